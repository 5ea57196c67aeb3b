/*
 * scene_test.cpp - a C++ caller of the scene-graph entry points through the
 * facade (include/slg_context.hpp): a group node with two mesh-node children
 * (translations and scales only, so the model matrices are exact), one
 * update, the model matrices checked against parent x child, one draw list
 * into a 128x128 RGBA8 framebuffer. Prints the covered pixels; exit 0 when
 * every check holds.
 */
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "slg_context.hpp"
#include "slg_programs.h"

int main()
{
    const unsigned W = 128, H = 128;
    slg::Context ctx;
    if (!ctx.valid())
    {
        std::fprintf(stderr, "context: %s\n", ctx.last_error().c_str());
        return 2;
    }

    /* a quad in z = 0: position, uv, normal */
    const float v[4][8] = {{-1, -1, 0, 0, 0, 0, 0, 1}, {1, -1, 0, 1, 0, 0, 0, 1}, {1, 1, 0, 1, 1, 0, 0, 1}, {-1, 1, 0, 0, 1, 0, 0, 1}};
    const uint32_t idx[6] = {0, 1, 2, 0, 2, 3};
    const size_t vbo = ctx.create_vbo();
    ctx.vbo(vbo).init(sizeof(v), v);
    const size_t ibo = ctx.create_ibo();
    ctx.ibo(ibo).init(6, SLG_VERTEX_DATA_INT, idx);
    const size_t vao = ctx.create_vao();
    ctx.vao(vao).set_vertex_buffer(vbo);
    ctx.vao(vao).set_index_buffer(ibo);
    ctx.vao(vao).set_binding(0, 0, 32, 3, SLG_VERTEX_DATA_FLOAT);

    std::vector<uint8_t> texels(4 * 4 * 4, 200);
    const size_t tex = ctx.create_texture();
    ctx.texture(tex).init(SLG_COLOR_RGBA_8U, 4, 4);
    ctx.texture(tex).set_texels(texels.data(), texels.size());

    const size_t color = ctx.create_texture();
    ctx.texture(color).init(SLG_COLOR_RGBA_8U, W, H);
    const size_t depth = ctx.create_texture();
    ctx.texture(depth).init(SLG_COLOR_R_FLOAT, W, H);
    const size_t fbo = ctx.create_framebuffer();
    ctx.framebuffer(fbo).reserve_color_buffers(1);
    ctx.framebuffer(fbo).attach_color_buffer(0, color);
    ctx.framebuffer(fbo).attach_depth_buffer(depth);

    slg_lambert_uniforms u;
    std::memset(&u, 0, sizeof(u));
    for (int i = 0; i < 4; ++i) u.vpMatrix[5 * i] = u.modelMatrix[5 * i] = 1.f;
    u.lightDir[2] = 1.f;
    u.ambient[0] = u.ambient[1] = u.ambient[2] = 0.1f;
    u.textureId = (uint32_t)tex;
    const size_t ubo = ctx.create_ubo();
    ctx.ubo(ubo).assign(u);
    const slg_vertex_shader vs = {2, SLG_CULL_OFF, SLG_PROGRAM_LAMBERT_TEX};
    const slg_fragment_shader fs = {2, 1, SLG_BLEND_OFF, SLG_DEPTH_TEST_LESS_THAN, SLG_DEPTH_MASK_ON, SLG_PROGRAM_LAMBERT_TEX};
    const size_t shader = ctx.create_shader(vs, fs, ubo);

    const size_t sceneId = ctx.create_scene();
    slg::SceneGraphRef scene = ctx.scene(sceneId);
    const size_t material = scene.insert_material(tex);
    const slg_mesh quad = {vao, 0, 6, SLG_RENDER_MODE_INDEXED_TRIANGLES, (uint32_t)material};
    const float hi[3] = {1.f, 1.f, 0.f}, lo[3] = {-1.f, -1.f, 0.f};
    const size_t mesh = scene.insert_mesh(quad, hi, lo);
    const slg_transform tg = {{0.25f, 0.f, 0.f}, {1.f, 1.f, 1.f}, {0.f, 0.f, 0.f, 1.f}, 0};
    const slg_transform ta = {{-0.5f, 0.f, 0.f}, {0.25f, 0.25f, 1.f}, {0.f, 0.f, 0.f, 1.f}, 0};
    const slg_transform tb = {{0.f, 0.5f, 0.f}, {0.25f, 0.25f, 1.f}, {0.f, 0.f, 0.f, 1.f}, 0};
    const size_t group = scene.insert_empty_node(SLG_SCENE_ROOT, tg);
    const size_t a = scene.insert_mesh_node(group, 1, &mesh, ta);
    const size_t b = scene.insert_mesh_node(group, 1, &mesh, tb);
    if (group == SLG_INVALID_ID || a == SLG_INVALID_ID || b == SLG_INVALID_ID || scene.update())
    {
        std::fprintf(stderr, "scene: %s\n", ctx.last_error().c_str());
        return 3;
    }

    float models[3 * 16];
    if (scene.model_matrices(models, 3)) return 4;
    const float wantA[3] = {-0.25f, 0.f, 0.f}, wantB[3] = {0.25f, 0.5f, 0.f};
    for (int k = 0; k < 3; ++k)
    {
        if (models[16 * a + 12 + k] != wantA[k] || models[16 * b + 12 + k] != wantB[k])
        {
            std::fprintf(stderr, "model translation %d differs\n", k);
            return 5;
        }
    }
    if (models[16 * a] != 0.25f || models[16 * b + 5] != 0.25f) return 6;

    const double clear[4] = {0.0, 0.0, 0.0, 1.0};
    ctx.clear_framebuffer(fbo, 0, clear, 1.0);
    float ident[16] = {};
    for (int i = 0; i < 4; ++i) ident[5 * i] = 1.f;
    if (scene.draw(fbo, shader, ident, ident)) return 7;
    if (ctx.finish() != SLG_OK)
    {
        std::fprintf(stderr, "finish: %s\n", ctx.last_error().c_str());
        return 8;
    }
    std::vector<uint8_t> img(W * H * 4);
    ctx.texture(color).read(img.data(), img.size());
    size_t covered = 0;
    for (size_t i = 0; i < W * H; ++i) covered += img[4 * i] != 0;
    std::printf("%zu\n", covered);
    /* two quads of 32 x 32 pixels (NDC half-size 0.25 of 128 px) */
    return (covered >= 2 * 30 * 30 && covered <= 2 * 34 * 34) ? 0 : 9;
}
