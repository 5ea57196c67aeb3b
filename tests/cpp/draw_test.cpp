/*
 * draw_test.cpp - a C++ caller of the GB300 draw path through the
 * SL_Context-shaped facade (include/slg_context.hpp), written the way
 * softlight/tests/sl_draw_test.cpp:108-194 uses SL_Context: one triangle,
 * flat colour, depth test off, into a 640x480 RGBA8 framebuffer. Writes the
 * colour attachment as raw RGBA8 to the path in argv[1].
 */
#include <cstdio>
#include <vector>

#include "slg_context.hpp"
#include "slg_programs.h"

int main(int argc, char** argv)
{
    const unsigned W = 640, H = 480;
    slg::Context ctx;
    if (!ctx.valid())
    {
        std::fprintf(stderr, "context: %s\n", ctx.last_error().c_str());
        return 2;
    }

    const float verts[3][9] = {
        {-0.9f, -0.9f, 0.f, 0, 0, 0, 0, 0, 0},
        { 0.9f, -0.9f, 0.f, 0, 0, 0, 0, 0, 0},
        { 0.0f,  0.9f, 0.f, 0, 0, 0, 0, 0, 0},
    };
    const size_t vbo = ctx.create_vbo();
    ctx.vbo(vbo).init(sizeof(verts), verts);
    const size_t vao = ctx.create_vao();
    ctx.vao(vao).set_vertex_buffer(vbo);
    ctx.vao(vao).set_binding(0, 0, 36, 3, SLG_VERTEX_DATA_FLOAT);

    const size_t color = ctx.create_texture();
    ctx.texture(color).init(SLG_COLOR_RGBA_8U, W, H);
    const size_t depth = ctx.create_texture();
    ctx.texture(depth).init(SLG_COLOR_R_FLOAT, W, H);
    const size_t fbo = ctx.create_framebuffer();
    ctx.framebuffer(fbo).reserve_color_buffers(1);
    ctx.framebuffer(fbo).attach_color_buffer(0, color);
    ctx.framebuffer(fbo).attach_depth_buffer(depth);

    slg_flat_uniforms u = {};
    for (int i = 0; i < 4; ++i) u.mvpMatrix[i * 5] = 1.f;
    u.color[0] = 1.f; u.color[1] = 0.5f; u.color[2] = 0.25f; u.color[3] = 1.f;
    const size_t ubo = ctx.create_ubo();
    ctx.ubo(ubo).assign(u);

    const slg_vertex_shader vs = {0, SLG_CULL_OFF, SLG_PROGRAM_FLAT_COLOR};
    const slg_fragment_shader fs = {0, 1, SLG_BLEND_OFF, SLG_DEPTH_TEST_OFF, SLG_DEPTH_MASK_OFF, SLG_PROGRAM_FLAT_COLOR};
    const size_t shader = ctx.create_shader(vs, fs, ubo);
    if (shader == SLG_INVALID_ID)
    {
        std::fprintf(stderr, "create_shader: %s\n", ctx.last_error().c_str());
        return 3;
    }

    const double clearColor[4] = {0.0, 0.0, 0.0, 1.0};
    ctx.clear_framebuffer(fbo, 0, clearColor, 1.0);
    const slg_mesh mesh = {vao, 0, 3, SLG_RENDER_MODE_TRIANGLES, 0};
    ctx.draw(mesh, shader, fbo);
    if (ctx.finish() != SLG_OK)
    {
        std::fprintf(stderr, "draw: %s\n", ctx.last_error().c_str());
        return 4;
    }

    std::vector<unsigned char> pixels(W * H * 4);
    if (ctx.texture(color).read(pixels.data(), pixels.size()) != SLG_OK) return 5;
    FILE* fh = std::fopen(argc > 1 ? argv[1] : "draw_test.rgba", "wb");
    if (!fh) return 6;
    std::fwrite(pixels.data(), 1, pixels.size(), fh);
    std::fclose(fh);
    return 0;
}
