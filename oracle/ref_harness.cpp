/*
 * ref_harness.cpp - drives SoftLight's own SL_Context (compiled unmodified
 * from the reference tree against oracle/ref_shim) through the C API of
 * include/slg.h with the prefix "slr_". Test infrastructure only: it lets the
 * CPU oracle (oracle/slo.cpp) be checked against the reference itself and
 * generates the golden fixtures under tests/golden.
 *
 * The built-in programs of include/slg_programs.h run as ordinary SoftLight
 * shader callbacks (SL_VertexShader::shader / SL_FragmentShader::shader); their
 * texture reads call the reference's sl_sample_bilinear
 * (softlight/include/softlight/SL_Sampler.hpp:187-218). Resource ids stored in
 * uniform blocks are resolved against the current context.
 */
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "softlight/SL_Color.hpp"
#include "softlight/SL_Context.hpp"
#include "softlight/SL_Framebuffer.hpp"
#include "softlight/SL_ImgFile.hpp"
#include "softlight/SL_IndexBuffer.hpp"
#include "softlight/SL_Mesh.hpp"
#include "softlight/SL_Sampler.hpp"
#include "softlight/SL_Shader.hpp"
#include "softlight/SL_Texture.hpp"
#include "softlight/SL_UniformBuffer.hpp"
#include "softlight/SL_VertexArray.hpp"
#include "softlight/SL_VertexBuffer.hpp"
#include "softlight/SL_BoundingBox.hpp"
#include "softlight/SL_Camera.hpp"
#include "softlight/SL_SceneGraph.hpp"
#include "softlight/SL_SceneNode.hpp"
#include "softlight/SL_Transform.hpp"

#include "../include/slg.h"
#include "../include/slg_programs.h"

namespace math = ls::math;

/* SL_Texture::init(const SL_ImgFile&) links against SL_ImgFile::data(), whose
 * definition needs FreeImage; image files are not used here. */
const void* SL_ImgFile::data() const { return nullptr; }

/* A reference scene graph with the materials the demos bind (the ambient
 * texture id per material). */
struct slr_scene
{
    SL_SceneGraph graph;
    std::vector<size_t> materials;
};

struct slr_context
{
    SL_Context ctx;
    std::string err;
    std::vector<size_t> shaderUbo; /* uniform block id of each shader */
    std::vector<std::unique_ptr<slr_scene>> scenes;

    /* SL_Context::create_shader stores &mUniforms[uboId]
     * (softlight/src/SL_Context.cpp:601), a pointer into a vector that a later
     * create_ubo may reallocate. Re-point every shader before drawing. */
    void bind_uniforms()
    {
        for (size_t i = 0; i < shaderUbo.size(); ++i)
        {
            if (shaderUbo[i] != SLG_INVALID_ID) ctx.shader(i).pUniforms = &ctx.ubo(shaderUbo[i]);
        }
    }
};

namespace
{

slr_context* g_current = nullptr;

struct RefEnv
{
    const SL_VertexBuffer* vbo;
    const SL_VertexArray* vao;
    const unsigned char* ubo;

    const float* vertex(uint64_t vertId) const
    {
        return vbo->element<const float>(vao->offset(0, (size_t)vertId));
    }
    const void* uniforms() const { return ubo; }
    const float* buffer(uint32_t vboId) const
    {
        return reinterpret_cast<const float*>(g_current->ctx.vbo(vboId).data());
    }
    slg_v4 sample_rgba8(uint32_t texId, float u, float v) const
    {
        const SL_Texture& t = g_current->ctx.texture(texId);
        const SL_ColorRGBA8 p = sl_sample_bilinear<SL_ColorRGBA8, SL_WrapMode::REPEAT>(t, u, v);
        const math::vec4 f = color_cast<float, uint8_t>(p);
        return slg_make_v4(f[0], f[1], f[2], f[3]);
    }
    slg_v4 sample_rgbaf(uint32_t texId, float u, float v) const
    {
        const SL_Texture& t = g_current->ctx.texture(texId);
        const SL_ColorRGBAf p = sl_sample_bilinear<SL_ColorRGBAf, SL_WrapMode::REPEAT>(t, u, v);
        return slg_make_v4(p[0], p[1], p[2], p[3]);
    }
};

template <uint32_t P>
math::vec4 vs_callback(SL_VertexParam& param)
{
    RefEnv env{param.pVbo, param.pVao, param.pUniforms->buffer()};
    slg_v4 vary[4];
    slg_v4 r;
    switch (P)
    {
        case SLG_PROGRAM_LAMBERT_TEX:      r = slg_vs_lambert(env, param.vertId, param.instanceId, vary); break;
        case SLG_PROGRAM_BLINN_PHONG_INST: r = slg_vs_blinn(env, param.vertId, param.instanceId, vary); break;
        case SLG_PROGRAM_VCOLOR_TEX_ALPHA:
        case SLG_PROGRAM_VCOLOR_TEXF:
        case SLG_PROGRAM_GBUFFER:
        case SLG_PROGRAM_VCOLOR_TEX_CUTOUT:
        case SLG_PROGRAM_FRAG_COORD:       r = slg_vs_vcolor(env, param.vertId, param.instanceId, vary); break;
        default:                           r = slg_vs_flat(env, param.vertId, param.instanceId, vary); break;
    }
    const int n = (P == SLG_PROGRAM_BLINN_PHONG_INST) ? 3 : (P == SLG_PROGRAM_FLAT_COLOR ? 0 : 2);
    for (int i = 0; i < n; ++i)
    {
        param.pVaryings[i] = math::vec4{vary[i].x, vary[i].y, vary[i].z, vary[i].w};
    }
    return math::vec4{r.x, r.y, r.z, r.w};
}

template <uint32_t P>
bool fs_callback(SL_FragmentParam& param)
{
    RefEnv env{nullptr, nullptr, param.pUniforms->buffer()};
    slg_v4 vary[4], outs[4];
    for (int i = 0; i < 4; ++i)
    {
        vary[i] = slg_make_v4(param.pVaryings[i][0], param.pVaryings[i][1], param.pVaryings[i][2], param.pVaryings[i][3]);
        outs[i] = slg_make_v4(0.f, 0.f, 0.f, 0.f);
    }
    bool r;
    switch (P)
    {
        case SLG_PROGRAM_LAMBERT_TEX:      r = slg_fs_lambert(env, vary, outs); break;
        case SLG_PROGRAM_BLINN_PHONG_INST: r = slg_fs_blinn(env, vary, outs); break;
        case SLG_PROGRAM_VCOLOR_TEX_ALPHA: r = slg_fs_vcolor_tex_alpha(env, vary, outs); break;
        case SLG_PROGRAM_VCOLOR_TEXF:      r = slg_fs_vcolor_texf(env, vary, outs); break;
        case SLG_PROGRAM_GBUFFER:          r = slg_fs_gbuffer(env, vary, outs); break;
        case SLG_PROGRAM_VCOLOR_TEX_CUTOUT: r = slg_fs_cutout(env, vary, outs); break;
        case SLG_PROGRAM_FRAG_COORD:
        {
            /* SL_FragmentParam::coord in and out: the reference writes the
             * depth the program leaves there */
            slg_frag_coord c;
            c.x = param.coord.x;
            c.y = param.coord.y;
            c.depth = param.coord.depth;
            r = slg_fs_frag_coord(env, &c, vary, outs);
            param.coord.depth = c.depth;
            break;
        }
        default:                           r = slg_fs_flat(env, vary, outs); break;
    }
    for (int i = 0; i < 4; ++i)
    {
        param.pOutputs[i] = math::vec4{outs[i].x, outs[i].y, outs[i].z, outs[i].w};
    }
    return r;
}

typedef math::vec4 (*VsFn)(SL_VertexParam&);
typedef bool (*FsFn)(SL_FragmentParam&);

VsFn vs_for(uint32_t p)
{
    switch (p)
    {
        case SLG_PROGRAM_LAMBERT_TEX:      return vs_callback<SLG_PROGRAM_LAMBERT_TEX>;
        case SLG_PROGRAM_BLINN_PHONG_INST: return vs_callback<SLG_PROGRAM_BLINN_PHONG_INST>;
        case SLG_PROGRAM_VCOLOR_TEX_ALPHA: return vs_callback<SLG_PROGRAM_VCOLOR_TEX_ALPHA>;
        case SLG_PROGRAM_VCOLOR_TEXF:      return vs_callback<SLG_PROGRAM_VCOLOR_TEXF>;
        case SLG_PROGRAM_FLAT_COLOR:       return vs_callback<SLG_PROGRAM_FLAT_COLOR>;
        case SLG_PROGRAM_GBUFFER:          return vs_callback<SLG_PROGRAM_GBUFFER>;
        case SLG_PROGRAM_VCOLOR_TEX_CUTOUT: return vs_callback<SLG_PROGRAM_VCOLOR_TEX_CUTOUT>;
        case SLG_PROGRAM_FRAG_COORD:       return vs_callback<SLG_PROGRAM_FRAG_COORD>;
        default:                           return nullptr;
    }
}

FsFn fs_for(uint32_t p)
{
    switch (p)
    {
        case SLG_PROGRAM_LAMBERT_TEX:      return fs_callback<SLG_PROGRAM_LAMBERT_TEX>;
        case SLG_PROGRAM_BLINN_PHONG_INST: return fs_callback<SLG_PROGRAM_BLINN_PHONG_INST>;
        case SLG_PROGRAM_VCOLOR_TEX_ALPHA: return fs_callback<SLG_PROGRAM_VCOLOR_TEX_ALPHA>;
        case SLG_PROGRAM_VCOLOR_TEXF:      return fs_callback<SLG_PROGRAM_VCOLOR_TEXF>;
        case SLG_PROGRAM_FLAT_COLOR:       return fs_callback<SLG_PROGRAM_FLAT_COLOR>;
        case SLG_PROGRAM_GBUFFER:          return fs_callback<SLG_PROGRAM_GBUFFER>;
        case SLG_PROGRAM_VCOLOR_TEX_CUTOUT: return fs_callback<SLG_PROGRAM_VCOLOR_TEX_CUTOUT>;
        case SLG_PROGRAM_FRAG_COORD:       return fs_callback<SLG_PROGRAM_FRAG_COORD>;
        default:                           return nullptr;
    }
}

SL_Mesh to_mesh(const slg_mesh* m)
{
    SL_Mesh r;
    r.vaoId = m->vaoId;
    r.elementBegin = m->elementBegin;
    r.elementEnd = m->elementEnd;
    r.mode = (SL_RenderMode)m->mode;
    r.materialId = m->materialId;
    return r;
}

size_t texel_bytes(const SL_Texture& t) { return (size_t)t.width() * t.height() * t.depth() * t.bpp(); }

} // namespace

extern "C" {

int slr_context_create(slr_context** out)
{
    *out = new slr_context();
    (*out)->ctx.num_threads(1);
    return SLG_OK;
}

void slr_context_destroy(slr_context* c) { delete c; }
const char* slr_last_error(const slr_context* c) { return c->err.c_str(); }
unsigned slr_num_threads(slr_context* c, unsigned n) { return n ? c->ctx.num_threads(n) : c->ctx.num_threads(); }

size_t slr_create_vbo(slr_context* c) { return c->ctx.create_vbo(); }
int slr_vbo_init(slr_context* c, size_t id, size_t n, const void* data)
{
    /* the GPU path pads vertex buffers by 64 bytes; do the same here */
    std::vector<uint8_t> tmp(n + 64, 0);
    if (data) std::memcpy(tmp.data(), data, n);
    return c->ctx.vbo(id).init(n + 64, tmp.data()) ? SLG_ERR_INVALID_ARG : SLG_OK;
}
int slr_vbo_assign(slr_context* c, size_t id, const void* data, size_t off, size_t n)
{
    c->ctx.vbo(id).assign(data, (ptrdiff_t)off, n);
    return SLG_OK;
}
size_t slr_create_ibo(slr_context* c) { return c->ctx.create_ibo(); }
int slr_ibo_init(slr_context* c, size_t id, size_t n, int type, const void* data)
{
    return c->ctx.ibo(id).init((uint32_t)n, (SL_DataType)type, data) ? SLG_ERR_INVALID_ARG : SLG_OK;
}
size_t slr_create_vao(slr_context* c) { return c->ctx.create_vao(); }
int slr_vao_set_vertex_buffer(slr_context* c, size_t vao, size_t vbo) { c->ctx.vao(vao).set_vertex_buffer(vbo); return SLG_OK; }
int slr_vao_set_index_buffer(slr_context* c, size_t vao, size_t ibo) { c->ctx.vao(vao).set_index_buffer(ibo); return SLG_OK; }
int slr_vao_set_binding(slr_context* c, size_t vao, unsigned bindId, ptrdiff_t offset, ptrdiff_t stride, unsigned comps, int type)
{
    SL_VertexArray& v = c->ctx.vao(vao);
    if (v.num_bindings() <= bindId) v.set_num_bindings(bindId + 1);
    v.set_binding(bindId, offset, stride, (SL_Dimension)(comps ? comps - 1 : 0), (SL_DataType)type);
    return SLG_OK;
}
size_t slr_create_texture(slr_context* c) { return c->ctx.create_texture(); }
int slr_texture_init(slr_context* c, size_t id, int type, uint16_t w, uint16_t h, uint16_t d)
{
    return c->ctx.texture(id).init((SL_ColorDataType)type, w, h, d) ? SLG_ERR_INVALID_ARG : SLG_OK;
}
int slr_texture_set_texels(slr_context* c, size_t id, const void* data, size_t n)
{
    SL_Texture& t = c->ctx.texture(id);
    if (n != texel_bytes(t)) return SLG_ERR_INVALID_ARG;
    std::memcpy(t.data(), data, n);
    return SLG_OK;
}
int slr_texture_read(slr_context* c, size_t id, void* dst, size_t n)
{
    const SL_Texture& t = c->ctx.texture(id);
    if (n != texel_bytes(t)) return SLG_ERR_INVALID_ARG;
    std::memcpy(dst, t.data(), n);
    return SLG_OK;
}
int slr_blit(slr_context* c, size_t out, size_t in)
{
    c->ctx.blit(out, in);
    return SLG_OK;
}
int slr_blit_rect(slr_context* c, size_t out, size_t in, uint16_t sx0, uint16_t sy0, uint16_t sx1, uint16_t sy1,
                  uint16_t dx0, uint16_t dy0, uint16_t dx1, uint16_t dy1)
{
    c->ctx.blit(out, in, sx0, sy0, sx1, sy1, dx0, dy0, dx1, dy1);
    return SLG_OK;
}
int slr_blit_read(slr_context* c, size_t in, int type, uint16_t w, uint16_t h, void* dst, size_t n)
{
    (void)n;
    SL_TextureView view;
    sl_texture_view_from_buffer(view, w, h, 1, (SL_ColorDataType)type, dst);
    c->ctx.blit(view, in);
    return SLG_OK;
}
size_t slr_create_framebuffer(slr_context* c) { return c->ctx.create_framebuffer(); }
int slr_fbo_reserve_color_buffers(slr_context* c, size_t fbo, unsigned n)
{
    return c->ctx.framebuffer(fbo).reserve_color_buffers(n) ? SLG_ERR_INVALID_ARG : SLG_OK;
}
int slr_fbo_attach_color_buffer(slr_context* c, size_t fbo, unsigned i, size_t tex)
{
    return c->ctx.framebuffer(fbo).attach_color_buffer(i, c->ctx.texture(tex).view()) ? SLG_ERR_INVALID_ARG : SLG_OK;
}
int slr_fbo_attach_depth_buffer(slr_context* c, size_t fbo, size_t tex)
{
    return c->ctx.framebuffer(fbo).attach_depth_buffer(c->ctx.texture(tex).view()) ? SLG_ERR_INVALID_ARG : SLG_OK;
}
size_t slr_create_ubo(slr_context* c)
{
    const size_t id = c->ctx.create_ubo();
    std::memset(c->ctx.ubo(id).buffer(), 0, SL_MAX_UNIFORM_BUFFER_SIZE);
    return id;
}
int slr_ubo_assign(slr_context* c, size_t id, const void* data, size_t n)
{
    if (n > SL_MAX_UNIFORM_BUFFER_SIZE) return SLG_ERR_INVALID_ARG;
    std::memcpy(c->ctx.ubo(id).buffer(), data, n);
    return SLG_OK;
}
size_t slr_create_shader(slr_context* c, const slg_vertex_shader* vs, const slg_fragment_shader* fs, size_t ubo)
{
    SL_VertexShader v;
    v.numVaryings = vs->numVaryings;
    v.cullMode = (SL_CullMode)vs->cullMode;
    v.shader = vs_for(vs->program);
    SL_FragmentShader f;
    f.numVaryings = fs->numVaryings;
    f.numOutputs = fs->numOutputs;
    f.blend = (SL_BlendMode)fs->blend;
    f.depthTest = (SL_DepthTest)fs->depthTest;
    f.depthMask = (SL_DepthMask)fs->depthMask;
    f.shader = fs_for(fs->program);
    if (!v.shader || !f.shader) return SLG_INVALID_ID;
    const size_t id = (ubo == SLG_INVALID_ID) ? c->ctx.create_shader(v, f) : c->ctx.create_shader(v, f, ubo);
    if (id != SLG_INVALID_ID)
    {
        c->shaderUbo.resize(id + 1, SLG_INVALID_ID);
        c->shaderUbo[id] = ubo;
    }
    return id;
}
int slr_clear_framebuffer(slr_context* c, size_t fbo, unsigned att, const double rgba[4], double depth)
{
    c->ctx.clear_framebuffer(fbo, att, math::vec4_t<double>{rgba[0], rgba[1], rgba[2], rgba[3]}, depth);
    return SLG_OK;
}
int slr_clear_color_buffer(slr_context* c, size_t fbo, unsigned att, const double rgba[4])
{
    c->ctx.clear_color_buffer(fbo, att, math::vec4_t<double>{rgba[0], rgba[1], rgba[2], rgba[3]});
    return SLG_OK;
}
int slr_clear_depth_buffer(slr_context* c, size_t fbo, double depth)
{
    c->ctx.clear_depth_buffer(fbo, depth);
    return SLG_OK;
}
int slr_draw(slr_context* c, const slg_mesh* m, size_t shader, size_t fbo)
{
    g_current = c;
    c->bind_uniforms();
    c->ctx.draw(to_mesh(m), shader, fbo);
    return SLG_OK;
}
int slr_draw_instanced(slr_context* c, const slg_mesh* m, size_t n, size_t shader, size_t fbo)
{
    g_current = c;
    c->bind_uniforms();
    if (n == 0) return SLG_OK;
    if (n == 1) c->ctx.draw(to_mesh(m), shader, fbo);
    else c->ctx.draw_instanced(to_mesh(m), n, shader, fbo);
    return SLG_OK;
}
int slr_draw_multiple(slr_context* c, const slg_mesh* ms, size_t n, size_t shader, size_t fbo)
{
    g_current = c;
    c->bind_uniforms();
    std::vector<SL_Mesh> v;
    for (size_t i = 0; i < n; ++i) v.push_back(to_mesh(&ms[i]));
    c->ctx.draw_multiple(v.data(), n, shader, fbo);
    return SLG_OK;
}
int slr_draw_batch(slr_context* c, const slg_draw_cmd* cmds, size_t n, size_t fbo)
{
    for (size_t i = 0; i < n; ++i)
    {
        slr_draw_instanced(c, &cmds[i].mesh, cmds[i].numInstances, cmds[i].shaderId, fbo);
    }
    return SLG_OK;
}
int slr_finish(slr_context*) { return SLG_OK; }

/*-----------------------------------------------------------------------------
 * Scene graph: the reference's SL_SceneGraph, SL_Transform, SL_BoundingBox and
 * sl_extract_frustum_planes / sl_is_visible drive the demos' traversal
 * (softlight/tests/sl_large_scene_test.cpp:678-740), which is caller code and
 * restated here: per mesh node the model and view-projection matrices, per
 * submesh the frustum test, the triangle-mode test, the material's texture
 * and SL_Context::draw.
-----------------------------------------------------------------------------*/
static SL_Transform make_transform(const slg_transform* t)
{
    SL_Transform r{(SL_TransformType)t->type};
    r.position(math::vec3{t->position[0], t->position[1], t->position[2]});
    r.scaling(math::vec3{t->scaling[0], t->scaling[1], t->scaling[2]});
    r.orientation(math::quat{t->orientation[0], t->orientation[1], t->orientation[2], t->orientation[3]});
    return r;
}

size_t slr_create_scene(slr_context* c)
{
    c->scenes.emplace_back(new slr_scene());
    return c->scenes.size() - 1;
}

int slr_scene_insert_mesh(slr_context* c, size_t sid, const slg_mesh* m, const float maxPoint[3], const float minPoint[3], size_t* out)
{
    SL_BoundingBox bb;
    bb.max_point(math::vec3{maxPoint[0], maxPoint[1], maxPoint[2]});
    bb.min_point(math::vec3{minPoint[0], minPoint[1], minPoint[2]});
    *out = c->scenes[sid]->graph.insert_mesh(to_mesh(m), bb);
    return SLG_OK;
}

int slr_scene_insert_material(slr_context* c, size_t sid, size_t tex, size_t* out)
{
    c->scenes[sid]->materials.push_back(tex);
    *out = c->scenes[sid]->materials.size() - 1;
    return SLG_OK;
}

int slr_scene_insert_node(slr_context* c, size_t sid, size_t parent, size_t n, const size_t* ids, const slg_transform* t, size_t* out)
{
    SL_SceneGraph& g = c->scenes[sid]->graph;
    const SL_Transform tr = make_transform(t);
    *out = n ? g.insert_mesh_node(parent, "node", n, ids, tr) : g.insert_empty_node(parent, "node", tr);
    return SLG_OK;
}

int slr_scene_set_transform(slr_context* c, size_t sid, size_t node, const slg_transform* t)
{
    SL_Transform& tr = c->scenes[sid]->graph.mCurrentTransforms[node];
    tr.type((SL_TransformType)t->type);
    tr.position(math::vec3{t->position[0], t->position[1], t->position[2]});
    tr.scaling(math::vec3{t->scaling[0], t->scaling[1], t->scaling[2]});
    tr.orientation(math::quat{t->orientation[0], t->orientation[1], t->orientation[2], t->orientation[3]});
    return SLG_OK;
}

int slr_scene_update(slr_context* c, size_t sid)
{
    c->scenes[sid]->graph.update();
    return SLG_OK;
}

int slr_scene_read_models(slr_context* c, size_t sid, float* out, size_t n)
{
    SL_SceneGraph& g = c->scenes[sid]->graph;
    if (n != g.mModelMatrices.size()) return SLG_ERR_INVALID_ARG;
    for (size_t i = 0; i < n; ++i) std::memcpy(out + 16 * i, &g.mModelMatrices[i], 64);
    return SLG_OK;
}

int slr_scene_draw(slr_context* c, size_t sid, size_t fbo, size_t shader, const float projection[16], const float view[16],
                   const float cullProjection[16])
{
    slr_scene& sc = *c->scenes[sid];
    SL_SceneGraph& g = sc.graph;
    math::mat4 p, v;
    std::memcpy(&p, projection, 64);
    std::memcpy(&v, view, 64);
    const bool cull = cullProjection != nullptr;
    math::vec4 planes[6];
    if (cull)
    {
        math::mat4 cp;
        std::memcpy(&cp, cullProjection, 64);
        sl_extract_frustum_planes(cp, planes);
    }
    const math::mat4 vp = p * v;
    const size_t ubo = c->shaderUbo[shader];
    slg_lambert_uniforms* u = reinterpret_cast<slg_lambert_uniforms*>(c->ctx.ubo(ubo).buffer());
    slg_lambert_uniforms saved;
    std::memcpy(&saved, u, sizeof(saved));
    for (size_t nodeId = 0; nodeId < g.mNodes.size(); ++nodeId)
    {
        const SL_SceneNode& n = g.mNodes[nodeId];
        if (n.type != NODE_TYPE_MESH) continue;
        const math::mat4& modelMat = g.mModelMatrices[nodeId];
        const math::mat4 mv = v * modelMat;
        std::memcpy(u->vpMatrix, &vp, 64);
        std::memcpy(u->modelMatrix, &modelMat, 64);
        const size_t numNodeMeshes = g.mNumNodeMeshes[n.dataId];
        const size_t* meshIds = g.mNodeMeshes[n.dataId].get();
        for (size_t k = 0; k < numNodeMeshes; ++k)
        {
            const size_t meshId = meshIds[k];
            const SL_Mesh& m = g.mMeshes[meshId];
            if (cull && !sl_is_visible(g.mMeshBounds[meshId], mv, planes)) continue;
            if (!(m.mode & SL_RenderMode::RENDER_MODE_TRIANGLES)) continue;
            u->textureId = (uint32_t)sc.materials[m.materialId];
            slg_mesh gm;
            gm.vaoId = m.vaoId;
            gm.elementBegin = m.elementBegin;
            gm.elementEnd = m.elementEnd;
            gm.mode = (uint32_t)m.mode;
            gm.materialId = m.materialId;
            slr_draw(c, &gm, shader, fbo);
        }
    }
    std::memcpy(u, &saved, sizeof(saved));
    return SLG_OK;
}

} // extern "C"
