/*
 * slg_context.hpp - header-only C++ facade with SoftLight's SL_Context shape
 * over the C ABI of slg.h.
 *
 * Method names, argument meaning and error conventions follow
 * softlight/include/softlight/SL_Context.hpp:59-306: create_* return size_t
 * ids ((size_t)-1 on error), draw / draw_multiple / draw_instanced are
 * `void ... noexcept` (errors are kept and reported by last_error() and by
 * finish()), and the resource objects are reached through accessors
 * (vao(id).set_binding(...), texture(id).init(...), framebuffer(id).
 * attach_color_buffer(...)) as in the reference. A SoftLight caller switches
 * by replacing SL_Context with slg::Context, SL_Mesh with slg_mesh and shader
 * function pointers with program ids (slg_programs.h).
 */
#ifndef SLG_CONTEXT_HPP
#define SLG_CONTEXT_HPP

#include <cstddef>
#include <string>

#include "slg.h"

namespace slg
{

class Context;

/* SL_VertexArray (softlight/include/softlight/SL_VertexArray.hpp:56-85) */
class VertexArrayRef
{
  public:
    VertexArrayRef(slg_context* c, size_t id) noexcept : mCtx(c), mId(id) {}
    void set_vertex_buffer(size_t vboId) noexcept { slg_vao_set_vertex_buffer(mCtx, mId, vboId); }
    void set_index_buffer(size_t iboId) noexcept { slg_vao_set_index_buffer(mCtx, mId, iboId); }
    void set_binding(size_t bindId, ptrdiff_t offset, ptrdiff_t stride, unsigned numComponents, int type) noexcept
    {
        slg_vao_set_binding(mCtx, mId, (unsigned)bindId, offset, stride, numComponents, type);
    }
  private:
    slg_context* mCtx;
    size_t mId;
};

/* SL_VertexBuffer (softlight/include/softlight/SL_VertexBuffer.hpp:33-49) */
class VertexBufferRef
{
  public:
    VertexBufferRef(slg_context* c, size_t id) noexcept : mCtx(c), mId(id) {}
    int init(size_t numBytes, const void* data = nullptr) noexcept { return slg_vbo_init(mCtx, mId, numBytes, data); }
    void assign(const void* data, ptrdiff_t offset, size_t numBytes) noexcept { slg_vbo_assign(mCtx, mId, data, (size_t)offset, numBytes); }
  private:
    slg_context* mCtx;
    size_t mId;
};

/* SL_IndexBuffer (softlight/src/SL_IndexBuffer.cpp:138) */
class IndexBufferRef
{
  public:
    IndexBufferRef(slg_context* c, size_t id) noexcept : mCtx(c), mId(id) {}
    int init(size_t numElements, int type, const void* data = nullptr) noexcept { return slg_ibo_init(mCtx, mId, numElements, type, data); }
  private:
    slg_context* mCtx;
    size_t mId;
};

/* SL_Texture (softlight/src/SL_Texture.cpp:276) */
class TextureRef
{
  public:
    TextureRef(slg_context* c, size_t id) noexcept : mCtx(c), mId(id) {}
    int init(int type, uint16_t w, uint16_t h, uint16_t d = 1) noexcept { return slg_texture_init(mCtx, mId, type, w, h, d); }
    int set_texels(const void* data, size_t numBytes) noexcept { return slg_texture_set_texels(mCtx, mId, data, numBytes); }
    int read(void* dst, size_t numBytes) noexcept { return slg_texture_read(mCtx, mId, dst, numBytes); }
  private:
    slg_context* mCtx;
    size_t mId;
};

/* SL_Framebuffer (softlight/src/SL_Framebuffer.cpp:823,855,908). Attachments
 * are texture ids where the reference passes SL_TextureView references. */
class FramebufferRef
{
  public:
    FramebufferRef(slg_context* c, size_t id) noexcept : mCtx(c), mId(id) {}
    int reserve_color_buffers(unsigned n) noexcept { return slg_fbo_reserve_color_buffers(mCtx, mId, n); }
    int attach_color_buffer(unsigned index, size_t texId) noexcept { return slg_fbo_attach_color_buffer(mCtx, mId, index, texId); }
    int attach_depth_buffer(size_t texId) noexcept { return slg_fbo_attach_depth_buffer(mCtx, mId, texId); }
  private:
    slg_context* mCtx;
    size_t mId;
};

/* SL_UniformBuffer: 1024 bytes (softlight/include/softlight/SL_UniformBuffer.hpp:12-20) */
class UniformBufferRef
{
  public:
    UniformBufferRef(slg_context* c, size_t id) noexcept : mCtx(c), mId(id) {}
    template <typename T> int assign(const T& block) noexcept
    {
        static_assert(sizeof(T) <= 1024, "uniform blocks hold at most 1024 bytes");
        return slg_ubo_assign(mCtx, mId, &block, sizeof(T));
    }
  private:
    slg_context* mCtx;
    size_t mId;
};

/* SL_SceneGraph (softlight/include/softlight/SL_SceneGraph.hpp:215):
 * insert_mesh / insert_empty_node / insert_mesh_node, a node's current
 * transform, update(), mModelMatrices, and the draw list of the mesh nodes
 * (the traversal SoftLight's demos write by hand). Insertion calls return
 * SLG_INVALID_ID on error. */
class SceneGraphRef
{
  public:
    SceneGraphRef(slg_context* c, size_t id) noexcept : mCtx(c), mId(id) {}
    size_t insert_mesh(const slg_mesh& m, const float maxPoint[3], const float minPoint[3]) noexcept
    {
        size_t out = SLG_INVALID_ID;
        return slg_scene_insert_mesh(mCtx, mId, &m, maxPoint, minPoint, &out) ? SLG_INVALID_ID : out;
    }
    size_t insert_material(size_t ambientTextureId) noexcept
    {
        size_t out = SLG_INVALID_ID;
        return slg_scene_insert_material(mCtx, mId, ambientTextureId, &out) ? SLG_INVALID_ID : out;
    }
    size_t insert_empty_node(size_t parentId, const slg_transform& t) noexcept
    {
        size_t out = SLG_INVALID_ID;
        return slg_scene_insert_node(mCtx, mId, parentId, 0, nullptr, &t, &out) ? SLG_INVALID_ID : out;
    }
    size_t insert_mesh_node(size_t parentId, size_t numSubMeshes, const size_t* subMeshIds, const slg_transform& t) noexcept
    {
        size_t out = SLG_INVALID_ID;
        return slg_scene_insert_node(mCtx, mId, parentId, numSubMeshes, subMeshIds, &t, &out) ? SLG_INVALID_ID : out;
    }
    int transform(size_t nodeId, const slg_transform& t) noexcept { return slg_scene_set_transform(mCtx, mId, nodeId, &t); }
    int update() noexcept { return slg_scene_update(mCtx, mId); }
    int model_matrices(float* out, size_t numNodes) noexcept { return slg_scene_read_models(mCtx, mId, out, numNodes); }
    int draw(size_t fboId, size_t shaderId, const float projection[16], const float view[16],
             const float cullProjection[16] = nullptr) noexcept
    {
        return slg_scene_draw(mCtx, mId, fboId, shaderId, projection, view, cullProjection);
    }
  private:
    slg_context* mCtx;
    size_t mId;
};

class Context
{
  public:
    Context() noexcept { mStatus = slg_context_create(&mCtx); }
    ~Context() noexcept { if (mCtx) slg_context_destroy(mCtx); }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;

    bool valid() const noexcept { return mCtx != nullptr && mStatus == SLG_OK; }
    std::string last_error() const { return mCtx ? std::string(slg_last_error(mCtx)) : std::string("no context"); }
    slg_context* handle() noexcept { return mCtx; }

    size_t create_vao() noexcept { return slg_create_vao(mCtx); }
    size_t create_vbo() noexcept { return slg_create_vbo(mCtx); }
    size_t create_ibo() noexcept { return slg_create_ibo(mCtx); }
    size_t create_texture() noexcept { return slg_create_texture(mCtx); }
    size_t create_framebuffer() noexcept { return slg_create_framebuffer(mCtx); }
    size_t create_ubo() noexcept { return slg_create_ubo(mCtx); }
    size_t create_shader(const slg_vertex_shader& vs, const slg_fragment_shader& fs, size_t uboId = SLG_INVALID_ID) noexcept
    {
        return slg_create_shader(mCtx, &vs, &fs, uboId);
    }

    VertexArrayRef vao(size_t id) noexcept { return VertexArrayRef(mCtx, id); }
    VertexBufferRef vbo(size_t id) noexcept { return VertexBufferRef(mCtx, id); }
    IndexBufferRef ibo(size_t id) noexcept { return IndexBufferRef(mCtx, id); }
    TextureRef texture(size_t id) noexcept { return TextureRef(mCtx, id); }
    FramebufferRef framebuffer(size_t id) noexcept { return FramebufferRef(mCtx, id); }
    UniformBufferRef ubo(size_t id) noexcept { return UniformBufferRef(mCtx, id); }
    size_t create_scene() noexcept { return slg_create_scene(mCtx); }
    SceneGraphRef scene(size_t id) noexcept { return SceneGraphRef(mCtx, id); }

    /* SL_Context::draw / draw_multiple / draw_instanced: void and noexcept as
     * in the reference; a failure is recorded for finish() / last_error(). */
    void draw(const slg_mesh& m, size_t shaderId, size_t fboId) noexcept { note(slg_draw(mCtx, &m, shaderId, fboId)); }
    void draw_multiple(const slg_mesh* m, size_t n, size_t shaderId, size_t fboId) noexcept { note(slg_draw_multiple(mCtx, m, n, shaderId, fboId)); }
    void draw_instanced(const slg_mesh& m, size_t n, size_t shaderId, size_t fboId) noexcept { note(slg_draw_instanced(mCtx, &m, n, shaderId, fboId)); }
    void draw_batch(const slg_draw_cmd* cmds, size_t n, size_t fboId) noexcept { note(slg_draw_batch(mCtx, cmds, n, fboId)); }

    /* SL_Context::blit (softlight/src/SL_Context.cpp:747-880); the window
     * buffer form becomes a read into host memory of the given format */
    void blit(size_t outTextureId, size_t inTextureId) noexcept { note(slg_blit(mCtx, outTextureId, inTextureId)); }
    void blit(size_t outTextureId, size_t inTextureId, uint16_t srcX0, uint16_t srcY0, uint16_t srcX1, uint16_t srcY1,
              uint16_t dstX0, uint16_t dstY0, uint16_t dstX1, uint16_t dstY1) noexcept
    {
        note(slg_blit_rect(mCtx, outTextureId, inTextureId, srcX0, srcY0, srcX1, srcY1, dstX0, dstY0, dstX1, dstY1));
    }
    int blit_read(size_t textureId, int colorType, uint16_t w, uint16_t h, void* dst, size_t numBytes) noexcept
    {
        return slg_blit_read(mCtx, textureId, colorType, w, h, dst, numBytes);
    }

    void clear_color_buffer(size_t fboId, unsigned attachment, const double rgba[4]) noexcept { note(slg_clear_color_buffer(mCtx, fboId, attachment, rgba)); }
    void clear_depth_buffer(size_t fboId, double depth) noexcept { note(slg_clear_depth_buffer(mCtx, fboId, depth)); }
    void clear_framebuffer(size_t fboId, unsigned attachment, const double rgba[4], double depth) noexcept
    {
        note(slg_clear_framebuffer(mCtx, fboId, attachment, rgba, depth));
    }

    unsigned num_threads() const noexcept { return slg_num_threads(mCtx, 0); }
    unsigned num_threads(unsigned n) noexcept { return slg_num_threads(mCtx, n); }

    /* Waits for queued draws; returns the first error since the last call. */
    int finish() noexcept
    {
        const int r = slg_finish(mCtx);
        const int first = mStatus != SLG_OK ? mStatus : r;
        mStatus = SLG_OK;
        return first;
    }

  private:
    void note(int r) noexcept { if (r != SLG_OK && mStatus == SLG_OK) mStatus = r; }
    slg_context* mCtx = nullptr;
    int mStatus = SLG_OK;
};

} // namespace slg

#endif /* SLG_CONTEXT_HPP */
