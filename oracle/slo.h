/*
 * slo.h - C API of the CPU oracle (test infrastructure, not product code).
 *
 * The oracle is a CPU restatement of SoftLight's triangle draw path (the
 * portable, non-SIMD branches, single-threaded ordering) used only by the
 * tests, the smoke check and the CPU-baseline leg of the benchmark to check
 * and time the GPU path. It exposes the same entry points as include/slg.h
 * with an "slo_" prefix so a scene can be built identically on both.
 */
#ifndef SLO_H
#define SLO_H

#include "../include/slg.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct slo_context slo_context;

int         slo_context_create(slo_context** outCtx);
void        slo_context_destroy(slo_context* ctx);
const char* slo_last_error(const slo_context* ctx);
unsigned    slo_num_threads(slo_context* ctx, unsigned n);

size_t slo_create_vbo(slo_context* ctx);
int    slo_vbo_init(slo_context* ctx, size_t vboId, size_t numBytes, const void* data);
int    slo_vbo_assign(slo_context* ctx, size_t vboId, const void* data, size_t offset, size_t numBytes);
size_t slo_create_ibo(slo_context* ctx);
int    slo_ibo_init(slo_context* ctx, size_t iboId, size_t numElements, int indexType, const void* data);
size_t slo_create_vao(slo_context* ctx);
int    slo_vao_set_vertex_buffer(slo_context* ctx, size_t vaoId, size_t vboId);
int    slo_vao_set_index_buffer(slo_context* ctx, size_t vaoId, size_t iboId);
int    slo_vao_set_binding(slo_context* ctx, size_t vaoId, unsigned bindId, ptrdiff_t offset,
                           ptrdiff_t stride, unsigned numComponents, int dataType);
size_t slo_create_texture(slo_context* ctx);
int    slo_texture_init(slo_context* ctx, size_t texId, int colorType, uint16_t w, uint16_t h, uint16_t d);
int    slo_texture_set_texels(slo_context* ctx, size_t texId, const void* data, size_t numBytes);
int    slo_texture_read(slo_context* ctx, size_t texId, void* dst, size_t numBytes);
int    slo_blit(slo_context* ctx, size_t outTextureId, size_t inTextureId);
int    slo_blit_rect(slo_context* ctx, size_t outTextureId, size_t inTextureId, uint16_t srcX0, uint16_t srcY0,
                     uint16_t srcX1, uint16_t srcY1, uint16_t dstX0, uint16_t dstY0, uint16_t dstX1, uint16_t dstY1);
int    slo_blit_read(slo_context* ctx, size_t inTextureId, int dstColorType, uint16_t dstW, uint16_t dstH, void* dst,
                     size_t numBytes);
size_t slo_create_framebuffer(slo_context* ctx);
int    slo_fbo_reserve_color_buffers(slo_context* ctx, size_t fboId, unsigned numColorBuffers);
int    slo_fbo_attach_color_buffer(slo_context* ctx, size_t fboId, unsigned index, size_t texId);
int    slo_fbo_attach_depth_buffer(slo_context* ctx, size_t fboId, size_t texId);
size_t slo_create_ubo(slo_context* ctx);
int    slo_ubo_assign(slo_context* ctx, size_t uboId, const void* data, size_t numBytes);
size_t slo_create_shader(slo_context* ctx, const slg_vertex_shader* vs,
                         const slg_fragment_shader* fs, size_t uboId);
int slo_clear_framebuffer(slo_context* ctx, size_t fboId, unsigned attachment, const double rgba[4], double depth);
int slo_clear_color_buffer(slo_context* ctx, size_t fboId, unsigned attachment, const double rgba[4]);
int slo_clear_depth_buffer(slo_context* ctx, size_t fboId, double depth);
int slo_draw(slo_context* ctx, const slg_mesh* m, size_t shaderId, size_t fboId);
int slo_draw_instanced(slo_context* ctx, const slg_mesh* m, size_t numInstances, size_t shaderId, size_t fboId);
int slo_draw_multiple(slo_context* ctx, const slg_mesh* meshes, size_t numMeshes, size_t shaderId, size_t fboId);
int slo_draw_batch(slo_context* ctx, const slg_draw_cmd* cmds, size_t numCmds, size_t fboId);
int slo_finish(slo_context* ctx);

/* Statistics of the last draw call: triangles pushed to bins and fragments
 * that passed the depth test. */
void slo_last_stats(const slo_context* ctx, uint64_t* numBins, uint64_t* numFragments);

#ifdef __cplusplus
}
#endif

#endif /* SLO_H */
