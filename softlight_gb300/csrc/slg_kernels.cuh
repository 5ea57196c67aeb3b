/*
 * slg_kernels.cuh - host-side entry points of the draw-path kernels.
 */
#ifndef SLG_KERNELS_CUH
#define SLG_KERNELS_CUH

#include <cuda_runtime.h>
#include "slg_device.cuh"

namespace slg
{

/* Enqueue one launch on s: ops' vertex stage, tile_scan, bin_fill, the tile
 * sort when the ordered raster may run, ops' raster stage. When ev is not
 * null, ev[0..4] are recorded before the vertex stage, after it, after
 * tile_scan, after bin_fill and after the raster. */
cudaError_t launch_pipeline(const Frame& f, const slg_pipeline_ops& ops, int keyCap, cudaStream_t s, cudaEvent_t* ev);

/* Largest tile grid whose lists a blended launch fills in key order (the
 * count and fill passes keep one word per tile and chunk in shared memory);
 * larger grids fill by atomics and sort per tile. */
constexpr int kMaxOrderedTiles = 4096;

/* Raises the dynamic shared-memory limits of the tile sort and of the
 * key-order fill once, so launches (and stream captures) need no attribute
 * calls. */
cudaError_t init_library_attributes(int keyCap);

/* The entry table of the built-in programs (slg_builtin_vertex.cu). */
const slg_pipeline_ops& builtin_pipeline();

/* Fill numTexels texels of bytesPerTexel bytes with value; skipped while
 * status (when not null) holds a capacity overflow. */
cudaError_t launch_clear(uint8_t* dst, size_t numTexels, int bytesPerTexel, const uint32_t value[8], const int32_t* status,
                         cudaStream_t s);

/* Nearest-neighbour blit of SL_BlitProcessor::blit_nearest over destination
 * pixels [x0, x0 + nx) x [y0, y0 + ny); all reads were checked in bounds. */
struct BlitArgs
{
    const uint8_t* src;
    uint8_t* dst;
    int32_t srcType, dstType;          /* slg_color_type */
    uint64_t srcW, dstW;
    uint64_t x0, y0, nx, ny;
    uint64_t foutW, foutH;             /* 16.16 source steps per destination pixel */
    uint64_t srcY0, srcY1;
    const int32_t* status;             /* skipped while it holds a capacity overflow; may be null */
};
cudaError_t launch_blit(const BlitArgs& a, cudaStream_t s);

/* Queued uniform-block uploads: a staging area of UboCopy records, then the
 * blocks' bytes (16-byte aligned); one CTA copies one block. */
struct UboCopy
{
    uint8_t* dst;
    uint32_t src;      /* byte offset of the block in the staging area */
    uint32_t words;    /* 4-byte words */
};
cudaError_t launch_ubo_scatter(const uint8_t* stage, uint32_t n, cudaStream_t s);

/* Scene graph: the device copy of a node (SL_SceneGraph's mNodeParentIds
 * and mCurrentTransforms, softlight/include/softlight/SL_SceneGraph.hpp:230-260). */
constexpr int kSceneMaxDepth = 64;    /* nodes on a path from a root, inclusive */
constexpr uint64_t kSceneRoot = ~0ull; /* SCENE_NODE_ROOT_ID */
struct SceneNodeGpu
{
    uint64_t parent;          /* kSceneRoot: attached to the root */
    float position[3];
    float scaling[3];
    float orientation[4];     /* quaternion x, y, z, w */
    uint32_t viewFps;         /* SL_TRANSFORM_TYPE_VIEW_FPS(_LOCKED_Y): R * TS instead of TS * R */
    uint32_t update;          /* recomputed by this update */
};

/* Recomputes the model matrices (16 floats per node, column-major) of the
 * n nodes in list (SL_SceneGraph::update's set for this call). */
cudaError_t launch_scene_update(const SceneNodeGpu* nodes, const uint32_t* list, uint32_t n, float* model, cudaStream_t s);

/* One draw of the scene's draw list: a submesh of a mesh node. */
struct SceneEntryGpu
{
    uint64_t node;
    uint32_t bounds;          /* bounding box index (8 floats: max xyzw, min xyzw) */
    uint32_t textureId;       /* the material's ambient texture */
    uint8_t* ubo;             /* the draw's slg_lambert_uniforms */
};

struct SceneDrawArgs
{
    const SceneEntryGpu* entries;
    uint32_t numEntries;
    int32_t cull;             /* frustum-cull by bounding box (sl_is_visible) */
    const float* model;       /* 16 floats per node */
    const float* bounds;
    DrawDesc* descs;          /* entry e's descriptor of the launch */
    float vp[16], view[16], planes[24];
    uint32_t templ[64];       /* the template uniform block, copied first */
    uint32_t templWords;
};

/* Writes each entry's uniform block (template, vpMatrix, modelMatrix,
 * textureId) and its descriptor's hidden flag. */
cudaError_t launch_scene_draw(const SceneDrawArgs& a, cudaStream_t s);

} // namespace slg

#endif /* SLG_KERNELS_CUH */
