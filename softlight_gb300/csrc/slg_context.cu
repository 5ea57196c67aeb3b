/*
 * slg_context.cu - host side of the GB300 draw path: the SL_Context-shaped
 * resource model and the C ABI declared in include/slg.h.
 *
 * The context owns device mirrors of every resource the reference's
 * SL_Context owns (softlight/include/softlight/SL_Context.hpp:66-82):
 * vertex/index/uniform buffers and textures live in HBM from init/assign
 * until the context is destroyed. Draws enqueue kernels on the context's
 * stream and return; results become visible to the host at slg_finish or
 * slg_texture_read, which also report any device-side error of the queued
 * draws.
 */
#include <algorithm>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/slg.h"
#include "slg_adjoint.cuh"
#include "slg_device.cuh"
#include "slg_kernels.cuh"

using slg::DrawDesc;
using slg::Frame;
using slg::TexView;

namespace
{

struct DevBuffer
{
    void*  ptr = nullptr;
    size_t bytes = 0;
};

struct Vbo { DevBuffer buf; size_t size = 0; };
struct Ibo { DevBuffer buf; int type = SLG_VERTEX_DATA_INVALID; size_t count = 0; uint64_t maxIndex = 0; };
struct Binding { ptrdiff_t offset = 0, stride = 0; unsigned comps = 0; int type = 0; };
struct Vao { size_t vbo = SLG_INVALID_ID, ibo = SLG_INVALID_ID; Binding bindings[8]; };
struct Texture { DevBuffer buf; int type = -1; uint16_t w = 0, h = 0, d = 0; unsigned bpt = 0; };
struct Fbo
{
    unsigned numColors = 0;
    size_t colors[4] = {SLG_INVALID_ID, SLG_INVALID_ID, SLG_INVALID_ID, SLG_INVALID_ID};
    size_t depth = SLG_INVALID_ID;
    DevBuffer vis;          /* visibility map, when enabled */
    bool visEnabled = false;
};
struct Ubo { DevBuffer buf; uint8_t shadow[1024] = {}; uint32_t pending = 0; /* bytes queued for upload */ };
struct Shader
{
    uint8_t cull, depthTest, depthMask, blend, numVaryings, numOutputs;
    uint32_t vsProgram, fsProgram;
    size_t ubo;
    uint32_t programSet;     /* 0: built-in programs, else 1 + the registration */
    uint32_t fsFlags;        /* SLG_PROGRAM_DISCARDS | SLG_PROGRAM_WRITES_DEPTH of the fragment program */
    uint32_t vertexBytes;    /* bytes the vertex program reads per vertex at binding 0 */
};

struct DrawRequest
{
    slg_mesh mesh;
    size_t numInstances;
    size_t shaderId;
    uint64_t primBase;
};

/* An operation that writes a framebuffer or what a later draw reads,
 * recorded from the last synchronisation point on so that it can be
 * replayed when a launch overflowed a buffer (settle). */
struct LogOp
{
    enum Kind { kLaunch, kNoalloc, kOpaque, kClearColor, kClearDepth, kBlit, kUbo } kind;
    std::vector<DrawRequest> reqs;     /* kLaunch */
    size_t fbo = 0;                    /* kLaunch, kNoalloc, clears */
    bool batch = false, multiple = false;
    slg_mesh mesh{};                   /* kNoalloc */
    size_t shader = 0;
    unsigned attachment = 0;           /* kClearColor */
    double value[4] = {0, 0, 0, 0};    /* clear colour, or depth in value[0] */
    size_t out = 0, in = 0;            /* kBlit */
    uint16_t rect[8] = {};
    size_t ubo = 0;                    /* kUbo: the block's bytes before and after */
    std::vector<uint8_t> before, after;
};

/* A registered program set (slg_register_programs): its kernels' entry
 * table and its programs. */
struct ProgramSet
{
    slg_pipeline_ops ops;
    std::vector<slg_program_info> programs;
};

/* Field widths of the packed formats 28..32 (RGB 332, RGB 565, RGBA 5551,
 * RGBA 4444, RGBA 1010102; softlight/include/softlight/SL_ColorCompressed.hpp),
 * from bit 0 up, and their texel bytes. */
const int kPackedWidths[5][4] = {{3, 3, 2, 0}, {5, 6, 5, 0}, {5, 5, 5, 1}, {4, 4, 4, 4}, {10, 10, 10, 2}};
const size_t kPackedBytes[5] = {1, 2, 2, 2, 4};

/* Bytes of a texel of SL_ColorDataType 0..32: components (type / 7 + 1) x
 * the size of u8, u16, u32, u64, half, float or double (type % 7), then the
 * packed formats (sl_bytes_per_color, softlight/src/SL_Color.cpp:12-56). */
size_t bytes_per_color(int type)
{
    if (type >= 28 && type <= 32) return kPackedBytes[type - 28];
    if (type < 0 || type > 27) return 0;
    static const size_t kind[7] = {1, 2, 4, 8, 2, 4, 8};
    return (size_t)(type / 7 + 1) * kind[type % 7];
}

bool core_color_type(int type)
{
    return type == SLG_COLOR_RGBA_8U || type == SLG_COLOR_RGBA_FLOAT || type == SLG_COLOR_R_FLOAT;
}

/* double -> unsigned as x86-64 code does it (cvttsd2si; 32-bit values from
 * the 64-bit form, 64-bit values from gcc's two-range sequence): the clear
 * colour conversion color_cast<T, double> of the reference build */
int64_t cvt_f64_i64(double v)
{
    return (v >= -9223372036854775808.0 && v < 9223372036854775808.0) ? (int64_t)v : INT64_MIN;
}

/* RGBA u32 clear values: the reference build converts four-lane u32
 * vectors with the vectorised SSE2 form (cvttpd2dq of x or of x - 2^31,
 * 0x80000000 out of int32 range); the conversion is undefined in C++ out of
 * range, identical within it. */
uint32_t d2u32_vec(double x)
{
    const bool big = x >= 2147483648.0;
    const double y = big ? x - 2147483648.0 : x;
    const uint32_t i = (y >= -2147483648.0 && y < 2147483648.0) ? (uint32_t)(int32_t)y : 0x80000000u;
    return big ? (i ^ 0x80000000u) : i;
}

uint64_t d2u_x86(double v, int kind)
{
    if (kind <= 1) return (uint64_t)(uint32_t)((v >= -2147483648.0 && v < 2147483648.0) ? (int32_t)v : INT32_MIN);
    if (kind == 2) return (uint64_t)cvt_f64_i64(v) & 0xFFFFFFFFull;
    if (!(v >= 9223372036854775808.0)) return (uint64_t)cvt_f64_i64(v);
    return (uint64_t)cvt_f64_i64(v - 9223372036854775808.0) ^ 0x8000000000000000ull;
}

size_t index_bytes(int type)
{
    switch (type)
    {
        case SLG_VERTEX_DATA_BYTE: return 1;
        case SLG_VERTEX_DATA_SHORT: return 2;
        case SLG_VERTEX_DATA_INT: return 4;
        default: return 0;
    }
}

bool valid_program(uint32_t p) { return p >= SLG_PROGRAM_LAMBERT_TEX && p <= SLG_PROGRAM_FRAG_COORD; }

/* SLG_PROGRAM_DISCARDS / SLG_PROGRAM_WRITES_DEPTH of a built-in fragment program. */
uint32_t builtin_program_flags(uint32_t p)
{
    if (p == SLG_PROGRAM_VCOLOR_TEX_CUTOUT) return SLG_PROGRAM_DISCARDS;
    if (p == SLG_PROGRAM_FRAG_COORD) return SLG_PROGRAM_DISCARDS | SLG_PROGRAM_WRITES_DEPTH;
    return 0;
}

constexpr size_t kDescRing = 4096;
constexpr uint64_t kMaxSlots = (1ull << 29) - 1; /* keys are slot << 3 | sub in 32 bits */
constexpr int kMaxLineExtent = 10922;            /* 3 * 10922 < 32768 */
constexpr uint32_t kAliasCap = 4096;             /* line address aliases per launch */
constexpr size_t kLogCap = 4096;                 /* recorded operations before a launch settles them */
constexpr uint64_t kMaxCacheEntries = 1ull << 25; /* vertex-cache entries per launch (80 B each) */
constexpr uint64_t kMinCachedSlots = 1ull << 16;  /* smaller launches run the programs per corner */
constexpr uint64_t kMaxBinChunks = 4096;          /* chunks of the key-order tile list fill */
constexpr uint64_t kMaxChunkCounts = 1ull << 24;  /* tiles x chunks it counts in (64 MB) */

} // namespace

/* A scene graph: SL_SceneGraph's node arrays (softlight/include/softlight/
 * SL_SceneGraph.hpp:224-300) on the host, the nodes' transforms and model
 * matrices and the draw list on the device. */
struct Scene
{
    std::vector<uint64_t> parents;              /* SLG_SCENE_ROOT or an earlier node */
    std::vector<uint32_t> depth;                /* nodes on the path from a root */
    std::vector<slg_transform> transforms;
    std::vector<uint8_t> dirty;
    std::vector<uint64_t> meshFirst, meshCount; /* per node, into nodeMeshes (count 0: empty node) */
    std::vector<uint64_t> nodeMeshes;
    std::vector<slg_mesh> meshes;
    std::vector<float> bounds;                  /* mMeshBounds: max xyzw, min xyzw per entry */
    std::vector<size_t> materials;              /* ambient texture per material */
    uint64_t modelsReady = 0;                   /* nodes whose device model matrix exists */
    DevBuffer dNodes, dList, dModel, dBounds, dEntries;

    /* the draw list: one entry per triangle-mode submesh of a mesh node */
    struct Entry
    {
        uint64_t node, mesh;
        size_t texture, ubo, shader;
    };
    std::vector<Entry> entries;
    std::vector<size_t> pool;                   /* ubo, shader pairs made for entries */
    bool listDirty = true;
    size_t listShader = SLG_INVALID_ID;
    size_t boundsUploaded = 0;
};

struct slg_context
{
    std::string err;
    cudaStream_t stream = nullptr;
    unsigned numThreads = 1;
    int tileW = 32, tileH = 32;
    int keyCap = 32768;   /* largest sortable tile list (128 KB of shared memory) */
    bool forceOrdered = false;
    int vsBlock = 128;          /* triangles per CTA of the vertex stage */
    bool batchGraphs = false;   /* replay slg_draw_batch launches as a CUDA graph */

    /* the last captured batch launch */
    struct GraphCache
    {
        cudaGraphExec_t exec = nullptr;
        std::vector<DrawDesc> descs;
        std::vector<uint64_t> starts;
        Frame frame;
        DevBuffer devDescs, devStarts;
    } graph;

    std::vector<Vbo> vbos;
    std::vector<Ibo> ibos;
    std::vector<Vao> vaos;
    std::vector<Texture> textures;
    std::vector<Fbo> fbos;
    std::vector<Ubo> ubos;
    std::vector<Shader> shaders;
    std::vector<Scene> scenes;
    std::vector<ProgramSet> programSets;   /* registered caller program sets */

    /* operations since the last synchronisation point (settle) */
    std::vector<LogOp> log;
    bool replaying = false;
    uint32_t aliasCap = kAliasCap;     /* line-alias events per launch */
    uint64_t ovfWant = 0;              /* clipped-triangle records the last overflow needed */
    bool sortFallback = false;         /* a tile list outgrew the shared-memory sort: keep sortScratch */
    DevBuffer sortScratch;

    /* uniform blocks assigned since the last launch, uploaded together
     * through a ring of pinned staging slots */
    std::vector<size_t> uboPending;
    struct UboStage
    {
        uint8_t* host = nullptr;
        size_t cap = 0;
        cudaEvent_t done = nullptr;
    } uboStage[4];
    int uboStageNext = 0;
    DevBuffer uboStageDev;

    /* resource tables visible to device programs */
    DevBuffer texTable, bufTable, vaoTable;
    bool tablesDirty = true;

    /* scratch */
    DevBuffer records, varyings, slotInfo, slotOvf, ovfCount, clipQueue, clipCount;
    DevBuffer aliasEvents, aliasCount; /* line address aliases (slg::AliasEvent) */
    DevBuffer cachePos, cacheVary;     /* post-transform vertex cache */
    DevBuffer recVerts;                /* per slot: cache entries of a cached record */
    uint64_t cacheCap = 0;
    DevBuffer tileCount, tileOffset, tileCursor, entries, status;
    DevBuffer blitBuf;      /* destination of slg_blit_read */
    DevBuffer rankOf, recOfRank, seqRec, seqKey, binBlocks;   /* blend order of a multi-mesh draw */
    uint64_t rankCap = 0;
    DevBuffer chunkCounts, itemKey;    /* tile lists in key order (Frame::chunkCounts) */
    DevBuffer tileOrder;               /* Frame::tileOrder */
    DevBuffer bestWords, ovfKey;       /* untiled order-free raster (Frame::bestWords) */
    bool forceTiled = false;           /* slg_set_raster_mode 2: order-free launches on tiles */
    bool forceUntiled = false;         /* slg_set_raster_mode 3: untiled where eligible */
    bool untiled = false;              /* the autotuner's pick for order-free triangle / point launches */
    bool sortKeysCapped = false;       /* slg_set_scratch_caps set a sort-key cap */
    uint64_t slotCap = 0, ovfCap = 0, tileCap = 0, entryCap = 0;

    /* draw descriptors: pinned host ring mirrored to a device ring */
    DrawDesc* hostDescs = nullptr;
    uint64_t* hostStarts = nullptr;
    DevBuffer devDescs, devStarts;
    size_t descHead = 0;

    int32_t* hostStatus = nullptr;
    cudaEvent_t stageEvents[5] = {};
    bool profileStages = false;

    int fail(int code, const std::string& msg) { err = msg; return code; }
    size_t fail_id(const std::string& msg) { err = msg; return SLG_INVALID_ID; }

    int cuda_fail(cudaError_t e, const char* what)
    {
        err = std::string(what) + ": " + cudaGetErrorString(e);
        return SLG_ERR_CUDA;
    }
};

namespace
{

int dev_alloc(slg_context* ctx, DevBuffer& b, size_t bytes, bool zero)
{
    if (b.bytes >= bytes && b.ptr)
    {
        if (zero)
        {
            cudaError_t e = cudaMemsetAsync(b.ptr, 0, bytes, ctx->stream);
            if (e != cudaSuccess) return ctx->cuda_fail(e, "cudaMemsetAsync");
        }
        return SLG_OK;
    }
    if (b.ptr)
    {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(b.ptr);
        b.ptr = nullptr;
        b.bytes = 0;
    }
    cudaError_t e = cudaMalloc(&b.ptr, bytes ? bytes : 16);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "cudaMalloc");
    b.bytes = bytes;
    if (zero)
    {
        e = cudaMemsetAsync(b.ptr, 0, bytes, ctx->stream);
        if (e != cudaSuccess) return ctx->cuda_fail(e, "cudaMemsetAsync");
    }
    return SLG_OK;
}

void dev_free(DevBuffer& b)
{
    if (b.ptr) cudaFree(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
}

void fill_vao_views(const slg_context* ctx, slg::VaoView* out)
{
    for (size_t i = 0; i < ctx->vaos.size(); ++i)
    {
        for (int k = 0; k < 8; ++k)
        {
            out[i].offset[k] = ctx->vaos[i].bindings[k].offset;
            out[i].stride[k] = ctx->vaos[i].bindings[k].stride;
        }
    }
}

/* The resource tables of a frame: textures, vertex buffers and vertex
 * arrays by id (device pointers to the uploaded tables). */
void set_tables(const slg_context* ctx, slg::Tables& t, const void* tex, const void* bufs, const void* vaos)
{
    t.textures = static_cast<const TexView*>(tex);
    t.buffers = static_cast<const uint8_t* const*>(bufs);
    t.vaos = static_cast<const slg::VaoView*>(vaos);
    t.numTextures = (uint32_t)ctx->textures.size();
    t.numBuffers = (uint32_t)ctx->vbos.size();
    t.numVaos = (uint32_t)ctx->vaos.size();
}

int upload_tables(slg_context* ctx)
{
    if (!ctx->tablesDirty) return SLG_OK;
    std::vector<TexView> tex(std::max<size_t>(1, ctx->textures.size()));
    for (size_t i = 0; i < ctx->textures.size(); ++i)
    {
        const Texture& t = ctx->textures[i];
        tex[i].texels = static_cast<const uint8_t*>(t.buf.ptr);
        tex[i].w = t.w;
        tex[i].h = t.h;
        tex[i].d = t.d;
        tex[i].type = t.type;
    }
    std::vector<const uint8_t*> bufs(std::max<size_t>(1, ctx->vbos.size()), nullptr);
    for (size_t i = 0; i < ctx->vbos.size(); ++i) bufs[i] = static_cast<const uint8_t*>(ctx->vbos[i].buf.ptr);
    std::vector<slg::VaoView> vaos(std::max<size_t>(1, ctx->vaos.size()));
    fill_vao_views(ctx, vaos.data());

    int r = dev_alloc(ctx, ctx->texTable, tex.size() * sizeof(TexView), false);
    if (r) return r;
    r = dev_alloc(ctx, ctx->bufTable, bufs.size() * sizeof(void*), false);
    if (r) return r;
    r = dev_alloc(ctx, ctx->vaoTable, vaos.size() * sizeof(slg::VaoView), false);
    if (r) return r;
    cudaStreamSynchronize(ctx->stream);
    cudaError_t e = cudaMemcpy(ctx->texTable.ptr, tex.data(), tex.size() * sizeof(TexView), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(ctx->bufTable.ptr, bufs.data(), bufs.size() * sizeof(void*), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(ctx->vaoTable.ptr, vaos.data(), vaos.size() * sizeof(slg::VaoView), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "table upload");
    ctx->tablesDirty = false;
    return SLG_OK;
}

int ensure_scratch(slg_context* ctx, uint64_t numSlots, uint64_t numTiles)
{
    int r;
    if (numSlots > ctx->slotCap || ctx->ovfWant > ctx->ovfCap)
    {
        const uint64_t cap = std::max<uint64_t>(std::max<uint64_t>(numSlots, ctx->slotCap), 1u << 16);
        const uint64_t ovf = std::max<uint64_t>(std::max<uint64_t>(std::min<uint64_t>(7 * cap, 1u << 22), cap / 2), ctx->ovfWant);
        const uint64_t recs = cap + ovf;
        if ((r = dev_alloc(ctx, ctx->records, recs * slg::kRecordVec4 * sizeof(float4), false))) return r;
        if ((r = dev_alloc(ctx, ctx->varyings, recs * slg::kVaryingVec4 * sizeof(float4), false))) return r;
        if ((r = dev_alloc(ctx, ctx->slotInfo, cap * sizeof(uint32_t), false))) return r;
        if ((r = dev_alloc(ctx, ctx->slotOvf, cap * sizeof(uint32_t), false))) return r;
        if ((r = dev_alloc(ctx, ctx->clipQueue, cap * sizeof(uint32_t), false))) return r;
        if ((r = dev_alloc(ctx, ctx->recVerts, cap * sizeof(uint4), false))) return r;
        ctx->slotCap = cap;
        ctx->ovfCap = ovf;
        const uint64_t wantEntries = std::max<uint64_t>(8 * cap, 32u << 20);
        if (wantEntries > ctx->entryCap)
        {
            if ((r = dev_alloc(ctx, ctx->entries, wantEntries * sizeof(uint32_t), false))) return r;
            ctx->entryCap = wantEntries;
        }
    }
    if (!ctx->ovfCount.ptr)
    {
        if ((r = dev_alloc(ctx, ctx->ovfCount, sizeof(uint32_t), true))) return r;
        if ((r = dev_alloc(ctx, ctx->clipCount, sizeof(uint32_t), true))) return r;
        if ((r = dev_alloc(ctx, ctx->aliasCount, sizeof(uint32_t), true))) return r;
    }
    if (ctx->aliasEvents.bytes < ctx->aliasCap * sizeof(slg::AliasEvent))
    {
        if ((r = dev_alloc(ctx, ctx->aliasEvents, ctx->aliasCap * sizeof(slg::AliasEvent), false))) return r;
    }
    if (ctx->sortFallback && ctx->sortScratch.bytes < 2 * ctx->entryCap * sizeof(uint32_t))
    {
        if ((r = dev_alloc(ctx, ctx->sortScratch, 2 * ctx->entryCap * sizeof(uint32_t), false))) return r;
    }
    if (numTiles > ctx->tileCap)
    {
        const uint64_t cap = numTiles;
        if ((r = dev_alloc(ctx, ctx->tileCount, cap * sizeof(uint32_t), true))) return r;
        if ((r = dev_alloc(ctx, ctx->tileOffset, (cap + 1) * sizeof(uint32_t), false))) return r;
        if ((r = dev_alloc(ctx, ctx->tileCursor, cap * sizeof(uint32_t), false))) return r;
        ctx->tileCap = cap;
    }
    return SLG_OK;
}

/* Waits for the queued work and completes it: replays launches that
 * overflowed a buffer and reports device-side conditions (defined below). */
int settle(slg_context* ctx);

/* Records an operation while launches may still have to be replayed. */
void log_op(slg_context* ctx, LogOp&& op) { ctx->log.push_back(std::move(op)); }

/* The clear value of a texel of `type` (SL_Context::clear_color_buffer ->
 * sl_match_color_for_type, softlight/src/SL_Color.cpp:137-192): per component
 * color_cast<T, double>, i.e. (T)(c * (double)max) for unsigned T, a half from
 * (float)c, (float)c or c. out: the texel's bytes (up to 32). */
int color_value(int type, const double rgba[4], uint32_t out[8])
{
    std::memset(out, 0, 8 * sizeof(uint32_t));
    const size_t bpt = bytes_per_color(type);
    if (!bpt) return -1;
    if (type >= 28)
    {
        /* rgba_cast<T, double> (SL_Color.cpp:180-184): (uint8_t or
         * uint16_t)(c * (double)max) per field, the field keeping its low bits */
        uint32_t bits = 0;
        int shift = 0;
        for (int j = 0; j < 4; ++j)
        {
            const int b = kPackedWidths[type - 28][j];
            if (!b) break;
            const uint32_t mask = (1u << b) - 1u;
            bits |= ((uint32_t)d2u_x86(rgba[j] * (double)mask, 0) & mask) << shift;
            shift += b;
        }
        out[0] = bits;
        return 0;
    }
    const int nc = type / 7 + 1, kind = type % 7;
    static const double kMax[4] = {255.0, 65535.0, 4294967295.0, 18446744073709551615.0};
    uint8_t* bytes = reinterpret_cast<uint8_t*>(out);
    for (int j = 0; j < nc; ++j)
    {
        uint8_t* c = bytes + (size_t)j * (bpt / nc);
        if (kind == 2 && nc == 4)
        {
            const uint32_t u = d2u32_vec(rgba[j] * kMax[kind]);
            std::memcpy(c, &u, 4);
        }
        else if (kind <= 3)
        {
            const uint64_t u = d2u_x86(rgba[j] * kMax[kind], kind);
            std::memcpy(c, &u, bpt / nc);   /* little-endian low bytes */
        }
        else if (kind == 4)
        {
            const uint16_t h = slg_float_to_half((float)rgba[j]);
            std::memcpy(c, &h, 2);
        }
        else if (kind == 5)
        {
            const float f = (float)rgba[j];
            std::memcpy(c, &f, 4);
        }
        else
        {
            std::memcpy(c, &rgba[j], 8);
        }
    }
    return 0;
}

/* Texels SL_ClearProcessor::clear_texture reaches (softlight/src/
 * SL_ClearProcessor.cpp:22-33): the w*h texels are dealt to the threads by
 * sl_calc_indexed_parition2<1> (softlight/include/softlight/SL_ShaderUtil.hpp:
 * 222-231), whose per-thread range count/threads + (1 - (count/threads) % 3)
 * is computed in size_t, so together the threads clear the prefix
 * [0, min(threads * range, count)); with one thread and count % 3 == 2 the
 * last texel keeps its value. */
uint64_t clear_extent(uint64_t count, unsigned threads)
{
    const uint64_t n = threads ? threads : 1u;
    const uint64_t total = count / n;
    const uint64_t range = total + (uint64_t(1) - total % 3u);
    const uint64_t reach = n * range;
    return (range != 0 && reach / range == n && reach < count) ? reach : count;
}

int clear_texture(slg_context* ctx, size_t texId, const double rgba[4])
{
    const Texture& t = ctx->textures[texId];
    uint32_t v[8];
    if (color_value(t.type, rgba, v)) return ctx->fail(SLG_ERR_INVALID_ARG, "unsupported clear format");
    const uint64_t texels = clear_extent((uint64_t)t.w * t.h, ctx->numThreads);
    cudaError_t e = slg::launch_clear(static_cast<uint8_t*>(t.buf.ptr), (size_t)texels, (int)t.bpt, v,
                                      static_cast<const int32_t*>(ctx->status.ptr), ctx->stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "clear launch");
    return SLG_OK;
}

/* The viewport and scissor matrix of SL_TriProcessor::execute with the
 * default SL_ViewportState (softlight/src/SL_TriProcessor.cpp:672-675,
 * softlight/src/SL_ViewportState.cpp:17-110); compiled with
 * -ffp-contract=off like the rest of the host code. */
void viewport_setup(float fboW, float fboH, float scissor[16], float viewport[4])
{
    auto mn = [](float a, float b) { return (b < a) ? b : a; };
    auto mx = [](float a, float b) { return (a < b) ? b : a; };
    const float invW = 1.f / fboW, invH = 1.f / fboH;
    float sx = 0.f * invW, sy = 0.f * invH;
    float sw = 65535.f * invW, sh = 65535.f * invH;
    if (sx < 0.f) { sw += sx; sx = 0.f; }
    if (sy < 0.f) { sh += sy; sy = 0.f; }
    sw = mn(1.f - sx, sw);
    sh = mn(1.f - sy, sh);
    const float nm00 = 1.f / sw, nm11 = 1.f / sh;
    const float nm30 = nm00 - 1.f, nm31 = nm11 - 1.f;
    const float m30 = sx * (-2.f * nm00) + nm30;
    const float m31 = sy * (-2.f * nm11) + nm31;
    const float m[16] = {nm00, 0, 0, 0, 0, nm11, 0, 0, 0, 0, 1, 0, m30, m31, 0, 1};
    std::memcpy(scissor, m, sizeof(m));
    const float vx = mn(mx(0.f + 0.f, 0.f), fboW);
    const float vy = mn(mx(0.f + 0.f, 0.f), fboH);
    viewport[0] = vx;
    viewport[1] = vy;
    viewport[2] = mn(mn(65535.f, (0.f + 65535.f) - vx), fboW - vx);
    viewport[3] = mn(mn(65535.f, (0.f + 65535.f) - vy), fboH - vy);
}

/* Bytes a program reads per vertex at binding 0 (include/slg_programs.h). */
size_t program_vertex_bytes(uint32_t program)
{
    switch (program)
    {
        case SLG_PROGRAM_LAMBERT_TEX:
        case SLG_PROGRAM_BLINN_PHONG_INST: return 32;
        case SLG_PROGRAM_VCOLOR_TEX_ALPHA:
        case SLG_PROGRAM_VCOLOR_TEXF:
        case SLG_PROGRAM_GBUFFER:
        case SLG_PROGRAM_VCOLOR_TEX_CUTOUT:
        case SLG_PROGRAM_FRAG_COORD:       return 36;
        default:                           return 12;
    }
}

/* Bytes of one component of SL_DataType (softlight/include/softlight/SL_Geometry.hpp:30). */
uint64_t vertex_type_bytes(int type)
{
    switch (type)
    {
        case SLG_VERTEX_DATA_BYTE:   return 1;
        case SLG_VERTEX_DATA_SHORT:  return 2;
        case SLG_VERTEX_DATA_INT:    return 4;
        case SLG_VERTEX_DATA_LONG:   return 8;
        case SLG_VERTEX_DATA_FLOAT:  return 4;
        case SLG_VERTEX_DATA_DOUBLE: return 8;
        default:                     return 0;
    }
}

bool texture_ok(const slg_context* ctx, uint32_t id, int type)
{
    return id < ctx->textures.size() && ctx->textures[id].buf.ptr && ctx->textures[id].type == type;
}

/* Vertices per primitive of the supported render modes (0 = unsupported). */
uint64_t render_mode_vertices(int mode)
{
    switch (mode)
    {
        case SLG_RENDER_MODE_POINTS:
        case SLG_RENDER_MODE_INDEXED_POINTS:    return 1;
        case SLG_RENDER_MODE_LINES:
        case SLG_RENDER_MODE_INDEXED_LINES:     return 2;
        case SLG_RENDER_MODE_TRIANGLES:
        case SLG_RENDER_MODE_INDEXED_TRIANGLES:
        case SLG_RENDER_MODE_TRI_WIRE:
        case SLG_RENDER_MODE_INDEXED_TRI_WIRE:  return 3;
        default:                                return 0;
    }
}

bool render_mode_indexed(int mode)
{
    return mode == SLG_RENDER_MODE_INDEXED_POINTS || mode == SLG_RENDER_MODE_INDEXED_LINES || mode == SLG_RENDER_MODE_INDEXED_TRIANGLES ||
           mode == SLG_RENDER_MODE_INDEXED_TRI_WIRE;
}

uint8_t render_mode_prim(int mode)
{
    switch (render_mode_vertices(mode))
    {
        case 1:  return slg::kPrimPoint;
        case 2:  return slg::kPrimLine;
        default: return (mode == SLG_RENDER_MODE_TRI_WIRE || mode == SLG_RENDER_MODE_INDEXED_TRI_WIRE) ? slg::kPrimWire : slg::kPrimTriangle;
    }
}

/* Host-side bounds checks of everything a draw's kernels will read: the
 * vertex range, the index range and the resource ids stored in the uniform
 * block. The reference performs none (SL_Context::draw, SL_Context.cpp:714);
 * here an invalid draw is rejected before any kernel is launched. */
int validate_draw(slg_context* ctx, const Shader& sh, const Vao& vao, const slg_mesh& m, size_t numInstances, size_t numElements)
{
    const Vbo& vbo = ctx->vbos[vao.vbo];
    const Binding& b0 = vao.bindings[0];
    if (b0.offset < 0 || b0.stride <= 0) return ctx->fail(SLG_ERR_INVALID_ARG, "binding 0 needs offset >= 0 and stride > 0");
    /* the reference reads whole primitives: a partial last line or triangle
     * reads the elements after elementEnd */
    const uint64_t perPrim = render_mode_vertices(m.mode);
    const uint64_t lastElement = m.elementBegin + perPrim * ((numElements + perPrim - 1) / perPrim) - 1;
    uint64_t maxVertex;
    if (render_mode_indexed(m.mode))
    {
        const Ibo& ibo = ctx->ibos[vao.ibo];
        if (lastElement >= ibo.count) return ctx->fail(SLG_ERR_INVALID_ARG, "element range exceeds the index buffer");
        maxVertex = ibo.maxIndex;
    }
    else
    {
        maxVertex = lastElement;
    }
    const uint64_t need = (uint64_t)b0.offset + (uint64_t)b0.stride * maxVertex + sh.vertexBytes;
    if (need > vbo.size + 64) return ctx->fail(SLG_ERR_INVALID_ARG, "vertex range exceeds the vertex buffer");

    /* a caller's programs may read any configured binding (SL_VertexArray::
     * offset(bindId, vertId)); each must stay inside the buffer for every
     * vertex the draw reaches. Uniform blocks are theirs to interpret. */
    if (sh.programSet != 0)
    {
        for (int k = 1; k < 8; ++k)
        {
            const Binding& b = vao.bindings[k];
            if (b.stride == 0 && b.comps == 0) continue;
            const uint64_t elem = (uint64_t)b.comps * vertex_type_bytes(b.type);
            if (b.offset < 0 || b.stride < 0 || (uint64_t)b.offset + (uint64_t)b.stride * maxVertex + elem > vbo.size + 64)
                return ctx->fail(SLG_ERR_INVALID_ARG, "vertex binding " + std::to_string(k) + " reaches past the vertex buffer");
        }
        return SLG_OK;
    }
    if (sh.ubo == SLG_INVALID_ID) return ctx->fail(SLG_ERR_INVALID_ARG, "built-in programs need a uniform block");
    const uint8_t* u = ctx->ubos[sh.ubo].shadow;
    uint32_t tex = 0, buf = 0;
    switch (sh.fsProgram)
    {
        case SLG_PROGRAM_LAMBERT_TEX:
            std::memcpy(&tex, u + offsetof(slg_lambert_uniforms, textureId), 4);
            if (!texture_ok(ctx, tex, SLG_COLOR_RGBA_8U)) return ctx->fail(SLG_ERR_INVALID_ARG, "uniform textureId is not an RGBA8 texture");
            break;
        case SLG_PROGRAM_BLINN_PHONG_INST:
            std::memcpy(&tex, u + offsetof(slg_blinn_uniforms, textureId), 4);
            if (!texture_ok(ctx, tex, SLG_COLOR_RGBA_8U)) return ctx->fail(SLG_ERR_INVALID_ARG, "uniform textureId is not an RGBA8 texture");
            break;
        case SLG_PROGRAM_VCOLOR_TEX_ALPHA:
        case SLG_PROGRAM_GBUFFER:
        case SLG_PROGRAM_VCOLOR_TEX_CUTOUT:
            std::memcpy(&tex, u + offsetof(slg_vcolor_uniforms, textureId), 4);
            if (!texture_ok(ctx, tex, SLG_COLOR_RGBA_8U)) return ctx->fail(SLG_ERR_INVALID_ARG, "uniform textureId is not an RGBA8 texture");
            break;
        case SLG_PROGRAM_VCOLOR_TEXF:
            std::memcpy(&tex, u + offsetof(slg_vcolor_uniforms, textureId), 4);
            if (!texture_ok(ctx, tex, SLG_COLOR_RGBA_FLOAT)) return ctx->fail(SLG_ERR_INVALID_ARG, "uniform textureId is not an RGBA float texture");
            break;
        default:
            break;
    }
    if (sh.vsProgram == SLG_PROGRAM_BLINN_PHONG_INST)
    {
        std::memcpy(&buf, u + offsetof(slg_blinn_uniforms, instanceBufferId), 4);
        if (buf >= ctx->vbos.size() || !ctx->vbos[buf].buf.ptr || ctx->vbos[buf].size < 64 * (uint64_t)numInstances)
            return ctx->fail(SLG_ERR_INVALID_ARG, "uniform instanceBufferId does not hold one matrix per instance");
    }
    if (sh.vsProgram == SLG_PROGRAM_BLINN_PHONG_INST && sh.fsProgram != SLG_PROGRAM_BLINN_PHONG_INST)
        return ctx->fail(SLG_ERR_INVALID_ARG, "program pair not supported");
    return SLG_OK;
}

/* Colour attachments of the framebuffer into the frame (SL_Framebuffer::
 * build_output_functions, softlight/src/SL_Framebuffer.cpp:1207-1231). A
 * program writing more outputs than the framebuffer has attachments would
 * call unset output functions in the reference; here it is rejected. */
int bind_attachments(slg_context* ctx, const Fbo& fbo, const Texture& depthTex, const DrawDesc* descs, size_t n, Frame& f)
{
    f.numColors = 0;
    for (unsigned k = 0; k < fbo.numColors && k < 4; ++k)
    {
        if (fbo.colors[k] == SLG_INVALID_ID || fbo.colors[k] >= ctx->textures.size()) break;
        const Texture& t = ctx->textures[fbo.colors[k]];
        if (!t.buf.ptr) break;
        if (t.w != depthTex.w || t.h != depthTex.h) return ctx->fail(SLG_ERR_INVALID_ARG, "colour and depth attachments differ in size");
        if (!bytes_per_color(t.type)) return ctx->fail(SLG_ERR_INVALID_ARG, "unsupported colour attachment format");
        f.colors[k] = static_cast<uint8_t*>(t.buf.ptr);
        f.colorTypes[k] = t.type;
        f.numColors = (int32_t)k + 1;
    }
    /* attachment 0 of another format is written like attachments 1..3 */
    f.generic0 = (f.numColors > 0 && !core_color_type(f.colorTypes[0])) ? 1 : 0;
    if (f.generic0) f.hasMrt = 1;
    for (size_t i = 0; i < n; ++i)
    {
        if (f.numColors > 0 && descs[i].numOutputs > f.numColors)
            return ctx->fail(SLG_ERR_INVALID_ARG, "the fragment program writes more outputs than the framebuffer has colour attachments");
        if (f.numColors > 1 && descs[i].numOutputs > 1) f.hasMrt = 1;
    }
    return SLG_OK;
}

/* The framebuffer's visibility map (slg_fbo_enable_visibility) into the
 * frame, after the checks that keep it exact: the order-free raster writes
 * it, so the launch must be order-free, of filled triangles or points, into
 * an R_FLOAT depth attachment. */
int bind_visibility(slg_context* ctx, const Fbo& fbo, Frame& f)
{
    if (!fbo.visEnabled) return SLG_OK;
    if (f.depthType != SLG_COLOR_R_FLOAT)
        return ctx->fail(SLG_ERR_INVALID_ARG, "a framebuffer with a visibility map needs an R_FLOAT depth attachment");
    if (f.hasLines || f.hasWire)
        return ctx->fail(SLG_ERR_INVALID_ARG, "a framebuffer with a visibility map takes filled triangle and point draws only");
    if (!f.orderFree)
        return ctx->fail(SLG_ERR_INVALID_ARG, "a framebuffer with a visibility map takes opaque draws only (no blending, one depth rule)");
    if (fbo.vis.bytes < (size_t)f.width * f.height * sizeof(uint32_t))
        return ctx->fail(SLG_ERR_INVALID_ARG, "visibility map is smaller than the framebuffer (enable it again after resizing)");
    f.ids = static_cast<uint32_t*>(fbo.vis.ptr);
    return SLG_OK;
}

/* Uploads the queued uniform blocks: with allocation allowed, one copy of a
 * packed staging slot and one scatter kernel; otherwise (the no-allocation
 * draw) one copy per block from its host copy. */
int flush_ubos(slg_context* ctx, bool allowAlloc)
{
    if (ctx->uboPending.empty()) return SLG_OK;
    cudaError_t e = cudaSuccess;
    if (!allowAlloc)
    {
        for (size_t id : ctx->uboPending)
        {
            Ubo& u = ctx->ubos[id];
            if (e == cudaSuccess) e = cudaMemcpyAsync(u.buf.ptr, u.shadow, u.pending, cudaMemcpyHostToDevice, ctx->stream);
            u.pending = 0;
        }
        ctx->uboPending.clear();
        return (e == cudaSuccess) ? SLG_OK : ctx->cuda_fail(e, "uniform block upload");
    }
    const size_t n = ctx->uboPending.size();
    const size_t header = (n * sizeof(slg::UboCopy) + 15) & ~(size_t)15;
    size_t bytes = header;
    for (size_t id : ctx->uboPending) bytes += (ctx->ubos[id].pending + 15) & ~15u;
    slg_context::UboStage& st = ctx->uboStage[ctx->uboStageNext];
    ctx->uboStageNext = (ctx->uboStageNext + 1) % 4;
    if (st.done) cudaEventSynchronize(st.done);   /* the slot's last copy has read it */
    else if ((e = cudaEventCreateWithFlags(&st.done, cudaEventDisableTiming)) != cudaSuccess) return ctx->cuda_fail(e, "ubo staging event");
    if (st.cap < bytes)
    {
        if (st.host) cudaFreeHost(st.host);
        st.host = nullptr;
        st.cap = 0;
        const size_t cap = std::max<size_t>(bytes, 64 << 10);
        if ((e = cudaMallocHost(&st.host, cap)) != cudaSuccess) return ctx->cuda_fail(e, "ubo staging");
        st.cap = cap;
    }
    int r = dev_alloc(ctx, ctx->uboStageDev, std::max<size_t>(bytes, 64 << 10), false);
    if (r) return r;
    slg::UboCopy* rec = reinterpret_cast<slg::UboCopy*>(st.host);
    size_t off = header;
    for (size_t k = 0; k < n; ++k)
    {
        Ubo& u = ctx->ubos[ctx->uboPending[k]];
        const uint32_t words = (u.pending + 3) / 4;   /* whole words of the 1024-byte block */
        rec[k].dst = static_cast<uint8_t*>(u.buf.ptr);
        rec[k].src = (uint32_t)off;
        rec[k].words = words;
        std::memcpy(st.host + off, u.shadow, (size_t)words * 4);
        off += ((size_t)words * 4 + 15) & ~(size_t)15;
        u.pending = 0;
    }
    ctx->uboPending.clear();
    e = cudaMemcpyAsync(ctx->uboStageDev.ptr, st.host, bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaEventRecord(st.done, ctx->stream);
    if (e == cudaSuccess) e = slg::launch_ubo_scatter(static_cast<const uint8_t*>(ctx->uboStageDev.ptr), (uint32_t)n, ctx->stream);
    return (e == cudaSuccess) ? SLG_OK : ctx->cuda_fail(e, "uniform block upload");
}

int build_desc(slg_context* ctx, const DrawRequest& req, uint64_t slotBase, DrawDesc& d, uint64_t& numSlots)
{
    const slg_mesh& m = req.mesh;
    if (req.shaderId >= ctx->shaders.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid shader id");
    if (m.vaoId >= ctx->vaos.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid vao id");
    const uint64_t perPrim = render_mode_vertices(m.mode);
    if (perPrim == 0)
        return ctx->fail(SLG_ERR_INVALID_ARG, "unsupported render mode");
    const Shader& sh = ctx->shaders[req.shaderId];
    const Vao& vao = ctx->vaos[m.vaoId];
    if (vao.vbo == SLG_INVALID_ID || !ctx->vbos[vao.vbo].buf.ptr) return ctx->fail(SLG_ERR_INVALID_ARG, "vao has no vertex buffer");
    const bool indexed = render_mode_indexed(m.mode);
    if (indexed && (vao.ibo == SLG_INVALID_ID || !ctx->ibos[vao.ibo].buf.ptr))
        return ctx->fail(SLG_ERR_INVALID_ARG, "indexed draw without index buffer");

    const size_t numElements = (m.elementEnd > m.elementBegin) ? (m.elementEnd - m.elementBegin) : 0;
    if (numElements && req.numInstances)
    {
        int r = validate_draw(ctx, sh, vao, m, req.numInstances, numElements);
        if (r) return r;
    }

    std::memset(&d, 0, sizeof(d));
    d.vbo = static_cast<const uint8_t*>(ctx->vbos[vao.vbo].buf.ptr);
    d.ibo = indexed ? static_cast<const uint8_t*>(ctx->ibos[vao.ibo].buf.ptr) : nullptr;
    d.ubo = (sh.ubo != SLG_INVALID_ID) ? static_cast<const uint8_t*>(ctx->ubos[sh.ubo].buf.ptr) : nullptr;
    d.b0Offset = vao.bindings[0].offset;
    d.b0Stride = vao.bindings[0].stride;
    d.elementBegin = m.elementBegin;
    d.numElements = (m.elementEnd > m.elementBegin) ? (m.elementEnd - m.elementBegin) : 0;
    d.numTris = (d.numElements + perPrim - 1) / perPrim;
    d.prim = render_mode_prim(m.mode);
    d.numInstances = std::max<size_t>(1, req.numInstances);
    d.slotBase = slotBase;
    d.primBase = req.primBase;
    /* post-transform vertex cache for indexed triangles whose vertices are
     * shared by enough corners: the program then runs once per vertex and
     * instance instead of once per corner (run_launch assigns the entries) */
    d.cacheBase = 0;
    d.cacheVerts = 0;
    if (indexed && (d.prim == slg::kPrimTriangle || d.prim == slg::kPrimWire))
    {
        const uint64_t verts = (uint64_t)ctx->ibos[vao.ibo].maxIndex + 1;
        if (2 * d.numTris >= verts) d.cacheVerts = verts;
    }
    d.indexType = indexed ? ctx->ibos[vao.ibo].type : -1;
    d.vsProgram = sh.vsProgram;
    d.fsProgram = sh.fsProgram;
    d.vaoId = (uint32_t)m.vaoId;
    d.cull = sh.cull;
    d.numVaryings = sh.numVaryings;
    d.depthTest = sh.depthTest;
    d.depthMask = sh.depthMask;
    d.blend = sh.blend;
    d.numOutputs = sh.numOutputs;
    numSlots = d.numTris * d.numInstances;
    if (req.numInstances == 0) numSlots = 0;
    return SLG_OK;
}

/* The kernels of program set `set` (0: built-in). */
const slg_pipeline_ops& pipeline_ops(const slg_context* ctx, uint32_t set)
{
    return set == 0 ? slg::builtin_pipeline() : ctx->programSets[set - 1].ops;
}

/* Replays the cached CUDA graph of a batch launch when the descriptors and
 * the launch parameters are unchanged (uniform-block contents may change:
 * they are read from device memory and were validated again on the host),
 * otherwise captures the pipeline of this launch into a new graph. */
int launch_batch_graph(slg_context* ctx, const Frame& frame, const DrawDesc* descs, const uint64_t* starts, size_t n,
                       const slg_pipeline_ops& ops)
{
    slg_context::GraphCache& g = ctx->graph;
    int r;
    if ((r = dev_alloc(ctx, g.devDescs, n * sizeof(DrawDesc), false))) return r;
    if ((r = dev_alloc(ctx, g.devStarts, (n + 1) * sizeof(uint64_t), false))) return r;
    Frame f = frame;
    f.draws = static_cast<const DrawDesc*>(g.devDescs.ptr);
    f.drawSlotStart = static_cast<const uint64_t*>(g.devStarts.ptr);

    const bool same = g.exec && g.descs.size() == n &&
                      std::memcmp(g.descs.data(), descs, n * sizeof(DrawDesc)) == 0 &&
                      std::memcmp(g.starts.data(), starts, (n + 1) * sizeof(uint64_t)) == 0 &&
                      std::memcmp(&g.frame, &f, sizeof(Frame)) == 0;
    cudaError_t e = cudaSuccess;
    if (!same)
    {
        if (g.exec)
        {
            cudaStreamSynchronize(ctx->stream);
            cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
        }
        e = cudaMemcpyAsync(g.devDescs.ptr, descs, n * sizeof(DrawDesc), cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(g.devStarts.ptr, starts, (n + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return ctx->cuda_fail(e, "graph descriptor upload");

        cudaGraph_t graph = nullptr;
        e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return ctx->cuda_fail(e, "cudaStreamBeginCapture");
        const cudaError_t le = slg::launch_pipeline(f, ops, ctx->keyCap, ctx->stream, nullptr);
        e = cudaStreamEndCapture(ctx->stream, &graph);
        if (le != cudaSuccess) e = le;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&g.exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (e != cudaSuccess)
        {
            g.exec = nullptr;
            return ctx->cuda_fail(e, "batch graph capture");
        }
        g.descs.assign(descs, descs + n);
        g.starts.assign(starts, starts + n + 1);
        g.frame = f;
    }
    e = cudaGraphLaunch(g.exec, ctx->stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "cudaGraphLaunch");
    return SLG_OK;
}

/* One launch of the pipeline over a sequence of draws that share a
 * framebuffer. The result equals issuing the draws one after another. */
/* Work enqueued between the descriptor upload and the pipeline (the scene
 * graph's draw-list kernel writes uniform blocks and hidden flags there). */
struct LaunchHook
{
    cudaError_t (*fn)(void* user, DrawDesc* devDescs, cudaStream_t s);
    void* user;
};

int run_launch(slg_context* ctx, const std::vector<DrawRequest>& reqs, size_t fboId, bool batch = false,
               const LaunchHook* hook = nullptr, bool multiple = false)
{
    if (fboId >= ctx->fbos.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid fbo id");
    const Fbo& fbo = ctx->fbos[fboId];
    if (fbo.depth == SLG_INVALID_ID) return ctx->fail(SLG_ERR_INVALID_ARG, "framebuffer has no depth attachment");
    if (reqs.empty()) return SLG_OK;
    if (ctx->log.size() >= kLogCap && !ctx->replaying)
    {
        /* a caller that never synchronises: complete the recorded work */
        const int settled = settle(ctx);
        if (settled) return settled;
    }
    if (reqs.size() + 1 > kDescRing) return ctx->fail(SLG_ERR_INVALID_ARG, "too many draws in one batch");

    /* a launch runs the kernels of one program set: draws whose shaders come
     * from different sets go out as consecutive launches, which gives the
     * same result as one */
    uint32_t programSet = 0;
    for (size_t i = 0; i < reqs.size(); ++i)
    {
        if (reqs[i].shaderId >= ctx->shaders.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid shader id");
        const uint32_t set = ctx->shaders[reqs[i].shaderId].programSet;
        if (i == 0)
        {
            programSet = set;
        }
        else if (set != programSet)
        {
            if (hook) return ctx->fail(SLG_ERR_INVALID_ARG, "a draw list mixes program sets");
            const std::vector<DrawRequest> head(reqs.begin(), reqs.begin() + i), tail(reqs.begin() + i, reqs.end());
            int r = run_launch(ctx, head, fboId, false, nullptr);
            return r ? r : run_launch(ctx, tail, fboId, false, nullptr);
        }
    }
    const slg_pipeline_ops& ops = pipeline_ops(ctx, programSet);

    int r = upload_tables(ctx);
    if (r) return r;
    if ((r = flush_ubos(ctx, true))) return r;

    const Texture& depthTex = ctx->textures[fbo.depth];
    const Texture* colorTex = (fbo.numColors > 0 && fbo.colors[0] != SLG_INVALID_ID) ? &ctx->textures[fbo.colors[0]] : nullptr;
    if (colorTex && (colorTex->w != depthTex.w || colorTex->h != depthTex.h))
        return ctx->fail(SLG_ERR_INVALID_ARG, "colour and depth attachments differ in size");

    /* descriptors into the ring */
    const size_t n = reqs.size();
    if (ctx->descHead + n + 1 > kDescRing)
    {
        cudaStreamSynchronize(ctx->stream);
        ctx->descHead = 0;
    }
    DrawDesc* descs = ctx->hostDescs + ctx->descHead;
    uint64_t* starts = ctx->hostStarts + ctx->descHead;
    uint64_t numSlots = 0;
    for (size_t i = 0; i < n; ++i)
    {
        uint64_t s = 0;
        if ((r = build_desc(ctx, reqs[i], numSlots, descs[i], s))) return r;
        starts[i] = numSlots;
        numSlots += s;
    }
    starts[n] = numSlots;
    if (numSlots > kMaxSlots) return ctx->fail(SLG_ERR_INVALID_ARG, "too many triangles in one launch (max 2^29-1)");
    /* the vertex cache costs a launch: used from kMinCachedSlots triangles on */
    uint64_t cacheEntries = 0;
    for (size_t i = 0; i < n; ++i)
    {
        descs[i].cacheBase = cacheEntries;
        const uint64_t add = descs[i].cacheVerts * descs[i].numInstances;
        if (descs[i].cacheVerts && numSlots >= kMinCachedSlots && starts[i + 1] > starts[i] && cacheEntries + add <= kMaxCacheEntries)
            cacheEntries += add;
        else descs[i].cacheVerts = 0;
    }
    if (cacheEntries > ctx->cacheCap)
    {
        if ((r = dev_alloc(ctx, ctx->cachePos, cacheEntries * sizeof(float4), false))) return r;
        if ((r = dev_alloc(ctx, ctx->cacheVary, cacheEntries * slg::kMaxVaryings * sizeof(float4), false))) return r;
        ctx->cacheCap = cacheEntries;
    }

    Frame f;
    std::memset(&f, 0, sizeof(f));
    for (size_t i = 0; i < n; ++i)
    {
        if (descs[i].prim == slg::kPrimLine) f.hasLines = 1;
        if (descs[i].prim == slg::kPrimWire) f.hasWire = 1;
    }
    f.width = depthTex.w;
    f.height = depthTex.h;
    if ((r = bind_attachments(ctx, fbo, depthTex, descs, n, f))) return r;
    /* launches with line or wireframe draws or several render targets use
     * the raster that carries those, compiled for one tile size */
    const bool edges = f.hasLines || f.hasWire || f.hasMrt;
    f.tileW = edges ? slg::kLineTile : ctx->tileW;
    f.tileH = edges ? slg::kLineTile : ctx->tileH;
    f.tilesX = (f.width + f.tileW - 1) / f.tileW;
    f.tilesY = (f.height + f.tileH - 1) / f.tileH;
    const uint64_t numTiles = (uint64_t)f.tilesX * f.tilesY;
    if ((r = ensure_scratch(ctx, numSlots, numTiles))) return r;

    DrawDesc* devDescs = static_cast<DrawDesc*>(ctx->devDescs.ptr) + ctx->descHead;
    uint64_t* devStarts = static_cast<uint64_t*>(ctx->devStarts.ptr) + ctx->descHead;
    cudaError_t e = cudaSuccess;

    f.color = colorTex ? static_cast<uint8_t*>(colorTex->buf.ptr) : nullptr;
    f.colorType = colorTex ? colorTex->type : SLG_COLOR_RGBA_8U;
    if (f.generic0) f.color = nullptr;
    f.depth = static_cast<float*>(depthTex.buf.ptr);
    f.depthType = depthTex.type;
    viewport_setup((float)f.width, (float)f.height, f.scissor, f.viewport);
    f.records = static_cast<float4*>(ctx->records.ptr);
    f.cachePos = static_cast<float4*>(ctx->cachePos.ptr);
    f.cacheVary = static_cast<float4*>(ctx->cacheVary.ptr);
    f.cacheEntries = cacheEntries;
    f.recVerts = static_cast<uint4*>(ctx->recVerts.ptr);
    f.allCached = cacheEntries > 0 ? 1 : 0;
    for (size_t i = 0; i < n; ++i)
    {
        if (starts[i + 1] > starts[i] && (descs[i].cacheVerts == 0 || descs[i].prim != slg::kPrimTriangle)) f.allCached = 0;
    }
    f.varyings = static_cast<float4*>(ctx->varyings.ptr);
    f.slotInfo = static_cast<uint32_t*>(ctx->slotInfo.ptr);
    f.slotOvf = static_cast<uint32_t*>(ctx->slotOvf.ptr);
    f.ovfCount = static_cast<uint32_t*>(ctx->ovfCount.ptr);
    f.clipQueue = static_cast<uint32_t*>(ctx->clipQueue.ptr);
    f.clipCount = static_cast<uint32_t*>(ctx->clipCount.ptr);
    f.ovfCap = (uint32_t)std::min<uint64_t>(ctx->ovfCap, 0xFFFFFFFFu);
    f.numSlots = numSlots;
    f.tileCount = static_cast<uint32_t*>(ctx->tileCount.ptr);
    f.tileOffset = static_cast<uint32_t*>(ctx->tileOffset.ptr);
    f.tileCursor = static_cast<uint32_t*>(ctx->tileCursor.ptr);
    f.entries = static_cast<uint32_t*>(ctx->entries.ptr);
    f.entryCap = (uint32_t)std::min<uint64_t>(ctx->entryCap, 0xFFFFFFFFu);
    f.status = static_cast<int32_t*>(ctx->status.ptr);
    f.draws = devDescs;
    f.drawSlotStart = devStarts;
    f.numDraws = (int32_t)n;
    /* order-free raster when nothing blends and every draw uses the same
     * order-independent depth rule (NOT_EQUAL depends on order) */
    f.orderFree = 1;
    f.freeDepthFunc = descs[0].depthTest;
    f.freeDepthMask = descs[0].depthMask;
    for (size_t i = 0; i < n; ++i)
    {
        /* a discarded fragment leaves an earlier one's colour and a written
         * coord.depth changes later tests: both need the order */
        const uint32_t flags = ctx->shaders[reqs[i].shaderId].fsFlags;
        if (descs[i].blend != SLG_BLEND_OFF || descs[i].depthTest == SLG_DEPTH_TEST_NOT_EQUAL ||
            descs[i].depthTest != f.freeDepthFunc || descs[i].depthMask != f.freeDepthMask || ctx->forceOrdered ||
            (flags & (SLG_PROGRAM_DISCARDS | SLG_PROGRAM_WRITES_DEPTH)))
        {
            f.orderFree = 0;
        }
    }
    /* a half depth is rounded on every write and re-read by later
     * fragments: the outcome depends on the order, not the set */
    if (f.depthType == SLG_COLOR_R_HALF) f.orderFree = 0;
    /* the ordered raster's depth bound holds while every pixel's depth moves
     * one way: one family of depth test, no program writing depth */
    f.depthBound = 0;
    {
        const auto family = [](uint8_t t) {
            return (t == SLG_DEPTH_TEST_LESS_THAN || t == SLG_DEPTH_TEST_LESS_EQUAL) ? 1
                 : (t == SLG_DEPTH_TEST_GREATER_THAN || t == SLG_DEPTH_TEST_GREATER_EQUAL) ? 2 : 0;
        };
        int32_t fam = family(descs[0].depthTest);
        for (size_t i = 0; i < n && fam; ++i)
        {
            if (family(descs[i].depthTest) != fam || (ctx->shaders[reqs[i].shaderId].fsFlags & SLG_PROGRAM_WRITES_DEPTH)) fam = 0;
        }
        f.depthBound = fam;
    }
    for (size_t i = 0; i < n; ++i)
    {
        /* the reference's Bresenham error term is int16: it stays exact while
         * 3 * dx fits, dx <= max(W, H) */
        if (descs[i].prim == slg::kPrimLine && std::max(f.width, f.height) > kMaxLineExtent)
            return ctx->fail(SLG_ERR_INVALID_ARG, "line draws need a framebuffer of at most 10922 x 10922");
    }
    if (f.hasLines)
    {
        f.aliasEvents = static_cast<slg::AliasEvent*>(ctx->aliasEvents.ptr);
        f.aliasCount = static_cast<uint32_t*>(ctx->aliasCount.ptr);
        f.aliasCap = ctx->aliasCap;
    }
    f.sortScratch = ctx->sortFallback ? static_cast<uint32_t*>(ctx->sortScratch.ptr) : nullptr;
    set_tables(ctx, f.tables, ctx->texTable.ptr, ctx->bufTable.ptr, ctx->vaoTable.ptr);

    f.vsBlock = ctx->vsBlock;

    if ((r = bind_visibility(ctx, fbo, f))) return r;

    /* one draw_multiple call over several meshes with blending: the
     * reference's flush groups interleave the meshes by primIndex */
    bool flushSort = multiple && n >= 2 && descs[0].blend != SLG_BLEND_OFF;
    for (size_t i = 0; i < n; ++i)
    {
        if (descs[i].prim != slg::kPrimTriangle && descs[i].prim != slg::kPrimWire) flushSort = false;
    }
    if (flushSort && numSlots > 0)
    {
        const uint64_t recs = ctx->slotCap + ctx->ovfCap;
        const uint64_t blocks = (numSlots + 1023) / 1024;
        if (recs > ctx->rankCap)
        {
            if ((r = dev_alloc(ctx, ctx->rankOf, recs * sizeof(uint32_t), false))) return r;
            if ((r = dev_alloc(ctx, ctx->recOfRank, recs * sizeof(uint32_t), false))) return r;
            if ((r = dev_alloc(ctx, ctx->seqRec, recs * sizeof(uint32_t), false))) return r;
            if ((r = dev_alloc(ctx, ctx->seqKey, recs * sizeof(unsigned long long), false))) return r;
            ctx->rankCap = recs;
        }
        if ((r = dev_alloc(ctx, ctx->binBlocks, (blocks + 1) * sizeof(uint32_t), false))) return r;
        f.rankOf = static_cast<uint32_t*>(ctx->rankOf.ptr);
        f.recOfRank = static_cast<uint32_t*>(ctx->recOfRank.ptr);
        f.seqRec = static_cast<uint32_t*>(ctx->seqRec.ptr);
        f.seqKey = static_cast<unsigned long long*>(ctx->seqKey.ptr);
        f.binBlocks = static_cast<uint32_t*>(ctx->binBlocks.ptr);
        f.rankGrid = (uint32_t)std::min<uint64_t>((recs + 1023) / 1024, 152 * 4);
    }

    /* ordered raster: the tile lists are filled in key order (no tile sort)
     * for tile grids of at most kMaxOrderedTiles tiles whose per-chunk
     * counts fit kMaxChunkCounts words; a sort-key cap set for testing keeps
     * the atomic fill and the tile sort */
    if (!f.orderFree && numSlots > 0 && !ctx->sortKeysCapped && (uint64_t)f.tilesX * f.tilesY <= (uint64_t)slg::kMaxOrderedTiles)
    {
        const uint64_t numTiles = (uint64_t)f.tilesX * f.tilesY;
        uint64_t chunks = std::min<uint64_t>(kMaxBinChunks, ((numSlots + 255) / 256 + 7) & ~7ull);
        chunks = std::min<uint64_t>(chunks, (kMaxChunkCounts / numTiles) & ~7ull);
        if (chunks >= 8)
        {
            const uint64_t recs = ctx->slotCap + ctx->ovfCap;
            const uint64_t blocks = (numSlots + 1023) / 1024;
            if ((r = dev_alloc(ctx, ctx->seqRec, recs * sizeof(uint32_t), false))) return r;
            if (!f.rankOf && (r = dev_alloc(ctx, ctx->itemKey, recs * sizeof(uint32_t), false))) return r;
            if ((r = dev_alloc(ctx, ctx->binBlocks, (blocks + 1) * sizeof(uint32_t), false))) return r;
            if ((r = dev_alloc(ctx, ctx->chunkCounts, numTiles * chunks * sizeof(uint32_t), false))) return r;
            if ((r = dev_alloc(ctx, ctx->tileOrder, numTiles * sizeof(uint32_t), false))) return r;
            f.seqRec = static_cast<uint32_t*>(ctx->seqRec.ptr);
            f.itemKey = f.rankOf ? nullptr : static_cast<uint32_t*>(ctx->itemKey.ptr);
            f.binBlocks = static_cast<uint32_t*>(ctx->binBlocks.ptr);
            f.chunkCounts = static_cast<uint32_t*>(ctx->chunkCounts.ptr);
            f.binChunks = (uint32_t)chunks;
            f.tileOrder = static_cast<uint32_t*>(ctx->tileOrder.ptr);
        }
    }

    /* order-free launches of triangles and points run untiled when the
     * autotuner picked it (or raster mode 3): every record is walked once
     * into per-pixel best words, no tile lists */
    if (f.orderFree && !f.hasLines && !f.hasWire && !f.hasMrt && !f.generic0 && numSlots > 0 && !ctx->forceTiled &&
        (ctx->untiled || ctx->forceUntiled))
    {
        const uint64_t pixels = (uint64_t)f.width * f.height;
        if ((r = dev_alloc(ctx, ctx->bestWords, pixels * sizeof(unsigned long long), false))) return r;
        if ((r = dev_alloc(ctx, ctx->ovfKey, std::max<uint64_t>(ctx->ovfCap, 1) * sizeof(uint32_t), false))) return r;
        f.bestWords = static_cast<unsigned long long*>(ctx->bestWords.ptr);
        f.ovfKey = static_cast<uint32_t*>(ctx->ovfKey.ptr);
    }

    /* from here on the launch is queued: a launch with a device-written
     * draw list (the scene graph's) cannot be replayed */
    {
        LogOp op;
        op.kind = hook ? LogOp::kOpaque : LogOp::kLaunch;
        if (!hook) op.reqs = reqs;
        op.fbo = fboId;
        op.batch = batch;
        op.multiple = multiple;
        log_op(ctx, std::move(op));
    }
    if (batch && ctx->batchGraphs && !ctx->profileStages && !hook)
    {
        return launch_batch_graph(ctx, f, descs, starts, n, ops);
    }

    e = cudaMemcpyAsync(devDescs, descs, n * sizeof(DrawDesc), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(devStarts, starts, (n + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "descriptor upload");
    ctx->descHead += n + 1;
    if (hook)
    {
        e = hook->fn(hook->user, devDescs, ctx->stream);
        if (e != cudaSuccess) return ctx->cuda_fail(e, "scene draw list");
    }

    e = slg::launch_pipeline(f, ops, ctx->keyCap, ctx->stream, ctx->profileStages ? ctx->stageEvents : nullptr);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "draw launch");
    return SLG_OK;
}

bool id_ok(size_t id, size_t n) { return id < n; }

/* The mode a mesh of draw_multiple is drawn with: the processor and raster
 * mode of the first mesh, the index use of its own mode. */
uint32_t multiple_mesh_mode(uint32_t first, uint32_t own)
{
    switch (first)
    {
        case SLG_RENDER_MODE_TRIANGLES:
        case SLG_RENDER_MODE_INDEXED_TRIANGLES:
        {
            const bool indexed = own == SLG_RENDER_MODE_INDEXED_TRIANGLES || own == SLG_RENDER_MODE_INDEXED_TRI_WIRE;
            return indexed ? SLG_RENDER_MODE_INDEXED_TRIANGLES : SLG_RENDER_MODE_TRIANGLES;
        }
        case SLG_RENDER_MODE_TRI_WIRE:
        case SLG_RENDER_MODE_INDEXED_TRI_WIRE:
        {
            const bool indexed = own == SLG_RENDER_MODE_INDEXED_TRIANGLES || own == SLG_RENDER_MODE_INDEXED_TRI_WIRE;
            return indexed ? SLG_RENDER_MODE_INDEXED_TRI_WIRE : SLG_RENDER_MODE_TRI_WIRE;
        }
        case SLG_RENDER_MODE_LINES:
        case SLG_RENDER_MODE_INDEXED_LINES:
            return own == SLG_RENDER_MODE_INDEXED_LINES ? SLG_RENDER_MODE_INDEXED_LINES : SLG_RENDER_MODE_LINES;
        case SLG_RENDER_MODE_POINTS:
        case SLG_RENDER_MODE_INDEXED_POINTS:
            return own == SLG_RENDER_MODE_INDEXED_POINTS ? SLG_RENDER_MODE_INDEXED_POINTS : SLG_RENDER_MODE_POINTS;
        default:
            return own;
    }
}

/*-----------------------------------------------------------------------------
 * Scene graph helpers
-----------------------------------------------------------------------------*/
/* mat4 * mat4 in the LightMath layer's order (column i = sum of a's columns
 * scaled by b's column i, left to right); host code is built without
 * contraction, like the kernels. */
void mat4_mul(const float* a, const float* b, float* out)
{
    float r[16];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            r[4 * i + j] = ((a[j] * b[4 * i] + a[4 + j] * b[4 * i + 1]) + a[8 + j] * b[4 * i + 2]) + a[12 + j] * b[4 * i + 3];
    std::memcpy(out, r, sizeof(r));
}

/* sl_extract_frustum_planes (softlight/src/SL_Camera.cpp:25-49): left, right,
 * bottom, top, near, far from the projection's rows, each scaled by
 * 1 / |xyz|. */
void frustum_planes(const float* p, float planes[24])
{
    for (int i = 0; i < 4; ++i)
    {
        const float w = p[4 * i + 3];
        planes[0 + i] = w + p[4 * i + 0];
        planes[4 + i] = w - p[4 * i + 0];
        planes[8 + i] = w + p[4 * i + 1];
        planes[12 + i] = w - p[4 * i + 1];
        planes[16 + i] = w + p[4 * i + 2];
        planes[20 + i] = w - p[4 * i + 2];
    }
    for (int k = 0; k < 6; ++k)
    {
        float* q = planes + 4 * k;
        const float lenInv = 1.f / std::sqrt((q[0] * q[0] + q[1] * q[1]) + q[2] * q[2]);
        for (int i = 0; i < 4; ++i) q[i] = q[i] * lenInv;
    }
}

Scene* scene_of(slg_context* ctx, size_t id)
{
    if (!id_ok(id, ctx->scenes.size())) return nullptr;
    return &ctx->scenes[id];
}

/* device model matrices for every node (identity for nodes never updated) */
int scene_models(slg_context* ctx, Scene& sc)
{
    const uint64_t n = sc.parents.size();
    if (sc.modelsReady == n) return SLG_OK;
    if (sc.dModel.bytes < n * 64)
    {
        DevBuffer grown;
        int r = dev_alloc(ctx, grown, std::max<size_t>(n * 64, sc.dModel.bytes * 2), false);
        if (r) return r;
        if (sc.modelsReady)
        {
            cudaError_t e = cudaMemcpyAsync(grown.ptr, sc.dModel.ptr, sc.modelsReady * 64, cudaMemcpyDeviceToDevice, ctx->stream);
            if (e != cudaSuccess) return ctx->cuda_fail(e, "scene models");
        }
        cudaStreamSynchronize(ctx->stream);
        dev_free(sc.dModel);
        sc.dModel = grown;
    }
    std::vector<float> ident((n - sc.modelsReady) * 16, 0.f);
    for (size_t k = 0; k < n - sc.modelsReady; ++k)
        for (int d = 0; d < 4; ++d) ident[16 * k + 5 * d] = 1.f;
    cudaError_t e = cudaMemcpyAsync(static_cast<float*>(sc.dModel.ptr) + 16 * sc.modelsReady, ident.data(), ident.size() * sizeof(float),
                                    cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "scene models");
    sc.modelsReady = n;
    return SLG_OK;
}

int check_transform(slg_context* ctx, const slg_transform* t)
{
    if (!t) return ctx->fail(SLG_ERR_INVALID_ARG, "null transform");
    if (t->type > 4) return ctx->fail(SLG_ERR_INVALID_ARG, "unknown transform type");
    return SLG_OK;
}

/* The draw list of the scene's mesh nodes for shaderId: entries reuse the
 * scene's shader / uniform-block pairs, made on first use. */
int scene_build_list(slg_context* ctx, Scene& sc, size_t shaderId)
{
    const Shader tmpl = ctx->shaders[shaderId];
    sc.entries.clear();
    size_t used = 0;
    for (size_t node = 0; node < sc.parents.size(); ++node)
    {
        for (uint64_t k = 0; k < sc.meshCount[node]; ++k)
        {
            const uint64_t meshId = sc.nodeMeshes[sc.meshFirst[node] + k];
            const slg_mesh& m = sc.meshes[meshId];
            if (!(m.mode & SLG_RENDER_MODE_TRIANGLES)) continue;
            if (m.materialId >= sc.materials.size()) return ctx->fail(SLG_ERR_INVALID_ARG, "scene mesh has no material");
            const size_t tex = sc.materials[m.materialId];
            if (!texture_ok(ctx, (uint32_t)tex, SLG_COLOR_RGBA_8U)) return ctx->fail(SLG_ERR_INVALID_ARG, "scene material texture is not an RGBA8 texture");
            if (used == sc.pool.size() / 2)
            {
                const size_t ubo = slg_create_ubo(ctx);
                if (ubo == SLG_INVALID_ID) return ctx->fail(SLG_ERR_NO_MEMORY, "scene uniform block");
                ctx->shaders.push_back(tmpl);
                sc.pool.push_back(ubo);
                sc.pool.push_back(ctx->shaders.size() - 1);
            }
            Scene::Entry en;
            en.node = node;
            en.mesh = meshId;
            en.texture = tex;
            en.ubo = sc.pool[2 * used];
            en.shader = sc.pool[2 * used + 1];
            ++used;
            Shader& sh = ctx->shaders[en.shader];
            sh = tmpl;
            sh.ubo = en.ubo;
            /* the host copy carries the texture the draw validates */
            std::memcpy(ctx->ubos[en.ubo].shadow, ctx->ubos[tmpl.ubo].shadow, sizeof(slg_lambert_uniforms));
            const uint32_t tex32 = (uint32_t)tex;
            std::memcpy(ctx->ubos[en.ubo].shadow + offsetof(slg_lambert_uniforms, textureId), &tex32, 4);
            sc.entries.push_back(en);
        }
    }
    if (sc.entries.size() + 1 > kDescRing) return ctx->fail(SLG_ERR_INVALID_ARG, "too many scene draws in one launch");
    std::vector<slg::SceneEntryGpu> dev(sc.entries.size());
    for (size_t i = 0; i < sc.entries.size(); ++i)
    {
        dev[i].node = sc.entries[i].node;
        dev[i].bounds = (uint32_t)sc.entries[i].mesh;
        dev[i].textureId = (uint32_t)sc.entries[i].texture;
        dev[i].ubo = static_cast<uint8_t*>(ctx->ubos[sc.entries[i].ubo].buf.ptr);
    }
    if (!dev.empty())
    {
        int r = dev_alloc(ctx, sc.dEntries, dev.size() * sizeof(slg::SceneEntryGpu), false);
        if (r) return r;
        cudaError_t e = cudaMemcpyAsync(sc.dEntries.ptr, dev.data(), dev.size() * sizeof(slg::SceneEntryGpu), cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return ctx->cuda_fail(e, "scene draw list upload");
    }
    sc.listDirty = false;
    sc.listShader = shaderId;
    return SLG_OK;
}

cudaError_t scene_draw_hook(void* user, DrawDesc* devDescs, cudaStream_t s)
{
    slg::SceneDrawArgs* a = static_cast<slg::SceneDrawArgs*>(user);
    a->descs = devDescs;
    return slg::launch_scene_draw(*a, s);
}

} // namespace

/*-----------------------------------------------------------------------------
 * C ABI
-----------------------------------------------------------------------------*/
extern "C" {

int slg_context_create(slg_context** outCtx)
{
    if (!outCtx) return SLG_ERR_INVALID_ARG;
    *outCtx = nullptr;
    slg_context* ctx = new (std::nothrow) slg_context();
    if (!ctx) return SLG_ERR_NO_MEMORY;
    cudaError_t e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMallocHost(&ctx->hostDescs, kDescRing * sizeof(DrawDesc));
    if (e == cudaSuccess) e = cudaMallocHost(&ctx->hostStarts, kDescRing * sizeof(uint64_t));
    if (e == cudaSuccess) e = cudaMallocHost(&ctx->hostStatus, 4 * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&ctx->devDescs.ptr, kDescRing * sizeof(DrawDesc));
    if (e == cudaSuccess) e = cudaMalloc(&ctx->devStarts.ptr, kDescRing * sizeof(uint64_t));
    /* the device status words (overflow bits and sizes), read and cleared by
     * settle; every launch of the context reports into them, the
     * no-allocation draw included */
    if (e == cudaSuccess) e = cudaMalloc(&ctx->status.ptr, 4 * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMemset(ctx->status.ptr, 0, 4 * sizeof(int32_t));
    for (int i = 0; i < 5 && e == cudaSuccess; ++i) e = cudaEventCreate(&ctx->stageEvents[i]);
    if (e == cudaSuccess) e = slg::init_library_attributes(ctx->keyCap);
    if (e == cudaSuccess) e = (cudaError_t)slg::builtin_pipeline().set_attributes();
    if (e != cudaSuccess)
    {
        slg_context_destroy(ctx);
        return SLG_ERR_CUDA;
    }
    ctx->devDescs.bytes = kDescRing * sizeof(DrawDesc);
    ctx->devStarts.bytes = kDescRing * sizeof(uint64_t);
    ctx->status.bytes = 4 * sizeof(int32_t);
    *outCtx = ctx;
    return SLG_OK;
}

void slg_context_destroy(slg_context* ctx)
{
    if (!ctx) return;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (Vbo& v : ctx->vbos) dev_free(v.buf);
    for (Ibo& v : ctx->ibos) dev_free(v.buf);
    for (Texture& t : ctx->textures) dev_free(t.buf);
    for (Ubo& u : ctx->ubos) dev_free(u.buf);
    for (Fbo& f : ctx->fbos) dev_free(f.vis);
    for (auto& st : ctx->uboStage)
    {
        if (st.host) cudaFreeHost(st.host);
        if (st.done) cudaEventDestroy(st.done);
    }
    dev_free(ctx->uboStageDev);
    for (Scene& sc : ctx->scenes)
    {
        dev_free(sc.dNodes);
        dev_free(sc.dList);
        dev_free(sc.dModel);
        dev_free(sc.dBounds);
        dev_free(sc.dEntries);
    }
    DevBuffer* scratch[] = {&ctx->texTable, &ctx->bufTable, &ctx->vaoTable, &ctx->records, &ctx->varyings, &ctx->slotInfo, &ctx->slotOvf,
                            &ctx->ovfCount, &ctx->clipQueue, &ctx->clipCount, &ctx->aliasEvents, &ctx->aliasCount,
                            &ctx->cachePos, &ctx->cacheVary, &ctx->recVerts,
                            &ctx->tileCount, &ctx->tileOffset,
                            &ctx->tileCursor, &ctx->entries, &ctx->blitBuf,
                            &ctx->rankOf, &ctx->recOfRank, &ctx->seqRec, &ctx->seqKey, &ctx->binBlocks,
                            &ctx->chunkCounts, &ctx->itemKey, &ctx->tileOrder, &ctx->bestWords, &ctx->ovfKey, &ctx->sortScratch,
                            &ctx->status, &ctx->devDescs, &ctx->devStarts};
    for (DevBuffer* b : scratch) dev_free(*b);
    if (ctx->graph.exec) cudaGraphExecDestroy(ctx->graph.exec);
    dev_free(ctx->graph.devDescs);
    dev_free(ctx->graph.devStarts);
    if (ctx->hostDescs) cudaFreeHost(ctx->hostDescs);
    if (ctx->hostStarts) cudaFreeHost(ctx->hostStarts);
    if (ctx->hostStatus) cudaFreeHost(ctx->hostStatus);
    for (cudaEvent_t ev : ctx->stageEvents) if (ev) cudaEventDestroy(ev);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char* slg_last_error(const slg_context* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

unsigned slg_num_threads(slg_context* ctx, unsigned n)
{
    if (n > 0) ctx->numThreads = n;
    return ctx->numThreads;
}

size_t slg_create_vbo(slg_context* ctx) { ctx->vbos.emplace_back(); ctx->tablesDirty = true; return ctx->vbos.size() - 1; }

int slg_vbo_init(slg_context* ctx, size_t id, size_t numBytes, const void* data)
{
    /* queued draws read the old contents: complete them first */
    if (!ctx->log.empty())
    {
        const int settled = settle(ctx);
        if (settled) return settled;
    }
    if (!id_ok(id, ctx->vbos.size())) return ctx->fail(SLG_ERR_INVALID_ID, "invalid vbo id");
    Vbo& v = ctx->vbos[id];
    int r = dev_alloc(ctx, v.buf, numBytes + 64, true);
    if (r) return r;
    v.size = numBytes;
    if (data && numBytes)
    {
        cudaError_t e = cudaMemcpyAsync(v.buf.ptr, data, numBytes, cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return ctx->cuda_fail(e, "vbo upload");
    }
    ctx->tablesDirty = true;
    return SLG_OK;
}

int slg_vbo_assign(slg_context* ctx, size_t id, const void* data, size_t offset, size_t numBytes)
{
    /* queued draws read the old contents: complete them first */
    if (!ctx->log.empty())
    {
        const int settled = settle(ctx);
        if (settled) return settled;
    }
    if (!id_ok(id, ctx->vbos.size())) return ctx->fail(SLG_ERR_INVALID_ID, "invalid vbo id");
    Vbo& v = ctx->vbos[id];
    if (offset + numBytes > v.size) return ctx->fail(SLG_ERR_INVALID_ARG, "vbo range");
    cudaError_t e = cudaMemcpyAsync(static_cast<uint8_t*>(v.buf.ptr) + offset, data, numBytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "vbo assign");
    return SLG_OK;
}

size_t slg_create_ibo(slg_context* ctx) { ctx->ibos.emplace_back(); return ctx->ibos.size() - 1; }

int slg_ibo_init(slg_context* ctx, size_t id, size_t numElements, int indexType, const void* data)
{
    /* queued draws read the old contents: complete them first */
    if (!ctx->log.empty())
    {
        const int settled = settle(ctx);
        if (settled) return settled;
    }
    if (!id_ok(id, ctx->ibos.size())) return ctx->fail(SLG_ERR_INVALID_ID, "invalid ibo id");
    const size_t ib = index_bytes(indexType);
    if (!ib) return ctx->fail(SLG_ERR_INVALID_ARG, "invalid index type");
    Ibo& v = ctx->ibos[id];
    /* padded like SL_IndexBuffer so a partial last triangle reads zeros */
    int r = dev_alloc(ctx, v.buf, numElements * ib + 16, true);
    if (r) return r;
    v.type = indexType;
    v.count = numElements;
    v.maxIndex = 0;
    for (size_t i = 0; data && i < numElements; ++i)
    {
        uint64_t x;
        if (ib == 1) x = static_cast<const uint8_t*>(data)[i];
        else if (ib == 2) { uint16_t t; std::memcpy(&t, static_cast<const uint8_t*>(data) + 2 * i, 2); x = t; }
        else { uint32_t t; std::memcpy(&t, static_cast<const uint8_t*>(data) + 4 * i, 4); x = t; }
        v.maxIndex = std::max(v.maxIndex, x);
    }
    if (data && numElements)
    {
        cudaError_t e = cudaMemcpyAsync(v.buf.ptr, data, numElements * ib, cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return ctx->cuda_fail(e, "ibo upload");
    }
    return SLG_OK;
}

size_t slg_create_vao(slg_context* ctx) { ctx->vaos.emplace_back(); ctx->tablesDirty = true; return ctx->vaos.size() - 1; }

int slg_vao_set_vertex_buffer(slg_context* ctx, size_t vao, size_t vbo)
{
    if (!id_ok(vao, ctx->vaos.size()) || !id_ok(vbo, ctx->vbos.size())) return ctx->fail(SLG_ERR_INVALID_ID, "invalid id");
    ctx->vaos[vao].vbo = vbo;
    return SLG_OK;
}

int slg_vao_set_index_buffer(slg_context* ctx, size_t vao, size_t ibo)
{
    if (!id_ok(vao, ctx->vaos.size()) || !id_ok(ibo, ctx->ibos.size())) return ctx->fail(SLG_ERR_INVALID_ID, "invalid id");
    ctx->vaos[vao].ibo = ibo;
    return SLG_OK;
}

int slg_vao_set_binding(slg_context* ctx, size_t vao, unsigned bindId, ptrdiff_t offset, ptrdiff_t stride,
                        unsigned numComponents, int dataType)
{
    if (!id_ok(vao, ctx->vaos.size()) || bindId >= 8) return ctx->fail(SLG_ERR_INVALID_ID, "invalid id");
    Binding& b = ctx->vaos[vao].bindings[bindId];
    b.offset = offset;
    b.stride = stride;
    b.comps = numComponents;
    b.type = dataType;
    ctx->tablesDirty = true;
    return SLG_OK;
}

size_t slg_create_texture(slg_context* ctx) { ctx->textures.emplace_back(); ctx->tablesDirty = true; return ctx->textures.size() - 1; }

int slg_texture_init(slg_context* ctx, size_t id, int colorType, uint16_t w, uint16_t h, uint16_t d)
{
    /* queued draws read the old contents: complete them first */
    if (!ctx->log.empty())
    {
        const int settled = settle(ctx);
        if (settled) return settled;
    }
    if (!id_ok(id, ctx->textures.size())) return ctx->fail(SLG_ERR_INVALID_ID, "invalid texture id");
    const size_t bpt = bytes_per_color(colorType);
    if (!bpt || !w || !h || !d) return ctx->fail(SLG_ERR_INVALID_ARG, "invalid texture format or size");
    Texture& t = ctx->textures[id];
    /* zero padding after the dense texels: bilinear filtering may read one
     * row and one texel past the end (softlight/include/softlight/SL_Sampler.hpp:200-201,
     * allocation padded by softlight/src/SL_Texture.cpp:28-56) */
    const size_t texels = (size_t)w * h * d;
    const size_t padded = texels + (size_t)w + 64;
    int r = dev_alloc(ctx, t.buf, padded * bpt, true);
    if (r) return r;
    t.type = colorType;
    t.w = w; t.h = h; t.d = d;
    t.bpt = (unsigned)bpt;
    ctx->tablesDirty = true;
    return SLG_OK;
}

int slg_texture_set_texels(slg_context* ctx, size_t id, const void* data, size_t numBytes)
{
    /* queued draws read the old contents: complete them first */
    if (!ctx->log.empty())
    {
        const int settled = settle(ctx);
        if (settled) return settled;
    }
    if (!id_ok(id, ctx->textures.size())) return ctx->fail(SLG_ERR_INVALID_ID, "invalid texture id");
    Texture& t = ctx->textures[id];
    if (!t.buf.ptr || numBytes != (size_t)t.w * t.h * t.d * t.bpt) return ctx->fail(SLG_ERR_INVALID_ARG, "texel byte count");
    cudaError_t e = cudaMemcpyAsync(t.buf.ptr, data, numBytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "texture upload");
    return SLG_OK;
}

int slg_texture_read(slg_context* ctx, size_t id, void* dst, size_t numBytes)
{
    if (!id_ok(id, ctx->textures.size())) return ctx->fail(SLG_ERR_INVALID_ID, "invalid texture id");
    Texture& t = ctx->textures[id];
    if (!t.buf.ptr || numBytes != (size_t)t.w * t.h * t.d * t.bpt) return ctx->fail(SLG_ERR_INVALID_ARG, "texel byte count");
    /* the texels as the queued draws leave them, then the copy */
    const int r = settle(ctx);
    cudaError_t e = cudaMemcpyAsync(dst, t.buf.ptr, numBytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "texture read");
    return r;
}

} // extern "C"

namespace
{

/* Geometry of SL_BlitProcessor::blit_nearest (softlight/src/SL_BlitProcessor.cpp:621-660)
 * for a source texture and a dstW x dstH destination, in the reference's
 * 64-bit unsigned arithmetic; rejects rectangles whose reads or writes the
 * reference would make out of bounds. */
int blit_geometry(slg_context* ctx, const Texture& src, uint64_t dstW, uint64_t dstH, uint16_t srcX0, uint16_t srcY0,
                  uint16_t srcX1, uint16_t srcY1, uint16_t dstX0, uint16_t dstY0, uint16_t dstX1, uint16_t dstY1,
                  slg::BlitArgs& a)
{
    if (srcX1 <= srcX0 || srcY1 <= srcY0 || dstX1 <= dstX0 || dstY1 <= dstY0)
        return ctx->fail(SLG_ERR_INVALID_ARG, "empty or inverted blit rectangle");
    if (dstY1 > dstH) return ctx->fail(SLG_ERR_INVALID_ARG, "blit rectangle extends below the destination");
    const uint64_t inW = (uint64_t)srcX1 - srcX0, inH = (uint64_t)srcY1 - srcY0;
    const uint64_t x0 = dstX0, x1 = std::min<uint64_t>(dstW, x0 + ((uint64_t)dstX1 - dstX0));
    const uint64_t y0 = dstY0, y1 = dstY1;
    std::memset(&a, 0, sizeof(a));
    a.foutW = ((inW << 16) / dstW) + 1u;
    a.foutH = ((inH << 16) / dstH) + 1u;
    a.x0 = x0;
    a.y0 = y0;
    a.nx = (x1 > x0) ? x1 - x0 : 0u;
    a.ny = y1 - y0;
    a.srcY0 = srcY0;
    a.srcY1 = srcY1;
    a.srcW = src.w;
    a.dstW = dstW;
    if (a.nx == 0u) return SLG_OK;
    const uint64_t maxSrcX = ((x1 - 1u) * a.foutW) >> 16;
    const uint64_t yfMin = (y0 * a.foutH) >> 16, yfMax = ((y1 - 1u) * a.foutH) >> 16;
    if (maxSrcX >= src.w || srcY0 + yfMax + 1u > srcY1 || srcY1 - (srcY0 + yfMin) - 1u >= src.h)
        return ctx->fail(SLG_ERR_INVALID_ARG, "blit rectangle reads outside the source texture");
    return SLG_OK;
}

bool blit_type_ok(int t) { return t == SLG_COLOR_RGBA_8U || t == SLG_COLOR_RGBA_FLOAT || t == SLG_COLOR_R_FLOAT; }

} // namespace

extern "C" {

int slg_blit_rect(slg_context* ctx, size_t outId, size_t inId, uint16_t srcX0, uint16_t srcY0, uint16_t srcX1,
                  uint16_t srcY1, uint16_t dstX0, uint16_t dstY0, uint16_t dstX1, uint16_t dstY1)
{
    if (!id_ok(outId, ctx->textures.size()) || !id_ok(inId, ctx->textures.size())) return ctx->fail(SLG_ERR_INVALID_ID, "invalid texture id");
    const Texture& src = ctx->textures[inId];
    Texture& dst = ctx->textures[outId];
    if (!src.buf.ptr || !dst.buf.ptr || !blit_type_ok(src.type) || !blit_type_ok(dst.type))
        return ctx->fail(SLG_ERR_INVALID_ARG, "blit needs initialised R float, RGBA8 or RGBA float textures");
    if (outId == inId) return ctx->fail(SLG_ERR_INVALID_ARG, "blit source and destination are the same texture");
    slg::BlitArgs a;
    int r = blit_geometry(ctx, src, dst.w, dst.h, srcX0, srcY0, srcX1, srcY1, dstX0, dstY0, dstX1, dstY1, a);
    if (r || a.nx == 0u) return r;
    a.src = static_cast<const uint8_t*>(src.buf.ptr);
    a.dst = static_cast<uint8_t*>(dst.buf.ptr);
    a.srcType = src.type;
    a.dstType = dst.type;
    a.status = static_cast<const int32_t*>(ctx->status.ptr);
    {
        LogOp op;
        op.kind = LogOp::kBlit;
        op.out = outId;
        op.in = inId;
        const uint16_t rect[8] = {srcX0, srcY0, srcX1, srcY1, dstX0, dstY0, dstX1, dstY1};
        std::memcpy(op.rect, rect, sizeof(rect));
        log_op(ctx, std::move(op));
    }
    cudaError_t e = slg::launch_blit(a, ctx->stream);
    return (e == cudaSuccess) ? SLG_OK : ctx->cuda_fail(e, "blit launch");
}

int slg_blit(slg_context* ctx, size_t outId, size_t inId)
{
    if (!id_ok(outId, ctx->textures.size()) || !id_ok(inId, ctx->textures.size())) return ctx->fail(SLG_ERR_INVALID_ID, "invalid texture id");
    const Texture& src = ctx->textures[inId];
    const Texture& dst = ctx->textures[outId];
    return slg_blit_rect(ctx, outId, inId, 0, 0, src.w, src.h, 0, 0, dst.w, dst.h);
}

int slg_blit_read(slg_context* ctx, size_t inId, int dstType, uint16_t dstW, uint16_t dstH, void* out, size_t numBytes)
{
    if (!id_ok(inId, ctx->textures.size())) return ctx->fail(SLG_ERR_INVALID_ID, "invalid texture id");
    const Texture& src = ctx->textures[inId];
    if (!src.buf.ptr || !blit_type_ok(src.type) || !blit_type_ok(dstType))
        return ctx->fail(SLG_ERR_INVALID_ARG, "blit needs R float, RGBA8 or RGBA float formats");
    const size_t bytes = (size_t)dstW * dstH * bytes_per_color(dstType);
    if (!out || numBytes != bytes || bytes == 0) return ctx->fail(SLG_ERR_INVALID_ARG, "destination byte count");
    slg::BlitArgs a;
    int r = blit_geometry(ctx, src, dstW, dstH, 0, 0, src.w, src.h, 0, 0, dstW, dstH, a);
    if (r) return r;
    if ((r = settle(ctx))) return r;   /* the source as the queued draws leave it */
    a.status = nullptr;
    if ((r = dev_alloc(ctx, ctx->blitBuf, bytes, false))) return r;
    a.src = static_cast<const uint8_t*>(src.buf.ptr);
    a.dst = static_cast<uint8_t*>(ctx->blitBuf.ptr);
    a.srcType = src.type;
    a.dstType = dstType;
    cudaError_t e = slg::launch_blit(a, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, ctx->blitBuf.ptr, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "blit read");
    return SLG_OK;
}

size_t slg_create_framebuffer(slg_context* ctx) { ctx->fbos.emplace_back(); return ctx->fbos.size() - 1; }

/* SL_Framebuffer::reserve_color_buffers (softlight/src/SL_Framebuffer.cpp:
 * 821-845): 1..4 attachments; a new count detaches every colour attachment. */
int slg_fbo_reserve_color_buffers(slg_context* ctx, size_t fbo, unsigned n)
{
    if (!id_ok(fbo, ctx->fbos.size())) return ctx->fail(SLG_ERR_INVALID_ID, "invalid fbo");
    Fbo& b = ctx->fbos[fbo];
    if (n == b.numColors) return SLG_OK;
    if (n < 1 || n > 4) return ctx->fail(SLG_ERR_INVALID_ARG, "a framebuffer has 1 to 4 colour attachments");
    for (size_t& c : b.colors) c = SLG_INVALID_ID;
    b.numColors = n;
    return SLG_OK;
}

int slg_fbo_attach_color_buffer(slg_context* ctx, size_t fbo, unsigned index, size_t tex)
{
    /* queued draws read the old contents: complete them first */
    if (!ctx->log.empty())
    {
        const int settled = settle(ctx);
        if (settled) return settled;
    }
    if (!id_ok(fbo, ctx->fbos.size()) || !id_ok(tex, ctx->textures.size()) || index >= ctx->fbos[fbo].numColors)
        return ctx->fail(SLG_ERR_INVALID_ARG, "invalid fbo attachment");
    ctx->fbos[fbo].colors[index] = tex;
    return SLG_OK;
}

int slg_fbo_attach_depth_buffer(slg_context* ctx, size_t fbo, size_t tex)
{
    /* queued draws read the old contents: complete them first */
    if (!ctx->log.empty())
    {
        const int settled = settle(ctx);
        if (settled) return settled;
    }
    if (!id_ok(fbo, ctx->fbos.size()) || !id_ok(tex, ctx->textures.size())) return ctx->fail(SLG_ERR_INVALID_ARG, "invalid fbo attachment");
    const int dt = ctx->textures[tex].type;
    if (dt != SLG_COLOR_R_HALF && dt != SLG_COLOR_R_FLOAT && dt != SLG_COLOR_R_DOUBLE)
        return ctx->fail(SLG_ERR_INVALID_ARG, "depth must be R_HALF, R_FLOAT or R_DOUBLE");
    ctx->fbos[fbo].depth = tex;
    return SLG_OK;
}

size_t slg_create_ubo(slg_context* ctx)
{
    ctx->ubos.emplace_back();
    if (dev_alloc(ctx, ctx->ubos.back().buf, 1024, true) != SLG_OK)
    {
        ctx->ubos.pop_back();
        return SLG_INVALID_ID;
    }
    return ctx->ubos.size() - 1;
}

/* SL_UniformBuffer contents: the host copy is written now; the device copy
 * before the next launch that reads uniform blocks (flush_ubos). */
int slg_ubo_assign(slg_context* ctx, size_t id, const void* data, size_t numBytes)
{
    if (!id_ok(id, ctx->ubos.size()) || numBytes > 1024 || (!data && numBytes)) return ctx->fail(SLG_ERR_INVALID_ARG, "invalid ubo");
    if (!numBytes) return SLG_OK;
    Ubo& u = ctx->ubos[id];
    if (!ctx->log.empty())
    {
        LogOp op;
        op.kind = LogOp::kUbo;
        op.ubo = id;
        op.before.assign(u.shadow, u.shadow + numBytes);
        op.after.assign(static_cast<const uint8_t*>(data), static_cast<const uint8_t*>(data) + numBytes);
        log_op(ctx, std::move(op));
    }
    std::memcpy(u.shadow, data, numBytes);
    if (!u.pending) ctx->uboPending.push_back(id);
    u.pending = std::max<uint32_t>(u.pending, (uint32_t)numBytes);
    return SLG_OK;
}

int slg_ubo_assign_many(slg_context* ctx, const size_t* ids, size_t count, const void* blocks, size_t blockStride, size_t numBytes)
{
    if (!count) return SLG_OK;
    if (!ids || !blocks || numBytes > 1024 || blockStride < numBytes) return ctx->fail(SLG_ERR_INVALID_ARG, "invalid ubo blocks");
    for (size_t k = 0; k < count; ++k)
        if (!id_ok(ids[k], ctx->ubos.size())) return ctx->fail(SLG_ERR_INVALID_ID, "invalid ubo id");
    if (!numBytes) return SLG_OK;
    const uint8_t* src = static_cast<const uint8_t*>(blocks);
    for (size_t k = 0; k < count; ++k)
    {
        Ubo& u = ctx->ubos[ids[k]];
        if (!ctx->log.empty())
        {
            LogOp op;
            op.kind = LogOp::kUbo;
            op.ubo = ids[k];
            op.before.assign(u.shadow, u.shadow + numBytes);
            op.after.assign(src + k * blockStride, src + k * blockStride + numBytes);
            log_op(ctx, std::move(op));
        }
        std::memcpy(u.shadow, src + k * blockStride, numBytes);
        if (!u.pending) ctx->uboPending.push_back(ids[k]);
        u.pending = std::max<uint32_t>(u.pending, (uint32_t)numBytes);
    }
    return SLG_OK;
}

size_t slg_create_shader(slg_context* ctx, const slg_vertex_shader* vs, const slg_fragment_shader* fs, size_t ubo)
{
    if (!vs || !fs) return ctx->fail_id("null shader");
    /* SL_Context::create_shader (softlight/src/SL_Context.cpp:492-505) */
    if (vs->numVaryings < fs->numVaryings || vs->numVaryings > 4 || fs->numVaryings > 4 || fs->numOutputs > 4)
        return ctx->fail_id("invalid varying or output count");
    /* the vertex and fragment program run in one set's kernels */
    /* program -> its set (0: built-in) and registration; both programs of a
     * shader must come from one set */
    const auto find = [&](uint32_t id, uint32_t& set, const slg_program_info*& info) {
        set = 0;
        info = nullptr;
        if (valid_program(id)) return true;
        for (size_t k = 0; k < ctx->programSets.size(); ++k)
            for (const slg_program_info& p : ctx->programSets[k].programs)
                if (p.id == id)
                {
                    set = (uint32_t)k + 1;
                    info = &p;
                    return true;
                }
        return false;
    };
    uint32_t set = 0, fSet = 0;
    const slg_program_info* vi = nullptr;
    const slg_program_info* fi = nullptr;
    if (!find(vs->program, set, vi) || !find(fs->program, fSet, fi)) return ctx->fail_id("unknown shader program");
    if (set != fSet) return ctx->fail_id("the vertex and fragment programs come from different program sets");
    const uint32_t fsFlags = fi ? fi->flags : builtin_program_flags(fs->program);
    const uint32_t vertexBytes = vi ? vi->vertexBytes : (uint32_t)program_vertex_bytes(vs->program);
    if (vs->cullMode > SLG_CULL_OFF || fs->depthTest > SLG_DEPTH_TEST_NOT_EQUAL || fs->blend > SLG_BLEND_SCREEN || fs->depthMask > 1)
        return ctx->fail_id("invalid pipeline state");
    if (ubo != SLG_INVALID_ID && !id_ok(ubo, ctx->ubos.size())) return ctx->fail_id("invalid ubo id");
    Shader s;
    s.cull = vs->cullMode;
    s.depthTest = fs->depthTest;
    s.depthMask = fs->depthMask;
    s.blend = fs->blend;
    s.numVaryings = fs->numVaryings;
    s.numOutputs = fs->numOutputs;
    s.vsProgram = vs->program;
    s.fsProgram = fs->program;
    s.ubo = ubo;
    s.programSet = set;
    s.fsFlags = fsFlags;
    s.vertexBytes = vertexBytes;
    ctx->shaders.push_back(s);
    return ctx->shaders.size() - 1;
}

int slg_register_programs(slg_context* ctx, const slg_pipeline_ops* ops, const slg_program_info* programs, size_t numPrograms)
{
    if (!ops || !programs || !numPrograms) return ctx->fail(SLG_ERR_INVALID_ARG, "null program set");
    if (ops->abiVersion != SLG_PIPELINE_ABI_VERSION || ops->frameBytes != sizeof(Frame))
        return ctx->fail(SLG_ERR_INVALID_ARG, "program set compiled against another version of the draw-path headers");
    if (!ops->set_attributes || !ops->launch_vertex || !ops->launch_raster) return ctx->fail(SLG_ERR_INVALID_ARG, "incomplete program set");
    for (size_t i = 0; i < numPrograms; ++i)
    {
        const slg_program_info& p = programs[i];
        if (p.id < SLG_PROGRAM_USER_FIRST) return ctx->fail(SLG_ERR_INVALID_ARG, "registered program ids start at SLG_PROGRAM_USER_FIRST");
        if (p.flags & ~(SLG_PROGRAM_DISCARDS | SLG_PROGRAM_WRITES_DEPTH)) return ctx->fail(SLG_ERR_INVALID_ARG, "unknown program flags");
        for (size_t j = 0; j < i; ++j)
            if (programs[j].id == p.id) return ctx->fail(SLG_ERR_INVALID_ARG, "program id listed twice");
        for (const ProgramSet& set : ctx->programSets)
            for (const slg_program_info& q : set.programs)
                if (q.id == p.id) return ctx->fail(SLG_ERR_INVALID_ARG, "program id already registered");
    }
    const cudaError_t e = (cudaError_t)ops->set_attributes();
    if (e != cudaSuccess) return ctx->cuda_fail(e, "program set kernel attributes");
    ProgramSet set;
    set.ops = *ops;
    set.programs.assign(programs, programs + numPrograms);
    ctx->programSets.push_back(std::move(set));
    return SLG_OK;
}

int slg_clear_color_buffer(slg_context* ctx, size_t fbo, unsigned att, const double rgba[4])
{
    if (!id_ok(fbo, ctx->fbos.size()) || att >= ctx->fbos[fbo].numColors || ctx->fbos[fbo].colors[att] == SLG_INVALID_ID)
        return ctx->fail(SLG_ERR_INVALID_ARG, "invalid fbo attachment");
    {
        LogOp op;
        op.kind = LogOp::kClearColor;
        op.fbo = fbo;
        op.attachment = att;
        for (int k = 0; k < 4; ++k) op.value[k] = rgba[k];
        log_op(ctx, std::move(op));
    }
    return clear_texture(ctx, ctx->fbos[fbo].colors[att], rgba);
}

int slg_clear_depth_buffer(slg_context* ctx, size_t fbo, double depth)
{
    if (!id_ok(fbo, ctx->fbos.size()) || ctx->fbos[fbo].depth == SLG_INVALID_ID) return ctx->fail(SLG_ERR_INVALID_ARG, "invalid fbo");
    {
        LogOp op;
        op.kind = LogOp::kClearDepth;
        op.fbo = fbo;
        op.value[0] = depth;
        log_op(ctx, std::move(op));
    }
    const double d[4] = {depth, 0, 0, 0};
    int r = clear_texture(ctx, ctx->fbos[fbo].depth, d);
    if (r || !ctx->fbos[fbo].visEnabled) return r;
    cudaError_t e = cudaMemsetAsync(ctx->fbos[fbo].vis.ptr, 0, ctx->fbos[fbo].vis.bytes, ctx->stream);
    return (e == cudaSuccess) ? SLG_OK : ctx->cuda_fail(e, "visibility clear");
}

int slg_clear_framebuffer(slg_context* ctx, size_t fbo, unsigned att, const double rgba[4], double depth)
{
    int r = slg_clear_color_buffer(ctx, fbo, att, rgba);
    if (r) return r;
    return slg_clear_depth_buffer(ctx, fbo, depth);
}

int slg_draw(slg_context* ctx, const slg_mesh* m, size_t shaderId, size_t fboId)
{
    return slg_draw_instanced(ctx, m, 1, shaderId, fboId);
}

int slg_draw_instanced(slg_context* ctx, const slg_mesh* m, size_t numInstances, size_t shaderId, size_t fboId)
{
    if (!m) return ctx->fail(SLG_ERR_INVALID_ARG, "null mesh");
    if (!numInstances) return SLG_OK;
    std::vector<DrawRequest> reqs(1);
    reqs[0] = {*m, numInstances, shaderId, 0};
    return run_launch(ctx, reqs, fboId);
}

int slg_draw_multiple(slg_context* ctx, const slg_mesh* meshes, size_t numMeshes, size_t shaderId, size_t fboId)
{
    if (!meshes || !numMeshes) return SLG_OK;
    std::vector<DrawRequest> reqs(numMeshes);
    for (size_t i = 0; i < numMeshes; ++i)
    {
        /* SL_ProcessorPool::run_shader_processors picks the processor and
         * the raster mode from the first mesh (softlight/src/
         * SL_ProcessorPool.cpp:333-357); each mesh only decides whether
         * its elements are indices (SL_TriProcessor.cpp:686-712,
         * SL_LineProcessor.cpp:207, SL_PointProcessor.cpp:77) */
        slg_mesh m = meshes[i];
        m.mode = multiple_mesh_mode(meshes[0].mode, meshes[i].mode);
        reqs[i] = {m, 1, shaderId, 0};
    }
    return run_launch(ctx, reqs, fboId, false, nullptr, true);
}

int slg_draw_batch(slg_context* ctx, const slg_draw_cmd* cmds, size_t numCmds, size_t fboId)
{
    if (!cmds || !numCmds) return SLG_OK;
    std::vector<DrawRequest> reqs;
    reqs.reserve(numCmds);
    for (size_t i = 0; i < numCmds; ++i)
    {
        if (cmds[i].numInstances == 0) continue;
        reqs.push_back({cmds[i].mesh, cmds[i].numInstances, cmds[i].shaderId, 0});
    }
    return run_launch(ctx, reqs, fboId, true);
}

int slg_set_vertex_block(slg_context* ctx, int threads)
{
    if (threads != 64 && threads != 128 && threads != 256) return ctx->fail(SLG_ERR_INVALID_ARG, "vertex block must be 64, 128 or 256");
    ctx->vsBlock = threads;
    return SLG_OK;
}

int slg_set_batch_graphs(slg_context* ctx, int enable)
{
    ctx->batchGraphs = enable != 0;
    return SLG_OK;
}

/* Times clear + slg_draw_batch for every supported tile size and vertex
 * block size and keeps the fastest; out = {tileW, tileH, vertex block}. */
int slg_autotune(slg_context* ctx, const slg_draw_cmd* cmds, size_t numCmds, size_t fboId,
                 const double rgba[4], double depth, int out[3])
{
    if (fboId >= ctx->fbos.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid fbo id");
    static const int tiles[][2] = {{8, 8}, {16, 16}, {32, 16}, {32, 32}, {64, 32}, {64, 64}};
    static const int blocks[] = {64, 128, 256};
    const bool graphs = ctx->batchGraphs, prof = ctx->profileStages;
    ctx->batchGraphs = false;
    ctx->profileStages = false;
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    float best = 1e30f;
    int bw = ctx->tileW, bh = ctx->tileH, bb = ctx->vsBlock;
    const bool hasColor = ctx->fbos[fboId].numColors > 0;
    auto frame = [&]() -> int {
        const int c = hasColor ? slg_clear_framebuffer(ctx, fboId, 0, rgba, depth) : slg_clear_depth_buffer(ctx, fboId, depth);
        return c ? c : slg_draw_batch(ctx, cmds, numCmds, fboId);
    };
    int status = SLG_OK;
    for (const auto& t : tiles)
    {
        for (int b : blocks)
        {
            ctx->tileW = t[0];
            ctx->tileH = t[1];
            ctx->vsBlock = b;
            int r = frame();
            if (!r) r = frame();
            if (!r) r = slg_finish(ctx);
            if (r == SLG_ERR_OVERFLOW) continue; /* this tile size overflows its lists */
            if (r) { status = r; break; }
            cudaEventRecord(t0, ctx->stream);
            for (int k = 0; k < 3 && !r; ++k) r = frame();
            cudaEventRecord(t1, ctx->stream);
            if (!r) r = slg_finish(ctx);
            if (r == SLG_ERR_OVERFLOW) continue;
            if (r) { status = r; break; }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, t0, t1);
            if (ms < best) { best = ms; bw = t[0]; bh = t[1]; bb = b; }
        }
        if (status) break;
    }
    /* then the untiled order-free raster (the tile size does not matter to
     * it; launches it does not apply to keep the tiles) */
    const bool wasUntiled = ctx->untiled;
    bool bu = wasUntiled && !status;
    if (!status && !ctx->forceTiled && !ctx->forceOrdered)
    {
        bu = false;
        ctx->tileW = bw;
        ctx->tileH = bh;
        ctx->untiled = true;
        for (int b : blocks)
        {
            ctx->vsBlock = b;
            int r = frame();
            if (!r) r = frame();
            if (!r) r = slg_finish(ctx);
            if (r == SLG_ERR_OVERFLOW) continue;
            if (r) { status = r; break; }
            cudaEventRecord(t0, ctx->stream);
            for (int k = 0; k < 3 && !r; ++k) r = frame();
            cudaEventRecord(t1, ctx->stream);
            if (!r) r = slg_finish(ctx);
            if (r == SLG_ERR_OVERFLOW) continue;
            if (r) { status = r; break; }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, t0, t1);
            if (ms < best) { best = ms; bb = b; bu = true; }
        }
    }
    ctx->untiled = status ? wasUntiled : bu;
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    ctx->tileW = bw;
    ctx->tileH = bh;
    ctx->vsBlock = bb;
    ctx->batchGraphs = graphs;
    ctx->profileStages = prof;
    if (out) { out[0] = bw; out[1] = bh; out[2] = bb; }
    return status;
}

/*-----------------------------------------------------------------------------
 * Scene graph (SL_SceneGraph, softlight/include/softlight/SL_SceneGraph.hpp:215)
-----------------------------------------------------------------------------*/
size_t slg_create_scene(slg_context* ctx)
{
    ctx->scenes.emplace_back();
    return ctx->scenes.size() - 1;
}

int slg_scene_insert_mesh(slg_context* ctx, size_t sceneId, const slg_mesh* mesh, const float maxPoint[3],
                          const float minPoint[3], size_t* outMeshId)
{
    Scene* sc = scene_of(ctx, sceneId);
    if (!sc) return ctx->fail(SLG_ERR_INVALID_ID, "invalid scene id");
    if (!mesh || !maxPoint || !minPoint || !outMeshId) return ctx->fail(SLG_ERR_INVALID_ARG, "null argument");
    if (mesh->vaoId >= ctx->vaos.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid vao id");
    sc->meshes.push_back(*mesh);
    const float b[8] = {maxPoint[0], maxPoint[1], maxPoint[2], 1.f, minPoint[0], minPoint[1], minPoint[2], 1.f};
    sc->bounds.insert(sc->bounds.end(), b, b + 8);
    sc->listDirty = true;
    *outMeshId = sc->meshes.size() - 1;
    return SLG_OK;
}

int slg_scene_insert_material(slg_context* ctx, size_t sceneId, size_t ambientTextureId, size_t* outMaterialId)
{
    Scene* sc = scene_of(ctx, sceneId);
    if (!sc) return ctx->fail(SLG_ERR_INVALID_ID, "invalid scene id");
    if (!outMaterialId) return ctx->fail(SLG_ERR_INVALID_ARG, "null argument");
    sc->materials.push_back(ambientTextureId);
    sc->listDirty = true;
    *outMaterialId = sc->materials.size() - 1;
    return SLG_OK;
}

int slg_scene_insert_node(slg_context* ctx, size_t sceneId, size_t parentId, size_t numSubMeshes, const size_t* subMeshIds,
                          const slg_transform* transform, size_t* outNodeId)
{
    Scene* sc = scene_of(ctx, sceneId);
    if (!sc) return ctx->fail(SLG_ERR_INVALID_ID, "invalid scene id");
    if (!outNodeId || (numSubMeshes && !subMeshIds)) return ctx->fail(SLG_ERR_INVALID_ARG, "null argument");
    int r = check_transform(ctx, transform);
    if (r) return r;
    if (parentId != SLG_SCENE_ROOT && parentId >= sc->parents.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid parent node");
    const uint32_t depth = (parentId == SLG_SCENE_ROOT) ? 1u : sc->depth[parentId] + 1u;
    if (depth > (uint32_t)slg::kSceneMaxDepth) return ctx->fail(SLG_ERR_INVALID_ARG, "scene paths hold at most 64 nodes");
    if (sc->parents.size() >= 0xFFFFFFFFull) return ctx->fail(SLG_ERR_INVALID_ARG, "too many scene nodes");
    for (size_t k = 0; k < numSubMeshes; ++k)
        if (subMeshIds[k] >= sc->meshes.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid submesh id");
    sc->parents.push_back(parentId == SLG_SCENE_ROOT ? slg::kSceneRoot : (uint64_t)parentId);
    sc->depth.push_back(depth);
    sc->transforms.push_back(*transform);
    sc->dirty.push_back(1);
    sc->meshFirst.push_back(sc->nodeMeshes.size());
    sc->meshCount.push_back(numSubMeshes);
    sc->nodeMeshes.insert(sc->nodeMeshes.end(), subMeshIds, subMeshIds + numSubMeshes);
    if (numSubMeshes)
    {
        /* insert_mesh_node appends a default box to mMeshBounds (max 1, min -1) */
        const float b[8] = {1.f, 1.f, 1.f, 1.f, -1.f, -1.f, -1.f, 1.f};
        sc->bounds.insert(sc->bounds.end(), b, b + 8);
    }
    sc->listDirty = true;
    *outNodeId = sc->parents.size() - 1;
    return SLG_OK;
}

int slg_scene_set_transform(slg_context* ctx, size_t sceneId, size_t nodeId, const slg_transform* transform)
{
    Scene* sc = scene_of(ctx, sceneId);
    if (!sc) return ctx->fail(SLG_ERR_INVALID_ID, "invalid scene id");
    if (nodeId >= sc->parents.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid node id");
    int r = check_transform(ctx, transform);
    if (r) return r;
    sc->transforms[nodeId] = *transform;
    sc->dirty[nodeId] = 1;
    return SLG_OK;
}

int slg_scene_update(slg_context* ctx, size_t sceneId)
{
    Scene* sc = scene_of(ctx, sceneId);
    if (!sc) return ctx->fail(SLG_ERR_INVALID_ID, "invalid scene id");
    int r = scene_models(ctx, *sc);
    if (r) return r;
    const size_t n = sc->parents.size();
    /* SL_SceneGraph::update's loop (SL_SceneGraph.cpp:269-290): a dirty node
     * and every following node until one whose parent precedes it; a node
     * updated this way is clean when the loop reaches it */
    std::vector<slg::SceneNodeGpu> nodes(n);
    std::vector<uint32_t> list;
    auto mark = [&](size_t j) {
        if (!nodes[j].update) list.push_back((uint32_t)j);
        nodes[j].update = 1;
        sc->dirty[j] = 0;
    };
    for (size_t i = 0; i < n; ++i)
    {
        if (!sc->dirty[i]) continue;
        mark(i);
        for (size_t j = i + 1; j < n; ++j)
        {
            if (sc->parents[j] < i)
            {
                i = j - 1;
                break;
            }
            mark(j);
        }
    }
    if (list.empty()) return SLG_OK;
    for (size_t i = 0; i < n; ++i)
    {
        const slg_transform& t = sc->transforms[i];
        slg::SceneNodeGpu& g = nodes[i];
        g.parent = sc->parents[i];
        std::memcpy(g.position, t.position, sizeof(g.position));
        std::memcpy(g.scaling, t.scaling, sizeof(g.scaling));
        std::memcpy(g.orientation, t.orientation, sizeof(g.orientation));
        /* apply_transform flips the order for the FPS view types (SL_Transform.cpp:319-328) */
        g.viewFps = (t.type == 1 || t.type == 3) ? 1u : 0u;
    }
    if ((r = dev_alloc(ctx, sc->dNodes, n * sizeof(slg::SceneNodeGpu), false))) return r;
    if ((r = dev_alloc(ctx, sc->dList, list.size() * sizeof(uint32_t), false))) return r;
    cudaError_t e = cudaMemcpyAsync(sc->dNodes.ptr, nodes.data(), n * sizeof(slg::SceneNodeGpu), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(sc->dList.ptr, list.data(), list.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess)
        e = slg::launch_scene_update(static_cast<const slg::SceneNodeGpu*>(sc->dNodes.ptr), static_cast<const uint32_t*>(sc->dList.ptr),
                                     (uint32_t)list.size(), static_cast<float*>(sc->dModel.ptr), ctx->stream);
    /* the host vectors are released on return: the copies must have read them */
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "scene update");
    return SLG_OK;
}

int slg_scene_read_models(slg_context* ctx, size_t sceneId, float* out, size_t numNodes)
{
    Scene* sc = scene_of(ctx, sceneId);
    if (!sc) return ctx->fail(SLG_ERR_INVALID_ID, "invalid scene id");
    if (!out || numNodes != sc->parents.size()) return ctx->fail(SLG_ERR_INVALID_ARG, "node count");
    int r = scene_models(ctx, *sc);
    if (r) return r;
    if (!numNodes) return SLG_OK;
    cudaError_t e = cudaMemcpyAsync(out, sc->dModel.ptr, numNodes * 64, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "scene model read");
    return SLG_OK;
}

int slg_scene_draw(slg_context* ctx, size_t sceneId, size_t fboId, size_t shaderId, const float projection[16],
                   const float view[16], const float cullProjection[16])
{
    Scene* sc = scene_of(ctx, sceneId);
    if (!sc) return ctx->fail(SLG_ERR_INVALID_ID, "invalid scene id");
    if (!projection || !view) return ctx->fail(SLG_ERR_INVALID_ARG, "null matrix");
    if (!id_ok(shaderId, ctx->shaders.size())) return ctx->fail(SLG_ERR_INVALID_ID, "invalid shader id");
    /* a copy: building the draw list appends to ctx->shaders */
    const Shader sh = ctx->shaders[shaderId];
    if (sh.vsProgram != SLG_PROGRAM_LAMBERT_TEX || sh.fsProgram != SLG_PROGRAM_LAMBERT_TEX || sh.ubo == SLG_INVALID_ID)
        return ctx->fail(SLG_ERR_INVALID_ARG, "scene draws take a SLG_PROGRAM_LAMBERT_TEX shader with a uniform block");
    if (fboId >= ctx->fbos.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid fbo id");
    int r = scene_models(ctx, *sc);
    if (r) return r;
    if (sc->listDirty || sc->listShader != shaderId)
    {
        if ((r = scene_build_list(ctx, *sc, shaderId))) return r;
    }
    if (sc->entries.empty()) return SLG_OK;
    if (sc->boundsUploaded != sc->bounds.size())
    {
        if ((r = dev_alloc(ctx, sc->dBounds, sc->bounds.size() * sizeof(float), false))) return r;
        cudaError_t e = cudaMemcpyAsync(sc->dBounds.ptr, sc->bounds.data(), sc->bounds.size() * sizeof(float), cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return ctx->cuda_fail(e, "scene bounds upload");
        sc->boundsUploaded = sc->bounds.size();
    }
    slg::SceneDrawArgs a;
    std::memset(&a, 0, sizeof(a));
    a.entries = static_cast<const slg::SceneEntryGpu*>(sc->dEntries.ptr);
    a.numEntries = (uint32_t)sc->entries.size();
    a.cull = cullProjection ? 1 : 0;
    a.model = static_cast<const float*>(sc->dModel.ptr);
    a.bounds = static_cast<const float*>(sc->dBounds.ptr);
    mat4_mul(projection, view, a.vp);
    std::memcpy(a.view, view, sizeof(a.view));
    if (cullProjection) frustum_planes(cullProjection, a.planes);
    static_assert(sizeof(slg_lambert_uniforms) <= sizeof(a.templ), "template block");
    std::memcpy(a.templ, ctx->ubos[sh.ubo].shadow, sizeof(slg_lambert_uniforms));
    a.templWords = sizeof(slg_lambert_uniforms) / 4;
    std::vector<DrawRequest> reqs;
    reqs.reserve(sc->entries.size());
    for (const Scene::Entry& en : sc->entries)
    {
        DrawRequest q;
        q.mesh = sc->meshes[en.mesh];
        q.numInstances = 1;
        q.shaderId = en.shader;
        q.primBase = 0;
        reqs.push_back(q);
    }
    const LaunchHook hook = {scene_draw_hook, &a};
    return run_launch(ctx, reqs, fboId, false, &hook);
}

int slg_finish(slg_context* ctx)
{
    return settle(ctx);
}

void* slg_context_stream(slg_context* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int slg_set_tile_size(slg_context* ctx, int tileW, int tileH)
{
    const bool ok = (tileW == 8 && tileH == 8) || (tileW == 16 && tileH == 16) || (tileW == 32 && tileH == 16) ||
                    (tileW == 32 && tileH == 32) || (tileW == 64 && tileH == 32) || (tileW == 64 && tileH == 64);
    if (!ok) return ctx->fail(SLG_ERR_INVALID_ARG, "unsupported tile size");
    cudaStreamSynchronize(ctx->stream);
    ctx->tileW = tileW;
    ctx->tileH = tileH;
    return SLG_OK;
}

int slg_set_raster_mode(slg_context* ctx, int mode)
{
    if (mode < 0 || mode > 3) return ctx->fail(SLG_ERR_INVALID_ARG, "raster mode must be 0, 1, 2 or 3");
    ctx->forceOrdered = (mode == 1);
    ctx->forceTiled = (mode == 2);
    ctx->forceUntiled = (mode == 3);
    return SLG_OK;
}

int slg_untiled_raster(const slg_context* ctx)
{
    return (!ctx->forceTiled && (ctx->untiled || ctx->forceUntiled)) ? 1 : 0;
}

int slg_profile_stages(slg_context* ctx, int enable)
{
    ctx->profileStages = enable != 0;
    return SLG_OK;
}

int slg_stage_times(slg_context* ctx, float ms[4])
{
    cudaError_t e = cudaEventSynchronize(ctx->stageEvents[4]);
    for (int i = 0; i < 4 && e == cudaSuccess; ++i) e = cudaEventElapsedTime(&ms[i], ctx->stageEvents[i], ctx->stageEvents[i + 1]);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "stage timing");
    return SLG_OK;
}

} // extern "C"

/*-----------------------------------------------------------------------------
 * slg_draw_noalloc: slg_draw with its per-launch scratch in one fixed device
 * array that exists from the moment the library is loaded.
 *
 * slg_draw keeps its scratch (triangle records, varyings, tile lists) in
 * context buffers that grow with cudaMalloc when a draw needs more. Some
 * callers cannot let a draw allocate: a render loop running under a fixed
 * device-memory budget, a thread that must not meet cudaMalloc/cudaFree's
 * implicit device-wide synchronisation in the middle of a frame, or code
 * running under an allocator hook that forbids new allocations once set-up
 * is over. For them this variant sizes every scratch array for a stated
 * worst case, rejects larger draws up front, and never allocates.
-----------------------------------------------------------------------------*/
namespace
{

constexpr uint64_t kNoAllocTris = SLG_NOALLOC_MAX_TRIANGLES;
constexpr uint64_t kNoAllocTiles = SLG_NOALLOC_MAX_TILES;
/* a clipped triangle is replaced by at most 7 sub-triangles, which live in
 * the overflow region behind the per-triangle records */
constexpr uint64_t kNoAllocOvf = 7 * kNoAllocTris;
constexpr uint64_t kNoAllocRecords = kNoAllocTris + kNoAllocOvf;
/* every record lands in at most every tile: no tile list can overflow */
constexpr uint64_t kNoAllocEntries = kNoAllocOvf * kNoAllocTiles;
constexpr size_t kNoAllocTextures = 256, kNoAllocBuffers = 256;

constexpr size_t align256(size_t n) { return (n + 255) & ~size_t(255); }

/* layout of the static scratch; the first kNoAllocZeroBytes must be zero
 * when the pipeline starts: ovfCount (+0), clipCount (+4), aliasCount (+8)
 * and the per-tile triangle counters (+256). The status words are the
 * context's own (allocated when the context is created), so errors of a
 * no-allocation draw are reported at slg_finish like those of slg_draw. */
constexpr size_t kOffCounters = 0;
constexpr size_t kOffTileCount = 256;
constexpr size_t kNoAllocZeroBytes = kOffTileCount + align256(kNoAllocTiles * sizeof(uint32_t));
constexpr size_t kOffTileOffset = kNoAllocZeroBytes;
constexpr size_t kOffTileCursor = kOffTileOffset + align256((kNoAllocTiles + 1) * sizeof(uint32_t));
constexpr size_t kOffSlotInfo = kOffTileCursor + align256(kNoAllocTiles * sizeof(uint32_t));
constexpr size_t kOffSlotOvf = kOffSlotInfo + align256(kNoAllocTris * sizeof(uint32_t));
constexpr size_t kOffClipQueue = kOffSlotOvf + align256(kNoAllocTris * sizeof(uint32_t));
constexpr size_t kOffTexTable = kOffClipQueue + align256(kNoAllocTris * sizeof(uint32_t));
constexpr size_t kOffBufTable = kOffTexTable + align256(kNoAllocTextures * sizeof(TexView));
constexpr size_t kOffVaoTable = kOffBufTable + align256(kNoAllocBuffers * sizeof(void*));
constexpr size_t kOffRecords = kOffVaoTable + align256(kNoAllocBuffers * sizeof(slg::VaoView));
constexpr size_t kOffVaryings = kOffRecords + align256(kNoAllocRecords * slg::kRecordVec4 * sizeof(float4));
constexpr size_t kOffEntries = kOffVaryings + align256(kNoAllocRecords * slg::kVaryingVec4 * sizeof(float4));
constexpr uint32_t kNoAllocAliases = kAliasCap;   /* as slg_draw: 4096 full-width line aliases */
constexpr size_t kOffAliases = kOffEntries + align256(kNoAllocEntries * sizeof(uint32_t));
constexpr size_t kNoAllocBytes = kOffAliases + align256(kNoAllocAliases * sizeof(slg::AliasEvent));
static_assert(kNoAllocBytes < (8u << 20), "static draw scratch stays under 8 MiB");
static_assert(offsetof(slg_cutout_uniforms, textureId) == offsetof(slg_vcolor_uniforms, textureId), "cutout block extends the vertex-colour block");
static_assert(kNoAllocZeroBytes % 4 == 0, "counters are cleared in whole words");

static __device__ __align__(256) unsigned char g_noallocScratch[kNoAllocBytes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noallocMutex;
unsigned char* g_noallocPtr[kNoAllocMaxDevices] = {};

/* Device address of the static scratch on the current device, looked up
 * once per device (with that device current) and cached. */
int noalloc_scratch(slg_context* ctx, unsigned char** out)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= kNoAllocMaxDevices) return ctx->fail(SLG_ERR_INVALID_ARG, "slg_draw_noalloc: device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_noallocMutex);
    if (!g_noallocPtr[dev])
    {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noallocScratch);
        if (e != cudaSuccess) return ctx->cuda_fail(e, "cudaGetSymbolAddress(static draw scratch)");
        g_noallocPtr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_noallocPtr[dev];
    return SLG_OK;
}

} // namespace

extern "C" int slg_draw_noalloc(slg_context* ctx, const slg_mesh* m, size_t shaderId, size_t fboId)
{
    if (!m) return ctx->fail(SLG_ERR_INVALID_ARG, "null mesh");
    if (fboId >= ctx->fbos.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid fbo id");
    const Fbo& fbo = ctx->fbos[fboId];
    if (fbo.depth == SLG_INVALID_ID) return ctx->fail(SLG_ERR_INVALID_ARG, "framebuffer has no depth attachment");
    const Texture& depthTex = ctx->textures[fbo.depth];
    const Texture* colorTex = (fbo.numColors > 0 && fbo.colors[0] != SLG_INVALID_ID) ? &ctx->textures[fbo.colors[0]] : nullptr;
    if (colorTex && (colorTex->w != depthTex.w || colorTex->h != depthTex.h))
        return ctx->fail(SLG_ERR_INVALID_ARG, "colour and depth attachments differ in size");

    unsigned char* scratch = nullptr;
    int r = noalloc_scratch(ctx, &scratch);
    if (r) return r;

    /* the descriptor goes through the context's pinned ring, as for slg_draw */
    if (ctx->descHead + 2 > kDescRing)
    {
        cudaStreamSynchronize(ctx->stream);
        ctx->descHead = 0;
    }
    DrawDesc* desc = ctx->hostDescs + ctx->descHead;
    uint64_t* starts = ctx->hostStarts + ctx->descHead;
    uint64_t numSlots = 0;
    const DrawRequest req = {*m, 1, shaderId, 0};
    if ((r = build_desc(ctx, req, 0, *desc, numSlots))) return r;
    desc->cacheVerts = 0; /* the static scratch has no vertex cache */
    if (numSlots == 0) return SLG_OK;
    if (numSlots > kNoAllocTris)
        return ctx->fail(SLG_ERR_INVALID_ARG, "slg_draw_noalloc: " + std::to_string(numSlots) + " triangles exceed the static limit of " +
                                                  std::to_string(kNoAllocTris));

    Frame f;
    std::memset(&f, 0, sizeof(f));
    f.hasLines = (desc->prim == slg::kPrimLine) ? 1 : 0;
    f.hasWire = (desc->prim == slg::kPrimWire) ? 1 : 0;
    f.width = depthTex.w;
    f.height = depthTex.h;
    if ((r = bind_attachments(ctx, fbo, depthTex, desc, 1, f))) return r;
    f.tileW = (f.hasLines || f.hasWire || f.hasMrt) ? slg::kLineTile : ctx->tileW;
    f.tileH = (f.hasLines || f.hasWire || f.hasMrt) ? slg::kLineTile : ctx->tileH;
    f.tilesX = (f.width + f.tileW - 1) / f.tileW;
    f.tilesY = (f.height + f.tileH - 1) / f.tileH;
    const uint64_t numTiles = (uint64_t)f.tilesX * f.tilesY;
    if (numTiles > kNoAllocTiles)
        return ctx->fail(SLG_ERR_INVALID_ARG, "slg_draw_noalloc: a " + std::to_string(f.width) + "x" + std::to_string(f.height) +
                                                  " framebuffer is " + std::to_string(numTiles) + " tiles of " + std::to_string(f.tileW) + "x" +
                                                  std::to_string(f.tileH) + ", over the static limit of " + std::to_string(kNoAllocTiles));
    f.depthType = depthTex.type;
    const Shader& shader = ctx->shaders[shaderId];
    f.orderFree = (desc->blend == SLG_BLEND_OFF && desc->depthTest != SLG_DEPTH_TEST_NOT_EQUAL && !ctx->forceOrdered &&
                   f.depthType != SLG_COLOR_R_HALF && !(shader.fsFlags & (SLG_PROGRAM_DISCARDS | SLG_PROGRAM_WRITES_DEPTH))) ? 1 : 0;
    f.freeDepthFunc = desc->depthTest;
    f.freeDepthMask = desc->depthMask;
    if ((r = bind_visibility(ctx, fbo, f))) return r;
    if (desc->prim == slg::kPrimLine)
    {
        if (std::max(f.width, f.height) > kMaxLineExtent)
            return ctx->fail(SLG_ERR_INVALID_ARG, "line draws need a framebuffer of at most 10922 x 10922");
        f.aliasEvents = reinterpret_cast<slg::AliasEvent*>(scratch + kOffAliases);
        f.aliasCount = reinterpret_cast<uint32_t*>(scratch + kOffCounters + 8);
        f.aliasCap = kNoAllocAliases;
    }

    /* resource tables: the context's when they are current, else a copy of
     * them into the static scratch */
    const size_t numTex = ctx->textures.size(), numBuf = ctx->vbos.size();
    cudaError_t e = cudaSuccess;
    const size_t numVao = ctx->vaos.size();
    if (!ctx->tablesDirty && ctx->texTable.ptr && ctx->bufTable.ptr && ctx->vaoTable.ptr)
    {
        set_tables(ctx, f.tables, ctx->texTable.ptr, ctx->bufTable.ptr, ctx->vaoTable.ptr);
    }
    else
    {
        if (numTex > kNoAllocTextures || numBuf > kNoAllocBuffers || numVao > kNoAllocBuffers)
            return ctx->fail(SLG_ERR_INVALID_ARG,
                             "slg_draw_noalloc: more than 256 textures, vertex buffers or vertex arrays since the last slg_draw");
        TexView tex[kNoAllocTextures];
        const uint8_t* bufs[kNoAllocBuffers];
        static thread_local slg::VaoView vaoViews[kNoAllocBuffers];   /* 32 KB: off the stack */
        for (size_t i = 0; i < numTex; ++i)
        {
            const Texture& t = ctx->textures[i];
            tex[i].texels = static_cast<const uint8_t*>(t.buf.ptr);
            tex[i].w = t.w;
            tex[i].h = t.h;
            tex[i].d = t.d;
            tex[i].type = t.type;
        }
        for (size_t i = 0; i < numBuf; ++i) bufs[i] = static_cast<const uint8_t*>(ctx->vbos[i].buf.ptr);
        if (numTex) e = cudaMemcpyAsync(scratch + kOffTexTable, tex, numTex * sizeof(TexView), cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess && numBuf)
            e = cudaMemcpyAsync(scratch + kOffBufTable, bufs, numBuf * sizeof(void*), cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess && numVao)
        {
            fill_vao_views(ctx, vaoViews);
            e = cudaMemcpyAsync(scratch + kOffVaoTable, vaoViews, numVao * sizeof(slg::VaoView), cudaMemcpyHostToDevice, ctx->stream);
        }
        if (e != cudaSuccess) return ctx->cuda_fail(e, "slg_draw_noalloc: table upload");
        set_tables(ctx, f.tables, scratch + kOffTexTable, scratch + kOffBufTable, scratch + kOffVaoTable);
    }

    starts[0] = 0;
    starts[1] = numSlots;
    DrawDesc* devDesc = static_cast<DrawDesc*>(ctx->devDescs.ptr) + ctx->descHead;
    uint64_t* devStarts = static_cast<uint64_t*>(ctx->devStarts.ptr) + ctx->descHead;
    e = cudaMemcpyAsync(devDesc, desc, sizeof(DrawDesc), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(devStarts, starts, 2 * sizeof(uint64_t), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(scratch + kOffCounters, 0, kNoAllocZeroBytes, ctx->stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "slg_draw_noalloc: descriptor upload");
    ctx->descHead += 2;

    f.color = colorTex ? static_cast<uint8_t*>(colorTex->buf.ptr) : nullptr;
    f.colorType = colorTex ? colorTex->type : SLG_COLOR_RGBA_8U;
    if (f.generic0) f.color = nullptr;
    f.depth = static_cast<float*>(depthTex.buf.ptr);
    f.depthType = depthTex.type;
    viewport_setup((float)f.width, (float)f.height, f.scissor, f.viewport);
    f.records = reinterpret_cast<float4*>(scratch + kOffRecords);
    f.varyings = reinterpret_cast<float4*>(scratch + kOffVaryings);
    f.slotInfo = reinterpret_cast<uint32_t*>(scratch + kOffSlotInfo);
    f.slotOvf = reinterpret_cast<uint32_t*>(scratch + kOffSlotOvf);
    f.ovfCount = reinterpret_cast<uint32_t*>(scratch + kOffCounters);
    f.clipCount = reinterpret_cast<uint32_t*>(scratch + kOffCounters + 4);
    f.status = static_cast<int32_t*>(ctx->status.ptr);
    f.clipQueue = reinterpret_cast<uint32_t*>(scratch + kOffClipQueue);
    f.ovfCap = (uint32_t)kNoAllocOvf;
    f.numSlots = numSlots;
    f.tileCount = reinterpret_cast<uint32_t*>(scratch + kOffTileCount);
    f.tileOffset = reinterpret_cast<uint32_t*>(scratch + kOffTileOffset);
    f.tileCursor = reinterpret_cast<uint32_t*>(scratch + kOffTileCursor);
    f.entries = reinterpret_cast<uint32_t*>(scratch + kOffEntries);
    f.entryCap = (uint32_t)kNoAllocEntries;
    f.draws = devDesc;
    f.drawSlotStart = devStarts;
    f.numDraws = 1;
    f.vsBlock = ctx->vsBlock;

    if (flush_ubos(ctx, false)) return SLG_ERR_CUDA;
    {
        LogOp op;
        op.kind = LogOp::kNoalloc;
        op.mesh = *m;
        op.shader = shaderId;
        op.fbo = fboId;
        log_op(ctx, std::move(op));
    }
    /* the static scratch bounds a tile list by kNoAllocEntries / tiles; the
     * shared-memory sort holds that many whatever the context's cap */
    e = slg::launch_pipeline(f, pipeline_ops(ctx, shader.programSet), std::max(ctx->keyCap, (int)kNoAllocRecords), ctx->stream, nullptr);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "slg_draw_noalloc: launch");
    return SLG_OK;
}

/*-----------------------------------------------------------------------------
 * Differentiable rendering (no reference counterpart; the reference has no
 * adjoint). An opaque draw into a framebuffer with a visibility map records,
 * per pixel, which triangle won the depth test; given that map,
 * slg_diff_shade evaluates the differentiable shading model of the
 * vertex-colour x float-texture program and slg_draw_adjoint its gradients
 * (model and layout: softlight_gb300/csrc/slg_adjoint.cu).
-----------------------------------------------------------------------------*/
namespace
{

bool device_visible(const void* p)
{
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, p) != cudaSuccess)
    {
        cudaGetLastError();
        return false;
    }
    return attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged || attr.type == cudaMemoryTypeHost;
}

int diff_args(slg_context* ctx, const slg_mesh* m, size_t shaderId, size_t fboId, slg::DiffArgs& a, uint64_t& vertexBytes)
{
    if (!m) return ctx->fail(SLG_ERR_INVALID_ARG, "null mesh");
    if (fboId >= ctx->fbos.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid fbo id");
    const Fbo& fbo = ctx->fbos[fboId];
    if (!fbo.visEnabled || fbo.depth == SLG_INVALID_ID)
        return ctx->fail(SLG_ERR_INVALID_ARG, "framebuffer has no visibility map (slg_fbo_enable_visibility)");
    const Texture& depthTex = ctx->textures[fbo.depth];
    if (fbo.vis.bytes < (size_t)depthTex.w * depthTex.h * sizeof(uint32_t))
        return ctx->fail(SLG_ERR_INVALID_ARG, "visibility map is smaller than the framebuffer");

    const DrawRequest req = {*m, 1, shaderId, 0};
    DrawDesc d;
    uint64_t numSlots = 0;
    int r = build_desc(ctx, req, 0, d, numSlots);
    if (r) return r;
    const Shader& sh = ctx->shaders[shaderId];
    if (d.prim != slg::kPrimTriangle) return ctx->fail(SLG_ERR_INVALID_ARG, "the differentiable model covers triangle draws only");
    if (sh.vsProgram != SLG_PROGRAM_VCOLOR_TEXF || sh.fsProgram != SLG_PROGRAM_VCOLOR_TEXF)
        return ctx->fail(SLG_ERR_INVALID_ARG, "the differentiable model covers SLG_PROGRAM_VCOLOR_TEXF draws only");
    if ((d.b0Offset & 3) || (d.b0Stride & 3)) return ctx->fail(SLG_ERR_INVALID_ARG, "binding 0 offset and stride must be multiples of 4 bytes");
    if (d.numElements / 3 > 0xFFFFFFFEull) return ctx->fail(SLG_ERR_INVALID_ARG, "too many triangles");
    uint32_t texId = 0;
    std::memcpy(&texId, ctx->ubos[sh.ubo].shadow + offsetof(slg_vcolor_uniforms, textureId), 4);
    const Texture& tex = ctx->textures[texId];   /* validated by build_desc */

    const Vao& vao = ctx->vaos[m->vaoId];
    const uint64_t maxVertex = (d.indexType >= 0) ? ctx->ibos[vao.ibo].maxIndex : (d.elementBegin + 3 * d.numTris - 1);
    vertexBytes = (uint64_t)d.b0Offset + (uint64_t)d.b0Stride * maxVertex + 9 * sizeof(float);

    std::memset(&a, 0, sizeof(a));
    a.vbo = d.vbo;
    a.b0Offset = d.b0Offset;
    a.b0Stride = d.b0Stride;
    a.ibo = d.ibo;
    a.indexType = d.indexType;
    a.elementBegin = d.elementBegin;
    a.numTris = (uint32_t)(d.numElements / 3);
    a.mvp = reinterpret_cast<const float*>(d.ubo + offsetof(slg_vcolor_uniforms, mvpMatrix));
    a.texels = static_cast<const float4*>(tex.buf.ptr);
    a.texW = tex.w;
    a.texH = tex.h;
    a.vis = static_cast<const uint32_t*>(fbo.vis.ptr);
    if (fbo.numColors > 0 && fbo.colors[0] != SLG_INVALID_ID && ctx->textures[fbo.colors[0]].type == SLG_COLOR_RGBA_FLOAT &&
        ctx->textures[fbo.colors[0]].w == depthTex.w && ctx->textures[fbo.colors[0]].h == depthTex.h)
        a.exact = static_cast<const float4*>(ctx->textures[fbo.colors[0]].buf.ptr);
    a.width = depthTex.w;
    a.height = depthTex.h;
    return SLG_OK;
}

} // namespace

extern "C" {

int slg_fbo_enable_visibility(slg_context* ctx, size_t fboId, int enable)
{
    if (fboId >= ctx->fbos.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid fbo id");
    Fbo& fbo = ctx->fbos[fboId];
    if (!enable)
    {
        cudaStreamSynchronize(ctx->stream);
        dev_free(fbo.vis);
        fbo.visEnabled = false;
        return SLG_OK;
    }
    if (fbo.depth == SLG_INVALID_ID) return ctx->fail(SLG_ERR_INVALID_ARG, "a visibility map needs a depth attachment");
    const Texture& d = ctx->textures[fbo.depth];
    int r = dev_alloc(ctx, fbo.vis, (size_t)d.w * d.h * sizeof(uint32_t), true);
    if (r) return r;
    fbo.visEnabled = true;
    return SLG_OK;
}

int slg_fbo_read_visibility(slg_context* ctx, size_t fboId, uint32_t* dst, size_t count)
{
    if (fboId >= ctx->fbos.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid fbo id");
    const Fbo& fbo = ctx->fbos[fboId];
    if (!fbo.visEnabled) return ctx->fail(SLG_ERR_INVALID_ARG, "framebuffer has no visibility map");
    if (!dst || count * sizeof(uint32_t) > fbo.vis.bytes) return ctx->fail(SLG_ERR_INVALID_ARG, "bad destination size");
    const int r = settle(ctx);
    cudaError_t e = cudaMemcpyAsync(dst, fbo.vis.ptr, count * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "visibility read");
    return r;
}

int slg_diff_shade(slg_context* ctx, const slg_mesh* m, size_t shaderId, size_t fboId, float* image, size_t count)
{
    slg::DiffArgs a;
    uint64_t vertexBytes = 0;
    int r = diff_args(ctx, m, shaderId, fboId, a, vertexBytes);
    if (r) return r;
    if (!image || ((uintptr_t)image & 15) || count < (size_t)a.width * a.height * 4 || !device_visible(image))
        return ctx->fail(SLG_ERR_INVALID_ARG, "image must be a 16-byte aligned device buffer of width*height*4 floats");
    a.image = reinterpret_cast<float4*>(image);
    if ((r = flush_ubos(ctx, true))) return r;
    cudaError_t e = slg::launch_diff_shade(a, ctx->stream);
    return (e == cudaSuccess) ? SLG_OK : ctx->cuda_fail(e, "diff shade launch");
}

int slg_draw_adjoint(slg_context* ctx, const slg_mesh* m, size_t shaderId, size_t fboId, const float* dImage, size_t dImageCount,
                     float* dVertices, size_t dVertexCount, float* dTexels, size_t dTexelCount)
{
    slg::DiffArgs a;
    uint64_t vertexBytes = 0;
    int r = diff_args(ctx, m, shaderId, fboId, a, vertexBytes);
    if (r) return r;
    if (!dImage || ((uintptr_t)dImage & 15) || dImageCount < (size_t)a.width * a.height * 4 || !device_visible(dImage))
        return ctx->fail(SLG_ERR_INVALID_ARG, "dImage must be a 16-byte aligned device buffer of width*height*4 floats");
    if (!dVertices || ((uintptr_t)dVertices & 3) || (uint64_t)dVertexCount * sizeof(float) < vertexBytes || !device_visible(dVertices))
        return ctx->fail(SLG_ERR_INVALID_ARG, "dVertices must be a device buffer covering the draw's vertices in the vertex buffer's layout");
    if (!dTexels || ((uintptr_t)dTexels & 15) || dTexelCount < (size_t)a.texW * a.texH * 4 || !device_visible(dTexels))
        return ctx->fail(SLG_ERR_INVALID_ARG, "dTexels must be a 16-byte aligned device buffer of texW*texH*4 floats");
    a.dImage = reinterpret_cast<const float4*>(dImage);
    a.dVertices = dVertices;
    a.dTexels = reinterpret_cast<float4*>(dTexels);
    if ((r = flush_ubos(ctx, true))) return r;
    cudaError_t e = slg::launch_diff_adjoint(a, ctx->stream);
    return (e == cudaSuccess) ? SLG_OK : ctx->cuda_fail(e, "adjoint launch");
}

} // extern "C"

/*-----------------------------------------------------------------------------
 * Completion and overflow recovery. Scratch buffers are sized from what
 * earlier launches needed; a launch that needs more than a buffer holds
 * sets a capacity bit in the status words, writes nothing, and every later
 * framebuffer write on the stream is skipped while the bit is set. At the
 * next synchronisation point the host grows the buffer and replays the
 * recorded operations from the launch that overflowed: the draws come out
 * as if the buffer had been large enough from the start.
-----------------------------------------------------------------------------*/
namespace
{

/* Grows the buffers whose capacity bits are set in `bits`. */
int grow_for(slg_context* ctx, int32_t bits, const int32_t* status)
{
    int r;
    if (bits & slg::kStatusEntryOverflow)
    {
        const uint64_t want = std::max<uint64_t>((uint64_t)(uint32_t)status[1] + ((uint64_t)(uint32_t)status[1] >> 1), ctx->entryCap + 1);
        if ((r = dev_alloc(ctx, ctx->entries, want * sizeof(uint32_t), false))) return r;
        ctx->entryCap = want;
    }
    if (bits & slg::kStatusOvfOverflow)
    {
        ctx->ovfWant = std::max<uint64_t>((uint64_t)(uint32_t)status[2] + ((uint64_t)(uint32_t)status[2] >> 1), ctx->ovfCap + 1);
    }
    if (bits & slg::kStatusTileOverflow)
    {
        ctx->sortFallback = true;
    }
    if (bits & slg::kStatusAliasOverflow)
    {
        ctx->aliasCap *= 4;
    }
    if (ctx->sortFallback && ctx->sortScratch.bytes < 2 * ctx->entryCap * sizeof(uint32_t))
    {
        if ((r = dev_alloc(ctx, ctx->sortScratch, 2 * ctx->entryCap * sizeof(uint32_t), false))) return r;
    }
    if (ctx->aliasEvents.ptr && ctx->aliasEvents.bytes < ctx->aliasCap * sizeof(slg::AliasEvent))
    {
        if ((r = dev_alloc(ctx, ctx->aliasEvents, ctx->aliasCap * sizeof(slg::AliasEvent), false))) return r;
    }
    return SLG_OK;
}

int replay(slg_context* ctx, const LogOp& op)
{
    switch (op.kind)
    {
        case LogOp::kLaunch:     return run_launch(ctx, op.reqs, op.fbo, op.batch, nullptr, op.multiple);
        case LogOp::kNoalloc:    return slg_draw_noalloc(ctx, &op.mesh, op.shader, op.fbo);
        case LogOp::kClearColor: return slg_clear_color_buffer(ctx, op.fbo, op.attachment, op.value);
        case LogOp::kClearDepth: return slg_clear_depth_buffer(ctx, op.fbo, op.value[0]);
        case LogOp::kBlit:
            return slg_blit_rect(ctx, op.out, op.in, op.rect[0], op.rect[1], op.rect[2], op.rect[3], op.rect[4], op.rect[5], op.rect[6],
                                 op.rect[7]);
        case LogOp::kUbo:        return slg_ubo_assign(ctx, op.ubo, op.after.data(), op.after.size());
        default:                 return ctx->fail(SLG_ERR_INVALID_ARG, "operation cannot be replayed");
    }
}

} // namespace

namespace
{

int settle(slg_context* ctx)
{
    int32_t* hs = ctx->hostStatus;
    for (int attempt = 0;; ++attempt)
    {
        cudaError_t e = cudaMemcpyAsync(hs, ctx->status.ptr, 4 * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return ctx->cuda_fail(e, "device status read");
        const int32_t bits = hs[0];
        if (!(bits & slg::kStatusSticky)) break;

        /* the launch that overflowed: the first not counted as done */
        const uint32_t done = (uint32_t)hs[3];
        size_t pos = ctx->log.size(), launches = 0;
        bool opaque = false;
        for (size_t i = 0; i < ctx->log.size(); ++i)
        {
            const LogOp::Kind k = ctx->log[i].kind;
            if (k == LogOp::kLaunch || k == LogOp::kNoalloc || k == LogOp::kOpaque)
            {
                if (launches == done && pos == ctx->log.size()) pos = i;
                ++launches;
            }
            if (pos != ctx->log.size() && k == LogOp::kOpaque) opaque = true;
        }
        int r = grow_for(ctx, bits, hs);
        std::vector<LogOp> ops;
        if (pos < ctx->log.size()) ops.assign(std::make_move_iterator(ctx->log.begin() + pos), std::make_move_iterator(ctx->log.end()));
        ctx->log.clear();
        e = cudaMemsetAsync(ctx->status.ptr, 0, 4 * sizeof(int32_t), ctx->stream);
        if (e != cudaSuccess) return ctx->cuda_fail(e, "device status reset");
        if (r) return r;
        if (opaque || ops.empty() || attempt == 3 || ctx->replaying)
        {
            std::string msg = "device-side status:";
            if (bits & slg::kStatusEntryOverflow) msg += " tile entries";
            if (bits & slg::kStatusOvfOverflow) msg += " clipped-triangle records";
            if (bits & slg::kStatusTileOverflow) msg += " triangles per tile";
            if (bits & slg::kStatusAliasOverflow) msg += " full-width line aliases";
            msg += opaque ? " (a scene-graph draw list cannot be replayed: the draws from the overflow on were skipped; buffers have been grown)"
                          : " (the draws from the overflow on were skipped; buffers have been grown)";
            return ctx->fail(SLG_ERR_OVERFLOW, msg);
        }
        /* undo the uniform blocks written after the overflow, then replay */
        for (size_t i = ops.size(); i--;)
        {
            if (ops[i].kind != LogOp::kUbo) continue;
            Ubo& u = ctx->ubos[ops[i].ubo];
            std::memcpy(u.shadow, ops[i].before.data(), ops[i].before.size());
            if (!u.pending) ctx->uboPending.push_back(ops[i].ubo);
            u.pending = std::max<uint32_t>(u.pending, (uint32_t)ops[i].before.size());
        }
        ctx->replaying = true;
        for (const LogOp& op : ops)
        {
            if ((r = replay(ctx, op))) break;
        }
        ctx->replaying = false;
        if (r) return r;
    }
    const int32_t bits = hs[0];
    ctx->log.clear();
    if (bits || hs[3])
    {
        cudaError_t e = cudaMemsetAsync(ctx->status.ptr, 0, 4 * sizeof(int32_t), ctx->stream);
        if (e != cudaSuccess) return ctx->cuda_fail(e, "device status reset");
    }
    if (bits & slg::kStatusUndeclaredDiscard)
    {
        return ctx->fail(SLG_ERR_INVALID_ARG, "device-side status: a fragment program discarded a fragment in a launch that took the "
                                              "order-free raster; register programs that return false with SLG_PROGRAM_DISCARDS "
                                              "(the affected pixels keep the wrong colour)");
    }
    if (bits & (slg::kStatusWireQueue | slg::kStatusAliasKeys))
    {
        std::string msg = "device-side status:";
        if (bits & slg::kStatusWireQueue)
            msg += " blended wireframe triangle revisiting a pixel after 600 queued fragments (queue flush order not reproduced)";
        if (bits & slg::kStatusAliasKeys) msg += " more than 4096 records cover a full-width line's shared pixel (not replayed)";
        return ctx->fail(SLG_ERR_OVERFLOW, msg);
    }
    return SLG_OK;
}

} // namespace

extern "C" int slg_set_scratch_caps(slg_context* ctx, size_t maxEntries, size_t maxClipRecords, unsigned maxSortKeys)
{
    const int settled = settle(ctx);
    if (settled) return settled;
    if (maxEntries)
    {
        const int r = dev_alloc(ctx, ctx->entries, maxEntries * sizeof(uint32_t), false);
        if (r) return r;
        ctx->entryCap = maxEntries;
    }
    if (maxClipRecords) ctx->ovfCap = std::min<uint64_t>(ctx->ovfCap, maxClipRecords);
    if (maxSortKeys)
    {
        ctx->keyCap = (int)std::max(2u, std::min(maxSortKeys, 32768u));
        ctx->sortKeysCapped = true;
    }
    return SLG_OK;
}
