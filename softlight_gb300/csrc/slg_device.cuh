/*
 * slg_device.cuh - device-side data layout and exact arithmetic helpers.
 *
 * All floating-point code in this library is compiled with --fmad=false,
 * -prec-div=true, -prec-sqrt=true and no flush-to-zero, so every expression
 * below is a sequence of separately rounded binary32 operations in the
 * written order. That is what makes coverage, depth and colour bit-identical
 * to SoftLight's portable CPU path (the vector-library conventions are listed
 * at the top of slg_kernels.cu).
 */
#ifndef SLG_DEVICE_CUH
#define SLG_DEVICE_CUH

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/slg.h"
#include "../../include/slg_half.h"
#include "../../include/slg_programs.h"

namespace slg
{

/*-----------------------------------------------------------------------------
 * Sizes
-----------------------------------------------------------------------------*/
constexpr int kMaxVaryings = 4;         /* SL_SHADER_MAX_VARYING_VECTORS (SL_Config.hpp:40) */
constexpr int kRecordVec4 = 8;          /* raster record: 8 x float4 = 128 bytes */
constexpr int kVaryingVec4 = 12;        /* 3 vertices x 4 varyings */
constexpr int kSubShift = 3;            /* key = slot << 3 | sub-triangle */

/*-----------------------------------------------------------------------------
 * Exact scalar helpers
-----------------------------------------------------------------------------*/
/* float -> int32 with x86 cvttss2si semantics: NaN or out of range gives
 * INT32_MIN. */
__device__ __forceinline__ int32_t f2i(float f)
{
    return (f >= -2147483648.f && f < 2147483648.f) ? __float2int_rz(f) : (int32_t)0x80000000;
}

__device__ __forceinline__ uint8_t f2u8(float f) { return (uint8_t)(uint32_t)f2i(f); }

__device__ __forceinline__ float lm_max(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float lm_min(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ int sign_mask(float f) { return (int)(__float_as_uint(f) >> 31); }

/*-----------------------------------------------------------------------------
 * Resource views
-----------------------------------------------------------------------------*/
struct TexView
{
    const uint8_t* texels; /* dense w*h*d texels followed by zero padding */
    uint32_t w, h, d;
    int32_t type;          /* slg_color_type */
};

/* SL_VertexArray's bindings (softlight/include/softlight/SL_VertexArray.hpp:
 * 20-34, 109-126): per binding the byte offset of vertex 0 and the stride. */
struct VaoView
{
    int64_t offset[8];
    int64_t stride[8];
};

struct Tables
{
    const TexView* textures;
    const uint8_t* const* buffers; /* vertex buffer base pointers by id */
    const VaoView* vaos;           /* vertex array bindings by id */
    uint32_t numTextures, numBuffers, numVaos;
};

/* One draw: what SL_ProcessorPool::run_shader_processors hands to
 * SL_TriProcessor (softlight/src/SL_ProcessorPool.cpp:280-327). */
struct DrawDesc
{
    const uint8_t* vbo;
    const uint8_t* ibo;
    const uint8_t* ubo;
    int64_t  b0Offset;
    int64_t  b0Stride;
    uint64_t elementBegin;
    uint64_t numElements;   /* elementEnd - elementBegin */
    uint64_t numTris;       /* primitives per instance: ceil(numElements / 3) triangles, or numElements points */
    uint64_t numInstances;
    uint64_t slotBase;      /* first slot of this draw in the launch */
    uint64_t primBase;      /* primIndex offset (draw_multiple keeps per-mesh primIndex) */
    uint64_t cacheBase;     /* first vertex-cache entry of the draw (non-decreasing over the launch's draws) */
    uint64_t cacheVerts;    /* cached vertices per instance (the index buffer's max index + 1); 0: not cached */
    int32_t  indexType;     /* -1: non-indexed */
    uint32_t vsProgram;
    uint32_t fsProgram;
    uint32_t vaoId;         /* the mesh's vertex array (Tables::vaos) */
    uint8_t  cull, numVaryings, depthTest, depthMask, blend, numOutputs, prim;
    uint8_t  hidden;        /* 1: culled as a whole by the scene-graph producer (set on the device) */
};

/* DrawDesc::prim */
enum PrimKind
{
    kPrimTriangle = 0,
    kPrimPoint = 1,
    kPrimLine = 2,
    kPrimWire = 3     /* triangles drawn as wireframe */
};

/* record r7.w: depth test | depth mask << 4 | one of these bits for a point,
 * a line or a wireframe triangle record (none for a filled triangle) */
constexpr uint32_t kRecordPoint = 1u << 5;
constexpr uint32_t kRecordLine = 1u << 6;
constexpr uint32_t kRecordWire = 1u << 7;
/* the record's varyings are the vertex cache's: Frame::recVerts holds the
 * slot's three cache entries (x, y, z) instead of copies */
constexpr uint32_t kRecordCached = 1u << 8;

/* Per-launch scratch and framebuffer description. */
/* Screen tile of launches that contain line or wireframe draws or write
 * several render targets: the raster kernels that carry those are compiled
 * for this tile size only. */
constexpr int kLineTile = 32;

/* A line whose last walk step (x = W on row y - 1) is stored at the address
 * of its first step (x = 0 on row y). SoftLight depth-tests line fragments
 * when it queues them and writes them when its 600-fragment queue is
 * flushed, so when fewer than 600 of the line's fragments were queued before
 * the last step, both steps are tested against the depth before the line.
 * The vertex stage logs such lines (depth mask on, depth test on); the
 * ordered raster counts `queued`; alias_fixup_kernel replays the pixel. */
struct AliasEvent
{
    uint32_t slot;      /* the line's record */
    uint32_t pixel;     /* linear index of the shared pixel (column 0) */
    uint32_t queued;    /* steps 0 < k < dx that passed the depth test */
    float    depth0;    /* the pixel's depth before the launch */
    uint8_t  colors[4][32]; /* the pixel's texel bytes before the launch, attachments 0..3 */
};

struct Frame
{
    /* framebuffer */
    uint8_t* color;         /* attachment 0, or null */
    float*   depth;         /* texels of depthType: R_HALF, R_FLOAT or R_DOUBLE */
    int32_t  depthType;
    int32_t  colorType;
    int32_t  width, height;
    int32_t  tileW, tileH, tilesX, tilesY;
    float    scissor[16];
    float    viewport[4];

    /* scratch */
    float4*   records;      /* (numSlots + ovfCap) x kRecordVec4 */
    float4*   varyings;     /* (numSlots + ovfCap) x kVaryingVec4 */
    uint32_t* slotInfo;     /* per slot: 0 none, 1 main record, 2+n: n clipped sub-records */
    uint32_t* slotOvf;      /* per slot: first overflow record (relative) */
    uint32_t* ovfCount;
    uint32_t  ovfCap;
    uint32_t* clipQueue;    /* slots of partially visible triangles (capacity numSlots) */
    uint32_t* clipCount;
    uint64_t  numSlots;
    uint32_t* tileCount;    /* numTiles, zero between launches */
    uint32_t* tileOffset;   /* numTiles + 1 */
    uint32_t* tileCursor;   /* numTiles */
    uint32_t* entries;      /* keys, grouped by tile */
    uint32_t  entryCap;
    int32_t*  status;       /* [0] error bits, [1] entries needed, [2] overflow records needed */

    const DrawDesc* draws;
    const uint64_t* drawSlotStart; /* numDraws + 1 */
    int32_t numDraws;
    Tables tables;

    /* raster mode of the launch: order-free when no draw blends and all
     * draws share one order-independent depth rule */
    int32_t orderFree;
    int32_t freeDepthFunc;
    int32_t freeDepthMask;

    /* threads per block of the vertex stage (64, 128 or 256): triangles per CTA */
    int32_t vsBlock;

    /* some draw of the launch is a line draw: the vertex stage variant with
     * the line set-up runs (kept apart from the triangle variant's registers) */
    int32_t hasLines;

    /* some draw of the launch is a wireframe draw (SL_RENDER_MODE_TRI_WIRE) */
    int32_t hasWire;

    /* post-transform vertex cache of indexed draws that reuse vertices: per
     * entry e = cacheBase + instance * cacheVerts + vertex the program's
     * position cachePos[e] and varying vi at cacheVary[vi * cacheEntries + e]
     * (one plane per varying); cacheEntries 0: unused */
    float4*  cachePos;
    float4*  cacheVary;
    uint64_t cacheEntries;
    uint4*   recVerts;      /* per slot: the cache entries of a kRecordCached record */
    int32_t  allCached;     /* every draw with slots is a cached triangle draw */

    /* colour attachments 0..numColors-1 (colors[0] == color); hasMrt: some
     * draw writes more than one of them (outputs k -> attachment k) */
    uint8_t* colors[4];
    int32_t  colorTypes[4];
    int32_t  numColors;
    int32_t  hasMrt;
    /* attachment 0 has a format other than RGBA8, RGBA float or R float: it
     * is written like attachments 1..3 (general raster, global memory) and
     * `color` is null */
    int32_t  generic0;

    /* line address aliases (AliasEvent); null without line draws. Order-free
     * launches take the ordered raster when any alias was logged. */
    AliasEvent* aliasEvents;
    uint32_t*   aliasCount;
    uint32_t    aliasCap;

    /* optional visibility map (order-free raster only): per pixel written,
     * 1 + the launch slot (triangle) of the winning fragment; null: off */
    uint32_t* ids;

    /* blend order of a multi-mesh draw (flush_sort_kernel): when recOfRank
     * is set, tile-list keys are ranks in the reference's rasterisation
     * order and recOfRank maps a rank to its record; null otherwise */
    uint32_t* rankOf;             /* per record: its rank */
    uint32_t* recOfRank;          /* per rank: the record */
    uint32_t* seqRec;             /* per bin in push order: the record */
    unsigned long long* seqKey;   /* per bin in push order: primIndex */
    uint32_t* binBlocks;          /* per 1024 slots: bins, then their exclusive scan; [numBlocks] = all bins */
    uint32_t  rankGrid;           /* CTAs of flush_sort_kernel */

    /* tile lists filled in key order (bin_count_ordered_kernel ..
     * bin_fill_ordered_kernel): the bins in key order are cut into binChunks
     * chunks, one warp each; chunkCounts (chunk-major, binChunks x
     * numTiles) holds each chunk's entries per tile, then their exclusive
     * scan over the chunks (the chunk's first position in each tile's list).
     * null: the lists are filled by atomics and sorted per tile when the
     * ordered raster needs them. */
    uint32_t* chunkCounts;
    uint32_t  binChunks;
    uint32_t* itemKey;            /* per bin in push order: its tile-list key (launches without recOfRank) */
    /* the order in which the ordered raster's CTAs take the tiles (longest
     * tile list first; written by tile_scan_kernel), for launches with
     * lists in key order; null: CTA i takes tile i */
    uint32_t* tileOrder;

    /* untiled order-free raster (raster_global_kernel): per pixel the best
     * word of raster_free_kernel in global memory, and per overflow record
     * (clipped fan) its key; null: the tiled rasters run */
    unsigned long long* bestWords;
    uint32_t* ovfKey;

    /* the ordered raster's depth bound (depth_range_rect): 1 when every
     * draw uses LESS / LESS_EQUAL, 2 when every draw uses GREATER /
     * GREATER_EQUAL, and no fragment program writes depth (the depth of a
     * pixel then only moves one way); 0 otherwise */
    int32_t depthBound;

    /* global-memory sort of tile lists longer than the shared-memory sort
     * holds: two words per tile entry (the list padded to a power of two at
     * twice its offset); null until a launch needed it */
    uint32_t* sortScratch;
};

enum StatusBits
{
    kStatusEntryOverflow = 1,
    kStatusOvfOverflow = 2,
    kStatusTileOverflow = 4,
    kStatusAliasOverflow = 8,
    kStatusWireQueue = 16,
    kStatusUndeclaredDiscard = 32,  /* a program discarded in an order-free launch */
    kStatusAliasKeys = 64           /* more records than the line-alias replay holds cover one pixel */
};

/* Capacity overflows. Once one is set, every later kernel that writes a
 * framebuffer skips its work until the host has read the status (at a
 * synchronisation point), grown the buffer and replayed the launches from
 * the first that overflowed. status[3] counts the launches that finished
 * before the first overflow. */
constexpr int32_t kStatusSticky = kStatusEntryOverflow | kStatusOvfOverflow | kStatusTileOverflow | kStatusAliasOverflow;

/*-----------------------------------------------------------------------------
 * Texture sampling: sl_sample_bilinear<color, SL_WrapMode::REPEAT, ORDERED>
 * (softlight/include/softlight/SL_Sampler.hpp:97-115,187-218)
-----------------------------------------------------------------------------*/
/* (uvw < 0 ? 1 : 0) + fmod(uvw, 1). uvw - trunc(uvw) is computed exactly
 * (Sterbenz for |uvw| >= 1, trunc = 0 below), so this form gives the same
 * binary32 result as the fmod form for every input (all 2^32 values
 * compared on the host), without the cost of a general fmodf. */
__device__ __forceinline__ float wrap_repeat(float uvw)
{
    return (uvw < 0.f ? 1.f : 0.f) + (uvw - truncf(uvw));
}

struct Bilinear
{
    uint32_t i00, i01, i10, i11;
    float omdx, omdy, dx, dy;
};

__device__ __forceinline__ Bilinear bilinear_coords(const TexView& t, float x, float y)
{
    const float xf = wrap_repeat(x) * (float)t.w;
    const float yf = wrap_repeat(y) * (float)t.h;
    const uint32_t xi0 = (uint32_t)f2i(xf) & 0xFFFFu;
    const uint32_t yi0 = (uint32_t)f2i(yf) & 0xFFFFu;
    const uint32_t xn = (xi0 + 1u) & 0xFFFFu;
    const uint32_t yn = (yi0 + 1u) & 0xFFFFu;
    const uint32_t xi1 = (t.w < xn) ? t.w : xn;
    const uint32_t yi1 = (t.h < yn) ? t.h : yn;
    Bilinear c;
    c.dx = xf - (float)xi0;
    c.dy = yf - (float)yi0;
    c.omdx = 1.f - c.dx;
    c.omdy = 1.f - c.dy;
    c.i00 = xi0 + t.w * yi0;
    c.i01 = xi0 + t.w * yi1;
    c.i10 = xi1 + t.w * yi0;
    c.i11 = xi1 + t.w * yi1;
    return c;
}

__device__ __forceinline__ float4 unpack_rgba8(uint32_t p)
{
    /* color_cast<float, uint8_t> (softlight/include/softlight/SL_Color.hpp:674) */
    return make_float4((float)(p & 0xFFu) * 0.00392156862745f, (float)((p >> 8) & 0xFFu) * 0.00392156862745f,
                       (float)((p >> 16) & 0xFFu) * 0.00392156862745f, (float)(p >> 24) * 0.00392156862745f);
}

__device__ __forceinline__ float4 bilinear_sum(const float4 p0, const float4 p1, const float4 p2, const float4 p3, const Bilinear& c)
{
    float4 r;
    r.x = (((p0.x * c.omdx) * c.omdy + (p1.x * c.omdx) * c.dy) + (p2.x * c.dx) * c.omdy) + (p3.x * c.dx) * c.dy;
    r.y = (((p0.y * c.omdx) * c.omdy + (p1.y * c.omdx) * c.dy) + (p2.y * c.dx) * c.omdy) + (p3.y * c.dx) * c.dy;
    r.z = (((p0.z * c.omdx) * c.omdy + (p1.z * c.omdx) * c.dy) + (p2.z * c.dx) * c.omdy) + (p3.z * c.dx) * c.dy;
    r.w = (((p0.w * c.omdx) * c.omdy + (p1.w * c.omdx) * c.dy) + (p2.w * c.dx) * c.omdy) + (p3.w * c.dx) * c.dy;
    return r;
}

__device__ __forceinline__ slg_v4 sample_rgba8(const TexView& t, float u, float v)
{
    const Bilinear c = bilinear_coords(t, u, v);
    const uint32_t* p = reinterpret_cast<const uint32_t*>(t.texels);
    const float4 s = bilinear_sum(unpack_rgba8(__ldg(p + c.i00)), unpack_rgba8(__ldg(p + c.i01)),
                                  unpack_rgba8(__ldg(p + c.i10)), unpack_rgba8(__ldg(p + c.i11)), c);
    /* color_cast<uint8_t, float>, then the shader's color_cast<float, uint8_t> */
    return slg_make_v4((float)f2u8(s.x * 255.f) * 0.00392156862745f, (float)f2u8(s.y * 255.f) * 0.00392156862745f,
                       (float)f2u8(s.z * 255.f) * 0.00392156862745f, (float)f2u8(s.w * 255.f) * 0.00392156862745f);
}

__device__ __forceinline__ slg_v4 sample_rgbaf(const TexView& t, float u, float v)
{
    const Bilinear c = bilinear_coords(t, u, v);
    const float4* p = reinterpret_cast<const float4*>(t.texels);
    const float4 s = bilinear_sum(__ldg(p + c.i00), __ldg(p + c.i01), __ldg(p + c.i10), __ldg(p + c.i11), c);
    return slg_make_v4(s.x, s.y, s.z, s.w);
}

/* Environment handed to the header-only programs (include/slg_programs.h). */
struct DevEnv
{
    const uint8_t* vbo;
    int64_t b0Offset, b0Stride;
    const uint8_t* ubo;
    Tables tables;

    __device__ __forceinline__ const float* vertex(uint64_t vertId) const
    {
        return reinterpret_cast<const float*>(vbo + b0Offset + b0Stride * (int64_t)vertId);
    }
    __device__ __forceinline__ const void* uniforms() const { return ubo; }
    __device__ __forceinline__ const float* buffer(uint32_t vboId) const
    {
        return reinterpret_cast<const float*>(tables.buffers[vboId]);
    }
    __device__ __forceinline__ slg_v4 sample_rgba8(uint32_t texId, float u, float v) const
    {
        return slg::sample_rgba8(tables.textures[texId], u, v);
    }
    __device__ __forceinline__ slg_v4 sample_rgbaf(uint32_t texId, float u, float v) const
    {
        return slg::sample_rgbaf(tables.textures[texId], u, v);
    }
};

__device__ __forceinline__ DevEnv make_env(const DrawDesc& d, const Tables& t)
{
    DevEnv e;
    e.vbo = d.vbo;
    e.b0Offset = d.b0Offset;
    e.b0Stride = d.b0Stride;
    e.ubo = d.ubo;
    e.tables = t;
    return e;
}

/* Program dispatch: the GPU counterpart of calling SL_Shader::pVertShader /
 * pFragShader through a function pointer (softlight/src/SL_TriProcessor.cpp:584-594,
 * softlight/src/SL_FragmentProcessor.cpp:501). */
__device__ __forceinline__ slg_v4 run_vertex_program(uint32_t program, const DevEnv& env, uint64_t vertId,
                                                     uint64_t instanceId, slg_v4* varyings)
{
    switch (program)
    {
        case SLG_PROGRAM_LAMBERT_TEX:      return slg_vs_lambert(env, vertId, instanceId, varyings);
        case SLG_PROGRAM_BLINN_PHONG_INST: return slg_vs_blinn(env, vertId, instanceId, varyings);
        case SLG_PROGRAM_VCOLOR_TEX_ALPHA:
        case SLG_PROGRAM_VCOLOR_TEXF:
        case SLG_PROGRAM_GBUFFER:
        case SLG_PROGRAM_VCOLOR_TEX_CUTOUT:
        case SLG_PROGRAM_FRAG_COORD:       return slg_vs_vcolor(env, vertId, instanceId, varyings);
        default:                           return slg_vs_flat(env, vertId, instanceId, varyings);
    }
}

__device__ __forceinline__ bool run_fragment_program(uint32_t program, const DevEnv& env, slg_frag_coord& coord, const slg_v4* varyings,
                                                     slg_v4* outputs)
{
    switch (program)
    {
        case SLG_PROGRAM_LAMBERT_TEX:       return slg_fs_lambert(env, varyings, outputs);
        case SLG_PROGRAM_BLINN_PHONG_INST:  return slg_fs_blinn(env, varyings, outputs);
        case SLG_PROGRAM_VCOLOR_TEX_ALPHA:  return slg_fs_vcolor_tex_alpha(env, varyings, outputs);
        case SLG_PROGRAM_VCOLOR_TEXF:       return slg_fs_vcolor_texf(env, varyings, outputs);
        case SLG_PROGRAM_GBUFFER:           return slg_fs_gbuffer(env, varyings, outputs);
        case SLG_PROGRAM_VCOLOR_TEX_CUTOUT: return slg_fs_cutout(env, varyings, outputs);
        case SLG_PROGRAM_FRAG_COORD:        return slg_fs_frag_coord(env, &coord, varyings, outputs);
        default:                            return slg_fs_flat(env, varyings, outputs);
    }
}

/* The library's own program set (include/slg_programs.h), in the form the
 * draw-path kernel templates take (slg_pipeline.cuh). */
struct BuiltinPrograms
{
    static __device__ __forceinline__ slg_v4 vertex(const DrawDesc& d, const Tables& t, uint64_t vertId, uint64_t instanceId,
                                                    slg_v4* varyings)
    {
        return run_vertex_program(d.vsProgram, make_env(d, t), vertId, instanceId, varyings);
    }
    static __device__ __forceinline__ bool fragment(const DrawDesc& d, const Tables& t, slg_frag_coord& coord, const slg_v4* varyings,
                                                    slg_v4* outputs)
    {
        return run_fragment_program(d.fsProgram, make_env(d, t), coord, varyings, outputs);
    }
};

} // namespace slg

#endif /* SLG_DEVICE_CUH */
