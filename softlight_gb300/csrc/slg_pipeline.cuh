/*
 * slg_pipeline.cuh - the draw-path kernels that run shader programs, as
 * templates over a program set.
 *
 * A program set P supplies the GPU counterparts of SoftLight's shader
 * callbacks (SL_VertexShader::shader / SL_FragmentShader::shader,
 * softlight/include/softlight/SL_Shader.hpp:41-119):
 *
 *   static __device__ slg_v4 P::vertex(const DrawDesc& d, const Tables& t,
 *                                      uint64_t vertId, uint64_t instanceId,
 *                                      slg_v4* varyings);
 *   static __device__ bool   P::fragment(const DrawDesc& d, const Tables& t,
 *                                        slg_frag_coord& coord,
 *                                        const slg_v4* varyings, slg_v4* outputs);
 *
 * d.vsProgram / d.fsProgram name the program. The library instantiates these
 * kernels for its built-in programs (slg_builtin.cuh); a caller instantiates
 * them for its own programs through include/slg_shader.cuh and registers the
 * result with slg_register_programs. The kernels that do not run programs
 * (tile scan, tile lists, key-order fill, tile sort, clears, blits) live in
 * slg_kernels.cu.
 *
 * Pipeline of one launch (one draw, one instanced draw or a batch of draws):
 *   0. vertex cache : the vertex program once per (draw, instance, vertex)
 *                  of indexed draws that share vertices.
 *   1. vs_setup  : one thread per triangle slot (draw, instance, element
 *                  triple): three positions (cache or vertex program),
 *                  back-face cull, clip-space classification, perspective
 *                  divide, viewport mapping, the sub-pixel reject and
 *                  barycentric set-up of SL_TriProcessor
 *                  (softlight/src/SL_TriProcessor.cpp:248-640); writes one
 *                  128-byte raster record (+ varyings) per surviving
 *                  triangle and counts, per screen tile, the records whose
 *                  bounding box touches it; partially visible triangles are
 *                  queued for clip_kernel (Sutherland-Hodgman,
 *                  SL_TriProcessor.cpp:370-519). In an untiled launch each
 *                  warp then walks the records it stored (step 4).
 *   2. tile lists: scan of the per-tile counts and the fill of every
 *                  record's key into each tile list it touches (library),
 *                  in key order for blended launches.
 *   3. raster    : one CTA per tile. The order-free raster (no blending, one
 *                  order-independent depth rule) folds fragments into a
 *                  per-pixel best word and shades each pixel once; the
 *                  ordered raster replays, per pixel and in submission order,
 *                  the reference's scan-line span, incremental barycentrics,
 *                  depth test, perspective-correct varyings, fragment
 *                  program, blend and depth write
 *                  (softlight/src/SL_TriRasterizer.cpp:807-923,
 *                  softlight/src/SL_FragmentProcessor.cpp:417-531).
 *   4. untiled   : the order-free rule without tiles (steps 2-3 skipped):
 *                  records walked once into per-pixel best words in global
 *                  memory, then a pixel-parallel resolve.
 *
 * Ordering. SoftLight with one thread rasterises triangles in the order
 * push_bin emits them. Every record gets the key slot << 3 | sub, where the
 * slot counts triangles in submission order across draws and instances and
 * sub orders the fan triangles of a clipped input (0 when unclipped). Each
 * tile processes its keys in ascending order, and each pixel is owned by
 * exactly one thread, so every pixel sees its fragments in the reference's
 * order. Nothing else depends on order.
 *
 * Vector-library conventions (LightMath, absent from the reference tree):
 *   fmadd(a,b,c) = a*b + c (two roundings); rcp(x) = 1/x;
 *   dot/sum fold left ((a0+a1)+a2)+a3; mix(a,b,t) = (b-a)*t + a;
 *   cross(vec4) = (a1*b2-a2*b1, a2*b0-a0*b2, a0*b1-a1*b0, 0);
 *   cross(vec2) = a0*b1 - a1*b0; max(a,b) = a<b ? b : a; min(a,b) = b<a ? b : a;
 *   vec4 <= / >= compare all components; mat4*vec4 folds columns left;
 *   float->int truncation gives INT32_MIN for NaN / out of range.
 */
#ifndef SLG_PIPELINE_CUH
#define SLG_PIPELINE_CUH

#include "slg_device.cuh"

namespace slg
{

/*-----------------------------------------------------------------------------
 * Vertex stage helpers
-----------------------------------------------------------------------------*/
__device__ __forceinline__ float4 to_f4(const slg_v4& v) { return make_float4(v.x, v.y, v.z, v.w); }

__device__ __forceinline__ float4 mat_mul(const float* m, const float4 v)
{
    float4 r;
    r.x = ((m[0] * v.x + m[4] * v.y) + m[8]  * v.z) + m[12] * v.w;
    r.y = ((m[1] * v.x + m[5] * v.y) + m[9]  * v.z) + m[13] * v.w;
    r.z = ((m[2] * v.x + m[6] * v.y) + m[10] * v.z) + m[14] * v.w;
    r.w = ((m[3] * v.x + m[7] * v.y) + m[11] * v.z) + m[15] * v.w;
    return r;
}

/* face_determinant, portable branch (SL_TriProcessor.cpp:98-115) */
__device__ __forceinline__ float face_determinant(const float4 p0, const float4 p1, const float4 p2)
{
    const float w0 = 1.f / p0.w;
    const float w1 = 1.f / p1.w;
    const float w2 = 1.f / p2.w;
    const float v0x = p0.x * w0, v0y = p0.y * w0;
    const float v1x = p1.x * w1, v1y = p1.y * w1;
    const float v2x = p2.x * w2, v2y = p2.y * w2;
    const float s = (v0x * (v1y - v2y) + v1x * (v2y - v0y)) + v2x * (v0y - v1y);
    return __fadd_rn(s, 0.f);
}

/* sl_ndc_clip_status, portable branch (SL_PostVertexTransform.hpp:651-673) */
__device__ __forceinline__ int clip_status(const float4 c0, const float4 c1, const float4 c2)
{
    auto inside = [](const float4 c) {
        const float w = c.w, nw = -c.w;
        return (c.x <= w && c.y <= w && c.z <= w && c.w <= w) && (c.x >= nw && c.y >= nw && c.z >= nw && c.w >= nw);
    };
    const bool vis = inside(c0) && inside(c1) && inside(c2);
    const bool part = c0.w > 0.f || c1.w > 0.f || c2.w > 0.f;
    return (vis ? 3 : 0) | (part ? 1 : 0);
}

/* sl_perspective_divide + sl_ndc_to_screen_coords, portable branches
 * (SL_PostVertexTransform.hpp:240-249,509-524) */
__device__ __forceinline__ float4 to_screen(const float4 v, const float* vp)
{
    const float wInv = 1.f / v.w;
    const float x = v.x * wInv, y = v.y * wInv, z = v.z * wInv;
    const float hw = vp[2] * 0.5f, hh = vp[3] * 0.5f;
    float4 r;
    r.x = lm_max(floorf((x + 1.f) * hw + vp[0]), 0.f);
    r.y = lm_max(floorf((y + 1.f) * hh + vp[1]), 0.f);
    r.z = z;
    r.w = wInv;
    return r;
}

/* The sub-pixel reject of SL_TriProcessor::push_bin (SL_TriProcessor.cpp:257-264) */
__device__ __forceinline__ bool bin_visible(const float4 p0, const float4 p1, const float4 p2)
{
    const float minX = lm_min(lm_min(p0.x, p1.x), p2.x);
    const float minY = lm_min(lm_min(p0.y, p1.y), p2.y);
    const float maxX = lm_max(lm_max(p0.x, p1.x), p2.x);
    const float maxY = lm_max(lm_max(p0.y, p1.y), p2.y);
    return !((maxX - minX < 1.f) || (maxY - minY < 1.f));
}

/* Raster record of one binned triangle: the barycentric set-up of push_bin
 * (SL_TriProcessor.cpp:271-314) and the per-triangle constants of
 * SL_ScanlineBounds::init (SL_ScanlineBounds.hpp:137-186), which the
 * reference recomputes per bin and thread and which are kept here.
 *   r0 = (v0y, v1y, v0x, v1x)        r1 = (p20y, p20x, p21xy, p10xy)
 *   r2 = (bc0.xyz, bc.w)             r3 = (bc1.xyz, z0)
 *   r4 = (bc2.xyz, z1)               r5 = (z2, w0, w1, w2)
 *   r6 = (minY, maxY, minX-1, maxX+1) as int32 bits
 *   r7 = (draw index, primIndex lo, primIndex hi, depth test | mask << 4) as uint32 bits */
struct Record { float4 r[kRecordVec4]; };

__device__ __forceinline__ void make_record(const float4 p0, const float4 p1, const float4 p2, uint32_t drawIndex,
                                            uint64_t primIndex, uint32_t depthFlags, Record& rec)
{
    const float xyx = p0.x - p1.x, xyy = p0.y - p1.y;
    const float zyx = p2.x - p1.x, zyy = p2.y - p1.y;
    const float denom = 1.f / (zyx * xyy - zyy * xyx);

    const float ddx0 = p1.y - p2.y, ddx1 = p2.y - p0.y, ddx2 = p0.y - p1.y;
    const float ddy0 = p2.x - p1.x, ddy1 = p0.x - p2.x, ddy2 = p1.x - p0.x;
    const float ddz0 = p1.x * p2.y - p2.x * p1.y;
    const float ddz1 = p2.x * p0.y - p0.x * p2.y;
    const float ddz2 = p0.x * p1.y - p1.x * p0.y;

    /* SL_ScanlineBounds::init: sort by y, descending */
    float4 a = p0, b = p1, c = p2, t;
    if (a.y < b.y) { t = a; a = b; b = t; }
    if (a.y < c.y) { t = a; a = c; c = t; }
    if (b.y < c.y) { t = b; b = c; c = t; }
    const float p2p0x = c.x - a.x, p2p0y = c.y - a.y;
    const float p2p1x = c.x - b.x, p2p1y = c.y - b.y;
    const float p1p0x = b.x - a.x, p1p0y = b.y - a.y;

    const float minX = lm_min(lm_min(p0.x, p1.x), p2.x);
    const float minY = lm_min(lm_min(p0.y, p1.y), p2.y);
    const float maxX = lm_max(lm_max(p0.x, p1.x), p2.x);
    const float maxY = lm_max(lm_max(p0.y, p1.y), p2.y);

    rec.r[0] = make_float4(a.y, b.y, a.x, b.x);
    rec.r[1] = make_float4(1.f / p2p0y, p2p0x, p2p1x * (1.f / p2p1y), p1p0x * (1.f / p1p0y));
    rec.r[2] = make_float4(ddx0 * denom, ddx1 * denom, ddx2 * denom, 0.f * denom);
    rec.r[3] = make_float4(ddy0 * denom, ddy1 * denom, ddy2 * denom, p0.z);
    rec.r[4] = make_float4(ddz0 * denom, ddz1 * denom, ddz2 * denom, p1.z);
    rec.r[5] = make_float4(p2.z, p0.w, p1.w, p2.w);
    rec.r[6] = make_float4(__int_as_float(f2i(minY)), __int_as_float(f2i(maxY)),
                           __int_as_float(f2i(minX) - 1), __int_as_float(f2i(maxX) + 1));
    rec.r[7] = make_float4(__uint_as_float(drawIndex), __uint_as_float((uint32_t)primIndex),
                           __uint_as_float((uint32_t)(primIndex >> 32)), __uint_as_float(depthFlags));
}

/* The depth texel as the reference compares it, (float)depth_type, and its
 * write, (depth_type)z (_sl_get_depth_texel, SL_TriRasterizer.cpp:95-101;
 * SL_FragmentProcessor.cpp:398-401,524-527). A half depth is re-read after
 * every write, so depth_quant rounds a written z the same way. */
__device__ __forceinline__ float depth_load(const Frame& f, size_t i)
{
    if (f.depthType == SLG_COLOR_R_HALF) return slg_half_to_float(reinterpret_cast<const uint16_t*>(f.depth)[i]);
    if (f.depthType == SLG_COLOR_R_DOUBLE) return (float)reinterpret_cast<const double*>(f.depth)[i];
    return f.depth[i];
}

__device__ __forceinline__ void depth_store(const Frame& f, size_t i, float z)
{
    if (f.depthType == SLG_COLOR_R_HALF) reinterpret_cast<uint16_t*>(f.depth)[i] = slg_float_to_half(z);
    else if (f.depthType == SLG_COLOR_R_DOUBLE) reinterpret_cast<double*>(f.depth)[i] = (double)z;
    else f.depth[i] = z;
}

__device__ __forceinline__ float depth_quant(bool halfDepth, float z)
{
    return halfDepth ? slg_half_to_float(slg_float_to_half(z)) : z;
}

/* The packed formats 28..32 (RGB 332, RGB 565, RGBA 5551, RGBA 4444,
 * RGBA 1010102; softlight/include/softlight/SL_ColorCompressed.hpp):
 * unsigned bitfields from bit 0 up, the field widths one nibble each. */
constexpr int kFirstPacked = 28;

__device__ __forceinline__ uint32_t packed_widths(int type)
{
    switch (type)
    {
        case 28: return 0x0233u;
        case 29: return 0x0565u;
        case 30: return 0x1555u;
        case 31: return 0x4444u;
        default: return 0x2AAAu;
    }
}

__device__ __forceinline__ int packed_bytes(int type) { return (type == 28) ? 1 : (type == 32) ? 4 : 2; }

/* bytes of a texel of colour format `type` (SL_ColorDataType 0..32) */
__device__ __forceinline__ int texel_bytes(int type)
{
    if (type >= kFirstPacked) return packed_bytes(type);
    const int kind = type % 7;
    return (type / 7 + 1) * ((kind == 0) ? 1 : (kind == 1 || kind == 4) ? 2 : (kind == 2 || kind == 5) ? 4 : 8);
}

/* r7.w of a triangle record: depth test, depth mask, wireframe bit */
__device__ __forceinline__ uint32_t record_flags(const DrawDesc& d)
{
    return (uint32_t)d.depthTest | ((uint32_t)d.depthMask << 4) | (d.prim == kPrimWire ? kRecordWire : 0u);
}

/* Flags blended wireframe triangles whose queue flush points matter
 * (defined with the wireframe raster below). */
static __device__ __noinline__ void wire_queue_check(const Frame& f, const float4* R);

/* Inclusive tile range touched by a record; empty when tx1 < tx0 or ty1 < ty0. */
struct TileRange { int tx0, tx1, ty0, ty1; };

__device__ __forceinline__ TileRange tile_range(const float4 r6, const Frame& f)
{
    const int minY = __float_as_int(r6.x), maxY = __float_as_int(r6.y);
    const int minX = __float_as_int(r6.z), maxX = __float_as_int(r6.w);
    TileRange t;
    if (maxY <= minY || maxX < minX || maxY <= 0 || minY >= f.height || maxX < 0 || minX >= f.width)
    {
        t.tx0 = 0; t.tx1 = -1; t.ty0 = 0; t.ty1 = -1;
        return t;
    }
    const int ylo = max(minY, 0), yhi = min(maxY - 1, f.height - 1);
    const int xlo = max(minX, 0), xhi = min(maxX, f.width - 1);
    t.tx0 = xlo / f.tileW;
    t.tx1 = xhi / f.tileW;
    t.ty0 = ylo / f.tileH;
    t.ty1 = yhi / f.tileH;
    return t;
}

__device__ __forceinline__ void count_tiles(const float4 r6, const Frame& f)
{
    const TileRange t = tile_range(r6, f);
    for (int ty = t.ty0; ty <= t.ty1; ++ty)
    {
        for (int tx = t.tx0; tx <= t.tx1; ++tx)
        {
            atomicAdd(&f.tileCount[ty * f.tilesX + tx], 1u);
        }
    }
}

/* Walks each lane's tile range in lock-step; lanes that hit the same tile in
 * the same step are grouped with __match_any_sync and one atomic per group
 * adds (or reserves) the group's size. fn(tile, groupBase + rankInGroup) is
 * called per lane and tile when `reserve` points at per-tile cursors; with
 * reserve == nullptr only the counts are added. Every lane of the warp must
 * call this. */
template <class Fn>
__device__ __forceinline__ void warp_tile_walk(const Frame& f, TileRange t, bool valid, uint32_t* counters, Fn&& fn)
{
    const unsigned lane = threadIdx.x & 31;
    bool active = valid && t.tx1 >= t.tx0 && t.ty1 >= t.ty0;
    int tx = t.tx0, ty = t.ty0;
    while (__any_sync(0xFFFFFFFFu, active))
    {
        const uint32_t tile = active ? (uint32_t)(ty * f.tilesX + tx) : 0xFFFFFFFFu;
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, tile);
        if (active)
        {
            const unsigned leader = __ffs(peers) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(&counters[tile], (uint32_t)__popc(peers));
            base = __shfl_sync(peers, base, leader);
            fn(tile, base + __popc(peers & ((1u << lane) - 1u)));
            if (++tx > t.tx1)
            {
                tx = t.tx0;
                if (++ty > t.ty1) active = false;
            }
        }
    }
}

__device__ __forceinline__ void store_record(const Frame& f, uint64_t recIndex, const Record& rec)
{
    float4* dst = f.records + recIndex * kRecordVec4;
#pragma unroll
    for (int i = 0; i < kRecordVec4; ++i)
    {
        dst[i] = rec.r[i];
    }
}

__device__ __forceinline__ void store_varyings(const Frame& f, uint64_t recIndex, int nv,
                                               const slg_v4* a, const slg_v4* b, const slg_v4* c)
{
    float4* dst = f.varyings + recIndex * kVaryingVec4;
#pragma unroll
    for (int i = 0; i < kMaxVaryings; ++i)
    {
        if (i < nv)
        {
            dst[i] = to_f4(a[i]);
            dst[4 + i] = to_f4(b[i]);
            dst[8 + i] = to_f4(c[i]);
        }
    }
}

__device__ __forceinline__ slg_v4 mix4(const slg_v4 a, const slg_v4 b, float t)
{
    return slg_make_v4((b.x - a.x) * t + a.x, (b.y - a.y) * t + a.y, (b.z - a.z) * t + a.z, (b.w - a.w) * t + a.w);
}

__device__ __forceinline__ float4 mix4(const float4 a, const float4 b, float t)
{
    return make_float4((b.x - a.x) * t + a.x, (b.y - a.y) * t + a.y, (b.z - a.z) * t + a.z, (b.w - a.w) * t + a.w);
}

/* Whether SoftLight's clipper leaves nothing of a triangle in its first
 * pass that changes it: at the first plane (clipEdges order) with a vertex
 * outside, all three are outside. The passes before it copy the triangle
 * unchanged, so the clipper returns at that pass with no vertex; such a
 * triangle is not queued. */
__device__ __forceinline__ bool clip_trivially_empty(const float4* c)
{
#pragma unroll
    for (int e = 0; e < 6; ++e)
    {
        const float ex = (e == 0) ? 1.f : (e == 1) ? -1.f : 0.f;
        const float ey = (e == 2) ? 1.f : (e == 3) ? -1.f : 0.f;
        const float ez = (e == 4) ? 1.f : (e == 5) ? -1.f : 0.f;
        int out = 0;
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            out += sign_mask(((c[k].x * ex + c[k].y * ey) + c[k].z * ez) + c[k].w * 1.f);
        }
        if (out == 3) return true;
        if (out > 0) return false;
    }
    return false;
}

/* SL_TriProcessor::clip_and_process_tris (SL_TriProcessor.cpp:370-519),
 * two triangles per warp, one per 16-lane half. Lane v of a half holds
 * polygon vertex v (v < 9): its clip position and its four varying slots,
 * as newVerts[v] and newVarys[v * 4 .. v * 4 + 3], plus its tempVerts /
 * tempVarys entries. Per clip plane every lane tests its vertex, a scan over
 * the half places each vertex's outputs (the crossing point with the
 * previous vertex, then the vertex if inside), and each output lane fetches
 * its one or two source vertices by shuffle, so every interpolation is the
 * reference's expression on the same operands. The reference's copy-back of
 * the varyings moves numNew vectors from each output vertex's first slot
 * (:471-475); slot 4 v + m is refreshed from tempVarys when v * 4 + m lies
 * in some range [4 i, 4 i + numNew), i < numNew, which copied_slot
 * evaluates per lane. Every lane of the warp calls it (no early exit: the
 * halves shuffle together); returns the half's slotInfo value. */
__device__ __forceinline__ bool copied_slot(int v, int m, int numNew)
{
    return (v < numNew && m < numNew) || (v >= 1 && v - 1 < numNew && m + 4 < numNew) || (v >= 2 && v - 2 < numNew && m + 8 < numNew);
}

constexpr int kClipLanes = 16;  /* lanes per clipped triangle */

__device__ __forceinline__ float4 shfl4(const float4 v, int src)
{
    return make_float4(__shfl_sync(0xFFFFFFFFu, v.x, src, kClipLanes), __shfl_sync(0xFFFFFFFFu, v.y, src, kClipLanes),
                       __shfl_sync(0xFFFFFFFFu, v.z, src, kClipLanes), __shfl_sync(0xFFFFFFFFu, v.w, src, kClipLanes));
}

__device__ __forceinline__ slg_v4 shfl4(const slg_v4 v, int src)
{
    return slg_make_v4(__shfl_sync(0xFFFFFFFFu, v.x, src, kClipLanes), __shfl_sync(0xFFFFFFFFu, v.y, src, kClipLanes),
                       __shfl_sync(0xFFFFFFFFu, v.z, src, kClipLanes), __shfl_sync(0xFFFFFFFFu, v.w, src, kClipLanes));
}

constexpr int kClipVerts = 9;   /* 3 + one per clip plane: the reference's array sizes */

template <class P>
__device__ __forceinline__ uint32_t clip_pair(const Frame& f, bool active, const DrawDesc& d, uint32_t drawIndex, uint64_t slot,
                                              uint64_t primIndex, uint64_t inst, uint64_t vid, float4 pos)
{
    const int lane = threadIdx.x & 31;
    const int sl = lane & (kClipLanes - 1);
    const int half = lane >> 4;
    const int nv = active ? d.numVaryings : 0;
    const slg_v4 zero4 = slg_make_v4(0.f, 0.f, 0.f, 0.f);
    slg_v4 cur[kMaxVaryings], tmp[kMaxVaryings];
#pragma unroll
    for (int i = 0; i < kMaxVaryings; ++i)
    {
        cur[i] = zero4;
        tmp[i] = zero4;
    }
    if (active && sl < 3)
    {
        if (d.cacheVerts)
        {
#pragma unroll
            for (int i = 0; i < kMaxVaryings; ++i)
            {
                if (i < nv)
                {
                    const float4 cv = f.cacheVary[(uint64_t)i * f.cacheEntries + vid];
                    cur[i] = slg_make_v4(cv.x, cv.y, cv.z, cv.w);
                }
            }
        }
        else
        {
            slg_v4 vary[kMaxVaryings];
            (void)P::vertex(d, f.tables, vid, inst, vary);
#pragma unroll
            for (int i = 0; i < kMaxVaryings; ++i)
            {
                if (i < nv) cur[i] = vary[i];
            }
        }
    }
    else
    {
        pos = make_float4(0.f, 0.f, 0.f, 0.f);
    }

    /* numTotal 0: no triangle in this half, or nothing left of it */
    int numTotal = active ? 3 : 0;
    for (int e = 0; e < 6; ++e)
    {
        /* clipEdges: +x, -x, +y, -y, +z, -z against w (SL_TriProcessor.cpp:384-393) */
        const float ex = (e == 0) ? 1.f : (e == 1) ? -1.f : 0.f;
        const float ey = (e == 2) ? 1.f : (e == 3) ? -1.f : 0.f;
        const float ez = (e == 4) ? 1.f : (e == 5) ? -1.f : 0.f;
        const bool mine = sl < numTotal;
        const float t = mine ? ((pos.x * ex + pos.y * ey) + pos.z * ez) + pos.w * 1.f : 0.f;
        const int vis = mine ? !sign_mask(t) : 0;
        if (__ballot_sync(0xFFFFFFFFu, mine && !vis) == 0u)
        {
            /* every vertex inside, in both halves: the outputs are the
             * inputs in order, so tempVerts / tempVarys take the current
             * values and the copy-back runs as for any pass */
            if (mine)
            {
#pragma unroll
                for (int i = 0; i < kMaxVaryings; ++i)
                {
                    if (i < nv) tmp[i] = cur[i];
                }
            }
            if (sl < kClipVerts && numTotal > 0)
            {
#pragma unroll
                for (int m = 0; m < kMaxVaryings; ++m)
                {
                    if (copied_slot(sl, m, numTotal)) cur[m] = tmp[m];
                }
            }
            continue;
        }
        const int prev = (sl == 0) ? max(numTotal - 1, 0) : sl - 1;
        const int visPrev = __shfl_sync(0xFFFFFFFFu, vis, prev, kClipLanes);
        const int cross = (mine && (visPrev ^ vis)) ? 1 : 0;
        const int cnt = cross + vis;
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < kClipLanes; o <<= 1)
        {
            const int n = __shfl_up_sync(0xFFFFFFFFu, incl, o, kClipLanes);
            if (sl >= o) incl += n;
        }
        int numNew = __shfl_sync(0xFFFFFFFFu, incl, kClipLanes - 1, kClipLanes);
        /* more than 9 vertices would overrun the reference's arrays: such a
         * polygon is not rendered */
        if (numNew > kClipVerts) numNew = 0;
        const int out0 = incl - cnt;
        /* the vertex k whose outputs hold output slot sl */
        int k = 0;
#pragma unroll
        for (int q = 1; q < kClipVerts; ++q)
        {
            if (__shfl_sync(0xFFFFFFFFu, out0, q, kClipLanes) <= sl && q < numTotal) k = q;
        }
        const int kOut0 = __shfl_sync(0xFFFFFFFFu, out0, k, kClipLanes);
        const int kCross = __shfl_sync(0xFFFFFFFFu, cross, k, kClipLanes);
        const bool isMix = kCross && sl == kOut0;
        const int srcA = isMix ? ((k == 0) ? numTotal - 1 : k - 1) : k;
        const float4 pa = shfl4(pos, srcA), pb = shfl4(pos, k);
        const float ta = __shfl_sync(0xFFFFFFFFu, t, srcA, kClipLanes), tb = __shfl_sync(0xFFFFFFFFu, t, k, kClipLanes);
        slg_v4 va[kMaxVaryings], vb[kMaxVaryings];
#pragma unroll
        for (int i = 0; i < kMaxVaryings; ++i)
        {
            va[i] = zero4;
            vb[i] = zero4;
            if (__any_sync(0xFFFFFFFFu, i < nv))
            {
                va[i] = shfl4(cur[i], srcA);
                vb[i] = shfl4(cur[i], k);
            }
        }
        if (sl < numNew)
        {
            if (isMix)
            {
                const float tt = ta * (1.f / (ta - tb));
                pos = mix4(pa, pb, tt);
#pragma unroll
                for (int i = 0; i < kMaxVaryings; ++i)
                {
                    if (i < nv) tmp[i] = mix4(va[i], vb[i], tt);
                }
            }
            else
            {
                pos = pb;
#pragma unroll
                for (int i = 0; i < kMaxVaryings; ++i)
                {
                    if (i < nv) tmp[i] = vb[i];
                }
            }
        }
        if (sl < kClipVerts && numNew > 0)
        {
#pragma unroll
            for (int m = 0; m < kMaxVaryings; ++m)
            {
                if (copied_slot(sl, m, numNew)) cur[m] = tmp[m];
            }
        }
        numTotal = numNew;
    }

    const float4 sp = (sl < numTotal) ? to_screen(pos, f.viewport) : make_float4(0.f, 0.f, 0.f, 0.f);

    /* fan (0, i+1, i+2) for i = numTotal-3 .. 0, in that order: lane i */
    const int i1 = min(sl + 1, kClipLanes - 1), i2 = min(sl + 2, kClipLanes - 1);
    const float4 a = shfl4(sp, 0), b = shfl4(sp, i1), c = shfl4(sp, i2);
    const bool fan = sl < numTotal - 2 && bin_visible(a, b, c);
    const uint32_t vmask = (__ballot_sync(0xFFFFFFFFu, fan) >> (half * kClipLanes)) & 0xFFFFu;
    const uint32_t survivors = (uint32_t)__popc(vmask);
    uint32_t base = 0;
    if (sl == 0 && survivors) base = atomicAdd(f.ovfCount, survivors);
    base = __shfl_sync(0xFFFFFFFFu, base, 0, kClipLanes);
    const bool fits = survivors && base + survivors <= f.ovfCap;
    if (sl == 0 && survivors)
    {
        if (fits)
        {
            f.slotOvf[slot] = base;
        }
        else
        {
            atomicOr(f.status, kStatusOvfOverflow);
            atomicMax(f.status + 2, (int)(base + survivors));
        }
    }

    slg_v4 v0[kMaxVaryings], v1[kMaxVaryings], v2[kMaxVaryings];
#pragma unroll
    for (int i = 0; i < kMaxVaryings; ++i)
    {
        v0[i] = zero4;
        v1[i] = zero4;
        v2[i] = zero4;
        if (__any_sync(0xFFFFFFFFu, i < nv))
        {
            v0[i] = shfl4(cur[i], 0);
            v1[i] = shfl4(cur[i], i1);
            v2[i] = shfl4(cur[i], i2);
        }
    }
    if (fan && fits)
    {
        /* records in fan order: those of higher i come first */
        const uint32_t sub = (uint32_t)__popc(vmask & ~((2u << sl) - 1u));
        Record rec;
        make_record(a, b, c, drawIndex, primIndex, record_flags(d), rec);
        if (d.prim == kPrimWire && d.blend != SLG_BLEND_OFF) wire_queue_check(f, rec.r);
        const uint64_t recIndex = f.numSlots + base + sub;
        store_record(f, recIndex, rec);
        store_varyings(f, recIndex, nv, v0, v1, v2);
        if (f.ovfKey) f.ovfKey[base + sub] = (uint32_t)(slot << kSubShift) | (sub + 1u);
        if (f.chunkCounts == nullptr && f.bestWords == nullptr) count_tiles(rec.r[6], f);
    }
    return fits ? 2u + survivors : 0u;
}

/* a / b in slot arithmetic: one 32-bit division when both fit (slots stay
 * below 2^29), the 64-bit routine otherwise; the same quotient either way */
__device__ __forceinline__ uint64_t udiv_slot(uint64_t a, uint64_t b)
{
    return ((a | b) >> 32) == 0 ? (uint64_t)((uint32_t)a / (uint32_t)b) : a / b;
}

__device__ __forceinline__ int find_draw(const Frame& f, uint64_t slot)
{
    int lo = 0, hi = f.numDraws - 1;
    while (lo < hi)
    {
        const int mid = (lo + hi + 1) >> 1;
        if (f.drawSlotStart[mid] <= slot) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ uint64_t read_index(const DrawDesc& d, uint64_t i)
{
    switch (d.indexType)
    {
        case SLG_VERTEX_DATA_BYTE:  return d.ibo[i];
        case SLG_VERTEX_DATA_SHORT: return reinterpret_cast<const uint16_t*>(d.ibo)[i];
        default:                    return reinterpret_cast<const uint32_t*>(d.ibo)[i];
    }
}

/*-----------------------------------------------------------------------------
 * Kernel 1: vertex processing, clipping, set-up and tile counting
 * (SL_TriProcessor::process_verts, SL_TriProcessor.cpp:527-640)
-----------------------------------------------------------------------------*/
/* SL_PointProcessor::process_verts for one point (softlight/src/SL_PointProcessor.cpp:63-110):
 * vertex program, scissor, the one-vertex clip status (fully inside
 * [-w, w] with w > 0, SL_PostVertexTransform.hpp:536-552), divide and
 * viewport. The fragment lands where SL_PointRasterizer addresses it: the
 * 16-bit screen coordinates at linear index x + W*y (SL_PointRasterizer.cpp:
 * 45-57), so x == W wraps to the next row; an index past the buffer (which
 * the reference would write out of bounds) is dropped. */
template <class P>
__device__ __forceinline__ uint32_t setup_point(const Frame& f, const DrawDesc& d, int di, uint64_t slot, uint64_t local,
                                                TileRange& tr, bool& counted)
{
    const uint64_t inst = udiv_slot(local, d.numTris);
    const uint64_t e = d.elementBegin + (local - inst * d.numTris);
    const uint64_t vid = (d.indexType >= 0) ? read_index(d, e) : e;
    slg_v4 vary[kMaxVaryings];
    float4 c = mat_mul(f.scissor, to_f4(P::vertex(d, f.tables, vid, inst, vary)));
    const float w = c.w, nw = -c.w;
    const bool visible = (w > 0.f) && (c.x <= w && c.y <= w && c.z <= w && c.w <= w) &&
                         (c.x >= nw && c.y >= nw && c.z >= nw && c.w >= nw);
    if (!visible)
    {
        return 0;
    }
    const float4 sc = to_screen(c, f.viewport);
    const uint64_t lin = (uint64_t)((uint32_t)f2i(sc.x) & 0xFFFFu) + (uint64_t)f.width * ((uint32_t)f2i(sc.y) & 0xFFFFu);
    if (lin >= (uint64_t)f.width * (uint64_t)f.height)
    {
        return 0;
    }
    const int px = (int)(lin % (uint64_t)f.width), py = (int)(lin / (uint64_t)f.width);
    Record rec;
    rec.r[0] = sc;
    rec.r[1] = rec.r[2] = rec.r[3] = rec.r[4] = rec.r[5] = make_float4(0.f, 0.f, 0.f, 0.f);
    rec.r[6] = make_float4(__int_as_float(py), __int_as_float(py + 1), __int_as_float(px), __int_as_float(px));
    rec.r[7] = make_float4(__uint_as_float((uint32_t)di), __uint_as_float((uint32_t)e), __uint_as_float((uint32_t)(e >> 32)),
                           __uint_as_float((uint32_t)d.depthTest | ((uint32_t)d.depthMask << 4) | kRecordPoint));
    store_record(f, slot, rec);
    float4* dst = f.varyings + slot * kVaryingVec4;
#pragma unroll
    for (int vi = 0; vi < kMaxVaryings; ++vi)
    {
        if (vi < d.numVaryings) dst[vi] = to_f4(vary[vi]);
    }
    tr = tile_range(rec.r[6], f);
    counted = true;
    return 1;
}

/*-----------------------------------------------------------------------------
 * Lines (SL_LineProcessor, softlight/src/SL_LineProcessor.cpp:51-279;
 * SL_LineRasterizer, softlight/src/SL_LineRasterizer.cpp:26-96). A line record:
 *   r0, r1 = screen positions of the two ends (x, y, z, w)
 *   r2     = (1 / |end1 - end0|, 0, 0, 0)
 *   r3     = Bresenham walk as int32 bits: (x1, x2, y1, steep | (yErr < 0) << 1)
 *   r4     = (dx, dErr, wraps, alias event + 1 or 0) as int32 bits
 *   r6     = pixel bounds, r7 = (draw, primIndex lo, hi, flags | kRecordLine)
-----------------------------------------------------------------------------*/
constexpr float kLineEpsilon = 1.0e-6f;   /* LS_EPSILON */

__device__ __forceinline__ float mixf(float a, float b, float t) { return (b - a) * t + a; }

/* _clip_segment of SL_LineProcessor::clip_and_process_lines (SL_LineProcessor.cpp:94-126) */
__device__ __forceinline__ bool clip_segment(float num, float denom, float& tE, float& tL)
{
    if (fabsf(denom) < kLineEpsilon) return num < 0.f;
    const float t = num / denom;
    if (denom > 0.f)
    {
        if (t > tL) return false;
        if (t > tE) tE = t;
    }
    else
    {
        if (t < tE) return false;
        if (t < tL) tL = t;
    }
    return true;
}

/* Screen-space clip of a partially visible line against the viewport
 * (SL_LineProcessor.cpp:63-166); false when nothing is left. */
__device__ __forceinline__ bool clip_line(const float* vp, float4& p0, float4& p1, slg_v4* va, slg_v4* vb, int nv)
{
    const float4 a = p0, b = p1;
    const float dx = b.x - a.x, dy = b.y - a.y;
    const float xMin = vp[0], yMin = vp[1], xMax = vp[2], yMax = vp[3];
    if (fabsf(dx) < kLineEpsilon && fabsf(dy) < kLineEpsilon)
    {
        if (a.x >= xMin && a.x <= xMax && a.y >= yMin && a.y <= yMax) return true;
    }
    const float ex = a.x - b.x, ey = a.y - b.y;
    const float dist = 1.f / sqrtf(ex * ex + ey * ey);
    float tE = 0.f, tL = 1.f;
    if (!(clip_segment(xMin - a.x, dx, tE, tL) && clip_segment(a.x - xMax, -dx, tE, tL) &&
          clip_segment(yMin - a.y, dy, tE, tL) && clip_segment(a.y - yMax, -dy, tE, tL)))
    {
        return false;
    }
    if (tL < 1.f)
    {
        p1.x = a.x + tL * dx;
        p1.y = a.y + tL * dy;
    }
    if (tE > 0.f)
    {
        p0.x = a.x + tE * dx;
        p0.y = a.y + tE * dy;
    }
    const float l0x = p0.x - a.x, l0y = p0.y - a.y, l1x = p1.x - b.x, l1y = p1.y - b.y;
    const float interp0 = sqrtf(((l0x * l0x + l0y * l0y) + 0.f) + 0.f) * dist;
    const float interp1 = sqrtf(((l1x * l1x + l1y * l1y) + 0.f) + 0.f) * dist;
    p0.z = mixf(a.z, b.z, interp0);
    p0.w = mixf(a.w, b.w, interp0);
    p1.z = mixf(b.z, a.z, interp1);
    p1.w = mixf(b.w, a.w, interp1);
#pragma unroll
    for (int vi = 0; vi < kMaxVaryings; ++vi)
    {
        if (vi < nv)
        {
            const slg_v4 u = va[vi], v = vb[vi];
            va[vi] = slg_make_v4(mixf(u.x, v.x, interp0), mixf(u.y, v.y, interp0), mixf(u.z, v.z, interp0), mixf(u.w, v.w, interp0));
            vb[vi] = slg_make_v4(mixf(v.x, u.x, interp1), mixf(v.y, u.y, interp1), mixf(v.z, u.z, interp1), mixf(v.w, u.w, interp1));
        }
    }
    return true;
}

/* float screen coordinate -> the int16 the Bresenham walk takes ((uint16_t) cast, then sl_lowp_t) */
__device__ __forceinline__ int lowp(float v) { return (int)(int16_t)(uint16_t)((uint32_t)f2i(v) & 0xFFFFu); }

/* SL_LineProcessor::process_verts for one segment (SL_LineProcessor.cpp:172-279). */
template <class P>
__device__ __forceinline__ uint32_t setup_line(const Frame& f, const DrawDesc& d, int di, uint64_t slot, uint64_t local,
                                               TileRange& tr, bool& counted)
{
    const uint64_t inst = udiv_slot(local, d.numTris);
    const uint64_t i = d.elementBegin + 2u * (local - inst * d.numTris);
    slg_v4 va[kMaxVaryings], vb[kMaxVaryings];
    const uint64_t vid0 = (d.indexType >= 0) ? read_index(d, i) : i;
    const uint64_t vid1 = (d.indexType >= 0) ? read_index(d, i + 1) : (i + 1);
    const float4 c0 = mat_mul(f.scissor, to_f4(P::vertex(d, f.tables, vid0, inst, va)));
    const float4 c1 = mat_mul(f.scissor, to_f4(P::vertex(d, f.tables, vid1, inst, vb)));
    if (c0.w < 0.f || c1.w < 0.f)
    {
        return 0;
    }
    /* sl_ndc_clip_status of two vertices (SL_PostVertexTransform.hpp:560-585) */
    const float w0 = c0.w, w1 = c1.w;
    const bool inside = (c0.x <= w0 && c0.y <= w0 && c0.z <= w0 && c0.w <= w0) && (c1.x <= w1 && c1.y <= w1 && c1.z <= w1 && c1.w <= w1) &&
                        (c0.x >= -w0 && c0.y >= -w0 && c0.z >= -w0 && c0.w >= -w0) && (c1.x >= -w1 && c1.y >= -w1 && c1.z >= -w1 && c1.w >= -w1);
    const int status = (inside ? 3 : 0) | ((w0 > 0.f || w1 > 0.f) ? 1 : 0);
    if (status == 0)
    {
        return 0;
    }
    float4 s0 = to_screen(c0, f.viewport), s1 = to_screen(c1, f.viewport);
    uint64_t primIndex = i;
    if (status == 1)
    {
        if (!clip_line(f.viewport, s0, s1, va, vb, d.numVaryings)) return 0;
        primIndex = i * inst + i;
    }

    /* sl_draw_line_bresenham set-up (softlight/include/softlight/SL_Geometry.hpp:314-333) */
    int x1 = lowp(s0.x), y1 = lowp(s0.y), x2 = lowp(s1.x), y2 = lowp(s1.y);
    const int minX = min(x1, x2), maxX = max(x1, x2), minY = min(y1, y2), maxY = max(y1, y2);
    const bool steep = abs(x1 - x2) < abs(y1 - y2);
    if (steep)
    {
        int t = x1; x1 = y1; y1 = t;
        t = x2; x2 = y2; y2 = t;
    }
    if (x1 > x2)
    {
        int t = x1; x1 = x2; x2 = t;
        t = y1; y1 = y2; y2 = t;
    }
    const int dxl = (int)(int16_t)(x2 - x1);
    const int dErr = (int)(int16_t)(abs((int)(int16_t)(y2 - y1)) * 2);
    const int yNeg = (y2 > y1) ? 0 : 1;
    const bool wraps = maxX >= f.width;   /* pixels at x = W land on the next row */

    /* the last step (x = W, row y2) is stored at the first step's address
     * (x = 0, row y1 = y2 + 1): logged for alias_fixup_kernel when the depth
     * state can tell the queue's test order from the sequential one */
    int aliasTag = 0;
    if (!steep && x1 == 0 && x2 == f.width && y2 == y1 - 1 && y1 < f.height && d.depthMask && d.depthTest != SLG_DEPTH_TEST_OFF &&
        f.aliasEvents)
    {
        const uint32_t e = atomicAdd(f.aliasCount, 1u);
        if (e < f.aliasCap)
        {
            AliasEvent& ev = f.aliasEvents[e];
            const uint32_t pix = (uint32_t)y1 * (uint32_t)f.width;
            ev.slot = (uint32_t)slot;
            ev.pixel = pix;
            ev.queued = 0;
            ev.depth0 = depth_load(f, pix);
            for (int k = 0; k < f.numColors; ++k)
            {
                const int bpt = texel_bytes(f.colorTypes[k]);
                for (int b = 0; b < bpt; ++b) ev.colors[k][b] = f.colors[k][(size_t)pix * bpt + b];
            }
            aliasTag = (int)e + 1;
        }
        else
        {
            atomicOr(f.status, kStatusAliasOverflow);
        }
    }

    Record rec;
    const float ex = s1.x - s0.x, ey = s1.y - s0.y;
    rec.r[0] = s0;
    rec.r[1] = s1;
    rec.r[2] = make_float4(1.f / sqrtf(ex * ex + ey * ey), 0.f, 0.f, 0.f);
    rec.r[3] = make_float4(__int_as_float(x1), __int_as_float(x2), __int_as_float(y1), __int_as_float((steep ? 1 : 0) | (yNeg << 1)));
    rec.r[4] = make_float4(__int_as_float(dxl), __int_as_float(dErr), __int_as_float(wraps ? 1 : 0), __int_as_float(aliasTag));
    rec.r[5] = make_float4(0.f, 0.f, 0.f, 0.f);
    rec.r[6] = wraps ? make_float4(__int_as_float(minY), __int_as_float(maxY + 2), __int_as_float(0), __int_as_float(f.width - 1))
                     : make_float4(__int_as_float(minY), __int_as_float(maxY + 1), __int_as_float(minX), __int_as_float(maxX));
    rec.r[7] = make_float4(__uint_as_float((uint32_t)di), __uint_as_float((uint32_t)primIndex), __uint_as_float((uint32_t)(primIndex >> 32)),
                           __uint_as_float((uint32_t)d.depthTest | ((uint32_t)d.depthMask << 4) | kRecordLine));
    store_record(f, slot, rec);
    float4* dst = f.varyings + slot * kVaryingVec4;
#pragma unroll
    for (int vi = 0; vi < kMaxVaryings; ++vi)
    {
        if (vi < d.numVaryings)
        {
            dst[vi] = to_f4(va[vi]);
            dst[4 + vi] = to_f4(vb[vi]);
        }
    }
    tr = tile_range(rec.r[6], f);
    counted = true;
    return 1;
}

/* The Bresenham walk of a line record. */
struct LineWalk
{
    int x1, x2, y1, dx, dErr, yErr;
    bool steep, wraps;
};

__device__ __forceinline__ LineWalk line_walk(const float4* R)
{
    LineWalk w;
    const float4 r3 = R[3], r4 = R[4];
    w.x1 = __float_as_int(r3.x);
    w.x2 = __float_as_int(r3.y);
    w.y1 = __float_as_int(r3.z);
    const int fl = __float_as_int(r3.w);
    w.steep = (fl & 1) != 0;
    w.yErr = (fl & 2) ? -1 : 1;
    w.dx = __float_as_int(r4.x);
    w.dErr = __float_as_int(r4.y);
    w.wraps = __float_as_int(r4.z) != 0;
    return w;
}

/* Pixel k (0..dx) of sl_draw_line_bresenham (SL_Geometry.hpp:335-363): the
 * error term stays in (-dx, dx], so before pixel k the minor coordinate has
 * moved ceil((k dErr - dx) / (2 dx)) steps. Returns the 16-bit (x, y) the
 * callback receives. */
__device__ __forceinline__ void line_pixel(const LineWalk& w, int k, uint32_t& X, uint32_t& Y)
{
    const int a = k * w.dErr - w.dx;
    const int m = (a <= 0) ? 0 : (a + 2 * w.dx - 1) / (2 * w.dx);
    const int p = (int)(int16_t)(w.x1 + k), q = (int)(int16_t)(w.y1 + w.yErr * m);
    X = (uint32_t)(w.steep ? q : p) & 0xFFFFu;
    Y = (uint32_t)(w.steep ? p : q) & 0xFFFFu;
}

/* Walk steps whose pixel can land in row y of the columns [x0, xLimit):
 * [kLo, kHi] with callback row y, plus kWrap (or -1), the step whose pixel
 * has x = W on row y - 1 and so is stored at (0, y). Inverting the closed
 * form above: minor step m is taken by the steps k with
 * 2 dx m - dx < k dErr <= 2 dx m + dx. */
struct LineRow { int kLo, kHi, kWrap; };

__device__ __forceinline__ LineRow line_row(const LineWalk& w, int y, int x0, int xLimit, int width)
{
    LineRow lr;
    lr.kLo = 0;
    lr.kHi = -1;
    lr.kWrap = -1;
    if (w.steep)
    {
        lr.kLo = lr.kHi = y - w.x1;
        if (w.wraps && x0 == 0) lr.kWrap = y - 1 - w.x1;
    }
    else
    {
        const int m = (y - w.y1) * w.yErr;
        if (m >= 0)
        {
            if (w.dErr == 0)
            {
                if (m == 0) lr.kHi = w.dx;
            }
            else
            {
                lr.kLo = (m == 0) ? 0 : (2 * w.dx * m - w.dx) / w.dErr + 1;
                lr.kHi = (2 * w.dx * m + w.dx) / w.dErr;
            }
        }
        lr.kLo = max(lr.kLo, x0 - w.x1);
        lr.kHi = min(lr.kHi, min(xLimit, width) - 1 - w.x1);
        if (w.wraps && x0 == 0) lr.kWrap = w.dx;
    }
    lr.kLo = max(lr.kLo, 0);
    lr.kHi = min(lr.kHi, w.dx);
    if (lr.kWrap > w.dx) lr.kWrap = -1;
    return lr;
}

/* Stored pixel of walk step k: SoftLight addresses the buffers with
 * x + W * y of the 16-bit callback coordinates, so x = W lands on the next
 * row; steps past the end of the buffer are dropped (false). */
__device__ __forceinline__ bool line_store_pixel(const LineWalk& w, int k, int width, int height, uint32_t& X, uint32_t& Y,
                                                 int& px, int& py)
{
    line_pixel(w, k, X, Y);
    const uint32_t lin = X + (uint32_t)width * Y;
    if (lin >= (uint32_t)width * (uint32_t)height) return false;
    py = (int)(lin / (uint32_t)width);
    px = (int)(lin - (uint32_t)py * (uint32_t)width);
    return true;
}

/* SL_LineRasterizer::render_line per pixel (SL_LineRasterizer.cpp:49-58):
 * interp = |p - end0| / |end1 - end0|, z = mix(z0, z1, interp). */
__device__ __forceinline__ float line_interp(const float4* R, uint32_t X, uint32_t Y)
{
    const float ex = (float)X - R[0].x, ey = (float)Y - R[0].y;
    return sqrtf(((ex * ex + ey * ey) + 0.f) + 0.f) * R[2].x;
}

/* kCached: every draw of the launch is an indexed triangle draw served by
 * the vertex cache, so the vertex programs are compiled out of this
 * instantiation (fewer registers, more resident warps). */
template <class P, bool kLines, bool kCached>
__device__ __forceinline__ uint32_t setup_slot(const Frame& f, uint64_t slot, TileRange& tr, bool& counted)
{
    const int di = (f.numDraws > 1) ? find_draw(f, slot) : 0;
    const DrawDesc& d = f.draws[di];
    if (d.hidden)
    {
        return 0;
    }
    const uint64_t local = slot - d.slotBase;
    if (!kCached && d.prim == kPrimPoint)
    {
        return setup_point<P>(f, d, di, slot, local, tr, counted);
    }
    if (!kCached && kLines && d.prim == kPrimLine)
    {
        return setup_line<P>(f, d, di, slot, local, tr, counted);
    }
    const uint64_t inst = udiv_slot(local, d.numTris);
    const uint64_t tri = local - inst * d.numTris;
    const uint64_t i = d.elementBegin + 3u * tri;

    /* positions first; the varyings are produced again per vertex only for
     * triangles that are stored (keeps three vertices' varyings out of the
     * registers while culling and set-up run) */
    float4 clip[3];
    uint64_t vids[3];
    const bool cached = kCached || d.cacheVerts != 0;
#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
        vids[k] = (d.indexType >= 0) ? read_index(d, i + k) : (i + k);
        if (cached)
        {
            vids[k] += d.cacheBase + inst * d.cacheVerts;
            clip[k] = f.cachePos[vids[k]];
        }
        else if (!kCached)
        {
            slg_v4 unused[kMaxVaryings];
            clip[k] = to_f4(P::vertex(d, f.tables, vids[k], inst, unused));
        }
    }

    if (d.cull != SLG_CULL_OFF)
    {
        const float det = face_determinant(clip[0], clip[1], clip[2]);
        const bool culled = (d.cull == SLG_CULL_FRONT_FACE) ^ (sign_mask(det) != 0);
        if (culled)
        {
            return 0;
        }
    }

#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
        clip[k] = mat_mul(f.scissor, clip[k]);
    }

    const uint64_t primIndex = d.primBase + d.numElements * inst + i;
    const int vis = clip_status(clip[0], clip[1], clip[2]);
    if (vis == 3)
    {
        const float4 s0 = to_screen(clip[0], f.viewport);
        const float4 s1 = to_screen(clip[1], f.viewport);
        const float4 s2 = to_screen(clip[2], f.viewport);
        if (bin_visible(s0, s1, s2))
        {
            Record rec;
            make_record(s0, s1, s2, (uint32_t)di, primIndex, record_flags(d) | (cached ? kRecordCached : 0u), rec);
            if (kLines && d.prim == kPrimWire && d.blend != SLG_BLEND_OFF) wire_queue_check(f, rec.r);
            store_record(f, slot, rec);
            tr = tile_range(rec.r[6], f);
            if (cached)
            {
                f.recVerts[slot] = make_uint4((uint32_t)vids[0], (uint32_t)vids[1], (uint32_t)vids[2], 0u);
                counted = true;
                return 1;
            }
            if (kCached)
            {
                return 0;
            }
            float4* dst = f.varyings + slot * kVaryingVec4;
            const int nv = d.numVaryings;
#pragma unroll
            for (int k = 0; k < 3; ++k)
            {
                slg_v4 vary[kMaxVaryings];
                (void)P::vertex(d, f.tables, vids[k], inst, vary);
#pragma unroll
                for (int vi = 0; vi < kMaxVaryings; ++vi)
                {
                    if (vi < nv) dst[4 * k + vi] = to_f4(vary[vi]);
                }
            }
            counted = true;
            return 1;
        }
        return 0;
    }
    if (vis == 1)
    {
        if (clip_trivially_empty(clip))
        {
            return 0;
        }
        /* partially visible: queued for clip_kernel */
        const uint32_t q = atomicAdd(f.clipCount, 1u);
        f.clipQueue[q] = (uint32_t)slot;
        return 0;
    }
    return 0;
}

/*-----------------------------------------------------------------------------
 * Kernel 1b: clipping of the queued partially visible triangles
 * (SL_TriProcessor::clip_and_process_tris, SL_TriProcessor.cpp:370-519)
-----------------------------------------------------------------------------*/
template <class P>
__global__ void __launch_bounds__(128) clip_kernel(const Frame f)
{
    const uint32_t count = *f.clipCount;
    const int lane = threadIdx.x & 31;
    const int sl = lane & (kClipLanes - 1);
    const uint32_t pairs = gridDim.x * (blockDim.x >> 5);
    for (uint32_t q0 = 2u * (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)); q0 < count; q0 += 2u * pairs)
    {
        /* half h of the warp clips queue entry q0 + h */
        const uint32_t q = q0 + (uint32_t)(lane >> 4);
        const bool active = q < count;
        const uint64_t slot = active ? f.clipQueue[q] : 0u;
        const int di = (active && f.numDraws > 1) ? find_draw(f, slot) : 0;
        const DrawDesc& d = f.draws[di];
        const uint64_t local = slot - d.slotBase;
        const uint64_t inst = active ? udiv_slot(local, d.numTris) : 0u;
        const uint64_t tri = local - inst * d.numTris;
        const uint64_t i = d.elementBegin + 3u * tri;
        /* lanes 0..2 of the half: the triangle's vertices */
        uint64_t vid = 0;
        float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
        if (active && sl < 3)
        {
            vid = (d.indexType >= 0) ? read_index(d, i + sl) : (i + sl);
            if (d.cacheVerts)
            {
                vid += d.cacheBase + inst * d.cacheVerts;
                p = mat_mul(f.scissor, f.cachePos[vid]);
            }
            else
            {
                slg_v4 vary[4];
                p = mat_mul(f.scissor, to_f4(P::vertex(d, f.tables, vid, inst, vary)));
            }
        }
        const uint64_t primIndex = d.primBase + d.numElements * inst + i;
        const uint32_t info = clip_pair<P>(f, active, d, (uint32_t)di, slot, primIndex, inst, vid, p);
        if (active && sl == 0) f.slotInfo[slot] = info;
    }
}

/* Kernel 0: the post-transform vertex cache. One thread per entry runs the
 * vertex program once for its (draw, instance, vertex); SoftLight runs it for
 * every triangle corner (SL_TriProcessor.cpp:125-234), which gives the same
 * values, so the triangle stage reads positions here and the raster reads
 * varyings here. */
template <class P>
__global__ void __launch_bounds__(256) vertex_cache_kernel(const Frame f)
{
    const uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= f.cacheEntries)
    {
        return;
    }
    /* the owner is the last draw whose first entry is <= e (uncached draws
     * own no entries, so one with the same base is never the last) */
    int lo = 0, hi = f.numDraws - 1;
    while (lo < hi)
    {
        const int mid = (lo + hi + 1) >> 1;
        if (f.draws[mid].cacheBase <= e) lo = mid;
        else hi = mid - 1;
    }
    const DrawDesc& d = f.draws[lo];
    if (d.hidden)
    {
        return;
    }
    const uint64_t local = e - d.cacheBase;
    const uint64_t inst = udiv_slot(local, d.cacheVerts);
    const uint64_t vid = local - inst * d.cacheVerts;
    slg_v4 vary[kMaxVaryings];
    f.cachePos[e] = to_f4(P::vertex(d, f.tables, vid, inst, vary));
#pragma unroll
    for (int vi = 0; vi < kMaxVaryings; ++vi)
    {
        if (vi < d.numVaryings) f.cacheVary[(uint64_t)vi * f.cacheEntries + e] = to_f4(vary[vi]);
    }
}


/*-----------------------------------------------------------------------------
 * Kernel 4: tile raster + shade
-----------------------------------------------------------------------------*/
__device__ __forceinline__ bool depth_cmp(int func, float z, float d)
{
    switch (func)
    {
        case SLG_DEPTH_TEST_LESS_THAN:     return z < d;
        case SLG_DEPTH_TEST_LESS_EQUAL:    return z <= d;
        case SLG_DEPTH_TEST_GREATER_THAN:  return z > d;
        case SLG_DEPTH_TEST_GREATER_EQUAL: return z >= d;
        case SLG_DEPTH_TEST_EQUAL:         return z == d;
        case SLG_DEPTH_TEST_NOT_EQUAL:     return z != d;
        default:                           return true;
    }
}

/* Colour formats of the tile buffer in shared memory. */
struct ColorRGBA8
{
    typedef uint32_t stored;
    static __device__ __forceinline__ float4 load(stored v) { return unpack_rgba8(v); }
    static __device__ __forceinline__ stored store(float4 c)
    {
        return (uint32_t)f2u8(c.x * 255.f) | ((uint32_t)f2u8(c.y * 255.f) << 8) |
               ((uint32_t)f2u8(c.z * 255.f) << 16) | ((uint32_t)f2u8(c.w * 255.f) << 24);
    }
    static __device__ __forceinline__ stored read(const uint8_t* p, size_t i) { return reinterpret_cast<const uint32_t*>(p)[i]; }
    static __device__ __forceinline__ void write(uint8_t* p, size_t i, stored v) { reinterpret_cast<uint32_t*>(p)[i] = v; }
};

struct ColorRGBAF
{
    typedef float4 stored;
    static __device__ __forceinline__ float4 load(stored v) { return v; }
    static __device__ __forceinline__ stored store(float4 c) { return c; }
    static __device__ __forceinline__ stored read(const uint8_t* p, size_t i) { return reinterpret_cast<const float4*>(p)[i]; }
    static __device__ __forceinline__ void write(uint8_t* p, size_t i, stored v) { reinterpret_cast<float4*>(p)[i] = v; }
};

struct ColorRF
{
    typedef float stored;
    static __device__ __forceinline__ float4 load(stored v) { return make_float4(v, 0.f, 0.f, 1.f); }
    static __device__ __forceinline__ stored store(float4 c) { return c.x; }
    static __device__ __forceinline__ stored read(const uint8_t* p, size_t i) { return reinterpret_cast<const float*>(p)[i]; }
    static __device__ __forceinline__ void write(uint8_t* p, size_t i, stored v) { reinterpret_cast<float*>(p)[i] = v; }
};

/* assign_alpha_pixel blend formulas (SL_Framebuffer.cpp:316-349) */
__device__ __forceinline__ float4 blend_color(int mode, const float4 s, const float4 d)
{
    const float sa = s.w;
    const float modulation = 1.f - sa;
    float4 r;
    if (mode == SLG_BLEND_ALPHA)
    {
        const float dstMod = modulation * d.w;
        const float dstAlpha = dstMod + sa;
        const float rc = 1.f / dstAlpha;
        r = make_float4((s.x * sa + d.x * dstMod) * rc, (s.y * sa + d.y * dstMod) * rc, (s.z * sa + d.z * dstMod) * rc, dstAlpha);
    }
    else if (mode == SLG_BLEND_PREMULTIPLED_ALPHA)
    {
        r = make_float4(d.x * modulation + s.x, d.y * modulation + s.y, d.z * modulation + s.z, d.w * modulation + s.w);
    }
    else if (mode == SLG_BLEND_ADDITIVE)
    {
        r = make_float4(s.x * sa + d.x, s.y * sa + d.y, s.z * sa + d.z, s.w * sa + d.w);
    }
    else
    {
        r = make_float4(s.x * sa + d.x * modulation, s.y * sa + d.y * modulation, s.z * sa + d.z * modulation, s.w * sa + d.w * modulation);
    }
    r.x = lm_min(lm_max(r.x, 0.f), 1.f);
    r.y = lm_min(lm_max(r.y, 0.f), 1.f);
    r.z = lm_min(lm_max(r.z, 0.f), 1.f);
    r.w = lm_min(lm_max(r.w, 0.f), 1.f);
    return r;
}

/*-----------------------------------------------------------------------------
 * Colour formats (SL_ColorDataType 0..27: R / RG / RGB / RGBA of u8, u16,
 * u32, u64, half, float, double). A fragment output is written as
 * color_cast<T, float> (SL_Color.hpp:606-660): integers (T)(x * (float)max),
 * half and double by conversion; the blend reads color_cast<float, T> of the
 * texel padded by assign_alpha_pixel (SL_Framebuffer.cpp:268-312): missing
 * green / blue are the format's minimum and alpha its maximum, and a
 * three-component texel is read as (r, r, r, max). Float -> unsigned
 * conversions follow the reference as compiled for x86-64 (cvttss2si, with
 * 32-bit values taken from its 64-bit form and 64-bit ones from gcc's
 * two-range sequence), so e.g. 1.0 stores 0 in a u32 or u64 channel, as the
 * reference does.
-----------------------------------------------------------------------------*/
__device__ __forceinline__ int format_components(int type) { return type / 7 + 1; }
__device__ __forceinline__ int format_kind(int type) { return type % 7; }   /* 0 u8 1 u16 2 u32 3 u64 4 half 5 float 6 double */
__device__ __forceinline__ int kind_bytes(int kind) { return (kind == 0) ? 1 : (kind == 1 || kind == 4) ? 2 : (kind == 2 || kind == 5) ? 4 : 8; }

/* cvttss2si with a 64-bit destination: NaN and out of range give INT64_MIN */
__device__ __forceinline__ uint64_t cvt_f32_i64(float x)
{
    return (x >= -9223372036854775808.f && x < 9223372036854775808.f) ? (uint64_t)__float2ll_rz(x) : 0x8000000000000000ull;
}

__device__ __forceinline__ uint64_t f2u_x86(float x, int kind)
{
    if (kind <= 1) return (uint64_t)(uint32_t)f2i(x);            /* u8 / u16: 32-bit cvttss2si */
    if (kind == 2) return cvt_f32_i64(x) & 0xFFFFFFFFull;        /* u32: low half of the 64-bit form */
    if (!(x >= 9223372036854775808.f)) return cvt_f32_i64(x);     /* u64 below 2^63 (and NaN) */
    return cvt_f32_i64(x - 9223372036854775808.f) ^ 0x8000000000000000ull;
}

/* RGBA u32 texels: converting an out-of-range or NaN float to unsigned is
 * undefined in C++, and for four-lane u32 vectors the reference build
 * (x86-64 SSE2) emits the vectorised form: x >= 2^31 ? cvttps2dq(x - 2^31)
 * ^ 2^31 : cvttps2dq(x), where cvttps2dq gives 0x80000000 out of int32
 * range. In-range values convert identically either way. */
__device__ __forceinline__ uint32_t f2u32_vec(float x)
{
    const bool big = x >= 2147483648.f;
    const float y = big ? x - 2147483648.f : x;
    const uint32_t i = (y >= -2147483648.f && y < 2147483648.f) ? (uint32_t)__float2int_rz(y) : 0x80000000u;
    return big ? (i ^ 0x80000000u) : i;
}

__device__ __forceinline__ float kind_max(int kind)
{
    return (kind == 0) ? 255.f : (kind == 1) ? 65535.f : (kind == 2) ? 4294967295.f : 18446744073709551615.f;
}

/* component j of texel i as float (color_cast<float, T>) */
__device__ __forceinline__ float component_load(int kind, int nc, const uint8_t* p, size_t i, int j)
{
    const uint8_t* c = p + (i * (size_t)nc + (size_t)j) * (size_t)kind_bytes(kind);
    switch (kind)
    {
        case 0: return (float)c[0] * 0.00392156862745f;
        case 1: return (float)*reinterpret_cast<const uint16_t*>(c) * (1.f / 65535.f);
        case 2: return (float)*reinterpret_cast<const uint32_t*>(c) * (1.f / 4294967295.f);
        case 3: return (float)*reinterpret_cast<const unsigned long long*>(c) * (1.f / 18446744073709551615.f);
        case 4: return slg_half_to_float(*reinterpret_cast<const uint16_t*>(c));
        case 5: return *reinterpret_cast<const float*>(c);
        default: return (float)*reinterpret_cast<const double*>(c);
    }
}

/* the format's maximum as float (the padding of a missing alpha) */
__device__ __forceinline__ float kind_one(int kind)
{
    switch (kind)
    {
        case 0: return 255.f * 0.00392156862745f;
        case 1: return 65535.f * (1.f / 65535.f);
        case 2: return 4294967295.f * (1.f / 4294967295.f);
        case 3: return 18446744073709551615.f * (1.f / 18446744073709551615.f);
        default: return 1.f;
    }
}

__device__ __forceinline__ void component_store(int kind, int nc, uint8_t* p, size_t i, int j, float x)
{
    uint8_t* c = p + (i * (size_t)nc + (size_t)j) * (size_t)kind_bytes(kind);
    switch (kind)
    {
        case 0: c[0] = (uint8_t)f2u_x86(x * 255.f, 0); break;
        case 1: *reinterpret_cast<uint16_t*>(c) = (uint16_t)f2u_x86(x * 65535.f, 1); break;
        case 2: *reinterpret_cast<uint32_t*>(c) = (nc == 4) ? f2u32_vec(x * 4294967295.f) : (uint32_t)f2u_x86(x * 4294967295.f, 2); break;
        case 3: *reinterpret_cast<unsigned long long*>(c) = f2u_x86(x * 18446744073709551615.f, 3); break;
        case 4: *reinterpret_cast<uint16_t*>(c) = slg_float_to_half(x); break;
        case 5: *reinterpret_cast<float*>(c) = x; break;
        default: *reinterpret_cast<double*>(c) = (double)x; break;
    }
}

/* Packed texels. Read (rgba_cast<float, T>, SL_ColorCompressed.hpp:165-184
 * and its siblings): each field (float)c / (float)max, alpha 1 for RGB 332
 * and RGB 565. Write (rgba_cast<T, float>, :112-132 and siblings): each
 * field (uint8_t or uint16_t)(x * (float)max) - cvttss2si's 32-bit result,
 * the field keeping its low bits. */
static __device__ __noinline__ float4 packed_load(int type, const uint8_t* p, size_t i)
{
    const int nb = packed_bytes(type);
    const uint32_t bits = (nb == 1) ? (uint32_t)p[i]
                        : (nb == 2) ? (uint32_t)reinterpret_cast<const uint16_t*>(p)[i]
                                    : reinterpret_cast<const uint32_t*>(p)[i];
    const uint32_t w = packed_widths(type);
    const int nc = (type <= 29) ? 3 : 4;
    float v[4] = {0.f, 0.f, 0.f, 1.f};
    int shift = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j)
    {
        if (j < nc)
        {
            const int b = (int)((w >> (4 * j)) & 15u);
            const uint32_t mask = (1u << b) - 1u;
            v[j] = (float)((bits >> shift) & mask) / (float)mask;
            shift += b;
        }
    }
    return make_float4(v[0], v[1], v[2], v[3]);
}

static __device__ __noinline__ void packed_store(int type, uint8_t* p, size_t i, const float4 c)
{
    const uint32_t w = packed_widths(type);
    const int nc = (type <= 29) ? 3 : 4;
    const float v[4] = {c.x, c.y, c.z, c.w};
    uint32_t bits = 0;
    int shift = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j)
    {
        if (j < nc)
        {
            const int b = (int)((w >> (4 * j)) & 15u);
            const uint32_t mask = (1u << b) - 1u;
            bits |= ((uint32_t)f2i(v[j] * (float)mask) & mask) << shift;
            shift += b;
        }
    }
    const int nb = packed_bytes(type);
    if (nb == 1) p[i] = (uint8_t)bits;
    else if (nb == 2) reinterpret_cast<uint16_t*>(p)[i] = (uint16_t)bits;
    else reinterpret_cast<uint32_t*>(p)[i] = bits;
}

/* A texel of an attachment, as the float4 the blend reads and from the
 * float4 a fragment writes (the three core formats keep their fast forms). */
__device__ __forceinline__ float4 texel_load(int type, const uint8_t* p, size_t i)
{
    if (type == SLG_COLOR_RGBA_FLOAT) return ColorRGBAF::load(ColorRGBAF::read(p, i));
    if (type == SLG_COLOR_R_FLOAT) return ColorRF::load(ColorRF::read(p, i));
    if (type == SLG_COLOR_RGBA_8U) return ColorRGBA8::load(ColorRGBA8::read(p, i));
    if (type >= kFirstPacked) return packed_load(type, p, i);
    const int nc = format_components(type), kind = format_kind(type);
    const float r = component_load(kind, nc, p, i, 0);
    if (nc == 1) return make_float4(r, 0.f, 0.f, kind_one(kind));
    if (nc == 3) return make_float4(r, r, r, kind_one(kind));
    const float g = component_load(kind, nc, p, i, 1);
    if (nc == 2) return make_float4(r, g, 0.f, kind_one(kind));
    return make_float4(r, g, component_load(kind, nc, p, i, 2), component_load(kind, nc, p, i, 3));
}

__device__ __forceinline__ void texel_store(int type, uint8_t* p, size_t i, const float4 c)
{
    if (type == SLG_COLOR_RGBA_FLOAT) ColorRGBAF::write(p, i, ColorRGBAF::store(c));
    else if (type == SLG_COLOR_R_FLOAT) ColorRF::write(p, i, ColorRF::store(c));
    else if (type == SLG_COLOR_RGBA_8U) ColorRGBA8::write(p, i, ColorRGBA8::store(c));
    else if (type >= kFirstPacked) packed_store(type, p, i, c);
    else
    {
        const int nc = format_components(type), kind = format_kind(type);
        const float v[4] = {c.x, c.y, c.z, c.w};
        for (int j = 0; j < nc; ++j) component_store(kind, nc, p, i, j, v[j]);
    }
}

/* Outputs 1..3 of a fragment into colour attachments 1..3, blended per
 * attachment: the reference's output mask writes pOutputs[k] to attachment k
 * for every k below the program's output count (SL_FragmentProcessor.cpp:
 * 376-395, SL_Framebuffer.cpp:1207-1231). reps: the fragment's visits. */
__device__ __forceinline__ void emit_extra_outputs(const Frame& f, const DrawDesc& dd, size_t gi, const slg_v4* outputs, int reps)
{
    const int n = min((int)dd.numOutputs, f.numColors);
    for (int k = f.generic0 ? 0 : 1; k < n; ++k)
    {
        uint8_t* p = f.colors[k];
        const int t = f.colorTypes[k];
        const float4 o = to_f4(outputs[k]);
        for (int r = 0; r < reps; ++r)
        {
            texel_store(t, p, gi, (dd.blend != SLG_BLEND_OFF) ? blend_color(dd.blend, o, texel_load(t, p, gi)) : o);
        }
    }
}

__device__ __forceinline__ uint64_t key_to_record(const Frame& f, uint32_t key)
{
    if (f.recOfRank)
    {
        return f.recOfRank[key];
    }
    const uint64_t slot = key >> kSubShift;
    const uint32_t sub = key & ((1u << kSubShift) - 1u);
    return (sub == 0) ? slot : (f.numSlots + f.slotOvf[slot] + (sub - 1));
}

/* In-place ascending bitonic sort of n keys in shared memory (n <= cap, cap a
 * power of two); entries n..p-1 are padded with 0xFFFFFFFF. */
static __device__ void sort_keys(uint32_t* s, int n)
{
    int p = 2;
    while (p < n) p <<= 1;
    for (int i = n + threadIdx.x; i < p; i += blockDim.x) s[i] = 0xFFFFFFFFu;
    __syncthreads();

    int unsorted = 0;
    for (int i = threadIdx.x; i + 1 < n; i += blockDim.x) unsorted |= (s[i] > s[i + 1]);
    if (!__syncthreads_or(unsorted))
    {
        return;
    }

    for (int k = 2; k <= p; k <<= 1)
    {
        for (int j = k >> 1; j > 0; j >>= 1)
        {
            for (int i = threadIdx.x; i < p; i += blockDim.x)
            {
                const int ixj = i ^ j;
                if (ixj > i)
                {
                    const uint32_t a = s[i], b = s[ixj];
                    const bool up = ((i & k) == 0);
                    if ((a > b) == up)
                    {
                        s[i] = b;
                        s[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
}

/* Per-triangle constants a thread needs for one scan-line. */
struct Span
{
    int32_t xMin, xMax;
};

/* SL_ScanlineBounds::step, portable branch (SL_ScanlineBounds.hpp:301-321) */
__device__ __forceinline__ Span scanline_span(const float4 r0, const float4 r1, float yf)
{
    const float d0 = yf - r0.x;
    const float d1 = yf - r0.y;
    const float alpha = d0 * r1.x;
    const int32_t lo = f2i(r1.y * alpha + r0.z);
    const int32_t sa = f2i(r1.z * d1 + r0.w);
    const int32_t sb = f2i(r1.w * d0 + r0.z);
    const int32_t hi = (d1 < 0.f) ? sa : sb;
    Span s;
    s.xMin = (lo >= hi) ? hi : lo;
    s.xMax = (lo >= hi) ? lo : hi;
    return s;
}

/* One thread's walk over the pixels x = xs + 4g of a scan-line span that lie
 * in [xFirst, xEnd): the incremental barycentrics of
 * SL_TriRasterizer.cpp:856-911 replayed exactly (bc0*xs + bcY, then one
 * addition of 4*bc0 per step, including the steps left of the tile). */
struct Chain
{
    float b0, b1, b2;       /* barycentrics at the current pixel */
    float s0, s1, s2;       /* 4 * bc0 */
    int x, xEnd;
};

/* The chain of the column class of myX0 (pixels myX0 + 4k below xLimit) on
 * a scan-line whose span sp is known to be non-empty. */
__device__ __forceinline__ bool chain_begin_span(const float4* R, float yf, const Span sp, int myX0, int xLimit, Chain& ch)
{
    const int xEnd = min(sp.xMax, xLimit);
    const int xs = sp.xMin + ((myX0 - sp.xMin) & 3);
    const int xFirst = max(xs, myX0);
    if (xFirst >= xEnd)
    {
        return false;
    }
    const float4 r2 = R[2], r3 = R[3], r4 = R[4];
    const float bcY0 = r3.x * yf + r4.x;
    const float bcY1 = r3.y * yf + r4.y;
    const float bcY2 = r3.z * yf + r4.z;
    const float xsf = (float)xs;
    ch.b0 = r2.x * xsf + bcY0;
    ch.b1 = r2.y * xsf + bcY1;
    ch.b2 = r2.z * xsf + bcY2;
    ch.s0 = r2.x * 4.f;
    ch.s1 = r2.y * 4.f;
    ch.s2 = r2.z * 4.f;
    for (int g = (xFirst - xs) >> 2; g > 0; --g)
    {
        ch.b0 += ch.s0;
        ch.b1 += ch.s1;
        ch.b2 += ch.s2;
    }
    ch.x = xFirst;
    ch.xEnd = xEnd;
    return true;
}

__device__ __forceinline__ bool chain_begin(const float4* R, float yf, int myX0, int xLimit, Chain& ch)
{
    const Span sp = scanline_span(R[0], R[1], yf);
    if (!((uint32_t)sp.xMin < (uint32_t)sp.xMax))
    {
        return false;
    }
    return chain_begin_span(R, yf, sp, myX0, xLimit, ch);
}

__device__ __forceinline__ void chain_step(Chain& ch)
{
    ch.b0 += ch.s0;
    ch.b1 += ch.s1;
    ch.b2 += ch.s2;
    ch.x += 4;
}

/* z = dot(depth, bc) with depth.w = 0 (SL_TriRasterizer.cpp:880) */
__device__ __forceinline__ float chain_depth(const float4* R, const Chain& ch)
{
    const float4 r2 = R[2], r3 = R[3], r4 = R[4], r5 = R[5];
    return __fadd_rn((r3.w * ch.b0 + r4.w * ch.b1) + r5.x * ch.b2, 0.f * r2.w);
}

/*-----------------------------------------------------------------------------
 * Wireframe (SL_TriRasterizer::render_wireframe, SL_TriRasterizer.cpp:116-204):
 * the same triangle records; per scan-line the left run of d0 pixels from the
 * span's start and, when the span is longer, the right run
 * [max(xMin, xMax - d1 - 1) + 1, xMax), where d0 / d1 are how far the span's
 * ends moved since the row above (at least 1). The runs overlap on narrow
 * rows: those pixels are visited twice with the same fragment. Barycentrics
 * are evaluated directly per pixel, bc = bc0 * x + (bc1 * y + bc2).
-----------------------------------------------------------------------------*/
constexpr uint32_t kFragQueue = 600;      /* SL_SHADER_MAX_QUEUED_FRAGS */

struct WireRow { int a0, a1, b0, b1; };   /* runs [a0, a1) and [b0, b1) */

__device__ __forceinline__ int abs_diff_wrap(int32_t a, int32_t b)
{
    const uint32_t d = (uint32_t)a - (uint32_t)b;
    return (int)(((int32_t)d < 0) ? (0u - d) : d);
}

__device__ __forceinline__ WireRow wire_row(const float4* R, float yf)
{
    WireRow w;
    w.a0 = w.a1 = w.b0 = w.b1 = 0;
    const Span s0 = scanline_span(R[0], R[1], yf);
    if (!((uint32_t)s0.xMin < (uint32_t)s0.xMax))
    {
        return w;
    }
    const Span s1 = scanline_span(R[0], R[1], yf - 1.f);
    const int d0 = max(abs_diff_wrap(s0.xMin, s1.xMin), 1);
    const int d1 = max(abs_diff_wrap(s0.xMax, s1.xMax), 1);
    const long long reach = (long long)s0.xMin + d0;
    w.a0 = s0.xMin;
    if (reach < (long long)s0.xMax)
    {
        w.a1 = (int)reach;
        w.b0 = max(s0.xMin, (int)((uint32_t)s0.xMax - (uint32_t)d1 - 1u)) + 1;
        w.b1 = s0.xMax;
    }
    else
    {
        w.a1 = s0.xMax;
    }
    return w;
}

/* visits of pixel x on a wire row: 0, 1 or 2 */
__device__ __forceinline__ int wire_visits(const WireRow& w, int x)
{
    return (x >= w.a0 && x < w.a1 ? 1 : 0) + (x >= w.b0 && x < w.b1 ? 1 : 0);
}

/* direct barycentrics and depth of pixel x on the row whose bcY is given */
__device__ __forceinline__ float wire_fragment(const float4* R, float bcY0, float bcY1, float bcY2, int x, float& b0, float& b1, float& b2)
{
    const float4 r2 = R[2], r3 = R[3], r4 = R[4], r5 = R[5];
    const float xf = (float)x;
    b0 = r2.x * xf + bcY0;
    b1 = r2.y * xf + bcY1;
    b2 = r2.z * xf + bcY2;
    return __fadd_rn((r3.w * b0 + r4.w * b1) + r5.x * b2, 0.f * r2.w);
}

/* A blended wireframe triangle can have a queue flush between the two
 * visits of a pixel, after which the second is tested against the first
 * one's write. That needs 600 queued fragments before the second visit, which
 * comes right after the row's left run; when some row with a revisited pixel
 * has that many visits before it, the order is not replayed (the two visits
 * are applied as one unflushed queue) and the launch reports
 * kStatusWireQueue. */
static __device__ __noinline__ void wire_queue_check(const Frame& f, const float4* R)
{
    const int minY = __float_as_int(R[6].x), maxY = __float_as_int(R[6].y);
    long long visits = 0;
    for (int y = minY; y < maxY; ++y)
    {
        const WireRow w = wire_row(R, (float)y);
        const bool twice = w.b1 > w.b0 && w.b0 < w.a1;
        if (twice && visits + (long long)(w.a1 - w.a0) >= (long long)kFragQueue)
        {
            atomicOr(f.status, kStatusWireQueue);
            return;
        }
        visits += (long long)(w.a1 - w.a0) + (long long)(w.b1 - w.b0);
    }
}

/* SL_FragCoordXYZ of a fragment (softlight/include/softlight/SL_ShaderUtil.hpp:
 * 668-673): the 16-bit screen coordinates and the depth the fragment was
 * tested with. */
__device__ __forceinline__ slg_frag_coord frag_coord(uint32_t x, uint32_t y, float depth)
{
    slg_frag_coord c;
    c.x = (uint16_t)x;
    c.y = (uint16_t)y;
    c.depth = depth;
    return c;
}

/* A point's coordinates as SL_PointRasterizer::render_point sets them
 * ((uint16_t) of the screen position, SL_PointRasterizer.cpp:47-50) and its
 * depth. */
__device__ __forceinline__ slg_frag_coord point_coord(const float4* R)
{
    const float4 r0 = R[0];
    return frag_coord((uint32_t)f2i(r0.x) & 0xFFFFu, (uint32_t)f2i(r0.y) & 0xFFFFu, r0.z);
}

/* The fragment program's outputs 1..3 (attachments 1..3, or 0..3 when
 * attachment 0 is not a core format) once the program has run. */
template <bool kExtra>
__device__ __forceinline__ void shade_extra(const Frame& f, const DrawDesc& dd, bool kept, const slg_v4* outputs, size_t gi, int reps)
{
    if (kExtra && kept && (f.numColors > 1 || f.generic0))
    {
        emit_extra_outputs(f, dd, gi, outputs, reps);
    }
}

/* Whether a fragment the program kept writes colour attachment 0. */
__device__ __forceinline__ bool writes_color(const DrawDesc& dd, bool kept) { return kept && dd.numOutputs > 0; }

/* Perspective correction, varying interpolation and the fragment program of
 * SL_FragmentProcessor::flush_tri_fragments (SL_FragmentProcessor.cpp:463-529,
 * interpolate_tri_varyings :308-330). fc is the fragment's SL_FragCoordXYZ
 * (x, y, depth) going in and what the program leaves in it coming out (the
 * reference writes fc.depth to the depth buffer after the program). Returns
 * the program's result: false when it discarded the fragment. */
template <class P, bool kExtra>
__device__ __forceinline__ bool shade(const Frame& f, const DrawDesc& dd, uint64_t rec, uint32_t recFlags, float bcw, const float4 r5,
                                      float b0, float b1, float b2, slg_frag_coord& fc, float4& out, size_t gi = 0, int reps = 1)
{
    const float bp0 = b0 * r5.y, bp1 = b1 * r5.z, bp2 = b2 * r5.w;
    const float bp3 = bcw * 0.f;
    const float persp = 1.f / (((bp0 + bp1) + bp2) + bp3);
    const float q0 = bp0 * persp, q1 = bp1 * persp, q2 = bp2 * persp;

    slg_v4 vary[4];
    /* varying vi of corner k is V_k[vi * stride]: planes of the vertex
     * cache, or the record's own copies */
    const float4 *V0, *V1, *V2;
    size_t stride;
    if (recFlags & kRecordCached)
    {
        const uint4 e = f.recVerts[rec];
        V0 = f.cacheVary + e.x;
        V1 = f.cacheVary + e.y;
        V2 = f.cacheVary + e.z;
        stride = (size_t)f.cacheEntries;
    }
    else
    {
        V0 = f.varyings + rec * kVaryingVec4;
        V1 = V0 + 4;
        V2 = V0 + 8;
        stride = 1;
    }
    const int nv = dd.numVaryings;
#pragma unroll
    for (int vi = 0; vi < kMaxVaryings; ++vi)
    {
        if (vi < nv)
        {
            const float4 a = V0[vi * stride], b = V1[vi * stride], c = V2[vi * stride];
            vary[vi] = slg_make_v4((a.x * q0 + b.x * q1) + c.x * q2, (a.y * q0 + b.y * q1) + c.y * q2,
                                   (a.z * q0 + b.z * q1) + c.z * q2, (a.w * q0 + b.w * q1) + c.w * q2);
        }
        else
        {
            vary[vi] = slg_make_v4(0.f, 0.f, 0.f, 0.f);
        }
    }
    slg_v4 outputs[4];
    const bool kept = P::fragment(dd, f.tables, fc, vary, outputs);
    out = to_f4(outputs[0]);
    shade_extra<kExtra>(f, dd, kept, outputs, gi, reps);
    return kept;
}

/* SL_PointRasterizer::render_point's shading (SL_PointRasterizer.cpp:59-90):
 * the point's varyings are handed to the fragment program unchanged. */
template <class P, bool kExtra>
__device__ __forceinline__ bool shade_point(const Frame& f, const DrawDesc& dd, uint64_t rec, slg_frag_coord& fc, float4& out, size_t gi = 0,
                                            int reps = 1)
{
    slg_v4 vary[kMaxVaryings];
    const float4* V = f.varyings + rec * kVaryingVec4;
#pragma unroll
    for (int vi = 0; vi < kMaxVaryings; ++vi)
    {
        const float4 v = (vi < dd.numVaryings) ? V[vi] : make_float4(0.f, 0.f, 0.f, 0.f);
        vary[vi] = slg_make_v4(v.x, v.y, v.z, v.w);
    }
    slg_v4 outputs[4];
    const bool kept = P::fragment(dd, f.tables, fc, vary, outputs);
    out = to_f4(outputs[0]);
    shade_extra<kExtra>(f, dd, kept, outputs, gi, reps);
    return kept;
}

/* SL_LineRasterizer's fragment shading (SL_FragmentProcessor.cpp:346-402,
 * interpolate_line_varyings :120-140): varyings mix(v0, v1, interp). */
template <class P, bool kExtra>
__device__ __forceinline__ bool shade_line(const Frame& f, const DrawDesc& dd, uint64_t rec, float interp, slg_frag_coord& fc, float4& out,
                                           size_t gi = 0, int reps = 1)
{
    slg_v4 vary[kMaxVaryings];
    const float4* V = f.varyings + rec * kVaryingVec4;
#pragma unroll
    for (int vi = 0; vi < kMaxVaryings; ++vi)
    {
        if (vi < dd.numVaryings)
        {
            const float4 a = V[vi], b = V[4 + vi];
            vary[vi] = slg_make_v4(mixf(a.x, b.x, interp), mixf(a.y, b.y, interp), mixf(a.z, b.z, interp), mixf(a.w, b.w, interp));
        }
        else
        {
            vary[vi] = slg_make_v4(0.f, 0.f, 0.f, 0.f);
        }
    }
    slg_v4 outputs[4];
    const bool kept = P::fragment(dd, f.tables, fc, vary, outputs);
    out = to_f4(outputs[0]);
    shade_extra<kExtra>(f, dd, kept, outputs, gi, reps);
    return kept;
}

/* Shared-memory pitch of a staged record: its 8 vectors and one unused, so
 * that lanes reading one vector of 32 different records spread over the
 * banks (a 128-byte pitch puts them all in the same four). */
constexpr int kStagedVec4 = kRecordVec4 + 1;

template <int TW, int TH, class Color>
struct RasterLayout
{
    static constexpr int kThreads = TH * 4;
    static constexpr int kStride = TW + 4;       /* row pitch of the tile buffers (bank spread) */
    static constexpr int kBatch = 48;            /* records staged per step (two buffers: 7 CTAs of 64x32 RGBA8 fit an SM) */
    static constexpr int kPix = TH * kStride;
    static constexpr size_t kRecBytes = sizeof(float4) * kBatch * kStagedVec4;
    /* ordered path: colour + depth tile, two record buffers (one batch is
     * walked while the next arrives), their keys, then each tile row's and
     * each 8-row band's depth range (lo, hi) at the start of a batch */
    static constexpr size_t kRecOff = sizeof(typename Color::stored) * kPix + sizeof(float) * kPix;
    static constexpr size_t kKeyOff = kRecOff + 2 * kRecBytes;
    static constexpr size_t kRowDOff = kKeyOff + 2 * sizeof(uint32_t) * kBatch;
    static constexpr size_t kBandDOff = kRowDOff + 2 * sizeof(float) * TH;
    /* the survivor count of each warp while a batch is gathered, and where
     * the next gathering resumes */
    static constexpr size_t kScanOff = kBandDOff + 2 * sizeof(float) * (TH / 8);
    static constexpr size_t ordered_bytes() { return kScanOff + sizeof(uint32_t) * (TH / 8 + 1); }
};

/* Starts copying records [b0, b0+cnt) of the tile list into shared memory
 * (cp.async, one commit group per call); their keys are stored directly.
 * The copies are complete for the calling thread after cp_async_wait, and
 * for the block after a barrier that follows it. */
__device__ __forceinline__ void stage_records_async(const Frame& f, const uint32_t* keys, int cnt, float4* sRec, uint32_t* sKey)
{
    for (int i = threadIdx.x; i < cnt * kRecordVec4; i += blockDim.x)
    {
        const int ri = i / kRecordVec4, part = i % kRecordVec4;
        const uint32_t key = keys[ri];
        if (part == 0) sKey[ri] = key;
        const float4* src = f.records + key_to_record(f, key) * kRecordVec4 + part;
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(sRec + ri * kStagedVec4 + part);
        asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src) : "memory");
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}

/* Waits for this thread's copies of all groups but the newest `pending`. */
template <int pending>
__device__ __forceinline__ void cp_async_wait()
{
    asm volatile("cp.async.wait_group %0;\n" ::"n"(pending) : "memory");
}

/* Stages records [b0, b0+cnt) of the tile list into shared memory. */
template <int Batch>
__device__ __forceinline__ void stage_records(const Frame& f, const uint32_t* keys, int cnt, float4* sRec, uint32_t* sKey)
{
    for (int i = threadIdx.x; i < cnt * kRecordVec4; i += blockDim.x)
    {
        const int ri = i / kRecordVec4, part = i % kRecordVec4;
        const uint32_t key = keys[ri];
        if (part == 0) sKey[ri] = key;
        sRec[ri * kStagedVec4 + part] = f.records[key_to_record(f, key) * kRecordVec4 + part];
    }
}

/* The warp owns rows [bandY0, bandY0 + 8): the 32 lanes test 32 staged
 * records at once against that band and the warp walks only the hits, in
 * order (ballot + find-first-set compaction). keep(ri, r6, lo, hi) may drop
 * a hit whose walk can change nothing, and bound its depths in the band;
 * fn(ri, lo, hi) walks it. */
template <class Keep, class Fn>
__device__ __forceinline__ void for_band_records(const float4* sRec, int cnt, int bandY0, Keep&& keep, Fn&& fn)
{
    const int lane = threadIdx.x & 31;
    for (int base = 0; base < cnt; base += 32)
    {
        const int ri = base + lane;
        bool hit = false;
        /* keep may narrow the record's depths in the band to [lo, hi] */
        float lo = __int_as_float(0xFF800000), hi = __int_as_float(0x7F800000);
        if (ri < cnt)
        {
            const float4 r6 = sRec[ri * kStagedVec4 + 6];
            hit = __float_as_int(r6.x) < bandY0 + 8 && __float_as_int(r6.y) > bandY0 && keep(ri, r6, lo, hi);
        }
        unsigned mask = __ballot_sync(0xFFFFFFFFu, hit);
        while (mask)
        {
            const int j = __ffs(mask) - 1;
            mask &= mask - 1;
            fn(base + j, __shfl_sync(0xFFFFFFFFu, lo, j), __shfl_sync(0xFFFFFFFFu, hi, j));
        }
    }
}

/*-----------------------------------------------------------------------------
 * Ordered raster: blending or order-dependent depth state. Keys are sorted
 * and every thread applies, for the pixels it owns, each fragment in
 * submission order: depth test, fragment program, blend, depth write.
-----------------------------------------------------------------------------*/
/* Whether the ordered raster renders this launch: always when it is not
 * order-free, and for an order-free launch whose line draws logged address
 * aliases (the order-free raster then stands aside). */
__device__ __forceinline__ bool ordered_raster_runs(const Frame& f)
{
    return !f.orderFree || (f.aliasCount != nullptr && *f.aliasCount != 0u);
}

/* Largest screen coordinate for which depth_range_rect holds: below it the
 * scan-line span arithmetic errs by far less than a pixel, so every span
 * lies in the record's [minX - 1, maxX + 1] (screen vertices are whole
 * pixels: to_screen floors them), as the tile binning also relies on. */
constexpr int kRectBoundMaxX = 1 << 20;

/* The depths a triangle record's walk can produce on rows [ya, yb] of
 * columns [xa, xb], as [lo, hi]. A fragment's depth, as the walk computes it
 * (chain_begin_span / chain_step / chain_depth), is the plane z = A x + B y
 * + C of the record's barycentric gradients plus rounding: the start value
 * bc0 * xs + (bc1 * y + bc2) (terms of size Binit, a few roundings), then k
 * additions of 4 * bc0 to values of size at most Bchain (one rounding each,
 * |error| <= 2^-24 * |value|), then the depth dot product (three roundings
 * on terms |z_i b_i|). The margin counts each rounding at 2^-21, eight
 * times the unit roundoff. Each walked chain starts at some xs in [xsMin,
 * xb] (xsMin <= the span's start, >= 0) and ends by xb; the plane takes its
 * extremes over the rectangle at its corners, and the rounding terms take
 * the largest start (|bc0| xb + |bc1| yb + |bc2|) and chain values (the
 * corners of [xsMin, xb] x [ya, yb], the barycentrics being affine) and the
 * longest chain, so the margin bounds the one of every walk there. NaNs
 * make the range NaN, which rejects nothing. */
__device__ __forceinline__ void depth_range_rect(const float4* R, int ya, int yb, int xa, int xb, int xsMin, float& lo, float& hi)
{
    const float4 r2 = R[2], r3 = R[3], r4 = R[4];
    const float z0 = r3.w, z1 = r4.w, z2 = R[5].x;
    const float bx[3] = {r2.x, r2.y, r2.z};
    const float ry[3] = {r3.x, r3.y, r3.z};
    const float rc[3] = {r4.x, r4.y, r4.z};
    const float yaf = (float)ya, ybf = (float)yb, xaf = (float)xa, xbf = (float)xb, xsf = (float)xsMin;
    float byA[3], byB[3];
    float binit = 0.f, bchain = 0.f;
#pragma unroll
    for (int i = 0; i < 3; ++i)
    {
        byA[i] = ry[i] * yaf + rc[i];
        byB[i] = ry[i] * ybf + rc[i];
        binit = fmaxf(binit, fabsf(bx[i] * xbf) + fabsf(ry[i] * ybf) + fabsf(rc[i]));
        bchain = fmaxf(bchain, fmaxf(fmaxf(fabsf(bx[i] * xsf + byA[i]), fabsf(bx[i] * xbf + byA[i])),
                                     fmaxf(fabsf(bx[i] * xsf + byB[i]), fabsf(bx[i] * xbf + byB[i]))));
    }
    const float A = (z0 * bx[0] + z1 * bx[1]) + z2 * bx[2];
    const float CA = (z0 * byA[0] + z1 * byA[1]) + z2 * byA[2];
    const float CB = (z0 * byB[0] + z1 * byB[1]) + z2 * byB[2];
    const float zaa = A * xaf + CA, zba = A * xbf + CA, zab = A * xaf + CB, zbb = A * xbf + CB;
    const float k = (float)((xb - xsMin) / 4 + 1);
    const float zs = (fabsf(z0) + fabsf(z1)) + fabsf(z2);
    const float margin = 4.76837158203125e-07f * zs * (4.f * binit + (k + 8.f) * bchain);   /* 2^-21 */
    lo = fminf(fminf(zaa, zba), fminf(zab, zbb)) - margin;
    hi = fmaxf(fmaxf(zaa, zba), fmaxf(zab, zbb)) + margin;
}

/* Whether no fragment of depth in [lo, hi] passes func against stored
 * depths in [dMin, dMax] (NaNs reject nothing). */
__device__ __forceinline__ bool depth_range_rejects(int func, float lo, float hi, float dMin, float dMax)
{
    switch (func)
    {
        case SLG_DEPTH_TEST_LESS_THAN:     return lo >= dMax;
        case SLG_DEPTH_TEST_LESS_EQUAL:    return lo > dMax;
        case SLG_DEPTH_TEST_GREATER_THAN:  return hi <= dMin;
        case SLG_DEPTH_TEST_GREATER_EQUAL: return hi < dMin;
        default:                           return false;
    }
}

/* Whether no pixel of the tile (rows [y0, yEnd), columns [x0, xLimit)) can
 * take a fragment of the staged triangle record R: depth_range_rect over the
 * record's box in the tile against the depth range of the 8-row bands the
 * box spans (bandD: (lo, hi) per band). A record whose box misses the tile's
 * columns has no pixel there either. Line, wireframe and point records, and
 * boxes reaching kRectBoundMaxX, are never rejected. */
__device__ __forceinline__ bool tile_rejects(const float4* R, const float4 r6, int y0, int yEnd, int x0, int xLimit, const float* bandD)
{
    const uint32_t flags = __float_as_uint(R[7].w);
    const int minX = __float_as_int(r6.z), maxX = __float_as_int(r6.w);
    if ((flags & (kRecordLine | kRecordWire | kRecordPoint)) || maxX >= kRectBoundMaxX || maxX < minX)
    {
        return false;
    }
    const int ya = max(__float_as_int(r6.x), y0);
    const int yb = min(__float_as_int(r6.y), yEnd) - 1;
    const int xsMin = max(minX - 2, 0);
    const int xa = max(x0, xsMin), xb = min(xLimit - 1, maxX);
    if (yb < ya || xb < xa)
    {
        return true;
    }
    float lo = __int_as_float(0x7F800000), hi = __int_as_float(0xFF800000);
    for (int b = (ya - y0) >> 3; b <= (yb - y0) >> 3; ++b)
    {
        lo = fminf(lo, bandD[2 * b]);
        hi = fmaxf(hi, bandD[2 * b + 1]);
    }
    float zlo, zhi;
    depth_range_rect(R, ya, yb, xa, xb, xsMin, zlo, zhi);
    return depth_range_rejects(flags & 0xF, zlo, zhi, lo, hi);
}

/* kGeneral: the instantiation that carries line and wireframe records and
 * writes several render targets (such launches use kLineTile tiles); the
 * others keep the triangle loop's registers. */
template <class P, int TW, int TH, class Color, bool kGeneral>
__global__ void __launch_bounds__(TH * 4, kGeneral ? 512 / (TH * 4) : 896 / (TH * 4)) raster_ordered_kernel(const Frame f)
{
    typedef RasterLayout<TW, TH, Color> L;
    typedef typename Color::stored Stored;
    extern __shared__ __align__(16) uint8_t smem[];
    Stored*   sColor = reinterpret_cast<Stored*>(smem);
    float*    sDepth = reinterpret_cast<float*>(smem + sizeof(Stored) * L::kPix);
    float4*   sRecBuf = reinterpret_cast<float4*>(smem + L::kRecOff);
    uint32_t* sKeyBuf = reinterpret_cast<uint32_t*>(smem + L::kKeyOff);
    float*    sRowD  = reinterpret_cast<float*>(smem + L::kRowDOff);
    float*    sBandD = reinterpret_cast<float*>(smem + L::kBandDOff);
    uint32_t* sScan  = reinterpret_cast<uint32_t*>(smem + L::kScanOff);

    /* longest tile lists first (tile_scan_kernel), so that the short ones
     * fill in behind them */
    const int tile = f.tileOrder ? (int)f.tileOrder[blockIdx.x] : (int)blockIdx.x;
    const uint32_t begin = f.tileOffset[tile];
    const uint32_t n = f.tileOffset[tile + 1] - begin;
    if (n == 0 || (f.status[0] & kStatusSticky) || !ordered_raster_runs(f))
    {
        return;
    }
    const uint32_t* sKeys = f.entries + begin; /* sorted by tile_sort_kernel */
    const bool halfDepth = f.depthType == SLG_COLOR_R_HALF;

    const int tx = tile % f.tilesX, ty = tile / f.tilesX;
    const int x0 = tx * TW, y0 = ty * TH;

    for (int i = threadIdx.x; i < TW * TH; i += blockDim.x)
    {
        const int px = i % TW, py = i / TW;
        const int gx = x0 + px, gy = y0 + py;
        if (gx < f.width && gy < f.height)
        {
            const size_t gi = (size_t)gx + (size_t)f.width * gy;
            sDepth[py * L::kStride + px] = depth_load(f, gi);
            if (f.color) sColor[py * L::kStride + px] = Color::read(f.color, gi);
        }
    }
    __syncthreads();

    const int r = threadIdx.x >> 2;
    const int c = threadIdx.x & 3;
    const int y = y0 + r;
    const int myX0 = x0 + c;
    const int xLimit = min(x0 + TW, f.width);
    const bool rowActive = (y < f.height);
    const float yf = (float)y;
    const int bandY0 = y0 + ((threadIdx.x >> 5) << 3);

    /* the depth range of this thread's pixels at the start of a batch: a
     * bound for the whole batch, since depth only moves one way
     * (Frame::depthBound); each tile row's range for the warp-wide record
     * test and each 8-row band's for the tile-wide one */
    float dMin = 0.f, dMax = 0.f;
    const auto batch_ranges = [&]() {
        if (f.depthBound && rowActive)
        {
            dMin = __int_as_float(0x7F800000);
            dMax = -dMin;
            for (int x = myX0; x < xLimit; x += 4)
            {
                const float d = sDepth[r * L::kStride + (x - x0)];
                dMin = fminf(dMin, d);
                dMax = fmaxf(dMax, d);
            }
        }
        if (f.depthBound)
        {
            float rowLo = rowActive ? dMin : __int_as_float(0x7F800000);
            float rowHi = rowActive ? dMax : __int_as_float(0xFF800000);
            rowLo = fminf(rowLo, __shfl_xor_sync(0xFFFFFFFFu, rowLo, 1));
            rowHi = fmaxf(rowHi, __shfl_xor_sync(0xFFFFFFFFu, rowHi, 1));
            rowLo = fminf(rowLo, __shfl_xor_sync(0xFFFFFFFFu, rowLo, 2));
            rowHi = fmaxf(rowHi, __shfl_xor_sync(0xFFFFFFFFu, rowHi, 2));
            if (c == 0)
            {
                sRowD[2 * r] = rowLo;
                sRowD[2 * r + 1] = rowHi;
            }
            if (!kGeneral)
            {
#pragma unroll
                for (int o = 4; o < 32; o <<= 1)
                {
                    rowLo = fminf(rowLo, __shfl_xor_sync(0xFFFFFFFFu, rowLo, o));
                    rowHi = fmaxf(rowHi, __shfl_xor_sync(0xFFFFFFFFu, rowHi, o));
                }
                if ((threadIdx.x & 31) == 0)
                {
                    sBandD[2 * (threadIdx.x >> 5)] = rowLo;
                    sBandD[2 * (threadIdx.x >> 5) + 1] = rowHi;
                }
            }
        }
    };

    /* Triangle launches under a depth bound gather each batch: the threads
     * test list entries [cursor, cursor + blockDim) straight from the
     * records (one each, tile_rejects against the bands' ranges at the
     * start of the batch), and only the records that can pass somewhere in
     * the tile are copied into the staging buffers, in list order, up to
     * kGather of them; the rest of the list is resumed at the first record
     * that did not fit. Most records of a deep scene end there, so the
     * batches, their barriers and their depth ranges are few. */
    constexpr int kGather = 2 * L::kBatch;
    const int nWarps = (int)(blockDim.x >> 5);
    const int yEnd = min(y0 + TH, f.height);
    const auto gather = [&](uint32_t& cursor) -> int {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        int cnt = 0;
        while (cnt < kGather && cursor < n)
        {
            const uint32_t i = cursor + threadIdx.x;
            bool take = false;
            uint32_t key = 0;
            const float4* Rg = f.records;
            float4 Rl[8];
            if (i < n)
            {
                key = sKeys[i];
                Rg = f.records + key_to_record(f, key) * kRecordVec4;
#pragma unroll
                for (int j = 2; j < 8; ++j)
                {
                    Rl[j] = Rg[j];
                }
                take = !tile_rejects(Rl, Rl[6], y0, yEnd, x0, xLimit, sBandD);
            }
            const unsigned m = __ballot_sync(0xFFFFFFFFu, take);
            if (lane == 0)
            {
                sScan[warp] = (uint32_t)__popc(m);
            }
            __syncthreads();
            int before = 0, total = 0;
            for (int w = 0; w < nWarps; ++w)
            {
                const int cw = (int)sScan[w];
                before += (w < warp) ? cw : 0;
                total += cw;
            }
            const int slot = cnt + before + __popc(m & ((1u << lane) - 1u));
            if (take && slot < kGather)
            {
                /* read again (L1) rather than held across the barrier */
                float4* dst = sRecBuf + slot * kStagedVec4;
#pragma unroll
                for (int j = 0; j < 8; ++j)
                {
                    dst[j] = Rg[j];
                }
                sKeyBuf[slot] = key;
            }
            if (take && slot == kGather)
            {
                sScan[nWarps] = i;
            }
            __syncthreads();
            if (cnt + total > kGather)
            {
                cursor = sScan[nWarps];
                cnt = kGather;
            }
            else
            {
                cursor += blockDim.x;
                cnt += total;
            }
        }
        return cnt;
    };
    const bool gathered = !kGeneral && f.depthBound;

    /* Otherwise batch k is walked from buffer k & 1 while batch k + 1 is
     * copied into the other (its last readers finished at the barrier
     * ending batch k - 1). */
    if (!gathered)
    {
        stage_records_async(f, sKeys, (int)min((uint32_t)L::kBatch, n), sRecBuf, sKeyBuf);
    }
    for (uint32_t b0 = 0, k = 0; b0 < n; ++k)
    {
        int cnt;
        float4* sRec;
        uint32_t* sRecKey;
        if (gathered)
        {
            batch_ranges();
            __syncthreads();
            cnt = gather(b0);
            sRec = sRecBuf;
            sRecKey = sKeyBuf;
        }
        else
        {
            cnt = (int)min((uint32_t)L::kBatch, n - b0);
            sRec = sRecBuf + (k & 1) * (L::kBatch * kStagedVec4);
            sRecKey = sKeyBuf + (k & 1) * L::kBatch;
            if (b0 + L::kBatch < n)
            {
                stage_records_async(f, sKeys + b0 + L::kBatch, (int)min((uint32_t)L::kBatch, n - b0 - L::kBatch),
                                    sRecBuf + ((k + 1) & 1) * (L::kBatch * kStagedVec4), sKeyBuf + ((k + 1) & 1) * L::kBatch);
                cp_async_wait<1>();
            }
            else
            {
                cp_async_wait<0>();
            }
            batch_ranges();
            __syncthreads();
            b0 += L::kBatch;
        }

        /* a triangle record none of whose pixels in the band can pass the
         * depth test is dropped for the whole warp (depth_range_rect over
         * its rows in the band and its columns in the tile) */
        const auto keep = [&](int ri, const float4 r6, float& zlo, float& zhi) {
            if (!f.depthBound)
            {
                return true;
            }
            const float4* R = sRec + ri * kStagedVec4;
            const uint32_t flags = __float_as_uint(R[7].w);
            const int minX = __float_as_int(r6.z), maxX = __float_as_int(r6.w);
            if ((flags & (kRecordLine | kRecordWire | kRecordPoint)) || maxX >= kRectBoundMaxX || maxX < minX)
            {
                return true;
            }
            const int ya = max(__float_as_int(r6.x), bandY0);
            const int yb = min(min(__float_as_int(r6.y), bandY0 + 8), f.height) - 1;
            const int xsMin = max(minX - 2, 0);
            const int xa = max(x0, xsMin), xb = min(xLimit - 1, maxX);
            if (yb < ya || xb < xa)
            {
                return false;
            }
            float lo = __int_as_float(0x7F800000), hi = __int_as_float(0xFF800000);
            for (int yy = ya; yy <= yb; ++yy)
            {
                lo = fminf(lo, sRowD[2 * (yy - y0)]);
                hi = fmaxf(hi, sRowD[2 * (yy - y0) + 1]);
            }
            depth_range_rect(R, ya, yb, xa, xb, xsMin, zlo, zhi);
            return !depth_range_rejects(flags & 0xF, zlo, zhi, lo, hi);
        };

        for_band_records(sRec, cnt, bandY0, keep, [&](int ri, float zlo, float zhi) {
            const float4* R = sRec + ri * kStagedVec4;
            const float4 r6 = R[6];
            if (!rowActive || y < __float_as_int(r6.x) || y >= __float_as_int(r6.y))
            {
                return;
            }
            const uint32_t flags = __float_as_uint(R[7].w);
            if (kGeneral && (flags & kRecordLine))
            {
                /* the walk steps of this row whose pixels this thread owns:
                 * one step on a steep line, every fourth on a flat one */
                const LineWalk w = line_walk(R);
                const LineRow lr = line_row(w, y, x0, xLimit, f.width);
                const DrawDesc& dd = f.draws[__float_as_uint(R[7].x)];
                const uint64_t rec = key_to_record(f, sRecKey[ri]);
                const int step = w.steep ? 1 : 4;
                const int kStart = w.steep ? lr.kLo : lr.kLo + ((myX0 - w.x1 - lr.kLo) & 3);
                const int nRow = (lr.kHi >= kStart) ? (lr.kHi - kStart) / step + 1 : 0;
                const int nAll = nRow + (lr.kWrap >= 0 ? 1 : 0);
                for (int j = 0; j < nAll; ++j)
                {
                    const int k = (j < nRow) ? kStart + j * step : lr.kWrap;
                    uint32_t X, Y;
                    int px, py;
                    if (!line_store_pixel(w, k, f.width, f.height, X, Y, px, py) || py != y || px < myX0 || px >= xLimit ||
                        ((px - myX0) & 3) != 0)
                    {
                        continue;
                    }
                    const float interp = line_interp(R, X, Y);
                    const float z = mixf(R[0].z, R[1].z, interp);
                    const int idx = r * L::kStride + (px - x0);
                    if (depth_cmp(flags & 0xF, z, sDepth[idx]))
                    {
                        const int aliasTag = __float_as_int(R[4].w);
                        if (aliasTag && k > 0 && k < w.dx)
                        {
                            /* a fragment SoftLight queues ahead of the line's last step */
                            atomicAdd(&f.aliasEvents[aliasTag - 1].queued, 1u);
                        }
                        float4 o;
                        slg_frag_coord fc = frag_coord(X, Y, z);
                        if (writes_color(dd, shade_line<P, kGeneral>(f, dd, rec, interp, fc, o, (size_t)px + (size_t)f.width * y)) &&
                            f.color)
                        {
                            sColor[idx] = (dd.blend != SLG_BLEND_OFF) ? Color::store(blend_color(dd.blend, o, Color::load(sColor[idx])))
                                                                      : Color::store(o);
                        }
                        if ((flags >> 4) & 1)
                        {
                            sDepth[idx] = depth_quant(halfDepth, fc.depth);
                        }
                    }
                }
                return;
            }
            if (kGeneral && (flags & kRecordWire))
            {
                /* this thread's pixels of the row's runs; a pixel visited twice
                 * takes its fragment twice (both visits are tested against the
                 * depth before the triangle: one unflushed queue) */
                const WireRow wr = wire_row(R, yf);
                const float bcY0 = R[3].x * yf + R[4].x, bcY1 = R[3].y * yf + R[4].y, bcY2 = R[3].z * yf + R[4].z;
                const DrawDesc& dd = f.draws[__float_as_uint(R[7].x)];
                const uint64_t rec = key_to_record(f, sRecKey[ri]);
                const int lo = max(wr.a0, myX0);
                const int xFirst = lo + ((myX0 - lo) & 3);
                const int xEnd = min(max(wr.a1, wr.b1), xLimit);
                for (int x = xFirst; x < xEnd; x += 4)
                {
                    const int n = wire_visits(wr, x);
                    if (n == 0)
                    {
                        continue;
                    }
                    float b0, b1, b2;
                    const float z = wire_fragment(R, bcY0, bcY1, bcY2, x, b0, b1, b2);
                    const int idx = r * L::kStride + (x - x0);
                    if (depth_cmp(flags & 0xF, z, sDepth[idx]))
                    {
                        float4 o;
                        slg_frag_coord fc = frag_coord((uint32_t)x, (uint32_t)y, z);
                        if (writes_color(dd, shade<P, kGeneral>(f, dd, rec, flags, R[2].w, R[5], b0, b1, b2, fc, o,
                                                               (size_t)x + (size_t)f.width * y, (dd.blend != SLG_BLEND_OFF) ? n : 1)) &&
                            f.color)
                        {
                            if (dd.blend != SLG_BLEND_OFF)
                            {
                                for (int v = 0; v < n; ++v) sColor[idx] = Color::store(blend_color(dd.blend, o, Color::load(sColor[idx])));
                            }
                            else
                            {
                                sColor[idx] = Color::store(o);
                            }
                        }
                        if ((flags >> 4) & 1)
                        {
                            sDepth[idx] = depth_quant(halfDepth, fc.depth);
                        }
                    }
                }
                return;
            }
            if (flags & kRecordPoint)
            {
                const int px = __float_as_int(r6.z);
                if (px < myX0 || px >= xLimit || ((px - myX0) & 3) != 0)
                {
                    return;
                }
                const int idx = r * L::kStride + (px - x0);
                const float z = R[0].z;
                if (depth_cmp(flags & 0xF, z, sDepth[idx]))
                {
                    const DrawDesc& dd = f.draws[__float_as_uint(R[7].x)];
                    float4 o;
                    slg_frag_coord fc = point_coord(R);
                    if (writes_color(dd, shade_point<P, kGeneral>(f, dd, key_to_record(f, sRecKey[ri]), fc, o, (size_t)px + (size_t)f.width * y)) &&
                        f.color)
                    {
                        sColor[idx] = (dd.blend != SLG_BLEND_OFF) ? Color::store(blend_color(dd.blend, o, Color::load(sColor[idx])))
                                                                  : Color::store(o);
                    }
                    if ((flags >> 4) & 1)
                    {
                        sDepth[idx] = depth_quant(halfDepth, fc.depth);
                    }
                }
                return;
            }
            const Span sp = scanline_span(R[0], R[1], yf);
            if (!((uint32_t)sp.xMin < (uint32_t)sp.xMax))
            {
                return;
            }
            const int depthFunc = flags & 0xF;
            /* the record's depths in the band against this thread's pixels */
            if (f.depthBound && depth_range_rejects(depthFunc, zlo, zhi, dMin, dMax))
            {
                return;
            }
            Chain ch;
            if (!chain_begin_span(R, yf, sp, myX0, xLimit, ch))
            {
                return;
            }
            const bool depthMask = (flags >> 4) & 1;
            const uint32_t drawIndex = __float_as_uint(R[7].x);
            for (; ch.x < ch.xEnd; chain_step(ch))
            {
                const float z = chain_depth(R, ch);
                const int idx = r * L::kStride + (ch.x - x0);
                if (depth_cmp(depthFunc, z, sDepth[idx]))
                {
                    const DrawDesc& dd = f.draws[drawIndex];
                    float4 o;
                    slg_frag_coord fc = frag_coord((uint32_t)ch.x, (uint32_t)y, z);
                    if (writes_color(dd, shade<P, kGeneral>(f, dd, key_to_record(f, sRecKey[ri]), flags, R[2].w, R[5], ch.b0, ch.b1, ch.b2, fc,
                                                           o, (size_t)ch.x + (size_t)f.width * y)) &&
                        f.color)
                    {
                        sColor[idx] = (dd.blend != SLG_BLEND_OFF) ? Color::store(blend_color(dd.blend, o, Color::load(sColor[idx])))
                                                                  : Color::store(o);
                    }
                    if (depthMask)
                    {
                        sDepth[idx] = depth_quant(halfDepth, fc.depth);
                    }
                }
            }
        });
        __syncthreads();
    }

    for (int i = threadIdx.x; i < TW * TH; i += blockDim.x)
    {
        const int px = i % TW, py = i / TW;
        const int gx = x0 + px, gy = y0 + py;
        if (gx < f.width && gy < f.height)
        {
            const size_t gi = (size_t)gx + (size_t)f.width * gy;
            depth_store(f, gi, sDepth[py * L::kStride + px]);
            if (f.color) Color::write(f.color, gi, sColor[py * L::kStride + px]);
        }
    }
}

/*-----------------------------------------------------------------------------
 * Order-free raster: no blending and one of the depth rules below for every
 * draw of the launch. The outcome of SoftLight's sequential per-pixel loop
 * (test against the current depth, write depth, overwrite colour) is then a
 * function of the fragment set alone:
 *   depth mask on,  LESS          : min z, ties -> earliest key
 *   depth mask on,  LESS_EQUAL    : min z, ties -> latest key
 *   depth mask on,  GREATER       : max z, ties -> earliest key
 *   depth mask on,  GREATER_EQUAL : max z, ties -> latest key
 *   depth mask on,  EQUAL         : latest key with z == d0
 *   any mask,       OFF           : latest key
 *   depth mask off, LT/LE/GT/GE/EQ: latest key passing against d0
 * (every built-in program writes colour unconditionally), so fragments may
 * be visited in any order and each pixel shaded once at the end.
 *
 * Task-parallel. A task is one scan-line of one staged
 * record inside the tile; a block-wide prefix sum over the records' row
 * counts deals the tasks to the threads densely, so triangles a few pixels
 * tall do not leave lanes idle. Each task walks its span with the four
 * column chains of the reference's 4-wide scan-line loop (chain_begin_span),
 * so every fragment's barycentrics and depth are the reference's bit for bit.
 *
 * Pass 1 folds each fragment that passes the depth test against the
 * pre-launch depth into the pixel's best word with a shared 64-bit
 * atomicMin; the word packs (depth order, key) so that its minimum is the
 * fragment the table above keeps. Pass 2 walks
 * the batch again and the pixel's winning fragment, unique by its key,
 * stores its barycentrics and depth; the resolve shades each pixel once.
-----------------------------------------------------------------------------*/
constexpr int kFreeThreads = 128;
constexpr int kFreeBatch = 128;   /* records staged per step */

template <int TW, int TH>
struct FreeLayout
{
    static constexpr int kPix = TW * TH;
    /* records staged per step: 96 for tiles of at most 64 pixels (less
     * shared memory, so 12 CTAs fit an SM), else kFreeBatch */
    static constexpr int kBatch = (TW * TH <= 64) ? 96 : kFreeBatch;
    /* resident CTAs the launch bounds ask for */
    static constexpr int kMinBlocks = (TW * TH <= 64) ? 12 : 4;
    static constexpr size_t kRecOff = 0;                                                   /* float4 [batch][kStagedVec4] */
    static constexpr size_t kBOff = kRecOff + sizeof(float4) * kBatch * kStagedVec4;        /* float4 (b0, b1, b2, z) per pixel */
    static constexpr size_t kBestOff = kBOff + sizeof(float4) * kPix;                      /* u64 per pixel */
    static constexpr size_t kD0Off = kBestOff + sizeof(unsigned long long) * kPix;         /* pre-launch depth per pixel */
    static constexpr size_t kKeyOff = kD0Off + sizeof(float) * kPix;                       /* u32 per staged record */
    static constexpr size_t kPreOff = kKeyOff + sizeof(uint32_t) * kBatch;                 /* u32 [threads + 1] row prefix */
    static constexpr size_t kWarpOff = kPreOff + sizeof(uint32_t) * (kFreeThreads + 4);    /* u32 per warp */
    static constexpr size_t kWonOff = kWarpOff + sizeof(uint32_t) * (kFreeThreads / 32);           /* u32 bit per scan-line task */
    static constexpr int kWonWords = (kBatch * TH + 31) / 32; /* a staged record has at most TH rows in the tile */
    static constexpr size_t bytes() { return kWonOff + sizeof(uint32_t) * kWonWords; }
};

/* Total order of depths as unsigned words (-0 and +0 equal, as they compare). */
__device__ __forceinline__ uint32_t depth_order(float z)
{
    const uint32_t u = __float_as_uint(z + 0.f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

/* Whether the depth rule prefers the larger key among equal depths (or
 * whenever depth does not decide). */
__device__ __forceinline__ bool free_key_max(int func, bool mask)
{
    return !mask || !(func == SLG_DEPTH_TEST_LESS_THAN || func == SLG_DEPTH_TEST_GREATER_THAN);
}

__device__ __forceinline__ unsigned long long free_pack(int func, bool mask, float z, uint32_t key)
{
    uint32_t zp = 0u;
    if (mask && (func == SLG_DEPTH_TEST_LESS_THAN || func == SLG_DEPTH_TEST_LESS_EQUAL)) zp = depth_order(z);
    if (mask && (func == SLG_DEPTH_TEST_GREATER_THAN || func == SLG_DEPTH_TEST_GREATER_EQUAL)) zp = ~depth_order(z);
    return ((unsigned long long)zp << 32) | (free_key_max(func, mask) ? ~key : key);
}

/* Walks the scan-line tasks of the staged batch. kStore false: fold every
 * passing fragment into sBest; true: the fragment equal to its pixel's
 * sBest stores (b0, b1, b2, z). */
template <int TW, int TH, bool kStore, bool kGeneral>
__device__ __forceinline__ void free_walk(const float4* sRec, const uint32_t* sKey, const uint32_t* sPre, int cnt, int x0, int y0,
                                          int xLimit, int width, int height, int func, bool mask, const float* sD0,
                                          unsigned long long* sBest, float4* sB, uint32_t* sWon)
{
    const uint32_t total = sPre[cnt];
    for (uint32_t i = threadIdx.x; i < total; i += kFreeThreads)
    {
        if (kStore && !((sWon[i >> 5] >> (i & 31)) & 1u))
        {
            continue;
        }
        /* sBest only decreases and packed values are unique per pixel, so a
         * fragment not below the value read here can never be its pixel's
         * final best: it is dropped, and only tasks with a fragment that
         * passed are walked again by the store pass */
        bool marked = false;
        auto fold = [&](int idx, unsigned long long p) {
            if (p < *reinterpret_cast<volatile unsigned long long*>(sBest + idx))
            {
                atomicMin(sBest + idx, p);
                if (kGeneral && !marked)
                {
                    marked = true;
                    atomicOr(sWon + (i >> 5), 1u << (i & 31));
                }
            }
        };
        int lo = 0, hi = cnt;
        while (hi - lo > 1)
        {
            const int mid = (lo + hi) >> 1;
            if (sPre[mid] <= i) lo = mid;
            else hi = mid;
        }
        const float4* R = sRec + lo * kStagedVec4;
        const int y = max(__float_as_int(R[6].x), y0) + (int)(i - sPre[lo]);
        if (kGeneral && (__float_as_uint(R[7].w) & kRecordLine))
        {
            /* the walk steps of this row; sB keeps (interp, 0, 0, z) */
            const LineWalk w = line_walk(R);
            const LineRow lr = line_row(w, y, x0, xLimit, width);
            const uint32_t key = sKey[lo];
            const int nRow = max(lr.kHi - lr.kLo + 1, 0);
            const int nAll = nRow + (lr.kWrap >= 0 ? 1 : 0);
            for (int j = 0; j < nAll; ++j)
            {
                const int kk = (j < nRow) ? lr.kLo + j : lr.kWrap;
                uint32_t X, Y;
                int px, py;
                if (!line_store_pixel(w, kk, width, height, X, Y, px, py) || py != y || px < x0 || px >= xLimit)
                {
                    continue;
                }
                const float interp = line_interp(R, X, Y);
                const float z = mixf(R[0].z, R[1].z, interp);
                const int idx = (y - y0) * TW + (px - x0);
                if (!depth_cmp(func, z, sD0[idx]))
                {
                    continue;
                }
                const unsigned long long p = free_pack(func, mask, z, key);
                if (kStore)
                {
                    if (sBest[idx] == p) sB[idx] = make_float4(interp, __uint_as_float(X | (Y << 16)), 0.f, z);
                }
                else
                {
                    fold(idx, p);
                }
            }
            continue;
        }
        if (kGeneral && (__float_as_uint(R[7].w) & kRecordWire))
        {
            /* each visited pixel once: the left run, then the right run past it */
            const float yf = (float)y;
            const WireRow wr = wire_row(R, yf);
            const float bcY0 = R[3].x * yf + R[4].x, bcY1 = R[3].y * yf + R[4].y, bcY2 = R[3].z * yf + R[4].z;
            const uint32_t key = sKey[lo];
            for (int run = 0; run < 2; ++run)
            {
                const int xa = max(run ? max(wr.b0, wr.a1) : wr.a0, x0);
                const int xb = min(run ? wr.b1 : wr.a1, xLimit);
                for (int x = xa; x < xb; ++x)
                {
                    float b0, b1, b2;
                    const float z = wire_fragment(R, bcY0, bcY1, bcY2, x, b0, b1, b2);
                    const int idx = (y - y0) * TW + (x - x0);
                    if (!depth_cmp(func, z, sD0[idx]))
                    {
                        continue;
                    }
                    const unsigned long long p = free_pack(func, mask, z, key);
                    if (kStore)
                    {
                        if (sBest[idx] == p) sB[idx] = make_float4(b0, b1, b2, z);
                    }
                    else
                    {
                        fold(idx, p);
                    }
                }
            }
            continue;
        }
        if (__float_as_uint(R[7].w) & kRecordPoint)
        {
            const int px = __float_as_int(R[6].z);
            const int idx = (y - y0) * TW + (px - x0);
            const float z = R[0].z;
            if (px < x0 || px >= xLimit || !depth_cmp(func, z, sD0[idx]))
            {
                continue;
            }
            const unsigned long long p = free_pack(func, mask, z, sKey[lo]);
            if (kStore)
            {
                if (sBest[idx] == p) sB[idx] = make_float4(0.f, 0.f, 0.f, z);
            }
            else
            {
                fold(idx, p);
            }
            continue;
        }
        const float yf = (float)y;
        const Span sp = scanline_span(R[0], R[1], yf);
        if (!((uint32_t)sp.xMin < (uint32_t)sp.xMax))
        {
            continue;
        }
        const uint32_t key = sKey[lo];
        const int rowBase = (y - y0) * TW - x0;
        /* the four column chains of chain_begin_span / chain_step /
         * chain_depth, with the row terms they share computed once */
        const float4 r2 = R[2], r3 = R[3], r4 = R[4], r5 = R[5];
        const float bcY0 = r3.x * yf + r4.x, bcY1 = r3.y * yf + r4.y, bcY2 = r3.z * yf + r4.z;
        const float s0 = r2.x * 4.f, s1 = r2.y * 4.f, s2 = r2.z * 4.f;
        const float zw = 0.f * r2.w;
        const int xEnd = min(sp.xMax, xLimit);
#pragma unroll 1
        for (int l = 0; l < 4; ++l)
        {
            const int myX0 = x0 + l;
            const int xs = sp.xMin + ((myX0 - sp.xMin) & 3);
            const int xFirst = max(xs, myX0);
            if (xFirst >= xEnd)
            {
                continue;
            }
            const float xsf = (float)xs;
            float b0 = r2.x * xsf + bcY0, b1 = r2.y * xsf + bcY1, b2 = r2.z * xsf + bcY2;
            for (int g = (xFirst - xs) >> 2; g > 0; --g)
            {
                b0 += s0;
                b1 += s1;
                b2 += s2;
            }
            for (int x = xFirst; x < xEnd; x += 4, b0 += s0, b1 += s1, b2 += s2)
            {
                const float z = __fadd_rn((r3.w * b0 + r4.w * b1) + r5.x * b2, zw);
                const int idx = rowBase + x;
                if (!depth_cmp(func, z, sD0[idx]))
                {
                    continue;
                }
                const unsigned long long p = free_pack(func, mask, z, key);
                if (kStore)
                {
                    if (sBest[idx] == p) sB[idx] = make_float4(b0, b1, b2, z);
                }
                else
                {
                    fold(idx, p);
                }
            }
        }
    }
}

/* Shades the winning fragment p (a best word) of pixel (x, y) once and
 * writes its colour, depth and visibility id. Triangle winners re-derive
 * their barycentrics and depth from the record with the walk's own chain
 * (the column class of x starts at the same xs and takes the same
 * (x - xs) / 4 additions); kGeneral launches pass what their store pass
 * kept (`stored`), which line winners need. */
template <class P, class Color, bool kGeneral>
__device__ __forceinline__ void resolve_winner(const Frame& f, unsigned long long p, bool keyMax, bool mask, int x, int y, float4 stored)
{
    const uint32_t key = keyMax ? ~(uint32_t)p : (uint32_t)p;
    const size_t gi = (size_t)x + (size_t)f.width * y;
    const uint64_t rec = key_to_record(f, key);
    const float4* R = f.records + rec * kRecordVec4;
    const DrawDesc& dd = f.draws[__float_as_uint(R[7].x)];
    const uint32_t kind = __float_as_uint(R[7].w);
    float4 b;
    if (kGeneral)
    {
        b = stored;
    }
    else if (kind & kRecordPoint)
    {
        b = make_float4(0.f, 0.f, 0.f, R[0].z);
    }
    else
    {
        const float yf = (float)y;
        Chain ch;
        (void)chain_begin_span(R, yf, scanline_span(R[0], R[1], yf), x, x + 1, ch);
        b = make_float4(ch.b0, ch.b1, ch.b2, chain_depth(R, ch));
    }
    if ((f.color || f.generic0) && dd.numOutputs > 0)
    {
        float4 o;
        bool kept;
        if (kind & kRecordPoint)
        {
            slg_frag_coord fc = point_coord(R);
            kept = shade_point<P, kGeneral>(f, dd, rec, fc, o, gi);
        }
        else if (kGeneral && (kind & kRecordLine))
        {
            /* stored.y keeps the line step's 16-bit (X, Y): X = W on the row
             * above for the step stored at column 0 */
            const uint32_t xy = __float_as_uint(b.y);
            slg_frag_coord fc = frag_coord(xy & 0xFFFFu, xy >> 16, b.w);
            kept = shade_line<P, kGeneral>(f, dd, rec, b.x, fc, o, gi);
        }
        else
        {
            slg_frag_coord fc = frag_coord((uint32_t)x, (uint32_t)y, b.w);
            kept = shade<P, kGeneral>(f, dd, rec, kind, R[2].w, R[5], b.x, b.y, b.z, fc, o, gi);
        }
        if (kept && f.color)
        {
            Color::write(f.color, gi, Color::store(o));
        }
        if (!kept)
        {
            /* the winner is the last fragment that passes, in the
             * reference's order; when it is discarded the pixel keeps an
             * earlier fragment's colour, which only the ordered raster
             * knows: programs that discard are registered as such and
             * their launches never come here */
            atomicOr(f.status, kStatusUndeclaredDiscard);
        }
    }
    if (mask)
    {
        depth_store(f, gi, b.w);
    }
    if (f.ids)
    {
        f.ids[gi] = (key >> kSubShift) + 1u;
    }
}

template <class P, int TW, int TH, class Color, bool kGeneral>
__global__ void __launch_bounds__(kFreeThreads, kGeneral ? 4 : FreeLayout<TW, TH>::kMinBlocks) raster_free_kernel(const Frame f, int depthFunc, int depthMask)
{
    typedef FreeLayout<TW, TH> L;
    extern __shared__ __align__(16) uint8_t smem[];
    float4* sRec = reinterpret_cast<float4*>(smem + L::kRecOff);
    float4* sB = reinterpret_cast<float4*>(smem + L::kBOff);
    unsigned long long* sBest = reinterpret_cast<unsigned long long*>(smem + L::kBestOff);
    float* sD0 = reinterpret_cast<float*>(smem + L::kD0Off);
    uint32_t* sKey = reinterpret_cast<uint32_t*>(smem + L::kKeyOff);
    uint32_t* sPre = reinterpret_cast<uint32_t*>(smem + L::kPreOff);
    uint32_t* sWarp = reinterpret_cast<uint32_t*>(smem + L::kWarpOff);
    uint32_t* sWon = reinterpret_cast<uint32_t*>(smem + L::kWonOff);

    const int tile = blockIdx.x;
    const uint32_t begin = f.tileOffset[tile];
    const uint32_t n = f.tileOffset[tile + 1] - begin;
    if (n == 0 || (f.status[0] & kStatusSticky) || ordered_raster_runs(f))
    {
        return;
    }
    const int tx = tile % f.tilesX, ty = tile / f.tilesX;
    const int x0 = tx * TW, y0 = ty * TH;
    const int xLimit = min(x0 + TW, f.width);
    const int yLimit = min(y0 + TH, f.height);
    const bool mask = depthMask != 0;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

    for (int i = threadIdx.x; i < L::kPix; i += kFreeThreads)
    {
        const int x = x0 + i % TW, y = y0 + i / TW;
        sBest[i] = ~0ull;
        sD0[i] = (x < xLimit && y < yLimit) ? depth_load(f, (size_t)x + (size_t)f.width * y) : 0.f;
    }

    for (uint32_t b0 = 0; b0 < n; b0 += L::kBatch)
    {
        const int cnt = (int)min((uint32_t)L::kBatch, n - b0);
        __syncthreads();
        stage_records<L::kBatch>(f, f.entries + begin + b0, cnt, sRec, sKey);
        __syncthreads();

        /* rows of each staged record inside the tile, prefix-summed */
        uint32_t rows = 0;
        if ((int)threadIdx.x < cnt)
        {
            const float4 r6 = sRec[threadIdx.x * kStagedVec4 + 6];
            const int ry0 = max(__float_as_int(r6.x), y0);
            const int ry1 = min(__float_as_int(r6.y), yLimit);
            rows = (ry1 > ry0) ? (uint32_t)(ry1 - ry0) : 0u;
        }
        uint32_t incl = rows;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1)
        {
            const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, off);
            if (lane >= off) incl += t;
        }
        if (lane == 31) sWarp[warp] = incl;
        __syncthreads();
        for (int w = 0; w < warp; ++w) incl += sWarp[w];
        sPre[threadIdx.x + 1] = incl;
        if (threadIdx.x == 0) sPre[0] = 0u;
        if (kGeneral)
        {
            for (int w = threadIdx.x; w < L::kWonWords; w += kFreeThreads) sWon[w] = 0u;
        }
        __syncthreads();

        free_walk<TW, TH, false, kGeneral>(sRec, sKey, sPre, cnt, x0, y0, xLimit, f.width, f.height, depthFunc, mask, sD0, sBest, sB, sWon);
        if (kGeneral)
        {
            /* line and wireframe fragments cannot be re-derived from the
             * pixel alone: the winners store their interpolants */
            __syncthreads();
            free_walk<TW, TH, true, kGeneral>(sRec, sKey, sPre, cnt, x0, y0, xLimit, f.width, f.height, depthFunc, mask, sD0, sBest, sB,
                                              sWon);
        }
    }
    __syncthreads();

    /* resolve: shade each pixel's winner once */
    const bool keyMax = free_key_max(depthFunc, mask);
    for (int i = threadIdx.x; i < L::kPix; i += kFreeThreads)
    {
        const unsigned long long p = sBest[i];
        if (p != ~0ull)
        {
            resolve_winner<P, Color, kGeneral>(f, p, keyMax, mask, x0 + i % TW, y0 + i / TW, kGeneral ? sB[i] : make_float4(0.f, 0.f, 0.f, 0.f));
        }
    }
}

/*-----------------------------------------------------------------------------
 * Untiled order-free raster, for launches of triangles and points: the
 * fragment set and the winner rule of raster_free_kernel without tile
 * lists. Every record is walked once, row by row (the tile version stages a
 * record once per tile it touches), and each fragment that passes against
 * the pre-launch depth is folded into its pixel's best word in global memory
 * (64-bit atomicMin, skipped when a plain read already shows a better word;
 * the words stay in L2). resolve_global_kernel then shades each pixel's
 * winner with resolve_winner. A warp takes 32 records at a time and deals
 * their rows to the lanes 32 per step, so triangles of any height keep the
 * lanes busy. The walk of a row runs the reference's four column chains
 * from the span's start: the chain of x starts at the same xs and takes the
 * same additions as in the tiled walk, so depths are identical.
-----------------------------------------------------------------------------*/
constexpr int kGlobalWarps = 4;

struct GroupRecs
{
    uint32_t start[32];   /* first task (row) of each record of the group */
    uint32_t rec[32];
    uint32_t key[32];
    int32_t  y0[32];      /* first row walked */
};

/* Folds a fragment of pixel gi into its best word when it passes against
 * the pre-launch depth. The word only decreases, so any earlier value of it
 * is an upper bound: a fragment not below what a plain (L1-cached, possibly
 * older) read returns can never win and issues no atomic. */
__device__ __forceinline__ void global_fold(const Frame& f, size_t gi, float z, uint32_t key, int func, bool mask)
{
    /* both reads issued together, then the tests */
    unsigned long long* w = f.bestWords + gi;
    const float d0 = depth_load(f, gi);
    const unsigned long long cur = *w;
    const unsigned long long p = free_pack(func, mask, z, key);
    if (depth_cmp(func, z, d0) && p < cur)
    {
        atomicMin(w, p);
    }
}

/* Walks 32 records, one named per lane (have: the lane holds one; rec: its
 * index; key: its ordering key), row by row into the best words: the group's
 * rows are dealt to the lanes 32 per step. Every lane of the warp calls it. */
__device__ __forceinline__ void walk_group(const Frame& f, bool have, uint64_t rec, uint32_t key, int depthFunc, bool mask, GroupRecs& g)
{
    const int lane = threadIdx.x & 31;
    uint32_t rows = 0;
    int ya = 0;
    if (have)
    {
        const float4 r6 = f.records[rec * kRecordVec4 + 6];
        ya = max(__float_as_int(r6.x), 0);
        const int yb = min(__float_as_int(r6.y), f.height);
        if (yb > ya && __float_as_int(r6.w) >= 0 && __float_as_int(r6.z) < f.width)
        {
            rows = (uint32_t)(yb - ya);
        }
    }
    uint32_t incl = rows;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += v;
    }
    const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    __syncwarp();
    g.start[lane] = incl - rows;
    g.rec[lane] = (uint32_t)min(rec, (uint64_t)0xFFFFFFFFu);
    g.key[lane] = key;
    g.y0[lane] = ya;
    __syncwarp();
    for (uint32_t e = lane; e < total; e += 32)
    {
        /* the record holding task e: the last one starting at or before
         * e (records without rows share their start with the next) */
        int lo = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1)
        {
            if (lo + step < 32 && g.start[lo + step] <= e) lo += step;
        }
        const uint32_t k = g.key[lo];
        const int y = g.y0[lo] + (int)(e - g.start[lo]);
        const float4* R = f.records + (uint64_t)g.rec[lo] * kRecordVec4;
        const size_t rowBase = (size_t)f.width * y;
        if (__float_as_uint(R[7].w) & kRecordPoint)
        {
            const int px = __float_as_int(R[6].z);
            if (px >= 0 && px < f.width) global_fold(f, rowBase + px, R[0].z, k, depthFunc, mask);
            continue;
        }
        const float yf = (float)y;
        const Span sp = scanline_span(R[0], R[1], yf);
        if (!((uint32_t)sp.xMin < (uint32_t)sp.xMax))
        {
            continue;
        }
        const float4 r2 = R[2], r3 = R[3], r4 = R[4], r5 = R[5];
        const float bcY0 = r3.x * yf + r4.x, bcY1 = r3.y * yf + r4.y, bcY2 = r3.z * yf + r4.z;
        const float s0 = r2.x * 4.f, s1 = r2.y * 4.f, s2 = r2.z * 4.f;
        const float zw = 0.f * r2.w;
        const int xEnd = min(sp.xMax, f.width);
        /* the four column chains from the span's start (chain_begin_span
         * with no catch-up: each starts at its first pixel) */
#pragma unroll 1
        for (int xs = sp.xMin; xs < min(sp.xMin + 4, xEnd); ++xs)
        {
            const float xsf = (float)xs;
            float b0 = r2.x * xsf + bcY0, b1 = r2.y * xsf + bcY1, b2 = r2.z * xsf + bcY2;
            for (int x = xs; x < xEnd; x += 4, b0 += s0, b1 += s1, b2 += s2)
            {
                global_fold(f, rowBase + x, __fadd_rn((r3.w * b0 + r4.w * b1) + r5.x * b2, zw), k, depthFunc, mask);
            }
        }
    }
    __syncwarp();
}

/* The clipped fans' records (vs_setup_kernel walks the slots' own records
 * as it stores them): records [numSlots, numSlots + ovfCount). */
template <class P>
__global__ void __launch_bounds__(kGlobalWarps * 32) raster_global_kernel(const Frame f, int depthFunc, int depthMask)
{
    __shared__ GroupRecs sG[kGlobalWarps];
    if (f.status[0] & kStatusSticky)
    {
        return;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    /* the count can pass the capacity only in a launch that overflowed,
     * which the sticky status already stopped */
    const uint64_t nOvf = min(*f.ovfCount, f.ovfCap);
    const uint64_t stride = (uint64_t)gridDim.x * kGlobalWarps * 32;
    for (uint64_t g0 = ((uint64_t)blockIdx.x * kGlobalWarps + warp) * 32; g0 < nOvf; g0 += stride)
    {
        const uint64_t j = g0 + lane;
        const bool have = j < nOvf;
        walk_group(f, have, f.numSlots + j, have ? f.ovfKey[j] : 0u, depthFunc, depthMask != 0, sG[warp]);
    }
}

template <class P, bool kLines, bool kCached>
__global__ void __launch_bounds__(256, kCached ? 6 : 1) vs_setup_kernel(const Frame f)
{
    const uint64_t slot = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    TileRange tr;
    tr.tx0 = 0; tr.tx1 = -1; tr.ty0 = 0; tr.ty1 = -1;
    bool counted = false;
    if (slot < f.numSlots)
    {
        f.slotInfo[slot] = setup_slot<P, kLines, kCached>(f, slot, tr, counted);
    }
    /* per-tile counts of the unclipped records, one atomic per group of
     * lanes touching the same tile (clipped records count themselves);
     * launches filling their lists in key order count per chunk instead,
     * untiled launches not at all */
    warp_tile_walk(f, tr, counted && f.chunkCounts == nullptr && f.bestWords == nullptr, f.tileCount, [](uint32_t, uint32_t) {});
    if (f.bestWords)
    {
        /* untiled launch: the warp walks the records its lanes just stored
         * (raster_global_kernel walks the clipped fans later) */
        __shared__ GroupRecs sG[8];
        const bool have = slot < f.numSlots && f.slotInfo[slot] == 1;
        walk_group(f, have, slot, (uint32_t)(slot << kSubShift), f.freeDepthFunc, f.freeDepthMask != 0, sG[threadIdx.x >> 5]);
    }
}

template <class P, class Color>
__global__ void __launch_bounds__(256) resolve_global_kernel(const Frame f, int depthFunc, int depthMask)
{
    if (f.status[0] & kStatusSticky)
    {
        return;
    }
    const bool mask = depthMask != 0;
    const bool keyMax = free_key_max(depthFunc, mask);
    /* one 16x16 block of pixels per CTA, so the pixels of a small triangle
     * share its record, cache entries and texels in L1 */
    const int gx = (f.width + 15) >> 4;
    const int x = (int)(blockIdx.x % (unsigned)gx) * 16 + (int)(threadIdx.x & 15);
    const int y = (int)(blockIdx.x / (unsigned)gx) * 16 + (int)(threadIdx.x >> 4);
    if (x >= f.width || y >= f.height)
    {
        return;
    }
    const unsigned long long p = f.bestWords[(size_t)x + (size_t)f.width * y];
    if (p != ~0ull)
    {
        resolve_winner<P, Color, false>(f, p, keyMax, mask, x, y, make_float4(0.f, 0.f, 0.f, 0.f));
    }
}

/*-----------------------------------------------------------------------------
 * Line address aliases (AliasEvent). After the ordered raster, each logged
 * pixel is replayed from its pre-launch state through every record that
 * covers it, in submission order. The aliasing line's two fragments there
 * follow SoftLight's queue (SL_LineRasterizer.cpp:49-85, flushed every
 * SL_SHADER_MAX_QUEUED_FRAGS = 600 queued fragments): when fewer than 600 of
 * the line's steps before the last one passed the depth test, the last step
 * is tested against the depth before the line; both writes then follow in
 * walk order.
-----------------------------------------------------------------------------*/
constexpr int kAliasThreads = 256;
constexpr int kAliasKeys = 4096;          /* records covering one pixel (power of two) */

template <class P, class Color>
__device__ void alias_replay(const Frame& f, const AliasEvent& ev, const uint32_t* keys, int m)
{
    typedef typename Color::stored Stored;
    const uint32_t gi = ev.pixel;
    const int py = (int)(gi / (uint32_t)f.width);
    const float yf = (float)py;

    const bool halfDepth = f.depthType == SLG_COLOR_R_HALF;
    /* the pixel's state before the launch */
    float depth = ev.depth0;
    for (int k = 0; k < f.numColors; ++k)
    {
        const int bpt = texel_bytes(f.colorTypes[k]);
        for (int b = 0; b < bpt; ++b) f.colors[k][(size_t)gi * bpt + b] = ev.colors[k][b];
    }
    Stored color{};
    if (f.color)
    {
        color = Color::read(f.color, gi);
    }
    auto put = [&](const DrawDesc& dd, bool kept, const float4 o) {
        if (writes_color(dd, kept) && f.color)
        {
            color = (dd.blend != SLG_BLEND_OFF) ? Color::store(blend_color(dd.blend, o, Color::load(color))) : Color::store(o);
        }
    };

    for (int i = 0; i < m; ++i)
    {
        const uint64_t rec = key_to_record(f, keys[i]);
        const float4* R = f.records + rec * kRecordVec4;
        const uint32_t flags = __float_as_uint(R[7].w);
        const int func = flags & 0xF;
        const bool mask = ((flags >> 4) & 1) != 0;
        const DrawDesc& dd = f.draws[__float_as_uint(R[7].x)];
        float4 o;
        if (flags & kRecordLine)
        {
            const LineWalk w = line_walk(R);
            const LineRow lr = line_row(w, py, 0, 1, f.width);
            int ks[2];
            int nk = 0;
            for (int k = lr.kLo; k <= lr.kHi && nk < 2; ++k) ks[nk++] = k;
            if (lr.kWrap >= 0 && nk < 2) ks[nk++] = lr.kWrap;
            int kh[2];
            uint32_t xh[2], yh[2];
            float zh[2], ih[2];
            int nh = 0;
            for (int j = 0; j < nk; ++j)
            {
                uint32_t X, Y;
                int px, qy;
                if (line_store_pixel(w, ks[j], f.width, f.height, X, Y, px, qy) && (uint32_t)qy * (uint32_t)f.width + (uint32_t)px == gi)
                {
                    xh[nh] = X;
                    yh[nh] = Y;
                    ih[nh] = line_interp(R, X, Y);
                    zh[nh] = mixf(R[0].z, R[1].z, ih[nh]);
                    kh[nh] = ks[j];
                    ++nh;
                }
            }
            const int tag = __float_as_int(R[4].w);
            const float before = depth;
            for (int j = 0; j < nh; ++j)
            {
                float against = depth;
                if (j == 1 && tag != 0 && kh[1] == w.dx)
                {
                    /* the last step: the first one is written before its test
                     * only if the queue was flushed in between */
                    const uint32_t queued = f.aliasEvents[tag - 1].queued + (depth_cmp(func, zh[0], before) ? 1u : 0u);
                    if (queued < kFragQueue) against = before;
                }
                if (depth_cmp(func, zh[j], against))
                {
                    slg_frag_coord fc = frag_coord(xh[j], yh[j], zh[j]);
                    put(dd, shade_line<P, true>(f, dd, rec, ih[j], fc, o, gi), o);
                    if (mask) depth = depth_quant(halfDepth, fc.depth);
                }
            }
        }
        else if (flags & kRecordWire)
        {
            const WireRow wr = wire_row(R, yf);
            const int n = wire_visits(wr, 0);
            if (n > 0)
            {
                float b0, b1, b2;
                const float z = wire_fragment(R, R[3].x * yf + R[4].x, R[3].y * yf + R[4].y, R[3].z * yf + R[4].z, 0, b0, b1, b2);
                if (depth_cmp(func, z, depth))
                {
                    slg_frag_coord fc = frag_coord(0u, (uint32_t)py, z);
                    const bool have = shade<P, true>(f, dd, rec, flags, R[2].w, R[5], b0, b1, b2, fc, o, gi, (dd.blend != SLG_BLEND_OFF) ? n : 1);
                    for (int v = 0; v < ((dd.blend != SLG_BLEND_OFF) ? n : 1); ++v) put(dd, have, o);
                    if (mask) depth = depth_quant(halfDepth, fc.depth);
                }
            }
        }
        else if (flags & kRecordPoint)
        {
            const float4 r6 = R[6];
            if (__float_as_int(r6.z) == 0 && __float_as_int(r6.x) == py && depth_cmp(func, R[0].z, depth))
            {
                slg_frag_coord fc = point_coord(R);
                put(dd, shade_point<P, true>(f, dd, rec, fc, o, gi), o);
                if (mask) depth = depth_quant(halfDepth, fc.depth);
            }
        }
        else
        {
            Chain ch;
            if (chain_begin(R, yf, 0, 1, ch) && ch.x == 0)
            {
                const float z = chain_depth(R, ch);
                if (depth_cmp(func, z, depth))
                {
                    slg_frag_coord fc = frag_coord(0u, (uint32_t)py, z);
                    put(dd, shade<P, true>(f, dd, rec, flags, R[2].w, R[5], ch.b0, ch.b1, ch.b2, fc, o, gi), o);
                    if (mask) depth = depth_quant(halfDepth, fc.depth);
                }
            }
        }
    }
    depth_store(f, gi, depth);
    if (f.color) Color::write(f.color, gi, color);
}

template <class P, class Color>
__global__ void __launch_bounds__(kAliasThreads) alias_fixup_kernel(const Frame f)
{
    __shared__ uint32_t sKeys[kAliasKeys];
    __shared__ uint32_t sCount;
    __shared__ int sSkip;
    if (f.status[0] & kStatusSticky)
    {
        return;
    }
    const uint32_t count = min(*f.aliasCount, f.aliasCap);
    for (uint32_t e = blockIdx.x; e < count; e += gridDim.x)
    {
        __syncthreads();
        if (threadIdx.x == 0)
        {
            sCount = 0;
            sSkip = 0;
        }
        __syncthreads();
        const AliasEvent ev = f.aliasEvents[e];
        /* one replay per pixel, by its first event */
        for (uint32_t j = threadIdx.x; j < e; j += blockDim.x)
        {
            if (f.aliasEvents[j].pixel == ev.pixel) sSkip = 1;
        }
        __syncthreads();
        const bool skip = sSkip != 0;
        const int py = (int)(ev.pixel / (uint32_t)f.width);
        const int tile = (py / f.tileH) * f.tilesX;
        const uint32_t begin = f.tileOffset[tile];
        const uint32_t n = f.tileOffset[tile + 1] - begin;
        if (!skip)
        {
            for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
            {
                const uint32_t key = f.entries[begin + i];
                const float4 r6 = f.records[key_to_record(f, key) * kRecordVec4 + 6];
                if (__float_as_int(r6.x) <= py && py < __float_as_int(r6.y) && __float_as_int(r6.z) <= 0)
                {
                    const uint32_t q = atomicAdd(&sCount, 1u);
                    if (q < (uint32_t)kAliasKeys) sKeys[q] = key;
                }
            }
        }
        __syncthreads();
        const int m = skip ? 0 : (int)sCount;
        if (m > kAliasKeys)
        {
            if (threadIdx.x == 0) atomicOr(f.status, kStatusAliasKeys);
            continue;
        }
        if (!skip)
        {
            sort_keys(sKeys, m);
            if (threadIdx.x == 0) alias_replay<P, Color>(f, ev, sKeys, m);
        }
    }
}


/*-----------------------------------------------------------------------------
 * Launchers of one program set. The raster stage is instantiated per colour
 * format of attachment 0 (RGBA8, RGBA float, R float: the formats the tile
 * buffers hold), so a program set can be compiled in four translation units.
-----------------------------------------------------------------------------*/
/* Vertex stage: post-transform vertex cache, vs_setup, clipping. */
template <class P>
cudaError_t launch_vertex_stage(const Frame& f, cudaStream_t s)
{
    const int vsBlock = (f.vsBlock == 64 || f.vsBlock == 256) ? f.vsBlock : 128;
    if (f.cacheEntries > 0)
    {
        vertex_cache_kernel<P><<<(unsigned)((f.cacheEntries + 255) / 256), 256, 0, s>>>(f);
    }
    if (f.bestWords)
    {
        /* the untiled raster's best words, reset before vs_setup_kernel walks into them */
        cudaMemsetAsync(f.bestWords, 0xFF, (size_t)f.width * f.height * sizeof(unsigned long long), s);
    }
    if (f.numSlots > 0)
    {
        const unsigned blocks = (unsigned)((f.numSlots + vsBlock - 1) / vsBlock);
        if (f.hasLines || f.hasWire) vs_setup_kernel<P, true, false><<<blocks, vsBlock, 0, s>>>(f);
        else if (f.allCached) vs_setup_kernel<P, false, true><<<blocks, vsBlock, 0, s>>>(f);
        else vs_setup_kernel<P, false, false><<<blocks, vsBlock, 0, s>>>(f);
        clip_kernel<P><<<152 * 4, 128, 0, s>>>(f);   /* 128 registers: four CTAs per SM */
    }
    return cudaGetLastError();
}

/* Raster of one tile size; tile_sort_kernel (library) has already sorted the
 * tile lists when the ordered raster may run. */
template <class P, int TW, int TH, class Color, bool kGeneral>
cudaError_t launch_raster_tiles(const Frame& f, int numTiles, cudaStream_t s)
{
    typedef RasterLayout<TW, TH, Color> L;
    if (f.orderFree)
    {
        raster_free_kernel<P, TW, TH, Color, kGeneral><<<numTiles, kFreeThreads, FreeLayout<TW, TH>::bytes(), s>>>(f, f.freeDepthFunc,
                                                                                                                  f.freeDepthMask);
    }
    if (!f.orderFree || f.aliasCount)
    {
        /* for an order-free launch with line draws both rasters are queued
         * and the device decides (ordered_raster_runs) */
        raster_ordered_kernel<P, TW, TH, Color, kGeneral><<<numTiles, L::kThreads, L::ordered_bytes(), s>>>(f);
    }
    if (f.aliasCount)
    {
        alias_fixup_kernel<P, Color><<<64, kAliasThreads, 0, s>>>(f);
    }
    return cudaGetLastError();
}

template <class P, int TW, int TH, class Color, bool kGeneral>
cudaError_t raster_attributes_tiles()
{
    typedef RasterLayout<TW, TH, Color> L;
    cudaError_t e = cudaFuncSetAttribute(raster_free_kernel<P, TW, TH, Color, kGeneral>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)FreeLayout<TW, TH>::bytes());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(raster_ordered_kernel<P, TW, TH, Color, kGeneral>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)L::ordered_bytes());
    return e;
}

/* Raster stage for attachment-0 format Color at the frame's tile size. */
template <class P, class Color>
cudaError_t launch_raster_color(const Frame& f, cudaStream_t s)
{
    const int numTiles = f.tilesX * f.tilesY;
    if (f.bestWords)
    {
        /* untiled order-free raster: the clipped fans walked (vs_setup_kernel
         * walked the rest), winners shaded */
        raster_global_kernel<P><<<152 * 16, kGlobalWarps * 32, 0, s>>>(f, f.freeDepthFunc, f.freeDepthMask);
        const unsigned blocks = (unsigned)(((f.width + 15) >> 4) * ((f.height + 15) >> 4));
        resolve_global_kernel<P, Color><<<blocks, 256, 0, s>>>(f, f.freeDepthFunc, f.freeDepthMask);
        return cudaGetLastError();
    }
    if (f.hasLines || f.hasWire || f.hasMrt)
    {
        /* the host sets kLineTile x kLineTile tiles for these launches */
        if (f.tileW != kLineTile || f.tileH != kLineTile) return cudaErrorInvalidValue;
        return launch_raster_tiles<P, kLineTile, kLineTile, Color, true>(f, numTiles, s);
    }
    if (f.tileW == 16 && f.tileH == 16) return launch_raster_tiles<P, 16, 16, Color, false>(f, numTiles, s);
    if (f.tileW == 32 && f.tileH == 16) return launch_raster_tiles<P, 32, 16, Color, false>(f, numTiles, s);
    if (f.tileW == 64 && f.tileH == 32) return launch_raster_tiles<P, 64, 32, Color, false>(f, numTiles, s);
    if (f.tileW == 64 && f.tileH == 64) return launch_raster_tiles<P, 64, 64, Color, false>(f, numTiles, s);
    if (f.tileW == 8 && f.tileH == 8) return launch_raster_tiles<P, 8, 8, Color, false>(f, numTiles, s);
    return launch_raster_tiles<P, 32, 32, Color, false>(f, numTiles, s);
}

/* Raises the dynamic shared-memory limits of the raster kernels of Color
 * once, so launches (and stream captures) need no attribute calls. */
template <class P, class Color>
cudaError_t raster_attributes_color()
{
    cudaError_t e = raster_attributes_tiles<P, 8, 8, Color, false>();
    if (e == cudaSuccess) e = raster_attributes_tiles<P, 16, 16, Color, false>();
    if (e == cudaSuccess) e = raster_attributes_tiles<P, 32, 16, Color, false>();
    if (e == cudaSuccess) e = raster_attributes_tiles<P, 32, 32, Color, false>();
    if (e == cudaSuccess) e = raster_attributes_tiles<P, 64, 32, Color, false>();
    if (e == cudaSuccess) e = raster_attributes_tiles<P, 64, 64, Color, false>();
    if (e == cudaSuccess) e = raster_attributes_tiles<P, kLineTile, kLineTile, Color, true>();
    return e;
}

/* The entry points of a program set, behind the plain-C table the library
 * calls (slg_pipeline_ops, include/slg.h). */
template <class P>
struct PipelineEntry
{
    static int set_attributes()
    {
        cudaError_t e = raster_attributes_color<P, ColorRGBA8>();
        if (e == cudaSuccess) e = raster_attributes_color<P, ColorRGBAF>();
        if (e == cudaSuccess) e = raster_attributes_color<P, ColorRF>();
        return (int)e;
    }
    static int vertex(const void* frame, void* stream)
    {
        return (int)launch_vertex_stage<P>(*static_cast<const Frame*>(frame), static_cast<cudaStream_t>(stream));
    }
    static int raster(const void* frame, void* stream)
    {
        const Frame& f = *static_cast<const Frame*>(frame);
        const cudaStream_t s = static_cast<cudaStream_t>(stream);
        switch (f.colorType)
        {
            case SLG_COLOR_RGBA_FLOAT: return (int)launch_raster_color<P, ColorRGBAF>(f, s);
            case SLG_COLOR_R_FLOAT:    return (int)launch_raster_color<P, ColorRF>(f, s);
            default:                   return (int)launch_raster_color<P, ColorRGBA8>(f, s);
        }
    }
    static slg_pipeline_ops ops()
    {
        slg_pipeline_ops o;
        o.abiVersion = SLG_PIPELINE_ABI_VERSION;
        o.frameBytes = (uint32_t)sizeof(Frame);
        o.set_attributes = &PipelineEntry<P>::set_attributes;
        o.launch_vertex = &PipelineEntry<P>::vertex;
        o.launch_raster = &PipelineEntry<P>::raster;
        return o;
    }
};

} // namespace slg

/* Explicit instantiations of a program set's kernels: the vertex stage and
 * the entry table in one translation unit, the raster stage of each colour
 * format in its own (or all in one), so the kernels compile in parallel. */
#define SLG_PIPELINE_EXTERN(P)                                                                                 \
    extern template cudaError_t slg::launch_raster_color<P, slg::ColorRGBA8>(const slg::Frame&, cudaStream_t); \
    extern template cudaError_t slg::launch_raster_color<P, slg::ColorRGBAF>(const slg::Frame&, cudaStream_t); \
    extern template cudaError_t slg::launch_raster_color<P, slg::ColorRF>(const slg::Frame&, cudaStream_t);    \
    extern template cudaError_t slg::raster_attributes_color<P, slg::ColorRGBA8>();                            \
    extern template cudaError_t slg::raster_attributes_color<P, slg::ColorRGBAF>();                            \
    extern template cudaError_t slg::raster_attributes_color<P, slg::ColorRF>();

#define SLG_PIPELINE_RASTER(P, Color)                                                                   \
    template cudaError_t slg::launch_raster_color<P, slg::Color>(const slg::Frame&, cudaStream_t);   \
    template cudaError_t slg::raster_attributes_color<P, slg::Color>();

#endif /* SLG_PIPELINE_CUH */
