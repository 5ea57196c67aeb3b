/*
 * slg_adjoint.cu - differentiable rendering of one opaque draw of the
 * vertex-colour x float-texture program (SLG_PROGRAM_VCOLOR_TEXF).
 *
 * SoftLight has no adjoint. The model differentiated here is the forward
 * shading of that draw over the coverage the exact rasteriser produced:
 * the order-free raster records, per pixel, which triangle won the depth
 * test (the visibility map); given that map the image is a smooth function
 * of the vertex positions, vertex colours, vertex uvs and texels:
 *
 *   n        = (2x/W - 1, 2y/H - 1)      pixel (x, y) sampled at integer
 *                                         coordinates, as the reference's
 *                                         scan-line loop samples it
 *   h_k      = (clip.x, clip.y, clip.w) of vertex k, clip = MVP (p, 1)
 *   h'_k     = h_k.xy - h_k.w n
 *   e_k      = cross(h'_{k+1}, h'_{k+2}),  l_k = e_k / (e_0 + e_1 + e_2)
 *              (perspective-correct barycentrics of the unsnapped
 *              triangle: the reference's screen barycentrics times 1/w,
 *              renormalised, in closed form)
 *   colour   = sum l_k C_k,  uv = sum l_k UV_k
 *   texel    = bilinear REPEAT sample with the reference's addressing
 *              (x = wrap(u) W, x0 = trunc x, x1 = min(x0 + 1, W), index
 *              x + W y into the padded texel array)
 *   out      = colour * texel
 *
 * The model covers a visible pixel when min l_k >= -1 and its triangle is
 * not a sliver: |e_0 + e_1 + e_2| >= 0.02 x the sum of the squared edge
 * lengths in the h' frame. The exact rasteriser snaps vertices to whole
 * pixels, so a sliver can own pixels well outside its unsnapped shape, where
 * l_k reach tens; and near-degenerate or edge-on triangles have barycentrics
 * that vary as 1/area. Such pixels (about 0.6% of the 512x512 sphere's) keep
 * the framebuffer's colour and carry no gradient.
 *
 * Nothing from the forward pass is stored but the visibility map (4 bytes a
 * pixel): the adjoint recomputes each pixel's barycentrics, varyings and
 * texture footprint from the vertex buffer and the texture, then runs the
 * chain rule backwards. A warp owns 32 consecutive pixels of a row; their
 * contributions are first summed over runs of lanes that share a triangle
 * (vertex gradients) or a bilinear cell (texel gradients) with warp
 * shuffles, then the last lane of each run adds the sums into per-tile
 * (32x8 pixels) shared-memory hash tables, one for vertices and one for
 * texels, with shared FP32 atomics; each tile flushes its tables to HBM
 * with one global FP32 atomic per touched vertex or texel component.
 */
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/slg.h"
#include "slg_adjoint.cuh"
#include "slg_device.cuh"

namespace slg
{
namespace
{

constexpr int kTileX = 32, kTileY = 8, kThreads = kTileX * kTileY;   /* one warp per row */
constexpr int kVertSlots = 512;   /* distinct vertices a tile can stage */
constexpr int kTexSlots = 1024;   /* distinct texels a tile can stage */
constexpr int kProbes = 16;       /* linear-probe bound; then the update goes straight to HBM */
constexpr int kVertFloats = 9;    /* pos[3], rgba[4], uv[2] */
constexpr uint32_t kEmpty = 0xFFFFFFFFu;
constexpr float kMinBarycentric = -1.f;
constexpr float kMinShape = 0.02f;   /* 0.29 for an equilateral triangle */

struct PixelModel
{
    uint32_t vid[3];
    float lam[3];
    float4 C[3];
    float2 U[3];
    float2 hp[3];
    float S, nx, ny;
    float4 colour, texel;
    uint32_t ti[4];
    float w[4];
    float dx, dy;
    float4 T[4];
};

__device__ __forceinline__ uint32_t vertex_id(const DiffArgs& a, uint64_t e)
{
    if (a.indexType < 0) return (uint32_t)e;
    switch (a.indexType)
    {
        case SLG_VERTEX_DATA_BYTE:  return a.ibo[e];
        case SLG_VERTEX_DATA_SHORT: return reinterpret_cast<const uint16_t*>(a.ibo)[e];
        default:                    return reinterpret_cast<const uint32_t*>(a.ibo)[e];
    }
}

__device__ __forceinline__ float wrap_unit(float t)
{
    return wrap_repeat(t);
}

__device__ __forceinline__ float4 f4_scale(float4 v, float s) { return make_float4(v.x * s, v.y * s, v.z * s, v.w * s); }
__device__ __forceinline__ float4 f4_add(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ __forceinline__ float4 f4_mul(float4 a, float4 b) { return make_float4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
__device__ __forceinline__ float f4_dot(float4 a, float4 b) { return ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w; }

/* Forward model at pixel (x, y) whose visibility id is `id`; false when the
 * pixel has no (valid) triangle or a degenerate one. Every texel index it
 * forms is at most W + W*H, inside the texture's zero padding. */
__device__ bool pixel_model(const DiffArgs& a, int x, int y, uint32_t id, PixelModel& m)
{
    if (id == 0u || id > a.numTris) return false;
    const uint64_t e0 = a.elementBegin + 3ull * (uint64_t)(id - 1u);
    m.nx = (2.f * (float)x) / (float)a.width - 1.f;
    m.ny = (2.f * (float)y) / (float)a.height - 1.f;
    const float* M = a.mvp;
#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
        const uint32_t vid = vertex_id(a, e0 + k);
        m.vid[k] = vid;
        const float* v = reinterpret_cast<const float*>(a.vbo + a.b0Offset + a.b0Stride * (int64_t)vid);
        const float p0 = v[0], p1 = v[1], p2 = v[2];
        m.C[k] = make_float4(v[3], v[4], v[5], v[6]);
        m.U[k] = make_float2(v[7], v[8]);
        const float cx = ((M[0] * p0 + M[4] * p1) + M[8] * p2) + M[12];
        const float cy = ((M[1] * p0 + M[5] * p1) + M[9] * p2) + M[13];
        const float cw = ((M[3] * p0 + M[7] * p1) + M[11] * p2) + M[15];
        m.hp[k] = make_float2(cx - cw * m.nx, cy - cw * m.ny);
    }
    float e[3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
        const float2 p = m.hp[(k + 1) % 3], q = m.hp[(k + 2) % 3];
        e[k] = p.x * q.y - p.y * q.x;
    }
    m.S = (e[0] + e[1]) + e[2];
    if (!(m.S != 0.f) || !isfinite(m.S)) return false;
    /* slivers and edge-on triangles (barycentrics vary as 1/area) are
     * outside the model: |2 x area| >= kMinShape x sum of squared edges */
    float e2 = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
        const float2 p = m.hp[(k + 1) % 3], q = m.hp[k];
        e2 += (p.x - q.x) * (p.x - q.x) + (p.y - q.y) * (p.y - q.y);
    }
    if (fabsf(m.S) < kMinShape * e2) return false;
#pragma unroll
    for (int k = 0; k < 3; ++k) m.lam[k] = e[k] / m.S;
    /* the model's domain: pixels within one triangle height of every edge of
     * the unsnapped triangle (barycentrics >= -1). Snapping lets slivers
     * cover pixels far outside their unsnapped shape, where extrapolation is
     * ill-conditioned; those pixels keep the exact colour and no gradient. */
    if (fminf(fminf(m.lam[0], m.lam[1]), m.lam[2]) < kMinBarycentric) return false;
    float4 col = make_float4(0.f, 0.f, 0.f, 0.f);
    float u = 0.f, vv = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
        col = f4_add(col, f4_scale(m.C[k], m.lam[k]));
        u += m.U[k].x * m.lam[k];
        vv += m.U[k].y * m.lam[k];
    }
    m.colour = col;

    const uint32_t W = a.texW, H = a.texH;
    const float xf = wrap_unit(u) * (float)W;
    const float yf = wrap_unit(vv) * (float)H;
    const uint32_t xi0 = (uint32_t)f2i(xf) & 0xFFFFu;
    const uint32_t yi0 = (uint32_t)f2i(yf) & 0xFFFFu;
    const uint32_t xi1 = min((xi0 + 1u) & 0xFFFFu, W);
    const uint32_t yi1 = min((yi0 + 1u) & 0xFFFFu, H);
    /* xi0 <= W and yi0 <= H hold for any float input (wrap_unit is in
     * [0, 1] or NaN, and f2i(NaN) masks to 0); clamp anyway */
    const uint32_t x0 = min(xi0, W), y0 = min(yi0, H);
    m.dx = xf - (float)xi0;
    m.dy = yf - (float)yi0;
    m.ti[0] = x0 + W * y0;
    m.ti[1] = x0 + W * yi1;
    m.ti[2] = xi1 + W * y0;
    m.ti[3] = xi1 + W * yi1;
    m.w[0] = (1.f - m.dx) * (1.f - m.dy);
    m.w[1] = (1.f - m.dx) * m.dy;
    m.w[2] = m.dx * (1.f - m.dy);
    m.w[3] = m.dx * m.dy;
    float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int j = 0; j < 4; ++j)
    {
        m.T[j] = __ldg(a.texels + m.ti[j]);
        t = f4_add(t, f4_scale(m.T[j], m.w[j]));
    }
    m.texel = t;
    return true;
}

__global__ void __launch_bounds__(kThreads) diff_shade_kernel(const DiffArgs a)
{
    const int x = blockIdx.x * kTileX + (threadIdx.x % kTileX);
    const int y = blockIdx.y * kTileY + (threadIdx.x / kTileX);
    if (x >= a.width || y >= a.height) return;
    const size_t gi = (size_t)x + (size_t)a.width * y;
    PixelModel m;
    float4 out = a.exact ? a.exact[gi] : make_float4(0.f, 0.f, 0.f, 0.f);
    if (pixel_model(a, x, y, a.vis[gi], m)) out = f4_mul(m.colour, m.texel);
    a.image[gi] = out;
}

/* Slot of `key` in a shared open-addressing table, inserting it if absent;
 * -1 after kProbes occupied slots. Keys never leave the table during a
 * kernel, so a slot read as `key` stays `key`. */
__device__ __forceinline__ int stage_slot(uint32_t* keys, int mask, uint32_t key)
{
    uint32_t h = (key * 2654435761u) >> 7;
#pragma unroll 1
    for (int p = 0; p < kProbes; ++p)
    {
        h &= (uint32_t)mask;
        const uint32_t cur = *(volatile uint32_t*)(keys + h);
        if (cur == key) return (int)h;
        if (cur == kEmpty)
        {
            const uint32_t prev = atomicCAS(keys + h, kEmpty, key);
            if (prev == kEmpty || prev == key) return (int)h;
        }
        ++h;
    }
    return -1;
}

/* Segmented inclusive sum of v over runs of equal `key` in consecutive lanes
 * (lane i and i + 1 in one run when their keys match): afterwards the last
 * lane of each run holds the run's totals. Returns whether this lane is the
 * last of its run. All 32 lanes must call it. */
template <int N>
__device__ __forceinline__ bool run_reduce(uint32_t key, float (&v)[N])
{
    const int lane = threadIdx.x & 31;
    const uint32_t prev = __shfl_up_sync(0xFFFFFFFFu, key, 1);
    const uint32_t heads = __ballot_sync(0xFFFFFFFFu, lane == 0 || key != prev);
    const int start = 31 - __clz(heads & (0xFFFFFFFFu >> (31 - lane)));
#pragma unroll
    for (int off = 1; off < 32; off <<= 1)
    {
        const bool take = lane - off >= start;
#pragma unroll
        for (int i = 0; i < N; ++i)
        {
            const float t = __shfl_up_sync(0xFFFFFFFFu, v[i], off);
            if (take) v[i] += t;
        }
    }
    return lane == 31 || ((heads >> (lane + 1)) & 1u);
}

/* One warp per 32-pixel row segment. Each pixel's contributions are summed
 * over runs of lanes with the same triangle (vertex gradients) and the same
 * bilinear cell (texel gradients) with warp shuffles; the last lane of each
 * run adds the run's sums into the tile's shared tables, which are flushed
 * to HBM with global FP32 atomics once per tile. */
__global__ void __launch_bounds__(kThreads) diff_adjoint_kernel(const DiffArgs a)
{
    __shared__ uint32_t vKey[kVertSlots];
    __shared__ float vVal[kVertSlots * kVertFloats];
    __shared__ uint32_t tKey[kTexSlots];
    __shared__ float4 tVal[kTexSlots];

    const int tid = threadIdx.x;
    for (int i = tid; i < kVertSlots; i += kThreads) vKey[i] = kEmpty;
    for (int i = tid; i < kVertSlots * kVertFloats; i += kThreads) vVal[i] = 0.f;
    for (int i = tid; i < kTexSlots; i += kThreads)
    {
        tKey[i] = kEmpty;
        tVal[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();

    const int x = blockIdx.x * kTileX + (tid % kTileX);
    const int y = blockIdx.y * kTileY + (tid / kTileX);
    PixelModel m;
    const bool live = x < a.width && y < a.height && pixel_model(a, x, y, a.vis[(size_t)x + (size_t)a.width * y], m);

    float vv[3 * kVertFloats];
    float tv[16];
#pragma unroll
    for (int i = 0; i < 3 * kVertFloats; ++i) vv[i] = 0.f;
#pragma unroll
    for (int i = 0; i < 16; ++i) tv[i] = 0.f;
    uint32_t triKey = kEmpty, cellKey = kEmpty;

    if (live)
    {
        triKey = a.vis[(size_t)x + (size_t)a.width * y];
        cellKey = m.ti[0];
        const float4 g = a.dImage[(size_t)x + (size_t)a.width * y];
        const float4 gc = f4_mul(g, m.texel);    /* dL/d colour varying */
        const float4 gt = f4_mul(g, m.colour);   /* dL/d texture sample */

        /* texture sample w.r.t. its cell coordinates, then uv */
        const float4 dSdx = f4_add(f4_add(f4_scale(m.T[0], -(1.f - m.dy)), f4_scale(m.T[1], -m.dy)),
                                   f4_add(f4_scale(m.T[2], 1.f - m.dy), f4_scale(m.T[3], m.dy)));
        const float4 dSdy = f4_add(f4_add(f4_scale(m.T[0], -(1.f - m.dx)), f4_scale(m.T[1], 1.f - m.dx)),
                                   f4_add(f4_scale(m.T[2], -m.dx), f4_scale(m.T[3], m.dx)));
        const float du = f4_dot(gt, dSdx) * (float)a.texW;
        const float dv = f4_dot(gt, dSdy) * (float)a.texH;

        /* barycentrics */
        float dl[3];
        float ldl = 0.f;
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            dl[k] = f4_dot(gc, m.C[k]) + (du * m.U[k].x + dv * m.U[k].y);
            ldl += m.lam[k] * dl[k];
        }
        float2 dhp[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            const float de = (dl[k] - ldl) / m.S;
            const int k1 = (k + 1) % 3, k2 = (k + 2) % 3;
            const float2 p = m.hp[k1], q = m.hp[k2];
            dhp[k1].x += q.y * de;
            dhp[k1].y -= q.x * de;
            dhp[k2].x -= p.y * de;
            dhp[k2].y += p.x * de;
        }

        const float* M = a.mvp;
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            /* clip gradient (x, y, 0, w), then positions: dp_c = sum_r M[r][c] dclip_r */
            const float dcx = dhp[k].x, dcy = dhp[k].y;
            const float dcw = -(m.nx * dcx + m.ny * dcy);
            float* o = vv + k * kVertFloats;
            o[0] = (M[0] * dcx + M[1] * dcy) + M[3] * dcw;
            o[1] = (M[4] * dcx + M[5] * dcy) + M[7] * dcw;
            o[2] = (M[8] * dcx + M[9] * dcy) + M[11] * dcw;
            o[3] = gc.x * m.lam[k];
            o[4] = gc.y * m.lam[k];
            o[5] = gc.z * m.lam[k];
            o[6] = gc.w * m.lam[k];
            o[7] = du * m.lam[k];
            o[8] = dv * m.lam[k];
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
        {
            tv[4 * j + 0] = gt.x * m.w[j];
            tv[4 * j + 1] = gt.y * m.w[j];
            tv[4 * j + 2] = gt.z * m.w[j];
            tv[4 * j + 3] = gt.w * m.w[j];
        }
    }

    if (run_reduce(triKey, vv) && triKey != kEmpty)
    {
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            const float* o = vv + k * kVertFloats;
            const int s = stage_slot(vKey, kVertSlots - 1, m.vid[k]);
            if (s >= 0)
            {
#pragma unroll
                for (int c = 0; c < kVertFloats; ++c) atomicAdd(&vVal[s * kVertFloats + c], o[c]);
            }
            else
            {
                float* dst = a.dVertices + (a.b0Offset + a.b0Stride * (int64_t)m.vid[k]) / 4;
#pragma unroll
                for (int c = 0; c < kVertFloats; ++c) atomicAdd(dst + c, o[c]);
            }
        }
    }

    if (run_reduce(cellKey, tv) && cellKey != kEmpty)
    {
        const uint32_t numTexels = a.texW * a.texH;
#pragma unroll
        for (int j = 0; j < 4; ++j)
        {
            if (m.ti[j] >= numTexels) continue;   /* zero padding: a constant */
            const float4 v = make_float4(tv[4 * j], tv[4 * j + 1], tv[4 * j + 2], tv[4 * j + 3]);
            const int s = stage_slot(tKey, kTexSlots - 1, m.ti[j]);
            if (s >= 0)
            {
                atomicAdd(&tVal[s].x, v.x);
                atomicAdd(&tVal[s].y, v.y);
                atomicAdd(&tVal[s].z, v.z);
                atomicAdd(&tVal[s].w, v.w);
            }
            else
            {
                atomicAdd(a.dTexels + m.ti[j], v);
            }
        }
    }
    __syncthreads();

    /* flush the tile's partial sums */
    for (int i = tid; i < kVertSlots; i += kThreads)
    {
        const uint32_t key = vKey[i];
        if (key == kEmpty) continue;
        float* dst = a.dVertices + (a.b0Offset + a.b0Stride * (int64_t)key) / 4;
#pragma unroll
        for (int c = 0; c < kVertFloats; ++c)
        {
            const float v = vVal[i * kVertFloats + c];
            if (v != 0.f) atomicAdd(dst + c, v);
        }
    }
    for (int i = tid; i < kTexSlots; i += kThreads)
    {
        const uint32_t key = tKey[i];
        if (key == kEmpty) continue;
        atomicAdd(a.dTexels + key, tVal[i]);
    }
}

} // namespace

cudaError_t launch_diff_shade(const DiffArgs& a, cudaStream_t s)
{
    const dim3 grid((a.width + kTileX - 1) / kTileX, (a.height + kTileY - 1) / kTileY);
    diff_shade_kernel<<<grid, kThreads, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_diff_adjoint(const DiffArgs& a, cudaStream_t s)
{
    const dim3 grid((a.width + kTileX - 1) / kTileX, (a.height + kTileY - 1) / kTileY);
    diff_adjoint_kernel<<<grid, kThreads, 0, s>>>(a);
    return cudaGetLastError();
}

} // namespace slg
