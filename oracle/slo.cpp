/*
 * slo.cpp - CPU oracle for the GB300 draw path (test infrastructure only).
 *
 * This file restates, in plain C++, the arithmetic and ordering of
 * SoftLight's triangle draw path as compiled WITHOUT any LS_X86_* / LS_ARM_*
 * macro, i.e. the portable branches of every #if ladder, with FP contraction
 * off and one thread. Nothing in the product links or calls it: the tests,
 * the smoke check and the benchmark's CPU-baseline leg use it as the checker
 * and as the timed CPU restatement.
 *
 * Each function names the reference code it follows (paths relative to the
 * SoftLight source tree). The reference's vector library (LightMath, an
 * absent git submodule) is restated with these definitions, shared with the
 * GPU path and with the compatibility shim used to build the reference
 * sources themselves:
 *   fmadd(a,b,c) = a*b + c (two roundings); rcp(x) = 1/x;
 *   dot / sum fold left: ((a0+a1)+a2)+a3;  mix(a,b,t) = (b-a)*t + a;
 *   cross(vec4 a, vec4 b) = (a1*b2-a2*b1, a2*b0-a0*b2, a0*b1-a1*b0, 0);
 *   cross(vec2 a, vec2 b) = a0*b1 - a1*b0;  max(a,b) = a<b ? b : a;
 *   min(a,b) = b<a ? b : a;  vec4 <= / >= compare all four components;
 *   mat4 * vec4 = m[0]*v0 + m[1]*v1 + m[2]*v2 + m[3]*v3 (columns, left fold);
 *   float -> int32 conversions behave like x86 cvttss2si (NaN / out of
 *   range -> INT32_MIN) so the result does not depend on the host ISA.
 */
#include "slo.h"
#include "../include/slg_half.h"
#include "../include/slg_programs.h"

#include <algorithm>
#include <condition_variable>
#include <functional>
#include <memory>
#include <mutex>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <array>
#include <vector>

namespace
{

/*-----------------------------------------------------------------------------
 * Restated LightMath helpers
-----------------------------------------------------------------------------*/
struct V4
{
    float v[4];
    float& operator[](int i) { return v[i]; }
    float operator[](int i) const { return v[i]; }
};

static inline V4 mk(float a, float b, float c, float d) { V4 r; r.v[0] = a; r.v[1] = b; r.v[2] = c; r.v[3] = d; return r; }
static inline V4 add(const V4& a, const V4& b) { return mk(a[0] + b[0], a[1] + b[1], a[2] + b[2], a[3] + b[3]); }
static inline V4 sub(const V4& a, const V4& b) { return mk(a[0] - b[0], a[1] - b[1], a[2] - b[2], a[3] - b[3]); }
static inline V4 mul(const V4& a, const V4& b) { return mk(a[0] * b[0], a[1] * b[1], a[2] * b[2], a[3] * b[3]); }
static inline V4 mulf(const V4& a, float s) { return mk(a[0] * s, a[1] * s, a[2] * s, a[3] * s); }
static inline float dot(const V4& a, const V4& b) { return ((a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]) + a[3] * b[3]; }
static inline float lm_max(float a, float b) { return (a < b) ? b : a; }
static inline float lm_min(float a, float b) { return (b < a) ? b : a; }
static inline V4 mix(const V4& a, const V4& b, float t)
{
    return mk((b[0] - a[0]) * t + a[0], (b[1] - a[1]) * t + a[1], (b[2] - a[2]) * t + a[2], (b[3] - a[3]) * t + a[3]);
}
static inline int sign_mask(float f) { uint32_t u; std::memcpy(&u, &f, 4); return (int)(u >> 31); }

static inline int32_t f2i(float f)
{
    if (!(f >= -2147483648.f && f < 2147483648.f))
    {
        return INT32_MIN;
    }
    return (int32_t)f;
}

static inline uint8_t f2u8(float f) { return (uint8_t)(uint32_t)f2i(f); }

/* mat4 (column-major, 16 floats) * vec4 as ls::math does it */
static inline V4 mat_mul(const float* m, const V4& v)
{
    V4 r;
    for (int row = 0; row < 4; ++row)
    {
        r[row] = ((m[0 + row] * v[0] + m[4 + row] * v[1]) + m[8 + row] * v[2]) + m[12 + row] * v[3];
    }
    return r;
}

/*-----------------------------------------------------------------------------
 * Resources
-----------------------------------------------------------------------------*/
struct Texture
{
    int type = -1;
    uint16_t w = 0, h = 0, d = 0;
    unsigned bpt = 0;
    std::vector<uint8_t> bytes;
};

struct Vbo { std::vector<uint8_t> bytes; };

struct Ibo
{
    int type = SLG_VERTEX_DATA_INVALID;
    size_t count = 0;
    std::vector<uint8_t> bytes;
};

struct Binding { ptrdiff_t offset = 0, stride = 0; unsigned comps = 0; int type = 0; };

struct Vao
{
    size_t vbo = SLG_INVALID_ID, ibo = SLG_INVALID_ID;
    Binding bindings[8];
};

struct Fbo
{
    unsigned numColors = 0;
    size_t colors[4] = {SLG_INVALID_ID, SLG_INVALID_ID, SLG_INVALID_ID, SLG_INVALID_ID};
    size_t depth = SLG_INVALID_ID;
};

struct Ubo { alignas(16) uint8_t bytes[1024]; };

struct Shader
{
    uint8_t cull, depthTest, depthMask, blend, numVaryings, numOutputs;
    uint32_t vsProgram, fsProgram;
    size_t ubo;
};

/* SL_TransformedVert (softlight/include/softlight/SL_ShaderUtil.hpp:612) */
struct TVert
{
    V4 vert;
    V4 varyings[4];
};

/* SL_FragmentBin (softlight/include/softlight/SL_ShaderUtil.hpp:627) */
struct Bin
{
    V4 screen[3];
    V4 bc[3];
    V4 varyings[12];
    size_t primIndex;
    uint32_t drawIndex;
};

/* The packed formats SL_COLOR_RGB_332 .. SL_COLOR_RGBA_1010102 (28..32,
 * softlight/include/softlight/SL_ColorCompressed.hpp): unsigned bitfields
 * allocated from bit 0 up, as gcc lays them out on little-endian targets. */
struct PackedFormat
{
    int nc, bytes;
    int bits[4], shift[4];
};

static const PackedFormat kPacked[5] = {
    {3, 1, {3, 3, 2, 0}, {0, 3, 6, 0}},          /* RGB 332 */
    {3, 2, {5, 6, 5, 0}, {0, 5, 11, 0}},         /* RGB 565 */
    {4, 2, {5, 5, 5, 1}, {0, 5, 10, 15}},        /* RGBA 5551 */
    {4, 2, {4, 4, 4, 4}, {0, 4, 8, 12}},         /* RGBA 4444 */
    {4, 4, {10, 10, 10, 2}, {0, 10, 20, 30}},    /* RGBA 1010102 */
};

/* bytes of a texel of SL_ColorDataType 0..32: components type / 7 + 1 of
 * u8, u16, u32, u64, half, float, double by type % 7, then the packed
 * formats (sl_bytes_per_color, softlight/src/SL_Color.cpp:12-56) */
static size_t bytes_per_color(int type)
{
    if (type >= 28 && type <= 32) return (size_t)kPacked[type - 28].bytes;
    if (type < 0 || type > 27) return 0;
    static const size_t kind[7] = {1, 2, 4, 8, 2, 4, 8};
    return (size_t)(type / 7 + 1) * kind[type % 7];
}

static size_t index_bytes(int type)
{
    switch (type)
    {
        case SLG_VERTEX_DATA_BYTE: return 1;
        case SLG_VERTEX_DATA_SHORT: return 2;
        case SLG_VERTEX_DATA_INT: return 4;
        default: return 0;
    }
}

} // namespace

/* A scene graph (SL_SceneGraph's node arrays, softlight/include/softlight/
 * SL_SceneGraph.hpp:224-300): nodes in insertion order, a parent before its
 * children. */
struct SloScene
{
    std::vector<uint64_t> parents;             /* SLG_SCENE_ROOT or an earlier node */
    std::vector<slg_transform> transforms;
    std::vector<uint8_t> dirty;
    std::vector<std::array<float, 16>> models;
    std::vector<std::vector<uint64_t>> nodeMeshes;   /* empty for an empty node */
    std::vector<slg_mesh> meshes;
    std::vector<std::array<float, 8>> bounds;  /* mMeshBounds: max xyzw, min xyzw */
    std::vector<size_t> materials;             /* ambient texture per material */
};

/* A fixed set of host threads, kept by the context, that run one phase
 * function at a time: run(fn) calls fn(t) on thread t for every t (the
 * calling thread takes t = 0) and returns when all have finished, like the
 * reference's persistent processor pool (SL_ProcessorPool.cpp:280-380). */
class WorkerPool
{
  public:
    explicit WorkerPool(unsigned n) : mN(n)
    {
        for (unsigned t = 1; t < n; ++t) mThreads.emplace_back([this, t]() { loop(t); });
    }
    ~WorkerPool()
    {
        {
            std::lock_guard<std::mutex> lk(mMutex);
            mStop = true;
            ++mGen;
        }
        mCv.notify_all();
        for (std::thread& th : mThreads) th.join();
    }
    unsigned size() const { return mN; }
    void run(const std::function<void(unsigned)>& fn)
    {
        {
            std::lock_guard<std::mutex> lk(mMutex);
            mFn = fn;
            mPending = mN - 1;
            ++mGen;
        }
        mCv.notify_all();
        mFn(0u);
        std::unique_lock<std::mutex> lk(mMutex);
        mDone.wait(lk, [this]() { return mPending == 0; });
    }

  private:
    void loop(unsigned t)
    {
        uint64_t seen = 0;
        for (;;)
        {
            {
                std::unique_lock<std::mutex> lk(mMutex);
                mCv.wait(lk, [&]() { return mGen != seen; });
                seen = mGen;
                if (mStop) return;
            }
            mFn(t);
            std::lock_guard<std::mutex> lk(mMutex);
            if (--mPending == 0) mDone.notify_one();
        }
    }
    std::function<void(unsigned)> mFn;
    unsigned mN;
    std::vector<std::thread> mThreads;
    std::mutex mMutex;
    std::condition_variable mCv, mDone;
    uint64_t mGen = 0;
    unsigned mPending = 0;
    bool mStop = false;
};

struct slo_context
{
    std::string err;
    unsigned numThreads = 1;
    std::vector<Vbo> vbos;
    std::vector<Ibo> ibos;
    std::vector<Vao> vaos;
    std::vector<Texture*> textures;
    std::vector<Fbo> fbos;
    std::vector<Ubo*> ubos;
    std::vector<Shader> shaders;
    std::vector<SloScene> scenes;
    uint64_t lastBins = 0, lastFrags = 0;
    std::unique_ptr<WorkerPool> pool;   /* host threads of the multi-threaded mode */

    ~slo_context()
    {
        for (Texture* t : textures) delete t;
        for (Ubo* u : ubos) delete u;
    }

    int fail(int code, const char* msg) { err = msg; return code; }
};

namespace
{

/*-----------------------------------------------------------------------------
 * Shader environment for the built-in programs
-----------------------------------------------------------------------------*/
/* sl_sample_bilinear<color, SL_WrapMode::REPEAT, ORDERED>
 * (softlight/include/softlight/SL_Sampler.hpp:97-115,187-218) */
static inline float wrap_repeat(float uvw)
{
    /* fmod(uvw, 1) as uvw - trunc(uvw): exact for every binary32 input
     * (Sterbenz for |uvw| >= 1, trunc = 0 below), so the same value as
     * the reference's fmod at a fraction of its cost */
    return (uvw < 0.f ? 1.f : 0.f) + (uvw - std::trunc(uvw));
}

struct BilinearCoords
{
    uint32_t i00, i01, i10, i11;
    float omdx, omdy, dx, dy;
};

static inline BilinearCoords bilinear_coords(const Texture& t, float x, float y)
{
    const float xf = wrap_repeat(x) * (float)t.w;
    const float yf = wrap_repeat(y) * (float)t.h;
    const uint16_t xi0 = (uint16_t)(uint32_t)f2i(xf);
    const uint16_t yi0 = (uint16_t)(uint32_t)f2i(yf);
    const uint16_t xn = (uint16_t)(xi0 + 1u);
    const uint16_t yn = (uint16_t)(yi0 + 1u);
    const uint16_t xi1 = (t.w < xn) ? t.w : xn;
    const uint16_t yi1 = (t.h < yn) ? t.h : yn;
    BilinearCoords c;
    c.dx = xf - (float)xi0;
    c.dy = yf - (float)yi0;
    c.omdx = 1.f - c.dx;
    c.omdy = 1.f - c.dy;
    c.i00 = (uint32_t)xi0 + (uint32_t)t.w * yi0;
    c.i01 = (uint32_t)xi0 + (uint32_t)t.w * yi1;
    c.i10 = (uint32_t)xi1 + (uint32_t)t.w * yi0;
    c.i11 = (uint32_t)xi1 + (uint32_t)t.w * yi1;
    return c;
}

static inline V4 sample_rgba8(const Texture& t, float x, float y)
{
    const BilinearCoords c = bilinear_coords(t, x, y);
    const uint8_t* p = t.bytes.data();
    V4 px[4];
    const uint32_t idx[4] = {c.i00, c.i01, c.i10, c.i11};
    for (int k = 0; k < 4; ++k)
    {
        const uint8_t* q = p + 4u * (size_t)idx[k];
        /* color_cast<float, uint8_t> (softlight/include/softlight/SL_Color.hpp:674) */
        px[k] = mk((float)q[0] * 0.00392156862745f, (float)q[1] * 0.00392156862745f,
                   (float)q[2] * 0.00392156862745f, (float)q[3] * 0.00392156862745f);
    }
    const V4 w0 = mulf(mulf(px[0], c.omdx), c.omdy);
    const V4 w1 = mulf(mulf(px[1], c.omdx), c.dy);
    const V4 w2 = mulf(mulf(px[2], c.dx), c.omdy);
    const V4 w3 = mulf(mulf(px[3], c.dx), c.dy);
    const V4 s = add(add(add(w0, w1), w2), w3);
    /* color_cast<uint8_t, float> then back to float in the shader */
    V4 r;
    for (int k = 0; k < 4; ++k)
    {
        r[k] = (float)f2u8(s[k] * 255.f) * 0.00392156862745f;
    }
    return r;
}

static inline V4 sample_rgbaf(const Texture& t, float x, float y)
{
    const BilinearCoords c = bilinear_coords(t, x, y);
    const float* p = reinterpret_cast<const float*>(t.bytes.data());
    V4 px[4];
    const uint32_t idx[4] = {c.i00, c.i01, c.i10, c.i11};
    for (int k = 0; k < 4; ++k)
    {
        const float* q = p + 4u * (size_t)idx[k];
        px[k] = mk(q[0], q[1], q[2], q[3]);
    }
    const V4 w0 = mulf(mulf(px[0], c.omdx), c.omdy);
    const V4 w1 = mulf(mulf(px[1], c.omdx), c.dy);
    const V4 w2 = mulf(mulf(px[2], c.dx), c.omdy);
    const V4 w3 = mulf(mulf(px[3], c.dx), c.dy);
    return add(add(add(w0, w1), w2), w3);
}

struct Env
{
    const slo_context* ctx;
    const uint8_t* vboBytes;
    Binding b0;
    const uint8_t* ubo;

    const float* vertex(uint64_t vertId) const
    {
        return reinterpret_cast<const float*>(vboBytes + b0.offset + b0.stride * (ptrdiff_t)vertId);
    }
    const void* uniforms() const { return ubo; }
    const float* buffer(uint32_t vboId) const
    {
        return reinterpret_cast<const float*>(ctx->vbos[vboId].bytes.data());
    }
    slg_v4 sample_rgba8(uint32_t texId, float u, float v) const
    {
        const V4 r = ::sample_rgba8(*ctx->textures[texId], u, v);
        return slg_make_v4(r[0], r[1], r[2], r[3]);
    }
    slg_v4 sample_rgbaf(uint32_t texId, float u, float v) const
    {
        const V4 r = ::sample_rgbaf(*ctx->textures[texId], u, v);
        return slg_make_v4(r[0], r[1], r[2], r[3]);
    }
};

static inline V4 from_slg(const slg_v4& a) { return mk(a.x, a.y, a.z, a.w); }
static inline slg_v4 to_slg(const V4& a) { return slg_make_v4(a[0], a[1], a[2], a[3]); }

static V4 run_vs(uint32_t program, const Env& env, uint64_t vertId, uint64_t instId, V4* varyings)
{
    slg_v4 vary[4];
    slg_v4 r;
    switch (program)
    {
        case SLG_PROGRAM_LAMBERT_TEX:      r = slg_vs_lambert(env, vertId, instId, vary); break;
        case SLG_PROGRAM_BLINN_PHONG_INST: r = slg_vs_blinn(env, vertId, instId, vary); break;
        case SLG_PROGRAM_VCOLOR_TEX_ALPHA:
        case SLG_PROGRAM_VCOLOR_TEXF:
        case SLG_PROGRAM_GBUFFER:
        case SLG_PROGRAM_VCOLOR_TEX_CUTOUT:
        case SLG_PROGRAM_FRAG_COORD:       r = slg_vs_vcolor(env, vertId, instId, vary); break;
        default:                           r = slg_vs_flat(env, vertId, instId, vary); break;
    }
    for (int i = 0; i < 4; ++i) varyings[i] = from_slg(vary[i]);
    return from_slg(r);
}

/* The fragment program with SL_FragmentParam's coord (x, y, depth) in and
 * out: the depth buffer receives coord.depth after the program
 * (SL_FragmentProcessor.cpp:501-529). */
static bool run_fs(uint32_t program, const Env& env, slg_frag_coord& coord, const V4* varyings, V4* outputs)
{
    slg_v4 vary[4], outs[4];
    for (int i = 0; i < 4; ++i) { vary[i] = to_slg(varyings[i]); outs[i] = slg_make_v4(0.f, 0.f, 0.f, 0.f); }
    bool r;
    switch (program)
    {
        case SLG_PROGRAM_LAMBERT_TEX:      r = slg_fs_lambert(env, vary, outs); break;
        case SLG_PROGRAM_BLINN_PHONG_INST: r = slg_fs_blinn(env, vary, outs); break;
        case SLG_PROGRAM_VCOLOR_TEX_ALPHA: r = slg_fs_vcolor_tex_alpha(env, vary, outs); break;
        case SLG_PROGRAM_VCOLOR_TEXF:      r = slg_fs_vcolor_texf(env, vary, outs); break;
        case SLG_PROGRAM_GBUFFER:          r = slg_fs_gbuffer(env, vary, outs); break;
        case SLG_PROGRAM_VCOLOR_TEX_CUTOUT: r = slg_fs_cutout(env, vary, outs); break;
        case SLG_PROGRAM_FRAG_COORD:       r = slg_fs_frag_coord(env, &coord, vary, outs); break;
        default:                           r = slg_fs_flat(env, vary, outs); break;
    }
    for (int i = 0; i < 4; ++i) outputs[i] = from_slg(outs[i]);
    return r;
}

static inline slg_frag_coord frag_coord(uint32_t x, uint32_t y, float depth)
{
    slg_frag_coord c;
    c.x = (uint16_t)x;
    c.y = (uint16_t)y;
    c.depth = depth;
    return c;
}

/*-----------------------------------------------------------------------------
 * Vertex stage (softlight/src/SL_TriProcessor.cpp)
-----------------------------------------------------------------------------*/
/* face_determinant, portable branch (SL_TriProcessor.cpp:98-115) */
static inline float face_determinant(const V4& p0, const V4& p1, const V4& p2)
{
    const float w0 = 1.f / p0[3];
    const float w1 = 1.f / p1[3];
    const float w2 = 1.f / p2[3];
    const V4 v0 = mulf(p0, w0);
    const V4 v1 = mulf(p1, w1);
    const V4 v2 = mulf(p2, w2);
    const V4 yCAB = mk(v2[1], v0[1], v1[1], 0.f);
    const V4 yBCA = mk(v1[1], v2[1], v0[1], 0.f);
    const V4 xABC = mk(v0[0], v1[0], v2[0], 0.f);
    return dot(xABC, sub(yBCA, yCAB));
}

/* sl_ndc_clip_status, portable branch (SL_PostVertexTransform.hpp:651-673) */
static inline int clip_status(const V4& c0, const V4& c1, const V4& c2)
{
    auto le = [](const V4& c, float w) { return c[0] <= w && c[1] <= w && c[2] <= w && c[3] <= w; };
    auto ge = [](const V4& c, float w) { return c[0] >= w && c[1] >= w && c[2] >= w && c[3] >= w; };
    const bool vis = le(c0, c0[3]) && le(c1, c1[3]) && le(c2, c2[3]) &&
                     ge(c0, -c0[3]) && ge(c1, -c1[3]) && ge(c2, -c2[3]);
    const bool part = c0[3] > 0.f || c1[3] > 0.f || c2[3] > 0.f;
    return (vis ? 3 : 0) | (part ? 1 : 0);
}

/* sl_perspective_divide, portable branch (SL_PostVertexTransform.hpp:240-249) */
static inline void perspective_divide(V4& v)
{
    const float wInv = 1.f / v[3];
    const V4 m = mulf(v, wInv);
    v = mk(m[0], m[1], m[2], wInv);
}

/* sl_ndc_to_screen_coords, portable branch (SL_PostVertexTransform.hpp:509-524) */
static inline void ndc_to_screen(V4& p, const V4& vp)
{
    const float w = vp[2] * 0.5f;
    const float h = vp[3] * 0.5f;
    p[0] = lm_max(std::floor((p[0] + 1.f) * w + vp[0]), 0.f);
    p[1] = lm_max(std::floor((p[1] + 1.f) * h + vp[1]), 0.f);
}

struct DrawState
{
    const slo_context* ctx;
    const Shader* shader;
    Env env;
    float scissor[16];
    V4 viewport;
    unsigned numVaryings;
    uint32_t drawIndex;
};

/* SL_TriProcessor::push_bin (SL_TriProcessor.cpp:248-342) */
static void push_bin(const DrawState& ds, std::vector<Bin>& bins, size_t primIndex, const TVert& a, const TVert& b, const TVert& c)
{
    const V4& p0 = a.vert;
    const V4& p1 = b.vert;
    const V4& p2 = c.vert;

    const float minX = lm_min(lm_min(p0[0], p1[0]), p2[0]);
    const float minY = lm_min(lm_min(p0[1], p1[1]), p2[1]);
    const float maxX = lm_max(lm_max(p0[0], p1[0]), p2[0]);
    const float maxY = lm_max(lm_max(p0[1], p1[1]), p2[1]);
    if ((maxX - minX < 1.f) || (maxY - minY < 1.f))
    {
        return;
    }

    const float xyx = p0[0] - p1[0], xyy = p0[1] - p1[1];
    const float zyx = p2[0] - p1[0], zyy = p2[1] - p1[1];
    const float denom = 1.f / (zyx * xyy - zyy * xyx);

    const V4 X = mk(p0[0], p1[0], p2[0], 0.f);
    const V4 Y = mk(p0[1], p1[1], p2[1], 0.f);
    const V4 ddx = mk(Y[1] * 1.f - Y[2] * 1.f, Y[2] * 1.f - Y[0] * 1.f, Y[0] * 1.f - Y[1] * 1.f, 0.f);
    const V4 ddy = mk(1.f * X[2] - 1.f * X[1], 1.f * X[0] - 1.f * X[2], 1.f * X[1] - 1.f * X[0], 0.f);
    const V4 ddz = mk(X[1] * Y[2] - X[2] * Y[1], X[2] * Y[0] - X[0] * Y[2], X[0] * Y[1] - X[1] * Y[0], 0.f);

    Bin bin;
    bin.screen[0] = p0;
    bin.screen[1] = p1;
    bin.screen[2] = p2;
    bin.bc[0] = mulf(ddx, denom);
    bin.bc[1] = mulf(ddy, denom);
    bin.bc[2] = mulf(ddz, denom);
    for (unsigned i = 0; i < ds.numVaryings; ++i)
    {
        bin.varyings[i + 0] = a.varyings[i];
        bin.varyings[i + 4] = b.varyings[i];
        bin.varyings[i + 8] = c.varyings[i];
    }
    bin.primIndex = primIndex;
    bin.drawIndex = ds.drawIndex;
    bins.push_back(bin);
}

/* SL_TriProcessor::clip_and_process_tris (SL_TriProcessor.cpp:370-519) */
static void clip_and_process(const DrawState& ds, std::vector<Bin>& bins, size_t primIndex, const TVert& a, const TVert& b, const TVert& c)
{
    const unsigned numVarys = ds.numVaryings;
    unsigned numTotalVerts = 3;
    V4 tempVerts[9], newVerts[9];
    V4 tempVarys[36], newVarys[36];
    std::memset(tempVerts, 0, sizeof(tempVerts));
    std::memset(newVerts, 0, sizeof(newVerts));
    std::memset(tempVarys, 0, sizeof(tempVarys));
    std::memset(newVarys, 0, sizeof(newVarys));
    static const float clipEdges[6][4] = {
        { 1.f,  0.f,  0.f, 1.f},
        {-1.f,  0.f,  0.f, 1.f},
        { 0.f,  1.f,  0.f, 1.f},
        { 0.f, -1.f,  0.f, 1.f},
        { 0.f,  0.f,  1.f, 1.f},
        { 0.f,  0.f, -1.f, 1.f},
    };

    newVerts[0] = a.vert;
    newVerts[1] = b.vert;
    newVerts[2] = c.vert;
    for (unsigned i = 0; i < numVarys; ++i)
    {
        newVarys[0 + i] = a.varyings[i];
        newVarys[4 + i] = b.varyings[i];
        newVarys[8 + i] = c.varyings[i];
    }

    for (int e = 0; e < 6; ++e)
    {
        const V4 edge = mk(clipEdges[e][0], clipEdges[e][1], clipEdges[e][2], clipEdges[e][3]);
        unsigned numNewVerts = 0;
        unsigned j = numTotalVerts - 1;
        V4 p0 = newVerts[numTotalVerts - 1];
        float t0 = dot(p0, edge);
        int visible0 = !sign_mask(t0);

        for (unsigned k = 0; k < numTotalVerts; ++k)
        {
            const V4 p1 = newVerts[k];
            const float t1 = dot(p1, edge);
            const int visible1 = !sign_mask(t1);

            if (visible0 ^ visible1)
            {
                const float t = t0 * (1.f / (t0 - t1));
                tempVerts[numNewVerts] = mix(p0, p1, t);
                for (unsigned i = 0; i < numVarys; ++i)
                {
                    tempVarys[numNewVerts * 4 + i] = mix(newVarys[j * 4 + i], newVarys[k * 4 + i], t);
                }
                ++numNewVerts;
            }

            if (visible1)
            {
                tempVerts[numNewVerts] = p1;
                for (unsigned i = 0; i < numVarys; ++i)
                {
                    tempVarys[numNewVerts * 4 + i] = newVarys[k * 4 + i];
                }
                ++numNewVerts;
            }

            j = k;
            p0 = p1;
            t0 = t1;
            visible0 = visible1;
        }

        if (!numNewVerts)
        {
            return;
        }

        numTotalVerts = numNewVerts;
        for (unsigned i = 0; i < numNewVerts; ++i)
        {
            newVerts[i] = tempVerts[i];
        }

        /* The reference copies numNewVerts vectors starting at each vertex's
         * varying slot (SL_TriProcessor.cpp:471-475), not numVarys; restated
         * slot by slot, bounded to the 36-slot arrays. */
        for (unsigned i = numNewVerts; i--;)
        {
            const unsigned offset = i * 4;
            for (unsigned m = 0; m < numNewVerts; ++m)
            {
                if (offset + m < 36)
                {
                    newVarys[offset + m] = tempVarys[offset + m];
                }
            }
        }
    }

    if (numTotalVerts < 3)
    {
        return;
    }

    for (unsigned i = 0; i < numTotalVerts; ++i)
    {
        perspective_divide(newVerts[i]);
        ndc_to_screen(newVerts[i], ds.viewport);
    }

    TVert q0, q1, q2;
    q0.vert = newVerts[0];
    for (unsigned i = 0; i < numVarys; ++i) q0.varyings[i] = newVarys[i];

    for (unsigned i = numTotalVerts - 2; i--;)
    {
        const unsigned j = i + 1;
        const unsigned k = i + 2;
        q1.vert = newVerts[j];
        q2.vert = newVerts[k];
        for (unsigned v = 0; v < numVarys; ++v)
        {
            q1.varyings[v] = newVarys[j * 4 + v];
            q2.varyings[v] = newVarys[k * 4 + v];
        }
        push_bin(ds, bins, primIndex, q0, q1, q2);
    }
}

/* get_next_vertex3, portable branch (SL_TriProcessor.cpp:125-234) */
static inline size_t read_index(const Ibo& ibo, size_t i)
{
    const uint8_t* p = ibo.bytes.data();
    switch (ibo.type)
    {
        case SLG_VERTEX_DATA_BYTE:  return p[i];
        case SLG_VERTEX_DATA_SHORT: { uint16_t v; std::memcpy(&v, p + 2 * i, 2); return v; }
        default:                    { uint32_t v; std::memcpy(&v, p + 4 * i, 4); return v; }
    }
}

/* SL_TriProcessor::process_verts<usingIndices> (SL_TriProcessor.cpp:527-640)
 * restricted to elements [first, last) of one mesh instance. */
static void process_verts(const DrawState& ds, const Ibo* ibo, const slg_mesh& m, size_t instanceId,
                          size_t first, size_t last, std::vector<Bin>& bins)
{
    const size_t numElements = m.elementEnd - m.elementBegin;
    const size_t primOffset = numElements * instanceId;
    const uint8_t cullMode = ds.shader->cull;
    TVert tv[3];

    for (size_t i = first; i < last; i += 3)
    {
        for (int k = 0; k < 3; ++k)
        {
            const size_t vertId = ibo ? read_index(*ibo, i + k) : (i + k);
            tv[k].vert = run_vs(ds.shader->vsProgram, ds.env, vertId, instanceId, tv[k].varyings);
        }

        if (cullMode != SLG_CULL_OFF)
        {
            const float det = face_determinant(tv[0].vert, tv[1].vert, tv[2].vert);
            const bool culled = (cullMode == SLG_CULL_FRONT_FACE) ^ (sign_mask(det) != 0);
            if (culled)
            {
                continue;
            }
        }

        for (int k = 0; k < 3; ++k)
        {
            tv[k].vert = mat_mul(ds.scissor, tv[k].vert);
        }

        const int vis = clip_status(tv[0].vert, tv[1].vert, tv[2].vert);
        if (vis == 3)
        {
            for (int k = 0; k < 3; ++k)
            {
                perspective_divide(tv[k].vert);
                ndc_to_screen(tv[k].vert, ds.viewport);
            }
            push_bin(ds, bins, primOffset + i, tv[0], tv[1], tv[2]);
        }
        else if (vis == 1)
        {
            clip_and_process(ds, bins, primOffset + i, tv[0], tv[1], tv[2]);
        }
    }
}

/*-----------------------------------------------------------------------------
 * Fragment stage
-----------------------------------------------------------------------------*/
struct Target
{
    uint8_t* bytes;
    int type;
    uint16_t w;
};

/* assign_pixel / assign_alpha_pixel, portable (SL_Framebuffer.cpp:45-80,271-368) */
/* float -> unsigned as the reference build does it on x86-64: cvttss2si,
 * 32-bit values from its 64-bit form, 64-bit values from gcc's two-range
 * sequence (so 1.0 * (float)UINT32_MAX stores 0) */
static inline uint64_t cvt_f32_i64(float x)
{
    return (x >= -9223372036854775808.f && x < 9223372036854775808.f) ? (uint64_t)(int64_t)x : 0x8000000000000000ull;
}

static inline uint64_t f2u_x86(float x, int kind)
{
    if (kind <= 1) return (uint64_t)(uint32_t)f2i(x);
    if (kind == 2) return cvt_f32_i64(x) & 0xFFFFFFFFull;
    if (!(x >= 9223372036854775808.f)) return cvt_f32_i64(x);
    return cvt_f32_i64(x - 9223372036854775808.f) ^ 0x8000000000000000ull;
}

/* RGBA u32 texels: converting an out-of-range or NaN float to unsigned is
 * undefined in C++, and for four-lane u32 vectors the reference build
 * (x86-64 SSE2) emits the vectorised form: x >= 2^31 ? cvttps2dq(x - 2^31)
 * ^ 2^31 : cvttps2dq(x), where cvttps2dq gives 0x80000000 out of int32
 * range. In-range values convert identically either way. */
static inline uint32_t f2u32_vec(float x)
{
    const bool big = x >= 2147483648.f;
    const float y = big ? x - 2147483648.f : x;
    const uint32_t i = (y >= -2147483648.f && y < 2147483648.f) ? (uint32_t)(int32_t)y : 0x80000000u;
    return big ? (i ^ 0x80000000u) : i;
}

static inline uint32_t d2u32_vec(double x)
{
    const bool big = x >= 2147483648.0;
    const double y = big ? x - 2147483648.0 : x;
    const uint32_t i = (y >= -2147483648.0 && y < 2147483648.0) ? (uint32_t)(int32_t)y : 0x80000000u;
    return big ? (i ^ 0x80000000u) : i;
}

/* component j of texel idx as float: color_cast<float, T> (SL_Color.hpp:640-670) */
static inline float component_get(const Target& t, size_t idx, int j)
{
    const int nc = t.type / 7 + 1, kind = t.type % 7;
    const size_t cb = bytes_per_color(t.type) / nc;
    const uint8_t* c = t.bytes + (idx * nc + j) * cb;
    switch (kind)
    {
        case 0: return (float)c[0] * 0.00392156862745f;
        case 1: { uint16_t v; std::memcpy(&v, c, 2); return (float)v * (1.f / 65535.f); }
        case 2: { uint32_t v; std::memcpy(&v, c, 4); return (float)v * (1.f / 4294967295.f); }
        case 3: { uint64_t v; std::memcpy(&v, c, 8); return (float)v * (1.f / 18446744073709551615.f); }
        case 4: { uint16_t v; std::memcpy(&v, c, 2); return slg_half_to_float(v); }
        case 5: { float v; std::memcpy(&v, c, 4); return v; }
        default: { double v; std::memcpy(&v, c, 8); return (float)v; }
    }
}

/* the format's maximum as float: the alpha a texel without one is read with */
static inline float kind_one(int kind)
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

/* color_cast<T, float> of one component (SL_Color.hpp:618-637) */
static inline void component_set(const Target& t, size_t idx, int j, float x)
{
    const int nc = t.type / 7 + 1, kind = t.type % 7;
    const size_t cb = bytes_per_color(t.type) / nc;
    uint8_t* c = t.bytes + (idx * nc + j) * cb;
    static const float kMax[4] = {255.f, 65535.f, 4294967295.f, 18446744073709551615.f};
    if (kind == 2 && nc == 4)
    {
        const uint32_t u = f2u32_vec(x * kMax[kind]);
        std::memcpy(c, &u, 4);
    }
    else if (kind <= 3)
    {
        const uint64_t u = f2u_x86(x * kMax[kind], kind);
        std::memcpy(c, &u, cb);   /* little-endian low bytes */
    }
    else if (kind == 4) { const uint16_t h = slg_float_to_half(x); std::memcpy(c, &h, 2); }
    else if (kind == 5) std::memcpy(c, &x, 4);
    else { const double d = (double)x; std::memcpy(c, &d, 8); }
}

/* Packed texels. Read (rgba_cast<float, T>, SL_ColorCompressed.hpp:165-184
 * and the like): each field as (float)c / (float)max, alpha 1 for the RGB
 * formats. Write (rgba_cast<T, float>, :112-132 and the like): each field
 * (uint8_t or uint16_t)(x * (float)max), i.e. cvttss2si's 32-bit result,
 * keeping the field's low bits. */
static inline uint32_t packed_bits(const Target& t, size_t idx)
{
    const PackedFormat& pf = kPacked[t.type - 28];
    uint32_t bits = 0;
    std::memcpy(&bits, t.bytes + idx * pf.bytes, pf.bytes);   /* little-endian */
    return bits;
}

static inline V4 packed_get(const Target& t, size_t idx)
{
    const PackedFormat& pf = kPacked[t.type - 28];
    const uint32_t bits = packed_bits(t, idx);
    V4 d = mk(0.f, 0.f, 0.f, 1.f);
    for (int j = 0; j < pf.nc; ++j)
    {
        const uint32_t mask = (1u << pf.bits[j]) - 1u;
        d[j] = (float)((bits >> pf.shift[j]) & mask) / (float)mask;
    }
    return d;
}

static inline void packed_set(const Target& t, size_t idx, const V4& c)
{
    const PackedFormat& pf = kPacked[t.type - 28];
    uint32_t bits = 0;
    for (int j = 0; j < pf.nc; ++j)
    {
        const uint32_t mask = (1u << pf.bits[j]) - 1u;
        bits |= ((uint32_t)f2i(c[j] * (float)mask) & mask) << pf.shift[j];
    }
    std::memcpy(t.bytes + idx * pf.bytes, &bits, pf.bytes);
}

/* assign_pixel / assign_alpha_pixel (softlight/src/SL_Framebuffer.cpp:45-80,
 * 266-366): the blend reads the texel padded with the format's min (green,
 * blue) and max (alpha), a three-component texel as (r, r, r, max); the
 * blended value is clamped to [0, 1]; components beyond the format's are
 * dropped. Packed formats read and write whole texels (SL_Framebuffer.cpp:
 * 85-145, 371-587, with the same blend and clamp). */
static inline void write_color(const Target& t, unsigned x, unsigned y, const V4& rgba, uint8_t blend)
{
    const size_t idx = (size_t)x + (size_t)t.w * y;
    const bool packed = t.type >= 28;
    const int nc = packed ? 0 : t.type / 7 + 1, kind = packed ? 0 : t.type % 7;
    V4 src = rgba;

    if (blend != SLG_BLEND_OFF)
    {
        V4 d;
        if (packed) d = packed_get(t, idx);
        else
        {
            const float r = component_get(t, idx, 0);
            if (nc == 1) d = mk(r, 0.f, 0.f, kind_one(kind));
            else if (nc == 2) d = mk(r, component_get(t, idx, 1), 0.f, kind_one(kind));
            else if (nc == 3) d = mk(r, r, r, kind_one(kind));
            else d = mk(r, component_get(t, idx, 1), component_get(t, idx, 2), component_get(t, idx, 3));
        }

        const float sa = rgba[3];
        const float modulation = 1.f - sa;
        if (blend == SLG_BLEND_ALPHA)
        {
            const float dstMod = modulation * d[3];
            const float dstAlpha = dstMod + sa;
            const float rc = 1.f / dstAlpha;
            d = mk((rgba[0] * sa + d[0] * dstMod) * rc, (rgba[1] * sa + d[1] * dstMod) * rc,
                   (rgba[2] * sa + d[2] * dstMod) * rc, dstAlpha);
        }
        else if (blend == SLG_BLEND_PREMULTIPLED_ALPHA)
        {
            d = mk(d[0] * modulation + rgba[0], d[1] * modulation + rgba[1], d[2] * modulation + rgba[2], d[3] * modulation + rgba[3]);
        }
        else if (blend == SLG_BLEND_ADDITIVE)
        {
            d = mk(rgba[0] * sa + d[0], rgba[1] * sa + d[1], rgba[2] * sa + d[2], rgba[3] * sa + d[3]);
        }
        else
        {
            d = mk(rgba[0] * sa + d[0] * modulation, rgba[1] * sa + d[1] * modulation,
                   rgba[2] * sa + d[2] * modulation, rgba[3] * sa + d[3] * modulation);
        }
        for (int k = 0; k < 4; ++k)
        {
            d[k] = lm_min(lm_max(d[k], 0.f), 1.f);
        }
        src = d;
    }

    if (packed) packed_set(t, idx, src);
    else for (int j = 0; j < nc; ++j) component_set(t, idx, j, src[j]);
}

static inline bool depth_cmp(uint8_t func, float z, float d)
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

struct RasterState
{
    const slo_context* ctx;
    uint8_t* depth;     /* R_HALF, R_FLOAT or R_DOUBLE texels */
    int depthType;
    uint16_t width;
    uint16_t height;
    Target colors[4];
    unsigned numOutputs;
    std::vector<const Shader*> shaders; /* per draw index */
    std::vector<Env> envs;               /* per draw index */
};

/* The depth texel as the rasterizers compare it, (float)depth_type, and the
 * write (depth_type)z (_sl_get_depth_texel, SL_TriRasterizer.cpp:95-101;
 * SL_FragmentProcessor.cpp:398-401, 524-527). */
static inline float dget(const RasterState& rs, size_t i)
{
    if (rs.depthType == SLG_COLOR_R_HALF) { uint16_t h; std::memcpy(&h, rs.depth + 2 * i, 2); return slg_half_to_float(h); }
    if (rs.depthType == SLG_COLOR_R_DOUBLE) { double d; std::memcpy(&d, rs.depth + 8 * i, 8); return (float)d; }
    float f;
    std::memcpy(&f, rs.depth + 4 * i, 4);
    return f;
}

static inline void dset(const RasterState& rs, size_t i, float z)
{
    if (rs.depthType == SLG_COLOR_R_HALF) { const uint16_t h = slg_float_to_half(z); std::memcpy(rs.depth + 2 * i, &h, 2); }
    else if (rs.depthType == SLG_COLOR_R_DOUBLE) { const double d = (double)z; std::memcpy(rs.depth + 8 * i, &d, 8); }
    else std::memcpy(rs.depth + 4 * i, &z, 4);
}

/* SL_FragmentProcessor::flush_tri_fragments for one fragment, portable
 * (SL_FragmentProcessor.cpp:417-531, interpolate_tri_varyings :308-330) */
static inline void shade_fragment(const RasterState& rs, const Bin& bin, int x, int y, float z, const V4& bcIn, uint64_t& frags)
{
    const Shader& sh = *rs.shaders[bin.drawIndex];
    const V4 homogenous = mk(bin.screen[0][3], bin.screen[1][3], bin.screen[2][3], 0.f);
    const V4 bc = mul(bcIn, homogenous);
    const float persp = 1.f / (((bc[0] + bc[1]) + bc[2]) + bc[3]);
    const V4 bcp = mulf(bc, persp);

    V4 varyings[4];
    for (unsigned i = 0; i < 4; ++i) varyings[i] = mk(0.f, 0.f, 0.f, 0.f);
    for (unsigned i = 0; i < sh.numVaryings; ++i)
    {
        const V4 v0 = mulf(bin.varyings[i + 0], bcp[0]);
        const V4 v1 = mulf(bin.varyings[i + 4], bcp[1]);
        const V4 v2 = mulf(bin.varyings[i + 8], bcp[2]);
        varyings[i] = add(add(v0, v1), v2);
    }

    V4 outputs[4];
    slg_frag_coord coord = frag_coord((uint32_t)x, (uint32_t)y, z);
    const bool haveOutputs = run_fs(sh.fsProgram, rs.envs[bin.drawIndex], coord, varyings, outputs);
    if (haveOutputs)
    {
        for (unsigned t = 0; t < sh.numOutputs && t < rs.numOutputs; ++t)
        {
            write_color(rs.colors[t], (unsigned)x, (unsigned)y, outputs[t], sh.blend);
        }
    }
    if (sh.depthMask == SLG_DEPTH_MASK_ON)
    {
        dset(rs, (size_t)x + (size_t)rs.width * y, coord.depth);
    }
    ++frags;
}

/* SL_TriRasterizer::render_triangle_simd, portable branch
 * (SL_TriRasterizer.cpp:807-923) with SL_ScanlineBounds init/step portable
 * branches (SL_ScanlineBounds.hpp:137-186,301-321). Only rows with
 * y % rowStride == rowPhase are drawn (the reference's scan-line
 * interleave across threads, SL_ScanlineBounds.hpp:32-50). */
/* The depth texel as the reference reads it, (float)depth_type
 * (_sl_get_depth_texel, SL_TriRasterizer.cpp:95-101), for a depth type
 * known at compile time. */
template <int DepthType>
static inline float depth_texel(const uint8_t* depth, size_t i)
{
    if (DepthType == SLG_COLOR_R_HALF) { uint16_t h; std::memcpy(&h, depth + 2 * i, 2); return slg_half_to_float(h); }
    if (DepthType == SLG_COLOR_R_DOUBLE) { double d; std::memcpy(&d, depth + 8 * i, 8); return (float)d; }
    float f;
    std::memcpy(&f, depth + 4 * i, 4);
    return f;
}

/* One bin with the depth type and depth test fixed at compile time, as the
 * reference instantiates render_triangle_simd per depth functor and type
 * (SL_TriRasterizer.cpp:965-1068). Four pixels are tested at once into a
 * mask and the passing ones queued (SL_SHADER_MAX_QUEUED_FRAGS, 600) and
 * shaded when the queue fills or the bin ends; a bin's pixels are
 * distinct, so the queue gives the same result as shading at once. */
template <int DepthType, int Func>
static void raster_bin_t(const RasterState& rs, const Bin& bin, int rowStride, int rowPhase, uint64_t& frags)
{
    const V4* pts = bin.screen;
    const int32_t bboxMinY = f2i(lm_min(lm_min(pts[0][1], pts[1][1]), pts[2][1]));
    const int32_t bboxMaxY = f2i(lm_max(lm_max(pts[0][1], pts[1][1]), pts[2][1]));

    int32_t y = bboxMinY;
    if (rowStride > 1)
    {
        /* sl_scanline_offset (SL_ScanlineBounds.hpp:32-50) */
        const int32_t n1 = rowStride - 1;
        y += n1 - ((bboxMinY + (n1 - rowPhase)) % rowStride);
    }
    if (y >= bboxMaxY)
    {
        return;
    }

    const V4 depth = mk(pts[0][2], pts[1][2], pts[2][2], 0.f);

    /* SL_ScanlineBounds::init */
    V4 p0 = pts[0], p1 = pts[1], p2 = pts[2];
    if (p0[1] < p1[1]) std::swap(p0, p1);
    if (p0[1] < p2[1]) std::swap(p0, p2);
    if (p1[1] < p2[1]) std::swap(p1, p2);
    const V4 p2p0 = sub(p2, p0);
    const V4 p2p1 = sub(p2, p1);
    const V4 p1p0 = sub(p1, p0);
    const float v0y = p0[1], v1y = p1[1], v0x = p0[0], v1x = p1[0];
    const float p20y = 1.f / p2p0[1];
    const float p20x = p2p0[0];
    const float p21xy = p2p1[0] * (1.f / p2p1[1]);
    const float p10xy = p1p0[0] * (1.f / p1p0[1]);

    const V4* bcs = bin.bc;
    const V4 bcX = mulf(bcs[0], 4.f);
    struct Frag { int32_t x, y; float z; V4 bc; };
    constexpr unsigned kQueue = 600;   /* SL_SHADER_MAX_QUEUED_FRAGS (SL_Config.hpp:46) */
    Frag queue[kQueue];
    unsigned numQueued = 0;

    do
    {
        const float yf = (float)y;

        /* SL_ScanlineBounds::step */
        const float d0 = yf - v0y;
        const float d1 = yf - v1y;
        const float alpha = d0 * p20y;
        const int32_t lo = f2i(p20x * alpha + v0x);
        const int32_t secondHalf = -(d1 < 0.f);
        const int32_t sa = f2i(p21xy * d1 + v1x);
        const int32_t sb = f2i(p10xy * d0 + v0x);
        const int32_t hi = (secondHalf & sa) | (~secondHalf & sb);
        const int32_t xMin = (lo >= hi) ? hi : lo;
        const int32_t xMax = (lo >= hi) ? lo : hi;

        if ((uint32_t)xMin < (uint32_t)xMax)
        {
            const V4 bcY = mk(bcs[1][0] * yf + bcs[2][0], bcs[1][1] * yf + bcs[2][1],
                              bcs[1][2] * yf + bcs[2][2], bcs[1][3] * yf + bcs[2][3]);
            V4 bc[4];
            int32_t x4[4];
            for (int k = 0; k < 4; ++k)
            {
                x4[k] = xMin + k;
                const float xf = (float)x4[k];
                bc[k] = mk(bcs[0][0] * xf + bcY[0], bcs[0][1] * xf + bcY[1],
                           bcs[0][2] * xf + bcY[2], bcs[0][3] * xf + bcY[3]);
            }

            const size_t rowBase = (size_t)rs.width * (size_t)y;
            do
            {
                bool pass[4];
                float z[4];
                for (int k = 0; k < 4; ++k)
                {
                    z[k] = dot(depth, bc[k]);
                    const bool in = x4[k] < xMax;
                    const float d = in ? depth_texel<DepthType>(rs.depth, rowBase + (size_t)x4[k]) : 0.f;
                    pass[k] = in & depth_cmp(Func, z[k], d);
                }
                if (pass[0] | pass[1] | pass[2] | pass[3])
                {
                    for (int k = 0; k < 4; ++k)
                    {
                        if (pass[k])
                        {
                            queue[numQueued++] = {x4[k], y, z[k], bc[k]};
                        }
                    }
                    if (numQueued > kQueue - 4)
                    {
                        for (unsigned q = 0; q < numQueued; ++q) shade_fragment(rs, bin, queue[q].x, queue[q].y, queue[q].z, queue[q].bc, frags);
                        numQueued = 0;
                    }
                }
                for (int k = 0; k < 4; ++k)
                {
                    bc[k] = add(bc[k], bcX);
                    x4[k] += 4;
                }
            }
            while (x4[0] < xMax);
        }

        y += rowStride;
    }
    while (y < bboxMaxY);
    for (unsigned q = 0; q < numQueued; ++q) shade_fragment(rs, bin, queue[q].x, queue[q].y, queue[q].z, queue[q].bc, frags);
}

static void raster_bin(const RasterState& rs, const Bin& bin, int rowStride, int rowPhase, uint64_t& frags)
{
    const uint8_t func = rs.shaders[bin.drawIndex]->depthTest;
#define SLO_RASTER_FUNCS(DT)                                                                                     \
    switch (func)                                                                                                \
    {                                                                                                            \
        case SLG_DEPTH_TEST_LESS_THAN:     return raster_bin_t<DT, SLG_DEPTH_TEST_LESS_THAN>(rs, bin, rowStride, rowPhase, frags);     \
        case SLG_DEPTH_TEST_LESS_EQUAL:    return raster_bin_t<DT, SLG_DEPTH_TEST_LESS_EQUAL>(rs, bin, rowStride, rowPhase, frags);    \
        case SLG_DEPTH_TEST_GREATER_THAN:  return raster_bin_t<DT, SLG_DEPTH_TEST_GREATER_THAN>(rs, bin, rowStride, rowPhase, frags);  \
        case SLG_DEPTH_TEST_GREATER_EQUAL: return raster_bin_t<DT, SLG_DEPTH_TEST_GREATER_EQUAL>(rs, bin, rowStride, rowPhase, frags); \
        case SLG_DEPTH_TEST_EQUAL:         return raster_bin_t<DT, SLG_DEPTH_TEST_EQUAL>(rs, bin, rowStride, rowPhase, frags);         \
        case SLG_DEPTH_TEST_NOT_EQUAL:     return raster_bin_t<DT, SLG_DEPTH_TEST_NOT_EQUAL>(rs, bin, rowStride, rowPhase, frags);     \
        default:                           return raster_bin_t<DT, SLG_DEPTH_TEST_OFF>(rs, bin, rowStride, rowPhase, frags);           \
    }
    if (rs.depthType == SLG_COLOR_R_HALF) { SLO_RASTER_FUNCS(SLG_COLOR_R_HALF) }
    if (rs.depthType == SLG_COLOR_R_DOUBLE) { SLO_RASTER_FUNCS(SLG_COLOR_R_DOUBLE) }
    SLO_RASTER_FUNCS(SLG_COLOR_R_FLOAT)
#undef SLO_RASTER_FUNCS
}

/* radix-sort of a flush group by primIndex when blending
 * (SL_VertexProcessor.cpp:110-119; stable) */
/*-----------------------------------------------------------------------------
 * Lines: SL_LineProcessor (softlight/src/SL_LineProcessor.cpp:25-279) and
 * SL_LineRasterizer::render_line (softlight/src/SL_LineRasterizer.cpp:26-90),
 * one thread, the bins in element order.
-----------------------------------------------------------------------------*/
struct LineVert
{
    V4 vert;
    V4 varyings[4];
};

/* sl_draw_line_bresenham (softlight/include/softlight/SL_Geometry.hpp:313-366),
 * sl_lowp_t = int16_t */
template <typename Fn>
static void line_bresenham(int16_t x1, int16_t y1, int16_t x2, int16_t y2, Fn&& fn)
{
    const bool steep = std::abs(x1 - x2) < std::abs(y1 - y2);
    if (steep)
    {
        std::swap(x1, y1);
        std::swap(x2, y2);
    }
    if (x1 > x2)
    {
        std::swap(x1, x2);
        std::swap(y1, y2);
    }
    const int16_t dx = (int16_t)(x2 - x1);
    const int16_t dy = (int16_t)(y2 - y1);
    const int16_t dErr = (int16_t)((dy < 0 ? -dy : dy) * 2);
    const int16_t yErr = (y2 > y1) ? 1 : -1;
    int16_t err = 0;
    int16_t y = y1;
    for (int16_t x = x1; x <= x2; ++x)
    {
        if (steep) fn((uint16_t)y, (uint16_t)x);
        else fn((uint16_t)x, (uint16_t)y);
        err = (int16_t)(err + dErr);
        if (err > dx)
        {
            y = (int16_t)(y + yErr);
            err = (int16_t)(err - 2 * dx);
        }
    }
}

/* SL_LineRasterizer::render_line + SL_FragmentProcessor::flush_line_fragments
 * (SL_FragmentProcessor.cpp:346-402): fragments are depth-tested when they
 * are queued and written when the queue of SL_SHADER_MAX_QUEUED_FRAGS (600)
 * is flushed or the line ends. */
static void render_line(const RasterState& rs, const DrawState& ds, const LineVert& a, const LineVert& b, uint64_t& frags)
{
    const Shader& sh = *ds.shader;
    const float z0 = a.vert[2], z1 = b.vert[2];
    const float sc0x = a.vert[0], sc0y = a.vert[1], sc1x = b.vert[0], sc1y = b.vert[1];
    const float ex = sc1x - sc0x, ey = sc1y - sc0y;
    const float dist = 1.f / std::sqrt(ex * ex + ey * ey);
    const size_t W = rs.width, H = rs.height;

    struct Frag { float interp, z; uint16_t x, y; };
    std::vector<Frag> queue;
    queue.reserve(600);
    const auto flush = [&]() {
        for (const Frag& q : queue)
        {
            V4 vary[4];
            for (unsigned i = 0; i < 4; ++i) vary[i] = mk(0.f, 0.f, 0.f, 0.f);
            for (unsigned i = 0; i < ds.numVaryings; ++i) vary[i] = mix(a.varyings[i], b.varyings[i], q.interp);
            V4 outputs[4];
            const size_t lin = (size_t)q.x + W * q.y;
            slg_frag_coord coord = frag_coord(q.x, q.y, q.z);
            if (run_fs(sh.fsProgram, ds.env, coord, vary, outputs))
            {
                for (unsigned t = 0; t < sh.numOutputs && t < rs.numOutputs; ++t)
                {
                    write_color(rs.colors[t], (unsigned)(lin % W), (unsigned)(lin / W), outputs[t], sh.blend);
                }
            }
            if (sh.depthMask == SLG_DEPTH_MASK_ON) dset(rs, lin, coord.depth);
            ++frags;
        }
        queue.clear();
    };
    const auto to_u16 = [](float v) { return (uint16_t)((uint32_t)f2i(v) & 0xFFFFu); };
    line_bresenham((int16_t)to_u16(sc0x), (int16_t)to_u16(sc0y), (int16_t)to_u16(sc1x), (int16_t)to_u16(sc1y),
                   [&](uint16_t x, uint16_t y) {
                       const float px = (float)x - sc0x, py = (float)y - sc0y;
                       const float currLen = std::sqrt(((px * px + py * py) + 0.f * 0.f) + 0.f * 0.f);
                       const float interp = currLen * dist;
                       const float z = (z1 - z0) * interp + z0;
                       const size_t lin = (size_t)x + W * y;
                       if (lin >= W * H) return; /* past the buffer: out of bounds in the reference */
                       if (!depth_cmp(sh.depthTest, z, dget(rs, lin))) return;
                       queue.push_back({interp, z, x, y});
                       if (queue.size() == 600) flush();
                   });
    flush();
}

/* _clip_segment of SL_LineProcessor::clip_and_process_lines (SL_LineProcessor.cpp:94-126) */
static bool clip_segment(float num, float denom, float& tE, float& tL)
{
    if (std::fabs(denom) < 1.0e-6f) return num < 0.f;
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

/* SL_LineProcessor::clip_and_process_lines (SL_LineProcessor.cpp:63-166) */
static void clip_and_render_line(const RasterState& rs, const DrawState& ds, const LineVert& a, const LineVert& b, uint64_t& frags)
{
    const float dx = b.vert[0] - a.vert[0], dy = b.vert[1] - a.vert[1];
    const float xMin = ds.viewport[0], yMin = ds.viewport[1], xMax = ds.viewport[2], yMax = ds.viewport[3];
    if (std::fabs(dx) < 1.0e-6f && std::fabs(dy) < 1.0e-6f)
    {
        if (a.vert[0] >= xMin && a.vert[0] <= xMax && a.vert[1] >= yMin && a.vert[1] <= yMax)
        {
            render_line(rs, ds, a, b, frags);
            return;
        }
    }
    LineVert p0 = a, p1 = b;
    const float lx = p0.vert[0] - p1.vert[0], ly = p0.vert[1] - p1.vert[1];
    const float dist = 1.f / std::sqrt(lx * lx + ly * ly);
    float tE = 0.f, tL = 1.f;
    const float x1 = p0.vert[0], y1 = p0.vert[1];
    if (!(clip_segment(xMin - x1, dx, tE, tL) && clip_segment(x1 - xMax, -dx, tE, tL) &&
          clip_segment(yMin - y1, dy, tE, tL) && clip_segment(y1 - yMax, -dy, tE, tL)))
    {
        return;
    }
    if (tL < 1.f)
    {
        p1.vert[0] = x1 + tL * dx;
        p1.vert[1] = y1 + tL * dy;
    }
    if (tE > 0.f)
    {
        p0.vert[0] = x1 + tE * dx;
        p0.vert[1] = y1 + tE * dy;
    }
    const V4 d0 = sub(p0.vert, a.vert), d1 = sub(p1.vert, b.vert);
    const float interp0 = std::sqrt(dot(d0, d0)) * dist;
    const float interp1 = std::sqrt(dot(d1, d1)) * dist;
    p0.vert[2] = (b.vert[2] - a.vert[2]) * interp0 + a.vert[2];
    p0.vert[3] = (b.vert[3] - a.vert[3]) * interp0 + a.vert[3];
    p1.vert[2] = (a.vert[2] - b.vert[2]) * interp1 + b.vert[2];
    p1.vert[3] = (a.vert[3] - b.vert[3]) * interp1 + b.vert[3];
    for (unsigned i = 0; i < ds.numVaryings; ++i)
    {
        p0.varyings[i] = mix(a.varyings[i], b.varyings[i], interp0);
        p1.varyings[i] = mix(b.varyings[i], a.varyings[i], interp1);
    }
    render_line(rs, ds, p0, p1, frags);
}

/* SL_LineProcessor::process_verts (SL_LineProcessor.cpp:172-279), one thread */
static void process_lines(const RasterState& rs, const DrawState& ds, const Ibo* ibo, const slg_mesh& m, size_t instanceId, uint64_t& frags)
{
    const Shader& sh = *ds.shader;
    for (size_t i = m.elementBegin; i < m.elementEnd; i += 2)
    {
        LineVert v0, v1;
        for (unsigned k = 0; k < 4; ++k) v0.varyings[k] = v1.varyings[k] = mk(0.f, 0.f, 0.f, 0.f);
        v0.vert = mat_mul(ds.scissor, run_vs(sh.vsProgram, ds.env, ibo ? read_index(*ibo, i) : i, instanceId, v0.varyings));
        v1.vert = mat_mul(ds.scissor, run_vs(sh.vsProgram, ds.env, ibo ? read_index(*ibo, i + 1) : i + 1, instanceId, v1.varyings));
        if (v0.vert[3] < 0.f || v1.vert[3] < 0.f) continue;
        /* sl_ndc_clip_status of two vertices (SL_PostVertexTransform.hpp:560-585) */
        const V4& c0 = v0.vert;
        const V4& c1 = v1.vert;
        const float w0 = c0[3], w1 = c1[3];
        const bool inside = (c0[0] <= w0 && c0[1] <= w0 && c0[2] <= w0 && c0[3] <= w0) &&
                            (c1[0] <= w1 && c1[1] <= w1 && c1[2] <= w1 && c1[3] <= w1) &&
                            (c0[0] >= -w0 && c0[1] >= -w0 && c0[2] >= -w0 && c0[3] >= -w0) &&
                            (c1[0] >= -w1 && c1[1] >= -w1 && c1[2] >= -w1 && c1[3] >= -w1);
        const int status = (inside ? 3 : 0) | ((w0 > 0.f || w1 > 0.f) ? 1 : 0);
        if (status == 0) continue;
        perspective_divide(v0.vert);
        perspective_divide(v1.vert);
        ndc_to_screen(v0.vert, ds.viewport);
        ndc_to_screen(v1.vert, ds.viewport);
        if (status == 3) render_line(rs, ds, v0, v1, frags);
        else clip_and_render_line(rs, ds, v0, v1, frags);
    }
}

/* SL_TriRasterizer::render_wireframe (softlight/src/SL_TriRasterizer.cpp:116-204):
 * per scan-line the left edge run of d0 pixels, then a jump to the right edge
 * run; d0 / d1 are how far the span's ends moved since the row above (at
 * least 1). Barycentrics are evaluated directly per pixel; each fragment is
 * depth-tested when it is queued and written when the thread's queue of
 * SL_SHADER_MAX_QUEUED_FRAGS (600) is flushed or the bin ends. */
static void raster_wire_bin(const RasterState& rs, const Bin& bin, int rowStride, int rowPhase, uint64_t& frags)
{
    const Shader& sh = *rs.shaders[bin.drawIndex];
    const V4* pts = bin.screen;
    const int32_t bboxMinY = f2i(lm_min(lm_min(pts[0][1], pts[1][1]), pts[2][1]));
    const int32_t bboxMaxY = f2i(lm_max(lm_max(pts[0][1], pts[1][1]), pts[2][1]));
    int32_t y0 = bboxMinY;
    if (rowStride > 1)
    {
        const int32_t n1 = rowStride - 1;
        y0 += n1 - ((bboxMinY + (n1 - rowPhase)) % rowStride);
    }

    /* SL_ScanlineBounds::init / step (SL_ScanlineBounds.hpp:137-186,301-321) */
    V4 p0 = pts[0], p1 = pts[1], p2 = pts[2];
    if (p0[1] < p1[1]) std::swap(p0, p1);
    if (p0[1] < p2[1]) std::swap(p0, p2);
    if (p1[1] < p2[1]) std::swap(p1, p2);
    const V4 p2p0 = sub(p2, p0), p2p1 = sub(p2, p1), p1p0 = sub(p1, p0);
    const float v0y = p0[1], v1y = p1[1], v0x = p0[0], v1x = p1[0];
    const float p20y = 1.f / p2p0[1];
    const float p20x = p2p0[0];
    const float p21xy = p2p1[0] * (1.f / p2p1[1]);
    const float p10xy = p1p0[0] * (1.f / p1p0[1]);
    const auto step = [&](float yf, int32_t& xMin, int32_t& xMax) {
        const float d0 = yf - v0y, d1 = yf - v1y;
        const float alpha = d0 * p20y;
        const int32_t lo = f2i(p20x * alpha + v0x);
        const int32_t sa = f2i(p21xy * d1 + v1x);
        const int32_t sb = f2i(p10xy * d0 + v0x);
        const int32_t hi = (d1 < 0.f) ? sa : sb;
        xMin = (lo >= hi) ? hi : lo;
        xMax = (lo >= hi) ? lo : hi;
    };
    /* int32 differences and abs as the reference computes them (wrapping) */
    const auto absdiff = [](int32_t a, int32_t b) {
        const uint32_t d = (uint32_t)a - (uint32_t)b;
        return (int32_t)(((int32_t)d < 0) ? (0u - d) : d);
    };

    const V4* bcs = bin.bc;
    const V4 depth = mk(pts[0][2], pts[1][2], pts[2][2], 0.f);
    struct Frag { int32_t x, y; float z; V4 bc; };
    std::vector<Frag> queue;
    queue.reserve(600);
    const auto flush = [&]() {
        for (const Frag& q : queue) shade_fragment(rs, bin, q.x, q.y, q.z, q.bc, frags);
        queue.clear();
    };
    for (int32_t y = y0; y < bboxMaxY; y += rowStride)
    {
        const float yf = (float)y;
        const V4 bcY = mk(bcs[1][0] * yf + bcs[2][0], bcs[1][1] * yf + bcs[2][1], bcs[1][2] * yf + bcs[2][2], bcs[1][3] * 0.f + bcs[2][3]);
        int32_t xMin0, xMax0, xMin1, xMax1;
        step(yf, xMin0, xMax0);
        step(yf - 1.f, xMin1, xMax1);
        const int32_t d0 = std::max(absdiff(xMin0, xMin1), 1);
        const int32_t d1 = std::max(absdiff(xMax0, xMax1), 1);
        for (int32_t ix = 0, x = xMin0; (uint32_t)x < (uint32_t)xMax0; ++ix, ++x)
        {
            if (ix == d0)
            {
                x = std::max(xMin0, (int32_t)((uint32_t)xMax0 - (uint32_t)d1 - 1u));
                continue;
            }
            const float xf = (float)x;
            const V4 bc = mk(bcs[0][0] * xf + bcY[0], bcs[0][1] * xf + bcY[1], bcs[0][2] * xf + bcY[2], bcs[0][3] * 0.f + bcY[3]);
            const float z = dot(depth, bc);
            const float d = dget(rs, (size_t)x + (size_t)rs.width * y);
            if (!depth_cmp(sh.depthTest, z, d)) continue;
            queue.push_back({x, y, z, bc});
            if (queue.size() == 600) flush();
        }
    }
    flush();
}

struct DrawItem
{
    slg_mesh mesh;
    size_t numInstances;
    size_t shaderId;
    bool multiple; /* part of a draw_multiple group sharing one bin stream */
};

} // namespace

/*-----------------------------------------------------------------------------
 * C API
-----------------------------------------------------------------------------*/
extern "C" {

int slo_context_create(slo_context** outCtx)
{
    if (!outCtx) return SLG_ERR_INVALID_ARG;
    *outCtx = new (std::nothrow) slo_context();
    return *outCtx ? SLG_OK : SLG_ERR_NO_MEMORY;
}

void slo_context_destroy(slo_context* ctx) { delete ctx; }
const char* slo_last_error(const slo_context* ctx) { return ctx ? ctx->err.c_str() : "null context"; }
unsigned slo_num_threads(slo_context* ctx, unsigned n)
{
    if (n > 0) ctx->numThreads = n;
    return ctx->numThreads;
}

size_t slo_create_vbo(slo_context* ctx) { ctx->vbos.emplace_back(); return ctx->vbos.size() - 1; }

int slo_vbo_init(slo_context* ctx, size_t id, size_t numBytes, const void* data)
{
    if (id >= ctx->vbos.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid vbo id");
    ctx->vbos[id].bytes.assign(numBytes + 64, 0);
    if (data) std::memcpy(ctx->vbos[id].bytes.data(), data, numBytes);
    return SLG_OK;
}

int slo_vbo_assign(slo_context* ctx, size_t id, const void* data, size_t offset, size_t numBytes)
{
    if (id >= ctx->vbos.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid vbo id");
    if (offset + numBytes + 64 > ctx->vbos[id].bytes.size()) return ctx->fail(SLG_ERR_INVALID_ARG, "vbo range");
    std::memcpy(ctx->vbos[id].bytes.data() + offset, data, numBytes);
    return SLG_OK;
}

size_t slo_create_ibo(slo_context* ctx) { ctx->ibos.emplace_back(); return ctx->ibos.size() - 1; }

int slo_ibo_init(slo_context* ctx, size_t id, size_t numElements, int indexType, const void* data)
{
    if (id >= ctx->ibos.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid ibo id");
    const size_t ib = index_bytes(indexType);
    if (!ib) return ctx->fail(SLG_ERR_INVALID_ARG, "invalid index type");
    Ibo& ibo = ctx->ibos[id];
    ibo.type = indexType;
    ibo.count = numElements;
    ibo.bytes.assign(numElements * ib + 16, 0); /* padded like SL_IndexBuffer */
    if (data) std::memcpy(ibo.bytes.data(), data, numElements * ib);
    return SLG_OK;
}

size_t slo_create_vao(slo_context* ctx) { ctx->vaos.emplace_back(); return ctx->vaos.size() - 1; }

int slo_vao_set_vertex_buffer(slo_context* ctx, size_t vao, size_t vbo)
{
    if (vao >= ctx->vaos.size() || vbo >= ctx->vbos.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid id");
    ctx->vaos[vao].vbo = vbo;
    return SLG_OK;
}

int slo_vao_set_index_buffer(slo_context* ctx, size_t vao, size_t ibo)
{
    if (vao >= ctx->vaos.size() || ibo >= ctx->ibos.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid id");
    ctx->vaos[vao].ibo = ibo;
    return SLG_OK;
}

int slo_vao_set_binding(slo_context* ctx, size_t vao, unsigned bindId, ptrdiff_t offset, ptrdiff_t stride,
                        unsigned numComponents, int dataType)
{
    if (vao >= ctx->vaos.size() || bindId >= 8) return ctx->fail(SLG_ERR_INVALID_ID, "invalid id");
    Binding& b = ctx->vaos[vao].bindings[bindId];
    b.offset = offset;
    b.stride = stride;
    b.comps = numComponents;
    b.type = dataType;
    return SLG_OK;
}

size_t slo_create_texture(slo_context* ctx) { ctx->textures.push_back(new Texture()); return ctx->textures.size() - 1; }

int slo_texture_init(slo_context* ctx, size_t id, int colorType, uint16_t w, uint16_t h, uint16_t d)
{
    if (id >= ctx->textures.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid texture id");
    const size_t bpt = bytes_per_color(colorType);
    if (!bpt || !w || !h || !d) return ctx->fail(SLG_ERR_INVALID_ARG, "invalid texture format or size");
    Texture& t = *ctx->textures[id];
    t.type = colorType;
    t.w = w; t.h = h; t.d = d;
    t.bpt = (unsigned)bpt;
    /* _sl_allocate_texture (SL_Texture.cpp:28-56): padded, zero-filled */
    const size_t pw = w + (4 - (w % 4));
    const size_t ph = h + (4 - (h % 4));
    const size_t pd = d + (4 - (d % 4));
    const size_t numBytes = pw * ph * pd * bpt;
    const size_t rem = 4 * bpt;
    t.bytes.assign(numBytes + (rem - (numBytes % rem)), 0);
    return SLG_OK;
}

int slo_texture_set_texels(slo_context* ctx, size_t id, const void* data, size_t numBytes)
{
    if (id >= ctx->textures.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid texture id");
    Texture& t = *ctx->textures[id];
    if (numBytes != (size_t)t.w * t.h * t.d * t.bpt) return ctx->fail(SLG_ERR_INVALID_ARG, "texel byte count");
    std::memcpy(t.bytes.data(), data, numBytes);
    return SLG_OK;
}

int slo_texture_read(slo_context* ctx, size_t id, void* dst, size_t numBytes)
{
    if (id >= ctx->textures.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid texture id");
    Texture& t = *ctx->textures[id];
    if (numBytes != (size_t)t.w * t.h * t.d * t.bpt) return ctx->fail(SLG_ERR_INVALID_ARG, "texel byte count");
    std::memcpy(dst, t.bytes.data(), numBytes);
    return SLG_OK;
}

/* SL_BlitProcessor::blit_nearest (softlight/src/SL_BlitProcessor.cpp:621-660) over a
 * destination of dstType texels, dstW x dstH, with the blit operators of
 * :20-420 (color_cast, softlight/include/softlight/SL_Color.hpp:600-690).
 * Index arithmetic is 64-bit unsigned (uint_fast32_t on LP64). */
static int blit_into(slo_context* ctx, const Texture& src, int dstType, uint64_t dstW, uint64_t dstH, uint8_t* out,
                     uint16_t srcX0, uint16_t srcY0, uint16_t srcX1, uint16_t srcY1, uint16_t dstX0, uint16_t dstY0,
                     uint16_t dstX1, uint16_t dstY1)
{
    if (srcX1 <= srcX0 || srcY1 <= srcY0 || dstX1 <= dstX0 || dstY1 <= dstY0)
        return ctx->fail(SLG_ERR_INVALID_ARG, "empty or inverted blit rectangle");
    if (dstY1 > dstH) return ctx->fail(SLG_ERR_INVALID_ARG, "blit rectangle extends below the destination");
    const uint64_t inW = (uint64_t)srcX1 - srcX0, inH = (uint64_t)srcY1 - srcY0, outW = (uint64_t)dstX1 - dstX0;
    const uint64_t x0 = dstX0, x1 = std::min<uint64_t>(dstW, x0 + outW);
    const uint64_t y0 = dstY0, y1 = dstY1;
    const uint64_t foutW = ((inW << 16) / dstW) + 1u;
    const uint64_t foutH = ((inH << 16) / dstH) + 1u;
    if (x1 <= x0) return SLG_OK;
    if (((x1 - 1u) * foutW >> 16) >= src.w || srcY0 + (((y1 - 1u) * foutH) >> 16) + 1u > srcY1 ||
        srcY1 - (srcY0 + ((y0 * foutH) >> 16)) - 1u >= src.h)
        return ctx->fail(SLG_ERR_INVALID_ARG, "blit rectangle reads outside the source texture");
    for (uint64_t y = y0; y < y1; ++y)
    {
        const uint64_t yf = (y * foutH) >> 16;
        const uint64_t srcY = srcY1 - (srcY0 + yf) - 1u;
        for (uint64_t x = x0; x < x1; ++x)
        {
            const uint64_t srcX = (x * foutW) >> 16;
            const uint64_t si = srcX + (uint64_t)src.w * srcY;
            const uint64_t di = x + dstW * y;
            float c[4];
            if (src.type == SLG_COLOR_RGBA_8U)
            {
                const uint8_t* q = &src.bytes[si * 4];
                for (int k = 0; k < 4; ++k) c[k] = (float)q[k] * 0.00392156862745f;
                if (dstType == SLG_COLOR_RGBA_8U) { std::memcpy(out + di * 4, q, 4); continue; }
            }
            else if (src.type == SLG_COLOR_RGBA_FLOAT)
            {
                std::memcpy(c, &src.bytes[si * 16], 16);
            }
            else
            {
                /* SL_Blit_R_to_*: (min, min, r, max) of the source type */
                float r;
                std::memcpy(&r, &src.bytes[si * 4], 4);
                if (dstType == SLG_COLOR_R_FLOAT) { std::memcpy(out + di * 4, &r, 4); continue; }
                c[0] = 0.f; c[1] = 0.f; c[2] = r; c[3] = 1.f;
            }
            if (dstType == SLG_COLOR_RGBA_8U)
            {
                uint8_t q[4];
                for (int k = 0; k < 4; ++k) q[k] = f2u8(c[k] * 255.f);
                std::memcpy(out + di * 4, q, 4);
            }
            else if (dstType == SLG_COLOR_RGBA_FLOAT)
            {
                std::memcpy(out + di * 16, c, 16);
            }
            else
            {
                std::memcpy(out + di * 4, &c[0], 4);
            }
        }
    }
    return SLG_OK;
}

static bool blit_type_ok(int t) { return t == SLG_COLOR_RGBA_8U || t == SLG_COLOR_RGBA_FLOAT || t == SLG_COLOR_R_FLOAT; }

int slo_blit_rect(slo_context* ctx, size_t outId, size_t inId, uint16_t srcX0, uint16_t srcY0, uint16_t srcX1,
                  uint16_t srcY1, uint16_t dstX0, uint16_t dstY0, uint16_t dstX1, uint16_t dstY1)
{
    if (outId >= ctx->textures.size() || inId >= ctx->textures.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid texture id");
    const Texture& src = *ctx->textures[inId];
    Texture& dst = *ctx->textures[outId];
    if (src.bytes.empty() || dst.bytes.empty() || !blit_type_ok(src.type) || !blit_type_ok(dst.type))
        return ctx->fail(SLG_ERR_INVALID_ARG, "blit needs initialised R float, RGBA8 or RGBA float textures");
    if (outId == inId) return ctx->fail(SLG_ERR_INVALID_ARG, "blit source and destination are the same texture");
    return blit_into(ctx, src, dst.type, dst.w, dst.h, dst.bytes.data(), srcX0, srcY0, srcX1, srcY1, dstX0, dstY0, dstX1, dstY1);
}

int slo_blit(slo_context* ctx, size_t outId, size_t inId)
{
    if (outId >= ctx->textures.size() || inId >= ctx->textures.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid texture id");
    const Texture& src = *ctx->textures[inId];
    const Texture& dst = *ctx->textures[outId];
    return slo_blit_rect(ctx, outId, inId, 0, 0, src.w, src.h, 0, 0, dst.w, dst.h);
}

int slo_blit_read(slo_context* ctx, size_t inId, int dstType, uint16_t dstW, uint16_t dstH, void* dst, size_t numBytes)
{
    if (inId >= ctx->textures.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid texture id");
    const Texture& src = *ctx->textures[inId];
    if (src.bytes.empty() || !blit_type_ok(src.type) || !blit_type_ok(dstType))
        return ctx->fail(SLG_ERR_INVALID_ARG, "blit needs R float, RGBA8 or RGBA float formats");
    const size_t bytes = (size_t)dstW * dstH * (dstType == SLG_COLOR_RGBA_FLOAT ? 16u : 4u);
    if (!dst || numBytes != bytes || bytes == 0) return ctx->fail(SLG_ERR_INVALID_ARG, "destination byte count");
    return blit_into(ctx, src, dstType, dstW, dstH, static_cast<uint8_t*>(dst), 0, 0, src.w, src.h, 0, 0, dstW, dstH);
}

size_t slo_create_framebuffer(slo_context* ctx) { ctx->fbos.emplace_back(); return ctx->fbos.size() - 1; }

/* SL_Framebuffer::reserve_color_buffers (softlight/src/SL_Framebuffer.cpp:821-845) */
int slo_fbo_reserve_color_buffers(slo_context* ctx, size_t fbo, unsigned n)
{
    if (fbo >= ctx->fbos.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid fbo");
    Fbo& b = ctx->fbos[fbo];
    if (n == b.numColors) return SLG_OK;
    if (n < 1 || n > 4) return ctx->fail(SLG_ERR_INVALID_ARG, "a framebuffer has 1 to 4 colour attachments");
    for (size_t& c : b.colors) c = SLG_INVALID_ID;
    b.numColors = n;
    return SLG_OK;
}

int slo_fbo_attach_color_buffer(slo_context* ctx, size_t fbo, unsigned index, size_t tex)
{
    if (fbo >= ctx->fbos.size() || tex >= ctx->textures.size() || index >= ctx->fbos[fbo].numColors)
        return ctx->fail(SLG_ERR_INVALID_ARG, "invalid fbo attachment");
    ctx->fbos[fbo].colors[index] = tex;
    return SLG_OK;
}

int slo_fbo_attach_depth_buffer(slo_context* ctx, size_t fbo, size_t tex)
{
    if (fbo >= ctx->fbos.size() || tex >= ctx->textures.size()) return ctx->fail(SLG_ERR_INVALID_ARG, "invalid fbo attachment");
    const int dt = ctx->textures[tex]->type;
    if (dt != SLG_COLOR_R_HALF && dt != SLG_COLOR_R_FLOAT && dt != SLG_COLOR_R_DOUBLE)
        return ctx->fail(SLG_ERR_INVALID_ARG, "depth must be R_HALF, R_FLOAT or R_DOUBLE");
    ctx->fbos[fbo].depth = tex;
    return SLG_OK;
}

size_t slo_create_ubo(slo_context* ctx)
{
    Ubo* u = new Ubo();
    std::memset(u->bytes, 0, sizeof(u->bytes));
    ctx->ubos.push_back(u);
    return ctx->ubos.size() - 1;
}

int slo_ubo_assign(slo_context* ctx, size_t id, const void* data, size_t numBytes)
{
    if (id >= ctx->ubos.size() || numBytes > 1024) return ctx->fail(SLG_ERR_INVALID_ARG, "invalid ubo");
    std::memcpy(ctx->ubos[id]->bytes, data, numBytes);
    return SLG_OK;
}

/* SL_Context::create_shader validation (SL_Context.cpp:488-541) */
size_t slo_create_shader(slo_context* ctx, const slg_vertex_shader* vs, const slg_fragment_shader* fs, size_t ubo)
{
    if (!vs || !fs) { ctx->err = "null shader"; return SLG_INVALID_ID; }
    if (vs->numVaryings < fs->numVaryings || vs->numVaryings > 4 || fs->numVaryings > 4 || fs->numOutputs > 4)
    {
        ctx->err = "invalid varying or output count";
        return SLG_INVALID_ID;
    }
    if (ubo != SLG_INVALID_ID && ubo >= ctx->ubos.size()) { ctx->err = "invalid ubo id"; return SLG_INVALID_ID; }
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
    ctx->shaders.push_back(s);
    return ctx->shaders.size() - 1;
}

/* SL_ClearProcessor::clear_texture's reach (softlight/src/SL_ClearProcessor.cpp:22-33
 * with sl_calc_indexed_parition2<1>, softlight/include/softlight/SL_ShaderUtil.hpp:222-231):
 * thread t clears [t*range, min((t+1)*range, w*h)) with
 * range = total + (1 - total % 3) in size_t, total = w*h / threads. */
static size_t clear_reach(size_t count, unsigned threads)
{
    size_t reach = 0;
    const size_t n = threads ? threads : 1u;
    const size_t total = count / n;
    const size_t range = total + (size_t(1) - (total % 3));
    for (size_t id = 0; id < n; ++id)
    {
        const size_t begin = range * id, end = begin + range;
        const size_t stop = end < count ? end : count;
        if (stop > begin && stop > reach) reach = stop;
    }
    return reach;
}

/* double -> unsigned as x86-64 code does it (cvttsd2si, as f2u_x86) */
static inline uint64_t d2u_x86(double v, int kind)
{
    const auto i64 = [](double w) { return (w >= -9223372036854775808.0 && w < 9223372036854775808.0) ? (uint64_t)(int64_t)w : 0x8000000000000000ull; };
    if (kind <= 1) return (uint64_t)(uint32_t)((v >= -2147483648.0 && v < 2147483648.0) ? (int32_t)v : INT32_MIN);
    if (kind == 2) return i64(v) & 0xFFFFFFFFull;
    if (!(v >= 9223372036854775808.0)) return i64(v);
    return i64(v - 9223372036854775808.0) ^ 0x8000000000000000ull;
}

/* SL_Context::clear_color_buffer / clear_depth_buffer: per component
 * color_cast<T, double> (sl_match_color_for_type, SL_Color.cpp:137-192;
 * SL_Context.cpp:897-913 for depth), over the texels the clear reaches */
static void clear_color(Texture& t, const double rgba[4], unsigned threads)
{
    const size_t n = clear_reach((size_t)t.w * t.h, threads);
    const size_t bpt = bytes_per_color(t.type);
    const bool packed = t.type >= 28;
    const int nc = packed ? 0 : t.type / 7 + 1, kind = packed ? 0 : t.type % 7;
    const size_t cb = packed ? 0 : bpt / nc;
    static const double kMax[4] = {255.0, 65535.0, 4294967295.0, 18446744073709551615.0};
    uint8_t texel[32] = {0};
    if (packed)
    {
        /* rgba_cast<T, double> (SL_Color.cpp:180-184): (uint8_t or
         * uint16_t)(c * (double)max) per field, low bits kept */
        const PackedFormat& pf = kPacked[t.type - 28];
        uint32_t bits = 0;
        for (int j = 0; j < pf.nc; ++j)
        {
            const uint32_t mask = (1u << pf.bits[j]) - 1u;
            bits |= ((uint32_t)d2u_x86(rgba[j] * (double)mask, 0) & mask) << pf.shift[j];
        }
        std::memcpy(texel, &bits, pf.bytes);
    }
    for (int j = 0; j < nc; ++j)
    {
        uint8_t* c = texel + j * cb;
        if (kind == 2 && nc == 4) { const uint32_t u = d2u32_vec(rgba[j] * kMax[kind]); std::memcpy(c, &u, 4); }
        else if (kind <= 3) { const uint64_t u = d2u_x86(rgba[j] * kMax[kind], kind); std::memcpy(c, &u, cb); }
        else if (kind == 4) { const uint16_t h = slg_float_to_half((float)rgba[j]); std::memcpy(c, &h, 2); }
        else if (kind == 5) { const float f = (float)rgba[j]; std::memcpy(c, &f, 4); }
        else std::memcpy(c, &rgba[j], 8);
    }
    /* one texel, then the filled prefix doubled: the texel pattern repeats */
    uint8_t* dst = t.bytes.data();
    const size_t total = bpt * n;
    if (total == 0) return;
    std::memcpy(dst, texel, bpt);
    for (size_t done = bpt; done < total;)
    {
        const size_t c = std::min(done, total - done);
        std::memcpy(dst + done, dst, c);
        done += c;
    }
}

int slo_clear_color_buffer(slo_context* ctx, size_t fbo, unsigned att, const double rgba[4])
{
    if (fbo >= ctx->fbos.size() || att >= ctx->fbos[fbo].numColors) return ctx->fail(SLG_ERR_INVALID_ARG, "invalid fbo");
    clear_color(*ctx->textures[ctx->fbos[fbo].colors[att]], rgba, ctx->numThreads);
    return SLG_OK;
}

int slo_clear_depth_buffer(slo_context* ctx, size_t fbo, double depth)
{
    if (fbo >= ctx->fbos.size() || ctx->fbos[fbo].depth == SLG_INVALID_ID) return ctx->fail(SLG_ERR_INVALID_ARG, "invalid fbo");
    const double d[4] = {depth, 0, 0, 0};
    clear_color(*ctx->textures[ctx->fbos[fbo].depth], d, ctx->numThreads);
    return SLG_OK;
}

int slo_clear_framebuffer(slo_context* ctx, size_t fbo, unsigned att, const double rgba[4], double depth)
{
    int r = slo_clear_color_buffer(ctx, fbo, att, rgba);
    if (r) return r;
    return slo_clear_depth_buffer(ctx, fbo, depth);
}

/* Runs a list of draw groups. Each group is what one SL_Context::draw,
 * draw_instanced or draw_multiple call hands to SL_TriProcessor::execute
 * (SL_TriProcessor.cpp:665-716): bins are produced in element order and
 * rasterised in that order (one thread), in flush groups of 1024. With more
 * than one host thread the vertex stage splits the element range into
 * contiguous chunks whose bins are concatenated in order, and the raster
 * stage splits scan-lines y % N across threads; both keep the one-thread
 * result. */
static int run_draws(slo_context* ctx, const std::vector<std::vector<DrawItem>>& groups, size_t fboId)
{
    if (fboId >= ctx->fbos.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid fbo id");
    const Fbo& fbo = ctx->fbos[fboId];
    if (fbo.depth == SLG_INVALID_ID) return ctx->fail(SLG_ERR_INVALID_ARG, "framebuffer has no depth attachment");
    Texture& depthTex = *ctx->textures[fbo.depth];

    RasterState rs;
    rs.ctx = ctx;
    rs.depth = depthTex.bytes.data();
    rs.depthType = depthTex.type;
    rs.width = depthTex.w;
    rs.height = depthTex.h;
    rs.numOutputs = 0;
    for (unsigned i = 0; i < fbo.numColors && i < 4; ++i)
    {
        if (fbo.colors[i] == SLG_INVALID_ID || fbo.colors[i] >= ctx->textures.size()) break;
        Texture& t = *ctx->textures[fbo.colors[i]];
        rs.colors[i].bytes = t.bytes.data();
        rs.colors[i].type = t.type;
        rs.colors[i].w = t.w;
        rs.numOutputs = i + 1;
    }

    /* SL_TriProcessor::execute viewport set-up (SL_TriProcessor.cpp:672-675,
     * SL_ViewportState.cpp:17-110) with the default viewport and scissor
     * (0, 0, 65535, 65535). */
    const float fboW = (float)depthTex.w, fboH = (float)depthTex.h;
    float scissor[16];
    {
        const float invW = 1.f / fboW, invH = 1.f / fboH;
        float sx = 0.f * invW, sy = 0.f * invH;
        float sw = 65535.f * invW, sh = 65535.f * invH;
        if (sx < 0.f) { sw += sx; sx = 0.f; }
        if (sy < 0.f) { sh += sy; sy = 0.f; }
        sw = lm_min(1.f - sx, sw);
        sh = lm_min(1.f - sy, sh);
        const float nm00 = 1.f / sw, nm11 = 1.f / sh;
        const float nm30 = nm00 - 1.f, nm31 = nm11 - 1.f;
        const float m30 = sx * (-2.f * nm00) + nm30;
        const float m31 = sy * (-2.f * nm11) + nm31;
        const float m[16] = {nm00, 0, 0, 0, 0, nm11, 0, 0, 0, 0, 1, 0, m30, m31, 0, 1};
        std::memcpy(scissor, m, sizeof(m));
    }
    V4 viewport;
    {
        const float vx = lm_min(lm_max(0.f + 0.f, 0.f), fboW);
        const float vy = lm_min(lm_max(0.f + 0.f, 0.f), fboH);
        viewport = mk(vx, vy, lm_min(lm_min(65535.f, (0.f + 65535.f) - vx), fboW - vx),
                      lm_min(lm_min(65535.f, (0.f + 65535.f) - vy), fboH - vy));
    }

    uint64_t totalBins = 0, totalFrags = 0;
    const unsigned nthreads = std::max(1u, ctx->numThreads);

    for (const std::vector<DrawItem>& group : groups)
    {
        /* one bin stream per group, in the order SL_TriProcessor::execute walks it */
        std::vector<DrawState> states;
        rs.shaders.clear();
        rs.envs.clear();
        for (size_t d = 0; d < group.size(); ++d)
        {
            const DrawItem& it = group[d];
            if (it.shaderId >= ctx->shaders.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid shader id");
            if (it.mesh.vaoId >= ctx->vaos.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid vao id");
            const Shader& sh = ctx->shaders[it.shaderId];
            const Vao& vao = ctx->vaos[it.mesh.vaoId];
            if (vao.vbo == SLG_INVALID_ID) return ctx->fail(SLG_ERR_INVALID_ARG, "vao has no vertex buffer");
            DrawState ds;
            ds.ctx = ctx;
            ds.shader = &sh;
            ds.env.ctx = ctx;
            ds.env.vboBytes = ctx->vbos[vao.vbo].bytes.data();
            ds.env.b0 = vao.bindings[0];
            ds.env.ubo = sh.ubo != SLG_INVALID_ID ? ctx->ubos[sh.ubo]->bytes : nullptr;
            std::memcpy(ds.scissor, scissor, sizeof(scissor));
            ds.viewport = viewport;
            ds.numVaryings = sh.numVaryings;
            ds.drawIndex = (uint32_t)d;
            states.push_back(ds);
            rs.shaders.push_back(&sh);
            rs.envs.push_back(ds.env);
        }

        /* enumerate (draw, instance) work units in execution order */
        struct Unit { size_t draw, instance; };
        std::vector<Unit> units;
        for (size_t d = 0; d < group.size(); ++d)
        {
            for (size_t inst = 0; inst < std::max<size_t>(1, group[d].numInstances); ++inst)
            {
                units.push_back({d, inst});
            }
        }

        const bool blending = group.empty() ? false : (ctx->shaders[group[0].shaderId].blend != SLG_BLEND_OFF);

        if (!group.empty() && (group[0].mesh.mode == SLG_RENDER_MODE_POINTS || group[0].mesh.mode == SLG_RENDER_MODE_INDEXED_POINTS))
        {
            /* SL_PointProcessor::process_verts and SL_PointRasterizer::render_point
             * (softlight/src/SL_PointProcessor.cpp:63-110, SL_PointRasterizer.cpp:26-90),
             * one thread: points in element order, each depth-tested and
             * written at once, at linear index x + W*y of its 16-bit screen
             * coordinates (an index past the buffer is dropped). */
            const size_t W = depthTex.w, H = depthTex.h;
            for (const Unit& u : units)
            {
                const DrawItem& it = group[u.draw];
                const DrawState& ds = states[u.draw];
                const Shader& sh = *ds.shader;
                const Vao& vao = ctx->vaos[it.mesh.vaoId];
                const bool indexed = (it.mesh.mode == SLG_RENDER_MODE_INDEXED_POINTS);
                const Ibo* ibo = (indexed && vao.ibo != SLG_INVALID_ID) ? &ctx->ibos[vao.ibo] : nullptr;
                if (indexed && !ibo) return ctx->fail(SLG_ERR_INVALID_ARG, "indexed draw without index buffer");
                for (size_t i = it.mesh.elementBegin; i < it.mesh.elementEnd; ++i)
                {
                    const size_t vertId = ibo ? read_index(*ibo, i) : i;
                    V4 vary[4];
                    for (int k = 0; k < 4; ++k) vary[k] = mk(0.f, 0.f, 0.f, 0.f);
                    V4 v = mat_mul(ds.scissor, run_vs(sh.vsProgram, ds.env, vertId, u.instance, vary));
                    const float w = v[3], nw = -v[3];
                    const bool visible = (w > 0.f) && (v[0] <= w && v[1] <= w && v[2] <= w && v[3] <= w) &&
                                         (v[0] >= nw && v[1] >= nw && v[2] >= nw && v[3] >= nw);
                    if (!visible) continue;
                    perspective_divide(v);
                    ndc_to_screen(v, ds.viewport);
                    const size_t x = (uint32_t)f2i(v[0]) & 0xFFFFu, y = (uint32_t)f2i(v[1]) & 0xFFFFu;
                    const size_t lin = x + W * y;
                    if (lin >= W * H) continue;
                    const float z = v[2];
                    if (!depth_cmp(sh.depthTest, z, dget(rs, lin))) continue;
                    V4 outputs[4];
                    slg_frag_coord coord = frag_coord((uint32_t)x, (uint32_t)y, z);
                    if (run_fs(sh.fsProgram, ds.env, coord, vary, outputs))
                    {
                        for (unsigned t = 0; t < sh.numOutputs && t < rs.numOutputs; ++t)
                        {
                            write_color(rs.colors[t], (unsigned)(lin % W), (unsigned)(lin / W), outputs[t], sh.blend);
                        }
                    }
                    if (sh.depthMask == SLG_DEPTH_MASK_ON) dset(rs, lin, coord.depth);
                    ++totalFrags;
                }
            }
            continue;
        }

        if (!group.empty() && (group[0].mesh.mode == SLG_RENDER_MODE_LINES || group[0].mesh.mode == SLG_RENDER_MODE_INDEXED_LINES))
        {
            for (const Unit& u : units)
            {
                const DrawItem& it = group[u.draw];
                const Vao& vao = ctx->vaos[it.mesh.vaoId];
                const bool indexed = (it.mesh.mode == SLG_RENDER_MODE_INDEXED_LINES);
                const Ibo* ibo = (indexed && vao.ibo != SLG_INVALID_ID) ? &ctx->ibos[vao.ibo] : nullptr;
                if (indexed && !ibo) return ctx->fail(SLG_ERR_INVALID_ARG, "indexed draw without index buffer");
                process_lines(rs, states[u.draw], ibo, it.mesh, u.instance, totalFrags);
            }
            continue;
        }

        /* Bins are produced in chunks of whole triangles, each chunk split
         * into contiguous per-thread slices (concatenated in order), and
         * rasterised in whole 1024-bin flush groups as they complete
         * (SL_VertexProcessor::flush_rasterizer, SL_VertexProcessor.cpp:
         * 84-181): the groups are sorted by primIndex when blending, and
         * thread t draws rows y % N == t of every bin in order, so each
         * pixel sees its fragments in the one-thread order. */
        const bool wire = !group.empty() && (group[0].mesh.mode == SLG_RENDER_MODE_TRI_WIRE ||
                                             group[0].mesh.mode == SLG_RENDER_MODE_INDEXED_TRI_WIRE);
        struct Slice { size_t unit, first, last; };   /* elements [first, last) of one unit */
        std::vector<const Ibo*> unitIbo(units.size(), nullptr);
        std::vector<size_t> unitStart(units.size() + 1, 0);
        for (size_t k = 0; k < units.size(); ++k)
        {
            const DrawItem& it = group[units[k].draw];
            const Vao& vao = ctx->vaos[it.mesh.vaoId];
            const bool indexed = (it.mesh.mode == SLG_RENDER_MODE_INDEXED_TRIANGLES || it.mesh.mode == SLG_RENDER_MODE_INDEXED_TRI_WIRE);
            unitIbo[k] = (indexed && vao.ibo != SLG_INVALID_ID) ? &ctx->ibos[vao.ibo] : nullptr;
            if (indexed && !unitIbo[k]) return ctx->fail(SLG_ERR_INVALID_ARG, "indexed draw without index buffer");
            const size_t begin = it.mesh.elementBegin, end = it.mesh.elementEnd;
            unitStart[k + 1] = unitStart[k] + ((end > begin) ? (end - begin + 2) / 3 : 0);
        }
        const size_t totalTris = unitStart[units.size()];
        /* the elements of global triangles [t0, t1), unit by unit */
        const auto slices_of = [&](size_t t0, size_t t1, std::vector<Slice>& out) {
            out.clear();
            size_t k = (size_t)(std::upper_bound(unitStart.begin(), unitStart.end(), t0) - unitStart.begin()) - 1;
            for (; k < units.size() && unitStart[k] < t1; ++k)
            {
                const size_t a = std::max(t0, unitStart[k]) - unitStart[k];
                const size_t b = std::min(t1, unitStart[k + 1]) - unitStart[k];
                if (a >= b) continue;
                const slg_mesh& m = group[units[k].draw].mesh;
                out.push_back({k, m.elementBegin + 3 * a, std::min(m.elementEnd, m.elementBegin + 3 * b)});
            }
        };
        const size_t chunkTris = std::max<size_t>(4096, 2048 * (size_t)nthreads);
        /* bins of a chunk stay in the producing thread's vector; `stream`
         * points at them in stream order. Bins left over past the last whole
         * flush group are copied to `carry` (fewer than 1024) before the
         * vectors are reused. */
        std::vector<std::vector<Bin>> parts(nthreads);
        std::vector<std::vector<Slice>> partSlices(nthreads);
        std::vector<Bin> carry, carryNext;
        std::vector<const Bin*> stream;
        std::vector<uint64_t> frags(nthreads, 0);
        size_t chunk0 = 0;
        bool vertexPhase = true;
        size_t rasterCount = 0;
        const auto work = [&](unsigned t) {
            if (vertexPhase)
            {
                parts[t].clear();
                for (const Slice& sl : partSlices[t])
                {
                    const Unit& u = units[sl.unit];
                    process_verts(states[u.draw], unitIbo[sl.unit], group[u.draw].mesh, u.instance, sl.first, sl.last, parts[t]);
                }
                return;
            }
            /* a local count: per-thread slots of one vector share cache lines */
            uint64_t count = 0;
            for (size_t i = 0; i < rasterCount; ++i)
            {
                if (wire) raster_wire_bin(rs, *stream[i], (int)nthreads, (int)t, count);
                else raster_bin(rs, *stream[i], (int)nthreads, (int)t, count);
            }
            frags[t] += count;
        };
        if (!ctx->pool || ctx->pool->size() != nthreads) ctx->pool.reset(new WorkerPool(nthreads));
        WorkerPool& pool = *ctx->pool;
        while (chunk0 < totalTris || !carry.empty())
        {
            stream.clear();
            for (const Bin& b : carry) stream.push_back(&b);
            const size_t chunk1 = std::min(totalTris, chunk0 + chunkTris);
            if (chunk0 < chunk1)
            {
                const size_t per = (chunk1 - chunk0 + nthreads - 1) / nthreads;
                for (unsigned t = 0; t < nthreads; ++t)
                {
                    const size_t a = std::min(chunk1, chunk0 + per * t), b = std::min(chunk1, chunk0 + per * (t + 1));
                    slices_of(a, b, partSlices[t]);
                }
                vertexPhase = true;
                pool.run(work);
                for (const std::vector<Bin>& p : parts)
                    for (const Bin& b : p) stream.push_back(&b);
            }
            chunk0 = chunk1;
            /* whole flush groups, or everything at the end of the stream */
            const size_t flushGroup = 1024; /* SL_SHADER_MAX_BINNED_PRIMS (SL_Config.hpp:53) */
            rasterCount = (chunk0 < totalTris) ? (stream.size() / flushGroup) * flushGroup : stream.size();
            if (blending)
            {
                /* the stable sort of bin ids (utils::sort_radix) */
                for (size_t b = 0; b < rasterCount; b += flushGroup)
                {
                    std::stable_sort(stream.begin() + b, stream.begin() + std::min(rasterCount, b + flushGroup),
                                     [](const Bin* l, const Bin* r) { return l->primIndex < r->primIndex; });
                }
            }
            if (rasterCount > 0)
            {
                vertexPhase = false;
                pool.run(work);
                totalBins += rasterCount;
            }
            carryNext.clear();
            for (size_t i = rasterCount; i < stream.size(); ++i) carryNext.push_back(*stream[i]);
            carry.swap(carryNext);
        }
        for (uint64_t f : frags) totalFrags += f;
    }

    ctx->lastBins = totalBins;
    ctx->lastFrags = totalFrags;
    return SLG_OK;
}

static bool valid_tri_mesh(const slg_mesh* m)
{
    return m && (m->mode == SLG_RENDER_MODE_TRIANGLES || m->mode == SLG_RENDER_MODE_INDEXED_TRIANGLES ||
                 m->mode == SLG_RENDER_MODE_POINTS || m->mode == SLG_RENDER_MODE_INDEXED_POINTS ||
                 m->mode == SLG_RENDER_MODE_LINES || m->mode == SLG_RENDER_MODE_INDEXED_LINES ||
                 m->mode == SLG_RENDER_MODE_TRI_WIRE || m->mode == SLG_RENDER_MODE_INDEXED_TRI_WIRE);
}

int slo_draw(slo_context* ctx, const slg_mesh* m, size_t shaderId, size_t fboId)
{
    return slo_draw_instanced(ctx, m, 1, shaderId, fboId);
}

int slo_draw_instanced(slo_context* ctx, const slg_mesh* m, size_t numInstances, size_t shaderId, size_t fboId)
{
    if (!valid_tri_mesh(m)) return ctx->fail(SLG_ERR_INVALID_ARG, "unsupported render mode");
    std::vector<std::vector<DrawItem>> groups(1);
    groups[0].push_back({*m, numInstances, shaderId, false});
    return run_draws(ctx, groups, fboId);
}

int slo_draw_multiple(slo_context* ctx, const slg_mesh* meshes, size_t numMeshes, size_t shaderId, size_t fboId)
{
    if (!meshes || !numMeshes) return SLG_OK;
    std::vector<std::vector<DrawItem>> groups(1);
    for (size_t i = 0; i < numMeshes; ++i)
    {
        if (!valid_tri_mesh(&meshes[i])) return ctx->fail(SLG_ERR_INVALID_ARG, "unsupported render mode");
        groups[0].push_back({meshes[i], 1, shaderId, true});
    }
    return run_draws(ctx, groups, fboId);
}

int slo_draw_batch(slo_context* ctx, const slg_draw_cmd* cmds, size_t numCmds, size_t fboId)
{
    std::vector<std::vector<DrawItem>> groups;
    for (size_t i = 0; i < numCmds; ++i)
    {
        if (!valid_tri_mesh(&cmds[i].mesh)) return ctx->fail(SLG_ERR_INVALID_ARG, "unsupported render mode");
        groups.push_back({{cmds[i].mesh, cmds[i].numInstances, cmds[i].shaderId, false}});
    }
    return run_draws(ctx, groups, fboId);
}

int slo_finish(slo_context*) { return SLG_OK; }

void slo_last_stats(const slo_context* ctx, uint64_t* numBins, uint64_t* numFragments)
{
    if (numBins) *numBins = ctx->lastBins;
    if (numFragments) *numFragments = ctx->lastFrags;
}

/*-----------------------------------------------------------------------------
 * Scene graph: SL_SceneGraph (softlight/src/SL_SceneGraph.cpp) with
 * SL_Transform (softlight/src/SL_Transform.cpp) and the mesh-node traversal
 * of SoftLight's scene demos (softlight/tests/sl_large_scene_test.cpp:678-740).
 * Matrix arithmetic in the order of the LightMath layer the reference is
 * built against: column-major, mat * vec sums the scaled columns left to
 * right.
-----------------------------------------------------------------------------*/
static void sg_mat_vec(const float* m, const float v[4], float out[4])
{
    for (int r = 0; r < 4; ++r) out[r] = ((m[r] * v[0] + m[4 + r] * v[1]) + m[8 + r] * v[2]) + m[12 + r] * v[3];
}

static std::array<float, 16> sg_mat_mul(const float* a, const float* b)
{
    std::array<float, 16> r;
    for (int c = 0; c < 4; ++c) sg_mat_vec(a, b + 4 * c, r.data() + 4 * c);
    return r;
}

/* get_rst_matrix / get_str_matrix (SL_Transform.cpp:408-432) with the
 * quaternion's rotation matrix; apply_transform swaps them for the FPS view
 * types (SL_Transform.cpp:319-328) */
static std::array<float, 16> sg_local(const slg_transform& t)
{
    const float x = t.orientation[0], y = t.orientation[1], z = t.orientation[2], w = t.orientation[3];
    const float xx = x * x, yy = y * y, zz = z * z, xy = x * y, xz = x * z, yz = y * z, wx = w * x, wy = w * y, wz = w * z;
    const float rot[16] = {1.f - 2.f * (yy + zz), 2.f * (xy + wz), 2.f * (xz - wy), 0.f,
                           2.f * (xy - wz), 1.f - 2.f * (xx + zz), 2.f * (yz + wx), 0.f,
                           2.f * (xz + wy), 2.f * (yz - wx), 1.f - 2.f * (xx + yy), 0.f,
                           0.f, 0.f, 0.f, 1.f};
    const float ts[16] = {t.scaling[0], 0.f, 0.f, 0.f, 0.f, t.scaling[1], 0.f, 0.f, 0.f, 0.f, t.scaling[2], 0.f,
                          t.position[0], t.position[1], t.position[2], 1.f};
    const bool fps = t.type == 1 || t.type == 3;
    return fps ? sg_mat_mul(rot, ts) : sg_mat_mul(ts, rot);
}

/* sl_is_visible(const SL_BoundingBox&, mv, planes) (SL_Camera.cpp:63-85) */
static bool sg_visible(const std::array<float, 8>& b, const float* mv, const float planes[24])
{
    float hi[4], lo[4];
    sg_mat_vec(mv, b.data(), hi);
    sg_mat_vec(mv, b.data() + 4, lo);
    float c[3], h[3];
    for (int k = 0; k < 3; ++k)
    {
        c[k] = (hi[k] + lo[k]) * 0.5f;
        h[k] = (hi[k] - lo[k]) * 0.5f;
    }
    const float radius = std::sqrt((h[0] * h[0] + h[1] * h[1]) + h[2] * h[2]);
    for (int i = 0; i < 6; ++i)
    {
        const float* p = planes + 4 * i;
        if ((((c[0] * p[0] + c[1] * p[1]) + c[2] * p[2]) + p[3]) + radius <= 0.f) return false;
    }
    return true;
}

static SloScene* sg_scene(slo_context* ctx, size_t id)
{
    return (id < ctx->scenes.size()) ? &ctx->scenes[id] : nullptr;
}

size_t slo_create_scene(slo_context* ctx)
{
    ctx->scenes.emplace_back();
    return ctx->scenes.size() - 1;
}

int slo_scene_insert_mesh(slo_context* ctx, size_t sceneId, const slg_mesh* mesh, const float maxPoint[3],
                          const float minPoint[3], size_t* outMeshId)
{
    SloScene* sc = sg_scene(ctx, sceneId);
    if (!sc) return ctx->fail(SLG_ERR_INVALID_ID, "invalid scene id");
    if (!mesh || !maxPoint || !minPoint || !outMeshId) return ctx->fail(SLG_ERR_INVALID_ARG, "null argument");
    if (mesh->vaoId >= ctx->vaos.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid vao id");
    sc->meshes.push_back(*mesh);
    sc->bounds.push_back({maxPoint[0], maxPoint[1], maxPoint[2], 1.f, minPoint[0], minPoint[1], minPoint[2], 1.f});
    *outMeshId = sc->meshes.size() - 1;
    return SLG_OK;
}

int slo_scene_insert_material(slo_context* ctx, size_t sceneId, size_t ambientTextureId, size_t* outMaterialId)
{
    SloScene* sc = sg_scene(ctx, sceneId);
    if (!sc) return ctx->fail(SLG_ERR_INVALID_ID, "invalid scene id");
    if (!outMaterialId) return ctx->fail(SLG_ERR_INVALID_ARG, "null argument");
    sc->materials.push_back(ambientTextureId);
    *outMaterialId = sc->materials.size() - 1;
    return SLG_OK;
}

/* insert_empty_node / insert_mesh_node (SL_SceneGraph.cpp:1180-1258): the
 * node is appended with the transform as given (dirty; its model matrix
 * the identity of a transform never applied), a mesh node's default
 * bounding box appended to mMeshBounds */
int slo_scene_insert_node(slo_context* ctx, size_t sceneId, size_t parentId, size_t numSubMeshes, const size_t* subMeshIds,
                          const slg_transform* transform, size_t* outNodeId)
{
    SloScene* sc = sg_scene(ctx, sceneId);
    if (!sc) return ctx->fail(SLG_ERR_INVALID_ID, "invalid scene id");
    if (!outNodeId || !transform || (numSubMeshes && !subMeshIds)) return ctx->fail(SLG_ERR_INVALID_ARG, "null argument");
    if (transform->type > 4) return ctx->fail(SLG_ERR_INVALID_ARG, "unknown transform type");
    if (parentId != SLG_SCENE_ROOT && parentId >= sc->parents.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid parent node");
    size_t depth = 1;
    for (uint64_t p = parentId; p != SLG_SCENE_ROOT; p = sc->parents[p]) ++depth;
    if (depth > 64) return ctx->fail(SLG_ERR_INVALID_ARG, "scene paths hold at most 64 nodes");
    for (size_t k = 0; k < numSubMeshes; ++k)
        if (subMeshIds[k] >= sc->meshes.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid submesh id");
    sc->parents.push_back(parentId);
    sc->transforms.push_back(*transform);
    sc->dirty.push_back(1);
    std::array<float, 16> ident{};
    ident[0] = ident[5] = ident[10] = ident[15] = 1.f;
    sc->models.push_back(ident);
    sc->nodeMeshes.emplace_back(subMeshIds, subMeshIds + numSubMeshes);
    if (numSubMeshes) sc->bounds.push_back({1.f, 1.f, 1.f, 1.f, -1.f, -1.f, -1.f, 1.f});
    *outNodeId = sc->parents.size() - 1;
    return SLG_OK;
}

int slo_scene_set_transform(slo_context* ctx, size_t sceneId, size_t nodeId, const slg_transform* transform)
{
    SloScene* sc = sg_scene(ctx, sceneId);
    if (!sc) return ctx->fail(SLG_ERR_INVALID_ID, "invalid scene id");
    if (nodeId >= sc->parents.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid node id");
    if (!transform || transform->type > 4) return ctx->fail(SLG_ERR_INVALID_ARG, "invalid transform");
    sc->transforms[nodeId] = *transform;
    sc->dirty[nodeId] = 1;
    return SLG_OK;
}

/* SL_SceneGraph::update (SL_SceneGraph.cpp:223-299) */
int slo_scene_update(slo_context* ctx, size_t sceneId)
{
    SloScene* sc = sg_scene(ctx, sceneId);
    if (!sc) return ctx->fail(SLG_ERR_INVALID_ID, "invalid scene id");
    const size_t n = sc->parents.size();
    auto update_node = [&](size_t j) {
        const std::array<float, 16> local = sg_local(sc->transforms[j]);
        sc->models[j] = (sc->parents[j] == SLG_SCENE_ROOT) ? local : sg_mat_mul(sc->models[sc->parents[j]].data(), local.data());
        sc->dirty[j] = 0;
    };
    for (size_t i = 0; i < n; ++i)
    {
        if (!sc->dirty[i]) continue;
        update_node(i);
        for (size_t j = i + 1; j < n; ++j)
        {
            if (sc->parents[j] < i)
            {
                i = j - 1;
                break;
            }
            update_node(j);
        }
    }
    return SLG_OK;
}

int slo_scene_read_models(slo_context* ctx, size_t sceneId, float* out, size_t numNodes)
{
    SloScene* sc = sg_scene(ctx, sceneId);
    if (!sc) return ctx->fail(SLG_ERR_INVALID_ID, "invalid scene id");
    if (!out || numNodes != sc->parents.size()) return ctx->fail(SLG_ERR_INVALID_ARG, "node count");
    for (size_t i = 0; i < numNodes; ++i) std::memcpy(out + 16 * i, sc->models[i].data(), 64);
    return SLG_OK;
}

/* The demos' traversal: per mesh node, model and vp * ... into the uniform
 * block; per submesh, the frustum test, the triangle-mode test, the
 * material's texture, then SL_Context::draw. The template block is written
 * for each draw and restored at the end. */
int slo_scene_draw(slo_context* ctx, size_t sceneId, size_t fboId, size_t shaderId, const float projection[16],
                   const float view[16], const float cullProjection[16])
{
    uint64_t bins = 0, frags = 0;
    SloScene* sc = sg_scene(ctx, sceneId);
    if (!sc) return ctx->fail(SLG_ERR_INVALID_ID, "invalid scene id");
    if (!projection || !view) return ctx->fail(SLG_ERR_INVALID_ARG, "null matrix");
    if (shaderId >= ctx->shaders.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid shader id");
    const Shader& sh = ctx->shaders[shaderId];
    if (sh.vsProgram != SLG_PROGRAM_LAMBERT_TEX || sh.fsProgram != SLG_PROGRAM_LAMBERT_TEX || sh.ubo == SLG_INVALID_ID)
        return ctx->fail(SLG_ERR_INVALID_ARG, "scene draws take a SLG_PROGRAM_LAMBERT_TEX shader with a uniform block");
    if (fboId >= ctx->fbos.size()) return ctx->fail(SLG_ERR_INVALID_ID, "invalid fbo id");

    /* sl_extract_frustum_planes (SL_Camera.cpp:25-49) */
    const bool cull = cullProjection != nullptr;
    float planes[24] = {};
    for (int i = 0; i < 4 && cull; ++i)
    {
        const float* col = cullProjection + 4 * i;
        planes[0 + i] = col[3] + col[0];
        planes[4 + i] = col[3] - col[0];
        planes[8 + i] = col[3] + col[1];
        planes[12 + i] = col[3] - col[1];
        planes[16 + i] = col[3] + col[2];
        planes[20 + i] = col[3] - col[2];
    }
    for (int k = 0; k < 6 && cull; ++k)
    {
        float* q = planes + 4 * k;
        const float lenInv = 1.f / std::sqrt((q[0] * q[0] + q[1] * q[1]) + q[2] * q[2]);
        for (int i = 0; i < 4; ++i) q[i] = q[i] * lenInv;
    }
    const std::array<float, 16> vp = sg_mat_mul(projection, view);

    Ubo& ubo = *ctx->ubos[sh.ubo];
    slg_lambert_uniforms saved;
    std::memcpy(&saved, ubo.bytes, sizeof(saved));
    int status = SLG_OK;
    for (size_t node = 0; node < sc->parents.size() && status == SLG_OK; ++node)
    {
        if (sc->nodeMeshes[node].empty()) continue;
        const std::array<float, 16>& model = sc->models[node];
        const std::array<float, 16> mv = sg_mat_mul(view, model.data());
        for (const uint64_t meshId : sc->nodeMeshes[node])
        {
            const slg_mesh& m = sc->meshes[meshId];
            if (cull && !sg_visible(sc->bounds[meshId], mv.data(), planes)) continue;
            if (!(m.mode & SLG_RENDER_MODE_TRIANGLES)) continue;
            if (m.materialId >= sc->materials.size())
            {
                status = ctx->fail(SLG_ERR_INVALID_ARG, "scene mesh has no material");
                break;
            }
            slg_lambert_uniforms u = saved;
            std::memcpy(u.vpMatrix, vp.data(), 64);
            std::memcpy(u.modelMatrix, model.data(), 64);
            u.textureId = (uint32_t)sc->materials[m.materialId];
            std::memcpy(ubo.bytes, &u, sizeof(u));
            status = slo_draw(ctx, &m, shaderId, fboId);
            bins += ctx->lastBins;
            frags += ctx->lastFrags;
        }
    }
    std::memcpy(ubo.bytes, &saved, sizeof(saved));
    /* the statistics of the whole draw list */
    ctx->lastBins = bins;
    ctx->lastFrags = frags;
    return status;
}

} // extern "C"
