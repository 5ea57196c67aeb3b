/*
 * slg_programs.h - built-in shader programs of the GB300 draw path.
 *
 * SoftLight shaders are C callbacks with the signatures
 *     vec4 vertex_shader(SL_VertexParam&)      (softlight/include/softlight/SL_Shader.hpp:41-66)
 *     bool fragment_shader(SL_FragmentParam&)  (softlight/include/softlight/SL_Shader.hpp:74-92)
 * Here each program is a pair of header-only functions with the same inputs
 * and outputs, compiled for the device (and, unchanged, for host-side
 * checking). The "environment" template argument supplies what SL_VertexParam
 * and SL_FragmentParam carry in the reference: the vertex bytes of binding 0
 * (SL_VertexArray::offset(0, vertId), softlight/include/softlight/SL_VertexArray.hpp:120),
 * the uniform block, other vertex buffers by id, and texture sampling.
 *
 * Arithmetic rules (identical on host and device): every operation is a
 * separately rounded IEEE-754 binary32 operation in the order written; no
 * fused multiply-add (device code is built with --fmad=false, host code with
 * -ffp-contract=off); square roots and divisions are correctly rounded. The
 * specular power is an exact product chain, not powf, so results do not
 * depend on a math library.
 *
 * Uniform blocks are plain structs of at most 1024 bytes (the size of
 * SL_UniformBuffer, softlight/include/softlight/SL_UniformBuffer.hpp:12-20).
 * Where a reference test stores host pointers in its uniform block (a texture,
 * an instance-matrix array: softlight/tests/sl_instancing_test.cpp:84-93),
 * these blocks store resource ids instead.
 */
#ifndef SLG_PROGRAMS_H
#define SLG_PROGRAMS_H

#include <stdint.h>
#include <math.h>

#if defined(__CUDACC__)
    #define SLG_HD __host__ __device__ __forceinline__
#else
    #define SLG_HD static inline
#endif

/*-----------------------------------------------------------------------------
 * Uniform block layouts (column-major 4x4 matrices, like ls::math::mat4)
-----------------------------------------------------------------------------*/
/* SLG_PROGRAM_LAMBERT_TEX. Vertex layout (binding 0): float pos[3], uv[2],
 * normal[3]; 32-byte stride, as Tuple<vec3, vec2, vec3> in
 * softlight/tests/sl_instancing_test.cpp:107. */
typedef struct slg_lambert_uniforms
{
    float    vpMatrix[16];
    float    modelMatrix[16];
    float    lightDir[4];   /* unit vector towards the light, w = 0 */
    float    ambient[4];    /* added to the Lambert factor per channel */
    uint32_t textureId;     /* RGBA8 texture, bilinear, REPEAT */
    uint32_t pad[3];
} slg_lambert_uniforms;

/* SLG_PROGRAM_BLINN_PHONG_INST. Same vertex layout as Lambert. */
typedef struct slg_blinn_uniforms
{
    float    vpMatrix[16];
    float    camPos[4];        /* w = 1 */
    float    lightPos[4][4];   /* w = 1 */
    float    lightColor[4][4];
    float    ambient[4];
    float    specularity;
    float    attenuation;      /* k in 1 / (1 + k*d^2) */
    uint32_t textureId;        /* RGBA8 texture, bilinear, REPEAT */
    uint32_t instanceBufferId; /* vertex buffer of column-major float 4x4 model matrices, one per instance */
} slg_blinn_uniforms;

/* SLG_PROGRAM_VCOLOR_TEX_ALPHA, SLG_PROGRAM_VCOLOR_TEXF and SLG_PROGRAM_GBUFFER.
 * Vertex layout (binding 0): float pos[3], rgba[4], uv[2]; 36-byte stride. */
typedef struct slg_vcolor_uniforms
{
    float    mvpMatrix[16];
    uint32_t textureId;        /* RGBA8 (TEX_ALPHA) or RGBA float (TEXF) texture, bilinear, REPEAT */
    uint32_t pad[3];
} slg_vcolor_uniforms;

/* SLG_PROGRAM_VCOLOR_TEX_CUTOUT. Same vertex layout and block prefix as
 * slg_vcolor_uniforms; fragments whose alpha (vertex alpha x texel alpha)
 * is below alphaRef are discarded. */
typedef struct slg_cutout_uniforms
{
    float    mvpMatrix[16];
    uint32_t textureId;        /* RGBA8 texture, bilinear, REPEAT */
    float    alphaRef;
    uint32_t pad[2];
} slg_cutout_uniforms;

/* SLG_PROGRAM_FRAG_COORD. Same vertex layout and block prefix as
 * slg_vcolor_uniforms. The fragment stage reads the fragment coordinate:
 * output (x * invSize[0], y * invSize[1], depth, vertex alpha); where
 * screenDoor != 0, fragments with ((x ^ y) & screenDoor) == 0 are
 * discarded; the depth written is depth * depthScale + depthBias. */
typedef struct slg_fragcoord_uniforms
{
    float    mvpMatrix[16];
    float    invSize[2];
    float    depthScale;
    float    depthBias;
    uint32_t screenDoor;
    uint32_t pad[3];
} slg_fragcoord_uniforms;

/* SLG_PROGRAM_FLAT_COLOR. Vertex layout: float pos[3] at binding 0. */
typedef struct slg_flat_uniforms
{
    float mvpMatrix[16];
    float color[4];
} slg_flat_uniforms;

/*-----------------------------------------------------------------------------
 * Minimal vector helpers with a fixed evaluation order
-----------------------------------------------------------------------------*/
typedef struct slg_v4 { float x, y, z, w; } slg_v4;

/* SL_FragCoordXYZ (softlight/include/softlight/SL_ShaderUtil.hpp:668-673),
 * same layout: the fragment's 16-bit screen coordinates and its depth. A
 * fragment program may change depth; that value is what is written to the
 * depth buffer (softlight/src/SL_FragmentProcessor.cpp:524-527). */
typedef struct slg_frag_coord
{
    uint16_t x;
    uint16_t y;
    float    depth;
} slg_frag_coord;

SLG_HD slg_v4 slg_make_v4(float x, float y, float z, float w) { slg_v4 r; r.x = x; r.y = y; r.z = z; r.w = w; return r; }
SLG_HD slg_v4 slg_v4_load(const float* p) { return slg_make_v4(p[0], p[1], p[2], p[3]); }
SLG_HD slg_v4 slg_add(slg_v4 a, slg_v4 b) { return slg_make_v4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
SLG_HD slg_v4 slg_sub(slg_v4 a, slg_v4 b) { return slg_make_v4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
SLG_HD slg_v4 slg_mul(slg_v4 a, slg_v4 b) { return slg_make_v4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
SLG_HD slg_v4 slg_scale(slg_v4 a, float s) { return slg_make_v4(a.x * s, a.y * s, a.z * s, a.w * s); }
SLG_HD float  slg_dot(slg_v4 a, slg_v4 b) { return ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w; }
SLG_HD float  slg_maxf(float a, float b) { return (a < b) ? b : a; }
SLG_HD float  slg_minf(float a, float b) { return (b < a) ? b : a; }
SLG_HD slg_v4 slg_min1(slg_v4 a) { return slg_make_v4(slg_minf(a.x, 1.f), slg_minf(a.y, 1.f), slg_minf(a.z, 1.f), slg_minf(a.w, 1.f)); }
SLG_HD slg_v4 slg_normalize(slg_v4 a) { return slg_scale(a, 1.f / sqrtf(slg_dot(a, a))); }

/* column-major m (m[4*col + row]) times column vector v, summed column by column */
SLG_HD slg_v4 slg_mat_mul_v4(const float* m, slg_v4 v)
{
    slg_v4 r;
    r.x = ((m[0] * v.x + m[4] * v.y) + m[8]  * v.z) + m[12] * v.w;
    r.y = ((m[1] * v.x + m[5] * v.y) + m[9]  * v.z) + m[13] * v.w;
    r.z = ((m[2] * v.x + m[6] * v.y) + m[10] * v.z) + m[14] * v.w;
    r.w = ((m[3] * v.x + m[7] * v.y) + m[11] * v.z) + m[15] * v.w;
    return r;
}

/* x^50 as an exact product chain: x^32 * x^16 * x^2 */
SLG_HD float slg_pow50(float x)
{
    const float x2 = x * x;
    const float x4 = x2 * x2;
    const float x8 = x4 * x4;
    const float x16 = x8 * x8;
    const float x32 = x16 * x16;
    return (x32 * x16) * x2;
}

/*-----------------------------------------------------------------------------
 * Programs. Env must provide:
 *   const float* vertex(uint64_t vertId) const     -> binding-0 bytes of a vertex
 *   const void*  uniforms() const                    -> uniform block
 *   const float* buffer(uint32_t vboId) const        -> a vertex buffer's bytes
 *   slg_v4 sample_rgba8(uint32_t texId, float u, float v) const
 *       = color_cast<float>(sl_sample_bilinear<RGBA8, REPEAT>)  (softlight/include/softlight/SL_Sampler.hpp:187-218)
 *   slg_v4 sample_rgbaf(uint32_t texId, float u, float v) const
 *       = sl_sample_bilinear<RGBA float, REPEAT>
 * Vertex programs write their varyings and return the clip-space position;
 * fragment programs read varyings, write outputs and return whether to write
 * colour (SL_FragmentShader semantics).
-----------------------------------------------------------------------------*/
template <class Env>
SLG_HD slg_v4 slg_vs_lambert(const Env& env, uint64_t vertId, uint64_t instanceId, slg_v4* varyings)
{
    (void)instanceId;
    const slg_lambert_uniforms* u = (const slg_lambert_uniforms*)env.uniforms();
    const float* v = env.vertex(vertId);
    const slg_v4 pos  = slg_make_v4(v[0], v[1], v[2], 1.f);
    const slg_v4 uv   = slg_make_v4(v[3], v[4], 0.f, 0.f);
    const slg_v4 norm = slg_make_v4(v[5], v[6], v[7], 0.f);
    const slg_v4 world = slg_mat_mul_v4(u->modelMatrix, pos);
    varyings[0] = uv;
    varyings[1] = slg_mat_mul_v4(u->modelMatrix, norm);
    return slg_mat_mul_v4(u->vpMatrix, world);
}

template <class Env>
SLG_HD bool slg_fs_lambert(const Env& env, const slg_v4* varyings, slg_v4* outputs)
{
    const slg_lambert_uniforms* u = (const slg_lambert_uniforms*)env.uniforms();
    const slg_v4 albedo = env.sample_rgba8(u->textureId, varyings[0].x, varyings[0].y);
    const slg_v4 n = slg_normalize(varyings[1]);
    const float lambert = slg_maxf(slg_dot(n, slg_v4_load(u->lightDir)), 0.f);
    const slg_v4 light = slg_make_v4(u->ambient[0] + lambert, u->ambient[1] + lambert, u->ambient[2] + lambert, 1.f);
    const slg_v4 rgba = slg_mul(albedo, light);
    outputs[0] = slg_make_v4(slg_minf(rgba.x, 1.f), slg_minf(rgba.y, 1.f), slg_minf(rgba.z, 1.f), 1.f);
    return true;
}

template <class Env>
SLG_HD slg_v4 slg_vs_blinn(const Env& env, uint64_t vertId, uint64_t instanceId, slg_v4* varyings)
{
    const slg_blinn_uniforms* u = (const slg_blinn_uniforms*)env.uniforms();
    const float* v = env.vertex(vertId);
    const float* model = env.buffer(u->instanceBufferId) + 16u * instanceId;
    const slg_v4 pos  = slg_make_v4(v[0], v[1], v[2], 1.f);
    const slg_v4 norm = slg_make_v4(v[5], v[6], v[7], 0.f);
    const slg_v4 world = slg_mat_mul_v4(model, pos);
    varyings[0] = world;
    varyings[1] = slg_make_v4(v[3], v[4], 0.f, 0.f);
    varyings[2] = slg_mat_mul_v4(model, norm);
    return slg_mat_mul_v4(u->vpMatrix, world);
}

template <class Env>
SLG_HD bool slg_fs_blinn(const Env& env, const slg_v4* varyings, slg_v4* outputs)
{
    const slg_blinn_uniforms* u = (const slg_blinn_uniforms*)env.uniforms();
    const slg_v4 world = varyings[0];
    const slg_v4 albedo = env.sample_rgba8(u->textureId, varyings[1].x, varyings[1].y);
    const slg_v4 n = slg_normalize(varyings[2]);
    const slg_v4 view = slg_normalize(slg_sub(slg_v4_load(u->camPos), world));
    slg_v4 acc = slg_mul(albedo, slg_v4_load(u->ambient));

    for (int i = 0; i < 4; ++i)
    {
        const slg_v4 ld = slg_sub(slg_v4_load(u->lightPos[i]), world);
        const float d2 = slg_dot(ld, ld);
        const slg_v4 l = slg_scale(ld, 1.f / sqrtf(d2));
        const float diffuse = slg_maxf(slg_dot(n, l), 0.f);
        const slg_v4 h = slg_normalize(slg_add(l, view));
        const float spec = slg_pow50(slg_maxf(slg_dot(n, h), 0.f)) * u->specularity;
        const float atten = 1.f / (1.f + u->attenuation * d2);
        const slg_v4 lit = slg_add(slg_scale(albedo, diffuse), slg_make_v4(spec, spec, spec, spec));
        acc = slg_add(acc, slg_mul(slg_v4_load(u->lightColor[i]), slg_scale(lit, atten)));
    }

    outputs[0] = slg_make_v4(slg_minf(acc.x, 1.f), slg_minf(acc.y, 1.f), slg_minf(acc.z, 1.f), 1.f);
    return true;
}

template <class Env>
SLG_HD slg_v4 slg_vs_vcolor(const Env& env, uint64_t vertId, uint64_t instanceId, slg_v4* varyings)
{
    (void)instanceId;
    const slg_vcolor_uniforms* u = (const slg_vcolor_uniforms*)env.uniforms();
    const float* v = env.vertex(vertId);
    varyings[0] = slg_make_v4(v[3], v[4], v[5], v[6]);
    varyings[1] = slg_make_v4(v[7], v[8], 0.f, 0.f);
    return slg_mat_mul_v4(u->mvpMatrix, slg_make_v4(v[0], v[1], v[2], 1.f));
}

template <class Env>
SLG_HD bool slg_fs_vcolor_tex_alpha(const Env& env, const slg_v4* varyings, slg_v4* outputs)
{
    const slg_vcolor_uniforms* u = (const slg_vcolor_uniforms*)env.uniforms();
    const slg_v4 c = varyings[0];
    const slg_v4 t = env.sample_rgba8(u->textureId, varyings[1].x, varyings[1].y);
    outputs[0] = slg_make_v4(c.x * t.x, c.y * t.y, c.z * t.z, c.w);
    return true;
}

template <class Env>
SLG_HD bool slg_fs_vcolor_texf(const Env& env, const slg_v4* varyings, slg_v4* outputs)
{
    const slg_vcolor_uniforms* u = (const slg_vcolor_uniforms*)env.uniforms();
    const slg_v4 t = env.sample_rgbaf(u->textureId, varyings[1].x, varyings[1].y);
    outputs[0] = slg_mul(varyings[0], t);
    return true;
}

/* SLG_PROGRAM_GBUFFER: the outputs of a deferred G-buffer pass, one per
 * render target (SL_FragmentParam::pOutputs[0..3]): vertex colour x texture
 * (vertex alpha), the texture sample, the vertex colour, and channel products
 * (r*g, g*b, b*r, texture alpha). Every output stays in [0, 1] for colours
 * and textures in [0, 1]. The texture is RGBA8 (slg_vcolor_uniforms::textureId). */
template <class Env>
SLG_HD bool slg_fs_gbuffer(const Env& env, const slg_v4* varyings, slg_v4* outputs)
{
    const slg_vcolor_uniforms* u = (const slg_vcolor_uniforms*)env.uniforms();
    const slg_v4 c = varyings[0];
    const slg_v4 uv = varyings[1];
    const slg_v4 t = env.sample_rgba8(u->textureId, uv.x, uv.y);
    outputs[0] = slg_make_v4(c.x * t.x, c.y * t.y, c.z * t.z, c.w);
    outputs[1] = t;
    outputs[2] = c;
    outputs[3] = slg_make_v4(c.x * c.y, c.y * c.z, c.z * c.x, t.w);
    return true;
}

/* SLG_PROGRAM_VCOLOR_TEX_CUTOUT: an alpha test. Returns false (the fragment
 * is discarded: no colour is written, depth still is) where the combined
 * alpha is below alphaRef. */
template <class Env>
SLG_HD bool slg_fs_cutout(const Env& env, const slg_v4* varyings, slg_v4* outputs)
{
    const slg_cutout_uniforms* u = (const slg_cutout_uniforms*)env.uniforms();
    const slg_v4 c = varyings[0];
    const slg_v4 t = env.sample_rgba8(u->textureId, varyings[1].x, varyings[1].y);
    const float a = c.w * t.w;
    if (a < u->alphaRef)
    {
        return false;
    }
    outputs[0] = slg_make_v4(c.x * t.x, c.y * t.y, c.z * t.z, a);
    return true;
}

/* SLG_PROGRAM_FRAG_COORD: reads and writes the fragment coordinate. */
template <class Env>
SLG_HD bool slg_fs_frag_coord(const Env& env, slg_frag_coord* coord, const slg_v4* varyings, slg_v4* outputs)
{
    const slg_fragcoord_uniforms* u = (const slg_fragcoord_uniforms*)env.uniforms();
    const uint32_t x = coord->x, y = coord->y;
    if (u->screenDoor != 0u && ((x ^ y) & u->screenDoor) == 0u)
    {
        return false;
    }
    const float depth = coord->depth;
    outputs[0] = slg_make_v4((float)x * u->invSize[0], (float)y * u->invSize[1], depth, varyings[0].w);
    coord->depth = depth * u->depthScale + u->depthBias;
    return true;
}

template <class Env>
SLG_HD slg_v4 slg_vs_flat(const Env& env, uint64_t vertId, uint64_t instanceId, slg_v4* varyings)
{
    (void)instanceId; (void)varyings;
    const slg_flat_uniforms* u = (const slg_flat_uniforms*)env.uniforms();
    const float* v = env.vertex(vertId);
    return slg_mat_mul_v4(u->mvpMatrix, slg_make_v4(v[0], v[1], v[2], 1.f));
}

template <class Env>
SLG_HD bool slg_fs_flat(const Env& env, const slg_v4* varyings, slg_v4* outputs)
{
    (void)varyings;
    const slg_flat_uniforms* u = (const slg_flat_uniforms*)env.uniforms();
    outputs[0] = slg_v4_load(u->color);
    return true;
}

#endif /* SLG_PROGRAMS_H */
