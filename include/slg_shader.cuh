/*
 * slg_shader.cuh - shader programs written by the caller, for the GB300 draw
 * path.
 *
 * In SoftLight a shader is a pair of host callbacks,
 *     ls::math::vec4 vertex(SL_VertexParam&)     (softlight/include/softlight/SL_Shader.hpp:41-66)
 *     bool           fragment(SL_FragmentParam&) (softlight/include/softlight/SL_Shader.hpp:74-92)
 * handed to SL_Context::create_shader. Here the same pair is a pair of
 * __device__ functions over parameter structs of the same shape
 * (slg::VertexParam, slg::FragmentParam below, device pointers inside). A
 * program set gathers a caller's programs behind two dispatch functions:
 *
 *     struct MyPrograms
 *     {
 *         static __device__ slg::vec4 vertex(uint32_t program, slg::VertexParam& p);
 *         static __device__ bool fragment(uint32_t program, slg::FragmentParam& p);
 *     };
 *     SLG_DEFINE_PROGRAMS(MyPrograms, my_programs)   // in one .cu file
 *
 * SLG_DEFINE_PROGRAMS compiles the draw-path kernels (vertex stage, clipping,
 * rasterisers) for the set in the caller's translation unit and defines
 *     extern "C" const slg_pipeline_ops* my_programs(void);
 * whose table the caller passes to slg_register_programs together with the
 * set's program ids (>= SLG_PROGRAM_USER_FIRST) and flags. Shaders created
 * with those ids (slg_create_shader) then draw like built-in ones. To
 * compile the set in four translation units in parallel, use
 * SLG_PROGRAMS_ENTRY(MyPrograms, my_programs) in one file and
 * SLG_PROGRAMS_RASTER(MyPrograms, ColorRGBA8 | ColorRGBAF | ColorRF) in three
 * others, all compiled with the library's flags (nvcc -gencode
 * arch=compute_103a,code=sm_103a --fmad=false -prec-div=true -prec-sqrt=true
 * -ftz=false -std=c++17 -I include).
 *
 * Semantics, as in SoftLight:
 *  - a vertex program writes numVaryings varyings into p.pVaryings and
 *    returns the clip-space position; it must be a pure function of the
 *    vertex, the instance and what it reads (the vertex stage may run it once
 *    per vertex rather than once per triangle corner);
 *  - a fragment program reads p.coord (16-bit x, y and the depth the
 *    fragment passed the depth test with) and p.pVaryings, writes
 *    p.pOutputs[0 .. numOutputs-1] and returns false to discard: no colour is
 *    written, depth still is (SL_FragmentProcessor.cpp:501-529); the depth
 *    written is p.coord.depth after the program. A program that may return
 *    false is registered with SLG_PROGRAM_DISCARDS, one that may change
 *    p.coord.depth with SLG_PROGRAM_WRITES_DEPTH;
 *  - where SoftLight's uniform blocks hold host pointers (a texture, an
 *    array), blocks hold resource ids and p.pResources resolves them.
 */
#ifndef SLG_SHADER_CUH
#define SLG_SHADER_CUH

#include <cstddef>
#include <cstdint>

#include "slg.h"
#include "slg_programs.h"
#include "../softlight_gb300/csrc/slg_pipeline.cuh"

namespace slg
{

typedef slg_v4 vec4;

/* SL_UniformBuffer (softlight/include/softlight/SL_UniformBuffer.hpp:12-20):
 * the shader's 1024-byte block. */
struct UniformBuffer
{
    const uint8_t* bytes;

    template <typename T>
    __device__ __forceinline__ const T* as() const { return reinterpret_cast<const T*>(bytes); }
    __device__ __forceinline__ const void* buffer() const { return bytes; }
};

/* SL_VertexBuffer (softlight/include/softlight/SL_VertexBuffer.hpp:40-43). */
struct VertexBuffer
{
    const uint8_t* bytes;

    template <typename T>
    __device__ __forceinline__ const T* element(ptrdiff_t offset) const { return reinterpret_cast<const T*>(bytes + offset); }
    __device__ __forceinline__ const void* data() const { return bytes; }
};

/* SL_VertexArray (softlight/include/softlight/SL_VertexArray.hpp:63-66,
 * 109-126): byte offsets of the bindings. */
struct VertexArray
{
    const VaoView* view;

    __device__ __forceinline__ ptrdiff_t offset(size_t bindId) const { return (ptrdiff_t)view->offset[bindId & 7]; }
    __device__ __forceinline__ ptrdiff_t offset(size_t bindId, size_t vertId) const
    {
        return (ptrdiff_t)(view->offset[bindId & 7] + view->stride[bindId & 7] * (int64_t)vertId);
    }
    __device__ __forceinline__ ptrdiff_t stride(size_t bindId) const { return (ptrdiff_t)view->stride[bindId & 7]; }
};

/* Textures and vertex buffers by id, for ids held in a uniform block. An id
 * that is not a texture of the sampled format reads zero. */
struct Resources
{
    Tables tables;

    __device__ __forceinline__ const TexView* texture(uint32_t id) const
    {
        return (id < tables.numTextures) ? &tables.textures[id] : nullptr;
    }
    /* color_cast<float>(sl_sample_bilinear<SL_ColorRGBA8, SL_WrapMode::REPEAT>)
     * (softlight/include/softlight/SL_Sampler.hpp:187-218) */
    __device__ __forceinline__ vec4 sample_rgba8(uint32_t id, float u, float v) const
    {
        const TexView* t = texture(id);
        return (t && t->type == SLG_COLOR_RGBA_8U) ? slg::sample_rgba8(*t, u, v) : slg_make_v4(0.f, 0.f, 0.f, 0.f);
    }
    /* sl_sample_bilinear<SL_ColorRGBAf, SL_WrapMode::REPEAT> */
    __device__ __forceinline__ vec4 sample_rgbaf(uint32_t id, float u, float v) const
    {
        const TexView* t = texture(id);
        return (t && t->type == SLG_COLOR_RGBA_FLOAT) ? slg::sample_rgbaf(*t, u, v) : slg_make_v4(0.f, 0.f, 0.f, 0.f);
    }
    __device__ __forceinline__ const uint8_t* buffer(uint32_t id) const { return (id < tables.numBuffers) ? tables.buffers[id] : nullptr; }
};

/* SL_VertexParam (softlight/include/softlight/SL_Shader.hpp:41-51) */
struct VertexParam
{
    const UniformBuffer* pUniforms;
    size_t vertId;
    size_t instanceId;
    const VertexArray* pVao;
    const VertexBuffer* pVbo;
    vec4* pVaryings;
    const Resources* pResources;
};

/* SL_FragCoordXYZ (softlight/include/softlight/SL_ShaderUtil.hpp:668-673) */
typedef slg_frag_coord FragCoordXYZ;

/* SL_FragmentParam (softlight/include/softlight/SL_Shader.hpp:74-84) */
struct FragmentParam
{
    FragCoordXYZ coord;
    const UniformBuffer* pUniforms;
    vec4 pVaryings[kMaxVaryings];
    vec4 pOutputs[4];
    const Resources* pResources;
};

/* A caller's program set in the form the draw-path kernels take
 * (slg_pipeline.cuh): builds the parameter structs from the draw and
 * resource tables and calls User::vertex / User::fragment. */
template <class User>
struct CallerPrograms
{
    static __device__ __forceinline__ slg_v4 vertex(const DrawDesc& d, const Tables& t, uint64_t vertId, uint64_t instanceId,
                                                    slg_v4* varyings)
    {
        const UniformBuffer u{d.ubo};
        const VertexBuffer vb{d.vbo};
        const VertexArray va{t.vaos + d.vaoId};
        const Resources r{t};
        VertexParam p{&u, (size_t)vertId, (size_t)instanceId, &va, &vb, varyings, &r};
        return User::vertex(d.vsProgram, p);
    }

    static __device__ __forceinline__ bool fragment(const DrawDesc& d, const Tables& t, slg_frag_coord& coord, const slg_v4* varyings,
                                                    slg_v4* outputs)
    {
        const UniformBuffer u{d.ubo};
        const Resources r{t};
        FragmentParam p;
        p.coord = coord;
        p.pUniforms = &u;
        p.pResources = &r;
#pragma unroll
        for (int i = 0; i < kMaxVaryings; ++i) p.pVaryings[i] = varyings[i];
#pragma unroll
        for (int i = 0; i < 4; ++i) p.pOutputs[i] = slg_make_v4(0.f, 0.f, 0.f, 0.f);
        const bool kept = User::fragment(d.fsProgram, p);
#pragma unroll
        for (int i = 0; i < 4; ++i) outputs[i] = p.pOutputs[i];
        coord.depth = p.coord.depth;
        return kept;
    }
};

} // namespace slg

/* The raster stage of program set User for one colour format of attachment 0
 * (ColorRGBA8, ColorRGBAF or ColorRF), in a translation unit of its own. */
#define SLG_PROGRAMS_RASTER(User, Color) SLG_PIPELINE_RASTER(slg::CallerPrograms<User>, Color)

/* The vertex stage of program set User and its entry table
 *     extern "C" const slg_pipeline_ops* name(void)
 * with the raster stages compiled elsewhere (SLG_PROGRAMS_RASTER). */
#define SLG_PROGRAMS_ENTRY(User, name)                                                                \
    SLG_PIPELINE_EXTERN(slg::CallerPrograms<User>)                                                    \
    extern "C" const slg_pipeline_ops* name(void)                                                     \
    {                                                                                                 \
        static const slg_pipeline_ops ops = slg::PipelineEntry<slg::CallerPrograms<User>>::ops();     \
        return &ops;                                                                                  \
    }

/* All of program set User in one translation unit. */
#define SLG_DEFINE_PROGRAMS(User, name)                                                               \
    SLG_PROGRAMS_RASTER(User, ColorRGBA8)                                                             \
    SLG_PROGRAMS_RASTER(User, ColorRGBAF)                                                             \
    SLG_PROGRAMS_RASTER(User, ColorRF)                                                                \
    extern "C" const slg_pipeline_ops* name(void)                                                     \
    {                                                                                                 \
        static const slg_pipeline_ops ops = slg::PipelineEntry<slg::CallerPrograms<User>>::ops();     \
        return &ops;                                                                                  \
    }

#endif /* SLG_SHADER_CUH */
