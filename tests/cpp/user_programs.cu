/*
 * user_programs.cu - a caller-defined program set, written as a SoftLight
 * user writes shaders (softlight/tests/sl_instancing_test.cpp:95-172): each
 * program reads its uniform block with pUniforms->as<T>(), its vertex with
 * pVbo->element<T>(pVao->offset(bind, vertId)), and its fragment position
 * from coord. Compiled four times (SLG_USER_PART 0..3: entry table and
 * vertex stage, then the raster stage for each colour format of attachment
 * 0) and linked into one shared library by tests/test_user_programs.py.
 *
 * Programs (ids from SLG_PROGRAM_USER_FIRST):
 *   256 vertex: position, colour, uv from one interleaved binding
 *       fragment: alpha test (vertex alpha x texel alpha < alphaRef discards)
 *   257 fragment: fragment coordinate as colour, screen-door discard,
 *       depth written as depth * scale + bias
 *   258 vertex: position from binding 0, colour from binding 1, uv from
 *       binding 2 of the same buffer (SL_VertexArray with three bindings)
 * The arithmetic is the built-in programs' (slg_fs_cutout,
 * slg_fs_frag_coord, slg_vs_vcolor), so the images must match theirs bit
 * for bit.
 */
#include "slg_shader.cuh"

namespace
{

struct CutoutUniforms      /* slg_cutout_uniforms */
{
    float    mvpMatrix[16];
    uint32_t textureId;
    float    alphaRef;
    uint32_t pad[2];
};

struct FragCoordUniforms   /* slg_fragcoord_uniforms */
{
    float    mvpMatrix[16];
    float    invSize[2];
    float    depthScale;
    float    depthBias;
    uint32_t screenDoor;
    uint32_t pad[3];
};

struct Vertex
{
    float pos[3];
    float rgba[4];
    float uv[2];
};

__device__ slg::vec4 interleaved_vert_shader(slg::VertexParam& param)
{
    const CutoutUniforms* u = param.pUniforms->as<CutoutUniforms>();
    const Vertex* v = param.pVbo->element<const Vertex>(param.pVao->offset(0, param.vertId));
    param.pVaryings[0] = slg_make_v4(v->rgba[0], v->rgba[1], v->rgba[2], v->rgba[3]);
    param.pVaryings[1] = slg_make_v4(v->uv[0], v->uv[1], 0.f, 0.f);
    return slg_mat_mul_v4(u->mvpMatrix, slg_make_v4(v->pos[0], v->pos[1], v->pos[2], 1.f));
}

__device__ slg::vec4 split_bindings_vert_shader(slg::VertexParam& param)
{
    const CutoutUniforms* u = param.pUniforms->as<CutoutUniforms>();
    const float* pos = param.pVbo->element<const float>(param.pVao->offset(0, param.vertId));
    const float* rgba = param.pVbo->element<const float>(param.pVao->offset(1, param.vertId));
    const float* uv = param.pVbo->element<const float>(param.pVao->offset(2, param.vertId));
    param.pVaryings[0] = slg_make_v4(rgba[0], rgba[1], rgba[2], rgba[3]);
    param.pVaryings[1] = slg_make_v4(uv[0], uv[1], 0.f, 0.f);
    return slg_mat_mul_v4(u->mvpMatrix, slg_make_v4(pos[0], pos[1], pos[2], 1.f));
}

__device__ bool cutout_frag_shader(slg::FragmentParam& fragParam)
{
    const CutoutUniforms* u = fragParam.pUniforms->as<CutoutUniforms>();
    const slg::vec4 c = fragParam.pVaryings[0];
    const slg::vec4 t = fragParam.pResources->sample_rgba8(u->textureId, fragParam.pVaryings[1].x, fragParam.pVaryings[1].y);
    const float a = c.w * t.w;
    if (a < u->alphaRef)
    {
        return false;
    }
    fragParam.pOutputs[0] = slg_make_v4(c.x * t.x, c.y * t.y, c.z * t.z, a);
    return true;
}

__device__ bool frag_coord_shader(slg::FragmentParam& fragParam)
{
    const FragCoordUniforms* u = fragParam.pUniforms->as<FragCoordUniforms>();
    const uint32_t x = fragParam.coord.x, y = fragParam.coord.y;
    if (u->screenDoor != 0u && ((x ^ y) & u->screenDoor) == 0u)
    {
        return false;
    }
    const float depth = fragParam.coord.depth;
    fragParam.pOutputs[0] = slg_make_v4((float)x * u->invSize[0], (float)y * u->invSize[1], depth, fragParam.pVaryings[0].w);
    fragParam.coord.depth = depth * u->depthScale + u->depthBias;
    return true;
}

} // namespace

struct TestPrograms
{
    static __device__ __forceinline__ slg::vec4 vertex(uint32_t program, slg::VertexParam& p)
    {
        return (program == 258u) ? split_bindings_vert_shader(p) : interleaved_vert_shader(p);
    }
    static __device__ __forceinline__ bool fragment(uint32_t program, slg::FragmentParam& p)
    {
        return (program == 257u) ? frag_coord_shader(p) : cutout_frag_shader(p);
    }
};

#if SLG_USER_PART == 0
SLG_PROGRAMS_ENTRY(TestPrograms, slg_test_user_programs)
#elif SLG_USER_PART == 1
SLG_PROGRAMS_RASTER(TestPrograms, ColorRGBA8)
#elif SLG_USER_PART == 2
SLG_PROGRAMS_RASTER(TestPrograms, ColorRGBAF)
#else
SLG_PROGRAMS_RASTER(TestPrograms, ColorRF)
#endif
