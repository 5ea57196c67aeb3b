/*
 * slg_adjoint.cuh - launchers of the differentiable-render kernels
 * (slg_adjoint.cu): the shading model of one opaque vertex-colour x float
 * texture draw over the visibility the exact rasteriser recorded, its image
 * and its adjoint.
 */
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace slg
{

struct DiffArgs
{
    /* geometry: vertex k of triangle t is element elementBegin + 3t + k */
    const uint8_t* vbo;
    int64_t b0Offset, b0Stride;     /* bytes; pos[3], rgba[4], uv[2] floats at the binding */
    const uint8_t* ibo;             /* null when not indexed */
    int32_t indexType;              /* slg_data_type of the indices, -1: none */
    uint64_t elementBegin;
    uint32_t numTris;
    const float* mvp;               /* column-major 4x4 in the uniform block */

    /* texture: RGBA float texels, w*h of them followed by >= w + 64 zero texels */
    const float4* texels;
    uint32_t texW, texH;

    /* framebuffer */
    const uint32_t* vis;            /* per pixel: 0, or 1 + the visible triangle */
    const float4* exact;            /* RGBA float colour attachment, or null */
    int32_t width, height;

    /* outputs */
    float4* image;                  /* forward: model image (w x h) */
    const float4* dImage;           /* adjoint: dL/d image (w x h) */
    float* dVertices;               /* adjoint: += gradients in the vertex buffer's layout */
    float4* dTexels;                /* adjoint: += gradients, texW * texH */
};

cudaError_t launch_diff_shade(const DiffArgs& a, cudaStream_t s);
cudaError_t launch_diff_adjoint(const DiffArgs& a, cudaStream_t s);

} // namespace slg
