/*
 * slg_kernels.cuh - host-side entry points of the draw-path kernels.
 */
#ifndef SLG_KERNELS_CUH
#define SLG_KERNELS_CUH

#include <cuda_runtime.h>
#include "slg_device.cuh"

namespace slg
{

/* Enqueue vs_setup, tile_scan, bin_fill and raster for one launch on s.
 * When ev is not null, ev[0..4] are recorded before vs_setup, after
 * vs_setup, after tile_scan, after bin_fill and after raster. */
cudaError_t launch_pipeline(const Frame& f, int keyCap, cudaStream_t s, cudaEvent_t* ev);

/* Raises the dynamic shared-memory limits of the raster and sort kernels
 * once, so launches (and stream captures) need no attribute calls. */
cudaError_t init_kernel_attributes(int keyCap);

/* Fill numTexels texels of 4 or 16 bytes with value. */
cudaError_t launch_clear(uint8_t* dst, size_t numTexels, int bytesPerTexel, const uint32_t value[8], cudaStream_t s);

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
};
cudaError_t launch_blit(const BlitArgs& a, cudaStream_t s);

} // namespace slg

#endif /* SLG_KERNELS_CUH */
