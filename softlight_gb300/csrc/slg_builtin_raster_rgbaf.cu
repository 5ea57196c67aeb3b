/*
 * slg_builtin_raster_rgbaf.cu - the built-in programs' raster stage for
 * colour attachment 0 in RGBA float (order-free and ordered rasters at every tile
 * size, line-address fix-up).
 */
#include "slg_pipeline.cuh"

SLG_PIPELINE_RASTER(slg::BuiltinPrograms, ColorRGBAF)
