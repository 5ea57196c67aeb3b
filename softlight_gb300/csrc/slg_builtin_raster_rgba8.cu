/*
 * slg_builtin_raster_rgba8.cu - the built-in programs' raster stage for
 * colour attachment 0 in RGBA8 (order-free and ordered rasters at every tile
 * size, line-address fix-up).
 */
#include "slg_pipeline.cuh"

SLG_PIPELINE_RASTER(slg::BuiltinPrograms, ColorRGBA8)
