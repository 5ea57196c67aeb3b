/*
 * slg_builtin_vertex.cu - the built-in programs' vertex stage (post-transform
 * vertex cache, vs_setup, clipping) and their entry table; their raster
 * stage is compiled per colour format in slg_builtin_raster_*.cu.
 */
#include "slg_pipeline.cuh"
#include "slg_kernels.cuh"

SLG_PIPELINE_EXTERN(slg::BuiltinPrograms)

namespace slg
{

const slg_pipeline_ops& builtin_pipeline()
{
    static const slg_pipeline_ops ops = PipelineEntry<BuiltinPrograms>::ops();
    return ops;
}

} // namespace slg
