// Stage kernels instantiated for the f32 storage mode.
#include "rgdn_kernels.cuh"

namespace rgdn
{
cudaError_t launch_stage_f32( const FrameArgs& a, int stage, int iter, cudaStream_t s )
{
    return launch_stage_t< MODE_F32 >( a, stage, iter, s );
}
}  // namespace rgdn
