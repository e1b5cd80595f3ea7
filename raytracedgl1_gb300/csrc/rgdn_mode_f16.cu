// Stage kernels instantiated for the f16 storage mode.
#include "rgdn_kernels.cuh"

namespace rgdn
{
cudaError_t launch_stage_f16( const FrameArgs& a, int stage, int iter, cudaStream_t s )
{
    return launch_stage_t< MODE_F16 >( a, stage, iter, s );
}
}  // namespace rgdn
