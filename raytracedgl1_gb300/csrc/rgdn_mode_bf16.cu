// Stage kernels instantiated for the bf16 storage mode.
#include "rgdn_kernels.cuh"

namespace rgdn
{
cudaError_t launch_stage_bf16( const FrameArgs& a, int stage, int iter, cudaStream_t s )
{
    return launch_stage_t< MODE_BF16 >( a, stage, iter, s );
}
}  // namespace rgdn
