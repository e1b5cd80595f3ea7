// Stage kernels instantiated for the ref storage mode.
#include "rgdn_kernels.cuh"

namespace rgdn
{
cudaError_t launch_stage_ref( const FrameArgs& a, int stage, int iter, cudaStream_t s )
{
    return launch_stage_t< MODE_REF >( a, stage, iter, s );
}
}  // namespace rgdn
