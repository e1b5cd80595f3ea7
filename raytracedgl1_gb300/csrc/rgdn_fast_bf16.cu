// FAST kernels (continuous arithmetic only: the a-trous weights and the variance) for the bf16
// storage mode, in their own translation unit.
#include "rgdn_kernels.cuh"

namespace rgdn
{
cudaError_t launch_fast_bf16( const FrameArgs& a, int stage, int iter, cudaStream_t s )
{
    return launch_fast_t< MODE_BF16 >( a, stage, iter, s );
}
cudaError_t launch_batch_fast_bf16( int stage, int iter, int slot, dim3 block, int grid, cudaStream_t s )
{
    return launch_batch_fast_t< MODE_BF16 >( stage, iter, slot, block, grid, s );
}
void* batch_slot_fast_bf16( int slot ) { return batch_slot_t( slot ); }
int batch_blocks_per_sm_fast_bf16( int stage ) { return batch_blocks_per_sm_fast_t< MODE_BF16 >( stage ); }
cudaError_t launch_atrous_tma_bf16( const FrameArgs& a, int iter, bool hist, const void* maps, cudaStream_t s )
{
    return launch_atrous_tma_t< MODE_BF16 >( a, iter, hist, maps, s );
}
}  // namespace rgdn
