// Stage kernels instantiated for the bf16 storage mode.
#include "rgdn_kernels.cuh"

namespace rgdn
{
cudaError_t launch_bloom_bf16( const BloomArgs& b, cudaStream_t s )
{
    return launch_bloom_t< MODE_BF16 >( b, s );
}
cudaError_t launch_final_bf16( const FinalArgs& f, cudaStream_t s )
{
    return launch_final_t< MODE_BF16 >( f, s );
}
cudaError_t launch_stage_bf16( const FrameArgs& a, int stage, int iter, cudaStream_t s )
{
    return launch_stage_t< MODE_BF16 >( a, stage, iter, s );
}
cudaError_t launch_batch_bf16( int stage, int iter, int slot, dim3 block, int grid, cudaStream_t s )
{
    return launch_batch_t< MODE_BF16 >( stage, iter, slot, block, grid, s );
}
void* batch_slot_bf16( int slot ) { return batch_slot_t( slot ); }
int batch_blocks_per_sm_bf16( int stage ) { return batch_blocks_per_sm_t< MODE_BF16 >( stage ); }
}  // namespace rgdn
