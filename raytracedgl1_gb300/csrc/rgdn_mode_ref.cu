// Stage kernels instantiated for the ref storage mode.
#include "rgdn_kernels.cuh"

namespace rgdn
{
cudaError_t launch_bloom_ref( const BloomArgs& b, cudaStream_t s )
{
    return launch_bloom_t< MODE_REF >( b, s );
}
cudaError_t launch_final_ref( const FinalArgs& f, cudaStream_t s )
{
    return launch_final_t< MODE_REF >( f, s );
}
cudaError_t launch_stage_ref( const FrameArgs& a, int stage, int iter, cudaStream_t s )
{
    return launch_stage_t< MODE_REF >( a, stage, iter, s );
}
cudaError_t launch_batch_ref( int stage, int iter, int slot, dim3 block, int grid, cudaStream_t s )
{
    return launch_batch_t< MODE_REF >( stage, iter, slot, block, grid, s );
}
void* batch_slot_ref( int slot ) { return batch_slot_t( slot ); }
int batch_blocks_per_sm_ref( int stage ) { return batch_blocks_per_sm_t< MODE_REF >( stage ); }
}  // namespace rgdn
