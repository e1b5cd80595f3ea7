// Stage kernels instantiated for the f32 storage mode.
#include "rgdn_kernels.cuh"

namespace rgdn
{
cudaError_t launch_bloom_f32( const BloomArgs& b, cudaStream_t s )
{
    return launch_bloom_t< MODE_F32 >( b, s );
}
cudaError_t launch_final_f32( const FinalArgs& f, cudaStream_t s )
{
    return launch_final_t< MODE_F32 >( f, s );
}
cudaError_t launch_stage_f32( const FrameArgs& a, int stage, int iter, cudaStream_t s )
{
    return launch_stage_t< MODE_F32 >( a, stage, iter, s );
}
cudaError_t launch_batch_f32( int stage, int iter, int slot, dim3 block, int grid, cudaStream_t s )
{
    return launch_batch_t< MODE_F32 >( stage, iter, slot, block, grid, s );
}
void* batch_slot_f32( int slot ) { return batch_slot_t( slot ); }
int batch_blocks_per_sm_f32( int stage ) { return batch_blocks_per_sm_t< MODE_F32 >( stage ); }
}  // namespace rgdn
