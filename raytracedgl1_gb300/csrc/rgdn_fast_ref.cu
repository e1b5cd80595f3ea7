// FAST kernels (continuous arithmetic only: the a-trous weights and the variance) for the ref
// storage mode, in their own translation unit.
#include "rgdn_kernels.cuh"

namespace rgdn
{
cudaError_t launch_fast_ref( const FrameArgs& a, int stage, int iter, cudaStream_t s )
{
    return launch_fast_t< MODE_REF >( a, stage, iter, s );
}
cudaError_t launch_batch_fast_ref( int stage, int iter, int slot, dim3 block, int grid, cudaStream_t s )
{
    return launch_batch_fast_t< MODE_REF >( stage, iter, slot, block, grid, s );
}
void* batch_slot_fast_ref( int slot ) { return batch_slot_t( slot ); }
int batch_blocks_per_sm_fast_ref( int stage ) { return batch_blocks_per_sm_fast_t< MODE_REF >( stage ); }
cudaError_t launch_atrous_tma_ref( const FrameArgs& a, int iter, bool hist, const void* maps, cudaStream_t s )
{
    return launch_atrous_tma_t< MODE_REF >( a, iter, hist, maps, s );
}
int atrous_tma_smem( int storage, int iter )
{
    switch( storage )
    {
        case MODE_REF: return atrous_tma_smem_t< MODE_REF >( iter );
        case MODE_F32: return atrous_tma_smem_t< MODE_F32 >( iter );
        case MODE_F16: return atrous_tma_smem_t< MODE_F16 >( iter );
        default: return atrous_tma_smem_t< MODE_BF16 >( iter );
    }
}
}  // namespace rgdn
