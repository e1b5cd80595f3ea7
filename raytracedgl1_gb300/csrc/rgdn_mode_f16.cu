// Stage kernels instantiated for the f16 storage mode.
#include "rgdn_kernels.cuh"

namespace rgdn
{
cudaError_t launch_bloom_f16( const BloomArgs& b, cudaStream_t s )
{
    return launch_bloom_t< MODE_F16 >( b, s );
}
// the volumetric kernels read and write fixed formats: one instantiation serves every mode
cudaError_t launch_process_scattering( const ScatterArgs& a, cudaStream_t s )
{
    return launch_scatter_t< MODE_F16 >( a, s );
}
cudaError_t launch_final_f16( const FinalArgs& f, cudaStream_t s )
{
    return launch_final_t< MODE_F16 >( f, s );
}
cudaError_t launch_stage_f16( const FrameArgs& a, int stage, int iter, cudaStream_t s )
{
    return launch_stage_t< MODE_F16 >( a, stage, iter, s );
}
cudaError_t launch_batch_f16( int stage, int iter, int slot, dim3 block, int grid, cudaStream_t s )
{
    return launch_batch_t< MODE_F16 >( stage, iter, slot, block, grid, s );
}
void* batch_slot_f16( int slot ) { return batch_slot_t( slot ); }
int batch_blocks_per_sm_f16( int stage ) { return batch_blocks_per_sm_t< MODE_F16 >( stage ); }
}  // namespace rgdn
