// rgdn_gradient_atrous_noalloc: the four gradient a-trous iterations for callers that are not
// allowed to allocate device memory.
//
// Who needs it: code that runs where a device allocation is forbidden or harmful —
// inside a host application that hands every plug-in a fixed memory budget and owns all
// allocations itself, or in a real-time frame loop where cudaMalloc / cudaFree would stall
// the device (they synchronise) and break a frame's timing. Such a caller already holds its
// gradient images; this entry point needs nothing else from it.
//
// Where the scratch lives: the iterations ping-pong through one intermediate image. Here that
// image is a file-scope __device__ array of fixed capacity (kMaxStrata rgba8 texels, 3.5 MiB),
// which every GPU that loads the library holds until the process exits. Host code cannot
// use the array's name as a device address (in host code it names a host-side shadow), so
// the address is taken with cudaGetSymbolAddress, with the device current, and passed to the
// kernel. It is looked up once per CUDA context: a context that is not the device's primary
// one, or the primary context created again after cudaDeviceReset, loads the module anew and
// may place the array elsewhere, so the cached address is keyed by the context handle.
#include <mutex>

#include "rgdn_kernels.cuh"

namespace
{

// One rgba8 texel per stratum: enough for a 3840x2160 render (1280 x 720 strata).
constexpr int kMaxStrata = 1280 * 720;
static __device__ __align__( 256 ) uint32_t g_gradientScratch[ kMaxStrata ];

constexpr int kMaxDevices = 64;
// per device: the context the address was taken in, and the address
void*         g_scratchContext[ kMaxDevices ] = {};
void*         g_scratchAddress[ kMaxDevices ] = {};
std::mutex    g_setupMutex;

// cuCtxGetCurrent through the runtime's driver entry point (the library links only cudart)
typedef int ( *CtxGetCurrentFn )( void** ctx );
CtxGetCurrentFn ctx_get_current_fn()
{
    static CtxGetCurrentFn fn   = nullptr;
    static bool            done = false;
    if( !done )
    {
        void*                           p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if( cudaGetDriverEntryPointByVersion( "cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q ) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess )
            fn = (CtxGetCurrentFn)p;
        done = true;
    }
    return fn;
}

__global__ void __launch_bounds__( 256 ) k_gradient_atrous_noalloc( const uint32_t* src, uint32_t* dst, uint32_t* hist,
                                                                     const rgdn::Uniform u, const int iter )
{
    __shared__ float u8[ 256 ];
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
    u8[ t ]     = (float)t / 255.0f;
    __syncthreads();
    const int gx = blockIdx.x * blockDim.x + threadIdx.x;
    const int gy = blockIdx.y * blockDim.y + threadIdx.y;
    if( gx >= u.GW || gy >= u.GH || gx * rgdn::STRATA >= u.W || gy * rgdn::STRATA >= u.H ) return;
    rgdn::dev::gradient_atrous_core( u, src, dst, hist, gx, gy, iter, u8 );
}

}  // namespace

extern "C" rgdn_status rgdn_gradient_atrous_noalloc( const uint32_t* samples, uint32_t* filtered, uint32_t* history,
                                                     uint32_t renderWidth, uint32_t renderHeight, rgdn_cuda_stream cudaStream )
{
    if( !samples || !filtered || !history || renderWidth < 2 || renderHeight < 1 || ( renderWidth & 1 ) ||
        ( (uintptr_t)samples & 3 ) || ( (uintptr_t)filtered & 3 ) || ( (uintptr_t)history & 3 ) )
        return RGDN_WRONG_FUNCTION_ARGUMENT;
    // iteration 0 reads the neighbours of `samples` while it writes `history`, and the later
    // iterations write `filtered`: three distinct images, as the reference's DISPingGradient /
    // DISGradientHistory are
    if( (const void*)samples == (const void*)history || (const void*)filtered == (const void*)samples || filtered == history )
        return RGDN_WRONG_FUNCTION_ARGUMENT;
    const uint32_t gw = ( renderWidth + 1 ) / 3 > 0 ? ( renderWidth + 1 ) / 3 : 1;
    const uint32_t gh = ( renderHeight + 1 ) / 3 > 0 ? ( renderHeight + 1 ) / 3 : 1;
    // the fixed scratch holds kMaxStrata texels: larger frames are refused, not truncated
    if( (uint64_t)gw * gh > (uint64_t)kMaxStrata ) return RGDN_WRONG_FUNCTION_ARGUMENT;

    int dev = 0;
    if( cudaGetDevice( &dev ) != cudaSuccess || dev < 0 || dev >= kMaxDevices ) return RGDN_DEVICE_ERROR;
    const CtxGetCurrentFn getCtx = ctx_get_current_fn();
    void*                 ctx    = nullptr;
    if( !getCtx || getCtx( &ctx ) != 0 ) return RGDN_DEVICE_ERROR;
    void* scratch = nullptr;
    {
        // set-up, once per device and context, with that device current
        std::lock_guard< std::mutex > g( g_setupMutex );
        if( !ctx || !g_scratchAddress[ dev ] || g_scratchContext[ dev ] != ctx )
        {
            void* p = nullptr;
            if( cudaGetSymbolAddress( &p, g_gradientScratch ) != cudaSuccess || !p ) return RGDN_DEVICE_ERROR;
            // with no context current before, the runtime has now made the primary one current
            if( !ctx && ( getCtx( &ctx ) != 0 || !ctx ) ) return RGDN_DEVICE_ERROR;
            g_scratchAddress[ dev ] = p;
            g_scratchContext[ dev ] = ctx;
        }
        scratch = g_scratchAddress[ dev ];
    }

    rgdn::Uniform u;
    memset( &u, 0, sizeof( u ) );
    u.W  = (int)renderWidth;
    u.H  = (int)renderHeight;
    u.GW = (int)gw;
    u.GH = (int)gh;
    u.rw = (float)renderWidth;
    u.rh = (float)renderHeight;

    // the reference's routing Ping -> Pong(+history) -> Ping -> Pong -> Ping, with the
    // scratch in the Pong role and `filtered` in the Ping role (samples are only read)
    uint32_t*       tmp = (uint32_t*)scratch;
    const uint32_t* src[ 4 ] = { samples, tmp, filtered, tmp };
    uint32_t*       dst[ 4 ] = { tmp, filtered, tmp, filtered };
    const dim3      blk( 32, 8 );
    const dim3      grid( ( gw + 31 ) / 32, ( gh + 7 ) / 8 );
    for( int it = 0; it < 4; it++ )
    {
        k_gradient_atrous_noalloc<<< grid, blk, 0, (cudaStream_t)cudaStream >>>( src[ it ], dst[ it ], it == 0 ? history : nullptr, u, it );
        if( cudaGetLastError() != cudaSuccess ) return RGDN_DEVICE_ERROR;
    }
    return RGDN_SUCCESS;
}
