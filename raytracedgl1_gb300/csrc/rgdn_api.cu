// C ABI of the denoise-and-expose path (include/rgdn.h): contexts, streams (one framebuffer
// set + history + tonemapping state each), stage sequencing and the tonemapping read-back.
//
// Host-side counterparts in the reference:
//   Denoiser::Denoise            Source/Denoiser.cpp:64-255 (stage order, iteration routing)
//   Tonemapping::CalculateExposure  Source/Tonemapping.cpp:59-165
//   Framebuffers                 Source/Framebuffers.cpp:34-49 (cur/_Prev by frameIndex),
//                                :640-699 (sizes, FORCE_SIZE_1_3 = (W+1)/3)
//   RgResult / Call<> wrapper    Source/RTGL1.cpp:145-195 (no exceptions cross the ABI)
#include <algorithm>
#include <cstddef>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <map>
#include <new>
#include <set>
#include <utility>
#include <vector>

#include <tuple>

#include "rgdn_codec.h"
#include "rgdn_host.h"

using namespace rgdn;

// the default path marks the frame's geometry record persisting in L2 (kGeomBothSlots: both
// frame slots' records, so the temporal pass's previous-frame taps hit as well), with up to
// kL2PersistMB of L2 set aside. On GB300 at 1080p: 0.5065 ms per frame with 48 MB and the
// current slot, 0.5068 with 34 MB, 0.5786 with 80 MB and both slots (too little L2 left for the
// passes' other planes), 0.517 without the window.
constexpr bool   kGeomL2Persist = true;
constexpr bool   kGeomBothSlots = false;
constexpr size_t kL2PersistMB   = 48;

namespace
{
// cuTensorMapEncodeTiled through the runtime's driver entry point (no libcuda link)
typedef CUresult ( *EncodeTiledFn )( CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*, const cuuint64_t*,
                                     const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                     CUtensorMapL2promotion, CUtensorMapFloatOOBfill );
EncodeTiledFn encode_tiled_fn()
{
    static EncodeTiledFn fn   = nullptr;
    static bool          done = false;
    if( !done )
    {
        void*                           p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if( cudaGetDriverEntryPointByVersion( "cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q ) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess )
            fn = (EncodeTiledFn)p;
        done = true;
    }
    return fn;
}

// The temporal pass's history-length decay pow(1 - g, 10) (CmSVGFTemporalAccumulation.comp:
// 339, 356) for the 256 unorm8 gradient values g = k / 255: the expression the exact kernels
// evaluate inline, in the same FP32 operations, so the fast kernels read the same bits.
__global__ void k_fill_decay( float* t )
{
    const int   k = threadIdx.x;
    const float g = (float)k / 255.0f;
    t[ k ]        = powf( 1.0f - g, 10.0f );
}
cudaError_t fill_decay_table( float* t )
{
    k_fill_decay<<< 1, 256 >>>( t );
    const cudaError_t e = cudaGetLastError();
    return e != cudaSuccess ? e : cudaDeviceSynchronize();
}
}  // namespace

namespace
{

struct FbDesc
{
    uint32_t format;
    bool     prev;
    bool     third;
    int      shift = 0;   // bloom mips: ((W+1) >> shift) x ((H+1) >> shift), at least 1
    uint32_t fixedW = 0, fixedH = 0;   // a size independent of the render size (the froxel volume)
};

uint32_t format_bytes( uint32_t f )
{
    switch( f )
    {
        case RGDN_FORMAT_R8_UINT: return 1;
        case RGDN_FORMAT_RG8_UNORM: case RGDN_FORMAT_R16_SFLOAT: return 2;
        case RGDN_FORMAT_RGBA8_UNORM: case RGDN_FORMAT_RG16_SFLOAT: case RGDN_FORMAT_R32_SFLOAT:
        case RGDN_FORMAT_R32_UINT: case RGDN_FORMAT_E5B9G9R9_UFLOAT: case RGDN_FORMAT_B10G11R11_UFLOAT:
        case RGDN_FORMAT_NORMAL_SPHERICAL: return 4;
        case RGDN_FORMAT_RGBA16_SFLOAT: case RGDN_FORMAT_RGBA16_BFLOAT: case RGDN_FORMAT_RG32_SFLOAT: return 8;
        case RGDN_FORMAT_RGBA32_SFLOAT: case RGDN_FORMAT_RGBA32_UINT: return 16;
        default: return 0;
    }
}

// Formats of every image per storage mode. REF is the reference's table
// (GenerateShaderCommon.py:802-887); the other modes change only colour / history images.
FbDesc fb_desc( uint32_t fb, uint32_t storage )
{
    const uint32_t col3 = storage == RGDN_STORAGE_REF ? RGDN_FORMAT_E5B9G9R9_UFLOAT
                        : storage == RGDN_STORAGE_FP32 ? RGDN_FORMAT_RGBA32_SFLOAT
                        : storage == RGDN_STORAGE_FP16 ? RGDN_FORMAT_RGBA16_SFLOAT
                                                       : RGDN_FORMAT_RGBA16_BFLOAT;
    const uint32_t colvar = storage == RGDN_STORAGE_REF ? RGDN_FORMAT_RGBA16_SFLOAT : col3;
    const uint32_t mom    = storage == RGDN_STORAGE_REF ? RGDN_FORMAT_RG16_SFLOAT : RGDN_FORMAT_RG32_SFLOAT;
    const uint32_t fvar   = storage == RGDN_STORAGE_REF ? RGDN_FORMAT_R16_SFLOAT : RGDN_FORMAT_R32_SFLOAT;
    const uint32_t pre    = storage == RGDN_STORAGE_REF ? RGDN_FORMAT_B10G11R11_UFLOAT
                          : storage == RGDN_STORAGE_FP32 ? RGDN_FORMAT_RGBA32_SFLOAT
                                                         : RGDN_FORMAT_RGBA16_SFLOAT;
    const uint32_t varpl  = ( storage == RGDN_STORAGE_FP16 || storage == RGDN_STORAGE_BF16 ) ? RGDN_FORMAT_R32_SFLOAT : RGDN_FORMAT_NONE;
    switch( fb )
    {
        case RGDN_FB_ALBEDO: return { RGDN_FORMAT_B10G11R11_UFLOAT, false, false };
        case RGDN_FB_IS_SKY: return { RGDN_FORMAT_R8_UINT, false, false };
        case RGDN_FB_NORMAL: return { RGDN_FORMAT_NORMAL_SPHERICAL, true, false };
        case RGDN_FB_METALLIC_ROUGHNESS: return { RGDN_FORMAT_RG8_UNORM, true, false };
        case RGDN_FB_DEPTH_WORLD: return { RGDN_FORMAT_R16_SFLOAT, true, false };
        case RGDN_FB_DEPTH_GRAD: return { RGDN_FORMAT_R16_SFLOAT, false, false };
        case RGDN_FB_MOTION: return { RGDN_FORMAT_RGBA16_SFLOAT, false, false };
        case RGDN_FB_UNFILTERED_DIRECT:
        case RGDN_FB_UNFILTERED_SPECULAR:
        case RGDN_FB_UNFILTERED_INDIR: return { RGDN_FORMAT_E5B9G9R9_UFLOAT, false, false };
        case RGDN_FB_SURFACE_POSITION: return { RGDN_FORMAT_RGBA32_SFLOAT, true, false };
        case RGDN_FB_VIEW_DIRECTION: return { RGDN_FORMAT_RGBA16_SFLOAT, false, false };
        case RGDN_FB_THROUGHPUT: return { RGDN_FORMAT_RGBA16_SFLOAT, false, false };
        case RGDN_FB_GRADIENT_INPUTS: return { RGDN_FORMAT_RG16_SFLOAT, true, false };
        case RGDN_FB_GRADIENT_RESHADED: return { RGDN_FORMAT_RG32_SFLOAT, false, false };
        case RGDN_FB_PRE_FINAL: return { pre, false, false };
        case RGDN_FB_HISTOGRAM_INPUT: return { RGDN_FORMAT_R16_SFLOAT, false, false };
        case RGDN_FB_ACCUM_HISTORY_LENGTH: return { colvar, true, false };
        case RGDN_FB_DIFF_TEMPORARY: return { col3, false, false };
        case RGDN_FB_DIFF_ACCUM_COLOR: return { col3, true, false };
        case RGDN_FB_DIFF_ACCUM_MOMENTS: return { mom, true, false };
        case RGDN_FB_DIFF_COLOR_HISTORY:
        case RGDN_FB_DIFF_PING_COLOR_AND_VARIANCE:
        case RGDN_FB_DIFF_PONG_COLOR_AND_VARIANCE: return { colvar, false, false };
        case RGDN_FB_SPEC_ACCUM_COLOR: return { col3, true, false };
        case RGDN_FB_SPEC_PING_COLOR:
        case RGDN_FB_SPEC_PONG_COLOR: return { col3, false, false };
        case RGDN_FB_INDIR_ACCUM: return { col3, true, false };
        case RGDN_FB_INDIR_PING:
        case RGDN_FB_INDIR_PONG: return { col3, false, false };
        case RGDN_FB_ATROUS_FILTERED_VARIANCE: return { fvar, false, false };
        case RGDN_FB_DIS_PING_GRADIENT:
        case RGDN_FB_DIS_PONG_GRADIENT: return { RGDN_FORMAT_RGBA8_UNORM, false, true };
        case RGDN_FB_DIS_GRADIENT_HISTORY: return { RGDN_FORMAT_RGBA8_UNORM, true, true };
        case RGDN_FB_GRADIENT_PREV_PIX: return { RGDN_FORMAT_R8_UINT, false, true };
        case RGDN_FB_DIFF_COLOR_HISTORY_VARIANCE:
        case RGDN_FB_DIFF_PING_VARIANCE:
        case RGDN_FB_DIFF_PONG_VARIANCE: return { varpl, false, false };
        case RGDN_FB_SCREEN_EMIS_RT: return { RGDN_FORMAT_B10G11R11_UFLOAT, false, false };
        case RGDN_FB_SCATTERING: return { RGDN_FORMAT_RGBA16_SFLOAT, true, false };
        case RGDN_FB_DEPTH_NDC: return { RGDN_FORMAT_R32_SFLOAT, false, false };
        case RGDN_FB_SCATTERING_HISTORY: return { RGDN_FORMAT_R16_SFLOAT, true, false };
        case RGDN_FB_SCATTER_VOLUME:
            return { RGDN_FORMAT_RGBA16_SFLOAT, true, false, 0, RGDN_VOLUME_SIZE_X, RGDN_VOLUME_SIZE_Y * RGDN_VOLUME_SIZE_Z };
        case RGDN_FB_FINAL:
        case RGDN_FB_BLOOM_INPUT:
        case RGDN_FB_BLOOM_RESULT: return { pre, false, false };
        case RGDN_FB_RESERVOIRS: return { RGDN_FORMAT_RGBA32_UINT, true, false };
        case RGDN_FB_BLOOM_MIP1: case RGDN_FB_BLOOM_MIP2: case RGDN_FB_BLOOM_MIP3: case RGDN_FB_BLOOM_MIP4:
        case RGDN_FB_BLOOM_MIP5: case RGDN_FB_BLOOM_MIP6: case RGDN_FB_BLOOM_MIP7: case RGDN_FB_BLOOM_MIP8:
            return { pre, false, false, (int)( fb - RGDN_FB_BLOOM_MIP1 ) + 1 };
        default: return { RGDN_FORMAT_NONE, false, false };
    }
}

constexpr size_t kAlign = 256;
inline size_t align_up( size_t v ) { return ( v + kAlign - 1 ) & ~( kAlign - 1 ); }

StageLauncher launcher_for( uint32_t storage, int stage )
{
    const bool fast = is_fast_kernel( stage );
    switch( storage )
    {
        case RGDN_STORAGE_REF: return fast ? launch_fast_ref : launch_stage_ref;
        case RGDN_STORAGE_FP32: return fast ? launch_fast_f32 : launch_stage_f32;
        case RGDN_STORAGE_FP16: return fast ? launch_fast_f16 : launch_stage_f16;
        case RGDN_STORAGE_BF16: return fast ? launch_fast_bf16 : launch_stage_bf16;
        default: return nullptr;
    }
}

// getColorBin of CmLuminanceHistogram.comp:41-54, evaluated on the host in FP32 for every
// fp16 bit pattern; the GPU histogram indexes this table with the fp16 bits it bins.
void build_bin_lut( uint8_t* lut, float minLog, float maxLog )
{
    const float inv = 1.0f / ( maxLog - minLog );
    for( uint32_t h = 0; h < 65536u; h++ )
    {
        const float lum = rgdn::f16_to_f32( (uint16_t)h );
        uint32_t    bin;
        if( lum < 0.001f ) bin = 0;
        else
        {
            const float ll = fminf( fmaxf( ( log2f( lum ) - minLog ) * inv, 0.0f ), 1.0f );
            bin            = (uint32_t)( ll * 254.0f + 1.0f );
        }
        lut[ h ] = (uint8_t)bin;
    }
}

}  // namespace

namespace rgdn
{


// bytes of one stream's single device block
size_t stream_layout( uint32_t W, uint32_t H, uint32_t storage, PlaneSlot* planes, uint8_t* base )
{
    const uint32_t GW = std::max( 1u, ( W + 1 ) / 3 ), GH = std::max( 1u, ( H + 1 ) / 3 );
    size_t off = 0;
    // tonemapping state, re-shade scene, histogram bin table, geometry records of the default
    // path (2 slots)
    off += align_up( sizeof( Tonemapping ) );
    off += align_up( sizeof( rgdn_reshade_scene ) );
    off += align_up( 65536 );
    off += 2 * align_up( (size_t)W * H * 16 );
    for( uint32_t fb = 0; fb < RGDN_FB_COUNT; fb++ )
    {
        FbDesc   d     = fb_desc( fb, storage );
        uint32_t texel = format_bytes( d.format );
        if( planes ) planes[ fb ] = PlaneSlot();
        if( d.format == RGDN_FORMAT_NONE ) continue;
        uint32_t w = d.third ? GW : W, h = d.third ? GH : H;
        if( d.shift ) w = std::max( 1u, ( W + 1 ) >> d.shift ), h = std::max( 1u, ( H + 1 ) >> d.shift );
        if( d.fixedW ) w = d.fixedW, h = d.fixedH;
        size_t   sz = (size_t)w * h * texel;
        for( int s = 0; s < ( d.prev ? 2 : 1 ); s++ )
        {
            if( planes ) planes[ fb ].ptr[ s ] = planes[ fb ].own[ s ] = base ? base + off : nullptr;
            off += align_up( sz );
        }
        if( planes )
        {
            planes[ fb ].w = w; planes[ fb ].h = h; planes[ fb ].texel = texel;
            planes[ fb ].format = d.format; planes[ fb ].prev = d.prev;
        }
    }
    return off;
}

const uint8_t* plane_ptr( const rgdn_stream* s, uint32_t fb, uint32_t fi )
{
    const PlaneSlot& p = s->planes[ fb ];
    return p.prev ? p.ptr[ fi & 1 ] : p.ptr[ 0 ];
}
uint8_t* plane_ptr_mut( rgdn_stream* s, uint32_t fb, uint32_t fi )
{
    PlaneSlot& p = s->planes[ fb ];
    return p.prev ? p.ptr[ fi & 1 ] : p.ptr[ 0 ];
}

rgdn_status check_params( const rgdn_frame_params* p )
{
    if( !p ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    uint32_t n = p->atrousIterations == 0 ? 4u : p->atrousIterations;
    if( n < 1 || n > (uint32_t)MAX_ATROUS_ITERATIONS ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    if( !( p->maxLogLuminance > p->minLogLuminance ) ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    return RGDN_SUCCESS;
}

void fill_args( rgdn_stream* s, uint32_t fi, const rgdn_frame_params* p, FrameArgs& a )
{
    memset( &a, 0, sizeof( a ) );
    Uniform& u = a.u;
    u.W = (int)s->W; u.H = (int)s->H; u.GW = (int)s->GW; u.GH = (int)s->GH;
    u.rw = (float)s->W; u.rh = (float)s->H;
    u.isx = 1.0f / ( u.rw / 2.0f );
    u.isy = 1.0f / u.rh;
    // proj * view, column-major, for the FAST virtual-motion reprojection
    for( int c = 0; c < 4; c++ )
        for( int r = 0; r < 4; r++ )
        {
            double v = 0.0, vPrev = 0.0;
            for( int k = 0; k < 4; k++ )
            {
                v += (double)p->projection[ k * 4 + r ] * (double)p->view[ c * 4 + k ];
                vPrev += (double)p->projectionPrev[ k * 4 + r ] * (double)p->viewPrev[ c * 4 + k ];
            }
            u.vp[ c * 4 + r ]     = (float)v;
            u.vpPrev[ c * 4 + r ] = (float)vPrev;
        }
    memcpy( u.view, p->view, sizeof( u.view ) );
    memcpy( u.viewPrev, p->viewPrev, sizeof( u.viewPrev ) );
    memcpy( u.proj, p->projection, sizeof( u.proj ) );
    memcpy( u.projPrev, p->projectionPrev, sizeof( u.projPrev ) );
    memcpy( u.camPos, p->cameraPosition, sizeof( u.camPos ) );
    memcpy( u.camPosPrev, p->cameraPositionPrev, sizeof( u.camPosPrev ) );
    u.timeDelta         = p->timeDelta;
    u.minLog            = p->minLogLuminance;
    u.maxLog            = p->maxLogLuminance;
    u.stopEyeAdaptation = p->stopEyeAdaptation;
    u.gradMultD         = p->gradientMultDiffuse;
    u.gradMultI         = p->gradientMultIndirect;
    u.gradMultS         = p->gradientMultSpecular;
    u.antiFirefly       = p->antiFireflyEnabled;
    u.lightmapCoverage  = p->lightmapScreenCoverage;
    u.debugFlags        = p->debugShowFlags;
    u.niter             = p->atrousIterations == 0 ? 4u : p->atrousIterations;
    u.flags             = p->flags;
    u.frameId           = p->frameId;

    const uint32_t pf = fi ^ 1u;
#define CUR( fb ) ( (void*)plane_ptr_mut( s, fb, fi ) )
#define PRV( fb ) ( (const void*)plane_ptr( s, fb, pf ) )
    a.albedo         = (const uint32_t*)CUR( RGDN_FB_ALBEDO );
    a.isSky          = (const uint8_t*)CUR( RGDN_FB_IS_SKY );
    a.normal         = (const uint32_t*)CUR( RGDN_FB_NORMAL );
    a.normalPrev     = (const uint32_t*)PRV( RGDN_FB_NORMAL );
    a.mr             = (const uint16_t*)CUR( RGDN_FB_METALLIC_ROUGHNESS );
    a.depth          = (const uint16_t*)CUR( RGDN_FB_DEPTH_WORLD );
    a.depthPrev      = (const uint16_t*)PRV( RGDN_FB_DEPTH_WORLD );
    a.depthGrad      = (const uint16_t*)CUR( RGDN_FB_DEPTH_GRAD );
    a.motion         = (const ushort4*)CUR( RGDN_FB_MOTION );
    a.unfD           = (const uint32_t*)CUR( RGDN_FB_UNFILTERED_DIRECT );
    a.unfS           = (const uint32_t*)CUR( RGDN_FB_UNFILTERED_SPECULAR );
    a.unfI           = (const uint32_t*)CUR( RGDN_FB_UNFILTERED_INDIR );
    a.surfPos        = (const float4*)CUR( RGDN_FB_SURFACE_POSITION );
    a.surfPosPrev    = (const float4*)PRV( RGDN_FB_SURFACE_POSITION );
    a.viewDir        = (const ushort4*)CUR( RGDN_FB_VIEW_DIRECTION );
    a.throughput     = (const ushort4*)CUR( RGDN_FB_THROUGHPUT );
    a.gradInputsPrev = (const uint32_t*)PRV( RGDN_FB_GRADIENT_INPUTS );
    a.reshaded       = (const float2*)CUR( RGDN_FB_GRADIENT_RESHADED );
    a.rs             = s->rsSet ? s->rsDev : nullptr;
    a.reservoirsPrev = (const uint4*)PRV( RGDN_FB_RESERVOIRS );
    a.mrPrev         = (const uint16_t*)PRV( RGDN_FB_METALLIC_ROUGHNESS );
    a.preFinal       = CUR( RGDN_FB_PRE_FINAL );
    a.histInput      = (uint16_t*)CUR( RGDN_FB_HISTOGRAM_INPUT );
    a.histLen        = CUR( RGDN_FB_ACCUM_HISTORY_LENGTH );
    a.histLenPrev    = PRV( RGDN_FB_ACCUM_HISTORY_LENGTH );
    a.diffTemp       = CUR( RGDN_FB_DIFF_TEMPORARY );
    a.diffAccumColor = CUR( RGDN_FB_DIFF_ACCUM_COLOR );
    a.moments        = CUR( RGDN_FB_DIFF_ACCUM_MOMENTS );
    a.momentsPrev    = PRV( RGDN_FB_DIFF_ACCUM_MOMENTS );
    a.diffHistory    = CUR( RGDN_FB_DIFF_COLOR_HISTORY );
    a.diffPing       = CUR( RGDN_FB_DIFF_PING_COLOR_AND_VARIANCE );
    a.diffPong       = CUR( RGDN_FB_DIFF_PONG_COLOR_AND_VARIANCE );
    a.varHistory     = (float*)CUR( RGDN_FB_DIFF_COLOR_HISTORY_VARIANCE );
    a.varPing        = (float*)CUR( RGDN_FB_DIFF_PING_VARIANCE );
    a.varPong        = (float*)CUR( RGDN_FB_DIFF_PONG_VARIANCE );
    a.specAccum      = CUR( RGDN_FB_SPEC_ACCUM_COLOR );
    a.specAccumPrev  = PRV( RGDN_FB_SPEC_ACCUM_COLOR );
    a.specPing       = CUR( RGDN_FB_SPEC_PING_COLOR );
    a.specPong       = CUR( RGDN_FB_SPEC_PONG_COLOR );
    a.indirAccum     = CUR( RGDN_FB_INDIR_ACCUM );
    a.indirAccumPrev = PRV( RGDN_FB_INDIR_ACCUM );
    a.indirPing      = CUR( RGDN_FB_INDIR_PING );
    a.indirPong      = CUR( RGDN_FB_INDIR_PONG );
    a.filtVar        = CUR( RGDN_FB_ATROUS_FILTERED_VARIANCE );
    a.disPing        = (uint32_t*)CUR( RGDN_FB_DIS_PING_GRADIENT );
    a.disPong        = (uint32_t*)CUR( RGDN_FB_DIS_PONG_GRADIENT );
    a.disHist        = (uint32_t*)CUR( RGDN_FB_DIS_GRADIENT_HISTORY );
    a.disHistPrev    = (const uint32_t*)PRV( RGDN_FB_DIS_GRADIENT_HISTORY );
    a.gradPrevPix    = (uint8_t*)CUR( RGDN_FB_GRADIENT_PREV_PIX );
#undef CUR
#undef PRV
    a.tm       = s->tm;
    a.geom     = s->geom[ fi & 1 ];
    a.geomPrev = s->geom[ ( fi & 1 ) ^ 1 ];
    a.binLut   = s->binLut;
    a.phiTab   = s->ctx->phiTab;
    a.thetaTab = s->ctx->thetaTab;
    a.decay10  = s->ctx->decayTab;
}

cudaEvent_t take_event( rgdn_stream* s )
{
    if( !s->eventPool.empty() )
    {
        cudaEvent_t e = s->eventPool.back();
        s->eventPool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if( cudaEventCreate( &e ) != cudaSuccess ) return nullptr;
    return e;
}

rgdn_status launch( rgdn_stream* s, const FrameArgs& a, int stage, int iter, cudaStream_t cs )
{
    // the plain temporal pass does not write the geometry record of its slot
    if( stage == RGDN_STAGE_TEMPORAL_ACCUMULATION ) s->geomValid[ a.geom == s->geom[ 0 ] ? 0 : 1 ] = false;
    StageLauncher L = launcher_for( s->storage, stage );
    if( !L ) return RGDN_INTERNAL_ERROR;
    cudaEvent_t ea = nullptr, eb = nullptr;
    if( s->timing )
    {
        ea = take_event( s );
        eb = take_event( s );
        if( !ea || !eb ) return RGDN_DEVICE_ERROR;
        cudaEventRecord( ea, cs );
    }
    cudaError_t e = L( a, stage, iter, cs );
    s->ctx->launches.fetch_add( 1, std::memory_order_relaxed );
    if( s->timing )
    {
        cudaEventRecord( eb, cs );
        s->pending.push_back( { stage, iter, ea, eb } );
    }
    return cuda_status( e );
}

// the histogram bin table follows the frame's luminance range
rgdn_status ensure_bin_lut( rgdn_stream* s, const rgdn_frame_params* p, cudaStream_t cs )
{
    if( s->lutMin == p->minLogLuminance && s->lutMax == p->maxLogLuminance ) return RGDN_SUCCESS;
    s->hostLut.resize( 65536 );
    build_bin_lut( s->hostLut.data(), p->minLogLuminance, p->maxLogLuminance );
    // pageable source: the call returns once the bytes are staged, so hostLut may change later
    cudaError_t e = cudaMemcpyAsync( s->binLut, s->hostLut.data(), 65536, cudaMemcpyHostToDevice, cs );
    if( e != cudaSuccess ) return RGDN_DEVICE_ERROR;
    s->lutMin = p->minLogLuminance;
    s->lutMax = p->maxLogLuminance;
    return RGDN_SUCCESS;
}

rgdn_status run_denoise_fused( rgdn_stream* s, uint32_t fi, const rgdn_frame_params* p, cudaStream_t cs );
bool        tma_atrous_ok( const rgdn_stream* s, int iter );
rgdn_status launch_atrous_tma( rgdn_stream* s, const FrameArgs& a, int iter, bool hist, cudaStream_t cs );

rgdn_status run_denoise( rgdn_stream* s, uint32_t fi, const rgdn_frame_params* p, cudaStream_t cs )
{
    if( !( p->flags & RGDN_FLAG_PLAIN ) ) return run_denoise_fused( s, fi, p, cs );
    FrameArgs a;
    fill_args( s, fi, p, a );
    rgdn_status r;
    if( !( p->flags & RGDN_FLAG_SKIP_GRADIENTS ) )
    {
        if( ( r = launch( s, a, RGDN_STAGE_GRADIENT_SAMPLES, 0, cs ) ) != RGDN_SUCCESS ) return r;
        for( int i = 0; i < 4; i++ )
            if( ( r = launch( s, a, RGDN_STAGE_GRADIENT_ATROUS, i, cs ) ) != RGDN_SUCCESS ) return r;
    }
    if( ( r = launch( s, a, RGDN_STAGE_TEMPORAL_ACCUMULATION, 0, cs ) ) != RGDN_SUCCESS ) return r;
    if( ( r = launch( s, a, RGDN_STAGE_ANTI_FIREFLY, 0, cs ) ) != RGDN_SUCCESS ) return r;
    if( ( r = launch( s, a, RGDN_STAGE_VARIANCE_ESTIMATION, 0, cs ) ) != RGDN_SUCCESS ) return r;
    for( uint32_t i = 0; i < a.u.niter; i++ )
        if( ( r = launch( s, a, RGDN_STAGE_ATROUS, (int)i, cs ) ) != RGDN_SUCCESS ) return r;
    return RGDN_SUCCESS;
}

// One reference stage on the default path's kernel (run_denoise_fused, and rgdn_denoise_stage
// with RGDN_FLAG_STAGE_DEFAULT): the temporal pass also writes the per-pixel geometry record the
// later passes read, the last a-trous iteration also bins the histogram, and the histogram stage
// itself is then empty. The caller has filled `a` for frame slot `fi` and made the bin table
// current.
rgdn_status launch_default_stage( rgdn_stream* s, const FrameArgs& a, uint32_t fi, const rgdn_frame_params* p, int stage, int iter,
                                  cudaStream_t cs, bool pairOk = false, bool afterGradients = false )
{
    const bool exact = ( p->flags & RGDN_FLAG_EXACT_MATH ) != 0;
    switch( stage )
    {
        case RGDN_STAGE_GRADIENT_SAMPLES:
        case RGDN_STAGE_GRADIENT_ATROUS: return launch( s, a, stage, iter, cs );
        case RGDN_STAGE_TEMPORAL_ACCUMULATION:
        {
            const bool  gp = s->geomValid[ fi ^ 1u ];
            // directly after this frame's gradient chain, the FAST pass reads all but the
            // gradient before it waits for the chain (k_temporal, EARLY)
            const int   tf = afterGradients ? ( gp ? KF_TEMPORAL_FAST_GP_EARLY : KF_TEMPORAL_FAST_EARLY ) : ( gp ? KF_TEMPORAL_FAST_GP : KF_TEMPORAL_FAST );
            const int   ta = exact ? ( gp ? KF_TEMPORAL_EXACT_GEOM_GP : KF_TEMPORAL_EXACT_GEOM ) : tf;
            rgdn_status r  = launch( s, a, ta, 0, cs );
            if( r == RGDN_SUCCESS ) s->geomValid[ fi ] = true;
            return r;
        }
        case RGDN_STAGE_ANTI_FIREFLY: return launch( s, a, KF_ANTI_FIREFLY_FAST, 0, cs );
        case RGDN_STAGE_VARIANCE_ESTIMATION: return launch( s, a, exact ? KF_VARIANCE_EXACT_GEOM : KF_VARIANCE_FAST, 0, cs );
        case RGDN_STAGE_ATROUS:
        {
            // a histogram no exposure pass consumed is discarded: this frame's replaces it
            if( iter == 0 && s->histPending )
            {
                if( cudaMemsetAsync( s->tm->histogram, 0, sizeof( s->tm->histogram ), cs ) != cudaSuccess ) return RGDN_DEVICE_ERROR;
                s->histPending = false;
            }
            const bool  last = iter + 1 == (int)a.u.niter;
            rgdn_status r;
            if( pairOk && iter == 1 ) return RGDN_SUCCESS;   // computed with iteration 0
            if( pairOk && iter == 0 ) r = launch( s, a, KF_ATROUS_PAIR01, 0, cs );
            else if( !exact && ( p->flags & RGDN_FLAG_TMA_STAGING ) && tma_atrous_ok( s, iter ) ) r = launch_atrous_tma( s, a, iter, last, cs );
            else
            {
                const int k = exact ? ( last ? KF_ATROUS_EXACT_HIST : KF_ATROUS_EXACT ) : ( last ? KF_ATROUS_FAST_HIST : KF_ATROUS_FAST );
                r = launch( s, a, k, iter, cs );
            }
            if( r == RGDN_SUCCESS && last ) s->histPending = true;
            return r;
        }
        case RGDN_STAGE_LUMINANCE_HISTOGRAM: return RGDN_SUCCESS;
        case RGDN_STAGE_LUMINANCE_AVG:
        {
            // binned by the last a-trous iteration, or by nothing (an average of an empty
            // histogram, as the plain path's order would give without its histogram pass)
            s->histPending = false;
            return launch( s, a, RGDN_STAGE_LUMINANCE_AVG, 0, cs );
        }
        default: return RGDN_WRONG_FUNCTION_ARGUMENT;
    }
}

// Default path: gradient samples and the 4 gradient a-trous iterations, temporal accumulation,
// anti-firefly on packed values, variance, the a-trous iterations, and the histogram
// accumulated by the last iteration (HistogramInput is still written). Continuous weights use
// FAST math.
rgdn_status run_denoise_fused( rgdn_stream* s, uint32_t fi, const rgdn_frame_params* p, cudaStream_t cs )
{
    rgdn_status r = ensure_bin_lut( s, p, cs );
    if( r != RGDN_SUCCESS ) return r;
    FrameArgs a;
    fill_args( s, fi, p, a );
    // the frame's geometry record persists in L2 for the launches of this frame
    struct WindowScope
    {
        WindowScope( const rgdn_stream* s, const FrameArgs& a )
        {
            const size_t one   = (size_t)s->W * s->H * 16;
            void*        base  = kGeomBothSlots ? (void*)s->geom[ 0 ] : (void*)a.geom;
            const size_t bytes = kGeomBothSlots ? (size_t)( (uint8_t*)s->geom[ 1 ] - (uint8_t*)s->geom[ 0 ] ) + one : one;
            if( kGeomL2Persist && s->ctx->l2Persist && a.geom && !tl_l2windowOff )
            {
                tl_l2window = { base, bytes, std::min( 1.0f, (float)s->ctx->l2Persist / (float)bytes ) };
                s->ctx->l2Dirty.store( true, std::memory_order_relaxed );
            }
        }
        ~WindowScope() { tl_l2window = L2Window{}; }
    } window( s, a );
    if( !( p->flags & RGDN_FLAG_SKIP_GRADIENTS ) )
    {
        if( ( r = launch_default_stage( s, a, fi, p, RGDN_STAGE_GRADIENT_SAMPLES, 0, cs ) ) != RGDN_SUCCESS ) return r;
        for( int i = 0; i < 4; i++ )
            if( ( r = launch_default_stage( s, a, fi, p, RGDN_STAGE_GRADIENT_ATROUS, i, cs ) ) != RGDN_SUCCESS ) return r;
    }
    const bool afterGradients = !( p->flags & RGDN_FLAG_SKIP_GRADIENTS );
    if( ( r = launch_default_stage( s, a, fi, p, RGDN_STAGE_TEMPORAL_ACCUMULATION, 0, cs, false, afterGradients ) ) != RGDN_SUCCESS ) return r;
    if( p->flags & RGDN_FLAG_AF_VARIANCE_FUSED )
        r = launch( s, a, ( p->flags & RGDN_FLAG_EXACT_MATH ) ? KF_AF_VARIANCE_EXACT : KF_AF_VARIANCE_FAST, 0, cs );
    else if( ( r = launch_default_stage( s, a, fi, p, RGDN_STAGE_ANTI_FIREFLY, 0, cs ) ) == RGDN_SUCCESS )
        r = launch_default_stage( s, a, fi, p, RGDN_STAGE_VARIANCE_ESTIMATION, 0, cs );
    if( r != RGDN_SUCCESS ) return r;
    // iterations 0 and 1 in one launch when asked for, with the FAST shared-memory kernels and at
    // least one more iteration after them
    const bool pairOk = ( p->flags & RGDN_FLAG_ATROUS_PAIR ) && a.u.niter >= 3 &&
                        !( p->flags & ( RGDN_FLAG_EXACT_MATH | RGDN_FLAG_TMA_STAGING ) );
    for( uint32_t i = 0; i < a.u.niter; i++ )
        if( ( r = launch_default_stage( s, a, fi, p, RGDN_STAGE_ATROUS, (int)i, cs, pairOk ) ) != RGDN_SUCCESS ) return r;
    return RGDN_SUCCESS;
}

// A map of a dense W x H plane of `tw` 4-byte words per texel with boxes of bw x bh texels:
// 2-D over words for texels up to 8 bytes, 3-D (word, x, y) for 16-byte texels, so no box
// dimension exceeds 256 elements.
bool tensor_map( rgdn_stream* s, const void* plane, int tw, int bw, int bh, CUtensorMap& out )
{
    const auto key = std::make_tuple( plane, tw, bw, bh );
    auto       it  = s->tmaps.find( key );
    if( it != s->tmaps.end() )
    {
        out = it->second;
        return true;
    }
    EncodeTiledFn fn = encode_tiled_fn();
    if( !fn ) return false;
    CUtensorMap      m;
    const cuuint32_t es[ 3 ] = { 1, 1, 1 };
    CUresult         r;
    if( tw == 4 )
    {
        const cuuint64_t dims[ 3 ]    = { 4, (cuuint64_t)s->W, (cuuint64_t)s->H };
        const cuuint64_t strides[ 2 ] = { 16, (cuuint64_t)s->W * 16 };
        const cuuint32_t box[ 3 ]     = { 4, (cuuint32_t)bw, (cuuint32_t)bh };
        r = fn( &m, CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, const_cast< void* >( plane ), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE );
    }
    else
    {
        const cuuint64_t dims[ 2 ]    = { (cuuint64_t)s->W * tw, (cuuint64_t)s->H };
        const cuuint64_t strides[ 1 ] = { (cuuint64_t)s->W * tw * 4 };
        const cuuint32_t box[ 2 ]     = { (cuuint32_t)( bw * tw ), (cuuint32_t)bh };
        r = fn( &m, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, const_cast< void* >( plane ), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE );
    }
    if( r != CUDA_SUCCESS ) return false;
    s->tmaps[ key ] = m;
    out             = m;
    return true;
}

// The TMA-staged a-trous needs 16-byte row pitches of every staged plane (W % 4 == 0 covers
// the 4-byte ones), steps up to 16, the driver's tensor-map encoder, and two stages that fit
// the 227 KB of shared memory a block may use.
bool tma_atrous_ok( const rgdn_stream* s, int iter )
{
    return ( s->W % 4 ) == 0 && iter <= 4 && encode_tiled_fn() != nullptr && atrous_tma_smem( (int)s->storage, iter ) <= 220 * 1024;
}

rgdn_status launch_atrous_tma( rgdn_stream* s, const FrameArgs& a, int iter, bool hist, cudaStream_t cs )
{
    // the sources of this iteration (the routing of atrous_io, CmSVGFAtrous.comp:237-276)
    const bool     odd = ( iter & 1 ) != 0;
    const void*    cv  = iter == 0 ? a.diffPing : iter == 1 ? a.diffHistory : ( odd ? a.diffPong : a.diffPing );
    const void*    var = iter == 0 ? a.varPing : iter == 1 ? a.varHistory : ( odd ? a.varPong : a.varPing );
    const void*    sp  = iter == 0 ? a.specPing : ( odd ? a.specPong : a.specPing );
    const void*    in  = iter == 0 ? a.indirPing : ( odd ? a.indirPong : a.indirPing );
    const TmaGeom  g   = tma_geometry( (int)s->storage, iter );
    const TmaTexel tx  = tma_texel( (int)s->storage );
    AtrousMaps     m;
    if( !tensor_map( s, cv, tx.cv / 4, g.rw, g.rh, m.cv ) || !tensor_map( s, sp, tx.col / 4, g.rw, g.rh, m.spec ) ||
        !tensor_map( s, in, tx.col / 4, g.rw, g.rh, m.indir ) || !tensor_map( s, a.geom, 4, g.rw, g.rh, m.geo ) )
        return RGDN_DEVICE_ERROR;
    if( tx.var ) { if( !var || !tensor_map( s, var, tx.var / 4, g.rw, g.rh, m.var ) ) return RGDN_DEVICE_ERROR; }
    else m.var = m.cv;
    cudaEvent_t ea = nullptr, eb = nullptr;
    if( s->timing )
    {
        ea = take_event( s );
        eb = take_event( s );
        if( !ea || !eb ) return RGDN_DEVICE_ERROR;
        cudaEventRecord( ea, cs );
    }
    cudaError_t e;
    switch( s->storage )
    {
        case RGDN_STORAGE_REF: e = launch_atrous_tma_ref( a, iter, hist, &m, cs ); break;
        case RGDN_STORAGE_FP32: e = launch_atrous_tma_f32( a, iter, hist, &m, cs ); break;
        case RGDN_STORAGE_FP16: e = launch_atrous_tma_f16( a, iter, hist, &m, cs ); break;
        default: e = launch_atrous_tma_bf16( a, iter, hist, &m, cs ); break;
    }
    s->ctx->launches.fetch_add( 1, std::memory_order_relaxed );
    if( s->timing )
    {
        cudaEventRecord( eb, cs );
        s->pending.push_back( { hist ? KF_ATROUS_TMA_HIST : KF_ATROUS_TMA, iter, ea, eb } );
    }
    return cuda_status( e );
}

rgdn_status run_exposure( rgdn_stream* s, uint32_t fi, const rgdn_frame_params* p, cudaStream_t cs )
{
    rgdn_status r = ensure_bin_lut( s, p, cs );
    if( r != RGDN_SUCCESS ) return r;
    FrameArgs a;
    fill_args( s, fi, p, a );
    if( !s->histPending && ( r = launch( s, a, RGDN_STAGE_LUMINANCE_HISTOGRAM, 0, cs ) ) != RGDN_SUCCESS ) return r;
    s->histPending = false;
    return launch( s, a, RGDN_STAGE_LUMINANCE_AVG, 0, cs );
}

// The Y row of the RGB -> XYZ matrix of the Rec.709 primaries with the D65 white (Lindbloom's
// construction: primaries' xyz columns scaled so that RGB (1, 1, 1) maps to the white's XYZ
// with Y = 1), in double precision.
static void rec709_luma( double y[ 3 ] )
{
    const double px[ 3 ] = { 0.64, 0.30, 0.15 }, py[ 3 ] = { 0.33, 0.60, 0.06 };
    const double wx = 0.3127, wy = 0.3290;
    double       m[ 3 ][ 3 ];
    for( int c = 0; c < 3; c++ )
    {
        m[ 0 ][ c ] = px[ c ];
        m[ 1 ][ c ] = py[ c ];
        m[ 2 ][ c ] = 1.0 - px[ c ] - py[ c ];
    }
    const double w[ 3 ] = { wx / wy, 1.0, ( 1.0 - wx - wy ) / wy };
    const double det = m[ 0 ][ 0 ] * ( m[ 1 ][ 1 ] * m[ 2 ][ 2 ] - m[ 1 ][ 2 ] * m[ 2 ][ 1 ] ) -
                       m[ 0 ][ 1 ] * ( m[ 1 ][ 0 ] * m[ 2 ][ 2 ] - m[ 1 ][ 2 ] * m[ 2 ][ 0 ] ) +
                       m[ 0 ][ 2 ] * ( m[ 1 ][ 0 ] * m[ 2 ][ 1 ] - m[ 1 ][ 1 ] * m[ 2 ][ 0 ] );
    // s = m^-1 w by Cramer's rule: column c of m replaced by w
    for( int c = 0; c < 3; c++ )
    {
        double a[ 3 ][ 3 ];
        for( int r = 0; r < 3; r++ )
            for( int k = 0; k < 3; k++ ) a[ r ][ k ] = k == c ? w[ r ] : m[ r ][ k ];
        const double dc = a[ 0 ][ 0 ] * ( a[ 1 ][ 1 ] * a[ 2 ][ 2 ] - a[ 1 ][ 2 ] * a[ 2 ][ 1 ] ) -
                          a[ 0 ][ 1 ] * ( a[ 1 ][ 0 ] * a[ 2 ][ 2 ] - a[ 1 ][ 2 ] * a[ 2 ][ 0 ] ) +
                          a[ 0 ][ 2 ] * ( a[ 1 ][ 0 ] * a[ 2 ][ 1 ] - a[ 1 ][ 1 ] * a[ 2 ][ 0 ] );
        y[ c ] = m[ 1 ][ c ] * ( dc / det );
    }
}

// The LPM setup and filter restated below follow AMD FidelityFX LPM, which carries this notice:
//   Copyright (c) 2017-2019 Advanced Micro Devices, Inc. All rights reserved.
//   Permission is hereby granted, free of charge, to any person obtaining a copy of this
//   software and associated documentation files (the "Software"), to deal in the Software
//   without restriction, including without limitation the rights to use, copy, modify, merge,
//   publish, distribute, sublicense, and/or sell copies of the Software, and to permit persons
//   to whom the Software is furnished to do so, subject to the following conditions:
//   The above copyright notice and this permission notice shall be included in all copies or
//   substantial portions of the Software.
//   THE SOFTWARE IS PROVIDED "AS IS", WITHOUT WARRANTY OF ANY KIND, EXPRESS OR IMPLIED,
//   INCLUDING BUT NOT LIMITED TO THE WARRANTIES OF MERCHANTABILITY, FITNESS FOR A PARTICULAR
//   PURPOSE AND NONINFRINGEMENT. IN NO EVENT SHALL THE AUTHORS OR COPYRIGHT HOLDERS BE LIABLE FOR
//   ANY CLAIM, DAMAGES OR OTHER LIABILITY, WHETHER IN AN ACTION OF CONTRACT, TORT OR OTHERWISE,
//   ARISING FROM, OUT OF OR IN CONNECTION WITH THE SOFTWARE OR THE USE OR OTHER DEALINGS IN THE
//   SOFTWARE.
// LpmSetupCustom.inl:40-70 for the 709 -> 709 arguments ImageComposition::SetupLpmParams
// passes, in FP32 in the setup's order; the luma coefficients are the Rec.709 Y row normalised
// to a unit sum
void lpm_setup_709( const float saturation[ 3 ], const float crosstalk[ 3 ], LpmConsts& o )
{
    const float hdrMax = 256.0f, exposure = 8.0f, shoulderContrast = 1.0f;
    const float contrast = 0.1f + 1.0f;
    for( int k = 0; k < 3; k++ ) o.saturation[ k ] = saturation[ k ] + contrast;
    o.contrast         = contrast;
    const float midIn  = hdrMax * 0.18f * exp2f( -exposure );
    const float midOut = 0.18f;
    const float cs     = contrast * shoulderContrast;
    const float z0 = -powf( midIn, contrast );
    const float z1 = powf( hdrMax, cs ) * powf( midIn, contrast );
    const float z2 = powf( hdrMax, contrast ) * powf( midIn, cs ) * midOut;
    const float z3 = powf( hdrMax, cs ) * midOut;
    const float z4 = powf( midIn, cs ) * midOut;
    o.toneScaleBias[ 0 ] = -( ( z0 + ( midOut * ( z1 - z2 ) ) * ( 1.0f / ( z3 - z4 ) ) ) * ( 1.0f / z4 ) );
    const float w0 = powf( hdrMax, cs ) * powf( midIn, contrast );
    const float w1 = powf( hdrMax, contrast ) * powf( midIn, cs ) * midOut;
    const float w2 = powf( hdrMax, cs ) * midOut;
    const float w3 = powf( midIn, cs ) * midOut;
    o.toneScaleBias[ 1 ] = ( w0 - w1 ) * ( 1.0f / ( w2 - w3 ) );
    double y[ 3 ];
    rec709_luma( y );
    float l[ 3 ] = { (float)y[ 0 ], (float)y[ 1 ], (float)y[ 2 ] };
    const float rs = 1.0f / ( l[ 0 ] + l[ 1 ] + l[ 2 ] );
    for( int k = 0; k < 3; k++ )
    {
        o.lumaT[ k ]     = l[ k ] * rs;
        o.rcpLumaT[ k ]  = 1.0f / o.lumaT[ k ];
        o.crosstalk[ k ] = crosstalk[ k ];
    }
}

}  // namespace rgdn

// ==========================================================================================
extern "C" {

uint32_t rgdn_api_version( void ) { return RGDN_API_VERSION; }

rgdn_status rgdn_histogram_bin_table( float minLog, float maxLog, uint8_t* out )
{
    if( !out || !( maxLog > minLog ) ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    build_bin_lut( out, minLog, maxLog );
    return RGDN_SUCCESS;
}

const char* rgdn_status_string( rgdn_status st )
{
    switch( st )
    {
        case RGDN_SUCCESS: return "success";
        case RGDN_WRONG_INSTANCE: return "wrong instance (null or destroyed handle)";
        case RGDN_DEVICE_ERROR: return "a CUDA call failed";
        case RGDN_INTERNAL_ERROR: return "internal error";
        case RGDN_WRONG_FUNCTION_CALL: return "wrong function call";
        case RGDN_WRONG_FUNCTION_ARGUMENT: return "wrong function argument";
        case RGDN_OUT_OF_BUDGET: return "out of the memory budget";
        case RGDN_TIMEOUT: return "timeout";
        case RGDN_NOT_READY: return "not ready";
        default: return "unknown status";
    }
}

rgdn_status rgdn_context_create( const rgdn_context_create_info* info, rgdn_context** out )
{
    if( !info || !out ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    *out = nullptr;
    int n = 0;
    if( cudaGetDeviceCount( &n ) != cudaSuccess || info->device < 0 || info->device >= n ) return RGDN_DEVICE_ERROR;
    if( cudaSetDevice( info->device ) != cudaSuccess ) return RGDN_DEVICE_ERROR;
    rgdn_context* c = new( std::nothrow ) rgdn_context();
    if( !c ) return RGDN_INTERNAL_ERROR;
    c->device = info->device;
    c->budget = info->memoryBudgetBytes;
    if( kGeomL2Persist && !( info->flags & RGDN_CONTEXT_NO_L2_PERSIST ) )
    {
        // L2 set aside for the geometry record (a limit of this process's context)
        int maxPersist = 0;
        if( cudaDeviceGetAttribute( &maxPersist, cudaDevAttrMaxPersistingL2CacheSize, info->device ) == cudaSuccess && maxPersist > 0 )
        {
            const size_t want = std::min< size_t >( (size_t)maxPersist, kL2PersistMB << 20 );
            if( cudaDeviceSetLimit( cudaLimitPersistingL2CacheSize, want ) == cudaSuccess ) c->l2Persist = want;
        }
        cudaGetLastError();
    }
    // normal decode tables: the correctly rounded sin/cos of the FP32 angles of Utils.h:132-133
    std::vector< float2 > ph( 65536 ), th( 65536 );
    for( uint32_t j = 0; j < 65536u; j++ )
    {
        const double phi = (double)rgdn::normal_phi( j );
        ph[ j ]          = make_float2( (float)sin( phi ), (float)cos( phi ) );
        const double tht = (double)rgdn::normal_theta( j );
        th[ j ]          = make_float2( (float)cos( tht ), (float)sin( tht ) );
    }
    if( cudaMalloc( &c->phiTab, 65536 * sizeof( float2 ) ) != cudaSuccess ||
        cudaMalloc( &c->thetaTab, 65536 * sizeof( float2 ) ) != cudaSuccess ||
        cudaMalloc( &c->decayTab, 256 * sizeof( float ) ) != cudaSuccess ||
        cudaMemcpy( c->phiTab, ph.data(), 65536 * sizeof( float2 ), cudaMemcpyHostToDevice ) != cudaSuccess ||
        cudaMemcpy( c->thetaTab, th.data(), 65536 * sizeof( float2 ), cudaMemcpyHostToDevice ) != cudaSuccess ||
        fill_decay_table( c->decayTab ) != cudaSuccess )
    {
        cudaFree( c->phiTab );
        cudaFree( c->thetaTab );
        cudaFree( c->decayTab );
        c->magic = 0;
        delete c;
        return RGDN_DEVICE_ERROR;
    }
    *out = c;
    return RGDN_SUCCESS;
}

rgdn_status rgdn_context_destroy( rgdn_context* c )
{
    if( !valid_ctx( c ) ) return RGDN_WRONG_INSTANCE;
    cudaSetDevice( c->device );
    std::vector< rgdn_stream* > left;
    {
        std::lock_guard< std::mutex > g( c->mtx );
        left.assign( c->streams.begin(), c->streams.end() );
    }
    batch_destroy( c );
    for( rgdn_stream* s : left ) rgdn_stream_destroy( s );
    cudaFree( c->phiTab );
    cudaFree( c->thetaTab );
    cudaFree( c->decayTab );
    if( c->l2Persist )
    {
        // the set-aside ends with the rgdn context that made it
        cudaCtxResetPersistingL2Cache();
        cudaDeviceSetLimit( cudaLimitPersistingL2CacheSize, 0 );
        cudaGetLastError();
    }
    c->magic = 0;
    delete c;
    return RGDN_SUCCESS;
}

rgdn_status rgdn_context_memory_used( rgdn_context* c, uint64_t* out )
{
    if( !valid_ctx( c ) ) return RGDN_WRONG_INSTANCE;
    if( !out ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    std::lock_guard< std::mutex > g( c->mtx );
    *out = c->used;
    return RGDN_SUCCESS;
}

rgdn_status rgdn_context_launch_count( rgdn_context* c, uint64_t* out )
{
    if( !valid_ctx( c ) ) return RGDN_WRONG_INSTANCE;
    if( !out ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    *out = c->launches.load();
    return RGDN_SUCCESS;
}

rgdn_status rgdn_stream_required_bytes( const rgdn_stream_create_info* info, uint64_t* out )
{
    if( !info || !out || info->width < 2 || info->height < 1 || ( info->width & 1 ) || info->storage > RGDN_STORAGE_BF16 )
        return RGDN_WRONG_FUNCTION_ARGUMENT;
    *out = stream_layout( info->width, info->height, info->storage, nullptr, nullptr );
    return RGDN_SUCCESS;
}

static rgdn_status stream_alloc( rgdn_stream* s, uint32_t W, uint32_t H )
{
    rgdn_context* c     = s->ctx;
    const size_t  bytes = stream_layout( W, H, s->storage, nullptr, nullptr );
    {
        std::lock_guard< std::mutex > g( c->mtx );
        if( c->budget && c->used + bytes > c->budget ) return RGDN_OUT_OF_BUDGET;
        c->used += bytes;
    }
    void* block = nullptr;
    if( cudaMalloc( &block, bytes ) != cudaSuccess || cudaMemset( block, 0, bytes ) != cudaSuccess )
    {
        cudaFree( block );
        cudaGetLastError();
        std::lock_guard< std::mutex > g( c->mtx );
        c->used -= bytes;
        return RGDN_OUT_OF_BUDGET;
    }
    s->block = block;
    s->bytes = bytes;
    s->W = W; s->H = H;
    s->GW = std::max( 1u, ( W + 1 ) / 3 );
    s->GH = std::max( 1u, ( H + 1 ) / 3 );
    stream_layout( W, H, s->storage, s->planes, (uint8_t*)block );
    s->tm     = (Tonemapping*)block;
    s->rsDev  = (rgdn_reshade_scene*)( (uint8_t*)block + align_up( sizeof( Tonemapping ) ) );
    s->binLut = (uint8_t*)s->rsDev + align_up( sizeof( rgdn_reshade_scene ) );
    s->geom[ 0 ] = (float4*)( s->binLut + align_up( 65536 ) );
    s->geom[ 1 ] = (float4*)( (uint8_t*)s->geom[ 0 ] + align_up( (size_t)W * H * 16 ) );
    s->geomValid[ 0 ] = s->geomValid[ 1 ] = false;
    s->tmaps.clear();
    s->lutMin = s->lutMax = NAN;
    return RGDN_SUCCESS;
}

static void stream_free( rgdn_stream* s )
{
    if( !s->block ) return;
    cudaFree( s->block );
    std::lock_guard< std::mutex > g( s->ctx->mtx );
    s->ctx->used -= s->bytes;
    s->block = nullptr;
    s->bytes = 0;
}

rgdn_status rgdn_stream_create( rgdn_context* c, const rgdn_stream_create_info* info, rgdn_stream** out )
{
    if( !valid_ctx( c ) ) return RGDN_WRONG_INSTANCE;
    if( !info || !out ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    *out = nullptr;
    if( info->width < 2 || info->height < 1 || ( info->width & 1 ) || info->storage > RGDN_STORAGE_BF16 ||
        info->width > 16384 || info->height > 16384 )
        return RGDN_WRONG_FUNCTION_ARGUMENT;
    if( cudaSetDevice( c->device ) != cudaSuccess ) return RGDN_DEVICE_ERROR;
    rgdn_stream* s = new( std::nothrow ) rgdn_stream();
    if( !s ) return RGDN_INTERNAL_ERROR;
    s->ctx     = c;
    s->storage = info->storage;
    rgdn_status r = stream_alloc( s, info->width, info->height );
    if( r != RGDN_SUCCESS )
    {
        s->magic = 0;
        delete s;
        return r;
    }
    {
        std::lock_guard< std::mutex > g( c->mtx );
        c->streams.insert( s );
    }
    *out = s;
    return RGDN_SUCCESS;
}

rgdn_status rgdn_stream_destroy( rgdn_stream* s )
{
    if( !valid_stream( s ) ) return RGDN_WRONG_INSTANCE;
    cudaSetDevice( s->ctx->device );
    cudaDeviceSynchronize();
    stream_free( s );
    for( auto& pd : s->pending )
    {
        cudaEventDestroy( pd.a );
        cudaEventDestroy( pd.b );
    }
    for( cudaEvent_t e : s->eventPool ) cudaEventDestroy( e );
    {
        std::lock_guard< std::mutex > g( s->ctx->mtx );
        s->ctx->streams.erase( s );
    }
    s->magic = 0;
    delete s;
    return RGDN_SUCCESS;
}

rgdn_status rgdn_stream_resize( rgdn_stream* s, uint32_t w, uint32_t h )
{
    if( !valid_stream( s ) ) return RGDN_WRONG_INSTANCE;
    if( w < 2 || h < 1 || ( w & 1 ) || w > 16384 || h > 16384 ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    if( w == s->W && h == s->H ) return RGDN_SUCCESS;
    cudaSetDevice( s->ctx->device );
    // Framebuffers::PrepareForSize waits for the device idle before reallocating
    cudaDeviceSynchronize();
    const uint32_t oldW = s->W, oldH = s->H;
    stream_free( s );
    rgdn_status r = stream_alloc( s, w, h );
    if( r != RGDN_SUCCESS )
    {
        // keep the stream usable at its old size when the new one does not fit
        if( stream_alloc( s, oldW, oldH ) != RGDN_SUCCESS ) return RGDN_DEVICE_ERROR;
        return r;
    }
    return RGDN_SUCCESS;
}

rgdn_status rgdn_stream_get_framebuffer( rgdn_stream* s, uint32_t fb, uint32_t frameIndex, rgdn_image* out )
{
    if( !valid_stream( s ) ) return RGDN_WRONG_INSTANCE;
    if( fb >= RGDN_FB_COUNT || !out || frameIndex > 1 ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    const PlaneSlot& p = s->planes[ fb ];
    out->data        = (void*)plane_ptr( s, fb, frameIndex );
    out->width       = p.w;
    out->height      = p.h;
    out->pitch_bytes = p.w * p.texel;
    out->texel_bytes = p.texel;
    out->format      = p.format;
    out->has_prev    = p.prev ? 1u : 0u;
    return RGDN_SUCCESS;
}

rgdn_status rgdn_stream_bind_framebuffer( rgdn_stream* s, uint32_t fb, uint32_t frameIndex, void* devicePtr )
{
    if( !valid_stream( s ) ) return RGDN_WRONG_INSTANCE;
    const bool producerPlane = fb <= RGDN_FB_GRADIENT_RESHADED || fb == RGDN_FB_SCREEN_EMIS_RT || fb == RGDN_FB_SCATTERING ||
                               fb == RGDN_FB_RESERVOIRS ||
                               fb == RGDN_FB_DEPTH_NDC || fb == RGDN_FB_SCATTER_VOLUME;
    if( !producerPlane || frameIndex > 1 || ( (uintptr_t)devicePtr & 15u ) ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    PlaneSlot& p    = s->planes[ fb ];
    const int  slot = p.prev ? (int)frameIndex : 0;
    p.ptr[ slot ]   = devicePtr ? (uint8_t*)devicePtr : p.own[ slot ];
    if( fb == RGDN_FB_NORMAL || fb == RGDN_FB_DEPTH_WORLD || fb == RGDN_FB_METALLIC_ROUGHNESS ) s->geomValid[ frameIndex ] = false;
    return RGDN_SUCCESS;
}

rgdn_status rgdn_stream_upload( rgdn_stream* s, uint32_t fb, uint32_t frameIndex, const void* src, size_t bytes, rgdn_cuda_stream cs )
{
    if( !valid_stream( s ) ) return RGDN_WRONG_INSTANCE;
    if( fb >= RGDN_FB_COUNT || frameIndex > 1 || !src ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    const PlaneSlot& p = s->planes[ fb ];
    if( !p.ptr[ 0 ] || bytes != (size_t)p.w * p.h * p.texel ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    cudaSetDevice( s->ctx->device );
    if( fb == RGDN_FB_NORMAL || fb == RGDN_FB_DEPTH_WORLD || fb == RGDN_FB_METALLIC_ROUGHNESS ) s->geomValid[ frameIndex ] = false;
    return cuda_status( cudaMemcpyAsync( plane_ptr_mut( s, fb, frameIndex ), src, bytes, cudaMemcpyDefault, (cudaStream_t)cs ) );
}

rgdn_status rgdn_stream_download( rgdn_stream* s, uint32_t fb, uint32_t frameIndex, void* dst, size_t bytes, rgdn_cuda_stream cs )
{
    if( !valid_stream( s ) ) return RGDN_WRONG_INSTANCE;
    if( fb >= RGDN_FB_COUNT || frameIndex > 1 || !dst ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    const PlaneSlot& p = s->planes[ fb ];
    if( !p.ptr[ 0 ] || bytes != (size_t)p.w * p.h * p.texel ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    cudaSetDevice( s->ctx->device );
    return cuda_status( cudaMemcpyAsync( dst, plane_ptr( s, fb, frameIndex ), bytes, cudaMemcpyDefault, (cudaStream_t)cs ) );
}

rgdn_status rgdn_denoise( rgdn_stream* s, uint32_t frameIndex, const rgdn_frame_params* p, rgdn_cuda_stream cs )
{
    if( !valid_stream( s ) ) return RGDN_WRONG_INSTANCE;
    if( frameIndex > 1 ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    rgdn_status r = check_params( p );
    if( r != RGDN_SUCCESS ) return r;
    cudaSetDevice( s->ctx->device );
    return run_denoise( s, frameIndex, p, (cudaStream_t)cs );
}

rgdn_status rgdn_bloom( rgdn_stream* s, uint32_t frameIndex, const rgdn_bloom_params* p, rgdn_cuda_stream cs )
{
    if( !valid_stream( s ) ) return RGDN_WRONG_INSTANCE;
    if( !p || frameIndex > 1 || !std::isfinite( p->bloomIntensity ) ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    cudaSetDevice( s->ctx->device );
    BloomArgs b = {};
    const uint32_t fbs[ 11 ] = { RGDN_FB_BLOOM_INPUT, RGDN_FB_BLOOM_MIP1, RGDN_FB_BLOOM_MIP2, RGDN_FB_BLOOM_MIP3, RGDN_FB_BLOOM_MIP4,
                                 RGDN_FB_BLOOM_MIP5,  RGDN_FB_BLOOM_MIP6, RGDN_FB_BLOOM_MIP7, RGDN_FB_BLOOM_MIP8, RGDN_FB_BLOOM_RESULT,
                                 RGDN_FB_FINAL };
    for( int k = 0; k < 11; k++ )
    {
        b.planes[ k ] = plane_ptr_mut( s, fbs[ k ], frameIndex );
        b.w[ k ]      = (int)s->planes[ fbs[ k ] ].w;
        b.h[ k ]      = (int)s->planes[ fbs[ k ] ].h;
    }
    b.W         = (int)s->W;
    b.H         = (int)s->H;
    b.intensity = p->bloomIntensity;
    cudaStream_t st = (cudaStream_t)cs;
    cudaEvent_t  ea = nullptr, eb = nullptr;
    if( s->timing )
    {
        ea = take_event( s );
        eb = take_event( s );
        if( !ea || !eb ) return RGDN_DEVICE_ERROR;
        cudaEventRecord( ea, st );
    }
    cudaError_t e;
    switch( s->storage )
    {
        case RGDN_STORAGE_REF: e = launch_bloom_ref( b, st ); break;
        case RGDN_STORAGE_FP32: e = launch_bloom_f32( b, st ); break;
        case RGDN_STORAGE_FP16: e = launch_bloom_f16( b, st ); break;
        default: e = launch_bloom_bf16( b, st ); break;
    }
    s->ctx->launches.fetch_add( BLOOM_LAUNCHES, std::memory_order_relaxed );
    if( s->timing )
    {
        cudaEventRecord( eb, st );
        s->pending.push_back( { KF_BLOOM, 0, ea, eb } );
    }
    return cuda_status( e );
}

// GLSL mat4 * mat4 (column-major), each element summed over k = 0..3 in FP32 without
// contraction: CmScatterAccum.comp:55 evaluates invView * invProjection before the vector
static void mat4_mul_f32( const float* a, const float* b, float* out )
{
    for( int c = 0; c < 4; c++ )
        for( int r = 0; r < 4; r++ )
        {
            volatile float acc = a[ 0 * 4 + r ] * b[ c * 4 + 0 ];
            for( int k = 1; k < 4; k++ )
            {
                volatile float prod = a[ k * 4 + r ] * b[ c * 4 + k ];
                acc                 = acc + prod;
            }
            out[ c * 4 + r ] = acc;
        }
}

rgdn_status rgdn_process_scattering( rgdn_stream* s, uint32_t frameIndex, const rgdn_volumetric_params* p, rgdn_cuda_stream cs )
{
    if( !valid_stream( s ) ) return RGDN_WRONG_INSTANCE;
    if( !p || frameIndex > 1 || p->volumeEnableType > RGDN_VOLUME_ENABLE_VOLUMETRIC || !std::isfinite( p->maxHistoryLength ) )
        return RGDN_WRONG_FUNCTION_ARGUMENT;
    if( p->volumeEnableType == RGDN_VOLUME_ENABLE_VOLUMETRIC && !( p->volumeCameraFar > p->volumeCameraNear ) ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    cudaSetDevice( s->ctx->device );
    ScatterArgs a = {};
    a.u.W         = (int)s->W;
    a.u.H         = (int)s->H;
    a.u.rw        = (float)s->W;
    a.u.rh        = (float)s->H;
    a.u.isx       = 1.0f / ( a.u.rw / 2.0f );
    a.u.isy       = 1.0f / a.u.rh;
    a.volume      = (ushort4*)plane_ptr_mut( s, RGDN_FB_SCATTER_VOLUME, frameIndex );
    a.nx          = RGDN_VOLUME_SIZE_X;
    a.ny          = RGDN_VOLUME_SIZE_Y;
    a.nz          = RGDN_VOLUME_SIZE_Z;
    a.motion      = (const ushort4*)plane_ptr( s, RGDN_FB_MOTION, frameIndex );
    a.depth       = (const uint16_t*)plane_ptr( s, RGDN_FB_DEPTH_WORLD, frameIndex );
    a.depthPrev   = (const uint16_t*)plane_ptr( s, RGDN_FB_DEPTH_WORLD, frameIndex ^ 1 );
    a.normal      = (const uint32_t*)plane_ptr( s, RGDN_FB_NORMAL, frameIndex );
    a.normalPrev  = (const uint32_t*)plane_ptr( s, RGDN_FB_NORMAL, frameIndex ^ 1 );
    a.depthNdc    = (const float*)plane_ptr( s, RGDN_FB_DEPTH_NDC, frameIndex );
    a.scatterPrev = (const ushort4*)plane_ptr( s, RGDN_FB_SCATTERING, frameIndex ^ 1 );
    a.historyPrev = (const uint16_t*)plane_ptr( s, RGDN_FB_SCATTERING_HISTORY, frameIndex ^ 1 );
    a.scatterOut  = (ushort4*)plane_ptr_mut( s, RGDN_FB_SCATTERING, frameIndex );
    a.historyOut  = (uint16_t*)plane_ptr_mut( s, RGDN_FB_SCATTERING_HISTORY, frameIndex );
    a.phiTab      = s->ctx->phiTab;
    a.thetaTab    = s->ctx->thetaTab;
    mat4_mul_f32( p->invView, p->invProjection, a.invViewProj );
    memcpy( a.volumeViewProj, p->volumeViewProj, sizeof( a.volumeViewProj ) );
    for( int k = 0; k < 3; k++ ) a.camPos[ k ] = p->cameraPosition[ k ], a.ambient[ k ] = p->volumeAmbient[ k ];
    a.volNear          = p->volumeCameraNear;
    a.volFar           = p->volumeCameraFar;
    a.density          = p->volumeScattering * 0.00005f;
    a.maxHistoryLength = p->maxHistoryLength;
    a.enableType       = p->volumeEnableType;
    a.frameId          = p->frameId;
    a.flags            = p->flags;
    a.irw              = 1.0f / a.u.rw;
    a.irh              = 1.0f / a.u.rh;
    a.iRange           = 1.0f / ( a.volFar - a.volNear );
    cudaStream_t st = (cudaStream_t)cs;
    cudaEvent_t  ea = nullptr, eb = nullptr;
    if( s->timing )
    {
        ea = take_event( s );
        eb = take_event( s );
        if( !ea || !eb ) return RGDN_DEVICE_ERROR;
        cudaEventRecord( ea, st );
    }
    const cudaError_t e = launch_process_scattering( a, st );
    s->ctx->launches.fetch_add( 2, std::memory_order_relaxed );
    if( s->timing )
    {
        cudaEventRecord( eb, st );
        s->pending.push_back( { KF_SCATTER_ACCUM, 0, ea, eb } );
    }
    return cuda_status( e );
}

rgdn_status rgdn_prepare_final( rgdn_stream* s, uint32_t frameIndex, const rgdn_final_params* p, rgdn_cuda_stream cs )
{
    if( !valid_stream( s ) ) return RGDN_WRONG_INSTANCE;
    if( !p || frameIndex > 1 ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    // LpmSetup: crosstalk in (0, 1] (one channel 1); finite tone parameters
    for( int k = 0; k < 3; k++ )
        if( !( p->crosstalk[ k ] > 0.0f && p->crosstalk[ k ] <= 1.0f ) || !std::isfinite( p->saturation[ k ] ) ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    if( !( p->luminanceWhitePoint > 0.0f ) || !std::isfinite( p->emissionMaxScreenColor ) || !std::isfinite( p->bloomEmissionMultiplier ) ||
        !( p->bloomThreshold >= 0.0f ) )
        return RGDN_WRONG_FUNCTION_ARGUMENT;
    cudaSetDevice( s->ctx->device );
    FinalArgs f        = {};
    f.W                = (int)s->W;
    f.H                = (int)s->H;
    f.rw               = (float)s->W;
    f.lightmapCoverage = p->lightmapScreenCoverage;
    f.whitePoint       = p->luminanceWhitePoint;
    f.emisMax          = p->emissionMaxScreenColor;
    f.bloomEvOffset    = p->bloomEmissionMultiplier;
    f.bloomThreshold   = p->bloomThreshold;
    f.flags            = p->flags;
    lpm_setup_709( p->saturation, p->crosstalk, f.lpm );
    f.preFinal   = plane_ptr( s, RGDN_FB_PRE_FINAL, frameIndex );
    f.screenEmis = (const uint32_t*)plane_ptr( s, RGDN_FB_SCREEN_EMIS_RT, frameIndex );
    f.scattering = (const ushort4*)plane_ptr( s, RGDN_FB_SCATTERING, frameIndex );
    f.throughput = (const ushort4*)plane_ptr( s, RGDN_FB_THROUGHPUT, frameIndex );
    f.tm         = s->tm;
    f.finalOut   = plane_ptr_mut( s, RGDN_FB_FINAL, frameIndex );
    f.bloomOut   = plane_ptr_mut( s, RGDN_FB_BLOOM_INPUT, frameIndex );
    cudaStream_t st = (cudaStream_t)cs;
    cudaEvent_t  ea = nullptr, eb = nullptr;
    if( s->timing )
    {
        ea = take_event( s );
        eb = take_event( s );
        if( !ea || !eb ) return RGDN_DEVICE_ERROR;
        cudaEventRecord( ea, st );
    }
    cudaError_t e;
    switch( s->storage )
    {
        case RGDN_STORAGE_REF: e = launch_final_ref( f, st ); break;
        case RGDN_STORAGE_FP32: e = launch_final_f32( f, st ); break;
        case RGDN_STORAGE_FP16: e = launch_final_f16( f, st ); break;
        default: e = launch_final_bf16( f, st ); break;
    }
    s->ctx->launches.fetch_add( 1, std::memory_order_relaxed );
    if( s->timing )
    {
        cudaEventRecord( eb, st );
        s->pending.push_back( { KF_PREPARE_FINAL, 0, ea, eb } );
    }
    return cuda_status( e );
}

rgdn_status rgdn_calculate_exposure( rgdn_stream* s, uint32_t frameIndex, const rgdn_frame_params* p, rgdn_cuda_stream cs )
{
    if( !valid_stream( s ) ) return RGDN_WRONG_INSTANCE;
    if( frameIndex > 1 ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    rgdn_status r = check_params( p );
    if( r != RGDN_SUCCESS ) return r;
    cudaSetDevice( s->ctx->device );
    return run_exposure( s, frameIndex, p, (cudaStream_t)cs );
}

rgdn_status rgdn_denoise_stage( rgdn_stream* s, uint32_t stage, uint32_t iteration, uint32_t frameIndex, const rgdn_frame_params* p,
                                rgdn_cuda_stream cs )
{
    if( !valid_stream( s ) ) return RGDN_WRONG_INSTANCE;
    if( frameIndex > 1 || stage >= RGDN_STAGE_COUNT ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    rgdn_status r = check_params( p );
    if( r != RGDN_SUCCESS ) return r;
    const uint32_t niter = p->atrousIterations == 0 ? 4u : p->atrousIterations;
    if( stage == RGDN_STAGE_GRADIENT_ATROUS && iteration > 3 ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    if( stage == RGDN_STAGE_ATROUS && iteration >= niter ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    cudaSetDevice( s->ctx->device );
    const bool def = ( p->flags & RGDN_FLAG_STAGE_DEFAULT ) != 0;
    if( ( def || stage == RGDN_STAGE_LUMINANCE_HISTOGRAM ) && ( r = ensure_bin_lut( s, p, (cudaStream_t)cs ) ) != RGDN_SUCCESS ) return r;
    FrameArgs a;
    fill_args( s, frameIndex, p, a );
    if( def ) return launch_default_stage( s, a, frameIndex, p, (int)stage, (int)iteration, (cudaStream_t)cs );
    return launch( s, a, (int)stage, (int)iteration, (cudaStream_t)cs );
}

rgdn_status rgdn_stream_set_reshade_scene( rgdn_stream* s, const rgdn_reshade_scene* scene )
{
    if( !valid_stream( s ) ) return RGDN_WRONG_INSTANCE;
    if( !scene )
    {
        s->rsSet = false;
        return RGDN_SUCCESS;
    }
    if( ( scene->lightCount && !scene->lights ) || ( scene->prevLightCount && !scene->prevToCur ) ||
        ( scene->occluderCount && !scene->occluders ) )
        return RGDN_WRONG_FUNCTION_ARGUMENT;
    cudaSetDevice( s->ctx->device );
    // a synchronous copy: frames already enqueued must not be in flight on another stream
    if( cudaMemcpy( s->rsDev, scene, sizeof( *scene ), cudaMemcpyHostToDevice ) != cudaSuccess ) return RGDN_DEVICE_ERROR;
    s->rsSet = true;
    return RGDN_SUCCESS;
}

rgdn_status rgdn_stream_set_timing( rgdn_stream* s, uint32_t enable )
{
    if( !valid_stream( s ) ) return RGDN_WRONG_INSTANCE;
    s->timing = enable != 0;
    return RGDN_SUCCESS;
}

rgdn_status rgdn_stream_read_timing( rgdn_stream* s, rgdn_stage_timing* out, uint32_t capacity, uint32_t* outCount )
{
    if( !valid_stream( s ) ) return RGDN_WRONG_INSTANCE;
    if( !outCount || ( capacity && !out ) ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    cudaSetDevice( s->ctx->device );
    std::map< std::pair< int, int >, std::pair< uint32_t, double > > agg;
    rgdn_status r = RGDN_SUCCESS;
    for( auto& pd : s->pending )
    {
        float ms = 0.0f;
        if( cudaEventSynchronize( pd.b ) != cudaSuccess || cudaEventElapsedTime( &ms, pd.a, pd.b ) != cudaSuccess ) r = RGDN_DEVICE_ERROR;
        auto& slot = agg[ { pd.stage, pd.iter } ];
        slot.first++;
        slot.second += ms;
        s->eventPool.push_back( pd.a );
        s->eventPool.push_back( pd.b );
    }
    s->pending.clear();
    uint32_t n = 0;
    for( auto& kv : agg )
    {
        if( n < capacity ) out[ n ] = { (uint32_t)kv.first.first, (uint32_t)kv.first.second, kv.second.first, (float)kv.second.second };
        n++;
    }
    *outCount = n;
    return r;
}

rgdn_status rgdn_stream_tonemapping_device( rgdn_stream* s, void** out )
{
    if( !valid_stream( s ) ) return RGDN_WRONG_INSTANCE;
    if( !out ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    *out = s->tm;
    return RGDN_SUCCESS;
}

rgdn_status rgdn_get_tonemapping( rgdn_stream* s, uint32_t* hist, float* avgLum, float* exposure, rgdn_cuda_stream cs )
{
    if( !valid_stream( s ) ) return RGDN_WRONG_INSTANCE;
    cudaSetDevice( s->ctx->device );
    Tonemapping h;
    if( cudaMemcpyAsync( &h, s->tm, sizeof( h ), cudaMemcpyDeviceToHost, (cudaStream_t)cs ) != cudaSuccess ||
        cudaStreamSynchronize( (cudaStream_t)cs ) != cudaSuccess )
        return RGDN_DEVICE_ERROR;
    if( hist ) memcpy( hist, h.histogram, sizeof( h.histogram ) );
    if( avgLum ) *avgLum = h.avgLuminance;
    if( exposure )
    {
        // Exposure.h:33-51 getAutoEV100 + ev100ToLuminousExposure
        const float lumAverage = fmaxf( 0.0f, h.avgLuminance );
        const float ev100      = log2f( lumAverage * 100.0f / 12.5f );
        const float maxLum     = 1.2f * exp2f( ev100 );
        *exposure              = maxLum > 0.0f ? 1.0f / maxLum : 0.0f;
    }
    return RGDN_SUCCESS;
}

rgdn_status rgdn_stream_take_device_errors( rgdn_stream* s, uint32_t* outFlags, rgdn_cuda_stream cs )
{
    if( !valid_stream( s ) ) return RGDN_WRONG_INSTANCE;
    if( !outFlags ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    cudaSetDevice( s->ctx->device );
    uint32_t     flags = 0;
    cudaStream_t st    = (cudaStream_t)cs;
    if( cudaMemcpyAsync( &flags, &s->tm->errorFlags, sizeof( flags ), cudaMemcpyDeviceToHost, st ) != cudaSuccess ||
        cudaStreamSynchronize( st ) != cudaSuccess )
        return RGDN_DEVICE_ERROR;
    if( flags && ( cudaMemsetAsync( &s->tm->errorFlags, 0, sizeof( uint32_t ), st ) != cudaSuccess ||
                   cudaStreamSynchronize( st ) != cudaSuccess ) )
        return RGDN_DEVICE_ERROR;
    *outFlags = flags;
    return RGDN_SUCCESS;
}

rgdn_status rgdn_stream_copy_tonemapping( rgdn_stream* s, void* dst, rgdn_cuda_stream cs )
{
    if( !valid_stream( s ) ) return RGDN_WRONG_INSTANCE;
    if( !dst ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    cudaSetDevice( s->ctx->device );
    const size_t bytes = offsetof( Tonemapping, avgLuminance ) + sizeof( float );
    return cuda_status( cudaMemcpyAsync( dst, s->tm, bytes, cudaMemcpyDefault, (cudaStream_t)cs ) );
}

rgdn_status rgdn_set_tonemapping( rgdn_stream* s, const uint32_t* hist, float avgLum, rgdn_cuda_stream cs )
{
    if( !valid_stream( s ) ) return RGDN_WRONG_INSTANCE;
    cudaSetDevice( s->ctx->device );
    Tonemapping h;
    memset( &h, 0, sizeof( h ) );
    if( hist ) memcpy( h.histogram, hist, sizeof( h.histogram ) );
    h.avgLuminance = avgLum;
    // pageable source: staged before the call returns
    if( cudaMemcpyAsync( s->tm, &h, sizeof( h ), cudaMemcpyHostToDevice, (cudaStream_t)cs ) != cudaSuccess ) return RGDN_DEVICE_ERROR;
    return cuda_status( cudaStreamSynchronize( (cudaStream_t)cs ) );
}

rgdn_status rgdn_submit_batch( rgdn_context* c, const rgdn_job* jobs, uint32_t n, rgdn_cuda_stream cs )
{
    if( !valid_ctx( c ) ) return RGDN_WRONG_INSTANCE;
    if( n && !jobs ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    for( uint32_t j = 0; j < n; j++ )
    {
        if( !valid_stream( jobs[ j ].stream ) || jobs[ j ].stream->ctx != c ) return RGDN_WRONG_INSTANCE;
        if( jobs[ j ].frameIndex > 1 ) return RGDN_WRONG_FUNCTION_ARGUMENT;
        rgdn_status r = check_params( jobs[ j ].params );
        if( r != RGDN_SUCCESS ) return r;
    }
    if( n == 0 ) return RGDN_SUCCESS;
    cudaSetDevice( c->device );
    return batch_submit( c, jobs, n, (cudaStream_t)cs );
}

rgdn_status rgdn_batch_get_config( rgdn_context* c, uint32_t storage, rgdn_batch_config* out )
{
    if( !valid_ctx( c ) ) return RGDN_WRONG_INSTANCE;
    if( !out || storage > RGDN_STORAGE_BF16 ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    cudaSetDevice( c->device );
    return batch_get_config( c, storage, out );
}

rgdn_status rgdn_batch_set_config( rgdn_context* c, uint32_t storage, const rgdn_batch_config* in )
{
    if( !valid_ctx( c ) ) return RGDN_WRONG_INSTANCE;
    if( !in || storage > RGDN_STORAGE_BF16 ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    cudaSetDevice( c->device );
    return batch_set_config( c, storage, in );
}

rgdn_status rgdn_batch_set_timing( rgdn_context* c, uint32_t enable )
{
    if( !valid_ctx( c ) ) return RGDN_WRONG_INSTANCE;
    cudaSetDevice( c->device );
    return batch_set_timing( c, enable != 0 );
}

rgdn_status rgdn_batch_read_timing( rgdn_context* c, rgdn_stage_timing* out, uint32_t capacity, uint32_t* outCount )
{
    if( !valid_ctx( c ) ) return RGDN_WRONG_INSTANCE;
    if( !outCount || ( capacity && !out ) ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    cudaSetDevice( c->device );
    return batch_read_timing( c, out, capacity, outCount );
}

}  // extern "C"
