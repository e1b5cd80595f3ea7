// Stage kernels of the A-SVGF denoise + luminance-histogram auto-exposure path, templated on
// the storage mode. Included once per mode by rgdn_mode_*.cu with RGDN_MODE defined.
//
// Every kernel restates one RayTracedGL1 compute shader (cited per kernel). Arithmetic is
// IEEE binary32 without fused multiply-add (the library is compiled with --fmad=false), in
// the shaders' expression and loop order, so threshold decisions (history length > 4, the
// depth/normal reprojection tests, floor() of reprojected positions) match a CPU evaluation
// of the same expressions bit for bit. Texel reads outside the image return zero texels.
//
// Layout: every image is a dense row-major W x H array of its texel type (no padding);
// threads map x -> threadIdx.x so that a warp reads 32 consecutive texels of a row.
#pragma once

#include <cuda.h>
#include <atomic>
#include <type_traits>
#include <utility>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "rgdn_codec.h"
#include "rgdn_internal.h"

namespace rgdn
{
// A launch that lets the kernel start while its predecessor in the stream drains
// (programmatic stream serialization; the kernels order their memory accesses with pdl_wait).
template< class... KP, class... A >
cudaError_t launch_pdl( void ( *kernel )( KP... ), dim3 grid, dim3 block, size_t smem, cudaStream_t s, A&&... args )
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim            = grid;
    cfg.blockDim           = block;
    cfg.dynamicSmemBytes   = smem;
    cfg.stream             = s;
    cudaLaunchAttribute at[ 2 ];
    at[ 0 ].id                                         = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[ 0 ].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs                                          = at;
    cfg.numAttrs                                       = 1;
    if( tl_l2window.ptr )
    {
        at[ 1 ].id                                 = cudaLaunchAttributeAccessPolicyWindow;
        at[ 1 ].val.accessPolicyWindow.base_ptr    = tl_l2window.ptr;
        at[ 1 ].val.accessPolicyWindow.num_bytes   = tl_l2window.bytes;
        at[ 1 ].val.accessPolicyWindow.hitRatio    = tl_l2window.hit;
        at[ 1 ].val.accessPolicyWindow.hitProp     = cudaAccessPropertyPersisting;
        at[ 1 ].val.accessPolicyWindow.missProp    = cudaAccessPropertyStreaming;
        cfg.numAttrs                               = 2;
    }
    return cudaLaunchKernelEx( &cfg, kernel, std::forward< A >( args )... );
}

namespace dev
{

// ------------------------------------------------------------------------------------------
// GLSL semantics
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ float gclamp( float x, float lo, float hi ) { return fminf( fmaxf( x, lo ), hi ); }
__device__ __forceinline__ float gsat( float x ) { return gclamp( x, 0.0f, 1.0f ); }
__device__ __forceinline__ float gmix( float x, float y, float a ) { return x * ( 1.0f - a ) + y * a; }
__device__ __forceinline__ float gsmoothstep( float e0, float e1, float x )
{
    float t = gclamp( ( x - e0 ) / ( e1 - e0 ), 0.0f, 1.0f );
    return t * t * ( 3.0f - 2.0f * t );
}
__device__ __forceinline__ float3 f3( float x, float y, float z ) { return make_float3( x, y, z ); }
__device__ __forceinline__ float3 add( float3 a, float3 b ) { return f3( a.x + b.x, a.y + b.y, a.z + b.z ); }
__device__ __forceinline__ float3 sub( float3 a, float3 b ) { return f3( a.x - b.x, a.y - b.y, a.z - b.z ); }
__device__ __forceinline__ float3 mul( float3 a, float3 b ) { return f3( a.x * b.x, a.y * b.y, a.z * b.z ); }
__device__ __forceinline__ float3 mul( float3 a, float s ) { return f3( a.x * s, a.y * s, a.z * s ); }
__device__ __forceinline__ float3 divs( float3 a, float s ) { return f3( a.x / s, a.y / s, a.z / s ); }
__device__ __forceinline__ float3 vmix( float3 x, float3 y, float a ) { return f3( gmix( x.x, y.x, a ), gmix( x.y, y.y, a ), gmix( x.z, y.z, a ) ); }
__device__ __forceinline__ float3 vmin( float3 a, float3 b ) { return f3( fminf( a.x, b.x ), fminf( a.y, b.y ), fminf( a.z, b.z ) ); }
__device__ __forceinline__ float3 vmax( float3 a, float3 b ) { return f3( fmaxf( a.x, b.x ), fmaxf( a.y, b.y ), fmaxf( a.z, b.z ) ); }
__device__ __forceinline__ float  dot3( float3 a, float3 b ) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 normalize3( float3 v )
{
    float l = sqrtf( dot3( v, v ) );
    return f3( v.x / l, v.y / l, v.z / l );
}
// Utils.h:54-57
__device__ __forceinline__ float luminance( float3 c ) { return 0.2125f * c.x + 0.7154f * c.y + 0.0721f * c.z; }

// column-major mat4 * vec4
__device__ __forceinline__ float4 mat_mul( const float* m, float4 v )
{
    return make_float4( m[ 0 ] * v.x + m[ 4 ] * v.y + m[ 8 ] * v.z + m[ 12 ] * v.w,
                        m[ 1 ] * v.x + m[ 5 ] * v.y + m[ 9 ] * v.z + m[ 13 ] * v.w,
                        m[ 2 ] * v.x + m[ 6 ] * v.y + m[ 10 ] * v.z + m[ 14 ] * v.w,
                        m[ 3 ] * v.x + m[ 7 ] * v.y + m[ 11 ] * v.z + m[ 15 ] * v.w );
}

__device__ __forceinline__ float h2f( uint16_t h ) { return f16_to_f32( h ); }
__device__ __forceinline__ float b2f( uint16_t h ) { return bf16_to_f32( h ); }

__device__ __forceinline__ bool inside( const Uniform& u, int x, int y ) { return x >= 0 && y >= 0 && x < u.W && y < u.H; }
__device__ __forceinline__ size_t idx( const Uniform& u, int x, int y ) { return (size_t)y * (size_t)u.W + (size_t)x; }

// Utils.h:124-140 through the decode tables
__device__ __forceinline__ float3 decode_normal( const FrameArgs& a, uint32_t p )
{
    const float2 ph = __ldg( &a.phiTab[ p >> 16 ] );
    const float2 th = __ldg( &a.thetaTab[ p & 0xFFFFu ] );
    return f3( ph.x * th.x, ph.x * th.y, ph.y );
}

// Geometry record (fused path): decoded normal + raw depth (fp16 bits) + metallic-roughness (rg8)
// — exactly the values the separate images decode to, fetched with one 16-byte load.
struct Geo
{
    float3   n;
    uint32_t bits;   // depth fp16 | mr << 16
};
__device__ __forceinline__ float4 geo_pack( float3 n, uint16_t depthBits, uint16_t mr )
{
    return make_float4( n.x, n.y, n.z, __uint_as_float( (uint32_t)depthBits | ( (uint32_t)mr << 16 ) ) );
}
__device__ __forceinline__ Geo geo_load( const float4* g, int i )
{
    const float4 r = g[ i ];
    return { make_float3( r.x, r.y, r.z ), __float_as_uint( r.w ) };
}
// the record of an all-zero texel (outside the image): normal code 0 decodes to (0, 0, 1)
__device__ __forceinline__ Geo geo_zero() { return { make_float3( 0.0f, 0.0f, 1.0f ), 0u }; }
__device__ __forceinline__ float geo_depth( const Geo& g ) { return __half2float( __ushort_as_half( (uint16_t)( g.bits & 0xFFFFu ) ) ); }
__device__ __forceinline__ uint32_t geo_rough8( const Geo& g ) { return g.bits >> 24; }
__device__ __forceinline__ uint32_t geo_metal8( const Geo& g ) { return ( g.bits >> 16 ) & 0xFFu; }

__device__ __forceinline__ float3 e5( uint32_t p )
{
    rgdn::f3 c = decode_e5( p );
    return make_float3( c.x, c.y, c.z );
}

// Math policy of the continuous weights. EXACT follows the shader expressions in IEEE binary32;
// FAST replaces only functions whose results feed continuous weights (no threshold follows):
// pow(x,128) by seven squarings, pow(x,y) by exp2(y*log2(x)) with an accurate log2 and the
// hardware exp2, exp by the hardware exp2, divisions by reciprocal multiplies, and fused
// multiply-adds in the sums. Every deviation is a few ulp of a weight.
__device__ __forceinline__ float ex2_approx( float x )
{
    float r;
    asm( "ex2.approx.ftz.f32 %0, %1;" : "=f"( r ) : "f"( x ) );
    return r;
}
__device__ __forceinline__ float lg2_approx( float x )
{
    float r;
    asm( "lg2.approx.ftz.f32 %0, %1;" : "=f"( r ) : "f"( x ) );
    return r;
}
__device__ __forceinline__ float rcp_approx( float x )
{
    float r;
    asm( "rcp.approx.ftz.f32 %0, %1;" : "=f"( r ) : "f"( x ) );
    return r;
}
__device__ __forceinline__ float sqrt_approx( float x )
{
    float r;
    asm( "sqrt.approx.ftz.f32 %0, %1;" : "=f"( r ) : "f"( x ) );
    return r;
}
template< bool FAST > struct Wm;
template<> struct Wm< false >
{
    __device__ static float  mix( float x, float y, float a ) { return gmix( x, y, a ); }
    __device__ static float3 vmix( float3 x, float3 y, float a ) { return ::rgdn::dev::vmix( x, y, a ); }
    __device__ static float pow128( float x ) { return powf( x, 128.0f ); }
    __device__ static float powv( float x, float y ) { return powf( x, y ); }
    __device__ static float pow01( float x, float y ) { return powf( x, y ); }
    __device__ static float expn( float x ) { return expf( x ); }
    __device__ static float madd( float a, float b, float c ) { return a * b + c; }
    __device__ static float lum( float3 c ) { return luminance( c ); }
    __device__ static float dot( float3 a, float3 b ) { return dot3( a, b ); }
    __device__ static float one_minus( float k, float x ) { return 1.0f - k * x; }
};
template<> struct Wm< true >
{
    __device__ static float pow128( float x )
    {
        x = x * x; x = x * x; x = x * x; x = x * x; x = x * x; x = x * x; x = x * x;
        return x;
    }
    __device__ static float powv( float x, float y ) { return ex2_approx( y * log2f( x ) ); }
    // x^y for x in [0, 1], y > 0: near 1 (d = 1 - x < 1/16, exact) ln x = -(d + d^2/2 + d^3/3 +
    // d^4/4 + d^5/5) to 1e-8 absolute; elsewhere the accurate log2
    __device__ static float pow01( float x, float y )
    {
        const float d = 1.0f - x;
        if( d < 0.0625f )
        {
            const float p  = __fmaf_rn( d, __fmaf_rn( d, __fmaf_rn( d, __fmaf_rn( d, 0.2f, 0.25f ), 0.33333334f ), 0.5f ), 1.0f );
            return ex2_approx( y * ( -d * p ) * 1.44269504088896341f );
        }
        return ex2_approx( y * log2f( x ) );
    }
    __device__ static float expn( float x ) { return ex2_approx( x * 1.44269504088896341f ); }
    __device__ static float madd( float a, float b, float c ) { return __fmaf_rn( a, b, c ); }
    // x + a (y - x)
    __device__ static float  mix( float x, float y, float a ) { return __fmaf_rn( a, y - x, x ); }
    __device__ static float3 vmix( float3 x, float3 y, float a ) { return f3( mix( x.x, y.x, a ), mix( x.y, y.y, a ), mix( x.z, y.z, a ) ); }
    // luminance and dot products as fused multiply-add chains
    __device__ static float lum( float3 c ) { return __fmaf_rn( 0.0721f, c.z, __fmaf_rn( 0.7154f, c.y, 0.2125f * c.x ) ); }
    __device__ static float dot( float3 a, float3 b ) { return __fmaf_rn( a.z, b.z, __fmaf_rn( a.y, b.y, a.x * b.x ) ); }
    // 1 - k * x
    __device__ static float one_minus( float k, float x ) { return __fmaf_rn( -k, x, 1.0f ); }
};

// ------------------------------------------------------------------------------------------
// Storage policy: element types of the colour / history images per mode
// ------------------------------------------------------------------------------------------
template< int M > struct Sto;

// the reference formats (GenerateShaderCommon.py:826-847)
template<> struct Sto< MODE_REF >
{
    static constexpr bool varPlane = false;
    __device__ static float3 ld3( const void* p, size_t i ) { return e5( static_cast< const uint32_t* >( p )[ i ] ); }
    __device__ static void   st3( void* p, size_t i, float3 v ) { static_cast< uint32_t* >( p )[ i ] = encode_e5( v.x, v.y, v.z ); }
    __device__ static float4 ldcv( const void* p, const float*, size_t i )
    {
        ushort4 h = static_cast< const ushort4* >( p )[ i ];
        return make_float4( h2f( h.x ), h2f( h.y ), h2f( h.z ), h2f( h.w ) );
    }
    // the same values through read-only global loads (ld.global.nc: free to move past shared stores)
    __device__ static float3 ld3_g( const void* p, size_t i ) { return e5( __ldg( static_cast< const uint32_t* >( p ) + i ) ); }
    __device__ static float4 ldcv_g( const void* p, const float*, size_t i )
    {
        const ushort4 h = __ldg( static_cast< const ushort4* >( p ) + i );
        return make_float4( h2f( h.x ), h2f( h.y ), h2f( h.z ), h2f( h.w ) );
    }
    __device__ static void stcv( void* p, float*, size_t i, float3 c, float var )
    {
        static_cast< ushort4* >( p )[ i ] = make_ushort4( f32_to_f16( c.x ), f32_to_f16( c.y ), f32_to_f16( c.z ), f32_to_f16( var ) );
    }
    __device__ static float2 ld2( const void* p, size_t i )
    {
        ushort2 h = static_cast< const ushort2* >( p )[ i ];
        return make_float2( h2f( h.x ), h2f( h.y ) );
    }
    __device__ static void st2( void* p, size_t i, float2 v ) { static_cast< ushort2* >( p )[ i ] = make_ushort2( f32_to_f16( v.x ), f32_to_f16( v.y ) ); }
    __device__ static float4 ld4( const void* p, size_t i )
    {
        ushort4 h = static_cast< const ushort4* >( p )[ i ];
        return make_float4( h2f( h.x ), h2f( h.y ), h2f( h.z ), h2f( h.w ) );
    }
    __device__ static void st4( void* p, size_t i, float4 v )
    {
        static_cast< ushort4* >( p )[ i ] = make_ushort4( f32_to_f16( v.x ), f32_to_f16( v.y ), f32_to_f16( v.z ), f32_to_f16( v.w ) );
    }
    __device__ static float ld1( const void* p, size_t i ) { return h2f( static_cast< const uint16_t* >( p )[ i ] ); }
    __device__ static void  st1( void* p, size_t i, float v ) { static_cast< uint16_t* >( p )[ i ] = f32_to_f16( v ); }
    __device__ static void  stpre( void* p, size_t i, float3 v ) { static_cast< uint32_t* >( p )[ i ] = encode_b10g11r11( v.x, v.y, v.z ); }
    __device__ static float3 ldpre( const void* p, size_t i )
    {
        const rgdn::f3 c = decode_b10g11r11( static_cast< const uint32_t* >( p )[ i ] );
        return make_float3( c.x, c.y, c.z );
    }
    // a value stored in PreFinal's format and read back
    __device__ static float3 qpre( float3 v )
    {
        const rgdn::f3 c = decode_b10g11r11( encode_b10g11r11( v.x, v.y, v.z ) );
        return make_float3( c.x, c.y, c.z );
    }
};

template<> struct Sto< MODE_F32 >
{
    static constexpr bool varPlane = false;
    __device__ static float3 ld3( const void* p, size_t i ) { float4 v = static_cast< const float4* >( p )[ i ]; return f3( v.x, v.y, v.z ); }
    __device__ static void   st3( void* p, size_t i, float3 v ) { static_cast< float4* >( p )[ i ] = make_float4( v.x, v.y, v.z, 0.0f ); }
    __device__ static float4 ldcv( const void* p, const float*, size_t i ) { return static_cast< const float4* >( p )[ i ]; }
    __device__ static void   stcv( void* p, float*, size_t i, float3 c, float var ) { static_cast< float4* >( p )[ i ] = make_float4( c.x, c.y, c.z, var ); }
    __device__ static float3 ld3_g( const void* p, size_t i ) { const float4 v = __ldg( static_cast< const float4* >( p ) + i ); return f3( v.x, v.y, v.z ); }
    __device__ static float4 ldcv_g( const void* p, const float*, size_t i ) { return __ldg( static_cast< const float4* >( p ) + i ); }
    __device__ static float2 ld2( const void* p, size_t i ) { return static_cast< const float2* >( p )[ i ]; }
    __device__ static void   st2( void* p, size_t i, float2 v ) { static_cast< float2* >( p )[ i ] = v; }
    __device__ static float4 ld4( const void* p, size_t i ) { return static_cast< const float4* >( p )[ i ]; }
    __device__ static void   st4( void* p, size_t i, float4 v ) { static_cast< float4* >( p )[ i ] = v; }
    __device__ static float  ld1( const void* p, size_t i ) { return static_cast< const float* >( p )[ i ]; }
    __device__ static void   st1( void* p, size_t i, float v ) { static_cast< float* >( p )[ i ] = v; }
    __device__ static void   stpre( void* p, size_t i, float3 v ) { static_cast< float4* >( p )[ i ] = make_float4( v.x, v.y, v.z, 0.0f ); }
    __device__ static float3 ldpre( const void* p, size_t i ) { float4 v = static_cast< const float4* >( p )[ i ]; return f3( v.x, v.y, v.z ); }
    __device__ static float3 qpre( float3 v ) { return v; }
};

// 16-bit colour / history with FP32 moments, FP32 variance planes, FP32 prefiltered variance
template< bool BF > struct Sto16
{
    static constexpr bool varPlane = true;
    __device__ static float    cv( uint16_t h ) { return BF ? b2f( h ) : h2f( h ); }
    __device__ static uint16_t pk( float f ) { return BF ? f32_to_bf16( f ) : f32_to_f16( f ); }
    __device__ static float3 ld3( const void* p, size_t i ) { ushort4 h = static_cast< const ushort4* >( p )[ i ]; return f3( cv( h.x ), cv( h.y ), cv( h.z ) ); }
    __device__ static void   st3( void* p, size_t i, float3 v ) { static_cast< ushort4* >( p )[ i ] = make_ushort4( pk( v.x ), pk( v.y ), pk( v.z ), 0 ); }
    __device__ static float3 ld3_g( const void* p, size_t i )
    {
        const ushort4 h = __ldg( static_cast< const ushort4* >( p ) + i );
        return f3( cv( h.x ), cv( h.y ), cv( h.z ) );
    }
    __device__ static float4 ldcv_g( const void* p, const float* var, size_t i )
    {
        const ushort4 h = __ldg( static_cast< const ushort4* >( p ) + i );
        return make_float4( cv( h.x ), cv( h.y ), cv( h.z ), __ldg( var + i ) );
    }
    __device__ static float4 ldcv( const void* p, const float* var, size_t i )
    {
        ushort4 h = static_cast< const ushort4* >( p )[ i ];
        return make_float4( cv( h.x ), cv( h.y ), cv( h.z ), var[ i ] );
    }
    __device__ static void stcv( void* p, float* var, size_t i, float3 c, float v )
    {
        static_cast< ushort4* >( p )[ i ] = make_ushort4( pk( c.x ), pk( c.y ), pk( c.z ), 0 );
        var[ i ] = v;
    }
    __device__ static float2 ld2( const void* p, size_t i ) { return static_cast< const float2* >( p )[ i ]; }
    __device__ static void   st2( void* p, size_t i, float2 v ) { static_cast< float2* >( p )[ i ] = v; }
    __device__ static float4 ld4( const void* p, size_t i )
    {
        ushort4 h = static_cast< const ushort4* >( p )[ i ];
        return make_float4( cv( h.x ), cv( h.y ), cv( h.z ), cv( h.w ) );
    }
    __device__ static void st4( void* p, size_t i, float4 v ) { static_cast< ushort4* >( p )[ i ] = make_ushort4( pk( v.x ), pk( v.y ), pk( v.z ), pk( v.w ) ); }
    __device__ static float ld1( const void* p, size_t i ) { return static_cast< const float* >( p )[ i ]; }
    __device__ static void  st1( void* p, size_t i, float v ) { static_cast< float* >( p )[ i ] = v; }
    // PreFinal is rgba16f in both 16-bit modes
    __device__ static void stpre( void* p, size_t i, float3 v )
    {
        static_cast< ushort4* >( p )[ i ] = make_ushort4( f32_to_f16( v.x ), f32_to_f16( v.y ), f32_to_f16( v.z ), 0 );
    }
    __device__ static float3 ldpre( const void* p, size_t i )
    {
        const ushort4 h = static_cast< const ushort4* >( p )[ i ];
        return f3( h2f( h.x ), h2f( h.y ), h2f( h.z ) );
    }
    __device__ static float3 qpre( float3 v ) { return f3( h2f( f32_to_f16( v.x ) ), h2f( f32_to_f16( v.y ) ), h2f( f32_to_f16( v.z ) ) ); }
};
template<> struct Sto< MODE_F16 > : Sto16< false > {};
template<> struct Sto< MODE_BF16 > : Sto16< true > {};

// zero-texel-outside-the-image loads of the mode-dependent images
template< int M > __device__ __forceinline__ float3 ld3z( const FrameArgs& a, const void* p, int x, int y )
{
    return inside( a.u, x, y ) ? Sto< M >::ld3( p, idx( a.u, x, y ) ) : f3( 0, 0, 0 );
}
template< int M > __device__ __forceinline__ float4 ldcvz( const FrameArgs& a, const void* p, const float* var, int x, int y )
{
    return inside( a.u, x, y ) ? Sto< M >::ldcv( p, var, idx( a.u, x, y ) ) : make_float4( 0, 0, 0, 0 );
}
__device__ __forceinline__ float ld_depth( const FrameArgs& a, const uint16_t* p, int x, int y )
{
    return inside( a.u, x, y ) ? h2f( p[ idx( a.u, x, y ) ] ) : 0.0f;
}
__device__ __forceinline__ uint32_t ld_u32( const FrameArgs& a, const uint32_t* p, int x, int y )
{
    return inside( a.u, x, y ) ? p[ idx( a.u, x, y ) ] : 0u;
}
__device__ __forceinline__ float ld_rough( const FrameArgs& a, int x, int y )
{
    return inside( a.u, x, y ) ? unorm8_to_f32( a.mr[ idx( a.u, x, y ) ] >> 8 ) : 0.0f;
}

// ------------------------------------------------------------------------------------------
// checkerboard helpers (ShaderCommonGLSLFunc.h:306-366)
// ------------------------------------------------------------------------------------------
struct Area
{
    int l, r, h;
};
__device__ __forceinline__ Area cb_area( const Uniform& u, int cx )
{
    const int sep   = u.W / 2;
    const int isOdd = cx >= sep ? 1 : 0;
    return { isOdd * sep, ( isOdd + 1 ) * sep, u.H };
}
__device__ __forceinline__ bool in_area( int x, int y, Area a ) { return y >= 0 && y < a.h && x >= a.l && x < a.r; }
__device__ __forceinline__ int2 regular_from_cb( const Uniform& u, int cx, int cy )
{
    const int sep   = u.W / 2;
    const int isOdd = cx >= sep ? 1 : 0;
    const int x     = cx - isOdd * sep;
    return make_int2( x * 2 + ( isOdd + cy ) % 2, cy );
}
// ShaderCommonGLSLFunc.h:271-277
__device__ __forceinline__ float2 prev_screen_pos( const Uniform& u, float2 m, int px, int py )
{
    const float sx = u.rw / 2.0f, sy = u.rh;
    // u.isx = 1 / sx and u.isy = 1 / sy, divided once on the host (IEEE, the same bits)
    return make_float2( ( ( (float)px + 0.5f ) * u.isx + m.x ) * sx, ( ( (float)py + 0.5f ) * u.isy + m.y ) * sy );
}
// ShaderCommonGLSLFunc.h:368-390
__device__ __forceinline__ bool test_depth( float z, float zPrev, float zMotion ) { return fabsf( z - zPrev + zMotion ) / fabsf( z ) < 0.1f; }
__device__ __forceinline__ bool test_normal( float3 n, float3 np ) { return dot3( n, np ) > 0.95f; }
// test_depth's decision from rz = rcp.approx(|z|) (relative error below 2^-22): the product
// n * rz lies within 2^-21 (relative) of the quotient n / |z|, so outside a band of 1e-6
// (relative) around 0.1 it decides as the rounded quotient would; inside the band, and for
// NaN, the IEEE quotient decides.
__device__ __forceinline__ bool test_depth_r( float z, float rz, float zPrev, float zMotion )
{
    const float n = fabsf( z - zPrev + zMotion );
    const float t = n * rz;
    if( t < 0.0999999f ) return true;
    if( t > 0.1000001f ) return false;
    return n / fabsf( z ) < 0.1f;
}
__device__ __forceinline__ float antilag( float g, float nf )
{
    float lambda = nf > 0.0001f ? gclamp( fabsf( g ) / nf, 0.0f, 1.0f ) : 0.0f;
    return gclamp( lambda, 0.0f, 1.0f );
}

__device__ __forceinline__ float4 unpack_rgba8( uint32_t c )
{
    return make_float4( unorm8_to_f32( c & 0xFFu ), unorm8_to_f32( ( c >> 8 ) & 0xFFu ), unorm8_to_f32( ( c >> 16 ) & 0xFFu ),
                        unorm8_to_f32( c >> 24 ) );
}
__device__ __forceinline__ uint32_t pack_rgba8( float x, float y, float z, float w )
{
    return f32_to_unorm8( x ) | ( f32_to_unorm8( y ) << 8 ) | ( f32_to_unorm8( z ) << 16 ) | ( f32_to_unorm8( w ) << 24 );
}
__device__ __forceinline__ float4 ld_rgba8z( const Uniform& u, const uint32_t* p, int x, int y )
{
    return ( x >= 0 && y >= 0 && x < u.GW && y < u.GH ) ? unpack_rgba8( p[ (size_t)y * u.GW + x ] ) : make_float4( 0, 0, 0, 0 );
}

// ==========================================================================================
// RtGradients.rgen:44-181 — image-space part of the gradient samples, one stratum
// ==========================================================================================
// unorm8 -> float through a table of the exact values u / 255
__device__ __forceinline__ float4 unpack_rgba8_t( uint32_t c, const float* u8 )
{
    return make_float4( u8[ c & 0xFFu ], u8[ ( c >> 8 ) & 0xFFu ], u8[ ( c >> 16 ) & 0xFFu ], u8[ c >> 24 ] );
}
__device__ __forceinline__ float4 ld_rgba8t( const Uniform& u, const uint32_t* p, int x, int y, const float* u8 )
{
    return ( x >= 0 && y >= 0 && x < u.GW && y < u.GH ) ? unpack_rgba8_t( p[ y * u.GW + x ], u8 ) : make_float4( 0, 0, 0, 0 );
}

// murmurHash33 (Random.h:280-287), the published MurmurHash2 mixing on three lanes
__device__ __forceinline__ uint3 murmur_hash33( uint3 src )
{
    const uint32_t M = 0x5bd1e995u;
    uint3          h = make_uint3( 1190494759u, 2147483647u, 3559788179u );
    src              = make_uint3( src.x * M, src.y * M, src.z * M );
    src              = make_uint3( src.x ^ ( src.x >> 24 ), src.y ^ ( src.y >> 24 ), src.z ^ ( src.z >> 24 ) );
    src              = make_uint3( src.x * M, src.y * M, src.z * M );
    auto mulx        = [ & ]( uint32_t k ) {
        h = make_uint3( h.x * M, h.y * M, h.z * M );
        h = make_uint3( h.x ^ k, h.y ^ k, h.z ^ k );
    };
    mulx( src.x );
    mulx( src.y );
    mulx( src.z );
    h = make_uint3( h.x ^ ( h.x >> 13 ), h.y ^ ( h.y >> 13 ), h.z ^ ( h.z >> 13 ) );
    h = make_uint3( h.x * M, h.y * M, h.z * M );
    return make_uint3( h.x ^ ( h.x >> 15 ), h.y ^ ( h.y >> 15 ), h.z ^ ( h.z >> 15 ) );
}
// Chris Wellons' lowbias32 (Random.h:243-251)
__device__ __forceinline__ uint32_t wellons_lowbias32( uint32_t x )
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
// getRandomSeed + packRandomSeed (Random.h:202-208, 289-300): 128 blue-noise layers of 128x128
__device__ __forceinline__ uint32_t random_seed( int px, int py, uint32_t frame )
{
    const uint3 h = murmur_hash33( make_uint3( (uint32_t)px, (uint32_t)py, frame ) );
    return ( ( h.z % 128u ) << 14 ) | ( ( h.y % 128u ) << 7 ) | ( h.x % 128u );
}

// ------------------------------------------------------------------------------------------
// Gradient re-shading (RtGradients.rgen:107-136): the previous frame's surface at a gradient
// sample, lit again by this frame's lights with the previous frame's reservoir and random seed.
// The light sample, the BRDF and the sample weight follow the shaders in IEEE binary32 and in
// their expression order; the shadow ray runs against the analytic occluders.
// ------------------------------------------------------------------------------------------
constexpr float kPi = 3.14159265358979323846f;   // M_PI (Utils.h:26)

// Utils.h:69-72, 142-146, Light.h:140-151
__device__ __forceinline__ float safe_positive_rcp( float f ) { return f <= 0.0f ? 0.0f : 1.0f / f; }
__device__ __forceinline__ float3 safe_normalize( float3 v )
{
    const float len = sqrtf( dot3( v, v ) );
    return len > 0.001f ? divs( v, len ) : f3( 0.0f, 1.0f, 0.0f );
}
__device__ __forceinline__ float safe_solid_angle( float a ) { return a > 0.0f && !isnan( a ) && !isinf( a ) ? gclamp( a, 0.0f, 4.0f * kPi ) : 0.0f; }
__device__ __forceinline__ float solid_angle_sphere( float radius, float dist )
{
    const float sinTheta = radius / fmaxf( radius, dist );
    const float cosTheta = sqrtf( 1.0f - sinTheta * sinTheta );
    return safe_solid_angle( 2.0f * kPi * ( 1.0f - cosTheta ) );
}
// sampleOrientedHemisphere (Random.h:175-201), the direction only
__device__ __forceinline__ float3 oriented_hemisphere( float3 n, float u1, float u2 )
{
    float       a   = 1.0f - 2.0f * u1;
    float       b   = sqrtf( 1.0f - a * a );
    const float phi = 2.0f * kPi * u2;
    a               = a * 0.98f;
    b               = b * 0.98f;
    return normalize3( f3( n.x + b * cosf( phi ), n.y + b * sinf( phi ), n.z + a ) );
}
// evalBRDFSmithGGX (BRDF.h:116-146) with D_GGX (BRDF.h:87-101) and getFresnelSchlick (BRDF.h:73-76)
__device__ __forceinline__ float3 brdf_smith_ggx( float3 n, float3 v, float3 l, float alpha, float3 specColor )
{
    alpha          = fmaxf( alpha, 0.005f );
    const float nl = fmaxf( dot3( n, l ), 0.0f );
    if( nl <= 0.0f ) return f3( 0.0f, 0.0f, 0.0f );
    const float  fr = powf( 1.0f - fmaxf( nl, 0.0f ), 5.0f );
    const float3 F  = f3( specColor.x + ( 1.0f - specColor.x ) * fr, specColor.y + ( 1.0f - specColor.y ) * fr,
                          specColor.z + ( 1.0f - specColor.z ) * fr );
    const float3 h       = normalize3( add( v, l ) );
    const float  alphaSq = alpha * alpha;
    const float  nm      = fmaxf( 0.0f, dot3( n, h ) );
    const float  dd      = nm * nm * ( alphaSq - 1.0f ) + 1.0f;
    const float  D       = alphaSq / kPi / ( dd * dd );
    const float  nv      = fmaxf( dot3( n, v ), 0.0f );
    const float  G2      = 0.5f / gmix( 2.0f * nl * nv, nl + nv, alpha );
    return mul( F, G2 * D );
}
// traceShadowRay (RaygenCommon.h:322-348) against the occluders: tMin 0.001, tMax the distance
// to the light point minus SHADOW_RAY_EPS (0.01)
__device__ __forceinline__ bool shadowed( const rgdn_reshade_scene& sc, float3 start, float3 end )
{
    float3      l           = sub( end, start );
    const float maxDistance = sqrtf( dot3( l, l ) );
    l                       = divs( l, maxDistance );
    const float tmin = 0.001f, tmax = maxDistance - 0.01f;
    for( uint32_t k = 0; k < sc.occluderCount; k++ )
    {
        const rgdn_occluder o = sc.occluders[ k ];
        if( o.type == RGDN_OCCLUDER_SPHERE )
        {
            const float3 oc   = sub( start, f3( o.data[ 0 ], o.data[ 1 ], o.data[ 2 ] ) );
            const float  b    = dot3( oc, l );
            const float  c    = dot3( oc, oc ) - o.data[ 3 ] * o.data[ 3 ];
            const float  disc = b * b - c;
            if( disc <= 0.0f ) continue;
            const float sq = sqrtf( disc );
            const float t0 = -b - sq, t1 = -b + sq;
            if( ( t0 >= tmin && t0 <= tmax ) || ( t1 >= tmin && t1 <= tmax ) ) return true;
        }
        else if( o.type == RGDN_OCCLUDER_RECT )
        {
            const int   ax = (int)o.data[ 0 ];
            const float so = ax == 0 ? start.x : ax == 1 ? start.y : start.z;
            const float dl = ax == 0 ? l.x : ax == 1 ? l.y : l.z;
            if( dl == 0.0f ) continue;
            const float t = ( o.data[ 1 ] - so ) / dl;
            if( !( t >= tmin && t <= tmax ) ) continue;
            const float3 q  = add( start, mul( l, t ) );
            const float  u0 = ax == 0 ? q.y : q.x, u1 = ax == 2 ? q.y : q.z;
            if( u0 >= o.data[ 2 ] && u0 <= o.data[ 3 ] && u1 >= o.data[ 4 ] && u1 <= o.data[ 5 ] ) return true;
        }
    }
    return false;
}
// forwardProjectedLuminance of the previous frame's pixel pp (checkerboard layout)
__device__ __forceinline__ float2 reshade_px( const FrameArgs& a, const int2 pp, const float* u8 )
{
    const Uniform&            u  = a.u;
    const rgdn_reshade_scene& sc = *a.rs;
    const int                 pi = pp.y * u.W + pp.x;
    const uint4               rv = a.reservoirsPrev[ pi ];
    const uint32_t            selectedPrev = rv.x & 65535u, Mres = ( rv.x >> 16 ) & 65535u;
    // isReservoirValid, then lightSources_Index_PrevToCur
    if( selectedPrev == 32767u || selectedPrev >= sc.prevLightCount ) return make_float2( 0.0f, 0.0f );
    const uint32_t sel = sc.prevToCur[ selectedPrev ];
    if( sel == 0xFFFFFFFFu || sel >= sc.lightCount ) return make_float2( 0.0f, 0.0f );
    // fetchGbufferSurface_NoAlbedoViewDir_Prev (Surface.inl:72-90) + the toViewerDir fix-up
    const float4   sp4  = a.surfPosPrev[ pi ];
    const float3   pos  = f3( sp4.x, sp4.y, sp4.z );
    const uint16_t mrb  = a.mrPrev[ pi ];
    const float    metallic = u8[ mrb & 0xFFu ], roughness = u8[ mrb >> 8 ];
    const float    spc  = 0.04f * ( 1.0f - metallic ) + 1.0f * metallic;   // getSpecularColor(1, metallic)
    const float3   n    = decode_normal( a, a.normalPrev[ pi ] );
    const float3   v    = normalize3( sub( f3( u.camPosPrev[ 0 ], u.camPosPrev[ 1 ], u.camPosPrev[ 2 ] ), pos ) );
    // getRandomSeed(prevShadingPix, frameId - 1), getLightPointRnd (RaygenCommon.h:624-627)
    const uint32_t seed = random_seed( pp.x, pp.y, u.frameId - 1u );
    const uint32_t rnd  = wellons_lowbias32( seed + 20u );   // RANDOM_SALT_LIGHT_POINT
    const float    r1   = (float)( rnd & 0xFFFFu ) / 65535.0f * 0.99f;
    const float    r2   = (float)( ( rnd & 0xFFFF0000u ) >> 16 ) / 65535.0f * 0.99f;
    // sampleSphereLight (Light.h:244-258)
    const rgdn_sphere_light L  = sc.lights[ sel ];
    const float3            c  = f3( L.center[ 0 ], L.center[ 1 ], L.center[ 2 ] );
    float3                  tc = sub( c, pos );
    const float             tl = sqrtf( dot3( tc, tc ) );
    tc                         = divs( tc, tl );
    const float3 ln            = oriented_hemisphere( f3( -tc.x, -tc.y, -tc.z ), r1, r2 );
    const float3 lpos          = add( c, mul( ln, L.radius ) );
    const float  dw            = solid_angle_sphere( L.radius, tl );
    const float3 col           = f3( L.color[ 0 ], L.color[ 1 ], L.color[ 2 ] );
    // shade (RaygenCommon.h:364-380) with calcSelectedSampleWeight (Reservoir.h:47-50)
    const float3 l  = safe_normalize( sub( lpos, pos ) );
    const float  nl = dot3( n, l );
    if( nl <= 0.0f ) return make_float2( 0.0f, 0.0f );
    const float  w    = safe_positive_rcp( __uint_as_float( rv.y ) ) * ( __uint_as_float( rv.z ) / (float)max( 1u, Mres ) );
    const float3 base = mul( col, dw * nl );
    float3       dif  = mul( mul( base, 1.0f / kPi ), w );
    float3       spe  = mul( mul( base, brdf_smith_ggx( n, v, l, roughness, f3( spc, spc, spc ) ) ), w );
    if( luminance( add( dif, spe ) ) <= 0.0f ) return make_float2( 0.0f, 0.0f );
    // traceVisibility (RaygenCommon.h:350-359): from the surface moved towards the viewer
    if( shadowed( sc, add( pos, mul( v, 0.01f ) ), lpos ) ) return make_float2( 0.0f, 0.0f );
    return make_float2( luminance( dif ), luminance( spe ) );
}

template< int M >
__device__ __forceinline__ void gradient_sample_px( const FrameArgs& a, uint32_t* dst, const int gx, const int gy, const float* u8 )
{
    const Uniform& u  = a.u;
    const int      gi = gy * u.GW + gx;
    if( u.gradMultD < 0.001f && u.gradMultI < 0.001f && u.gradMultS < 0.001f )
    {
        dst[ gi ]           = 0u;
        a.gradPrevPix[ gi ] = STRATA * STRATA + 1;
        return;
    }
    const uint32_t prevStrataPos = a.gradPrevPix[ gi ];
    // the 9 stratum positions: motion first, then the previous frame's luminance at the
    // forward-projected pixel (two rounds of independent loads instead of 18 in sequence)
    int2   ipos[ STRATA * STRATA ];
    float2 ilum[ STRATA * STRATA ];
#pragma unroll
    for( int k = 0; k < STRATA * STRATA; k++ )
    {
        const int cx = gx * STRATA + k % STRATA, cy = gy * STRATA + k / STRATA;
        float2    m  = make_float2( 0, 0 );
        if( inside( u, cx, cy ) )
        {
            const ushort4 mo = a.motion[ cy * u.W + cx ];
            m                = make_float2( h2f( mo.x ), h2f( mo.y ) );
        }
        const float2 pp = prev_screen_pos( u, m, cx, cy );
        ipos[ k ]       = make_int2( (int)floorf( pp.x ), (int)floorf( pp.y ) );
    }
#pragma unroll
    for( int k = 0; k < STRATA * STRATA; k++ )
    {
        float2 il = make_float2( 0, 0 );
        if( inside( u, ipos[ k ].x, ipos[ k ].y ) )
        {
            const uint32_t g = a.gradInputsPrev[ ipos[ k ].y * u.W + ipos[ k ].x ];
            il               = make_float2( h2f( (uint16_t)( g & 0xFFFFu ) ), h2f( (uint16_t)( g >> 16 ) ) );
        }
        ilum[ k ] = il;
    }
    int2     prevShadingPix = make_int2( 0, 0 ), curShadingPix = make_int2( 0, 0 );
    uint32_t curStrataPos   = 0;
    float2   prevLum        = make_float2( 0, 0 );
    // (a) the brightest sample of the stratum, skipping last frame's position (RtGradients.rgen:65-96)
#pragma unroll
    for( int k = 0; k < STRATA * STRATA; k++ )
    {
        if( (uint32_t)k == prevStrataPos ) continue;
        if( fmaxf( ilum[ k ].x, ilum[ k ].y ) > fmaxf( prevLum.x, prevLum.y ) )
        {
            prevShadingPix = ipos[ k ];
            curShadingPix  = make_int2( gx * STRATA + k % STRATA, gy * STRATA + k / STRATA );
            curStrataPos   = (uint32_t)k;
            prevLum        = ilum[ k ];
        }
    }
    const bool skyCur = inside( u, curShadingPix.x, curShadingPix.y ) && a.isSky[ curShadingPix.y * u.W + curShadingPix.x ] != 0;
    if( !in_area( prevShadingPix.x, prevShadingPix.y, cb_area( u, curShadingPix.x ) ) || skyCur ||
        ( prevLum.x <= 0.0f && prevLum.y <= 0.0f ) )
    {
        dst[ gi ]           = 0u;
        a.gradPrevPix[ gi ] = STRATA * STRATA + 1;
        return;
    }
    // in the render area, so inside the image
    const int    pi  = prevShadingPix.y * u.W + prevShadingPix.x;
    // the re-shaded luminance: computed here from the lights (RtGradients.rgen:107-136), or the
    // producer's image
    const float2 fpl = a.rs ? reshade_px( a, prevShadingPix, u8 ) : a.reshaded[ pi ];
    float g0, g1, g2;
    {
        const float gs = fpl.x - prevLum.x;
        const float nf = fmaxf( fpl.x, prevLum.x );
        g0             = antilag( gs, nf );
    }
    {
        float        gs         = fmaxf( 0.0f, prevLum.x - fpl.x );
        const float  nf         = fmaxf( fpl.x, prevLum.x );
        const float  brightness = luminance( Sto< M >::ld3( a.indirAccumPrev, (size_t)pi ) );
        gs = gs * ( 1.0f - gsmoothstep( 1.0f, 10.0f, brightness ) );
        g1 = antilag( gs, nf );
    }
    {
        const float gs = fpl.y - prevLum.y;
        const float nf = fmaxf( fpl.y, prevLum.y );
        g2             = antilag( gs, nf );
    }
    g0 = g0 * u.gradMultD;
    g1 = g1 * u.gradMultI;
    g2 = g2 * u.gradMultS;
    const float4 gp = ld_rgba8t( u, a.disHistPrev, prevShadingPix.x / STRATA, prevShadingPix.y / STRATA, u8 );
    g0 = gmix( g0, gp.x, 0.5f );
    g1 = gmix( g1, gp.y, 0.5f );
    g2 = gmix( g2, gp.z, 0.5f );
    dst[ gi ]           = pack_rgba8( g0, g1, g2, 0.0f );
    a.gradPrevPix[ gi ] = (uint8_t)curStrataPos;
}

// CmASVGFGradientAtrous.comp:42-105 — one iteration, one stratum, from `src` into `dst`
// (and `hist` on iteration 0), all GW x GH rgba8 images
// One filtered gradient texel (CmASVGFGradientAtrous.comp:42-95) from the packed rgba8 source
// texels that `fetch(qx, qy)` returns (0 outside the gradient image); returns it packed.
template< class Fetch >
__device__ __forceinline__ uint32_t gradient_atrous_texel( const Uniform& u, Fetch fetch, const int gx, const int gy, const int iter,
                                                           const float* u8 )
{
    const int   step = 1 << iter;
    const Area  a0   = cb_area( u, gx * STRATA );
    const Area  ga   = { a0.l / STRATA, a0.r / STRATA, a0.h / STRATA };
    const float kern[ 2 ][ 2 ] = { { 1.0f, 0.5f }, { 0.5f, 0.25f } };
    float3 out = f3( 0, 0, 0 );
    float  ws  = 0.0f;
#pragma unroll
    for( int yy = -1; yy <= 1; yy++ )
    {
#pragma unroll
        for( int xx = -1; xx <= 1; xx++ )
        {
            const int    qx = gx + xx * step, qy = gy + yy * step;
            const float4 g  = unpack_rgba8_t( fetch( qx, qy ), u8 );
            const float  w  = kern[ yy < 0 ? -yy : yy ][ xx < 0 ? -xx : xx ] * ( in_area( qx, qy, ga ) ? 1.0f : 0.0f );
            out = add( out, mul( f3( g.x, g.y, g.z ), w ) );
            ws  = ws + w;
        }
    }
    out = divs( out, ws );
    return pack_rgba8( out.x, out.y, out.z, 0.0f );
}

__device__ __forceinline__ void gradient_atrous_core( const Uniform& u, const uint32_t* src, uint32_t* dst, uint32_t* hist, const int gx,
                                                      const int gy, const int iter, const float* u8 )
{
    auto fetch = [ & ]( int x, int y ) { return ( x >= 0 && y >= 0 && x < u.GW && y < u.GH ) ? src[ y * u.GW + x ] : 0u; };
    const uint32_t packed = gradient_atrous_texel( u, fetch, gx, gy, iter, u8 );
    const int      gi     = gy * u.GW + gx;
    dst[ gi ] = packed;
    if( iter == 0 && hist ) hist[ gi ] = packed;
}

// the stream's ping-pong routing (CmASVGFGradientAtrous.comp:89-104)
__device__ __forceinline__ void gradient_atrous_px( const FrameArgs& a, const int gx, const int gy, const int iter, const float* u8 )
{
    const uint32_t* src = ( iter % 2 == 0 ) ? a.disPing : a.disPong;
    uint32_t*       dst = ( iter % 2 == 0 ) ? a.disPong : a.disPing;
    gradient_atrous_core( a.u, src, dst, a.disHist, gx, gy, iter, u8 );
}

// u / 255 for the 256 unorm8 codes, each the correctly rounded binary32 quotient: folded at
// compile time (IEEE division, as the device's) into a table in global memory, so a block fills
// its shared copy with loads instead of 256 divisions
struct U8Table
{
    float v[ 256 ];
};
constexpr U8Table make_u8_table()
{
    U8Table t{};
    for( int k = 0; k < 256; k++ ) t.v[ k ] = (float)k / 255.0f;
    return t;
}
static __device__ const U8Table g_u8 = make_u8_table();
__device__ __forceinline__ float u8_value( int k ) { return __ldg( &g_u8.v[ k ] ); }

__device__ __forceinline__ void fill_u8( float* u8, int t )
{
    u8[ t ] = u8_value( t );
}

// Programmatic dependent launch. Every kernel of the path lets its successor's blocks be
// scheduled once all of its own blocks have started (they then fill the SMs freed by this
// grid's last wave), and waits for its predecessor's grid to complete, with its writes visible,
// before the first global-memory access. Without a programmatic dependency both are no-ops.
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile( "griddepcontrol.launch_dependents;" ::: "memory" ); }
__device__ __forceinline__ void pdl_wait() { asm volatile( "griddepcontrol.wait;" ::: "memory" ); }

// Tile functions: one thread per pixel (or stratum) of the blockDim-sized tile (bx, by) of
// frame `a`. The single-frame kernels run one tile per block; the batched kernels loop a
// persistent block over the tiles of many frames.
template< int M > __device__ __forceinline__ void gradient_samples_tile( const FrameArgs& a, uint32_t* dst, int bx, int by, const float* u8 )
{
    const int gx = bx * blockDim.x + threadIdx.x;
    const int gy = by * blockDim.y + threadIdx.y;
    if( gx >= a.u.GW || gy >= a.u.GH || gx * STRATA >= a.u.W || gy * STRATA >= a.u.H ) return;
    gradient_sample_px< M >( a, dst, gx, gy, u8 );
}
__device__ __forceinline__ void gradient_atrous_tile( const FrameArgs& a, int iter, int bx, int by, const float* u8 )
{
    const int gx = bx * blockDim.x + threadIdx.x;
    const int gy = by * blockDim.y + threadIdx.y;
    if( gx >= a.u.GW || gy >= a.u.GH || gx * STRATA >= a.u.W || gy * STRATA >= a.u.H ) return;
    gradient_atrous_px( a, gx, gy, iter, u8 );
}

// The first kernel of a frame lets its dependents launch only after its own wait: every kernel
// enqueued before the frame has then completed, so the temporal pass that follows the gradient
// chain may read the frame's inputs and history before its own wait (k_temporal, EARLY).
template< int M > __global__ void __launch_bounds__( 256, 6 ) k_gradient_samples( const FrameArgs a, uint32_t* dst )
{
    __shared__ float u8[ 256 ];
    fill_u8( u8, threadIdx.y * blockDim.x + threadIdx.x );
    pdl_wait();
    pdl_launch_dependents();
    __syncthreads();
    gradient_samples_tile< M >( a, dst, blockIdx.x, blockIdx.y, u8 );
}

template< int M > __global__ void __launch_bounds__( 256 ) k_gradient_atrous( const FrameArgs a, const int iter )
{
    __shared__ float u8[ 256 ];
    pdl_launch_dependents();
    fill_u8( u8, threadIdx.y * blockDim.x + threadIdx.x );
    pdl_wait();
    __syncthreads();
    gradient_atrous_tile( a, iter, blockIdx.x, blockIdx.y, u8 );
}

// ==========================================================================================
// CmSVGFTemporalAccumulation.comp:57-384 — reprojection + temporal accumulation
// ==========================================================================================
__device__ __forceinline__ float spec_min_accum( const Uniform& u )
{
    const float td  = u.timeDelta;
    const float fps = td <= 0.0f ? 0.0f : 1.0f / td;
    return gclamp( 0.2f * fps, 0.0f, 128.0f );
}
template< bool FAST > __device__ __forceinline__ float spec_accum_speed( const Uniform& u, float Amax, float r, float NoV, float par )
{
    using X              = Wm< FAST >;
    const float acos01sq = 1.0f - NoV;
    const float aa       = X::powv( gsat( acos01sq ), 0.66f );
    const float b        = 1.1f + r * r;
    const float ps       = ( b + aa ) / ( b - aa );
    const float powScale = 1.0f + par * ps;
    float       f        = 1.0f - ( FAST ? ex2_approx( -200.0f * r * r ) : exp2f( -200.0f * r * r ) );
    f                    = f * X::powv( gsat( r ), 0.5f * powScale );
    const float A        = 256.0f * f;
    return gclamp( A, spec_min_accum( u ), Amax );
}
template< bool FAST > __device__ __forceinline__ float spec_dominant( float nv, float r )
{
    const float aa = 0.298475f * ( FAST ? __logf( 39.4115f - 39.0029f * r ) : logf( 39.4115f - 39.0029f * r ) );
    const float f  = Wm< FAST >::powv( gclamp( 1.0f - nv, 0.0f, 1.0f ), 10.8649f ) * ( 1.0f - aa ) + aa;
    return gclamp( f, 0.0f, 1.0f );
}
__device__ __forceinline__ float parallax( const Uniform& u, float3 pos, float3 posPrev )
{
    const float3 camDelta = f3( u.camPosPrev[ 0 ] - u.camPos[ 0 ], u.camPosPrev[ 1 ] - u.camPos[ 1 ], u.camPosPrev[ 2 ] - u.camPos[ 2 ] );
    const float3 v        = normalize3( pos );
    const float3 vPrev    = normalize3( sub( posPrev, camDelta ) );
    const float  cosa     = gsat( dot3( v, vPrev ) );
    const float  par      = sqrtf( 1.0f - cosa * cosa ) / fmaxf( cosa, 1e-6f );
    return par * 60.0f;
}

// FAST: continuous specular terms in hardware exp2/log2/sqrt, shared subexpressions, the
// precombined view-projection matrices, fused multiply-adds in the continuous sums and blends,
// the depth test through a reciprocal (exact near its threshold) and the history-length decay
// from the device table (the same bits as the inline powf). GEOM: write this frame's geometry
// record. GEOMPREV: read the previous frame's record (decoded normal + depth, the same values)
// at the taps.
// the temporal pass reads each in-area tap's history together with its geometry
constexpr bool kTemporalEarlyHistory = true;
// the temporal pass reads the surface positions before the taps rather than where they are used
constexpr bool kTemporalEarlySurfPos = false;
// the temporal pass prefetches the history rows under its bilinear footprint into L2 (once
// 4 % faster; with the geometry record persisting in L2 and the other later changes the pass ran
// 98.8 us without the prefetch against 102.4 with it, A/B/A/B on GB300)
constexpr bool kTemporalL2Prefetch = false;
// the temporal pass reads this frame's unfiltered colours and view ray before its taps
constexpr bool kTemporalEarlyInputs = true;
template< int M, bool FAST, bool GEOM, bool GEOMPREV, bool EARLY = false >
__device__ __forceinline__ void temporal_tile( const FrameArgs& a, int bx, int by, const float* u8 )
{
    using S          = Sto< M >;
    using X          = Wm< FAST >;
    const Uniform& u = a.u;
    const int      px = bx * blockDim.x + threadIdx.x;
    const int      py = by * blockDim.y + threadIdx.y;
    if( px >= u.W || py >= u.H ) return;
    const int i = py * u.W + px;

    // this frame's unfiltered colours and view ray, used only after the taps: read before them
    // (kTemporalEarlyInputs) or after them, so that they hold no registers across the tap loop
    float3 unfilteredDiff, unfilteredIndir, unfilteredSpec;
    float4 rayInfo;
    auto   ldInputs = [ & ]() {
        unfilteredDiff     = e5( a.unfD[ i ] );
        unfilteredIndir    = e5( a.unfI[ i ] );
        unfilteredSpec     = e5( a.unfS[ i ] );
        const ushort4 rv   = a.viewDir[ i ];
        rayInfo            = make_float4( h2f( rv.x ), h2f( rv.y ), h2f( rv.z ), h2f( rv.w ) );
    };
    if( kTemporalEarlyInputs ) ldInputs();
    const Area     chArea          = cb_area( u, px );
    const ushort4  mo              = a.motion[ i ];
    const float    motionZ         = h2f( mo.z );
    const uint16_t zBits           = a.depth[ i ];
    const float    z               = h2f( zBits );
    const float    rz              = FAST ? rcp_approx( fabsf( z ) ) : 0.0f;
    const float3   normal          = decode_normal( a, a.normal[ i ] );
    const uint16_t mrBits          = a.mr[ i ];
    const float    roughness       = u8[ mrBits >> 8 ];
    if( GEOM ) a.geom[ i ] = geo_pack( normal, zBits, mrBits );


    int2   pixPrev;
    float2 subPix;
    {
        const float2 posPrev = prev_screen_pos( u, make_float2( h2f( mo.x ), h2f( mo.y ) ), px, py );
        const float  fx = floorf( posPrev.x - 0.5f ), fy = floorf( posPrev.y - 0.5f );
        pixPrev = make_int2( (int)fx, (int)fy );
        subPix  = make_float2( ( posPrev.x - 0.5f ) - fx, ( posPrev.y - 0.5f ) - fy );
    }
    const float bw[ 2 ][ 2 ] = {
        { ( 1.0f - subPix.x ) * ( 1.0f - subPix.y ), subPix.x * ( 1.0f - subPix.y ) },
        { ( 1.0f - subPix.x ) * subPix.y, subPix.x * subPix.y },
    };
    // FAST: an L2 prefetch of the history rows under the bilinear footprint, so the history
    // loads that follow the reprojection tests find them on chip
    if( FAST && kTemporalL2Prefetch && pixPrev.x >= 0 && pixPrev.y >= 0 && pixPrev.x + 1 < u.W && pixPrev.y + 1 < u.H )
    {
        const TmaTexel tx = tma_texel( M == MODE_REF ? RGDN_STORAGE_REF : M == MODE_F32 ? RGDN_STORAGE_FP32 : RGDN_STORAGE_FP16 );
        const int      mb = M == MODE_REF ? 4 : 8;   // moments
#pragma unroll
        for( int r = 0; r < 2; r++ )
        {
            const size_t q = (size_t)( pixPrev.y + r ) * u.W + pixPrev.x;
            asm volatile( "prefetch.global.L2 [%0];" ::"l"( static_cast< const char* >( a.diffHistory ) + q * tx.cv ) );
            asm volatile( "prefetch.global.L2 [%0];" ::"l"( static_cast< const char* >( a.momentsPrev ) + q * mb ) );
            asm volatile( "prefetch.global.L2 [%0];" ::"l"( static_cast< const char* >( a.histLenPrev ) + q * tx.cv ) );
            asm volatile( "prefetch.global.L2 [%0];" ::"l"( static_cast< const char* >( a.specAccumPrev ) + q * tx.col ) );
            asm volatile( "prefetch.global.L2 [%0];" ::"l"( static_cast< const char* >( a.indirAccumPrev ) + q * tx.col ) );
            if( tx.var ) asm volatile( "prefetch.global.L2 [%0];" ::"l"( a.varHistory + q ) );
        }
    }
    // the surface positions the specular terms read once a tap is accepted: loaded with the
    // taps (kTemporalEarlySurfPos) or where they are used
    float4 sp4 = make_float4( 0, 0, 0, 0 ), spp4 = make_float4( 0, 0, 0, 0 );
    auto   ldSurf = [ & ]() {
        sp4  = a.surfPos[ i ];
        spp4 = inside( u, pixPrev.x, pixPrev.y ) ? a.surfPosPrev[ pixPrev.y * u.W + pixPrev.x ] : make_float4( 0, 0, 0, 0 );
    };
    if( kTemporalEarlySurfPos ) ldSurf();

    float4 histLenDIS     = make_float4( 0, 0, 0, 0 );
    float3 diffPrev       = f3( 0, 0, 0 );
    float2 momentsPrev    = make_float2( 0, 0 );
    float3 specPrevOnSurf = f3( 0, 0, 0 );
    float3 indirPrev      = f3( 0, 0, 0 );
    float  weightSum      = 0.0f;

#pragma unroll
    for( int yy = 0; yy <= 1; yy++ )
    {
#pragma unroll
        for( int xx = 0; xx <= 1; xx++ )
        {
            const int qx = pixPrev.x + xx, qy = pixPrev.y + yy;
            // in_area implies inside the image; a tap outside the area is rejected whatever
            // its texel holds
            if( !in_area( qx, qy, chArea ) ) continue;
            const int q = qy * u.W + qx;
            float     dP;
            float3    nP;
            if( GEOMPREV )
            {
                const Geo gp = geo_load( a.geomPrev, q );
                dP           = geo_depth( gp );
                nP           = gp.n;
            }
            else
            {
                dP = h2f( a.depthPrev[ q ] );
                nP = decode_normal( a, a.normalPrev[ q ] );
            }
            // FAST: the tap's history is read with its geometry, before the tests decide
            // whether it counts, so the two loads are in flight together
            float4 dc, hl;
            float2 m;
            float3 sp, ip;
            auto   ldHist = [ & ]() {
                dc = S::ldcv( a.diffHistory, a.varHistory, q );
                m  = S::ld2( a.momentsPrev, q );
                hl = S::ld4( a.histLenPrev, q );
                sp = S::ld3( a.specAccumPrev, q );
                ip = S::ld3( a.indirAccumPrev, q );
            };
            if( FAST && kTemporalEarlyHistory ) ldHist();
            const bool okDepth = FAST ? test_depth_r( z, rz, dP, motionZ ) : test_depth( z, dP, motionZ );
            if( okDepth && test_normal( normal, nP ) )
            {
                // FAST: fused multiply-adds for the continuous sums; the diffuse history length
                // (the variance pass switches on it) and the weight sum stay IEEE
                const float w = bw[ yy ][ xx ];
                if( !( FAST && kTemporalEarlyHistory ) ) ldHist();
                if constexpr( FAST )
                {
                    // the fourteen continuous sums as seven packed FP32 FMAs (the bits of the
                    // scalar FMAs)
                    const float2 ww = make_float2( w, w );
                    const float2 p0 = __ffma2_rn( make_float2( dc.x, dc.y ), ww, make_float2( diffPrev.x, diffPrev.y ) );
                    const float2 p1 = __ffma2_rn( make_float2( dc.z, m.x ), ww, make_float2( diffPrev.z, momentsPrev.x ) );
                    const float2 p2 = __ffma2_rn( make_float2( m.y, hl.y ), ww, make_float2( momentsPrev.y, histLenDIS.y ) );
                    const float2 p3 = __ffma2_rn( make_float2( hl.z, hl.w ), ww, make_float2( histLenDIS.z, histLenDIS.w ) );
                    const float2 p4 = __ffma2_rn( make_float2( sp.x, sp.y ), ww, make_float2( specPrevOnSurf.x, specPrevOnSurf.y ) );
                    const float2 p5 = __ffma2_rn( make_float2( sp.z, ip.x ), ww, make_float2( specPrevOnSurf.z, indirPrev.x ) );
                    const float2 p6 = __ffma2_rn( make_float2( ip.y, ip.z ), ww, make_float2( indirPrev.y, indirPrev.z ) );
                    diffPrev       = f3( p0.x, p0.y, p1.x );
                    momentsPrev    = make_float2( p1.y, p2.x );
                    histLenDIS     = make_float4( histLenDIS.x + w * hl.x, p2.y, p3.x, p3.y );
                    specPrevOnSurf = f3( p4.x, p4.y, p5.x );
                    indirPrev      = f3( p5.y, p6.x, p6.y );
                }
                else
                {
                    diffPrev       = f3( dc.x * w + diffPrev.x, dc.y * w + diffPrev.y, dc.z * w + diffPrev.z );
                    momentsPrev    = make_float2( w * m.x + momentsPrev.x, w * m.y + momentsPrev.y );
                    histLenDIS     = make_float4( histLenDIS.x + w * hl.x, w * hl.y + histLenDIS.y, w * hl.z + histLenDIS.z, w * hl.w + histLenDIS.w );
                    specPrevOnSurf = f3( w * sp.x + specPrevOnSurf.x, w * sp.y + specPrevOnSurf.y, w * sp.z + specPrevOnSurf.z );
                    indirPrev      = f3( w * ip.x + indirPrev.x, w * ip.y + indirPrev.y, w * ip.z + indirPrev.z );
                }
                weightSum = weightSum + w;
            }
        }
    }

    // the filtered gradients (unorm8) and, FAST, their history-length decay from the table
    float aD = 0.0f, aI = 0.0f, aS = 0.0f, decD = 1.0f, decI = 1.0f;
    // EARLY: the gradient chain that writes them is the only work this pass waits for
    if( EARLY ) pdl_wait();
    if( !( u.flags & RGDN_FLAG_SKIP_GRADIENTS ) )
    {
        const int      gx = px / STRATA, gy = py / STRATA;
        const uint32_t g  = ( gx < u.GW && gy < u.GH ) ? a.disPing[ gy * u.GW + gx ] : 0u;
        aD = u8[ g & 0xFFu ];
        aI = u8[ ( g >> 8 ) & 0xFFu ];
        aS = u8[ ( g >> 16 ) & 0xFFu ];
        if( FAST )
        {
            decD = __ldg( &a.decay10[ g & 0xFFu ] );
            decI = __ldg( &a.decay10[ ( g >> 8 ) & 0xFFu ] );
        }
    }

    if( !kTemporalEarlyInputs ) ldInputs();
    const float  l          = X::lum( unfilteredDiff );
    const float2 moments    = make_float2( l, l * l );
    const bool   hasHistory = weightSum > 0.0001f;
    // FAST: the one IEEE reciprocal both the continuous averages and the diffuse history
    // length use
    const float invWS = ( FAST && hasHistory ) ? 1.0f / weightSum : 0.0f;

    float3 specColorAccum;
    float  specHistoryLengthAccum, specHitDistanceAccum;

    if( hasHistory )
    {
        specPrevOnSurf                  = FAST ? mul( specPrevOnSurf, invWS ) : divs( specPrevOnSurf, weightSum );
        const float specHistoryLength   = FAST ? histLenDIS.z * invWS : histLenDIS.z / weightSum;
        const float specHitDistancePrev = FAST ? histLenDIS.w * invWS : histLenDIS.w / weightSum;

        if( !kTemporalEarlySurfPos ) ldSurf();
        const float3 surfPos     = f3( sp4.x, sp4.y, sp4.z );
        const float3 surfPosPrev = f3( spp4.x, spp4.y, spp4.z );
        const float nv = fmaxf( 0.0f, X::dot( normal, f3( -rayInfo.x, -rayInfo.y, -rayInfo.z ) ) );
        if constexpr( FAST )
        {
            const float td   = u.timeDelta;
            const float minA = gclamp( 0.2f * ( td <= 0.0f ? 0.0f : rcp_approx( td ) ), 0.0f, 128.0f );
            const float oma  = 1.0f - aS;
            const float A    = gclamp( 1.0f + specHistoryLength * ( oma * oma * oma * oma * oma ), minA, 256.0f );
            // getParallax (:58-69): normalize(pos) . normalize(posPrev - cameraDelta)
            const float3 camDelta = f3( u.camPosPrev[ 0 ] - u.camPos[ 0 ], u.camPosPrev[ 1 ] - u.camPos[ 1 ], u.camPosPrev[ 2 ] - u.camPos[ 2 ] );
            const float3 pp   = sub( surfPosPrev, camDelta );
            const float  cosa = gsat( X::dot( surfPos, pp ) * rsqrtf( X::dot( surfPos, surfPos ) ) * rsqrtf( X::dot( pp, pp ) ) );
            const float  par  = __fdividef( sqrt_approx( X::one_minus( cosa, cosa ) ), fmaxf( cosa, 1e-6f ) ) * 60.0f;
            // getSpecAccumSpeed (:80-92) for the surface and the virtual motion share every
            // term but the parallax
            const float aa = ex2_approx( 0.66f * __log2f( gsat( 1.0f - nv ) ) );
            const float b  = X::madd( roughness, roughness, 1.1f );
            const float ps = __fdividef( b + aa, b - aa );
            const float f0 = 1.0f - ex2_approx( -200.0f * roughness * roughness );
            const float lr = __log2f( gsat( roughness ) );
            const float AOnSurf = gclamp( 256.0f * ( f0 * ex2_approx( 0.5f * X::madd( par, ps, 1.0f ) * lr ) ), minA, A );
            // getSpecularDominantFactor (:93-99)
            const float da    = 0.298475f * __logf( X::madd( -39.0029f, roughness, 39.4115f ) );
            const float domin = gclamp( X::madd( ex2_approx( 10.8649f * __log2f( gclamp( 1.0f - nv, 0.0f, 1.0f ) ) ), 1.0f - da, da ), 0.0f, 1.0f );

            const float  invA          = __fdividef( 1.0f, 1.0f + AOnSurf );
            const float3 specOnSurf    = X::vmix( specPrevOnSurf, unfilteredSpec, invA );
            const float  hitDistOnSurf = X::mix( specHitDistancePrev, rayInfo.w, invA );
            specColorAccum         = specOnSurf;
            specHistoryLengthAccum = AOnSurf;
            specHitDistanceAccum   = hitDistOnSurf;

            const float  hd = hitDistOnSurf * domin;
            const float3 v  = f3( X::madd( rayInfo.x, hd, surfPos.x ), X::madd( rayInfo.y, hd, surfPos.y ), X::madd( rayInfo.z, hd, surfPos.z ) );
            // screen-space motion of the virtual position through proj*view (only x, y, w)
            const float* m  = u.vp;
            const float* mp = u.vpPrev;
            const float cxC = X::madd( m[ 0 ], v.x, X::madd( m[ 4 ], v.y, X::madd( m[ 8 ], v.z, m[ 12 ] ) ) );
            const float cyC = X::madd( m[ 1 ], v.x, X::madd( m[ 5 ], v.y, X::madd( m[ 9 ], v.z, m[ 13 ] ) ) );
            const float cwC = X::madd( m[ 3 ], v.x, X::madd( m[ 7 ], v.y, X::madd( m[ 11 ], v.z, m[ 15 ] ) ) );
            const float cxP = X::madd( mp[ 0 ], v.x, X::madd( mp[ 4 ], v.y, X::madd( mp[ 8 ], v.z, mp[ 12 ] ) ) );
            const float cyP = X::madd( mp[ 1 ], v.x, X::madd( mp[ 5 ], v.y, X::madd( mp[ 9 ], v.z, mp[ 13 ] ) ) );
            const float cwP = X::madd( mp[ 3 ], v.x, X::madd( mp[ 7 ], v.y, X::madd( mp[ 11 ], v.z, mp[ 15 ] ) ) );
            const float hC = 0.5f * rcp_approx( cwC ), hP = 0.5f * rcp_approx( cwP );
            // (ndcPrev * 0.5 + 0.5) - (ndcCur * 0.5 + 0.5)
            const float2 specMotion = make_float2( X::madd( cxP, hP, -cxC * hC ), X::madd( cyP, hP, -cyC * hC ) );
            const float2 spp = prev_screen_pos( u, specMotion, px, py );
            const float  fx = floorf( spp.x - 0.5f ), fy = floorf( spp.y - 0.5f );
            const int2   pixPrevS = make_int2( (int)fx, (int)fy );
            const float2 subPixS  = make_float2( ( spp.x - 0.5f ) - fx, ( spp.y - 0.5f ) - fy );
            float weightSumVirtual = 0.0f;
#pragma unroll
            for( int yy = 0; yy <= 1; yy++ )
            {
#pragma unroll
                for( int xx = 0; xx <= 1; xx++ )
                {
                    const int qx = pixPrevS.x + xx, qy = pixPrevS.y + yy;
                    if( !in_area( qx, qy, chArea ) ) continue;
                    const int q = qy * u.W + qx;
                    float     dP;
                    float3    nP;
                    if( GEOMPREV )
                    {
                        const Geo gp = geo_load( a.geomPrev, q );
                        dP           = geo_depth( gp );
                        nP           = gp.n;
                    }
                    else
                    {
                        dP = h2f( a.depthPrev[ q ] );
                        nP = decode_normal( a, a.normalPrev[ q ] );
                    }
                    const float w = ( xx ? subPixS.x : 1.0f - subPixS.x ) * ( yy ? subPixS.y : 1.0f - subPixS.y );
                    if( test_depth_r( z, rz, dP, motionZ ) && test_normal( normal, nP ) ) weightSumVirtual = weightSumVirtual + w;
                }
            }
            if( weightSumVirtual > 0.0001f )
            {
                // with the shader's confidence 1, mix(1/(1+Amin), 1/(1+Avirt), 1) leaves Avirt
                const float Avirt    = gclamp( 256.0f * ( f0 * ex2_approx( 0.5f * lr ) ), minA, A );
                const float invAv    = __fdividef( 1.0f, 1.0f + Avirt );
                const float Ahitdist = fminf( Avirt, 16.0f );
                const float3 specVirt = X::vmix( specPrevOnSurf, unfilteredSpec, invAv );
                const float  aa2      = X::mix( invA, invAv, domin );
                specColorAccum         = X::vmix( specOnSurf, specVirt, domin );
                specHistoryLengthAccum = __fdividef( 1.0f, aa2 ) - 1.0f;
                specHitDistanceAccum   = X::mix( specHitDistancePrev, rayInfo.w, __fdividef( 1.0f, 1.0f + Ahitdist ) );
            }
        }
        else
        {
            const float A       = gclamp( 1.0f + specHistoryLength * powf( 1.0f - aS, 5.0f ), spec_min_accum( u ), 256.0f );
            const float par     = parallax( u, surfPos, surfPosPrev );
            const float AOnSurf = spec_accum_speed< false >( u, A, roughness, nv, par );
            const float domin   = spec_dominant< false >( nv, roughness );

            const float3 specOnSurf    = vmix( specPrevOnSurf, unfilteredSpec, 1.0f / ( 1.0f + AOnSurf ) );
            const float  hitDistOnSurf = gmix( specHitDistancePrev, rayInfo.w, 1.0f / ( 1.0f + AOnSurf ) );

            specColorAccum         = specOnSurf;
            specHistoryLengthAccum = AOnSurf;
            specHitDistanceAccum   = hitDistOnSurf;

            const float3 rayDir     = f3( rayInfo.x, rayInfo.y, rayInfo.z );
            const float3 virtualPos = add( surfPos, mul( mul( rayDir, hitDistOnSurf ), domin ) );

            int2   pixPrevS;
            float2 subPixS;
            {
                const float4 vp   = make_float4( virtualPos.x, virtualPos.y, virtualPos.z, 1.0f );
                const float4 vsc  = mat_mul( u.view, vp );
                const float4 vsp  = mat_mul( u.viewPrev, vp );
                const float4 csc  = mat_mul( u.proj, vsc );
                const float4 csp  = mat_mul( u.projPrev, vsp );
                const float3 ndcC = f3( csc.x / csc.w, csc.y / csc.w, csc.z / csc.w );
                const float3 ndcP = f3( csp.x / csp.w, csp.y / csp.w, csp.z / csp.w );
                const float2 ssC  = make_float2( ndcC.x * 0.5f + 0.5f, ndcC.y * 0.5f + 0.5f );
                const float2 ssP  = make_float2( ndcP.x * 0.5f + 0.5f, ndcP.y * 0.5f + 0.5f );
                const float2 spp  = prev_screen_pos( u, make_float2( ssP.x - ssC.x, ssP.y - ssC.y ), px, py );
                const float  fx = floorf( spp.x - 0.5f ), fy = floorf( spp.y - 0.5f );
                pixPrevS = make_int2( (int)fx, (int)fy );
                subPixS  = make_float2( ( spp.x - 0.5f ) - fx, ( spp.y - 0.5f ) - fy );
            }
            const float bws[ 2 ][ 2 ] = {
                { ( 1.0f - subPixS.x ) * ( 1.0f - subPixS.y ), subPixS.x * ( 1.0f - subPixS.y ) },
                { ( 1.0f - subPixS.x ) * subPixS.y, subPixS.x * subPixS.y },
            };
            float weightSumVirtual = 0.0f;
#pragma unroll
            for( int yy = 0; yy <= 1; yy++ )
            {
#pragma unroll
                for( int xx = 0; xx <= 1; xx++ )
                {
                    const int qx = pixPrevS.x + xx, qy = pixPrevS.y + yy;
                    if( !in_area( qx, qy, chArea ) ) continue;
                    const int    q  = qy * u.W + qx;
                    const float  dP = h2f( a.depthPrev[ q ] );
                    const float3 nP = decode_normal( a, a.normalPrev[ q ] );
                    // the shader also accumulates SpecAccumColor_Prev here but never uses the sum
                    if( test_depth( z, dP, motionZ ) && test_normal( normal, nP ) ) weightSumVirtual = weightSumVirtual + bws[ yy ][ xx ];
                }
            }
            if( weightSumVirtual > 0.0001f )
            {
                float       Avirt      = spec_accum_speed< false >( u, A, roughness, nv, 0.0f );
                const float confidence = 1.0f;
                const float Amin       = fminf( Avirt, 3.0f * sqrtf( roughness ) );
                float       aa         = gmix( 1.0f / ( 1.0f + Amin ), 1.0f / ( 1.0f + Avirt ), confidence );
                Avirt                  = 1.0f / aa - 1.0f;
                const float Ahitdist   = fminf( Avirt, 16.0f );
                const float3 specVirt  = vmix( specPrevOnSurf, unfilteredSpec, 1.0f / ( 1.0f + Avirt ) );
                const float amount     = domin;
                aa                     = gmix( 1.0f / ( 1.0f + AOnSurf ), 1.0f / ( 1.0f + Avirt ), amount );
                specColorAccum         = vmix( specOnSurf, specVirt, amount );
                specHistoryLengthAccum = 1.0f / aa - 1.0f;
                specHitDistanceAccum   = gmix( specHitDistancePrev, rayInfo.w, 1.0f / ( 1.0f + Ahitdist ) );
            }
        }
    }
    else
    {
        specColorAccum         = unfilteredSpec;
        specHistoryLengthAccum = 1.0f;
        specHitDistanceAccum   = rayInfo.w;
    }

    float3 diffColorAccum, indirAccum;
    float2 diffMomentsAccum;
    float  diffHL, indirHL;
    if( hasHistory )
    {
        const float inv = FAST ? invWS : 1.0f / weightSum;
        diffPrev        = mul( diffPrev, inv );
        momentsPrev     = make_float2( momentsPrev.x * inv, momentsPrev.y * inv );
        indirPrev       = mul( indirPrev, inv );
        float dHL       = histLenDIS.x * inv;
        float iHL       = histLenDIS.y * inv;
        {
            // the history length stays IEEE (variance switches on it); its reciprocal only
            // blends, so FAST takes the hardware one
            dHL = dHL * ( FAST ? decD : powf( 1.0f - aD, 10.0f ) );
            dHL = gclamp( dHL + 1.0f, 1.0f, 256.0f );
            const float rD     = FAST ? __fdividef( 1.0f, dHL ) : 1.0f / dHL;
            float alphaColor   = fmaxf( 0.01f, rD );
            float alphaMoments = fmaxf( 0.01f, rD );
            alphaColor         = X::mix( alphaColor, 1.0f, aD );
            alphaMoments       = X::mix( alphaMoments, 1.0f, aD );
            diffColorAccum     = X::vmix( diffPrev, unfilteredDiff, alphaColor );
            diffMomentsAccum   = make_float2( X::mix( momentsPrev.x, moments.x, alphaMoments ), X::mix( momentsPrev.y, moments.y, alphaMoments ) );
            diffHL             = dHL;
        }
        {
            iHL = iHL * ( FAST ? decI : powf( 1.0f - aI, 10.0f ) );
            iHL = gclamp( iHL + 1.0f, 1.0f, 256.0f );
            float alphaColor = fmaxf( 0.01f, FAST ? __fdividef( 1.0f, iHL ) : 1.0f / iHL );
            alphaColor       = X::mix( alphaColor, 1.0f, aI );
            indirAccum       = X::vmix( indirPrev, unfilteredIndir, alphaColor );
            indirHL          = iHL;
        }
    }
    else
    {
        diffColorAccum   = unfilteredDiff;
        diffMomentsAccum = moments;
        diffHL           = 1.0f;
        indirAccum       = unfilteredIndir;
        indirHL          = 1.0f;
    }

    S::st3( a.diffTemp, i, diffColorAccum );
    S::st2( a.moments, i, diffMomentsAccum );
    S::st4( a.histLen, i, make_float4( diffHL, indirHL, specHistoryLengthAccum, specHitDistanceAccum ) );
    S::st3( a.specAccum, i, specColorAccum );
    S::st3( a.indirAccum, i, indirAccum );
}

// NT threads per block (32 x NT/32 tiles), MINB resident blocks per SM. EARLY (only directly after
// the gradient chain, whose first kernel releases its dependents after its own wait): everything
// but the filtered gradient is read before this grid waits for the chain, so the reprojection
// and the taps overlap the chain's last kernels. The gradient chain writes nothing else this
// pass reads, and reads nothing this pass writes.
template< int M, bool FAST, bool GEOM, bool GEOMPREV, int NT = 256, int MINB = 1, bool EARLY = false >
__global__ void __launch_bounds__( NT, MINB ) k_temporal( const FrameArgs a )
{
    __shared__ float u8[ 256 ];
    pdl_launch_dependents();
    for( int k = threadIdx.y * blockDim.x + threadIdx.x; k < 256; k += NT ) fill_u8( u8, k );
    if( !EARLY ) pdl_wait();
    __syncthreads();
    temporal_tile< M, FAST, GEOM, GEOMPREV, EARLY >( a, blockIdx.x, blockIdx.y, u8 );
}

// ==========================================================================================
// CmAntiFirefly.comp:96-158 — 5x5 min/max clamp (the centre excluded)
// ==========================================================================================
template< int M > __global__ void __launch_bounds__( 256 ) k_antifirefly( const FrameArgs a )
{
    using S          = Sto< M >;
    const Uniform& u = a.u;
    const int      px = blockIdx.x * blockDim.x + threadIdx.x;
    const int      py = blockIdx.y * blockDim.y + threadIdx.y;
    if( px >= u.W || py >= u.H ) return;
    const size_t i = idx( u, px, py );
    float3 cd = S::ld3( a.diffTemp, i ), cs = S::ld3( a.specAccum, i ), ci = S::ld3( a.indirAccum, i );
    if( u.antiFirefly != 0 )
    {
        const float MAXF = 1000000.0f;
        float3 mnD = f3( MAXF, MAXF, MAXF ), mnS = mnD, mnI = mnD;
        float3 mxD = f3( -MAXF, -MAXF, -MAXF ), mxS = mxD, mxI = mxD;
#pragma unroll
        for( int oy = -2; oy <= 2; oy++ )
        {
#pragma unroll
            for( int ox = -2; ox <= 2; ox++ )
            {
                if( ox == 0 && oy == 0 ) continue;
                const float3 od = ld3z< M >( a, a.diffTemp, px + ox, py + oy );
                const float3 os = ld3z< M >( a, a.specAccum, px + ox, py + oy );
                const float3 oi = ld3z< M >( a, a.indirAccum, px + ox, py + oy );
                mnD = vmin( mnD, od ); mnS = vmin( mnS, os ); mnI = vmin( mnI, oi );
                mxD = vmax( mxD, od ); mxS = vmax( mxS, os ); mxI = vmax( mxI, oi );
            }
        }
        cd = vmin( vmax( cd, mnD ), mxD );
        cs = vmin( vmax( cs, mnS ), mxS );
        ci = vmin( vmax( ci, mnI ), mxI );
    }
    S::st3( a.diffAccumColor, i, cd );
    S::st3( a.specPing, i, cs );
    S::st3( a.indirPing, i, ci );
}

// ==========================================================================================
// CmSVGFEstimateVariance.comp:129-206
// ==========================================================================================
// colourAt(dx, dy) returns DiffAccumColor at (px+dx, py+dy), zero outside the image
template< int M, bool FAST, bool GEOMIN, class ColorAt >
__device__ __forceinline__ void variance_px( const FrameArgs& a, const int px, const int py, const int i, ColorAt colorAt, float3& outC,
                                             float& outV )
{
    using S          = Sto< M >;
    using X          = Wm< FAST >;
    const Geo   gc   = GEOMIN ? geo_load( a.geom, i ) : geo_zero();
    const float cz   = GEOMIN ? geo_depth( gc ) : h2f( a.depth[ i ] );
    float3      pc   = colorAt( 0, 0 );
    if( cz < 0.0f || cz > MAX_RAY_LENGTH )
    {
        outC = pc;
        outV = 0.0f;
        return;
    }
    const float  histLen = S::ld4( a.histLen, (size_t)i ).x;
    const float2 tm      = S::ld2( a.moments, (size_t)i );
    const float  THR     = 4.0f;
    // FAST: hardware reciprocals and fused multiply-adds in the continuous terms; the history
    // length switch and the validity tests stay IEEE
    if( histLen > THR )
    {
        float tv = fmaxf( 0.0f, FAST ? X::madd( -tm.x, tm.x, tm.y ) : tm.y - tm.x * tm.x );
        tv       = FAST ? tv * rcp_approx( fmaxf( 1.0f, histLen - THR ) ) : tv / fmaxf( 1.0f, histLen - THR );
        outC     = pc;
        outV     = tv;
        return;
    }
    const float  l   = X::lum( pc );
    float2       sm  = make_float2( l + tm.x, X::madd( l, l, tm.y ) );
    float        ws  = 1.0f;
    const float3 cnd = GEOMIN ? gc.n : decode_normal( a, a.normal[ i ] );
#pragma unroll
    for( int yy = -1; yy <= 1; yy++ )
    {
#pragma unroll
        for( int xx = -1; xx <= 1; xx++ )
        {
            if( xx == 0 && yy == 0 ) continue;
            const int    qx  = px + xx, qy = py + yy;
            const float3 cq  = colorAt( xx, yy );
            const float  lq  = X::lum( cq );
            const bool   in  = inside( a.u, qx, qy );
            const int    q   = in ? qy * a.u.W + qx : 0;
            float        zq;
            float3       nq;
            if( GEOMIN )
            {
                const Geo gq = in ? geo_load( a.geom, q ) : geo_zero();
                zq           = geo_depth( gq );
                nq           = gq.n;
            }
            else
            {
                zq = in ? h2f( a.depth[ q ] ) : 0.0f;
                nq = decode_normal( a, in ? a.normal[ q ] : 0u );
            }
            const float  mz  = fmaxf( cz, zq );
            const float  rcp = mz <= 0.0f ? 0.0f : ( FAST ? rcp_approx( mz ) : 1.0f / mz );
            const float  wz  = X::expn( -fabsf( cz - zq ) * rcp );
            const float  wn  = X::pow128( fmaxf( 0.0f, X::dot( cnd, nq ) ) );
            const float  w   = wz * wn;
            if( !isnan( w ) )
            {
                const float lw = lq * w;
                sm = make_float2( sm.x + lw, FAST ? X::madd( lq, lw, sm.y ) : sm.y + lq * lq * w );
                pc = f3( X::madd( cq.x, w, pc.x ), X::madd( cq.y, w, pc.y ), X::madd( cq.z, w, pc.z ) );
                ws = ws + w;
            }
        }
    }
    const float inv = ws <= 0.0f ? 0.0f : ( FAST ? rcp_approx( ws ) : 1.0f / ws );
    sm              = make_float2( sm.x * inv, sm.y * inv );
    outC            = mul( pc, inv );
    outV            = fmaxf( 0.0f, FAST ? X::madd( -sm.x, sm.x, sm.y ) : sm.y - sm.x * sm.x ) * ( 1.0f + 2.0f * ( 1.0f - histLen / THR ) );
}

template< int M > __global__ void __launch_bounds__( 256 ) k_variance( const FrameArgs a )
{
    using S          = Sto< M >;
    const Uniform& u = a.u;
    const int      px = blockIdx.x * blockDim.x + threadIdx.x;
    const int      py = blockIdx.y * blockDim.y + threadIdx.y;
    if( px >= u.W || py >= u.H ) return;
    const int i = py * u.W + px;
    float3    c;
    float     v;
    variance_px< M, false, false >( a, px, py, i, [ & ]( int dx, int dy ) { return ld3z< M >( a, a.diffAccumColor, px + dx, py + dy ); }, c, v );
    S::stcv( a.diffPing, a.varPing, (size_t)i, c, v );
}

// ==========================================================================================
// Anti-firefly for the default path (CmAntiFirefly.comp:120-158), the same results as
// k_antifirefly: min / max are exact in any representation of the stored values, so 16-bit
// storage clamps on packed half2 / bf16x2 pairs without converting, fp32 on floats, and the
// shared-exponent storage on decoded floats. Blocks whose 5x5 footprint lies inside the image
// skip the bounds tests. Every stored colour is non-negative and finite, so the shader's
// +-1e6 initial extrema never survive the 24 taps and the first tap seeds them.
// ==========================================================================================
template< int M > struct AfOps;
template<> struct AfOps< MODE_F16 >
{
    using V = uint2;   // (r,g) (b,0) as two half2
    __device__ static V ld( const void* p, int i ) { return static_cast< const uint2* >( p )[ i ]; }
    __device__ static V zero() { return make_uint2( 0u, 0u ); }
    __device__ static uint32_t mn2( uint32_t a, uint32_t b )
    {
        __half2 r = __hmin2( *reinterpret_cast< __half2* >( &a ), *reinterpret_cast< __half2* >( &b ) );
        return *reinterpret_cast< uint32_t* >( &r );
    }
    __device__ static uint32_t mx2( uint32_t a, uint32_t b )
    {
        __half2 r = __hmax2( *reinterpret_cast< __half2* >( &a ), *reinterpret_cast< __half2* >( &b ) );
        return *reinterpret_cast< uint32_t* >( &r );
    }
    __device__ static V mn( V a, V b ) { return make_uint2( mn2( a.x, b.x ), mn2( a.y, b.y ) ); }
    __device__ static V mx( V a, V b ) { return make_uint2( mx2( a.x, b.x ), mx2( a.y, b.y ) ); }
    __device__ static void st( void* p, int i, V v ) { static_cast< uint2* >( p )[ i ] = v; }
};
template<> struct AfOps< MODE_BF16 >
{
    using V = uint2;
    __device__ static V ld( const void* p, int i ) { return static_cast< const uint2* >( p )[ i ]; }
    __device__ static V zero() { return make_uint2( 0u, 0u ); }
    __device__ static uint32_t mn2( uint32_t a, uint32_t b )
    {
        __nv_bfloat162 r = __hmin2( *reinterpret_cast< __nv_bfloat162* >( &a ), *reinterpret_cast< __nv_bfloat162* >( &b ) );
        return *reinterpret_cast< uint32_t* >( &r );
    }
    __device__ static uint32_t mx2( uint32_t a, uint32_t b )
    {
        __nv_bfloat162 r = __hmax2( *reinterpret_cast< __nv_bfloat162* >( &a ), *reinterpret_cast< __nv_bfloat162* >( &b ) );
        return *reinterpret_cast< uint32_t* >( &r );
    }
    __device__ static V mn( V a, V b ) { return make_uint2( mn2( a.x, b.x ), mn2( a.y, b.y ) ); }
    __device__ static V mx( V a, V b ) { return make_uint2( mx2( a.x, b.x ), mx2( a.y, b.y ) ); }
    __device__ static void st( void* p, int i, V v ) { static_cast< uint2* >( p )[ i ] = v; }
};
template<> struct AfOps< MODE_F32 >
{
    using V = float3;   // rgb of the rgba32f texel (alpha is written 0)
    __device__ static V ld( const void* p, int i )
    {
        const float4 v = static_cast< const float4* >( p )[ i ];
        return f3( v.x, v.y, v.z );
    }
    __device__ static V zero() { return f3( 0, 0, 0 ); }
    __device__ static V mn( V a, V b ) { return vmin( a, b ); }
    __device__ static V mx( V a, V b ) { return vmax( a, b ); }
    __device__ static void st( void* p, int i, V v ) { static_cast< float4* >( p )[ i ] = make_float4( v.x, v.y, v.z, 0.0f ); }
};
template<> struct AfOps< MODE_REF >
{
    using V = float3;
    __device__ static V ld( const void* p, int i ) { return e5( static_cast< const uint32_t* >( p )[ i ] ); }
    __device__ static V zero() { return f3( 0, 0, 0 ); }
    __device__ static V mn( V a, V b ) { return vmin( a, b ); }
    __device__ static V mx( V a, V b ) { return vmax( a, b ); }
    __device__ static void st( void* p, int i, V v ) { static_cast< uint32_t* >( p )[ i ] = encode_e5( v.x, v.y, v.z ); }
};

template< int M, bool INTERIOR >
__device__ __forceinline__ void af_signal( const FrameArgs& a, const void* src, void* dst, int px, int py, int i )
{
    using O          = AfOps< M >;
    using V          = typename O::V;
    const Uniform& u = a.u;
    V c = O::ld( src, i );
    if( u.antiFirefly != 0 )
    {
        V mn = c, mx = c;
        bool first = true;
#pragma unroll
        for( int oy = -2; oy <= 2; oy++ )
        {
#pragma unroll
            for( int ox = -2; ox <= 2; ox++ )
            {
                if( ox == 0 && oy == 0 ) continue;
                const int qx = px + ox, qy = py + oy;
                const V   v  = ( INTERIOR || inside( u, qx, qy ) ) ? O::ld( src, qy * u.W + qx ) : O::zero();
                if( first )
                {
                    mn = mx = v;
                    first = false;
                }
                else
                {
                    mn = O::mn( mn, v );
                    mx = O::mx( mx, v );
                }
            }
        }
        c = O::mn( O::mx( c, mn ), mx );
    }
    O::st( dst, i, c );
}

// The 5x5 clamp (the centre excluded) of a tile of 32 columns x 8 RP rows, blockDim 32 x 8,
// one signal after the other:
//   1. the thread of column x and row group ty loads its column's RP + 4 texels (zeros outside
//      the image) into registers and forms, for each of its RP rows, the minimum and maximum of
//      the 5 rows around it (v5) and of the 4 rows without it (v4), from minima of row pairs;
//   2. v5 of every column, the two halo columns on each side included, goes to shared memory;
//   3. the pixel combines its own v4 with v5 of the columns x-2, x-1, x+1, x+2 and clamps its
//      centre, still in registers.
// min and max are exact, so this is the 24-tap clamp of af_signal value for value. Shared
// memory carries only the v5 pairs: one 16-byte store and four 16-byte loads per pixel and
// signal for the packed 16-bit texels.
template< int M > struct AfOpsRows
{
    static constexpr int RP = 4;   // output rows per thread
};
template< int M > struct AfPair
{
    typename AfOps< M >::V mn, mx;
};
template< int M > struct AfShared
{
    static constexpr int RP = AfOpsRows< M >::RP, TH = 8 * RP, RW = 32 + 4;
    AfPair< M >          v5[ TH ][ RW ];
};
static_assert( sizeof( AfShared< MODE_F32 > ) <= 48 * 1024 && sizeof( AfShared< MODE_F16 > ) <= 48 * 1024,
               "the anti-firefly tile must fit static shared memory" );

// Rows r0 - 2 .. r0 + RP + 1 of column x of one signal, zeros outside the image: writes v5 of
// rows r0 .. r0 + RP - 1 to the shared column `col` (rows `row0` ...), and returns v4 and the
// centre texel of each row (when v4 is non-null).
template< int M >
__device__ __forceinline__ void af_column( const Uniform& u, const void* src, const int x, const int r0, AfShared< M >& sh, const int row0,
                                           const int col, typename AfOps< M >::V* c, AfPair< M >* v4 )
{
    using O          = AfOps< M >;
    using V          = typename O::V;
    constexpr int RP = AfOpsRows< M >::RP;
    const bool    colIn = x >= 0 && x < u.W;
    V             v[ RP + 4 ];
#pragma unroll
    for( int k = 0; k < RP + 4; k++ )
    {
        const int y = r0 - 2 + k;
        v[ k ]      = ( colIn && y >= 0 && y < u.H ) ? O::ld( src, y * u.W + x ) : O::zero();
    }
#pragma unroll
    for( int r = 0; r < RP; r++ )
    {
        // rows r-2, r-1 and r+1, r+2 around row r (v[r + 2])
        const V     mn4 = O::mn( O::mn( v[ r ], v[ r + 1 ] ), O::mn( v[ r + 3 ], v[ r + 4 ] ) );
        const V     mx4 = O::mx( O::mx( v[ r ], v[ r + 1 ] ), O::mx( v[ r + 3 ], v[ r + 4 ] ) );
        AfPair< M > p5;
        p5.mn                       = O::mn( mn4, v[ r + 2 ] );
        p5.mx                       = O::mx( mx4, v[ r + 2 ] );
        sh.v5[ row0 + r ][ col ] = p5;
        if( v4 )
        {
            v4[ r ].mn = mn4;
            v4[ r ].mx = mx4;
            c[ r ]     = v[ r + 2 ];
        }
    }
}

// One signal of the tile (every thread of the block takes part): rows r0 .. r0 + RP - 1 of
// column x clamped into dst; keep (when non-null) receives the clamped texels of the rows
// inside the image.
template< int M >
__device__ __forceinline__ void af_tile_signal( const Uniform& u, const void* src, void* dst, const int bx, const int x, const int r0,
                                                AfShared< M >& sh, typename AfOps< M >::V* keep )
{
    using O          = AfOps< M >;
    using V          = typename O::V;
    constexpr int RP = AfShared< M >::RP;
    const int     tx = threadIdx.x, ty = threadIdx.y;
    V             c[ RP ];
    AfPair< M >   v4[ RP ];
    af_column< M >( u, src, x, r0, sh, ty * RP, tx + 2, c, v4 );
    // the halo columns: local 0, 1 (x0 - 2, x0 - 1) and 34, 35 (x0 + 32, x0 + 33)
    if( tx < 4 )
    {
        const int lc = tx < 2 ? tx : 32 + tx;
        af_column< M >( u, src, bx * 32 - 2 + lc, r0, sh, ty * RP, lc, nullptr, nullptr );
    }
    __syncthreads();
    if( x < u.W )
    {
#pragma unroll
        for( int r = 0; r < RP; r++ )
        {
            if( r0 + r >= u.H ) break;
            const AfPair< M >* row = &sh.v5[ ty * RP + r ][ tx ];
            V mn = O::mn( O::mn( row[ 0 ].mn, row[ 1 ].mn ), O::mn( row[ 3 ].mn, row[ 4 ].mn ) );
            V mx = O::mx( O::mx( row[ 0 ].mx, row[ 1 ].mx ), O::mx( row[ 3 ].mx, row[ 4 ].mx ) );
            mn   = O::mn( mn, v4[ r ].mn );
            mx   = O::mx( mx, v4[ r ].mx );
            const V v = O::mn( O::mx( c[ r ], mn ), mx );
            O::st( dst, ( r0 + r ) * u.W + x, v );
            if( keep ) keep[ r ] = v;
        }
    }
    __syncthreads();   // the next signal reuses the v5 rows
}

template< int M > __device__ __forceinline__ void antifirefly_fast_tile( const FrameArgs& a, int bx, int by, AfShared< M >& sh )
{
    using O          = AfOps< M >;
    using SH         = AfShared< M >;
    constexpr int RP = SH::RP;
    const Uniform& u = a.u;
    const int      tx = threadIdx.x, ty = threadIdx.y;
    const int      x  = bx * 32 + tx;
    const int      r0 = by * SH::TH + ty * RP;
    if( u.antiFirefly == 0 )
    {
        if( x >= u.W ) return;
#pragma unroll
        for( int r = 0; r < RP; r++ )
        {
            if( r0 + r >= u.H ) break;
            const int i = ( r0 + r ) * u.W + x;
            O::st( a.diffAccumColor, i, O::ld( a.diffTemp, i ) );
            O::st( a.specPing, i, O::ld( a.specAccum, i ) );
            O::st( a.indirPing, i, O::ld( a.indirAccum, i ) );
        }
        return;
    }
#pragma unroll
    for( int k = 0; k < 3; k++ )
    {
        const void* src = k == 0 ? a.diffTemp : k == 1 ? a.specAccum : a.indirAccum;
        void*       dst = k == 0 ? a.diffAccumColor : k == 1 ? a.specPing : a.indirPing;
        af_tile_signal< M >( u, src, dst, bx, x, r0, sh, nullptr );
    }
}

template< int M > __global__ void __launch_bounds__( 256, ( M == MODE_F16 || M == MODE_BF16 ) ? 4 : 3 ) k_antifirefly_fast( const FrameArgs a )
{
    __shared__ AfShared< M > sh;
    pdl_launch_dependents();
    pdl_wait();
    antifirefly_fast_tile< M >( a, blockIdx.x, blockIdx.y, sh );
}

// Variance for the default path: the geometry record instead of the depth / normal images
template< int M, bool FAST > __device__ __forceinline__ void variance_geo_tile( const FrameArgs& a, int bx, int by )
{
    using S          = Sto< M >;
    const Uniform& u = a.u;
    const int      px = bx * blockDim.x + threadIdx.x;
    const int      py = by * blockDim.y + threadIdx.y;
    if( px >= u.W || py >= u.H ) return;
    const int i = py * u.W + px;
    float3    c;
    float     v;
    variance_px< M, FAST, true >( a, px, py, i, [ & ]( int dx, int dy ) { return ld3z< M >( a, a.diffAccumColor, px + dx, py + dy ); }, c, v );
    S::stcv( a.diffPing, a.varPing, (size_t)i, c, v );
}
template< int M, bool FAST > __global__ void __launch_bounds__( 256, 8 ) k_variance_geo( const FrameArgs a )
{
    pdl_launch_dependents();
    pdl_wait();
    variance_geo_tile< M, FAST >( a, blockIdx.x, blockIdx.y );
}

// ------------------------------------------------------------------------------------------
// Anti-firefly and variance in one launch (RGDN_FLAG_AF_VARIANCE_FUSED). The block clamps its
// 32 x 32 tile as antifirefly_fast_tile does and keeps the diffuse results, together with those
// of the tile's one-pixel ring (each clamped here from its own 5 x 5 neighbourhood), in shared
// memory as the texels DIFF_ACCUM_COLOR stores. The variance estimate of the tile's pixels then
// reads its 3 x 3 colours there (CmSVGFEstimateVariance.comp:168-205) instead of from memory.
// min and max are exact and the colours are the stored texels, so the results are those of
// k_antifirefly_fast followed by k_variance_geo, bit for bit.
// ------------------------------------------------------------------------------------------
// the texel DIFF_ACCUM_COLOR stores for a clamped value of AfOps< M >, and its decoded colour
// (Sto< M >::ld3 of that texel)
template< int M > struct AfRaw;
template<> struct AfRaw< MODE_REF >
{
    using R = uint32_t;
    __device__ static R      raw( float3 v ) { return encode_e5( v.x, v.y, v.z ); }
    __device__ static R      zero() { return 0u; }
    __device__ static float3 col( R r ) { return e5( r ); }
};
template<> struct AfRaw< MODE_F32 >
{
    using R = float3;
    __device__ static R      raw( float3 v ) { return v; }
    __device__ static R      zero() { return f3( 0, 0, 0 ); }
    __device__ static float3 col( R r ) { return r; }
};
template< bool BF > struct AfRaw16
{
    using R = uint2;
    __device__ static R     raw( uint2 v ) { return v; }
    __device__ static R     zero() { return make_uint2( 0u, 0u ); }
    __device__ static float cv( uint32_t h ) { return BF ? b2f( (uint16_t)h ) : h2f( (uint16_t)h ); }
    __device__ static float3 col( R r ) { return f3( cv( r.x & 0xFFFFu ), cv( r.x >> 16 ), cv( r.y & 0xFFFFu ) ); }
};
template<> struct AfRaw< MODE_F16 > : AfRaw16< false > {};
template<> struct AfRaw< MODE_BF16 > : AfRaw16< true > {};

template< int M > struct AfVarShared
{
    AfShared< M >           af;
    typename AfRaw< M >::R d[ AfShared< M >::TH + 2 ][ 34 ];   // rows / columns -1 .. 32 of the tile
};

template< int M, bool FAST > __device__ __forceinline__ void af_variance_tile( const FrameArgs& a, int bx, int by, AfVarShared< M >& sh )
{
    using O          = AfOps< M >;
    using V          = typename O::V;
    using RW         = AfRaw< M >;
    using S          = Sto< M >;
    constexpr int RP = AfShared< M >::RP, TH = AfShared< M >::TH;
    const Uniform& u = a.u;
    const int      tx = threadIdx.x, ty = threadIdx.y;
    const int      x  = bx * 32 + tx;
    const int      r0 = by * TH + ty * RP;
    V              keep[ RP ];
    if( u.antiFirefly == 0 )
    {
        if( x < u.W )
        {
#pragma unroll
            for( int r = 0; r < RP; r++ )
            {
                if( r0 + r >= u.H ) break;
                const int i = ( r0 + r ) * u.W + x;
                keep[ r ]   = O::ld( a.diffTemp, i );
                O::st( a.diffAccumColor, i, keep[ r ] );
                O::st( a.specPing, i, O::ld( a.specAccum, i ) );
                O::st( a.indirPing, i, O::ld( a.indirAccum, i ) );
            }
        }
    }
    else
    {
        af_tile_signal< M >( u, a.specAccum, a.specPing, bx, x, r0, sh.af, nullptr );
        af_tile_signal< M >( u, a.indirAccum, a.indirPing, bx, x, r0, sh.af, nullptr );
        af_tile_signal< M >( u, a.diffTemp, a.diffAccumColor, bx, x, r0, sh.af, keep );
    }
#pragma unroll
    for( int r = 0; r < RP; r++ )
        sh.d[ ty * RP + r + 1 ][ tx + 1 ] = ( x < u.W && r0 + r < u.H ) ? RW::raw( keep[ r ] ) : RW::zero();
    // the ring: rows -1 and TH (34 texels each), then columns -1 and 32 (TH texels each)
    const int t = ty * 32 + tx;
    if( t < 2 * 34 + 2 * TH )
    {
        int lx, ly;
        if( t < 68 ) { lx = t % 34; ly = t < 34 ? 0 : TH + 1; }
        else { lx = t < 68 + TH ? 0 : 33; ly = 1 + ( t - 68 ) % TH; }
        const int gx = bx * 32 - 1 + lx, gy = by * TH - 1 + ly;
        typename RW::R v = RW::zero();
        if( gx >= 0 && gy >= 0 && gx < u.W && gy < u.H )
        {
            V c = O::ld( a.diffTemp, gy * u.W + gx );
            if( u.antiFirefly != 0 )
            {
                // the 24-tap clamp of af_signal, zeros outside the image
                V    mn = c, mx = c;
                bool first = true;
#pragma unroll
                for( int oy = -2; oy <= 2; oy++ )
                {
#pragma unroll
                    for( int ox = -2; ox <= 2; ox++ )
                    {
                        if( ox == 0 && oy == 0 ) continue;
                        const int qx = gx + ox, qy = gy + oy;
                        const V   q  = inside( u, qx, qy ) ? O::ld( a.diffTemp, qy * u.W + qx ) : O::zero();
                        mn           = first ? q : O::mn( mn, q );
                        mx           = first ? q : O::mx( mx, q );
                        first        = false;
                    }
                }
                c = O::mn( O::mx( c, mn ), mx );
            }
            v = RW::raw( c );
        }
        sh.d[ ly ][ lx ] = v;
    }
    __syncthreads();
    if( x >= u.W ) return;
#pragma unroll 1
    for( int r = 0; r < RP; r++ )
    {
        const int y = r0 + r;
        if( y >= u.H ) break;
        const int i = y * u.W + x;
        float3    c;
        float     var;
        variance_px< M, FAST, true >( a, x, y, i, [ & ]( int dx, int dy ) { return RW::col( sh.d[ ty * RP + r + 1 + dy ][ tx + 1 + dx ] ); }, c, var );
        S::stcv( a.diffPing, a.varPing, (size_t)i, c, var );
    }
}

template< int M, bool FAST >
__global__ void __launch_bounds__( 256, ( M == MODE_F16 || M == MODE_BF16 ) ? 4 : 3 ) k_af_variance( const FrameArgs a )
{
    __shared__ AfVarShared< M > sh;
    pdl_launch_dependents();
    pdl_wait();
    af_variance_tile< M, FAST >( a, blockIdx.x, blockIdx.y, sh );
}

// ==========================================================================================
// CmSVGFAtrous_Iter0.comp:158-335 and CmSVGFAtrous.comp:71-349 — one a-trous iteration;
// the last one composes PreFinal and HistogramInput instead of storing ping/pong.
// ==========================================================================================
// FAST: the hardware reciprocal (the power is an exponent of a continuous weight)
template< bool FAST = false > __device__ __forceinline__ float spec_power( float alpha )
{
    return fmaxf( 0.01f, ( FAST ? 2.0f * rcp_approx( alpha * alpha + 1e-4f ) : 2.0f / ( alpha * alpha + 1e-4f ) ) - 2.0f );
}

struct AtrousIO
{
    const void*  diffSrc;
    const float* varSrc;
    const void*  specSrc;
    const void*  indirSrc;
    void*        diffDst;
    float*       varDst;
    void*        specDst;
    void*        indirDst;
};

template< int M > __device__ __forceinline__ AtrousIO atrous_io( const FrameArgs& a, int iter )
{
    AtrousIO io;
    if( iter == 0 )
    {
        io = { a.diffPing, a.varPing, a.specPing, a.indirPing, a.diffHistory, a.varHistory, a.specPong, a.indirPong };
    }
    else
    {
        const bool odd = ( iter & 1 ) != 0;
        io.diffSrc  = iter == 1 ? a.diffHistory : ( odd ? a.diffPong : a.diffPing );
        io.varSrc   = iter == 1 ? a.varHistory : ( odd ? a.varPong : a.varPing );
        io.specSrc  = odd ? a.specPong : a.specPing;
        io.indirSrc = odd ? a.indirPong : a.indirPing;
        io.diffDst  = odd ? a.diffPing : a.diffPong;
        io.varDst   = odd ? a.varPing : a.varPong;
        io.specDst  = odd ? a.specPing : a.specPong;
        io.indirDst = odd ? a.indirPing : a.indirPong;
    }
    return io;
}

// BRDF.h:49-64
__device__ __forceinline__ float material_ambient( float3 albedo )
{
    const float l = luminance( albedo );
    const float q = ( l - 0.02f ) / 0.02f;
    return l > 0.02f ? 1.0f : 1.0f - q * q;
}

// CmSVGFAtrous.comp:278-348; returns the histogram input value (fp16 bits)
// B10G11R11 channel to FP32 by assembling the bits: exponent e in 1..30 becomes e + 112 with the
// mantissa shifted up; e = 0 gives (2^-14 + m 2^(-14-k)) - 2^-14, an exact difference; e = 31
// gives Inf or the canonical NaN. The values of rgdn::ufloat_to_f32, without a conversion.
__device__ __forceinline__ float ufloat_bits( uint32_t v, int mbits )
{
    const uint32_t e = v >> mbits, m = v & ( ( 1u << mbits ) - 1u );
    if( e == 31u ) return __uint_as_float( m ? 0x7FC00000u : 0x7F800000u );
    const float f = __uint_as_float( ( ( e ? e + 112u : 113u ) << 23 ) | ( m << ( 23 - mbits ) ) );
    return e ? f : f - 6.103515625e-05f;
}
__device__ __forceinline__ float3 decode_b10g11r11_bits( uint32_t p )
{
    return f3( ufloat_bits( p & 0x7FFu, 6 ), ufloat_bits( ( p >> 11 ) & 0x7FFu, 6 ), ufloat_bits( ( p >> 22 ) & 0x3FFu, 5 ) );
}

// The G-buffer texels the composition reads, loaded before the last iteration's taps so their
// latency overlaps the filtering
struct ComposeIn
{
    uint32_t albedo;   // B10G11R11 at the pixel's regular-layout position
    ushort4  throughput;
    uint32_t sky;
    uint32_t mr;
    int      rx, ri;   // regular-layout column and index
};
__device__ __forceinline__ ComposeIn compose_load( const FrameArgs& a, int px, int py, int i )
{
    const int2 rp = regular_from_cb( a.u, px, py );
    ComposeIn  c;
    c.rx         = rp.x;
    c.ri         = rp.y * a.u.W + rp.x;
    c.albedo     = a.albedo[ c.ri ];
    c.throughput = a.throughput[ i ];
    c.sky        = a.isSky[ i ];
    c.mr         = a.mr[ i ];
    return c;
}

// FAST: fused multiply-adds and a reciprocal multiply in the continuous terms (the composed
// colour and the histogram input both are); unorm8 through the table u8 (the same values)
template< int M, bool FAST >
__device__ __forceinline__ uint16_t compose( const FrameArgs& a, int px, const ComposeIn& in, float3 filteredDiff, float3 filteredSpec,
                                             float3 filteredIndir, const float* u8 )
{
    using X           = Wm< FAST >;
    const Uniform& u  = a.u;
    const int      ri = in.ri;
    float3         albedo = decode_b10g11r11_bits( in.albedo );
    const ushort4  tp = in.throughput;
    const float3   throughput = f3( h2f( tp.x ), h2f( tp.y ), h2f( tp.z ) );
    if( u.debugFlags & RGDN_DEBUG_SHOW_FLAG_ALBEDO_WHITE ) albedo = f3( 1.0f, 1.0f, 1.0f );
    float3 ill;
    if( in.sky == 0 )
    {
        const uint32_t mrb       = in.mr;
        const float    metallic  = u8[ mrb & 0xFFu ];
        const float    roughness = u8[ mrb >> 8 ];
        const float3   diffuse = filteredDiff, indirect = filteredIndir;
        // smoothstep(0.5, 0.75, roughness): the division by 0.25 is the exact product by 4
        const float    st       = gsat( ( roughness - 0.5f ) * 4.0f );
        const float3   specular = X::vmix( filteredSpec, indirect, st * st * ( 3.0f - 2.0f * st ) );
        const float3   ro_s     = X::vmix( f3( 0.04f, 0.04f, 0.04f ), albedo, metallic );
        const float3   ro_d     = mul( albedo, 1.0f - metallic );
        const float3   di       = add( diffuse, indirect );
        ill = f3( X::madd( di.x, ro_d.x, specular.x * ro_s.x ), X::madd( di.y, ro_d.y, specular.y * ro_s.y ),
                  X::madd( di.z, ro_d.z, specular.z * ro_s.z ) );
        if( u.debugFlags & RGDN_DEBUG_SHOW_FLAG_ONLY_DIRECT_DIFFUSE ) ill = mul( diffuse, albedo );
        else if( u.debugFlags & RGDN_DEBUG_SHOW_FLAG_ONLY_SPECULAR ) ill = mul( specular, ro_s );
        else if( u.debugFlags & RGDN_DEBUG_SHOW_FLAG_ONLY_INDIRECT_DIFFUSE ) ill = indirect;
        ill = mul( ill, throughput );
        // MaterialAmbient (BRDF.h:49-64)
        const float l = X::lum( albedo );
        const float q = FAST ? ( l - 0.02f ) * 50.0f : ( l - 0.02f ) / 0.02f;
        ill           = mul( ill, l > 0.02f ? 1.0f : X::one_minus( q, q ) );
    }
    else ill = mul( albedo, throughput );

    const uint16_t hin = f32_to_f16( fmaxf( 0.0f, X::lum( ill ) ) );
    a.histInput[ ri ] = hin;
    if( (float)in.rx < u.lightmapCoverage * u.rw ) ill = mul( albedo, throughput );
    Sto< M >::stpre( a.preFinal, ri, vmax( f3( 0, 0, 0 ), ill ) );
    return hin;
}

// FP16 pairs through the packed converter
__device__ __forceinline__ float4 ld_h4( const ushort4* p, int i )
{
    const ushort4 h  = p[ i ];
    const float2  lo = __half22float2( __halves2half2( __ushort_as_half( h.x ), __ushort_as_half( h.y ) ) );
    const float2  hi = __half22float2( __halves2half2( __ushort_as_half( h.z ), __ushort_as_half( h.w ) ) );
    return make_float4( lo.x, lo.y, hi.x, hi.y );
}

// one a-trous iteration for one pixel (CmSVGFAtrous_Iter0.comp:196-304, CmSVGFAtrous.comp:71-220)
// INTERIOR: every tap of the pixel lies inside the image and inside the pixel's checkerboard
// half, so the bounds and render-area tests are statically true (the caller checks this for
// the whole block)
// The centre pixel's terms every tap's weights use, and the running sums.
struct AtrousCtr
{
    float3 normal;
    float  z, l, wLumMul, roughness, wRoughMul, nwSpec, gradDepth, rz1, rz2;
    Area   chArea;
};
constexpr float kLog2e     = 1.44269504088896341f;   // log2(e)
constexpr float kSqrtLog2e = 1.20112240878644913f;   // sqrt(log2(e))
struct AtrousAcc
{
    float3 d, s, i;
    float  var, ws, wsS, wsI;
};

// One tap (xx, yy) of the dilated 3x3 stencil (CmSVGFAtrous.comp:163-235): its edge-stopping
// weights and its contribution to the sums. Both a-trous loops below run this same code, so
// their results are identical.
//
// FAST evaluates every weight in the exponent domain (one hardware exp2 per weight): with
// L = log2 max(n.n_q, 0) (clamped at -126, where every weight it enters is 0 in FP32),
//   wBase = 2^( -(w_z sqrt(log2 e))^2 + 128 L + log2 kernel ),
//   wDiff = 2^( that - w_l log2 e ),   wSpec = w_r' 2^( that + p L ),
// the same products as exp(-w_z^2) * n^128 * kernel, exp(-w_l) and n^p. atrous_terms folds the
// constant factors into rz1, rz2 and wLumMul.
// lq is the tap colour's luminance, Wm< FAST >::lum of (cvq.x, cvq.y, cvq.z)
template< bool FAST, bool INTERIOR >
__device__ __forceinline__ void atrous_accum_l( const AtrousCtr& c, AtrousAcc& acc, const int xx, const int yy, const int qx, const int qy,
                                                const float rq, const float3 nq, const float zq, const float4 cvq, const float lq,
                                                const float3 sq, const float3 iq )
{
    using X = Wm< FAST >;
    if constexpr( FAST )
    {
        const float3 dq    = f3( cvq.x, cvq.y, cvq.z );
        const float  nn    = fmaxf( 0.0f, X::dot( c.normal, nq ) );
        const int    man   = ( xx < 0 ? -xx : xx ) + ( yy < 0 ? -yy : yy );
        const float  L     = fmaxf( lg2_approx( nn ), -126.0f );
        const float  wz    = fabsf( c.z - zq ) * ( man == 1 ? c.rz1 : c.rz2 );
        // log2 of the wavelet kernel {1, 0.5, 0.25} by Manhattan distance
        const float  eBase = __fmaf_rn( -wz, wz, __fmaf_rn( 128.0f, L, -(float)man ) );
        float        w_r   = fmaxf( 0.0f, X::one_minus( 10.0f, fabsf( c.roughness - rq ) ) ) * c.wRoughMul;
        const float  insideA = ( INTERIOR || in_area( qx, qy, c.chArea ) ) ? 1.0f : 0.0f;
        const float  wBase = ex2_approx( eBase ) * insideA;
        const float  wDiff = ex2_approx( eBase - fabsf( c.l - lq ) * c.wLumMul ) * insideA;
        const float  wSpec = w_r * ex2_approx( __fmaf_rn( c.nwSpec, L, eBase ) ) * insideA;
        const float  wInd  = wBase;
        // the sums in packed FP32 pairs (two independent round-to-nearest FMAs or adds per
        // instruction, the bits of the scalar forms): (d.xy), (d.z, var), (s.xy), (s.z, i.z),
        // (i.xy), (ws, wsS)
        const float2 wDD = make_float2( wDiff, wDiff ), wSS = make_float2( wSpec, wSpec ), wII = make_float2( wInd, wInd );
        const float2 dxy = __ffma2_rn( make_float2( dq.x, dq.y ), wDD, make_float2( acc.d.x, acc.d.y ) );
        const float2 dzv = __ffma2_rn( make_float2( dq.z, cvq.w * wDiff ), wDD, make_float2( acc.d.z, acc.var ) );
        const float2 sxy = __ffma2_rn( make_float2( sq.x, sq.y ), wSS, make_float2( acc.s.x, acc.s.y ) );
        const float2 szi = __ffma2_rn( make_float2( sq.z, iq.z ), make_float2( wSpec, wInd ), make_float2( acc.s.z, acc.i.z ) );
        const float2 ixy = __ffma2_rn( make_float2( iq.x, iq.y ), wII, make_float2( acc.i.x, acc.i.y ) );
        const float2 wsp = __fadd2_rn( make_float2( acc.ws, acc.wsS ), make_float2( wDiff, wSpec ) );
        acc.d   = f3( dxy.x, dxy.y, dzv.x );
        acc.var = dzv.y;
        acc.s   = f3( sxy.x, sxy.y, szi.x );
        acc.i   = f3( ixy.x, ixy.y, szi.y );
        acc.ws  = wsp.x;
        acc.wsS = wsp.y;
        acc.wsI = acc.wsI + wInd;
        return;
    }
    const float kern[ 2 ][ 2 ] = { { 1.0f, 0.5f }, { 0.5f, 0.25f } };
    const float3 dq  = f3( cvq.x, cvq.y, cvq.z );
    const float  nn  = fmaxf( 0.0f, X::dot( c.normal, nq ) );
    const int    man = ( xx < 0 ? -xx : xx ) + ( yy < 0 ? -yy : yy );

    const float w_z = FAST ? fabsf( c.z - zq ) * ( man == 1 ? c.rz1 : c.rz2 )
                           : fabsf( c.z - zq ) / fmaxf( c.gradDepth * (float)man, 0.01f );
    const float w_n = X::pow128( nn );
    const float w_l = fabsf( c.l - lq ) * c.wLumMul;
    float       w_r = fmaxf( 0.0f, X::one_minus( 10.0f, fabsf( c.roughness - rq ) ) ) * c.wRoughMul;
    // pow(nn, p) is finite for nn in [0,1], so a zero w_r stays zero without it
    if( c.nwSpec > 0.0f && w_r > 0.0f ) w_r = w_r * X::pow01( nn, c.nwSpec );
    const float waveletW = kern[ yy < 0 ? -yy : yy ][ xx < 0 ? -xx : xx ];
    const float insideA  = ( INTERIOR || in_area( qx, qy, c.chArea ) ) ? 1.0f : 0.0f;
    const float wBase    = X::expn( -w_z * w_z ) * w_n * waveletW * insideA;
    const float wDiff    = wBase * X::expn( -w_l );
    const float wSpec    = wBase * w_r;
    const float wInd     = wBase;

    acc.d   = f3( X::madd( dq.x, wDiff, acc.d.x ), X::madd( dq.y, wDiff, acc.d.y ), X::madd( dq.z, wDiff, acc.d.z ) );
    acc.s   = f3( X::madd( sq.x, wSpec, acc.s.x ), X::madd( sq.y, wSpec, acc.s.y ), X::madd( sq.z, wSpec, acc.s.z ) );
    acc.i   = f3( X::madd( iq.x, wInd, acc.i.x ), X::madd( iq.y, wInd, acc.i.y ), X::madd( iq.z, wInd, acc.i.z ) );
    acc.var = X::madd( cvq.w * wDiff, wDiff, acc.var );
    acc.ws  = acc.ws + wDiff;
    acc.wsS = acc.wsS + wSpec;
    acc.wsI = acc.wsI + wInd;
}
template< bool FAST, bool INTERIOR >
__device__ __forceinline__ void atrous_accum( const AtrousCtr& c, AtrousAcc& acc, const int xx, const int yy, const int qx, const int qy,
                                              const float rq, const float3 nq, const float zq, const float4 cvq, const float3 sq,
                                              const float3 iq )
{
    atrous_accum_l< FAST, INTERIOR >( c, acc, xx, yy, qx, qy, rq, nq, zq, cvq, Wm< FAST >::lum( f3( cvq.x, cvq.y, cvq.z ) ), sq, iq );
}

// The centre pixel's weight terms, from its colour (acc.d), normal, depth, depth gradient (in
// c), roughness byte, prefiltered variance and specular history length; resets the weight sums.
template< bool FAST >
__device__ __forceinline__ void atrous_terms_r( AtrousCtr& c, AtrousAcc& acc, const float roughness, const float prefVar, const float hS,
                                                const int iter )
{
    c.l             = Wm< FAST >::lum( acc.d );
    c.wLumMul       = FAST ? kLog2e * rcp_approx( 4.0f * prefVar + 0.00001f ) : 1.0f / ( 4.0f * prefVar + 0.00001f );
    c.roughness     = roughness;
    c.wRoughMul     = gclamp( c.roughness * 30.0f - (float)iter, 0.0f, 1.0f );
    const float nws = gclamp( hS / 8.0f, 0.0f, 1.0f );
    c.nwSpec        = gclamp( spec_power< FAST >( c.roughness * c.roughness ), 8.0f, 1024.0f ) * nws;
    // FAST: one reciprocal per tap distance class (|x|+|y| = 1 or 2), scaled for the exponent
    // domain
    c.rz1  = FAST ? kSqrtLog2e * rcp_approx( fmaxf( c.gradDepth * 1.0f, 0.01f ) ) : 0.0f;
    c.rz2  = FAST ? kSqrtLog2e * rcp_approx( fmaxf( c.gradDepth * 2.0f, 0.01f ) ) : 0.0f;
    acc.ws = acc.wsS = acc.wsI = 1.0f;
}
template< bool FAST >
__device__ __forceinline__ void atrous_terms( AtrousCtr& c, AtrousAcc& acc, const float* u8, const uint32_t rough8, const float prefVar,
                                              const float hS, const int iter )
{
    atrous_terms_r< FAST >( c, acc, u8[ rough8 ], prefVar, hS, iter );
}

// The centre pixel: loads, the invalid-depth early out and the per-pixel weight terms
// (CmSVGFAtrous_Iter0.comp:158-243 / CmSVGFAtrous.comp:71-160). Returns false when the pixel
// keeps its own values (invalid depth).
template< int M, bool FAST, bool GEOMIN >
__device__ __forceinline__ bool atrous_centre( const FrameArgs& a, const AtrousIO& io, const int iter, const int px, const int py, const int i,
                                               const float* u8, AtrousCtr& c, AtrousAcc& acc )
{
    using S          = Sto< M >;
    const Uniform& u = a.u;
    c.chArea         = cb_area( u, px );
    const float4 cv  = S::ldcv( io.diffSrc, io.varSrc, (size_t)i );
    acc.d            = f3( cv.x, cv.y, cv.z );
    acc.var          = cv.w;
    acc.s            = S::ld3( io.specSrc, (size_t)i );
    acc.i            = S::ld3( io.indirSrc, (size_t)i );
    const Geo gc     = GEOMIN ? geo_load( a.geom, i ) : geo_zero();
    c.z              = GEOMIN ? geo_depth( gc ) : h2f( a.depth[ i ] );
    c.gradDepth      = h2f( a.depthGrad[ i ] );

    if( c.z < 0.0f || c.z > MAX_RAY_LENGTH )
    {
        if( iter == 0 )
        {
            acc.d = f3( 0, 0, 0 ); acc.var = 0.0f; acc.s = f3( 0, 0, 0 ); acc.i = f3( 0, 0, 0 );
        }
        return false;
    }
    c.normal = GEOMIN ? gc.n : decode_normal( a, a.normal[ i ] );
    float prefVar;
    if( iter == 0 )
    {
        // prefilterLuminanceVariance (CmSVGFAtrous_Iter0.comp:158-187)
        const float g[ 2 ][ 2 ] = { { 0.25f, 0.125f }, { 0.125f, 0.0625f } };
        float r = 0.0f;
#pragma unroll
        for( int yy = -1; yy <= 1; yy++ )
        {
#pragma unroll
            for( int xx = -1; xx <= 1; xx++ )
                r = r + ldcvz< M >( a, io.diffSrc, io.varSrc, px + xx, py + yy ).w * g[ xx < 0 ? -xx : xx ][ yy < 0 ? -yy : yy ];
        }
        r = FAST ? sqrt_approx( fmaxf( r, 0.0f ) ) : sqrtf( fmaxf( r, 0.0f ) );
        S::st1( a.filtVar, (size_t)i, r );
        prefVar = r;
    }
    else prefVar = S::ld1( a.filtVar, (size_t)i );
    atrous_terms< FAST >( c, acc, u8, GEOMIN ? geo_rough8( gc ) : ( a.mr[ i ] >> 8 ), prefVar, S::ld4( a.histLen, (size_t)i ).z, iter );
    return true;
}

// FAST: the hardware reciprocals of the weight sums (each sum is at least the centre weight 1)
template< bool FAST >
__device__ __forceinline__ void atrous_finish( AtrousAcc& acc, float3& outDiff, float& outVar, float3& outSpec, float3& outInd )
{
    const float inv  = FAST ? rcp_approx( acc.ws ) : 1.0f / acc.ws;
    const float invS = FAST ? rcp_approx( acc.wsS ) : 1.0f / acc.wsS;
    const float invI = FAST ? rcp_approx( acc.wsI ) : 1.0f / acc.wsI;
    outDiff = mul( acc.d, inv );
    outVar  = acc.var * ( inv * inv );   // outVariance *= invWeightSum * invWeightSum (CmSVGFAtrous.comp:217)
    outSpec = mul( acc.s, invS );
    outInd  = mul( acc.i, invI );
}

template< int M, bool FAST, bool INTERIOR, bool GEOMIN >
__device__ __forceinline__ void atrous_px( const FrameArgs& a, const AtrousIO& io, const int iter, const int px, const int py,
                                           const int i, const float* u8, float3& outDiff, float& outVar, float3& outSpec,
                                           float3& outInd )
{
    using S          = Sto< M >;
    const Uniform& u = a.u;
    const int      step = 1 << iter;
    AtrousCtr      c;
    AtrousAcc      acc;
    if( !atrous_centre< M, FAST, GEOMIN >( a, io, iter, px, py, i, u8, c, acc ) )
    {
        outDiff = acc.d; outVar = acc.var; outSpec = acc.s; outInd = acc.i;
        return;
    }
#pragma unroll
    for( int yy = -1; yy <= 1; yy++ )
    {
#pragma unroll
        for( int xx = -1; xx <= 1; xx++ )
        {
            if( xx == 0 && yy == 0 ) continue;
            const int  qx = px + xx * step, qy = py + yy * step;
            const bool in = INTERIOR || inside( u, qx, qy );
            const int  q  = in ? qy * u.W + qx : 0;
            float      rq, zq;
            float3     nq;
            if( GEOMIN )
            {
                const Geo gq = in ? geo_load( a.geom, q ) : geo_zero();
                rq           = u8[ geo_rough8( gq ) ];
                nq           = gq.n;
                zq           = geo_depth( gq );
            }
            else
            {
                rq = in ? u8[ a.mr[ q ] >> 8 ] : 0.0f;
                nq = decode_normal( a, in ? a.normal[ q ] : 0u );
                zq = in ? h2f( a.depth[ q ] ) : 0.0f;
            }
            const float3 sq  = in ? S::ld3( io.specSrc, (size_t)q ) : f3( 0, 0, 0 );
            const float4 cvq = in ? S::ldcv( io.diffSrc, io.varSrc, (size_t)q ) : make_float4( 0, 0, 0, 0 );
            const float3 iq  = in ? S::ld3( io.indirSrc, (size_t)q ) : f3( 0, 0, 0 );
            atrous_accum< FAST, INTERIOR >( c, acc, xx, yy, qx, qy, rq, nq, zq, cvq, sq, iq );
        }
    }
    atrous_finish< FAST >( acc, outDiff, outVar, outSpec, outInd );
}

// The tile of one a-trous iteration. HIST adds the bins of this tile's HistogramInput values
// to the block's shared histogram `hist` (the caller zeroes and flushes it).
// the last a-trous iteration loads the composition's G-buffer texels before its taps (held in
// registers across the taps: slower) or after them
constexpr bool kComposeEarlyLoads = false;
template< int M, bool FAST, bool HIST, bool GEOMIN >
__device__ __forceinline__ void atrous_tile( const FrameArgs& a, const int iter, int bx, int by, const float* u8, uint32_t* hist )
{
    using S = Sto< M >;
    const Uniform& u  = a.u;
    const int      px = bx * blockDim.x + threadIdx.x;
    const int      py = by * blockDim.y + threadIdx.y;
    if( px < u.W && py < u.H )
    {
        const int      i    = py * u.W + px;
        const AtrousIO io   = atrous_io< M >( a, iter );
        const bool     last = iter + 1 == (int)u.niter;
        float3         outDiff, outSpec, outInd;
        float          outVar;
        // block-uniform: the block's taps are all inside the image and inside one checkerboard half
        const int  step = 1 << iter, sep = u.W / 2;
        const int  bx0 = bx * blockDim.x, bx1 = bx0 + blockDim.x - 1;
        const int  by0 = by * blockDim.y, by1 = by0 + blockDim.y - 1;
        const bool interior = bx0 - step >= 0 && by0 - step >= 0 && bx1 + step < u.W && by1 + step < u.H &&
                              ( bx1 + step < sep || bx0 - step >= sep );
        ComposeIn cin;
        if( last && kComposeEarlyLoads ) cin = compose_load( a, px, py, i );
        if( interior ) atrous_px< M, FAST, true, GEOMIN >( a, io, iter, px, py, i, u8, outDiff, outVar, outSpec, outInd );
        else atrous_px< M, FAST, false, GEOMIN >( a, io, iter, px, py, i, u8, outDiff, outVar, outSpec, outInd );
        if( last && !kComposeEarlyLoads ) cin = compose_load( a, px, py, i );
        if( !last )
        {
            S::stcv( io.diffDst, io.varDst, (size_t)i, outDiff, outVar );
            S::st3( io.specDst, (size_t)i, outSpec );
            S::st3( io.indirDst, (size_t)i, outInd );
        }
        else
        {
            const uint16_t hin = compose< M, FAST >( a, px, cin, outDiff, outSpec, outInd, u8 );
            if( HIST )
            {
                // one shared atomic per distinct bin of the warp
                const uint32_t bin    = __ldg( &a.binLut[ hin ] );
                const uint32_t peers  = __match_any_sync( __activemask(), bin );
                if( ( ( threadIdx.y * blockDim.x + threadIdx.x ) & 31 ) == (uint32_t)( __ffs( peers ) - 1 ) )
                    atomicAdd( &hist[ bin ], (uint32_t)__popc( peers ) );
            }
        }
    }
}

// NT threads per block (32 x NT/32 tiles), MINB resident blocks per SM. ITER >= 0 builds the
// kernel for that iteration (the argument `iter` is then ITER): the step is a constant, so the
// taps of a stencil row share one address and differ by immediate offsets.
template< int M, bool FAST, bool HIST, bool GEOMIN, int NT = 256, int MINB = 3, int ITER = -1 >
__global__ void __launch_bounds__( NT, MINB ) k_atrous( const FrameArgs a, const int iterArg )
{
    const int iter = ITER >= 0 ? ITER : iterArg;
    __shared__ float    u8[ 256 ];
    __shared__ uint32_t hist[ HIST ? 256 : 1 ];
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
    pdl_launch_dependents();
#pragma unroll
    for( int k = t; k < 256; k += NT )
    {
        u8[ k ] = u8_value( k );
        if( HIST ) hist[ k ] = 0u;
    }
    pdl_wait();
    __syncthreads();
    atrous_tile< M, FAST, HIST, GEOMIN >( a, iter, blockIdx.x, blockIdx.y, u8, hist );
    if( HIST )
    {
        __syncthreads();
#pragma unroll
        for( int k = t; k < 256; k += NT )
            if( hist[ k ] ) atomicAdd( &a.tm->histogram[ k ], hist[ k ] );
    }
}

// ==========================================================================================
// A-trous from footprints decoded once into shared memory (the fused iterations 0 + 1 below).
//
// Every texel a block's taps read is loaded once (coalesced rows, read-only loads), decoded to
// FP32 and kept in four float4 planes of shared memory: (normal, depth), (colour, variance),
// (specular, colour luminance) and (indirect, roughness). The taps then read shared memory at
// compile-time offsets. The arithmetic is atrous_px's, in the same order, so the results equal
// the direct kernel's bit for bit.
// ==========================================================================================
// One texel of an a-trous footprint as the staged planes hold it: (normal, depth),
// (colour, variance), (specular, luminance of the colour), (indirect, roughness). A texel outside
// the image is the zero texel the direct kernel substitutes (normal code 0 decodes to (0, 0, 1)).
template< int M >
__device__ __forceinline__ void atrous_stage_texel( const FrameArgs& a, const AtrousIO& io, const int gx, const int gy, const float* u8,
                                                    float4& vg, float4& vc, float4& vs, float4& vi )
{
    using S = Sto< M >;
    vg = make_float4( 0.0f, 0.0f, 1.0f, 0.0f );
    vc = vs = vi = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
    if( inside( a.u, gx, gy ) )
    {
        const int    q  = gy * a.u.W + gx;
        const float4 gr = __ldg( a.geom + q );
        const Geo    g  = { make_float3( gr.x, gr.y, gr.z ), __float_as_uint( gr.w ) };
        const float3 sp = S::ld3_g( io.specSrc, (size_t)q );
        const float3 in = S::ld3_g( io.indirSrc, (size_t)q );
        vc = S::ldcv_g( io.diffSrc, io.varSrc, (size_t)q );
        vg = make_float4( g.n.x, g.n.y, g.n.z, geo_depth( g ) );
        vs = make_float4( sp.x, sp.y, sp.z, Wm< true >::lum( f3( vc.x, vc.y, vc.z ) ) );
        vi = make_float4( in.x, in.y, in.z, u8[ geo_rough8( g ) ] );
    }
}

// The result of one a-trous pixel; `pref` tells whether iteration 0 computed the prefiltered
// variance (not for an invalid-depth centre, which keeps its values and writes no variance).
struct AtrousOut
{
    float3 d, s, i;
    float  var, prefVar;
    bool   pref;
};

// One pixel of a-trous iteration ITER (step STEP) from staged planes: the colour planes C, Sp, I
// with centre texel cc and tap offsets dy * RC + dx * STEP, the static plane G with centre cg
// and tap offsets dy * RG + dx * STEP. The arithmetic and its order are atrous_px's (FAST).
// Iteration 0 prefilters the variance from C (STEP 1); later iterations take `prefVar`.
template< int ITER, int STEP, int RC, int RG >
__device__ __forceinline__ AtrousOut atrous_sm_px( const FrameArgs& a, const int px, const int py, const int i, const bool interior,
                                                   const float4* G, const float4* C, const float4* Sp, const float4* I, const int cg,
                                                   const int cc, float prefVar, const float hS )
{
    AtrousCtr c;
    AtrousAcc acc;
    AtrousOut o;
    o.pref          = false;
    c.chArea        = cb_area( a.u, px );
    const float4 cv = C[ cc ], cs = Sp[ cc ], ci = I[ cc ], cgv = G[ cg ];
    acc.d           = f3( cv.x, cv.y, cv.z );
    acc.var         = cv.w;
    acc.s           = f3( cs.x, cs.y, cs.z );
    acc.i           = f3( ci.x, ci.y, ci.z );
    c.z             = cgv.w;
    c.gradDepth     = h2f( a.depthGrad[ i ] );
    if( c.z < 0.0f || c.z > MAX_RAY_LENGTH )
    {
        // invalid depth keeps its own values (iteration 0: zeros), CmSVGFAtrous_Iter0.comp:208-216
        if( ITER == 0 ) { acc.d = f3( 0, 0, 0 ); acc.var = 0.0f; acc.s = f3( 0, 0, 0 ); acc.i = f3( 0, 0, 0 ); }
        o.d = acc.d; o.var = acc.var; o.s = acc.s; o.i = acc.i; o.prefVar = 0.0f;
        return o;
    }
    c.normal = f3( cgv.x, cgv.y, cgv.z );
    if( ITER == 0 )
    {
        // prefilterLuminanceVariance (CmSVGFAtrous_Iter0.comp:158-187), step-1 neighbours
        const float gw[ 2 ][ 2 ] = { { 0.25f, 0.125f }, { 0.125f, 0.0625f } };
        float       r            = 0.0f;
#pragma unroll
        for( int yy = -1; yy <= 1; yy++ )
        {
#pragma unroll
            for( int xx = -1; xx <= 1; xx++ )
                r = r + C[ cc + yy * RC + xx ].w * gw[ xx < 0 ? -xx : xx ][ yy < 0 ? -yy : yy ];
        }
        prefVar = sqrt_approx( fmaxf( r, 0.0f ) );   // the FAST form of atrous_centre
        o.pref  = true;
    }
    o.prefVar = prefVar;
    atrous_terms_r< true >( c, acc, ci.w, prefVar, hS, ITER );
    auto taps = [ & ]( auto interiorTag ) {
        constexpr bool IN = decltype( interiorTag )::value;
#pragma unroll
        for( int yy = -1; yy <= 1; yy++ )
        {
#pragma unroll
            for( int xx = -1; xx <= 1; xx++ )
            {
                if( xx == 0 && yy == 0 ) continue;
                const int    ec = cc + yy * RC + xx * STEP, eg = cg + yy * RG + xx * STEP;
                const float4 tg = G[ eg ], tc = C[ ec ], ts = Sp[ ec ], ti = I[ ec ];
                atrous_accum_l< true, IN >( c, acc, xx, yy, px + xx * STEP, py + yy * STEP, ti.w, f3( tg.x, tg.y, tg.z ), tg.w, tc, ts.w,
                                            f3( ts.x, ts.y, ts.z ), f3( ti.x, ti.y, ti.z ) );
            }
        }
    };
    if( interior ) taps( std::true_type() );
    else taps( std::false_type() );
    atrous_finish< true >( acc, o.d, o.var, o.s, o.i );
    return o;
}

// ==========================================================================================
// A-trous iterations 0 and 1 in one launch (fusion depth 2).
//
// The block stages iteration 0's sources over its 32 x 8 tile widened by 3 (1 for iteration 0's
// taps, 2 for iteration 1's), computes iteration 0 over the tile widened by 2, keeps those
// results in shared memory exactly as they would be stored and read back (the storage mode's
// quantisation), and then computes iteration 1 (step 2) over the tile. Iteration 0's images are
// written for the tile's own pixels, but iteration 1 reads none of them back: its sources never
// leave the chip. The arithmetic is the single-iteration kernels', so the planes are the same
// bit for bit. The extra cost is iteration 0 over (36 x 12) / (32 x 8) = 1.69 times the tile's
// pixels.
// ==========================================================================================
struct AtPair
{
    static constexpr int TW = 32, TH = 8;
    static constexpr int RW0 = TW + 6, RH0 = TH + 6, N0 = RW0 * RH0;   // iteration 0's sources: tile +- 3
    static constexpr int RW1 = TW + 4, RH1 = TH + 4, N1 = RW1 * RH1;   // iteration 0's results: tile +- 2
    static constexpr int SMEM = ( 4 * N0 + 3 * N1 ) * (int)sizeof( float4 ) + TW * TH * (int)sizeof( float );
};

// the value `v` takes once stored in and read back from a colour + variance / colour plane of
// storage mode M
template< int M > __device__ __forceinline__ float4 stored_cv( float3 c, float var )
{
    alignas( 16 ) uint8_t tex[ 16 ];
    float                 vv;
    Sto< M >::stcv( tex, &vv, 0, c, var );
    return Sto< M >::ldcv( tex, &vv, 0 );
}
template< int M > __device__ __forceinline__ float3 stored_c3( float3 c )
{
    alignas( 16 ) uint8_t tex[ 16 ];
    Sto< M >::st3( tex, 0, c );
    return Sto< M >::ld3( tex, 0 );
}
template< int M > __device__ __forceinline__ float stored_1( float v )
{
    alignas( 16 ) uint8_t tex[ 4 ];
    Sto< M >::st1( tex, 0, v );
    return Sto< M >::ld1( tex, 0 );
}

// the pair's tile (bx, by) of frame `a`, one 32 x 8 block; `smem` holds AtPair::SMEM bytes
template< int M >
__device__ __forceinline__ void atrous_pair_tile( const FrameArgs& a, const int bx, const int by, float4* smem, const float* u8 )
{
    using P = AtPair;
    using S = Sto< M >;
    float4* const    sG = smem;           // iteration 0's sources over tile +- 3
    float4* const    sC = sG + P::N0;
    float4* const    sS = sC + P::N0;
    float4* const    sI = sS + P::N0;
    float4* const    tC = sI + P::N0;     // iteration 0's results over tile +- 2
    float4* const    tS = tC + P::N1;
    float4* const    tI = tS + P::N1;
    float* const     tP = reinterpret_cast< float* >( tI + P::N1 );   // prefiltered variance of the tile
    const int        t = threadIdx.y * 32 + threadIdx.x;

    const Uniform& u   = a.u;
    const AtrousIO io0 = atrous_io< M >( a, 0 ), io1 = atrous_io< M >( a, 1 );
    const int      x0 = bx * P::TW, y0 = by * P::TH;
#pragma unroll
    for( int k = 0; k < ( P::N0 + 255 ) / 256; k++ )
    {
        const int e = t + 256 * k;
        if( e < P::N0 )
        {
            const int r = e / P::RW0, c = e - r * P::RW0;
            atrous_stage_texel< M >( a, io0, x0 - 3 + c, y0 - 3 + r, u8, sG[ e ], sC[ e ], sS[ e ], sI[ e ] );
        }
    }
    __syncthreads();

    const int sep = u.W / 2;
    // iteration 0 over tile +- 2; a pixel outside the image is the zero texel iteration 1 reads
    // there (the roughness stays the staged one, which is zero outside the image as well)
    {
        const int  xa = x0 - 2, ya = y0 - 2, xb = x0 + P::TW + 1, yb = y0 + P::TH + 1;
        const bool interior = xa - 1 >= 0 && ya - 1 >= 0 && xb + 1 < u.W && yb + 1 < u.H && ( xb + 1 < sep || xa - 1 >= sep );
#pragma unroll 1
        for( int e = t; e < P::N1; e += 256 )
        {
            const int r = e / P::RW1, c = e - r * P::RW1;
            const int px = xa + c, py = ya + r;
            const int ce = ( r + 1 ) * P::RW0 + c + 1;
            float4    vc = make_float4( 0.0f, 0.0f, 0.0f, 0.0f ), vs = vc, vi = make_float4( 0.0f, 0.0f, 0.0f, sI[ ce ].w );
            if( inside( u, px, py ) )
            {
                const int       i  = py * u.W + px;
                const bool      own = c >= 2 && c < 2 + P::TW && r >= 2 && r < 2 + P::TH;
                const AtrousOut o  = atrous_sm_px< 0, 1, P::RW0, P::RW0 >( a, px, py, i, interior, sG, sC, sS, sI, ce, ce, 0.0f,
                                                                            S::ld4( a.histLen, (size_t)i ).z );
                if( own )
                {
                    // iteration 0's images, for the tile's own pixels: DiffColorHistory and the
                    // prefiltered variance, which later passes read, and the specular / indirect
                    // pong images (iteration 1 takes them from shared memory, but with three
                    // iterations nothing overwrites them, so the frame's planes stay the
                    // single launches')
                    if( o.pref ) S::st1( a.filtVar, (size_t)i, o.prefVar );
                    S::stcv( io0.diffDst, io0.varDst, (size_t)i, o.d, o.var );
                    S::st3( io0.specDst, (size_t)i, o.s );
                    S::st3( io0.indirDst, (size_t)i, o.i );
                    tP[ ( r - 2 ) * P::TW + c - 2 ] = o.pref ? stored_1< M >( o.prefVar ) : 0.0f;
                }
                vc = stored_cv< M >( o.d, o.var );
                const float3 sp = stored_c3< M >( o.s ), in = stored_c3< M >( o.i );
                vs = make_float4( sp.x, sp.y, sp.z, Wm< true >::lum( f3( vc.x, vc.y, vc.z ) ) );
                vi = make_float4( in.x, in.y, in.z, vi.w );
            }
            tC[ e ] = vc;
            tS[ e ] = vs;
            tI[ e ] = vi;
        }
    }
    __syncthreads();

    // iteration 1 (step 2) over the tile
    {
        const int  x1 = x0 + P::TW - 1, y1 = y0 + P::TH - 1;
        const bool interior = x0 - 2 >= 0 && y0 - 2 >= 0 && x1 + 2 < u.W && y1 + 2 < u.H && ( x1 + 2 < sep || x0 - 2 >= sep );
        const int  px = x0 + threadIdx.x, py = y0 + threadIdx.y;
        if( px < u.W && py < u.H )
        {
            const int       i  = py * u.W + px;
            const int       cc = ( threadIdx.y + 2 ) * P::RW1 + threadIdx.x + 2;
            const int       cg = ( threadIdx.y + 3 ) * P::RW0 + threadIdx.x + 3;
            const AtrousOut o  = atrous_sm_px< 1, 2, 2 * P::RW1, 2 * P::RW0 >( a, px, py, i, interior, sG, tC, tS, tI, cg, cc, tP[ t ],
                                                                              S::ld4( a.histLen, (size_t)i ).z );
            S::stcv( io1.diffDst, io1.varDst, (size_t)i, o.d, o.var );
            S::st3( io1.specDst, (size_t)i, o.s );
            S::st3( io1.indirDst, (size_t)i, o.i );
        }
    }
}

template< int M, int MINB >
__global__ void __launch_bounds__( 256, MINB ) k_atrous_pair01( const FrameArgs a )
{
    extern __shared__ float4 smem[];
    __shared__ float         u8[ 256 ];
    const int                t = threadIdx.y * 32 + threadIdx.x;
    pdl_launch_dependents();
    u8[ t ] = u8_value( t );
    pdl_wait();
    __syncthreads();
    atrous_pair_tile< M >( a, blockIdx.x, blockIdx.y, smem, u8 );
}

// ==========================================================================================
// A-trous with shared-memory staging by the Tensor Memory Accelerator (opt-in).
//
// A 32x8 output tile reads its 3x3 dilated taps from shared memory. The tap footprint of each
// source image (colour+variance, variance plane, specular, indirect, geometry record) is
// copied by TMA (cp.async.bulk.tensor.2d) before any arithmetic: one box of
// (32 + 2 sx) x (8 + 2 s) texels for steps s <= 8, or three 8-row bands (rows -s, 0, +s) for
// s = 16, with sx = s rounded up to 4 texels so every box starts on a 16-byte boundary.
// Texels outside the image arrive as zeros (TMA out-of-bounds fill), which is the zero-texel
// rule; only the geometry record needs a patch there (a zero normal code decodes to (0,0,1)).
// Completion is an mbarrier transaction count; the wait is bounded and a timeout sets an
// error bit in the stream's tonemapping block instead of hanging.
// ==========================================================================================
__device__ __forceinline__ uint32_t smem_u32( const void* p ) { return (uint32_t)__cvta_generic_to_shared( p ); }
__device__ __forceinline__ void mbar_init( uint64_t* bar, uint32_t count )
{
    asm volatile( "mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"( smem_u32( bar ) ), "r"( count ) : "memory" );
}
__device__ __forceinline__ void fence_async_shared() { asm volatile( "fence.proxy.async.shared::cta;" ::: "memory" ); }
__device__ __forceinline__ void mbar_arrive_expect_tx( uint64_t* bar, uint32_t bytes )
{
    asm volatile( "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"( smem_u32( bar ) ), "r"( bytes ) : "memory" );
}
__device__ __forceinline__ void tma_load_2d( void* dst, const CUtensorMap* tm, int x, int y, uint64_t* bar )
{
    asm volatile( "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
                      smem_u32( dst ) ),
                  "l"( (uint64_t)tm ), "r"( x ), "r"( y ), "r"( smem_u32( bar ) )
                  : "memory" );
}
__device__ __forceinline__ void tma_load_3d( void* dst, const CUtensorMap* tm, int x, int y, int z, uint64_t* bar )
{
    asm volatile( "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
                      smem_u32( dst ) ),
                  "l"( (uint64_t)tm ), "r"( x ), "r"( y ), "r"( z ), "r"( smem_u32( bar ) )
                  : "memory" );
}
__device__ __forceinline__ bool mbar_try_wait( uint64_t* bar, uint32_t phase )
{
    uint32_t ok;
    asm volatile( "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                  : "=r"( ok )
                  : "r"( smem_u32( bar ) ), "r"( phase )
                  : "memory" );
    return ok != 0;
}
// bounded wait: false after `limit` polls (the error bit is then set by the caller)
__device__ __forceinline__ bool mbar_wait_bounded( uint64_t* bar, uint32_t phase, int limit = 1 << 22 )
{
    for( int k = 0; k < limit; k++ )
        if( mbar_try_wait( bar, phase ) ) return true;
    return false;
}

template< int M > __host__ __device__ __forceinline__ TmaGeom tma_geom( int iter ) { return tma_geometry( M, iter ); }

template< int M > struct TmaLd;
template<> struct TmaLd< MODE_REF >
{
    __device__ static float4 cv( const uint8_t* b, const uint8_t*, int k )
    {
        const ushort4 h = reinterpret_cast< const ushort4* >( b )[ k ];
        return make_float4( h2f( h.x ), h2f( h.y ), h2f( h.z ), h2f( h.w ) );
    }
    __device__ static float3 col( const uint8_t* b, int k ) { return e5( reinterpret_cast< const uint32_t* >( b )[ k ] ); }
};
template<> struct TmaLd< MODE_F32 >
{
    __device__ static float4 cv( const uint8_t* b, const uint8_t*, int k ) { return reinterpret_cast< const float4* >( b )[ k ]; }
    __device__ static float3 col( const uint8_t* b, int k )
    {
        const float4 v = reinterpret_cast< const float4* >( b )[ k ];
        return f3( v.x, v.y, v.z );
    }
};
template< bool BF > struct TmaLd16
{
    __device__ static float cvt( uint16_t h ) { return BF ? b2f( h ) : h2f( h ); }
    __device__ static float4 cv( const uint8_t* b, const uint8_t* var, int k )
    {
        const ushort4 h = reinterpret_cast< const ushort4* >( b )[ k ];
        return make_float4( cvt( h.x ), cvt( h.y ), cvt( h.z ), reinterpret_cast< const float* >( var )[ k ] );
    }
    __device__ static float3 col( const uint8_t* b, int k )
    {
        const ushort4 h = reinterpret_cast< const ushort4* >( b )[ k ];
        return f3( cvt( h.x ), cvt( h.y ), cvt( h.z ) );
    }
};
template<> struct TmaLd< MODE_F16 > : TmaLd16< false > {};
template<> struct TmaLd< MODE_BF16 > : TmaLd16< true > {};

template< int M, bool FAST, bool INTERIOR >
__device__ __forceinline__ void atrous_px_tma( const FrameArgs& a, const AtrousIO& io, const TmaGeom& g, const uint8_t* sm, const int iter,
                                               const int px, const int py, const int tx, const int ty, const int i, const float* u8,
                                               float3& outDiff, float& outVar, float3& outSpec, float3& outInd )
{
    using S          = Sto< M >;
    using L          = TmaLd< M >;
    const Uniform& u = a.u;
    const int      step = g.s;
    // shared-memory texel index of tap (dx, dy) of this thread's pixel
    auto kidx = [ & ]( int dx, int dy ) {
        const int row = g.nb == 3 ? ( dy + 1 ) * g.th + ty : step + ty + dy * step;
        return row * g.rw + g.sx + tx + dx * step;
    };
    const uint8_t* bCv  = sm + g.offCv;
    const uint8_t* bVar = sm + g.offVar;
    const uint8_t* bSp  = sm + g.offSpec;
    const uint8_t* bIn  = sm + g.offInd;
    const float4*  bGeo = reinterpret_cast< const float4* >( sm + g.offGeo );
    const int      k0   = kidx( 0, 0 );
    const float4   cv   = L::cv( bCv, bVar, k0 );
    AtrousCtr      c;
    AtrousAcc      acc;
    acc.d            = f3( cv.x, cv.y, cv.z );
    acc.var          = cv.w;
    acc.s            = L::col( bSp, k0 );
    acc.i            = L::col( bIn, k0 );
    const float4 gc4 = bGeo[ k0 ];
    const Geo    gc  = { make_float3( gc4.x, gc4.y, gc4.z ), __float_as_uint( gc4.w ) };
    c.z              = geo_depth( gc );
    c.gradDepth      = h2f( a.depthGrad[ i ] );
    if( c.z < 0.0f || c.z > MAX_RAY_LENGTH )
    {
        if( iter == 0 )
        {
            acc.d = f3( 0, 0, 0 ); acc.var = 0.0f; acc.s = f3( 0, 0, 0 ); acc.i = f3( 0, 0, 0 );
        }
        outDiff = acc.d; outVar = acc.var; outSpec = acc.s; outInd = acc.i;
        return;
    }
    c.chArea = cb_area( u, px );
    c.normal = gc.n;
    float prefVar;
    if( iter == 0 )
    {
        // prefilterLuminanceVariance (CmSVGFAtrous_Iter0.comp:158-187); the staged footprint
        // covers +-1 and holds zeros outside the image
        const float gk[ 2 ][ 2 ] = { { 0.25f, 0.125f }, { 0.125f, 0.0625f } };
        float r = 0.0f;
#pragma unroll
        for( int yy = -1; yy <= 1; yy++ )
        {
#pragma unroll
            for( int xx = -1; xx <= 1; xx++ ) r = r + L::cv( bCv, bVar, kidx( xx, yy ) ).w * gk[ xx < 0 ? -xx : xx ][ yy < 0 ? -yy : yy ];
        }
        r = FAST ? sqrt_approx( fmaxf( r, 0.0f ) ) : sqrtf( fmaxf( r, 0.0f ) );
        S::st1( a.filtVar, (size_t)i, r );
        prefVar = r;
    }
    else prefVar = S::ld1( a.filtVar, (size_t)i );
    atrous_terms< FAST >( c, acc, u8, geo_rough8( gc ), prefVar, S::ld4( a.histLen, (size_t)i ).z, iter );

#pragma unroll
    for( int yy = -1; yy <= 1; yy++ )
    {
#pragma unroll
        for( int xx = -1; xx <= 1; xx++ )
        {
            if( xx == 0 && yy == 0 ) continue;
            const int    qx  = px + xx * step, qy = py + yy * step;
            const int    k   = kidx( xx, yy );
            const float4 gq4 = bGeo[ k ];
            Geo          gq  = { make_float3( gq4.x, gq4.y, gq4.z ), __float_as_uint( gq4.w ) };
            if( !INTERIOR && !inside( u, qx, qy ) ) gq = geo_zero();
            atrous_accum< FAST, INTERIOR >( c, acc, xx, yy, qx, qy, u8[ geo_rough8( gq ) ], gq.n, geo_depth( gq ), L::cv( bCv, bVar, k ),
                                            L::col( bSp, k ), L::col( bIn, k ) );
        }
    }
    atrous_finish< FAST >( acc, outDiff, outVar, outSpec, outInd );
}

// Issues the TMA copies of tile (x0, y0)'s footprint into one stage (thread 0 only).
// `extraTx` bytes are expected on top of what the copies deliver: 0, except under
// RGDN_FLAG_TEST_TMA_TIMEOUT, where the barrier can then never complete
template< int M >
__device__ __forceinline__ void tma_issue_tile( const TmaGeom& g, const AtrousMaps& maps, uint8_t* st, uint64_t* bar, int x0, int y0,
                                                uint32_t extraTx )
{
    constexpr TmaTexel tx   = { M == MODE_REF ? 8 : M == MODE_F32 ? 16 : 8, ( M == MODE_F16 || M == MODE_BF16 ) ? 4 : 0,
                                M == MODE_REF ? 4 : M == MODE_F32 ? 16 : 8 };
    const int          box  = g.rw * g.rh;
    mbar_arrive_expect_tx( bar, (uint32_t)( box * g.nb * ( tx.cv + tx.var + 2 * tx.col + 16 ) ) + extraTx );
    // one plane: nb bands of rw x rh texels; 16-byte texels through a 3-D map (word, x, y),
    // the others through a 2-D map of 4-byte words
    auto plane = [ & ]( int off, const CUtensorMap* m, int texBytes ) {
        const int xt = x0 - g.sx;
        for( int b = 0; b < g.nb; b++ )
        {
            const int y = g.nb == 3 ? y0 + ( b - 1 ) * g.s : y0 - g.s;
            if( texBytes == 16 ) tma_load_3d( st + off + b * box * texBytes, m, 0, xt, y, bar );
            else tma_load_2d( st + off + b * box * texBytes, m, xt * ( texBytes / 4 ), y, bar );
        }
    };
    plane( g.offCv, &maps.cv, tx.cv );
    if( tx.var ) plane( g.offVar, &maps.var, tx.var );
    plane( g.offSpec, &maps.spec, tx.col );
    plane( g.offInd, &maps.indir, tx.col );
    plane( g.offGeo, &maps.geo, 16 );
}

// Persistent TMA-staged a-trous iteration: block b computes tiles b, b + gridDim.x, ... Each
// tile's footprint is staged in shared memory by TMA; while the block computes tile k from one
// stage, the copies of tile k+1 fill the other, so the taps never wait on global memory.
// Waits are bounded: a timeout sets bit 0 of the stream's error flags and returns once the
// block's copies are accounted for (see the timeout branch).
template< int M, bool FAST, bool HIST >
__global__ void __launch_bounds__( 256, 3 ) k_atrous_tma( const FrameArgs a, const int iter, const __grid_constant__ AtrousMaps maps )
{
    using S = Sto< M >;
    extern __shared__ __align__( 128 ) uint8_t sm[];
    __shared__ __align__( 8 ) uint64_t bar[ 2 ];
    __shared__ float    u8[ 256 ];
    __shared__ uint32_t hist[ HIST ? 256 : 1 ];
    const Uniform& u      = a.u;
    const int      t      = threadIdx.y * blockDim.x + threadIdx.x;
    const TmaGeom  g      = tma_geom< M >( iter );
    const int      tilesX = ( u.W + g.tw - 1 ) / g.tw;
    const int      total  = tilesX * ( ( u.H + g.th - 1 ) / g.th );
    const int      G      = (int)gridDim.x;
    // RGDN_FLAG_TEST_TMA_TIMEOUT: every stage expects 16 bytes more than its copies bring, and
    // the waits give up after a short limit
    const bool     testTimeout = ( u.flags & RGDN_FLAG_TEST_TMA_TIMEOUT ) != 0;
    const uint32_t extraTx     = testTimeout ? 16u : 0u;
    const int      limit       = testTimeout ? ( 1 << 14 ) : ( 1 << 22 );
    pdl_launch_dependents();
    pdl_wait();
    if( t == 0 )
    {
        mbar_init( &bar[ 0 ], 1 );
        mbar_init( &bar[ 1 ], 1 );
        fence_async_shared();
    }
    u8[ t ] = u8_value( t );
    if( HIST ) hist[ t ] = 0u;
    __syncthreads();
    const int first = (int)blockIdx.x;
    if( t == 0 && first < total ) tma_issue_tile< M >( g, maps, sm, &bar[ 0 ], ( first % tilesX ) * g.tw, ( first / tilesX ) * g.th, extraTx );

    const AtrousIO io   = atrous_io< M >( a, iter );
    const bool     last = iter + 1 == (int)u.niter;
    const int      sep  = u.W / 2;
    int            k    = 0;
    for( int tile = first; tile < total; tile += G, k++ )
    {
        const int st   = k & 1;
        const int next = tile + G;
        // the other stage was released by the barrier that ended the previous tile
        if( t == 0 && next < total )
            tma_issue_tile< M >( g, maps, sm + ( st ^ 1 ) * g.bytes, &bar[ st ^ 1 ], ( next % tilesX ) * g.tw, ( next / tilesX ) * g.th,
                                 extraTx );
        const bool ready = __syncthreads_and( mbar_wait_bounded( &bar[ st ], ( k >> 1 ) & 1, limit ) ? 1 : 0 ) != 0;
        if( !ready )
        {
            // The copies did not complete in time: flag the stream and leave the outputs
            // untouched. The block may not exit while a copy it issued can still write its
            // shared memory, and at this point two stages may have copies outstanding: this
            // tile's (the wait just gave up on them) and the next tile's (issued above). Thread 0
            // waits for both stages again, each up to the full limit, so copies that are only
            // slow land before the memory is released. (A barrier that expects more bytes than
            // its copies bring never completes even after they have landed: both waits then run
            // out, which is the test's case.)
            if( t == 0 )
            {
                atomicOr( &a.tm->errorFlags, RGDN_DEVICE_ERROR_TMA_WAIT );
                mbar_wait_bounded( &bar[ st ], ( k >> 1 ) & 1, limit );
                if( next < total ) mbar_wait_bounded( &bar[ st ^ 1 ], ( ( k + 1 ) >> 1 ) & 1, limit );
            }
            return;
        }
        const uint8_t* stage = sm + st * g.bytes;
        const int      x0 = ( tile % tilesX ) * g.tw, y0 = ( tile / tilesX ) * g.th;
        const int      px = x0 + threadIdx.x, py = y0 + threadIdx.y;
        if( px < u.W && py < u.H )
        {
            const int  i = py * u.W + px;
            float3     outDiff, outSpec, outInd;
            float      outVar;
            const bool interior = x0 - g.s >= 0 && y0 - g.s >= 0 && x0 + g.tw - 1 + g.s < u.W && y0 + g.th - 1 + g.s < u.H &&
                                  ( x0 + g.tw - 1 + g.s < sep || x0 - g.s >= sep );
            if( interior )
                atrous_px_tma< M, FAST, true >( a, io, g, stage, iter, px, py, threadIdx.x, threadIdx.y, i, u8, outDiff, outVar, outSpec, outInd );
            else
                atrous_px_tma< M, FAST, false >( a, io, g, stage, iter, px, py, threadIdx.x, threadIdx.y, i, u8, outDiff, outVar, outSpec, outInd );
            if( !last )
            {
                S::stcv( io.diffDst, io.varDst, (size_t)i, outDiff, outVar );
                S::st3( io.specDst, (size_t)i, outSpec );
                S::st3( io.indirDst, (size_t)i, outInd );
            }
            else
            {
                const uint16_t hin = compose< M, FAST >( a, px, compose_load( a, px, py, i ), outDiff, outSpec, outInd, u8 );
                if( HIST )
                {
                    const uint32_t bin   = __ldg( &a.binLut[ hin ] );
                    const uint32_t peers = __match_any_sync( __activemask(), bin );
                    if( ( t & 31 ) == (uint32_t)( __ffs( peers ) - 1 ) ) atomicAdd( &hist[ bin ], (uint32_t)__popc( peers ) );
                }
            }
        }
        __syncthreads();   // every thread is done with this stage before it is refilled
    }
    if( HIST && hist[ t ] ) atomicAdd( &a.tm->histogram[ t ], hist[ t ] );
}

template< int M, bool FAST, bool HIST > cudaError_t launch_atrous_tma( const FrameArgs& a, int iter, const AtrousMaps& maps, cudaStream_t s )
{
    const TmaGeom g = tma_geom< M >( iter );
    // per iteration: the dynamic shared memory attribute and the resident blocks per SM
    static int attrBytes = 0, perSM[ MAX_ATROUS_ITERATIONS ] = {}, sms = 0;
    if( attrBytes < 2 * g.bytes )
    {
        cudaError_t e = cudaFuncSetAttribute( k_atrous_tma< M, FAST, HIST >, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * g.bytes );
        if( e != cudaSuccess ) return e;
        attrBytes = 2 * g.bytes;
    }
    if( !perSM[ iter ] )
    {
        int dev = 0;
        if( cudaGetDevice( &dev ) != cudaSuccess || cudaDeviceGetAttribute( &sms, cudaDevAttrMultiProcessorCount, dev ) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor( &perSM[ iter ], k_atrous_tma< M, FAST, HIST >, 256, 2 * g.bytes ) != cudaSuccess ||
            perSM[ iter ] <= 0 )
            return cudaErrorInvalidConfiguration;
    }
    const int total = ( ( a.u.W + g.tw - 1 ) / g.tw ) * ( ( a.u.H + g.th - 1 ) / g.th );
    const int grid  = total < perSM[ iter ] * sms ? total : perSM[ iter ] * sms;
    return launch_pdl( k_atrous_tma< M, FAST, HIST >, grid, dim3( g.tw, g.th ), 2 * g.bytes, s, a, iter, maps );
}

// ==========================================================================================
// CmLuminanceHistogram.comp:60-86 — 256-bin histogram of HistogramInput. Bins come from a
// 65536-entry table indexed by the fp16 bits (built on the host from getColorBin, :41-54).
// ==========================================================================================
template< int M > __global__ void __launch_bounds__( 256 ) k_histogram( const FrameArgs a )
{
    __shared__ uint32_t sh[ 256 ];
    const Uniform& u = a.u;
    const int      t = threadIdx.y * blockDim.x + threadIdx.x;
    sh[ t ]          = 0u;
    __syncthreads();
    const int px = blockIdx.x * blockDim.x + threadIdx.x;
    const int py = blockIdx.y * blockDim.y + threadIdx.y;
    if( px < u.W && py < u.H ) atomicAdd( &sh[ __ldg( &a.binLut[ a.histInput[ idx( u, px, py ) ] ] ) ], 1u );
    __syncthreads();
    if( sh[ t ] ) atomicAdd( &a.tm->histogram[ t ], sh[ t ] );
}

// CmLuminanceAvg.comp:39-89 — weighted average bin, eye adaptation, histogram clear
__device__ __forceinline__ void luminance_avg_job( const FrameArgs& a, uint32_t* sh, uint32_t& count0 )
{
    const Uniform& u  = a.u;
    Tonemapping*   tm = a.tm;
    const int      t  = threadIdx.x;
    const uint32_t c  = tm->histogram[ t ];
    sh[ t ]           = c * (uint32_t)t;
    if( t == 0 ) count0 = c;
    __syncthreads();
    tm->histogram[ t ] = 0u;
    for( int cutoff = 128; cutoff > 0; cutoff >>= 1 )
    {
        if( t < cutoff ) sh[ t ] += sh[ t + cutoff ];
        __syncthreads();
    }
    if( t != 0 || u.stopEyeAdaptation != 0 ) return;
    const float minL       = u.minLog, maxL = u.maxLog;
    const float range      = maxL - minL;
    const float pixelCount = u.rw * u.rh;
    const float black      = (float)count0;
    const float wla        = ( (float)sh[ 0 ] / fmaxf( pixelCount - black, 1.0f ) ) - 1.0f;
    const float wal        = (float)exp2( (double)( wla / 254.0f * range + minL ) );
    const float last       = tm->avgLuminance;
    const float tt         = 1.0f - (float)exp( (double)( -u.timeDelta * 1.1f ) );
    const float adapted    = last + ( wal - last ) * tt;
    tm->avgLuminance       = fminf( adapted, (float)exp2( (double)maxL ) );
}
template< int M > __global__ void __launch_bounds__( 256 ) k_luminance_avg( const FrameArgs a )
{
    __shared__ uint32_t sh[ 256 ];
    __shared__ uint32_t count0;
    pdl_launch_dependents();
    pdl_wait();
    luminance_avg_job( a, sh, count0 );
}

// ==========================================================================================
// Batched steps: persistent kernels, one per stage, looping over the tiles of every frame of
// the step. Their grids are a single wave, so each block lets the next stage launch only when it
// has finished its tiles (pdl_launch_dependents at the end): the next stage's blocks then take
// over the SMs as this stage's blocks drain. The step's tile tables and frame arguments are in this module's constant slot
// c_batch[slot] (internal linkage: every translation unit has its own copy, which the host
// fills for the kernels it launches). Every index into it is warp-uniform (derived from
// blockIdx, gridDim and constant data), so the frame arguments live in uniform registers.
// ==========================================================================================
static __constant__ BatchConst c_batch[ BATCH_SLOTS ];

// A batched launch covers the jobs [j0, j1) of its slot's table (one group of the step): the
// launch argument `sarg` packs slot | j0 << 8 | j1 << 16. Tile numbers of a launch count from
// the group's first tile, start[kind][j0].
struct BatchRange
{
    int slot, j0, j1;
};
__device__ __forceinline__ BatchRange batch_range( const int sarg ) { return { sarg & 0xff, ( sarg >> 8 ) & 0xff, ( sarg >> 16 ) & 0xff }; }

// Runs body(args, job, tile x, tile y) for the block's tiles of launch kind `kind`: tile t of
// the launch goes to block t mod gridDim.x. The loop runs job by job, so a job's arguments are
// resolved once per job and the tile coordinates advance by a fixed stride without a division
// per tile. GRAD: tiles cover the gradient image (GW x GH) instead of the render (W x H).
// Every thread of the block runs every iteration, so body may use barriers.
template< bool GRAD, class F > __device__ __forceinline__ void batch_tiles( const int sarg, const int kind, F&& body )
{
    const BatchRange  br   = batch_range( sarg );
    const BatchConst& bc   = c_batch[ br.slot ];
    const int         base = bc.start[ kind ][ br.j0 ];
    const int         G    = (int)gridDim.x;
    for( int j = br.j0; j < br.j1; j++ )
    {
        const int s0 = bc.start[ kind ][ j ] - base, s1 = bc.start[ kind ][ j + 1 ] - base;
        int       r  = ( (int)blockIdx.x - s0 ) % G;
        r            = r < 0 ? r + G : r;
        if( s0 + r >= s1 ) continue;
        const FrameArgs& a  = bc.jobs[ j ];
        const int        tx = ( ( GRAD ? a.u.GW : a.u.W ) + (int)blockDim.x - 1 ) / (int)blockDim.x;
        const int        gq = G / tx, gr = G - gq * tx;
        int              by = r / tx, bx = r - by * tx;
        for( int lt = r; lt < s1 - s0; lt += G )
        {
            body( a, j, bx, by );
            bx += gr;
            by += gq;
            if( bx >= tx )
            {
                bx -= tx;
                by++;
            }
        }
    }
}

template< int M > __global__ void __launch_bounds__( 256, 6 ) kb_gradient_samples( const int sarg )
{
    __shared__ float u8[ 256 ];
    fill_u8( u8, threadIdx.y * blockDim.x + threadIdx.x );
    pdl_wait();
    __syncthreads();
    batch_tiles< true >( sarg, BS_GRADIENT, [ & ]( const FrameArgs& a, int, int bx, int by ) { gradient_samples_tile< M >( a, a.disPing, bx, by, u8 ); } );
    pdl_launch_dependents();
}

template< int M > __global__ void __launch_bounds__( 256 ) kb_gradient_atrous( const int sarg, const int iter )
{
    __shared__ float u8[ 256 ];
    fill_u8( u8, threadIdx.y * blockDim.x + threadIdx.x );
    pdl_wait();
    __syncthreads();
    batch_tiles< true >( sarg, BS_GRADIENT, [ & ]( const FrameArgs& a, int, int bx, int by ) { gradient_atrous_tile( a, iter, bx, by, u8 ); } );
    pdl_launch_dependents();
}

// FAST temporal accumulation writing the geometry record. GPM: 0 = no job has a valid previous
// record, 1 = every job has one, 2 = it depends on the job. The block of a job's first tile also
// clears a histogram that no exposure pass consumed (before the last a-trous iteration adds
// this frame's).
template< int M, int GPM > __global__ void __launch_bounds__( 256 ) kb_temporal( const int sarg )
{
    __shared__ float u8[ 256 ];
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
    fill_u8( u8, t );
    pdl_wait();
    __syncthreads();
    batch_tiles< false >( sarg, BS_TEMPORAL, [ & ]( const FrameArgs& a, int j, int bx, int by ) {
        const uint32_t f = c_batch[ sarg & 0xff ].jobFlags[ j ];
        if( bx == 0 && by == 0 && ( f & BATCH_JOB_CLEAR_HIST ) ) a.tm->histogram[ t ] = 0u;
        if( GPM == 1 || ( GPM == 2 && ( f & BATCH_JOB_GEOM_PREV ) ) ) temporal_tile< M, true, true, true >( a, bx, by, u8 );
        else temporal_tile< M, true, true, false >( a, bx, by, u8 );
    } );
    pdl_launch_dependents();
}

// One tile per block instead of persistent blocks: block b of the launch takes tile b of the
// step's tile table, in the job j with start[kind][j] <= b < start[kind][j + 1] (a block-uniform
// binary search over the constant table, which skips jobs without tiles of this kind). The
// execution shape of the single-frame kernels: 128-thread 32x4 tiles, 7 blocks per SM, the
// dependent launch triggered at the start.
template< bool GRAD > __device__ __forceinline__ bool batch_tile_of_block( const int sarg, const int kind, int& j, int& bx, int& by )
{
    const BatchRange  br = batch_range( sarg );
    const BatchConst& bc = c_batch[ br.slot ];
    const int         b  = (int)blockIdx.x + bc.start[ kind ][ br.j0 ];
    int               lo = br.j0, hi = br.j1;
    if( b >= bc.start[ kind ][ hi ] ) return false;
    while( hi - lo > 1 )
    {
        const int mid = ( lo + hi ) >> 1;
        if( bc.start[ kind ][ mid ] <= b ) lo = mid;
        else hi = mid;
    }
    j                  = lo;
    const FrameArgs& a = bc.jobs[ j ];
    const int        t = b - bc.start[ kind ][ j ];
    const int        tx = ( ( GRAD ? a.u.GW : a.u.W ) + (int)blockDim.x - 1 ) / (int)blockDim.x;
    by                 = t / tx;
    bx                 = t - by * tx;
    return true;
}

template< int M, int GPM > __global__ void __launch_bounds__( 128, 7 ) kt_temporal( const int sarg )
{
    __shared__ float u8[ 256 ];
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
    pdl_launch_dependents();
    for( int k = t; k < 256; k += 128 ) fill_u8( u8, k );
    int        j = 0, bx = 0, by = 0;
    const bool has = batch_tile_of_block< false >( sarg, BS_TEMPORAL, j, bx, by );
    pdl_wait();
    __syncthreads();
    if( !has ) return;
    const FrameArgs& a = c_batch[ sarg & 0xff ].jobs[ j ];
    const uint32_t   f = c_batch[ sarg & 0xff ].jobFlags[ j ];
    if( bx == 0 && by == 0 && ( f & BATCH_JOB_CLEAR_HIST ) )
        for( int k = t; k < 256; k += 128 ) a.tm->histogram[ k ] = 0u;
    if( GPM == 1 || ( GPM == 2 && ( f & BATCH_JOB_GEOM_PREV ) ) ) temporal_tile< M, true, true, true >( a, bx, by, u8 );
    else temporal_tile< M, true, true, false >( a, bx, by, u8 );
}

// blockDim 32 x 8 over tiles of 32 columns x af_tile_rows rows (the tile function's layout); a
// barrier ends each tile before the next reuses the shared rows
template< int M > __global__ void __launch_bounds__( 256 ) kb_antifirefly( const int sarg )
{
    __shared__ AfShared< M > sh;
    pdl_wait();
    batch_tiles< false >( sarg, BS_ANTI_FIREFLY, [ & ]( const FrameArgs& a, int, int bx, int by ) {
        antifirefly_fast_tile< M >( a, bx, by, sh );
        __syncthreads();
    } );
    pdl_launch_dependents();
}

// register cap: the occupancy of the single-frame kernel (5 blocks of 256 per SM)

template< int M > __global__ void __launch_bounds__( 256, 5 ) kb_variance( const int sarg )
{
    pdl_wait();
    batch_tiles< false >( sarg, BS_VARIANCE, [ & ]( const FrameArgs& a, int, int bx, int by ) { variance_geo_tile< M, true >( a, bx, by ); } );
    pdl_launch_dependents();
}

// Variance with one 32 x 8 tile of the step's table per block, built for 8 blocks per SM as the
// single-frame kernel (the block finds its job by a search of the tile table)
template< int M > __global__ void __launch_bounds__( 256, 8 ) kt_variance( const int sarg )
{
    pdl_launch_dependents();
    int        j = 0, bx = 0, by = 0;
    const bool has = batch_tile_of_block< false >( sarg, BS_VARIANCE, j, bx, by );
    pdl_wait();
    if( !has ) return;
    variance_geo_tile< M, true >( c_batch[ sarg & 0xff ].jobs[ j ], bx, by );
}

// A-trous iteration `iter` over the jobs that run it. A job's last iteration composes PreFinal
// and bins its HistogramInput into the block's shared histogram, which is flushed into that
// job's tonemapping state when the block moves to another job and at the end.
// HM: 0 = the iteration is no job's last, 1 = it is every job's last, 2 = it depends on the job.
// MINB: resident blocks per SM the kernel is built for (the register budget).
template< int M, int HM, int MINB >
__global__ void __launch_bounds__( 256, MINB ) kb_atrous( const int sarg, const int iter )
{
    __shared__ float    u8[ 256 ];
    __shared__ uint32_t hist[ HM ? 256 : 1 ];
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
    u8[ t ]     = u8_value( t );
    if( HM ) hist[ t ] = 0u;
    pdl_wait();
    __syncthreads();
    int  histJob = -1;
    auto flush   = [ & ]() {
        __syncthreads();
        const uint32_t c = hist[ t ];
        if( c ) atomicAdd( &c_batch[ sarg & 0xff ].jobs[ histJob ].tm->histogram[ t ], c );
        hist[ t ] = 0u;
        __syncthreads();
    };
    batch_tiles< false >( sarg, BS_ATROUS0 + iter, [ & ]( const FrameArgs& a, int j, int bx, int by ) {
        if( HM == 0 ) atrous_tile< M, true, false, true >( a, iter, bx, by, u8, hist );
        else if( HM == 1 || iter + 1 == (int)a.u.niter )
        {
            if( histJob != j )
            {
                if( histJob >= 0 ) flush();
                histJob = j;
            }
            atrous_tile< M, true, true, true >( a, iter, bx, by, u8, hist );
        }
        else atrous_tile< M, true, false, true >( a, iter, bx, by, u8, hist );
    } );
    if( HM && histJob >= 0 ) flush();
    pdl_launch_dependents();
}

// One 32x4 tile per 128-thread block (see kt_temporal); a tile of a job's last iteration bins
// its HistogramInput in the block's shared histogram and flushes it into that job's state.
template< int M, int HM > __global__ void __launch_bounds__( 128, 7 ) kt_atrous( const int sarg, const int iter )
{
    __shared__ float    u8[ 256 ];
    __shared__ uint32_t hist[ HM ? 256 : 1 ];
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
    pdl_launch_dependents();
    for( int k = t; k < 256; k += 128 )
    {
        u8[ k ] = u8_value( k );
        if( HM ) hist[ k ] = 0u;
    }
    int        j = 0, bx = 0, by = 0;
    const bool has = batch_tile_of_block< false >( sarg, BS_ATROUS0 + iter, j, bx, by );
    pdl_wait();
    __syncthreads();
    if( !has ) return;
    const FrameArgs& a = c_batch[ sarg & 0xff ].jobs[ j ];
    if( HM == 1 || ( HM == 2 && iter + 1 == (int)a.u.niter ) )
    {
        atrous_tile< M, true, true, true >( a, iter, bx, by, u8, hist );
        __syncthreads();
        for( int k = t; k < 256; k += 128 )
            if( hist[ k ] ) atomicAdd( &a.tm->histogram[ k ], hist[ k ] );
    }
    else atrous_tile< M, true, false, true >( a, iter, bx, by, u8, hist );
}

// a-trous iterations 0 and 1 of a batched step in one launch: one 32 x 8 tile of the
// BS_ATROUS0 table per block (every job runs at least 3 iterations)
template< int M > __global__ void __launch_bounds__( 256, 3 ) kt_atrous_pair01( const int sarg )
{
    extern __shared__ float4 smem[];
    __shared__ float         u8[ 256 ];
    const int                t = threadIdx.y * 32 + threadIdx.x;
    pdl_launch_dependents();
    u8[ t ] = u8_value( t );
    int        j = 0, bx = 0, by = 0;
    const bool has = batch_tile_of_block< false >( sarg, BS_ATROUS0, j, bx, by );
    pdl_wait();
    __syncthreads();
    if( !has ) return;
    atrous_pair_tile< M >( c_batch[ sarg & 0xff ].jobs[ j ], bx, by, smem, u8 );
}

// one block per job of the group (strided), as k_luminance_avg
template< int M > __global__ void __launch_bounds__( 256 ) kb_luminance_avg( const int sarg )
{
    __shared__ uint32_t sh[ 256 ];
    __shared__ uint32_t count0;
    pdl_wait();
    const BatchRange br = batch_range( sarg );
    for( int j = br.j0 + (int)blockIdx.x; j < br.j1; j += gridDim.x )
    {
        __syncthreads();
        luminance_avg_job( c_batch[ br.slot ].jobs[ j ], sh, count0 );
    }
    pdl_launch_dependents();
}


// ==========================================================================================
// CmCheckerboard.comp:27-69 and CmPrepareFinal.comp:57-187: the checkerboard resolve of split
// pixels, volumetric scattering, exposure, tonemapping and the bloom input, per regular pixel.
// IEEE arithmetic in the shaders' order (a per-pixel pass, off the denoiser's hot loop).
// ==========================================================================================
// resolveCheckerboard (CmCheckerboard.comp:27-39): the cross mean of the four neighbours,
// without a horizontal neighbour across a checkerboard half's edge, mixed half-half with the
// centre; neighbours outside the image read zero
template< class Ld > __device__ __forceinline__ float3 cb_resolve( const FinalArgs& f, Ld ld, const int x, const int y, const int cbx, const float3 c )
{
    const int    sep = f.W / 2;
    const float  lf  = ( cbx == 0 || cbx == sep ) ? 0.0f : 1.0f;
    const float  rf  = ( cbx == sep || cbx == f.W ) ? 0.0f : 1.0f;
    const float3 l = ld( x - 1, y ), r = ld( x + 1, y ), d = ld( x, y + 1 ), u = ld( x, y - 1 );
    const float3 cross = f3( 0.25f * l.x * lf + 0.25f * r.x * rf + 0.25f * d.x + 0.25f * u.x,
                             0.25f * l.y * lf + 0.25f * r.y * rf + 0.25f * d.y + 0.25f * u.y,
                             0.25f * l.z * lf + 0.25f * r.z * rf + 0.25f * d.z + 0.25f * u.z );
    return vmix( c, cross, 0.5f );
}

// uncharted2Tonemap (CmPrepareFinal.comp:69-87)
__device__ __forceinline__ float u2_op( float x )
{
    const float A = 0.15f, B = 0.50f, C = 0.10f, D = 0.20f, E = 0.02f, F = 0.30f;
    return ( ( x * ( A * x + C * B ) + D * E ) / ( x * ( A * x + B ) + D * F ) ) - E / F;
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
// LpmMap (ffx_lpm.h, AMD FidelityFX LPM 1.0) with LPM_CONFIG_709_709 and no shoulder: the ratio
// of the colour to its maximum, raised to the saturation powers; luma tone-mapped by
// luma^c / (luma^c * scale + bias); the ratio scaled to hit that luma without clipping; then
// the missing luma of clipped channels moved to the others through the crosstalk capacities,
// twice. The operation order is the shader's.
// FAST: pow(x, y) as the hardware exp2(y log2 x) and the reciprocals by rcp.approx, as the
// shader's own pow and division compile on a GPU; the result is continuous in each of them
template< bool FAST > __device__ __forceinline__ float lpm_pow( float x, float y ) { return FAST ? ex2_approx( y * lg2_approx( x ) ) : powf( x, y ); }
template< bool FAST > __device__ __forceinline__ float lpm_rcp( float x ) { return FAST ? rcp_approx( x ) : 1.0f / x; }
template< bool FAST > __device__ __forceinline__ float3 lpm_709( float3 c, const LpmConsts& k )
{
    const float rcpMax = lpm_rcp< FAST >( fmaxf( c.x, fmaxf( c.y, c.z ) ) );
    float       rR = c.x * rcpMax, rG = c.y * rcpMax, rB = c.z * rcpMax;
    // pow(x, +-0) is 1 for every x, NaN included: the default saturation 0 needs no pow
    rR = k.saturation[ 0 ] == 0.0f ? 1.0f : lpm_pow< FAST >( rR, k.saturation[ 0 ] );
    rG = k.saturation[ 1 ] == 0.0f ? 1.0f : lpm_pow< FAST >( rG, k.saturation[ 1 ] );
    rB = k.saturation[ 2 ] == 0.0f ? 1.0f : lpm_pow< FAST >( rB, k.saturation[ 2 ] );
    float luma = c.y * k.lumaT[ 1 ] + ( c.x * k.lumaT[ 0 ] + ( c.z * k.lumaT[ 2 ] ) );
    luma       = lpm_pow< FAST >( luma, k.contrast );
    luma       = luma * lpm_rcp< FAST >( luma * k.toneScaleBias[ 0 ] + k.toneScaleBias[ 1 ] );
    const float lumaRatio  = rR * k.lumaT[ 0 ] + rG * k.lumaT[ 1 ] + rB * k.lumaT[ 2 ];
    const float ratioScale = gsat( luma * lpm_rcp< FAST >( lumaRatio ) );
    float       cR = gsat( rR * ratioScale ), cG = gsat( rG * ratioScale ), cB = gsat( rB * ratioScale );
    const float capR = -k.crosstalk[ 0 ] * cR + k.crosstalk[ 0 ];
    const float capG = -k.crosstalk[ 1 ] * cG + k.crosstalk[ 1 ];
    const float capB = -k.crosstalk[ 2 ] * cB + k.crosstalk[ 2 ];
    float lumaAdd = gsat( ( -cB ) * k.lumaT[ 2 ] + ( ( -cR ) * k.lumaT[ 0 ] + ( ( -cG ) * k.lumaT[ 1 ] + luma ) ) );
    const float t = lumaAdd * lpm_rcp< FAST >( capG * k.lumaT[ 1 ] + ( capR * k.lumaT[ 0 ] + ( capB * k.lumaT[ 2 ] ) ) );
    cR      = gsat( t * capR + cR );
    cG      = gsat( t * capG + cG );
    cB      = gsat( t * capB + cB );
    lumaAdd = gsat( ( -cB ) * k.lumaT[ 2 ] + ( ( -cR ) * k.lumaT[ 0 ] + ( ( -cG ) * k.lumaT[ 1 ] + luma ) ) );
    cR      = gsat( lumaAdd * k.rcpLumaT[ 0 ] + cR );
    cG      = gsat( lumaAdd * k.rcpLumaT[ 1 ] + cG );
    cB      = gsat( lumaAdd * k.rcpLumaT[ 2 ] + cB );
    return f3( cR, cG, cB );
}

template< int M, bool FAST > __global__ void __launch_bounds__( 256 ) k_prepare_final( const FinalArgs f )
{
    using S     = Sto< M >;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    pdl_launch_dependents();
    pdl_wait();
    // getAutoEV100, ev100ToLuminousExposure (Exposure.h:14-51): the same for every pixel, so one
    // thread of the block evaluates them
    __shared__ float shExp[ 2 ];
    if( threadIdx.x == 0 && threadIdx.y == 0 )
    {
        const float ev     = log2f( fmaxf( 0.0f, f.tm->avgLuminance ) * 100.0f / 12.5f );
        const float maxLum = 1.2f * exp2f( ev );
        shExp[ 0 ]         = maxLum > 0.0f ? 1.0f / maxLum : 0.0f;
        shExp[ 1 ]         = exp2f( ev + f.bloomEvOffset - 3.0f );
    }
    __syncthreads();
    if( x >= f.W || y >= f.H ) return;
    const float exposure = shExp[ 0 ], el = shExp[ 1 ];
    const int   i        = y * f.W + x;
    // getCheckerboardPix (ShaderCommonGLSLFunc.h:321-329)
    const int sep = f.W / 2;
    const int odd = ( x + y % 2 ) % 2;
    const int cbx = odd * sep + x / 2;
    float3    hdr = S::ldpre( f.preFinal, (size_t)i );
    float3    emis = decode_b10g11r11_bits( f.screenEmis[ i ] );
    // needResolveCheckerboard: wasSplit(Throughput.a) (ShaderCommonGLSLFunc.h:435-444). CmCheckerboard
    // stores the resolved values into Final and ScreenEmission (CmCheckerboard.comp:66-76), which
    // CmPrepareFinal reads back, so they pass through those formats: Final has PreFinal's,
    // ScreenEmission ScreenEmisRT's B10G11R11. Values that were not resolved came from those
    // formats and pass through unchanged.
    if( h2f( f.throughput[ y * f.W + cbx ].w ) > 0.5f )
    {
        auto inImg = [ & ]( int qx, int qy ) { return qx >= 0 && qy >= 0 && qx < f.W && qy < f.H; };
        hdr  = cb_resolve( f, [ & ]( int qx, int qy ) { return inImg( qx, qy ) ? S::ldpre( f.preFinal, (size_t)( qy * f.W + qx ) ) : f3( 0, 0, 0 ); }, x, y, cbx, hdr );
        emis = cb_resolve( f, [ & ]( int qx, int qy ) { return inImg( qx, qy ) ? decode_b10g11r11_bits( f.screenEmis[ qy * f.W + qx ] ) : f3( 0, 0, 0 ); }, x, y, cbx, emis );
        hdr  = S::qpre( hdr );
        emis = decode_b10g11r11_bits( encode_b10g11r11( emis.x, emis.y, emis.z ) );
    }
    if( f.flags & RGDN_FINAL_APPLY_SCATTERING )
    {
        const ushort4 v = f.scattering[ i ];
        const float   a = h2f( v.w );
        hdr             = f3( hdr.x * a + h2f( v.x ), hdr.y * a + h2f( v.y ), hdr.z * a + h2f( v.z ) );
    }
    // finalizeColor (CmPrepareFinal.comp:101-113)
    float3 color;
    if( (float)x < f.lightmapCoverage * f.rw )
    {
        const float w = u2_op( f.whitePoint );
        if constexpr( FAST )
        {
            const float iw = rcp_approx( w );
            color          = f3( u2_op( 2.0f * hdr.x ) * iw, u2_op( 2.0f * hdr.y ) * iw, u2_op( 2.0f * hdr.z ) * iw );
        }
        else color = f3( u2_op( 2.0f * hdr.x ) / w, u2_op( 2.0f * hdr.y ) / w, u2_op( 2.0f * hdr.z ) / w );
    }
    else
    {
        const float3 c = f3( hdr.x * exposure + emis.x * f.emisMax, hdr.y * exposure + emis.y * f.emisMax, hdr.z * exposure + emis.z * f.emisMax );
        color          = lpm_709< FAST >( c, f.lpm );
    }
    // getBloomInput (CmPrepareFinal.comp:116-133)
    float3 bloom = f3( ( hdr.x + emis.x * el ) * exposure, ( hdr.y + emis.y * el ) * exposure, ( hdr.z + emis.z * el ) * exposure );
    if( isnan( bloom.x ) || isnan( bloom.y ) || isnan( bloom.z ) || isinf( bloom.x ) || isinf( bloom.y ) || isinf( bloom.z ) )
        bloom = f3( 0, 0, 0 );
    if constexpr( FAST )
    {
        const float st = gsat( luminance( bloom ) * rcp_approx( f.bloomThreshold ) );   // smoothstep( 0, threshold, . )
        bloom          = mul( bloom, st * st * ( 3.0f - 2.0f * st ) );
    }
    else bloom = mul( bloom, gsmoothstep( 0.0f, f.bloomThreshold, luminance( bloom ) ) );
    S::stpre( f.finalOut, (size_t)i, color );
    S::stpre( f.bloomOut, (size_t)i, bloom );
}


// ==========================================================================================
// CmBloomDownsample.comp, CmBloomUpsample.comp, CmBloomApply.comp: the bloom pyramid over
// images in PRE_FINAL's format. textureLod with the framebuffers' bilinear clamp-to-edge
// sampler is evaluated in FP32 (texel centres at +0.5, weights from the fractional position).
// ==========================================================================================
// One bloom texel: (r, g) as a pair for the packed FP32x2 operations, b alone. Each packed
// lane rounds as the scalar operation does (no contraction), so results equal a scalar
// evaluation bit for bit.
struct P3
{
    float2 rg;
    float  b;
};
__device__ __forceinline__ float3 f3of( P3 p ) { return f3( p.rg.x, p.rg.y, p.b ); }
__device__ __forceinline__ P3     padd( P3 a, P3 b ) { return { __fadd2_rn( a.rg, b.rg ), a.b + b.b }; }
__device__ __forceinline__ P3     pmul( P3 a, float s ) { return { __fmul2_rn( a.rg, make_float2( s, s ) ), a.b * s }; }
// gmix per channel: x (1 - a) + y a
__device__ __forceinline__ P3 pmix( P3 x, P3 y, float a )
{
    const float w = 1.0f - a;
    return { __fadd2_rn( __fmul2_rn( x.rg, make_float2( w, w ) ), __fmul2_rn( y.rg, make_float2( a, a ) ) ), x.b * w + y.b * a };
}
__device__ __forceinline__ float plum( P3 c ) { return 0.2125f * c.rg.x + 0.7154f * c.rg.y + 0.0721f * c.b; }

// a texel of an image in PRE_FINAL's format
template< int M > __device__ __forceinline__ P3 bloom_ld( const void* p, size_t i )
{
    const float3 c = Sto< M >::ldpre( p, i );
    return { make_float2( c.x, c.y ), c.z };
}

// one coordinate of the bilinear clamp-to-edge sampler: x = u n - 0.5, the texel pair
// (floor(x), floor(x) + 1) clamped to [0, n - 1] and the weight x - floor(x)
struct BlAxis
{
    int   i0, i1;
    float f;
};
__device__ __forceinline__ BlAxis bl_axis( float u, int n )
{
    const float x  = u * (float)n - 0.5f;
    const float fx = floorf( x );
    const int   ix = (int)fx;
    return { min( max( ix, 0 ), n - 1 ), min( max( ix + 1, 0 ), n - 1 ), x - fx };
}
template< int M > __device__ __forceinline__ P3 bl_sample( const void* img, int w, const BlAxis& ax, const BlAxis& ay )
{
    const P3 t00 = bloom_ld< M >( img, (size_t)( ay.i0 * w + ax.i0 ) ), t10 = bloom_ld< M >( img, (size_t)( ay.i0 * w + ax.i1 ) );
    const P3 t01 = bloom_ld< M >( img, (size_t)( ay.i1 * w + ax.i0 ) ), t11 = bloom_ld< M >( img, (size_t)( ay.i1 * w + ax.i1 ) );
    return pmix( pmix( t00, t10, ax.f ), pmix( t01, t11, ax.f ), ay.f );
}

// One texel of downsample step k (CmBloomDownsample.comp:15-136): src is BLOOM_INPUT (k = 0)
// or mip k, dst mip k + 1. 13 bilinear taps at offsets of -2..2 source texels, five 2x2 boxes
// of them, Karis weights 1 / (1 + luminance) on step 0. When each offset's texel pair starts
// where the previous one's ends (the usual case; rounding near a texel edge can break it) the
// 6x6 source window is read once, a row at a time, and each row's horizontal lerps serve the
// taps above and below it. Every tap is the same expression either way.
template< int M >
__device__ __forceinline__ void bloom_down_texel( const void* src, int sw, int sh, void* dst, int dw, int x, int y, int k, float4 st )
{
    const float idx = st.x, idy = st.y;
    const float u = ( (float)x + 0.5f ) * idx, v = ( (float)y + 0.5f ) * idy;
    if( u > 1.0f || v > 1.0f ) return;
    const float isx = st.z, isy = st.w;
    BlAxis      ax[ 5 ], ay[ 5 ];
    bool        chain = true;
#pragma unroll
    for( int j = 0; j < 5; j++ )
    {
        ax[ j ] = bl_axis( u + (float)( j - 2 ) * isx, sw );
        ay[ j ] = bl_axis( v + (float)( j - 2 ) * isy, sh );
        if( j > 0 ) chain = chain && ax[ j - 1 ].i1 == ax[ j ].i0 && ay[ j - 1 ].i1 == ay[ j ].i0;
    }
    // the boxes' sums in tap order: b0 = t3 t4 t8 t9, b1 = t0 t1 t5 t6, b2 = t1 t2 t6 t7,
    // b3 = t5 t6 t10 t11, b4 = t6 t7 t11 t12 (tap (ox, oy) on the 5x5 offset grid: t0 (-2,-2),
    // t1 (0,-2), t2 (2,-2), t3 (-1,-1), t4 (1,-1), t5 (-2,0), t6 (0,0), t7 (2,0), t8 (-1,1),
    // t9 (1,1), t10 (-2,2), t11 (0,2), t12 (2,2))
    P3 s0, s1, s2, s3, s4;
    if( chain )
    {
        int col[ 6 ];
#pragma unroll
        for( int j = 0; j < 5; j++ ) col[ j ] = ax[ j ].i0;
        col[ 5 ] = ax[ 4 ].i1;
        P3 hp[ 5 ] = {}, hc[ 5 ] = {};
#pragma unroll
        for( int r = 0; r < 6; r++ )
        {
            const int row = r < 5 ? ay[ r ].i0 : ay[ 4 ].i1;
            P3        t[ 6 ];
#pragma unroll
            for( int c = 0; c < 6; c++ ) t[ c ] = bloom_ld< M >( src, (size_t)( row * sw + col[ c ] ) );
#pragma unroll
            for( int j = 0; j < 5; j++ )
                if( ( j & 1 ) == 0 || ( r >= 1 && r <= 4 ) ) hc[ j ] = pmix( t[ j ], t[ j + 1 ], ax[ j ].f );
            if( r > 0 )
            {
                const int   yj = r - 1;
                const float b  = ay[ yj ].f;
                if( ( yj & 1 ) == 0 )
                {
                    const P3 ta = pmix( hp[ 0 ], hc[ 0 ], b ), tb = pmix( hp[ 2 ], hc[ 2 ], b ), tc = pmix( hp[ 4 ], hc[ 4 ], b );
                    if( yj == 0 ) s1 = padd( ta, tb ), s2 = padd( tb, tc );
                    else if( yj == 2 ) s1 = padd( padd( s1, ta ), tb ), s2 = padd( padd( s2, tb ), tc ), s3 = padd( ta, tb ), s4 = padd( tb, tc );
                    else s3 = padd( padd( s3, ta ), tb ), s4 = padd( padd( s4, tb ), tc );
                }
                else
                {
                    const P3 ta = pmix( hp[ 1 ], hc[ 1 ], b ), tb = pmix( hp[ 3 ], hc[ 3 ], b );
                    s0 = yj == 1 ? padd( ta, tb ) : padd( padd( s0, ta ), tb );
                }
            }
#pragma unroll
            for( int j = 0; j < 5; j++ ) hp[ j ] = hc[ j ];
        }
    }
    else
    {
        auto     tap = [ & ]( int xj, int yj ) { return bl_sample< M >( src, sw, ax[ xj ], ay[ yj ] ); };
        const P3 t0 = tap( 0, 0 ), t1 = tap( 2, 0 ), t2 = tap( 4, 0 ), t3 = tap( 1, 1 ), t4 = tap( 3, 1 );
        const P3 t5 = tap( 0, 2 ), t6 = tap( 2, 2 ), t7 = tap( 4, 2 ), t8 = tap( 1, 3 ), t9 = tap( 3, 3 );
        const P3 t10 = tap( 0, 4 ), t11 = tap( 2, 4 ), t12 = tap( 4, 4 );
        s0 = padd( padd( padd( t3, t4 ), t8 ), t9 );
        s1 = padd( padd( padd( t0, t1 ), t5 ), t6 );
        s2 = padd( padd( padd( t1, t2 ), t6 ), t7 );
        s3 = padd( padd( padd( t5, t6 ), t10 ), t11 );
        s4 = padd( padd( padd( t6, t7 ), t11 ), t12 );
    }
    const P3 b0 = pmul( s0, 0.25f ), b1 = pmul( s1, 0.25f ), b2 = pmul( s2, 0.25f ), b3 = pmul( s3, 0.25f ), b4 = pmul( s4, 0.25f );
    P3       r;
    if( k == 0 )
    {
        // partial Karis average: each box weighted by 1 / (1 + luminance)
        auto kw = []( P3 bx ) { return 1.0f / ( 1.0f + plum( bx ) ); };
        r       = padd( padd( padd( padd( pmul( b0, 0.5f * kw( b0 ) ), pmul( b1, 0.125f * kw( b1 ) ) ), pmul( b2, 0.125f * kw( b2 ) ) ),
                              pmul( b3, 0.125f * kw( b3 ) ) ),
                        pmul( b4, 0.125f * kw( b4 ) ) );
    }
    else r = padd( padd( padd( padd( pmul( b0, 0.5f ), pmul( b1, 0.125f ) ), pmul( b2, 0.125f ) ), pmul( b3, 0.125f ) ), pmul( b4, 0.125f ) );
    Sto< M >::stpre( dst, (size_t)( y * dw + x ), f3of( r ) );
}

// One texel of upsample step k (CmBloomUpsample.comp:15-104): a 3x3 tent of bilinear taps of
// src (mip k + 1) around the texel's centre plus half a source texel, plus dst's own texel for
// k > 0; dst is mip k, or BLOOM_RESULT for k = 0. The chained case reads the 4x4 source window
// once and shares each row's lerps between the taps above and below it.
template< int M >
__device__ __forceinline__ void bloom_up_texel( const void* src, int sw, int sh, void* dst, int dw, int x, int y, int k, float4 st )
{
    const float isx = st.x, isy = st.y;
    const float iux = st.z, iuy = st.w;
    const float u = ( (float)x + 0.5f ) * iux + 0.5f * isx, v = ( (float)y + 0.5f ) * iuy + 0.5f * isy;
    if( u > 1.0f || v > 1.0f ) return;
    BlAxis ax[ 3 ], ay[ 3 ];
    bool   chain = true;
#pragma unroll
    for( int j = 0; j < 3; j++ )
    {
        ax[ j ] = bl_axis( u + (float)( j - 1 ) * isx, sw );
        ay[ j ] = bl_axis( v + (float)( j - 1 ) * isy, sh );
        if( j > 0 ) chain = chain && ax[ j - 1 ].i1 == ax[ j ].i0 && ay[ j - 1 ].i1 == ay[ j ].i0;
    }
    auto wt = []( int q, int j ) { return ( q == 1 ? 2.0f : 1.0f ) * ( j == 1 ? 0.125f : 0.0625f ); };   // 1 2 1 / 2 4 2 / 1 2 1 over 16
    P3   r  = { make_float2( 0.0f, 0.0f ), 0.0f };
    if( chain )
    {
        const int col[ 4 ] = { ax[ 0 ].i0, ax[ 1 ].i0, ax[ 2 ].i0, ax[ 2 ].i1 };
        P3        hp[ 3 ] = {}, hc[ 3 ];
#pragma unroll
        for( int rr = 0; rr < 4; rr++ )
        {
            const int row = rr < 3 ? ay[ rr ].i0 : ay[ 2 ].i1;
            P3        t[ 4 ];
#pragma unroll
            for( int c = 0; c < 4; c++ ) t[ c ] = bloom_ld< M >( src, (size_t)( row * sw + col[ c ] ) );
#pragma unroll
            for( int j = 0; j < 3; j++ ) hc[ j ] = pmix( t[ j ], t[ j + 1 ], ax[ j ].f );
            if( rr > 0 )
#pragma unroll
                for( int j = 0; j < 3; j++ ) r = padd( r, pmul( pmix( hp[ j ], hc[ j ], ay[ rr - 1 ].f ), wt( rr - 1, j ) ) );
#pragma unroll
            for( int j = 0; j < 3; j++ ) hp[ j ] = hc[ j ];
        }
    }
    else
    {
#pragma unroll
        for( int q = 0; q < 3; q++ )
#pragma unroll
            for( int j = 0; j < 3; j++ ) r = padd( r, pmul( bl_sample< M >( src, sw, ax[ j ], ay[ q ] ), wt( q, j ) ) );
    }
    if( k > 0 ) r = padd( r, bloom_ld< M >( dst, (size_t)( y * dw + x ) ) );
    Sto< M >::stpre( dst, (size_t)( y * dw + x ), f3of( r ) );
}

// MINB 4 for the large steps (more warps in flight at 64 registers), 1 for the small coarse
// steps, whose single wave is bound by one texel's chain of dependent loads; the B10G11R11
// decode of the reference storage mode would spill at 64 registers, so it always takes 1
template< int M, int MINB >
__global__ void __launch_bounds__( 256, M == MODE_REF ? 1 : MINB ) k_bloom_down( const void* src, int sw, int sh, void* dst, int dw, int dh, int k, float4 st )
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    pdl_launch_dependents();
    pdl_wait();
    if( x >= dw || y >= dh ) return;
    bloom_down_texel< M >( src, sw, sh, dst, dw, x, y, k, st );
}

// Upsample step k for the 2x2 quad of dst texels at (x0, y0): the four texels' tents read the
// same 4x4 source window when their texel pairs chain and coincide (the usual case, as dst has
// twice src's resolution), so the window is read once, each row's lerps serve both rows of the
// quad, and each texel keeps its own weights. Returns false, having written nothing, when the
// quad is not complete, a texel is outside the uv <= 1 range or the windows differ.
template< int M >
__device__ __forceinline__ bool bloom_up_quad( const void* src, int sw, int sh, void* dst, int dw, int dh, int x0, int y0, int k, float4 st )
{
    if( x0 + 1 >= dw || y0 + 1 >= dh ) return false;
    const float isx = st.x, isy = st.y;
    const float iux = st.z, iuy = st.w;
    BlAxis      ax[ 2 ][ 3 ], ay[ 2 ][ 3 ];
    bool        ok = true;
#pragma unroll
    for( int i = 0; i < 2; i++ )
    {
        const float u = ( (float)( x0 + i ) + 0.5f ) * iux + 0.5f * isx, v = ( (float)( y0 + i ) + 0.5f ) * iuy + 0.5f * isy;
        ok            = ok && u <= 1.0f && v <= 1.0f;
#pragma unroll
        for( int j = 0; j < 3; j++ )
        {
            ax[ i ][ j ] = bl_axis( u + (float)( j - 1 ) * isx, sw );
            ay[ i ][ j ] = bl_axis( v + (float)( j - 1 ) * isy, sh );
        }
        ok = ok && ax[ i ][ 0 ].i1 == ax[ i ][ 1 ].i0 && ax[ i ][ 1 ].i1 == ax[ i ][ 2 ].i0 && ay[ i ][ 0 ].i1 == ay[ i ][ 1 ].i0 &&
             ay[ i ][ 1 ].i1 == ay[ i ][ 2 ].i0;
    }
#pragma unroll
    for( int j = 0; j < 3; j++ ) ok = ok && ax[ 0 ][ j ].i0 == ax[ 1 ][ j ].i0 && ay[ 0 ][ j ].i0 == ay[ 1 ][ j ].i0;
    ok = ok && ax[ 0 ][ 2 ].i1 == ax[ 1 ][ 2 ].i1 && ay[ 0 ][ 2 ].i1 == ay[ 1 ][ 2 ].i1;
    if( !ok ) return false;
    auto      wt       = []( int q, int j ) { return ( q == 1 ? 2.0f : 1.0f ) * ( j == 1 ? 0.125f : 0.0625f ); };
    const int col[ 4 ] = { ax[ 0 ][ 0 ].i0, ax[ 0 ][ 1 ].i0, ax[ 0 ][ 2 ].i0, ax[ 0 ][ 2 ].i1 };
    P3        r[ 2 ][ 2 ];
#pragma unroll
    for( int q = 0; q < 4; q++ ) r[ q >> 1 ][ q & 1 ] = { make_float2( 0.0f, 0.0f ), 0.0f };
    P3 hp[ 2 ][ 3 ] = {}, hc[ 2 ][ 3 ];
#pragma unroll
    for( int rr = 0; rr < 4; rr++ )
    {
        const int row = rr < 3 ? ay[ 0 ][ rr ].i0 : ay[ 0 ][ 2 ].i1;
        P3        t[ 4 ];
#pragma unroll
        for( int c = 0; c < 4; c++ ) t[ c ] = bloom_ld< M >( src, (size_t)( row * sw + col[ c ] ) );
#pragma unroll
        for( int xi = 0; xi < 2; xi++ )
#pragma unroll
            for( int j = 0; j < 3; j++ ) hc[ xi ][ j ] = pmix( t[ j ], t[ j + 1 ], ax[ xi ][ j ].f );
        if( rr > 0 )
#pragma unroll
            for( int yi = 0; yi < 2; yi++ )
#pragma unroll
                for( int xi = 0; xi < 2; xi++ )
#pragma unroll
                    for( int j = 0; j < 3; j++ )
                        r[ yi ][ xi ] = padd( r[ yi ][ xi ], pmul( pmix( hp[ xi ][ j ], hc[ xi ][ j ], ay[ yi ][ rr - 1 ].f ), wt( rr - 1, j ) ) );
#pragma unroll
        for( int xi = 0; xi < 2; xi++ )
#pragma unroll
            for( int j = 0; j < 3; j++ ) hp[ xi ][ j ] = hc[ xi ][ j ];
    }
#pragma unroll
    for( int q = 0; q < 4; q++ )
    {
        const size_t i = (size_t)( ( y0 + ( q >> 1 ) ) * dw + x0 + ( q & 1 ) );
        P3           o = r[ q >> 1 ][ q & 1 ];
        if( k > 0 ) o = padd( o, bloom_ld< M >( dst, i ) );
        Sto< M >::stpre( dst, i, f3of( o ) );
    }
    return true;
}

// one thread per dst texel (the small coarse steps)
template< int M >
__global__ void __launch_bounds__( 256 ) k_bloom_up( const void* src, int sw, int sh, void* dst, int dw, int dh, int k, float4 st )
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    pdl_launch_dependents();
    pdl_wait();
    if( x >= dw || y >= dh ) return;
    bloom_up_texel< M >( src, sw, sh, dst, dw, x, y, k, st );
}

// one thread per 2x2 quad of dst texels, blocks of 32x4 threads (the large steps)
template< int M >
__global__ void __launch_bounds__( 128 ) k_bloom_up_quad( const void* src, int sw, int sh, void* dst, int dw, int dh, int k, float4 st )
{
    const int x0 = 2 * ( blockIdx.x * blockDim.x + threadIdx.x ), y0 = 2 * ( blockIdx.y * blockDim.y + threadIdx.y );
    pdl_launch_dependents();
    pdl_wait();
    if( x0 >= dw || y0 >= dh ) return;
    if( bloom_up_quad< M >( src, sw, sh, dst, dw, dh, x0, y0, k, st ) ) return;
#pragma unroll 1
    for( int q = 0; q < 4; q++ )
    {
        const int x = x0 + ( q & 1 ), y = y0 + ( q >> 1 );
        if( x < dw && y < dh ) bloom_up_texel< M >( src, sw, sh, dst, dw, x, y, k, st );
    }
}

// FINAL += intensity * BLOOM_RESULT(uv) (CmBloomApply.comp:45-76, lens dirt not included)
template< int M > __global__ void __launch_bounds__( 256 ) k_bloom_apply( const void* result, void* finalImg, int W, int H, float2 inv, float intensity )
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    pdl_launch_dependents();
    pdl_wait();
    if( x >= W || y >= H ) return;
    const float u = ( (float)x + 0.5f ) * inv.x, v = ( (float)y + 0.5f ) * inv.y;   // inv = (1 / W, 1 / H)
    if( u > 1.0f || v > 1.0f ) return;
    const P3     bloom = pmul( bl_sample< M >( result, W, bl_axis( u, W ), bl_axis( v, H ) ), intensity );
    const size_t i     = (size_t)( y * W + x );
    Sto< M >::stpre( finalImg, i, f3of( padd( bloom_ld< M >( finalImg, i ), bloom ) ) );
}

// ==========================================================================================
// Volumetric::ProcessScattering: CmVolumetricProcess.comp and CmScatterAccum.comp
// ==========================================================================================
__device__ __forceinline__ float4 h4f( ushort4 h ) { return make_float4( h2f( h.x ), h2f( h.y ), h2f( h.z ), h2f( h.w ) ); }
__device__ __forceinline__ ushort4 f4h( float4 v ) { return make_ushort4( f32_to_f16( v.x ), f32_to_f16( v.y ), f32_to_f16( v.z ), f32_to_f16( v.w ) ); }
__device__ __forceinline__ float4 vmix4( float4 x, float4 y, float a )
{
    return make_float4( gmix( x.x, y.x, a ), gmix( x.y, y.y, a ), gmix( x.z, y.z, a ), gmix( x.w, y.w, a ) );
}

// CmVolumetricProcess.comp:58-79 (accumulateScattering, store): one thread per froxel column,
// front to back. The running (light, extinction) stays in FP32; cell z stores
// (light, exp(-extinction)) over the cell's own (in-scatter, extinction), which it has read.
template< int M > __global__ void __launch_bounds__( 128 ) k_volume_process( ushort4* vol, int nx, int ny, int nz )
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    pdl_launch_dependents();
    pdl_wait();
    if( x >= nx || y >= ny ) return;
    const size_t  slice = (size_t)nx * ny;
    ushort4*      col   = vol + (size_t)y * nx + x;
    // The column is walked in chunks of VP cells, the next chunk's loads issued before the
    // current chunk's stores: every cell is still read before it is written, and the loads of a
    // chunk are in flight together instead of one per step.
    constexpr int VP = 8;
    ushort4       cur[ VP ], nxt[ VP ];
#pragma unroll
    for( int j = 0; j < VP; j++ ) cur[ j ] = j < nz ? col[ j * slice ] : make_ushort4( 0, 0, 0, 0 );
    float4 acc = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
    float  e   = 1.0f;
    for( int z0 = 0; z0 < nz; z0 += VP )
    {
#pragma unroll
        for( int j = 0; j < VP; j++ ) nxt[ j ] = z0 + VP + j < nz ? col[ ( z0 + VP + j ) * slice ] : make_ushort4( 0, 0, 0, 0 );
#pragma unroll
        for( int j = 0; j < VP; j++ )
        {
            const int z = z0 + j;
            if( z >= nz ) break;
            const float4 v = h4f( cur[ j ] );
            if( z == 0 ) acc = v;
            else
            {
                const float t = gsat( e );   // saturate( exp( -front.a ) )
                acc           = make_float4( acc.x + t * v.x, acc.y + t * v.y, acc.z + t * v.z, acc.w + v.w );
            }
            e                = expf( -acc.w );
            col[ z * slice ] = f4h( make_float4( acc.x, acc.y, acc.z, e ) );
        }
#pragma unroll
        for( int j = 0; j < VP; j++ ) cur[ j ] = nxt[ j ];
    }
}

// an index from a floor()ed coordinate: NaN to 0, magnitudes beyond 2^30 saturated, so that
// the conversion is defined for every input
__device__ __forceinline__ int safe_floor_int( float f ) { return f == f ? (int)fminf( fmaxf( f, -1073741824.0f ), 1073741824.0f ) : 0; }

// textureLod of the processed volume with the linear clamp-to-edge sampler (Volumetric.cpp:
// 236-256): lerps along x, then y, then z, in FP32
__device__ __forceinline__ float4 volume_trilinear( const ushort4* vol, int nx, int ny, int nz, float3 sp )
{
    auto axis = []( float u, int n, int& i0, int& i1, float& f ) {
        const float x  = u * (float)n - 0.5f;
        const float fx = floorf( x );
        const int   ix = safe_floor_int( fx );
        i0             = min( max( ix, 0 ), n - 1 );
        i1             = min( max( ix, -1 ) + 1, n - 1 );
        f              = x - fx;
    };
    int   x0, x1, y0, y1, z0, z1;
    float fx, fy, fz;
    axis( sp.x, nx, x0, x1, fx );
    axis( sp.y, ny, y0, y1, fy );
    axis( sp.z, nz, z0, z1, fz );
    auto t = [ & ]( int x, int y, int z ) { return h4f( vol[ ( (size_t)z * ny + y ) * nx + x ] ); };
    const float4 c00 = vmix4( t( x0, y0, z0 ), t( x1, y0, z0 ), fx ), c10 = vmix4( t( x0, y1, z0 ), t( x1, y1, z0 ), fx );
    const float4 c01 = vmix4( t( x0, y0, z1 ), t( x1, y0, z1 ), fx ), c11 = vmix4( t( x0, y1, z1 ), t( x1, y1, z1 ), fx );
    return vmix4( vmix4( c00, c10, fy ), vmix4( c01, c11, fy ), fz );
}

// volume_toSamplePosition_T (Volumetric.h:38-58) with VOLUMETRIC_DISTANCE_POW 1
// FAST: reciprocal multiplies and the hardware square root (continuous in every term)
template< bool FAST > __device__ __forceinline__ float3 volume_sample_pos( const ScatterArgs& a, float3 w )
{
    const float4 ndc = mat_mul( a.volumeViewProj, make_float4( w.x, w.y, w.z, 1.0f ) );
    const float  iw  = FAST ? rcp_approx( ndc.w ) : 0.0f;
    const float  nx = FAST ? ndc.x * iw : ndc.x / ndc.w, ny = FAST ? ndc.y * iw : ndc.y / ndc.w;
    const float  dx = w.x - a.camPos[ 0 ], dy = w.y - a.camPos[ 1 ], dz = w.z - a.camPos[ 2 ];
    const float  d2 = dx * dx + dy * dy + dz * dz;
    const float  dist = FAST ? sqrt_approx( d2 ) : sqrtf( d2 );
    const float  zr   = FAST ? ( dist - a.volNear ) * a.iRange : ( dist - a.volNear ) / ( a.volFar - a.volNear );
    const float  z    = gclamp( zr, 0.0f, 1.0f );   // pow( z, 1 ) == z
    return f3( nx * 0.5f + 0.5f, ny * 0.5f + 0.5f, z );
}

// fializeScattering (CmScatterAccum.comp:41-95) at regular pixel (rx, ry); depthCb is
// DEPTH_WORLD at its checkerboard position
template< bool FAST >
__device__ __forceinline__ float4 finalize_scattering( const ScatterArgs& a, int rx, int ry, float depthCb, const float* inv255 )
{
    if( a.enableType == RGDN_VOLUME_ENABLE_VOLUMETRIC )
    {
        const float  sx  = FAST ? (float)rx * a.irw : (float)rx / a.u.rw, sy = FAST ? (float)ry * a.irh : (float)ry / a.u.rh;
        const float4 ndc = make_float4( sx * 2.0f - 1.0f, sy * 2.0f - 1.0f, a.depthNdc[ (size_t)ry * a.u.W + rx ], 1.0f );
        const float4 wp  = mat_mul( a.invViewProj, ndc );
        const float  iw  = FAST ? rcp_approx( wp.w ) : 0.0f;
        const float3 pos = FAST ? f3( wp.x * iw, wp.y * iw, wp.z * iw ) : f3( wp.x / wp.w, wp.y / wp.w, wp.z / wp.w );
        // rnd8_4( getRandomSeed( pix, frameId ), 0 ).xyz
        // byte / 255 from a table of the IEEE quotients
        const uint32_t rnd = wellons_lowbias32( random_seed( rx, ry, a.frameId ) );
        const float    r0 = inv255[ rnd & 0xFFu ], r1 = inv255[ ( rnd >> 8 ) & 0xFFu ], r2 = inv255[ ( rnd >> 16 ) & 0xFFu ];
        // sampleHemisphere (Random.h:73-92)
        const float u1 = r0 * 0.99f, u2 = r1 * 0.99f;
        const float rr = FAST ? sqrt_approx( u1 ) : sqrtf( u1 ), phi = ( 2.0f * 3.14159265358979f ) * u2;
        const float hz = FAST ? sqrt_approx( 1.0f - u1 ) : sqrtf( 1.0f - u1 );
        float       sphi, cphi;
        if( FAST ) __sincosf( phi, &sphi, &cphi );
        else sincosf( phi, &sphi, &cphi );
        const float3 basis = f3( -( rr * cphi ), -( rr * sphi ), -hz );
        // volume_sampleDithered (Volumetric.h:92-104), dither radius 2; / 64 is the exact * 2^-6
        float3      sp = volume_sample_pos< FAST >( a, pos );
        const float k  = r2 * 2.0f;
        const float dx = FAST ? ( k * basis.x ) * ( 1.0f / (float)RGDN_VOLUME_SIZE_X ) : ( k * basis.x ) / (float)a.nx;
        const float dy = FAST ? ( k * basis.y ) * ( 1.0f / (float)RGDN_VOLUME_SIZE_Y ) : ( k * basis.y ) / (float)a.ny;
        sp             = f3( sp.x + dx, sp.y + dy, sp.z + ( k * basis.z ) * 0.015625f );
        return volume_trilinear( a.volume, a.nx, a.ny, a.nz, sp );
    }
    if( a.enableType == RGDN_VOLUME_ENABLE_SIMPLE )
    {
        if( depthCb > MAX_RAY_LENGTH ) return make_float4( 0.0f, 0.0f, 0.0f, 1.0f );
        const float f = FAST ? ex2_approx( ( -depthCb * a.density ) * 1.44269504088896341f ) : expf( -depthCb * a.density );
        return make_float4( a.ambient[ 0 ] * ( 1.0f - f ), a.ambient[ 1 ] * ( 1.0f - f ), a.ambient[ 2 ] * ( 1.0f - f ), f );
    }
    return make_float4( 0.0f, 0.0f, 0.0f, 1.0f );
}

// CmScatterAccum.comp:97-161 for checkerboard pixel (cx, cy); returns the new scattering and
// history length
template< bool FAST >
__device__ __forceinline__ float4 scatter_pixel( const ScatterArgs& a, int cx, int cy, const float* inv255, float& histOut )
{
    const size_t ci    = (size_t)cy * a.u.W + cx;
    const float4 mo    = h4f( a.motion[ ci ] );
    const float  depth = h2f( a.depth[ ci ] );
    auto         nrm   = [ & ]( uint32_t p ) {
        const float2 ph = __ldg( &a.phiTab[ p >> 16 ] ), th = __ldg( &a.thetaTab[ p & 0xFFFFu ] );
        return f3( ph.x * th.x, ph.x * th.y, ph.y );
    };
    const float3 normal = nrm( a.normal[ ci ] );
    const float  rz     = rcp_approx( fabsf( depth ) );   // testReprojectedDepth through test_depth_r
    const float2 pp     = prev_screen_pos( a.u, make_float2( mo.x, mo.y ), cx, cy );
    const float  fpx = floorf( pp.x - 0.5f ), fpy = floorf( pp.y - 0.5f );
    const int    px = safe_floor_int( fpx ), py = safe_floor_int( fpy );
    const float  sx = ( pp.x - 0.5f ) - fpx, sy = ( pp.y - 0.5f ) - fpy;
    const float  bw[ 2 ][ 2 ] = { { ( 1.0f - sx ) * ( 1.0f - sy ), sx * ( 1.0f - sy ) }, { ( 1.0f - sx ) * sy, sx * sy } };
    const Area   area = cb_area( a.u, cx );
    float4       acc  = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
    float        hist = 0.0f, wsum = 0.0f;
#pragma unroll
    for( int yy = 0; yy <= 1; yy++ )
#pragma unroll
        for( int xx = 0; xx <= 1; xx++ )
        {
            const int qx = px + xx, qy = py + yy;
            if( !in_area( qx, qy, area ) ) continue;
            const size_t qi = (size_t)qy * a.u.W + qx;
            if( test_depth_r( depth, rz, h2f( a.depthPrev[ qi ] ), mo.z ) && test_normal( normal, nrm( a.normalPrev[ qi ] ) ) )
            {
                const float  w  = bw[ yy ][ xx ];
                const int2   r  = regular_from_cb( a.u, qx, qy );
                const size_t ri = (size_t)r.y * a.u.W + r.x;
                const float4 v  = h4f( a.scatterPrev[ ri ] );
                acc             = make_float4( acc.x + w * v.x, acc.y + w * v.y, acc.z + w * v.z, acc.w + w * v.w );
                hist            = hist + w * h2f( a.historyPrev[ ri ] );
                wsum            = wsum + w;
            }
        }
    const bool ok = wsum > 0.0001f;
    if( FAST )
    {
        const float iws = rcp_approx( wsum );
        hist            = ok ? hist * iws : 0.0f;
        acc             = ok ? make_float4( acc.x * iws, acc.y * iws, acc.z * iws, acc.w * iws ) : make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
    }
    else
    {
        hist = ok ? hist / wsum : 0.0f;
        acc  = ok ? make_float4( acc.x / wsum, acc.y / wsum, acc.z / wsum, acc.w / wsum ) : make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
    }
    hist           = gclamp( hist + 1.0f, 1.0f, fmaxf( 1.0f, a.maxHistoryLength ) );
    const int2 reg = regular_from_cb( a.u, cx, cy );
    histOut        = hist;
    return vmix4( acc, finalize_scattering< FAST >( a, reg.x, reg.y, depth, inv255 ), FAST ? rcp_approx( hist ) : 1.0f / hist );
}

// One thread per checkerboard pixel. (One thread per pair (cx, cx + W/2), whose regular pixels
// are neighbours, wrote full sectors but ran 10 % slower: half the warps to hide latency.)
template< int M, bool FAST > __global__ void __launch_bounds__( 256, 6 ) k_scatter_accum( const ScatterArgs a )
{
    __shared__ float inv255[ 256 ];
    for( int t = threadIdx.y * blockDim.x + threadIdx.x; t < 256; t += blockDim.x * blockDim.y ) inv255[ t ] = u8_value( t );
    __syncthreads();
    const int cx = blockIdx.x * blockDim.x + threadIdx.x, cy = blockIdx.y * blockDim.y + threadIdx.y;
    pdl_launch_dependents();
    pdl_wait();
    if( cx >= a.u.W || cy >= a.u.H ) return;
    float        hist;
    const float4 acc = scatter_pixel< FAST >( a, cx, cy, inv255, hist );
    const int2   reg = regular_from_cb( a.u, cx, cy );
    const size_t ri  = (size_t)reg.y * a.u.W + reg.x;
    a.scatterOut[ ri ] = f4h( acc );
    a.historyOut[ ri ] = f32_to_f16( hist );
}

}  // namespace dev


// ------------------------------------------------------------------------------------------
// launcher for one mode
// ------------------------------------------------------------------------------------------
template< int M > cudaError_t launch_stage_t( const FrameArgs& a, int stage, int iter, cudaStream_t s )
{
    cudaError_t e = cudaSuccess;
    const dim3 blk( 32, 8 );
    const dim3 grid( ( a.u.W + 31 ) / 32, ( a.u.H + 7 ) / 8 );
    const dim3 gridG( ( a.u.GW + 31 ) / 32, ( a.u.GH + 7 ) / 8 );
    switch( stage )
    {
        case RGDN_STAGE_GRADIENT_SAMPLES: e = launch_pdl( dev::k_gradient_samples< M >, gridG, blk, 0, s, a, a.disPing ); break;
        case RGDN_STAGE_GRADIENT_ATROUS: e = launch_pdl( dev::k_gradient_atrous< M >, gridG, blk, 0, s, a, iter ); break;
        case RGDN_STAGE_TEMPORAL_ACCUMULATION: e = launch_pdl( dev::k_temporal< M, false, false, false >, grid, blk, 0, s, a ); break;
        case KF_TEMPORAL_EXACT_GEOM: e = launch_pdl( dev::k_temporal< M, false, true, false >, grid, blk, 0, s, a ); break;
        case KF_TEMPORAL_EXACT_GEOM_GP: e = launch_pdl( dev::k_temporal< M, false, true, true >, grid, blk, 0, s, a ); break;
        case KF_TEMPORAL_FAST:
            e = launch_pdl( dev::k_temporal< M, true, true, false, 128, 8 >, dim3( grid.x, ( a.u.H + 3 ) / 4 ), dim3( 32, 4 ), 0, s, a );
            break;
        case KF_TEMPORAL_FAST_GP:
            e = launch_pdl( dev::k_temporal< M, true, true, true, 128, 8 >, dim3( grid.x, ( a.u.H + 3 ) / 4 ), dim3( 32, 4 ), 0, s, a );
            break;
        case KF_TEMPORAL_FAST_EARLY:
            e = launch_pdl( dev::k_temporal< M, true, true, false, 128, 8, true >, dim3( grid.x, ( a.u.H + 3 ) / 4 ), dim3( 32, 4 ), 0, s, a );
            break;
        case KF_TEMPORAL_FAST_GP_EARLY:
            e = launch_pdl( dev::k_temporal< M, true, true, true, 128, 8, true >, dim3( grid.x, ( a.u.H + 3 ) / 4 ), dim3( 32, 4 ), 0, s, a );
            break;
        case KF_ANTI_FIREFLY_FAST:
            e = launch_pdl( dev::k_antifirefly_fast< M >, dim3( grid.x, ( a.u.H + dev::AfShared< M >::TH - 1 ) / dev::AfShared< M >::TH ), blk, 0, s, a );
            break;
        case KF_VARIANCE_EXACT_GEOM: e = launch_pdl( dev::k_variance_geo< M, false >, grid, blk, 0, s, a ); break;
        case RGDN_STAGE_ANTI_FIREFLY: dev::k_antifirefly< M ><<< grid, blk, 0, s >>>( a ); break;
        case RGDN_STAGE_VARIANCE_ESTIMATION: dev::k_variance< M ><<< grid, blk, 0, s >>>( a ); break;
        case RGDN_STAGE_ATROUS: e = launch_pdl( dev::k_atrous< M, false, false, false >, grid, blk, 0, s, a, iter ); break;
        case KF_ATROUS_EXACT: e = launch_pdl( dev::k_atrous< M, false, false, true >, grid, blk, 0, s, a, iter ); break;
        case RGDN_STAGE_LUMINANCE_HISTOGRAM: dev::k_histogram< M ><<< grid, blk, 0, s >>>( a ); break;
        case RGDN_STAGE_LUMINANCE_AVG: e = launch_pdl( dev::k_luminance_avg< M >, 1, 256, 0, s, a ); break;
        case KF_ATROUS_EXACT_HIST: e = launch_pdl( dev::k_atrous< M, false, true, true >, grid, blk, 0, s, a, iter ); break;
        default: return cudaErrorInvalidValue;
    }
    return e != cudaSuccess ? e : cudaGetLastError();
}

// the bloom pyramid over planes[0] = BLOOM_INPUT, planes[1..8] = mips, planes[9] = BLOOM_RESULT,
// planes[10] = FINAL; w/h per plane
template< int M > cudaError_t launch_bloom_t( const BloomArgs& b, cudaStream_t s )
{
    const dim3  blk( 32, 8 );
    auto        grid  = []( int w, int h ) { return dim3( ( w + 31 ) / 32, ( h + 7 ) / 8 ); };
    auto        large = [ & ]( int p ) { return (long long)b.w[ p ] * b.h[ p ] >= BLOOM_LARGE_TEXELS; };
    cudaError_t e     = cudaSuccess;
    // the texel steps of level k in uv, (2^(k+1) / W, 2^(k+1) / H, 2^k / W, 2^k / H): the IEEE
    // quotients every texel of the shaders computes, evaluated once
    auto st = [ & ]( int k ) {
        return make_float4( (float)( 1 << ( k + 1 ) ) / (float)b.W, (float)( 1 << ( k + 1 ) ) / (float)b.H, (float)( 1 << k ) / (float)b.W,
                            (float)( 1 << k ) / (float)b.H );
    };
    for( int k = 0; k < 8 && e == cudaSuccess; k++ )
        e = launch_pdl( large( k + 1 ) ? dev::k_bloom_down< M, 4 > : dev::k_bloom_down< M, 1 >, grid( b.w[ k + 1 ], b.h[ k + 1 ] ), blk, 0, s,
                        (const void*)b.planes[ k ], b.w[ k ], b.h[ k ], b.planes[ k + 1 ], b.w[ k + 1 ], b.h[ k + 1 ], k, st( k ) );
    for( int k = 7; k >= 0 && e == cudaSuccess; k-- )
    {
        const int d = k == 0 ? 9 : k;
        if( large( d ) )
            e = launch_pdl( dev::k_bloom_up_quad< M >, dim3( ( b.w[ d ] + 63 ) / 64, ( b.h[ d ] + 7 ) / 8 ), dim3( 32, 4 ), 0, s,
                            (const void*)b.planes[ k + 1 ], b.w[ k + 1 ], b.h[ k + 1 ], b.planes[ d ], b.w[ d ], b.h[ d ], k, st( k ) );
        else
            e = launch_pdl( dev::k_bloom_up< M >, grid( b.w[ d ], b.h[ d ] ), blk, 0, s, (const void*)b.planes[ k + 1 ], b.w[ k + 1 ], b.h[ k + 1 ],
                            b.planes[ d ], b.w[ d ], b.h[ d ], k, st( k ) );
    }
    if( e == cudaSuccess )
        e = launch_pdl( dev::k_bloom_apply< M >, grid( b.W, b.H ), blk, 0, s, (const void*)b.planes[ 9 ], b.planes[ 10 ], b.W, b.H,
                        make_float2( 1.0f / (float)b.W, 1.0f / (float)b.H ), b.intensity );
    return e != cudaSuccess ? e : cudaGetLastError();
}

template< int M > cudaError_t launch_scatter_t( const ScatterArgs& a, cudaStream_t s )
{
    cudaError_t e = launch_pdl( dev::k_volume_process< M >, dim3( ( a.nx + 31 ) / 32, ( a.ny + 3 ) / 4 ), dim3( 32, 4 ), 0, s, a.volume, a.nx, a.ny, a.nz );
    const dim3 g( ( a.u.W + 31 ) / 32, ( a.u.H + 7 ) / 8 ), b( 32, 8 );
    if( e == cudaSuccess )
        e = ( a.flags & RGDN_VOLUME_EXACT_MATH ) ? launch_pdl( dev::k_scatter_accum< M, false >, g, b, 0, s, a )
                                                  : launch_pdl( dev::k_scatter_accum< M, true >, g, b, 0, s, a );
    return e != cudaSuccess ? e : cudaGetLastError();
}

template< int M > cudaError_t launch_final_t( const FinalArgs& f, cudaStream_t s )
{
    const dim3        g( ( f.W + 31 ) / 32, ( f.H + 7 ) / 8 ), b( 32, 8 );
    const cudaError_t e = ( f.flags & RGDN_FINAL_EXACT_MATH ) ? launch_pdl( dev::k_prepare_final< M, false >, g, b, 0, s, f )
                                                             : launch_pdl( dev::k_prepare_final< M, true >, g, b, 0, s, f );
    return e != cudaSuccess ? e : cudaGetLastError();
}

// a-trous iterations 0 and 1 in one launch (the caller ensures iteration 1 is not the last)
template< int M > cudaError_t launch_atrous_pair01( const FrameArgs& a, cudaStream_t s )
{
    using P     = dev::AtPair;
    auto kernel = dev::k_atrous_pair01< M, 3 >;
    static std::atomic< uint64_t > enabled( 0 );
    int                            d = 0;
    if( cudaGetDevice( &d ) != cudaSuccess ) return cudaErrorInvalidDevice;
    const uint64_t bit = 1ull << ( d & 63 );
    if( !( enabled.load( std::memory_order_relaxed ) & bit ) )
    {
        const cudaError_t e = cudaFuncSetAttribute( kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, P::SMEM );
        if( e != cudaSuccess ) return e;
        enabled.fetch_or( bit, std::memory_order_relaxed );
    }
    return launch_pdl( kernel, dim3( ( a.u.W + P::TW - 1 ) / P::TW, ( a.u.H + P::TH - 1 ) / P::TH ), dim3( 32, 8 ), P::SMEM, s, a );
}

// The default a-trous kernel (32x4 tiles, 7 blocks per SM), built per iteration for the first
// five iterations (steps 1 to 16)
template< int M, bool HIST > cudaError_t launch_atrous_fast( const FrameArgs& a, const int iter, cudaStream_t s )
{
    const dim3 grid( ( a.u.W + 31 ) / 32, ( a.u.H + 3 ) / 4 ), blk( 32, 4 );
    switch( iter )
    {
        case 0: return launch_pdl( dev::k_atrous< M, true, HIST, true, 128, 7, 0 >, grid, blk, 0, s, a, iter );
        case 1: return launch_pdl( dev::k_atrous< M, true, HIST, true, 128, 7, 1 >, grid, blk, 0, s, a, iter );
        case 2: return launch_pdl( dev::k_atrous< M, true, HIST, true, 128, 7, 2 >, grid, blk, 0, s, a, iter );
        case 3: return launch_pdl( dev::k_atrous< M, true, HIST, true, 128, 7, 3 >, grid, blk, 0, s, a, iter );
        case 4: return launch_pdl( dev::k_atrous< M, true, HIST, true, 128, 7, 4 >, grid, blk, 0, s, a, iter );
        default: return launch_pdl( dev::k_atrous< M, true, HIST, true, 128, 7 >, grid, blk, 0, s, a, iter );
    }
}

// Kernels whose results are continuous in every arithmetic operation (no threshold follows
// them), in their own translation units (rgdn_fast_*.cu); their weighted sums use explicit
// fused multiply-adds.
template< int M > cudaError_t launch_fast_t( const FrameArgs& a, int stage, int iter, cudaStream_t s )
{
    cudaError_t e = cudaSuccess;
    const dim3 blk( 32, 8 );
    const dim3 grid( ( a.u.W + 31 ) / 32, ( a.u.H + 7 ) / 8 );
    switch( stage )
    {
        case KF_ATROUS_FAST: e = launch_atrous_fast< M, false >( a, iter, s ); break;
        case KF_ATROUS_FAST_HIST: e = launch_atrous_fast< M, true >( a, iter, s ); break;
        case KF_VARIANCE_FAST: e = launch_pdl( dev::k_variance_geo< M, true >, grid, blk, 0, s, a ); break;
        case KF_ATROUS_PAIR01: e = launch_atrous_pair01< M >( a, s ); break;
        case KF_AF_VARIANCE_FAST:
        case KF_AF_VARIANCE_EXACT:
        {
            const dim3 g( grid.x, ( a.u.H + dev::AfShared< M >::TH - 1 ) / dev::AfShared< M >::TH );
            e = stage == KF_AF_VARIANCE_FAST ? launch_pdl( dev::k_af_variance< M, true >, g, blk, 0, s, a )
                                             : launch_pdl( dev::k_af_variance< M, false >, g, blk, 0, s, a );
            break;
        }
        default: return cudaErrorInvalidValue;
    }
    return e != cudaSuccess ? e : cudaGetLastError();
}

// Batched launches. `iter` carries variants in its high bits: for the temporal pass the
// previous-record mode GPM (bits 8-9); for a-trous the histogram mode HM (bits 8-9) and the
// resident blocks per SM it is built for (bits 10-12: 3 or 4, i.e. 80 or 64 registers).
template< int M > cudaError_t launch_batch_t( int stage, int iter, int slot, dim3 block, int grid, cudaStream_t s )
{
    cudaError_t e = cudaSuccess;
    const int v = ( iter >> 8 ) & 3, it = iter & 0xff;
    switch( stage )
    {
        case RGDN_STAGE_GRADIENT_SAMPLES: e = launch_pdl( dev::kb_gradient_samples< M >, grid, block, 0, s, slot ); break;
        case RGDN_STAGE_GRADIENT_ATROUS: e = launch_pdl( dev::kb_gradient_atrous< M >, grid, block, 0, s, slot, it ); break;
        case RGDN_STAGE_TEMPORAL_ACCUMULATION:
            if( ( ( iter >> 10 ) & 7 ) == 7 )
            {
                if( v == 0 ) e = launch_pdl( dev::kt_temporal< M, 0 >, grid, block, 0, s, slot );
                else if( v == 1 ) e = launch_pdl( dev::kt_temporal< M, 1 >, grid, block, 0, s, slot );
                else e = launch_pdl( dev::kt_temporal< M, 2 >, grid, block, 0, s, slot );
            }
            else if( v == 0 ) e = launch_pdl( dev::kb_temporal< M, 0 >, grid, block, 0, s, slot );
            else if( v == 1 ) e = launch_pdl( dev::kb_temporal< M, 1 >, grid, block, 0, s, slot );
            else e = launch_pdl( dev::kb_temporal< M, 2 >, grid, block, 0, s, slot );
            break;
        case RGDN_STAGE_ANTI_FIREFLY: e = launch_pdl( dev::kb_antifirefly< M >, grid, block, 0, s, slot ); break;
        case RGDN_STAGE_LUMINANCE_AVG: e = launch_pdl( dev::kb_luminance_avg< M >, grid, 256, 0, s, slot ); break;
        default: return cudaErrorInvalidValue;
    }
    return e != cudaSuccess ? e : cudaGetLastError();
}
template< int M > cudaError_t launch_batch_fast_t( int stage, int iter, int slot, dim3 block, int grid, cudaStream_t s )
{
    cudaError_t e = cudaSuccess;
    switch( stage )
    {
        case RGDN_STAGE_VARIANCE_ESTIMATION:
            e = ( ( iter >> 10 ) & 7 ) == 7 ? launch_pdl( dev::kt_variance< M >, grid, block, 0, s, slot )
                                            : launch_pdl( dev::kb_variance< M >, grid, block, 0, s, slot );
            break;
        case RGDN_STAGE_ATROUS:
        {
            const int hm = ( iter >> 8 ) & 3, occ = ( iter >> 10 ) & 7, it = iter & 0xff;
            switch( occ * 4 + hm )
            {
                case 12: e = launch_pdl( dev::kb_atrous< M, 0, 3 >, grid, block, 0, s, slot, it ); break;
                case 13: e = launch_pdl( dev::kb_atrous< M, 1, 3 >, grid, block, 0, s, slot, it ); break;
                case 14: e = launch_pdl( dev::kb_atrous< M, 2, 3 >, grid, block, 0, s, slot, it ); break;
                case 16: e = launch_pdl( dev::kb_atrous< M, 0, 4 >, grid, block, 0, s, slot, it ); break;
                case 17: e = launch_pdl( dev::kb_atrous< M, 1, 4 >, grid, block, 0, s, slot, it ); break;
                case 18: e = launch_pdl( dev::kb_atrous< M, 2, 4 >, grid, block, 0, s, slot, it ); break;
                case 24:
                case 25:
                case 26:
                {
                    // occupancy code 6: iterations 0 and 1 in one launch (fusion depth 2)
                    auto kernel = dev::kt_atrous_pair01< M >;
                    static std::atomic< uint64_t > enabled( 0 );
                    int                            d = 0;
                    if( cudaGetDevice( &d ) != cudaSuccess ) return cudaErrorInvalidDevice;
                    const uint64_t bit = 1ull << ( d & 63 );
                    if( !( enabled.load( std::memory_order_relaxed ) & bit ) )
                    {
                        if( ( e = cudaFuncSetAttribute( kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dev::AtPair::SMEM ) ) != cudaSuccess )
                            return e;
                        enabled.fetch_or( bit, std::memory_order_relaxed );
                    }
                    e = launch_pdl( kernel, grid, block, dev::AtPair::SMEM, s, slot );
                    break;
                }
                case 28: e = launch_pdl( dev::kt_atrous< M, 0 >, grid, block, 0, s, slot, it ); break;
                case 29: e = launch_pdl( dev::kt_atrous< M, 1 >, grid, block, 0, s, slot, it ); break;
                case 30: e = launch_pdl( dev::kt_atrous< M, 2 >, grid, block, 0, s, slot, it ); break;
                default: return cudaErrorInvalidValue;
            }
            break;
        }
        default: return cudaErrorInvalidValue;
    }
    return e != cudaSuccess ? e : cudaGetLastError();
}
template< class K > int blocks_per_sm( K kernel, int threads = 256 )
{
    int n = 0;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor( &n, kernel, threads, 0 ) == cudaSuccess ? n : 0;
}
template< int M > int batch_blocks_per_sm_t( int stage )
{
    switch( stage )
    {
        case RGDN_STAGE_GRADIENT_SAMPLES: return blocks_per_sm( dev::kb_gradient_samples< M > );
        case RGDN_STAGE_GRADIENT_ATROUS: return blocks_per_sm( dev::kb_gradient_atrous< M > );
        case RGDN_STAGE_TEMPORAL_ACCUMULATION: return blocks_per_sm( dev::kb_temporal< M, 2 > );
        case RGDN_STAGE_TEMPORAL_ACCUMULATION | ( 7 << 10 ): return blocks_per_sm( dev::kt_temporal< M, 2 >, 128 );
        case RGDN_STAGE_ANTI_FIREFLY: return blocks_per_sm( dev::kb_antifirefly< M > );
        case RGDN_STAGE_LUMINANCE_AVG: return blocks_per_sm( dev::kb_luminance_avg< M > );
        default: return 0;
    }
}
template< int M > int batch_blocks_per_sm_fast_t( int stage )
{
    switch( stage )
    {
        case RGDN_STAGE_VARIANCE_ESTIMATION: return blocks_per_sm( dev::kb_variance< M > );
        case RGDN_STAGE_ATROUS | ( 3 << 10 ): return blocks_per_sm( dev::kb_atrous< M, 2, 3 > );
        case RGDN_STAGE_ATROUS | ( 4 << 10 ): return blocks_per_sm( dev::kb_atrous< M, 2, 4 > );
        case RGDN_STAGE_ATROUS | ( 7 << 10 ): return blocks_per_sm( dev::kt_atrous< M, 2 >, 128 );
        default: return 0;
    }
}
// device address of this module's constant slot (for the host's copy of a step's table);
// internal linkage, like c_batch: every translation unit answers for its own module
static inline void* batch_slot_t( int slot )
{
    void* p = nullptr;
    if( slot < 0 || slot >= BATCH_SLOTS || cudaGetSymbolAddress( &p, dev::c_batch ) != cudaSuccess ) return nullptr;
    return static_cast< BatchConst* >( p ) + slot;
}

template< int M > cudaError_t launch_atrous_tma_t( const FrameArgs& a, int iter, bool hist, const void* maps, cudaStream_t s )
{
    const AtrousMaps& m = *static_cast< const AtrousMaps* >( maps );
    return hist ? dev::launch_atrous_tma< M, true, true >( a, iter, m, s ) : dev::launch_atrous_tma< M, true, false >( a, iter, m, s );
}
template< int M > int atrous_tma_smem_t( int iter ) { return 2 * dev::tma_geom< M >( iter ).bytes; }

}  // namespace rgdn
