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

#include <cooperative_groups.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "rgdn_codec.h"
#include "rgdn_internal.h"

namespace rgdn
{
namespace dev
{
namespace cg = cooperative_groups;

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
template< bool FAST > struct Wm;
template<> struct Wm< false >
{
    __device__ static float pow128( float x ) { return powf( x, 128.0f ); }
    __device__ static float powv( float x, float y ) { return powf( x, y ); }
    __device__ static float expn( float x ) { return expf( x ); }
    __device__ static float madd( float a, float b, float c ) { return a * b + c; }
};
template<> struct Wm< true >
{
    __device__ static float pow128( float x )
    {
        x = x * x; x = x * x; x = x * x; x = x * x; x = x * x; x = x * x; x = x * x;
        return x;
    }
    __device__ static float powv( float x, float y ) { return ex2_approx( y * log2f( x ) ); }
    __device__ static float expn( float x ) { return ex2_approx( x * 1.44269504088896341f ); }
    __device__ static float madd( float a, float b, float c ) { return __fmaf_rn( a, b, c ); }
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
};

template<> struct Sto< MODE_F32 >
{
    static constexpr bool varPlane = false;
    __device__ static float3 ld3( const void* p, size_t i ) { float4 v = static_cast< const float4* >( p )[ i ]; return f3( v.x, v.y, v.z ); }
    __device__ static void   st3( void* p, size_t i, float3 v ) { static_cast< float4* >( p )[ i ] = make_float4( v.x, v.y, v.z, 0.0f ); }
    __device__ static float4 ldcv( const void* p, const float*, size_t i ) { return static_cast< const float4* >( p )[ i ]; }
    __device__ static void   stcv( void* p, float*, size_t i, float3 c, float var ) { static_cast< float4* >( p )[ i ] = make_float4( c.x, c.y, c.z, var ); }
    __device__ static float2 ld2( const void* p, size_t i ) { return static_cast< const float2* >( p )[ i ]; }
    __device__ static void   st2( void* p, size_t i, float2 v ) { static_cast< float2* >( p )[ i ] = v; }
    __device__ static float4 ld4( const void* p, size_t i ) { return static_cast< const float4* >( p )[ i ]; }
    __device__ static void   st4( void* p, size_t i, float4 v ) { static_cast< float4* >( p )[ i ] = v; }
    __device__ static float  ld1( const void* p, size_t i ) { return static_cast< const float* >( p )[ i ]; }
    __device__ static void   st1( void* p, size_t i, float v ) { static_cast< float* >( p )[ i ] = v; }
    __device__ static void   stpre( void* p, size_t i, float3 v ) { static_cast< float4* >( p )[ i ] = make_float4( v.x, v.y, v.z, 0.0f ); }
};

// 16-bit colour / history with FP32 moments, FP32 variance planes, FP32 prefiltered variance
template< bool BF > struct Sto16
{
    static constexpr bool varPlane = true;
    __device__ static float    cv( uint16_t h ) { return BF ? b2f( h ) : h2f( h ); }
    __device__ static uint16_t pk( float f ) { return BF ? f32_to_bf16( f ) : f32_to_f16( f ); }
    __device__ static float3 ld3( const void* p, size_t i ) { ushort4 h = static_cast< const ushort4* >( p )[ i ]; return f3( cv( h.x ), cv( h.y ), cv( h.z ) ); }
    __device__ static void   st3( void* p, size_t i, float3 v ) { static_cast< ushort4* >( p )[ i ] = make_ushort4( pk( v.x ), pk( v.y ), pk( v.z ), 0 ); }
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
    const float isx = 1.0f / sx, isy = 1.0f / sy;
    return make_float2( ( ( (float)px + 0.5f ) * isx + m.x ) * sx, ( ( (float)py + 0.5f ) * isy + m.y ) * sy );
}
// ShaderCommonGLSLFunc.h:368-390
__device__ __forceinline__ bool test_depth( float z, float zPrev, float zMotion ) { return fabsf( z - zPrev + zMotion ) / fabsf( z ) < 0.1f; }
__device__ __forceinline__ bool test_normal( float3 n, float3 np ) { return dot3( n, np ) > 0.95f; }
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

template< int M > __device__ __forceinline__ void gradient_sample_px( const FrameArgs& a, const int gx, const int gy, const float* u8 )
{
    const Uniform& u  = a.u;
    const int      gi = gy * u.GW + gx;
    if( u.gradMultD < 0.001f && u.gradMultI < 0.001f && u.gradMultS < 0.001f )
    {
        a.disPing[ gi ]     = 0u;
        a.gradPrevPix[ gi ] = STRATA * STRATA + 1;
        return;
    }
    const uint32_t prevStrataPos = a.gradPrevPix[ gi ];
    int2     prevShadingPix = make_int2( 0, 0 ), curShadingPix = make_int2( 0, 0 );
    uint32_t curStrataPos   = 0;
    float2   prevLum        = make_float2( 0, 0 );
    for( int yy = 0; yy < STRATA; yy++ )
    {
        for( int xx = 0; xx < STRATA; xx++ )
        {
            if( (uint32_t)( yy * STRATA + xx ) == prevStrataPos ) continue;
            const int cx = gx * STRATA + xx, cy = gy * STRATA + yy;
            float2    m  = make_float2( 0, 0 );
            if( inside( u, cx, cy ) )
            {
                const ushort4 mo = a.motion[ cy * u.W + cx ];
                m                = make_float2( h2f( mo.x ), h2f( mo.y ) );
            }
            const float2 pp = prev_screen_pos( u, m, cx, cy );
            const int2   ip = make_int2( (int)floorf( pp.x ), (int)floorf( pp.y ) );
            float2       il = make_float2( 0, 0 );
            if( inside( u, ip.x, ip.y ) )
            {
                const uint32_t g = a.gradInputsPrev[ ip.y * u.W + ip.x ];
                il               = make_float2( h2f( (uint16_t)( g & 0xFFFFu ) ), h2f( (uint16_t)( g >> 16 ) ) );
            }
            if( fmaxf( il.x, il.y ) > fmaxf( prevLum.x, prevLum.y ) )
            {
                prevShadingPix = ip;
                curShadingPix  = make_int2( cx, cy );
                curStrataPos   = (uint32_t)( yy * STRATA + xx );
                prevLum        = il;
            }
        }
    }
    const bool skyCur = inside( u, curShadingPix.x, curShadingPix.y ) && a.isSky[ curShadingPix.y * u.W + curShadingPix.x ] != 0;
    if( !in_area( prevShadingPix.x, prevShadingPix.y, cb_area( u, curShadingPix.x ) ) || skyCur ||
        ( prevLum.x <= 0.0f && prevLum.y <= 0.0f ) )
    {
        a.disPing[ gi ]     = 0u;
        a.gradPrevPix[ gi ] = STRATA * STRATA + 1;
        return;
    }
    // in the render area, so inside the image
    const int    pi  = prevShadingPix.y * u.W + prevShadingPix.x;
    // the re-shaded luminance is a boundary input (RtGradients.rgen:107-136)
    const float2 fpl = a.reshaded[ pi ];
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
    a.disPing[ gi ]     = pack_rgba8( g0, g1, g2, 0.0f );
    a.gradPrevPix[ gi ] = (uint8_t)curStrataPos;
}

// CmASVGFGradientAtrous.comp:42-105 — one iteration, one stratum, from `src` into `dst`
// (and `hist` on iteration 0), all GW x GH rgba8 images
__device__ __forceinline__ void gradient_atrous_core( const Uniform& u, const uint32_t* src, uint32_t* dst, uint32_t* hist, const int gx,
                                                      const int gy, const int iter, const float* u8 )
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
            const float4 g  = ld_rgba8t( u, src, qx, qy, u8 );
            const float  w  = kern[ yy < 0 ? -yy : yy ][ xx < 0 ? -xx : xx ] * ( in_area( qx, qy, ga ) ? 1.0f : 0.0f );
            out = add( out, mul( f3( g.x, g.y, g.z ), w ) );
            ws  = ws + w;
        }
    }
    out = divs( out, ws );
    const uint32_t packed = pack_rgba8( out.x, out.y, out.z, 0.0f );
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

__device__ __forceinline__ void fill_u8( float* u8, int t )
{
    u8[ t ] = (float)t / 255.0f;
}

template< int M > __global__ void __launch_bounds__( 256 ) k_gradient_samples( const FrameArgs a )
{
    __shared__ float u8[ 256 ];
    fill_u8( u8, threadIdx.y * blockDim.x + threadIdx.x );
    __syncthreads();
    const int gx = blockIdx.x * blockDim.x + threadIdx.x;
    const int gy = blockIdx.y * blockDim.y + threadIdx.y;
    if( gx >= a.u.GW || gy >= a.u.GH || gx * STRATA >= a.u.W || gy * STRATA >= a.u.H ) return;
    gradient_sample_px< M >( a, gx, gy, u8 );
}

template< int M > __global__ void __launch_bounds__( 256 ) k_gradient_atrous( const FrameArgs a, const int iter )
{
    __shared__ float u8[ 256 ];
    fill_u8( u8, threadIdx.y * blockDim.x + threadIdx.x );
    __syncthreads();
    const int gx = blockIdx.x * blockDim.x + threadIdx.x;
    const int gy = blockIdx.y * blockDim.y + threadIdx.y;
    if( gx >= a.u.GW || gy >= a.u.GH || gx * STRATA >= a.u.W || gy * STRATA >= a.u.H ) return;
    gradient_atrous_px( a, gx, gy, iter, u8 );
}

// The whole gradient chain in one cooperative launch: samples, then the 4 a-trous
// iterations, separated by grid-wide barriers (every block is co-resident; the
// launch fails instead of starting if the grid does not fit).
template< int M > __global__ void __launch_bounds__( 256 ) k_gradient_fused( const FrameArgs a )
{
    __shared__ float u8[ 256 ];
    fill_u8( u8, threadIdx.x );
    __syncthreads();
    cg::grid_group grid   = cg::this_grid();
    const Uniform& u      = a.u;
    const int      n      = u.GW * u.GH;
    const int      stride = gridDim.x * blockDim.x;
    for( int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride )
    {
        const int gx = k % u.GW, gy = k / u.GW;
        if( gx * STRATA < u.W && gy * STRATA < u.H ) gradient_sample_px< M >( a, gx, gy, u8 );
    }
    for( int iter = 0; iter < 4; iter++ )
    {
        grid.sync();
        for( int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride )
        {
            const int gx = k % u.GW, gy = k / u.GW;
            if( gx * STRATA < u.W && gy * STRATA < u.H ) gradient_atrous_px( a, gx, gy, iter, u8 );
        }
    }
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

template< int M, bool FAST > __global__ void __launch_bounds__( 256 ) k_temporal( const FrameArgs a )
{
    using S          = Sto< M >;
    const Uniform& u = a.u;
    const int      px = blockIdx.x * blockDim.x + threadIdx.x;
    const int      py = blockIdx.y * blockDim.y + threadIdx.y;
    if( px >= u.W || py >= u.H ) return;
    const size_t i = idx( u, px, py );

    const float3  unfilteredDiff  = e5( a.unfD[ i ] );
    const float3  unfilteredIndir = e5( a.unfI[ i ] );
    const float3  unfilteredSpec  = e5( a.unfS[ i ] );
    const ushort4 rv              = a.viewDir[ i ];
    const float4  rayInfo         = make_float4( h2f( rv.x ), h2f( rv.y ), h2f( rv.z ), h2f( rv.w ) );
    const Area    chArea          = cb_area( u, px );
    const ushort4 mo              = a.motion[ i ];
    const float   motionZ         = h2f( mo.z );
    const float   z               = h2f( a.depth[ i ] );
    const float3  normal          = decode_normal( a, a.normal[ i ] );
    const float   roughness       = unorm8_to_f32( a.mr[ i ] >> 8 );

    const float l = luminance( unfilteredDiff );
    const float2 moments = make_float2( l, l * l );

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
            const int   qx = pixPrev.x + xx, qy = pixPrev.y + yy;
            const bool  in = inside( u, qx, qy );
            const size_t q = in ? idx( u, qx, qy ) : 0;
            const float  dP = in ? h2f( a.depthPrev[ q ] ) : 0.0f;
            const float3 nP = decode_normal( a, in ? a.normalPrev[ q ] : 0u );
            const bool ok = in_area( qx, qy, chArea ) && test_depth( z, dP, motionZ ) && test_normal( normal, nP );
            if( ok )
            {
                // in_area implies inside the image
                const float  w  = bw[ yy ][ xx ];
                const float4 dc = S::ldcv( a.diffHistory, a.varHistory, q );
                diffPrev        = add( diffPrev, mul( f3( dc.x, dc.y, dc.z ), w ) );
                const float2 m  = S::ld2( a.momentsPrev, q );
                momentsPrev     = make_float2( momentsPrev.x + w * m.x, momentsPrev.y + w * m.y );
                const float4 hl = S::ld4( a.histLenPrev, q );
                histLenDIS = make_float4( histLenDIS.x + w * hl.x, histLenDIS.y + w * hl.y, histLenDIS.z + w * hl.z, histLenDIS.w + w * hl.w );
                const float3 sp = S::ld3( a.specAccumPrev, q );
                specPrevOnSurf  = add( specPrevOnSurf, f3( w * sp.x, w * sp.y, w * sp.z ) );
                const float3 ip = S::ld3( a.indirAccumPrev, q );
                indirPrev       = add( indirPrev, f3( w * ip.x, w * ip.y, w * ip.z ) );
                weightSum       = weightSum + w;
            }
        }
    }

    float aD = 0.0f, aI = 0.0f, aS = 0.0f;
    if( !( u.flags & RGDN_FLAG_SKIP_GRADIENTS ) )
    {
        const float4 g = ld_rgba8z( u, a.disPing, px / STRATA, py / STRATA );
        aD = g.x; aI = g.y; aS = g.z;
    }

    float3 specColorAccum;
    float  specHistoryLengthAccum, specHitDistanceAccum;

    if( weightSum > 0.0001f )
    {
        specPrevOnSurf                = divs( specPrevOnSurf, weightSum );
        const float specHistoryLength   = histLenDIS.z / weightSum;
        const float specHitDistancePrev = histLenDIS.w / weightSum;

        const float4 sp4     = a.surfPos[ i ];
        const float3 surfPos = f3( sp4.x, sp4.y, sp4.z );
        float3       surfPosPrev = f3( 0, 0, 0 );
        if( inside( u, pixPrev.x, pixPrev.y ) )
        {
            const float4 spp = a.surfPosPrev[ idx( u, pixPrev.x, pixPrev.y ) ];
            surfPosPrev      = f3( spp.x, spp.y, spp.z );
        }
        const float nv = fmaxf( 0.0f, dot3( normal, f3( -rayInfo.x, -rayInfo.y, -rayInfo.z ) ) );

        const float A       = gclamp( 1.0f + specHistoryLength * Wm< FAST >::powv( 1.0f - aS, 5.0f ), spec_min_accum( u ), 256.0f );
        const float par     = parallax( u, surfPos, surfPosPrev );
        const float AOnSurf = spec_accum_speed< FAST >( u, A, roughness, nv, par );
        const float domin   = spec_dominant< FAST >( nv, roughness );

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
                const int    qx = pixPrevS.x + xx, qy = pixPrevS.y + yy;
                const bool   in = inside( u, qx, qy );
                const size_t q  = in ? idx( u, qx, qy ) : 0;
                const float  dP = in ? h2f( a.depthPrev[ q ] ) : 0.0f;
                const float3 nP = decode_normal( a, in ? a.normalPrev[ q ] : 0u );
                const bool ok = in_area( qx, qy, chArea ) && test_depth( z, dP, motionZ ) && test_normal( normal, nP );
                // the shader also accumulates SpecAccumColor_Prev here but never uses the sum
                if( ok ) weightSumVirtual = weightSumVirtual + bws[ yy ][ xx ];
            }
        }
        if( weightSumVirtual > 0.0001f )
        {
            float       Avirt      = spec_accum_speed< FAST >( u, A, roughness, nv, 0.0f );
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
    else
    {
        specColorAccum         = unfilteredSpec;
        specHistoryLengthAccum = 1.0f;
        specHitDistanceAccum   = rayInfo.w;
    }

    float3 diffColorAccum, indirAccum;
    float2 diffMomentsAccum;
    float  diffHL, indirHL;
    if( weightSum > 0.0001f )
    {
        const float inv = 1.0f / weightSum;
        diffPrev        = mul( diffPrev, inv );
        momentsPrev     = make_float2( momentsPrev.x * inv, momentsPrev.y * inv );
        indirPrev       = mul( indirPrev, inv );
        float dHL       = histLenDIS.x * inv;
        float iHL       = histLenDIS.y * inv;
        {
            dHL = dHL * powf( 1.0f - aD, 10.0f );
            dHL = gclamp( dHL + 1.0f, 1.0f, 256.0f );
            float alphaColor   = fmaxf( 0.01f, 1.0f / dHL );
            float alphaMoments = fmaxf( 0.01f, 1.0f / dHL );
            alphaColor         = gmix( alphaColor, 1.0f, aD );
            alphaMoments       = gmix( alphaMoments, 1.0f, aD );
            diffColorAccum     = vmix( diffPrev, unfilteredDiff, alphaColor );
            diffMomentsAccum   = make_float2( gmix( momentsPrev.x, moments.x, alphaMoments ), gmix( momentsPrev.y, moments.y, alphaMoments ) );
            diffHL             = dHL;
        }
        {
            iHL = iHL * powf( 1.0f - aI, 10.0f );
            iHL = gclamp( iHL + 1.0f, 1.0f, 256.0f );
            float alphaColor = fmaxf( 0.01f, 1.0f / iHL );
            alphaColor       = gmix( alphaColor, 1.0f, aI );
            indirAccum       = vmix( indirPrev, unfilteredIndir, alphaColor );
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
template< int M, bool FAST, class ColorAt >
__device__ __forceinline__ void variance_px( const FrameArgs& a, const int px, const int py, const int i, ColorAt colorAt, float3& outC,
                                             float& outV )
{
    using S          = Sto< M >;
    using X          = Wm< FAST >;
    const float cz   = h2f( a.depth[ i ] );
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
    if( histLen > THR )
    {
        float tv = fmaxf( 0.0f, tm.y - tm.x * tm.x );
        tv       = tv / fmaxf( 1.0f, histLen - THR );
        outC     = pc;
        outV     = tv;
        return;
    }
    const float  l   = luminance( pc );
    float2       sm  = make_float2( l + tm.x, l * l + tm.y );
    float        ws  = 1.0f;
    const float3 cnd = decode_normal( a, a.normal[ i ] );
#pragma unroll
    for( int yy = -1; yy <= 1; yy++ )
    {
#pragma unroll
        for( int xx = -1; xx <= 1; xx++ )
        {
            if( xx == 0 && yy == 0 ) continue;
            const int    qx  = px + xx, qy = py + yy;
            const float3 cq  = colorAt( xx, yy );
            const float  lq  = luminance( cq );
            const bool   in  = inside( a.u, qx, qy );
            const int    q   = in ? qy * a.u.W + qx : 0;
            const float  zq  = in ? h2f( a.depth[ q ] ) : 0.0f;
            const float  mz  = fmaxf( cz, zq );
            const float  rcp = mz <= 0.0f ? 0.0f : 1.0f / mz;
            const float  wz  = X::expn( -fabsf( cz - zq ) * rcp );
            const float  wn  = X::pow128( fmaxf( 0.0f, dot3( cnd, decode_normal( a, in ? a.normal[ q ] : 0u ) ) ) );
            const float  w   = wz * wn;
            if( !isnan( w ) )
            {
                sm = make_float2( sm.x + lq * w, sm.y + lq * lq * w );
                pc = add( pc, mul( cq, w ) );
                ws = ws + w;
            }
        }
    }
    const float inv = ws <= 0.0f ? 0.0f : 1.0f / ws;
    sm              = make_float2( sm.x * inv, sm.y * inv );
    outC            = mul( pc, inv );
    outV            = fmaxf( 0.0f, sm.y - sm.x * sm.x ) * ( 1.0f + 2.0f * ( 1.0f - histLen / THR ) );
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
    variance_px< M, false >( a, px, py, i, [ & ]( int dx, int dy ) { return ld3z< M >( a, a.diffAccumColor, px + dx, py + dy ); }, c, v );
    S::stcv( a.diffPing, a.varPing, (size_t)i, c, v );
}

// ==========================================================================================
// Anti-firefly + variance in one kernel (CmAntiFirefly.comp + CmSVGFEstimateVariance.comp).
// A 32x8 tile: the three signals are staged with a 3-texel halo, the 5x5 ring minimum and
// maximum come from row extrema (min over the 4 rows above/below of the 5-wide row extremum,
// and the 4 same-row neighbours), the anti-firefly diffuse result on a 1-texel halo is
// quantised through the storage format exactly as if it had been stored to DiffAccumColor,
// and the variance reads it from shared memory. Results equal the two separate kernels.
// ==========================================================================================
constexpr int AFV_TX = 32, AFV_TY = 8;
constexpr int AFV_IW = AFV_TX + 6, AFV_IH = AFV_TY + 6;   // staged inputs: tile +-3
constexpr int AFV_AW = AFV_TX + 2, AFV_AH = AFV_TY + 2;   // anti-firefly results: tile +-1

template< int M > __device__ __forceinline__ float3 quantize3( float3 v )
{
    if( M == MODE_REF ) return e5( encode_e5( v.x, v.y, v.z ) );
    return v;  // fp32 / fp16 / bf16 channels of a clamp are already representable
}

template< int M, bool FAST > __global__ void __launch_bounds__( 256 ) k_af_variance( const FrameArgs a )
{
    using S = Sto< M >;
    __shared__ float v[ 3 ][ AFV_IH ][ AFV_IW ];
    __shared__ float rmn[ 3 ][ AFV_IH ][ AFV_AW ];
    __shared__ float rmx[ 3 ][ AFV_IH ][ AFV_AW ];
    __shared__ float afd[ 3 ][ AFV_AH ][ AFV_AW ];
    const Uniform& u   = a.u;
    const int      t   = threadIdx.y * AFV_TX + threadIdx.x;
    const int      x0  = blockIdx.x * AFV_TX, y0 = blockIdx.y * AFV_TY;
    const bool     af  = u.antiFirefly != 0;
    const float    MAXF = 1000000.0f;

    for( int sig = 0; sig < 3; sig++ )
    {
        const void* src = sig == 0 ? a.diffTemp : sig == 1 ? a.specAccum : a.indirAccum;
        for( int k = t; k < AFV_IW * AFV_IH; k += 256 )
        {
            const int    lx = k % AFV_IW, ly = k / AFV_IW;
            const float3 c  = ld3z< M >( a, src, x0 - 3 + lx, y0 - 3 + ly );
            v[ 0 ][ ly ][ lx ] = c.x;
            v[ 1 ][ ly ][ lx ] = c.y;
            v[ 2 ][ ly ][ lx ] = c.z;
        }
        __syncthreads();
        if( af )
        {
            for( int k = t; k < AFV_AW * AFV_IH; k += 256 )
            {
                const int rx = k % AFV_AW, ry = k / AFV_AW;
#pragma unroll
                for( int c = 0; c < 3; c++ )
                {
                    const float* r = &v[ c ][ ry ][ rx ];
                    rmn[ c ][ ry ][ rx ] = fminf( fminf( fminf( r[ 0 ], r[ 1 ] ), fminf( r[ 2 ], r[ 3 ] ) ), r[ 4 ] );
                    rmx[ c ][ ry ][ rx ] = fmaxf( fmaxf( fmaxf( r[ 0 ], r[ 1 ] ), fmaxf( r[ 2 ], r[ 3 ] ) ), r[ 4 ] );
                }
            }
            __syncthreads();
        }
        for( int k = t; k < AFV_AW * AFV_AH; k += 256 )
        {
            const int ax = k % AFV_AW, ay = k / AFV_AW;
            const int gx = x0 - 1 + ax, gy = y0 - 1 + ay;
            float3    res;
            float*    ctr[ 3 ];
            float     o[ 3 ];
#pragma unroll
            for( int c = 0; c < 3; c++ )
            {
                const float center = v[ c ][ ay + 2 ][ ax + 2 ];
                if( af )
                {
                    const float* row = &v[ c ][ ay + 2 ][ ax ];
                    float mn = fminf( fminf( fminf( rmn[ c ][ ay ][ ax ], rmn[ c ][ ay + 1 ][ ax ] ), fminf( rmn[ c ][ ay + 3 ][ ax ], rmn[ c ][ ay + 4 ][ ax ] ) ),
                                      fminf( fminf( row[ 0 ], row[ 1 ] ), fminf( row[ 3 ], row[ 4 ] ) ) );
                    float mx = fmaxf( fmaxf( fmaxf( rmx[ c ][ ay ][ ax ], rmx[ c ][ ay + 1 ][ ax ] ), fmaxf( rmx[ c ][ ay + 3 ][ ax ], rmx[ c ][ ay + 4 ][ ax ] ) ),
                                      fmaxf( fmaxf( row[ 0 ], row[ 1 ] ), fmaxf( row[ 3 ], row[ 4 ] ) ) );
                    mn   = fminf( MAXF, mn );
                    mx   = fmaxf( -MAXF, mx );
                    o[ c ] = fminf( fmaxf( center, mn ), mx );
                }
                else o[ c ] = center;
                (void)ctr;
            }
            res = f3( o[ 0 ], o[ 1 ], o[ 2 ] );
            const bool in = inside( u, gx, gy );
            if( sig == 0 )
            {
                const float3 q = in ? quantize3< M >( res ) : f3( 0, 0, 0 );
                afd[ 0 ][ ay ][ ax ] = q.x;
                afd[ 1 ][ ay ][ ax ] = q.y;
                afd[ 2 ][ ay ][ ax ] = q.z;
            }
            else if( in && ax >= 1 && ax <= AFV_TX && ay >= 1 && ay <= AFV_TY )
                S::st3( sig == 1 ? a.specPing : a.indirPing, (size_t)( gy * u.W + gx ), res );
        }
        __syncthreads();
    }

    const int px = x0 + threadIdx.x, py = y0 + threadIdx.y;
    if( px >= u.W || py >= u.H ) return;
    const int i = py * u.W + px;
    float3    c;
    float     var;
    variance_px< M, FAST >( a, px, py, i,
                            [ & ]( int dx, int dy ) {
                                const int ax = threadIdx.x + 1 + dx, ay = threadIdx.y + 1 + dy;
                                return f3( afd[ 0 ][ ay ][ ax ], afd[ 1 ][ ay ][ ax ], afd[ 2 ][ ay ][ ax ] );
                            },
                            c, var );
    S::stcv( a.diffPing, a.varPing, (size_t)i, c, var );
}

// ==========================================================================================
// CmSVGFAtrous_Iter0.comp:158-335 and CmSVGFAtrous.comp:71-349 — one a-trous iteration;
// the last one composes PreFinal and HistogramInput instead of storing ping/pong.
// ==========================================================================================
__device__ __forceinline__ float spec_power( float alpha ) { return fmaxf( 0.01f, 2.0f / ( alpha * alpha + 1e-4f ) - 2.0f ); }

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
template< int M > __device__ __forceinline__ uint16_t compose( const FrameArgs& a, int px, int py, size_t i, float3 filteredDiff, float3 filteredSpec,
                                                            float3 filteredIndir )
{
    const Uniform& u  = a.u;
    const int2     rp = regular_from_cb( u, px, py );
    const size_t   ri = idx( u, rp.x, rp.y );
    const rgdn::f3 al = decode_b10g11r11( a.albedo[ ri ] );
    float3         albedo = f3( al.x, al.y, al.z );
    const ushort4  tp = a.throughput[ i ];
    const float3   throughput = f3( h2f( tp.x ), h2f( tp.y ), h2f( tp.z ) );
    if( u.debugFlags & RGDN_DEBUG_SHOW_FLAG_ALBEDO_WHITE ) albedo = f3( 1.0f, 1.0f, 1.0f );
    float3 ill;
    if( a.isSky[ i ] == 0 )
    {
        const uint16_t mrb       = a.mr[ i ];
        const float    metallic  = unorm8_to_f32( mrb & 0xFFu );
        const float    roughness = unorm8_to_f32( mrb >> 8 );
        const float3   diffuse = filteredDiff, indirect = filteredIndir;
        const float3   specular = vmix( filteredSpec, indirect, gsmoothstep( 0.5f, 0.5f + 0.25f, roughness ) );
        const float3   ro_s     = vmix( f3( 0.04f, 0.04f, 0.04f ), albedo, metallic );
        const float3   ro_d     = mul( albedo, 1.0f - metallic );
        ill = add( mul( add( diffuse, indirect ), ro_d ), mul( specular, ro_s ) );
        if( u.debugFlags & RGDN_DEBUG_SHOW_FLAG_ONLY_DIRECT_DIFFUSE ) ill = mul( diffuse, albedo );
        else if( u.debugFlags & RGDN_DEBUG_SHOW_FLAG_ONLY_SPECULAR ) ill = mul( specular, vmix( f3( 0.04f, 0.04f, 0.04f ), albedo, metallic ) );
        else if( u.debugFlags & RGDN_DEBUG_SHOW_FLAG_ONLY_INDIRECT_DIFFUSE ) ill = indirect;
        ill = mul( ill, throughput );
        ill = mul( ill, material_ambient( albedo ) );
    }
    else ill = mul( albedo, throughput );

    const uint16_t hin = f32_to_f16( fmaxf( 0.0f, luminance( ill ) ) );
    a.histInput[ ri ] = hin;
    if( (float)rp.x < u.lightmapCoverage * u.rw ) ill = mul( albedo, throughput );
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
template< int M, bool FAST >
__device__ __forceinline__ void atrous_px( const FrameArgs& a, const AtrousIO& io, const int iter, const int px, const int py,
                                           const int i, const float* u8, float3& outDiff, float& outVar, float3& outSpec,
                                           float3& outInd )
{
    using S          = Sto< M >;
    using X          = Wm< FAST >;
    const Uniform& u = a.u;
    const int      step   = 1 << iter;
    const Area     chArea = cb_area( u, px );
    const float4   cv     = S::ldcv( io.diffSrc, io.varSrc, (size_t)i );
    outDiff = f3( cv.x, cv.y, cv.z );
    outVar  = cv.w;
    outSpec = S::ld3( io.specSrc, (size_t)i );
    outInd  = S::ld3( io.indirSrc, (size_t)i );
    const float z         = h2f( a.depth[ i ] );
    const float gradDepth = h2f( a.depthGrad[ i ] );

    if( z < 0.0f || z > MAX_RAY_LENGTH )
    {
        if( iter == 0 )
        {
            outDiff = f3( 0, 0, 0 ); outVar = 0.0f; outSpec = f3( 0, 0, 0 ); outInd = f3( 0, 0, 0 );
        }
        return;
    }
    const float3 normal = decode_normal( a, a.normal[ i ] );
    const float  l      = luminance( outDiff );
    float        prefVar;
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
        r = sqrtf( fmaxf( r, 0.0f ) );
        S::st1( a.filtVar, (size_t)i, r );
        prefVar = r;
    }
    else prefVar = S::ld1( a.filtVar, (size_t)i );

    const float wLumMul   = 1.0f / ( 4.0f * prefVar + 0.00001f );
    const float roughness = u8[ a.mr[ i ] >> 8 ];
    const float wRoughMul = gclamp( roughness * 30.0f - (float)iter, 0.0f, 1.0f );
    const float hS        = S::ld4( a.histLen, (size_t)i ).z;
    const float nws       = gclamp( hS / 8.0f, 0.0f, 1.0f );
    float       nwSpec    = spec_power( roughness * roughness );
    nwSpec                = gclamp( nwSpec, 8.0f, 1024.0f );
    nwSpec                = nwSpec * nws;
    // FAST: one reciprocal per tap distance class (|x|+|y| = 1 or 2)
    const float rz1 = FAST ? 1.0f / fmaxf( gradDepth * 1.0f, 0.01f ) : 0.0f;
    const float rz2 = FAST ? 1.0f / fmaxf( gradDepth * 2.0f, 0.01f ) : 0.0f;

    const float kern[ 2 ][ 2 ] = { { 1.0f, 0.5f }, { 0.5f, 0.25f } };
    float ws = 1.0f, wsS = 1.0f, wsI = 1.0f;
#pragma unroll
    for( int yy = -1; yy <= 1; yy++ )
    {
#pragma unroll
        for( int xx = -1; xx <= 1; xx++ )
        {
            if( xx == 0 && yy == 0 ) continue;
            const int    qx  = px + xx * step, qy = py + yy * step;
            const bool   in  = inside( u, qx, qy );
            const int    q   = in ? qy * u.W + qx : 0;
            const float  rq  = in ? u8[ a.mr[ q ] >> 8 ] : 0.0f;
            const float3 nq  = decode_normal( a, in ? a.normal[ q ] : 0u );
            const float  zq  = in ? h2f( a.depth[ q ] ) : 0.0f;
            const float3 sq  = in ? S::ld3( io.specSrc, (size_t)q ) : f3( 0, 0, 0 );
            const float4 cvq = in ? S::ldcv( io.diffSrc, io.varSrc, (size_t)q ) : make_float4( 0, 0, 0, 0 );
            const float3 dq  = f3( cvq.x, cvq.y, cvq.z );
            const float  lq  = luminance( dq );
            const float  nn  = fmaxf( 0.0f, dot3( normal, nq ) );
            const float3 iq  = in ? S::ld3( io.indirSrc, (size_t)q ) : f3( 0, 0, 0 );
            const int    man = ( xx < 0 ? -xx : xx ) + ( yy < 0 ? -yy : yy );

            const float w_z = FAST ? fabsf( z - zq ) * ( man == 1 ? rz1 : rz2 )
                                   : fabsf( z - zq ) / fmaxf( gradDepth * (float)man, 0.01f );
            const float w_n = X::pow128( nn );
            const float w_l = fabsf( l - lq ) * wLumMul;
            float       w_r = fmaxf( 0.0f, 1.0f - 10.0f * fabsf( roughness - rq ) ) * wRoughMul;
            if( nwSpec > 0.0f ) w_r = w_r * X::powv( nn, nwSpec );
            const float waveletW = kern[ yy < 0 ? -yy : yy ][ xx < 0 ? -xx : xx ];
            const float insideA  = in_area( qx, qy, chArea ) ? 1.0f : 0.0f;
            const float wBase    = X::expn( -w_z * w_z ) * w_n * waveletW * insideA;
            const float wDiff    = wBase * X::expn( -w_l );
            const float wSpec    = wBase * w_r;
            const float wInd     = wBase;

            outDiff = f3( X::madd( dq.x, wDiff, outDiff.x ), X::madd( dq.y, wDiff, outDiff.y ), X::madd( dq.z, wDiff, outDiff.z ) );
            outSpec = f3( X::madd( sq.x, wSpec, outSpec.x ), X::madd( sq.y, wSpec, outSpec.y ), X::madd( sq.z, wSpec, outSpec.z ) );
            outInd  = f3( X::madd( iq.x, wInd, outInd.x ), X::madd( iq.y, wInd, outInd.y ), X::madd( iq.z, wInd, outInd.z ) );
            outVar  = X::madd( cvq.w * wDiff, wDiff, outVar );
            ws      = ws + wDiff;
            wsS     = wsS + wSpec;
            wsI     = wsI + wInd;
        }
    }
    const float inv = 1.0f / ws, invS = 1.0f / wsS, invI = 1.0f / wsI;
    outDiff = mul( outDiff, inv );
    outVar  = outVar * inv * inv;
    outSpec = mul( outSpec, invS );
    outInd  = mul( outInd, invI );
}

// One a-trous iteration over the frame. HIST: the last iteration also accumulates the
// luminance histogram of the HistogramInput values it writes (CmLuminanceHistogram.comp,
// fused: no second read of the image).
template< int M, bool FAST, bool HIST > __global__ void __launch_bounds__( 256 ) k_atrous( const FrameArgs a, const int iter )
{
    using S = Sto< M >;
    __shared__ float    u8[ 256 ];
    __shared__ uint32_t hist[ HIST ? 256 : 1 ];
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
    u8[ t ]     = (float)t / 255.0f;
    if( HIST ) hist[ t ] = 0u;
    __syncthreads();

    const Uniform& u  = a.u;
    const int      px = blockIdx.x * blockDim.x + threadIdx.x;
    const int      py = blockIdx.y * blockDim.y + threadIdx.y;
    if( px < u.W && py < u.H )
    {
        const int      i    = py * u.W + px;
        const AtrousIO io   = atrous_io< M >( a, iter );
        const bool     last = iter + 1 == (int)u.niter;
        float3         outDiff, outSpec, outInd;
        float          outVar;
        atrous_px< M, FAST >( a, io, iter, px, py, i, u8, outDiff, outVar, outSpec, outInd );
        if( !last )
        {
            S::stcv( io.diffDst, io.varDst, (size_t)i, outDiff, outVar );
            S::st3( io.specDst, (size_t)i, outSpec );
            S::st3( io.indirDst, (size_t)i, outInd );
        }
        else
        {
            const uint16_t hin = compose< M >( a, px, py, (size_t)i, outDiff, outSpec, outInd );
            if( HIST ) atomicAdd( &hist[ __ldg( &a.binLut[ hin ] ) ], 1u );
        }
    }
    if( HIST )
    {
        __syncthreads();
        if( hist[ t ] ) atomicAdd( &a.tm->histogram[ t ], hist[ t ] );
    }
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
template< int M > __global__ void __launch_bounds__( 256 ) k_luminance_avg( const FrameArgs a )
{
    __shared__ uint32_t sh[ 256 ];
    __shared__ uint32_t count0;
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

}  // namespace dev

// ------------------------------------------------------------------------------------------
// launcher for one mode
// ------------------------------------------------------------------------------------------
template< int M > cudaError_t launch_stage_t( const FrameArgs& a, int stage, int iter, cudaStream_t s )
{
    const dim3 blk( 32, 8 );
    const dim3 grid( ( a.u.W + 31 ) / 32, ( a.u.H + 7 ) / 8 );
    const dim3 gridG( ( a.u.GW + 31 ) / 32, ( a.u.GH + 7 ) / 8 );
    switch( stage )
    {
        case RGDN_STAGE_GRADIENT_SAMPLES: dev::k_gradient_samples< M ><<< gridG, blk, 0, s >>>( a ); break;
        case RGDN_STAGE_GRADIENT_ATROUS: dev::k_gradient_atrous< M ><<< gridG, blk, 0, s >>>( a, iter ); break;
        case RGDN_STAGE_TEMPORAL_ACCUMULATION: dev::k_temporal< M, false ><<< grid, blk, 0, s >>>( a ); break;
        case KF_TEMPORAL_FAST: dev::k_temporal< M, true ><<< grid, blk, 0, s >>>( a ); break;
        case KF_AF_VARIANCE: dev::k_af_variance< M, false ><<< grid, blk, 0, s >>>( a ); break;
        case KF_AF_VARIANCE_FAST: dev::k_af_variance< M, true ><<< grid, blk, 0, s >>>( a ); break;
        case KF_GRADIENT_FUSED:
        {
            // one co-resident wave: blocks per SM from the occupancy calculator
            static int blocksPerGrid = 0;
            if( blocksPerGrid == 0 )
            {
                int dev = 0, sms = 0, perSm = 0;
                cudaGetDevice( &dev );
                cudaDeviceGetAttribute( &sms, cudaDevAttrMultiProcessorCount, dev );
                cudaOccupancyMaxActiveBlocksPerMultiprocessor( &perSm, dev::k_gradient_fused< M >, 256, 0 );
                blocksPerGrid = sms * ( perSm > 0 ? perSm : 1 );
            }
            const int need   = ( a.u.GW * a.u.GH + 255 ) / 256;
            const int blocks = need < blocksPerGrid ? ( need > 0 ? need : 1 ) : blocksPerGrid;
            void*     args[] = { (void*)&a };
            return cudaLaunchCooperativeKernel( (const void*)dev::k_gradient_fused< M >, dim3( blocks ), dim3( 256 ), args, 0, s );
        }
        case RGDN_STAGE_ANTI_FIREFLY: dev::k_antifirefly< M ><<< grid, blk, 0, s >>>( a ); break;
        case RGDN_STAGE_VARIANCE_ESTIMATION: dev::k_variance< M ><<< grid, blk, 0, s >>>( a ); break;
        case RGDN_STAGE_ATROUS: dev::k_atrous< M, false, false ><<< grid, blk, 0, s >>>( a, iter ); break;
        case RGDN_STAGE_LUMINANCE_HISTOGRAM: dev::k_histogram< M ><<< grid, blk, 0, s >>>( a ); break;
        case RGDN_STAGE_LUMINANCE_AVG: dev::k_luminance_avg< M ><<< 1, 256, 0, s >>>( a ); break;
        case KF_ATROUS_FAST: dev::k_atrous< M, true, false ><<< grid, blk, 0, s >>>( a, iter ); break;
        case KF_ATROUS_FAST_HIST: dev::k_atrous< M, true, true ><<< grid, blk, 0, s >>>( a, iter ); break;
        case KF_ATROUS_EXACT_HIST: dev::k_atrous< M, false, true ><<< grid, blk, 0, s >>>( a, iter ); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace rgdn
