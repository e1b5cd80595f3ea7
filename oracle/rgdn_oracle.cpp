// ============================================================================================
//  CPU ORACLE — TEST INFRASTRUCTURE ONLY.
//
//  A line-by-line C++ restatement of RayTracedGL1's image-space denoise-and-expose shaders.
//  Only the tests, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm use
//  it, as the checker. The product library never links, loads or calls anything here.
//
//  Parity status: PINNED to the reference's own shader sources for the compute stages. The
//  reference path is GLSL for Vulkan, which no machine here runs; oracle/glsl_ref/ runs those
//  GLSL sources on the CPU instead (a mechanical rewrite to C++ over a GLSL runtime written
//  for it), dispatched as the reference dispatches them, and tests/test_ref_shaders.py
//  requires every plane and the tonemapping buffer to equal this oracle's bit for bit after
//  every stage: the gradient samples (RtGradients.rgen's main(), its ray-traced forward
//  projection read from the boundary input RGDN_FB_GRADIENT_RESHADED), the gradient a-trous,
//  temporal accumulation, anti-firefly, variance, the a-trous iterations with the composition,
//  the histogram and the adaptation, the bloom pyramid, the volumetric scattering
//  (CmVolumetricProcess + CmScatterAccum) and the final composition (CmCheckerboard +
//  CmPrepareFinal, the LPM control block from the reference's own CPU-side LpmSetup)
//  and the bloom's application (committed vectors in tests/golden, and live where the
//  reference checkout is present). The re-shading of the analytic scene
//  stay pinned only by the codecs' known-answer tests from the public specs they implement
//  (IEEE-754 binary16/bfloat16, EXT_texture_shared_exponent, the Vulkan B10G11R11
//  unsigned-float layout) and the closed-form known-answer tests in tests/.
//
//  Conventions shared with the GPU path (each is a choice where GLSL leaves freedom):
//   * texelFetch / imageLoad outside the image returns an all-zero texel (raw bits 0, then
//     decoded: a zero normal code decodes to (0,0,1)).
//   * min/max/clamp follow IEEE minNum/maxNum (a NaN operand yields the other operand).
//   * mix(x,y,a) = x*(1-a) + y*a; smoothstep per the GLSL definition.
//   * round() rounds half away from zero (EXT_texture_shared_exponent's floor(x+0.5) for x>=0).
//   * float->fp16/bf16 conversion rounds to nearest even; fp16 overflow gives Inf.
//   * float->unorm8 = round(clamp(x,0,1)*255); unorm8->float = u / 255.0.
//   * B10G11R11 conversion rounds to nearest even, clamps to the largest finite value,
//     maps negatives and NaN to 0.
//   * sin/cos of the spherical normal decode are the correctly rounded float values of the
//     float angle (computed here through double precision).
//   * the histogram shaders' groupMemoryBarrier-only synchronisation is read as the
//     intended race-free semantics (CmLuminanceHistogram.comp:60-86, CmLuminanceAvg.comp:39-89).
//   * the single-thread tail of CmLuminanceAvg.comp evaluates exp2/exp through double
//     precision and rounds to float.
//   * arithmetic is plain IEEE binary32 with no fused multiply-add contraction
//     (build with -ffp-contract=off); sums run in the shader's loop order.
//
//  Template parameter T = float restates the shaders in FP32; T = double with the F64
//  storage mode is the FP64 error reference (no quantisation of internal buffers).
// ============================================================================================

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <type_traits>
#include <vector>

#include "../include/rgdn.h"

namespace orc
{

// --------------------------------------------------------------------------------------------
// Scalar / vector helpers with GLSL semantics
// --------------------------------------------------------------------------------------------

template< class T > struct V2 { T x, y; };
template< class T > struct V3 { T x, y, z; };
template< class T > struct V4 { T x, y, z, w; };

// float literal for T=float, double literal for T=double (no double rounding of constants)
#define K( lit ) ( std::is_same< T, float >::value ? (T)( lit##f ) : (T)( lit ) )

inline float  o_fmin( float a, float b ) { return fminf( a, b ); }
inline double o_fmin( double a, double b ) { return fmin( a, b ); }
inline float  o_fmax( float a, float b ) { return fmaxf( a, b ); }
inline double o_fmax( double a, double b ) { return fmax( a, b ); }
inline float  o_abs( float a ) { return fabsf( a ); }
inline double o_abs( double a ) { return fabs( a ); }
inline float  o_sqrt( float a ) { return sqrtf( a ); }
inline double o_sqrt( double a ) { return sqrt( a ); }
inline float  o_exp( float a ) { return expf( a ); }
inline double o_exp( double a ) { return exp( a ); }
inline float  o_exp2( float a ) { return exp2f( a ); }
inline double o_exp2( double a ) { return exp2( a ); }
inline float  o_log( float a ) { return logf( a ); }
inline double o_log( double a ) { return log( a ); }
inline float  o_log2( float a ) { return log2f( a ); }
inline double o_log2( double a ) { return log2( a ); }
inline float  o_pow( float a, float b ) { return powf( a, b ); }
inline double o_pow( double a, double b ) { return pow( a, b ); }
inline float  o_floor( float a ) { return floorf( a ); }
inline double o_floor( double a ) { return floor( a ); }

template< class T > inline T gclamp( T x, T lo, T hi ) { return o_fmin( o_fmax( x, lo ), hi ); }
template< class T > inline T gsat( T x ) { return gclamp( x, (T)0, (T)1 ); }
template< class T > inline T gmix( T x, T y, T a ) { return x * ( (T)1 - a ) + y * a; }
template< class T > inline T gsmoothstep( T e0, T e1, T x )
{
    T t = gclamp( ( x - e0 ) / ( e1 - e0 ), (T)0, (T)1 );
    return t * t * ( (T)3 - (T)2 * t );
}

template< class T > inline V3< T > operator+( V3< T > a, V3< T > b ) { return { a.x + b.x, a.y + b.y, a.z + b.z }; }
template< class T > inline V3< T > operator-( V3< T > a, V3< T > b ) { return { a.x - b.x, a.y - b.y, a.z - b.z }; }
template< class T > inline V3< T > operator*( V3< T > a, V3< T > b ) { return { a.x * b.x, a.y * b.y, a.z * b.z }; }
template< class T > inline V3< T > operator*( V3< T > a, T s ) { return { a.x * s, a.y * s, a.z * s }; }
template< class T > inline V3< T > operator*( T s, V3< T > a ) { return { s * a.x, s * a.y, s * a.z }; }
template< class T > inline V3< T > operator/( V3< T > a, T s ) { return { a.x / s, a.y / s, a.z / s }; }
template< class T > inline V3< T > vmix( V3< T > x, V3< T > y, T a )
{
    return { gmix( x.x, y.x, a ), gmix( x.y, y.y, a ), gmix( x.z, y.z, a ) };
}
template< class T > inline V3< T > vmin( V3< T > a, V3< T > b ) { return { o_fmin( a.x, b.x ), o_fmin( a.y, b.y ), o_fmin( a.z, b.z ) }; }
template< class T > inline V3< T > vmax( V3< T > a, V3< T > b ) { return { o_fmax( a.x, b.x ), o_fmax( a.y, b.y ), o_fmax( a.z, b.z ) }; }
template< class T > inline V3< T > vclamp( V3< T > x, V3< T > lo, V3< T > hi ) { return vmin( vmax( x, lo ), hi ); }
template< class T > inline T dot3( V3< T > a, V3< T > b ) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template< class T > inline V3< T > normalize3( V3< T > v )
{
    T len = o_sqrt( dot3( v, v ) );
    return { v.x / len, v.y / len, v.z / len };
}
// Utils.h:54-57
template< class T > inline T luminance( V3< T > c ) { return K( 0.2125 ) * c.x + K( 0.7154 ) * c.y + K( 0.0721 ) * c.z; }
template< class T > inline V3< T > xyz( V4< T > v ) { return { v.x, v.y, v.z }; }

// column-major mat4 * vec4 (the reference uniform's float[16] layout), summed column by column
template< class T > inline V4< T > mat_mul( const float* m, V4< T > v )
{
    V4< T > r;
    T*      rp = &r.x;
    for( int row = 0; row < 4; row++ )
    {
        rp[ row ] = (T)m[ 0 * 4 + row ] * v.x + (T)m[ 1 * 4 + row ] * v.y + (T)m[ 2 * 4 + row ] * v.z +
                    (T)m[ 3 * 4 + row ] * v.w;
    }
    return r;
}

// --------------------------------------------------------------------------------------------
// Codecs (restated from the public specifications)
// --------------------------------------------------------------------------------------------

inline uint32_t fbits( float f ) { uint32_t u; memcpy( &u, &f, 4 ); return u; }
inline float    bitsf( uint32_t u ) { float f; memcpy( &f, &u, 4 ); return f; }

// IEEE-754 binary32 -> binary16, round to nearest even
uint16_t f32_to_f16( float f )
{
    uint32_t x    = fbits( f );
    uint32_t sign = ( x >> 16 ) & 0x8000u;
    uint32_t ex   = ( x >> 23 ) & 0xFFu;
    uint32_t man  = x & 0x7FFFFFu;
    if( ex == 0xFF )
    {
        if( man ) return (uint16_t)( sign | 0x7E00u | ( man >> 13 ) );   // quiet NaN, payload kept
        return (uint16_t)( sign | 0x7C00u );
    }
    int e = (int)ex - 127 + 15;
    if( e >= 31 ) return (uint16_t)( sign | 0x7C00u );
    if( e <= 0 )
    {
        if( e < -10 ) return (uint16_t)sign;  // below half the smallest subnormal
        uint32_t sig   = man | 0x800000u;
        int      shift = 14 - e;              // 24-bit significand -> subnormal mantissa
        uint32_t q     = sig >> shift;
        uint32_t rem   = sig & ( ( 1u << shift ) - 1 );
        uint32_t half  = 1u << ( shift - 1 );
        if( rem > half || ( rem == half && ( q & 1 ) ) ) q++;
        return (uint16_t)( sign | q );        // q == 0x400 carries into the exponent field
    }
    uint32_t q    = man >> 13;
    uint32_t rem  = man & 0x1FFFu;
    uint32_t res  = ( (uint32_t)e << 10 ) | q;
    if( rem > 0x1000u || ( rem == 0x1000u && ( q & 1 ) ) ) res++;  // carry may reach Inf
    return (uint16_t)( sign | res );
}

float f16_to_f32( uint16_t h )
{
    uint32_t sign = ( (uint32_t)h & 0x8000u ) << 16;
    uint32_t ex   = ( h >> 10 ) & 0x1Fu;
    uint32_t man  = h & 0x3FFu;
    if( ex == 0 )
    {
        float v = (float)man * 5.9604644775390625e-08f;  // 2^-24
        return sign ? -v : v;
    }
    if( ex == 31 ) return bitsf( sign | 0x7F800000u | ( man << 13 ) );
    return bitsf( sign | ( ( ex - 15 + 127 ) << 23 ) | ( man << 13 ) );
}

uint16_t f32_to_bf16( float f )
{
    uint32_t x = fbits( f );
    if( ( x & 0x7F800000u ) == 0x7F800000u && ( x & 0x7FFFFFu ) ) return (uint16_t)( ( x >> 16 ) | 0x40u );
    uint32_t lsb = ( x >> 16 ) & 1u;
    x += 0x7FFFu + lsb;
    return (uint16_t)( x >> 16 );
}
float bf16_to_f32( uint16_t b ) { return bitsf( (uint32_t)b << 16 ); }

// unsigned small float with 5 exponent bits (bias 15) and `mbits` mantissa bits
uint32_t f32_to_uf( float f, int mbits )
{
    const uint32_t maxFinite = ( 30u << mbits ) | ( ( 1u << mbits ) - 1 );
    if( !( f > 0.0f ) ) return 0;             // negative, zero, NaN
    uint32_t x   = fbits( f );
    uint32_t ex  = ( x >> 23 ) & 0xFFu;
    uint32_t man = x & 0x7FFFFFu;
    if( ex == 0xFF ) return maxFinite;        // +Inf clamps
    int      e   = (int)ex - 127 + 15;
    uint32_t sig = ex ? ( man | 0x800000u ) : man;
    int      shift;
    if( e >= 1 ) shift = 23 - mbits;
    else
    {
        shift = 23 - mbits + ( 1 - e );
        e     = 0;
        if( shift > 24 ) return 0;
    }
    uint32_t q    = sig >> shift;
    uint32_t rem  = sig & ( ( 1u << shift ) - 1 );
    uint32_t half = 1u << ( shift - 1 );
    if( rem > half || ( rem == half && ( q & 1 ) ) ) q++;
    uint32_t res;
    if( e == 0 ) res = q;                                      // subnormal (q may carry to 1<<mbits)
    else
    {
        if( q == ( 2u << mbits ) ) { q >>= 1; e++; }
        res = ( (uint32_t)e << mbits ) | ( q & ( ( 1u << mbits ) - 1 ) );
    }
    if( res > maxFinite ) res = maxFinite;
    return res;
}

float uf_to_f32( uint32_t v, int mbits )
{
    uint32_t e = v >> mbits;
    uint32_t m = v & ( ( 1u << mbits ) - 1 );
    if( e == 0 ) return ldexpf( (float)m, -14 - mbits );
    if( e == 31 ) return m ? NAN : INFINITY;
    return ldexpf( (float)( ( 1u << mbits ) | m ), (int)e - 15 - mbits );
}

uint32_t encode_b10g11r11( float r, float g, float b )
{
    return f32_to_uf( r, 6 ) | ( f32_to_uf( g, 6 ) << 11 ) | ( f32_to_uf( b, 5 ) << 22 );
}
void decode_b10g11r11( uint32_t p, float* out )
{
    out[ 0 ] = uf_to_f32( p & 0x7FFu, 6 );
    out[ 1 ] = uf_to_f32( ( p >> 11 ) & 0x7FFu, 6 );
    out[ 2 ] = uf_to_f32( ( p >> 22 ) & 0x3FFu, 5 );
}

inline float o_roundf( float x ) { return roundf( x ); }

// Utils.h:152-192 encodeE5B9G9R9, with floor(log2(x)) taken from the exponent field
uint32_t encode_e5( float r, float g, float b )
{
    const int N = 9, B = 15, Np2 = 1 << N;
    r = o_fmin( o_fmax( r, 0.0f ), 65408.0f );
    g = o_fmin( o_fmax( g, 0.0f ), 65408.0f );
    b = o_fmin( o_fmax( b, 0.0f ), 65408.0f );
    float max_c = o_fmax( r, o_fmax( g, b ) );
    if( max_c == 0.0f ) return 0;
    uint32_t bits   = fbits( max_c );
    int      ex     = (int)( ( bits >> 23 ) & 0xFF );
    int      flog2  = ex ? ex - 127 : -127;            // subnormals are far below -B-1
    int      exp_p  = std::max( -B - 1, flog2 ) + 1 + B;
    int      max_s  = (int)o_roundf( max_c * ldexpf( 1.0f, -( exp_p - B - N ) ) );
    int      exp_sh = max_s != Np2 ? exp_p : exp_p + 1;
    float    s      = ldexpf( 1.0f, -( exp_sh - B - N ) );
    uint32_t rs     = (uint32_t)o_roundf( r * s );
    uint32_t gs     = (uint32_t)o_roundf( g * s );
    uint32_t bs     = (uint32_t)o_roundf( b * s );
    return ( (uint32_t)exp_sh << 27 ) | ( bs << 18 ) | ( gs << 9 ) | rs;
}

// Utils.h:194-207
void decode_e5( uint32_t p, float* out )
{
    int   e = (int)( p >> 27 );
    float s = ldexpf( 1.0f, e - 15 - 9 );
    out[ 0 ] = s * (float)( p & 0x1FFu );
    out[ 1 ] = s * (float)( ( p >> 9 ) & 0x1FFu );
    out[ 2 ] = s * (float)( ( p >> 18 ) & 0x1FFu );
}

// Utils.h:124-140 decodeNormal
template< class T > V3< T > decode_normal( uint32_t packed )
{
    uint32_t j = packed >> 16;
    uint32_t k = packed & 0xFFFFu;
    if constexpr( std::is_same< T, float >::value )
    {
        float phi   = (float)j * 3.14159265f / 65535.0f;
        float theta = (float)( k * 2u ) * 3.14159265f / 65536.0f;
        float sp    = (float)sin( (double)phi );
        float cp    = (float)cos( (double)phi );
        float st    = (float)sin( (double)theta );
        float ct    = (float)cos( (double)theta );
        return { sp * ct, sp * st, cp };
    }
    else
    {
        double phi   = (double)j * M_PI / 65535.0;
        double theta = (double)( k * 2u ) * M_PI / 65536.0;
        return { sin( phi ) * cos( theta ), sin( phi ) * sin( theta ), cos( phi ) };
    }
}

// Utils.h:108-122 encodeNormal (used by the known-answer tests only)
uint32_t encode_normal( float x, float y, float z )
{
    const float PI    = 3.14159265f;
    float       phi   = acosf( z );
    float       theta = atan2f( y, x );
    theta             = theta < 0 ? theta + 2 * PI : theta;
    uint32_t j        = (uint32_t)o_roundf( phi * 65535.0f / PI );
    uint32_t kk       = ( (uint32_t)o_roundf( theta * 65536.0f / ( 2 * PI ) ) ) % 65536u;
    return ( j << 16 ) | kk;
}

// CmLuminanceHistogram.comp:41-54 getColorBin
uint32_t color_bin( float inputLum, float minLog, float maxLog )
{
    float inv = 1.0f / ( maxLog - minLog );
    if( inputLum < 0.001f ) return 0;
    float ll = gclamp( ( log2f( inputLum ) - minLog ) * inv, 0.0f, 1.0f );
    return (uint32_t)( ll * 254.0f + 1.0f );
}

// --------------------------------------------------------------------------------------------
// Images
// --------------------------------------------------------------------------------------------

enum Fmt : uint32_t
{
    F_NONE     = RGDN_FORMAT_NONE,
    F_R8U      = RGDN_FORMAT_R8_UINT,
    F_RG8      = RGDN_FORMAT_RG8_UNORM,
    F_RGBA8    = RGDN_FORMAT_RGBA8_UNORM,
    F_R16F     = RGDN_FORMAT_R16_SFLOAT,
    F_RG16F    = RGDN_FORMAT_RG16_SFLOAT,
    F_RGBA16F  = RGDN_FORMAT_RGBA16_SFLOAT,
    F_RGBA16BF = RGDN_FORMAT_RGBA16_BFLOAT,
    F_R32F     = RGDN_FORMAT_R32_SFLOAT,
    F_RG32F    = RGDN_FORMAT_RG32_SFLOAT,
    F_RGBA32F  = RGDN_FORMAT_RGBA32_SFLOAT,
    F_R32U     = RGDN_FORMAT_R32_UINT,
    F_E5       = RGDN_FORMAT_E5B9G9R9_UFLOAT,
    F_B10G11R11= RGDN_FORMAT_B10G11R11_UFLOAT,
    F_NORMAL   = RGDN_FORMAT_NORMAL_SPHERICAL,
    F_RGBA32U  = RGDN_FORMAT_RGBA32_UINT,
    // oracle-only, FP64 error reference
    F_R64F     = 100,
    F_RG64F    = 101,
    F_RGBA64F  = 102,
};

inline uint32_t fmt_bytes( uint32_t f )
{
    switch( f )
    {
        case F_R8U: return 1;
        case F_RG8: return 2;
        case F_R16F: return 2;
        case F_RGBA8: case F_RG16F: case F_R32F: case F_R32U: case F_E5: case F_B10G11R11: case F_NORMAL: return 4;
        case F_RGBA16F: case F_RGBA16BF: case F_RG32F: case F_R64F: return 8;
        case F_RGBA32F: case F_RG64F: case F_RGBA32U: return 16;
        case F_RGBA64F: return 32;
        default: return 0;
    }
}

enum StorageMode : uint32_t { M_REF = 0, M_F32 = 1, M_F16 = 2, M_BF16 = 3, M_F64 = 4 };

struct FbInfo
{
    uint32_t fmt;
    bool     prev;
    bool     third;    // 1/3 resolution
    int      shift = 0;   // Framebuffers.cpp:669-692 FORCE_SIZE_BLOOM: (size + 1) / 2^shift, at least 1
    int      fixedW = 0, fixedH = 0;   // a size independent of the render size
};

// The oracle's own format table (the reference's is GenerateShaderCommon.py:802-887).
FbInfo fb_info( uint32_t fb, uint32_t mode )
{
    const bool f64  = mode == M_F64;
    uint32_t col3   = mode == M_REF ? F_E5 : mode == M_F32 ? F_RGBA32F : mode == M_F16 ? F_RGBA16F : mode == M_BF16 ? F_RGBA16BF : F_RGBA64F;
    uint32_t colvar = mode == M_REF ? F_RGBA16F : mode == M_F32 ? F_RGBA32F : mode == M_F16 ? F_RGBA16F : mode == M_BF16 ? F_RGBA16BF : F_RGBA64F;
    uint32_t hlen   = colvar;
    uint32_t mom    = mode == M_REF ? F_RG16F : f64 ? F_RG64F : F_RG32F;
    uint32_t fvar   = mode == M_REF ? F_R16F : f64 ? F_R64F : F_R32F;
    uint32_t pre    = mode == M_REF ? F_B10G11R11 : mode == M_F32 ? F_RGBA32F : f64 ? F_RGBA64F : F_RGBA16F;
    uint32_t dis    = f64 ? F_RGBA64F : F_RGBA8;
    uint32_t varpl  = ( mode == M_F16 || mode == M_BF16 ) ? F_R32F : F_NONE;
    switch( fb )
    {
        case RGDN_FB_ALBEDO: return { F_B10G11R11, false, false };
        case RGDN_FB_IS_SKY: return { F_R8U, false, false };
        case RGDN_FB_NORMAL: return { F_NORMAL, true, false };
        case RGDN_FB_METALLIC_ROUGHNESS: return { F_RG8, true, false };
        case RGDN_FB_DEPTH_WORLD: return { F_R16F, true, false };
        case RGDN_FB_DEPTH_GRAD: return { F_R16F, false, false };
        case RGDN_FB_MOTION: return { F_RGBA16F, false, false };
        case RGDN_FB_UNFILTERED_DIRECT:
        case RGDN_FB_UNFILTERED_SPECULAR:
        case RGDN_FB_UNFILTERED_INDIR: return { F_E5, false, false };
        case RGDN_FB_SURFACE_POSITION: return { F_RGBA32F, true, false };
        case RGDN_FB_VIEW_DIRECTION: return { F_RGBA16F, false, false };
        case RGDN_FB_THROUGHPUT: return { F_RGBA16F, false, false };
        case RGDN_FB_GRADIENT_INPUTS: return { F_RG16F, true, false };
        case RGDN_FB_GRADIENT_RESHADED: return { F_RG32F, false, false };
        case RGDN_FB_PRE_FINAL: return { pre, false, false };
        case RGDN_FB_HISTOGRAM_INPUT: return { F_R16F, false, false };
        case RGDN_FB_ACCUM_HISTORY_LENGTH: return { hlen, true, false };
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
        case RGDN_FB_DIS_PONG_GRADIENT: return { dis, false, true };
        case RGDN_FB_DIS_GRADIENT_HISTORY: return { dis, true, true };
        case RGDN_FB_GRADIENT_PREV_PIX: return { F_R8U, false, true };
        case RGDN_FB_DIFF_COLOR_HISTORY_VARIANCE:
        case RGDN_FB_DIFF_PING_VARIANCE:
        case RGDN_FB_DIFF_PONG_VARIANCE: return { varpl, false, false };
        // GenerateShaderCommon.py:820-863 ScreenEmisRT, Scattering, Final, BloomInput (the last
        // two in PreFinal's format per storage mode)
        case RGDN_FB_SCREEN_EMIS_RT: return { F_B10G11R11, false, false };
        case RGDN_FB_SCATTERING: return { F_RGBA16F, true, false };
        // GenerateShaderCommon.py:810, 854-855 DepthNdc, ScatteringHistory; Volumetric.cpp:31,
        // 259-290 the scattering volume (RGBA16F, two slots), as an image of X x (Y * Z) texels
        case RGDN_FB_DEPTH_NDC: return { F_R32F, false, false };
        case RGDN_FB_SCATTERING_HISTORY: return { F_R16F, true, false };
        case RGDN_FB_SCATTER_VOLUME: return { F_RGBA16F, true, false, 0, RGDN_VOLUME_SIZE_X, RGDN_VOLUME_SIZE_Y * RGDN_VOLUME_SIZE_Z };
        case RGDN_FB_FINAL:
        case RGDN_FB_BLOOM_INPUT:
        case RGDN_FB_BLOOM_RESULT: return { pre, false, false };
        case RGDN_FB_BLOOM_MIP1: case RGDN_FB_BLOOM_MIP2: case RGDN_FB_BLOOM_MIP3: case RGDN_FB_BLOOM_MIP4:
        case RGDN_FB_BLOOM_MIP5: case RGDN_FB_BLOOM_MIP6: case RGDN_FB_BLOOM_MIP7: case RGDN_FB_BLOOM_MIP8:
            return { pre, false, false, (int)( fb - RGDN_FB_BLOOM_MIP1 ) + 1 };
        // GenerateShaderCommon.py Reservoirs (R32G32B32A32_UINT, stored with _Prev)
        case RGDN_FB_RESERVOIRS: return { F_RGBA32U, true, false };
        default: return { F_NONE, false, false };
    }
}

struct Plane
{
    int                    w = 0, h = 0;
    uint32_t               fmt = F_NONE;
    uint32_t               texel = 0;
    std::vector< uint8_t > bytes;

    void init( int W, int H, uint32_t f )
    {
        w = W; h = H; fmt = f; texel = fmt_bytes( f );
        bytes.assign( (size_t)W * H * texel, 0 );
    }
    bool     inside( int x, int y ) const { return x >= 0 && y >= 0 && x < w && y < h; }
    uint8_t* at( int x, int y ) { return bytes.data() + ( (size_t)y * w + x ) * texel; }
    const uint8_t* at( int x, int y ) const { return bytes.data() + ( (size_t)y * w + x ) * texel; }

    uint32_t raw_u32( int x, int y ) const
    {
        if( !inside( x, y ) ) return 0;
        uint32_t v; memcpy( &v, at( x, y ), 4 ); return v;
    }
    uint32_t raw_u8( int x, int y ) const { return inside( x, y ) ? *at( x, y ) : 0u; }
    // one 32-bit word k of a texel (RGBA32_UINT)
    uint32_t raw_word( int x, int y, int k ) const
    {
        if( !inside( x, y ) ) return 0;
        uint32_t v; memcpy( &v, at( x, y ) + 4 * k, 4 ); return v;
    }

    // texelFetch with the OOB-is-zero convention, decoded to T
    template< class T > V4< T > fetch( int x, int y ) const
    {
        V4< T > r = { 0, 0, 0, 0 };
        if( !inside( x, y ) ) { if( fmt == F_E5 || fmt == F_B10G11R11 || fmt == F_NORMAL ) {} return r; }
        const uint8_t* p = at( x, y );
        switch( fmt )
        {
            case F_R8U: r.x = (T)p[ 0 ]; break;
            case F_RG8: r.x = (T)( (float)p[ 0 ] / 255.0f ); r.y = (T)( (float)p[ 1 ] / 255.0f ); break;
            case F_RGBA8:
                r.x = (T)( (float)p[ 0 ] / 255.0f ); r.y = (T)( (float)p[ 1 ] / 255.0f );
                r.z = (T)( (float)p[ 2 ] / 255.0f ); r.w = (T)( (float)p[ 3 ] / 255.0f ); break;
            case F_R16F: { uint16_t h; memcpy( &h, p, 2 ); r.x = (T)f16_to_f32( h ); break; }
            case F_RG16F: { uint16_t h[ 2 ]; memcpy( h, p, 4 ); r.x = (T)f16_to_f32( h[ 0 ] ); r.y = (T)f16_to_f32( h[ 1 ] ); break; }
            case F_RGBA16F: { uint16_t h[ 4 ]; memcpy( h, p, 8 ); r.x = (T)f16_to_f32( h[ 0 ] ); r.y = (T)f16_to_f32( h[ 1 ] ); r.z = (T)f16_to_f32( h[ 2 ] ); r.w = (T)f16_to_f32( h[ 3 ] ); break; }
            case F_RGBA16BF: { uint16_t h[ 4 ]; memcpy( h, p, 8 ); r.x = (T)bf16_to_f32( h[ 0 ] ); r.y = (T)bf16_to_f32( h[ 1 ] ); r.z = (T)bf16_to_f32( h[ 2 ] ); r.w = (T)bf16_to_f32( h[ 3 ] ); break; }
            case F_R32F: { float f; memcpy( &f, p, 4 ); r.x = (T)f; break; }
            case F_RG32F: { float f[ 2 ]; memcpy( f, p, 8 ); r.x = (T)f[ 0 ]; r.y = (T)f[ 1 ]; break; }
            case F_RGBA32F: { float f[ 4 ]; memcpy( f, p, 16 ); r.x = (T)f[ 0 ]; r.y = (T)f[ 1 ]; r.z = (T)f[ 2 ]; r.w = (T)f[ 3 ]; break; }
            case F_R32U: { uint32_t u; memcpy( &u, p, 4 ); r.x = (T)u; break; }
            case F_E5: { uint32_t u; memcpy( &u, p, 4 ); float c[ 3 ]; decode_e5( u, c ); r.x = (T)c[ 0 ]; r.y = (T)c[ 1 ]; r.z = (T)c[ 2 ]; break; }
            case F_B10G11R11: { uint32_t u; memcpy( &u, p, 4 ); float c[ 3 ]; decode_b10g11r11( u, c ); r.x = (T)c[ 0 ]; r.y = (T)c[ 1 ]; r.z = (T)c[ 2 ]; break; }
            case F_R64F: { double d; memcpy( &d, p, 8 ); r.x = (T)d; break; }
            case F_RG64F: { double d[ 2 ]; memcpy( d, p, 16 ); r.x = (T)d[ 0 ]; r.y = (T)d[ 1 ]; break; }
            case F_RGBA64F: { double d[ 4 ]; memcpy( d, p, 32 ); r.x = (T)d[ 0 ]; r.y = (T)d[ 1 ]; r.z = (T)d[ 2 ]; r.w = (T)d[ 3 ]; break; }
            default: break;
        }
        return r;
    }

    // imageStore; stores outside the image are dropped
    template< class T > void store( int x, int y, V4< T > v )
    {
        if( !inside( x, y ) ) return;
        uint8_t* p = at( x, y );
        switch( fmt )
        {
            case F_R8U: p[ 0 ] = (uint8_t)(uint32_t)v.x; break;
            case F_RG8: p[ 0 ] = unorm8( (float)v.x ); p[ 1 ] = unorm8( (float)v.y ); break;
            case F_RGBA8: p[ 0 ] = unorm8( (float)v.x ); p[ 1 ] = unorm8( (float)v.y ); p[ 2 ] = unorm8( (float)v.z ); p[ 3 ] = unorm8( (float)v.w ); break;
            case F_R16F: { uint16_t h = f32_to_f16( (float)v.x ); memcpy( p, &h, 2 ); break; }
            case F_RG16F: { uint16_t h[ 2 ] = { f32_to_f16( (float)v.x ), f32_to_f16( (float)v.y ) }; memcpy( p, h, 4 ); break; }
            case F_RGBA16F: { uint16_t h[ 4 ] = { f32_to_f16( (float)v.x ), f32_to_f16( (float)v.y ), f32_to_f16( (float)v.z ), f32_to_f16( (float)v.w ) }; memcpy( p, h, 8 ); break; }
            case F_RGBA16BF: { uint16_t h[ 4 ] = { f32_to_bf16( (float)v.x ), f32_to_bf16( (float)v.y ), f32_to_bf16( (float)v.z ), f32_to_bf16( (float)v.w ) }; memcpy( p, h, 8 ); break; }
            case F_R32F: { float f = (float)v.x; memcpy( p, &f, 4 ); break; }
            case F_RG32F: { float f[ 2 ] = { (float)v.x, (float)v.y }; memcpy( p, f, 8 ); break; }
            case F_RGBA32F: { float f[ 4 ] = { (float)v.x, (float)v.y, (float)v.z, (float)v.w }; memcpy( p, f, 16 ); break; }
            case F_R32U: { uint32_t u = (uint32_t)v.x; memcpy( p, &u, 4 ); break; }
            case F_E5: { uint32_t u = encode_e5( (float)v.x, (float)v.y, (float)v.z ); memcpy( p, &u, 4 ); break; }
            case F_B10G11R11: { uint32_t u = encode_b10g11r11( (float)v.x, (float)v.y, (float)v.z ); memcpy( p, &u, 4 ); break; }
            case F_R64F: { double d = (double)v.x; memcpy( p, &d, 8 ); break; }
            case F_RG64F: { double d[ 2 ] = { (double)v.x, (double)v.y }; memcpy( p, d, 16 ); break; }
            case F_RGBA64F: { double d[ 4 ] = { (double)v.x, (double)v.y, (double)v.z, (double)v.w }; memcpy( p, d, 32 ); break; }
            default: break;
        }
    }
    void store_u8( int x, int y, uint32_t v ) { if( inside( x, y ) ) *at( x, y ) = (uint8_t)v; }
    // v stored in this plane's format and read back
    template< class T > V3< T > requant( V3< T > v ) const
    {
        Plane one;
        one.init( 1, 1, fmt );
        one.store< T >( 0, 0, { v.x, v.y, v.z, (T)0 } );
        const V4< T > r = one.fetch< T >( 0, 0 );
        return { r.x, r.y, r.z };
    }

    static uint8_t unorm8( float f )
    {
        float c = o_fmin( o_fmax( f, 0.0f ), 1.0f );
        return (uint8_t)o_roundf( c * 255.0f );
    }
};

struct Stream
{
    int      W = 0, H = 0, GW = 0, GH = 0;
    uint32_t mode = M_REF;
    Plane    planes[ RGDN_FB_COUNT ][ 2 ];
    uint32_t hist[ 256 ] = {};
    double   avgLum      = 0.0;
    // the re-shade scene (rgdn_stream_set_reshade_scene), host copies
    bool                              rsSet = false;
    std::vector< rgdn_sphere_light > lights;
    std::vector< uint32_t >           prevToCur;
    std::vector< rgdn_occluder >      occluders;

    void init( int w, int h, uint32_t m )
    {
        W = w; H = h; mode = m;
        GW = std::max( 1, ( w + 1 ) / 3 );   // Framebuffers.cpp:690-697 FORCE_SIZE_1_3
        GH = std::max( 1, ( h + 1 ) / 3 );
        for( uint32_t fb = 0; fb < RGDN_FB_COUNT; fb++ )
        {
            FbInfo fi = fb_info( fb, m );
            for( int s = 0; s < 2; s++ )
            {
                if( fi.fmt == F_NONE || ( s == 1 && !fi.prev ) ) { planes[ fb ][ s ] = Plane(); continue; }
                int pw = fi.third ? GW : W, ph = fi.third ? GH : H;
                if( fi.shift ) pw = std::max( 1, ( W + 1 ) >> fi.shift ), ph = std::max( 1, ( H + 1 ) >> fi.shift );
                if( fi.fixedW ) pw = fi.fixedW, ph = fi.fixedH;
                planes[ fb ][ s ].init( pw, ph, fi.fmt );
            }
        }
        memset( hist, 0, sizeof( hist ) );
        avgLum = 0.0;
    }
    // Framebuffers::FrameIndexToFBIndex (Framebuffers.cpp:34-49)
    Plane& cur( uint32_t fb, uint32_t fi ) { return fb_info( fb, mode ).prev ? planes[ fb ][ fi & 1 ] : planes[ fb ][ 0 ]; }
    Plane& prv( uint32_t fb, uint32_t fi ) { return fb_info( fb, mode ).prev ? planes[ fb ][ ( fi & 1 ) ^ 1 ] : planes[ fb ][ 0 ]; }
};

// --------------------------------------------------------------------------------------------
// Parallel loop over rows (the CPU baseline uses every host core)
// --------------------------------------------------------------------------------------------
template< class F > void parallel_rows( int h, int nthreads, F&& fn )
{
    if( nthreads <= 1 || h < 2 * nthreads )
    {
        for( int y = 0; y < h; y++ ) fn( y );
        return;
    }
    std::atomic< int >         next( 0 );
    std::vector< std::thread > ts;
    for( int t = 0; t < nthreads; t++ )
    {
        ts.emplace_back( [ & ]() {
            for( ;; )
            {
                int y = next.fetch_add( 1 );
                if( y >= h ) break;
                fn( y );
            }
        } );
    }
    for( auto& t : ts ) t.join();
}

// --------------------------------------------------------------------------------------------
// The stages
// --------------------------------------------------------------------------------------------

constexpr int   STRATA         = 3;        // COMPUTE_ASVGF_STRATA_SIZE (ShaderCommonC.h:150)
constexpr float MAX_RAY_LENGTH = 10000.0f; // ShaderCommonC.h:167

uint32_t wellons_lowbias32( uint32_t x );
uint32_t random_seed( int px, int py, uint32_t frame );

template< class T > struct Denoise
{
    Stream&                  s;
    uint32_t                 fi;
    const rgdn_frame_params& p;
    int                      nthreads;

    int W() const { return s.W; }
    int H() const { return s.H; }
    // ShGlobalUniform.renderWidth / renderHeight are floats (VulkanDevice.cpp:184-185)
    float RW() const { return (float)s.W; }
    float RH() const { return (float)s.H; }

    // ShaderCommonGLSLFunc.h:306-357
    int sep() const { return s.W / 2; }
    static int odd_regular( int x, int y ) { return ( x + y % 2 ) % 2; }
    V2< int > regular_from_cb( int cx, int cy ) const
    {
        int isOdd = cx >= sep() ? 1 : 0;
        int x     = cx - isOdd * sep();
        return { x * 2 + ( isOdd + cy ) % 2, cy };
    }
    struct Area { int l, r, h; };
    Area cb_area( int cx, int /*cy*/ ) const
    {
        int isOdd = cx >= sep() ? 1 : 0;
        return { isOdd * sep(), ( isOdd + 1 ) * sep(), s.H };
    }
    static bool in_area( int x, int y, Area a ) { return y >= 0 && y < a.h && x >= a.l && x < a.r; }
    // ShaderCommonGLSLFunc.h:368-376
    static bool test_depth( T z, T zPrev, T zMotion ) { return o_abs( z - zPrev + zMotion ) / o_abs( z ) < K( 0.1 ); }
    static bool test_normal( V3< T > n, V3< T > np ) { return dot3( n, np ) > K( 0.95 ); }
    // ShaderCommonGLSLFunc.h:383-390
    static T antilag( T g, T nf )
    {
        T lambda = nf > K( 0.0001 ) ? gclamp( o_abs( g ) / nf, (T)0, (T)1 ) : (T)0;
        return gclamp( lambda, (T)0, (T)1 );
    }
    // ShaderCommonGLSLFunc.h:271-277
    V2< T > prev_screen_pos( V2< T > motion, int px, int py ) const
    {
        T sx  = (T)RW() / K( 2.0 );
        T sy  = (T)RH();
        T isx = (T)1 / sx, isy = (T)1 / sy;
        return { ( ( (T)px + K( 0.5 ) ) * isx + motion.x ) * sx, ( ( (T)py + K( 0.5 ) ) * isy + motion.y ) * sy };
    }

    Plane& C( uint32_t fb ) { return s.cur( fb, fi ); }
    Plane& P( uint32_t fb ) { return s.prv( fb, fi ); }
    uint32_t mode() const { return s.mode; }
    bool     has_var_plane() const { return mode() == M_F16 || mode() == M_BF16; }

    V3< T > fetch3( Plane& pl, int x, int y ) { return xyz( pl.template fetch< T >( x, y ) ); }
    void    store3( Plane& pl, int x, int y, V3< T > v ) { pl.template store< T >( x, y, { v.x, v.y, v.z, (T)0 } ); }
    V3< T > fetch_normal( Plane& pl, int x, int y ) { return decode_normal< T >( pl.raw_u32( x, y ) ); }

    uint32_t var_plane_of( uint32_t fb )
    {
        return fb == RGDN_FB_DIFF_COLOR_HISTORY ? RGDN_FB_DIFF_COLOR_HISTORY_VARIANCE
             : fb == RGDN_FB_DIFF_PING_COLOR_AND_VARIANCE ? RGDN_FB_DIFF_PING_VARIANCE
                                                          : RGDN_FB_DIFF_PONG_VARIANCE;
    }
    // colour + variance images: variance in .w, or in a separate FP32 plane (16-bit modes)
    V4< T > fetch_cv( uint32_t fb, int x, int y )
    {
        V4< T > v = C( fb ).template fetch< T >( x, y );
        if( has_var_plane() ) v.w = C( var_plane_of( fb ) ).template fetch< T >( x, y ).x;
        return v;
    }
    void store_cv( uint32_t fb, int x, int y, V3< T > c, T var )
    {
        if( has_var_plane() )
        {
            C( fb ).template store< T >( x, y, { c.x, c.y, c.z, (T)0 } );
            C( var_plane_of( fb ) ).template store< T >( x, y, { var, 0, 0, 0 } );
        }
        else C( fb ).template store< T >( x, y, { c.x, c.y, c.z, var } );
    }

    // ---------------------------------------------------------------- RtGradients.rgen:107-136
    // forwardProjectedLuminance of previous-frame pixel (px, py): the previous surface
    // (Surface.inl:72-90) lit by this frame's light selected through the previous reservoir
    // (Reservoir.h:138-146, lightSources_Index_PrevToCur), with the previous frame's seed
    // (Random.h:289-300) and light point (RaygenCommon.h:624-627, Light.h:244-258), shaded
    // (RaygenCommon.h:364-380, BRDF.h:34-146) and shadow-tested (RaygenCommon.h:322-359) against
    // the analytic occluders.
    static T safe_positive_rcp( T f ) { return f <= (T)0 ? (T)0 : (T)1 / f; }
    static V3< T > normalize_( V3< T > v ) { return v / o_sqrt( dot3( v, v ) ); }
    static V3< T > safe_normalize( V3< T > v )
    {
        T len = o_sqrt( dot3( v, v ) );
        return len > K( 0.001 ) ? v / len : V3< T >{ 0, 1, 0 };
    }
    static T safe_solid_angle( T a )
    {
        return a > (T)0 && !std::isnan( a ) && !std::isinf( a ) ? gclamp( a, (T)0, (T)4 * K( 3.14159265358979323846 ) ) : (T)0;
    }
    static T o_cos_( T x ) { if constexpr( std::is_same< T, float >::value ) return cosf( x ); else return cos( x ); }
    static T o_sin_( T x ) { if constexpr( std::is_same< T, float >::value ) return sinf( x ); else return sin( x ); }
    V3< T > brdf_smith_ggx( V3< T > n, V3< T > v, V3< T > l, T alpha, V3< T > specColor ) const
    {
        const T PI = K( 3.14159265358979323846 );
        alpha      = o_fmax( alpha, K( 0.005 ) );
        const T nl = o_fmax( dot3( n, l ), (T)0 );
        if( nl <= (T)0 ) return { 0, 0, 0 };
        const T       fr = o_pow( (T)1 - o_fmax( nl, (T)0 ), K( 5.0 ) );
        const V3< T > F  = { specColor.x + ( (T)1 - specColor.x ) * fr, specColor.y + ( (T)1 - specColor.y ) * fr,
                             specColor.z + ( (T)1 - specColor.z ) * fr };
        const V3< T > h       = normalize_( v + l );
        const T       alphaSq = alpha * alpha;
        const T       nm      = o_fmax( (T)0, dot3( n, h ) );
        const T       dd      = nm * nm * ( alphaSq - (T)1 ) + (T)1;
        const T       D       = alphaSq / PI / ( dd * dd );
        const T       nv      = o_fmax( dot3( n, v ), (T)0 );
        const T       G2      = K( 0.5 ) / gmix( (T)2 * nl * nv, nl + nv, alpha );
        return F * ( G2 * D );
    }
    bool shadowed( V3< T > start, V3< T > end ) const
    {
        V3< T >  l           = end - start;
        const T  maxDistance = o_sqrt( dot3( l, l ) );
        l                    = l / maxDistance;
        const T tmin = K( 0.001 ), tmax = maxDistance - K( 0.01 );
        for( const rgdn_occluder& o : s.occluders )
        {
            if( o.type == RGDN_OCCLUDER_SPHERE )
            {
                const V3< T > oc   = start - V3< T >{ (T)o.data[ 0 ], (T)o.data[ 1 ], (T)o.data[ 2 ] };
                const T       b    = dot3( oc, l );
                const T       c    = dot3( oc, oc ) - (T)o.data[ 3 ] * (T)o.data[ 3 ];
                const T       disc = b * b - c;
                if( disc <= (T)0 ) continue;
                const T sq = o_sqrt( disc );
                const T t0 = -b - sq, t1 = -b + sq;
                if( ( t0 >= tmin && t0 <= tmax ) || ( t1 >= tmin && t1 <= tmax ) ) return true;
            }
            else if( o.type == RGDN_OCCLUDER_RECT )
            {
                const int ax = (int)o.data[ 0 ];
                const T   so = ax == 0 ? start.x : ax == 1 ? start.y : start.z;
                const T   dl = ax == 0 ? l.x : ax == 1 ? l.y : l.z;
                if( dl == (T)0 ) continue;
                const T t = ( (T)o.data[ 1 ] - so ) / dl;
                if( !( t >= tmin && t <= tmax ) ) continue;
                const V3< T > q  = start + l * t;
                const T       u0 = ax == 0 ? q.y : q.x, u1 = ax == 2 ? q.y : q.z;
                if( u0 >= (T)o.data[ 2 ] && u0 <= (T)o.data[ 3 ] && u1 >= (T)o.data[ 4 ] && u1 <= (T)o.data[ 5 ] ) return true;
            }
        }
        return false;
    }
    V2< T > reshade( int px, int py )
    {
        const T  PI  = K( 3.14159265358979323846 );
        Plane&   res = P( RGDN_FB_RESERVOIRS );
        const uint32_t r0 = res.raw_word( px, py, 0 );
        const uint32_t selectedPrev = r0 & 65535u, Mres = ( r0 >> 16 ) & 65535u;
        if( selectedPrev == 32767u || selectedPrev >= s.prevToCur.size() ) return { 0, 0 };   // LIGHT_INDEX_NONE
        const uint32_t sel = s.prevToCur[ selectedPrev ];
        if( sel == 0xFFFFFFFFu || sel >= s.lights.size() ) return { 0, 0 };
        float tpdf, wsum;
        {
            uint32_t a = res.raw_word( px, py, 1 ), b = res.raw_word( px, py, 2 );
            memcpy( &tpdf, &a, 4 );
            memcpy( &wsum, &b, 4 );
        }
        const V4< T > sp   = P( RGDN_FB_SURFACE_POSITION ).template fetch< T >( px, py );
        const V3< T > pos  = { sp.x, sp.y, sp.z };
        const V4< T > mr   = P( RGDN_FB_METALLIC_ROUGHNESS ).template fetch< T >( px, py );
        const T       metallic = mr.x, roughness = mr.y;
        const T       spc  = K( 0.04 ) * ( (T)1 - metallic ) + (T)1 * metallic;   // getSpecularColor(vec3(1), metallic)
        const V3< T > n    = fetch_normal( P( RGDN_FB_NORMAL ), px, py );
        const V3< T > cam  = { (T)p.cameraPositionPrev[ 0 ], (T)p.cameraPositionPrev[ 1 ], (T)p.cameraPositionPrev[ 2 ] };
        const V3< T > v    = normalize_( cam - pos );
        const uint32_t seed = random_seed( px, py, p.frameId - 1u );
        const uint32_t rnd  = wellons_lowbias32( seed + 20u );   // RANDOM_SALT_LIGHT_POINT
        const T        r1   = (T)( (float)( rnd & 0xFFFFu ) / 65535.0f ) * K( 0.99 );
        const T        r2   = (T)( (float)( ( rnd & 0xFFFF0000u ) >> 16 ) / 65535.0f ) * K( 0.99 );
        const rgdn_sphere_light& L = s.lights[ sel ];
        const V3< T > c   = { (T)L.center[ 0 ], (T)L.center[ 1 ], (T)L.center[ 2 ] };
        V3< T >       tc  = c - pos;
        const T       tl  = o_sqrt( dot3( tc, tc ) );
        tc                = tc / tl;
        // sampleOrientedHemisphere(-toLightCenter.dir, u1, u2) (Random.h:175-201)
        V3< T > ln;
        {
            T       a   = (T)1 - (T)2 * r1;
            T       b   = o_sqrt( (T)1 - a * a );
            const T phi = (T)2 * PI * r2;
            a = a * K( 0.98 );
            b = b * K( 0.98 );
            ln = normalize_( V3< T >{ -tc.x + b * o_cos_( phi ), -tc.y + b * o_sin_( phi ), -tc.z + a } );
        }
        const V3< T > lpos = c + ln * (T)L.radius;
        T             dw;
        {
            const T sinTheta = (T)L.radius / o_fmax( (T)L.radius, tl );
            const T cosTheta = o_sqrt( (T)1 - sinTheta * sinTheta );
            dw               = safe_solid_angle( (T)2 * PI * ( (T)1 - cosTheta ) );
        }
        const V3< T > col = { (T)L.color[ 0 ], (T)L.color[ 1 ], (T)L.color[ 2 ] };
        const V3< T > l   = safe_normalize( lpos - pos );
        const T       nl  = dot3( n, l );
        if( nl <= (T)0 ) return { 0, 0 };
        const T       w    = safe_positive_rcp( (T)tpdf ) * ( (T)wsum / (T)std::max( 1u, Mres ) );
        const V3< T > base = col * ( dw * nl );
        const V3< T > dif  = ( base * ( (T)1 / PI ) ) * w;
        const V3< T > spe  = ( base * brdf_smith_ggx( n, v, l, roughness, { spc, spc, spc } ) ) * w;
        if( luminance( dif + spe ) <= (T)0 ) return { 0, 0 };
        if( shadowed( pos + v * K( 0.01 ), lpos ) ) return { 0, 0 };
        return { luminance( dif ), luminance( spe ) };
    }

    // ---------------------------------------------------------------- RtGradients.rgen:44-181
    void gradient_samples()
    {
        Plane& ping     = C( RGDN_FB_DIS_PING_GRADIENT );
        Plane& prevPix  = C( RGDN_FB_GRADIENT_PREV_PIX );
        Plane& motion   = C( RGDN_FB_MOTION );
        Plane& gInPrev  = P( RGDN_FB_GRADIENT_INPUTS );
        Plane& isSky    = C( RGDN_FB_IS_SKY );
        Plane& reshaded = C( RGDN_FB_GRADIENT_RESHADED );
        Plane& indirPrv = P( RGDN_FB_INDIR_ACCUM );
        Plane& disHist  = P( RGDN_FB_DIS_GRADIENT_HISTORY );
        const bool allOff = p.gradientMultDiffuse < 0.001f && p.gradientMultIndirect < 0.001f && p.gradientMultSpecular < 0.001f;

        parallel_rows( s.GH, nthreads, [ & ]( int gy ) {
            for( int gx = 0; gx < s.GW; gx++ )
            {
                if( gx * STRATA >= W() || gy * STRATA >= H() ) continue;
                if( allOff )
                {
                    ping.template store< T >( gx, gy, { 0, 0, 0, 0 } );
                    prevPix.store_u8( gx, gy, STRATA * STRATA + 1 );
                    continue;
                }
                const uint32_t prevStrataPos = prevPix.raw_u8( gx, gy );
                V2< int > prevShadingPix = { 0, 0 }, curShadingPix = { 0, 0 };
                uint32_t  curStrataPos   = 0;
                V2< T >   prevLum        = { 0, 0 };
                for( int yy = 0; yy < STRATA; yy++ )
                {
                    for( int xx = 0; xx < STRATA; xx++ )
                    {
                        if( (uint32_t)( yy * STRATA + xx ) == prevStrataPos ) continue;
                        int     cx = gx * STRATA + xx, cy = gy * STRATA + yy;
                        V4< T > m  = motion.template fetch< T >( cx, cy );
                        V2< T > pp = prev_screen_pos( { m.x, m.y }, cx, cy );
                        V2< int > ip = { (int)o_floor( pp.x ), (int)o_floor( pp.y ) };
                        V4< T >   il = gInPrev.template fetch< T >( ip.x, ip.y );
                        if( o_fmax( il.x, il.y ) > o_fmax( prevLum.x, prevLum.y ) )
                        {
                            prevShadingPix = ip;
                            curShadingPix  = { cx, cy };
                            curStrataPos   = (uint32_t)( yy * STRATA + xx );
                            prevLum        = { il.x, il.y };
                        }
                    }
                }
                if( !in_area( prevShadingPix.x, prevShadingPix.y, cb_area( curShadingPix.x, curShadingPix.y ) ) ||
                    isSky.raw_u8( curShadingPix.x, curShadingPix.y ) != 0 ||
                    ( prevLum.x <= (T)0 && prevLum.y <= (T)0 ) )
                {
                    ping.template store< T >( gx, gy, { 0, 0, 0, 0 } );
                    prevPix.store_u8( gx, gy, STRATA * STRATA + 1 );
                    continue;
                }
                V4< T > fpl = reshaded.template fetch< T >( prevShadingPix.x, prevShadingPix.y );
                if( s.rsSet )
                {
                    const V2< T > r = reshade( prevShadingPix.x, prevShadingPix.y );
                    fpl.x = r.x;
                    fpl.y = r.y;
                }
                T g[ 3 ];
                {
                    T gs = fpl.x - prevLum.x;
                    T nf = o_fmax( fpl.x, prevLum.x );
                    g[ 0 ] = antilag( gs, nf );
                }
                {
                    T gs = o_fmax( (T)0, prevLum.x - fpl.x );
                    T nf = o_fmax( fpl.x, prevLum.x );
                    T brightness = luminance( fetch3( indirPrv, prevShadingPix.x, prevShadingPix.y ) );
                    gs = gs * ( (T)1 - gsmoothstep( K( 1.0 ), K( 10.0 ), brightness ) );
                    g[ 1 ] = antilag( gs, nf );
                }
                {
                    T gs = fpl.y - prevLum.y;
                    T nf = o_fmax( fpl.y, prevLum.y );
                    g[ 2 ] = antilag( gs, nf );
                }
                g[ 0 ] = g[ 0 ] * (T)p.gradientMultDiffuse;
                g[ 1 ] = g[ 1 ] * (T)p.gradientMultIndirect;
                g[ 2 ] = g[ 2 ] * (T)p.gradientMultSpecular;
                V4< T > gp = disHist.template fetch< T >( prevShadingPix.x / STRATA, prevShadingPix.y / STRATA );
                g[ 0 ] = gmix( g[ 0 ], gp.x, K( 0.5 ) );
                g[ 1 ] = gmix( g[ 1 ], gp.y, K( 0.5 ) );
                g[ 2 ] = gmix( g[ 2 ], gp.z, K( 0.5 ) );
                ping.template store< T >( gx, gy, { g[ 0 ], g[ 1 ], g[ 2 ], (T)0 } );
                prevPix.store_u8( gx, gy, curStrataPos );
            }
        } );
    }

    // ---------------------------------------------------------------- CmASVGFGradientAtrous.comp:42-105
    void gradient_atrous( uint32_t iter )
    {
        Plane& ping = C( RGDN_FB_DIS_PING_GRADIENT );
        Plane& pong = C( RGDN_FB_DIS_PONG_GRADIENT );
        Plane& src  = ( iter % 2 == 0 ) ? ping : pong;
        Plane& dst  = ( iter % 2 == 0 ) ? pong : ping;
        Plane& hist = C( RGDN_FB_DIS_GRADIENT_HISTORY );
        const int   step = 1 << iter;
        const T     kern[ 2 ][ 2 ] = { { K( 1.0 ), K( 0.5 ) }, { K( 0.5 ), K( 0.25 ) } };

        parallel_rows( s.GH, nthreads, [ & ]( int gy ) {
            for( int gx = 0; gx < s.GW; gx++ )
            {
                if( gx * STRATA >= W() || gy * STRATA >= H() ) continue;
                Area a0 = cb_area( gx * STRATA, gy * STRATA );
                Area ga = { a0.l / STRATA, a0.r / STRATA, a0.h / STRATA };
                V3< T > out = { 0, 0, 0 };
                T       ws  = 0;
                for( int yy = -1; yy <= 1; yy++ )
                    for( int xx = -1; xx <= 1; xx++ )
                    {
                        int qx = gx + xx * step, qy = gy + yy * step;
                        V3< T > gq = fetch3( src, qx, qy );
                        T w = kern[ std::abs( yy ) ][ std::abs( xx ) ] * ( in_area( qx, qy, ga ) ? (T)1 : (T)0 );
                        out = out + gq * w;
                        ws  = ws + w;
                    }
                out = out / ws;
                dst.template store< T >( gx, gy, { out.x, out.y, out.z, (T)0 } );
                if( iter == 0 ) hist.template store< T >( gx, gy, { out.x, out.y, out.z, (T)0 } );
            }
        } );
    }

    // ---------------------------------------------------------------- CmSVGFTemporalAccumulation.comp:57-99
    T parallax( V3< T > pos, V3< T > posPrev )
    {
        V3< T > camDelta = { (T)p.cameraPositionPrev[ 0 ] - (T)p.cameraPosition[ 0 ],
                             (T)p.cameraPositionPrev[ 1 ] - (T)p.cameraPosition[ 1 ],
                             (T)p.cameraPositionPrev[ 2 ] - (T)p.cameraPosition[ 2 ] };
        V3< T > v     = normalize3( pos );
        V3< T > vPrev = normalize3( posPrev - camDelta );
        T       cosa  = gsat( dot3( v, vPrev ) );
        T       par   = o_sqrt( (T)1 - cosa * cosa ) / o_fmax( cosa, K( 1e-6 ) );
        return par * K( 60.0 );
    }
    T spec_min_accum() const
    {
        T td  = (T)p.timeDelta;
        T fps = td <= (T)0 ? (T)0 : (T)1 / td;
        return gclamp( K( 0.2 ) * fps, (T)0, K( 128.0 ) );
    }
    T spec_accum_speed( T Amax, T r, T NoV, T par )
    {
        T acos01sq = (T)1 - NoV;
        T a        = o_pow( gsat( acos01sq ), K( 0.66 ) );
        T b        = K( 1.1 ) + r * r;
        T ps       = ( b + a ) / ( b - a );
        T powScale = (T)1 + par * ps;
        T f        = (T)1 - o_exp2( K( -200.0 ) * r * r );
        f          = f * o_pow( gsat( r ), K( 0.5 ) * powScale );
        T A        = K( 256.0 ) * f;
        return gclamp( A, spec_min_accum(), Amax );
    }
    static T spec_dominant( T nv, T r )
    {
        T a = K( 0.298475 ) * o_log( K( 39.4115 ) - K( 39.0029 ) * r );
        T f = o_pow( gclamp( (T)1 - nv, (T)0, (T)1 ), K( 10.8649 ) ) * ( (T)1 - a ) + a;
        return gclamp( f, (T)0, (T)1 );
    }

    // ---------------------------------------------------------------- CmSVGFTemporalAccumulation.comp:101-384
    void temporal_accumulation()
    {
        Plane& unfD   = C( RGDN_FB_UNFILTERED_DIRECT );
        Plane& unfI   = C( RGDN_FB_UNFILTERED_INDIR );
        Plane& unfS   = C( RGDN_FB_UNFILTERED_SPECULAR );
        Plane& viewD  = C( RGDN_FB_VIEW_DIRECTION );
        Plane& motion = C( RGDN_FB_MOTION );
        Plane& depth  = C( RGDN_FB_DEPTH_WORLD );
        Plane& depthP = P( RGDN_FB_DEPTH_WORLD );
        Plane& nrm    = C( RGDN_FB_NORMAL );
        Plane& nrmP   = P( RGDN_FB_NORMAL );
        Plane& mr     = C( RGDN_FB_METALLIC_ROUGHNESS );
        Plane& spos   = C( RGDN_FB_SURFACE_POSITION );
        Plane& sposP  = P( RGDN_FB_SURFACE_POSITION );
        Plane& momP   = P( RGDN_FB_DIFF_ACCUM_MOMENTS );
        Plane& hlenP  = P( RGDN_FB_ACCUM_HISTORY_LENGTH );
        Plane& specP  = P( RGDN_FB_SPEC_ACCUM_COLOR );
        Plane& indirP = P( RGDN_FB_INDIR_ACCUM );
        Plane& grad   = C( RGDN_FB_DIS_PING_GRADIENT );
        const bool gradients = !( p.flags & RGDN_FLAG_SKIP_GRADIENTS );

        parallel_rows( H(), nthreads, [ & ]( int py ) {
            for( int px = 0; px < W(); px++ )
            {
                const V3< T > unfilteredDiff  = fetch3( unfD, px, py );
                const V3< T > unfilteredIndir = fetch3( unfI, px, py );
                const V3< T > unfilteredSpec  = fetch3( unfS, px, py );
                const V4< T > rayInfo         = viewD.template fetch< T >( px, py );
                const Area    chArea          = cb_area( px, py );
                const V4< T > mo              = motion.template fetch< T >( px, py );
                const T       motionZ         = mo.z;
                const T       z               = depth.template fetch< T >( px, py ).x;
                const V3< T > normal          = fetch_normal( nrm, px, py );
                const T       roughness       = mr.template fetch< T >( px, py ).y;

                const T       l       = luminance( unfilteredDiff );
                const V2< T > moments = { l, l * l };

                V2< int > pixPrev;
                V2< T >   subPix;
                {
                    V2< T > posPrev = prev_screen_pos( { mo.x, mo.y }, px, py );
                    T fx = o_floor( posPrev.x - K( 0.5 ) ), fy = o_floor( posPrev.y - K( 0.5 ) );
                    pixPrev = { (int)fx, (int)fy };
                    subPix  = { ( posPrev.x - K( 0.5 ) ) - fx, ( posPrev.y - K( 0.5 ) ) - fy };
                }
                const T bw[ 2 ][ 2 ] = {
                    { ( (T)1 - subPix.x ) * ( (T)1 - subPix.y ), subPix.x * ( (T)1 - subPix.y ) },
                    { ( (T)1 - subPix.x ) * subPix.y, subPix.x * subPix.y },
                };

                V4< T > histLenDIS     = { 0, 0, 0, 0 };
                V3< T > diffPrev       = { 0, 0, 0 };
                V2< T > momentsPrev    = { 0, 0 };
                V3< T > specPrevOnSurf = { 0, 0, 0 };
                V3< T > indirPrev      = { 0, 0, 0 };
                T       weightSum      = 0;

                for( int yy = 0; yy <= 1; yy++ )
                    for( int xx = 0; xx <= 1; xx++ )
                    {
                        int     qx = pixPrev.x + xx, qy = pixPrev.y + yy;
                        T       dP = depthP.template fetch< T >( qx, qy ).x;
                        V3< T > nP = fetch_normal( nrmP, qx, qy );
                        bool ok = in_area( qx, qy, chArea ) && test_depth( z, dP, motionZ ) && test_normal( normal, nP );
                        if( ok )
                        {
                            const T w = bw[ yy ][ xx ];
                            V4< T > dc = fetch_cv( RGDN_FB_DIFF_COLOR_HISTORY, qx, qy );
                            diffPrev = diffPrev + xyz( dc ) * w;
                            V4< T > m = momP.template fetch< T >( qx, qy );
                            momentsPrev = { momentsPrev.x + w * m.x, momentsPrev.y + w * m.y };
                            V4< T > hl = hlenP.template fetch< T >( qx, qy );
                            histLenDIS = { histLenDIS.x + w * hl.x, histLenDIS.y + w * hl.y, histLenDIS.z + w * hl.z, histLenDIS.w + w * hl.w };
                            specPrevOnSurf = specPrevOnSurf + w * fetch3( specP, qx, qy );
                            indirPrev      = indirPrev + w * fetch3( indirP, qx, qy );
                            weightSum      = weightSum + w;
                        }
                    }

                T aD = 0, aI = 0, aS = 0;
                if( gradients )
                {
                    V4< T > g = grad.template fetch< T >( px / STRATA, py / STRATA );
                    aD = g.x; aI = g.y; aS = g.z;
                }

                V3< T > specColorAccum;
                T       specHistoryLengthAccum, specHitDistanceAccum;

                if( weightSum > K( 0.0001 ) )
                {
                    specPrevOnSurf = specPrevOnSurf / weightSum;
                    const T specHistoryLength   = histLenDIS.z / weightSum;
                    const T specHitDistancePrev = histLenDIS.w / weightSum;

                    const V3< T > surfPos     = fetch3( spos, px, py );
                    const V3< T > surfPosPrev = fetch3( sposP, pixPrev.x, pixPrev.y );
                    T nv = o_fmax( (T)0, dot3( normal, V3< T >{ -rayInfo.x, -rayInfo.y, -rayInfo.z } ) );

                    const T A = gclamp( (T)1 + specHistoryLength * o_pow( (T)1 - aS, K( 5.0 ) ), spec_min_accum(), K( 256.0 ) );
                    const T par     = parallax( surfPos, surfPosPrev );
                    T       AOnSurf = spec_accum_speed( A, roughness, nv, par );

                    const V3< T > specOnSurf    = vmix( specPrevOnSurf, unfilteredSpec, (T)1 / ( (T)1 + AOnSurf ) );
                    const T       hitDistOnSurf = gmix( specHitDistancePrev, rayInfo.w, (T)1 / ( (T)1 + AOnSurf ) );

                    specColorAccum         = specOnSurf;
                    specHistoryLengthAccum = AOnSurf;
                    specHitDistanceAccum   = hitDistOnSurf;

                    const V3< T > rayDir     = { rayInfo.x, rayInfo.y, rayInfo.z };
                    const V3< T > virtualPos = surfPos + rayDir * hitDistOnSurf * spec_dominant( nv, roughness );

                    V2< int > pixPrevS;
                    V2< T >   subPixS;
                    {
                        V4< T > vp   = { virtualPos.x, virtualPos.y, virtualPos.z, (T)1 };
                        V4< T > vsc  = mat_mul( p.view, vp );
                        V4< T > vsp  = mat_mul( p.viewPrev, vp );
                        V4< T > csc  = mat_mul( p.projection, vsc );
                        V4< T > csp  = mat_mul( p.projectionPrev, vsp );
                        V3< T > ndcC = { csc.x / csc.w, csc.y / csc.w, csc.z / csc.w };
                        V3< T > ndcP = { csp.x / csp.w, csp.y / csp.w, csp.z / csp.w };
                        V2< T > ssC  = { ndcC.x * K( 0.5 ) + K( 0.5 ), ndcC.y * K( 0.5 ) + K( 0.5 ) };
                        V2< T > ssP  = { ndcP.x * K( 0.5 ) + K( 0.5 ), ndcP.y * K( 0.5 ) + K( 0.5 ) };
                        V2< T > specMotion = { ssP.x - ssC.x, ssP.y - ssC.y };
                        V2< T > spp = prev_screen_pos( specMotion, px, py );
                        T fx = o_floor( spp.x - K( 0.5 ) ), fy = o_floor( spp.y - K( 0.5 ) );
                        pixPrevS = { (int)fx, (int)fy };
                        subPixS  = { ( spp.x - K( 0.5 ) ) - fx, ( spp.y - K( 0.5 ) ) - fy };
                    }
                    const T bws[ 2 ][ 2 ] = {
                        { ( (T)1 - subPixS.x ) * ( (T)1 - subPixS.y ), subPixS.x * ( (T)1 - subPixS.y ) },
                        { ( (T)1 - subPixS.x ) * subPixS.y, subPixS.x * subPixS.y },
                    };
                    V3< T > specPrevVirtual  = { 0, 0, 0 };
                    T       weightSumVirtual = 0;
                    for( int yy = 0; yy <= 1; yy++ )
                        for( int xx = 0; xx <= 1; xx++ )
                        {
                            int     qx = pixPrevS.x + xx, qy = pixPrevS.y + yy;
                            T       dP = depthP.template fetch< T >( qx, qy ).x;
                            V3< T > nP = fetch_normal( nrmP, qx, qy );
                            bool ok = in_area( qx, qy, chArea ) && test_depth( z, dP, motionZ ) && test_normal( normal, nP );
                            if( ok )
                            {
                                const T w = bws[ yy ][ xx ];
                                specPrevVirtual  = specPrevVirtual + w * fetch3( specP, qx, qy );
                                weightSumVirtual = weightSumVirtual + w;
                            }
                        }
                    if( weightSumVirtual > K( 0.0001 ) )
                    {
                        specPrevVirtual = specPrevVirtual / weightSumVirtual;  // computed, unused (as in the shader)
                        T Avirt      = spec_accum_speed( A, roughness, nv, (T)0 );
                        T confidence = 1;
                        T Amin       = o_fmin( Avirt, K( 3.0 ) * o_sqrt( roughness ) );
                        T a          = gmix( (T)1 / ( (T)1 + Amin ), (T)1 / ( (T)1 + Avirt ), confidence );
                        Avirt        = (T)1 / a - (T)1;
                        T Ahitdist   = o_fmin( Avirt, K( 16.0 ) );
                        V3< T > specVirt = vmix( specPrevOnSurf, unfilteredSpec, (T)1 / ( (T)1 + Avirt ) );
                        T amount     = spec_dominant( nv, roughness );
                        a            = gmix( (T)1 / ( (T)1 + AOnSurf ), (T)1 / ( (T)1 + Avirt ), amount );
                        specColorAccum         = vmix( specOnSurf, specVirt, amount );
                        specHistoryLengthAccum = (T)1 / a - (T)1;
                        specHitDistanceAccum   = gmix( specHitDistancePrev, rayInfo.w, (T)1 / ( (T)1 + Ahitdist ) );
                    }
                }
                else
                {
                    specColorAccum         = unfilteredSpec;
                    specHistoryLengthAccum = 1;
                    specHitDistanceAccum   = rayInfo.w;
                }

                V3< T > diffColorAccum, indirAccum;
                V2< T > diffMomentsAccum;
                T       diffHL, indirHL;
                if( weightSum > K( 0.0001 ) )
                {
                    const T inv = (T)1 / weightSum;
                    diffPrev    = diffPrev * inv;
                    momentsPrev = { momentsPrev.x * inv, momentsPrev.y * inv };
                    indirPrev   = indirPrev * inv;
                    T dHL = histLenDIS.x * inv;
                    T iHL = histLenDIS.y * inv;
                    {
                        dHL = dHL * o_pow( (T)1 - aD, K( 10.0 ) );
                        dHL = gclamp( dHL + (T)1, (T)1, K( 256.0 ) );
                        T alphaColor   = o_fmax( K( 0.01 ), (T)1 / dHL );
                        T alphaMoments = o_fmax( K( 0.01 ), (T)1 / dHL );
                        alphaColor     = gmix( alphaColor, (T)1, aD );
                        alphaMoments   = gmix( alphaMoments, (T)1, aD );
                        diffColorAccum   = vmix( diffPrev, unfilteredDiff, alphaColor );
                        diffMomentsAccum = { gmix( momentsPrev.x, moments.x, alphaMoments ), gmix( momentsPrev.y, moments.y, alphaMoments ) };
                        diffHL = dHL;
                    }
                    {
                        iHL = iHL * o_pow( (T)1 - aI, K( 10.0 ) );
                        iHL = gclamp( iHL + (T)1, (T)1, K( 256.0 ) );
                        T alphaColor = o_fmax( K( 0.01 ), (T)1 / iHL );
                        alphaColor   = gmix( alphaColor, (T)1, aI );
                        indirAccum   = vmix( indirPrev, unfilteredIndir, alphaColor );
                        indirHL      = iHL;
                    }
                }
                else
                {
                    diffColorAccum   = unfilteredDiff;
                    diffMomentsAccum = moments;
                    diffHL           = 1;
                    indirAccum       = unfilteredIndir;
                    indirHL          = 1;
                }

                store3( C( RGDN_FB_DIFF_TEMPORARY ), px, py, diffColorAccum );
                C( RGDN_FB_DIFF_ACCUM_MOMENTS ).template store< T >( px, py, { diffMomentsAccum.x, diffMomentsAccum.y, 0, 0 } );
                C( RGDN_FB_ACCUM_HISTORY_LENGTH ).template store< T >( px, py, { diffHL, indirHL, specHistoryLengthAccum, specHitDistanceAccum } );
                store3( C( RGDN_FB_SPEC_ACCUM_COLOR ), px, py, specColorAccum );
                store3( C( RGDN_FB_INDIR_ACCUM ), px, py, indirAccum );
            }
        } );
    }

    // ---------------------------------------------------------------- CmAntiFirefly.comp:96-158
    void anti_firefly()
    {
        Plane& d   = C( RGDN_FB_DIFF_TEMPORARY );
        Plane& sp  = C( RGDN_FB_SPEC_ACCUM_COLOR );
        Plane& in  = C( RGDN_FB_INDIR_ACCUM );
        const T MAXF = K( 1000000.0 );
        parallel_rows( H(), nthreads, [ & ]( int py ) {
            for( int px = 0; px < W(); px++ )
            {
                V3< T > cd = fetch3( d, px, py ), cs = fetch3( sp, px, py ), ci = fetch3( in, px, py );
                if( p.antiFireflyEnabled != 0 )
                {
                    V3< T > mnD = { MAXF, MAXF, MAXF }, mnS = mnD, mnI = mnD;
                    V3< T > mxD = { -MAXF, -MAXF, -MAXF }, mxS = mxD, mxI = mxD;
                    for( int i = -2; i <= 2; i++ )
                        for( int j = -2; j <= 2; j++ )
                        {
                            if( i == 0 && j == 0 ) continue;
                            // GET_SDATA(i, j): i is the x offset, j the y offset
                            V3< T > od = fetch3( d, px + i, py + j ), os = fetch3( sp, px + i, py + j ), oi = fetch3( in, px + i, py + j );
                            mnD = vmin( mnD, od ); mnS = vmin( mnS, os ); mnI = vmin( mnI, oi );
                            mxD = vmax( mxD, od ); mxS = vmax( mxS, os ); mxI = vmax( mxI, oi );
                        }
                    cd = vclamp( cd, mnD, mxD );
                    cs = vclamp( cs, mnS, mxS );
                    ci = vclamp( ci, mnI, mxI );
                }
                store3( C( RGDN_FB_DIFF_ACCUM_COLOR ), px, py, cd );
                store3( C( RGDN_FB_SPEC_PING_COLOR ), px, py, cs );
                store3( C( RGDN_FB_INDIR_PING ), px, py, ci );
            }
        } );
    }

    // ---------------------------------------------------------------- CmSVGFEstimateVariance.comp:129-206
    void variance()
    {
        Plane& col   = C( RGDN_FB_DIFF_ACCUM_COLOR );
        Plane& nrm   = C( RGDN_FB_NORMAL );
        Plane& depth = C( RGDN_FB_DEPTH_WORLD );
        Plane& hlen  = C( RGDN_FB_ACCUM_HISTORY_LENGTH );
        Plane& mom   = C( RGDN_FB_DIFF_ACCUM_MOMENTS );
        const T THR  = K( 4.0 );
        parallel_rows( H(), nthreads, [ & ]( int py ) {
            for( int px = 0; px < W(); px++ )
            {
                const T       cz   = depth.template fetch< T >( px, py ).x;
                const uint32_t cn  = nrm.raw_u32( px, py );
                V3< T >       pc   = fetch3( col, px, py );
                if( cz < (T)0 || cz > (T)MAX_RAY_LENGTH )
                {
                    store_cv( RGDN_FB_DIFF_PING_COLOR_AND_VARIANCE, px, py, pc, (T)0 );
                    continue;
                }
                const T       histLen = hlen.template fetch< T >( px, py ).x;
                const V4< T > tm4     = mom.template fetch< T >( px, py );
                const V2< T > tm      = { tm4.x, tm4.y };
                if( histLen > THR )
                {
                    T tv = o_fmax( (T)0, tm.y - tm.x * tm.x );
                    tv   = tv / o_fmax( (T)1, histLen - THR );
                    store_cv( RGDN_FB_DIFF_PING_COLOR_AND_VARIANCE, px, py, pc, tv );
                    continue;
                }
                const T l  = luminance( pc );
                V2< T > sm = { l + tm.x, l * l + tm.y };
                T       ws = 1;
                const V3< T > cnd = decode_normal< T >( cn );
                for( int yy = -1; yy <= 1; yy++ )
                    for( int xx = -1; xx <= 1; xx++ )
                    {
                        if( xx == 0 && yy == 0 ) continue;
                        int qx = px + xx, qy = py + yy;
                        const V3< T > cq = fetch3( col, qx, qy );
                        const T       lq = luminance( cq );
                        const T       zq = depth.template fetch< T >( qx, qy ).x;
                        const T       mz = o_fmax( cz, zq );
                        const T       rcp = mz <= (T)0 ? (T)0 : (T)1 / mz;
                        const T wz = o_exp( -o_abs( cz - zq ) * rcp );
                        const T wn = o_pow( o_fmax( (T)0, dot3( cnd, decode_normal< T >( nrm.raw_u32( qx, qy ) ) ) ), K( 128.0 ) );
                        const T w  = wz * wn;
                        if( !std::isnan( w ) )
                        {
                            sm = { sm.x + lq * w, sm.y + lq * lq * w };
                            pc = pc + cq * w;
                            ws = ws + w;
                        }
                    }
                const T inv = ws <= (T)0 ? (T)0 : (T)1 / ws;
                sm = { sm.x * inv, sm.y * inv };
                pc = pc * inv;
                const T sv = o_fmax( (T)0, sm.y - sm.x * sm.x ) * ( (T)1 + (T)2 * ( (T)1 - histLen / THR ) );
                store_cv( RGDN_FB_DIFF_PING_COLOR_AND_VARIANCE, px, py, pc, sv );
            }
        } );
    }

    // ---------------------------------------------------------------- BRDF.h:27-29, 49-64
    static T spec_power( T alpha ) { return o_fmax( K( 0.01 ), K( 2.0 ) / ( alpha * alpha + K( 1e-4 ) ) - K( 2.0 ) ); }
    static V3< T > specular_color( V3< T > albedo, T metallic )
    {
        V3< T > mn = { K( 0.04 ), K( 0.04 ), K( 0.04 ) };
        return vmix( mn, albedo, metallic );
    }
    static T material_ambient( V3< T > albedo )
    {
        T l = luminance( albedo );
        T q = ( l - K( 0.02 ) ) / K( 0.02 );
        return l > K( 0.02 ) ? (T)1 : (T)1 - q * q;
    }

    // ---------------------------------------------------------------- CmSVGFAtrous_Iter0.comp / CmSVGFAtrous.comp
    void atrous( uint32_t iter, uint32_t niter )
    {
        // routing (CmSVGFAtrous.comp:237-276, generalised to niter iterations)
        uint32_t diffSrc, specSrc, indirSrc, diffDst = 0, specDst = 0, indirDst = 0;
        if( iter == 0 )
        {
            diffSrc = RGDN_FB_DIFF_PING_COLOR_AND_VARIANCE; specSrc = RGDN_FB_SPEC_PING_COLOR; indirSrc = RGDN_FB_INDIR_PING;
            diffDst = RGDN_FB_DIFF_COLOR_HISTORY; specDst = RGDN_FB_SPEC_PONG_COLOR; indirDst = RGDN_FB_INDIR_PONG;
        }
        else
        {
            diffSrc  = iter == 1 ? RGDN_FB_DIFF_COLOR_HISTORY : ( iter % 2 == 0 ? RGDN_FB_DIFF_PING_COLOR_AND_VARIANCE : RGDN_FB_DIFF_PONG_COLOR_AND_VARIANCE );
            specSrc  = iter % 2 == 1 ? RGDN_FB_SPEC_PONG_COLOR : RGDN_FB_SPEC_PING_COLOR;
            indirSrc = iter % 2 == 1 ? RGDN_FB_INDIR_PONG : RGDN_FB_INDIR_PING;
            diffDst  = iter % 2 == 1 ? RGDN_FB_DIFF_PING_COLOR_AND_VARIANCE : RGDN_FB_DIFF_PONG_COLOR_AND_VARIANCE;
            specDst  = iter % 2 == 1 ? RGDN_FB_SPEC_PING_COLOR : RGDN_FB_SPEC_PONG_COLOR;
            indirDst = iter % 2 == 1 ? RGDN_FB_INDIR_PING : RGDN_FB_INDIR_PONG;
        }
        const bool last = iter + 1 == niter;
        const int  step = 1 << iter;
        const T    kern[ 2 ][ 2 ] = { { K( 1.0 ), K( 0.5 ) }, { K( 0.5 ), K( 0.25 ) } };

        Plane& depth = C( RGDN_FB_DEPTH_WORLD );
        Plane& dgrad = C( RGDN_FB_DEPTH_GRAD );
        Plane& mr    = C( RGDN_FB_METALLIC_ROUGHNESS );
        Plane& nrm   = C( RGDN_FB_NORMAL );
        Plane& hlen  = C( RGDN_FB_ACCUM_HISTORY_LENGTH );
        Plane& specS = C( specSrc );
        Plane& indS  = C( indirSrc );
        Plane& fvar  = C( RGDN_FB_ATROUS_FILTERED_VARIANCE );

        parallel_rows( H(), nthreads, [ & ]( int py ) {
            for( int px = 0; px < W(); px++ )
            {
                const Area chArea = cb_area( px, py );
                V4< T >    cv     = fetch_cv( diffSrc, px, py );
                V3< T >    outDiff = xyz( cv );
                T          outVar  = cv.w;
                V3< T >    outSpec = fetch3( specS, px, py );
                V3< T >    outInd  = fetch3( indS, px, py );
                const T    z       = depth.template fetch< T >( px, py ).x;
                const T    gradDepth = dgrad.template fetch< T >( px, py ).x;

                if( z < (T)0 || z > (T)MAX_RAY_LENGTH )
                {
                    if( iter == 0 )
                    {
                        // CmSVGFAtrous_Iter0.comp:208-216: zeros; the prefiltered variance is not written
                        outDiff = { 0, 0, 0 }; outVar = 0; outSpec = { 0, 0, 0 }; outInd = { 0, 0, 0 };
                    }
                    // iterations >= 1 pass the inputs through (CmSVGFAtrous.comp:96-99)
                }
                else
                {
                    const V3< T > normal = fetch_normal( nrm, px, py );
                    const T       l      = luminance( outDiff );
                    T             prefVar;
                    if( iter == 0 )
                    {
                        // prefilterLuminanceVariance (CmSVGFAtrous_Iter0.comp:158-187)
                        const T g[ 2 ][ 2 ] = { { K( 0.25 ), K( 0.125 ) }, { K( 0.125 ), K( 0.0625 ) } };
                        T r = 0;
                        for( int yy = -1; yy <= 1; yy++ )
                            for( int xx = -1; xx <= 1; xx++ )
                                r = r + fetch_cv( diffSrc, px + xx, py + yy ).w * g[ std::abs( xx ) ][ std::abs( yy ) ];
                        r = o_sqrt( o_fmax( r, (T)0 ) );
                        fvar.template store< T >( px, py, { r, 0, 0, 0 } );
                        prefVar = r;
                    }
                    else prefVar = fvar.template fetch< T >( px, py ).x;

                    const T wLumMul = (T)1 / ( K( 4.0 ) * prefVar + K( 0.00001 ) );
                    const V4< T > mrc = mr.template fetch< T >( px, py );
                    const T roughness = mrc.y;
                    const T wRoughMul = gclamp( roughness * K( 30.0 ) - (T)iter, (T)0, (T)1 );
                    const T hS  = hlen.template fetch< T >( px, py ).z;
                    const T nws = gclamp( hS / K( 8.0 ), (T)0, (T)1 );
                    T nwSpec = spec_power( roughness * roughness );
                    nwSpec   = gclamp( nwSpec, K( 8.0 ), K( 1024.0 ) );
                    nwSpec   = nwSpec * nws;

                    T ws = 1, wsS = 1, wsI = 1;
                    for( int yy = -1; yy <= 1; yy++ )
                        for( int xx = -1; xx <= 1; xx++ )
                        {
                            if( xx == 0 && yy == 0 ) continue;
                            const int qx = px + xx * step, qy = py + yy * step;
                            const T       rq  = mr.template fetch< T >( qx, qy ).y;
                            const V3< T > nq  = fetch_normal( nrm, qx, qy );
                            const T       zq  = depth.template fetch< T >( qx, qy ).x;
                            const V3< T > sq  = fetch3( specS, qx, qy );
                            const V4< T > cvq = fetch_cv( diffSrc, qx, qy );
                            const V3< T > dq  = xyz( cvq );
                            const T       vq  = cvq.w;
                            const T       lq  = luminance( dq );
                            const T       nn  = o_fmax( (T)0, dot3( normal, nq ) );
                            const V3< T > iq  = fetch3( indS, qx, qy );

                            const T w_z = o_abs( z - zq ) / o_fmax( gradDepth * (T)( std::abs( xx ) + std::abs( yy ) ), K( 0.01 ) );
                            const T w_n = o_pow( nn, K( 128.0 ) );
                            const T w_l = o_abs( l - lq ) * wLumMul;
                            T w_r = o_fmax( (T)0, (T)1 - K( 10.0 ) * o_abs( roughness - rq ) ) * wRoughMul;
                            if( nwSpec > (T)0 ) w_r = w_r * o_pow( nn, nwSpec );
                            const T waveletW = kern[ std::abs( yy ) ][ std::abs( xx ) ];
                            const T inside   = in_area( qx, qy, chArea ) ? (T)1 : (T)0;
                            const T wBase    = o_exp( -w_z * w_z ) * w_n * waveletW * inside;
                            const T wDiff    = wBase * o_exp( -w_l );
                            const T wSpec    = wBase * w_r;
                            const T wInd     = wBase;

                            outDiff = outDiff + dq * wDiff;
                            outSpec = outSpec + sq * wSpec;
                            outInd  = outInd + iq * wInd;
                            outVar  = outVar + vq * wDiff * wDiff;
                            ws  = ws + wDiff;
                            wsS = wsS + wSpec;
                            wsI = wsI + wInd;
                        }
                    const T inv = (T)1 / ws, invS = (T)1 / wsS, invI = (T)1 / wsI;
                    outDiff = outDiff * inv;
                    outVar  = outVar * ( inv * inv );   // outVariance *= invWeightSum * invWeightSum
                    outSpec = outSpec * invS;
                    outInd  = outInd * invI;
                }

                if( !last )
                {
                    store_cv( diffDst, px, py, outDiff, outVar );
                    store3( C( specDst ), px, py, outSpec );
                    store3( C( indirDst ), px, py, outInd );
                }
                else compose( px, py, outDiff, outSpec, outInd );
            }
        } );
    }

    // ---------------------------------------------------------------- CmSVGFAtrous.comp:278-348
    void compose( int px, int py, V3< T > filteredDiff, V3< T > filteredSpec, V3< T > filteredIndir )
    {
        V2< int > rp = regular_from_cb( px, py );
        V3< T > albedo     = fetch3( C( RGDN_FB_ALBEDO ), rp.x, rp.y );
        V3< T > throughput = fetch3( C( RGDN_FB_THROUGHPUT ), px, py );
        if( p.debugShowFlags & RGDN_DEBUG_SHOW_FLAG_ALBEDO_WHITE ) albedo = { 1, 1, 1 };
        V3< T > ill;
        if( C( RGDN_FB_IS_SKY ).raw_u8( px, py ) == 0 )
        {
            V4< T > mrFb = C( RGDN_FB_METALLIC_ROUGHNESS ).template fetch< T >( px, py );
            T metallic = mrFb.x, roughness = mrFb.y;
            V3< T > diffuse = filteredDiff, indirect = filteredIndir;
            V3< T > specular = vmix( filteredSpec, indirect, gsmoothstep( K( 0.5 ), K( 0.5 ) + K( 0.25 ), roughness ) );
            V3< T > ro_s = specular_color( albedo, metallic );
            V3< T > ro_d = albedo * ( (T)1 - metallic );
            ill = ( diffuse + indirect ) * ro_d + specular * ro_s;
            if( p.debugShowFlags & RGDN_DEBUG_SHOW_FLAG_ONLY_DIRECT_DIFFUSE ) ill = diffuse * albedo;
            else if( p.debugShowFlags & RGDN_DEBUG_SHOW_FLAG_ONLY_SPECULAR ) ill = specular * specular_color( albedo, metallic );
            else if( p.debugShowFlags & RGDN_DEBUG_SHOW_FLAG_ONLY_INDIRECT_DIFFUSE ) ill = indirect;
            ill = ill * throughput;
            ill = ill * material_ambient( albedo );
        }
        else ill = albedo * throughput;

        C( RGDN_FB_HISTOGRAM_INPUT ).template store< T >( rp.x, rp.y, { o_fmax( (T)0, luminance( ill ) ), 0, 0, 0 } );
        // classicShading (ShaderCommonGLSLFunc.h:492-495)
        if( (float)rp.x < p.lightmapScreenCoverage * RW() ) ill = albedo * throughput;
        V3< T > z0 = { 0, 0, 0 };
        V3< T > o  = vmax( z0, ill );
        C( RGDN_FB_PRE_FINAL ).template store< T >( rp.x, rp.y, { o.x, o.y, o.z, (T)0 } );
    }

    // ---------------------------------------------------------------- CmLuminanceHistogram.comp:60-86
    void histogram()
    {
        Plane& hin = C( RGDN_FB_HISTOGRAM_INPUT );
        // per-row histograms summed in row order (integer sums are order-independent)
        std::vector< std::vector< uint32_t > > rows( H(), std::vector< uint32_t >( 256, 0 ) );
        parallel_rows( H(), nthreads, [ & ]( int py ) {
            for( int px = 0; px < W(); px++ )
            {
                uint16_t h; memcpy( &h, hin.at( px, py ), 2 );
                rows[ py ][ color_bin( f16_to_f32( h ), p.minLogLuminance, p.maxLogLuminance ) ]++;
            }
        } );
        for( int y = 0; y < H(); y++ )
            for( int b = 0; b < 256; b++ ) s.hist[ b ] += rows[ y ][ b ];
    }

    // ---------------------------------------------------------------- CmLuminanceAvg.comp:39-89
    void luminance_avg()
    {
        uint32_t sum = 0;
        for( uint32_t i = 0; i < 256; i++ ) sum += s.hist[ i ] * i;
        const uint32_t count0 = s.hist[ 0 ];
        for( int i = 0; i < 256; i++ ) s.hist[ i ] = 0;
        if( p.stopEyeAdaptation != 0 ) return;
        if constexpr( std::is_same< T, float >::value )
        {
            float minL = p.minLogLuminance, maxL = p.maxLogLuminance;
            float range      = maxL - minL;
            float pixelCount = RW() * RH();
            float black      = (float)count0;
            float wla        = ( (float)sum / o_fmax( pixelCount - black, 1.0f ) ) - 1.0f;
            float wal        = (float)exp2( (double)( wla / 254.0f * range + minL ) );
            float last       = (float)s.avgLum;
            float t          = 1.0f - (float)exp( (double)( -p.timeDelta * 1.1f ) );
            float adapted    = last + ( wal - last ) * t;
            s.avgLum         = o_fmin( adapted, (float)exp2( (double)maxL ) );
        }
        else
        {
            double minL = p.minLogLuminance, maxL = p.maxLogLuminance;
            double range = maxL - minL;
            double pixelCount = RW() * (double)RH();
            double wla   = ( (double)sum / fmax( pixelCount - (double)count0, 1.0 ) ) - 1.0;
            double wal   = exp2( wla / 254.0 * range + minL );
            double t     = 1.0 - exp( -(double)p.timeDelta * 1.1 );
            double adapt = s.avgLum + ( wal - s.avgLum ) * t;
            s.avgLum     = fmin( adapt, exp2( maxL ) );
        }
    }
};


// ============================================================================================
//  Exposure application and tonemapping: CmCheckerboard.comp:27-69 + CmPrepareFinal.comp:57-187
// ============================================================================================

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
// AMD FidelityFX LPM 1.0 (vendored as Shaders/LPM/ffx_lpm.h), the 709 -> 709 configuration
// without shoulder tuning that ImageComposition uses. Setup: LpmSetupCustom.inl:40-70;
// LpmColRgbToXyz / LpmMatInv3x3 (ffx_lpm.h:157-210) for the luma coefficients. Filter:
// LpmMap (ffx_lpm.h:727-812) with con, soft, con2, clip, scaleOnly and shoulder all false.
template< class T > struct Lpm
{
    T saturation[ 3 ], contrast, tsb[ 2 ], lumaT[ 3 ], rcpLumaT[ 3 ], crosstalk[ 3 ];
};

template< class T > Lpm< T > lpm_setup( const float sat[ 3 ], const float ct[ 3 ] )
{
    Lpm< T > L;
    const T hdrMax = (T)256, exposure = (T)8, shoulderContrast = (T)1;
    T       contrast = K( 0.1 ) + (T)1;
    for( int k = 0; k < 3; k++ ) L.saturation[ k ] = (T)sat[ k ] + contrast;
    L.contrast     = contrast;
    const T midIn  = hdrMax * K( 0.18 ) * o_exp2( -exposure );
    const T midOut = K( 0.18 );
    const T cs     = contrast * shoulderContrast;
    const T z0     = -o_pow( midIn, contrast );
    const T z1     = o_pow( hdrMax, cs ) * o_pow( midIn, contrast );
    const T z2     = o_pow( hdrMax, contrast ) * o_pow( midIn, cs ) * midOut;
    const T z3     = o_pow( hdrMax, cs ) * midOut;
    const T z4     = o_pow( midIn, cs ) * midOut;
    L.tsb[ 0 ]     = -( ( z0 + ( midOut * ( z1 - z2 ) ) * ( (T)1 / ( z3 - z4 ) ) ) * ( (T)1 / z4 ) );
    const T w0     = o_pow( hdrMax, cs ) * o_pow( midIn, contrast );
    const T w1     = o_pow( hdrMax, contrast ) * o_pow( midIn, cs ) * midOut;
    const T w2     = o_pow( hdrMax, cs ) * midOut;
    const T w3     = o_pow( midIn, cs ) * midOut;
    L.tsb[ 1 ]     = ( w0 - w1 ) * ( (T)1 / ( w2 - w3 ) );
    // RGB -> XYZ of the 709 primaries and the D65 white: the primaries' xyz as columns, scaled
    // per primary by inverse(columns) . white XYZ (Y = 1); the Y row gives the luma weights
    const T xy[ 3 ][ 2 ] = { { K( 0.64 ), K( 0.33 ) }, { K( 0.30 ), K( 0.60 ) }, { K( 0.15 ), K( 0.06 ) } };
    const T wxy[ 2 ]     = { K( 0.3127 ), K( 0.3290 ) };
    T       m[ 3 ][ 3 ];   // m[row][primary]
    for( int c = 0; c < 3; c++ )
    {
        m[ 0 ][ c ] = xy[ c ][ 0 ];
        m[ 1 ][ c ] = xy[ c ][ 1 ];
        m[ 2 ][ c ] = (T)1 - ( xy[ c ][ 0 ] + xy[ c ][ 1 ] );
    }
    const T wr = (T)1 / wxy[ 1 ];
    const T w[ 3 ] = { wxy[ 0 ] * wr, wxy[ 1 ] * wr, ( (T)1 - ( wxy[ 0 ] + wxy[ 1 ] ) ) * wr };
    // inverse by cofactors
    const T det = m[ 0 ][ 0 ] * ( m[ 1 ][ 1 ] * m[ 2 ][ 2 ] - m[ 2 ][ 1 ] * m[ 1 ][ 2 ] ) - m[ 0 ][ 1 ] * ( m[ 1 ][ 0 ] * m[ 2 ][ 2 ] - m[ 1 ][ 2 ] * m[ 2 ][ 0 ] ) +
                  m[ 0 ][ 2 ] * ( m[ 1 ][ 0 ] * m[ 2 ][ 1 ] - m[ 1 ][ 1 ] * m[ 2 ][ 0 ] );
    const T id = (T)1 / det;
    T inv[ 3 ][ 3 ];
    inv[ 0 ][ 0 ] = ( m[ 1 ][ 1 ] * m[ 2 ][ 2 ] - m[ 2 ][ 1 ] * m[ 1 ][ 2 ] ) * id;
    inv[ 0 ][ 1 ] = ( m[ 0 ][ 2 ] * m[ 2 ][ 1 ] - m[ 0 ][ 1 ] * m[ 2 ][ 2 ] ) * id;
    inv[ 0 ][ 2 ] = ( m[ 0 ][ 1 ] * m[ 1 ][ 2 ] - m[ 0 ][ 2 ] * m[ 1 ][ 1 ] ) * id;
    inv[ 1 ][ 0 ] = ( m[ 1 ][ 2 ] * m[ 2 ][ 0 ] - m[ 1 ][ 0 ] * m[ 2 ][ 2 ] ) * id;
    inv[ 1 ][ 1 ] = ( m[ 0 ][ 0 ] * m[ 2 ][ 2 ] - m[ 0 ][ 2 ] * m[ 2 ][ 0 ] ) * id;
    inv[ 1 ][ 2 ] = ( m[ 1 ][ 0 ] * m[ 0 ][ 2 ] - m[ 0 ][ 0 ] * m[ 1 ][ 2 ] ) * id;
    inv[ 2 ][ 0 ] = ( m[ 1 ][ 0 ] * m[ 2 ][ 1 ] - m[ 2 ][ 0 ] * m[ 1 ][ 1 ] ) * id;
    inv[ 2 ][ 1 ] = ( m[ 2 ][ 0 ] * m[ 0 ][ 1 ] - m[ 0 ][ 0 ] * m[ 2 ][ 1 ] ) * id;
    inv[ 2 ][ 2 ] = ( m[ 0 ][ 0 ] * m[ 1 ][ 1 ] - m[ 1 ][ 0 ] * m[ 0 ][ 1 ] ) * id;
    T y[ 3 ];
    for( int c = 0; c < 3; c++ )
    {
        const T sc = inv[ c ][ 0 ] * w[ 0 ] + inv[ c ][ 1 ] * w[ 1 ] + inv[ c ][ 2 ] * w[ 2 ];
        y[ c ]     = m[ 1 ][ c ] * sc;
    }
    const T rs = (T)1 / ( y[ 0 ] + y[ 1 ] + y[ 2 ] );
    for( int k = 0; k < 3; k++ )
    {
        L.lumaT[ k ]     = y[ k ] * rs;
        L.rcpLumaT[ k ]  = (T)1 / L.lumaT[ k ];
        L.crosstalk[ k ] = (T)ct[ k ];
    }
    return L;
}

template< class T > V3< T > lpm_filter( V3< T > c, const Lpm< T >& L )
{
    const T rcpMax = (T)1 / o_fmax( c.x, o_fmax( c.y, c.z ) );
    T       rR = c.x * rcpMax, rG = c.y * rcpMax, rB = c.z * rcpMax;
    rR = o_pow( rR, L.saturation[ 0 ] );
    rG = o_pow( rG, L.saturation[ 1 ] );
    rB = o_pow( rB, L.saturation[ 2 ] );
    T luma = c.y * L.lumaT[ 1 ] + ( c.x * L.lumaT[ 0 ] + ( c.z * L.lumaT[ 2 ] ) );
    luma   = o_pow( luma, L.contrast );
    luma   = luma * ( (T)1 / ( luma * L.tsb[ 0 ] + L.tsb[ 1 ] ) );
    const T lumaRatio  = rR * L.lumaT[ 0 ] + rG * L.lumaT[ 1 ] + rB * L.lumaT[ 2 ];
    const T ratioScale = gsat( luma * ( (T)1 / lumaRatio ) );
    T       cR = gsat( rR * ratioScale ), cG = gsat( rG * ratioScale ), cB = gsat( rB * ratioScale );
    const T capR = -L.crosstalk[ 0 ] * cR + L.crosstalk[ 0 ];
    const T capG = -L.crosstalk[ 1 ] * cG + L.crosstalk[ 1 ];
    const T capB = -L.crosstalk[ 2 ] * cB + L.crosstalk[ 2 ];
    T lumaAdd = gsat( ( -cB ) * L.lumaT[ 2 ] + ( ( -cR ) * L.lumaT[ 0 ] + ( ( -cG ) * L.lumaT[ 1 ] + luma ) ) );
    const T t = lumaAdd * ( (T)1 / ( capG * L.lumaT[ 1 ] + ( capR * L.lumaT[ 0 ] + ( capB * L.lumaT[ 2 ] ) ) ) );
    cR      = gsat( t * capR + cR );
    cG      = gsat( t * capG + cG );
    cB      = gsat( t * capB + cB );
    lumaAdd = gsat( ( -cB ) * L.lumaT[ 2 ] + ( ( -cR ) * L.lumaT[ 0 ] + ( ( -cG ) * L.lumaT[ 1 ] + luma ) ) );
    cR      = gsat( lumaAdd * L.rcpLumaT[ 0 ] + cR );
    cG      = gsat( lumaAdd * L.rcpLumaT[ 1 ] + cG );
    cB      = gsat( lumaAdd * L.rcpLumaT[ 2 ] + cB );
    return { cR, cG, cB };
}

// uncharted2TonemapOp (CmPrepareFinal.comp:69-80)
template< class T > T u2_op( T x )
{
    const T A = K( 0.15 ), B = K( 0.50 ), C = K( 0.10 ), D = K( 0.20 ), E = K( 0.02 ), F = K( 0.30 );
    return ( ( x * ( A * x + C * B ) + D * E ) / ( x * ( A * x + B ) + D * F ) ) - E / F;
}

template< class T > void prepare_final( Stream& s, uint32_t fi, const rgdn_final_params& p, int nthreads )
{
    const Lpm< T > L     = lpm_setup< T >( p.saturation, p.crosstalk );
    const int      W     = s.W, H = s.H, sep = W / 2;
    Plane&         pre   = s.cur( RGDN_FB_PRE_FINAL, fi );
    Plane&         emisP = s.cur( RGDN_FB_SCREEN_EMIS_RT, fi );
    Plane&         scat  = s.cur( RGDN_FB_SCATTERING, fi );
    Plane&         thr   = s.cur( RGDN_FB_THROUGHPUT, fi );
    Plane&         outF  = s.cur( RGDN_FB_FINAL, fi );
    Plane&         outB  = s.cur( RGDN_FB_BLOOM_INPUT, fi );
    // getAutoEV100 / ev100ToLuminousExposure (Exposure.h:14-51); the tonemapping SSBO holds a float
    const T avg      = (T)( std::is_same< T, float >::value ? (double)(float)s.avgLum : s.avgLum );
    const T ev       = o_log2( o_fmax( (T)0, avg ) * (T)100 / K( 12.5 ) );
    const T maxLum   = K( 1.2 ) * o_exp2( ev );
    const T exposure = maxLum > (T)0 ? (T)1 / maxLum : (T)0;
    const T quarter  = K( 0.25 );
    auto resolve = [ & ]( Plane& src, int x, int y, int cbx, V3< T > c ) {
        const T lf = ( cbx == 0 || cbx == sep ) ? (T)0 : (T)1;
        const T rf = ( cbx == sep || cbx == W ) ? (T)0 : (T)1;
        const V3< T > l = xyz( src.fetch< T >( x - 1, y ) ), r = xyz( src.fetch< T >( x + 1, y ) );
        const V3< T > d = xyz( src.fetch< T >( x, y + 1 ) ), u = xyz( src.fetch< T >( x, y - 1 ) );
        const V3< T > cross = { quarter * l.x * lf + quarter * r.x * rf + quarter * d.x + quarter * u.x,
                                quarter * l.y * lf + quarter * r.y * rf + quarter * d.y + quarter * u.y,
                                quarter * l.z * lf + quarter * r.z * rf + quarter * d.z + quarter * u.z };
        return vmix( c, cross, K( 0.5 ) );
    };
    parallel_rows( H, nthreads, [ & ]( int y ) {
        for( int x = 0; x < W; x++ )
        {
            const int cbx  = ( ( x + y % 2 ) % 2 ) * sep + x / 2;   // getCheckerboardPix
            V3< T >   hdr  = xyz( pre.fetch< T >( x, y ) );
            V3< T >   emis = xyz( emisP.fetch< T >( x, y ) );
            if( thr.fetch< T >( cbx, y ).w > K( 0.5 ) )   // wasSplit
            {
                // CmCheckerboard stores the resolved values into Final (PreFinal's format) and
                // ScreenEmission (ScreenEmisRT's format), and CmPrepareFinal reads them back
                // (CmCheckerboard.comp:66-76, CmPrepareFinal.comp:147-150)
                hdr  = outF.requant< T >( resolve( pre, x, y, cbx, hdr ) );
                emis = emisP.requant< T >( resolve( emisP, x, y, cbx, emis ) );
            }
            if( p.flags & RGDN_FINAL_APPLY_SCATTERING )
            {
                const V4< T > v = scat.fetch< T >( x, y );
                hdr             = { hdr.x * v.w + v.x, hdr.y * v.w + v.y, hdr.z * v.w + v.z };
            }
            V3< T > color;
            if( (T)x < (T)p.lightmapScreenCoverage * (T)W )   // classicShading
            {
                const T w = u2_op< T >( (T)p.luminanceWhitePoint );
                color     = { u2_op< T >( (T)2 * hdr.x ) / w, u2_op< T >( (T)2 * hdr.y ) / w, u2_op< T >( (T)2 * hdr.z ) / w };
            }
            else
            {
                const T em = (T)p.emissionMaxScreenColor;
                color      = lpm_filter< T >( { hdr.x * exposure + emis.x * em, hdr.y * exposure + emis.y * em, hdr.z * exposure + emis.z * em }, L );
            }
            const T el    = o_exp2( ev + (T)p.bloomEmissionMultiplier - (T)3 );
            V3< T > bloom = { ( hdr.x + emis.x * el ) * exposure, ( hdr.y + emis.y * el ) * exposure, ( hdr.z + emis.z * el ) * exposure };
            if( std::isnan( bloom.x ) || std::isnan( bloom.y ) || std::isnan( bloom.z ) || std::isinf( bloom.x ) || std::isinf( bloom.y ) ||
                std::isinf( bloom.z ) )
                bloom = { 0, 0, 0 };
            bloom = bloom * gsmoothstep( (T)0, (T)p.bloomThreshold, luminance( bloom ) );
            outF.store< T >( x, y, { color.x, color.y, color.z, (T)0 } );
            outB.store< T >( x, y, { bloom.x, bloom.y, bloom.z, (T)0 } );
        }
    } );
}

// --------------------------------------------------------------------------------------------
//  Bloom: CmBloomDownsample.comp:15-136, CmBloomUpsample.comp:15-104, CmBloomApply.comp:45-76
//  (without the lens-dirt texture term). textureLod through the framebuffers' bilinear
//  clamp-to-edge sampler (Framebuffers.cpp:187-209), evaluated exactly in T.
// --------------------------------------------------------------------------------------------
template< class T > V3< T > bilinear( const Plane& img, T u, T v )
{
    const T   x  = u * (T)img.w - K( 0.5 ), y = v * (T)img.h - K( 0.5 );
    const T   fx = o_floor( x ), fy = o_floor( y );
    const T   a  = x - fx, b = y - fy;
    const int ix = (int)fx, iy = (int)fy;
    const int x0 = std::min( std::max( ix, 0 ), img.w - 1 ), x1 = std::min( std::max( ix + 1, 0 ), img.w - 1 );
    const int y0 = std::min( std::max( iy, 0 ), img.h - 1 ), y1 = std::min( std::max( iy + 1, 0 ), img.h - 1 );
    const V3< T > t00 = xyz( img.fetch< T >( x0, y0 ) ), t10 = xyz( img.fetch< T >( x1, y0 ) );
    const V3< T > t01 = xyz( img.fetch< T >( x0, y1 ) ), t11 = xyz( img.fetch< T >( x1, y1 ) );
    return vmix( vmix( t00, t10, a ), vmix( t01, t11, a ), b );
}

template< class T > void bloom( Stream& s, uint32_t fi, float intensity )
{
    const int W = s.W, H = s.H;
    auto      mip = [ & ]( int k ) -> Plane& { return s.cur( k == 0 ? RGDN_FB_BLOOM_INPUT : RGDN_FB_BLOOM_MIP1 + ( k - 1 ), fi ); };
    const T   q = K( 0.25 ), h2 = K( 0.5 ), e8 = K( 0.125 );
    for( int k = 0; k < 8; k++ )
    {
        const Plane& src = mip( k );
        Plane&       dst = mip( k + 1 );
        const T      idx = (T)( 1 << ( k + 1 ) ) / (T)W, idy = (T)( 1 << ( k + 1 ) ) / (T)H;
        const T      isx = (T)( 1 << k ) / (T)W, isy = (T)( 1 << k ) / (T)H;
        for( int y = 0; y < dst.h; y++ )
            for( int x = 0; x < dst.w; x++ )
            {
                const T u = ( (T)x + h2 ) * idx, v = ( (T)y + h2 ) * idy;
                if( u > (T)1 || v > (T)1 ) continue;
                auto tap = [ & ]( T ox, T oy ) { return bilinear< T >( src, u + ox * isx, v + oy * isy ); };
                const V3< T > t0 = tap( -2, -2 ), t1 = tap( 0, -2 ), t2 = tap( 2, -2 ), t3 = tap( -1, -1 ), t4 = tap( 1, -1 );
                const V3< T > t5 = tap( -2, 0 ), t6 = tap( 0, 0 ), t7 = tap( 2, 0 ), t8 = tap( -1, 1 ), t9 = tap( 1, 1 );
                const V3< T > t10 = tap( -2, 2 ), t11 = tap( 0, 2 ), t12 = tap( 2, 2 );
                const V3< T > b0 = ( t3 + t4 + t8 + t9 ) * q, b1 = ( t0 + t1 + t5 + t6 ) * q, b2 = ( t1 + t2 + t6 + t7 ) * q;
                const V3< T > b3 = ( t5 + t6 + t10 + t11 ) * q, b4 = ( t6 + t7 + t11 + t12 ) * q;
                V3< T >       r;
                if( k == 0 )
                {
                    auto kw = []( V3< T > bx ) { return (T)1 / ( (T)1 + luminance( bx ) ); };   // getKarisWeight
                    r       = b0 * ( h2 * kw( b0 ) ) + b1 * ( e8 * kw( b1 ) ) + b2 * ( e8 * kw( b2 ) ) + b3 * ( e8 * kw( b3 ) ) + b4 * ( e8 * kw( b4 ) );
                }
                else r = b0 * h2 + b1 * e8 + b2 * e8 + b3 * e8 + b4 * e8;
                dst.store< T >( x, y, { r.x, r.y, r.z, (T)0 } );
            }
    }
    const T wt[ 3 ][ 3 ] = { { K( 0.0625 ), K( 0.125 ), K( 0.0625 ) }, { K( 0.125 ), K( 0.25 ), K( 0.125 ) }, { K( 0.0625 ), K( 0.125 ), K( 0.0625 ) } };
    for( int k = 7; k >= 0; k-- )
    {
        const Plane& src = mip( k + 1 );
        Plane&       dst = k == 0 ? s.cur( RGDN_FB_BLOOM_RESULT, fi ) : mip( k );
        const T      isx = (T)( 1 << ( k + 1 ) ) / (T)W, isy = (T)( 1 << ( k + 1 ) ) / (T)H;
        const T      iux = (T)( 1 << k ) / (T)W, iuy = (T)( 1 << k ) / (T)H;
        for( int y = 0; y < dst.h; y++ )
            for( int x = 0; x < dst.w; x++ )
            {
                const T u = ( (T)x + h2 ) * iux + h2 * isx, v = ( (T)y + h2 ) * iuy + h2 * isy;
                if( u > (T)1 || v > (T)1 ) continue;
                V3< T > r = { 0, 0, 0 };
                for( int oy = -1; oy <= 1; oy++ )
                    for( int ox = -1; ox <= 1; ox++ ) r = r + bilinear< T >( src, u + (T)ox * isx, v + (T)oy * isy ) * wt[ oy + 1 ][ ox + 1 ];
                if( k > 0 ) r = r + xyz( dst.fetch< T >( x, y ) );
                dst.store< T >( x, y, { r.x, r.y, r.z, (T)0 } );
            }
    }
    const Plane& res = s.cur( RGDN_FB_BLOOM_RESULT, fi );
    Plane&       fin = s.cur( RGDN_FB_FINAL, fi );
    for( int y = 0; y < H; y++ )
        for( int x = 0; x < W; x++ )
        {
            const T u = ( (T)x + h2 ) * ( (T)1 / (T)W ), v = ( (T)y + h2 ) * ( (T)1 / (T)H );
            if( u > (T)1 || v > (T)1 ) continue;
            const V3< T > c = xyz( fin.fetch< T >( x, y ) ) + bilinear< T >( res, u, v ) * (T)intensity;
            fin.store< T >( x, y, { c.x, c.y, c.z, (T)0 } );
        }
}

// --------------------------------------------------------------------------------------------
//  Volumetric::ProcessScattering (Volumetric.cpp:71-190)
// --------------------------------------------------------------------------------------------
// CmVolumetricProcess.comp:38-79: each froxel column integrated front to back in place; the
// running (light, extinction) in T, cell z storing (light, exp(-extinction))
template< class T > void volume_process( Stream& s, uint32_t fi )
{
    Plane&    vol = s.cur( RGDN_FB_SCATTER_VOLUME, fi );
    const int nx = RGDN_VOLUME_SIZE_X, ny = RGDN_VOLUME_SIZE_Y, nz = RGDN_VOLUME_SIZE_Z;
    for( int y = 0; y < ny; y++ )
        for( int x = 0; x < nx; x++ )
        {
            V4< T > acc = vol.fetch< T >( x, y );
            T       e   = o_exp( -acc.w );
            vol.store< T >( x, y, { acc.x, acc.y, acc.z, e } );
            for( int z = 1; z < nz; z++ )
            {
                const V4< T > v = vol.fetch< T >( x, z * ny + y );
                const T       t = gsat( e );   // saturate( exp( -front.a ) )
                acc             = { acc.x + t * v.x, acc.y + t * v.y, acc.z + t * v.z, acc.w + v.w };
                e               = o_exp( -acc.w );
                vol.store< T >( x, z * ny + y, { acc.x, acc.y, acc.z, e } );
            }
        }
}

// Random.h:243-251 wellonsLowBias32, 280-287 murmurHash33, 202-208 + 289-300 getRandomSeed
uint32_t wellons_lowbias32( uint32_t x )
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
void murmur_hash33( const uint32_t in[ 3 ], uint32_t h[ 3 ] )
{
    const uint32_t M      = 0x5bd1e995u;
    uint32_t       src[3] = { in[ 0 ], in[ 1 ], in[ 2 ] };
    h[ 0 ] = 1190494759u, h[ 1 ] = 2147483647u, h[ 2 ] = 3559788179u;
    for( int c = 0; c < 3; c++ )
    {
        src[ c ] *= M;
        src[ c ] ^= src[ c ] >> 24;
        src[ c ] *= M;
    }
    for( int k = 0; k < 3; k++ )
        for( int c = 0; c < 3; c++ )
        {
            h[ c ] *= M;
            h[ c ] ^= src[ k ];
        }
    for( int c = 0; c < 3; c++ )
    {
        h[ c ] ^= h[ c ] >> 13;
        h[ c ] *= M;
        h[ c ] ^= h[ c ] >> 15;
    }
}
uint32_t random_seed( int px, int py, uint32_t frame )
{
    const uint32_t in[ 3 ] = { (uint32_t)px, (uint32_t)py, frame };
    uint32_t       h[ 3 ];
    murmur_hash33( in, h );
    return ( ( h[ 2 ] % 128u ) << 14 ) | ( ( h[ 1 ] % 128u ) << 7 ) | ( h[ 0 ] % 128u );
}

// floor()ed coordinate to an index: NaN to 0, saturated beyond 2^30
template< class T > int safe_floor_int( T f ) { return f == f ? (int)std::min( std::max( f, (T)-1073741824.0 ), (T)1073741824.0 ) : 0; }

template< class T > V4< T > mat_mul_t( const T* m, V4< T > v )
{
    V4< T > r;
    T*      rp = &r.x;
    for( int row = 0; row < 4; row++ ) rp[ row ] = m[ row ] * v.x + m[ 4 + row ] * v.y + m[ 8 + row ] * v.z + m[ 12 + row ] * v.w;
    return r;
}
template< class T > V4< T > vmix4( V4< T > x, V4< T > y, T a ) { return { gmix( x.x, y.x, a ), gmix( x.y, y.y, a ), gmix( x.z, y.z, a ), gmix( x.w, y.w, a ) }; }

template< class T > struct Scatter
{
    Stream&                       s;
    uint32_t                      fi;
    const rgdn_volumetric_params& p;
    T                             invViewProj[ 16 ], viewProj[ 16 ];

    Scatter( Stream& st, uint32_t f, const rgdn_volumetric_params& pp ) : s( st ), fi( f ), p( pp )
    {
        // invView * invProjection (CmScatterAccum.comp:55), each element summed over k in order
        for( int c = 0; c < 4; c++ )
            for( int r = 0; r < 4; r++ )
            {
                T acc = (T)p.invView[ r ] * (T)p.invProjection[ c * 4 ];
                for( int k = 1; k < 4; k++ ) acc = acc + (T)p.invView[ k * 4 + r ] * (T)p.invProjection[ c * 4 + k ];
                invViewProj[ c * 4 + r ] = acc;
            }
        for( int k = 0; k < 16; k++ ) viewProj[ k ] = (T)p.volumeViewProj[ k ];
    }

    // textureLod of the volume, linear clamp-to-edge: x, then y, then z
    V4< T > trilinear( V3< T > sp )
    {
        Plane&    vol = s.cur( RGDN_FB_SCATTER_VOLUME, fi );
        const int n[ 3 ] = { RGDN_VOLUME_SIZE_X, RGDN_VOLUME_SIZE_Y, RGDN_VOLUME_SIZE_Z };
        const T   u[ 3 ] = { sp.x, sp.y, sp.z };
        int       i0[ 3 ], i1[ 3 ];
        T         f[ 3 ];
        for( int d = 0; d < 3; d++ )
        {
            const T x  = u[ d ] * (T)n[ d ] - K( 0.5 );
            const T fx = o_floor( x );
            const int ix = safe_floor_int( fx );
            i0[ d ] = std::min( std::max( ix, 0 ), n[ d ] - 1 );
            i1[ d ] = std::min( std::max( ix, -1 ) + 1, n[ d ] - 1 );
            f[ d ]  = x - fx;
        }
        auto t = [ & ]( int x, int y, int z ) { return vol.fetch< T >( x, z * n[ 1 ] + y ); };
        const V4< T > c00 = vmix4( t( i0[ 0 ], i0[ 1 ], i0[ 2 ] ), t( i1[ 0 ], i0[ 1 ], i0[ 2 ] ), f[ 0 ] );
        const V4< T > c10 = vmix4( t( i0[ 0 ], i1[ 1 ], i0[ 2 ] ), t( i1[ 0 ], i1[ 1 ], i0[ 2 ] ), f[ 0 ] );
        const V4< T > c01 = vmix4( t( i0[ 0 ], i0[ 1 ], i1[ 2 ] ), t( i1[ 0 ], i0[ 1 ], i1[ 2 ] ), f[ 0 ] );
        const V4< T > c11 = vmix4( t( i0[ 0 ], i1[ 1 ], i1[ 2 ] ), t( i1[ 0 ], i1[ 1 ], i1[ 2 ] ), f[ 0 ] );
        return vmix4( vmix4( c00, c10, f[ 1 ] ), vmix4( c01, c11, f[ 1 ] ), f[ 2 ] );
    }

    // volume_toSamplePosition_T (Volumetric.h:38-58), VOLUMETRIC_DISTANCE_POW 1
    V3< T > sample_pos( V3< T > w )
    {
        const V4< T > ndc = mat_mul_t( viewProj, V4< T >{ w.x, w.y, w.z, (T)1 } );
        const T       nx = ndc.x / ndc.w, ny = ndc.y / ndc.w;
        const T       dx = w.x - (T)p.cameraPosition[ 0 ], dy = w.y - (T)p.cameraPosition[ 1 ], dz = w.z - (T)p.cameraPosition[ 2 ];
        const T       dist = o_sqrt( dx * dx + dy * dy + dz * dz );
        const T       z    = gclamp( ( dist - (T)p.volumeCameraNear ) / ( (T)p.volumeCameraFar - (T)p.volumeCameraNear ), (T)0, (T)1 );
        return { nx * K( 0.5 ) + K( 0.5 ), ny * K( 0.5 ) + K( 0.5 ), z };
    }

    // fializeScattering (CmScatterAccum.comp:41-95)
    V4< T > finalize( int rx, int ry, T depthCb )
    {
        if( p.volumeEnableType == RGDN_VOLUME_ENABLE_VOLUMETRIC )
        {
            const T       sx  = (T)rx / (T)(float)s.W, sy = (T)ry / (T)(float)s.H;
            const T       dn  = s.cur( RGDN_FB_DEPTH_NDC, fi ).fetch< T >( rx, ry ).x;
            const V4< T > wp  = mat_mul_t( invViewProj, V4< T >{ sx * K( 2.0 ) - K( 1.0 ), sy * K( 2.0 ) - K( 1.0 ), dn, (T)1 } );
            const V3< T > pos = { wp.x / wp.w, wp.y / wp.w, wp.z / wp.w };
            const uint32_t rnd = wellons_lowbias32( random_seed( rx, ry, p.frameId ) );   // rnd8_4( seed, 0 )
            const T        r0 = (T)( rnd & 0xFFu ) / K( 255.0 ), r1 = (T)( ( rnd >> 8 ) & 0xFFu ) / K( 255.0 );
            const T        r2 = (T)( ( rnd >> 16 ) & 0xFFu ) / K( 255.0 );
            // sampleHemisphere (Random.h:73-92), unitBasis = -offset
            const T u1 = r0 * K( 0.99 ), u2 = r1 * K( 0.99 );
            const T rr = o_sqrt( u1 ), hz = o_sqrt( (T)1 - u1 );
            const T phi = ( K( 2.0 ) * K( 3.14159265358979 ) ) * u2;
            const V3< T > basis = { -( rr * (T)std::cos( phi ) ), -( rr * (T)std::sin( phi ) ), -hz };
            // volume_sampleDithered (Volumetric.h:92-104), dither radius 2
            V3< T >  sp = sample_pos( pos );
            const T  k  = r2 * K( 2.0 );
            sp          = { sp.x + ( k * basis.x ) / (T)RGDN_VOLUME_SIZE_X, sp.y + ( k * basis.y ) / (T)RGDN_VOLUME_SIZE_Y,
                            sp.z + ( k * basis.z ) / (T)RGDN_VOLUME_SIZE_Z };
            return trilinear( sp );
        }
        if( p.volumeEnableType == RGDN_VOLUME_ENABLE_SIMPLE )
        {
            if( depthCb > (T)MAX_RAY_LENGTH ) return { 0, 0, 0, 1 };
            const T density = (T)( p.volumeScattering * 0.00005f );
            const T f       = o_exp( -depthCb * density );
            return { (T)p.volumeAmbient[ 0 ] * ( (T)1 - f ), (T)p.volumeAmbient[ 1 ] * ( (T)1 - f ), (T)p.volumeAmbient[ 2 ] * ( (T)1 - f ), f };
        }
        return { 0, 0, 0, 1 };
    }

    // CmScatterAccum.comp:97-161
    void accumulate()
    {
        const int W = s.W, H = s.H, sep = W / 2;
        const T   sxs = (T)(float)s.W / K( 2.0 ), sys = (T)(float)s.H;
        const T   isx = (T)1 / sxs, isy = (T)1 / sys;
        Plane &   motion = s.cur( RGDN_FB_MOTION, fi ), &depthC = s.cur( RGDN_FB_DEPTH_WORLD, fi ), &depthP = s.prv( RGDN_FB_DEPTH_WORLD, fi );
        Plane &   nrmC = s.cur( RGDN_FB_NORMAL, fi ), &nrmP = s.prv( RGDN_FB_NORMAL, fi );
        Plane &   scP = s.prv( RGDN_FB_SCATTERING, fi ), &hP = s.prv( RGDN_FB_SCATTERING_HISTORY, fi );
        Plane &   scC = s.cur( RGDN_FB_SCATTERING, fi ), &hC = s.cur( RGDN_FB_SCATTERING_HISTORY, fi );
        auto      regular = [ & ]( int cx, int cy ) {
            const int isOdd = cx >= sep ? 1 : 0, x = cx - isOdd * sep;
            return V2< int >{ x * 2 + ( isOdd + cy ) % 2, cy };
        };
        for( int cy = 0; cy < H; cy++ )
            for( int cx = 0; cx < W; cx++ )
            {
                const V4< T > mo     = motion.fetch< T >( cx, cy );
                const T       depth  = depthC.fetch< T >( cx, cy ).x;
                const V3< T > normal = decode_normal< T >( nrmC.raw_u32( cx, cy ) );
                // getPrevScreenPos (ShaderCommonGLSLFunc.h:271-277)
                const T  ppx = ( ( (T)cx + K( 0.5 ) ) * isx + mo.x ) * sxs, ppy = ( ( (T)cy + K( 0.5 ) ) * isy + mo.y ) * sys;
                const T  fpx = o_floor( ppx - K( 0.5 ) ), fpy = o_floor( ppy - K( 0.5 ) );
                const int px = safe_floor_int( fpx ), py = safe_floor_int( fpy );
                const T  sx = ( ppx - K( 0.5 ) ) - fpx, sy = ( ppy - K( 0.5 ) ) - fpy;
                const T  bw[ 2 ][ 2 ] = { { ( (T)1 - sx ) * ( (T)1 - sy ), sx * ( (T)1 - sy ) }, { ( (T)1 - sx ) * sy, sx * sy } };
                const int isOdd = cx >= sep ? 1 : 0, al = isOdd * sep, ar = ( isOdd + 1 ) * sep;
                V4< T >  acc = { 0, 0, 0, 0 };
                T        hist = 0, wsum = 0;
                for( int yy = 0; yy <= 1; yy++ )
                    for( int xx = 0; xx <= 1; xx++ )
                    {
                        const int qx = px + xx, qy = py + yy;
                        if( !( qy >= 0 && qy < H && qx >= al && qx < ar ) ) continue;
                        const T       dP = depthP.fetch< T >( qx, qy ).x;
                        const V3< T > nP = decode_normal< T >( nrmP.raw_u32( qx, qy ) );
                        if( o_abs( depth - dP + mo.z ) / o_abs( depth ) < K( 0.1 ) && dot3( normal, nP ) > K( 0.95 ) )
                        {
                            const T         w = bw[ yy ][ xx ];
                            const V2< int > r = regular( qx, qy );
                            const V4< T >   v = scP.fetch< T >( r.x, r.y );
                            acc               = { acc.x + w * v.x, acc.y + w * v.y, acc.z + w * v.z, acc.w + w * v.w };
                            hist              = hist + w * hP.fetch< T >( r.x, r.y ).x;
                            wsum              = wsum + w;
                        }
                    }
                const bool ok = wsum > K( 0.0001 );
                hist          = ok ? hist / wsum : (T)0;
                acc           = ok ? V4< T >{ acc.x / wsum, acc.y / wsum, acc.z / wsum, acc.w / wsum } : V4< T >{ 0, 0, 0, 0 };
                hist          = gclamp( hist + (T)1, (T)1, o_fmax( (T)1, (T)p.maxHistoryLength ) );
                const V2< int > reg = regular( cx, cy );
                acc                 = vmix4( acc, finalize( reg.x, reg.y, depth ), (T)1 / hist );
                scC.store< T >( reg.x, reg.y, acc );
                hC.store< T >( reg.x, reg.y, { hist, 0, 0, 0 } );
            }
    }
};

}  // namespace orc

// ============================================================================================
//  extern "C" interface (ctypes)
// ============================================================================================

extern "C" {

struct orc_stream
{
    orc::Stream s;
};

orc_stream* orc_stream_create( uint32_t w, uint32_t h, uint32_t mode )
{
    if( w == 0 || h == 0 || ( w & 1 ) || mode > orc::M_F64 ) return nullptr;
    auto* o = new orc_stream();
    o->s.init( (int)w, (int)h, mode );
    return o;
}

void orc_stream_destroy( orc_stream* o ) { delete o; }

// host pointer of a plane + its description; returns NULL if absent
void* orc_stream_plane( orc_stream* o, uint32_t fb, uint32_t frameIndex, uint32_t* outW, uint32_t* outH, uint32_t* outTexel, uint32_t* outFmt )
{
    if( !o || fb >= RGDN_FB_COUNT ) return nullptr;
    orc::Plane& pl = o->s.cur( fb, frameIndex );
    if( outW ) *outW = (uint32_t)pl.w;
    if( outH ) *outH = (uint32_t)pl.h;
    if( outTexel ) *outTexel = pl.texel;
    if( outFmt ) *outFmt = pl.fmt;
    return pl.bytes.empty() ? nullptr : pl.bytes.data();
}

// the re-shade scene from host arrays (lights == NULL clears it)
void orc_set_reshade_scene( orc_stream* o, const rgdn_sphere_light* lights, uint32_t lightCount, const uint32_t* prevToCur,
                            uint32_t prevLightCount, const rgdn_occluder* occluders, uint32_t occluderCount )
{
    if( !o ) return;
    o->s.rsSet = lights != nullptr;
    o->s.lights.assign( lights, lights ? lights + lightCount : lights );
    o->s.prevToCur.assign( prevToCur, prevToCur ? prevToCur + prevLightCount : prevToCur );
    o->s.occluders.assign( occluders, occluders ? occluders + occluderCount : occluders );
}

// forwardProjectedLuminance of previous-frame pixel (px, py) for frame slot frameIndex (the
// re-shading alone, for the known-answer tests)
int orc_reshade( orc_stream* o, uint32_t frameIndex, int px, int py, const rgdn_frame_params* p, int f64, double out[ 2 ] )
{
    if( !o || !p || !out || !o->s.rsSet ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    if( f64 )
    {
        orc::Denoise< double > dn{ o->s, frameIndex, *p, 1 };
        const auto r = dn.reshade( px, py );
        out[ 0 ] = r.x; out[ 1 ] = r.y;
    }
    else
    {
        orc::Denoise< float > dn{ o->s, frameIndex, *p, 1 };
        const auto r = dn.reshade( px, py );
        out[ 0 ] = r.x; out[ 1 ] = r.y;
    }
    return RGDN_SUCCESS;
}

uint32_t orc_stream_grad_width( orc_stream* o ) { return o ? (uint32_t)o->s.GW : 0; }
uint32_t orc_stream_grad_height( orc_stream* o ) { return o ? (uint32_t)o->s.GH : 0; }

static int run_stage_t( orc::Stream& s, uint32_t stage, uint32_t iter, uint32_t fi, const rgdn_frame_params* p, int nthreads )
{
    const uint32_t niter = p->atrousIterations == 0 ? 4u : p->atrousIterations;
    if( niter > 6 ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    auto go = [ & ]( auto dn ) -> int {
        switch( stage )
        {
            case RGDN_STAGE_GRADIENT_SAMPLES: dn.gradient_samples(); break;
            case RGDN_STAGE_GRADIENT_ATROUS:
                if( iter > 3 ) return RGDN_WRONG_FUNCTION_ARGUMENT;
                dn.gradient_atrous( iter );
                break;
            case RGDN_STAGE_TEMPORAL_ACCUMULATION: dn.temporal_accumulation(); break;
            case RGDN_STAGE_ANTI_FIREFLY: dn.anti_firefly(); break;
            case RGDN_STAGE_VARIANCE_ESTIMATION: dn.variance(); break;
            case RGDN_STAGE_ATROUS:
                if( iter >= niter ) return RGDN_WRONG_FUNCTION_ARGUMENT;
                dn.atrous( iter, niter );
                break;
            case RGDN_STAGE_LUMINANCE_HISTOGRAM: dn.histogram(); break;
            case RGDN_STAGE_LUMINANCE_AVG: dn.luminance_avg(); break;
            default: return RGDN_WRONG_FUNCTION_ARGUMENT;
        }
        return RGDN_SUCCESS;
    };
    if( s.mode == orc::M_F64 ) return go( orc::Denoise< double >{ s, fi, *p, nthreads } );
    return go( orc::Denoise< float >{ s, fi, *p, nthreads } );
}

// one stage (the per-stage parity checks)
int orc_stage( orc_stream* o, uint32_t stage, uint32_t iter, uint32_t frameIndex, const rgdn_frame_params* p, int nthreads )
{
    if( !o || !p ) return RGDN_WRONG_INSTANCE;
    return run_stage_t( o->s, stage, iter, frameIndex & 1, p, nthreads );
}

// Denoiser::Denoise preceded by the image-space gradient sampling
int orc_denoise( orc_stream* o, uint32_t frameIndex, const rgdn_frame_params* p, int nthreads )
{
    if( !o || !p ) return RGDN_WRONG_INSTANCE;
    const uint32_t niter = p->atrousIterations == 0 ? 4u : p->atrousIterations;
    if( niter > 6 ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    const uint32_t fi = frameIndex & 1;
    int r = RGDN_SUCCESS;
    if( !( p->flags & RGDN_FLAG_SKIP_GRADIENTS ) )
    {
        r |= run_stage_t( o->s, RGDN_STAGE_GRADIENT_SAMPLES, 0, fi, p, nthreads );
        for( uint32_t i = 0; i < 4; i++ ) r |= run_stage_t( o->s, RGDN_STAGE_GRADIENT_ATROUS, i, fi, p, nthreads );
    }
    r |= run_stage_t( o->s, RGDN_STAGE_TEMPORAL_ACCUMULATION, 0, fi, p, nthreads );
    r |= run_stage_t( o->s, RGDN_STAGE_ANTI_FIREFLY, 0, fi, p, nthreads );
    r |= run_stage_t( o->s, RGDN_STAGE_VARIANCE_ESTIMATION, 0, fi, p, nthreads );
    for( uint32_t i = 0; i < niter; i++ ) r |= run_stage_t( o->s, RGDN_STAGE_ATROUS, i, fi, p, nthreads );
    return r;
}

// Tonemapping::CalculateExposure
int orc_calculate_exposure( orc_stream* o, uint32_t frameIndex, const rgdn_frame_params* p, int nthreads )
{
    if( !o || !p ) return RGDN_WRONG_INSTANCE;
    int r = run_stage_t( o->s, RGDN_STAGE_LUMINANCE_HISTOGRAM, 0, frameIndex & 1, p, nthreads );
    r |= run_stage_t( o->s, RGDN_STAGE_LUMINANCE_AVG, 0, frameIndex & 1, p, nthreads );
    return r;
}

// ImageComposition::PrepareForRaster + Finalize: CmCheckerboard + CmPrepareFinal
int orc_prepare_final( orc_stream* o, uint32_t frameIndex, const rgdn_final_params* p, int nthreads )
{
    if( !o || !p ) return RGDN_WRONG_INSTANCE;
    if( o->s.mode == orc::M_F64 ) orc::prepare_final< double >( o->s, frameIndex & 1, *p, nthreads );
    else orc::prepare_final< float >( o->s, frameIndex & 1, *p, nthreads );
    return RGDN_SUCCESS;
}

// Volumetric::ProcessScattering
int orc_process_scattering( orc_stream* o, uint32_t frameIndex, const rgdn_volumetric_params* p )
{
    if( !o || !p ) return RGDN_WRONG_INSTANCE;
    const uint32_t fi = frameIndex & 1;
    if( o->s.mode == orc::M_F64 )
    {
        orc::volume_process< double >( o->s, fi );
        orc::Scatter< double >( o->s, fi, *p ).accumulate();
    }
    else
    {
        orc::volume_process< float >( o->s, fi );
        orc::Scatter< float >( o->s, fi, *p ).accumulate();
    }
    return RGDN_SUCCESS;
}
// getRandomSeed + rnd8_4 (for the known-answer tests)
uint32_t orc_random_seed( int x, int y, uint32_t frame ) { return orc::random_seed( x, y, frame ); }
uint32_t orc_wellons_lowbias32( uint32_t x ) { return orc::wellons_lowbias32( x ); }

// Bloom::Prepare + Apply
int orc_bloom( orc_stream* o, uint32_t frameIndex, float intensity )
{
    if( !o ) return RGDN_WRONG_INSTANCE;
    if( o->s.mode == orc::M_F64 ) orc::bloom< double >( o->s, frameIndex & 1, intensity );
    else orc::bloom< float >( o->s, frameIndex & 1, intensity );
    return RGDN_SUCCESS;
}

// the LPM constants (saturation[3], contrast, toneScaleBias[2], lumaT[3], rcpLumaT[3],
// crosstalk[3]) and one filtered colour, for the known-answer tests
void orc_lpm_setup( const float* saturation3, const float* crosstalk3, float* out16 )
{
    const orc::Lpm< float > L = orc::lpm_setup< float >( saturation3, crosstalk3 );
    const float v[ 16 ] = { L.saturation[ 0 ], L.saturation[ 1 ], L.saturation[ 2 ], L.contrast, L.tsb[ 0 ], L.tsb[ 1 ],
                            L.lumaT[ 0 ], L.lumaT[ 1 ], L.lumaT[ 2 ], L.rcpLumaT[ 0 ], L.rcpLumaT[ 1 ], L.rcpLumaT[ 2 ],
                            L.crosstalk[ 0 ], L.crosstalk[ 1 ], L.crosstalk[ 2 ], 0.0f };
    memcpy( out16, v, sizeof( v ) );
}
void orc_lpm_filter( const float* saturation3, const float* crosstalk3, float* rgb )
{
    const orc::Lpm< float > L = orc::lpm_setup< float >( saturation3, crosstalk3 );
    const orc::V3< float >  c = orc::lpm_filter< float >( { rgb[ 0 ], rgb[ 1 ], rgb[ 2 ] }, L );
    rgb[ 0 ] = c.x; rgb[ 1 ] = c.y; rgb[ 2 ] = c.z;
}

// Exposure.h:33-51, evaluated on the host in FP32
float orc_exposure_from_avg( float avgLuminance )
{
    float lumAverage = orc::o_fmax( 0.0f, avgLuminance );
    float ev100      = log2f( lumAverage * 100.0f / 12.5f );
    float maxLum     = 1.2f * exp2f( ev100 );
    return maxLum > 0.0f ? 1.0f / maxLum : 0.0f;
}

void orc_get_tonemapping( orc_stream* o, uint32_t* hist, float* avgLum, double* avgLum64 )
{
    if( !o ) return;
    if( hist ) memcpy( hist, o->s.hist, sizeof( o->s.hist ) );
    if( avgLum ) *avgLum = (float)o->s.avgLum;
    if( avgLum64 ) *avgLum64 = o->s.avgLum;
}

void orc_set_tonemapping( orc_stream* o, const uint32_t* hist, float avgLum )
{
    if( !o ) return;
    if( hist ) memcpy( o->s.hist, hist, sizeof( o->s.hist ) );
    o->s.avgLum = (double)avgLum;
}

// ---- codecs, exported for the known-answer tests ------------------------------------------
uint16_t orc_f32_to_f16( float f ) { return orc::f32_to_f16( f ); }
float    orc_f16_to_f32( uint16_t h ) { return orc::f16_to_f32( h ); }
uint16_t orc_f32_to_bf16( float f ) { return orc::f32_to_bf16( f ); }
float    orc_bf16_to_f32( uint16_t h ) { return orc::bf16_to_f32( h ); }
uint32_t orc_encode_e5( float r, float g, float b ) { return orc::encode_e5( r, g, b ); }
void     orc_decode_e5( uint32_t p, float* out3 ) { orc::decode_e5( p, out3 ); }
uint32_t orc_encode_b10g11r11( float r, float g, float b ) { return orc::encode_b10g11r11( r, g, b ); }
void     orc_decode_b10g11r11( uint32_t p, float* out3 ) { orc::decode_b10g11r11( p, out3 ); }
uint32_t orc_encode_normal( float x, float y, float z ) { return orc::encode_normal( x, y, z ); }
void     orc_decode_normal( uint32_t p, float* out3 )
{
    orc::V3< float > n = orc::decode_normal< float >( p );
    out3[ 0 ] = n.x; out3[ 1 ] = n.y; out3[ 2 ] = n.z;
}
uint32_t orc_color_bin( float lum, float minLog, float maxLog ) { return orc::color_bin( lum, minLog, maxLog ); }
uint8_t  orc_unorm8( float f ) { return orc::Plane::unorm8( f ); }

}  // extern "C"
