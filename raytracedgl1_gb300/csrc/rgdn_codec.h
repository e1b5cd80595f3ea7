// Texel codecs of the denoiser's framebuffer formats, callable from CUDA device code and
// host C++ alike. Each one implements a public specification; the reference's uses are cited.
//
//   E5B9G9R9 shared-exponent colour      Source/Shaders/Utils.h:150-207
//                                        (EXT_texture_shared_exponent)
//   spherical 16:16 normal code          Source/Shaders/Utils.h:105-140
//   B10G11R11 unsigned float             Vulkan VK_FORMAT_B10G11R11_UFLOAT_PACK32
//   binary16 / bfloat16 / unorm8         IEEE-754, Vulkan unorm conversion
//
// Rounding choices (identical on host and device):
//   * round() in the E5 encoder rounds half away from zero;
//   * float -> fp16 / bf16 rounds to nearest even (fp16 overflow gives Inf);
//   * float -> unorm8 is round(clamp(x,0,1) * 255), unorm8 -> float is u / 255;
//   * float -> 11/10-bit unsigned float rounds to nearest even, clamps to the largest finite
//     value, and maps negative values and NaN to zero.
#pragma once

#include <stdint.h>

#if defined( __CUDACC__ )
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#define RGDN_HD __host__ __device__ __forceinline__
#else
#include <math.h>
#include <string.h>
#define RGDN_HD inline
#endif

namespace rgdn
{

RGDN_HD uint32_t f2u( float f )
{
#if defined( __CUDA_ARCH__ )
    return __float_as_uint( f );
#else
    uint32_t u;
    memcpy( &u, &f, 4 );
    return u;
#endif
}

RGDN_HD float u2f( uint32_t u )
{
#if defined( __CUDA_ARCH__ )
    return __uint_as_float( u );
#else
    float f;
    memcpy( &f, &u, 4 );
    return f;
#endif
}

// 2^k for k in the normal exponent range [-126, 127]
RGDN_HD float exp2i( int k ) { return u2f( (uint32_t)( k + 127 ) << 23 ); }

RGDN_HD float fmin_( float a, float b )
{
#if defined( __CUDA_ARCH__ )
    return fminf( a, b );
#else
    return fminf( a, b );
#endif
}
RGDN_HD float fmax_( float a, float b ) { return fmaxf( a, b ); }

// ---------------------------------------------------------------- binary16
RGDN_HD uint16_t f32_to_f16( float f )
{
#if defined( __CUDA_ARCH__ )
    return __half_as_ushort( __float2half_rn( f ) );
#else
    uint32_t x    = f2u( f );
    uint32_t sign = ( x >> 16 ) & 0x8000u;
    uint32_t e8   = ( x >> 23 ) & 0xFFu;
    uint32_t mant = x & 0x7FFFFFu;
    if( e8 == 0xFFu ) return (uint16_t)( sign | ( mant ? ( 0x7E00u | ( mant >> 13 ) ) : 0x7C00u ) );
    int e = (int)e8 - 112;  // rebias 127 -> 15
    if( e >= 31 ) return (uint16_t)( sign | 0x7C00u );
    if( e <= 0 )
    {
        if( e < -10 ) return (uint16_t)sign;
        uint32_t sig   = mant | 0x800000u;
        uint32_t shift = (uint32_t)( 14 - e );
        uint32_t q     = sig >> shift;
        uint32_t r     = sig & ( ( 1u << shift ) - 1u );
        uint32_t h     = 1u << ( shift - 1u );
        q += ( r > h || ( r == h && ( q & 1u ) ) ) ? 1u : 0u;
        return (uint16_t)( sign | q );
    }
    uint32_t v = ( (uint32_t)e << 10 ) | ( mant >> 13 );
    uint32_t r = mant & 0x1FFFu;
    v += ( r > 0x1000u || ( r == 0x1000u && ( v & 1u ) ) ) ? 1u : 0u;
    return (uint16_t)( sign | v );
#endif
}

RGDN_HD float f16_to_f32( uint16_t h )
{
#if defined( __CUDA_ARCH__ )
    return __half2float( __ushort_as_half( h ) );
#else
    uint32_t sign = ( (uint32_t)h & 0x8000u ) << 16;
    uint32_t e    = ( h >> 10 ) & 0x1Fu;
    uint32_t m    = h & 0x3FFu;
    if( e == 0 )
    {
        float v = (float)m * 5.9604644775390625e-08f;
        return sign ? -v : v;
    }
    if( e == 31 ) return u2f( sign | 0x7F800000u | ( m << 13 ) );
    return u2f( sign | ( ( e + 112u ) << 23 ) | ( m << 13 ) );
#endif
}

// ---------------------------------------------------------------- bfloat16
RGDN_HD uint16_t f32_to_bf16( float f )
{
#if defined( __CUDA_ARCH__ )
    return __bfloat16_as_ushort( __float2bfloat16_rn( f ) );
#else
    uint32_t x = f2u( f );
    if( ( x & 0x7F800000u ) == 0x7F800000u && ( x & 0x7FFFFFu ) ) return (uint16_t)( ( x >> 16 ) | 0x40u );
    x += 0x7FFFu + ( ( x >> 16 ) & 1u );
    return (uint16_t)( x >> 16 );
#endif
}
RGDN_HD float bf16_to_f32( uint16_t b ) { return u2f( (uint32_t)b << 16 ); }

// ---------------------------------------------------------------- unorm8
RGDN_HD uint32_t f32_to_unorm8( float f )
{
    float c = fmin_( fmax_( f, 0.0f ), 1.0f );
    return (uint32_t)roundf( c * 255.0f );
}
RGDN_HD float unorm8_to_f32( uint32_t u ) { return (float)u / 255.0f; }

// ---------------------------------------------------------------- E5B9G9R9 (Utils.h:162-207)
RGDN_HD uint32_t encode_e5( float r, float g, float b )
{
    r           = fmin_( fmax_( r, 0.0f ), 65408.0f );
    g           = fmin_( fmax_( g, 0.0f ), 65408.0f );
    b           = fmin_( fmax_( b, 0.0f ), 65408.0f );
    float max_c = fmax_( r, fmax_( g, b ) );
    if( max_c == 0.0f ) return 0u;
    // floor(log2(max_c)) from the exponent field; subnormals fall under the -16 floor
    int e8    = (int)( ( f2u( max_c ) >> 23 ) & 0xFFu );
    int flog  = e8 ? e8 - 127 : -127;
    int exp_p = ( flog > -16 ? flog : -16 ) + 16;                 // in [0, 31]
    int max_s = (int)roundf( max_c * exp2i( 24 - exp_p ) );       // exact scaling
    int exp_s = max_s != 512 ? exp_p : exp_p + 1;
    float s   = exp2i( 24 - exp_s );
    uint32_t rs = (uint32_t)roundf( r * s );
    uint32_t gs = (uint32_t)roundf( g * s );
    uint32_t bs = (uint32_t)roundf( b * s );
    return ( (uint32_t)exp_s << 27 ) | ( bs << 18 ) | ( gs << 9 ) | rs;
}

struct f3
{
    float x, y, z;
};

RGDN_HD f3 decode_e5( uint32_t p )
{
    float s = exp2i( (int)( p >> 27 ) - 24 );
    return { s * (float)( p & 0x1FFu ), s * (float)( ( p >> 9 ) & 0x1FFu ), s * (float)( ( p >> 18 ) & 0x1FFu ) };
}

// ---------------------------------------------------------------- B10G11R11 unsigned floats
RGDN_HD uint32_t f32_to_ufloat( float f, int mbits )
{
    const uint32_t maxFinite = ( 30u << mbits ) | ( ( 1u << mbits ) - 1u );
    if( !( f > 0.0f ) ) return 0u;
    uint32_t x  = f2u( f );
    uint32_t e8 = ( x >> 23 ) & 0xFFu;
    if( e8 == 0xFFu ) return maxFinite;
    int      e     = (int)e8 - 112;
    uint32_t sig   = e8 ? ( ( x & 0x7FFFFFu ) | 0x800000u ) : ( x & 0x7FFFFFu );
    int      shift = 23 - mbits;
    if( e < 1 )
    {
        shift += 1 - e;
        e = 0;
        if( shift > 24 ) return 0u;
    }
    uint32_t q = sig >> shift;
    uint32_t r = sig & ( ( 1u << shift ) - 1u );
    uint32_t h = 1u << ( shift - 1 );
    q += ( r > h || ( r == h && ( q & 1u ) ) ) ? 1u : 0u;
    uint32_t v;
    if( e == 0 ) v = q;
    else
    {
        if( q == ( 2u << mbits ) )
        {
            q >>= 1;
            e++;
        }
        v = ( (uint32_t)e << mbits ) | ( q & ( ( 1u << mbits ) - 1u ) );
    }
    return v > maxFinite ? maxFinite : v;
}

RGDN_HD float ufloat_to_f32( uint32_t v, int mbits )
{
    uint32_t e = v >> mbits;
    uint32_t m = v & ( ( 1u << mbits ) - 1u );
    if( e == 0 ) return (float)m * exp2i( -14 - mbits );
    if( e == 31 ) return u2f( m ? 0x7FC00000u : 0x7F800000u );
    return (float)( ( 1u << mbits ) | m ) * exp2i( (int)e - 15 - mbits );
}

RGDN_HD uint32_t encode_b10g11r11( float r, float g, float b )
{
    return f32_to_ufloat( r, 6 ) | ( f32_to_ufloat( g, 6 ) << 11 ) | ( f32_to_ufloat( b, 5 ) << 22 );
}
RGDN_HD f3 decode_b10g11r11( uint32_t p )
{
    return { ufloat_to_f32( p & 0x7FFu, 6 ), ufloat_to_f32( ( p >> 11 ) & 0x7FFu, 6 ), ufloat_to_f32( ( p >> 22 ) & 0x3FFu, 5 ) };
}

// ---------------------------------------------------------------- spherical normal code
// Angles exactly as Utils.h:124-140 forms them in FP32: phi = j*pi/65535, theta = (2k)*pi/65536.
RGDN_HD float normal_phi( uint32_t j ) { return (float)j * 3.14159265f / 65535.0f; }
RGDN_HD float normal_theta( uint32_t k ) { return (float)( k * 2u ) * 3.14159265f / 65536.0f; }

}  // namespace rgdn
