// The run-time part of glsl.h: format conversions, plane access, and the workgroup scheduler
// with fibers for barrier(). Test infrastructure only.
#include "glsl.h"

#include <cstdlib>

namespace glsl
{

thread_local Invocation* g_inv = nullptr;

std::map< std::string, Plane >& planes()
{
    static std::map< std::string, Plane > m;
    return m;
}
std::map< std::string, int >& formats()
{
    static std::map< std::string, int > m;
    return m;
}

// IEEE binary16 from binary32, round to nearest even; overflow to infinity
uint16_t f32_to_f16( float f )
{
    uint32_t u;
    std::memcpy( &u, &f, 4 );
    const uint32_t sign = ( u >> 16 ) & 0x8000u;
    const uint32_t e8   = ( u >> 23 ) & 0xFFu;
    uint32_t       m    = u & 0x7FFFFFu;
    if( e8 == 0xFFu ) return (uint16_t)( sign | 0x7C00u | ( m ? 0x200u : 0u ) );
    int e = (int)e8 - 127 + 15;
    if( e >= 31 ) return (uint16_t)( sign | 0x7C00u );
    if( e <= 0 )
    {
        if( e < -10 ) return (uint16_t)sign;
        m |= 0x800000u;
        const int      shift = 14 - e;
        uint32_t       q     = m >> shift;
        const uint32_t rem   = m & ( ( 1u << shift ) - 1u );
        const uint32_t half  = 1u << ( shift - 1 );
        if( rem > half || ( rem == half && ( q & 1u ) ) ) q++;
        return (uint16_t)( sign | q );
    }
    uint32_t       q   = ( (uint32_t)e << 10 ) | ( m >> 13 );
    const uint32_t rem = m & 0x1FFFu;
    if( rem > 0x1000u || ( rem == 0x1000u && ( q & 1u ) ) ) q++;   // may carry into the exponent
    return (uint16_t)( sign | q );
}

float f16_to_f32( uint16_t h )
{
    const uint32_t sign = ( (uint32_t)h & 0x8000u ) << 16;
    const uint32_t e    = ( h >> 10 ) & 0x1Fu;
    const uint32_t m    = h & 0x3FFu;
    uint32_t       u;
    if( e == 0 )
    {
        const float v = (float)m * ( 1.0f / 16777216.0f );   // m * 2^-24, exact
        return sign ? -v : v;
    }
    if( e == 31 ) u = sign | 0x7F800000u | ( m << 13 );
    else u = sign | ( ( e + 112u ) << 23 ) | ( m << 13 );
    float f;
    std::memcpy( &f, &u, 4 );
    return f;
}

// unsigned 11- / 10-bit floats (5-bit exponent, bias 15)
static float ufloat_to_f32( uint32_t v, int mbits )
{
    const uint32_t e = v >> mbits, m = v & ( ( 1u << mbits ) - 1u );
    if( e == 0 ) return std::ldexp( (float)m, -14 - mbits );
    if( e == 31 ) return m ? NAN : INFINITY;
    return std::ldexp( 1.0f + (float)m / (float)( 1u << mbits ), (int)e - 15 );
}
static uint32_t f32_to_ufloat( float f, int mbits )
{
    if( !( f > 0.0f ) ) return 0u;   // negative, zero, NaN
    const uint32_t maxv = ( 30u << mbits ) | ( ( 1u << mbits ) - 1u );
    if( std::isinf( f ) ) return 31u << mbits;
    int   e;
    float fr = std::frexp( f, &e );   // f = fr * 2^e, fr in [0.5, 1)
    int   eb = e - 1 + 15;            // biased exponent of 1.m form
    if( eb <= 0 )
    {
        // subnormal: m = f * 2^(14 + mbits), rounded to nearest even
        const float    s = std::ldexp( f, 14 + mbits );
        const uint32_t q = (uint32_t)std::nearbyint( s );
        return q;   // q == 1 << mbits carries into the smallest normal
    }
    const float    s = std::ldexp( fr * 2.0f - 1.0f, mbits );
    uint32_t       q = (uint32_t)std::nearbyint( s );
    uint32_t       r = ( (uint32_t)eb << mbits ) + q;   // a carry moves to the next exponent
    return r > maxv ? maxv : r;
}

int fmt_bytes( int fmt )
{
    switch( fmt )
    {
        case FMT_r8: case FMT_r8ui: return 1;
        case FMT_rg8: case FMT_r16f: case FMT_r16ui: return 2;
        case FMT_rgba8: case FMT_rg16f: case FMT_r32f: case FMT_r32ui: case FMT_r11f_g11f_b10f: return 4;
        case FMT_rgba16f: case FMT_rg32f: case FMT_rg32ui: return 8;
        case FMT_rgba32f: case FMT_rgba32ui: return 16;
        default: return 0;
    }
}

static uint8_t* texel( Plane& p, const ivec2& pix )
{
    if( !p.data || pix.x < 0 || pix.y < 0 || pix.x >= p.w || pix.y >= p.h ) return nullptr;
    return p.data + ( (size_t)pix.y * p.w + pix.x ) * fmt_bytes( p.fmt );
}

static uint8_t unorm8( float f )
{
    const float c = f < 0.0f ? 0.0f : f > 1.0f ? 1.0f : f;
    return (uint8_t)std::round( c * 255.0f );
}

vec4 load_f( Plane& p, ivec2 pix )
{
    const uint8_t* t = texel( p, pix );
    vec4           r( 0.0f, 0.0f, 0.0f, 1.0f );
    if( !t ) return vec4( 0.0f );
    uint16_t h[ 4 ];
    float    f[ 4 ];
    uint32_t u;
    switch( p.fmt )
    {
        case FMT_r8: r.x = t[ 0 ] / 255.0f; break;
        case FMT_rg8: r.x = t[ 0 ] / 255.0f; r.y = t[ 1 ] / 255.0f; break;
        case FMT_rgba8: r = vec4( t[ 0 ] / 255.0f, t[ 1 ] / 255.0f, t[ 2 ] / 255.0f, t[ 3 ] / 255.0f ); break;
        case FMT_r16f: std::memcpy( h, t, 2 ); r.x = f16_to_f32( h[ 0 ] ); break;
        case FMT_rg16f: std::memcpy( h, t, 4 ); r.x = f16_to_f32( h[ 0 ] ); r.y = f16_to_f32( h[ 1 ] ); break;
        case FMT_rgba16f:
            std::memcpy( h, t, 8 );
            r = vec4( f16_to_f32( h[ 0 ] ), f16_to_f32( h[ 1 ] ), f16_to_f32( h[ 2 ] ), f16_to_f32( h[ 3 ] ) );
            break;
        case FMT_r32f: std::memcpy( f, t, 4 ); r.x = f[ 0 ]; break;
        case FMT_rg32f: std::memcpy( f, t, 8 ); r.x = f[ 0 ]; r.y = f[ 1 ]; break;
        case FMT_rgba32f: std::memcpy( f, t, 16 ); r = vec4( f[ 0 ], f[ 1 ], f[ 2 ], f[ 3 ] ); break;
        case FMT_r11f_g11f_b10f:
            std::memcpy( &u, t, 4 );
            r.x = ufloat_to_f32( u & 0x7FFu, 6 );
            r.y = ufloat_to_f32( ( u >> 11 ) & 0x7FFu, 6 );
            r.z = ufloat_to_f32( u >> 22, 5 );
            break;
        default: std::abort();
    }
    return r;
}

vec4 bilinear( Plane& p, const vec2& uv )
{
    if( !p.data ) return vec4( 0.0f );
    const float x = uv.x * (float)p.w - 0.5f, y = uv.y * (float)p.h - 0.5f;
    const float fx = std::floor( x ), fy = std::floor( y );
    const float a = x - fx, b = y - fy;
    const int   ix = (int)fx, iy = (int)fy;
    auto        cl = []( int v, int n ) { return v < 0 ? 0 : v > n - 1 ? n - 1 : v; };
    const int   x0 = cl( ix, p.w ), x1 = cl( ix + 1, p.w ), y0 = cl( iy, p.h ), y1 = cl( iy + 1, p.h );
    const vec4  t00 = load_f( p, ivec2( x0, y0 ) ), t10 = load_f( p, ivec2( x1, y0 ) );
    const vec4  t01 = load_f( p, ivec2( x0, y1 ) ), t11 = load_f( p, ivec2( x1, y1 ) );
    return mix( mix( t00, t10, a ), mix( t01, t11, a ), b );
}

// a 3-D image's texel as a texel of the w x (h d) plane of its slices
static bool slice_pix( const Plane& p, const ivec3& c, ivec2& pix )
{
    if( !p.data || c.x < 0 || c.y < 0 || c.z < 0 || c.x >= p.w || c.y >= p.h || c.z >= p.d ) return false;
    pix = ivec2( c.x, c.z * p.h + c.y );
    return true;
}
static Plane slices( const Plane& p )
{
    Plane q = p;
    q.h     = p.h * p.d;
    q.d     = 1;
    return q;
}
vec4 load_f3( Plane& p, ivec3 c )
{
    ivec2 pix;
    if( !slice_pix( p, c, pix ) ) return vec4( 0.0f );
    Plane q = slices( p );
    return load_f( q, pix );
}
void store_f3( Plane& p, ivec3 c, const vec4& v )
{
    ivec2 pix;
    if( !slice_pix( p, c, pix ) ) return;
    Plane q = slices( p );
    store_f( q, pix, v );
}

vec4 trilinear( Plane& p, const vec3& uvw )
{
    if( !p.data ) return vec4( 0.0f );
    const int n[ 3 ] = { p.w, p.h, p.d };
    int       i0[ 3 ], i1[ 3 ];
    float     f[ 3 ];
    for( int k = 0; k < 3; k++ )
    {
        const float x  = uvw.v[ k ] * (float)n[ k ] - 0.5f;
        const float fx = std::floor( x );
        // NaN to 0; beyond the int range saturated
        const int ix = fx == fx ? (int)std::min( std::max( fx, -1073741824.0f ), 1073741824.0f ) : 0;
        i0[ k ] = std::min( std::max( ix, 0 ), n[ k ] - 1 );
        i1[ k ] = std::min( std::max( ix, -1 ) + 1, n[ k ] - 1 );
        f[ k ]  = x - fx;
    }
    auto t = [ & ]( int x, int y, int z ) { return load_f3( p, ivec3( x, y, z ) ); };
    const vec4 c00 = mix( t( i0[ 0 ], i0[ 1 ], i0[ 2 ] ), t( i1[ 0 ], i0[ 1 ], i0[ 2 ] ), f[ 0 ] );
    const vec4 c10 = mix( t( i0[ 0 ], i1[ 1 ], i0[ 2 ] ), t( i1[ 0 ], i1[ 1 ], i0[ 2 ] ), f[ 0 ] );
    const vec4 c01 = mix( t( i0[ 0 ], i0[ 1 ], i1[ 2 ] ), t( i1[ 0 ], i0[ 1 ], i1[ 2 ] ), f[ 0 ] );
    const vec4 c11 = mix( t( i0[ 0 ], i1[ 1 ], i1[ 2 ] ), t( i1[ 0 ], i1[ 1 ], i1[ 2 ] ), f[ 0 ] );
    return mix( mix( c00, c10, f[ 1 ] ), mix( c01, c11, f[ 1 ] ), f[ 2 ] );
}

uvec4 load_u( Plane& p, ivec2 pix )
{
    const uint8_t* t = texel( p, pix );
    uvec4          r( 0u, 0u, 0u, 1u );
    if( !t ) return uvec4( 0u );
    uint32_t u[ 4 ];
    uint16_t s;
    switch( p.fmt )
    {
        case FMT_r8ui: r.x = t[ 0 ]; break;
        case FMT_r16ui: std::memcpy( &s, t, 2 ); r.x = s; break;
        case FMT_r32ui: std::memcpy( u, t, 4 ); r.x = u[ 0 ]; break;
        case FMT_rg32ui: std::memcpy( u, t, 8 ); r.x = u[ 0 ]; r.y = u[ 1 ]; break;
        case FMT_rgba32ui: std::memcpy( u, t, 16 ); r = uvec4( u[ 0 ], u[ 1 ], u[ 2 ], u[ 3 ] ); break;
        default: std::abort();
    }
    return r;
}

void store_f( Plane& p, ivec2 pix, const vec4& v )
{
    uint8_t* t = texel( p, pix );
    if( !t ) return;
    uint16_t h[ 4 ];
    uint32_t u;
    switch( p.fmt )
    {
        case FMT_r8: t[ 0 ] = unorm8( v.x ); break;
        case FMT_rg8: t[ 0 ] = unorm8( v.x ); t[ 1 ] = unorm8( v.y ); break;
        case FMT_rgba8: for( int i = 0; i < 4; i++ ) t[ i ] = unorm8( v.v[ i ] ); break;
        case FMT_r16f: h[ 0 ] = f32_to_f16( v.x ); std::memcpy( t, h, 2 ); break;
        case FMT_rg16f: h[ 0 ] = f32_to_f16( v.x ); h[ 1 ] = f32_to_f16( v.y ); std::memcpy( t, h, 4 ); break;
        case FMT_rgba16f:
            for( int i = 0; i < 4; i++ ) h[ i ] = f32_to_f16( v.v[ i ] );
            std::memcpy( t, h, 8 );
            break;
        case FMT_r32f: std::memcpy( t, &v.x, 4 ); break;
        case FMT_rg32f: std::memcpy( t, v.v, 8 ); break;
        case FMT_rgba32f: std::memcpy( t, v.v, 16 ); break;
        case FMT_r11f_g11f_b10f:
            u = f32_to_ufloat( v.x, 6 ) | ( f32_to_ufloat( v.y, 6 ) << 11 ) | ( f32_to_ufloat( v.z, 5 ) << 22 );
            std::memcpy( t, &u, 4 );
            break;
        default: std::abort();
    }
}

void store_u( Plane& p, ivec2 pix, const uvec4& v )
{
    uint8_t* t = texel( p, pix );
    if( !t ) return;
    switch( p.fmt )
    {
        case FMT_r8ui: t[ 0 ] = (uint8_t)v.x; break;
        case FMT_r16ui: { const uint16_t s = (uint16_t)v.x; std::memcpy( t, &s, 2 ); break; }
        case FMT_r32ui: std::memcpy( t, &v.x, 4 ); break;
        case FMT_rg32ui: std::memcpy( t, v.v, 8 ); break;
        case FMT_rgba32ui: std::memcpy( t, v.v, 16 ); break;
        default: std::abort();
    }
}

// ------------------------------------------------------------------------------------------
// dispatch
// ------------------------------------------------------------------------------------------
namespace
{
ucontext_t        g_sched;
void ( *g_entry )() = nullptr;
constexpr size_t  kStack = 512 * 1024;

void fiber_main()
{
    g_entry();
    g_inv->done = true;
    swapcontext( &g_inv->ctx, &g_sched );
}
}  // namespace

thread_local bool g_fibers = false;

void barrier()
{
    if( !g_fibers ) return;
    swapcontext( &g_inv->ctx, &g_sched );
}

void dispatch( void ( *entry )(), uvec3 groups, uvec3 local, bool fibers )
{
    const uint                n = local.x * local.y * local.z;
    std::vector< Invocation > inv( n );
    std::vector< char >       stacks( fibers ? (size_t)n * kStack : 0 );
    g_entry  = entry;
    g_fibers = fibers;
    for( uint gz = 0; gz < groups.z; gz++ )
        for( uint gy = 0; gy < groups.y; gy++ )
            for( uint gx = 0; gx < groups.x; gx++ )
            {
                uint k = 0;
                for( uint lz = 0; lz < local.z; lz++ )
                    for( uint ly = 0; ly < local.y; ly++ )
                        for( uint lx = 0; lx < local.x; lx++, k++ )
                        {
                            Invocation& v = inv[ k ];
                            v.lid         = uvec3( lx, ly, lz );
                            v.wg          = uvec3( gx, gy, gz );
                            v.gid         = uvec3( gx * local.x + lx, gy * local.y + ly, gz * local.z + lz );
                            v.lindex      = k;
                            v.done        = false;
                        }
                if( !fibers )
                {
                    for( uint i = 0; i < n; i++ )
                    {
                        g_inv = &inv[ i ];
                        entry();
                    }
                    continue;
                }
                for( uint i = 0; i < n; i++ )
                {
                    getcontext( &inv[ i ].ctx );
                    inv[ i ].ctx.uc_stack.ss_sp   = stacks.data() + (size_t)i * kStack;
                    inv[ i ].ctx.uc_stack.ss_size = kStack;
                    inv[ i ].ctx.uc_link          = nullptr;
                    makecontext( &inv[ i ].ctx, fiber_main, 0 );
                }
                // rounds: every unfinished fiber runs to its next barrier (or its end)
                for( bool left = true; left; )
                {
                    left = false;
                    for( uint i = 0; i < n; i++ )
                    {
                        if( inv[ i ].done ) continue;
                        g_inv = &inv[ i ];
                        swapcontext( &g_sched, &inv[ i ].ctx );
                        left = left || !inv[ i ].done;
                    }
                }
            }
    g_inv    = nullptr;
    g_fibers = false;
}

}  // namespace glsl

// ------------------------------------------------------------------------------------------
// host interface
// ------------------------------------------------------------------------------------------
extern "C" {
// Binds host memory (dense rows of w x h texels in the image's declared format) to the image
// `name` and to the sampler named after it; returns the texel size, 0 for an undeclared image.
int ref_bind( const char* name, void* data, int w, int h )
{
    auto it = glsl::formats().find( name );
    if( it == glsl::formats().end() ) return 0;
    glsl::Plane& p = glsl::planes()[ name ];
    p.data         = static_cast< uint8_t* >( data );
    p.w            = w;
    p.h            = h;
    p.d            = 1;
    p.fmt          = it->second;
    return glsl::fmt_bytes( p.fmt );
}
// Binds a 3-D image (d slices of w x h texels) to `name` and the samplers named after it. A name
// that only samplers use (such as a _Sampler_Prev) takes the format `fmt`; a declared image keeps
// its declared format. Returns the texel size, 0 if the format is unknown.
int ref_bind3d( const char* name, void* data, int w, int h, int d, int fmt )
{
    auto it = glsl::formats().find( name );
    if( it == glsl::formats().end() )
    {
        if( fmt < 0 || fmt >= glsl::FMT_none ) return 0;
        glsl::formats()[ name ] = fmt;
        it                      = glsl::formats().find( name );
    }
    glsl::Plane& p = glsl::planes()[ name ];
    p.data         = static_cast< uint8_t* >( data );
    p.w            = w;
    p.h            = h;
    p.d            = d;
    p.fmt          = it->second;
    return glsl::fmt_bytes( p.fmt );
}
// the texel size of a declared image, 0 if none has that name
int ref_texel_bytes( const char* name )
{
    auto it = glsl::formats().find( name );
    return it == glsl::formats().end() ? 0 : glsl::fmt_bytes( it->second );
}
void ref_unbind_all()
{
    for( auto& kv : glsl::planes() ) kv.second = glsl::Plane{};
}
}
