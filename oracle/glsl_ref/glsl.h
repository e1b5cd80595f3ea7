// GLSL compute-shader semantics in C++, for running the reference's own shader sources on the
// CPU as the oracle's check (test infrastructure: nothing of the product links it).
//
// oracle/glsl_ref/build.py turns a preprocessed shader into C++ that includes this header:
// multi-component swizzles become swz<...>() (read) and swzw<...>() (write) calls, float
// literals get an f suffix, layout-qualified declarations become the GLSL_* macros below, and
// out / inout parameters become references. This header supplies the types (vectors with
// .x/.y/.z/.w and .r/.g/.b/.a members, column-major matrices), the built-in functions in binary32,
// images and samplers over host planes in the framebuffer formats, the compute built-in
// variables, shared memory and barrier().
//
// Execution: a dispatch runs its workgroups one after another. Within a workgroup each
// invocation runs as a fiber (ucontext) with its own stack, and barrier() (also
// groupMemoryBarrier() and memoryBarrierShared(), read as the synchronisation their shaders
// intend) hands control to the next fiber; every fiber reaches the barrier before any passes
// it. Shared variables are namespace-scope statics of the translation unit.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <string>
#include <type_traits>
#include <ucontext.h>
#include <vector>

namespace glsl
{

typedef uint32_t uint;

// ------------------------------------------------------------------------------------------
// vectors
// ------------------------------------------------------------------------------------------
template< class T, int N > struct vec;

template< class T, int N > struct vec_storage;
template< class T > struct vec_storage< T, 2 >
{
    union
    {
        struct { T x, y; };
        struct { T r, g; };
        struct { T s, t; };
        T v[ 2 ];
    };
};
template< class T > struct vec_storage< T, 3 >
{
    union
    {
        struct { T x, y, z; };
        struct { T r, g, b; };
        struct { T s, t, p; };
        T v[ 3 ];
    };
};
template< class T > struct vec_storage< T, 4 >
{
    union
    {
        struct { T x, y, z, w; };
        struct { T r, g, b, a; };
        struct { T s, t, p, q; };
        T v[ 4 ];
    };
};

template< class T > struct is_vec : std::false_type {};
template< class T, int N > struct is_vec< vec< T, N > > : std::true_type {};
template< class T > constexpr bool is_scalar_v = std::is_arithmetic< T >::value;

// components of the constructor arguments, in order
template< class T, int N > struct Filler
{
    T*  out;
    int n = 0;
    template< class S > void put( S s )
    {
        if constexpr( is_scalar_v< S > )
        {
            if( n < N ) out[ n++ ] = (T)s;
        }
        else
        {
            for( int i = 0; i < S::size; i++ )
                if( n < N ) out[ n++ ] = (T)s.v[ i ];
        }
    }
};

template< class T, int... I > struct SwzRef;

template< class T, int N > struct vec : vec_storage< T, N >
{
    static constexpr int size = N;
    using elem                = T;
    using vec_storage< T, N >::v;

    vec() { for( int i = 0; i < N; i++ ) v[ i ] = T( 0 ); }
    // one scalar: every component
    template< class S, typename std::enable_if< is_scalar_v< S >, int >::type = 0 > explicit vec( S s )
    {
        for( int i = 0; i < N; i++ ) v[ i ] = (T)s;
    }
    // the same size, another component type (GLSL's implicit conversions and constructors)
    template< class U > vec( const vec< U, N >& o )
    {
        for( int i = 0; i < N; i++ ) v[ i ] = (T)o.v[ i ];
    }
    // a larger vector: its first N components
    template< class U, int M, typename std::enable_if< ( M > N ), int >::type = 0 > explicit vec( const vec< U, M >& o )
    {
        for( int i = 0; i < N; i++ ) v[ i ] = (T)o.v[ i ];
    }
    // several arguments: their components in order
    template< class A, class B, class... R > vec( A a, B b, R... r )
    {
        Filler< T, N > f{ v };
        f.put( a );
        f.put( b );
        ( f.put( r ), ... );
    }
    vec( const vec& o ) { for( int i = 0; i < N; i++ ) v[ i ] = o.v[ i ]; }
    vec& operator=( const vec& o )
    {
        for( int i = 0; i < N; i++ ) v[ i ] = o.v[ i ];
        return *this;
    }

    T&       operator[]( int i ) { return v[ i ]; }
    const T& operator[]( int i ) const { return v[ i ]; }

    template< int... I > vec< T, (int)sizeof...( I ) > swz() const { return vec< T, (int)sizeof...( I ) >( v[ I ]... ); }
    template< int... I > SwzRef< T, I... > swzw() { return SwzRef< T, I... >{ v }; }

#define GLSL_COMPOUND( OP )                                                                              \
    vec& operator OP##=( const vec& o )                                                                   \
    {                                                                                                     \
        for( int i = 0; i < N; i++ ) v[ i ] = v[ i ] OP o.v[ i ];                                         \
        return *this;                                                                                     \
    }                                                                                                     \
    template< class S, typename std::enable_if< is_scalar_v< S >, int >::type = 0 > vec& operator OP##=( S s ) \
    {                                                                                                     \
        for( int i = 0; i < N; i++ ) v[ i ] = v[ i ] OP (T)s;                                             \
        return *this;                                                                                     \
    }
    GLSL_COMPOUND( + )
    GLSL_COMPOUND( - )
    GLSL_COMPOUND( * )
    GLSL_COMPOUND( / )
    GLSL_COMPOUND( % )
    GLSL_COMPOUND( ^ )
    GLSL_COMPOUND( & )
    GLSL_COMPOUND( | )
    GLSL_COMPOUND( << )
    GLSL_COMPOUND( >> )
#undef GLSL_COMPOUND
};

// a 1-component "swizzle" of a vector is its scalar, which the vec constructor accepts
template< class T, int... I > struct SwzRef
{
    T* v;
    static constexpr int n = (int)sizeof...( I );
    SwzRef& operator=( const vec< T, n >& o )
    {
        const int idx[] = { I... };
        const vec< T, n > c = o;   // the source may alias the target
        for( int k = 0; k < n; k++ ) v[ idx[ k ] ] = c.v[ k ];
        return *this;
    }
    template< class S, typename std::enable_if< is_scalar_v< S >, int >::type = 0 > SwzRef& operator=( S s )
    {
        return *this = vec< T, n >( s );
    }
    operator vec< T, n >() const { return vec< T, n >( v[ I ]... ); }
#define GLSL_SWZ_COMPOUND( OP )                                       \
    SwzRef& operator OP##=( const vec< T, n >& o )                      \
    {                                                                   \
        vec< T, n > c = *this;                                          \
        c OP## = o;                                                     \
        return *this = c;                                               \
    }                                                                   \
    template< class S, typename std::enable_if< is_scalar_v< S >, int >::type = 0 > SwzRef& operator OP##=( S s ) \
    {                                                                   \
        vec< T, n > c = *this;                                          \
        c OP## = s;                                                     \
        return *this = c;                                               \
    }
    GLSL_SWZ_COMPOUND( + )
    GLSL_SWZ_COMPOUND( - )
    GLSL_SWZ_COMPOUND( * )
    GLSL_SWZ_COMPOUND( / )
#undef GLSL_SWZ_COMPOUND
};

typedef vec< float, 2 >    vec2;
typedef vec< float, 3 >    vec3;
typedef vec< float, 4 >    vec4;
typedef vec< int, 2 >      ivec2;
typedef vec< int, 3 >      ivec3;
typedef vec< int, 4 >      ivec4;
typedef vec< uint32_t, 2 > uvec2;
typedef vec< uint32_t, 3 > uvec3;
typedef vec< uint32_t, 4 > uvec4;
typedef vec< bool, 2 >     bvec2;
typedef vec< bool, 3 >     bvec3;
typedef vec< bool, 4 >     bvec4;

// component-wise operators (vector op vector, vector op scalar, scalar op vector)
#define GLSL_BINOP( OP )                                                                                       \
    template< class T, int N > vec< T, N > operator OP( const vec< T, N >& a, const vec< T, N >& b )            \
    {                                                                                                            \
        vec< T, N > r;                                                                                           \
        for( int i = 0; i < N; i++ ) r.v[ i ] = a.v[ i ] OP b.v[ i ];                                            \
        return r;                                                                                                \
    }                                                                                                            \
    template< class T, int N, class S, typename std::enable_if< is_scalar_v< S >, int >::type = 0 >           \
    vec< T, N > operator OP( const vec< T, N >& a, S s )                                                       \
    {                                                                                                            \
        vec< T, N > r;                                                                                           \
        for( int i = 0; i < N; i++ ) r.v[ i ] = a.v[ i ] OP (T)s;                                                \
        return r;                                                                                                \
    }                                                                                                            \
    template< class T, int N, class S, typename std::enable_if< is_scalar_v< S >, int >::type = 0 >           \
    vec< T, N > operator OP( S s, const vec< T, N >& a )                                                       \
    {                                                                                                            \
        vec< T, N > r;                                                                                           \
        for( int i = 0; i < N; i++ ) r.v[ i ] = (T)s OP a.v[ i ];                                                \
        return r;                                                                                                \
    }
GLSL_BINOP( + )
GLSL_BINOP( - )
GLSL_BINOP( * )
GLSL_BINOP( / )
GLSL_BINOP( % )
GLSL_BINOP( & )
GLSL_BINOP( | )
GLSL_BINOP( ^ )
GLSL_BINOP( << )
GLSL_BINOP( >> )
#undef GLSL_BINOP
// a float vector with an integer vector: the integer one converts to float (GLSL's implicit
// conversion)
#define GLSL_MIXOP( OP )                                                                                \
    template< int N, class I, typename std::enable_if< std::is_integral< I >::value, int >::type = 0 >   \
    vec< float, N > operator OP( const vec< float, N >& a, const vec< I, N >& b )                         \
    {                                                                                                     \
        return a OP vec< float, N >( b );                                                                 \
    }                                                                                                     \
    template< int N, class I, typename std::enable_if< std::is_integral< I >::value, int >::type = 0 >   \
    vec< float, N > operator OP( const vec< I, N >& a, const vec< float, N >& b )                         \
    {                                                                                                     \
        return vec< float, N >( a ) OP b;                                                                 \
    }
GLSL_MIXOP( + )
GLSL_MIXOP( - )
GLSL_MIXOP( * )
GLSL_MIXOP( / )
#undef GLSL_MIXOP

template< class T, int N > vec< T, N > operator-( const vec< T, N >& a )
{
    vec< T, N > r;
    for( int i = 0; i < N; i++ ) r.v[ i ] = -a.v[ i ];
    return r;
}
template< class T, int N > vec< T, N > operator~( const vec< T, N >& a )
{
    vec< T, N > r;
    for( int i = 0; i < N; i++ ) r.v[ i ] = ~a.v[ i ];
    return r;
}
template< class T, int N > bool operator==( const vec< T, N >& a, const vec< T, N >& b )
{
    for( int i = 0; i < N; i++ )
        if( !( a.v[ i ] == b.v[ i ] ) ) return false;
    return true;
}
template< class T, int N > bool operator!=( const vec< T, N >& a, const vec< T, N >& b ) { return !( a == b ); }

// swizzle proxies in expressions: as their vector value
template< class T, int... I > vec< T, (int)sizeof...( I ) > val( const SwzRef< T, I... >& s ) { return s; }

// ------------------------------------------------------------------------------------------
// matrices (column-major, C columns of R rows)
// ------------------------------------------------------------------------------------------
template< int C, int R > struct mat
{
    vec< float, R > c[ C ];
    mat() {}
    explicit mat( float d )
    {
        for( int i = 0; i < C; i++ )
            for( int j = 0; j < R; j++ ) c[ i ].v[ j ] = i == j ? d : 0.0f;
    }
    template< int C2, int R2, typename std::enable_if< ( C2 != C || R2 != R ), int >::type = 0 > explicit mat( const mat< C2, R2 >& o )
    {
        for( int i = 0; i < C; i++ )
            for( int j = 0; j < R; j++ ) c[ i ].v[ j ] = ( i < C2 && j < R2 ) ? o.c[ i ].v[ j ] : ( i == j ? 1.0f : 0.0f );
    }
    template< class... A, typename std::enable_if< ( sizeof...( A ) == C && C > 1 ), int >::type = 0 > mat( const vec< float, R >& c0, A... rest )
    {
        const vec< float, R > cols[] = { c0, rest... };
        for( int i = 0; i < C; i++ ) c[ i ] = cols[ i ];
    }
    vec< float, R >&       operator[]( int i ) { return c[ i ]; }
    const vec< float, R >& operator[]( int i ) const { return c[ i ]; }
};
typedef mat< 2, 2 > mat2;
typedef mat< 3, 3 > mat3;
typedef mat< 4, 4 > mat4;
typedef mat< 2, 3 > mat2x3;
typedef mat< 2, 4 > mat2x4;
typedef mat< 3, 2 > mat3x2;
typedef mat< 3, 4 > mat3x4;
typedef mat< 4, 2 > mat4x2;
typedef mat< 4, 3 > mat4x3;

template< int C, int R > vec< float, R > operator*( const mat< C, R >& m, const vec< float, C >& x )
{
    vec< float, R > r;
    for( int j = 0; j < R; j++ )
    {
        float s = 0.0f;
        for( int i = 0; i < C; i++ ) s = s + m.c[ i ].v[ j ] * x.v[ i ];
        r.v[ j ] = s;
    }
    return r;
}
template< int C, int R > vec< float, C > operator*( const vec< float, R >& x, const mat< C, R >& m )
{
    vec< float, C > r;
    for( int i = 0; i < C; i++ )
    {
        float s = 0.0f;
        for( int j = 0; j < R; j++ ) s = s + x.v[ j ] * m.c[ i ].v[ j ];
        r.v[ i ] = s;
    }
    return r;
}
template< int K, int C, int R > mat< C, R > operator*( const mat< K, R >& a, const mat< C, K >& b )
{
    mat< C, R > r;
    for( int i = 0; i < C; i++ ) r.c[ i ] = a * b.c[ i ];
    return r;
}
template< int C, int R > mat< R, C > transpose( const mat< C, R >& m )
{
    mat< R, C > r;
    for( int i = 0; i < C; i++ )
        for( int j = 0; j < R; j++ ) r.c[ j ].v[ i ] = m.c[ i ].v[ j ];
    return r;
}

// ------------------------------------------------------------------------------------------
// built-in functions (binary32; scalars of integer type convert as GLSL's implicit conversions)
// ------------------------------------------------------------------------------------------
template< class T > using fl = typename std::conditional< std::is_integral< T >::value, float, T >::type;

#define GLSL_UNARY( NAME, EXPR )                                                     \
    template< class T, typename std::enable_if< is_scalar_v< T >, int >::type = 0 > \
    inline fl< T > NAME( T x_ )                                                      \
    {                                                                                \
        const fl< T > x = (fl< T >)x_;                                               \
        return EXPR;                                                                 \
    }                                                                                \
    template< class T, int N > inline vec< T, N > NAME( const vec< T, N >& a )       \
    {                                                                                \
        vec< T, N > r;                                                               \
        for( int i = 0; i < N; i++ ) r.v[ i ] = NAME( a.v[ i ] );                    \
        return r;                                                                    \
    }
GLSL_UNARY( sqrt, std::sqrt( x ) )
GLSL_UNARY( inversesqrt, 1.0f / std::sqrt( x ) )
GLSL_UNARY( exp, std::exp( x ) )
GLSL_UNARY( exp2, std::exp2( x ) )
GLSL_UNARY( log, std::log( x ) )
GLSL_UNARY( log2, std::log2( x ) )
// GLSL leaves the precision of sin and cos open; this takes the correctly rounded value of the
// binary32 argument (through binary64), as the oracle's normal decoding does
GLSL_UNARY( sin, (fl< T >)std::sin( (double)x ) )
GLSL_UNARY( cos, (fl< T >)std::cos( (double)x ) )
GLSL_UNARY( tan, std::tan( x ) )
GLSL_UNARY( asin, std::asin( x ) )
GLSL_UNARY( acos, std::acos( x ) )
GLSL_UNARY( floor, std::floor( x ) )
GLSL_UNARY( ceil, std::ceil( x ) )
GLSL_UNARY( trunc, std::trunc( x ) )
GLSL_UNARY( round, std::round( x ) )
GLSL_UNARY( fract, x - std::floor( x ) )
GLSL_UNARY( radians, x * 0.017453292519943295f )
#undef GLSL_UNARY

template< class T, typename std::enable_if< is_scalar_v< T >, int >::type = 0 > inline T abs( T x ) { return x < T( 0 ) ? -x : x; }
inline float abs( float x ) { return std::fabs( x ); }
template< class T, int N > inline vec< T, N > abs( const vec< T, N >& a )
{
    vec< T, N > r;
    for( int i = 0; i < N; i++ ) r.v[ i ] = abs( a.v[ i ] );
    return r;
}
template< class T, typename std::enable_if< is_scalar_v< T >, int >::type = 0 > inline T sign( T x )
{
    return x > T( 0 ) ? T( 1 ) : x < T( 0 ) ? T( -1 ) : T( 0 );
}
template< class T, int N > inline vec< T, N > sign( const vec< T, N >& a )
{
    vec< T, N > r;
    for( int i = 0; i < N; i++ ) r.v[ i ] = sign( a.v[ i ] );
    return r;
}
inline float atan( float y, float x ) { return std::atan2( y, x ); }
inline float atan( float x ) { return std::atan( x ); }
template< class A, class B > inline float pow( A x, B y ) { return std::pow( (float)x, (float)y ); }
template< class T, int N > inline vec< T, N > pow( const vec< T, N >& a, const vec< T, N >& b )
{
    vec< T, N > r;
    for( int i = 0; i < N; i++ ) r.v[ i ] = std::pow( a.v[ i ], b.v[ i ] );
    return r;
}
inline float mod( float x, float y ) { return x - y * std::floor( x / y ); }
template< int N > inline vec< float, N > mod( const vec< float, N >& a, float y )
{
    vec< float, N > r;
    for( int i = 0; i < N; i++ ) r.v[ i ] = mod( a.v[ i ], y );
    return r;
}
template< int N > inline vec< float, N > mod( const vec< float, N >& a, const vec< float, N >& y )
{
    vec< float, N > r;
    for( int i = 0; i < N; i++ ) r.v[ i ] = mod( a.v[ i ], y.v[ i ] );
    return r;
}

// min / max / clamp: the common type of scalars (GLSL converts int literals to the float type)
template< class A, class B > using common = typename std::common_type< A, B >::type;
template< class A, class B, typename std::enable_if< is_scalar_v< A > && is_scalar_v< B >, int >::type = 0 >
inline common< A, B > min( A a, B b )
{
    using C = common< A, B >;
    return (C)b < (C)a ? (C)b : (C)a;
}
template< class A, class B, typename std::enable_if< is_scalar_v< A > && is_scalar_v< B >, int >::type = 0 >
inline common< A, B > max( A a, B b )
{
    using C = common< A, B >;
    return (C)a < (C)b ? (C)b : (C)a;
}
inline float min( float a, float b ) { return std::fmin( a, b ); }
inline float max( float a, float b ) { return std::fmax( a, b ); }
template< class T, int N > inline vec< T, N > min( const vec< T, N >& a, const vec< T, N >& b )
{
    vec< T, N > r;
    for( int i = 0; i < N; i++ ) r.v[ i ] = min( a.v[ i ], b.v[ i ] );
    return r;
}
template< class T, int N > inline vec< T, N > max( const vec< T, N >& a, const vec< T, N >& b )
{
    vec< T, N > r;
    for( int i = 0; i < N; i++ ) r.v[ i ] = max( a.v[ i ], b.v[ i ] );
    return r;
}
template< class T, int N, class S, typename std::enable_if< is_scalar_v< S >, int >::type = 0 >
inline vec< T, N > min( const vec< T, N >& a, S s ) { return min( a, vec< T, N >( s ) ); }
template< class T, int N, class S, typename std::enable_if< is_scalar_v< S >, int >::type = 0 >
inline vec< T, N > max( const vec< T, N >& a, S s ) { return max( a, vec< T, N >( s ) ); }
template< class X, class L, class H, typename std::enable_if< is_scalar_v< X >, int >::type = 0 >
inline common< X, common< L, H > > clamp( X x, L lo, H hi )
{
    return min( max( x, lo ), hi );
}
template< class T, int N > inline vec< T, N > clamp( const vec< T, N >& x, const vec< T, N >& lo, const vec< T, N >& hi )
{
    return min( max( x, lo ), hi );
}
template< class T, int N, class L, class H, typename std::enable_if< is_scalar_v< L > && is_scalar_v< H >, int >::type = 0 >
inline vec< T, N > clamp( const vec< T, N >& x, L lo, H hi )
{
    return min( max( x, vec< T, N >( lo ) ), vec< T, N >( hi ) );
}

// mix(x, y, a) = x * (1 - a) + y * a (GLSL's definition, binary32, no contraction)
template< class A, class B, class C, typename std::enable_if< is_scalar_v< A > && is_scalar_v< C >, int >::type = 0 >
inline float mix( A x, B y, C a )
{
    return (float)x * ( 1.0f - (float)a ) + (float)y * (float)a;
}
template< class T, int N, class C, typename std::enable_if< is_scalar_v< C >, int >::type = 0 >
inline vec< T, N > mix( const vec< T, N >& x, const vec< T, N >& y, C a )
{
    vec< T, N > r;
    for( int i = 0; i < N; i++ ) r.v[ i ] = x.v[ i ] * ( T( 1 ) - (T)a ) + y.v[ i ] * (T)a;
    return r;
}
template< class T, int N > inline vec< T, N > mix( const vec< T, N >& x, const vec< T, N >& y, const vec< T, N >& a )
{
    vec< T, N > r;
    for( int i = 0; i < N; i++ ) r.v[ i ] = x.v[ i ] * ( T( 1 ) - a.v[ i ] ) + y.v[ i ] * a.v[ i ];
    return r;
}
template< class T, int N > inline vec< T, N > mix( const vec< T, N >& x, const vec< T, N >& y, const vec< bool, N >& a )
{
    vec< T, N > r;
    for( int i = 0; i < N; i++ ) r.v[ i ] = a.v[ i ] ? y.v[ i ] : x.v[ i ];
    return r;
}
inline float step( float edge, float x ) { return x < edge ? 0.0f : 1.0f; }
inline float smoothstep( float e0, float e1, float x )
{
    const float t = clamp( ( x - e0 ) / ( e1 - e0 ), 0.0f, 1.0f );
    return t * t * ( 3.0f - 2.0f * t );
}

template< int N > inline float dot( const vec< float, N >& a, const vec< float, N >& b )
{
    float s = a.v[ 0 ] * b.v[ 0 ];
    for( int i = 1; i < N; i++ ) s = s + a.v[ i ] * b.v[ i ];
    return s;
}
inline vec3 cross( const vec3& a, const vec3& b )
{
    return vec3( a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y );
}
template< int N > inline float length( const vec< float, N >& a ) { return std::sqrt( dot( a, a ) ); }
inline float length( float a ) { return std::fabs( a ); }
template< int N > inline float distance( const vec< float, N >& a, const vec< float, N >& b ) { return length( a - b ); }
template< int N > inline vec< float, N > normalize( const vec< float, N >& a ) { return a / length( a ); }
inline vec3 reflect( const vec3& i, const vec3& n ) { return i - 2.0f * dot( n, i ) * n; }

inline bool isnan( float x ) { return std::isnan( x ); }
inline bool isinf( float x ) { return std::isinf( x ); }
template< int N > inline vec< bool, N > isnan( const vec< float, N >& a )
{
    vec< bool, N > r;
    for( int i = 0; i < N; i++ ) r.v[ i ] = std::isnan( a.v[ i ] );
    return r;
}
template< int N > inline vec< bool, N > isinf( const vec< float, N >& a )
{
    vec< bool, N > r;
    for( int i = 0; i < N; i++ ) r.v[ i ] = std::isinf( a.v[ i ] );
    return r;
}
template< int N > inline bool any( const vec< bool, N >& a )
{
    for( int i = 0; i < N; i++ )
        if( a.v[ i ] ) return true;
    return false;
}
template< int N > inline bool all( const vec< bool, N >& a )
{
    for( int i = 0; i < N; i++ )
        if( !a.v[ i ] ) return false;
    return true;
}
#define GLSL_CMP( NAME, OP )                                                              \
    template< class T, int N > inline vec< bool, N > NAME( const vec< T, N >& a, const vec< T, N >& b ) \
    {                                                                                     \
        vec< bool, N > r;                                                                 \
        for( int i = 0; i < N; i++ ) r.v[ i ] = a.v[ i ] OP b.v[ i ];                     \
        return r;                                                                         \
    }
GLSL_CMP( lessThan, < )
GLSL_CMP( lessThanEqual, <= )
GLSL_CMP( greaterThan, > )
GLSL_CMP( greaterThanEqual, >= )
GLSL_CMP( equal, == )
GLSL_CMP( notEqual, != )
#undef GLSL_CMP

inline uint  floatBitsToUint( float f ) { uint u; std::memcpy( &u, &f, 4 ); return u; }
inline int   floatBitsToInt( float f ) { int u; std::memcpy( &u, &f, 4 ); return u; }
inline float uintBitsToFloat( uint u ) { float f; std::memcpy( &f, &u, 4 ); return f; }
inline float intBitsToFloat( int u ) { float f; std::memcpy( &f, &u, 4 ); return f; }
template< int N > inline vec< uint, N > floatBitsToUint( const vec< float, N >& a )
{
    vec< uint, N > r;
    for( int i = 0; i < N; i++ ) r.v[ i ] = floatBitsToUint( a.v[ i ] );
    return r;
}
template< int N > inline vec< float, N > uintBitsToFloat( const vec< uint, N >& a )
{
    vec< float, N > r;
    for( int i = 0; i < N; i++ ) r.v[ i ] = uintBitsToFloat( a.v[ i ] );
    return r;
}

// binary16 <-> binary32, round to nearest even (packHalf2x16, the 16-bit float formats)
uint16_t f32_to_f16( float f );
float    f16_to_f32( uint16_t h );
inline uint packHalf2x16( const vec2& v ) { return (uint)f32_to_f16( v.x ) | ( (uint)f32_to_f16( v.y ) << 16 ); }
inline vec2 unpackHalf2x16( uint u ) { return vec2( f16_to_f32( (uint16_t)( u & 0xFFFFu ) ), f16_to_f32( (uint16_t)( u >> 16 ) ) ); }
inline uint packUnorm4x8( const vec4& v )
{
    uint r = 0;
    for( int i = 0; i < 4; i++ ) r |= (uint)std::round( clamp( v.v[ i ], 0.0f, 1.0f ) * 255.0f ) << ( 8 * i );
    return r;
}
inline vec4 unpackUnorm4x8( uint u )
{
    return vec4( ( u & 0xFFu ) / 255.0f, ( ( u >> 8 ) & 0xFFu ) / 255.0f, ( ( u >> 16 ) & 0xFFu ) / 255.0f, ( u >> 24 ) / 255.0f );
}
inline uint bitfieldExtract( uint v, int off, int bits ) { return bits == 32 ? v : ( v >> off ) & ( ( 1u << bits ) - 1u ); }
inline uint bitfieldInsert( uint base, uint ins, int off, int bits )
{
    const uint m = bits == 32 ? 0xFFFFFFFFu : ( ( 1u << bits ) - 1u ) << off;
    return ( base & ~m ) | ( ( ins << off ) & m );
}

// atomics on buffer and shared memory (one invocation runs at a time)
template< class T, class U > inline T atomicAdd( T& mem, U v )
{
    const T old = mem;
    mem         = mem + (T)v;
    return old;
}
template< class T, class U > inline T atomicMax( T& mem, U v )
{
    const T old = mem;
    mem         = mem < (T)v ? (T)v : mem;
    return old;
}

// ------------------------------------------------------------------------------------------
// images and samplers over host planes
// ------------------------------------------------------------------------------------------
enum Fmt
{
    FMT_r8, FMT_rg8, FMT_rgba8, FMT_r16f, FMT_rg16f, FMT_rgba16f, FMT_r32f, FMT_rg32f, FMT_rgba32f,
    FMT_r8ui, FMT_r16ui, FMT_r32ui, FMT_rg32ui, FMT_rgba32ui, FMT_r11f_g11f_b10f, FMT_none
};
int fmt_bytes( int fmt );

struct Plane
{
    uint8_t* data = nullptr;
    int      w = 0, h = 0, fmt = FMT_none;
    int      d = 1;   // depth of a 3-D image: slices of w x h texels, z-major
};
std::map< std::string, Plane >& planes();   // by image name, shared by every shader of the library
std::map< std::string, int >&   formats();  // the format each image is declared with

struct ImageBase
{
    const char* name;
    int         fmt;
    Plane*      p = nullptr;
    ImageBase( const char* n, int f ) : name( n ), fmt( f ) { formats()[ n ] = f; }
    Plane& plane()
    {
        if( !p ) p = &planes()[ name ];
        return *p;
    }
};
struct image2D : ImageBase { using ImageBase::ImageBase; };
struct uimage2D : ImageBase { using ImageBase::ImageBase; };
struct iimage2D : ImageBase { using ImageBase::ImageBase; };
// a sampler reads the plane of the image its name extends ("framebufX_Sampler" -> "framebufX")
struct SamplerBase
{
    std::string base;
    Plane*      p = nullptr;
    explicit SamplerBase( const char* n ) : base( n )
    {
        const size_t k = base.rfind( "_Sampler" );
        if( k != std::string::npos ) base.erase( k, 8 );
    }
    Plane& plane()
    {
        if( !p ) p = &planes()[ base ];
        return *p;
    }
};
struct sampler2D : SamplerBase { using SamplerBase::SamplerBase; };
struct usampler2D : SamplerBase { using SamplerBase::SamplerBase; };
struct isampler2D : SamplerBase { using SamplerBase::SamplerBase; };
struct image3D : ImageBase { using ImageBase::ImageBase; };
struct sampler3D : SamplerBase { using SamplerBase::SamplerBase; };
// declared for the blue-noise array of Random.h, which the shaders run here do not read
struct texture2DArray : SamplerBase { using SamplerBase::SamplerBase; };
// the texture table (globalTextures[]): every element an unbound sampler (zero texels, size 0)
struct SamplerTable
{
    sampler2D none{ "" };
    sampler2D& operator[]( uint ) { return none; }
    sampler2D& operator[]( int ) { return none; }
};
template< class T > inline T nonuniformEXT( T i ) { return i; }

// texel load / store in the plane's format (outside the plane: zero on load, dropped on store)
vec4  load_f( Plane& p, ivec2 pix );
uvec4 load_u( Plane& p, ivec2 pix );
void  store_f( Plane& p, ivec2 pix, const vec4& v );
void  store_u( Plane& p, ivec2 pix, const uvec4& v );

inline vec4  imageLoad( image2D& im, const ivec2& pix ) { return load_f( im.plane(), pix ); }
inline uvec4 imageLoad( uimage2D& im, const ivec2& pix ) { return load_u( im.plane(), pix ); }
inline void  imageStore( image2D& im, const ivec2& pix, const vec4& v ) { store_f( im.plane(), pix, v ); }
inline void  imageStore( uimage2D& im, const ivec2& pix, const uvec4& v ) { store_u( im.plane(), pix, v ); }
inline vec4  texelFetch( sampler2D& s, const ivec2& pix, int ) { return load_f( s.plane(), pix ); }
inline uvec4 texelFetch( usampler2D& s, const ivec2& pix, int ) { return load_u( s.plane(), pix ); }
// Filtered reads: the framebuffers' sampler is bilinear with clamp-to-edge addressing. GLSL and
// Vulkan leave the weights' precision to the device (subTexelPrecisionBits); this takes them
// exactly in binary32: x = u w - 1/2, the texels floor(x) and floor(x) + 1 clamped to the edge,
// the weight x - floor(x), mix(x, y, a) = x (1 - a) + y a, rows first. Only LOD 0 is read.
vec4 bilinear( Plane& p, const vec2& uv );
inline vec4 textureLod( sampler2D& s, const vec2& uv, float ) { return bilinear( s.plane(), uv ); }
// the images here have one mip level, so an explicit gradient selects LOD 0 as well
inline vec4 textureGrad( sampler2D& s, const vec2& uv, const vec2&, const vec2& ) { return bilinear( s.plane(), uv ); }
// 3-D images: texel (x, y, z) of a w x h x d image; outside it, zero on load and dropped on store
vec4 load_f3( Plane& p, ivec3 c );
void store_f3( Plane& p, ivec3 c, const vec4& v );
inline vec4 imageLoad( image3D& im, const ivec3& c ) { return load_f3( im.plane(), c ); }
inline void imageStore( image3D& im, const ivec3& c, const vec4& v ) { store_f3( im.plane(), c, v ); }
inline vec4 texelFetch( sampler3D& s, const ivec3& c, int ) { return load_f3( s.plane(), c ); }
inline vec4 texelFetch( texture2DArray&, const ivec3&, int ) { return vec4( 0.0f ); }
// Linear filtering of a 3-D image with clamp-to-edge addressing, the weights exactly in
// binary32 as bilinear() takes them: along x, then y, then z.
vec4 trilinear( Plane& p, const vec3& uvw );
inline vec4 textureLod( sampler3D& s, const vec3& uvw, float ) { return trilinear( s.plane(), uvw ); }
inline vec4 texture( sampler2D& s, const vec2& uv ) { return bilinear( s.plane(), uv ); }
inline ivec2 imageSize( ImageBase& im ) { return ivec2( im.plane().w, im.plane().h ); }
inline ivec2 textureSize( SamplerBase& s, int ) { return ivec2( s.plane().w, s.plane().h ); }

// ------------------------------------------------------------------------------------------
// compute built-ins, dispatch and barriers
// ------------------------------------------------------------------------------------------
struct Invocation
{
    uvec3      gid, lid, wg;
    uint       lindex = 0;
    ucontext_t ctx;
    bool       done = false;
};
extern thread_local Invocation* g_inv;
void barrier();
inline void groupMemoryBarrier() { barrier(); }
inline void memoryBarrierShared() { barrier(); }
inline void memoryBarrier() {}

// runs `entry` over groups (gx, gy, gz) of (lx, ly, lz) invocations; `fibers`: barrier() in use
void dispatch( void ( *entry )(), uvec3 groups, uvec3 local, bool fibers );

}  // namespace glsl

#define gl_GlobalInvocationID ( glsl::g_inv->gid )
#define gl_LocalInvocationID ( glsl::g_inv->lid )
#define gl_WorkGroupID ( glsl::g_inv->wg )
#define gl_LocalInvocationIndex ( glsl::g_inv->lindex )

// declarations the build script writes for layout-qualified GLSL declarations
#define GLSL_IMAGE( TYPE, NAME, FMT ) static glsl::TYPE NAME( #NAME, glsl::FMT_##FMT )
#define GLSL_SAMPLER( TYPE, NAME ) static glsl::TYPE NAME( #NAME )
