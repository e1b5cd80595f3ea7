// Procedural scene generator: the synthetic stand-in for RayTracedGL1's path tracer, which
// produces the denoiser's G-buffer and noisy demodulated radiance (RaygenPrimary.inl:326-347,
// RtRaygenDirect.rgen:59-67). The reference ships no captured frames, so every input of the
// denoise-and-expose path is drawn here: analytic spheres and planes are ray-cast per pixel in
// the reference's checkerboard layout and written in the reference's framebuffer formats.
//
//   * camera translating `cameraPxPerFrame` pixels per frame (measured at the focus depth);
//   * one sphere moving `spherePxPerFrame` pixels per frame for disocclusions;
//   * noisy direct / specular / indirect radiance: analytic shading x exp(N(0, sigma)) per
//     channel, with fireflies (probability `fireflyProb`, x `fireflyMult`);
//   * GradientInputs = (lum direct, lum specular) of the noisy samples (RtRaygenDirect.rgen:66);
//   * GradientReshaded = the previous frame's samples re-lit by this frame's light intensity
//     (the analytic value of RtGradients.rgen:107-136's forwardProjectedLuminance);
//   * frame parameters (matrices, camera positions, time step, tonemapping range) as
//     VulkanDevice::FillUniform fills them (VulkanDevice.cpp:142-300).
//
// Randomness is counter-based (a hash of seed, frame, pixel, channel): any frame can be
// generated independently, in parallel, with identical results.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

#include "../../include/rgdn.h"
#include "rgdn_codec.h"

namespace
{

struct D3
{
    double x, y, z;
};
inline D3     operator+( D3 a, D3 b ) { return { a.x + b.x, a.y + b.y, a.z + b.z }; }
inline D3     operator-( D3 a, D3 b ) { return { a.x - b.x, a.y - b.y, a.z - b.z }; }
inline D3     operator*( D3 a, double s ) { return { a.x * s, a.y * s, a.z * s }; }
inline double dot( D3 a, D3 b ) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double len( D3 a ) { return std::sqrt( dot( a, a ) ); }
inline D3     nrm( D3 a ) { double l = len( a ); return { a.x / l, a.y / l, a.z / l }; }

// splitmix64 finaliser: a counter-based hash
inline uint64_t mix64( uint64_t z )
{
    z += 0x9E3779B97F4A7C15ull;
    z = ( z ^ ( z >> 30 ) ) * 0xBF58476D1CE4E5B9ull;
    z = ( z ^ ( z >> 27 ) ) * 0x94D049BB133111EBull;
    return z ^ ( z >> 31 );
}
inline double u01( uint64_t h ) { return ( (double)( h >> 11 ) + 0.5 ) * ( 1.0 / 9007199254740992.0 ); }
inline double gauss( uint64_t h1, uint64_t h2 )
{
    return std::sqrt( -2.0 * std::log( u01( h1 ) ) ) * std::cos( 6.283185307179586 * u01( h2 ) );
}

struct Material
{
    D3     albedo;
    double metallic, roughness;
};

struct Hit
{
    bool   hit = false;
    double t   = 1e30;
    D3     p{}, n{};
    int    mat = -1;
    int    obj = -1;
};

// Vulkan-style projection of the reference (Matrix.cpp:380-395), column-major
void make_projection( float* m, float aspect, float fovY, float zn, float zf )
{
    const float th = tanf( fovY * 0.5f );
    memset( m, 0, 16 * sizeof( float ) );
    m[ 0 ]  = 1.0f / ( aspect * th );
    m[ 5 ]  = -1.0f / th;
    m[ 10 ] = zf / ( zn - zf );
    m[ 11 ] = -1.0f;
    m[ 14 ] = ( zf * zn ) / ( zn - zf );
}

// view matrix of a camera at `eye` looking along -z (no rotation), column-major
void make_view( float* m, D3 eye )
{
    memset( m, 0, 16 * sizeof( float ) );
    m[ 0 ] = m[ 5 ] = m[ 10 ] = m[ 15 ] = 1.0f;
    m[ 12 ] = (float)-eye.x;
    m[ 13 ] = (float)-eye.y;
    m[ 14 ] = (float)-eye.z;
}

}  // namespace

extern "C" {

// Scene description (all fields have defaults through rgdn_scene_desc_default)
typedef struct rgdn_scene_desc
{
    uint64_t seed;
    float    sigma;            // log-normal sigma of the radiance noise
    float    fireflyProb;      // probability of a firefly sample
    float    fireflyMult;      // firefly multiplier
    float    cameraPxPerFrame; // horizontal camera motion, in pixels per frame at the focus depth
    float    spherePxPerFrame; // motion of the moving sphere, pixels per frame (0 = none)
    float    timeDelta;        // seconds per frame
    float    ev100Min, ev100Max;
    float    lightFlickerFrom; // frame index from which the light is brighter (antilag test), <0 = never
    float    lightFlickerGain;
    uint32_t atrousIterations;
    uint32_t antiFirefly;
    uint32_t reshadeLights;    // 1: GradientInputs from a sphere light shaded as the reference's direct
                               // pass does (so the device re-shading reproduces them), and reservoirs
} rgdn_scene_desc;

void rgdn_scene_desc_default( rgdn_scene_desc* d )
{
    d->seed             = 1;
    d->sigma            = 1.0f;
    d->fireflyProb      = 0.001f;
    d->fireflyMult      = 100.0f;
    d->cameraPxPerFrame = 2.0f;
    d->spherePxPerFrame = 8.0f;
    d->timeDelta        = 1.0f / 60.0f;
    d->ev100Min         = 0.0f;
    d->ev100Max         = 10.0f;
    d->lightFlickerFrom = 20.0f;
    d->lightFlickerGain = 2.0f;
    d->atrousIterations = 4;
    d->antiFirefly      = 1;
    d->reshadeLights    = 0;
}

struct rgdn_scene
{
    uint32_t        W, H;
    rgdn_scene_desc d;
    float           proj[ 16 ];
    double          fovY = 60.0 * M_PI / 180.0;
    double          focusDepth = 7.0;
};

rgdn_scene* rgdn_scene_create( uint32_t width, uint32_t height, const rgdn_scene_desc* desc )
{
    if( width < 2 || height < 1 || ( width & 1 ) ) return nullptr;
    auto* s = new rgdn_scene();
    s->W    = width;
    s->H    = height;
    if( desc ) s->d = *desc;
    else rgdn_scene_desc_default( &s->d );
    make_projection( s->proj, (float)width / (float)height, (float)s->fovY, 0.1f, 10000.0f );
    return s;
}

void rgdn_scene_destroy( rgdn_scene* s ) { delete s; }

}  // extern "C"

namespace
{

// camera x offset for frame f: cameraPxPerFrame pixels of image motion at focusDepth
D3 camera_eye( const rgdn_scene* s, double f )
{
    const double tanh = std::tan( s->fovY * 0.5 );
    const double aspect = (double)s->W / (double)s->H;
    const double dxPerPx = 2.0 * aspect * tanh * s->focusDepth / (double)s->W;
    return { -3.0 + f * s->d.cameraPxPerFrame * dxPerPx, 1.6, 6.0 };
}

D3 moving_sphere_center( const rgdn_scene* s, double f )
{
    const double tanh = std::tan( s->fovY * 0.5 );
    const double aspect = (double)s->W / (double)s->H;
    const double depth  = 6.0 + 3.0;   // camera z 6, sphere z -3
    const double dxPerPx = 2.0 * aspect * tanh * depth / (double)s->W;
    double x = -4.0 + std::fmod( f * s->d.spherePxPerFrame * dxPerPx, 9.0 );
    return { x, 1.2, -3.0 };
}

double light_gain( const rgdn_scene* s, int frame )
{
    return ( s->d.lightFlickerFrom >= 0.0f && frame >= (int)s->d.lightFlickerFrom ) ? (double)s->d.lightFlickerGain : 1.0;
}

const Material kMaterials[] = {
    { { 0.60, 0.60, 0.58 }, 0.0, 0.80 },  // ground
    { { 0.55, 0.32, 0.22 }, 0.0, 0.60 },  // back wall
    { { 0.90, 0.70, 0.30 }, 1.0, 0.20 },  // gold sphere
    { { 0.20, 0.40, 0.80 }, 0.0, 0.35 },  // blue sphere
    { { 0.015, 0.015, 0.015 }, 0.0, 0.05 },  // dark glossy sphere (ambient attenuation branch)
    { { 0.80, 0.15, 0.15 }, 0.3, 0.50 },  // moving red sphere
    { { 0.70, 0.75, 0.70 }, 0.0, 1.00 },  // rough box-ish sphere
};

struct SceneAtFrame
{
    D3 spheres[ 5 ];
    double radii[ 5 ];
    int mats[ 5 ];
};

SceneAtFrame scene_at( const rgdn_scene* s, double f )
{
    SceneAtFrame sc;
    sc.spheres[ 0 ] = { -2.0, 1.0, -1.0 }; sc.radii[ 0 ] = 1.0;  sc.mats[ 0 ] = 2;
    sc.spheres[ 1 ] = { 1.5, 0.7, 0.0 };   sc.radii[ 1 ] = 0.7;  sc.mats[ 1 ] = 3;
    sc.spheres[ 2 ] = { 0.0, 0.5, 2.0 };   sc.radii[ 2 ] = 0.5;  sc.mats[ 2 ] = 4;
    sc.spheres[ 3 ] = moving_sphere_center( s, f ); sc.radii[ 3 ] = 0.8; sc.mats[ 3 ] = 5;
    sc.spheres[ 4 ] = { 3.5, 1.5, -4.0 };  sc.radii[ 4 ] = 1.5;  sc.mats[ 4 ] = 6;
    if( s->d.spherePxPerFrame <= 0.0f ) sc.spheres[ 3 ] = { -4.0, 1.2, -3.0 };
    return sc;
}

Hit trace( const SceneAtFrame& sc, D3 o, D3 d )
{
    Hit h;
    // ground plane y = 0
    if( d.y < -1e-9 )
    {
        double t = -o.y / d.y;
        if( t > 1e-4 && t < h.t ) { h.hit = true; h.t = t; h.p = o + d * t; h.n = { 0, 1, 0 }; h.mat = 0; h.obj = 0; }
    }
    // back wall z = -8, x in [-12, 12], y in [0, 6]
    if( d.z < -1e-9 )
    {
        double t = ( -8.0 - o.z ) / d.z;
        D3     p = o + d * t;
        if( t > 1e-4 && t < h.t && std::fabs( p.x ) <= 12.0 && p.y >= 0.0 && p.y <= 6.0 )
        { h.hit = true; h.t = t; h.p = p; h.n = { 0, 0, 1 }; h.mat = 1; h.obj = 1; }
    }
    for( int i = 0; i < 5; i++ )
    {
        D3     oc = o - sc.spheres[ i ];
        double b  = dot( oc, d );
        double c  = dot( oc, oc ) - sc.radii[ i ] * sc.radii[ i ];
        double disc = b * b - c;
        if( disc <= 0 ) continue;
        double t = -b - std::sqrt( disc );
        if( t > 1e-4 && t < h.t )
        {
            h.hit = true; h.t = t; h.p = o + d * t; h.n = nrm( h.p - sc.spheres[ i ] ); h.mat = sc.mats[ i ]; h.obj = 2 + i;
        }
    }
    return h;
}

// column-major mat4 * (p, 1)
void xform( const float* m, D3 p, double out[ 4 ] )
{
    for( int r = 0; r < 4; r++ )
        out[ r ] = (double)m[ 0 + r ] * p.x + (double)m[ 4 + r ] * p.y + (double)m[ 8 + r ] * p.z + (double)m[ 12 + r ];
}

// encodeNormal of Utils.h:108-122, in FP32 like the shader
uint32_t encode_normal( float x, float y, float z )
{
    const float PI    = 3.14159265f;
    float       phi   = acosf( std::max( -1.0f, std::min( 1.0f, z ) ) );
    float       theta = atan2f( y, x );
    theta             = theta < 0 ? theta + 2 * PI : theta;
    uint32_t j        = (uint32_t)roundf( phi * 65535.0f / PI );
    uint32_t k        = ( (uint32_t)roundf( theta * 65536.0f / ( 2 * PI ) ) ) % 65536u;
    return ( j << 16 ) | k;
}

inline double lum( D3 c ) { return 0.2125 * c.x + 0.7154 * c.y + 0.0721 * c.z; }

struct Sample
{
    D3 direct, spec, indir;
};

const D3 kLightPos = { 3.0, 5.0, 2.0 };
// the sphere light of the re-shading scenes: kLightPos, radius 0.25, white of this intensity
// (times the frame's light gain): dw * color / pi matches the point light's 30 / d^2 at range
constexpr double kLightRadius = 0.25, kLightColor = 480.0;

// Random.h hashes (the host twins of the kernels' getRandomSeed / wellonsLowBias32)
uint32_t wellons( uint32_t x )
{
    x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16;
    return x;
}
uint32_t seed_of( int px, int py, uint32_t frame )
{
    const uint32_t M = 0x5bd1e995u;
    uint32_t       src[ 3 ] = { (uint32_t)px, (uint32_t)py, frame }, h[ 3 ] = { 1190494759u, 2147483647u, 3559788179u };
    for( auto& v : src ) { v *= M; v ^= v >> 24; v *= M; }
    for( int k = 0; k < 3; k++ )
        for( auto& v : h ) { v *= M; v ^= src[ k ]; }
    for( auto& v : h ) { v ^= v >> 13; v *= M; v ^= v >> 15; }
    return ( ( h[ 2 ] % 128u ) << 14 ) | ( ( h[ 1 ] % 128u ) << 7 ) | ( h[ 0 ] % 128u );
}


// noisy demodulated radiance of a surface point at frame `frame` for checkerboard pixel `pix`
Sample shade( const rgdn_scene* s, const Hit& h, D3 viewDir, int frame, uint64_t pixId, double gain )
{
    const Material& m = kMaterials[ h.mat ];
    D3     toL  = kLightPos - h.p;
    double dist = len( toL );
    D3     l    = toL * ( 1.0 / dist );
    double nl   = std::max( 0.0, dot( h.n, l ) );
    double I    = 30.0 * gain / ( dist * dist );
    D3     v    = viewDir * -1.0;
    D3     hv   = nrm( l + v );
    double nh   = std::max( 0.0, dot( h.n, hv ) );
    double a    = std::max( 0.02, m.roughness * m.roughness );
    double spec = std::pow( nh, 2.0 / ( a * a ) - 2.0 + 1.0 ) * nl * 0.5;
    double base[ 3 ] = { I * nl, I * spec, 0.25 * ( 0.6 + 0.4 * h.n.y ) * gain };
    Sample out;
    D3*    dst[ 3 ] = { &out.direct, &out.spec, &out.indir };
    const uint64_t key = mix64( s->d.seed ^ mix64( (uint64_t)frame * 0x100000001B3ull + pixId ) );
    for( int sig = 0; sig < 3; sig++ )
    {
        double c[ 3 ];
        uint64_t kf = mix64( key + 101 * (uint64_t)sig );
        bool firefly = u01( mix64( kf + 7 ) ) < (double)s->d.fireflyProb;
        for( int ch = 0; ch < 3; ch++ )
        {
            double z = gauss( mix64( kf + 11 + 2 * (uint64_t)ch ), mix64( kf + 12 + 2 * (uint64_t)ch ) );
            c[ ch ]  = base[ sig ] * std::exp( (double)s->d.sigma * z ) * ( firefly ? (double)s->d.fireflyMult : 1.0 );
        }
        *dst[ sig ] = { c[ 0 ], c[ 1 ], c[ 2 ] };
    }
    return out;
}

// The direct-light sample of RtRaygenDirect for checkerboard pixel (cx, cy) of `frame` at the
// surface (p, n) seen from `eye`: the sphere light's point drawn with the pixel's seed
// (getLightPointRnd), shade() with the Lambertian and Smith-GGX terms, a sample weight of 1
// (the reservoirs written say so) and the shadow ray against the scene; luminances (diffuse,
// specular). In double precision, on the quantised metallic / roughness the G-buffer stores.
void light_sample( const SceneAtFrame& sc, D3 p, D3 n, D3 eye, double metallic, double roughness, int cx, int cy, uint32_t frame,
                   double gain, double out[ 2 ] )
{
    out[ 0 ] = out[ 1 ] = 0.0;
    const double PI  = 3.14159265358979323846;
    const uint32_t rnd = wellons( seed_of( cx, cy, frame ) + 20u );
    const double r1 = (double)( rnd & 0xFFFFu ) / 65535.0 * 0.99, r2 = (double)( rnd >> 16 ) / 65535.0 * 0.99;
    D3           tc = kLightPos - p;
    const double tl = len( tc );
    tc              = tc * ( 1.0 / tl );
    double a = 1.0 - 2.0 * r1, b = std::sqrt( 1.0 - a * a );
    const double phi = 2.0 * PI * r2;
    a *= 0.98; b *= 0.98;
    const D3     ln   = nrm( D3{ -tc.x + b * std::cos( phi ), -tc.y + b * std::sin( phi ), -tc.z + a } );
    const D3     lpos = kLightPos + ln * kLightRadius;
    const double sinT = kLightRadius / std::max( kLightRadius, tl ), cosT = std::sqrt( 1.0 - sinT * sinT );
    const double dw   = 2.0 * PI * ( 1.0 - cosT );
    const D3     l    = nrm( lpos - p );
    const double nl   = dot( n, l );
    if( nl <= 0.0 ) return;
    const D3     v     = nrm( eye - p );
    const double col   = kLightColor * gain;
    const double dif   = dw * nl * col / PI;
    const double alpha = std::max( roughness, 0.005 );
    const double spc   = 0.04 * ( 1.0 - metallic ) + metallic;
    const double F     = spc + ( 1.0 - spc ) * std::pow( 1.0 - nl, 5.0 );
    const D3     h     = nrm( v + l );
    const double nm = std::max( 0.0, dot( n, h ) ), dd = nm * nm * ( alpha * alpha - 1.0 ) + 1.0;
    const double D  = alpha * alpha / PI / ( dd * dd );
    const double nv = std::max( dot( n, v ), 0.0 );
    const double G2 = 0.5 / ( 2.0 * nl * nv * ( 1.0 - alpha ) + ( nl + nv ) * alpha );
    const double spe = dw * nl * col * F * G2 * D;
    // shadow ray from the surface moved towards the viewer, tMin 0.001, up to 0.01 short of the light
    const D3     st = p + v * 0.01;
    D3           dl = lpos - st;
    const double md = len( dl );
    dl              = dl * ( 1.0 / md );
    const Hit hs    = trace( sc, st, dl );
    if( hs.hit && hs.t >= 0.001 && hs.t <= md - 0.01 ) return;
    out[ 0 ] = lum( D3{ dif, dif, dif } );
    out[ 1 ] = lum( D3{ spe, spe, spe } );
}

template< class F > void parallel_rows( int h, int nthreads, F&& fn )
{
    if( nthreads <= 1 )
    {
        for( int y = 0; y < h; y++ ) fn( y );
        return;
    }
    std::atomic< int > next( 0 );
    std::vector< std::thread > ts;
    for( int t = 0; t < nthreads; t++ )
        ts.emplace_back( [ & ]() {
            for( ;; )
            {
                int y = next.fetch_add( 1 );
                if( y >= h ) break;
                fn( y );
            }
        } );
    for( auto& t : ts ) t.join();
}

}  // namespace

extern "C" {

// Host output buffers for one frame, each W*H texels in the reference format of the
// framebuffer named in the comment (checkerboard layout unless noted). NULL = skip.
typedef struct rgdn_scene_frame
{
    uint32_t* albedo;          // RGDN_FB_ALBEDO, B10G11R11, regular layout
    uint8_t*  isSky;           // RGDN_FB_IS_SKY
    uint32_t* normal;          // RGDN_FB_NORMAL
    uint16_t* metallicRoughness; // RGDN_FB_METALLIC_ROUGHNESS, rg8 (x = metallic, y = roughness)
    uint16_t* depthWorld;      // RGDN_FB_DEPTH_WORLD, r16f
    uint16_t* depthGrad;       // RGDN_FB_DEPTH_GRAD, r16f
    uint16_t* motion;          // RGDN_FB_MOTION, rgba16f
    uint32_t* unfilteredDirect;   // E5
    uint32_t* unfilteredSpecular; // E5
    uint32_t* unfilteredIndir;    // E5
    float*    surfacePosition; // rgba32f
    uint16_t* viewDirection;   // rgba16f
    uint16_t* throughput;      // rgba16f
    uint16_t* gradientInputs;  // rg16f
    float*    gradientReshaded;// rg32f, indexed by previous-frame pixel
    uint32_t* reservoirs;      // RGDN_FB_RESERVOIRS, uint32 x4 (written when reshadeLights)
} rgdn_scene_frame;

// Generates frame `frame` into `out` and fills `params` (may be NULL).
int rgdn_scene_generate( const rgdn_scene* s, uint32_t frame, rgdn_scene_frame* out, rgdn_frame_params* params, int nthreads )
{
    if( !s || !out ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    const int    W = (int)s->W, H = (int)s->H, sep = W / 2;
    const double f = (double)frame;
    const D3     eye = camera_eye( s, f ), eyePrev = camera_eye( s, f - 1.0 );
    float        view[ 16 ], viewPrev[ 16 ];
    make_view( view, eye );
    make_view( viewPrev, eyePrev );
    const SceneAtFrame sc = scene_at( s, f ), scPrev = scene_at( s, f - 1.0 );
    const double gainCur = light_gain( s, (int)frame ), gainPrev = light_gain( s, (int)frame - 1 );
    const double tanh = std::tan( s->fovY * 0.5 ), aspect = (double)W / (double)H;

    if( params )
    {
        memset( params, 0, sizeof( *params ) );
        memcpy( params->view, view, sizeof( view ) );
        memcpy( params->viewPrev, viewPrev, sizeof( viewPrev ) );
        memcpy( params->projection, s->proj, sizeof( s->proj ) );
        memcpy( params->projectionPrev, s->proj, sizeof( s->proj ) );
        params->cameraPosition[ 0 ]     = (float)eye.x;
        params->cameraPosition[ 1 ]     = (float)eye.y;
        params->cameraPosition[ 2 ]     = (float)eye.z;
        params->cameraPositionPrev[ 0 ] = (float)eyePrev.x;
        params->cameraPositionPrev[ 1 ] = (float)eyePrev.y;
        params->cameraPositionPrev[ 2 ] = (float)eyePrev.z;
        params->timeDelta               = std::max( s->d.timeDelta, 0.001f );
        // VulkanDevice.cpp:204-210
        float lmin = exp2f( s->d.ev100Min ) * 12.5f / 100.0f;
        float lmax = exp2f( s->d.ev100Max ) * 12.5f / 100.0f;
        params->minLogLuminance        = log2f( lmin );
        params->maxLogLuminance        = log2f( lmax );
        params->stopEyeAdaptation      = 0;
        params->gradientMultDiffuse    = 0.5f;   // DrawFrameInfo.h defaults
        params->gradientMultIndirect   = 0.2f;
        params->gradientMultSpecular   = 0.5f;
        params->antiFireflyEnabled     = s->d.antiFirefly;
        params->lightmapScreenCoverage = 0.0f;
        params->debugShowFlags         = 0;
        params->atrousIterations       = s->d.atrousIterations;
        params->flags                  = 0;
        params->frameId                = frame;
    }

    // primary ray through regular pixel (rx + ox, ry + oy), world space
    auto ray_dir = [ & ]( double rx, double ry ) -> D3 {
        double ndcx = 2.0 * rx / (double)W - 1.0;
        double ndcy = 2.0 * ry / (double)H - 1.0;
        // inverse of the projection above: x_v = ndcx * aspect * tanh, y_v = -ndcy * tanh, z_v = -1
        return nrm( D3{ ndcx * aspect * tanh, -ndcy * tanh, -1.0 } );
    };
    auto project_screen = [ & ]( const float* v, D3 p, double& sx, double& sy, double& clipZ, double& viewLen ) {
        double vs[ 4 ], cs[ 4 ];
        xform( v, p, vs );
        D3 vsp = { vs[ 0 ], vs[ 1 ], vs[ 2 ] };
        xform( s->proj, vsp, cs );
        sx = ( cs[ 0 ] / cs[ 3 ] ) * 0.5 + 0.5;
        sy = ( cs[ 1 ] / cs[ 3 ] ) * 0.5 + 0.5;
        clipZ = cs[ 2 ];
        viewLen = len( vsp );
    };


    parallel_rows( H, nthreads, [ & ]( int y ) {
        for( int cx = 0; cx < W; cx++ )
        {
            const size_t idx   = (size_t)y * W + cx;
            const int    isOdd = cx >= sep ? 1 : 0;
            const int    rx    = ( cx - isOdd * sep ) * 2 + ( isOdd + y ) % 2;
            const size_t ridx  = (size_t)y * W + rx;
            const D3     dir   = ray_dir( rx + 0.5, y + 0.5 );
            const Hit    h     = trace( sc, eye, dir );

            if( !h.hit )
            {
                D3 sky = { 0.35 + 0.25 * std::max( 0.0, dir.y ), 0.55 + 0.2 * std::max( 0.0, dir.y ), 0.95 };
                if( out->albedo ) out->albedo[ ridx ] = rgdn::encode_b10g11r11( (float)sky.x, (float)sky.y, (float)sky.z );
                if( out->isSky ) out->isSky[ idx ] = 1;
                if( out->normal ) out->normal[ idx ] = encode_normal( 0.0f, 0.0f, 0.0f );
                if( out->metallicRoughness ) out->metallicRoughness[ idx ] = 0;
                if( out->depthWorld ) out->depthWorld[ idx ] = rgdn::f32_to_f16( 20000.0f );
                if( out->depthGrad ) out->depthGrad[ idx ] = 0;
                if( out->motion ) { for( int c = 0; c < 4; c++ ) out->motion[ idx * 4 + c ] = 0; }
                if( out->unfilteredDirect ) out->unfilteredDirect[ idx ] = 0;
                if( out->unfilteredSpecular ) out->unfilteredSpecular[ idx ] = 0;
                if( out->unfilteredIndir ) out->unfilteredIndir[ idx ] = 0;
                if( out->surfacePosition ) { for( int c = 0; c < 4; c++ ) out->surfacePosition[ idx * 4 + c ] = 10000000.0f; }
                if( out->viewDirection )
                {
                    out->viewDirection[ idx * 4 + 0 ] = rgdn::f32_to_f16( (float)dir.x );
                    out->viewDirection[ idx * 4 + 1 ] = rgdn::f32_to_f16( (float)dir.y );
                    out->viewDirection[ idx * 4 + 2 ] = rgdn::f32_to_f16( (float)dir.z );
                    out->viewDirection[ idx * 4 + 3 ] = 0;
                }
                if( out->throughput )
                {
                    for( int c = 0; c < 3; c++ ) out->throughput[ idx * 4 + c ] = rgdn::f32_to_f16( 1.0f );
                    out->throughput[ idx * 4 + 3 ] = 0;
                }
                if( out->gradientInputs ) { out->gradientInputs[ idx * 2 ] = 0; out->gradientInputs[ idx * 2 + 1 ] = 0; }
                if( out->reservoirs )
                {
                    out->reservoirs[ idx * 4 + 0 ] = 32767u;   // LIGHT_INDEX_NONE, M 0
                    out->reservoirs[ idx * 4 + 1 ] = out->reservoirs[ idx * 4 + 2 ] = out->reservoirs[ idx * 4 + 3 ] = 0u;
                }
            }
            else
            {
                const Material& m = kMaterials[ h.mat ];
                if( out->albedo ) out->albedo[ ridx ] = rgdn::encode_b10g11r11( (float)m.albedo.x, (float)m.albedo.y, (float)m.albedo.z );
                if( out->isSky ) out->isSky[ idx ] = 0;
                if( out->normal ) out->normal[ idx ] = encode_normal( (float)h.n.x, (float)h.n.y, (float)h.n.z );
                if( out->metallicRoughness )
                    out->metallicRoughness[ idx ] = (uint16_t)( rgdn::f32_to_unorm8( (float)m.metallic ) | ( rgdn::f32_to_unorm8( (float)m.roughness ) << 8 ) );

                double sx, sy, cz, vlen, sxp, syp, czp, vlenp;
                project_screen( view, h.p, sx, sy, cz, vlen );
                // the surface point one frame earlier (the moving sphere carries it along)
                D3 pPrev = h.p;
                if( h.obj == 2 + 3 ) pPrev = h.p - ( sc.spheres[ 3 ] - scPrev.spheres[ 3 ] );
                project_screen( viewPrev, pPrev, sxp, syp, czp, vlenp );
                if( out->depthWorld ) out->depthWorld[ idx ] = rgdn::f32_to_f16( (float)vlen );
                if( out->motion )
                {
                    out->motion[ idx * 4 + 0 ] = rgdn::f32_to_f16( (float)( sxp - sx ) );
                    out->motion[ idx * 4 + 1 ] = rgdn::f32_to_f16( (float)( syp - sy ) );
                    out->motion[ idx * 4 + 2 ] = rgdn::f32_to_f16( (float)( vlenp - vlen ) );
                    out->motion[ idx * 4 + 3 ] = 0;
                }
                if( out->depthGrad )
                {
                    // clip-space depth of the tangent-plane hits of the rays one pixel right / down
                    // (HitInfo.inl:336: gradDepth = (clipZ_AX - clipZ, clipZ_AY - clipZ))
                    double g[ 2 ];
                    for( int a = 0; a < 2; a++ )
                    {
                        D3     d2 = ray_dir( rx + 0.5 + ( a == 0 ? 1.0 : 0.0 ), y + 0.5 + ( a == 1 ? 1.0 : 0.0 ) );
                        double dn = dot( d2, h.n );
                        double t  = std::fabs( dn ) > 1e-9 ? dot( h.p - eye, h.n ) / dn : h.t;
                        D3     p2 = eye + d2 * t;
                        double s2x, s2y, c2, l2;
                        project_screen( view, p2, s2x, s2y, c2, l2 );
                        g[ a ] = c2 - cz;
                    }
                    out->depthGrad[ idx ] = rgdn::f32_to_f16( (float)std::sqrt( g[ 0 ] * g[ 0 ] + g[ 1 ] * g[ 1 ] ) );
                }
                const Sample smp = shade( s, h, dir, (int)frame, idx, gainCur );
                if( out->unfilteredDirect ) out->unfilteredDirect[ idx ] = rgdn::encode_e5( (float)smp.direct.x, (float)smp.direct.y, (float)smp.direct.z );
                if( out->unfilteredSpecular ) out->unfilteredSpecular[ idx ] = rgdn::encode_e5( (float)smp.spec.x, (float)smp.spec.y, (float)smp.spec.z );
                if( out->unfilteredIndir ) out->unfilteredIndir[ idx ] = rgdn::encode_e5( (float)smp.indir.x, (float)smp.indir.y, (float)smp.indir.z );
                if( out->surfacePosition )
                {
                    out->surfacePosition[ idx * 4 + 0 ] = (float)h.p.x;
                    out->surfacePosition[ idx * 4 + 1 ] = (float)h.p.y;
                    out->surfacePosition[ idx * 4 + 2 ] = (float)h.p.z;
                    out->surfacePosition[ idx * 4 + 3 ] = 0.0f;
                }
                if( out->viewDirection )
                {
                    out->viewDirection[ idx * 4 + 0 ] = rgdn::f32_to_f16( (float)dir.x );
                    out->viewDirection[ idx * 4 + 1 ] = rgdn::f32_to_f16( (float)dir.y );
                    out->viewDirection[ idx * 4 + 2 ] = rgdn::f32_to_f16( (float)dir.z );
                    out->viewDirection[ idx * 4 + 3 ] = rgdn::f32_to_f16( (float)len( kLightPos - h.p ) );
                }
                if( out->throughput )
                {
                    for( int c = 0; c < 3; c++ ) out->throughput[ idx * 4 + c ] = rgdn::f32_to_f16( 1.0f );
                    out->throughput[ idx * 4 + 3 ] = 0;
                }
                if( out->gradientInputs )
                {
                    double gl[ 2 ] = { lum( smp.direct ), lum( smp.spec ) };
                    if( s->d.reshadeLights )
                    {
                        // the same quantised metallic / roughness the G-buffer holds
                        const double metal = (double)rgdn::f32_to_unorm8( (float)m.metallic ) / 255.0;
                        const double rough = (double)rgdn::f32_to_unorm8( (float)m.roughness ) / 255.0;
                        light_sample( sc, h.p, h.n, eye, metal, rough, cx, y, frame, gainCur, gl );
                    }
                    out->gradientInputs[ idx * 2 + 0 ] = rgdn::f32_to_f16( (float)gl[ 0 ] );
                    out->gradientInputs[ idx * 2 + 1 ] = rgdn::f32_to_f16( (float)gl[ 1 ] );
                }
                if( out->reservoirs )
                {
                    // light 0 chosen with a weight of 1: targetPdf 1, weightSum 1, M 1
                    out->reservoirs[ idx * 4 + 0 ] = ( 1u << 16 ) | 0u;
                    out->reservoirs[ idx * 4 + 1 ] = out->reservoirs[ idx * 4 + 2 ] = 0x3F800000u;
                    out->reservoirs[ idx * 4 + 3 ] = 0u;
                }
            }

            if( out->gradientReshaded )
            {
                // the same pixel of the previous frame, re-lit with this frame's light intensity
                const Hit hp = trace( scPrev, eyePrev, ray_dir( rx + 0.5, y + 0.5 ) );
                if( hp.hit && frame > 0 )
                {
                    const D3     dp  = ray_dir( rx + 0.5, y + 0.5 );
                    const Sample sp  = shade( s, hp, dp, (int)frame - 1, idx, gainPrev );
                    const double rel = gainCur / gainPrev;
                    // the previous sample's luminance as it was stored (fp16), re-lit
                    float ld = rgdn::f16_to_f32( rgdn::f32_to_f16( (float)lum( sp.direct ) ) );
                    float ls = rgdn::f16_to_f32( rgdn::f32_to_f16( (float)lum( sp.spec ) ) );
                    out->gradientReshaded[ idx * 2 + 0 ] = (float)( ld * rel );
                    out->gradientReshaded[ idx * 2 + 1 ] = (float)( ls * rel );
                }
                else
                {
                    out->gradientReshaded[ idx * 2 + 0 ] = 0.0f;
                    out->gradientReshaded[ idx * 2 + 1 ] = 0.0f;
                }
            }
        }
    } );
    return RGDN_SUCCESS;
}

// The re-shading scene of `frame`: its sphere light (index 0, the previous frame's light 0 maps
// to it) and the analytic occluders (the five spheres at this frame, the ground plane, the back
// wall). Returns the counts; NULL outputs are skipped.
void rgdn_scene_reshade( const rgdn_scene* s, uint32_t frame, rgdn_sphere_light* light, rgdn_occluder* occluders, uint32_t* occluderCount )
{
    if( !s ) return;
    const double gain = light_gain( s, (int)frame );
    if( light )
    {
        memset( light, 0, sizeof( *light ) );
        light->center[ 0 ] = (float)kLightPos.x;
        light->center[ 1 ] = (float)kLightPos.y;
        light->center[ 2 ] = (float)kLightPos.z;
        light->radius      = (float)kLightRadius;
        light->color[ 0 ] = light->color[ 1 ] = light->color[ 2 ] = (float)( kLightColor * gain );
    }
    if( occluders )
    {
        const SceneAtFrame sc = scene_at( s, (double)frame );
        uint32_t           k  = 0;
        for( int i = 0; i < 5; i++, k++ )
        {
            occluders[ k ].type = RGDN_OCCLUDER_SPHERE;
            occluders[ k ].data[ 0 ] = (float)sc.spheres[ i ].x;
            occluders[ k ].data[ 1 ] = (float)sc.spheres[ i ].y;
            occluders[ k ].data[ 2 ] = (float)sc.spheres[ i ].z;
            occluders[ k ].data[ 3 ] = (float)sc.radii[ i ];
            occluders[ k ].data[ 4 ] = occluders[ k ].data[ 5 ] = occluders[ k ].data[ 6 ] = 0.0f;
        }
        const float inf = std::numeric_limits< float >::infinity();
        occluders[ k ].type = RGDN_OCCLUDER_RECT;   // ground y = 0
        const float g[ 7 ] = { 1.0f, 0.0f, -inf, inf, -inf, inf, 0.0f };
        memcpy( occluders[ k ].data, g, sizeof( g ) );
        k++;
        occluders[ k ].type = RGDN_OCCLUDER_RECT;   // back wall z = -8, |x| <= 12, 0 <= y <= 6
        const float w[ 7 ] = { 2.0f, -8.0f, -12.0f, 12.0f, 0.0f, 6.0f, 0.0f };
        memcpy( occluders[ k ].data, w, sizeof( w ) );
        k++;
        if( occluderCount ) *occluderCount = k;
    }
}

}  // extern "C"
