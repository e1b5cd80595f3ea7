// Internal interface between the C ABI host code (rgdn_api.cu) and the stage kernels
// (rgdn_kernels.cuh, instantiated once per storage mode in rgdn_mode_*.cu).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/rgdn.h"

namespace rgdn
{

enum Mode : int
{
    MODE_REF  = RGDN_STORAGE_REF,
    MODE_F32  = RGDN_STORAGE_FP32,
    MODE_F16  = RGDN_STORAGE_FP16,
    MODE_BF16 = RGDN_STORAGE_BF16,
};

constexpr int   STRATA         = 3;        // COMPUTE_ASVGF_STRATA_SIZE (ShaderCommonC.h:150)
constexpr float MAX_RAY_LENGTH = 10000.0f; // MAX_RAY_LENGTH (ShaderCommonC.h:167)
constexpr int   MAX_ATROUS_ITERATIONS = 6;

// ShTonemapping (ShaderCommonC.h:344-348), one per stream, device resident
struct Tonemapping
{
    uint32_t histogram[ 256 ];
    float    avgLuminance;
    uint32_t errorFlags;   // device-side failures (RGDN_DEVICE_ERROR_*)
};

// The subset of ShGlobalUniform (ShaderCommonC.h:209-304) this path reads, plus sizes.
struct Uniform
{
    int      W, H;           // render size (image size)
    int      GW, GH;         // gradient image size ((W+1)/3, (H+1)/3)
    float    rw, rh;         // renderWidth / renderHeight as floats
    float    isx, isy;       // 1 / (renderWidth / 2), 1 / renderHeight (ShaderCommonGLSLFunc.h:273-274)
    float    view[ 16 ], viewPrev[ 16 ], proj[ 16 ], projPrev[ 16 ];
    float    vp[ 16 ], vpPrev[ 16 ];   // proj * view, projPrev * viewPrev (FAST path only)
    float    camPos[ 3 ], camPosPrev[ 3 ];
    float    timeDelta, minLog, maxLog;
    uint32_t stopEyeAdaptation;
    float    gradMultD, gradMultI, gradMultS;
    uint32_t antiFirefly;
    float    lightmapCoverage;
    uint32_t debugFlags;
    uint32_t niter;
    uint32_t flags;
    uint32_t frameId;        // GlobalUniform::frameId (re-shading seeds)
};

// Device addresses of every plane the kernels touch, resolved for one frameIndex
// (cur = frameIndex, prev = frameIndex ^ 1 for double-buffered images). 16-byte aligned and
// sized: the batched kernels copy it into shared memory as int4.
struct alignas( 16 ) FrameArgs
{
    Uniform u;
    // G-buffer (reference formats)
    const uint32_t* albedo;          // B10G11R11, regular layout
    const uint8_t*  isSky;
    const uint32_t* normal;
    const uint32_t* normalPrev;
    const uint16_t* mr;              // rg8: low byte metallic, high byte roughness
    const uint16_t* depth;           // r16f
    const uint16_t* depthPrev;
    const uint16_t* depthGrad;
    const ushort4*  motion;          // rgba16f
    const uint32_t* unfD;
    const uint32_t* unfS;
    const uint32_t* unfI;
    const float4*   surfPos;
    const float4*   surfPosPrev;
    const ushort4*  viewDir;         // rgba16f
    const ushort4*  throughput;      // rgba16f
    const uint32_t* gradInputsPrev;  // rg16f
    const float2*   reshaded;        // rg32f
    // gradient re-shading on the device (null: `reshaded` is the producer's image)
    const rgdn_reshade_scene* rs;
    const uint4*              reservoirsPrev;   // RGBA32_UINT, previous slot
    const uint16_t*           mrPrev;           // metallic-roughness, previous slot
    // outputs
    void*     preFinal;
    uint16_t* histInput;             // r16f, regular layout
    // history / intermediates (mode-dependent element types)
    void*       histLen;
    const void* histLenPrev;
    void*       diffTemp;
    void*       diffAccumColor;
    void*       moments;
    const void* momentsPrev;
    void*       diffHistory;         // DiffColorHistory
    void*       diffPing;
    void*       diffPong;
    float*      varHistory;          // FP32 variance planes (16-bit modes only)
    float*      varPing;
    float*      varPong;
    void*       specAccum;
    const void* specAccumPrev;
    void*       specPing;
    void*       specPong;
    void*       indirAccum;
    const void* indirAccumPrev;
    void*       indirPing;
    void*       indirPong;
    void*       filtVar;
    // gradients, 1/3 resolution, rgba8
    uint32_t*       disPing;
    uint32_t*       disPong;
    uint32_t*       disHist;
    const uint32_t* disHistPrev;
    uint8_t*        gradPrevPix;
    // per-pixel geometry record of the current frame, written by the fused temporal pass:
    // (decoded normal xyz, bits: depth fp16 | metallic-roughness rg8 << 16)
    float4*       geom;
    const float4* geomPrev;   // the previous frame's record (valid when the host says so)
    // tonemapping
    Tonemapping*   tm;
    const uint8_t* binLut;           // 65536-entry fp16 bits -> histogram bin
    // normal decode tables: phi[j] = (sin, cos), theta[k] = (cos, sin)
    const float2* phiTab;
    const float2* thetaTab;
    // pow(1 - k/255, 10) for the 256 unorm8 gradient values k, computed on the device with the
    // powf the exact path calls inline (the same bits): the history-length decay
    const float* decay10;
};

// AMD LPM constants of the 709 -> 709 configuration without shoulder tuning (the ones
// LpmFilter reads with LPM_CONFIG_709_709): saturation powers, contrast, tone scale / bias,
// luma coefficients and their reciprocals, crosstalk.
struct LpmConsts
{
    float saturation[ 3 ], contrast, toneScaleBias[ 2 ], lumaT[ 3 ], rcpLumaT[ 3 ], crosstalk[ 3 ];
};
// LpmSetup (LpmSetupCustom.inl) for ImageComposition::SetupLpmParams' arguments
// (ImageComposition.cpp:384-394): 709 primaries and D65 in and out, no soft gap, hdrMax 256,
// exposure 8 stops, contrast 0.1, shoulder contrast 1.
void lpm_setup_709( const float saturation[ 3 ], const float crosstalk[ 3 ], LpmConsts& out );

// Arguments of the exposure / tonemapping kernel (rgdn_prepare_final), regular pixel layout.
struct FinalArgs
{
    int             W, H;
    float           rw;               // render width as float
    float           lightmapCoverage;
    float           whitePoint, emisMax, bloomEvOffset, bloomThreshold;
    uint32_t        flags;            // RGDN_FINAL_*
    LpmConsts       lpm;
    const void*     preFinal;         // PRE_FINAL (the storage mode's format)
    const uint32_t* screenEmis;       // B10G11R11
    const ushort4*  scattering;       // rgba16f
    const ushort4*  throughput;       // rgba16f, checkerboard layout
    const Tonemapping* tm;
    void*           finalOut;         // PRE_FINAL's format
    void*           bloomOut;
};
// The bloom pyramid's planes: [0] BLOOM_INPUT, [1..8] BLOOM_MIP1..8, [9] BLOOM_RESULT, [10] FINAL
struct BloomArgs
{
    void* planes[ 11 ];
    int   w[ 11 ], h[ 11 ];
    int   W, H;
    float intensity;
};
// 8 downsample launches, 8 upsample launches, the apply
constexpr int BLOOM_LAUNCHES = 17;
// levels of at least this many texels take the wide builds (2x2 quads per thread for the
// upsample, 4 blocks per SM for the downsample)
constexpr long long BLOOM_LARGE_TEXELS = 65536;
cudaError_t launch_bloom_ref( const BloomArgs& b, cudaStream_t s );
cudaError_t launch_bloom_f32( const BloomArgs& b, cudaStream_t s );
cudaError_t launch_bloom_f16( const BloomArgs& b, cudaStream_t s );
cudaError_t launch_bloom_bf16( const BloomArgs& b, cudaStream_t s );
// Volumetric::ProcessScattering: the froxel volume (RGBA16F, nx x (ny * nz) texels, z-major
// slices) integrated in place, then the screen-space accumulation. Fixed formats: the same
// kernels serve every storage mode.
struct ScatterArgs
{
    Uniform        u;                 // W, H, rw, rh, isx, isy
    ushort4*       volume;            // SCATTER_VOLUME[frameIndex], processed in place
    int            nx, ny, nz;
    const ushort4* motion;            // checkerboard layout
    const uint16_t* depth;            // DEPTH_WORLD cur / prev, checkerboard layout
    const uint16_t* depthPrev;
    const uint32_t* normal;           // NORMAL cur / prev, checkerboard layout
    const uint32_t* normalPrev;
    const float*   depthNdc;          // regular layout
    const ushort4* scatterPrev;       // SCATTERING prev, regular layout
    const uint16_t* historyPrev;      // SCATTERING_HISTORY prev, regular layout
    ushort4*       scatterOut;        // SCATTERING cur
    uint16_t*      historyOut;        // SCATTERING_HISTORY cur
    const float2*  phiTab;            // normal decode tables
    const float2*  thetaTab;
    float          invViewProj[ 16 ]; // invView * invProjection, column-major (FP32 on the host)
    float          volumeViewProj[ 16 ];
    float          camPos[ 3 ];
    float          volNear, volFar;
    float          irw, irh, iRange;  // 1 / renderWidth, 1 / renderHeight, 1 / (far - near)
    float          ambient[ 3 ];
    float          density;           // volumeScattering * 0.00005
    float          maxHistoryLength;
    uint32_t       enableType;
    uint32_t       frameId;
    uint32_t       flags;             // RGDN_VOLUME_EXACT_MATH
};
cudaError_t launch_process_scattering( const ScatterArgs& a, cudaStream_t s );
cudaError_t launch_final_ref( const FinalArgs& f, cudaStream_t s );
cudaError_t launch_final_f32( const FinalArgs& f, cudaStream_t s );
cudaError_t launch_final_f16( const FinalArgs& f, cudaStream_t s );
cudaError_t launch_final_bf16( const FinalArgs& f, cudaStream_t s );

// Kernels of the default (fused, fast-math) path, beyond the per-stage rgdn_stage ids.
enum FusedKernel : int
{
    KF_ATROUS_FAST      = 100,   // a-trous iteration with FAST weights
    KF_ATROUS_FAST_HIST = 101,   // last iteration + composition + fused histogram
    KF_TEMPORAL_FAST    = 102,   // temporal accumulation, FAST specular weights
    KF_ANTI_FIREFLY_FAST = 103,  // anti-firefly, packed min/max (exact)
    KF_VARIANCE_FAST     = 104,  // variance reading the geometry record, FAST weights
    KF_ATROUS_EXACT_HIST = 106,  // last iteration + fused histogram, IEEE math
    KF_ATROUS_EXACT      = 107,  // a-trous iteration reading the geometry record, IEEE math
    KF_TEMPORAL_EXACT_GEOM = 108,  // temporal accumulation writing the geometry record, IEEE math
    KF_VARIANCE_EXACT_GEOM = 109,  // variance reading the geometry record, IEEE math
    KF_TEMPORAL_FAST_GP    = 110,  // KF_TEMPORAL_FAST reading the previous frame's geometry record
    KF_TEMPORAL_EXACT_GEOM_GP = 111,
    KF_ATROUS_TMA          = 112,  // TMA-staged a-trous iteration (timing label)
    KF_ATROUS_TMA_HIST     = 113,  // TMA-staged last iteration + fused histogram (timing label)
    KF_PREPARE_FINAL       = 114,  // exposure, tonemapping and bloom input (timing label)
    KF_BLOOM               = 115,  // the bloom pyramid and its application (timing label)
    KF_SCATTER_ACCUM       = 117,  // volume integration + screen-space accumulation (timing label)
    KF_ATROUS_PAIR01       = 122,  // a-trous iterations 0 and 1 in one launch (fusion depth 2)
    KF_AF_VARIANCE_FAST    = 123,  // anti-firefly + variance in one launch, FAST variance weights
    KF_AF_VARIANCE_EXACT   = 124,  // anti-firefly + variance in one launch, IEEE math
    KF_TEMPORAL_FAST_EARLY    = 125,  // KF_TEMPORAL_FAST reading all but the gradient before its wait
    KF_TEMPORAL_FAST_GP_EARLY = 126,  // KF_TEMPORAL_FAST_GP likewise
};

// An address range the launches of this thread mark persisting in L2 while it is set (the
// default path sets it to the frame's geometry record, which every later pass reads per tap)
struct L2Window
{
    void*  ptr   = nullptr;
    size_t bytes = 0;
    float  hit   = 0.0f;
};
inline thread_local L2Window tl_l2window;
// set while a batched step runs frames side by side on several lanes: their windows would
// compete for the same set-aside L2, which measured slower than none
inline thread_local bool tl_l2windowOff = false;

// Launches one stage for one frame. Returns the CUDA error of the launch.
typedef cudaError_t ( *StageLauncher )( const FrameArgs& a, int stage, int iter, cudaStream_t s );

cudaError_t launch_stage_ref( const FrameArgs& a, int stage, int iter, cudaStream_t s );
cudaError_t launch_stage_f32( const FrameArgs& a, int stage, int iter, cudaStream_t s );
cudaError_t launch_stage_f16( const FrameArgs& a, int stage, int iter, cudaStream_t s );
cudaError_t launch_stage_bf16( const FrameArgs& a, int stage, int iter, cudaStream_t s );
// the FAST kernels (KF_ATROUS_FAST, KF_ATROUS_FAST_HIST, KF_VARIANCE_FAST)
cudaError_t launch_fast_ref( const FrameArgs& a, int stage, int iter, cudaStream_t s );
cudaError_t launch_fast_f32( const FrameArgs& a, int stage, int iter, cudaStream_t s );
cudaError_t launch_fast_f16( const FrameArgs& a, int stage, int iter, cudaStream_t s );
cudaError_t launch_fast_bf16( const FrameArgs& a, int stage, int iter, cudaStream_t s );
// Tensor maps of the five images one TMA-staged a-trous iteration reads
struct AtrousMaps
{
    CUtensorMap cv, var, spec, indir, geo;
};

// Rows of the anti-firefly tile (32 columns, 4 rows per thread of a 32 x 8 block; the kernel and
// the batched tile tables agree on it).
__host__ __device__ inline int af_tile_rows( int ) { return 32; }

// Shared-memory staging of one TMA-staged a-trous iteration (kernel and host agree on it).
// The output tile is tw x th pixels (one per thread). Each source plane's tap footprint is one
// box of rw x rh texels (steps up to 8: rows -s..th+s) or three bands of rw x th texels
// (step 16: rows -s, 0, +s), with a column halo sx = s rounded up to 4 texels so every box
// starts on a 16-byte boundary. Planes of 16-byte texels are addressed through 3-D maps
// (4 words x W x H), the others through 2-D maps of 4-byte words, so no box dimension exceeds
// the TMA limit of 256 elements. The kernel keeps two stages of `bytes` each.
struct TmaGeom
{
    int s, sx, tw, th, rw, rh, nb;
    int offCv, offVar, offSpec, offInd, offGeo, bytes;
};
// texel bytes of the staged planes per storage mode: colour+variance, variance plane, colour
struct TmaTexel
{
    int cv, var, col;
};
__host__ __device__ inline TmaTexel tma_texel( int storage )
{
    switch( storage )
    {
        case RGDN_STORAGE_REF: return { 8, 0, 4 };
        case RGDN_STORAGE_FP32: return { 16, 0, 16 };
        default: return { 8, 4, 8 };
    }
}
__host__ __device__ inline int tma_align128( int v ) { return ( v + 127 ) & ~127; }
__host__ __device__ inline TmaGeom tma_geometry( int storage, int iter )
{
    TmaGeom g;
    g.s  = 1 << iter;
    g.sx = ( g.s + 3 ) & ~3;
    g.tw = g.s > 8 ? 64 : 32;
    g.th = g.s > 8 ? 4 : 8;
    g.nb = g.s > 8 ? 3 : 1;
    g.rh = g.s > 8 ? g.th : g.th + 2 * g.s;
    g.rw = g.tw + 2 * g.sx;
    const TmaTexel tx     = tma_texel( storage );
    const int      texels = g.rw * g.rh * g.nb;
    int            off    = 0;
    g.offCv   = off; off = tma_align128( off + texels * tx.cv );
    g.offVar  = off; off = tma_align128( off + texels * tx.var );
    g.offSpec = off; off = tma_align128( off + texels * tx.col );
    g.offInd  = off; off = tma_align128( off + texels * tx.col );
    g.offGeo  = off; off = tma_align128( off + texels * 16 );
    g.bytes   = off;
    return g;
}

// TMA-staged a-trous iteration (FAST weights) with the tensor maps of its sources
// (`maps` points to the kernels' AtrousMaps: 5 CUtensorMap for colour+variance, variance,
// specular, indirect, geometry), and the dynamic shared memory one launch needs
cudaError_t launch_atrous_tma_ref( const FrameArgs& a, int iter, bool hist, const void* maps, cudaStream_t s );
cudaError_t launch_atrous_tma_f32( const FrameArgs& a, int iter, bool hist, const void* maps, cudaStream_t s );
cudaError_t launch_atrous_tma_f16( const FrameArgs& a, int iter, bool hist, const void* maps, cudaStream_t s );
cudaError_t launch_atrous_tma_bf16( const FrameArgs& a, int iter, bool hist, const void* maps, cudaStream_t s );
int atrous_tma_smem( int storage, int iter );
inline bool is_fast_kernel( int stage )
{
    return stage == KF_ATROUS_FAST || stage == KF_ATROUS_FAST_HIST || stage == KF_VARIANCE_FAST || stage == KF_ATROUS_PAIR01 ||
           stage == KF_AF_VARIANCE_FAST || stage == KF_AF_VARIANCE_EXACT;
}

// ------------------------------------------------------------------------------------------
// Batched steps: one persistent launch per stage covers the frames of many streams.
//
// A step's job table (tile tables and every frame's FrameArgs) is copied from pinned host
// memory into one of BATCH_SLOTS __constant__ slots of each kernel module at the head of the
// step. The kernels index their slot with a warp-uniform job index, so the compiler keeps the
// frame arguments in uniform registers and constant-bank operands, as it does for the
// single-frame kernels' parameters, instead of spending per-thread registers on them. A
// captured graph of a step (two copies + the launches) is valid for any set of up to MAX_BATCH
// frames with the same launch sequence.
// ------------------------------------------------------------------------------------------
constexpr int MAX_BATCH   = 32;
constexpr int BATCH_SLOTS = 2;

// tile tables of a step, one per launch kind
enum BatchKind : int
{
    BS_GRADIENT = 0,     // gradient samples and gradient a-trous (over the 1/3-resolution image)
    BS_TEMPORAL,
    BS_ANTI_FIREFLY,
    BS_VARIANCE,
    BS_ATROUS0,          // a-trous iteration i uses BS_ATROUS0 + i
    BS_COUNT = BS_ATROUS0 + MAX_ATROUS_ITERATIONS
};

constexpr uint32_t BATCH_JOB_GEOM_PREV  = 1u;   // the previous frame's geometry record is valid
constexpr uint32_t BATCH_JOB_CLEAR_HIST = 2u;   // discard a histogram no exposure pass consumed

// Tile t of launch kind k belongs to the job j with start[k][j] <= t < start[k][j+1]; a job
// without work in that launch has start[k][j] == start[k][j+1]. A job's tiles run row-major
// over its image, blockDim.x x blockDim.y pixels each.
struct BatchConst
{
    int       n;
    uint32_t  jobFlags[ MAX_BATCH ];
    int       start[ BS_COUNT ][ MAX_BATCH + 1 ];
    FrameArgs jobs[ MAX_BATCH ];
};
static_assert( BATCH_SLOTS * sizeof( BatchConst ) <= 63 * 1024, "the job-table slots must fit the 64 KiB constant bank" );

// One stage of a batched step over constant slot `slot`: `grid` persistent blocks of `block`
// threads (256 in all). Stages: RGDN_STAGE_GRADIENT_SAMPLES, _GRADIENT_ATROUS (iter 0..3),
// _TEMPORAL_ACCUMULATION, _ANTI_FIREFLY, _LUMINANCE_AVG (launch_batch_*) and
// _VARIANCE_ESTIMATION, _ATROUS (launch_batch_fast_*: the FAST translation units). `iter` also
// carries launch variants in its high bits (see launch_batch_t).
cudaError_t launch_batch_ref( int stage, int iter, int slot, dim3 block, int grid, cudaStream_t s );
cudaError_t launch_batch_f32( int stage, int iter, int slot, dim3 block, int grid, cudaStream_t s );
cudaError_t launch_batch_f16( int stage, int iter, int slot, dim3 block, int grid, cudaStream_t s );
cudaError_t launch_batch_bf16( int stage, int iter, int slot, dim3 block, int grid, cudaStream_t s );
cudaError_t launch_batch_fast_ref( int stage, int iter, int slot, dim3 block, int grid, cudaStream_t s );
cudaError_t launch_batch_fast_f32( int stage, int iter, int slot, dim3 block, int grid, cudaStream_t s );
cudaError_t launch_batch_fast_f16( int stage, int iter, int slot, dim3 block, int grid, cudaStream_t s );
cudaError_t launch_batch_fast_bf16( int stage, int iter, int slot, dim3 block, int grid, cudaStream_t s );
// resident blocks per SM of a batched stage's kernel (256-thread blocks), 0 on error
int batch_blocks_per_sm_ref( int stage );
int batch_blocks_per_sm_f32( int stage );
int batch_blocks_per_sm_f16( int stage );
int batch_blocks_per_sm_bf16( int stage );
int batch_blocks_per_sm_fast_ref( int stage );
int batch_blocks_per_sm_fast_f32( int stage );
int batch_blocks_per_sm_fast_f16( int stage );
int batch_blocks_per_sm_fast_bf16( int stage );
// device address of a translation unit's constant slot (the current device), nullptr on error
void* batch_slot_ref( int slot );
void* batch_slot_f32( int slot );
void* batch_slot_f16( int slot );
void* batch_slot_bf16( int slot );
void* batch_slot_fast_ref( int slot );
void* batch_slot_fast_f32( int slot );
void* batch_slot_fast_f16( int slot );
void* batch_slot_fast_bf16( int slot );
inline bool is_batch_fast_stage( int stage ) { return stage == RGDN_STAGE_VARIANCE_ESTIMATION || stage == RGDN_STAGE_ATROUS; }

}  // namespace rgdn
