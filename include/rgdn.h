/*
 * rgdn.h — C ABI of the GB300-native A-SVGF denoiser and luminance-histogram
 * auto-exposure (the image-space "denoise-and-expose" path of RayTracedGL1).
 *
 * Every entry point takes plain pointers and sizes; CUDA streams are passed as
 * `rgdn_cuda_stream` (ABI-identical to `cudaStream_t`, NULL = legacy default
 * stream). No C++ exceptions cross this boundary; every call returns an
 * `rgdn_status`.
 *
 * Mapping onto the reference (paths inside the RayTracedGL1 tree):
 *
 *   RTGL1::Denoiser::Denoise(cmd, frameIndex, uniform)     Source/Denoiser.cpp:64-255
 *       -> rgdn_denoise(stream, frameIndex, params, cudaStream)
 *   RTGL1::PathTracer::CalculateGradientsSamples(...)     Source/PathTracer.cpp:196-219
 *       (image-space part of RtGradients.rgen) is the first stage of rgdn_denoise
 *   RTGL1::Tonemapping::CalculateExposure(cmd, frameIndex, uniform)
 *                                                          Source/Tonemapping.cpp:59-165
 *       -> rgdn_calculate_exposure(stream, frameIndex, params, cudaStream)
 *   RTGL1::Tonemapping::GetDescSet (ShTonemapping SSBO)   Source/Tonemapping.h:36-55
 *       -> rgdn_stream_tonemapping_device / rgdn_get_tonemapping
 *   RTGL1::Framebuffers (images + _Prev swap by frameIndex)
 *                                                          Source/Framebuffers.cpp:34-49,640-699
 *       -> rgdn_stream_* (a stream owns one framebuffer set + history + tonemapping state)
 *   RgResult                                               Include/RTGL1/RTGL1.h:78-94
 *       -> rgdn_status (same numeric values where a code exists in both)
 */
#ifndef RGDN_H_
#define RGDN_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RGDN_API_VERSION 1

/* Status codes. Values 0..13 keep the meaning of RgResult (RTGL1.h:78-94). */
typedef enum rgdn_status
{
    RGDN_SUCCESS                 = 0,  /* RG_RESULT_SUCCESS */
    RGDN_WRONG_INSTANCE          = 3,  /* RG_RESULT_WRONG_INSTANCE: null / destroyed handle */
    RGDN_DEVICE_ERROR            = 5,  /* RG_RESULT_GRAPHICS_API_ERROR: a CUDA call failed */
    RGDN_INTERNAL_ERROR          = 6,  /* RG_RESULT_INTERNAL_ERROR */
    RGDN_WRONG_FUNCTION_CALL     = 10, /* RG_RESULT_WRONG_FUNCTION_CALL */
    RGDN_WRONG_FUNCTION_ARGUMENT = 11, /* RG_RESULT_WRONG_FUNCTION_ARGUMENT */
    RGDN_OUT_OF_BUDGET           = 64, /* admission refused: the memory budget is exhausted */
    RGDN_TIMEOUT                 = 65, /* a bounded host wait ran out */
    RGDN_NOT_READY               = 66, /* asynchronous work still in flight */
} rgdn_status;

/* Storage precision of the denoiser's colour and history buffers.
 * G-buffer inputs always keep the reference formats.
 *   REF  — the reference formats exactly (E5B9G9R9 colour, rgba16f history, rg16f moments)
 *          (Source/Generated/GenerateShaderCommon.py:802-887)
 *   FP32 — fp32 colour / history / moments
 *   FP16 — fp16 colour / history, fp32 moments and fp32 variance
 *   BF16 — bf16 colour / history, fp32 moments and fp32 variance                   */
typedef enum rgdn_storage
{
    RGDN_STORAGE_REF  = 0,
    RGDN_STORAGE_FP32 = 1,
    RGDN_STORAGE_FP16 = 2,
    RGDN_STORAGE_BF16 = 3,
} rgdn_storage;

/* Element formats of framebuffer planes. */
typedef enum rgdn_format
{
    RGDN_FORMAT_NONE = 0,
    RGDN_FORMAT_R8_UINT,          /* 1 B */
    RGDN_FORMAT_RG8_UNORM,        /* 2 B */
    RGDN_FORMAT_RGBA8_UNORM,      /* 4 B */
    RGDN_FORMAT_R16_SFLOAT,       /* 2 B */
    RGDN_FORMAT_RG16_SFLOAT,      /* 4 B */
    RGDN_FORMAT_RGBA16_SFLOAT,    /* 8 B */
    RGDN_FORMAT_RGBA16_BFLOAT,    /* 8 B (bf16 x4) */
    RGDN_FORMAT_R32_SFLOAT,       /* 4 B */
    RGDN_FORMAT_RG32_SFLOAT,      /* 8 B */
    RGDN_FORMAT_RGBA32_SFLOAT,    /* 16 B */
    RGDN_FORMAT_R32_UINT,         /* 4 B */
    RGDN_FORMAT_E5B9G9R9_UFLOAT,  /* 4 B, shared exponent (EXT_texture_shared_exponent) */
    RGDN_FORMAT_B10G11R11_UFLOAT, /* 4 B */
    RGDN_FORMAT_NORMAL_SPHERICAL, /* 4 B, (phi:16 | theta:16) code of Source/Shaders/Utils.h:105-140 */
    RGDN_FORMAT_RGBA32_UINT,      /* 16 B */
} rgdn_format;

/* The framebuffer images of one stream. Names follow the reference's framebuffer
 * table (GenerateShaderCommon.py:802-887). "prev" images (STORE_PREV there) have
 * two physical planes; frameIndex selects the current one, frameIndex^1 is _Prev.
 *
 * Producer-written, current frame (the G-buffer; checkerboarded layout unless noted):   */
typedef enum rgdn_framebuf
{
    RGDN_FB_ALBEDO = 0,               /* B10G11R11, regular (non-checkerboard) pixel layout */
    RGDN_FB_IS_SKY,                   /* R8_UINT */
    RGDN_FB_NORMAL,                   /* NORMAL_SPHERICAL, prev */
    RGDN_FB_METALLIC_ROUGHNESS,       /* RG8_UNORM, prev */
    RGDN_FB_DEPTH_WORLD,              /* R16_SFLOAT, prev */
    RGDN_FB_DEPTH_GRAD,               /* R16_SFLOAT */
    RGDN_FB_MOTION,                   /* RGBA16_SFLOAT: xy cur->prev screen uv, z linear depth delta */
    RGDN_FB_UNFILTERED_DIRECT,        /* E5B9G9R9 */
    RGDN_FB_UNFILTERED_SPECULAR,      /* E5B9G9R9 */
    RGDN_FB_UNFILTERED_INDIR,         /* E5B9G9R9 */
    RGDN_FB_SURFACE_POSITION,         /* RGBA32_SFLOAT, prev */
    RGDN_FB_VIEW_DIRECTION,           /* RGBA16_SFLOAT: xyz ray direction, w hit distance */
    RGDN_FB_THROUGHPUT,               /* RGBA16_SFLOAT */
    RGDN_FB_GRADIENT_INPUTS,          /* RG16_SFLOAT: (lum diffuse, lum specular), prev */
    RGDN_FB_GRADIENT_RESHADED,        /* RG32_SFLOAT: previous-frame surface re-shaded with this
                                         frame's lights, indexed by previous-frame pixel
                                         (RtGradients.rgen:107-136 "forwardProjectedLuminance") */
    /* Outputs */
    RGDN_FB_PRE_FINAL,                /* REF: B10G11R11; FP32: RGBA32F; FP16/BF16: RGBA16F; regular layout */
    RGDN_FB_HISTOGRAM_INPUT,          /* R16_SFLOAT, regular layout */
    /* Denoiser history and intermediates */
    RGDN_FB_ACCUM_HISTORY_LENGTH,     /* prev */
    RGDN_FB_DIFF_TEMPORARY,
    RGDN_FB_DIFF_ACCUM_COLOR,         /* prev */
    RGDN_FB_DIFF_ACCUM_MOMENTS,       /* prev */
    RGDN_FB_DIFF_COLOR_HISTORY,
    RGDN_FB_DIFF_PING_COLOR_AND_VARIANCE,
    RGDN_FB_DIFF_PONG_COLOR_AND_VARIANCE,
    RGDN_FB_SPEC_ACCUM_COLOR,         /* prev */
    RGDN_FB_SPEC_PING_COLOR,
    RGDN_FB_SPEC_PONG_COLOR,
    RGDN_FB_INDIR_ACCUM,              /* prev */
    RGDN_FB_INDIR_PING,
    RGDN_FB_INDIR_PONG,
    RGDN_FB_ATROUS_FILTERED_VARIANCE,
    /* Gradient (A-SVGF) images at 1/3 resolution: ((W+1)/3) x ((H+1)/3) */
    RGDN_FB_DIS_PING_GRADIENT,        /* RGBA8_UNORM */
    RGDN_FB_DIS_PONG_GRADIENT,        /* RGBA8_UNORM */
    RGDN_FB_DIS_GRADIENT_HISTORY,     /* RGBA8_UNORM, prev (double-buffered here; single in the
                                         reference, where sampling reads it before a-trous writes) */
    RGDN_FB_GRADIENT_PREV_PIX,        /* R8_UINT */
    /* FP32 variance planes of the colour+variance images (FP16/BF16 storage only) */
    RGDN_FB_DIFF_COLOR_HISTORY_VARIANCE,
    RGDN_FB_DIFF_PING_VARIANCE,
    RGDN_FB_DIFF_PONG_VARIANCE,
    /* exposure application and tonemapping (rgdn_prepare_final), regular pixel layout */
    RGDN_FB_SCREEN_EMIS_RT,           /* B10G11R11: the producer's screen-space emission */
    RGDN_FB_SCATTERING,               /* RGBA16_SFLOAT: volumetric in-scattering (rgb), transmittance (a);
                                         prev (rgdn_process_scattering accumulates it over frames) */
    RGDN_FB_FINAL,                    /* the exposed, tonemapped image (PRE_FINAL's format) */
    RGDN_FB_BLOOM_INPUT,              /* bloom input (PRE_FINAL's format) */
    /* bloom (rgdn_bloom): mip k is ((W+1) >> k) x ((H+1) >> k), at least 1x1; PRE_FINAL's format */
    RGDN_FB_BLOOM_MIP1,
    RGDN_FB_BLOOM_MIP2,
    RGDN_FB_BLOOM_MIP3,
    RGDN_FB_BLOOM_MIP4,
    RGDN_FB_BLOOM_MIP5,
    RGDN_FB_BLOOM_MIP6,
    RGDN_FB_BLOOM_MIP7,
    RGDN_FB_BLOOM_MIP8,
    RGDN_FB_BLOOM_RESULT,             /* W x H */
    /* volumetric scattering (rgdn_process_scattering) */
    RGDN_FB_DEPTH_NDC,                /* R32_SFLOAT: NDC depth of the primary hit, regular layout */
    RGDN_FB_SCATTERING_HISTORY,       /* R16_SFLOAT: history length of SCATTERING, regular layout, prev */
    RGDN_FB_SCATTER_VOLUME,           /* RGBA16_SFLOAT froxel volume of RGDN_VOLUME_SIZE_X x _Y x _Z
                                         cells as an image of X x (Y * Z) texels, z-major slices
                                         (cell (x, y, z) at row z * Y + y); rgb in-scattered light,
                                         a extinction along the cell; prev (two slots, as the
                                         reference's scattering[2]) */
    /* gradient re-shading on the device (rgdn_stream_set_reshade_scene) */
    RGDN_FB_RESERVOIRS,               /* RGBA32_UINT: the direct-light reservoir of each pixel as
                                         packReservoir stores it (Reservoir.h:116-136): x = M << 16 |
                                         selected light, y = bits of the selected target pdf, z = bits of
                                         the weight sum; prev (the producer writes it every frame) */
    RGDN_FB_COUNT
} rgdn_framebuf;

/* One plane of one framebuffer image. */
typedef struct rgdn_image
{
    void*    data;        /* device pointer (NULL if the image does not exist in this storage mode) */
    uint32_t width;
    uint32_t height;
    uint32_t pitch_bytes; /* row stride */
    uint32_t texel_bytes;
    uint32_t format;      /* rgdn_format */
    uint32_t has_prev;    /* 1 if the image is double-buffered by frameIndex */
} rgdn_image;

/* Per-frame parameters: the fields of ShGlobalUniform (ShaderCommonC.h:209-304)
 * that this path reads, as VulkanDevice::FillUniform fills them
 * (Source/VulkanDevice.cpp:142-300). Matrices are column-major float[16] like the
 * reference's uniform. */
typedef struct rgdn_frame_params
{
    float    view[ 16 ];
    float    viewPrev[ 16 ];
    float    projection[ 16 ];
    float    projectionPrev[ 16 ];
    float    cameraPosition[ 4 ];
    float    cameraPositionPrev[ 4 ];
    float    timeDelta;             /* seconds, >= 0.001 in the reference */
    float    minLogLuminance;       /* log2(2^ev100Min * 12.5 / 100) */
    float    maxLogLuminance;       /* log2(2^ev100Max * 12.5 / 100) */
    uint32_t stopEyeAdaptation;
    float    gradientMultDiffuse;   /* clamped to [0,1] by the caller, as FillUniform does */
    float    gradientMultIndirect;
    float    gradientMultSpecular;
    uint32_t antiFireflyEnabled;
    float    lightmapScreenCoverage;
    uint32_t debugShowFlags;        /* DEBUG_SHOW_FLAG_* of ShaderCommonC.h */
    uint32_t atrousIterations;      /* 0 or 4 = the reference's 4 iterations; 1..6 allowed */
    uint32_t flags;                 /* RGDN_FLAG_* */
    uint32_t frameId;               /* GlobalUniform::frameId: seeds the re-shaded light samples */
} rgdn_frame_params;

/* rgdn_frame_params.flags */
#define RGDN_FLAG_PLAIN              0x1u /* one kernel per reference dispatch, IEEE math (no fusion) */
#define RGDN_FLAG_SKIP_GRADIENTS     0x2u /* GRADIENT_ESTIMATION_ENABLED == 0 behaviour */
#define RGDN_FLAG_EXACT_MATH         0x4u /* fused kernels, but the plain path's IEEE math: the same
                                             results as RGDN_FLAG_PLAIN bit for bit (the default
                                             path uses hardware exp2/log2 for continuous weights) */
#define RGDN_FLAG_TMA_STAGING        0x8u /* a-trous taps staged in shared memory by the Tensor
                                             Memory Accelerator (widths divisible by 4, up to 5
                                             iterations); the same results as the default kernels */
#define RGDN_FLAG_AF_VARIANCE_FUSED  0x20u /* anti-firefly and variance estimation in one launch: each
                                             block keeps its tile's clamped diffuse colours (and
                                             their one-pixel ring) in shared memory for the
                                             variance's 3x3; the same results bit for bit (on
                                             GB300 about 8 % slower than the two launches) */
#define RGDN_FLAG_ATROUS_PAIR        0x40u /* a-trous iterations 0 and 1 in one launch (fusion depth 2,
                                             with 3 or more iterations): iteration 0 over the tile
                                             widened by 2 in shared memory, then iteration 1; the
                                             same results bit for bit */
#define RGDN_FLAG_TEST_TMA_TIMEOUT   0x80000000u /* tests only, with RGDN_FLAG_TMA_STAGING: every stage of
                                             the TMA-staged a-trous expects 16 bytes more than its
                                             copies deliver, so each block's first bounded wait runs
                                             out (after a short limit) with all its copies landed:
                                             the pass sets RGDN_DEVICE_ERROR_TMA_WAIT and leaves its
                                             outputs as they were */
#define RGDN_FLAG_STAGE_DEFAULT      0x10u /* rgdn_denoise_stage runs the default path's kernel for
                                             the stage (with RGDN_FLAG_EXACT_MATH: its IEEE form)
                                             instead of the one-kernel-per-dispatch form; the last
                                             a-trous iteration then also bins the histogram, and
                                             RGDN_STAGE_LUMINANCE_HISTOGRAM does nothing */

/* debugShowFlags bits used on this path (ShaderCommonC.h:156-166) */
#define RGDN_DEBUG_SHOW_FLAG_ONLY_DIRECT_DIFFUSE   ( 1u << 5 )
#define RGDN_DEBUG_SHOW_FLAG_ONLY_SPECULAR         ( 1u << 6 )
#define RGDN_DEBUG_SHOW_FLAG_ONLY_INDIRECT_DIFFUSE ( 1u << 7 )
#define RGDN_DEBUG_SHOW_FLAG_ALBEDO_WHITE          ( 1u << 9 )

/* Individual stages, for the plain path and per-stage checking. */
typedef enum rgdn_stage
{
    RGDN_STAGE_GRADIENT_SAMPLES = 0,  /* RtGradients.rgen:44-181 (image-space part) */
    RGDN_STAGE_GRADIENT_ATROUS,       /* CmASVGFGradientAtrous.comp, iteration 0..3 */
    RGDN_STAGE_TEMPORAL_ACCUMULATION, /* CmSVGFTemporalAccumulation.comp */
    RGDN_STAGE_ANTI_FIREFLY,          /* CmAntiFirefly.comp */
    RGDN_STAGE_VARIANCE_ESTIMATION,   /* CmSVGFEstimateVariance.comp */
    RGDN_STAGE_ATROUS,                /* CmSVGFAtrous_Iter0.comp (0) / CmSVGFAtrous.comp (>=1) */
    RGDN_STAGE_LUMINANCE_HISTOGRAM,   /* CmLuminanceHistogram.comp */
    RGDN_STAGE_LUMINANCE_AVG,         /* CmLuminanceAvg.comp */
    RGDN_STAGE_COUNT
} rgdn_stage;

typedef struct CUstream_st* rgdn_cuda_stream; /* == cudaStream_t */

typedef struct rgdn_context rgdn_context;
typedef struct rgdn_stream  rgdn_stream;

typedef struct rgdn_context_create_info
{
    int      device;               /* CUDA device ordinal */
    uint64_t memoryBudgetBytes;    /* 0 = no budget; stream creation beyond it fails with OUT_OF_BUDGET */
    uint32_t flags;                /* RGDN_CONTEXT_* */
} rgdn_context_create_info;
/* By default a context sets aside up to 48 MB of L2 for persisting accesses (a limit of the
 * process's CUDA context, lifted again when the rgdn context is destroyed), and each frame of
 * the default path marks its geometry record persisting while it runs alone: every later pass
 * reads that record at each tap (on GB300 a 1080p frame took 0.507 against 0.517 ms). A
 * context that runs several frames side by side (batched steps on several lanes, serving)
 * measured about 1 % slower with the set-aside than without; it passes
 * RGDN_CONTEXT_NO_L2_PERSIST. */
#define RGDN_CONTEXT_NO_L2_PERSIST 0x1u

typedef struct rgdn_stream_create_info
{
    uint32_t width;                /* render width, must be even (VulkanDevice.cpp:186-188) */
    uint32_t height;
    uint32_t storage;              /* rgdn_storage */
} rgdn_stream_create_info;

/* ---- context ---------------------------------------------------------------------- */
/* Replaces the Denoiser/Tonemapping constructors (Denoiser.cpp:28-55,
 * Tonemapping.cpp:30-46): selects the device, builds the shared tables. */
rgdn_status rgdn_context_create( const rgdn_context_create_info* info, rgdn_context** outCtx );
rgdn_status rgdn_context_destroy( rgdn_context* ctx );
/* Bytes held by all streams of the context. */
rgdn_status rgdn_context_memory_used( rgdn_context* ctx, uint64_t* outBytes );

/* ---- streams: one camera stream = one framebuffer set + history ------------------- */
/* Framebuffers::PrepareForSize (Framebuffers.cpp:216-230) + Tonemapping buffer creation
 * (Tonemapping.cpp:183-191). All images and the tonemapping state start at zero. */
rgdn_status rgdn_stream_create( rgdn_context* ctx, const rgdn_stream_create_info* info, rgdn_stream** outStream );
rgdn_status rgdn_stream_destroy( rgdn_stream* stream );
/* Reallocates every image at the new size (history is lost, as on a reference resize). */
rgdn_status rgdn_stream_resize( rgdn_stream* stream, uint32_t width, uint32_t height );
/* Bytes a stream of this size and storage needs (for admission control). */
rgdn_status rgdn_stream_required_bytes( const rgdn_stream_create_info* info, uint64_t* outBytes );
/* Framebuffers::GetImageHandles (Framebuffers.cpp:34-49): the plane of `fb` that
 * frameIndex (0 or 1) selects. A producer writes the G-buffer there directly. */
rgdn_status rgdn_stream_get_framebuffer( rgdn_stream* stream, uint32_t fb, uint32_t frameIndex, rgdn_image* outImage );
/* Points a producer-written G-buffer image (RGDN_FB_ALBEDO .. RGDN_FB_GRADIENT_RESHADED,
 * RGDN_FB_SCREEN_EMIS_RT, RGDN_FB_SCATTERING, RGDN_FB_DEPTH_NDC, RGDN_FB_SCATTER_VOLUME) of slot frameIndex at caller-owned device memory (dense rows, 16-byte aligned). An image
 * without a previous-frame slot (no _Prev in the reference) has one binding whatever frameIndex
 * says, so a caller that alternates buffers binds it again before each frame. This lets a renderer
 * that already holds its G-buffer in HBM hand it over without a copy — the role of the
 * reference's shared Framebuffers images (PathTracer writes, Denoiser reads). NULL restores
 * the stream's own plane. The memory must stay valid while work using it is in flight. */
rgdn_status rgdn_stream_bind_framebuffer( rgdn_stream* stream, uint32_t fb, uint32_t frameIndex, void* devicePtr );
/* Copies `bytes` (== pitch*height) into / out of a framebuffer plane; `src`/`dst` may be
 * host (pageable or pinned) or device memory. Enqueued on cudaStream. */
rgdn_status rgdn_stream_upload( rgdn_stream* stream, uint32_t fb, uint32_t frameIndex, const void* src, size_t bytes, rgdn_cuda_stream cudaStream );
rgdn_status rgdn_stream_download( rgdn_stream* stream, uint32_t fb, uint32_t frameIndex, void* dst, size_t bytes, rgdn_cuda_stream cudaStream );

/* ---- the hot path ----------------------------------------------------------------- */
/* Denoiser::Denoise (Denoiser.cpp:64-255) preceded by the image-space gradient sampling
 * of RtGradients.rgen: gradient samples, 4x gradient a-trous, temporal accumulation,
 * anti-firefly, variance, N x a-trous with the final composition into PRE_FINAL and
 * HISTOGRAM_INPUT. Asynchronous on cudaStream. */
rgdn_status rgdn_denoise( rgdn_stream* stream, uint32_t frameIndex, const rgdn_frame_params* params, rgdn_cuda_stream cudaStream );
/* Tonemapping::CalculateExposure (Tonemapping.cpp:59-165): 256-bin log-luminance
 * histogram of HISTOGRAM_INPUT, then the adapted average luminance. */
rgdn_status rgdn_calculate_exposure( rgdn_stream* stream, uint32_t frameIndex, const rgdn_frame_params* params, rgdn_cuda_stream cudaStream );
/* ---- exposure application and tonemapping ------------------------------------------
 * ImageComposition::PrepareForRaster + Finalize (ImageComposition.cpp:87-155) without the
 * rasterised geometry between them, in one kernel per pixel of the regular layout:
 *   CmCheckerboard.comp      PRE_FINAL and SCREEN_EMIS_RT, resolved from their cross
 *                            neighbours where the primary ray was split (THROUGHPUT.a > 0.5)
 *   CmPrepareFinal.comp      volumetric scattering (optional), then finalizeColor: uncharted2
 *                            under classic shading, else exposure (from the stream's adapted
 *                            average luminance) + screen emission through AMD LPM (709 -> 709);
 *                            and the bloom input
 * into FINAL and BLOOM_INPUT. Call after rgdn_calculate_exposure. The debug views of
 * processDebug and the SHIPPING_HACK acid fog are not part of it. */
typedef struct rgdn_final_params
{
    float    luminanceWhitePoint;      /* uncharted2 white point (classic shading); reference default 10 */
    float    emissionMaxScreenColor;   /* screen emission scale; default 1.5 */
    float    bloomEmissionMultiplier;  /* EV offset of screen emission in the bloom input; default 16 */
    float    bloomThreshold;           /* bloom input threshold (inputThreshold); default 4 */
    float    saturation[ 3 ];          /* LPM per-channel saturation (<0 less, >0 more); default 0 */
    float    crosstalk[ 3 ];           /* LPM crosstalk, one channel 1, others in (0, 1]; default 1 */
    float    lightmapScreenCoverage;   /* classic shading where x < coverage * width */
    uint32_t flags;                    /* RGDN_FINAL_* */
} rgdn_final_params;
#define RGDN_FINAL_APPLY_SCATTERING 0x1u /* hdr = hdr * scattering.a + scattering.rgb */
#define RGDN_FINAL_EXACT_MATH       0x2u /* IEEE powf and divisions in the shader's order; the
                                            default evaluates pow as the hardware exp2(y log2 x)
                                            and divides by reciprocal multiplies, as a GPU
                                            compiles the shader */
rgdn_status rgdn_prepare_final( rgdn_stream* stream, uint32_t frameIndex, const rgdn_final_params* params, rgdn_cuda_stream cudaStream );

/* ---- bloom -------------------------------------------------------------------------
 * Bloom::Prepare + Apply (Bloom.cpp:94-240): 8 downsampling steps of BLOOM_INPUT
 * (CmBloomDownsample.comp: 13-tap, partial Karis average on the first) into BLOOM_MIP1..8,
 * 8 upsampling steps (CmBloomUpsample.comp: 3x3 tent, adding each mip's own downsample) into
 * BLOOM_MIP7..1 and BLOOM_RESULT, then FINAL += intensity * BLOOM_RESULT (CmBloomApply.comp,
 * at render size, without the lens-dirt texture term). Bilinear reads are clamp-to-edge in
 * FP32. Call after rgdn_prepare_final. */
typedef struct rgdn_bloom_params
{
    float bloomIntensity;   /* reference default 1 */
} rgdn_bloom_params;
rgdn_status rgdn_bloom( rgdn_stream* stream, uint32_t frameIndex, const rgdn_bloom_params* params, rgdn_cuda_stream cudaStream );

/* ---- volumetric scattering ---------------------------------------------------------
 * Volumetric::ProcessScattering (Volumetric.cpp:71-190), between rgdn_denoise and
 * rgdn_calculate_exposure as VulkanDevice::Render orders them:
 *  1. CmVolumetricProcess.comp: each froxel column of SCATTER_VOLUME[frameIndex] integrated
 *     front to back in place (rgb: light scattered in so far, a: transmittance exp(-sum a));
 *  2. CmScatterAccum.comp: per pixel, the previous SCATTERING reprojected (2x2 bilinear with
 *     the depth and normal tests of the denoiser) and mixed with this frame's value by
 *     1 / history length into SCATTERING and SCATTERING_HISTORY. This frame's value is the
 *     processed volume sampled at the pixel's world position with a hashed dither
 *     (VOLUMETRIC), exponential fog from the ray length (SIMPLE), or (0, 0, 0, 1) (NONE).
 * The froxel illumination that RtVolumetric.rgen traces is an input: the producer writes
 * SCATTER_VOLUME. Matrices are column-major, as GLSL mat4. */
#define RGDN_VOLUME_SIZE_X 160 /* VOLUMETRIC_SIZE_X (ShaderCommonC.h:189-191) */
#define RGDN_VOLUME_SIZE_Y 88
#define RGDN_VOLUME_SIZE_Z 64
#define RGDN_VOLUME_ENABLE_NONE       0u /* VOLUME_ENABLE_* (ShaderCommonC.h:195-197) */
#define RGDN_VOLUME_ENABLE_SIMPLE     1u
#define RGDN_VOLUME_ENABLE_VOLUMETRIC 2u
typedef struct rgdn_volumetric_params
{
    float    invView[ 16 ];          /* GlobalUniform::invView */
    float    invProjection[ 16 ];    /* GlobalUniform::invProjection */
    float    volumeViewProj[ 16 ];   /* GlobalUniform::volumeViewProj */
    float    cameraPosition[ 4 ];    /* xyz */
    float    volumeCameraNear;
    float    volumeCameraFar;        /* > volumeCameraNear */
    float    volumeAmbient[ 3 ];     /* SIMPLE mode fog colour */
    float    volumeScattering;       /* SIMPLE mode density (times 0.00005) */
    float    maxHistoryLength;       /* RgDrawFrameVolumetricParams::maxHistoryLength; 0 after a
                                        history reset */
    uint32_t volumeEnableType;       /* RGDN_VOLUME_ENABLE_* */
    uint32_t frameId;                /* GlobalUniform::frameId: seeds the per-pixel dither */
    uint32_t flags;                  /* RGDN_VOLUME_EXACT_MATH */
} rgdn_volumetric_params;
#define RGDN_VOLUME_EXACT_MATH 0x1u /* IEEE divisions, square roots, sin/cos and exp in the
                                       accumulation; the default uses the hardware reciprocal,
                                       square root, sin/cos and exp2 for its continuous terms
                                       (the reprojection tests decide exactly either way) */
rgdn_status rgdn_process_scattering( rgdn_stream* stream, uint32_t frameIndex, const rgdn_volumetric_params* params, rgdn_cuda_stream cudaStream );

/* ---- gradient re-shading on the device --------------------------------------------------
 * RtGradients.rgen:107-136 re-lights the previous frame's surface at each gradient sample with
 * this frame's lights (processDirectIllumination with the previous frame's reservoir and random
 * seed, a shadow ray against the scene). By default the producer supplies that luminance as
 * RGDN_FB_GRADIENT_RESHADED. With a re-shade scene set, the gradient-samples kernel computes it
 * itself from RGDN_FB_RESERVOIRS (previous slot), the previous slot's SURFACE_POSITION, NORMAL and
 * METALLIC_ROUGHNESS, this frame's sphere lights and the scene's analytic occluders, which stand
 * in for the reference's acceleration structure (no triangle meshes on this path). Every surface
 * counts as matched by the visibility buffer, since analytic surfaces have exact positions. */
typedef struct rgdn_sphere_light
{
    float center[ 3 ];
    float radius;
    float color[ 3 ];
    float pad;
} rgdn_sphere_light;   /* SphereLight (Light.h:31-36), ShLightEncoded's LIGHT_TYPE_SPHERE */

#define RGDN_OCCLUDER_SPHERE 0u   /* data: center xyz, radius */
#define RGDN_OCCLUDER_RECT   1u   /* data: axis (0 = x, 1 = y, 2 = z) as float, plane offset along it,
                                     then min, max of the first and min, max of the second of the
                                     other two coordinates in x, y, z order (data[6] unused): an
                                     axis-aligned rectangle (an unbounded plane with +-inf) */
typedef struct rgdn_occluder
{
    uint32_t type;
    float    data[ 7 ];
} rgdn_occluder;

typedef struct rgdn_reshade_scene
{
    const rgdn_sphere_light* lights;         /* device: this frame's lights (lightSources) */
    uint32_t                 lightCount;
    const uint32_t*          prevToCur;      /* device: lightSources_Index_PrevToCur, prevLightCount
                                                entries; 0xFFFFFFFF = the light is gone */
    uint32_t                 prevLightCount;
    const rgdn_occluder*     occluders;      /* device: shadow-ray geometry */
    uint32_t                 occluderCount;
} rgdn_reshade_scene;

/* Sets (scene != NULL) or clears the re-shade scene of a stream; the arrays must stay valid for
 * every frame denoised with them. The frame's rgdn_frame_params.frameId seeds the samples. */
rgdn_status rgdn_stream_set_reshade_scene( rgdn_stream* stream, const rgdn_reshade_scene* scene );

/* One stage alone (per-stage checking): the plain path's kernel, or with
 * RGDN_FLAG_STAGE_DEFAULT the default path's. `iteration` selects the a-trous or gradient
 * a-trous iteration. */
rgdn_status rgdn_denoise_stage( rgdn_stream* stream, uint32_t stage, uint32_t iteration, uint32_t frameIndex, const rgdn_frame_params* params, rgdn_cuda_stream cudaStream );

/* ShTonemapping { uint histogram[256]; float avgLuminance; } (ShaderCommonC.h:344-348):
 * device address (what Tonemapping::GetDescSet exposes to later passes). */
rgdn_status rgdn_stream_tonemapping_device( rgdn_stream* stream, void** outDevicePtr );
/* Synchronous read of the tonemapping state after the work on cudaStream. `exposure`
 * is ev100ToLuminousExposure(getAutoEV100()) of Exposure.h:33-51. Any out pointer may be NULL. */
rgdn_status rgdn_get_tonemapping( rgdn_stream* stream, uint32_t* outHistogram256, float* outAvgLuminance, float* outExposure, rgdn_cuda_stream cudaStream );
/* Device-side failures of the stream's kernels since the last call, read and cleared after the
 * work on cudaStream (synchronising it). Every wait inside a kernel is bounded; one that runs
 * out sets a bit and lets the kernel finish, so the frames since the last call are unreliable
 * but the device is not hung:
 *   bit 0  a TMA-staged a-trous pass stopped waiting for its copies (RGDN_FLAG_TMA_STAGING) */
#define RGDN_DEVICE_ERROR_TMA_WAIT 1u
rgdn_status rgdn_stream_take_device_errors( rgdn_stream* stream, uint32_t* outFlags, rgdn_cuda_stream cudaStream );
/* Asynchronous copy, in cudaStream order, of { uint histogram[256]; float avgLuminance; }
 * (1028 bytes) to dst (host, pinned for overlap, or device). No reference counterpart: later
 * passes of the reference read the SSBO on the GPU. */
rgdn_status rgdn_stream_copy_tonemapping( rgdn_stream* stream, void* dst, rgdn_cuda_stream cudaStream );
/* Overwrites the tonemapping state (test fixtures, stream migration). */
rgdn_status rgdn_set_tonemapping( rgdn_stream* stream, const uint32_t* histogram256, float avgLuminance, rgdn_cuda_stream cudaStream );

/* ---- batching ---------------------------------------------------------------------- */
typedef struct rgdn_job
{
    rgdn_stream*             stream;
    uint32_t                 frameIndex;
    const rgdn_frame_params* params;
} rgdn_job;
/* rgdn_denoise + rgdn_calculate_exposure for n frames of (possibly) different streams
 * and sizes, with one launch per stage covering all of them. No reference counterpart: the
 * reference records one stream's dispatches per call (Denoiser.cpp:64-255).
 *
 * Jobs run in order; consecutive default-path jobs (no PLAIN, EXACT_MATH or TMA_STAGING
 * flag) of one storage mode on distinct streams form a step of up to 32 frames. A step is
 * one persistent launch per stage (gradient samples, 4 gradient a-trous, temporal
 * accumulation, anti-firefly, variance, each a-trous iteration, luminance average) whose
 * blocks loop over the tiles of all its frames; the frames' arguments are copied to the
 * device at the start of the step. Once the autotuner has settled, a step replays a captured
 * CUDA graph. Other jobs run as rgdn_denoise + rgdn_calculate_exposure. The results are those
 * of the single-stream calls, bit for bit. Up to 2 steps per device are in flight (the
 * process shares two constant-memory job tables per device); a third waits on the host for
 * the oldest. */
rgdn_status rgdn_submit_batch( rgdn_context* ctx, const rgdn_job* jobs, uint32_t n, rgdn_cuda_stream cudaStream );

/* Tile shapes of the batched kernels. 32x8, 16x16 and 64x4: persistent blocks of 256 threads,
 * as many as are resident, each looping over tiles. 32x4 (temporal accumulation and a-trous
 * only): one tile per 128-thread block, 7 resident per SM, the launch shape of the single-frame
 * kernels. */
#define RGDN_TILE_32X8  0u
#define RGDN_TILE_16X16 1u
#define RGDN_TILE_64X4  2u
#define RGDN_TILE_32X4  3u
#define RGDN_TILE_32X8_PER_BLOCK 4u   /* variance: one 32x8 tile per 256-thread block */
/* The launch configuration of batched steps for one storage mode. The autotuner starts from
 * 32x8 tiles everywhere and, over the first 15 steps, times every candidate of every launch
 * (tile shape; for a-trous also the register budget and the fusion depth) on the work being
 * submitted, keeps the fastest, then times 2 whole steps at each of 4 candidate groupings
 * (groupPixels, singleFramePixels) and keeps the fastest; then steps switch to graph replay
 * (steps with a single-frame group are launched directly). Candidates give identical results. */
typedef struct rgdn_batch_config
{
    uint32_t temporalTile;        /* RGDN_TILE_* */
    uint32_t antiFireflyTile;     /* always RGDN_TILE_32X8 (its shared-memory tile) */
    uint32_t varianceTile;
    uint32_t atrousTile[ 6 ];     /* per a-trous iteration */
    uint32_t atrousBlocksPerSM[ 6 ];/* register budget of each a-trous iteration's kernel: built
                                     for 3 or 4 resident blocks per SM (80 or 64 registers per
                                     thread); 0 = 3. With RGDN_TILE_32X4 it is 7 (0 or 7). */
    uint32_t useGraphs;           /* replay a captured graph per step (off while timing) */
    uint32_t tuned;               /* read: the autotuner has settled (set_config settles it) */
    uint32_t atrousFusionDepth;   /* 1: one launch per a-trous iteration; 2: iterations 0 and 1 in
                                     one launch (32x8 tiles, iteration 0 recomputed over the tile
                                     widened by 2) in steps whose frames all run 3 or more
                                     iterations; 0 = 1 */
    uint64_t groupPixels;         /* the step's frames run in groups of consecutive frames of at
                                     most this many pixels (a larger frame is a group of its own);
                                     a group runs every stage before the next group starts, so the
                                     planes one stage writes are still in L2 when the group's next
                                     stage reads them. 0 = no bound */
    uint64_t singleFramePixels;   /* a frame of at least this many pixels is a group of its own; a
                                     group of one frame runs on the single-frame kernels, its
                                     arguments passed as kernel parameters. 0 = never alone */
} rgdn_batch_config;
rgdn_status rgdn_batch_get_config( rgdn_context* ctx, uint32_t storage, rgdn_batch_config* outConfig );
/* Fixes the configuration of a storage mode and ends its autotuning. */
rgdn_status rgdn_batch_set_config( rgdn_context* ctx, uint32_t storage, const rgdn_batch_config* config );

/* ---- serving ---------------------------------------------------------------------------- */
/* No reference counterpart (the reference renders one camera per process). A request loop
 * that denoises frames of many camera streams with continuous batching: a frame submitted
 * while earlier steps run on the GPU joins the next step, which is enqueued at once, so steps
 * follow each other on the device without a gap (and overlap, on two CUDA streams, when no
 * camera stream is in both). Each stream's history stays resident. A stream's memory is
 * allocated when its first frame is scheduled and the context's budget
 * (rgdn_context_create_info.memoryBudgetBytes) admits it; until then its frames wait.
 * A step takes the oldest frame of each of up to maxFramesPerStep streams, in arrival
 * order, while the step's pixels stay within maxPixelsPerStep. The frames of one stream run
 * in submission order, one per step. Results are those of rgdn_denoise +
 * rgdn_calculate_exposure on the stream alone, bit for bit. */
typedef struct rgdn_server rgdn_server;
typedef struct rgdn_server_create_info
{
    uint32_t storage;            /* rgdn_storage of every stream of the server */
    uint32_t maxFramesPerStep;   /* 1..32 (0 = 32) */
    uint64_t maxPixelsPerStep;   /* bound on one step's work, i.e. its latency (0 = none) */
    uint32_t maxQueuedPerStream; /* a stream's frames waiting beyond this many are dropped,
                                    oldest first (a late frame is stale); 0 = keep all */
    uint32_t stepsInFlight;      /* steps enqueued ahead of the GPU: 1..3 (0 = 2); more than 2
                                    also wait for the two job tables of the device */
    uint32_t evictIdleMs;        /* a stream idle this long may lose its memory (and history)
                                    to admit another; 0 = never evict */
    uint32_t hostCopy;           /* RGDN_HOST_COPY_*: how RGDN_REQUEST_COPY planes in pinned host
                                    memory reach the device */
} rgdn_server_create_info;
#define RGDN_HOST_COPY_ENGINE 0u /* cudaMemcpyAsync per plane (the copy engines) */
#define RGDN_HOST_COPY_SM     1u /* one kernel per frame loads the pinned planes over the host link
                                    (mapped host memory) and stores them to the stream's planes;
                                    planes that are not device-mapped, or not 16-byte aligned and
                                    sized, still go through cudaMemcpyAsync */

/* G-buffer source of a request: planes RGDN_FB_ALBEDO .. RGDN_FB_GRADIENT_RESHADED */
#define RGDN_GBUFFER_PLANES 15

/* Copies `count` (1 .. RGDN_GBUFFER_PLANES) host ranges src[k] of bytes[k] into device memory
 * dst[k], asynchronously on cudaStream, the way a served frame's planes reach the device: with
 * RGDN_HOST_COPY_SM the ranges in pinned, device-mapped host memory with 16-byte aligned
 * addresses and sizes are loaded by one kernel (32 blocks) over the host link, and the others go
 * through cudaMemcpyAsync; with RGDN_HOST_COPY_ENGINE every range goes through cudaMemcpyAsync.
 * For a renderer that streams its G-buffer from host memory into device planes it binds with
 * rgdn_stream_bind_framebuffer. The reference has no counterpart: its G-buffer is written on the
 * device by its ray-tracing pipeline. */
rgdn_status rgdn_copy_host_planes( void* const* dst, const void* const* src, const size_t* bytes, uint32_t count,
                                   uint32_t hostCopy, rgdn_cuda_stream cudaStream );
#define RGDN_REQUEST_COPY 0u   /* gbuffer[] are host (pinned or pageable) or device pointers; copied
                                  into the stream's planes inside the step */
#define RGDN_REQUEST_BIND 1u   /* gbuffer[] are device pointers used in place (no copy); they must
                                  stay valid until the frame completes */
typedef struct rgdn_frame_request
{
    uint32_t          stream;                           /* id from rgdn_server_open_stream */
    uint32_t          gbufferMode;                      /* RGDN_REQUEST_* */
    const void*       gbuffer[ RGDN_GBUFFER_PLANES ];   /* dense rows; NULL keeps the plane */
    void*             preFinalOut;                      /* optional destination of PRE_FINAL
                                                           (host or device, dense rows) */
    rgdn_frame_params params;
} rgdn_frame_request;

/* rgdn_server_wait result states */
#define RGDN_FRAME_DONE    0u
#define RGDN_FRAME_DROPPED 1u   /* superseded by newer frames of the stream (maxQueuedPerStream) */
typedef struct rgdn_frame_result
{
    uint32_t state;          /* RGDN_FRAME_* */
    uint32_t frameIndex;     /* the stream's frame slot the frame ran in */
    float    latencyMs;      /* submission to completion seen by the host */
    float    queueMs;        /* submission to the step's enqueue */
} rgdn_frame_result;

typedef struct rgdn_server_stats
{
    uint64_t framesDone, framesDropped, steps, pixelsDone;
    uint32_t residentStreams, queuedFrames;
    uint64_t residentBytes;
    float    p50Ms, p99Ms, maxMs;     /* latency of the frames done since the last reset */
    float    meanFramesPerStep;
    double   busySeconds;             /* wall time with at least one step on the GPU */
    float    p99AllMs;                /* p99 over every finished request, a dropped one counting as
                                         an unbounded latency (+infinity once drops pass 1 %) */
    float    dropRate;                /* framesDropped / (framesDone + framesDropped) */
    /* one step's parts, p50 and p99 over the steps done since the last reset: the host time to
     * enqueue it (plane copies, tables, launches), then on the device the G-buffer copies in,
     * the kernels and the PRE_FINAL copies out (CUDA events on the step's stream) */
    float    issueP50Ms, issueP99Ms;
    float    copyInP50Ms, copyInP99Ms;
    float    kernelsP50Ms, kernelsP99Ms;
    float    copyOutP50Ms, copyOutP99Ms;
} rgdn_server_stats;

rgdn_status rgdn_server_create( rgdn_context* ctx, const rgdn_server_create_info* info, rgdn_server** outServer );
/* Completes every submitted frame, then frees the server's streams. */
rgdn_status rgdn_server_destroy( rgdn_server* server );
rgdn_status rgdn_server_open_stream( rgdn_server* server, uint32_t width, uint32_t height, uint32_t* outStreamId );
/* Waits for the stream's frames, then frees its memory. */
rgdn_status rgdn_server_close_stream( rgdn_server* server, uint32_t streamId );
/* Queues one frame; thread-safe. The request's buffers must stay valid until it completes. */
rgdn_status rgdn_server_submit( rgdn_server* server, const rgdn_frame_request* request, uint64_t* outTicket );
/* Waits up to timeoutMs (0 = poll) for a ticket: RGDN_SUCCESS with the result (the ticket is
 * then released), RGDN_TIMEOUT, or RGDN_WRONG_FUNCTION_ARGUMENT for an unknown ticket. */
rgdn_status rgdn_server_wait( rgdn_server* server, uint64_t ticket, uint32_t timeoutMs, rgdn_frame_result* outResult );
/* Blocks until every frame submitted so far has completed or been dropped. */
rgdn_status rgdn_server_drain( rgdn_server* server );
rgdn_status rgdn_server_stats_get( rgdn_server* server, rgdn_server_stats* outStats );
rgdn_status rgdn_server_stats_reset( rgdn_server* server );
/* The stream behind an id (NULL until admitted), for reading its images and tonemapping state
 * between frames. */
rgdn_status rgdn_server_get_stream( rgdn_server* server, uint32_t streamId, rgdn_stream** outStream );

/* ---- without device allocation ----------------------------------------------------------- */
/* No counterpart in the reference. The four gradient a-trous iterations
 * (CmASVGFGradientAtrous.comp, as RGDN_STAGE_GRADIENT_ATROUS 0..3) for a caller that may not
 * allocate device memory — a host application that owns every allocation through a fixed
 * budget, or a frame loop that cannot afford the device synchronisation of cudaMalloc /
 * cudaFree. The caller passes its own images (rgba8 per stratum, ((W+1)/3) x ((H+1)/3), dense
 * rows, 4-byte aligned): `samples` (read only), `filtered` (the result, the reference's final
 * DISPingGradient) and `history` (iteration 0's output, DISGradientHistory). The one
 * intermediate image lives in a fixed array inside the library: at most 1280 x 720 strata
 * (3840x2160 renders); larger sizes return RGDN_WRONG_FUNCTION_ARGUMENT. Nothing is allocated.
 * The first call on a device looks the array up (cudaGetSymbolAddress) with that device
 * current, and so does the first call in any other CUDA context (a non-primary context, or the
 * primary one created again after cudaDeviceReset); make that first call before capturing a
 * stream. All calls share the one array: calls whose work overlaps on the GPU (other streams,
 * other threads) race on it and must be serialised by the caller. The three images must not
 * overlap; equal pointers return RGDN_WRONG_FUNCTION_ARGUMENT. */
rgdn_status rgdn_gradient_atrous_noalloc( const uint32_t* samples, uint32_t* filtered, uint32_t* history, uint32_t renderWidth,
                                          uint32_t renderHeight, rgdn_cuda_stream cudaStream );

/* ---- per-kernel timing (tracing) ----------------------------------------------------- */
/* With timing on, every kernel the stream launches is bracketed by two CUDA events on the
 * launching stream. rgdn_stream_read_timing waits for them and returns, per (stage,
 * iteration), the launches and the summed device time since the last read. The reference
 * only labels its dispatches (CmdLabel, Source/Denoiser.cpp:90-205); this is the timed form. */
typedef struct rgdn_stage_timing
{
    uint32_t stage;       /* rgdn_stage */
    uint32_t iteration;
    uint32_t launches;
    float    totalMs;
} rgdn_stage_timing;
rgdn_status rgdn_stream_set_timing( rgdn_stream* stream, uint32_t enable );
rgdn_status rgdn_stream_read_timing( rgdn_stream* stream, rgdn_stage_timing* out, uint32_t capacity, uint32_t* outCount );
/* Per-launch device timing of batched steps (as rgdn_stream_set_timing; stage ids are
 * rgdn_stage, totals per (stage, iteration)). Timed steps use direct launches, not graphs.
 * A group of one frame (rgdn_batch_config.groupPixels) runs on the single-frame kernels and is
 * timed as a whole under the id RGDN_BATCH_SINGLE_FRAME_GROUP. */
#define RGDN_BATCH_SINGLE_FRAME_GROUP 200u
rgdn_status rgdn_batch_set_timing( rgdn_context* ctx, uint32_t enable );
rgdn_status rgdn_batch_read_timing( rgdn_context* ctx, rgdn_stage_timing* out, uint32_t capacity, uint32_t* outCount );

/* ---- misc -------------------------------------------------------------------------- */
/* getColorBin (CmLuminanceHistogram.comp:41-54) for every fp16 bit pattern of the
 * HistogramInput image: out[h] = bin of the fp16 value with bits h. This is the table the
 * GPU histogram indexes; exported so a caller can bin HistogramInput texels identically. */
rgdn_status rgdn_histogram_bin_table( float minLogLuminance, float maxLogLuminance, uint8_t* out65536 );
const char* rgdn_status_string( rgdn_status status );
/* Number of kernels this library launched since the context was created (all streams). */
rgdn_status rgdn_context_launch_count( rgdn_context* ctx, uint64_t* outCount );
uint32_t    rgdn_api_version( void );

#ifdef __cplusplus
}
#endif

#endif /* RGDN_H_ */
