"""ctypes binding of ``include/rgdn.h`` (librgdn.so). Loading fails loudly when the library
is missing: there is no Python or CPU fallback for any compute entry point."""
from __future__ import annotations

import ctypes as C
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "librgdn.so")

# ---- enums (values from include/rgdn.h) -------------------------------------------------
SUCCESS, WRONG_INSTANCE, DEVICE_ERROR, INTERNAL_ERROR = 0, 3, 5, 6
WRONG_FUNCTION_CALL, WRONG_FUNCTION_ARGUMENT = 10, 11
OUT_OF_BUDGET, TIMEOUT, NOT_READY = 64, 65, 66

STORAGE_REF, STORAGE_FP32, STORAGE_FP16, STORAGE_BF16 = 0, 1, 2, 3
STORAGE_NAMES = {"ref": STORAGE_REF, "fp32": STORAGE_FP32, "fp16": STORAGE_FP16, "bf16": STORAGE_BF16}

FORMAT_NAMES = [
    "NONE", "R8_UINT", "RG8_UNORM", "RGBA8_UNORM", "R16_SFLOAT", "RG16_SFLOAT", "RGBA16_SFLOAT",
    "RGBA16_BFLOAT", "R32_SFLOAT", "RG32_SFLOAT", "RGBA32_SFLOAT", "R32_UINT", "E5B9G9R9_UFLOAT",
    "B10G11R11_UFLOAT", "NORMAL_SPHERICAL",
]

FB_NAMES = [
    "ALBEDO", "IS_SKY", "NORMAL", "METALLIC_ROUGHNESS", "DEPTH_WORLD", "DEPTH_GRAD", "MOTION",
    "UNFILTERED_DIRECT", "UNFILTERED_SPECULAR", "UNFILTERED_INDIR", "SURFACE_POSITION",
    "VIEW_DIRECTION", "THROUGHPUT", "GRADIENT_INPUTS", "GRADIENT_RESHADED", "PRE_FINAL",
    "HISTOGRAM_INPUT", "ACCUM_HISTORY_LENGTH", "DIFF_TEMPORARY", "DIFF_ACCUM_COLOR",
    "DIFF_ACCUM_MOMENTS", "DIFF_COLOR_HISTORY", "DIFF_PING_COLOR_AND_VARIANCE",
    "DIFF_PONG_COLOR_AND_VARIANCE", "SPEC_ACCUM_COLOR", "SPEC_PING_COLOR", "SPEC_PONG_COLOR",
    "INDIR_ACCUM", "INDIR_PING", "INDIR_PONG", "ATROUS_FILTERED_VARIANCE", "DIS_PING_GRADIENT",
    "DIS_PONG_GRADIENT", "DIS_GRADIENT_HISTORY", "GRADIENT_PREV_PIX",
    "DIFF_COLOR_HISTORY_VARIANCE", "DIFF_PING_VARIANCE", "DIFF_PONG_VARIANCE",
    "SCREEN_EMIS_RT", "SCATTERING", "FINAL", "BLOOM_INPUT",
    "BLOOM_MIP1", "BLOOM_MIP2", "BLOOM_MIP3", "BLOOM_MIP4", "BLOOM_MIP5", "BLOOM_MIP6", "BLOOM_MIP7",
    "BLOOM_MIP8", "BLOOM_RESULT",
    "DEPTH_NDC", "SCATTERING_HISTORY", "SCATTER_VOLUME", "RESERVOIRS",
]
FB = {n: i for i, n in enumerate(FB_NAMES)}
FB_COUNT = len(FB_NAMES)

# G-buffer images a producer writes every frame
GBUFFER = ["ALBEDO", "IS_SKY", "NORMAL", "METALLIC_ROUGHNESS", "DEPTH_WORLD", "DEPTH_GRAD", "MOTION",
           "UNFILTERED_DIRECT", "UNFILTERED_SPECULAR", "UNFILTERED_INDIR", "SURFACE_POSITION",
           "VIEW_DIRECTION", "THROUGHPUT", "GRADIENT_INPUTS", "GRADIENT_RESHADED"]

STAGE_GRADIENT_SAMPLES, STAGE_GRADIENT_ATROUS, STAGE_TEMPORAL_ACCUMULATION = 0, 1, 2
STAGE_ANTI_FIREFLY, STAGE_VARIANCE_ESTIMATION, STAGE_ATROUS = 3, 4, 5
STAGE_LUMINANCE_HISTOGRAM, STAGE_LUMINANCE_AVG = 6, 7

FLAG_PLAIN, FLAG_SKIP_GRADIENTS, FLAG_EXACT_MATH, FLAG_TMA_STAGING, FLAG_STAGE_DEFAULT = 0x1, 0x2, 0x4, 0x8, 0x10
FLAG_ATROUS_PAIR = 0x40
FLAG_AF_VARIANCE_FUSED = 0x20
FLAG_TEST_TMA_TIMEOUT = 0x80000000


class FinalParams(C.Structure):
    """rgdn_final_params: ImageComposition's tonemapping, bloom and emission parameters."""
    _fields_ = [
        ("luminanceWhitePoint", C.c_float), ("emissionMaxScreenColor", C.c_float),
        ("bloomEmissionMultiplier", C.c_float), ("bloomThreshold", C.c_float),
        ("saturation", C.c_float * 3), ("crosstalk", C.c_float * 3),
        ("lightmapScreenCoverage", C.c_float), ("flags", C.c_uint32),
    ]

    @staticmethod
    def defaults() -> "FinalParams":
        """The reference's defaults (DrawFrameInfo.h: tonemapping, bloom, textures params)."""
        p = FinalParams()
        p.luminanceWhitePoint, p.emissionMaxScreenColor = 10.0, 1.5
        p.bloomEmissionMultiplier, p.bloomThreshold = 16.0, 4.0
        p.saturation[:] = (0.0, 0.0, 0.0)
        p.crosstalk[:] = (1.0, 1.0, 1.0)
        return p

    def copy(self) -> "FinalParams":
        c = FinalParams()
        C.pointer(c)[0] = self
        return c


FINAL_APPLY_SCATTERING = 0x1
FINAL_EXACT_MATH = 0x2


class BloomParams(C.Structure):
    """rgdn_bloom_params."""
    _fields_ = [("bloomIntensity", C.c_float)]


VOLUME_SIZE = (160, 88, 64)   # RGDN_VOLUME_SIZE_X, _Y, _Z
VOLUME_ENABLE_NONE, VOLUME_ENABLE_SIMPLE, VOLUME_ENABLE_VOLUMETRIC = 0, 1, 2
VOLUME_EXACT_MATH = 0x1


class VolumetricParams(C.Structure):
    """rgdn_volumetric_params: the GlobalUniform fields of Volumetric::ProcessScattering."""
    _fields_ = [
        ("invView", C.c_float * 16), ("invProjection", C.c_float * 16), ("volumeViewProj", C.c_float * 16),
        ("cameraPosition", C.c_float * 4), ("volumeCameraNear", C.c_float), ("volumeCameraFar", C.c_float),
        ("volumeAmbient", C.c_float * 3), ("volumeScattering", C.c_float), ("maxHistoryLength", C.c_float),
        ("volumeEnableType", C.c_uint32), ("frameId", C.c_uint32), ("flags", C.c_uint32),
    ]


class FrameParams(C.Structure):
    """rgdn_frame_params: the ShGlobalUniform fields this path reads."""
    _fields_ = [
        ("view", C.c_float * 16), ("viewPrev", C.c_float * 16),
        ("projection", C.c_float * 16), ("projectionPrev", C.c_float * 16),
        ("cameraPosition", C.c_float * 4), ("cameraPositionPrev", C.c_float * 4),
        ("timeDelta", C.c_float), ("minLogLuminance", C.c_float), ("maxLogLuminance", C.c_float),
        ("stopEyeAdaptation", C.c_uint32),
        ("gradientMultDiffuse", C.c_float), ("gradientMultIndirect", C.c_float),
        ("gradientMultSpecular", C.c_float), ("antiFireflyEnabled", C.c_uint32),
        ("lightmapScreenCoverage", C.c_float), ("debugShowFlags", C.c_uint32),
        ("atrousIterations", C.c_uint32), ("flags", C.c_uint32), ("frameId", C.c_uint32),
    ]

    def copy(self) -> "FrameParams":
        p = FrameParams()
        C.memmove(C.byref(p), C.byref(self), C.sizeof(FrameParams))
        return p


class SphereLight(C.Structure):
    """rgdn_sphere_light: SphereLight (Light.h:31-36)."""
    _fields_ = [("center", C.c_float * 3), ("radius", C.c_float), ("color", C.c_float * 3), ("pad", C.c_float)]


OCCLUDER_SPHERE, OCCLUDER_RECT = 0, 1


class Occluder(C.Structure):
    _fields_ = [("type", C.c_uint32), ("data", C.c_float * 7)]


class ReshadeScene(C.Structure):
    """rgdn_reshade_scene: device arrays of this frame's lights, the previous-to-current light
    index map and the shadow-ray occluders."""
    _fields_ = [("lights", C.c_void_p), ("lightCount", C.c_uint32), ("prevToCur", C.c_void_p),
                ("prevLightCount", C.c_uint32), ("occluders", C.c_void_p), ("occluderCount", C.c_uint32)]


class Image(C.Structure):
    _fields_ = [("data", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32),
                ("pitch_bytes", C.c_uint32), ("texel_bytes", C.c_uint32), ("format", C.c_uint32),
                ("has_prev", C.c_uint32)]


class ContextCreateInfo(C.Structure):
    _fields_ = [("device", C.c_int), ("memoryBudgetBytes", C.c_uint64), ("flags", C.c_uint32)]


CONTEXT_NO_L2_PERSIST = 0x1


class StreamCreateInfo(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("storage", C.c_uint32)]


class StageTiming(C.Structure):
    _fields_ = [("stage", C.c_uint32), ("iteration", C.c_uint32), ("launches", C.c_uint32),
                ("totalMs", C.c_float)]


class BatchConfig(C.Structure):
    """rgdn_batch_config: launch configuration of batched steps for one storage mode."""
    _fields_ = [("temporalTile", C.c_uint32), ("antiFireflyTile", C.c_uint32),
                ("varianceTile", C.c_uint32), ("atrousTile", C.c_uint32 * 6),
                ("atrousBlocksPerSM", C.c_uint32 * 6), ("useGraphs", C.c_uint32), ("tuned", C.c_uint32),
                ("atrousFusionDepth", C.c_uint32), ("groupPixels", C.c_uint64),
                ("singleFramePixels", C.c_uint64)]


TILE_32X8, TILE_16X16, TILE_64X4, TILE_32X4, TILE_32X8_PER_BLOCK = 0, 1, 2, 3, 4
DEVICE_ERROR_TMA_WAIT = 1

GBUFFER_PLANES = 15
REQUEST_COPY, REQUEST_BIND = 0, 1
FRAME_DONE, FRAME_DROPPED = 0, 1


class ServerCreateInfo(C.Structure):
    _fields_ = [("storage", C.c_uint32), ("maxFramesPerStep", C.c_uint32), ("maxPixelsPerStep", C.c_uint64),
                ("maxQueuedPerStream", C.c_uint32), ("stepsInFlight", C.c_uint32), ("evictIdleMs", C.c_uint32),
                ("hostCopy", C.c_uint32)]


HOST_COPY_ENGINE, HOST_COPY_SM = 0, 1


class FrameRequest(C.Structure):
    _fields_ = [("stream", C.c_uint32), ("gbufferMode", C.c_uint32), ("gbuffer", C.c_void_p * 15),
                ("preFinalOut", C.c_void_p), ("params", FrameParams)]


class FrameResult(C.Structure):
    _fields_ = [("state", C.c_uint32), ("frameIndex", C.c_uint32), ("latencyMs", C.c_float), ("queueMs", C.c_float)]


class ServerStats(C.Structure):
    _fields_ = [("framesDone", C.c_uint64), ("framesDropped", C.c_uint64), ("steps", C.c_uint64),
                ("pixelsDone", C.c_uint64), ("residentStreams", C.c_uint32), ("queuedFrames", C.c_uint32),
                ("residentBytes", C.c_uint64), ("p50Ms", C.c_float), ("p99Ms", C.c_float), ("maxMs", C.c_float),
                ("meanFramesPerStep", C.c_float), ("busySeconds", C.c_double), ("p99AllMs", C.c_float),
                ("dropRate", C.c_float), ("issueP50Ms", C.c_float), ("issueP99Ms", C.c_float),
                ("copyInP50Ms", C.c_float), ("copyInP99Ms", C.c_float), ("kernelsP50Ms", C.c_float),
                ("kernelsP99Ms", C.c_float), ("copyOutP50Ms", C.c_float), ("copyOutP99Ms", C.c_float)]


class Job(C.Structure):
    _fields_ = [("stream", C.c_void_p), ("frameIndex", C.c_uint32), ("params", C.POINTER(FrameParams))]


# (name, restype, argtypes) of every entry point declared in include/rgdn.h
_VP, _U32, _U64, _SZ, _I = C.c_void_p, C.c_uint32, C.c_uint64, C.c_size_t, C.c_int
_PFP = C.POINTER(FrameParams)
SIGNATURES = [
    ("rgdn_context_create", _I, [C.POINTER(ContextCreateInfo), C.POINTER(_VP)]),
    ("rgdn_context_destroy", _I, [_VP]),
    ("rgdn_context_memory_used", _I, [_VP, C.POINTER(_U64)]),
    ("rgdn_stream_create", _I, [_VP, C.POINTER(StreamCreateInfo), C.POINTER(_VP)]),
    ("rgdn_stream_destroy", _I, [_VP]),
    ("rgdn_stream_resize", _I, [_VP, _U32, _U32]),
    ("rgdn_stream_required_bytes", _I, [C.POINTER(StreamCreateInfo), C.POINTER(_U64)]),
    ("rgdn_stream_get_framebuffer", _I, [_VP, _U32, _U32, C.POINTER(Image)]),
    ("rgdn_stream_bind_framebuffer", _I, [_VP, _U32, _U32, _VP]),
    ("rgdn_stream_upload", _I, [_VP, _U32, _U32, _VP, _SZ, _VP]),
    ("rgdn_stream_download", _I, [_VP, _U32, _U32, _VP, _SZ, _VP]),
    ("rgdn_denoise", _I, [_VP, _U32, _PFP, _VP]),
    ("rgdn_calculate_exposure", _I, [_VP, _U32, _PFP, _VP]),
    ("rgdn_prepare_final", _I, [_VP, _U32, C.POINTER(FinalParams), _VP]),
    ("rgdn_bloom", _I, [_VP, _U32, C.POINTER(BloomParams), _VP]),
    ("rgdn_process_scattering", _I, [_VP, _U32, C.POINTER(VolumetricParams), _VP]),
    ("rgdn_denoise_stage", _I, [_VP, _U32, _U32, _U32, _PFP, _VP]),
    ("rgdn_stream_tonemapping_device", _I, [_VP, C.POINTER(_VP)]),
    ("rgdn_get_tonemapping", _I, [_VP, C.POINTER(_U32), C.POINTER(C.c_float), C.POINTER(C.c_float), _VP]),
    ("rgdn_set_tonemapping", _I, [_VP, C.POINTER(_U32), C.c_float, _VP]),
    ("rgdn_stream_copy_tonemapping", _I, [_VP, _VP, _VP]),
    ("rgdn_stream_take_device_errors", _I, [_VP, C.POINTER(_U32), _VP]),
    ("rgdn_submit_batch", _I, [_VP, C.POINTER(Job), _U32, _VP]),
    ("rgdn_status_string", C.c_char_p, [_I]),
    ("rgdn_context_launch_count", _I, [_VP, C.POINTER(_U64)]),
    ("rgdn_api_version", _U32, []),
    ("rgdn_histogram_bin_table", _I, [C.c_float, C.c_float, C.POINTER(C.c_uint8)]),
    ("rgdn_gradient_atrous_noalloc", _I, [_VP, _VP, _VP, _U32, _U32, _VP]),
    ("rgdn_stream_set_reshade_scene", _I, [_VP, C.POINTER(ReshadeScene)]),
    ("rgdn_stream_set_timing", _I, [_VP, _U32]),
    ("rgdn_stream_read_timing", _I, [_VP, C.POINTER(StageTiming), _U32, C.POINTER(_U32)]),
    ("rgdn_batch_get_config", _I, [_VP, _U32, C.POINTER(BatchConfig)]),
    ("rgdn_batch_set_config", _I, [_VP, _U32, C.POINTER(BatchConfig)]),
    ("rgdn_batch_set_timing", _I, [_VP, _U32]),
    ("rgdn_batch_read_timing", _I, [_VP, C.POINTER(StageTiming), _U32, C.POINTER(_U32)]),
    ("rgdn_server_create", _I, [_VP, C.POINTER(ServerCreateInfo), C.POINTER(_VP)]),
    ("rgdn_server_destroy", _I, [_VP]),
    ("rgdn_server_open_stream", _I, [_VP, _U32, _U32, C.POINTER(_U32)]),
    ("rgdn_server_close_stream", _I, [_VP, _U32]),
    ("rgdn_server_submit", _I, [_VP, C.POINTER(FrameRequest), C.POINTER(_U64)]),
    ("rgdn_server_wait", _I, [_VP, _U64, _U32, C.POINTER(FrameResult)]),
    ("rgdn_server_drain", _I, [_VP]),
    ("rgdn_server_stats_get", _I, [_VP, C.POINTER(ServerStats)]),
    ("rgdn_server_stats_reset", _I, [_VP]),
    ("rgdn_server_get_stream", _I, [_VP, _U32, C.POINTER(_VP)]),
    ("rgdn_copy_host_planes", _I, [C.POINTER(_VP), C.POINTER(_VP), C.POINTER(_SZ), _U32, _U32, _VP]),
]

STAGE_NAMES = ["gradient_samples", "gradient_atrous", "temporal_accumulation", "anti_firefly",
               "variance_estimation", "atrous", "luminance_histogram", "luminance_avg"]
# kernels of the default fused path (ids above the rgdn_stage range, see rgdn_internal.h)
KERNEL_NAMES = dict(enumerate(STAGE_NAMES))
KERNEL_NAMES.update({100: "atrous_fast", 101: "atrous_fast_hist", 102: "temporal_fast",
                     103: "anti_firefly_fast", 104: "variance_fast", 106: "atrous_exact_hist",
                     107: "atrous_exact", 108: "temporal_exact_geom", 109: "variance_exact_geom",
                     110: "temporal_fast_gp", 111: "temporal_exact_geom_gp", 112: "atrous_tma",
                     113: "atrous_tma_hist", 114: "prepare_final", 115: "bloom",
                     117: "process_scattering", 122: "atrous_pair", 123: "af_variance_fast",
                     124: "af_variance_exact", 125: "temporal_fast", 126: "temporal_fast_gp",
                     200: "single_frame_group"})

_lib = None


def load() -> C.CDLL:
    """Loads librgdn.so; raises if it was not built (run raytracedgl1_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -m raytracedgl1_gb300.build` "
                          "(the denoiser has no fallback without its CUDA library)")
    lib = C.CDLL(LIB_PATH)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class RgdnError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = load().rgdn_status_string(status).decode()
        super().__init__(f"{what}: {msg} (status {status})" if what else f"{msg} (status {status})")


def check(status: int, what: str = "") -> None:
    if status != SUCCESS:
        raise RgdnError(status, what)
