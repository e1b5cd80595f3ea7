"""Runs the reference's own shaders (oracle/_ref/librgdn_refshaders.so, built by build.py from
the reference's GLSL sources) beside the oracle, stage by stage, on the same state: test
infrastructure that pins the oracle to the reference.

Each stage is dispatched the way Denoiser::Denoise and Tonemapping::CalculateExposure
dispatch it (Source/Denoiser.cpp:92-253, Source/Tonemapping.cpp:106-165): 16x16 groups over the
render size, the gradient a-trous over renderWidth / 3 (a float, rounded up), the luminance
average as one group of 256. The gradient samples before them run as
PathTracer::CalculateGradientsSamples launches them (Source/PathTracer.cpp:196-218). The reference's framebuffers are bound by name to copies of the
oracle's planes (frame slot fi as framebufX, slot fi ^ 1 as framebufX_Prev), in the reference
framebuffer formats (the oracle's MODE_REF).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(os.path.dirname(HERE), "_ref", "librgdn_refshaders.so")

_lib = None


def load(path: str = LIB) -> C.CDLL:
    global _lib
    if _lib is None:
        _lib = C.CDLL(path)
        _lib.ref_bind.argtypes = [C.c_char_p, C.c_void_p, C.c_int, C.c_int]
        _lib.ref_bind.restype = C.c_int
        _lib.ref_texel_bytes.argtypes = [C.c_char_p]
        _lib.ref_texel_bytes.restype = C.c_int
    return _lib


def ref_name(fb: str) -> str:
    """The reference's image name of a framebuffer (DIFF_ACCUM_COLOR -> framebufDiffAccumColor,
    BLOOM_MIP1 -> framebufBloom_Mip1)."""
    words = fb.split("_")
    if words[0] == "BLOOM" and len(words) > 1 and words[1] in ("MIP1", "MIP2", "MIP3", "MIP4", "MIP5", "MIP6",
                                                               "MIP7", "MIP8", "RESULT"):
        return "framebufBloom_" + words[1].capitalize()
    return "framebuf" + "".join(w if w in ("DIS", "RT") else w.capitalize() for w in words)


def stage_plan(W: int, H: int, niter: int = 4):
    """(oracle stage, iteration, reference entry point, groups) in the reference's frame order:
    the gradient samples (RtGradients.rgen's main, launched over ceil(W / 3) x ceil(H / 3) as
    PathTracer::CalculateGradientsSamples launches it, one invocation per group here), then
    Denoise and CalculateExposure."""
    from raytracedgl1_gb300 import _native as N
    gw, gh = -(-W // 3), -(-H // 3)
    full = ((W + 15) // 16, (H + 15) // 16)
    plan = [(N.STAGE_GRADIENT_SAMPLES, 0, "RtGradients_main", (gw, gh))]
    plan += [(N.STAGE_GRADIENT_ATROUS, i, f"CmASVGFGradientAtrous_{i}", ((gw + 15) // 16, (gh + 15) // 16)) for i in range(4)]
    plan += [(N.STAGE_TEMPORAL_ACCUMULATION, 0, "CmSVGFTemporalAccumulation", full),
             (N.STAGE_ANTI_FIREFLY, 0, "CmAntiFirefly", full),
             (N.STAGE_VARIANCE_ESTIMATION, 0, "CmSVGFEstimateVariance", full)]
    plan += [(N.STAGE_ATROUS, i, "CmSVGFAtrous_Iter0" if i == 0 else f"CmSVGFAtrous_{i}", full) for i in range(niter)]
    plan += [(N.STAGE_LUMINANCE_HISTOGRAM, 0, "CmLuminanceHistogram", full),
             (N.STAGE_LUMINANCE_AVG, 0, "CmLuminanceAvg", (1, 1))]
    return plan


# Planes the reference keeps in one image and the oracle in two frame slots: the gradient history
# (DISGradientHistory, FRAMEBUF_FLAGS_FORCE_SIZE_1_3 without a _Prev image) is read by the gradient
# samples before this frame's gradient a-trous overwrites it, so at that point the reference's
# image holds the previous frame's history, which the oracle keeps in the previous frame's slot.
# For these entry points the previous slot is bound under the reference's (current) name.
PREV_AS_CURRENT = {"RtGradients_main": ("DIS_GRADIENT_HISTORY",)}


class RefRun:
    """The reference shaders' state for one frame: copies of the oracle's planes bound by name."""

    def __init__(self, W: int, H: int, lib: C.CDLL | None = None):
        self.W, self.H = W, H
        self.lib = lib or load()
        self.arrays: dict = {}

    def bind_from(self, planes: dict, fi: int, tag: str | None = None) -> None:
        """planes: {(fb name, slot): array}; binds copies (kept in self.arrays) for the entry point
        `tag` (see PREV_AS_CURRENT)."""
        self.arrays = {}
        prev_as_current = PREV_AS_CURRENT.get(tag, ())
        for (fb, slot), arr in planes.items():
            if fb in prev_as_current:
                if slot == fi:
                    continue
                name = ref_name(fb)
            else:
                name = ref_name(fb) + ("" if slot == fi else "_Prev")
            if not self.lib.ref_texel_bytes(name.encode()):
                continue
            a = np.ascontiguousarray(arr).copy()
            self.lib.ref_bind(name.encode(), a.ctypes.data, a.shape[1], a.shape[0])
            self.arrays[(fb, slot)] = a

    def run(self, tag: str, groups, params, tonemapping=None):
        """Dispatches one reference shader; `tonemapping` (histogram uint32[256], avg float) is the
        buffer's state before it, and the state after it is returned."""
        f = getattr(self.lib, f"ref_{tag}_set_uniform", None)
        if f is not None:
            f(C.byref(params), C.c_float(self.W), C.c_float(self.H))
        tm = getattr(self.lib, f"ref_{tag}_tonemapping", None) if tonemapping is not None else None
        ptr = None
        if tm is not None:
            tm.restype = C.c_void_p
            ptr = tm()
            h32 = np.ascontiguousarray(np.asarray(tonemapping[0], dtype=np.uint32))
            a32 = np.array([tonemapping[1]], dtype=np.float32)
            C.memmove(ptr, h32.ctypes.data, 1024)
            C.memmove(ptr + 1024, a32.ctypes.data, 4)
        getattr(self.lib, f"ref_{tag}_dispatch")(int(groups[0]), int(groups[1]))
        if ptr is None:
            return None
        return (np.frombuffer(C.string_at(ptr, 1024), dtype=np.uint32).copy(),
                float(np.frombuffer(C.string_at(ptr + 1024, 4), dtype=np.float32)[0]))


def oracle_planes(o, fi: int) -> dict:
    """Copies of every plane of an OracleStream: {(fb name, slot): array}, the previous-frame slot
    only for planes that have one."""
    from raytracedgl1_gb300 import _native as N
    out = {}
    for fb in N.FB_NAMES:
        cur, prev = o.plane(fb, fi), o.plane(fb, fi ^ 1)
        if cur is None:
            continue
        out[(fb, fi)] = np.ascontiguousarray(cur).copy()
        # a plane without a previous-frame slot answers both slots with the same memory
        if prev is not None and prev.ctypes.data != cur.ctypes.data:
            out[(fb, fi ^ 1)] = np.ascontiguousarray(prev).copy()
    return out


def differing(a: dict, b: dict) -> list:
    """[(fb, slot, texels that differ)] between two plane sets (keys of a)."""
    bad = []
    for key, x in a.items():
        y = b[key]
        if not np.array_equal(x.view(np.uint8), y.view(np.uint8)):
            xx = x.reshape(x.shape[0], x.shape[1], -1)
            yy = y.reshape(y.shape[0], y.shape[1], -1)
            bad.append((key[0], key[1], int(np.count_nonzero(np.any(xx != yy, axis=-1)))))
    return bad


def run_reference_final(W: int, H: int, planes: dict, fi: int, params, final, avg_luminance: float,
                        lib: C.CDLL | None = None) -> dict:
    """ImageComposition::PrepareForRaster + Finalize as the reference records them
    (Source/ImageComposition.cpp:87-155): CmCheckerboard over the render size, the LPM control
    block from ImageComposition::SetupLpmParams's LpmSetup call (lpm_setup_ref.cpp), then
    CmPrepareFinal, both in 16x16 groups. `planes` are the oracle's {(fb, slot): array} in the
    reference formats; SCREEN_EMISSION, which the oracle's single pass keeps on chip, is a scratch
    B10G11R11 image here. Returns the reference's planes after both shaders."""
    lib = lib or load()
    run = RefRun(W, H, lib)
    planes = dict(planes)
    planes[("SCREEN_EMISSION", fi)] = np.zeros((H, W), dtype=np.uint32)
    run.bind_from(planes, fi)
    groups = ((W + 15) // 16, (H + 15) // 16)
    ctl = np.zeros(96, dtype=np.uint32)
    sat = np.array(final.saturation[:], dtype=np.float32)
    ct = np.array(final.crosstalk[:], dtype=np.float32)
    lib.ref_lpm_setup(sat.ctypes.data_as(C.c_void_p), ct.ctypes.data_as(C.c_void_p), ctl.ctypes.data_as(C.c_void_p))
    for tag in ("CmCheckerboard", "CmPrepareFinal"):
        getattr(lib, f"ref_{tag}_set_uniform")(C.byref(params), C.c_float(W), C.c_float(H))
        getattr(lib, f"ref_{tag}_set_final")(C.byref(final))
    for name, data in (("lpm", ctl), ("tonemapping", np.array([avg_luminance], dtype=np.float32))):
        f = getattr(lib, f"ref_CmPrepareFinal_{name}")
        f.restype = C.c_void_p
        # the tonemapping buffer: 256 histogram words, then avgLuminance
        C.memmove(f() + (1024 if name == "tonemapping" else 0), data.ctypes.data, data.nbytes)
    for tag in ("CmCheckerboard", "CmPrepareFinal"):
        getattr(lib, f"ref_{tag}_dispatch")(int(groups[0]), int(groups[1]))
    return run.arrays


FMT_RGBA16F = 5   # glsl::FMT_rgba16f


def run_reference_scattering(W: int, H: int, planes: dict, fi: int, params, vparams, lib: C.CDLL | None = None) -> dict:
    """Volumetric::ProcessScattering as the reference records it (Source/Volumetric.cpp:71-190):
    CmVolumetricProcess over the froxel columns (the volume integrated in place), then
    CmScatterAccum over the render size with maxHistoryLength as its push constant. The oracle's
    SCATTER_VOLUME planes (X x (Y Z) texels, z-major) are bound as the 3-D images g_volumetric
    (this frame) and g_volumetric_Prev (the previous frame's, read through
    g_volumetric_Sampler_Prev). Returns the reference's planes after both shaders."""
    from raytracedgl1_gb300 import _native as N
    lib = lib or load()
    lib.ref_bind3d.argtypes = [C.c_char_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]
    lib.ref_bind3d.restype = C.c_int
    run = RefRun(W, H, lib)
    planes = dict(planes)
    vols = {slot: planes.pop(("SCATTER_VOLUME", slot)) for slot in (fi, fi ^ 1) if ("SCATTER_VOLUME", slot) in planes}
    run.bind_from(planes, fi)
    X, Y, Z = N.VOLUME_SIZE
    for slot, vol in vols.items():
        a = np.ascontiguousarray(vol).copy()
        name = b"g_volumetric" if slot == fi else b"g_volumetric_Prev"
        if not lib.ref_bind3d(name, a.ctypes.data, X, Y, Z, FMT_RGBA16F):
            raise RuntimeError(f"ref_bind3d {name!r}")
        run.arrays[("SCATTER_VOLUME", slot)] = a
    for tag in ("CmVolumetricProcess", "CmScatterAccum"):
        getattr(lib, f"ref_{tag}_set_uniform")(C.byref(params), C.c_float(W), C.c_float(H))
        getattr(lib, f"ref_{tag}_set_volumetric")(C.byref(vparams))
    push = lib.ref_CmScatterAccum_push
    push.restype = C.c_void_p
    C.memmove(push(), np.array([vparams.maxHistoryLength], dtype=np.float32).ctypes.data, 4)
    for tag, (w, h) in (("CmVolumetricProcess", (X, Y)), ("CmScatterAccum", (W, H))):
        local = (C.c_uint * 3)()
        getattr(lib, f"ref_{tag}_local")(local)
        getattr(lib, f"ref_{tag}_dispatch")(-(-w // local[0]), -(-h // local[1]))
    return run.arrays

