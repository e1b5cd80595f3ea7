"""CPU ORACLE — test infrastructure only (see rgdn_oracle.cpp's header).

Python binding of ``librgdn_oracle.so``, the C++ restatement of RayTracedGL1's denoise and
auto-exposure shaders. Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline / reference arm import this module, as the checker; the product never does.

Parity status: unpinned against the reference itself (its GLSL path cannot run here and its
tests hold no golden vectors); the codecs are pinned by spec known-answer tests.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librgdn_oracle.so")

MODE_REF, MODE_F32, MODE_F16, MODE_BF16, MODE_F64 = 0, 1, 2, 3, 4

# oracle-only FP64 formats, and the numpy view of every format
_NUMPY = {
    1: (np.uint8, 1), 2: (np.uint8, 2), 3: (np.uint8, 4), 4: (np.uint16, 1), 5: (np.uint16, 2),
    6: (np.uint16, 4), 7: (np.uint16, 4), 8: (np.float32, 1), 9: (np.float32, 2), 10: (np.float32, 4),
    11: (np.uint32, 1), 12: (np.uint32, 1), 13: (np.uint32, 1), 14: (np.uint32, 1), 15: (np.uint32, 4),
    100: (np.float64, 1), 101: (np.float64, 2), 102: (np.float64, 4),
}

_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} missing: build it with `python -m raytracedgl1_gb300.build`")
    from raytracedgl1_gb300._native import FinalParams, FrameParams, VolumetricParams
    lib = C.CDLL(LIB_PATH)
    P = C.POINTER
    sig = {
        "orc_stream_create": (C.c_void_p, [C.c_uint32, C.c_uint32, C.c_uint32]),
        "orc_stream_destroy": (None, [C.c_void_p]),
        "orc_stream_plane": (C.c_void_p, [C.c_void_p, C.c_uint32, C.c_uint32, P(C.c_uint32), P(C.c_uint32),
                                          P(C.c_uint32), P(C.c_uint32)]),
        "orc_stream_grad_width": (C.c_uint32, [C.c_void_p]),
        "orc_stream_grad_height": (C.c_uint32, [C.c_void_p]),
        "orc_stage": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, P(FrameParams), C.c_int]),
        "orc_denoise": (C.c_int, [C.c_void_p, C.c_uint32, P(FrameParams), C.c_int]),
        "orc_calculate_exposure": (C.c_int, [C.c_void_p, C.c_uint32, P(FrameParams), C.c_int]),
        "orc_exposure_from_avg": (C.c_float, [C.c_float]),
        "orc_prepare_final": (C.c_int, [C.c_void_p, C.c_uint32, P(FinalParams), C.c_int]),
        "orc_bloom": (C.c_int, [C.c_void_p, C.c_uint32, C.c_float]),
        "orc_process_scattering": (C.c_int, [C.c_void_p, C.c_uint32, P(VolumetricParams)]),
        "orc_random_seed": (C.c_uint32, [C.c_int, C.c_int, C.c_uint32]),
        "orc_set_reshade_scene": (None, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32]),
        "orc_reshade": (C.c_int, [C.c_void_p, C.c_uint32, C.c_int, C.c_int, P(FrameParams), C.c_int, P(C.c_double)]),
        "orc_wellons_lowbias32": (C.c_uint32, [C.c_uint32]),
        "orc_lpm_setup": (None, [P(C.c_float), P(C.c_float), P(C.c_float)]),
        "orc_lpm_filter": (None, [P(C.c_float), P(C.c_float), P(C.c_float)]),
        "orc_get_tonemapping": (None, [C.c_void_p, P(C.c_uint32), P(C.c_float), P(C.c_double)]),
        "orc_set_tonemapping": (None, [C.c_void_p, P(C.c_uint32), C.c_float]),
        "orc_f32_to_f16": (C.c_uint16, [C.c_float]),
        "orc_f16_to_f32": (C.c_float, [C.c_uint16]),
        "orc_f32_to_bf16": (C.c_uint16, [C.c_float]),
        "orc_bf16_to_f32": (C.c_float, [C.c_uint16]),
        "orc_encode_e5": (C.c_uint32, [C.c_float, C.c_float, C.c_float]),
        "orc_decode_e5": (None, [C.c_uint32, P(C.c_float)]),
        "orc_encode_b10g11r11": (C.c_uint32, [C.c_float, C.c_float, C.c_float]),
        "orc_decode_b10g11r11": (None, [C.c_uint32, P(C.c_float)]),
        "orc_encode_normal": (C.c_uint32, [C.c_float, C.c_float, C.c_float]),
        "orc_decode_normal": (None, [C.c_uint32, P(C.c_float)]),
        "orc_color_bin": (C.c_uint32, [C.c_float, C.c_float, C.c_float]),
        "orc_unorm8": (C.c_uint8, [C.c_float]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def nthreads_default() -> int:
    return max(1, os.cpu_count() or 1)


class OracleStream:
    """CPU twin of a librgdn stream: same framebuffer table, same byte layouts (modes 0-3)."""

    def __init__(self, width: int, height: int, mode: int = MODE_REF):
        self.lib = load()
        self.h = self.lib.orc_stream_create(width, height, mode)
        if not self.h:
            raise ValueError("bad oracle stream size / mode")
        self.width, self.height, self.mode = width, height, mode

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_stream_destroy(self.h)
            self.h = None

    def plane(self, fb, frame_index: int = 0) -> np.ndarray | None:
        """Zero-copy numpy view of a plane (writes go into the oracle's state)."""
        from raytracedgl1_gb300._native import FB
        fbi = FB[fb] if isinstance(fb, str) else fb
        w, h, t, f = C.c_uint32(), C.c_uint32(), C.c_uint32(), C.c_uint32()
        p = self.lib.orc_stream_plane(self.h, fbi, frame_index, C.byref(w), C.byref(h), C.byref(t), C.byref(f))
        if not p:
            return None
        dt, ch = _NUMPY[f.value]
        n = w.value * h.value * ch
        arr = np.ctypeslib.as_array(C.cast(p, C.POINTER(np.ctypeslib.as_ctypes_type(dt))), shape=(n,))
        return arr.reshape((h.value, w.value) if ch == 1 else (h.value, w.value, ch))

    def fmt(self, fb) -> int:
        from raytracedgl1_gb300._native import FB
        fbi = FB[fb] if isinstance(fb, str) else fb
        w, h, t, f = C.c_uint32(), C.c_uint32(), C.c_uint32(), C.c_uint32()
        self.lib.orc_stream_plane(self.h, fbi, 0, C.byref(w), C.byref(h), C.byref(t), C.byref(f))
        return f.value

    def load(self, fb, frame_index: int, data: np.ndarray) -> None:
        dst = self.plane(fb, frame_index)
        dst[...] = data.reshape(dst.shape).view(dst.dtype) if data.dtype != dst.dtype else data.reshape(dst.shape)

    def stage(self, stage: int, iteration: int, frame_index: int, params, nthreads: int = 0) -> None:
        r = self.lib.orc_stage(self.h, stage, iteration, frame_index, C.byref(params), nthreads or nthreads_default())
        if r != 0:
            raise RuntimeError(f"orc_stage failed: {r}")

    def denoise(self, frame_index: int, params, nthreads: int = 0) -> None:
        r = self.lib.orc_denoise(self.h, frame_index, C.byref(params), nthreads or nthreads_default())
        if r != 0:
            raise RuntimeError(f"orc_denoise failed: {r}")

    def calculate_exposure(self, frame_index: int, params, nthreads: int = 0) -> None:
        r = self.lib.orc_calculate_exposure(self.h, frame_index, C.byref(params), nthreads or nthreads_default())
        if r != 0:
            raise RuntimeError(f"orc_calculate_exposure failed: {r}")

    def prepare_final(self, frame_index: int, params, nthreads: int = 0) -> None:
        """CmCheckerboard + CmPrepareFinal into FINAL and BLOOM_INPUT (rgdn_final_params)."""
        r = self.lib.orc_prepare_final(self.h, frame_index, C.byref(params), nthreads or nthreads_default())
        if r != 0:
            raise RuntimeError(f"orc_prepare_final failed: {r}")

    def process_scattering(self, frame_index: int, params) -> None:
        """The volume integration and the scattering accumulation (rgdn_process_scattering)."""
        r = self.lib.orc_process_scattering(self.h, frame_index, C.byref(params))
        if r != 0:
            raise RuntimeError(f"orc_process_scattering failed: {r}")

    def bloom(self, frame_index: int, intensity: float = 1.0) -> None:
        """The bloom pyramid of BLOOM_INPUT added to FINAL (rgdn_bloom)."""
        r = self.lib.orc_bloom(self.h, frame_index, C.c_float(intensity))
        if r != 0:
            raise RuntimeError(f"orc_bloom failed: {r}")

    def tonemapping(self):
        hist = (C.c_uint32 * 256)()
        avg = C.c_float()
        avg64 = C.c_double()
        self.lib.orc_get_tonemapping(self.h, hist, C.byref(avg), C.byref(avg64))
        return np.frombuffer(hist, dtype=np.uint32).copy(), avg.value, self.lib.orc_exposure_from_avg(avg.value)

    def set_reshade_scene(self, lights=None, prev_to_cur=None, occluders=None) -> None:
        """Gradient re-shading from these host arrays (numpy structured / ctypes arrays of
        rgdn_sphere_light, uint32, rgdn_occluder); lights None clears it."""
        if lights is None:
            self.lib.orc_set_reshade_scene(self.h, None, 0, None, 0, None, 0)
            return
        self._rs = (lights, prev_to_cur, occluders)   # keep the buffers alive
        self.lib.orc_set_reshade_scene(self.h, C.cast(lights, C.c_void_p), len(lights),
                                       C.cast(prev_to_cur, C.c_void_p), len(prev_to_cur),
                                       C.cast(occluders, C.c_void_p) if occluders is not None else None,
                                       len(occluders) if occluders is not None else 0)

    def reshade(self, frame_index: int, px: int, py: int, params, f64: bool = False):
        """The re-shaded (diffuse, specular) luminance of previous-frame pixel (px, py)."""
        out = (C.c_double * 2)()
        r = self.lib.orc_reshade(self.h, frame_index, px, py, C.byref(params), 1 if f64 else 0, out)
        if r != 0:
            raise RuntimeError(f"orc_reshade failed: {r}")
        return out[0], out[1]

    def set_tonemapping(self, hist, avg: float) -> None:
        h = (C.c_uint32 * 256)(*[int(x) for x in hist]) if hist is not None else None
        self.lib.orc_set_tonemapping(self.h, h, C.c_float(avg))


# --- codecs for the known-answer tests ---------------------------------------------------
def encode_e5(r, g, b) -> int:
    return load().orc_encode_e5(r, g, b)


def decode_e5(p: int):
    out = (C.c_float * 3)()
    load().orc_decode_e5(p, out)
    return tuple(out)


def encode_b10g11r11(r, g, b) -> int:
    return load().orc_encode_b10g11r11(r, g, b)


def decode_b10g11r11(p: int):
    out = (C.c_float * 3)()
    load().orc_decode_b10g11r11(p, out)
    return tuple(out)


def f32_to_f16(x: float) -> int:
    return load().orc_f32_to_f16(x)


def f16_to_f32(h: int) -> float:
    return load().orc_f16_to_f32(h)


def f32_to_bf16(x: float) -> int:
    return load().orc_f32_to_bf16(x)


def encode_normal(x, y, z) -> int:
    return load().orc_encode_normal(x, y, z)


def decode_normal(p: int):
    out = (C.c_float * 3)()
    load().orc_decode_normal(p, out)
    return tuple(out)


def color_bin(lum: float, min_log: float, max_log: float) -> int:
    return load().orc_color_bin(lum, min_log, max_log)


# --- AMD LPM (709 -> 709, no shoulder) for the known-answer tests -------------------------
def lpm_setup(saturation=(0.0, 0.0, 0.0), crosstalk=(1.0, 1.0, 1.0)) -> dict:
    """The LpmFilter constants: saturation powers, contrast, tone scale/bias, luma weights."""
    sat, ct, out = (C.c_float * 3)(*saturation), (C.c_float * 3)(*crosstalk), (C.c_float * 16)()
    load().orc_lpm_setup(sat, ct, out)
    v = list(out)
    return {"saturation": v[0:3], "contrast": v[3], "tone_scale_bias": v[4:6], "luma": v[6:9],
            "rcp_luma": v[9:12], "crosstalk": v[12:15]}


def lpm_filter(rgb, saturation=(0.0, 0.0, 0.0), crosstalk=(1.0, 1.0, 1.0)):
    sat, ct, c = (C.c_float * 3)(*saturation), (C.c_float * 3)(*crosstalk), (C.c_float * 3)(*rgb)
    load().orc_lpm_filter(sat, ct, c)
    return tuple(c)
