"""Seeded synthetic frames (librgdn_scene.so): the G-buffer and noisy radiance a path tracer
would hand to the denoiser, in the reference's framebuffer formats and checkerboard layout.
Used by the tests, the smoke check and the benchmark as the stand-in for captured frames."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _native as N

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib", "librgdn_scene.so")


class SceneDesc(C.Structure):
    _fields_ = [
        ("seed", C.c_uint64), ("sigma", C.c_float), ("fireflyProb", C.c_float),
        ("fireflyMult", C.c_float), ("cameraPxPerFrame", C.c_float), ("spherePxPerFrame", C.c_float),
        ("timeDelta", C.c_float), ("ev100Min", C.c_float), ("ev100Max", C.c_float),
        ("lightFlickerFrom", C.c_float), ("lightFlickerGain", C.c_float),
        ("atrousIterations", C.c_uint32), ("antiFirefly", C.c_uint32), ("reshadeLights", C.c_uint32),
    ]


class SceneFrame(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in (
        "albedo", "isSky", "normal", "metallicRoughness", "depthWorld", "depthGrad", "motion",
        "unfilteredDirect", "unfilteredSpecular", "unfilteredIndir", "surfacePosition",
        "viewDirection", "throughput", "gradientInputs", "gradientReshaded", "reservoirs")]


# framebuffer name -> (SceneFrame field, dtype, channels)
_LAYOUT = {
    "ALBEDO": ("albedo", np.uint32, 1),
    "IS_SKY": ("isSky", np.uint8, 1),
    "NORMAL": ("normal", np.uint32, 1),
    "METALLIC_ROUGHNESS": ("metallicRoughness", np.uint8, 2),
    "DEPTH_WORLD": ("depthWorld", np.uint16, 1),
    "DEPTH_GRAD": ("depthGrad", np.uint16, 1),
    "MOTION": ("motion", np.uint16, 4),
    "UNFILTERED_DIRECT": ("unfilteredDirect", np.uint32, 1),
    "UNFILTERED_SPECULAR": ("unfilteredSpecular", np.uint32, 1),
    "UNFILTERED_INDIR": ("unfilteredIndir", np.uint32, 1),
    "SURFACE_POSITION": ("surfacePosition", np.float32, 4),
    "VIEW_DIRECTION": ("viewDirection", np.uint16, 4),
    "THROUGHPUT": ("throughput", np.uint16, 4),
    "GRADIENT_INPUTS": ("gradientInputs", np.uint16, 2),
    "GRADIENT_RESHADED": ("gradientReshaded", np.float32, 2),
    "RESERVOIRS": ("reservoirs", np.uint32, 4),
}

_lib = None


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -m raytracedgl1_gb300.build`")
        lib = C.CDLL(LIB_PATH)
        lib.rgdn_scene_desc_default.argtypes = [C.POINTER(SceneDesc)]
        lib.rgdn_scene_create.restype = C.c_void_p
        lib.rgdn_scene_create.argtypes = [C.c_uint32, C.c_uint32, C.POINTER(SceneDesc)]
        lib.rgdn_scene_destroy.argtypes = [C.c_void_p]
        lib.rgdn_scene_generate.restype = C.c_int
        lib.rgdn_scene_generate.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(SceneFrame),
                                            C.POINTER(N.FrameParams), C.c_int]
        lib.rgdn_scene_reshade.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(N.SphereLight),
                                           C.POINTER(N.Occluder), C.POINTER(C.c_uint32)]
        _lib = lib
    return _lib


def default_desc(**overrides) -> SceneDesc:
    d = SceneDesc()
    _load().rgdn_scene_desc_default(C.byref(d))
    for k, v in overrides.items():
        setattr(d, k, v)
    return d


class Scene:
    def __init__(self, width: int, height: int, **desc):
        self.lib = _load()
        self.desc = default_desc(**desc)
        self.handle = self.lib.rgdn_scene_create(width, height, C.byref(self.desc))
        if not self.handle:
            raise ValueError("scene size must be even and non-empty")
        self.width, self.height = width, height

    def __del__(self):
        if getattr(self, "handle", None):
            self.lib.rgdn_scene_destroy(self.handle)
            self.handle = None

    def planes(self) -> list:
        """The framebuffers this scene writes: RESERVOIRS only for a re-shading scene."""
        return [n for n in _LAYOUT if n != "RESERVOIRS" or self.desc.reshadeLights]

    def alloc(self, pinned=None) -> dict:
        """Host buffers for one frame. `pinned`: optional callable(nbytes) -> numpy uint8 array."""
        out = {}
        for name in self.planes():
            _, dt, ch = _LAYOUT[name]
            shape = (self.height, self.width) if ch == 1 else (self.height, self.width, ch)
            if pinned is not None:
                nbytes = int(np.prod(shape)) * np.dtype(dt).itemsize
                out[name] = pinned(nbytes).view(dt).reshape(shape)
            else:
                out[name] = np.empty(shape, dtype=dt)
        return out

    def generate(self, frame: int, out: dict | None = None, nthreads: int = 0):
        """Fills (or allocates) the G-buffer of `frame`; returns (buffers, FrameParams)."""
        if out is None:
            out = self.alloc()
        sf = SceneFrame()
        for name in self.planes():
            setattr(sf, _LAYOUT[name][0], out[name].ctypes.data)
        params = N.FrameParams()
        if nthreads <= 0:
            nthreads = min(32, os.cpu_count() or 1)
        r = self.lib.rgdn_scene_generate(self.handle, frame, C.byref(sf), C.byref(params), nthreads)
        N.check(r, "rgdn_scene_generate")
        return out, params

    def reshade(self, frame: int):
        """The re-shading scene of `frame`: (lights, previous-to-current light map, occluders) as
        ctypes arrays (one sphere light, light 0 of the previous frame mapped to it, seven
        occluders), for rgdn_stream_set_reshade_scene (after a copy to the device) and the oracle."""
        light = (N.SphereLight * 1)()
        occ = (N.Occluder * 16)()
        n = C.c_uint32()
        self.lib.rgdn_scene_reshade(self.handle, frame, light, occ, C.byref(n))
        return light, (C.c_uint32 * 1)(0), (N.Occluder * n.value)(*occ[:n.value])
