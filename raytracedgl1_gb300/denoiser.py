"""Python host mirror of the reference's interface for this path, over the C ABI.

    RTGL1::Denoiser      (Source/Denoiser.h:31-69)     -> Denoiser.Denoise(frameIndex, uniform)
    RTGL1::Tonemapping   (Source/Tonemapping.h:33-79)  -> Tonemapping.CalculateExposure(frameIndex, uniform)
    RTGL1::Framebuffers  (Source/Framebuffers.h)       -> Framebuffers (per stream)

Errors surface as ``RgdnError`` carrying the C status (the reference turns RgException into
RgResult at its API, Source/RTGL1.cpp:145-195). Every compute call goes through librgdn.so;
there is no Python fallback.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _native as N

# numpy view of each texel format: (dtype, channels per texel)
FORMAT_NUMPY = {
    1: (np.uint8, 1),    # R8_UINT
    2: (np.uint8, 2),    # RG8_UNORM
    3: (np.uint8, 4),    # RGBA8_UNORM
    4: (np.uint16, 1),   # R16_SFLOAT (bits)
    5: (np.uint16, 2),   # RG16_SFLOAT
    6: (np.uint16, 4),   # RGBA16_SFLOAT
    7: (np.uint16, 4),   # RGBA16_BFLOAT
    8: (np.float32, 1),  # R32_SFLOAT
    9: (np.float32, 2),  # RG32_SFLOAT
    10: (np.float32, 4),  # RGBA32_SFLOAT
    11: (np.uint32, 1),  # R32_UINT
    12: (np.uint32, 1),  # E5B9G9R9
    13: (np.uint32, 1),  # B10G11R11
    14: (np.uint32, 1),  # NORMAL_SPHERICAL
    15: (np.uint32, 4),  # RGBA32_UINT
}


def _stream_handle(cuda_stream) -> Optional[int]:
    """Accepts None (legacy default stream), an int handle, or a torch.cuda.Stream."""
    if cuda_stream is None:
        return None
    if isinstance(cuda_stream, int):
        return cuda_stream
    return int(cuda_stream.cuda_stream)


class Context:
    """One CUDA device, its normal-decode tables and the streams' memory budget."""

    def __init__(self, device: int = 0, memory_budget_bytes: int = 0, flags: int = 0):
        """flags: CONTEXT_* (CONTEXT_NO_L2_PERSIST for contexts that run frames side by side)."""
        self.lib = N.load()
        info = N.ContextCreateInfo(device, memory_budget_bytes, flags)
        h = C.c_void_p()
        N.check(self.lib.rgdn_context_create(C.byref(info), C.byref(h)), "rgdn_context_create")
        self.handle = h

    def close(self) -> None:
        if self.handle:
            N.check(self.lib.rgdn_context_destroy(self.handle), "rgdn_context_destroy")
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def memory_used(self) -> int:
        v = C.c_uint64()
        N.check(self.lib.rgdn_context_memory_used(self.handle, C.byref(v)))
        return v.value

    def launch_count(self) -> int:
        v = C.c_uint64()
        N.check(self.lib.rgdn_context_launch_count(self.handle, C.byref(v)))
        return v.value

    def submit_batch(self, jobs, cuda_stream=None) -> None:
        """jobs: iterable of (Stream, frameIndex, FrameParams)."""
        jobs = list(jobs)
        arr = (N.Job * len(jobs))()
        keep = []
        for i, (s, fi, p) in enumerate(jobs):
            keep.append(p)
            arr[i] = N.Job(s.handle, fi, C.pointer(p))
        N.check(self.lib.rgdn_submit_batch(self.handle, arr, len(jobs), _stream_handle(cuda_stream)),
                "rgdn_submit_batch")

    def batch_config(self, storage: int) -> "N.BatchConfig":
        cfg = N.BatchConfig()
        N.check(self.lib.rgdn_batch_get_config(self.handle, storage, C.byref(cfg)), "rgdn_batch_get_config")
        return cfg

    def set_batch_config(self, storage: int, cfg: "N.BatchConfig") -> None:
        N.check(self.lib.rgdn_batch_set_config(self.handle, storage, C.byref(cfg)), "rgdn_batch_set_config")

    def set_batch_timing(self, enable: bool) -> None:
        N.check(self.lib.rgdn_batch_set_timing(self.handle, 1 if enable else 0), "rgdn_batch_set_timing")

    def read_batch_timing(self) -> dict:
        """{(stage name, iteration): (launches, total ms)} of the timed batched launches."""
        buf = (N.StageTiming * 64)()
        n = C.c_uint32()
        N.check(self.lib.rgdn_batch_read_timing(self.handle, buf, 64, C.byref(n)), "rgdn_batch_read_timing")
        return {(N.KERNEL_NAMES.get(buf[i].stage, str(buf[i].stage)), buf[i].iteration): (buf[i].launches, buf[i].totalMs)
                for i in range(min(n.value, 64))}


def required_bytes(width: int, height: int, storage: int) -> int:
    lib = N.load()
    info = N.StreamCreateInfo(width, height, storage)
    v = C.c_uint64()
    N.check(lib.rgdn_stream_required_bytes(C.byref(info), C.byref(v)), "rgdn_stream_required_bytes")
    return v.value


class Stream:
    """One camera stream: its framebuffer set, temporal history and tonemapping state."""

    def __init__(self, ctx: Context, width: int, height: int, storage: int = N.STORAGE_REF):
        self.ctx, self.lib = ctx, ctx.lib
        info = N.StreamCreateInfo(width, height, storage)
        h = C.c_void_p()
        N.check(self.lib.rgdn_stream_create(ctx.handle, C.byref(info), C.byref(h)), "rgdn_stream_create")
        self.handle = h
        self.width, self.height, self.storage = width, height, storage

    @classmethod
    def borrowed(cls, ctx: Context, handle, width: int, height: int, storage: int) -> "Stream":
        """A view of a stream another owner (a Server) created and destroys."""
        s = cls.__new__(cls)
        s.ctx, s.lib, s.handle = ctx, ctx.lib, handle
        s.width, s.height, s.storage = width, height, storage
        s._borrowed = True
        return s

    def close(self) -> None:
        if self.handle and not getattr(self, "_borrowed", False):
            N.check(self.lib.rgdn_stream_destroy(self.handle), "rgdn_stream_destroy")
        self.handle = None

    def __del__(self):
        try:
            if self.ctx.handle:
                self.close()
        except Exception:
            pass

    def resize(self, width: int, height: int) -> None:
        N.check(self.lib.rgdn_stream_resize(self.handle, width, height), "rgdn_stream_resize")
        self.width, self.height = width, height

    # --- Framebuffers --------------------------------------------------------------------
    def image(self, fb, frame_index: int = 0) -> N.Image:
        fb = N.FB[fb] if isinstance(fb, str) else fb
        img = N.Image()
        N.check(self.lib.rgdn_stream_get_framebuffer(self.handle, fb, frame_index, C.byref(img)),
                "rgdn_stream_get_framebuffer")
        return img

    def bind(self, fb, frame_index: int, device_ptr: int | None) -> None:
        """Zero-copy: the G-buffer image `fb` of slot frame_index reads caller device memory."""
        fbi = N.FB[fb] if isinstance(fb, str) else fb
        N.check(self.lib.rgdn_stream_bind_framebuffer(self.handle, fbi, frame_index,
                                                      C.c_void_p(device_ptr) if device_ptr else None),
                f"bind {fb}")

    def upload(self, fb, frame_index: int, src, cuda_stream=None) -> None:
        """src: a numpy array (host) or an (int device pointer, nbytes) pair."""
        fbi = N.FB[fb] if isinstance(fb, str) else fb
        if isinstance(src, tuple):
            ptr, nbytes = src
        else:
            arr = np.ascontiguousarray(src)
            ptr, nbytes = arr.ctypes.data, arr.nbytes
        N.check(self.lib.rgdn_stream_upload(self.handle, fbi, frame_index, C.c_void_p(ptr), nbytes,
                                            _stream_handle(cuda_stream)), f"upload {fb}")
        if not isinstance(src, tuple) and cuda_stream is None:
            self.synchronize()

    def download(self, fb, frame_index: int = 0, cuda_stream=None) -> np.ndarray:
        img = self.image(fb, frame_index)
        if not img.data:
            raise N.RgdnError(N.WRONG_FUNCTION_ARGUMENT, f"{fb} does not exist in this storage mode")
        dt, ch = FORMAT_NUMPY[img.format]
        shape = (img.height, img.width) if ch == 1 else (img.height, img.width, ch)
        out = np.empty(shape, dtype=dt)
        fbi = N.FB[fb] if isinstance(fb, str) else fb
        N.check(self.lib.rgdn_stream_download(self.handle, fbi, frame_index, C.c_void_p(out.ctypes.data),
                                              out.nbytes, _stream_handle(cuda_stream)), f"download {fb}")
        self.synchronize(cuda_stream)
        return out

    def synchronize(self, cuda_stream=None) -> None:
        # a tonemapping read synchronises the stream; cheap (1 KB)
        N.check(self.lib.rgdn_get_tonemapping(self.handle, None, None, None, _stream_handle(cuda_stream)))

    # --- tonemapping state ---------------------------------------------------------------
    def take_device_errors(self, cuda_stream=None) -> int:
        """Device-side failure flags since the last call (N.DEVICE_ERROR_*), cleared."""
        out = C.c_uint32()
        N.check(self.lib.rgdn_stream_take_device_errors(self.handle, C.byref(out), _stream_handle(cuda_stream)),
                "rgdn_stream_take_device_errors")
        return out.value

    def tonemapping(self, cuda_stream=None):
        hist = (C.c_uint32 * 256)()
        avg = C.c_float()
        exp = C.c_float()
        N.check(self.lib.rgdn_get_tonemapping(self.handle, hist, C.byref(avg), C.byref(exp),
                                              _stream_handle(cuda_stream)), "rgdn_get_tonemapping")
        return np.frombuffer(hist, dtype=np.uint32).copy(), avg.value, exp.value

    def set_tonemapping(self, hist, avg_luminance: float, cuda_stream=None) -> None:
        h = (C.c_uint32 * 256)(*[int(x) for x in hist]) if hist is not None else None
        N.check(self.lib.rgdn_set_tonemapping(self.handle, h, C.c_float(avg_luminance),
                                              _stream_handle(cuda_stream)), "rgdn_set_tonemapping")

    def tonemapping_device_ptr(self) -> int:
        p = C.c_void_p()
        N.check(self.lib.rgdn_stream_tonemapping_device(self.handle, C.byref(p)))
        return p.value

    # --- per-kernel timing ----------------------------------------------------------------
    def set_timing(self, enable: bool) -> None:
        N.check(self.lib.rgdn_stream_set_timing(self.handle, 1 if enable else 0))

    def read_timing(self) -> dict:
        """{(stage name, iteration): (launches, total ms)} since the last read."""
        cap = 64
        buf = (N.StageTiming * cap)()
        n = C.c_uint32()
        N.check(self.lib.rgdn_stream_read_timing(self.handle, buf, cap, C.byref(n)), "rgdn_stream_read_timing")
        return {(N.KERNEL_NAMES.get(t.stage, str(t.stage)), t.iteration): (t.launches, t.totalMs)
                for t in buf[:min(n.value, cap)]}

    def set_reshade_scene(self, lights_ptr=None, light_count=0, prev_to_cur_ptr=None, prev_light_count=0,
                          occluders_ptr=None, occluder_count=0) -> None:
        """Gradient re-shading on the device from these device arrays (rgdn_sphere_light,
        uint32 previous-to-current light indices, rgdn_occluder); lights_ptr None clears it, and
        the producer's RGDN_FB_GRADIENT_RESHADED image is used again."""
        if lights_ptr is None:
            N.check(self.lib.rgdn_stream_set_reshade_scene(self.handle, None), "rgdn_stream_set_reshade_scene")
            return
        sc = N.ReshadeScene(lights_ptr, light_count, prev_to_cur_ptr, prev_light_count, occluders_ptr, occluder_count)
        N.check(self.lib.rgdn_stream_set_reshade_scene(self.handle, C.byref(sc)), "rgdn_stream_set_reshade_scene")

    # --- stages --------------------------------------------------------------------------
    def stage(self, stage: int, iteration: int, frame_index: int, params: N.FrameParams,
              cuda_stream=None) -> None:
        N.check(self.lib.rgdn_denoise_stage(self.handle, stage, iteration, frame_index, C.byref(params),
                                            _stream_handle(cuda_stream)), f"rgdn_denoise_stage {stage}")


class Denoiser:
    """Denoiser::Denoise(cmd, frameIndex, uniform) — Source/Denoiser.cpp:64-255."""

    def __init__(self, stream: Stream):
        self.stream = stream

    def Denoise(self, frameIndex: int, uniform: N.FrameParams, cuda_stream=None) -> None:
        s = self.stream
        N.check(s.lib.rgdn_denoise(s.handle, frameIndex, C.byref(uniform), _stream_handle(cuda_stream)),
                "rgdn_denoise")


class ImageComposition:
    """ImageComposition::PrepareForRaster + Finalize (Source/ImageComposition.cpp:87-155), without
    rasterised geometry in between: CmCheckerboard.comp + CmPrepareFinal.comp into FINAL and
    BLOOM_INPUT, from PRE_FINAL, SCREEN_EMIS_RT, SCATTERING and the adapted average luminance."""

    def __init__(self, stream: Stream):
        self.stream = stream

    def Finalize(self, frameIndex: int, params: N.FinalParams = None, cuda_stream=None) -> None:
        s = self.stream
        p = params if params is not None else N.FinalParams.defaults()
        N.check(s.lib.rgdn_prepare_final(s.handle, frameIndex, C.byref(p), _stream_handle(cuda_stream)),
                "rgdn_prepare_final")


class Bloom:
    """Bloom::Prepare + Apply (Source/Bloom.cpp:94-240): the 8-level bloom pyramid of BLOOM_INPUT,
    added to FINAL with the given intensity (without the lens-dirt texture term)."""

    def __init__(self, stream: Stream):
        self.stream = stream

    def Apply(self, frameIndex: int, bloomIntensity: float = 1.0, cuda_stream=None) -> None:
        s = self.stream
        p = N.BloomParams(bloomIntensity)
        N.check(s.lib.rgdn_bloom(s.handle, frameIndex, C.byref(p), _stream_handle(cuda_stream)), "rgdn_bloom")


class Volumetric:
    """Volumetric::ProcessScattering (Source/Volumetric.cpp:71-190): the froxel volume of
    SCATTER_VOLUME integrated front to back in place, then SCATTERING and SCATTERING_HISTORY
    accumulated over frames per pixel. Call between Denoise and CalculateExposure."""

    def __init__(self, stream: Stream):
        self.stream = stream

    def ProcessScattering(self, frameIndex: int, params: N.VolumetricParams, cuda_stream=None) -> None:
        s = self.stream
        N.check(s.lib.rgdn_process_scattering(s.handle, frameIndex, C.byref(params), _stream_handle(cuda_stream)),
                "rgdn_process_scattering")


class Tonemapping:
    """Tonemapping::CalculateExposure(cmd, frameIndex, uniform) — Source/Tonemapping.cpp:59-165."""

    def __init__(self, stream: Stream):
        self.stream = stream

    def CalculateExposure(self, frameIndex: int, uniform: N.FrameParams, cuda_stream=None) -> None:
        s = self.stream
        N.check(s.lib.rgdn_calculate_exposure(s.handle, frameIndex, C.byref(uniform),
                                              _stream_handle(cuda_stream)), "rgdn_calculate_exposure")

    def GetTonemapping(self, cuda_stream=None):
        """(histogram[256], avgLuminance, exposure) after the work on cuda_stream."""
        return self.stream.tonemapping(cuda_stream)


def histogram_bin_table(min_log: float, max_log: float) -> np.ndarray:
    lib = N.load()
    out = np.empty(65536, dtype=np.uint8)
    N.check(lib.rgdn_histogram_bin_table(C.c_float(min_log), C.c_float(max_log),
                                         out.ctypes.data_as(C.POINTER(C.c_uint8))))
    return out


def copy_host_planes(copies, host_copy: int = N.HOST_COPY_SM, cuda_stream=None) -> None:
    """rgdn_copy_host_planes: copies [(device pointer, host pointer, bytes), ...] (at most
    RGDN_GBUFFER_PLANES) asynchronously on cuda_stream, pinned device-mapped ranges by one SM
    kernel with HOST_COPY_SM, the others (and all with HOST_COPY_ENGINE) by cudaMemcpyAsync."""
    lib = N.load()
    n = len(copies)
    dst = (C.c_void_p * n)(*[c[0] for c in copies])
    src = (C.c_void_p * n)(*[c[1] for c in copies])
    nb = (C.c_size_t * n)(*[c[2] for c in copies])
    N.check(lib.rgdn_copy_host_planes(dst, src, nb, n, host_copy, _stream_handle(cuda_stream)), "rgdn_copy_host_planes")


class Server:
    """rgdn_server: continuous batching of frame requests from many camera streams, each
    stream's history resident on the device, admission under the context's memory budget."""

    def __init__(self, ctx: Context, storage: int, max_frames_per_step: int = 0, max_pixels_per_step: int = 0,
                 max_queued_per_stream: int = 0, steps_in_flight: int = 2, evict_idle_ms: int = 0,
                 host_copy: int = N.HOST_COPY_ENGINE):
        self.ctx, self.lib, self.storage = ctx, ctx.lib, storage
        info = N.ServerCreateInfo(storage, max_frames_per_step, max_pixels_per_step, max_queued_per_stream,
                                  steps_in_flight, evict_idle_ms, host_copy)
        h = C.c_void_p()
        N.check(self.lib.rgdn_server_create(ctx.handle, C.byref(info), C.byref(h)), "rgdn_server_create")
        self.handle = h
        self.sizes = {}

    def close(self) -> None:
        if self.handle:
            N.check(self.lib.rgdn_server_destroy(self.handle), "rgdn_server_destroy")
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def open_stream(self, width: int, height: int) -> int:
        v = C.c_uint32()
        N.check(self.lib.rgdn_server_open_stream(self.handle, width, height, C.byref(v)), "rgdn_server_open_stream")
        self.sizes[v.value] = (width, height)
        return v.value

    def close_stream(self, sid: int) -> None:
        N.check(self.lib.rgdn_server_close_stream(self.handle, sid), "rgdn_server_close_stream")
        self.sizes.pop(sid, None)

    @staticmethod
    def request(sid: int, params: N.FrameParams, gbuffer: dict, mode: int = N.REQUEST_COPY,
                pre_final_out: int | None = None) -> N.FrameRequest:
        """gbuffer: {G-buffer image name: pointer (host or device int)}."""
        r = N.FrameRequest()
        r.stream, r.gbufferMode = sid, mode
        for name, ptr in gbuffer.items():
            r.gbuffer[N.GBUFFER.index(name)] = ptr
        r.preFinalOut = pre_final_out
        C.memmove(C.byref(r.params), C.byref(params), C.sizeof(N.FrameParams))
        return r

    def submit(self, request: N.FrameRequest) -> int:
        t = C.c_uint64()
        N.check(self.lib.rgdn_server_submit(self.handle, C.byref(request), C.byref(t)), "rgdn_server_submit")
        return t.value

    def wait(self, ticket: int, timeout_ms: int = 60000) -> N.FrameResult:
        res = N.FrameResult()
        N.check(self.lib.rgdn_server_wait(self.handle, ticket, timeout_ms, C.byref(res)), "rgdn_server_wait")
        return res

    def drain(self) -> None:
        N.check(self.lib.rgdn_server_drain(self.handle), "rgdn_server_drain")

    def stats(self) -> dict:
        st = N.ServerStats()
        N.check(self.lib.rgdn_server_stats_get(self.handle, C.byref(st)), "rgdn_server_stats_get")
        return {name: getattr(st, name) for name, _ in N.ServerStats._fields_}

    def reset_stats(self) -> None:
        N.check(self.lib.rgdn_server_stats_reset(self.handle), "rgdn_server_stats_reset")

    def stream(self, sid: int) -> Optional[Stream]:
        h = C.c_void_p()
        N.check(self.lib.rgdn_server_get_stream(self.handle, sid, C.byref(h)), "rgdn_server_get_stream")
        if not h.value:
            return None
        w, hh = self.sizes[sid]
        return Stream.borrowed(self.ctx, h, w, hh, self.storage)
