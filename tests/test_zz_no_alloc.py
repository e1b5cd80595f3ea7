"""rgdn_gradient_atrous_noalloc against the stream path (RGDN_STAGE_GRADIENT_ATROUS x4).

The entry point serves callers that may not allocate device memory (a host that owns every
allocation, or a frame loop that cannot take cudaMalloc's device synchronisation); its one
intermediate image is a fixed array inside the library. This file is collected last so that a
run stopping at its first failure has already run every other test; it also passes alone.
"""
import ctypes as C

import numpy as np
import pytest

from raytracedgl1_gb300 import _native as N
from raytracedgl1_gb300.denoiser import Context, Stream
from raytracedgl1_gb300.scene import Scene

pytestmark = pytest.mark.gpu


def stream_reference(ctx, W, H, seed, frames=3):
    """Gradient samples and the 4 filtered iterations through the stream's own images."""
    sc = Scene(W, H, seed=seed, lightFlickerFrom=1.0)
    s = Stream(ctx, W, H, N.STORAGE_REF)
    for f in range(frames):
        fi = f & 1
        bufs, p = sc.generate(f)
        for name, arr in bufs.items():
            s.upload(name, fi, arr)
        s.stage(N.STAGE_GRADIENT_SAMPLES, 0, fi, p)
        samples = s.download("DIS_PING_GRADIENT", fi)
        for i in range(4):
            s.stage(N.STAGE_GRADIENT_ATROUS, i, fi, p)
        # finish the frame so the next one sees a consistent history
        for st, it in [(N.STAGE_TEMPORAL_ACCUMULATION, 0), (N.STAGE_ANTI_FIREFLY, 0),
                       (N.STAGE_VARIANCE_ESTIMATION, 0)] + [(N.STAGE_ATROUS, i) for i in range(4)]:
            s.stage(st, it, fi, p)
    out = (samples, s.download("DIS_PING_GRADIENT", fi), s.download("DIS_GRADIENT_HISTORY", fi))
    s.close()
    return out


def call_noalloc(samples, W, H):
    import torch
    dev = torch.device("cuda", 0)
    src = torch.from_numpy(np.ascontiguousarray(samples).view(np.uint8).reshape(-1)).to(dev)
    filtered = torch.full_like(src, 0xAB)   # poisoned: every texel must be overwritten
    history = torch.full_like(src, 0xCD)
    lib = N.load()
    st = torch.cuda.current_stream(dev)
    r = lib.rgdn_gradient_atrous_noalloc(C.c_void_p(src.data_ptr()), C.c_void_p(filtered.data_ptr()),
                                         C.c_void_p(history.data_ptr()), W, H, C.c_void_p(st.cuda_stream))
    assert r == N.SUCCESS, lib.rgdn_status_string(r)
    torch.cuda.synchronize(dev)
    shape = samples.shape
    return filtered.cpu().numpy().reshape(shape), history.cpu().numpy().reshape(shape)


def test_noalloc_matches_stream_path_twice_in_a_row():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ctx = Context(0)
    # two calls in a row, different sizes: the second sees the first call's leftover scratch
    for (W, H), seed in (((130, 76), 31), ((64, 37), 32)):
        samples, ref_filtered, ref_history = stream_reference(ctx, W, H, seed)
        filtered, history = call_noalloc(samples, W, H)
        assert np.array_equal(filtered, ref_filtered), f"{W}x{H}: filtered gradients differ"
        assert np.array_equal(history, ref_history), f"{W}x{H}: gradient history differs"
    ctx.close()


def test_noalloc_at_the_stated_maximum():
    """3840x2160 (exactly the 1280 x 720 strata the fixed scratch holds) is accepted and gives the
    stream path's images bit for bit, on seeded random samples."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    W, H = 3840, 2160
    ctx = Context(0)
    s = Stream(ctx, W, H, N.STORAGE_REF)
    rng = np.random.default_rng(41)
    shape = (s.image("DIS_PING_GRADIENT", 0).height, s.image("DIS_PING_GRADIENT", 0).width)
    assert shape == (720, 1280)
    samples = rng.integers(0, 256, size=shape + (4,), dtype=np.uint8)   # rgba8 per stratum
    s.upload("DIS_PING_GRADIENT", 0, samples)
    p = N.FrameParams()
    p.minLogLuminance, p.maxLogLuminance = -3.0, 7.0
    for i in range(4):
        s.stage(N.STAGE_GRADIENT_ATROUS, i, 0, p)
    ref_filtered, ref_history = s.download("DIS_PING_GRADIENT", 0), s.download("DIS_GRADIENT_HISTORY", 0)
    s.close()
    ctx.close()
    filtered, history = call_noalloc(samples, W, H)
    assert np.array_equal(filtered, ref_filtered), "filtered gradients differ at the maximum size"
    assert np.array_equal(history, ref_history), "gradient history differs at the maximum size"


def test_noalloc_rejects_oversized_and_bad_arguments():
    lib = N.load()
    bufs = [(C.c_uint32 * 4)() for _ in range(3)]
    a, b, c = (C.cast(x, C.c_void_p) for x in bufs)
    # 3842 x 2162 needs 1281 x 721 strata, beyond the fixed 1280 x 720 scratch
    assert lib.rgdn_gradient_atrous_noalloc(a, b, c, 3842, 2162, None) == N.WRONG_FUNCTION_ARGUMENT
    assert lib.rgdn_gradient_atrous_noalloc(a, b, c, 63, 36, None) == N.WRONG_FUNCTION_ARGUMENT   # odd width
    assert lib.rgdn_gradient_atrous_noalloc(None, b, c, 64, 36, None) == N.WRONG_FUNCTION_ARGUMENT
    # the three images must be distinct
    assert lib.rgdn_gradient_atrous_noalloc(a, b, a, 64, 36, None) == N.WRONG_FUNCTION_ARGUMENT   # history = samples
    assert lib.rgdn_gradient_atrous_noalloc(a, a, c, 64, 36, None) == N.WRONG_FUNCTION_ARGUMENT   # filtered = samples
    assert lib.rgdn_gradient_atrous_noalloc(a, b, b, 64, 36, None) == N.WRONG_FUNCTION_ARGUMENT   # filtered = history
