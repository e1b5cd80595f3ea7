"""GPU parity: librgdn's CUDA stages against the CPU oracle, through the C ABI.

Per stage: the GPU's whole framebuffer state is copied into the oracle, the one stage runs on
both, then every plane of both frame slots is compared — planes the stage does not write must
stay bit-identical, planes it writes must agree to within the storage format's quantum
(fp32 storage: 1e-3 relative per texel, the FP32-mode bar).

End to end: the GPU and the oracle run the same frames independently (no state sync), and the
outputs are compared per pixel. Histograms are compared bit-exact on the same HistogramInput.
"""
import numpy as np
import pytest

from raytracedgl1_gb300 import _native as N
from raytracedgl1_gb300.denoiser import Bloom, Denoiser, ImageComposition, Stream, Tonemapping, Volumetric
from raytracedgl1_gb300.scene import Scene

import oracle
from tests import _formats as F

pytestmark = pytest.mark.gpu

MODES = [("ref", N.STORAGE_REF), ("fp32", N.STORAGE_FP32), ("fp16", N.STORAGE_FP16), ("bf16", N.STORAGE_BF16)]
# sizes: W%3 in {1, 2, 0}, odd heights, a width whose half is odd
SIZES = [(64, 36), (50, 23), (34, 17)]

# The FP32 variance planes hold E[l^2] - E[l]^2 of weighted moments: the cancellation scales
# an ulp of the weights (CUDA's and the host's expf / powf differ by up to one) by
# E[l^2] / variance, so they get a wider per-texel bound than the other FP32 planes.
VARIANCE_PLANES = ("DIFF_PING_VARIANCE", "DIFF_PONG_VARIANCE", "DIFF_COLOR_HISTORY_VARIANCE")
VARIANCE_TOL = 2e-2

# per-texel tolerance (relative to the texel's largest channel) of each stored format
TOL = {F.F_E5: 2.0 ** -7, F.F_RGBA16F: 2.0 ** -9, F.F_RG16F: 2.0 ** -9, F.F_R16F: 2.0 ** -9,
       F.F_RGBA16BF: 2.0 ** -6, F.F_RGBA8: 1.01 / 255.0, F.F_B10G11R11: 2.0 ** -5,
       F.F_R32F: 1e-3, F.F_RG32F: 1e-3, F.F_RGBA32F: 1e-3}


def gpu_planes(s: Stream):
    out = {}
    for name in N.FB_NAMES:
        img = s.image(name, 0)
        if not img.data:
            continue
        for slot in ((0, 1) if img.has_prev else (0,)):
            out[(name, slot)] = (s.download(name, slot), img.format)
    return out


def sync_to_oracle(s: Stream, o: oracle.OracleStream):
    for (name, slot), (arr, fmt) in gpu_planes(s).items():
        assert o.fmt(name) == fmt, f"format table mismatch for {name}"
        o.plane(name, slot)[...] = arr
    hist, avg, _ = s.tonemapping()
    o.set_tonemapping(hist, avg)


def compare_state(s: Stream, o: oracle.OracleStream, what: str, max_diff_frac: float = 0.02):
    worst = []
    for (name, slot), (g, fmt) in gpu_planes(s).items():
        c = o.plane(name, slot)
        if np.array_equal(g, c):
            continue
        gd, cd = F.decode(g, fmt), F.decode(c, fmt)
        if fmt in (F.F_R8U, F.F_R32U, F.F_NORMAL, F.F_RGBA32U):
            bad = int(np.count_nonzero(gd != cd))
            raise AssertionError(f"{what}: integer plane {name}[{slot}] differs at {bad} texels")
        scale = np.percentile(np.abs(cd[np.isfinite(cd)]), 99) if np.isfinite(cd).any() else 1.0
        err = F.texel_rel_err(gd, cd, atol=max(1e-6, 1e-4 * float(scale)))
        tol = VARIANCE_TOL if name in VARIANCE_PLANES else TOL[fmt]
        ndiff = int(np.count_nonzero(np.any(g != c, axis=-1) if g.ndim == 3 else g != c))
        frac = ndiff / err.size
        worst.append((name, slot, float(err.max()), frac))
        assert err.max() <= tol, f"{what}: {name}[{slot}] max texel rel err {err.max():.3e} > {tol:.3e}"
        if fmt not in (F.F_R32F, F.F_RG32F, F.F_RGBA32F):
            # quantised planes: ulp-level differences of the transcendentals flip a stored
            # quantum only rarely; fp32 planes are held to the 1e-3 relative bar alone
            assert frac <= max_diff_frac, f"{what}: {name}[{slot}] {frac:.2%} of texels differ"
    return worst


def upload_frame(s, o, bufs, fi):
    for name, arr in bufs.items():
        s.upload(name, fi, arr)
        if o is not None:
            o.load(name, fi, arr)


STAGE_SEQ = None


def stage_sequence(niter: int):
    seq = [(N.STAGE_GRADIENT_SAMPLES, 0)] + [(N.STAGE_GRADIENT_ATROUS, i) for i in range(4)]
    seq += [(N.STAGE_TEMPORAL_ACCUMULATION, 0), (N.STAGE_ANTI_FIREFLY, 0), (N.STAGE_VARIANCE_ESTIMATION, 0)]
    seq += [(N.STAGE_ATROUS, i) for i in range(niter)]
    seq += [(N.STAGE_LUMINANCE_HISTOGRAM, 0), (N.STAGE_LUMINANCE_AVG, 0)]
    return seq


@pytest.mark.parametrize("mode_name,mode", MODES)
@pytest.mark.parametrize("size", SIZES)
def test_stage_parity(ctx, mode_name, mode, size):
    W, H = size
    sc = Scene(W, H, seed=7, lightFlickerFrom=2.0)
    s = Stream(ctx, W, H, mode)
    o = oracle.OracleStream(W, H, mode)
    for f in range(4):
        fi = f & 1
        bufs, p = sc.generate(f)
        upload_frame(s, None, bufs, fi)
        for stage, it in stage_sequence(4):
            sync_to_oracle(s, o)
            s.stage(stage, it, fi, p)
            o.stage(stage, it, fi, p)
            compare_state(s, o, f"{mode_name} {W}x{H} frame {f} stage {stage}.{it}")
            if stage == N.STAGE_LUMINANCE_HISTOGRAM or stage == N.STAGE_LUMINANCE_AVG:
                hg, ag, _ = s.tonemapping()
                ho, ao, _ = o.tonemapping()
                assert np.array_equal(hg, ho), "histogram not bit-exact"
                assert np.float32(ag) == np.float32(ao), f"avgLuminance {ag!r} != {ao!r}"
    s.close()


@pytest.mark.parametrize("mode_name,mode", MODES)
def test_five_iterations_and_flags(ctx, mode_name, mode):
    """N=5 a-trous (the generalised routing), anti-firefly off, debug flags, gradients off."""
    W, H = 64, 36
    sc = Scene(W, H, seed=3)
    s = Stream(ctx, W, H, mode)
    o = oracle.OracleStream(W, H, mode)
    variants = [dict(atrousIterations=5), dict(antiFireflyEnabled=0), dict(debugShowFlags=1 << 6),
                dict(debugShowFlags=(1 << 9) | (1 << 5)), dict(lightmapScreenCoverage=0.3),
                dict(gradientMultDiffuse=0.0, gradientMultIndirect=0.0, gradientMultSpecular=0.0),
                dict(flags=N.FLAG_SKIP_GRADIENTS), dict(stopEyeAdaptation=1)]
    for f, var in enumerate(variants):
        fi = f & 1
        bufs, p = sc.generate(f)
        for k, v in var.items():
            setattr(p, k, v)
        upload_frame(s, None, bufs, fi)
        niter = p.atrousIterations or 4
        for stage, it in stage_sequence(niter):
            if p.flags & N.FLAG_SKIP_GRADIENTS and stage in (N.STAGE_GRADIENT_SAMPLES, N.STAGE_GRADIENT_ATROUS):
                continue
            sync_to_oracle(s, o)
            s.stage(stage, it, fi, p)
            o.stage(stage, it, fi, p)
            compare_state(s, o, f"{mode_name} variant {var} stage {stage}.{it}")
    s.close()


def run_frames(s, o, sc, frames, denoise_gpu=True):
    for f in range(frames):
        fi = f & 1
        bufs, p = sc.generate(f)
        upload_frame(s, o, bufs, fi)
        Denoiser(s).Denoise(fi, p)
        Tonemapping(s).CalculateExposure(fi, p)
        o.denoise(fi, p)
        o.calculate_exposure(fi, p)
    return (frames - 1) & 1


@pytest.mark.parametrize("mode_name,mode", MODES)
def test_end_to_end(ctx, mode_name, mode):
    """Independent multi-frame runs; PRE_FINAL compared per pixel."""
    W, H = 96, 54
    sc = Scene(W, H, seed=11, lightFlickerFrom=4.0)
    s = Stream(ctx, W, H, mode)
    o = oracle.OracleStream(W, H, mode)
    fi = run_frames(s, o, sc, 8)
    img = s.image("PRE_FINAL", fi)
    g = F.decode(s.download("PRE_FINAL", fi), img.format)
    c = F.decode(o.plane("PRE_FINAL", fi), img.format)
    err = F.texel_rel_err(g, c, atol=1e-4 * float(np.percentile(c, 99)))
    if mode == N.STORAGE_FP32:
        # the FP32-mode bar: 1e-3 relative per pixel
        assert err.max() <= 1e-3, f"max rel err {err.max():.3e}"
    else:
        # quantised storage: discrete flips of one quantum propagate over frames;
        # almost every pixel stays within 1e-2 and the image PSNR stays high
        assert np.mean(err <= 1e-2) >= 0.99, f"{np.mean(err <= 1e-2):.4f} of pixels within 1e-2"
        assert F.psnr(g, c) > 50.0
    s.close()


@pytest.mark.parametrize("path", ["plain", "fused"])
@pytest.mark.parametrize("mode_name,mode", MODES[:2])
def test_histogram_bit_exact_same_input(ctx, mode_name, mode, path):
    """Given the same HistogramInput bytes, the histogram and avgLuminance are bit-exact —
    for the separate histogram kernel (plain path) and for the histogram fused into the last
    a-trous iteration (default path)."""
    W, H = 128, 72
    sc = Scene(W, H, seed=5)
    s = Stream(ctx, W, H, mode)
    o = oracle.OracleStream(W, H, mode)
    run_frames(s, o, sc, 3)
    for f in range(3, 6):
        fi = f & 1
        bufs, p = sc.generate(f)
        if path == "plain":
            p.flags = N.FLAG_PLAIN
        upload_frame(s, o, bufs, fi)
        h0, a0, _ = s.tonemapping()
        assert h0.sum() == 0   # cleared by the previous exposure pass
        Denoiser(s).Denoise(fi, p)
        hd, _, _ = s.tonemapping()   # fused: this frame's histogram already accumulated
        # the oracle bins the GPU's HistogramInput from the same starting state
        o.plane("HISTOGRAM_INPUT", fi)[...] = s.download("HISTOGRAM_INPUT", fi)
        o.set_tonemapping(h0, a0)
        o.stage(N.STAGE_LUMINANCE_HISTOGRAM, 0, fi, p)
        ho = o.tonemapping()[0].copy()
        assert ho.sum() == W * H
        if path == "fused":
            assert np.array_equal(hd, ho), "fused histogram differs"
        else:
            assert hd.sum() == 0
        Tonemapping(s).CalculateExposure(fi, p)
        o.stage(N.STAGE_LUMINANCE_AVG, 0, fi, p)
        hg, ag, eg = s.tonemapping()
        hc, ao, eo = o.tonemapping()
        assert hg.sum() == 0 and hc.sum() == 0  # both cleared for the next frame
        assert np.float32(ag) == np.float32(ao)
        assert np.float32(eg) == np.float32(eo)
        if path == "plain":
            # the separate histogram kernel alone, on the same input
            s.set_tonemapping(None, ag)
            s.stage(N.STAGE_LUMINANCE_HISTOGRAM, 0, fi, p)
            assert np.array_equal(s.tonemapping()[0], ho)
            s.set_tonemapping(None, ag)
    s.close()


@pytest.mark.parametrize("mode_name,mode", MODES)
@pytest.mark.parametrize("size", [(82, 46), (250, 151)])
def test_fused_exact_equals_plain(ctx, mode_name, mode, size):
    """The default path's kernels with IEEE math reproduce the one-kernel-per-dispatch path bit
    for bit on every plane, on one tile row and on many (250x151: odd height, interior and
    edge tiles of every kernel)."""
    W, H = size
    sc = Scene(W, H, seed=13, lightFlickerFrom=3.0)
    a = Stream(ctx, W, H, mode)
    b = Stream(ctx, W, H, mode)
    for f in range(6):
        fi = f & 1
        bufs, p = sc.generate(f)
        p.atrousIterations = 5 if f % 2 else 4
        upload_frame(a, None, bufs, fi)
        upload_frame(b, None, bufs, fi)
        pa, pb = p.copy(), p.copy()
        pa.flags = N.FLAG_PLAIN
        pb.flags = N.FLAG_EXACT_MATH
        Denoiser(a).Denoise(fi, pa)
        Tonemapping(a).CalculateExposure(fi, pa)
        Denoiser(b).Denoise(fi, pb)
        Tonemapping(b).CalculateExposure(fi, pb)
        ga, gb = gpu_planes(a), gpu_planes(b)
        for key in ga:
            assert np.array_equal(ga[key][0], gb[key][0]), f"frame {f}: {key} differs"
        ta, tb = a.tonemapping(), b.tonemapping()
        assert np.array_equal(ta[0], tb[0]) and ta[1] == tb[1]
    a.close()
    b.close()


@pytest.mark.parametrize("mode_name,mode", MODES)
def test_fast_math_close_to_exact(ctx, mode_name, mode):
    """The default path (hardware exp2/log2/rcp and fused multiply-adds in continuous terms)
    stays within the parity tolerance of the exact path over a frame sequence, and is as close
    to the FP64 oracle as the exact path is."""
    W, H = 96, 54
    sc = Scene(W, H, seed=17, lightFlickerFrom=3.0)
    a = Stream(ctx, W, H, mode)
    b = Stream(ctx, W, H, mode)
    o = oracle.OracleStream(W, H, oracle.MODE_F64)
    for f in range(8):
        fi = f & 1
        bufs, p = sc.generate(f)
        upload_frame(a, o, bufs, fi)
        upload_frame(b, None, bufs, fi)
        o.denoise(fi, p)
        pa = p.copy()
        pa.flags = N.FLAG_PLAIN
        for s, q in ((a, pa), (b, p)):
            Denoiser(s).Denoise(fi, q)
            Tonemapping(s).CalculateExposure(fi, q)
    img = a.image("PRE_FINAL", fi)
    ga = F.decode(a.download("PRE_FINAL", fi), img.format)
    gb = F.decode(b.download("PRE_FINAL", fi), img.format)
    err = F.texel_rel_err(gb, ga, atol=1e-4 * float(np.percentile(ga, 99)))
    ref = F.decode(o.plane("PRE_FINAL", fi), o.fmt("PRE_FINAL"))[..., :3]
    psnr_exact, psnr_fast = F.psnr(ga[..., :3], ref), F.psnr(gb[..., :3], ref)
    stats = (f"p99 {np.percentile(err, 99):.3e} p99.9 {np.percentile(err, 99.9):.3e} max {err.max():.3e}; "
             f"PSNR vs FP64: exact {psnr_exact:.2f} dB, default {psnr_fast:.2f} dB")
    if mode == N.STORAGE_FP32:
        assert err.max() <= 1e-3, stats
    elif mode == N.STORAGE_REF:
        # The reference formats quantise coarsely: E5B9G9R9 history (9-bit mantissas), unorm8
        # gradients and a B10G11R11 PreFinal (2^-6 for R and G, 2^-5 for B). An ulp-level
        # difference can move a stored code, and where it moves the unorm8 indirect gradient
        # (RtGradients.rgen weighs it by the indirect history's brightness) the indirect
        # history length of that pixel changes, a local difference of several quanta. So
        # almost every texel stays within one PreFinal quantum, and the default path is as
        # accurate against FP64 as the exact path.
        assert np.mean(err <= 2.0 ** -5) >= 0.99, stats
        assert psnr_fast >= psnr_exact - 1.5, stats
    else:
        assert np.mean(err <= 1e-2) >= 0.99, stats
        assert np.percentile(err, 99.9) <= 4e-2, stats
        assert psnr_fast >= psnr_exact - 0.5, stats
    a.close()
    b.close()


@pytest.mark.parametrize("mode_name,mode", MODES)
def test_fast_math_keeps_history_length(ctx, mode_name, mode):
    """The default path approximates only continuous weights: the diffuse history length (the
    variance pass switches on it, and the temporal pass derives it from the reprojection tests,
    the gradients and the decay table) is bit-identical to the one-kernel-per-dispatch path's
    over a sequence with disocclusions and gradient resets."""
    W, H = 96, 54
    sc = Scene(W, H, seed=23, lightFlickerFrom=2.0)
    a = Stream(ctx, W, H, mode)
    b = Stream(ctx, W, H, mode)
    for f in range(8):
        fi = f & 1
        bufs, p = sc.generate(f)
        upload_frame(a, None, bufs, fi)
        upload_frame(b, None, bufs, fi)
        pa = p.copy()
        pa.flags = N.FLAG_PLAIN
        for s, q in ((a, pa), (b, p)):
            Denoiser(s).Denoise(fi, q)
        ha = a.download("ACCUM_HISTORY_LENGTH", fi)[..., 0]
        hb = b.download("ACCUM_HISTORY_LENGTH", fi)[..., 0]
        assert np.array_equal(ha, hb), f"frame {f}: {int(np.sum(ha != hb))} history lengths differ"
    a.close()
    b.close()


@pytest.mark.parametrize("mode_name,mode", MODES)
def test_tma_staging_equals_default(ctx, mode_name, mode):
    """The TMA-staged a-trous computes the default kernels' arithmetic: identical planes."""
    W, H = 96, 54   # width divisible by 4: every iteration takes the TMA path
    sc = Scene(W, H, seed=19, lightFlickerFrom=2.0)
    a = Stream(ctx, W, H, mode)
    b = Stream(ctx, W, H, mode)
    for f in range(5):
        fi = f & 1
        bufs, p = sc.generate(f)
        p.atrousIterations = 5 if f % 2 else 4
        upload_frame(a, None, bufs, fi)
        upload_frame(b, None, bufs, fi)
        pb = p.copy()
        pb.flags = N.FLAG_TMA_STAGING
        for s, q in ((a, p), (b, pb)):
            Denoiser(s).Denoise(fi, q)
            Tonemapping(s).CalculateExposure(fi, q)
        ga, gb = gpu_planes(a), gpu_planes(b)
        for key in ga:
            assert np.array_equal(ga[key][0], gb[key][0]), f"frame {f}: {key} differs"
        assert np.array_equal(a.tonemapping()[0], b.tonemapping()[0])
    a.close()
    b.close()


@pytest.mark.parametrize("mode_name,mode", MODES)
@pytest.mark.parametrize("size", [(96, 54), (250, 151), (330, 97)])
def test_atrous_pair_equals_single(ctx, mode_name, mode, size):
    """A-trous iterations 0 and 1 in one launch (fusion depth 2: iteration 0 over the tile widened
    by 2 in shared memory, its results quantised as stored) give the single-iteration kernels'
    planes bit for bit, with partial tiles on the right and bottom edges and 4, 5 and 6
    iterations."""
    W, H = size
    sc = Scene(W, H, seed=29, lightFlickerFrom=2.0)
    a = Stream(ctx, W, H, mode)
    b = Stream(ctx, W, H, mode)
    for f in range(5):
        fi = f & 1
        bufs, p = sc.generate(f)
        p.atrousIterations = (4, 5, 6)[f % 3]
        upload_frame(a, None, bufs, fi)
        upload_frame(b, None, bufs, fi)
        pa = p.copy()
        pa.flags = N.FLAG_ATROUS_PAIR   # iterations 0 and 1 in one launch
        for s, q in ((a, pa), (b, p)):
            Denoiser(s).Denoise(fi, q)
            Tonemapping(s).CalculateExposure(fi, q)
        ga, gb = gpu_planes(a), gpu_planes(b)
        for key in ga:
            assert np.array_equal(ga[key][0], gb[key][0]), f"frame {f}: {key} differs"
        ta, tb = a.tonemapping(), b.tonemapping()
        assert np.array_equal(ta[0], tb[0]) and ta[1] == tb[1]
    a.close()
    b.close()


@pytest.mark.parametrize("mode_name,mode", MODES)
@pytest.mark.parametrize("size", [(64, 36), (50, 23), (98, 65)])
def test_af_variance_fused_equals_separate(ctx, mode_name, mode, size):
    """Anti-firefly and variance in one launch (RGDN_FLAG_AF_VARIANCE_FUSED: the tile's clamped
    diffuse colours and their one-pixel ring kept in shared memory for the variance's 3x3) give
    the two kernels' planes bit for bit: partial tiles on the right and bottom edges, tiles whose
    ring crosses the image edge, anti-firefly off on one frame, default and IEEE math."""
    W, H = size
    sc = Scene(W, H, seed=31, lightFlickerFrom=2.0)
    a = Stream(ctx, W, H, mode)
    b = Stream(ctx, W, H, mode)
    for f in range(6):
        fi = f & 1
        bufs, p = sc.generate(f)
        if f == 3:
            p.antiFireflyEnabled = 0
        if f >= 4:
            p.flags |= N.FLAG_EXACT_MATH
        upload_frame(a, None, bufs, fi)
        upload_frame(b, None, bufs, fi)
        pa = p.copy()
        pa.flags |= N.FLAG_AF_VARIANCE_FUSED
        for s, q in ((a, pa), (b, p)):
            Denoiser(s).Denoise(fi, q)
            Tonemapping(s).CalculateExposure(fi, q)
        ga, gb = gpu_planes(a), gpu_planes(b)
        for key in ga:
            assert np.array_equal(ga[key][0], gb[key][0]), f"frame {f}: {key} differs"
        ta, tb = a.tonemapping(), b.tonemapping()
        assert np.array_equal(ta[0], tb[0]) and ta[1] == tb[1]
    a.close()
    b.close()


def test_inputs_written_by_a_kernel_just_before_denoise(ctx):
    """The frame's G-buffer written by a kernel enqueued on the same CUDA stream right before
    rgdn_denoise (a renderer's last pass) is what the frame reads: the temporal pass reads its
    inputs before it waits for the gradient chain, which is safe only because the chain's first
    kernel releases its dependents after every earlier kernel has completed. At 1920x1080 the
    copy of the 164 MB G-buffer takes long enough that an early read would see stale planes; the
    planes must equal a stream whose inputs were copied and synchronised before each frame."""
    torch = pytest.importorskip("torch")
    W, H = 1920, 1080
    sc = Scene(W, H, seed=37, lightFlickerFrom=2.0)
    a = Stream(ctx, W, H, N.STORAGE_FP16)
    b = Stream(ctx, W, H, N.STORAGE_FP16)
    cs = torch.cuda.Stream()
    frames = []
    for f in range(4):
        bufs, p = sc.generate(f)
        frames.append(({k: torch.from_numpy(np.ascontiguousarray(v).view(np.uint8).reshape(-1)).cuda() for k, v in bufs.items()}, p))
    # each stream reads two device G-buffer sets, bound for the frame's slot before each frame (a
    # plane without a previous-frame slot has one binding, so it follows the current set): a's set
    # refilled on cs right before its frame, b's refilled and synchronised
    sets = {s: [{k: torch.zeros_like(t) for k, t in frames[0][0].items()} for _ in range(2)] for s in ("a", "b")}
    zero = torch.zeros(1, dtype=torch.uint8, device="cuda:0")
    torch.cuda.synchronize()
    for f, (bufs, p) in enumerate(frames):
        fi = f & 1
        for name, st in (("a", a), ("b", b)):
            for k, t in sets[name][fi].items():
                st.bind(k, fi, t.data_ptr())
        with torch.cuda.stream(cs):
            for k, t in bufs.items():
                # the producer's pass: a kernel (not a copy-engine copy), not synchronised
                torch.bitwise_or(t, zero, out=sets["a"][fi][k])
        Denoiser(a).Denoise(fi, p, cs)
        Tonemapping(a).CalculateExposure(fi, p, cs)
        for k, t in bufs.items():
            sets["b"][fi][k].copy_(t)
        torch.cuda.synchronize()
        Denoiser(b).Denoise(fi, p)
        Tonemapping(b).CalculateExposure(fi, p)
        torch.cuda.synchronize()
        for name in ("PRE_FINAL", "DIFF_TEMPORARY", "ACCUM_HISTORY_LENGTH", "DIFF_COLOR_HISTORY", "SPEC_ACCUM_COLOR"):
            assert np.array_equal(a.download(name, fi), b.download(name, fi)), f"frame {f}: {name} differs"
        ta, tb = a.tonemapping(), b.tonemapping()
        assert np.array_equal(ta[0], tb[0]) and ta[1] == tb[1]
    a.close()
    b.close()


def reshade_bind(s, o, sc, f):
    """Frame f's re-shading scene: device copies bound to GPU stream s, host arrays to the oracle
    o (None to skip). Returns the device buffers, which must outlive the frames that use them."""
    import torch
    lt, m, occ = sc.reshade(f)
    dev = [torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8).to("cuda:0") for arr in (lt, m, occ)]
    s.set_reshade_scene(dev[0].data_ptr(), len(lt), dev[1].data_ptr(), len(m), dev[2].data_ptr(), len(occ))
    if o is not None:
        o.set_reshade_scene(lt, m, occ)
    return dev


@pytest.mark.parametrize("mode_name,mode", MODES)
@pytest.mark.parametrize("size", [(64, 36), (50, 23)])
def test_reshade_stage_parity(ctx, mode_name, mode, size):
    """Gradient samples that re-shade the previous surface on the device (RtGradients.rgen:107-136:
    the previous reservoir's light, the previous seed, the shadow ray against the scene's
    occluders) against the oracle's restatement, stage by stage, with the light's intensity
    doubling at frame 2."""
    W, H = size
    sc = Scene(W, H, seed=9, reshadeLights=1, lightFlickerFrom=2.0)
    s = Stream(ctx, W, H, mode)
    o = oracle.OracleStream(W, H, mode)
    for f in range(4):
        fi = f & 1
        bufs, p = sc.generate(f)
        keep = reshade_bind(s, o, sc, f)
        upload_frame(s, None, bufs, fi)
        for stage, it in stage_sequence(4):
            sync_to_oracle(s, o)
            s.stage(stage, it, fi, p)
            o.stage(stage, it, fi, p)
            compare_state(s, o, f"reshade {mode_name} {W}x{H} frame {f} stage {stage}.{it}")
        s.synchronize()
        del keep
    s.close()


def test_reshade_gradients_follow_the_light(ctx):
    """With the re-shading on the device, a static scene under a steady light gives (almost) no
    gradient, and doubling the light gives the antilag value the reference's formula predicts
    (|2L - L| / 2L * gradientMultDiffuse, halved by the temporal mix) over the lit surfaces; the
    batched step computes the same planes."""
    W, H = 96, 54
    sc = Scene(W, H, seed=4, reshadeLights=1, cameraPxPerFrame=0.0, spherePxPerFrame=0.0, lightFlickerFrom=3.0)
    s = Stream(ctx, W, H, N.STORAGE_FP16)
    b = Stream(ctx, W, H, N.STORAGE_FP16)
    diff = []
    for f in range(4):
        fi = f & 1
        bufs, p = sc.generate(f)
        keep = [reshade_bind(s, None, sc, f), reshade_bind(b, None, sc, f)]
        upload_frame(s, None, bufs, fi)
        upload_frame(b, None, bufs, fi)
        s.stage(N.STAGE_GRADIENT_SAMPLES, 0, fi, p)
        diff.append(F.decode(s.download("DIS_PING_GRADIENT", fi), F.F_RGBA8)[..., 0])
        for it in range(4):
            s.stage(N.STAGE_GRADIENT_ATROUS, it, fi, p)
        for st, it in [(N.STAGE_TEMPORAL_ACCUMULATION, 0), (N.STAGE_ANTI_FIREFLY, 0), (N.STAGE_VARIANCE_ESTIMATION, 0)] + \
                [(N.STAGE_ATROUS, i) for i in range(4)]:
            s.stage(st, it, fi, p)
        Tonemapping(s).CalculateExposure(fi, p)
        ctx.submit_batch([(b, fi, p)])
        s.synchronize()
        b.synchronize()
        # the diffuse channel depends on the gradient chain alone
        assert np.array_equal(s.download("DIS_GRADIENT_HISTORY", fi)[..., 0], b.download("DIS_GRADIENT_HISTORY", fi)[..., 0])
        del keep
    lit3 = diff[3] > 0.05
    assert float(np.mean(diff[2])) < 0.01, float(np.mean(diff[2]))
    assert np.mean(lit3) > 0.3, float(np.mean(lit3))
    # 0.5 (antilag of a doubling) * 0.5 (gradientMultDiffuse), mixed half and half with a history
    # of about 0: 0.125, one unorm8 step either way
    assert abs(float(np.median(diff[3][lit3])) - 0.125) <= 1.5 / 255.0, float(np.median(diff[3][lit3]))
    s.close()
    b.close()


def test_batch_equals_sequential(ctx):
    """rgdn_submit_batch over streams of different sizes == each stream alone."""
    sizes = [(64, 36), (48, 30), (96, 54)]
    scenes = [Scene(w, h, seed=20 + i) for i, (w, h) in enumerate(sizes)]
    a = [Stream(ctx, w, h, N.STORAGE_FP16) for w, h in sizes]
    b = [Stream(ctx, w, h, N.STORAGE_FP16) for w, h in sizes]
    for f in range(4):
        fi = f & 1
        jobs = []
        for i, sc in enumerate(scenes):
            bufs, p = sc.generate(f)
            upload_frame(a[i], None, bufs, fi)
            upload_frame(b[i], None, bufs, fi)
            Denoiser(a[i]).Denoise(fi, p)
            Tonemapping(a[i]).CalculateExposure(fi, p)
            jobs.append((b[i], fi, p))
        ctx.submit_batch(jobs)
    for i in range(len(sizes)):
        assert np.array_equal(a[i].download("PRE_FINAL", 1), b[i].download("PRE_FINAL", 1))
        ha, aa, _ = a[i].tonemapping()
        hb, ab, _ = b[i].tonemapping()
        assert np.array_equal(ha, hb) and aa == ab
    for x in a + b:
        x.close()


def test_error_paths(ctx):
    with pytest.raises(N.RgdnError) as e:
        Stream(ctx, 63, 36)
    assert e.value.status == N.WRONG_FUNCTION_ARGUMENT
    s = Stream(ctx, 64, 36)
    p = N.FrameParams()
    p.minLogLuminance, p.maxLogLuminance = -3.0, 7.0
    p.atrousIterations = 9
    with pytest.raises(N.RgdnError) as e:
        Denoiser(s).Denoise(0, p)
    assert e.value.status == N.WRONG_FUNCTION_ARGUMENT
    p.atrousIterations = 4
    with pytest.raises(N.RgdnError):
        Denoiser(s).Denoise(2, p)
    with pytest.raises(N.RgdnError):
        s.upload("NORMAL", 0, np.zeros(10, np.uint32))
    s.close()
    lib = N.load()
    assert lib.rgdn_denoise(None, 0, p, None) == N.WRONG_INSTANCE


def _final_inputs(W, H, mode, seed):
    """Identical PRE_FINAL, SCREEN_EMIS_RT, SCATTERING and THROUGHPUT bytes for a GPU stream and
    the oracle: HDR colours up to 40 (some above the LPM mid level, some clipped), emission,
    volumetric scattering, and about a fifth of the primary rays split."""
    rng = np.random.default_rng(seed)
    o = oracle.OracleStream(W, H, mode)
    hdr = rng.uniform(0.0, 1.0, (H, W, 3)) ** 3 * 40.0
    pre = o.plane("PRE_FINAL", 0)
    if mode == N.STORAGE_REF:
        pre[...] = np.array([[oracle.encode_b10g11r11(*hdr[y, x]) for x in range(W)] for y in range(H)], np.uint32)
    elif mode == N.STORAGE_FP32:
        pre[..., :3] = hdr.astype(np.float32)
    else:
        pre[..., :3] = hdr.astype(np.float16).view(np.uint16)
    em = rng.uniform(0.0, 2.0, (H, W, 3)) * (rng.uniform(size=(H, W, 1)) < 0.3)
    o.plane("SCREEN_EMIS_RT", 0)[...] = np.array([[oracle.encode_b10g11r11(*em[y, x]) for x in range(W)] for y in range(H)], np.uint32)
    sc = np.concatenate([rng.uniform(0.0, 0.3, (H, W, 3)), rng.uniform(0.5, 1.0, (H, W, 1))], axis=2)
    o.plane("SCATTERING", 0)[...] = sc.astype(np.float16).view(np.uint16)
    thr = np.zeros((H, W, 4), np.float16)
    thr[..., :3] = 1.0
    thr[..., 3] = (rng.uniform(size=(H, W)) < 0.2).astype(np.float16)
    o.plane("THROUGHPUT", 0)[...] = thr.view(np.uint16)
    return o


@pytest.mark.parametrize("exact", [False, True])
@pytest.mark.parametrize("mode_name,mode", MODES)
@pytest.mark.parametrize("size", [(64, 36), (50, 23)])
def test_prepare_final_parity(ctx, mode_name, mode, size, exact):
    """rgdn_prepare_final (CmCheckerboard + CmPrepareFinal: split-pixel resolve, scattering,
    uncharted2 / exposure + emission through LPM, bloom input) against the oracle on the same
    inputs: classic shading on the left 30 %, non-default LPM saturation and crosstalk, with
    and without scattering; in the default hardware pow / reciprocal form and in the IEEE form
    (RGDN_FINAL_EXACT_MATH), both to the same bounds."""
    W, H = size
    o = _final_inputs(W, H, mode, seed=W + H)
    s = Stream(ctx, W, H, mode)
    for name in ("PRE_FINAL", "SCREEN_EMIS_RT", "SCATTERING", "THROUGHPUT"):
        s.upload(name, 0, o.plane(name, 0))
    for avg in (0.35, 2.5):
        s.set_tonemapping(None, avg)
        o.set_tonemapping(None, avg)
        for flags in (0, N.FINAL_APPLY_SCATTERING):
            p = N.FinalParams.defaults()
            p.lightmapScreenCoverage = 0.3
            p.saturation[:] = (-0.1, 0.0, 0.15)
            p.crosstalk[:] = (1.0, 0.5, 0.25)
            p.flags = flags | (N.FINAL_EXACT_MATH if exact else 0)
            ImageComposition(s).Finalize(0, p)
            o.prepare_final(0, p)
            for name in ("FINAL", "BLOOM_INPUT"):
                img = s.image(name, 0)
                g = F.decode(s.download(name, 0), img.format)
                c = F.decode(o.plane(name, 0), img.format)
                err = F.texel_rel_err(g, c, atol=1e-6)
                assert err.max() <= TOL[img.format], f"{name} avg {avg} flags {flags}: max rel err {err.max():.3e}"
                if img.format != F.F_RGBA32F:
                    # quantised outputs: ulp-level differences of pow / exp2 move a code rarely
                    assert np.mean(err > 0) <= 0.02, f"{name}: {np.mean(err > 0):.2%} of texels differ"
    s.close()


@pytest.mark.parametrize("mode_name,mode", MODES)
def test_prepare_final_classic_exact_is_bit_exact(ctx, mode_name, mode):
    """With classic shading over the whole width and RGDN_FINAL_EXACT_MATH, FINAL is uncharted2
    of the (resolved) HDR colour in IEEE arithmetic on both sides, so it must equal the oracle's
    bit for bit, split pixels included: the resolved colour passes through FINAL's format between
    CmCheckerboard and CmPrepareFinal on both."""
    W, H = 50, 23
    o = _final_inputs(W, H, mode, seed=7)
    split = o.plane("THROUGHPUT", 0)[..., 3].view(np.float16) > 0.5
    assert split.sum() > 100
    s = Stream(ctx, W, H, mode)
    for name in ("PRE_FINAL", "SCREEN_EMIS_RT", "SCATTERING", "THROUGHPUT"):
        s.upload(name, 0, o.plane(name, 0))
    s.set_tonemapping(None, 0.35)
    o.set_tonemapping(None, 0.35)
    p = N.FinalParams.defaults()
    p.lightmapScreenCoverage = 1.0
    p.flags = N.FINAL_EXACT_MATH
    ImageComposition(s).Finalize(0, p)
    o.prepare_final(0, p)
    assert np.array_equal(s.download("FINAL", 0), o.plane("FINAL", 0))
    s.close()


def _encode_pre(rgb: np.ndarray, fmt: int) -> np.ndarray:
    """HDR colours as the bytes of a pre-tonemapping plane of the given storage format."""
    H, W, _ = rgb.shape
    if fmt == F.F_B10G11R11:
        return np.array([[oracle.encode_b10g11r11(*rgb[y, x]) for x in range(W)] for y in range(H)], np.uint32)
    rgba = np.concatenate([rgb, np.zeros((H, W, 1))], axis=2)
    if fmt == F.F_RGBA32F:
        return rgba.astype(np.float32)
    if fmt == F.F_RGBA16F:
        return rgba.astype(np.float16).view(np.uint16)
    assert fmt == F.F_RGBA16BF
    b = rgba.astype(np.float32).view(np.uint32).astype(np.uint64)
    return ((b + 0x7FFF + ((b >> 16) & 1)) >> 16).astype(np.uint16)


BLOOM_PLANES = ["BLOOM_INPUT"] + [f"BLOOM_MIP{k}" for k in range(1, 9)] + ["BLOOM_RESULT", "FINAL"]


@pytest.mark.parametrize("mode_name,mode", MODES)
@pytest.mark.parametrize("size", [(320, 180), (302, 163)])
def test_bloom_parity(ctx, mode_name, mode, size):
    """rgdn_bloom (8 downsample steps with the Karis-weighted first one, 8 tent upsample steps,
    the apply onto FINAL) against the oracle. Every bloom plane starts from the same random
    bytes on both sides, so the texels the uv > 1 guards skip must keep them; an odd height
    gives mips whose sizes do not halve evenly."""
    W, H = size
    rng = np.random.default_rng(W * 7 + H)
    o = oracle.OracleStream(W, H, mode)
    s = Stream(ctx, W, H, mode)
    for name in BLOOM_PLANES:
        img = s.image(name, 0)
        rgb = rng.uniform(0.0, 1.0, (img.height, img.width, 3)) ** 4 * (24.0 if name == "BLOOM_INPUT" else 2.0)
        data = _encode_pre(rgb, img.format)
        o.plane(name, 0)[...] = data
        s.upload(name, 0, data)
    Bloom(s).Apply(0, 0.7)
    o.bloom(0, 0.7)
    for name in BLOOM_PLANES[1:]:
        img = s.image(name, 0)
        g = F.decode(s.download(name, 0), img.format)
        c = F.decode(o.plane(name, 0), img.format)
        err = F.texel_rel_err(g, c, atol=1e-6)
        assert err.max() <= TOL[img.format], f"{name}: max rel err {err.max():.3e}"
        if img.format == F.F_RGBA32F:
            assert err.max() <= 1e-5, f"{name}: max rel err {err.max():.3e}"
    s.close()


def _volumetric_params(mode, frame_id):
    """Matrices that place every pixel's world position inside the froxel volume: world =
    NDC through a slightly skewed inverse view-projection, a volume projection with a small
    perspective term, the camera behind the screen."""
    p = N.VolumetricParams()
    iv = np.eye(4, dtype=np.float32)
    iv[3, 0] = 0.05                      # column 3 (translation) x
    ip = np.eye(4, dtype=np.float32)
    ip[1, 0] = 0.02                      # column 1, row 0: skew
    vp = np.eye(4, dtype=np.float32)
    vp[2, 3] = 0.1                       # column 2, row 3: w = 1 + 0.1 z
    p.invView[:] = iv.reshape(-1)        # rows of this array are GLSL columns
    p.invProjection[:] = ip.reshape(-1)
    p.volumeViewProj[:] = vp.reshape(-1)
    p.cameraPosition[:] = (0.0, 0.0, -1.0, 0.0)
    p.volumeCameraNear, p.volumeCameraFar = 0.5, 3.0
    p.volumeAmbient[:] = (0.2, 0.4, 0.8)
    p.volumeScattering = 300.0
    p.maxHistoryLength = 6.0
    p.volumeEnableType = mode
    p.frameId = frame_id
    return p


@pytest.mark.parametrize("exact", [False, True])
@pytest.mark.parametrize("vmode", [N.VOLUME_ENABLE_NONE, N.VOLUME_ENABLE_SIMPLE, N.VOLUME_ENABLE_VOLUMETRIC])
@pytest.mark.parametrize("size", [(64, 36), (50, 23)])
def test_process_scattering_parity(ctx, vmode, size, exact):
    """rgdn_process_scattering (CmVolumetricProcess + CmScatterAccum) against the oracle over
    two frames of the synthetic scene: the volume integrated in place, then SCATTERING and
    SCATTERING_HISTORY reprojected from the previous frame (random history on the first, the
    first frame's output on the second) and mixed with this frame's fog or volume sample; in the
    default hardware-math form and the IEEE form (RGDN_VOLUME_EXACT_MATH), both to the same
    bounds."""
    W, H = size
    rng = np.random.default_rng(W * 31 + H + vmode)
    sc = Scene(W, H, seed=W + vmode)
    s = Stream(ctx, W, H, N.STORAGE_FP16)
    o = oracle.OracleStream(W, H, oracle.MODE_F32)
    nz, ny, nx = N.VOLUME_SIZE[2], N.VOLUME_SIZE[1], N.VOLUME_SIZE[0]
    for fi in (0, 1):
        vol = np.concatenate([rng.uniform(0, 0.5, (ny * nz, nx, 3)), rng.uniform(0, 0.1, (ny * nz, nx, 1))], axis=2)
        upload_frame(s, o, {"SCATTER_VOLUME": vol.astype(np.float16).view(np.uint16)}, fi)
    prev = np.concatenate([rng.uniform(0, 1, (H, W, 3)), rng.uniform(0.2, 1, (H, W, 1))], axis=2)
    upload_frame(s, o, {"SCATTERING": prev.astype(np.float16).view(np.uint16),
                        "SCATTERING_HISTORY": rng.uniform(1, 5, (H, W)).astype(np.float16).view(np.uint16)}, 1)
    for f in range(2):
        fi = f & 1
        bufs, _ = sc.generate(f)
        upload_frame(s, o, {k: bufs[k] for k in ("NORMAL", "DEPTH_WORLD", "MOTION")}, fi)
        upload_frame(s, o, {"DEPTH_NDC": rng.uniform(0.1, 0.9, (H, W)).astype(np.float32)}, fi)
        p = _volumetric_params(vmode, 100 + f)
        p.flags = N.VOLUME_EXACT_MATH if exact else 0
        Volumetric(s).ProcessScattering(fi, p)
        o.process_scattering(fi, p)
        for name in ("SCATTER_VOLUME", "SCATTERING", "SCATTERING_HISTORY"):
            img = s.image(name, fi)
            g = F.decode(s.download(name, fi), img.format)
            c = F.decode(o.plane(name, fi), img.format)
            err = F.texel_rel_err(g, c, atol=1e-6)
            assert err.max() <= TOL[img.format], f"frame {f} {name}: max rel err {err.max():.3e}"
            assert np.mean(err > 0) <= 0.02, f"frame {f} {name}: {np.mean(err > 0):.2%} of texels differ"
    s.close()


def test_bloom_parity_1080p(ctx):
    """The bloom pyramid at the headline size (1920x1080, fp16 storage): every level of 64K
    texels or more takes the wide builds (2x2-quad upsample, 4 blocks per SM), the coarse levels
    the per-texel kernels; all mips, BLOOM_RESULT and FINAL against the oracle."""
    W, H = 1920, 1080
    rng = np.random.default_rng(11)
    o = oracle.OracleStream(W, H, N.STORAGE_FP16)
    s = Stream(ctx, W, H, N.STORAGE_FP16)
    for name in BLOOM_PLANES:
        img = s.image(name, 0)
        rgb = rng.uniform(0.0, 1.0, (img.height, img.width, 3)) ** 4 * (24.0 if name == "BLOOM_INPUT" else 2.0)
        data = _encode_pre(rgb, img.format)
        o.plane(name, 0)[...] = data
        s.upload(name, 0, data)
    Bloom(s).Apply(0, 0.8)
    o.bloom(0, 0.8)
    for name in BLOOM_PLANES[1:]:
        img = s.image(name, 0)
        err = F.texel_rel_err(F.decode(s.download(name, 0), img.format), F.decode(o.plane(name, 0), img.format), atol=1e-6)
        assert err.max() <= TOL[img.format], f"{name}: max rel err {err.max():.3e}"
        assert np.mean(err > 0) <= 0.02, f"{name}: {np.mean(err > 0):.2%} of texels differ"
    s.close()


def test_process_scattering_parity_1080p(ctx):
    """Volumetric scattering (VOLUMETRIC mode) at 1920x1080 on one frame of the synthetic scene
    with a random froxel volume and history: the integrated volume, SCATTERING and
    SCATTERING_HISTORY against the oracle."""
    W, H = 1920, 1080
    rng = np.random.default_rng(5)
    sc = Scene(W, H, seed=5)
    s = Stream(ctx, W, H, N.STORAGE_FP16)
    o = oracle.OracleStream(W, H, oracle.MODE_F32)
    nz, ny, nx = N.VOLUME_SIZE[2], N.VOLUME_SIZE[1], N.VOLUME_SIZE[0]
    vol = np.concatenate([rng.uniform(0, 0.5, (ny * nz, nx, 3)), rng.uniform(0, 0.1, (ny * nz, nx, 1))], axis=2)
    upload_frame(s, o, {"SCATTER_VOLUME": vol.astype(np.float16).view(np.uint16)}, 0)
    prev = np.concatenate([rng.uniform(0, 1, (H, W, 3)), rng.uniform(0.2, 1, (H, W, 1))], axis=2)
    upload_frame(s, o, {"SCATTERING": prev.astype(np.float16).view(np.uint16),
                        "SCATTERING_HISTORY": rng.uniform(1, 5, (H, W)).astype(np.float16).view(np.uint16)}, 1)
    for f in range(2):
        bufs, _ = sc.generate(f)
        upload_frame(s, o, {k: bufs[k] for k in ("NORMAL", "DEPTH_WORLD", "MOTION")}, f & 1)
    upload_frame(s, o, {"DEPTH_NDC": rng.uniform(0.1, 0.9, (H, W)).astype(np.float32)}, 0)
    p = _volumetric_params(N.VOLUME_ENABLE_VOLUMETRIC, 7)
    Volumetric(s).ProcessScattering(0, p)
    o.process_scattering(0, p)
    for name in ("SCATTER_VOLUME", "SCATTERING", "SCATTERING_HISTORY"):
        img = s.image(name, 0)
        err = F.texel_rel_err(F.decode(s.download(name, 0), img.format), F.decode(o.plane(name, 0), img.format), atol=1e-6)
        assert err.max() <= TOL[img.format], f"{name}: max rel err {err.max():.3e}"
        assert np.mean(err > 0) <= 0.02, f"{name}: {np.mean(err > 0):.2%} of texels differ"
    s.close()


def test_process_scattering_bound_inputs(ctx):
    """A producer that owns its images binds them (rgdn_stream_bind_framebuffer) instead of
    uploading: the froxel volume (processed in place in the caller's memory), the NDC depth and
    the G-buffer planes the accumulation reads give SCATTERING bits equal to the uploaded
    stream's. Output-only images cannot be bound."""
    torch = pytest.importorskip("torch")
    W, H = 64, 36
    rng = np.random.default_rng(21)
    sc = Scene(W, H, seed=21)
    up = Stream(ctx, W, H, N.STORAGE_FP16)
    bd = Stream(ctx, W, H, N.STORAGE_FP16)
    nz, ny, nx = N.VOLUME_SIZE[2], N.VOLUME_SIZE[1], N.VOLUME_SIZE[0]
    vol = np.concatenate([rng.uniform(0, 0.5, (ny * nz, nx, 3)), rng.uniform(0, 0.1, (ny * nz, nx, 1))], axis=2)
    inputs = {"SCATTER_VOLUME": vol.astype(np.float16).view(np.uint16),
              "DEPTH_NDC": rng.uniform(0.1, 0.9, (H, W)).astype(np.float32)}
    bufs, _ = sc.generate(0)
    inputs.update({k: bufs[k] for k in ("NORMAL", "DEPTH_WORLD", "MOTION")})
    keep = []
    for name, arr in inputs.items():
        up.upload(name, 0, arr)
        t = torch.from_numpy(np.ascontiguousarray(arr).view(np.uint8).reshape(-1).copy()).cuda()
        keep.append(t)
        bd.bind(name, 0, t.data_ptr())
    torch.cuda.synchronize()
    p = _volumetric_params(N.VOLUME_ENABLE_VOLUMETRIC, 3)
    Volumetric(up).ProcessScattering(0, p)
    Volumetric(bd).ProcessScattering(0, p)
    for name in ("SCATTERING", "SCATTERING_HISTORY"):
        assert np.array_equal(up.download(name, 0), bd.download(name, 0)), name
    processed = keep[0].cpu().numpy().view(np.uint16).reshape(up.download("SCATTER_VOLUME", 0).shape)
    assert np.array_equal(processed, up.download("SCATTER_VOLUME", 0))
    with pytest.raises(N.RgdnError):
        bd.bind("SCATTERING_HISTORY", 0, keep[1].data_ptr())
    for name in inputs:
        bd.bind(name, 0, None)
    up.close()
    bd.close()


def test_process_scattering_rejects_bad_params(ctx):
    s = Stream(ctx, 64, 36)
    p = _volumetric_params(N.VOLUME_ENABLE_VOLUMETRIC, 0)
    p.volumeCameraFar = p.volumeCameraNear
    with pytest.raises(N.RgdnError) as e:
        Volumetric(s).ProcessScattering(0, p)
    assert e.value.status == N.WRONG_FUNCTION_ARGUMENT
    p = _volumetric_params(3, 0)
    with pytest.raises(N.RgdnError):
        Volumetric(s).ProcessScattering(0, p)
    s.close()


def test_prepare_final_rejects_bad_params(ctx):
    s = Stream(ctx, 64, 36)
    p = N.FinalParams.defaults()
    p.crosstalk[1] = 0.0
    with pytest.raises(N.RgdnError) as e:
        ImageComposition(s).Finalize(0, p)
    assert e.value.status == N.WRONG_FUNCTION_ARGUMENT
    p = N.FinalParams.defaults()
    with pytest.raises(N.RgdnError):
        ImageComposition(s).Finalize(2, p)
    s.close()


def test_device_errors_clear_on_a_clean_run(ctx):
    """Every bounded wait inside a kernel that runs out leaves a flag for
    rgdn_stream_take_device_errors; frames on the default and the TMA-staged paths leave none."""
    W, H = 96, 54
    sc = Scene(W, H, seed=29)
    s = Stream(ctx, W, H, N.STORAGE_FP16)
    for f in range(4):
        bufs, p = sc.generate(f)
        if f >= 2:
            p.flags |= N.FLAG_TMA_STAGING
        upload_frame(s, None, bufs, f & 1)
        Denoiser(s).Denoise(f & 1, p)
        Tonemapping(s).CalculateExposure(f & 1, p)
        assert s.take_device_errors() == 0
    s.close()


def test_tma_wait_runs_out_and_reports(ctx):
    """A TMA-staged a-trous pass whose barriers cannot complete gives up after its bounded wait,
    sets RGDN_DEVICE_ERROR_TMA_WAIT and returns, and the stream stays usable. The failure is made
    on purpose without any copy left in flight: under RGDN_FLAG_TEST_TMA_TIMEOUT every stage
    expects 16 bytes more than its copies deliver, so every copy lands while the barrier phase
    never completes."""
    W, H = 96, 54   # width divisible by 4: every iteration takes the TMA path
    sc = Scene(W, H, seed=31)
    s = Stream(ctx, W, H, N.STORAGE_FP16)
    bufs, p = sc.generate(0)
    upload_frame(s, None, bufs, 0)
    p.flags |= N.FLAG_TMA_STAGING | N.FLAG_TEST_TMA_TIMEOUT
    Denoiser(s).Denoise(0, p)
    s.synchronize()
    assert s.take_device_errors() & N.DEVICE_ERROR_TMA_WAIT
    assert s.take_device_errors() == 0   # taken and cleared
    # the context and the stream still work: a normal frame reports nothing
    for f in (1, 2):
        bufs, p = sc.generate(f)
        upload_frame(s, None, bufs, f & 1)
        p.flags |= N.FLAG_TMA_STAGING
        Denoiser(s).Denoise(f & 1, p)
        Tonemapping(s).CalculateExposure(f & 1, p)
        assert s.take_device_errors() == 0
    img = s.image("PRE_FINAL", 0)
    assert np.isfinite(F.decode(s.download("PRE_FINAL", 0), img.format)).all()
    s.close()


def test_budget_admission(cuda_ok):
    from raytracedgl1_gb300.denoiser import Context, required_bytes
    need = required_bytes(64, 36, N.STORAGE_REF)
    c = Context(0, memory_budget_bytes=need * 2 + 10)
    s1 = Stream(c, 64, 36)
    s2 = Stream(c, 64, 36)
    with pytest.raises(N.RgdnError) as e:
        Stream(c, 64, 36)
    assert e.value.status == N.OUT_OF_BUDGET
    s1.close()
    s3 = Stream(c, 64, 36)
    assert c.memory_used() == 2 * need
    s2.close(); s3.close()
    c.close()
