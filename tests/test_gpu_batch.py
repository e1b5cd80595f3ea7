"""Batched steps (rgdn_submit_batch): one persistent launch per stage covers the frames of many
streams of uneven size. Every result must equal the single-stream calls (rgdn_denoise +
rgdn_calculate_exposure) bit for bit: through the autotuner's candidate steps (each launch
kind cycles through every tile shape and register budget), then through graph replay.
"""
import numpy as np
import pytest

from raytracedgl1_gb300 import _native as N
from raytracedgl1_gb300.denoiser import Context, Denoiser, Stream, Tonemapping
from raytracedgl1_gb300.scene import Scene

pytestmark = pytest.mark.gpu

MODES = [("ref", N.STORAGE_REF), ("fp32", N.STORAGE_FP32), ("fp16", N.STORAGE_FP16), ("bf16", N.STORAGE_BF16)]
# uneven sizes: W % 3 in {0, 1, 2}, odd heights, a width whose half is odd, one wide tile row
SIZES = [(64, 36), (50, 23), (34, 17), (96, 54), (130, 9)]


def planes(s: Stream):
    out = {}
    for name in N.FB_NAMES:
        img = s.image(name, 0)
        if not img.data:
            continue
        for slot in ((0, 1) if img.has_prev else (0,)):
            out[(name, slot)] = s.download(name, slot)
    return out


def assert_same(a: Stream, b: Stream, what: str, full: bool):
    if full:
        pa, pb = planes(a), planes(b)
        for key in pa:
            assert np.array_equal(pa[key], pb[key]), f"{what}: {key} differs"
    else:
        for slot in (0, 1):
            assert np.array_equal(a.download("PRE_FINAL", slot), b.download("PRE_FINAL", slot)), f"{what}: PRE_FINAL"
    ha, la, _ = a.tonemapping()
    hb, lb, _ = b.tonemapping()
    assert np.array_equal(ha, hb), f"{what}: histogram differs"
    assert la == lb, f"{what}: avgLuminance {la} != {lb}"


def frame_params(sc, f, i):
    bufs, p = sc.generate(f)
    # mixed iteration counts: an a-trous launch where some frames end and others go on
    p.atrousIterations = (4, 5, 4, 3, 5)[i % 5]
    if i == 2:
        p.flags |= N.FLAG_SKIP_GRADIENTS
    return bufs, p


@pytest.mark.parametrize("mode_name,mode", MODES)
def test_batch_equals_sequential_through_tuning_and_graphs(mode_name, mode):
    ctx = Context(0)
    scenes = [Scene(w, h, seed=40 + i, lightFlickerFrom=3.0) for i, (w, h) in enumerate(SIZES)]
    seq = [Stream(ctx, w, h, mode) for w, h in SIZES]
    bat = [Stream(ctx, w, h, mode) for w, h in SIZES]
    # 15 steps tuning the launches (the fused first two a-trous iterations among them), 8 tuning
    # the group size, then graph replay
    frames = 27
    for f in range(frames):
        fi = f & 1
        jobs = []
        for i, sc in enumerate(scenes):
            bufs, p = frame_params(sc, f, i)
            for s in (seq[i], bat[i]):
                for name, arr in bufs.items():
                    s.upload(name, fi, arr)
            Denoiser(seq[i]).Denoise(fi, p)
            Tonemapping(seq[i]).CalculateExposure(fi, p)
            jobs.append((bat[i], fi, p))
        ctx.submit_batch(jobs)
        for i in range(len(SIZES)):
            assert_same(seq[i], bat[i], f"{mode_name} frame {f} stream {i}", full=(f % 6 == 5 or f == frames - 1))
    cfg = ctx.batch_config(mode)
    assert cfg.tuned == 1 and cfg.useGraphs == 1
    for s in seq + bat:
        s.close()
    ctx.close()


def test_batch_splits_steps_and_falls_back():
    """Two frames of one stream in one submission, a PLAIN job between them and two storage
    modes: steps split where they must, and the order of the jobs is kept."""
    ctx = Context(0)
    W, H = 48, 30
    sa, sb = Scene(W, H, seed=60), Scene(40, 22, seed=61)
    A = [Stream(ctx, W, H, N.STORAGE_FP16) for _ in range(2)]
    B = [Stream(ctx, 40, 22, N.STORAGE_FP32) for _ in range(2)]
    for f in range(0, 8, 2):
        b0, p0 = sa.generate(f)
        b1, p1 = sa.generate(f + 1)
        c0, q0 = sb.generate(f)
        qp = q0.copy()
        qp.flags |= N.FLAG_PLAIN
        for s in A:
            for name, arr in b0.items():
                s.upload(name, 0, arr)
            for name, arr in b1.items():
                s.upload(name, 1, arr)
        for s in B:
            for name, arr in c0.items():
                s.upload(name, 0, arr)
        # sequential reference, in job order
        for s, fi, p in ((A[0], 0, p0), (B[0], 0, qp), (A[0], 1, p1)):
            Denoiser(s).Denoise(fi, p)
            Tonemapping(s).CalculateExposure(fi, p)
        ctx.submit_batch([(A[1], 0, p0), (B[1], 0, qp), (A[1], 1, p1)])
        assert_same(A[0], A[1], f"A frame {f}", full=True)
        assert_same(B[0], B[1], f"B frame {f}", full=True)
    for s in A + B:
        s.close()
    ctx.close()


@pytest.mark.parametrize("shape,occ,depth,group,single", [(0, 3, 1, 0, 0), (1, 4, 1, 0, 0), (2, 4, 1, 1, 0), (2, 3, 1, 0, 0),
                                                          (0, 4, 1, 2000, 0), (3, 7, 1, 2000, 2000), (0, 3, 2, 1, 1),
                                                          (3, 7, 2, 0, 0), (3, 7, 2, 2000, 0), (0, 3, 2, 0, 2000)])
def test_batch_fixed_configs(shape, occ, depth, group, single):
    """A configuration set through rgdn_batch_set_config (no tuning) gives the same results.
    Shape 3 is the 128-thread 32x4 tile (temporal and a-trous; variance then runs one 32x8 tile
    per block). Fusion depth 2 runs a-trous iterations 0 and 1 in one launch; the last frame has
    a stream running only two iterations, where the step falls back to one launch per iteration.
    Group size 0 runs the three frames as one group, 2000 pixels as two (64x36, then 50x23 with
    34x17), 1 pixel as three; a single-frame size of 2000 pixels runs 64x36 alone on the
    single-frame kernels, 1 pixel every frame."""
    ctx = Context(0)
    cfg = N.BatchConfig()
    cfg.temporalTile = shape
    cfg.antiFireflyTile = 0
    # the 128-thread configurations take the variance's one-tile-per-block form
    cfg.varianceTile = shape if shape != N.TILE_32X4 else N.TILE_32X8_PER_BLOCK
    for i in range(6):
        cfg.atrousTile[i] = (shape + i) % 3 if shape != N.TILE_32X4 else N.TILE_32X4
        cfg.atrousBlocksPerSM[i] = occ
    cfg.useGraphs = 1
    cfg.atrousFusionDepth = depth
    cfg.groupPixels = group
    cfg.singleFramePixels = single
    ctx.set_batch_config(N.STORAGE_BF16, cfg)
    got = ctx.batch_config(N.STORAGE_BF16)
    assert got.tuned == 1 and got.temporalTile == shape and got.atrousFusionDepth == depth
    assert got.groupPixels == group and got.singleFramePixels == single
    assert list(got.atrousBlocksPerSM)[1:] == [occ] * 5
    sizes = SIZES[:3]
    scenes = [Scene(w, h, seed=70 + i) for i, (w, h) in enumerate(sizes)]
    seq = [Stream(ctx, w, h, N.STORAGE_BF16) for w, h in sizes]
    bat = [Stream(ctx, w, h, N.STORAGE_BF16) for w, h in sizes]
    for f in range(5):
        fi = f & 1
        jobs = []
        for i, sc in enumerate(scenes):
            bufs, p = sc.generate(f)
            p.atrousIterations = 2 if (f == 4 and i == 1) else 5
            for s in (seq[i], bat[i]):
                for name, arr in bufs.items():
                    s.upload(name, fi, arr)
            Denoiser(seq[i]).Denoise(fi, p)
            Tonemapping(seq[i]).CalculateExposure(fi, p)
            jobs.append((bat[i], fi, p))
        ctx.submit_batch(jobs)
    for i in range(len(sizes)):
        assert_same(seq[i], bat[i], f"stream {i}", full=True)
    for s in seq + bat:
        s.close()
    ctx.close()


def test_batch_timing_and_launch_count():
    ctx = Context(0)
    sizes = SIZES[:2]
    scenes = [Scene(w, h, seed=80 + i) for i, (w, h) in enumerate(sizes)]
    streams = [Stream(ctx, w, h, N.STORAGE_FP16) for w, h in sizes]
    ctx.set_batch_timing(True)
    before = ctx.launch_count()
    jobs = []
    for i, sc in enumerate(scenes):
        bufs, p = sc.generate(0)
        p.atrousIterations = 5
        for name, arr in bufs.items():
            streams[i].upload(name, 0, arr)
        jobs.append((streams[i], 0, p))
    ctx.submit_batch(jobs)
    t = ctx.read_batch_timing()
    # one launch per stage for both frames: 5 gradient, 3, 5 a-trous, 1 luminance average
    assert ctx.launch_count() - before == 14
    assert t[("temporal_accumulation", 0)][0] == 1
    assert [t[("atrous", i)][0] for i in range(5)] == [1] * 5
    assert t[("gradient_atrous", 3)][0] == 1 and t[("luminance_avg", 0)][0] == 1
    assert all(ms > 0 for _, ms in t.values())
    ctx.set_batch_timing(False)
    for s in streams:
        s.close()
    ctx.close()


def test_batch_groups_launch_per_group():
    """Groups of frames: with a group size and a single-frame size of 2000 pixels the frames
    64x36, 50x23 and 34x17 form the groups {64x36} and {50x23, 34x17}. The first runs on the
    single-frame kernels, the other on the batched kernels over jobs 1..2 of the step's table;
    each launches the whole stage sequence, in order, with the same results as one stream per
    call."""
    ctx = Context(0)
    cfg = ctx.batch_config(N.STORAGE_FP16)
    cfg.groupPixels = 2000
    cfg.singleFramePixels = 2000
    cfg.useGraphs = 1
    ctx.set_batch_config(N.STORAGE_FP16, cfg)
    sizes = SIZES[:1] + SIZES[1:3]
    scenes = [Scene(w, h, seed=90 + i) for i, (w, h) in enumerate(sizes)]
    seq = [Stream(ctx, w, h, N.STORAGE_FP16) for w, h in sizes]
    bat = [Stream(ctx, w, h, N.STORAGE_FP16) for w, h in sizes]
    for f in range(4):
        timed = f == 3
        ctx.set_batch_timing(timed)
        jobs = []
        for i, sc in enumerate(scenes):
            bufs, p = sc.generate(f)
            p.atrousIterations = 5
            for s in (seq[i], bat[i]):
                for name, arr in bufs.items():
                    s.upload(name, f & 1, arr)
            Denoiser(seq[i]).Denoise(f & 1, p)
            Tonemapping(seq[i]).CalculateExposure(f & 1, p)
            jobs.append((bat[i], f & 1, p))
        before = ctx.launch_count()
        ctx.submit_batch(jobs)
        # 14 launches per group (5 gradient, 3, 5 a-trous, 1 luminance average), two groups
        assert ctx.launch_count() - before == 28
        if timed:
            t = ctx.read_batch_timing()
            assert t[("single_frame_group", 0)][0] == 1 and t[("temporal_accumulation", 0)][0] == 1
            assert t[("luminance_avg", 0)][0] == 1
        for i in range(len(sizes)):
            assert_same(seq[i], bat[i], f"frame {f} stream {i}", full=True)
    ctx.set_batch_timing(False)
    for s in seq + bat:
        s.close()
    ctx.close()
