"""Closed-form known-answer tests of the CPU oracle's stages (the reference ships none; these
follow from the shader math itself)."""
import math

import numpy as np
import pytest

import oracle
from raytracedgl1_gb300 import _native as N
from raytracedgl1_gb300.scene import Scene
from tests import _formats as F


def params(**kw):
    p = N.FrameParams()
    for i in range(4):
        p.view[i * 5] = p.viewPrev[i * 5] = p.projection[i * 5] = p.projectionPrev[i * 5] = 1.0
    p.timeDelta = 1.0 / 60.0
    p.minLogLuminance, p.maxLogLuminance = -3.0, 7.0
    p.gradientMultDiffuse, p.gradientMultIndirect, p.gradientMultSpecular = 0.5, 0.2, 0.5
    p.antiFireflyEnabled = 1
    p.atrousIterations = 4
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def test_first_frame_resets_history():
    """With zeroed history every reprojection test fails: weightSum = 0, so the temporal
    accumulation outputs the unfiltered signal, history length 1, moments (l, l^2)
    (CmSVGFTemporalAccumulation.comp:310-376)."""
    W, H = 32, 18
    sc = Scene(W, H, seed=2)
    bufs, p = sc.generate(0)
    o = oracle.OracleStream(W, H, oracle.MODE_F32)
    for k, v in bufs.items():
        o.load(k, 0, v)
    o.stage(N.STAGE_TEMPORAL_ACCUMULATION, 0, 0, p)
    unf = F.decode_e5(bufs["UNFILTERED_DIRECT"])
    dt = o.plane("DIFF_TEMPORARY", 0)[..., :3]
    assert np.array_equal(dt, unf)
    hl = o.plane("ACCUM_HISTORY_LENGTH", 0)
    assert np.all(hl[..., 0] == 1.0) and np.all(hl[..., 1] == 1.0) and np.all(hl[..., 2] == 1.0)
    l = (np.float32(0.2125) * unf[..., 0] + np.float32(0.7154) * unf[..., 1]) + np.float32(0.0721) * unf[..., 2]
    m = o.plane("DIFF_ACCUM_MOMENTS", 0)
    assert np.array_equal(m[..., 0], l) and np.array_equal(m[..., 1], l * l)


def _flat_state(o, W, H, color, var, depth=5.0, normal_code=None):
    """A flat, fully valid surface: one depth, one normal, one colour and variance."""
    code = normal_code if normal_code is not None else oracle.encode_normal(0.0, 1.0, 0.0)
    o.plane("DEPTH_WORLD", 0)[...] = np.float16(depth).view(np.uint16)
    o.plane("DEPTH_GRAD", 0)[...] = np.float16(0.01).view(np.uint16)
    o.plane("NORMAL", 0)[...] = code
    o.plane("METALLIC_ROUGHNESS", 0)[...] = [0, 128]
    cv = o.plane("DIFF_PING_COLOR_AND_VARIANCE", 0)
    cv[..., :3] = color
    cv[..., 3] = var
    for name in ("SPEC_PING_COLOR", "INDIR_PING"):
        o.plane(name, 0)[..., :3] = color
    hl = o.plane("ACCUM_HISTORY_LENGTH", 0)
    hl[...] = [8.0, 8.0, 8.0, 1.0]


@pytest.mark.parametrize("niter", [4, 5])
def test_atrous_constant_image_invariant(niter):
    """Normalised edge-stopping weights keep a constant image constant through every
    a-trous iteration (CmSVGFAtrous.comp:212-219)."""
    W, H = 40, 24
    o = oracle.OracleStream(W, H, oracle.MODE_F32)
    c = np.array([0.7, 0.3, 1.9], dtype=np.float32)
    _flat_state(o, W, H, c, 0.01)
    o.plane("ALBEDO", 0)[...] = oracle.encode_b10g11r11(1.0, 1.0, 1.0)
    o.plane("THROUGHPUT", 0)[...] = np.float16(1.0).view(np.uint16)
    p = params(atrousIterations=niter)
    for i in range(niter):
        o.stage(N.STAGE_ATROUS, i, 0, p)
    # metallic 0, roughness 128/255: composition = (diff + indir) * albedo + spec' * 0.04
    r = 128.0 / 255.0
    t = min(max((r - 0.5) / 0.25, 0.0), 1.0)
    spec_w = t * t * (3 - 2 * t)
    expect = (c + c) * 1.0 + (c * (1 - spec_w) + c * spec_w) * 0.04
    pre = o.plane("PRE_FINAL", 0)[..., :3]
    assert np.allclose(pre, expect, rtol=2e-6)


def test_antifirefly_clamps_isolated_spike():
    W, H = 20, 12
    o = oracle.OracleStream(W, H, oracle.MODE_F32)
    base = np.array([1.0, 2.0, 3.0], np.float32)
    for name in ("DIFF_TEMPORARY", "SPEC_ACCUM_COLOR", "INDIR_ACCUM"):
        pl = o.plane(name, 0)
        pl[..., :3] = base
        pl[6, 9, :3] = base * 1000
    o.stage(N.STAGE_ANTI_FIREFLY, 0, 0, params())
    for name in ("DIFF_ACCUM_COLOR", "SPEC_PING_COLOR", "INDIR_PING"):
        assert np.allclose(o.plane(name, 0)[6, 9, :3], base)
    # disabled: passthrough
    o.stage(N.STAGE_ANTI_FIREFLY, 0, 0, params(antiFireflyEnabled=0))
    assert np.allclose(o.plane("DIFF_ACCUM_COLOR", 0)[6, 9, :3], base * 1000)


def test_variance_temporal_branch():
    """History > 4: variance = max(0, E[l^2] - E[l]^2) / max(1, h - 4)
    (CmSVGFEstimateVariance.comp:153-161)."""
    W, H = 16, 8
    o = oracle.OracleStream(W, H, oracle.MODE_F32)
    o.plane("DEPTH_WORLD", 0)[...] = np.float16(3.0).view(np.uint16)
    o.plane("DIFF_ACCUM_COLOR", 0)[..., :3] = 0.5
    o.plane("ACCUM_HISTORY_LENGTH", 0)[..., 0] = 10.0
    m = o.plane("DIFF_ACCUM_MOMENTS", 0)
    m[..., 0] = 0.5
    m[..., 1] = 0.5
    o.stage(N.STAGE_VARIANCE_ESTIMATION, 0, 0, params())
    v = o.plane("DIFF_PING_COLOR_AND_VARIANCE", 0)[..., 3]
    assert np.allclose(v, (np.float32(0.5) - np.float32(0.25)) / np.float32(6.0))
    # sky / invalid depth: variance 0, colour passes through
    o.plane("DEPTH_WORLD", 0)[...] = np.float16(20000.0).view(np.uint16)
    o.stage(N.STAGE_VARIANCE_ESTIMATION, 0, 0, params())
    assert np.all(o.plane("DIFF_PING_COLOR_AND_VARIANCE", 0)[..., 3] == 0)


def test_luminance_avg_closed_form():
    """All pixels in bin b: average = exp2((b-1)/254 * range + minLog); one adaptation step
    t = 1 - exp(-dt * 1.1) from the previous value (CmLuminanceAvg.comp:70-88)."""
    W, H = 32, 16
    o = oracle.OracleStream(W, H, oracle.MODE_F32)
    b = 128
    hist = np.zeros(256, np.uint32)
    hist[b] = W * H
    o.set_tonemapping(hist, 0.5)
    p = params()
    o.stage(N.STAGE_LUMINANCE_AVG, 0, 0, p)
    h, avg, exposure = o.tonemapping()
    target = 2.0 ** ((b - 1) / 254.0 * 10.0 - 3.0)
    t = 1.0 - math.exp(-p.timeDelta * 1.1)
    assert h.sum() == 0
    assert avg == pytest.approx(0.5 + (target - 0.5) * t, rel=1e-6)
    # Exposure.h: EV100 = log2(L*100/12.5); exposure = 1 / (1.2 * 2^EV100) = 12.5 / (120 L)
    assert exposure == pytest.approx(12.5 / (120.0 * avg), rel=1e-5)
    # stopEyeAdaptation: histogram still cleared, luminance kept
    o.set_tonemapping(hist, 0.25)
    o.stage(N.STAGE_LUMINANCE_AVG, 0, 0, params(stopEyeAdaptation=1))
    h, avg, _ = o.tonemapping()
    assert h.sum() == 0 and avg == 0.25


def test_histogram_counts_every_pixel():
    W, H = 30, 10
    o = oracle.OracleStream(W, H, oracle.MODE_REF)
    rng = np.random.default_rng(4)
    lum = np.exp(rng.normal(0, 3, (H, W))).astype(np.float16)
    o.plane("HISTOGRAM_INPUT", 0)[...] = lum.view(np.uint16)
    o.stage(N.STAGE_LUMINANCE_HISTOGRAM, 0, 0, params())
    h, _, _ = o.tonemapping()
    ref = np.bincount([oracle.color_bin(float(v), -3.0, 7.0) for v in lum.astype(np.float32).ravel()],
                      minlength=256)
    assert np.array_equal(h, ref) and h.sum() == W * H


def test_gradient_atrous_constant():
    W, H = 36, 18
    o = oracle.OracleStream(W, H, oracle.MODE_REF)
    o.plane("DIS_PING_GRADIENT", 0)[...] = [100, 50, 200, 0]
    for i in range(4):
        o.stage(N.STAGE_GRADIENT_ATROUS, i, 0, params())
    g = o.plane("DIS_PING_GRADIENT", 0)
    gw = (W + 1) // 3  # strata inside the render area keep the constant
    assert np.all(g[:, :gw, :3] == [100, 50, 200])
    assert np.all(o.plane("DIS_GRADIENT_HISTORY", 0)[..., :3] == [100, 50, 200])


def test_composition_writes_every_regular_pixel_once():
    """getRegularPixFromCheckerboardPix is a bijection: the last a-trous iteration writes every
    regular pixel of HistogramInput / PreFinal (ShaderCommonGLSLFunc.h:331-342)."""
    W, H = 24, 7
    o = oracle.OracleStream(W, H, oracle.MODE_F32)
    _flat_state(o, W, H, np.array([1.0, 1.0, 1.0], np.float32), 0.0)
    alb = o.plane("ALBEDO", 0)
    codes = np.arange(W * H, dtype=np.float32).reshape(H, W) + 1.0
    for y in range(H):
        for x in range(W):
            alb[y, x] = oracle.encode_b10g11r11(float(codes[y, x]), 0.0, 0.0)
    o.plane("IS_SKY", 0)[...] = 1  # sky: illuminated = albedo * throughput
    o.plane("THROUGHPUT", 0)[...] = np.float16(1.0).view(np.uint16)
    o.stage(N.STAGE_ATROUS, 3, 0, params())
    pre = o.plane("PRE_FINAL", 0)[..., 0]
    expect = F.decode_b10g11r11(alb)[..., 0]
    assert np.array_equal(pre, expect)


def test_fp64_and_fp32_oracles_agree():
    W, H = 48, 27
    sc = Scene(W, H, seed=9)
    o32 = oracle.OracleStream(W, H, oracle.MODE_F32)
    o64 = oracle.OracleStream(W, H, oracle.MODE_F64)
    for f in range(5):
        fi = f & 1
        bufs, p = sc.generate(f)
        for k, v in bufs.items():
            o32.load(k, fi, v)
            o64.load(k, fi, v)
        for o in (o32, o64):
            o.denoise(fi, p)
            o.calculate_exposure(fi, p)
    a = o32.plane("PRE_FINAL", fi)[..., :3].astype(np.float64)
    b = o64.plane("PRE_FINAL", fi)[..., :3]
    assert F.psnr(a, b) > 70.0


# --- exposure application and tonemapping (CmCheckerboard + CmPrepareFinal) ----------------
def test_lpm_setup_709():
    """LpmSetup for ImageComposition's arguments: luma weights are the Rec.709 Y row (D65),
    contrast 1 + 0.1, and the luma curve l^c / (l^c s + b) maps the mid level 0.18 to 0.18
    and hdrMax 256 to 1 (the two conditions its scale and bias are solved from)."""
    k = oracle.lpm_setup()
    assert k["luma"] == pytest.approx([0.2126390, 0.7151687, 0.0721923], abs=2e-6)
    assert sum(k["luma"]) == pytest.approx(1.0, abs=1e-6)
    assert k["contrast"] == pytest.approx(1.1) and k["saturation"] == pytest.approx([1.1] * 3)
    s, b = k["tone_scale_bias"]
    tone = lambda l: l ** 1.1 / (l ** 1.1 * s + b)
    assert tone(0.18) == pytest.approx(0.18, rel=1e-5)
    assert tone(256.0) == pytest.approx(1.0, rel=1e-5)
    assert oracle.lpm_setup(saturation=(-0.1, 0.0, 0.2))["saturation"] == pytest.approx([1.0, 1.1, 1.3])


def test_lpm_filter_grey_and_luma():
    """A grey stays grey on the luma curve; an in-gamut colour keeps its luma on the curve
    (the filter is luma-preserving); every output lies in [0, 1]."""
    k = oracle.lpm_setup()
    s, b = k["tone_scale_bias"]
    tone = lambda l: l ** 1.1 / (l ** 1.1 * s + b)
    for v in (0.003, 0.05, 0.18, 1.0, 7.5, 100.0):
        out = oracle.lpm_filter((v, v, v))
        assert out == pytest.approx((tone(v),) * 3, rel=2e-5)
    rgb = (0.3, 0.2, 0.1)
    out = oracle.lpm_filter(rgb)
    luma = lambda c: sum(w * x for w, x in zip(k["luma"], c))
    assert luma(out) == pytest.approx(tone(luma(rgb)), rel=1e-4)
    for c in ((50.0, 0.1, 0.0), (0.0, 0.0, 3.0), (1e4, 1e4, 0.5)):
        out = oracle.lpm_filter(c)
        assert all(0.0 <= x <= 1.0 for x in out)


def test_prepare_final_closed_form():
    """FINAL and BLOOM_INPUT of an fp32 stream against the formulas of CmPrepareFinal:
    uncharted2 left of the classic-shading edge, LPM of the exposed colour right of it, and
    the bloom input; one pixel with a split primary ray takes the cross-resolved colour."""
    W, H = 8, 4
    o = oracle.OracleStream(W, H, oracle.MODE_F32)
    rng = np.random.default_rng(3)
    hdr = rng.uniform(0.0, 6.0, (H, W, 4)).astype(np.float32)
    hdr[..., 3] = 0
    o.load("PRE_FINAL", 0, hdr)
    emis = np.array([[oracle.encode_b10g11r11(0.25, 0.5, 0.0)] * W] * H, np.uint32)
    o.load("SCREEN_EMIS_RT", 0, emis)
    thr = np.zeros((H, W, 4), np.uint16)
    thr[2, 1, 3] = 0x3C00   # throughput.a = 1 at checkerboard pixel (1, 2): regular pixel (2, 2)
    o.load("THROUGHPUT", 0, thr)
    avg = 0.4
    o.set_tonemapping(np.zeros(256), avg)
    p = N.FinalParams.defaults()
    p.lightmapScreenCoverage = 0.25   # classic shading for x < 2
    o.prepare_final(0, p)
    fin = o.plane("FINAL", 0)[..., :3].astype(np.float64)
    bloom = o.plane("BLOOM_INPUT", 0)[..., :3].astype(np.float64)
    exposure = 1.0 / (1.2 * avg * 100.0 / 12.5)
    e = np.array(oracle.decode_b10g11r11(int(emis[0, 0])))
    op = lambda x: ((x * (0.15 * x + 0.05) + 0.004) / (x * (0.15 * x + 0.5) + 0.06)) - 0.02 / 0.3
    for y in range(H):
        for x in range(W):
            c = hdr[y, x, :3].astype(np.float64)
            if (x, y) == (2, 2):
                cross = 0.25 * (hdr[2, 1, :3] + hdr[2, 3, :3] + hdr[3, 2, :3] + hdr[1, 2, :3])
                c = 0.5 * c + 0.5 * cross
            if x < 2:
                want = op(2.0 * c) / op(10.0)
            else:
                want = np.array(oracle.lpm_filter(tuple(c * exposure + e * 1.5)))
            assert fin[y, x] == pytest.approx(want, rel=2e-5, abs=1e-6), (x, y)
            b = (c + e * 2.0 ** (math.log2(avg * 8.0) + 16.0 - 3.0)) * exposure
            l = 0.2125 * b[0] + 0.7154 * b[1] + 0.0721 * b[2]
            t = min(max(l / 4.0, 0.0), 1.0)
            assert bloom[y, x] == pytest.approx(b * t * t * (3 - 2 * t), rel=2e-5, abs=1e-6), (x, y)


def test_bloom_constant_image():
    """A constant BLOOM_INPUT c through the pyramid of a 1920x1080 frame.

    - The Karis-weighted first downsample gives c' = c / (1 + lum(c)); the later downsamples
      keep it, so mip 8 (7x4, only ever written by the downsample) is c'.
    - Each upsample adds its own level, so mip k tops out at (9 - k) c' and BLOOM_RESULT at
      8 c'. FINAL gains intensity times BLOOM_RESULT.
    - The upsample's uv > 1 guard (CmBloomUpsample.comp:88-91) leaves the last column and row
      of every upsampled level unadded. Through the coarse levels (mip 8 spans 7.5 texels of
      uv but holds 7) this lowers the right and bottom of the frame, while the upper left
      (rows < 500, columns < 1280) stays exactly 8 c'."""
    W, H = 1920, 1080
    o = oracle.OracleStream(W, H, oracle.MODE_F64)
    c = np.array([0.5, 1.0, 2.0])
    o.plane("BLOOM_INPUT", 0)[..., :3] = c
    o.plane("FINAL", 0)[..., :3] = 0.25
    o.plane("BLOOM_RESULT", 0)[...] = -1.0
    o.bloom(0, 0.5)
    lum = 0.2125 * c[0] + 0.7154 * c[1] + 0.0721 * c[2]
    cp = c / (1 + lum)
    mip8 = o.plane("BLOOM_MIP8", 0)[..., :3]
    assert mip8.shape == (4, 7, 3)
    assert mip8 == pytest.approx(np.broadcast_to(cp, mip8.shape), rel=1e-12)
    for k in range(1, 8):
        m = o.plane(f"BLOOM_MIP{k}", 0)[..., :3] / cp
        assert m.max() == pytest.approx(9 - k, rel=1e-12) and m.min() == pytest.approx(1.0, rel=1e-12), k
    res = o.plane("BLOOM_RESULT", 0)
    assert res[:500, :1280, :3] == pytest.approx(np.broadcast_to(8 * cp, (500, 1280, 3)), rel=1e-12)
    fin = o.plane("FINAL", 0)[..., :3]
    assert fin[:500, :1280] == pytest.approx(np.broadcast_to(0.25 + 4 * cp, (500, 1280, 3)), rel=1e-12)
    assert np.all(res[:, W - 1] == -1.0) and np.all(res[H - 1, :] == -1.0)
    inner = res[: H - 1, : W - 1, :3] / cp
    assert inner.min() > 1.0 and inner.max() <= 8.0 * (1 + 1e-12)


def _f16(x):
    return np.asarray(x, np.float16).view(np.uint16)


def test_volume_process_closed_form():
    """CmVolumetricProcess on a volume of constant in-scatter L and extinction d per cell:
    cell z holds L * sum_{i<=z} exp(-i d) and transmittance exp(-(z + 1) d), within one fp16
    rounding of the stored cell."""
    o = oracle.OracleStream(64, 36, oracle.MODE_F64)
    vol = o.plane("SCATTER_VOLUME", 0)
    assert vol.shape == (N.VOLUME_SIZE[1] * N.VOLUME_SIZE[2], N.VOLUME_SIZE[0], 4)
    L, d = np.array([0.5, 0.25, 0.125]), 0.05
    vol[...] = _f16(np.concatenate([L, [d]]))
    o.process_scattering(0, N.VolumetricParams())
    v = vol.view(np.float16).astype(np.float64).reshape(N.VOLUME_SIZE[2], N.VOLUME_SIZE[1], N.VOLUME_SIZE[0], 4)
    dq, Lq = float(np.float16(d)), L.astype(np.float16).astype(np.float64)
    for z in range(N.VOLUME_SIZE[2]):
        rgb = Lq * sum(math.exp(-i * dq) for i in range(z + 1))
        assert v[z, 3, 7, :3] == pytest.approx(rgb, rel=2.0 ** -10), z
        assert v[z, 80, 150, 3] == pytest.approx(math.exp(-(z + 1) * dq), rel=2.0 ** -10), z


def _scatter_stream(W, H, depth, motion_x=0.0):
    o = oracle.OracleStream(W, H, oracle.MODE_F32)
    n = oracle.encode_normal(0.0, 0.0, 1.0)
    for fi in (0, 1):
        o.plane("NORMAL", fi)[...] = n
        o.plane("DEPTH_WORLD", fi)[...] = _f16(depth)
    mo = np.zeros((H, W, 4), np.float32)
    mo[..., 0] = motion_x
    o.plane("MOTION", 0)[...] = _f16(mo)
    o.plane("MOTION", 1)[...] = _f16(mo)
    return o


def test_scatter_simple_fog_and_history():
    """CmScatterAccum in SIMPLE mode. A frame without history writes the fog
    (ambient (1 - f), f), f = exp(-depth * scattering * 0.00005), with history length 1; sky
    (ray length above MAX_RAY_LENGTH) writes (0, 0, 0, 1). A static next frame finds all four
    taps valid and mixes with weight 1/2 (history 2), capped by maxHistoryLength."""
    W, H = 16, 8
    depth = np.full((H, W), 40.0)
    depth[:, 3] = 20000.0
    o = _scatter_stream(W, H, depth, motion_x=5.0)   # reprojects outside the image: no history
    p = N.VolumetricParams()
    p.volumeEnableType = N.VOLUME_ENABLE_SIMPLE
    p.volumeScattering = 100.0
    p.volumeAmbient[:] = (0.5, 1.0, 2.0)
    p.maxHistoryLength = 1.5
    o.process_scattering(0, p)
    sc = o.plane("SCATTERING", 0).view(np.float16).astype(np.float64)
    hist = o.plane("SCATTERING_HISTORY", 0).view(np.float16).astype(np.float64)
    f = math.exp(-float(np.float16(40.0)) * float(np.float32(100.0) * np.float32(0.00005)))
    fog = np.array([0.5 * (1 - f), 1.0 * (1 - f), 2.0 * (1 - f), f])
    cb_sky = {(2 * (3 - 0) + (0 + y) % 2, y) for y in range(H)}   # regular pixels of checkerboard column 3
    for y in range(H):
        for x in range(W):
            want = np.array([0, 0, 0, 1.0]) if (x, y) in cb_sky else fog
            assert sc[y, x] == pytest.approx(want, rel=2.0 ** -10, abs=1e-6), (x, y)
            assert hist[y, x] == 1.0
    # static second frame: history of 1 everywhere, mixed with 1 / min(1 + 1, 1.5)
    o.plane("MOTION", 1)[...] = _f16(np.zeros((H, W, 4), np.float32))
    o.process_scattering(1, p)
    sc1 = o.plane("SCATTERING", 1).view(np.float16).astype(np.float64)
    h1 = o.plane("SCATTERING_HISTORY", 1).view(np.float16).astype(np.float64)
    assert np.all(h1 == 1.5)
    assert sc1[4, 8] == pytest.approx(fog, rel=2.0 ** -9)


def test_random_seed_restatement():
    """getRandomSeed / rnd8_4's hashes (Random.h:243-300) against an independent Python
    restatement of MurmurHash2's mixing and lowbias32."""
    M, U = 0x5BD1E995, 0xFFFFFFFF

    def murmur33(v):
        src = [(((c * M) & U) ^ (((c * M) & U) >> 24)) * M & U for c in v]
        h = [1190494759, 2147483647, 3559788179]
        for k in src:
            h = [((x * M) & U) ^ k for x in h]
        h = [x ^ (x >> 13) for x in h]
        h = [(x * M) & U for x in h]
        return [x ^ (x >> 15) for x in h]

    def lowbias32(x):
        x ^= x >> 16
        x = (x * 0x7FEB352D) & U
        x ^= x >> 15
        x = (x * 0x846CA68B) & U
        return x ^ (x >> 16)

    lib = oracle.load()
    for (x, y, f) in [(0, 0, 0), (1, 2, 3), (1919, 1079, 123456), (640, 17, 0xFFFFFFFF)]:
        h = murmur33([x, y, f])
        seed = ((h[2] % 128) << 14) | ((h[1] % 128) << 7) | (h[0] % 128)
        assert lib.orc_random_seed(x, y, f) == seed
        assert lib.orc_wellons_lowbias32(seed) == lowbias32(seed)
    assert lowbias32(0) == 0 and lib.orc_wellons_lowbias32(1) == lowbias32(1)


def _reshade_stream(normal=(0.0, 1.0, 0.0), roughness=1.0, metallic=0.0):
    """An oracle stream whose previous slot holds one surface point at the origin, seen from a
    camera 5 above and 5 in front, with the reservoir of light 0 (weight 1)."""
    from raytracedgl1_gb300 import _native as N
    o = oracle.OracleStream(8, 4, oracle.MODE_F32)
    prev = 0   # frame slot 1 reads slot 0 as its previous frame
    o.plane("SURFACE_POSITION", prev)[...] = 0.0
    o.plane("NORMAL", prev)[...] = oracle.encode_normal(*normal)
    mr = o.plane("METALLIC_ROUGHNESS", prev)
    mr[..., 0], mr[..., 1] = round(metallic * 255), round(roughness * 255)
    res = o.plane("RESERVOIRS", prev)
    res[..., 0], res[..., 1], res[..., 2], res[..., 3] = (1 << 16) | 0, 0x3F800000, 0x3F800000, 0
    p = N.FrameParams()
    p.minLogLuminance, p.maxLogLuminance = -3.0, 7.0
    p.cameraPositionPrev[:] = (0.0, 5.0, 5.0, 0.0)
    p.frameId = 7
    return o, p


def _light(center, radius, color):
    from raytracedgl1_gb300 import _native as N
    lt = (N.SphereLight * 1)()
    lt[0].center[:] = center
    lt[0].radius = radius
    lt[0].color[:] = (color, color, color)
    return lt


def test_reshade_closed_form_and_its_zero_cases():
    """RtGradients.rgen:107-136 re-shading (oracle restatement): a surface facing a small sphere
    light straight above it gets the Lambertian term dw * nl * color / pi with dw the light's solid
    angle and nl within the light's angular radius of 1; the sample is zero when an occluder
    blocks the shadow ray, when the reservoir's light is gone or invalid, and for a surface facing
    away."""
    import ctypes as C
    import math
    from raytracedgl1_gb300 import _native as N
    o, p = _reshade_stream()
    lt = _light((0.0, 5.0, 0.0), 0.25, 100.0)
    o.set_reshade_scene(lt, (C.c_uint32 * 1)(0), (N.Occluder * 0)())
    d, s = o.reshade(1, 3, 2, p, f64=True)
    sin_t = 0.25 / 5.0
    dw = 2.0 * math.pi * (1.0 - math.sqrt(1.0 - sin_t * sin_t))
    ref = dw * 100.0 / math.pi   # luminance of a white light: the weights sum to 1
    assert 0.995 * ref <= d <= ref * 1.0000001, (d, ref)
    assert s > 0.0
    # FP32: 1 - cos(theta) of a small light cancels (the shader's own arithmetic), about 1e-4
    d32, _ = o.reshade(1, 3, 2, p, f64=False)
    assert abs(d32 - d) <= 1e-3 * d
    # an occluding sphere half way
    occ = (N.Occluder * 1)()
    occ[0].type = N.OCCLUDER_SPHERE
    occ[0].data[:4] = (0.0, 2.5, 0.0, 0.5)
    o.set_reshade_scene(lt, (C.c_uint32 * 1)(0), occ)
    assert o.reshade(1, 3, 2, p) == (0.0, 0.0)
    # a rectangle that misses the ray (beside it) changes nothing
    occ[0].type = N.OCCLUDER_RECT
    occ[0].data[:] = (1.0, 2.5, 3.0, 4.0, -1.0, 1.0, 0.0)   # y = 2.5, x in [3, 4], z in [-1, 1]
    o.set_reshade_scene(lt, (C.c_uint32 * 1)(0), occ)
    assert o.reshade(1, 3, 2, p, f64=True)[0] == d
    occ[0].data[:] = (1.0, 2.5, -1.0, 1.0, -1.0, 1.0, 0.0)  # the same plane across the ray
    o.set_reshade_scene(lt, (C.c_uint32 * 1)(0), occ)
    assert o.reshade(1, 3, 2, p) == (0.0, 0.0)
    # the previous frame's light is gone, or the reservoir holds no light
    o.set_reshade_scene(lt, (C.c_uint32 * 1)(0xFFFFFFFF), (N.Occluder * 0)())
    assert o.reshade(1, 3, 2, p) == (0.0, 0.0)
    o.set_reshade_scene(lt, (C.c_uint32 * 1)(0), (N.Occluder * 0)())
    o.plane("RESERVOIRS", 0)[..., 0] = 32767
    assert o.reshade(1, 3, 2, p) == (0.0, 0.0)
    # facing away from the light
    o2, p2 = _reshade_stream(normal=(0.0, -1.0, 0.0))
    o2.set_reshade_scene(lt, (C.c_uint32 * 1)(0), (N.Occluder * 0)())
    assert o2.reshade(1, 3, 2, p2) == (0.0, 0.0)


def test_reshade_specular_follows_roughness():
    """The Smith-GGX term (BRDF.h:116-146): with the camera on the mirror direction of the light,
    a smooth metal's specular luminance exceeds a rough dielectric's by orders of magnitude."""
    import ctypes as C
    from raytracedgl1_gb300 import _native as N
    lt = _light((0.0, 5.0, -5.0), 0.25, 100.0)
    spec = []
    for rough, metal in ((1.0, 0.0), (0.1, 1.0)):
        o, p = _reshade_stream(roughness=rough, metallic=metal)
        o.set_reshade_scene(lt, (C.c_uint32 * 1)(0), (N.Occluder * 0)())
        spec.append(o.reshade(1, 3, 2, p, f64=True)[1])
    assert spec[1] > 100.0 * spec[0] > 0.0, spec
