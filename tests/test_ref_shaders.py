"""The oracle against the reference's own shaders.

The reference's A-SVGF and tonemapping compute shaders (Source/Shaders/CmASVGFGradientAtrous.comp,
CmSVGFTemporalAccumulation.comp, CmAntiFirefly.comp, CmSVGFEstimateVariance.comp,
CmSVGFAtrous_Iter0.comp, CmSVGFAtrous.comp, CmLuminanceHistogram.comp, CmLuminanceAvg.comp), the
main() of its gradient-sample shader (RtGradients.rgen, with the ray-traced forward projection
read from the boundary input RGDN_FB_GRADIENT_RESHADED) and its bloom pyramid
(CmBloomDownsample.comp, CmBloomUpsample.comp) run on the CPU from their GLSL sources
(oracle/glsl_ref: a mechanical rewrite to C++ over a GLSL runtime), dispatched as
PathTracer::CalculateGradientsSamples, Denoiser::Denoise, Tonemapping::CalculateExposure and
Bloom::Prepare dispatch them. Every plane of both frame slots and the tonemapping buffer must equal
the oracle's bit for bit after every stage.

- test_oracle_matches_reference_vectors: from the committed vectors (tests/golden, written by
  tests/golden/make_ref_shader_vectors.py), wherever the oracle builds.
- test_oracle_matches_reference_shaders_live: the same, live, at sizes with partial workgroups
  and odd gradient images, where the reference checkout is present (it builds oracle/_ref first).
- test_a_planted_mistake_is_caught: an input changed on the oracle's side only (a moments texel
  before the variance pass; the forward-projected luminance before the gradient samples) must
  show up as a difference at that stage.
- test_oracle_bloom_*: the bloom pyramid (every bloom image) and its application onto FINAL
  (CmBloomApply through the effect framework's UpscaledPing/UpscaledPong images), from the
  committed vectors and live.
- test_oracle_scattering_*: Volumetric::ProcessScattering (CmVolumetricProcess + CmScatterAccum)
  in the three volume modes, the froxel volume bound as a 3-D image.
- test_oracle_final_*: the final composition, CmCheckerboard + CmPrepareFinal (the LPM control
  block from the reference's own CPU-side LpmSetup), with split checkerboard pixels, classic
  shading on part of the image, screen emission, scattering, non-default saturation and
  crosstalk; from the committed vectors and live.
"""
import glob
import os

import numpy as np
import pytest

import oracle
from oracle.glsl_ref import runner
from raytracedgl1_gb300 import _native as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "ref_shaders_*.npz")))
from oracle.glsl_ref.build import REFERENCE  # noqa: E402


def load_state(o, z, fi):
    for key in z.files:
        if key.startswith("s0/"):
            _, fb, slot = key.split("/")
            o.load(fb, int(slot), z[key])


def expected_state(z, k, state):
    for key in z.files:
        if key.startswith(f"k{k}/") and key.count("/") == 2:
            _, fb, slot = key.split("/")
            state[(fb, int(slot))] = z[key]
    return state


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_oracle_matches_reference_vectors(path):
    z = np.load(path)
    W, H, fi, _ = (int(v) for v in z["meta"])
    p = N.FrameParams.from_buffer_copy(bytes(z["params"]))
    o = oracle.OracleStream(W, H, oracle.MODE_REF)
    load_state(o, z, fi)
    o.set_tonemapping(z["tm0/hist"], float(z["tm0/avg"]))
    state = runner.oracle_planes(o, fi)
    assert len(state) > 40
    bad = []
    for k, (stage, it, tag, _) in enumerate(runner.stage_plan(W, H)):
        o.stage(stage, it, fi, p)
        state = expected_state(z, k, state)
        diff = runner.differing(state, runner.oracle_planes(o, fi))
        hist, avg, _ = o.tonemapping()
        if diff:
            bad.append((tag, diff))
        if not np.array_equal(hist, z[f"k{k}/hist"]) or np.float32(avg) != z[f"k{k}/avg"]:
            bad.append((tag, "tonemapping"))
    assert not bad, bad


def _live_ready():
    if not os.path.isdir(os.path.join(REFERENCE, "Source", "Shaders")):
        return "the reference checkout is not present"
    from oracle.glsl_ref import build
    if not os.path.exists(build.LIB) or os.path.getmtime(build.LIB) < max(
            os.path.getmtime(os.path.join(build.HERE, f)) for f in ("glsl.h", "glsl_rt.cpp", "build.py")):
        try:
            build.build(REFERENCE)
        except Exception as e:   # no compiler or no cpp: nothing to compare against
            return f"the reference shaders did not build: {e}"
    return None


def run_both(W, H, plant=None):
    """The oracle and the reference shaders from the same state, stage by stage; returns the
    stages whose results differ. plant(o, fi, k): a change made on the oracle's side only."""
    from tests.golden.make_ref_shader_vectors import start_state
    o, p, fi = start_state(W, H)
    ref = runner.RefRun(W, H)
    bad = []
    for k, (stage, it, tag, groups) in enumerate(runner.stage_plan(W, H)):
        hist, avg, _ = o.tonemapping()
        ref.bind_from(runner.oracle_planes(o, fi), fi, tag)
        tm = ref.run(tag, groups, p, (hist, avg))
        if plant:
            plant(o, fi, k)
        o.stage(stage, it, fi, p)
        diff = runner.differing(ref.arrays, runner.oracle_planes(o, fi))
        if diff:
            bad.append((tag, diff))
        if tm is not None:
            h2, a2, _ = o.tonemapping()
            if not np.array_equal(tm[0], h2) or np.float32(tm[1]) != np.float32(a2):
                bad.append((tag, "tonemapping"))
    return bad


# partial workgroups and odd gradient images, and the benchmark's 640x360 and 1920x1080 frames
# (the last about a minute)
@pytest.mark.parametrize("size", [(64, 36), (98, 33), (100, 34), (130, 9), (250, 151), (16, 6), (640, 360), (1920, 1080)])
def test_oracle_matches_reference_shaders_live(size):
    why = _live_ready()
    if why:
        pytest.skip(why)
    assert run_both(*size) == []


def _plant_moments(o, fi, k):
    # before the variance stage (plan index 7), one texel of the accumulated moments changes
    if k == 7:
        m = o.plane("DIFF_ACCUM_MOMENTS", fi)
        m[5, 7] = m[5, 7] + np.array(1000, dtype=m.dtype)


def _plant_reshaded(o, fi, k):
    # before the gradient samples (plan index 0), the forward-projected luminance doubles
    if k == 0:
        r = o.plane("GRADIENT_RESHADED", fi)
        r[...] = r * np.float32(2)


@pytest.mark.parametrize("plant,first", [(_plant_moments, "CmSVGFEstimateVariance"),
                                         (_plant_reshaded, "RtGradients_main")])
def test_a_planted_mistake_is_caught(plant, first):
    """A change made on the oracle's side only shows up at the stage that reads it."""
    why = _live_ready()
    if why:
        pytest.skip(why)
    bad = run_both(64, 36, plant)
    assert bad and bad[0][0] == first, bad


GOLDEN_BLOOM = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "ref_bloom_*.npz")))


def oracle_bloom(W, H, inp, final):
    """The oracle's bloom over `inp`, applied onto `final`: {(fb, slot): plane} of every bloom
    image and FINAL."""
    from tests.golden.make_ref_shader_vectors import BLOOM_INTENSITY
    o = oracle.OracleStream(W, H, oracle.MODE_REF)
    o.load("BLOOM_INPUT", 0, inp)
    o.load("FINAL", 0, final)
    o.bloom(0, BLOOM_INTENSITY)
    return {k: a for k, a in runner.oracle_planes(o, 0).items() if k[0].startswith("BLOOM") or k[0] == "FINAL"}


@pytest.mark.parametrize("path", GOLDEN_BLOOM, ids=[os.path.basename(p) for p in GOLDEN_BLOOM])
def test_oracle_bloom_matches_reference_vectors(path):
    z = np.load(path)
    W, H = (int(v) for v in z["meta"])
    expected = {}
    for key in z.files:
        if key != "meta":
            fb, slot = key.split("/")
            expected[(fb, int(slot))] = z[key]
    assert len(expected) == 11
    from tests.golden.make_ref_shader_vectors import SEED, bloom_input
    got = oracle_bloom(W, H, expected[("BLOOM_INPUT", 0)], bloom_input(W, H, seed=SEED + 1))
    assert runner.differing(expected, got) == []


@pytest.mark.parametrize("size", [(64, 36), (250, 151), (1280, 720)])
def test_oracle_bloom_matches_reference_shaders_live(size):
    why = _live_ready()
    if why:
        pytest.skip(why)
    from tests.golden.make_ref_shader_vectors import SEED, bloom_input, run_reference_bloom
    W, H = size
    inp, fin = bloom_input(W, H), bloom_input(W, H, seed=SEED + 1)
    ref = run_reference_bloom(W, H, inp, fin)
    # the reference writes no texel of a mip whose uv passes 1 (CmBloomDownsample.comp:123), so
    # the smallest mips of a small frame stay empty; the input and the first mips are not
    assert len(ref) == 11
    assert all(np.count_nonzero(ref[(fb, 0)]) for fb in ("BLOOM_INPUT", "BLOOM_MIP1", "BLOOM_MIP2", "BLOOM_RESULT", "FINAL"))
    assert not np.array_equal(ref[("FINAL", 0)], fin)
    assert runner.differing(ref, oracle_bloom(W, H, inp, fin)) == []


GOLDEN_FINAL = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "ref_final_*.npz")))


@pytest.mark.parametrize("path", GOLDEN_FINAL, ids=[os.path.basename(p) for p in GOLDEN_FINAL])
def test_oracle_final_matches_reference_vectors(path):
    """The oracle's prepare_final (CmCheckerboard + CmPrepareFinal with the LPM filter) against the
    reference's outputs for the same inputs: FINAL and BLOOM_INPUT bit for bit."""
    z = np.load(path)
    W, H = (int(v) for v in z["meta"])
    cases = sorted({k.split("/")[0] for k in z.files if k != "meta"})
    assert len(cases) == 2
    for c in cases:
        p = N.FrameParams.from_buffer_copy(bytes(z[f"{c}/params"]))
        f = N.FinalParams.from_buffer_copy(bytes(z[f"{c}/final"]))
        fi = int(z[f"{c}/fi"])
        o = oracle.OracleStream(W, H, oracle.MODE_REF)
        for key in z.files:
            if key.startswith(f"{c}/in/"):
                o.load(key.split("/")[2], fi, z[key])
        o.set_tonemapping(np.zeros(256, dtype=np.uint32), float(z[f"{c}/avg"]))
        o.prepare_final(fi, f)
        for fb in ("FINAL", "BLOOM_INPUT"):
            exp = z[f"{c}/out/{fb}"]
            assert np.count_nonzero(exp) > exp.size // 2
            assert np.array_equal(o.plane(fb, fi), exp), (c, fb)


@pytest.mark.parametrize("size,sat,ct,scat", [
    ((64, 36), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), True),
    ((98, 33), (0.3, -0.2, 0.1), (1.0, 0.5, 0.25), True),
    ((130, 9), (-0.5, 0.0, 0.5), (0.25, 1.0, 0.5), False),
    ((250, 151), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), True),
])
def test_oracle_final_matches_reference_shaders_live(size, sat, ct, scat):
    why = _live_ready()
    if why:
        pytest.skip(why)
    from tests.golden.make_ref_shader_vectors import final_case, run_reference_final_case
    o, p, f, fi = final_case(*size, saturation=sat, crosstalk=ct, scattering=scat)
    ref = run_reference_final_case(o, p, f, fi)
    o.prepare_final(fi, f)
    got = {fb: o.plane(fb, fi) for fb in ref}
    assert runner.differing({(fb, 0): a for fb, a in ref.items()}, {(fb, 0): a for fb, a in got.items()}) == []


def test_final_planted_mistake_is_caught():
    """A PRE_FINAL texel at a split pixel's neighbour changed on the oracle's side only moves the
    resolved pixels beside it."""
    why = _live_ready()
    if why:
        pytest.skip(why)
    from tests.golden.make_ref_shader_vectors import final_case, run_reference_final_case
    o, p, f, fi = final_case(64, 36)
    ref = run_reference_final_case(o, p, f, fi)
    pre = o.plane("PRE_FINAL", fi)
    pre[10, 30] = pre[10, 30] ^ np.uint32(1 << 12)
    o.prepare_final(fi, f)
    assert not np.array_equal(o.plane("FINAL", fi), ref["FINAL"])


GOLDEN_SCATTER = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "ref_scattering_*.npz")))


@pytest.mark.parametrize("path", GOLDEN_SCATTER, ids=[os.path.basename(p) for p in GOLDEN_SCATTER])
def test_oracle_scattering_matches_reference_vectors(path):
    """The oracle's process_scattering (CmVolumetricProcess + CmScatterAccum) against the
    reference's outputs in the three volume modes: SCATTERING and SCATTERING_HISTORY bit for bit,
    the processed volume by its SHA-256."""
    import hashlib
    from tests.golden.make_ref_shader_vectors import SEED, volume_input
    z = np.load(path)
    W, H = (int(v) for v in z["meta"])
    modes = sorted({k.split("/")[0] for k in z.files if k != "meta"})
    assert len(modes) == 3
    for m in modes:
        p = N.FrameParams.from_buffer_copy(bytes(z[f"{m}/params"]))
        vp = N.VolumetricParams.from_buffer_copy(bytes(z[f"{m}/vparams"]))
        o = oracle.OracleStream(W, H, oracle.MODE_REF)
        o.load("SCATTER_VOLUME", 1, volume_input(SEED * 2 + 1))
        for key in z.files:
            if key.startswith(f"{m}/in/"):
                _, _, fb, slot = key.split("/")
                o.load(fb, int(slot), z[key])
        o.process_scattering(1, vp)
        for fb in ("SCATTERING", "SCATTERING_HISTORY"):
            assert np.array_equal(o.plane(fb, 1), z[f"{m}/out/{fb}"]), (m, fb)
        digest = hashlib.sha256(o.plane("SCATTER_VOLUME", 1).tobytes()).digest()
        assert digest == bytes(z[f"{m}/out/SCATTER_VOLUME_sha256"]), m


@pytest.mark.parametrize("size", [(64, 36), (50, 23), (250, 151)])
@pytest.mark.parametrize("mode", [N.VOLUME_ENABLE_NONE, N.VOLUME_ENABLE_SIMPLE, N.VOLUME_ENABLE_VOLUMETRIC])
def test_oracle_scattering_matches_reference_shaders_live(size, mode):
    why = _live_ready()
    if why:
        pytest.skip(why)
    from tests.golden.make_ref_shader_vectors import scattering_case
    W, H = size
    o, p, vp, fi = scattering_case(W, H, mode)
    ref = runner.run_reference_scattering(W, H, runner.oracle_planes(o, fi), fi, p, vp)
    o.process_scattering(fi, vp)
    got = runner.oracle_planes(o, fi)
    keys = [("SCATTER_VOLUME", fi), ("SCATTERING", fi), ("SCATTERING_HISTORY", fi)]
    assert runner.differing({k: ref[k] for k in keys}, got) == []

