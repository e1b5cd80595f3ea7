"""Writes tests/golden/ref_shaders_<W>x<H>.npz: the reference's own shaders (oracle/glsl_ref,
built from the reference's GLSL sources) run over one frame of the seeded scene, stage by stage,
from a starting state, so that the oracle can be checked against the reference where the
reference checkout is absent (tests/test_ref_shaders.py).

The starting state is the oracle's, in the reference framebuffer formats, after three frames of
the scene, with the fourth frame's G-buffer loaded. Each stage's planes are the reference
shaders' own, carried from stage to stage, from the fourth frame's gradient samples on:
  s0/<fb>/<slot>        every plane of both frame slots before the gradient samples
  k<n>/<fb>/<slot>      the planes that stage n of stage_plan() changed, after it
  k<n>/hist, k<n>/avg   the tonemapping buffer after stage n (histogram, average luminance)
  tm0/hist, tm0/avg     the tonemapping buffer before the first stage
  params                the frame's rgdn_frame_params bytes; meta: W, H, fi, seed

Usage (where the reference checkout and a C++ compiler are present):
  python oracle/glsl_ref/build.py && python tests/golden/make_ref_shader_vectors.py 64 36 34 17

It also writes, at the first size, tests/golden/ref_bloom_<W>x<H>.npz: bloom_input() and every
bloom image after the reference's pyramid (Bloom::Prepare's eight downsampling and eight upsampling
steps); and tests/golden/ref_final_<W>x<H>.npz: two final_case() states (the inputs FINAL_INPUTS,
the frame and final parameters, the adapted average luminance) and FINAL and BLOOM_INPUT after the
reference's CmCheckerboard + CmPrepareFinal.
"""
import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle.glsl_ref import runner  # noqa: E402
from raytracedgl1_gb300 import _native as N  # noqa: E402
from raytracedgl1_gb300.scene import Scene  # noqa: E402

SEED = 5
WARM = 3


def start_state(W, H, seed=SEED):
    """The oracle after WARM frames, with the next frame's G-buffer loaded: (stream, params, fi)."""
    sc = Scene(W, H, seed=seed, lightFlickerFrom=1.0)
    o = oracle.OracleStream(W, H, oracle.MODE_REF)
    for f in range(WARM + 1):
        fi = f & 1
        bufs, p = sc.generate(f)
        p.atrousIterations = 4
        for n, a in bufs.items():
            o.load(n, fi, np.ascontiguousarray(a))
        if f < WARM:
            o.denoise(fi, p)
            o.calculate_exposure(fi, p)
    return o, p, fi


def generate(W, H, seed=SEED) -> dict:
    o, p, fi = start_state(W, H, seed)
    planes = runner.oracle_planes(o, fi)
    hist, avg, _ = o.tonemapping()
    out = {"params": np.frombuffer(bytes(p), dtype=np.uint8), "meta": np.array([W, H, fi, seed], dtype=np.int64),
           "tm0/hist": hist.astype(np.uint32), "tm0/avg": np.float32(avg)}
    for (fb, slot), a in planes.items():
        out[f"s0/{fb}/{slot}"] = a
    ref = runner.RefRun(W, H)
    tm = (hist, avg)
    for k, (stage, it, tag, groups) in enumerate(runner.stage_plan(W, H)):
        ref.bind_from(planes, fi, tag)
        r = ref.run(tag, groups, p, tm)
        for key, a in ref.arrays.items():
            if not np.array_equal(a.view(np.uint8), planes[key].view(np.uint8)):
                out[f"k{k}/{key[0]}/{key[1]}"] = a.copy()
        planes.update({key: a.copy() for key, a in ref.arrays.items()})
        if r is not None:
            tm = r
        out[f"k{k}/hist"] = np.asarray(tm[0], dtype=np.uint32)
        out[f"k{k}/avg"] = np.float32(tm[1])
    return out


def bloom_input(W, H, seed=SEED) -> np.ndarray:
    """Random B10G11R11 texels (each channel's exponent 0..29, so finite) for BLOOM_INPUT."""
    rng = np.random.default_rng(seed)
    r = (rng.integers(0, 30, (H, W)) << 6) | rng.integers(0, 64, (H, W))
    g = (rng.integers(0, 30, (H, W)) << 6) | rng.integers(0, 64, (H, W))
    b = (rng.integers(0, 30, (H, W)) << 5) | rng.integers(0, 32, (H, W))
    return (r | (g << 11) | (b << 22)).astype(np.uint32)


def bloom_plan(W, H):
    """(reference entry point, groups) of Bloom::Prepare (Source/Bloom.cpp:129-187)."""
    plan = []
    for i in range(8):
        w, h = -(-W // (1 << (i + 1))), -(-H // (1 << (i + 1)))
        plan.append((f"CmBloomDownsample_{i}", ((w + 15) // 16, (h + 15) // 16)))
    for i in range(7, -1, -1):
        w, h = -(-W // (1 << i)), -(-H // (1 << i))
        plan.append((f"CmBloomUpsample_{i}", ((w + 15) // 16, (h + 15) // 16)))
    return plan


def run_reference_bloom(W, H, inp: np.ndarray) -> dict:
    """The reference's bloom pyramid over `inp`: {(fb, slot): plane} of every bloom image."""
    o = oracle.OracleStream(W, H, oracle.MODE_REF)
    o.load("BLOOM_INPUT", 0, inp)
    ref = runner.RefRun(W, H)
    ref.bind_from(runner.oracle_planes(o, 0), 0)
    p = N.FrameParams()
    for tag, groups in bloom_plan(W, H):
        ref.run(tag, groups, p)
    return {k: a for k, a in ref.arrays.items() if k[0].startswith("BLOOM")}


def final_case(W, H, seed=SEED, saturation=(0.0, 0.0, 0.0), crosstalk=(1.0, 1.0, 1.0), coverage=0.25,
               scattering=True):
    """The oracle after start_state's frame is denoised and exposed, ready for the final
    composition, with inputs the scene leaves trivial made varied (seeded): 40 % of the pixels
    split by the checkerboard (THROUGHPUT.a = 1 at their checkerboard position), screen emission
    on 20 % of the pixels, a volumetric SCATTERING image (rgb in [0, 0.05), a in [0.6, 1)).
    Returns (stream, frame params, final params, fi)."""
    o, p, fi = start_state(W, H, seed)
    o.denoise(fi, p)
    o.calculate_exposure(fi, p)
    rng = np.random.default_rng(seed + 17)
    thr = o.plane("THROUGHPUT", fi)
    a = thr[..., 3].view(np.float16)
    a[...] = np.where(rng.random((H, W)) < 0.4, np.float16(1.0), a)
    r = (rng.integers(0, 15, (H, W)) << 6) | rng.integers(0, 64, (H, W))
    g = (rng.integers(0, 15, (H, W)) << 6) | rng.integers(0, 64, (H, W))
    b = (rng.integers(0, 15, (H, W)) << 5) | rng.integers(0, 32, (H, W))
    o.plane("SCREEN_EMIS_RT", fi)[...] = (r | (g << 11) | (b << 22)).astype(np.uint32) * (rng.random((H, W)) < 0.2)
    v = np.empty((H, W, 4), np.float32)
    v[..., :3] = rng.uniform(0.0, 0.05, (H, W, 3))
    v[..., 3] = rng.uniform(0.6, 1.0, (H, W))
    if not scattering:
        v[...] = (0.0, 0.0, 0.0, 1.0)
    o.plane("SCATTERING", fi)[...] = v.astype(np.float16).view(np.uint16)
    f = N.FinalParams.defaults()
    f.saturation[:] = saturation
    f.crosstalk[:] = crosstalk
    f.lightmapScreenCoverage = coverage
    # the reference always applies the scattering image; without the flag it holds (0, 0, 0, 1)
    f.flags = N.FINAL_APPLY_SCATTERING if scattering else 0
    return o, p, f, fi


FINAL_INPUTS = ("PRE_FINAL", "SCREEN_EMIS_RT", "THROUGHPUT", "SCATTERING")
FINAL_OUTPUTS = ("FINAL", "BLOOM_INPUT")


def run_reference_final_case(o, p, f, fi) -> dict:
    """The reference's CmCheckerboard + CmPrepareFinal over the oracle's state: {fb: plane} of
    FINAL and BLOOM_INPUT."""
    _, avg, _ = o.tonemapping()
    ref = runner.run_reference_final(o.width, o.height, runner.oracle_planes(o, fi), fi, p, f, avg)
    return {fb: ref[(fb, fi)] for fb in FINAL_OUTPUTS}


def main(argv):
    sizes = [(int(argv[i]), int(argv[i + 1])) for i in range(0, len(argv), 2)] or [(64, 36)]
    here = os.path.dirname(os.path.abspath(__file__))
    for W, H in sizes:
        path = os.path.join(here, f"ref_shaders_{W}x{H}.npz")
        np.savez_compressed(path, **generate(W, H))
        print(path, os.path.getsize(path))
    # the bloom pyramid (CmBloomDownsample / CmBloomUpsample) at the first size
    W, H = sizes[0]
    out = {"meta": np.array([W, H], dtype=np.int64)}
    for (fb, slot), a in run_reference_bloom(W, H, bloom_input(W, H)).items():
        out[f"{fb}/{slot}"] = a
    path = os.path.join(here, f"ref_bloom_{W}x{H}.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path))
    # the final composition (CmCheckerboard + CmPrepareFinal) at the first size, default and
    # non-default LPM saturation / crosstalk
    out = {"meta": np.array([W, H], dtype=np.int64)}
    for c, (sat, ct) in enumerate([((0.0, 0.0, 0.0), (1.0, 1.0, 1.0)), ((0.3, -0.2, 0.1), (1.0, 0.5, 0.25))]):
        o, p, f, fi = final_case(W, H, saturation=sat, crosstalk=ct)
        _, avg, _ = o.tonemapping()
        out[f"c{c}/params"] = np.frombuffer(bytes(p), dtype=np.uint8)
        out[f"c{c}/final"] = np.frombuffer(bytes(f), dtype=np.uint8)
        out[f"c{c}/avg"] = np.float32(avg)
        out[f"c{c}/fi"] = np.int64(fi)
        for fb in FINAL_INPUTS:
            out[f"c{c}/in/{fb}"] = o.plane(fb, fi).copy()
        for fb, a in run_reference_final_case(o, p, f, fi).items():
            out[f"c{c}/out/{fb}"] = a
    path = os.path.join(here, f"ref_final_{W}x{H}.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path))


if __name__ == "__main__":
    main(sys.argv[1:])
