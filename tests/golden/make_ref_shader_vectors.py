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

It also writes tests/golden/ref_bloom_<W>x<H>.npz at the first size: bloom_input() and every bloom
image after the reference's pyramid (Bloom::Prepare's eight downsampling and eight upsampling
steps).
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


if __name__ == "__main__":
    main(sys.argv[1:])
