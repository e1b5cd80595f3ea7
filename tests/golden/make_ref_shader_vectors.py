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
steps), and FINAL after Bloom::Apply over a second bloom_input() as the source image; and tests/golden/ref_final_<W>x<H>.npz: two final_case() states (the inputs FINAL_INPUTS,
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


BLOOM_INTENSITY = 0.7


def run_reference_bloom(W, H, inp: np.ndarray, final: np.ndarray) -> dict:
    """The reference's bloom over `inp`: the pyramid (Bloom::Prepare), then Bloom::Apply
    (Source/Bloom.cpp:194-240, CmBloomApply with the effect source UpscaledPing = `final` and the
    target UpscaledPong, intensity BLOOM_INTENSITY, no lens dirt). Returns {(fb, slot): plane} of
    every bloom image and ("FINAL", 0), the applied target."""
    o = oracle.OracleStream(W, H, oracle.MODE_REF)
    o.load("BLOOM_INPUT", 0, inp)
    ref = runner.RefRun(W, H)
    ref.bind_from(runner.oracle_planes(o, 0), 0)
    p = N.FrameParams()
    for tag, groups in bloom_plan(W, H):
        ref.run(tag, groups, p)
    out = {k: a for k, a in ref.arrays.items() if k[0].startswith("BLOOM")}
    lib = ref.lib
    src = np.ascontiguousarray(final, dtype=np.uint32).copy()
    dst = np.zeros((H, W), dtype=np.uint32)
    lib.ref_bind(b"framebufUpscaledPing", src.ctypes.data, W, H)
    lib.ref_bind(b"framebufUpscaledPong", dst.ctypes.data, W, H)
    bp = N.BloomParams()
    bp.bloomIntensity = BLOOM_INTENSITY
    lib.ref_CmBloomApply_1_set_uniform(C.byref(p), C.c_float(W), C.c_float(H))
    lib.ref_CmBloomApply_1_set_bloom(C.byref(bp))
    local = (C.c_uint * 3)()
    lib.ref_CmBloomApply_1_local(local)
    lib.ref_CmBloomApply_1_dispatch(-(-W // local[0]), -(-H // local[1]))
    out[("FINAL", 0)] = dst
    return out


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


def volume_input(seed: int) -> np.ndarray:
    """A SCATTER_VOLUME plane ((Y Z) x X texels of RGBA16F) from an integer hash of the texel
    index (the same bits on every machine): rgb in [0, 0.5), a in [0, 0.1)."""
    X, Y, Z = N.VOLUME_SIZE
    i = np.arange(Y * Z * X * 4, dtype=np.uint32) + np.uint32(seed * 0x9E3779B9 & 0xFFFFFFFF)
    h = i
    h = h ^ (h >> np.uint32(16)); h = h * np.uint32(0x7feb352d)
    h = h ^ (h >> np.uint32(15)); h = h * np.uint32(0x846ca68b)
    h = h ^ (h >> np.uint32(16))
    u = (h >> np.uint32(8)).astype(np.float32) * np.float32(1.0 / 16777216.0)
    u = u.reshape(Y * Z, X, 4)
    u[..., :3] *= np.float32(0.5)
    u[..., 3] *= np.float32(0.1)
    return u.astype(np.float16).view(np.uint16)


SCATTER_INPUTS = (("NORMAL", 0), ("NORMAL", 1), ("DEPTH_WORLD", 0), ("DEPTH_WORLD", 1), ("MOTION", 1),
                  ("DEPTH_NDC", 1), ("SCATTERING", 0), ("SCATTERING_HISTORY", 0))


def volumetric_params(mode: int, frame_id: int):
    """Matrices that place every pixel's world position inside the froxel volume: world = NDC
    through a slightly skewed inverse view-projection, a volume projection with a small
    perspective term, the camera behind the screen."""
    p = N.VolumetricParams()
    iv = np.eye(4, dtype=np.float32)
    iv[3, 0] = 0.05
    ip = np.eye(4, dtype=np.float32)
    ip[1, 0] = 0.02
    vp = np.eye(4, dtype=np.float32)
    vp[2, 3] = 0.1
    p.invView[:] = iv.reshape(-1)          # rows of these arrays are GLSL columns
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


def scattering_case(W, H, mode, seed=SEED):
    """The oracle ready for the second frame's Volumetric::ProcessScattering: frame 0's scattering
    processed over a random history, frame 1's G-buffer and NDC depth loaded, both volumes from
    volume_input(). Returns (stream, frame params, volumetric params, fi = 1)."""
    rng = np.random.default_rng(seed + 31 * mode)
    sc = Scene(W, H, seed=seed + mode)
    o = oracle.OracleStream(W, H, oracle.MODE_REF)
    for fi in (0, 1):
        o.load("SCATTER_VOLUME", fi, volume_input(seed * 2 + fi))
    prev = np.concatenate([rng.uniform(0, 1, (H, W, 3)), rng.uniform(0.2, 1, (H, W, 1))], axis=2)
    o.load("SCATTERING", 1, prev.astype(np.float16).view(np.uint16))
    o.load("SCATTERING_HISTORY", 1, rng.uniform(1, 5, (H, W)).astype(np.float16).view(np.uint16))
    for f in range(2):
        fi = f & 1
        bufs, p = sc.generate(f)
        for k in ("NORMAL", "DEPTH_WORLD", "MOTION"):
            o.load(k, fi, np.ascontiguousarray(bufs[k]))
        o.load("DEPTH_NDC", fi, rng.uniform(0.1, 0.9, (H, W)).astype(np.float32))
        vp = volumetric_params(mode, 100 + f)
        if f == 0:
            o.process_scattering(fi, vp)
    return o, p, vp, 1


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
    for (fb, slot), a in run_reference_bloom(W, H, bloom_input(W, H), bloom_input(W, H, seed=SEED + 1)).items():
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
    # Volumetric::ProcessScattering in each volume mode at the first size: the 2-D inputs and
    # outputs, this frame's volume by its volume_input() seed (the previous frame's is not read:
    # CmVolumetricProcess's temporal weight is 0) and the processed volume by its SHA-256
    import hashlib
    out = {"meta": np.array([W, H], dtype=np.int64)}
    for mode in (N.VOLUME_ENABLE_NONE, N.VOLUME_ENABLE_SIMPLE, N.VOLUME_ENABLE_VOLUMETRIC):
        o, p, vp, fi = scattering_case(W, H, mode)
        out[f"m{mode}/params"] = np.frombuffer(bytes(p), dtype=np.uint8)
        out[f"m{mode}/vparams"] = np.frombuffer(bytes(vp), dtype=np.uint8)
        for fb, slot in SCATTER_INPUTS:
            out[f"m{mode}/in/{fb}/{slot}"] = o.plane(fb, slot).copy()
        ref = runner.run_reference_scattering(W, H, runner.oracle_planes(o, fi), fi, p, vp)
        for fb in ("SCATTERING", "SCATTERING_HISTORY"):
            out[f"m{mode}/out/{fb}"] = ref[(fb, fi)]
        out[f"m{mode}/out/SCATTER_VOLUME_sha256"] = np.frombuffer(
            hashlib.sha256(ref[("SCATTER_VOLUME", fi)].tobytes()).digest(), dtype=np.uint8)
    path = os.path.join(here, f"ref_scattering_{W}x{H}.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path))


if __name__ == "__main__":
    main(sys.argv[1:])
