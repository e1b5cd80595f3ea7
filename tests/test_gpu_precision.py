"""Storage precision against the FP64 oracle: fp32 / fp16 / bf16 colour and history storage
(FP32 arithmetic, fp32 moments and variance in every mode) on the precision-sweep scene
(radiance sigma 2, 1 % fireflies x1000) at a reduced size, after a frame sequence long enough
for the history to carry the error forward.

Metrics of PRE_FINAL against the FP64 oracle (no quantisation of any buffer):
  max-rel  max over pixels of |x - ref| / max(|ref| over the pixel's channels, 1e-3 * p99(ref))
  PSNR     10 log10(max(ref)^2 / mean squared error)
"""
import numpy as np
import pytest

from raytracedgl1_gb300 import _native as N
from raytracedgl1_gb300.denoiser import Denoiser, Stream, Tonemapping
from raytracedgl1_gb300.scene import Scene

import oracle
from tests import _formats as F

pytestmark = pytest.mark.gpu

SWEEP = dict(sigma=2.0, fireflyProb=0.01, fireflyMult=1000.0)
# lower bounds (dB) of PSNR against FP64, per storage mode
PSNR_MIN = {N.STORAGE_FP32: 60.0, N.STORAGE_FP16: 40.0, N.STORAGE_BF16: 30.0}


def metrics(x: np.ndarray, ref: np.ndarray):
    x = x[..., :3].astype(np.float64)
    ref = ref[..., :3].astype(np.float64)
    atol = 1e-3 * float(np.percentile(np.abs(ref), 99))
    return float(F.texel_rel_err(x, ref, atol=atol).max()), F.psnr(x, ref)


def test_storage_precision_vs_fp64(ctx):
    W, H, frames = 192, 108, 12
    sc = Scene(W, H, seed=5, **SWEEP)
    seq = [sc.generate(f) for f in range(frames)]
    o = oracle.OracleStream(W, H, oracle.MODE_F64)
    gpu = {m: Stream(ctx, W, H, m) for m in PSNR_MIN}
    for f, (bufs, p) in enumerate(seq):
        fi = f & 1
        p.atrousIterations = 5
        for k, v in bufs.items():
            o.load(k, fi, v)
        o.denoise(fi, p, 8)
        o.calculate_exposure(fi, p, 8)
        for s in gpu.values():
            for k, v in bufs.items():
                s.upload(k, fi, v)
            Denoiser(s).Denoise(fi, p)
            Tonemapping(s).CalculateExposure(fi, p)
    fi = (frames - 1) & 1
    ref = F.decode(o.plane("PRE_FINAL", fi), o.fmt("PRE_FINAL"))
    res = {}
    for m, s in gpu.items():
        img = s.image("PRE_FINAL", fi)
        res[m] = metrics(F.decode(s.download("PRE_FINAL", fi), img.format), ref)
        s.close()
    for m, (mr, ps) in res.items():
        print(f"storage {m}: max-rel {mr:.3e}  PSNR {ps:.1f} dB")
        assert ps >= PSNR_MIN[m], f"storage {m}: PSNR {ps:.1f} dB < {PSNR_MIN[m]}"
    # more storage bits, less error
    assert res[N.STORAGE_FP32][1] > res[N.STORAGE_FP16][1] > res[N.STORAGE_BF16][1]
