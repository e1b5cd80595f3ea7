"""Vectorised numpy decoders of the framebuffer formats (test-side reading of planes),
and the per-texel comparison used by the parity tests."""
from __future__ import annotations

import numpy as np

F_R8U, F_RG8, F_RGBA8, F_R16F, F_RG16F, F_RGBA16F, F_RGBA16BF = 1, 2, 3, 4, 5, 6, 7
F_R32F, F_RG32F, F_RGBA32F, F_R32U, F_E5, F_B10G11R11, F_NORMAL = 8, 9, 10, 11, 12, 13, 14
F_RGBA32U = 15
F_R64F, F_RG64F, F_RGBA64F = 100, 101, 102


def decode_e5(p: np.ndarray) -> np.ndarray:
    p = p.astype(np.uint32)
    s = np.ldexp(np.float32(1.0), (p >> 27).astype(np.int32) - 24).astype(np.float32)
    r = (p & 0x1FF).astype(np.float32) * s
    g = ((p >> 9) & 0x1FF).astype(np.float32) * s
    b = ((p >> 18) & 0x1FF).astype(np.float32) * s
    return np.stack([r, g, b], axis=-1)


def _uf(v: np.ndarray, mbits: int) -> np.ndarray:
    e = (v >> mbits).astype(np.int32)
    m = (v & ((1 << mbits) - 1)).astype(np.float32)
    norm = np.ldexp((m + np.float32(1 << mbits)), e - 15 - mbits)
    den = np.ldexp(m, -14 - mbits)
    out = np.where(e == 0, den, norm).astype(np.float32)
    return np.where(e == 31, np.float32(np.inf), out)


def decode_b10g11r11(p: np.ndarray) -> np.ndarray:
    p = p.astype(np.uint32)
    return np.stack([_uf(p & 0x7FF, 6), _uf((p >> 11) & 0x7FF, 6), _uf((p >> 22) & 0x3FF, 5)], axis=-1)


def decode(arr: np.ndarray, fmt: int) -> np.ndarray:
    """Plane (as stored) -> float array (..., channels)."""
    if fmt == F_E5:
        return decode_e5(arr)
    if fmt == F_B10G11R11:
        return decode_b10g11r11(arr)
    if fmt in (F_R16F, F_RG16F, F_RGBA16F):
        return arr.view(np.float16).astype(np.float32)
    if fmt == F_RGBA16BF:
        return (arr.astype(np.uint32) << 16).view(np.float32)
    if fmt in (F_RG8, F_RGBA8):
        return arr.astype(np.float32) / np.float32(255.0)
    if fmt in (F_R8U, F_R32U, F_NORMAL, F_RGBA32U):
        return arr.astype(np.float64)
    return arr.astype(np.float64) if arr.dtype == np.float64 else arr.astype(np.float32)


# relative precision of one storage quantum, per format (for the quantised modes)
QUANTUM = {F_E5: 2.0 ** -8, F_RGBA16F: 2.0 ** -10, F_RG16F: 2.0 ** -10, F_R16F: 2.0 ** -10,
           F_RGBA16BF: 2.0 ** -7, F_RGBA8: 1.0 / 255.0, F_B10G11R11: 2.0 ** -5,
           F_R32F: 2.0 ** -22, F_RG32F: 2.0 ** -22, F_RGBA32F: 2.0 ** -22}


def texel_rel_err(a: np.ndarray, b: np.ndarray, atol: float = 1e-6) -> np.ndarray:
    """Per texel: max |a-b| over channels / max(max |b| over channels, atol).
    Relative to the texel's largest channel, like a shared-exponent quantum."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if a.ndim == 2:
        a = a[..., None]
        b = b[..., None]
    both_inf = np.isinf(a) & np.isinf(b) & (np.sign(a) == np.sign(b))
    both_nan = np.isnan(a) & np.isnan(b)
    d = np.where(both_inf | both_nan, 0.0, np.abs(a - b))
    d = np.where(np.isnan(d), np.inf, d)
    scale = np.maximum(np.nanmax(np.where(np.isinf(b), 0, np.abs(b)), axis=-1), atol)
    return np.max(d, axis=-1) / scale


def psnr(a: np.ndarray, ref: np.ndarray) -> float:
    a = np.asarray(a, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    peak = float(np.max(np.abs(ref))) or 1.0
    mse = float(np.mean((a - ref) ** 2))
    return float("inf") if mse == 0 else 10.0 * np.log10(peak * peak / mse)
