"""Known-answer tests of the texel codecs (CPU). Values come from the public specifications
the codecs implement: IEEE-754 binary16 (numpy's float16 as the independent reference),
bfloat16 round-to-nearest-even, EXT_texture_shared_exponent (E5B9G9R9), the 11/10-bit
unsigned floats of B10G11R11, and the spherical normal code of Utils.h:105-140."""
import math

import numpy as np
import pytest

import oracle
from tests import _formats as F


def test_f16_decode_all_patterns():
    for h in range(0, 65536, 7):
        ref = np.array([h], dtype=np.uint16).view(np.float16).astype(np.float32)[0]
        got = np.float32(oracle.f16_to_f32(h))
        if np.isnan(ref):
            assert np.isnan(got)
        else:
            assert got == ref, hex(h)


def test_f16_encode_matches_ieee_rne():
    rng = np.random.default_rng(0)
    vals = np.concatenate([
        rng.standard_normal(4000).astype(np.float32) * np.float32(1000),
        rng.standard_normal(2000).astype(np.float32) * np.float32(1e-5),  # subnormal range
        np.array([0.0, -0.0, 65504.0, 65519.99, 65520.0, 1e9, -1e9, 2.0 ** -24, 2.0 ** -25,
                  2.0 ** -25 * 1.0000001, 2.0 ** -14, 1.0 + 2.0 ** -11, 1.0 + 3 * 2.0 ** -11,
                  np.inf, -np.inf], dtype=np.float32),
    ])
    for v in vals:
        ref = np.array([v], dtype=np.float32).astype(np.float16).view(np.uint16)[0]
        assert oracle.f32_to_f16(float(v)) == ref, (v, hex(int(ref)))


@pytest.mark.parametrize("bits,expect", [
    (0x3F800000, 0x3F80),  # 1.0
    (0x3F808000, 0x3F80),  # tie -> even
    (0x3F818000, 0x3F82),  # tie -> even (up)
    (0x3F808001, 0x3F81),  # above the tie
    (0x7F7FFFFF, 0x7F80),  # rounds to +Inf
    (0xC0490FDB, 0xC049),  # -pi
])
def test_bf16_rne(bits, expect):
    v = np.array([bits], dtype=np.uint32).view(np.float32)[0]
    assert oracle.f32_to_bf16(float(v)) == expect


def _e5_spec(r, g, b):
    """EXT_texture_shared_exponent, section 'Shared exponent texture format' (N=9, B=15)."""
    N, B, Emax = 9, 15, 31
    sharedexp_max = (2 ** N - 1) / 2 ** N * 2 ** (Emax - B)
    rc, gc, bc = (max(0.0, min(sharedexp_max, x)) for x in (r, g, b))
    maxrgb = max(rc, gc, bc)
    if maxrgb == 0:
        return 0
    exp_p = max(-B - 1, math.floor(math.log2(maxrgb))) + 1 + B
    maxm = math.floor(maxrgb / 2.0 ** (exp_p - B - N) + 0.5)
    exp_s = exp_p + 1 if maxm == 2 ** N else exp_p
    den = 2.0 ** (exp_s - B - N)
    rs, gs, bs = (math.floor(x / den + 0.5) for x in (rc, gc, bc))
    return (exp_s << 27) | (bs << 18) | (gs << 9) | rs


@pytest.mark.parametrize("rgb", [
    (1.0, 1.0, 1.0), (0.0, 0.0, 0.0), (65408.0, 0.0, 0.0), (1e9, 2.0, 0.5), (1e-9, 0.0, 0.0),
    (0.25, 0.5, 0.125), (511.5, 1.0, 0.0), (511.4, 1.0, 0.0), (3.14159, 2.71828, 1.41421),
    (-1.0, 0.5, 0.25), (6.1035e-5, 3.0517e-5, 0.0), (2.0 ** -16, 2.0 ** -17, 0.0),
])
def test_e5_encode_spec(rgb):
    r, g, b = (float(np.float32(x)) for x in rgb)
    assert oracle.encode_e5(r, g, b) == _e5_spec(r, g, b)


def test_e5_roundtrip_and_canonical():
    rng = np.random.default_rng(1)
    for _ in range(3000):
        c = (np.exp(rng.normal(0, 4, 3)) * rng.uniform(0, 1, 3)).astype(np.float32)
        p = oracle.encode_e5(*map(float, c))
        d = np.array(oracle.decode_e5(p), dtype=np.float32)
        mx = float(min(c.max(), 65408.0))
        if mx > 2.0 ** -15:
            assert np.all(np.abs(d - np.minimum(c, 65408)) <= mx * 2.0 ** -8 + 2.0 ** -24)
        assert oracle.encode_e5(*map(float, d)) == p  # canonical codes are fixed points
        assert np.allclose(F.decode_e5(np.array([p], np.uint32))[0], d, rtol=0, atol=0)


@pytest.mark.parametrize("v,bits11", [
    (1.0, 15 << 6), (0.0, 0), (-3.0, 0), (65024.0, (30 << 6) | 63), (1e6, (30 << 6) | 63),
    (2.0 ** -15, 32), (2.0 ** -20, 1), (2.0 ** -21, 0), (1.0 + 2.0 ** -7, 15 << 6),
    (1.0 + 3 * 2.0 ** -7, (15 << 6) | 2), (float("nan"), 0), (float("inf"), (30 << 6) | 63),
])
def test_b10g11r11_red_channel(v, bits11):
    assert oracle.encode_b10g11r11(v, 0.0, 0.0) & 0x7FF == bits11


def test_b10g11r11_roundtrip():
    rng = np.random.default_rng(2)
    for _ in range(2000):
        c = np.exp(rng.normal(-1, 3, 3)).astype(np.float32)
        p = oracle.encode_b10g11r11(*map(float, c))
        d = np.array(oracle.decode_b10g11r11(p))
        assert np.allclose(d, F.decode_b10g11r11(np.array([p], np.uint32))[0])
        cc = np.minimum(c, [65024, 65024, 64512])
        tol = np.array([2.0 ** -7, 2.0 ** -7, 2.0 ** -6]) * cc + 2.0 ** -19
        assert np.all(np.abs(d - cc) <= tol)


def test_normal_code():
    assert np.allclose(oracle.decode_normal(0), (0.0, 0.0, 1.0))
    rng = np.random.default_rng(3)
    for _ in range(2000):
        n = rng.normal(size=3)
        n /= np.linalg.norm(n)
        d = np.array(oracle.decode_normal(oracle.encode_normal(*map(float, n))))
        assert np.linalg.norm(d - n) < 2e-4


@pytest.mark.parametrize("lum,expect", [
    (0.0, 0), (0.0009, 0), (0.001, 1), (0.125, 1), (128.0, 255), (1e6, 255), (4.0, 128),
    (-1.0, 0), (float("inf"), 255),
])
def test_color_bin_edges(lum, expect):
    # VulkanDevice.cpp:204-210 with the default ev100 range [0, 10]: minLog -3, maxLog 7
    assert oracle.color_bin(lum, -3.0, 7.0) == expect


def test_product_bin_table_matches_oracle():
    """librgdn's host-built histogram table == the oracle's getColorBin, every fp16 pattern."""
    from raytracedgl1_gb300.denoiser import histogram_bin_table
    for lo, hi in [(-3.0, 7.0), (-5.5, 2.25), (0.0, 1.0)]:
        t = histogram_bin_table(lo, hi)
        vals = np.arange(65536, dtype=np.uint32).astype(np.uint16).view(np.float16).astype(np.float32)
        ref = np.array([oracle.color_bin(float(v), lo, hi) for v in vals], dtype=np.uint8)
        assert np.array_equal(t, ref)
