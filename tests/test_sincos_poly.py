"""The FMA-pipe sin/cos polynomials of the split kernels, checked on the CPU.

The coefficients are read from csrc/split_frame.cuh and evaluated in float32 the way the
kernels do (one rounding per FMA, Horner order, the 1.5 * 2^23 rounding trick), so a
coefficient edited without refitting, or a reduction step changed, fails here:
  - poly_sincos / poly_sincos2: full-turn reduction, degree 11/12;
  - poly_sincos2_half: half-turn reduction, degree 9/8, (-1)^n taken from bit 0 of the
    rounded value (the sign mask the kernel puts on the amplitude).
"""
import os
import re

import numpy as np
import pytest

CSRC = os.path.join(os.path.dirname(__file__), "..", "holographic-projector-simulations_gb300",
                    "csrc")
F32 = np.float32
MAGIC = 12582912.0


def _body(name: str) -> str:
    src = open(os.path.join(CSRC, "split_frame.cuh")).read()
    start = src.index(f"void {name}(")
    return src[start:src.index("\n}\n", start)]


def _floats(text: str) -> list[float]:
    """Float literals of a function body in source order, without the rounding constant."""
    vals = [float(x) for x in re.findall(r"(-?\d+\.\d+(?:e[+-]\d+)?)f\b", text)]
    return [v for v in vals if v != MAGIC]


def _fma(a, b, c):
    # float64 holds the product of two float32 values exactly: one rounding, as FMA
    return (a.astype(np.float64) * b + c).astype(F32)


def _rnd(x):
    return np.asarray(x, dtype=np.float64).astype(F32)


def _horner(coefs, x2):
    """coefs in the kernel's order: the first FMA is fma(coefs[0], x2, coefs[1])."""
    acc = _fma(np.full_like(x2, F32(coefs[0])), x2, F32(coefs[1]))
    for c in coefs[2:]:
        acc = _fma(acc, x2, F32(c))
    return acc


def full_turn(th):
    body = _body("poly_sincos2")
    k = _floats(body)
    # constants in source order: 1 / 2pi, then 6 sin and 7 cos coefficients
    scale, s_c, c_c = k[0], k[1:7], k[7:14]
    assert len(k) == 14
    t = _rnd(th.astype(np.float64) * F32(scale))
    n = _rnd(_rnd(t.astype(np.float64) + MAGIC).astype(np.float64) - MAGIC)
    f = _rnd(t.astype(np.float64) - n)
    f2 = _rnd(f.astype(np.float64) * f)
    s = _rnd(_horner(s_c, f2).astype(np.float64) * f)
    c = _horner(c_c, f2)
    return s.astype(np.float64), c.astype(np.float64)


def half_turn(th):
    body = _body("poly_sincos2_half")
    k = _floats(body)
    scale, s_c, c_c = k[0], k[1:6], k[6:11]
    assert len(k) == 11
    assert "12582912.0f" in body and "0x8000000080000000ull" in body
    h = _rnd(th.astype(np.float64) * F32(scale))
    u = _rnd(h.astype(np.float64) + MAGIC)
    g = _rnd(h.astype(np.float64) - _rnd(u.astype(np.float64) - MAGIC))
    g2 = _rnd(g.astype(np.float64) * g)
    s = _rnd(_horner(s_c, g2).astype(np.float64) * g)
    c = _horner(c_c, g2)
    sign = np.where((u.view(np.uint32) & 1) == 1, -1.0, 1.0)
    return sign * s, sign * c


def _errors(fn, th):
    s, c = fn(th)
    x = th.astype(np.float64)
    return np.abs(s - np.sin(x)).max(), np.abs(c - np.cos(x)).max()


def test_half_turn_within_its_bound_on_one_turn():
    th = np.linspace(-np.pi, np.pi, 400_001).astype(F32)
    es, ec = _errors(half_turn, th)
    assert es <= 2.5e-7 and ec <= 3.5e-7, (es, ec)


def test_full_turn_within_its_bound_on_one_turn():
    th = np.linspace(-np.pi, np.pi, 400_001).astype(F32)
    es, ec = _errors(full_turn, th)
    assert es <= 1.0e-6 and ec <= 1.0e-6, (es, ec)


def test_half_turn_no_worse_than_full_turn_on_wide_arguments():
    # beyond one turn both are limited by the float32 rounding of th / (pi or 2 pi)
    rng = np.random.default_rng(3)
    th = rng.uniform(-60.0, 60.0, 400_000).astype(F32)
    hs, hc = _errors(half_turn, th)
    fs, fc = _errors(full_turn, th)
    assert max(hs, hc) <= 1.1 * max(fs, fc), (hs, hc, fs, fc)
    assert max(hs, hc) < 6e-6


def test_half_turn_sign_at_quadrant_boundaries():
    # odd multiples of pi flip both sin and cos; the result stays continuous across the
    # boundaries of the reduction (g = +-1/2)
    k = np.arange(-6, 6)
    for off in (-1e-3, 0.0, 1e-3):
        th = (np.pi * (k + 0.5) + off).astype(F32)
        s, c = half_turn(th)
        x = th.astype(np.float64)
        assert np.abs(s - np.sin(x)).max() < 1.5e-6
        assert np.abs(c - np.cos(x)).max() < 1.5e-6


def half_turns_given(h, sin7):
    """poly_sincos2_ht: the angle arrives in half turns (h = theta / pi); SIN7 selects the
    degree-7 sine (the first of the two sine coefficient sets in the source)."""
    body = _body("poly_sincos2_ht")
    k = _floats(body)
    assert len(k) == 4 + 5 + 5  # degree-7 sine, degree-9 sine, degree-8 cosine
    s_c = k[0:4] if sin7 else k[4:9]
    c_c = k[9:14]
    u = _rnd(h.astype(np.float64) + MAGIC)
    g = _rnd(h.astype(np.float64) - _rnd(u.astype(np.float64) - MAGIC))
    g2 = _rnd(g.astype(np.float64) * g)
    s = _rnd(_horner(s_c, g2).astype(np.float64) * g)
    c = _horner(c_c, g2)
    sign = np.where((u.view(np.uint32) & 1) == 1, -1.0, 1.0)
    return sign * s, sign * c


@pytest.mark.parametrize("sin7,bound", [(True, 8.0e-7), (False, 2.5e-7)])
def test_half_turns_given_within_bound(sin7, bound):
    # the tensor cores deliver h = theta / pi; over two turns of theta
    h = np.linspace(-2.0, 2.0, 400_001).astype(F32)
    s, c = half_turns_given(h, sin7)
    x = np.pi * h.astype(np.float64)
    assert np.abs(s - np.sin(x)).max() <= bound
    assert np.abs(c - np.cos(x)).max() <= 3.5e-7
    # the degree-9 set is the one poly_sincos2_half uses
    if not sin7:
        assert _floats(_body("poly_sincos2_ht"))[4:] == _floats(_body("poly_sincos2_half"))[1:]
