"""CPU tests: the oracle pinned against the reference's own golden data.

The fixtures under tests/golden/ were produced by tests/golden/make_golden.py
from the reference itself (its host-compiled phasor_displacement and its
NumPy prototype); these tests read only the committed files.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, LAM, grid, rel_l2


@pytest.mark.parametrize("tag", ["6328", "650"])
def test_pairs_match_reference_host_function(orc, tag):
    g = np.load(os.path.join(GOLDEN, f"pairs_{tag}.npz"))
    lam = float(g["lam"])
    out = np.array([orc.phasor(a, p, u, v, int(s), lam)
                    for a, p, u, v, s in zip(g["amp"], g["phase"], g["u"], g["v"], g["sign"])])
    ref = g["ref"][:, 0] + 1j * g["ref"][:, 1]
    same = np.mean(out == ref)
    rel = np.abs(out - ref) / np.abs(ref)
    # the reference's norm3d_host is pow(s, 0.5); the oracle uses sqrt: they
    # agree bit for bit except for rare last-ulp distances (x k r ~ 1e7 rad/m)
    assert same > 0.99, same
    assert rel.max() < 2e-9, rel.max()


def test_known_answer_unit_source_at_lambda(orc):
    """py/test_util.py:49-64: amp 1/lambda, phase ~ 2.449e-16 (direction=+1 = Backwards)."""
    ka = json.load(open(os.path.join(GOLDEN, "known_answer.json")))
    lam = ka["lambda"]
    c = orc.phasor(1.0, 0.0, [0.0, 0.0, 0.0], [0.0, 0.0, lam], ka["sign_cuda"], lam)
    assert abs(c) == pytest.approx(ka["amp_asserted"], rel=1e-15)
    assert abs(np.angle(c) - ka["phase_asserted"]) < 1e-15
    assert ka["amp"] == ka["amp_asserted"] and ka["phase"] == ka["phase_asserted"]


def test_small_transform_matches_reference_terms(orc):
    g = np.load(os.path.join(GOLDEN, "transform_small.npz"))
    lam = float(g["lam"])
    y = orc.transform(g["amp"], g["phase"], g["u"], g["v"], -1, lam)
    assert rel_l2(y, g["y"]) < 1e-10
    yn, _ = orc.normalize_amp(y)
    a, p = orc.to_polar(yn)
    assert np.max(np.abs(a - g["y_amp"])) < 1e-9
    assert np.max(np.abs(np.angle(np.exp(1j * (p - g["y_phase"]))))) < 1e-8
    z = orc.transform(g["y_amp"], g["y_phase"], g["v"], g["w"], +1, lam)
    assert rel_l2(z, g["z"]) < 1e-10


def test_prototype_agrees_with_oracle(orc):
    """py/ prototype (map_sum_kernel, direction=+1) vs the oracle's Backwards sum."""
    g = np.load(os.path.join(GOLDEN, "transform_small.npz"))
    y = orc.transform(g["amp"], g["phase"], g["u"], g["v"], -1, float(g["lam"]))
    proto = g["proto_y_amp"] * np.exp(1j * g["proto_y_phase"])
    assert rel_l2(proto, y) < 1e-8


def test_normalize_threshold(orc):
    """normalize_amp leaves fields with max |y| < 1e-6 unchanged (cuda/transform.cu:112-115)."""
    y = np.array([1e-7 + 0j, 3e-7j, -2e-7 + 1e-8j])
    yn, mx = orc.normalize_amp(y)
    assert np.array_equal(yn, y) and mx < 1e-6
    y2 = np.array([3 + 4j, 1 + 0j, -0.5j])
    yn2, mx2 = orc.normalize_amp(y2)
    assert mx2 == 5.0
    assert np.array_equal(yn2.real, y2.real / 5.0) and np.array_equal(yn2.imag, y2.imag / 5.0)


def test_unit_phasor_invariant(orc):
    """TEST_CONST_PHASE analogue on the oracle side: a coherent focus.

    Sources whose phases cancel k r at one target add up to sum a_n / r_n there."""
    lam = LAM
    u = grid(8, 10e-6, 0.2)
    v = np.array([[0.0, 0.0, 0.0]])
    r = np.linalg.norm(u - v, axis=1)
    k = orc.wavenumber(lam)
    amp = np.ones(len(u))
    phase = k * r  # Backwards: phase - k r = 0
    y = orc.transform(amp, phase, u, v, -1, lam)
    assert y[0].real == pytest.approx(np.sum(1 / r), rel=1e-9)
    assert abs(y[0].imag) < 1e-6 * np.sum(1 / r)


def test_philox_known_answers(orc):
    """Random123's published philox4x32-10 known-answer vectors."""
    kat = [
        ((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
        ((0xffffffff,) * 4, (0xffffffff,) * 2, (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
        ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
         (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)),
    ]
    for ctr, key, out in kat:
        assert tuple(int(x) for x in orc.philox(ctr, key)) == out


def test_mc_oracle_full_sampling_is_brute_force(orc):
    rng = np.random.default_rng(3)
    u = grid(16, 10e-6, 0.35)
    v = grid(12, 7.56e-6, 0.0)
    amp, phase = rng.uniform(0, 1, len(u)), rng.uniform(0, 2 * np.pi, len(u))
    so = rng.permutation(len(u)).astype(np.int32)
    to = rng.permutation(len(v)).astype(np.int32)
    y = orc.transform(amp, phase, u, v, -1, LAM)
    ymc = orc.transform_mc(amp, phase, u, v, -1, LAM, so, to, seed=7, sub=1, block=32)
    assert rel_l2(ymc, y) < 1e-13


def test_mc_oracle_is_unbiased(orc):
    rng = np.random.default_rng(4)
    u = grid(16, 10e-6, 0.35)
    v = grid(4, 7.56e-6, 0.0)
    amp, phase = rng.uniform(0, 1, len(u)), rng.uniform(0, 2 * np.pi, len(u))
    so = np.arange(len(u), dtype=np.int32)
    to = np.arange(len(v), dtype=np.int32)
    y = orc.transform(amp, phase, u, v, -1, LAM)
    runs = np.array([orc.transform_mc(amp, phase, u, v, -1, LAM, so, to, seed=s, sub=16,
                                      block=16) for s in range(400)])
    single = np.mean([rel_l2(r, y) for r in runs[:20]])
    mean_err = rel_l2(runs.mean(0), y)
    # averaging 400 independent estimates shrinks the error ~ 1/sqrt(400)
    assert mean_err < 3.0 * single / np.sqrt(400)


def test_oracle_rejects_bad_arguments(orc):
    with pytest.raises(ValueError):
        orc.transform([1.0], [0.0], [0, 0, 1], [0, 0, 0], -1, -1.0)
