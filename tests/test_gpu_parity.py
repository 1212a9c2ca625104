"""GPU parity: every precision mode against the CPU FP64 oracle, through the C ABI.

Tolerances (relative L2 over the field):
  HOLO_FP64    1e-12  (same rounding sequence per term as the oracle)
  HOLO_SPLIT32 1e-5   (the precision target of the split-precision path)
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, LAM, chain64, chain512, grid, max_phase_err, rel_l2

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "split32": 1e-5}


@pytest.mark.parametrize("prec", ["fp64", "split32"])
def test_golden_small_transform(holo, orc, prec):
    g = np.load(os.path.join(GOLDEN, "transform_small.npz"))
    lam = float(g["lam"])
    y = holo.transform(g["amp"], g["phase"], g["u"], g["v"], -1, lam, precision=prec)
    ref = orc.transform(g["amp"], g["phase"], g["u"], g["v"], -1, lam)
    assert rel_l2(y, ref) < TOL[prec]
    # against the reference's own terms (pow vs sqrt distance: <= 1e-10)
    assert rel_l2(y, g["y"]) < max(TOL[prec], 1e-10)
    z = holo.transform(g["y_amp"], g["y_phase"], g["v"], g["w"], +1, lam, precision=prec)
    assert rel_l2(z, g["z"]) < max(TOL[prec], 1e-10)


@pytest.mark.parametrize("prec", ["fp64", "split32"])
def test_chain64(holo, orc, prec):
    """64^2 chain: 4096 sources -> 65,536 projector pixels -> 4096 projection points."""
    amp, phase, u, v, w = chain64()
    y = holo.transform(amp, phase, u, v, -1, LAM, precision=prec)
    y_ref = orc.transform(amp, phase, u, v, -1, LAM)
    assert rel_l2(y, y_ref) < TOL[prec]
    yn, _ = orc.normalize_amp(y_ref)
    ya, yp = orc.to_polar(yn)
    z = holo.transform(ya, yp, v, w, +1, LAM, precision=prec)
    z_ref = orc.transform(ya, yp, v, w, +1, LAM)
    assert rel_l2(z, z_ref) < TOL[prec]
    if prec == "split32":
        assert max_phase_err(y, y_ref) < 1e-3


@pytest.mark.parametrize("prec", ["fp64", "split32"])
def test_project_chain_matches_oracle(holo, orc, prec):
    """holo_project: normalised polar y and z (cuda/main.cu:186, 213-216 semantics)."""
    amp, phase, u, v, w = chain64(seed=5)
    u, v, w = u[:1024], v[:16384], w[:2048]
    amp, phase = amp[:1024], phase[:1024]
    ya, yp, za, zp = holo.project(amp, phase, u, v, w, LAM, precision=prec)
    y = orc.transform(amp, phase, u, v, -1, LAM)
    yn, _ = orc.normalize_amp(y)
    ra, rp = orc.to_polar(yn)
    assert rel_l2(ya * np.exp(1j * yp), ra * np.exp(1j * rp)) < TOL[prec] * 10
    z = orc.transform(ra, rp, v, w, +1, LAM)
    zn, _ = orc.normalize_amp(z)
    qa, qp = orc.to_polar(zn)
    assert rel_l2(za * np.exp(1j * zp), qa * np.exp(1j * qp)) < max(TOL[prec] * 10, 1e-10)
    assert np.max(ya) == pytest.approx(1.0) and np.max(za) == pytest.approx(1.0)


def test_project_pinned_host_buffers(holo):
    """Page-locked CPU inputs: the outputs come back page-locked, complete when the call
    returns (the copies are asynchronous) and equal to the device-resident call's."""
    import torch
    amp, phase, u, v, w = chain64(seed=7)
    u, v, w = u[:2048], v[:8192], w[:1024]
    amp, phase = amp[:2048], phase[:2048]
    host = [torch.from_numpy(np.ascontiguousarray(a).reshape(-1)).pin_memory()
            for a in (amp, phase, u, v, w)]
    outs = holo.project(*host, LAM, precision="split32")
    assert all(o.is_pinned() and not o.is_cuda for o in outs)
    dev = holo.project(*[h.cuda() for h in host], LAM, precision="split32")
    for o, d in zip(outs, dev):
        assert np.array_equal(o.numpy(), d.cpu().numpy())


@pytest.mark.parametrize("prec", ["fp64", "split32"])
@pytest.mark.parametrize("n,m", [(1, 1), (1, 3000), (7, 5), (513, 2049), (3000, 1),
                                 (1025, 777)])
def test_ragged_sizes(holo, orc, prec, n, m):
    rng = np.random.default_rng(n * 31 + m)
    u = np.column_stack([rng.uniform(-1e-3, 1e-3, (n, 2)), np.full(n, 0.3)])
    v = np.column_stack([rng.uniform(-2e-3, 2e-3, (m, 2)), np.zeros(m)])
    amp, phase = rng.uniform(0, 1, n), rng.uniform(0, 2 * np.pi, n)
    for sign in (-1, 1):
        y = holo.transform(amp, phase, u, v, sign, LAM, precision=prec)
        assert rel_l2(y, orc.transform(amp, phase, u, v, sign, LAM)) < TOL[prec]


@pytest.mark.parametrize("n,m", [(1000, 777), (1025, 2049), (3, 600), (5000, 1)])
def test_tensor_core_variants_ragged(holo, orc, n, m):
    """Every tensor-core build on sizes that fill neither the 1024- (768-) source tiles nor
    the 512-target tiles: the padding sources, the targets past M in the last tile and the
    per-item staging of target records must all drop out."""
    rng = np.random.default_rng(n + 7 * m)
    u = grid(int(np.ceil(np.sqrt(n))), 10e-6, 0.35)[:n]
    v = grid(int(np.ceil(np.sqrt(m))), 7.56e-6, 0.0)[:m]
    amp, phase = rng.uniform(0, 1, n), rng.uniform(0, 2 * np.pi, n)
    refs = {s: orc.transform(amp, phase, u, v, s, LAM) for s in (-1, 1)}
    tc = [var for var in holo.variants("split32") if var["pair_loop"] == 3]
    assert tc, "no tensor-core build in the variant table"
    for var in tc:
        for s in (-1, 1):
            y = holo.transform(amp, phase, u, v, s, LAM, precision="split32",
                               variant=var["variant"])
            assert rel_l2(y, refs[s]) < TOL["split32"], (var, s)


@pytest.mark.parametrize("prec", ["fp64", "split32"])
def test_tilted_and_3d_geometry(holo, orc, prec):
    """Non-parallel planes and a 3-D cloud (the frame basis is built per tile pair)."""
    rng = np.random.default_rng(11)
    n, m = 2000, 5000
    s = rng.uniform(-1.5e-3, 1.5e-3, (n, 2))
    u = np.column_stack([s[:, 0], s[:, 1], 0.25 + 0.3 * s[:, 0]])  # tilted source plane
    v = np.column_stack([rng.uniform(-2e-3, 2e-3, (m, 2)), rng.uniform(-5e-4, 5e-4, m)])
    amp, phase = rng.uniform(0, 1, n), rng.uniform(0, 2 * np.pi, n)
    y = holo.transform(amp, phase, u, v, -1, LAM, precision=prec)
    assert rel_l2(y, orc.transform(amp, phase, u, v, -1, LAM)) < TOL[prec]


@pytest.mark.parametrize("prec", ["fp64", "split32"])
def test_const_phase_counts_sources(holo, prec):
    """TEST_CONST_PHASE (cuda/superposition.cu:113-116): every term 1+0i, so y_m == N exactly,
    through source splits, partial sums and the scatter back to caller order."""
    amp, phase, u, v, _ = chain64()
    for n, m in ((4096, 65536), (4096, 300), (1000, 5000)):
        y = holo.transform(amp[:n], phase[:n], u[:n], v[:m], -1, LAM, precision=prec,
                           flags=holo.FLAG_CONST_PHASE)
        assert np.all(y.real == n) and np.all(y.imag == 0)


@pytest.mark.parametrize("prec", ["fp64", "split32"])
def test_deterministic(holo, prec):
    amp, phase, u, v, _ = chain64(seed=2)
    a = holo.transform(amp, phase, u, v[:20000], -1, LAM, precision=prec)
    b = holo.transform(amp, phase, u, v[:20000], -1, LAM, precision=prec)
    assert np.array_equal(a, b)


def test_chain512_split_vs_fp64_kernel(holo, orc):
    """512^2 sources -> 1024^2 projector at full source count: split-FP32 vs the FP64
    kernel (validated above against the CPU oracle) on a seeded 4096-target subset, and
    vs the CPU oracle on 64 targets."""
    import torch
    amp, phase, u, v, _ = chain512()
    rng = np.random.default_rng(1)
    idx = np.sort(rng.choice(len(v), 4096, replace=False))
    ys = holo.transform(amp, phase, u, v[idx], -1, LAM, precision="split32")
    yd = holo.transform(amp, phase, u, v[idx], -1, LAM, precision="fp64")
    err = rel_l2(ys, yd)
    print(f"chain512 subset: rel-L2 {err:.3e}, max phase err {max_phase_err(ys, yd):.3e}")
    assert err < 1e-5
    yc = orc.transform_subset(amp, phase, u, v, idx[:64], -1, LAM)
    assert rel_l2(yd[:64], yc) < 1e-12
    # the full 2.75e11-pair pass runs on device buffers
    dev = torch.device("cuda:0")
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a).reshape(-1), device=dev)
    y_full = holo.transform(t(amp), t(phase), t(u), t(v), -1, LAM, precision="split32")
    torch.cuda.synchronize()
    y_full = y_full.cpu().numpy()
    assert rel_l2(y_full[idx], yd) < 1e-5


def test_plan_reuse_and_orders(holo, orc):
    amp, phase, u, v, _ = chain64(seed=3)
    with holo.Plan(u, v[:30000], "split32") as pl:
        so, to = pl.order(0), pl.order(1)
        assert np.array_equal(np.sort(so), np.arange(len(u)))
        assert np.array_equal(np.sort(to), np.arange(30000))
        for seed in range(2):
            ph = np.random.default_rng(seed).uniform(0, 2 * np.pi, len(u))
            y = pl.execute(amp, ph, -1, LAM)
            assert rel_l2(y, orc.transform(amp, ph, u, v[:30000], -1, LAM)) < 1e-5


def test_torch_device_path_is_async_and_matches(holo, orc):
    import torch
    amp, phase, u, v, _ = chain64(seed=4)
    dev = torch.device("cuda:0")
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a).reshape(-1), device=dev)
    y = holo.transform(t(amp), t(phase), t(u), t(v), -1, LAM, precision="split32")
    assert y.is_cuda and y.dtype == torch.complex128
    torch.cuda.synchronize()
    assert rel_l2(y.cpu().numpy(), orc.transform(amp, phase, u, v, -1, LAM)) < 1e-5
    holo.handle(0).status()


def test_invalid_arguments_return_status(holo):
    amp, phase, u, v, _ = chain64()
    with pytest.raises(ValueError):  # the Python layer rejects it first
        holo.transform(amp, phase, u, v, 0, LAM)
    lib, h = holo._native.load(), holo.handle(0)
    a, p, uu, vv = (np.ascontiguousarray(x) for x in (amp, phase, u, v))
    y = np.zeros(2 * len(v))
    rc = lib.holo_transform(h.h, 0, LAM, a.ctypes.data, p.ctypes.data, uu.ctypes.data, len(a),
                            vv.ctypes.data, len(v), y.ctypes.data, 1, None)
    assert rc == -1 and b"sign" in lib.holo_last_error_string()
    with pytest.raises(holo.HoloError):
        holo.transform(amp, phase, u, v, -1, float("nan"))
    with pytest.raises(holo.HoloError):
        holo.transform(amp, phase, u, v, -1, LAM, precision="split32", variant=99)
    import torch
    with pytest.raises(holo.HoloError):  # mixed host and device pointers
        holo.transform(torch.as_tensor(amp, device="cuda:0"), phase, u, v, -1, LAM)
    holo.handle(0).status()  # nothing left on the device error word


@pytest.mark.parametrize("prec", ["fp64", "split32"])
@pytest.mark.parametrize("on_device", [False, True])
def test_empty_inputs(holo, prec, on_device):
    """No sources: every target's sum is the empty sum 0; no targets: an empty result."""
    import torch
    if on_device:
        put = lambda a: torch.as_tensor(np.ascontiguousarray(a).reshape(-1), device="cuda:0")
    else:
        put = lambda a: np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
    e = np.zeros(0)
    v = grid(10, 7.56e-6, 0.0)
    y = holo.transform(put(e), put(e), put(e), put(v), -1, LAM, precision=prec)
    y = y.cpu().numpy() if on_device else y
    assert y.shape == (100,) and np.all(y == 0)
    u = grid(4, 10e-6, 0.35)
    y = holo.transform(put(np.ones(16)), put(np.zeros(16)), put(u), put(e), -1, LAM,
                       precision=prec)
    assert tuple(y.shape) == (0,)
    holo.handle(0).status()


def test_maximum_point_counts(holo):
    """The largest planes the tiler takes, 4096 x 4096 points per side: that many targets
    from 64 sources, and that many sources onto 256 targets, match the FP64 kernel (the
    oracle at this size, itself checked against the C oracle above) within the split
    tolerance.  One point more on either side is rejected with HOLO_ERR_INVALID; the
    buffers are real and of the claimed size, so nothing could be read out of bounds even
    if the check were missing."""
    import torch
    lim = 4096 * 4096
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(40)
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a).reshape(-1), device=dev)

    def check(u, v):
        n = len(u)
        amp, phase = t(rng.uniform(0, 1, n)), t(rng.uniform(0, 2 * np.pi, n))
        y32 = holo.transform(amp, phase, t(u), t(v), -1, LAM, precision="split32")
        y64 = holo.transform(amp, phase, t(u), t(v), -1, LAM, precision="fp64")
        err = float(torch.linalg.vector_norm(y32 - y64) / torch.linalg.vector_norm(y64))
        assert y32.numel() == len(v) and err < 1e-5, err

    check(grid(8, 10e-6, 0.35), grid(4096, 7.56e-6, 0.0))  # 64 -> 4096^2
    check(grid(4096, 10e-6, 0.35), grid(16, 7.56e-6, 0.0))  # 4096^2 -> 256
    torch.cuda.empty_cache()

    over = lim + 1
    src = t(grid(8, 10e-6, 0.35))
    amp, phase = t(np.ones(64)), t(np.zeros(64))
    with pytest.raises(holo.HoloError) as e:  # M above the limit
        holo.transform(amp, phase, src, torch.zeros(3 * over, dtype=torch.float64, device=dev),
                       -1, LAM, precision="split32")
    assert e.value.code == holo._native.ERR_INVALID and "supported" in str(e.value)
    u_over = torch.zeros(over, 3, dtype=torch.float64, device=dev)
    u_over[:, 2] = 0.35
    with pytest.raises(holo.HoloError) as e:  # N above the limit
        holo.transform(torch.ones(over, dtype=torch.float64, device=dev),
                       torch.zeros(over, dtype=torch.float64, device=dev), u_over,
                       t(grid(16, 7.56e-6, 0.0)), -1, LAM, precision="split32")
    assert e.value.code == holo._native.ERR_INVALID and "supported" in str(e.value)
    holo.handle(0).status()


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-10), ("split32", 1e-5)])
def test_reference_wave_amplitude_only(holo, orc, prec, tol):
    """PROJECT_PHASE=0 path (cuda/transform.cu:379-395) restated with the oracle, in both
    precisions."""
    amp, phase, u, v, _ = chain64(seed=6)
    u, amp, phase, v = u[:512], amp[:512], phase[:512], v[:8192]
    ya, yp, _, _ = holo.project(amp, phase, u, v, None, LAM, precision=prec,
                                reference_wave=True, reference_distance=0.25)
    y = orc.transform(amp, phase, u, v, -1, LAM)
    src = np.array([[0.0, 0.0, v[0, 2] - 0.25]])
    yr = orc.transform([1.0], [0.0], src, v, +1, LAM)
    yn, _ = orc.normalize_amp(y)
    rn, _ = orc.normalize_amp(yr)
    expect_amp = np.abs(yn + rn)
    expect_phase = np.angle(rn)
    assert np.max(np.abs(ya - expect_amp)) < 10 * tol
    assert np.max(np.abs(np.angle(np.exp(1j * (yp - expect_phase))))) < 10 * tol
    assert rel_l2(ya * np.exp(1j * yp), expect_amp * np.exp(1j * expect_phase)) < tol


@pytest.mark.parametrize("prec", ["fp64", "split32"])
def test_every_kernel_variant(holo, orc, prec):
    """Each kernel variant (tile shapes, FMA-pipe sin/cos share, curvature term on or off)
    meets the precision target on a 32x32 -> 64x64 patch of the 64^2 -> 256^2 planes, both
    signs.  The variants without the curvature term are exact enough here because the
    planes are 0.35 m apart and the tiles are a fraction of a millimetre wide."""
    rng = np.random.default_rng(11)
    u, v = grid(32, 10e-6, 0.35), grid(64, 7.56e-6, 0.0)
    amp, phase = rng.uniform(0, 1, len(u)), rng.uniform(0, 2 * np.pi, len(u))
    refs = {s: orc.transform(amp, phase, u, v, s, LAM) for s in (-1, 1)}
    for var in holo.variants(prec):
        for s in (-1, 1):
            y = holo.transform(amp, phase, u, v, s, LAM, precision=prec,
                               variant=var["variant"])
            assert rel_l2(y, refs[s]) < TOL[prec], (var, s)
