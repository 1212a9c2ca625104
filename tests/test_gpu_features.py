"""GPU tests of the extensions around the hot path: Monte Carlo estimator,
adjoint (autograd), batched persistent launch, and the reference-compatible CLI."""
import json
import math
import os
import subprocess
import time

import numpy as np
import pytest

from conftest import LAM, chain64, grid, rel_l2

pytestmark = pytest.mark.gpu


# ---- Monte Carlo (1/16, 64^2 -> 256^2) --------------------------------------------------
def test_mc_matches_oracle_restatement(holo, orc):
    """Same strata, blocks and Philox picks as the oracle, given the plan's tile orders."""
    amp, phase, u, v, _ = chain64()
    v = v[:16384]
    with holo.Plan(u, v, "split32") as pl:
        so, to = pl.order(0), pl.order(1)
        for sub in (16, 5):
            y = pl.execute_mc(amp, phase, -1, LAM, seed=123, subsample=sub, targets_per_block=256)
            ref = orc.transform_mc(amp, phase, u, v, -1, LAM, so, to, seed=123, sub=sub, block=256)
            assert rel_l2(y, ref) < 1e-5


def test_mc_full_sampling_is_brute_force(holo, orc):
    amp, phase, u, v, _ = chain64()
    v = v[:8192]
    y = holo.transform_mc(amp, phase, u, v, -1, LAM, seed=1, subsample=1, targets_per_block=256)
    assert rel_l2(y, orc.transform(amp, phase, u, v, -1, LAM)) < 1e-5


def test_mc16_error_and_unbiasedness(holo, orc):
    """64^2 -> 256^2 with 1/16 of the sources per block of 256 targets, x16 (report rel-L2)."""
    amp, phase, u, v, _ = chain64()
    v = v[:4096]
    ref = orc.transform(amp, phase, u, v, -1, LAM)
    runs = np.array([holo.transform_mc(amp, phase, u, v, -1, LAM, seed=s, subsample=16,
                                       targets_per_block=256) for s in range(64)])
    single = np.mean([rel_l2(r, ref) for r in runs])
    mean_err = rel_l2(runs.mean(0), ref)
    print(f"mc16: MC rel-L2 single {single:.3f}, mean of 64 {mean_err:.3f}")
    assert mean_err < 2.0 * single / math.sqrt(64)


# ---- adjoint (phase-only holograms) -----------------------------------------------------
def _small_problem(seed=0, n=256, m=4096):
    import torch
    rng = np.random.default_rng(seed)
    u = grid(16, 7.56e-6, 0.0)[:n]
    v = grid(64, 10e-6, 0.35)[:m]
    amp = rng.uniform(0.5, 1.0, n)
    phase = rng.uniform(0, 2 * np.pi, n)
    target = rng.uniform(0, 2, m)
    dev = torch.device("cuda:0")
    T = lambda a: torch.as_tensor(a, dtype=torch.float64, device=dev)
    return T(amp), T(phase), T(u), T(v), T(target)


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-9), ("split32", 1e-4)])
def test_adjoint_matches_dense_autograd(holo, prec, tol):
    import torch
    from holo_gb300 import torch_ops
    amp, phase, u, v, target = _small_problem()
    a1 = amp.clone().requires_grad_(True)
    p1 = phase.clone().requires_grad_(True)
    z = torch_ops.dense_reference(a1, p1, u, v, +1, LAM)
    torch_ops.intensity_loss(z, target).backward()
    a2 = amp.clone().requires_grad_(True)
    p2 = phase.clone().requires_grad_(True)
    with holo.Plan(u.reshape(-1), v.reshape(-1), prec) as pl:
        z2 = torch_ops.huygens(a2, p2, pl, +1, LAM)
        assert rel_l2(z2.detach().cpu(), z.detach().cpu()) < max(tol, 1e-11)
        torch_ops.intensity_loss(z2, target).backward()
    assert rel_l2(p2.grad.cpu(), p1.grad.cpu()) < tol
    assert rel_l2(a2.grad.cpu(), a1.grad.cpu()) < tol


def test_adjoint_central_differences(holo):
    """dL/dphi against FP64 central differences (h = 1e-3) on 64 random phases."""
    import torch
    from holo_gb300 import torch_ops
    amp, phase, u, v, target = _small_problem(seed=1)
    with holo.Plan(u.reshape(-1), v.reshape(-1), "fp64") as pl:
        p = phase.clone().requires_grad_(True)
        torch_ops.intensity_loss(torch_ops.huygens(amp, p, pl, +1, LAM), target).backward()
        g = p.grad.cpu().numpy()
        rng = np.random.default_rng(2)
        idx = rng.choice(len(g), 64, replace=False)
        h = 1e-3
        fd = []
        for i in idx:
            pp, pm = phase.clone(), phase.clone()
            pp[i] += h
            pm[i] -= h
            lp = float(torch_ops.intensity_loss(torch_ops.huygens(amp, pp, pl, +1, LAM), target))
            lm = float(torch_ops.intensity_loss(torch_ops.huygens(amp, pm, pl, +1, LAM), target))
            fd.append((lp - lm) / (2 * h))
    fd = np.array(fd)
    assert rel_l2(g[idx], fd) < 1e-5


def test_adjoint_cost_ratio(holo):
    """Backward (adjoint) costs <= 2.5x the forward pass at a size where kernels dominate."""
    import torch
    from holo_gb300 import torch_ops
    dev = torch.device("cuda:0")
    u = torch.as_tensor(grid(512, 7.56e-6, 0.0), device=dev).reshape(-1)
    v = torch.as_tensor(grid(256, 10e-6, 0.35), device=dev).reshape(-1)
    n = u.numel() // 3
    amp = torch.ones(n, dtype=torch.float64, device=dev)
    phase = torch.rand(n, dtype=torch.float64, device=dev) * 2 * math.pi
    with holo.Plan(u, v, "split32") as pl:
        g = torch.randn(v.numel() // 3, 2, dtype=torch.float64, device=dev)
        for _ in range(2):
            pl.execute(amp, phase, +1, LAM)
            pl.adjoint(amp, phase, g, +1, LAM)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(3):
            pl.execute(amp, phase, +1, LAM)
        torch.cuda.synchronize()
        fwd = time.perf_counter() - t0
        t0 = time.perf_counter()
        for _ in range(3):
            pl.adjoint(amp, phase, g, +1, LAM)
        torch.cuda.synchronize()
        bwd = time.perf_counter() - t0
    print(f"adjoint/forward time ratio {bwd / fwd:.2f}")
    assert bwd / fwd <= 2.5


def test_phase_hologram_optimisation_decreases_loss(holo):
    import torch
    from holo_gb300 import torch_ops
    dev = torch.device("cuda:0")
    pp = torch.as_tensor(grid(128, 7.56e-6, 0.0), device=dev)
    tp = torch.as_tensor(grid(64, 10e-6, 0.35), device=dev)
    rng = np.random.default_rng(0)
    yy, xx = np.meshgrid(np.arange(64), np.arange(64), indexing="ij")
    img = sum(rng.uniform(0.2, 1) * np.exp(-((xx - rng.uniform(0, 64)) ** 2 +
                                            (yy - rng.uniform(0, 64)) ** 2) / (2 * 4.0 ** 2))
              for _ in range(8)).ravel()
    target = torch.as_tensor(img / img.mean(), device=dev)
    _, losses = torch_ops.optimise_phase_hologram(pp, tp, target, LAM, steps=30, lr=0.05)
    assert losses[-1] < 0.7 * losses[0]


# ---- batched persistent launch (uneven) ---------------------------------------------------
def test_batched_matches_individual(holo, orc):
    import torch
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(9)
    probs, host = [], []
    for i in range(7):
        ns = int(np.exp(rng.uniform(np.log(1024), np.log(65536))))
        side = int(math.ceil(math.sqrt(ns)))
        u = grid(side, 10e-6, rng.uniform(0.2, 0.5))[:ns]
        mside = [128, 256][i % 2]
        v = grid(mside, 7.56e-6, 0.0)
        amp, phase = rng.uniform(0, 1, ns), rng.uniform(0, 2 * np.pi, ns)
        T = lambda a: torch.as_tensor(np.ascontiguousarray(a).reshape(-1), device=dev)
        y = torch.zeros(2 * len(v), dtype=torch.float64, device=dev)
        sign = -1 if i % 3 else 1
        probs.append(holo.Problem(T(amp), T(phase), T(u), T(v), sign, LAM, y))
        host.append((amp, phase, u, v, sign))
    with holo.Batch(probs, "split32") as b:
        b.execute()
        torch.cuda.synchronize()
        b.execute()  # replay of the captured graph
        torch.cuda.synchronize()
        assert b.pairs == sum(len(h[0]) * len(h[3]) for h in host)
    for pb, (amp, phase, u, v, sign) in zip(probs, host):
        yb = pb.y.cpu().numpy().view(np.complex128)
        yi = holo.transform(amp, phase, u, v, sign, LAM, precision="split32")
        assert rel_l2(yb, yi) < 1e-5  # the batch may run another variant than the planner
        idx = np.arange(0, len(v), 97)
        assert rel_l2(yb[idx], orc.transform_subset(amp, phase, u, v, idx, sign, LAM)) < 1e-5
    holo.handle(0).status()


# ---- CLI: the reference's file interface ---------------------------------------------------
def _cli(holo):
    return os.path.join(os.path.dirname(holo.__file__), "holo")


def test_cli_file_mode_chain(holo, orc, tmp_path):
    rng = np.random.default_rng(21)
    u = grid(16, 10e-6, 0.35)
    v = grid(48, 7.56e-6, 0.0)
    w = grid(16, 10e-6, 0.35)
    amp, phase = rng.uniform(0, 1, len(u)), rng.uniform(0, 2 * np.pi, len(u))
    holo.io.write_inputs(str(tmp_path), amp, phase, u, v, w)
    r = subprocess.run([_cli(holo), "-f", str(tmp_path), "-F", "--lambda", str(LAM)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    y = orc.transform(amp, phase, u, v, -1, LAM)
    yn, _ = orc.normalize_amp(y)
    ya, yp = orc.to_polar(yn)
    got_a = holo.io.read_dat(str(tmp_path / "y0_amp.dat"))
    got_p = holo.io.read_dat(str(tmp_path / "y0_phase.dat"))
    assert np.max(np.abs(got_a - ya)) < 1e-12
    assert rel_l2(got_a * np.exp(1j * got_p), ya * np.exp(1j * yp)) < 1e-12
    z = orc.transform(ya, yp, v, w, +1, LAM)
    zn, _ = orc.normalize_amp(z)
    za, zp = orc.to_polar(zn)
    got_za = holo.io.read_dat(str(tmp_path / "z0_0_amp.dat"))
    got_zp = holo.io.read_dat(str(tmp_path / "z0_0_phase.dat"))
    assert rel_l2(got_za * np.exp(1j * got_zp), za * np.exp(1j * zp)) < 1e-11
    assert np.array_equal(holo.io.read_dat(str(tmp_path / "v0.dat")), v.ravel())
    assert np.array_equal(holo.io.read_dat(str(tmp_path / "w0_0.dat")), w.ravel())
    meta = holo.io.parse_out_json(str(tmp_path / "out.json"))
    assert [m["phasor"] for m in meta] == ["y0", "z0_0"]
    assert [m["pos"] for m in meta] == ["v0", "w0_0"]
    assert meta[0]["len"] == len(v) and meta[0]["dims"] == 3 and meta[0]["precision"] == 8
    assert meta[0]["amp_sum"] == pytest.approx(np.sum(got_a), rel=1e-5)
    for k in ("phase_sum", "x_offset", "width", "randomized", "aspect_ratio", "timestamp",
              "runtime", "flops"):
        assert k in meta[0]


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("split32", 1e-5)])
def test_cli_check_writes_accuracy_keys(holo, orc, tmp_path, prec, tol):
    """--check K: every pass compared with the FP64 sum at K targets; out.json carries
    pairs_per_s on every line and check_targets / rel_l2 / max_phase_err after the
    reference's keys (cuda/util.h:358-396).  The reported y-pass error is checked here
    against the oracle at the same targets."""
    rng = np.random.default_rng(23)
    u = grid(32, 10e-6, 0.35)
    v = grid(128, 7.56e-6, 0.0)
    w = grid(32, 10e-6, 0.35)
    amp, phase = rng.uniform(0, 1, len(u)), rng.uniform(0, 2 * np.pi, len(u))
    holo.io.write_inputs(str(tmp_path), amp, phase, u, v, w)
    r = subprocess.run([_cli(holo), "-f", str(tmp_path), "-F", "--lambda", str(LAM),
                        "--precision", prec, "--check", "300"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    meta = holo.io.parse_out_json(str(tmp_path / "out.json"))
    assert [m["phasor"] for m in meta] == ["y0", "z0_0"]
    for m in meta:
        assert m["pairs_per_s"] > 0 and m["check_targets"] == 300
        assert 0 <= m["rel_l2"] < tol and 0 <= m["max_phase_err"] < 1e3 * tol
    # the y line's error, recomputed: the file field scaled back by max |y| against the oracle
    M, K = len(v), 300
    idx = ((np.arange(K) + 0.5) * M / K).astype(np.int64)
    exact = orc.transform_subset(amp, phase, u, v, idx, -1, LAM)
    ya = holo.io.read_dat(str(tmp_path / "y0_amp.dat"))
    yp = holo.io.read_dat(str(tmp_path / "y0_phase.dat"))
    scale = np.abs(orc.transform(amp, phase, u, v, -1, LAM)).max()
    got = ya[idx] * scale * np.exp(1j * yp[idx])
    assert rel_l2(got, exact) < tol
    if prec == "fp64":  # same scale as the CLI's to ~1e-16: the two figures agree
        assert meta[0]["rel_l2"] == pytest.approx(rel_l2(got, exact), abs=1e-13)


def test_cli_ref_compat_and_w0_fallback(holo, orc, tmp_path):
    rng = np.random.default_rng(22)
    u = grid(8, 10e-6, 0.35)
    v = grid(24, 7.56e-6, 0.0)
    amp, phase = rng.uniform(0, 1, len(u)), rng.uniform(0, 2 * np.pi, len(u))
    holo.io.write_inputs(str(tmp_path), amp, phase, u, v)
    holo.io.write_dat(str(tmp_path / "w0.dat"), grid(8, 10e-6, 0.35))  # the reference's name
    r = subprocess.run([_cli(holo), "-f", str(tmp_path), "-F", "--ref-compat", "--lambda",
                        str(LAM)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    # the reference's -F: z from x at u onto v, Forwards (cuda/main.cu:219)
    z = orc.transform(amp, phase, u, v, +1, LAM)
    zn, _ = orc.normalize_amp(z)
    za, _ = orc.to_polar(zn)
    assert np.max(np.abs(holo.io.read_dat(str(tmp_path / "z0_0_amp.dat")) - za)) < 1e-12


def test_cli_generated_mode(holo, tmp_path):
    r = subprocess.run([_cli(holo), "-x", "16", "-y", "4096", "-z", "1024", "-Z", "2",
                        "--out", str(tmp_path), "--precision", "split32"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    meta = holo.io.parse_out_json(str(tmp_path / "out.json"))
    assert [m["phasor"] for m in meta] == ["x0", "y0", "z0_0", "z0_1"]
    ya = holo.io.read_dat(str(tmp_path / "y0_amp.dat"))
    assert ya.size == 4096 and ya.max() == pytest.approx(1.0)
    u = holo.io.read_dat(str(tmp_path / "u0.dat")).reshape(-1, 3)
    assert np.allclose(u[:, 2], 0.35) and np.allclose(np.hypot(u[:, 0], u[:, 1]), 0.5e-3)
    # the two projection planes ran as one batched launch: each equals its own pass
    yp = holo.io.read_dat(str(tmp_path / "y0_phase.dat"))
    v = holo.io.read_dat(str(tmp_path / "v0.dat")).reshape(-1, 3)
    for j in range(2):
        w = holo.io.read_dat(str(tmp_path / f"w0_{j}.dat")).reshape(-1, 3)
        z = holo.transform(ya, yp, v, w, +1, 0.65e-6, precision="split32")  # CLI default
        za = np.abs(z) / np.abs(z).max()
        zf = holo.io.read_dat(str(tmp_path / f"z0_{j}_amp.dat"))
        assert zf.size == 1024 and np.max(np.abs(zf - za)) < 1e-4


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("split32", 1e-4)])
def test_cli_generated_plane_sweep(holo, tmp_path, prec, tol):
    """-X 3 -Z 2 (cuda/main.cu:125-199): three object planes of different width, height and
    projector width; their x -> y passes run as one batched launch and their six y -> z
    passes as another.  Files and metadata come out in the reference's per-plane order, and
    every plane equals its own single pass."""
    r = subprocess.run([_cli(holo), "-x", "16", "-y", "4096", "-z", "1024", "-X", "3", "-Z", "2",
                        "-o", "1e-4", "-O", "3e-4", "-l", "3e-3", "-L", "4e-3", "-w", "0.3",
                        "-W", "0.4", "--out", str(tmp_path), "--precision", prec],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    meta = holo.io.parse_out_json(str(tmp_path / "out.json"))
    assert [m["phasor"] for m in meta] == [n for i in range(3)
                                           for n in (f"x{i}", f"y{i}", f"z{i}_0", f"z{i}_1")]
    rd = lambda name: holo.io.read_dat(str(tmp_path / name))

    def norm_polar(y):
        return np.abs(y) / np.abs(y).max(), np.angle(y)

    z_heights = []
    for i in range(3):
        xa, xp = rd(f"x{i}_amp.dat"), rd(f"x{i}_phase.dat")
        u, v = rd(f"u{i}.dat").reshape(-1, 3), rd(f"v{i}.dat").reshape(-1, 3)
        z_heights.append(u[0, 2])
        ya, yp = rd(f"y{i}_amp.dat"), rd(f"y{i}_phase.dat")
        ea, _ = norm_polar(holo.transform(xa, xp, u, v, -1, 0.65e-6, precision="fp64"))
        assert np.max(np.abs(ya - ea)) < tol
        for j in range(2):
            w = rd(f"w{i}_{j}.dat").reshape(-1, 3)
            za = rd(f"z{i}_{j}_amp.dat")
            qa, _ = norm_polar(holo.transform(ya, yp, v, w, +1, 0.65e-6, precision="fp64"))
            assert za.size == 1024 and np.max(np.abs(za - qa)) < tol
    assert z_heights[0] == pytest.approx(0.3) and z_heights[2] == pytest.approx(0.4)
    assert not np.array_equal(rd("v0.dat"), rd("v2.dat"))


def test_cli_generated_lattices(holo, tmp_path):
    """The projector lattice of the generated-data mode, built on the device
    (cuda/init.h:89-158): cell centres of a 64 x 64 grid over the 3.584 mm default width
    exactly; with -r the reference's cuRAND jitter keeps every point within its cell's
    random range, and two runs agree bit for bit; an aspect ratio below 1 (where the
    reference reads past its random numbers) runs too."""
    def run(out, *extra):
        r = subprocess.run([_cli(holo), "-x", "4", "-y", "4096", "-z", "256", *extra,
                            "--out", str(out), "--precision", "split32"],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        return holo.io.read_dat(str(out / "v0.dat")).reshape(-1, 3)

    (tmp_path / "a").mkdir()
    v = run(tmp_path / "a")
    x = y = 64
    width = 512 * 7e-6  # the projector's default width (N_sqrt pixels of 7 um)
    dx = width / x
    i, j = np.divmod(np.arange(x * y), y)
    cx = i * dx - (width - dx) / 2
    cy = j * dx - (width - dx) / 2
    assert np.allclose(v[:, 0], cx, rtol=0, atol=1e-15) and np.allclose(v[:, 1], cy, rtol=0,
                                                                        atol=1e-15)
    assert np.all(v[:, 2] == 0.0)
    for name in ("b", "c"):
        (tmp_path / name).mkdir()
    vb, vc = run(tmp_path / "b", "-r"), run(tmp_path / "c", "-r")
    assert np.array_equal(vb, vc)
    half = 0.5 * (dx - 0.5 * 0.05 * dx)
    assert np.all(np.abs(vb[:, 0] - cx) <= half + 1e-15)
    assert np.all(np.abs(vb[:, 1] - cy) <= half + 1e-15)
    assert np.mean(np.abs(vb[:, 0] - cx)) > 0.1 * half  # jittered, not the centres
    (tmp_path / "d").mkdir()
    vd = run(tmp_path / "d", "-r", "-a", "0.5")
    assert np.all(np.isfinite(vd))


def test_batched_short_source_tile_groups(holo, orc):
    """Closer planes need narrower tile pairs: 10 um sources 0.2-0.35 m above a 128^2 grid of
    7.56 um select the tensor-core builds with 256- and 512-source tiles and the 1024-source
    one, and a wide set at 0.2 m a CUDA-core variant; one batch holds the four groups, each
    drained by its own work-queue kernel (the short-tile builds keep two partial-sum
    buffers per tile parity)."""
    import torch
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(31)
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a).reshape(-1), device=dev)
    v = grid(128, 7.56e-6, 0.0)
    cases, planned = [], set()
    for ns, z0, sign in ((4096, 0.2, -1), (16384, 0.25, 1), (4096, 0.35, -1),
                         (40000, 0.2, 1)):
        u = grid(int(math.ceil(math.sqrt(ns))), 10e-6, z0)[:ns]
        with holo.Plan(u, v, "split32") as pl:
            planned.add(pl.info()["variant"])
        amp, phase = rng.uniform(0, 1, ns), rng.uniform(0, 2 * np.pi, ns)
        cases.append((amp, phase, u, sign))
    tc_tiles = {var["source_tile"] for var in holo.variants("split32")
                if var["pair_loop"] == 3 and var["variant"] in planned}
    assert {256, 512, 1024} <= tc_tiles, (planned, "these geometries no longer select the "
                                                   "short-tile tensor-core builds")
    probs = [holo.Problem(T(a), T(p), T(u), T(v), s, LAM,
                          torch.zeros(2 * len(v), dtype=torch.float64, device=dev))
             for a, p, u, s in cases]
    with holo.Batch(probs, "split32") as b:
        b.execute()
        torch.cuda.synchronize()
        b.execute()
        torch.cuda.synchronize()
    idx = np.arange(0, len(v), 61)
    for pb, (amp, phase, u, sign) in zip(probs, cases):
        yb = pb.y.cpu().numpy().view(np.complex128)
        assert rel_l2(yb[idx], orc.transform_subset(amp, phase, u, v, idx, sign, LAM)) < 1e-5


def test_batched_mixed_geometry_groups(holo, orc):
    """Problems of one batch keep the variant their own plan picks: 64^2 -> 128^2 grids of
    27 um pitch 0.35 m apart need the smallest tiles (256 targets x 256 sources) and the
    curvature correction -- with tiles of 1024 the dropped curvature term alone would
    reach ~7e-5 rad -- while the 10 um / 7.56 um problems run the fast variant; the
    batch then holds two groups, each drained by its own queue kernel."""
    import torch
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(21)
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a).reshape(-1), device=dev)
    easy = (grid(64, 10e-6, 0.35), grid(128, 7.56e-6, 0.0))
    hard = (grid(64, 27e-6, 0.35), grid(128, 27e-6, 0.0))
    with holo.Plan(hard[0], hard[1], "split32") as pl:
        info = pl.info()
        assert info["target_tile"] <= 512 and info["path_error_bound_m"] <= 3.2e-13, info
    cases = []
    for u, v in (easy, hard, easy):
        amp, phase = rng.uniform(0, 1, len(u)), rng.uniform(0, 2 * np.pi, len(u))
        cases.append((amp, phase, u, v))
    probs = [holo.Problem(T(a), T(p), T(u), T(v), -1, LAM,
                          torch.zeros(2 * len(v), dtype=torch.float64, device=dev))
             for a, p, u, v in cases]
    with holo.Batch(probs, "split32") as b:
        b.execute()
        torch.cuda.synchronize()
    for pb, (amp, phase, u, v) in zip(probs, cases):
        yb = pb.y.cpu().numpy().view(np.complex128)
        idx = np.arange(0, len(v), 13)
        assert rel_l2(yb[idx], orc.transform_subset(amp, phase, u, v, idx, -1, LAM)) < 1e-5


@pytest.mark.parametrize("shape", ["line", "log-line", "dotted-circle"])
def test_cli_generated_object_shapes(holo, tmp_path, shape):
    """--shape selects the reference's other object shapes (cuda/init.h:175-222): 16 points
    of the default 1 mm wide object 0.35 m above the projector."""
    r = subprocess.run([_cli(holo), "-x", "16", "-y", "1024", "-z", "256", "--shape", shape,
                        "--out", str(tmp_path), "--precision", "split32"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    u = holo.io.read_dat(str(tmp_path / "u0.dat")).reshape(-1, 3)
    n, width = 16, 1e-3
    i = np.arange(n)
    assert np.allclose(u[:, 2], 0.35)
    if shape == "line":
        assert np.allclose(u[:, 0], i * width / (n - 1) - width / 2, rtol=0, atol=1e-15)
        assert np.all(u[:, 1] == 0.0)
    elif shape == "log-line":
        x = 10.0 ** np.linspace(0.0, np.log10(1.0 + width), n) - 1 + width / 2
        assert np.allclose(u[:, 0], x, rtol=0, atol=1e-15)
        assert np.all(u[:, 1] == 0.0)
    else:
        ang = i[1:] * 2 * np.pi / (n - 1) + 0.1125
        assert np.all(u[0, :2] == 0.0)  # the centre point
        assert np.allclose(u[1:, 0], np.sin(ang) * width / 2, rtol=0, atol=1e-15)
        assert np.allclose(u[1:, 1], np.cos(ang) * width / 2, rtol=0, atol=1e-15)
    ya = holo.io.read_dat(str(tmp_path / "y0_amp.dat"))
    assert ya.size == 1024 and ya.max() == pytest.approx(1.0)


def test_cli_rejects_bad_files(holo, tmp_path):
    holo.io.write_inputs(str(tmp_path), [1.0, 2.0], [0.0], [0, 0, 1, 0, 0, 1], [0, 0, 0])
    r = subprocess.run([_cli(holo), "-f", str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 2 and "inconsistent" in r.stderr


# ---- failure path: a bounded device wait that runs out -----------------------------------
def test_bounded_wait_timeout_is_reported_and_the_context_survives(holo, orc):
    """A wait on a barrier that nothing completes gives up after ~1 ms of SM clock, raises
    the handle's error word (HOLO_ERR_TIMEOUT on the next status check, then cleared), and
    the same handle computes correctly afterwards -- no GPU fault is involved."""
    lib, h = holo._native.load(), holo.handle(0)
    h.status()  # nothing pending
    assert lib.holo_selftest_bounded_wait(h.h, 2_000_000, None) == 0
    rc = lib.holo_device_status(h.h, None)
    assert rc == holo._native.ERR_TIMEOUT, rc
    assert b"ran out" in lib.holo_last_error_string()
    assert lib.holo_device_status(h.h, None) == 0  # cleared by the report
    assert lib.holo_selftest_bounded_wait(h.h, 0, None) == holo._native.ERR_INVALID
    amp, phase, u, v, _ = chain64(seed=4)
    u, amp, phase, v = u[:1024], amp[:1024], phase[:1024], v[:4096]
    for prec, tol in (("fp64", 1e-12), ("split32", 1e-5)):
        y = holo.transform(amp, phase, u, v, -1, LAM, precision=prec)
        assert rel_l2(y, orc.transform(amp, phase, u, v, -1, LAM)) < tol
