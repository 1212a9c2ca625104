"""Parity at the benchmark configurations' full scale, the autotuner, and the planner's
error bound on random geometries.

- config 4: 64 uneven problems (up to 262,144 sources and 1024^2 targets) as one batched
  launch against the FP64 kernel at sampled targets of every problem;
- config 5: the split-precision adjoint of the 1024^2 -> 512^2 y -> z pass against the
  FP64 adjoint at sampled sources;
- the autotuner (holo_autotune, its JSON table, reloading, and the planner refusing a
  tuned variant whose error bound fails; the reference's counterpart is the dispatch
  switch of cuda/transform.cu:50-104 over the geometry of cuda/init.h:42-84);
- seeded tilted, wide and close planes: the measured error of every target against the
  FP64 kernel stays within the phase bound k * holo_plan_error_bound.
"""
import json
import math

import numpy as np
import pytest

from conftest import LAM, grid, rel_l2

pytestmark = pytest.mark.gpu


def _dev_t():
    import torch
    dev = torch.device("cuda:0")
    return dev, (lambda a: torch.as_tensor(np.ascontiguousarray(a).reshape(-1), device=dev))


def test_batch64_full_scale_against_fp64(holo):
    """Config 4 at full size: N log-uniform in [1024, 262144] on square-ish 10 um grids,
    z0 U[0.2, 0.5] m, projectors 128^2 .. 1024^2 (at least one of each size), one
    batched launch; every problem within 1e-5 of the FP64 kernel at 512 targets."""
    import torch
    dev, t = _dev_t()
    rng = np.random.default_rng(0)
    sides = [128, 256, 512, 1024] + list(rng.choice([128, 256, 512, 1024], 60))
    host, probs = [], []
    for side in sides:
        ns = int(np.exp(rng.uniform(np.log(1024), np.log(262144))))
        sq = int(np.ceil(np.sqrt(ns)))
        u = grid(sq, 10e-6, rng.uniform(0.2, 0.5))[:ns]
        v = grid(int(side), 7.56e-6, 0.0)
        amp, phase = rng.uniform(0, 1, ns), rng.uniform(0, 2 * np.pi, ns)
        y = torch.full((2 * len(v),), float("nan"), dtype=torch.float64, device=dev)
        host.append((amp, phase, u, v))
        probs.append(holo.Problem(t(amp), t(phase), t(u), t(v), -1, LAM, y))
    assert max(len(h[0]) for h in host) > 131072
    with holo.Batch(probs, "split32") as b:
        b.execute()
        b.execute()  # a replay of the captured graph gives the same fields
    torch.cuda.synchronize()
    worst = 0.0
    for (amp, phase, u, v), p in zip(host, probs):
        yb = p.y.cpu().numpy().view(np.complex128)
        assert np.all(np.isfinite(yb))
        idx = np.sort(rng.choice(len(v), min(512, len(v)), replace=False))
        y64 = holo.transform(t(amp), t(phase), t(u), t(v[idx]), -1, LAM,
                             precision="fp64").cpu().numpy()
        worst = max(worst, rel_l2(yb[idx], y64))
    assert worst < 1e-5, worst
    holo.handle(0).status()


def test_adjoint_split_full_scale_against_fp64(holo):
    """Config 5's adjoint at full size: 1024^2 projector sources (unit amplitude, random
    phases) -> 512^2 targets, Forwards.  The gradient of every source depends only on that
    source and all targets, so the FP64 adjoint of 1024 sampled sources alone is the
    exact reference for those sources."""
    import torch
    dev, t = _dev_t()
    g = torch.Generator(device="cpu").manual_seed(3)
    u = grid(1024, 7.56e-6, 0.0)
    v = grid(512, 10e-6, 0.35)
    n, m = len(u), len(v)
    amp = torch.ones(n, dtype=torch.float64, device=dev)
    phase = (torch.rand(n, generator=g, dtype=torch.float64) * 2 * math.pi).to(dev)
    grad_y = torch.randn(2 * m, generator=g, dtype=torch.float64).to(dev)
    du, dv = t(u), t(v)
    with holo.Plan(du, dv, "split32") as pl:
        ga, gp = pl.adjoint(amp, phase, grad_y, +1, LAM)
    rng = np.random.default_rng(4)
    idx = np.sort(rng.choice(n, 1024, replace=False))
    it = torch.as_tensor(idx, device=dev)
    ea, ep = holo.adjoint(amp[it], phase[it], t(u[idx]), dv, grad_y, +1, LAM, precision="fp64")
    ga, gp, ea, ep = (x.cpu().numpy() for x in (ga[it], gp[it], ea, ep))
    assert rel_l2(ga, ea) < 1e-5 and rel_l2(gp, ep) < 1e-5
    # the complex adjoint field w_n = grad_amp - i grad_phase / a_n, as one vector
    assert rel_l2(ga - 1j * gp, ea - 1j * ep) < 1e-5
    holo.handle(0).status()


def test_autotuner_records_persists_and_reloads(holo, tmp_path, monkeypatch):
    """holo_autotune times every variant on a synthetic problem and records the fastest
    for the size bucket; api.autotune writes the JSON table ($HOLO_TUNE_CACHE) that a
    fresh handle loads."""
    from holo_gb300 import api
    cache = tmp_path / "tune.json"
    monkeypatch.setenv("HOLO_TUNE_CACHE", str(cache))
    n, m = 1024, 16384
    bucket = holo.size_bucket(n, m)
    h = holo.handle(0)
    try:
        res = api.autotune(n, m, "split32", repeats=1)
        assert res["bucket"] == bucket and res["pairs_per_s"] > 0
        assert 0 <= res["variant"] < len(holo.variants("split32"))
        assert h.get_variant("split32", bucket) == res["variant"]
        assert json.loads(cache.read_text())["split32"][str(bucket)] == res["variant"]
        fresh = api.Handle(0)
        try:
            assert fresh.get_variant("split32", bucket) == -1
            api.load_tuning(fresh)
            assert fresh.get_variant("split32", bucket) == res["variant"]
        finally:
            fresh.close()
    finally:
        h.set_variant("split32", bucket, -1)


def test_tuned_variant_refused_where_its_bound_fails(holo):
    """A variant recorded for a bucket is the planner's first candidate, taken where its
    error bound holds and refused where it does not: variant 13 drops the curvature
    term, which is fine 0.35 m from the projector and not 0.05 m from it (where the
    curvature-corrected builds on narrower tiles still meet the budget)."""
    dev, t = _dev_t()
    rng = np.random.default_rng(5)
    u_far, u_near = grid(64, 10e-6, 0.35), grid(64, 10e-6, 0.05)
    v = grid(256, 7.56e-6, 0.0)
    amp, phase = rng.uniform(0, 1, len(u_far)), rng.uniform(0, 2 * np.pi, len(u_far))
    bucket = holo.size_bucket(len(u_far), len(v))
    h = holo.handle(0)
    h.set_variant("split32", bucket, 13)
    try:
        with holo.Plan(t(u_far), t(v), "split32") as pl:
            assert pl.info()["variant"] == 13
        with holo.Plan(t(u_near), t(v), "split32") as pl:
            info = pl.info()
            y = pl.execute(t(amp), t(phase), -1, LAM).cpu().numpy()
        assert info["variant"] != 13
        assert info["path_error_bound_m"] <= 3.2e-13
        y64 = holo.transform(t(amp), t(phase), t(u_near), t(v), -1, LAM,
                             precision="fp64").cpu().numpy()
        assert rel_l2(y, y64) < 1e-5
    finally:
        h.set_variant("split32", bucket, -1)


def _rot(ax, ay):
    cx, sx, cy, sy = math.cos(ax), math.sin(ax), math.cos(ay), math.sin(ay)
    rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
    ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    return ry @ rx


@pytest.mark.parametrize("case", range(8))
def test_random_geometry_error_within_bound(holo, case):
    """Seeded tilted, wide and close planes.  Per target m the error of the split sum is
    at most the largest term error times sum_n |a_n| / r_nm, and a term's error is at most
    k times the plan's path-length bound (plus the FP32 sin/cos and summation floor,
    taken as 5e-6): max_m |y32 - y64| / sum_n |a_n| / r_nm <= 2 k bound + 5e-6."""
    dev, t = _dev_t()
    rng = np.random.default_rng(100 + case)
    ns_side = int(rng.choice([48, 64, 96, 128]))
    pitch_s = float(rng.choice([10e-6, 20e-6, 40e-6]))  # wide planes: up to 5 mm
    z0 = float(rng.uniform(0.02, 0.5))                 # close planes down to 2 cm
    u = grid(ns_side, pitch_s, 0.0) @ _rot(rng.uniform(-0.5, 0.5), rng.uniform(-0.5, 0.5)).T
    u += np.array([rng.uniform(-2e-3, 2e-3), rng.uniform(-2e-3, 2e-3), z0])
    nt_side = int(rng.choice([128, 192, 256]))
    v = grid(nt_side, 7.56e-6, 0.0) @ _rot(rng.uniform(-0.3, 0.3), 0.0).T
    amp, phase = rng.uniform(0, 1, len(u)), rng.uniform(0, 2 * np.pi, len(u))
    sign = int(rng.choice([-1, 1]))
    with holo.Plan(t(u), t(v), "split32") as pl:
        bound = pl.info()["path_error_bound_m"]
        y = pl.execute(t(amp), t(phase), sign, LAM).cpu().numpy()
    assert math.isfinite(bound)
    idx = np.sort(rng.choice(len(v), 256, replace=False))
    y64 = holo.transform(t(amp), t(phase), t(u), t(v[idx]), sign, LAM,
                         precision="fp64").cpu().numpy()
    r = np.linalg.norm(v[idx, None, :] - u[None, :, :], axis=2)
    scale = (amp[None, :] / r).sum(1)
    k = 2 * math.pi / LAM
    err = np.max(np.abs(y[idx] - y64) / scale)
    assert err <= 2 * k * bound + 5e-6, (case, err, k * bound, z0, pitch_s, ns_side)
    if bound <= 3.2e-13:  # the planner's budget held: the precision target holds too
        assert rel_l2(y[idx], y64) < 1e-5
