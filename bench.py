#!/usr/bin/env python
"""Benchmark of the Huygens superposition hot path on GB300.

Workload (one step): the x -> y -> z chain of a 512x512 source grid (10 um
pitch, z = 0.35 m, Gaussian-blob amplitudes, uniform phases, seed 0) through a
1024x1024 projector (7.56 um, z = 0) back onto the 512x512 grid: two passes of
2.75e11 pair evaluations each, split-FP32 precision, normalised polar outputs.

  value     pair-evals/s with inputs resident in HBM (holo_project on device buffers)
  e2e       the same through the C ABI with page-locked host buffers (copies inside
            the timing)
  roofline  the pair kernel's lane-op rate on its busier pipe (FP32 FMA or XU/MUFU;
            ops per pair from the planned variant's pair model and sin/cos split)
            against that pipe's rate on this GPU measured by holo_probe_peak
  cpu_baseline  the C oracle (FP64, all host threads) on a bounded target sample

``--impl reference`` times the reference's own CPU algorithm for this path --
the oracle port, all host threads -- on the same workload, one bounded target
sample per step.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)
LAM = 632.8e-9
METRIC = "pair-evals/s split-FP32 vs FP64 on 1 GB300 at rel-L2≤1e-5; % FP32/SFU peak"
FLOP_PER_PAIR = 29   # the reference's FLOP_PER_POINT (cuda/macros.h:71-80)


def pipe_ops_per_pair(variant: dict) -> tuple[float, float]:
    """(MUFU ops, FP32-pipe ops) per pair of a split-kernel variant, by pair model:
    0 (curvature correction): 3 MUFU (rsqrt, sin, cos) + 12 FP32; 1 (without it):
    3 + 10; 2 (1/q series, no rsqrt): 2 + 8; 3 (phase from tensor-core MMAs): 2 + 3.
    `fma_sincos_targets` of every `targets_per_thread` take sin/cos from the FMA-pipe
    polynomial instead (-2 MUFU; +16 FP32 for the full-turn form of the CUDA-core loops,
    +13 for the half-turn form of the tensor-core kernel); with warp-specialised sin/cos
    (pair loop 2) a quarter of the warps do."""
    f = variant["fma_sincos_targets"] / variant["targets_per_thread"]
    if variant.get("pair_loop", 0) == 2:
        f = 0.25
    poly = 16.0
    if variant.get("pair_loop", 0) == 3:  # tensor-core phase: `fma_sincos_targets` of 16 pairs
        f = variant["fma_sincos_targets"] / 16.0
        poly = 13.0
    mufu, fp32 = {0: (3.0, 12.0), 1: (3.0, 10.0), 2: (2.0, 8.0),
                  3: (2.0, 3.0)}[variant.get("pair_model", 0)]
    return mufu - 2.0 * f, fp32 + poly * f


WORKLOAD = "chain512: 512^2 sources -> 1024^2 projector -> 512^2 projection (x->y->z)"
# committed ncu summaries whose `key: value` lines the roofline reads
PROF_TRAFFIC = os.path.join(REPO, "profiles", "k_split_traffic_chain512.md")
PROF_MIX = os.path.join(REPO, "profiles", "k_split_tc_mix_chain512_slice.md")
PROF_FP64 = os.path.join(REPO, "profiles", "k_fp64_chain512_slice.md")


def profile_figures(path: str) -> dict:
    """The `key: number` lines of a committed profile summary (empty if absent)."""
    out = {}
    if not os.path.exists(path):
        return out
    for line in open(path):
        key, sep, val = line.partition(":")
        if sep and key.strip() and " " not in key.strip():
            try:
                out[key.strip()] = float(val.split()[0])
            except (ValueError, IndexError):
                pass
    return out


def grid(n, pitch, z):
    c = (np.arange(n) - (n - 1) / 2.0) * pitch
    X, Y = np.meshgrid(c, c, indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), np.full(n * n, z)], axis=1)


def workload(seed=0):
    rng = np.random.default_rng(seed)
    n = 512
    yy, xx = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    img = np.zeros((n, n))
    for _ in range(8):
        cx, cy = rng.uniform(0, n, 2)
        sigma = rng.uniform(5, 40)
        img += rng.uniform(0.2, 1.0) * np.exp(-((xx - cx) ** 2 + (yy - cy) ** 2) / (2 * sigma ** 2))
    amp = (img / img.max()).ravel()
    phase = rng.uniform(0.0, 2 * np.pi, n * n)
    u = grid(512, 10e-6, 0.35)
    v = grid(1024, 7.56e-6, 0.0)
    return amp, phase, u, v, u.copy()


class ClockSampler:
    """nvidia-smi samples during the timed region (clocks and throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.idx)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=10)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        load = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": max(mx), "samples": len(sm),
                "power_w_max": max(power) if power else None, "reasons": sorted(reasons)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def slowest_rank_seconds(local_seconds: float, world: int, device=None) -> float:
    """The whole job's time over `world` replicas: the slowest rank's (MAX all-reduce;
    the process group must be up when world > 1)."""
    if world <= 1:
        return local_seconds
    import torch
    import torch.distributed as dist
    tt = torch.tensor([local_seconds], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt)


def whole_job_rate(units_per_rank: float, world: int, seconds: float) -> float:
    """Units all `world` replicas processed, per second of the slowest rank."""
    return world * units_per_rank / seconds


# The CPU baseline is the repo's C oracle, not the reference's NumPy prototype
# (py/util.py:92-147): the prototype imports numba and pandas and calls an undefined
# global, and the reference sources are not on the GPU host.  Measured in the build
# container (Xeon, 2.7 GHz), the prototype ran 1.35e7 pair-evals/s per core with the
# minimal import shims, the C oracle 3.5e7: the oracle is the faster baseline.
PROTOTYPE_NOTE = ("C-oracle substitute for the reference's NumPy prototype (py/util.py:92-147), "
                  "which ran 1.35e7 pair-evals/s per core where both were measured (the oracle "
                  "3.5e7); the prototype cannot run on the GPU host")


def cpu_baseline(amp, phase, u, v, seconds: float = 12.0) -> dict:
    """The C oracle (FP64, every host thread) on a bounded sample of y-pass targets."""
    import oracle
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(7)
    probe = rng.choice(len(v), threads, replace=False)
    t0 = time.perf_counter()
    oracle.transform_subset(amp, phase, u, v, probe, -1, LAM, threads)
    rate = threads * len(amp) / max(time.perf_counter() - t0, 1e-6)
    n_t = int(max(threads, min(len(v), rate * seconds / len(amp))))
    idx = rng.choice(len(v), n_t, replace=False)
    t0 = time.perf_counter()
    oracle.transform_subset(amp, phase, u, v, idx, -1, LAM, threads)
    dt = time.perf_counter() - t0
    return {"value": n_t * len(amp) / dt, "unit": "pair-evals/s", "cores": threads,
            "kind": "port",
            "sample": f"{n_t} random targets of the y pass x all {len(amp)} sources "
                      f"(FP64 C oracle, {dt:.1f} s)",
            "substitute_for": PROTOTYPE_NOTE}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    oracle.build()
    amp, phase, u, v, w = workload()
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(11)
    # the z pass takes the normalised projector field as its sources; its values
    # do not change the work, so seeded stand-ins keep each step bounded
    y_amp = rng.uniform(0, 1, len(v))
    y_phase = rng.uniform(-np.pi, np.pi, len(v))
    # size each step to about 3 s of CPU work, split between the two passes by pair count
    t0 = time.perf_counter()
    oracle.transform_subset(amp, phase, u, v, np.arange(threads), -1, LAM, threads)
    rate = threads * len(amp) / max(time.perf_counter() - t0, 1e-6)
    pairs_step = max(rate * 3.0, 2.0 * threads * len(v))
    n_y = max(threads, int(pairs_step / 2 / len(amp)))
    n_z = max(threads, int(pairs_step / 2 / len(v)))

    def step(i):
        iy = rng.choice(len(v), n_y, replace=False)
        iz = rng.choice(len(w), n_z, replace=False)
        oracle.transform_subset(amp, phase, u, v, iy, -1, LAM, threads)
        oracle.transform_subset(y_amp, y_phase, v, w, iz, +1, LAM, threads)
        return n_y * len(amp) + n_z * len(v)

    for i in range(args.warmup):
        step(i)
    t0 = time.perf_counter()
    pairs = sum(step(i) for i in range(args.steps))
    dt = time.perf_counter() - t0
    value = pairs / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "pair-evals/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, chain512 shapes)",
        "config": {"workload": WORKLOAD, "sample": f"{n_y} y-pass + {n_z} z-pass targets per step"},
        "cpu_baseline": {"value": value, "unit": "pair-evals/s", "cores": threads, "kind": "port",
                         "sample": f"{n_y} y targets x {len(amp)} sources + {n_z} z targets x "
                                   f"{len(v)} sources per step, FP64 C oracle (restatement of "
                                   "cuda/superposition.cu:35-51); the reference's own host code "
                                   "cannot be built on the GPU host",
                         "substitute_for": PROTOTYPE_NOTE},
        "e2e": {"value": value, "unit": "pair-evals/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_profile_case(args):
    """Two launches of the pair kernel on a slice of the chain512 y pass (512^2 sources
    onto the central 256^2 of the projector); the second is the one to capture."""
    import torch
    import __graft_entry__ as entry
    entry._load_build_module().build()
    holo = entry.load_package()
    amp, phase, u, v, _ = workload()
    side = 1024
    # central 256^2 patch (split32) or 64^2 patch (fp64, ~0.1 s per launch)
    lo, hi = (384, 640) if args.precision == "split32" else (480, 544)
    vv = v.reshape(side, side, 3)[lo:hi, lo:hi].reshape(-1, 3)
    dev = torch.device("cuda", 0)
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a).reshape(-1), device=dev)
    args_ = (t(amp), t(phase), t(u), t(vv))
    if args.variants:  # one forced kernel variant instead of the planner's choice
        var = int(args.variants.split(",")[0])
        for _ in range(2):
            holo.transform(*args_, -1, LAM, precision=args.precision, variant=var)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": {"variant": var},
                          "pairs_per_launch": len(amp) * len(vv)}))
        return
    with holo.Plan(args_[2], args_[3], args.precision) as pl:
        for _ in range(2):
            pl.execute(args_[0], args_[1], -1, LAM)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": pl.info(), "pairs_per_launch": len(amp) * len(vv)}))


def mc_expected_rel_l2(amp, u, v, y, sub, n_sample=256, seed=7):
    """Expected rel-L2 of stratified sampling (one source drawn per stratum of `sub`,
    weight `sub`) for sources with independent uniform phases: the error variance per
    target is (sub - 1) sum_n |a_n / r_n|^2, so rel-L2 ~ sqrt((sub - 1) sum_mn
    |a_n / r_mn|^2) / |y|; sum_mn taken from `n_sample` random targets."""
    idx = np.random.default_rng(seed).choice(len(v), size=min(n_sample, len(v)), replace=False)
    d2 = ((v[idx, None, :] - u[None, :, :]) ** 2).sum(-1)
    power = float((amp[None, :] ** 2 / d2).sum()) * len(v) / len(idx)
    return float(np.sqrt((sub - 1) * power) / np.linalg.norm(y))


def _events_ms(fn, reps=1):
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        out = fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps, out


def _t(dev):
    import torch
    return lambda a: torch.as_tensor(np.ascontiguousarray(a).reshape(-1), device=dev)


def chain64_inputs(seed=0):
    """64^2 sources (10 um, z = 0.35 m) -> 256^2 projector (7.56 um, z = 0) -> the 64^2
    grid again; amplitudes U[0,1), phases U[0, 2 pi)."""
    rng = np.random.default_rng(seed)
    u = grid(64, 10e-6, 0.35)
    v = grid(256, 7.56e-6, 0.0)
    amp = rng.uniform(0, 1, len(u))
    phase = rng.uniform(0, 2 * np.pi, len(u))
    return amp, phase, u, v, u.copy()


def cpu_chain64(threads=None):
    """The CPU leg for the 64^2 -> 256^2 -> 64^2 chain: the FP64 C oracle (all host
    threads) runs the whole chain, normalisation included; its timing is the chain's
    CPU baseline and its fields the reference the GPU chains are compared with."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    oracle.build()
    threads = threads or os.cpu_count() or 1
    amp, phase, u, v, w = chain64_inputs()
    t0 = time.perf_counter()
    y = oracle.transform(amp, phase, u, v, -1, LAM, threads)
    yn, _ = oracle.normalize_amp(y)
    ya, yp = oracle.to_polar(yn)
    z = oracle.transform(ya, yp, v, w, +1, LAM, threads)
    zn, _ = oracle.normalize_amp(z)
    dt = time.perf_counter() - t0
    pairs = len(amp) * len(v) + len(v) * len(w)
    return {"seconds": dt, "pair_evals_per_s": pairs / dt, "cores": threads, "kind": "port",
            "what": "FP64 C oracle (restatement of cuda/superposition.cu:35-51), whole chain"}, \
        yn, zn


def wl_chain64(holo, dev, reps=5, cpu=None):
    """Both precisions through the one-shot x -> y -> z call (planning included), and
    the normalised fields against the oracle chain when `cpu` = cpu_chain64() is given."""
    t = _t(dev)
    amp, phase, u, v, w = chain64_inputs()
    d = [t(a) for a in (amp, phase, u, v, w)]
    pairs = len(u) * len(v) + len(v) * len(w)
    out = {"pairs_per_chain": pairs,
           "config": "64^2 sources -> 256^2 projector -> 64^2 projection, lambda 632.8 nm"}
    for prec in ("fp64", "split32"):
        holo.project(*d, LAM, precision=prec)
        ms, r = _events_ms(lambda: holo.project(*d, LAM, precision=prec), reps=reps)
        ya, yp, za, zp = (x.cpu().numpy() for x in r)
        row = {"ms_per_chain": ms, "pair_evals_per_s": pairs / (ms * 1e-3)}
        if cpu is not None:
            _, yo, zo = cpu
            yg, zg = ya * np.exp(1j * yp), za * np.exp(1j * zp)
            row.update({"y_rel_l2_vs_oracle": float(np.linalg.norm(yg - yo) / np.linalg.norm(yo)),
                        "z_rel_l2_vs_oracle": float(np.linalg.norm(zg - zo) / np.linalg.norm(zo)),
                        "y_max_phase_err_rad": float(np.max(np.abs(np.angle(yg / yo)))),
                        "z_max_phase_err_rad": float(np.max(np.abs(np.angle(zg / zo))))})
        out[prec] = row
    if cpu is not None:
        out["cpu_oracle"] = cpu[0]
        out["split32_over_cpu"] = out["split32"]["pair_evals_per_s"] / cpu[0]["pair_evals_per_s"]
    return out


def wl_mc16(holo, dev, reps=3):
    """x -> y of the 64^2 -> 256^2 chain with 1/16 of the sources per block of 256
    targets, against the FP64 brute force on the same targets."""
    t = _t(dev)
    amp, phase, u, v, _ = chain64_inputs()
    d = [t(a) for a in (amp, phase, u, v)]
    y64 = holo.transform(*d, -1, LAM, precision="fp64").cpu().numpy()
    holo.transform_mc(*d, -1, LAM, seed=1, subsample=16, targets_per_block=256)
    ms, ymc = _events_ms(lambda: holo.transform_mc(*d, -1, LAM, seed=2, subsample=16,
                                                   targets_per_block=256), reps=reps)
    ymc = ymc.cpu().numpy()
    ms_bf, _ = _events_ms(lambda: holo.transform(*d, -1, LAM, precision="split32"), reps=reps)
    return {"mc_ms": ms, "brute_force_split32_ms": ms_bf,
            "sampled_pair_evals_per_s": len(u) // 16 * len(v) / (ms * 1e-3),
            "effective_pair_evals_per_s": len(u) * len(v) / (ms * 1e-3),
            "mc_rel_l2_vs_fp64": float(np.linalg.norm(ymc - y64) / np.linalg.norm(y64)),
            "mc_expected_rel_l2": mc_expected_rel_l2(amp, u, v, y64, 16),
            "config": "x->y pass of the 64^2 -> 256^2 chain, 1/16 of the sources per block of "
                      "256 targets, Philox-seeded, weight 16"}


def batch64_problems(dev, seed=0):
    """64 problems: N log-uniform in [1024, 262144] on square-ish 10 um grids at z0
    U[0.2, 0.5] m, projectors of 128^2 .. 1024^2 at 7.56 um, amplitudes U[0,1), phases
    U[0, 2 pi)."""
    import torch
    t = _t(dev)
    rng = np.random.default_rng(seed)
    host, pairs = [], 0
    for i in range(64):
        ns = int(np.exp(rng.uniform(np.log(1024), np.log(262144))))
        side = int(np.ceil(np.sqrt(ns)))
        u = grid(side, 10e-6, rng.uniform(0.2, 0.5))[:ns]
        v = grid(int(rng.choice([128, 256, 512, 1024])), 7.56e-6, 0.0)
        amp, phase = rng.uniform(0, 1, ns), rng.uniform(0, 2 * np.pi, ns)
        host.append((amp, phase, u, v))
        pairs += ns * len(v)
    probs = [(t(a), t(p), t(u), t(v), torch.zeros(2 * len(v), dtype=torch.float64, device=dev))
             for a, p, u, v in host]
    return host, probs, pairs


def wl_batch64(holo, dev, reps=3, check_targets=512):
    """The 64 problems as one batched persistent launch (CUDA graph replay) against
    launching each problem's planned transform alone; the batch's fields against the
    FP64 kernel at `check_targets` random targets of every problem."""
    import torch
    host, probs, pairs = batch64_problems(dev)
    P = [holo.Problem(a, p, u, v, -1, LAM, y) for a, p, u, v, y in probs]
    with holo.Batch(P, "split32") as b:
        b.execute()
        ms_b, _ = _events_ms(b.execute, reps=reps)
    plans = [holo.Plan(p.u, p.v, "split32") for p in P]
    for pl, p in zip(plans, P):
        pl.execute(p.amp, p.phase, -1, LAM)
    ms_s, _ = _events_ms(lambda: [pl.execute(p.amp, p.phase, -1, LAM)
                                  for pl, p in zip(plans, P)], reps=max(1, reps - 1))
    variants = sorted({pl.info()["variant"] for pl in plans})
    for pl in plans:
        pl.close()
    rng = np.random.default_rng(3)
    errs, phase_errs = [], []
    for (amp, phase, u, v), (_, _, _, _, y) in zip(host, probs):
        idx = np.sort(rng.choice(len(v), min(check_targets, len(v)), replace=False))
        yb = y.cpu().numpy().view(np.complex128)[idx]
        y64 = holo.transform(*(_t(dev)(a) for a in (amp, phase, u, v[idx])), -1, LAM,
                             precision="fp64").cpu().numpy()
        errs.append(float(np.linalg.norm(yb - y64) / np.linalg.norm(y64)))
        phase_errs.append(float(np.max(np.abs(np.angle(yb / y64)))))
    torch.cuda.synchronize()
    return {"problems": 64, "pairs": pairs, "batched_ms": ms_b, "sequential_ms": ms_s,
            "batched_pair_evals_per_s": pairs / (ms_b * 1e-3),
            "sequential_pair_evals_per_s": pairs / (ms_s * 1e-3),
            "speedup_batched_over_sequential": ms_s / ms_b,
            "split_vs_fp64_rel_l2_worst": max(errs),
            "split_vs_fp64_rel_l2_median": float(np.median(errs)),
            "split_vs_fp64_max_phase_err_rad": max(phase_errs),
            "check": f"{check_targets} random targets per problem, FP64 kernel",
            "planned_variants_one_by_one": variants,
            "config": "N log-uniform [1024, 262144], M in {128^2..1024^2}, z0 U[0.2,0.5] m"}


def adam1024_inputs(dev, seed=0):
    """1024^2 projector pixels (7.56 um, z = 0), 512^2 target grid (10 um, z = 0.35 m),
    target intensity: 8 Gaussian blobs normalised to unit mean."""
    t = _t(dev)
    rng = np.random.default_rng(seed)
    pp = t(grid(1024, 7.56e-6, 0.0)).reshape(-1, 3)
    tp = t(grid(512, 10e-6, 0.35)).reshape(-1, 3)
    n = 512
    yy, xx = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    img = np.zeros((n, n))
    for _ in range(8):
        cx, cy = rng.uniform(0, n, 2)
        img += rng.uniform(0.2, 1) * np.exp(-((xx - cx) ** 2 + (yy - cy) ** 2) /
                                             (2 * rng.uniform(5, 40) ** 2))
    return pp, tp, t((img / img.mean()).ravel())


def wl_adam1024(holo, dev, steps=100, warmup=3, reps=3):
    """100 Adam steps (lr 0.05) of 1024^2 projector phases onto a 512^2 target intensity
    (forward y -> z + hand-written adjoint per step), then forward, adjoint and the Adam
    update timed apart with CUDA events."""
    import torch
    from holo_gb300 import torch_ops
    pp, tp, target = adam1024_inputs(dev)
    # untimed warm-up run: first calls into the autograd engine, Adam and the kernels
    torch_ops.optimise_phase_hologram(pp, tp, target, LAM, steps=warmup, lr=0.05)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _, losses = torch_ops.optimise_phase_hologram(pp, tp, target, LAM, steps=steps, lr=0.05)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    n, m = pp.shape[0], tp.shape[0]
    g = torch.Generator(device="cpu").manual_seed(1)
    amp = torch.ones(n, dtype=torch.float64, device=dev)
    phase = (torch.rand(n, generator=g, dtype=torch.float64) * 2 * np.pi).to(dev)
    grad_y = torch.randn(2 * m, generator=g, dtype=torch.float64).to(dev)
    with holo.Plan(pp.reshape(-1), tp.reshape(-1), "split32") as pl:
        pl.execute(amp, phase, +1, LAM)
        pl.adjoint(amp, phase, grad_y, +1, LAM)
        fwd_ms, _ = _events_ms(lambda: pl.execute(amp, phase, +1, LAM), reps=reps)
        adj_ms, _ = _events_ms(lambda: pl.adjoint(amp, phase, grad_y, +1, LAM), reps=reps)
    p32 = phase.float().clone().requires_grad_(True)
    opt = torch.optim.Adam([p32], lr=0.05)
    p32.grad = torch.randn(n, generator=g).to(dev)
    opt.step()
    adam_ms, _ = _events_ms(opt.step, reps=10)
    return {"adam_steps": steps, "seconds": dt, "s_per_step": dt / steps,
            "pair_evals_per_s": 2 * n * m * steps / dt,
            "loss_first": losses[0], "loss_last": losses[-1],
            "forward_ms": fwd_ms, "adjoint_ms": adj_ms, "adam_update_ms": adam_ms,
            "adjoint_over_forward": adj_ms / fwd_ms,
            "config": "1024^2 phases -> 512^2 target intensity, forward + adjoint per step"}


def run_other_workload(args):
    """The chain64, mc16, batch64 and adam1024 workloads alone: one JSON line each (the
    default run carries them in the headline line's extra.workloads)."""
    import torch
    import __graft_entry__ as entry
    entry._load_build_module().build()
    holo = entry.load_package()
    dev = torch.device("cuda", 0)
    out = {"workload": args.workload, "data": "synthetic (seeded)"}
    if args.workload == "chain64":
        out.update(wl_chain64(holo, dev, cpu=cpu_chain64()))
    elif args.workload == "mc16":
        out.update(wl_mc16(holo, dev))
    elif args.workload == "batch64":
        out.update(wl_batch64(holo, dev))
    else:
        out.update(wl_adam1024(holo, dev, steps=args.adam_steps))
    print(json.dumps(out), flush=True)


def run_sweep(args):
    """One JSON line per split-FP32 variant: pair kernel rate on the chain512 y pass
    (512^2 -> 1024^2)."""
    import torch
    import __graft_entry__ as entry
    entry._load_build_module().build()
    holo = entry.load_package()
    amp, phase, u, v, _ = workload()
    dev = torch.device("cuda", 0)
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a).reshape(-1), device=dev)
    d = [t(a) for a in (amp, phase, u, v)]
    h = holo.handle(0)
    ref = None
    only = {int(x) for x in args.variants.split(",")} if args.variants else None
    for var in holo.variants("split32"):
        if only is not None and var["variant"] not in only:
            continue
        try:
            holo.transform(*d, -1, LAM, precision="split32", variant=var["variant"])
            torch.cuda.synchronize()
            h.profile_begin()
            for _ in range(2):
                y = holo.transform(*d, -1, LAM, precision="split32", variant=var["variant"])
            ms, n = h.profile_end()
        except holo.HoloError as e:
            print(json.dumps({"variant": var, "error": str(e)}), flush=True)
            continue
        yv = y.cpu().numpy()
        if ref is None:
            ref = yv
        rate = 2 * len(amp) * len(v) / (ms * 1e-3)
        print(json.dumps({"variant": var, "kernel_pairs_per_s": rate, "ms": ms / n,
                          "rel_l2_vs_first": float(np.linalg.norm(yv - ref) /
                                                   np.linalg.norm(ref))}),
              flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="split32", choices=["split32", "fp64"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extra-workloads", action="store_true",
                    help="skip the chain64, mc16, batch64 and adam1024 measurements that the "
                         "default run adds to its line (extra.workloads)")
    ap.add_argument("--adam-steps", type=int, default=100,
                    help="Adam steps of the adam1024 workload (default 100)")
    ap.add_argument("--profile-case", action="store_true",
                    help="small case for ncu: two split-FP32 passes of the 512^2 sources onto "
                         "a 256^2 patch of the projector (1.7e10 pairs each), then exit")
    ap.add_argument("--variants", default="",
                    help="comma-separated variant numbers to restrict --sweep-variants to "
                         "(--profile-case: the first one is forced)")
    ap.add_argument("--sweep-variants", action="store_true",
                    help="time every split-FP32 kernel variant on the chain512 y pass, then exit")
    ap.add_argument("--workload", default="chain512",
                    choices=["chain512", "chain64", "mc16", "batch64", "adam1024"],
                    help="chain512 (default) is the headline line; the others print their own "
                         "JSON line: chain64 the 64^2 -> 256^2 -> 64^2 chain in FP64 and "
                         "split-FP32, mc16 its x -> y pass with 1/16 of the sources (Monte "
                         "Carlo), batch64 64 uneven problems batched against one by one, "
                         "adam1024 100 Adam steps of a 1024^2 phase hologram onto 512^2")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.profile_case:
        return run_profile_case(args)
    if args.sweep_variants:
        return run_sweep(args)
    if args.workload != "chain512":
        return run_other_workload(args)

    import torch
    import torch.distributed as dist
    import __graft_entry__ as entry

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    entry._load_build_module().build()
    holo = entry.load_package()
    from holo_gb300 import api

    dev = torch.device("cuda", local)
    amp, phase, u, v, w = workload()
    N, M, P = len(amp), len(v), len(w)
    pairs_step = N * M + M * P
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a).reshape(-1), device=dev)
    d_amp, d_phase, d_u, d_v, d_w = (t(a) for a in (amp, phase, u, v, w))
    h = holo.handle(local)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > 129 MB L2

    def step():
        return holo.project(d_amp, d_phase, d_u, d_v, d_w, LAM, precision=args.precision)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(max(args.warmup, 3)):
        step()
    barrier()
    gpu_idx = os.environ.get("CUDA_VISIBLE_DEVICES", str(local)).split(",")[local] \
        if os.environ.get("CUDA_VISIBLE_DEVICES") else str(local)
    clocks = ClockSampler(gpu_idx)
    clocks.start()
    launches0 = api.kernel_launches()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    barrier()
    h.profile_begin()
    wall0 = time.perf_counter()
    for i in range(args.steps):
        flush.fill_(float(i))  # L2 flush between timed steps, outside the events
        ev[i][0].record()
        step()
        ev[i][1].record()
    barrier()
    wall = time.perf_counter() - wall0
    kern_ms, kern_launches = h.profile_end()
    launches = api.kernel_launches() - launches0
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_s = slowest_rank_seconds(sum(step_ms) * 1e-3, world, dev)
    value = whole_job_rate(pairs_step * args.steps, world, total_s)

    # e2e: the C ABI with page-locked host buffers, copies inside the timing (the outputs
    # are page-locked too: the API allocates them like the inputs)
    e2e_steps = max(3, args.steps)
    host = [torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64).reshape(-1)).pin_memory()
            for a in (amp, phase, u, v, w)]
    holo.project(*host, LAM, precision=args.precision)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        holo.project(*host, LAM, precision=args.precision)
    barrier()
    e2e_s = slowest_rank_seconds((time.perf_counter() - t0) / e2e_steps, world, dev)
    h2d = 8 * (2 * N + 3 * N + 3 * M + 3 * P)
    d2h = 8 * (2 * M + 2 * P)

    # roofline of the pair kernel: FP32 and MUFU (XU pipe) issue rates against measured peaks
    kern_pairs_s = pairs_step * args.steps / (kern_ms * 1e-3) if kern_ms > 0 else 0.0
    mufu_peak = h.probe_peak(0)
    ffma_peak = h.probe_peak(1)
    with holo.Plan(d_u, d_v, args.precision) as pl:
        info = pl.info()
    var = next(x for x in holo.variants(args.precision) if x["variant"] == info["variant"]) \
        if args.precision == "split32" else None
    MUFU_PER_PAIR, FP32_PER_PAIR = pipe_ops_per_pair(var) if var else (0.0, 0.0)
    ops_source = "pair model of the planned variant"
    # lane-ops per pair counted by ncu on the same variant (XU instructions x 32, FMA-pipe
    # instructions x 32 with packed f32x2 ones counted twice, per pair evaluated)
    mix = profile_figures(PROF_MIX)
    if var and mix.get("variant") == var["variant"] and "xu_lane_ops_per_pair" in mix:
        MUFU_PER_PAIR = mix["xu_lane_ops_per_pair"]
        FP32_PER_PAIR = mix["fma_lane_ops_per_pair"]
        ops_source = "ncu instruction counts (profiles/k_split_tc_mix_chain512_slice.md)"
    achieved = kern_pairs_s * MUFU_PER_PAIR
    # DRAM bytes per pair-kernel launch (the y pass) from the committed ncu capture
    traffic = None
    if args.precision == "split32":
        traffic = profile_figures(PROF_TRAFFIC).get("bytes_per_launch_y_pass")
        traffic = int(traffic) if traffic else None
    # the pair rate this variant could reach if its busiest pipe ran at the measured peak
    bound_rate = min(mufu_peak / MUFU_PER_PAIR if MUFU_PER_PAIR else float("inf"),
                     ffma_peak / FP32_PER_PAIR if FP32_PER_PAIR else float("inf")) if var else None
    # the bound named is the busier of the two pipes (FP32 FMA pipe, XU/MUFU pipe)
    fp32_ops = kern_pairs_s * FP32_PER_PAIR
    xu_frac = achieved / mufu_peak if mufu_peak else 0.0
    fp32_frac = fp32_ops / ffma_peak if ffma_peak else 0.0
    busy_fp32 = fp32_frac > xu_frac
    roofline = {"bound": "fp32" if busy_fp32 else "xu",
                "achieved": (fp32_ops if busy_fp32 else achieved) / 1e9,
                "peak": (ffma_peak if busy_fp32 else mufu_peak) / 1e9,
                "unit": "Gop/s", "frac": fp32_frac if busy_fp32 else xu_frac,
                "traffic": traffic,
                "note": "compute-bound on the FP32 (FMA) and XU (MUFU) pipes: the busier pipe's "
                        "lane-ops of the pair kernel per second vs that pipe's rate measured by "
                        "holo_probe_peak (FFMA / sin.approx throughput kernels); neither HBM nor "
                        "tensor cores bound this path",
                "xu_frac": xu_frac, "xu_achieved_gops": achieved / 1e9,
                "xu_peak_gops": mufu_peak / 1e9,
                "variant": var, "mufu_per_pair": MUFU_PER_PAIR, "fp32_per_pair": FP32_PER_PAIR,
                "ops_per_pair_source": ops_source,
                "fp32_frac": fp32_frac,
                "fma_peak_gops": ffma_peak / 1e9,
                "pairs_per_s_frac_of_pipe_bound": kern_pairs_s / bound_rate if bound_rate else None,
                "kernel_pairs_per_s": kern_pairs_s,
                "kernel_ms_per_launch": kern_ms / max(kern_launches, 1),
                "kernel_launches": kern_launches}
    # the same kernel against the measured copy bandwidth and bf16 GEMM rate: it
    # moves ~1e-4 bytes per pair and runs 4 TF32 MMAs of K = 8 per pair (64 FLOP; TF32
    # issues at half the bf16 rate), far from both
    peaks_path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path) and kern_launches and var and var.get("pair_loop") == 3:
        peaks = json.load(open(peaks_path))
        launch_s = kern_ms * 1e-3 / kern_launches
        tc_tflops = 64.0 * kern_pairs_s / 1e12
        roofline["measured_peaks"] = {
            "source": "MEASURED_PEAKS.json (copy bandwidth; cuBLAS bf16 burst)",
            "hbm_gbs": peaks.get("hbm_gbs"),
            "dram_gbs": traffic / launch_s / 1e9 if traffic else None,
            "hbm_frac": traffic / launch_s / 1e9 / peaks["hbm_gbs"]
            if traffic and peaks.get("hbm_gbs") else None,
            "bf16_tflops": peaks.get("bf16_tflops"),
            "tf32_mma_tflops": tc_tflops,
            "tensor_frac_of_bf16": tc_tflops / peaks["bf16_tflops"]
            if peaks.get("bf16_tflops") else None}

    # split-FP32 vs the plain FP64 kernel on a bounded target subset; the split result
    # is the full y pass (the timed tiling and variant) read at those targets
    rng = np.random.default_rng(1)
    idx = np.sort(rng.choice(M, 8192, replace=False))
    d_vs = t(v[idx])
    holo.transform(d_amp, d_phase, d_u, d_vs, -1, LAM, precision="fp64")
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    y64 = holo.transform(d_amp, d_phase, d_u, d_vs, -1, LAM, precision="fp64")
    e1.record()
    barrier()
    fp64_rate = N * len(idx) / (e0.elapsed_time(e1) * 1e-3)
    with holo.Plan(d_u, d_v, args.precision) as pl:
        y32 = pl.execute(d_amp, d_phase, -1, LAM)[torch.as_tensor(idx, device=dev)]
        acc_variant = pl.info()["variant"]
    torch.cuda.synchronize()
    a32, a64 = y32.cpu().numpy(), y64.cpu().numpy()
    rel = float(np.linalg.norm(a32 - a64) / np.linalg.norm(a64))
    phase_err = float(np.max(np.abs(np.angle(a32 / a64))))
    h.status()
    # roofline of the FP64 kernel: its FP64-pipe lane-ops per pair (ncu count on a slice of
    # the same y pass) at the measured pair rate, against the DFMA probe's rate
    dfma_peak = h.probe_peak(3)
    f64 = profile_figures(PROF_FP64)
    fp64_roofline = {"bound": "fp64", "pair_evals_per_s": fp64_rate, "peak_gops": dfma_peak / 1e9,
                     "unit": "Gop/s", "peak_source": "holo_probe_peak kind 3 (DFMA chains)"}
    if "fp64_pipe_slots_per_pair" in f64:
        # pipe slots: the DFMA/DADD/DMUL arithmetic plus the pipe's other FP64 instructions
        ops = f64["fp64_pipe_slots_per_pair"]
        fp64_roofline.update({"fp64_pipe_slots_per_pair": ops,
                              "fp64_arith_per_pair": f64.get("fp64_lane_ops_per_pair"),
                              "achieved_gops": fp64_rate * ops / 1e9,
                              "frac": fp64_rate * ops / dfma_peak if dfma_peak else None,
                              "ops_per_pair_source": "ncu counters on a slice of the same pass "
                                                     "(profiles/k_fp64_chain512_slice.md)"})

    if rank != 0:
        return
    cpu = cpu64 = None
    if not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        cpu = cpu_baseline(amp, phase, u, v)
        if world == 1 and not args.no_extra_workloads:
            cpu64 = cpu_chain64()
    # the other workloads, measured after the headline (N = 1 only)
    extra = None
    if world == 1 and not args.no_extra_workloads:
        t_extra = time.perf_counter()
        extra = {"workloads": {
            "chain64": wl_chain64(holo, dev, cpu=cpu64),
            "mc16": wl_mc16(holo, dev),
            "batch64": wl_batch64(holo, dev),
            "adam1024": wl_adam1024(holo, dev, steps=args.adam_steps)}}
        extra["seconds"] = time.perf_counter() - t_extra
        h.status()
    line = {
        "metric": METRIC, "value": value, "unit": "pair-evals/s", "n_gpus": world,
        "steps": args.steps, "warmup": max(args.warmup, 3),
        "ms_per_step": 1e3 * total_s / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if args.precision == "split32" else "f64",
        "data": "synthetic (seeded; chain512 shapes and value distributions)",
        "config": {"workload": WORKLOAD, "precision": args.precision, "lambda_m": LAM,
                   "pairs_per_step": pairs_step, "l2": "flushed between timed steps (256 MB write)",
                   "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": {"value": whole_job_rate(pairs_step, world, e2e_s), "unit": "pair-evals/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": 1e3 * e2e_s, "steps": e2e_steps,
                "timing": "wall clock around the steps, host copies and a final synchronize "
                          "included"},
        "gpu_launches": launches,
        "clocks": clk,
        "fp64_kernel_pairs_per_s": fp64_rate,
        "fp64_roofline": fp64_roofline,
        "fp64_frac": fp64_roofline.get("frac"),
        "split_over_fp64": kern_pairs_s / fp64_rate if fp64_rate else None,
        "rel_l2_split_vs_fp64": rel, "max_phase_err_rad": phase_err,
        "accuracy_check": {"targets": len(idx), "variant": acc_variant,
                           "precision": args.precision},
        "flops_29_per_pair": value * FLOP_PER_PAIR,
        "wall_s_timed": wall,
        "published_reference_pairs_per_s": {"value": 5.3e10, "what": "reference kernel #2, "
                                            "FP64, Quadro GV100, N=1920x1080 (README figure)"},
        "extra": extra,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
