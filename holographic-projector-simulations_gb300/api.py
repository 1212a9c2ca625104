"""Python host API over the C ABI (include/holo.h).

Arrays may be NumPy arrays or PyTorch tensors.  CUDA tensors run
asynchronously on the current torch stream of their device; NumPy arrays and
CPU tensors go through the library's host-pointer path (copy in, compute on
the GPU, copy out).  Results come back in the kind of container that came in.

Names mirror the reference's interface for this path:
  transform_full  cuda/transform.cu:147-340  raw complex sum, one direction
  time_transform  cuda/transform.cu:346-406  timed, normalised, polar output
  phasor_displacement / map_sum_kernel / projector_setup
                  py/util.py:92-175 (the NumPy prototype's names and signs)
"""
from __future__ import annotations

import ctypes
import json
import os
import threading
import time
from dataclasses import dataclass

import numpy as np

from . import _native as N

try:  # torch is optional for the NumPy path
    import torch
except ImportError:  # pragma: no cover
    torch = None

PRECISIONS = {"fp64": N.FP64, "split32": N.SPLIT32, N.FP64: N.FP64, N.SPLIT32: N.SPLIT32}
DIRECTIONS = {"Forwards": N.FORWARDS, "Backwards": N.BACKWARDS, "forwards": N.FORWARDS,
              "backwards": N.BACKWARDS, 1: N.FORWARDS, -1: N.BACKWARDS}
DEFAULT_LAMBDA = 0.65e-6  # the reference's LAMBDA default (cuda/macros.h:23-25)


def _precision(p) -> int:
    try:
        return PRECISIONS[p]
    except KeyError:
        raise ValueError(f"precision must be 'fp64' or 'split32', got {p!r}") from None


def _sign(d) -> int:
    try:
        return DIRECTIONS[d]
    except KeyError:
        raise ValueError(f"direction must be +1/-1 or 'Forwards'/'Backwards', got {d!r}") from None


# ---- buffers ------------------------------------------------------------------------
def _is_tensor(x) -> bool:
    return torch is not None and isinstance(x, torch.Tensor)


class _Buf:
    """A contiguous float64 view of an input, with its pointer and placement."""

    def __init__(self, x, count: int | None = None, name: str = "array"):
        if _is_tensor(x):
            t = x.detach()
            if t.is_complex():
                t = torch.view_as_real(t)
            t = t.to(torch.float64).contiguous()
            self.obj, self.ptr, self.device = t, t.data_ptr(), t.is_cuda
            self.dev_index = t.device.index if t.is_cuda else None
            self.n = t.numel()
        else:
            a = np.asarray(x)
            if np.iscomplexobj(a):
                a = np.ascontiguousarray(a, np.complex128).view(np.float64)
            a = np.ascontiguousarray(a, dtype=np.float64)
            self.obj, self.ptr, self.device, self.dev_index = a, a.ctypes.data, False, None
            self.n = a.size
        if count is not None and self.n != count:
            raise ValueError(f"{name}: expected {count} values, got {self.n}")


def _is_pinned(t) -> bool:
    try:
        return bool(t.is_pinned())
    except RuntimeError:  # no accelerator to ask
        return False


def _empty_like(ref: _Buf, count: int):
    if ref.device:
        t = torch.empty(count, dtype=torch.float64, device=f"cuda:{ref.dev_index}")
        return t, t.data_ptr()
    if _is_tensor(ref.obj):
        # page-locked inputs get page-locked outputs: the library's device-to-host copies
        # then run at the link's rate instead of through the driver's staging buffer
        t = torch.empty(count, dtype=torch.float64, pin_memory=_is_pinned(ref.obj))
        return t, t.data_ptr()
    a = np.empty(count, dtype=np.float64)
    return a, a.ctypes.data


def _stream(ref: _Buf):
    if ref.device:
        return ctypes.c_void_p(torch.cuda.current_stream(ref.dev_index).cuda_stream)
    return None


def _as_complex(buf):
    if _is_tensor(buf):
        return torch.view_as_complex(buf.view(-1, 2))
    return buf.view(np.complex128)


# ---- handle -------------------------------------------------------------------------
class Handle:
    """One libholo handle (device memory pool, variant table) per device."""

    def __init__(self, device: int = 0):
        self.lib = N.load()
        h = ctypes.c_void_p()
        N.check(self.lib.holo_create(device, ctypes.byref(h)))
        self.h = h
        self.device = device

    def close(self) -> None:
        if self.h:
            self.lib.holo_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):  # pragma: no cover - interpreter shutdown order varies
        try:
            self.close()
        except Exception:
            pass

    def status(self, stream=None) -> None:
        N.check(self.lib.holo_device_status(self.h, stream))

    # variants / autotuner
    def set_variant(self, precision, bucket: int, variant: int) -> None:
        N.check(self.lib.holo_set_variant(self.h, _precision(precision), bucket, variant))

    def get_variant(self, precision, bucket: int) -> int:
        v = ctypes.c_int()
        N.check(self.lib.holo_get_variant(self.h, _precision(precision), bucket, ctypes.byref(v)))
        return v.value

    def autotune(self, n: int, m: int, precision="split32", repeats: int = 3):
        v, r = ctypes.c_int(), ctypes.c_double()
        N.check(self.lib.holo_autotune(self.h, _precision(precision), n, m, repeats, None,
                                       ctypes.byref(v), ctypes.byref(r)))
        return v.value, r.value

    # measurement
    def profile_begin(self) -> None:
        N.check(self.lib.holo_profile_begin(self.h))

    def profile_end(self) -> tuple[float, int]:
        """(total ms, launches) of the pair-evaluation kernels since profile_begin."""
        ms, n = ctypes.c_double(), ctypes.c_int()
        N.check(self.lib.holo_profile_end(self.h, ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def probe_peak(self, kind: int) -> float:
        """Measured lane-instructions/s of the MUFU (kind 0), FP32 FMA (kind 1) or packed
        FP32-pair FMA (kind 2, two FMAs each) pipe."""
        r = ctypes.c_double()
        N.check(self.lib.holo_probe_peak(self.h, kind, ctypes.byref(r)))
        return r.value


def kernel_launches() -> int:
    n = ctypes.c_longlong()
    N.check(N.load().holo_kernel_launches(ctypes.byref(n)))
    return n.value


_handles: dict[int, Handle] = {}
_hlock = threading.Lock()


def handle(device: int = 0) -> Handle:
    with _hlock:
        if device not in _handles:
            _handles[device] = Handle(device)
            load_tuning(_handles[device])
        return _handles[device]


def _device_of(*bufs: _Buf) -> int:
    for b in bufs:
        if b.device:
            return b.dev_index or 0
    return 0


# ---- one-shot transforms ------------------------------------------------------------
_TILINGS = {N.TILE_HILBERT: "hilbert", N.TILE_PACKED: "packed", -1: "none"}


def tile_order(points, tiling: str = "hilbert") -> np.ndarray:
    """Tile order of a point set (xyz triples, NumPy or torch): order[i] = input index
    of the i-th point in tile order, by the Hilbert or the packed tiling."""
    codes = {v: k for k, v in _TILINGS.items() if k >= 0}
    if tiling not in codes:
        raise ValueError(f"tiling must be one of {sorted(codes)}")
    b = _Buf(points, name="points")
    if b.n % 3:
        raise ValueError("points must hold xyz triples")
    n = b.n // 3
    h = handle(_device_of(b))
    out = np.zeros(max(n, 1), np.int32)
    N.check(h.lib.holo_tile_order(h.h, b.ptr, n, codes[tiling], out.ctypes.data, _stream(b)))
    return out[:n]


def transform(amp, phase, u, v, sign: int, lam: float = DEFAULT_LAMBDA, precision="split32",
              variant: int | None = None, flags: int = 0):
    """y_m = sum_n a_n exp(i(phi_n + sign k r_nm)) / r_nm for every target (complex)."""
    a = _Buf(amp, name="amp")
    n = a.n
    p = _Buf(phase, n, "phase")
    uu = _Buf(u, 3 * n, "u")
    vv = _Buf(v, name="v")
    if vv.n % 3:
        raise ValueError("v must hold xyz triples")
    m = vv.n // 3
    h = handle(_device_of(a, p, uu, vv))
    out, optr = _empty_like(a if a.device else vv, 2 * m)
    s = _stream(a if a.device else vv)
    if variant is None and flags == 0:
        rc = h.lib.holo_transform(h.h, _sign(sign), lam, a.ptr, p.ptr, uu.ptr, n, vv.ptr, m, optr,
                                  _precision(precision), s)
        N.check(rc)
    elif flags:
        with Plan(u, v, precision, device=h.device) as pl:
            return pl.execute(amp, phase, sign, lam, flags=flags)
    else:
        N.check(h.lib.holo_transform_variant(h.h, _sign(sign), lam, a.ptr, p.ptr, uu.ptr, n,
                                             vv.ptr, m, optr, _precision(precision), variant, s))
    return _as_complex(out)


def transform_mc(amp, phase, u, v, sign: int, lam: float = DEFAULT_LAMBDA, seed: int = 0,
                 subsample: int = 16, targets_per_block: int = 256):
    """Monte Carlo estimate: every block of targets sums 1/subsample of the sources."""
    a = _Buf(amp, name="amp")
    n = a.n
    p = _Buf(phase, n, "phase")
    uu = _Buf(u, 3 * n, "u")
    vv = _Buf(v, name="v")
    m = vv.n // 3
    h = handle(_device_of(a, p, uu, vv))
    out, optr = _empty_like(a if a.device else vv, 2 * m)
    N.check(h.lib.holo_transform_mc(h.h, _sign(sign), lam, a.ptr, p.ptr, uu.ptr, n, vv.ptr, m,
                                    optr, seed, subsample, targets_per_block,
                                    _stream(a if a.device else vv)))
    return _as_complex(out)


def adjoint(amp, phase, u, v, grad_y, sign: int, lam: float = DEFAULT_LAMBDA,
            precision="split32"):
    """(dL/d amp, dL/d phase) of a real loss L given grad_y = dL/dRe y + i dL/dIm y."""
    with Plan(u, v, precision, device=_device_of(_Buf(amp))) as pl:
        return pl.adjoint(amp, phase, grad_y, sign, lam)


def normalize_polar(y):
    """normalize_amp + polar output: (|y|/max, atan2) and max |y| (cuda/transform.cu:106-139)."""
    b = _Buf(y, name="y")
    m = b.n // 2
    h = handle(_device_of(b))
    amp, aptr = _empty_like(b, m)
    ph, pptr = _empty_like(b, m)
    mx = ctypes.c_double()
    N.check(h.lib.holo_normalize_polar(h.h, b.ptr, m, aptr, pptr, ctypes.byref(mx), _stream(b)))
    return amp, ph, mx.value


def project(x_amp, x_phase, u, v, w=None, lam: float = DEFAULT_LAMBDA, precision="split32",
            reference_wave: bool = False, reference_distance: float = 0.25):
    """x -> y -> z: y = normalised polar Backwards(x, u -> v); z = Forwards(y, v -> w)."""
    a = _Buf(x_amp, name="x_amp")
    n = a.n
    p = _Buf(x_phase, n, "x_phase")
    uu = _Buf(u, 3 * n, "u")
    vv = _Buf(v, name="v")
    m = vv.n // 3
    ww = _Buf(w if w is not None else np.zeros(0), name="w")
    if w is not None and _is_tensor(w) and ww.device != a.device:
        raise ValueError("w must live with the other inputs")
    pcount = ww.n // 3
    h = handle(_device_of(a, p, uu, vv))
    ref = a if a.device else vv
    ya, yap = _empty_like(ref, m)
    yp, ypp = _empty_like(ref, m)
    za, zap = _empty_like(ref, pcount)
    zp, zpp = _empty_like(ref, pcount)
    N.check(h.lib.holo_project(h.h, lam, a.ptr, p.ptr, uu.ptr, n, vv.ptr, m,
                               ww.ptr if pcount else None, pcount, yap, ypp,
                               zap if pcount else None, zpp if pcount else None,
                               _precision(precision), int(bool(reference_wave)),
                               reference_distance, _stream(ref)))
    return ya, yp, za, zp


# ---- plans ----------------------------------------------------------------------------
class Plan:
    """Positions fixed, amplitudes/phases per call (the tiling is built once)."""

    def __init__(self, u, v, precision="split32", device: int | None = None):
        uu = _Buf(u, name="u")
        vv = _Buf(v, name="v")
        if uu.n % 3 or vv.n % 3:
            raise ValueError("u and v must hold xyz triples")
        self.n, self.m = uu.n // 3, vv.n // 3
        self.precision = _precision(precision)
        self.h = handle(device if device is not None else _device_of(uu, vv))
        self._keep = (uu, vv)
        self._ref = uu if uu.device else vv
        p = ctypes.c_void_p()
        N.check(self.h.lib.holo_plan_create(self.h.h, uu.ptr, self.n, vv.ptr, self.m,
                                            self.precision, _stream(self._ref), ctypes.byref(p)))
        self.p = p

    def close(self) -> None:
        if self.p:
            self.h.lib.holo_plan_destroy(self.p)
            self.p = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass

    def execute(self, amp, phase, sign: int, lam: float = DEFAULT_LAMBDA, out=None,
                flags: int = 0):
        a = _Buf(amp, self.n, "amp")
        p = _Buf(phase, self.n, "phase")
        if out is None:
            out, optr = _empty_like(a, 2 * self.m)
        else:
            ob = _Buf(out, 2 * self.m, "out")
            if ob.obj is not out and not (_is_tensor(out) and out.is_contiguous()):
                raise ValueError("out must be a contiguous float64 buffer of 2*M values")
            optr = ob.ptr
        N.check(self.h.lib.holo_plan_execute_flags(self.p, _sign(sign), lam, a.ptr, p.ptr, optr,
                                                   flags, _stream(a)))
        return _as_complex(out)

    def execute_mc(self, amp, phase, sign: int, lam: float = DEFAULT_LAMBDA, seed: int = 0,
                   subsample: int = 16, targets_per_block: int = 256):
        a = _Buf(amp, self.n, "amp")
        p = _Buf(phase, self.n, "phase")
        out, optr = _empty_like(a, 2 * self.m)
        N.check(self.h.lib.holo_plan_execute_mc(self.p, _sign(sign), lam, a.ptr, p.ptr, optr,
                                                seed, subsample, targets_per_block, _stream(a)))
        return _as_complex(out)

    def adjoint(self, amp, phase, grad_y, sign: int, lam: float = DEFAULT_LAMBDA):
        a = _Buf(amp, self.n, "amp")
        p = _Buf(phase, self.n, "phase")
        g = _Buf(grad_y, 2 * self.m, "grad_y")
        ga, gaptr = _empty_like(a, self.n)
        gp, gpptr = _empty_like(a, self.n)
        N.check(self.h.lib.holo_plan_adjoint(self.p, _sign(sign), lam, a.ptr, p.ptr, g.ptr,
                                             gaptr, gpptr, _stream(a)))
        return ga, gp

    def tiling(self) -> dict:
        """The tiling of the plan's sources and targets: "hilbert" or "packed" ("none"
        for an FP64 plan, which keeps the caller's order)."""
        ts, tt = ctypes.c_int(), ctypes.c_int()
        N.check(self.h.lib.holo_plan_tiling(self.p, ctypes.byref(ts), ctypes.byref(tt)))
        return {"sources": _TILINGS[ts.value], "targets": _TILINGS[tt.value]}

    def order(self, which: int) -> np.ndarray:
        n = self.n if which == 0 else self.m
        out = np.zeros(max(n, 1), np.int32)
        N.check(self.h.lib.holo_plan_get_order(self.p, which, out.ctypes.data))
        return out[:n]

    def info(self) -> dict:
        v, s, tt, cs = (ctypes.c_int() for _ in range(4))
        N.check(self.h.lib.holo_plan_info(self.p, ctypes.byref(v), ctypes.byref(s),
                                          ctypes.byref(tt), ctypes.byref(cs)))
        b = ctypes.c_double()
        N.check(self.h.lib.holo_plan_error_bound(self.p, ctypes.byref(b)))
        return {"variant": v.value, "splits": s.value, "target_tile": tt.value,
                "source_tile": cs.value, "path_error_bound_m": b.value}


# ---- batches ----------------------------------------------------------------------------
@dataclass
class Problem:
    amp: object
    phase: object
    u: object
    v: object
    sign: int
    lam: float
    y: object  # float64 buffer of 2*M values (device)


class Batch:
    """Many uneven problems in one persistent launch, replayed from a CUDA graph."""

    def __init__(self, problems: list[Problem], precision="split32", device: int = 0):
        self.h = handle(device)
        arr = (N.HoloProblem * max(1, len(problems)))()
        self._keep = []
        for i, pb in enumerate(problems):
            bufs = [_Buf(x) for x in (pb.amp, pb.phase, pb.u, pb.v, pb.y)]
            for b, x in zip(bufs, (pb.amp, pb.phase, pb.u, pb.v, pb.y)):
                if not b.device:
                    raise ValueError("batched problems need CUDA tensors")
            self._keep.append(bufs)
            arr[i] = N.HoloProblem(bufs[0].ptr, bufs[1].ptr, bufs[2].ptr, bufs[0].n, bufs[3].ptr,
                                   bufs[3].n // 3, _sign(pb.sign), pb.lam, bufs[4].ptr)
        self._arr = arr
        b = ctypes.c_void_p()
        s = ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)
        N.check(self.h.lib.holo_batch_create(self.h.h, arr, len(problems), _precision(precision),
                                             s, ctypes.byref(b)))
        self.b = b
        pairs = ctypes.c_longlong()
        N.check(self.h.lib.holo_batch_pairs(b, ctypes.byref(pairs)))
        self.pairs = pairs.value

    def execute(self) -> None:
        s = ctypes.c_void_p(torch.cuda.current_stream(self.h.device).cuda_stream)
        N.check(self.h.lib.holo_batch_execute(self.b, s))

    def close(self) -> None:
        if self.b:
            self.h.lib.holo_batch_destroy(self.b)
            self.b = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


# ---- variants and the persisted autotuning table ----------------------------------------
def variants(precision="split32") -> list[dict]:
    L = N.load()
    pr = _precision(precision)
    out = []
    for i in range(L.holo_variant_count(pr)):
        t, r, c, q, k, lp = (ctypes.c_int() for _ in range(6))
        N.check(L.holo_variant_describe(pr, i, ctypes.byref(t), ctypes.byref(r), ctypes.byref(c),
                                        ctypes.byref(q), ctypes.byref(k), ctypes.byref(lp)))
        out.append({"variant": i, "threads": t.value, "targets_per_thread": r.value,
                    "source_tile": c.value, "target_tile": t.value * r.value,
                    "fma_sincos_targets": q.value, "pair_model": k.value,
                    "pair_loop": lp.value})
    return out


def size_bucket(n: int, m: int) -> int:
    return N.load().holo_size_bucket(n, m)


def tuning_path() -> str:
    return os.environ.get("HOLO_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "holo_gb300",
                                       "tune.json"))


def load_tuning(h: Handle) -> None:
    path = tuning_path()
    if not os.path.exists(path):
        return
    try:
        with open(path) as f:
            table = json.load(f)
        for prec, buckets in table.items():
            for bucket, var in buckets.items():
                h.set_variant(prec, int(bucket), int(var))
    except (OSError, ValueError, N.HoloError):
        pass  # a stale or foreign cache is ignored


def autotune(n: int, m: int, precision="split32", repeats: int = 3, device: int = 0,
             save: bool = True) -> dict:
    """Time every kernel variant on an n x m problem; record the best for its size bucket."""
    h = handle(device)
    best, rate = h.autotune(n, m, precision, repeats)
    bucket = size_bucket(n, m)
    if save:
        path = tuning_path()
        os.makedirs(os.path.dirname(path), exist_ok=True)
        table = {}
        if os.path.exists(path):
            try:
                with open(path) as f:
                    table = json.load(f)
            except (OSError, ValueError):
                table = {}
        key = "split32" if _precision(precision) == N.SPLIT32 else "fp64"
        table.setdefault(key, {})[str(bucket)] = best
        with open(path, "w") as f:
            json.dump(table, f, indent=1)
    return {"bucket": bucket, "variant": best, "pairs_per_s": rate}


# ---- the reference's names ----------------------------------------------------------------
def transform_full(x, u, v, direction, lam: float = DEFAULT_LAMBDA, precision="fp64"):
    """transform_full<direction>(x, u, v) (cuda/transform.cu:147-340): x is N x (amp, phase)."""
    xb = np.asarray(x, dtype=np.float64).reshape(-1, 2) if not _is_tensor(x) else x.reshape(-1, 2)
    return transform(xb[:, 0], xb[:, 1], u, v, _sign(direction), lam, precision)


def time_transform(x, u, v, direction, lam: float = DEFAULT_LAMBDA, precision="fp64"):
    """time_transform (cuda/transform.cu:346-406): returns (M x (amp, phase), runtime seconds)."""
    t0 = time.perf_counter()
    y = transform_full(x, u, v, direction, lam, precision)
    amp, ph, _ = normalize_polar(torch.view_as_real(y).reshape(-1) if _is_tensor(y)
                                 else y.view(np.float64))
    dt = time.perf_counter() - t0
    if _is_tensor(amp):
        return torch.stack([amp, ph], dim=1), dt
    return np.stack([amp, ph], axis=1), dt


def phasor_displacement(amplitude, phase, w, v, direction=1, lam: float = DEFAULT_LAMBDA):
    """py/util.py:92-108: terms a/r exp(i(phase - direction k r)) of sources w at target v."""
    w = np.asarray(w, dtype=np.float64).reshape(-1, 3)
    amp = np.broadcast_to(np.asarray(amplitude, dtype=np.float64), (w.shape[0],))
    ph = np.broadcast_to(np.asarray(phase, dtype=np.float64), (w.shape[0],))
    v = np.asarray(v, dtype=np.float64).reshape(1, 3)
    # one term per source: a transform with one target per call is wasteful, so
    # evaluate each source against the target as its own one-source sum
    out = np.empty(w.shape[0], np.complex128)
    for i in range(w.shape[0]):
        out[i] = transform(amp[i:i + 1], ph[i:i + 1], w[i], v, -int(direction), lam, "fp64")[0]
    return out


def map_sum_kernel(x, y, w, v, direction=1, distance=1, plane_wave_intensity=0.0,
                   lam: float = DEFAULT_LAMBDA, precision="fp64"):
    """py/util.py:133-147: y[m] = polar(sum_n phasor(x_n at w_n, v_m)) in place.

    The prototype's direction=+1 is the CUDA path's Backwards (phase - k r)."""
    x = np.asarray(x, dtype=np.float64).reshape(-1, 2)
    c = np.asarray(transform(x[:, 0], x[:, 1], w, v, -int(direction), lam, precision))
    if abs(plane_wave_intensity) > 0:
        c = c + plane_wave_intensity
    amp, ph = np.abs(c), np.angle(c)
    if np.sign(distance) == -1:
        ph = -ph
    y[:, 0] = amp
    y[:, 1] = ph


def projector_setup(x, y, z, w, v, u, plane_wave_intensity=1, lam: float = DEFAULT_LAMBDA,
                    precision="fp64"):
    """py/util.py:166-175: y from x (direction -1, with a plane wave), then z from y."""
    map_sum_kernel(x, y, w, v, direction=-1, plane_wave_intensity=plane_wave_intensity, lam=lam,
                   precision=precision)
    y[:, 0] /= np.max(y[:, 0])
    map_sum_kernel(y, z, v, u, lam=lam, precision=precision)
    z[:, 0] /= np.max(z[:, 0])
