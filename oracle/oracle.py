"""ctypes binding of the CPU FP64 oracle (oracle/holo_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` and
by the CPU-baseline leg of ``bench.py`` -- as the checker, never as the thing
measured or shipped.  ``build()`` compiles ``liboracle.so`` with the Makefile
beside this file.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

_dp = ctypes.POINTER(ctypes.c_double)
_i64p = ctypes.POINTER(ctypes.c_int64)
_i32p = ctypes.POINTER(ctypes.c_int32)
_u32p = ctypes.POINTER(ctypes.c_uint32)
_lib = None


def build(with_reference: bool = False) -> None:
    """Compile liboracle.so (and the reference probes when asked and present)."""
    target = "all" if with_reference else "oracle"
    subprocess.run(["make", "-s", "-C", HERE, target], check=True)


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.oracle_wavenumber.restype = ctypes.c_double
        L.oracle_wavenumber.argtypes = [ctypes.c_double]
        L.oracle_phasor.restype = None
        L.oracle_phasor.argtypes = [ctypes.c_double, ctypes.c_double, _dp, _dp, ctypes.c_int,
                                    ctypes.c_double, _dp]
        L.oracle_transform.restype = ctypes.c_int
        L.oracle_transform.argtypes = [ctypes.c_size_t, _dp, _dp, _dp, ctypes.c_size_t, _dp,
                                       ctypes.c_int, ctypes.c_double, _dp, ctypes.c_int]
        L.oracle_transform_subset.restype = ctypes.c_int
        L.oracle_transform_subset.argtypes = [ctypes.c_size_t, _dp, _dp, _dp, _dp, _i64p,
                                              ctypes.c_size_t, ctypes.c_int, ctypes.c_double,
                                              _dp, ctypes.c_int]
        L.oracle_normalize_amp.restype = ctypes.c_double
        L.oracle_normalize_amp.argtypes = [_dp, ctypes.c_size_t]
        L.oracle_to_polar.restype = None
        L.oracle_to_polar.argtypes = [_dp, ctypes.c_size_t, _dp, _dp]
        L.oracle_philox4x32_10.restype = None
        L.oracle_philox4x32_10.argtypes = [_u32p, _u32p, _u32p]
        L.oracle_transform_mc.restype = ctypes.c_int
        L.oracle_transform_mc.argtypes = [ctypes.c_size_t, _dp, _dp, _dp, ctypes.c_size_t, _dp,
                                          ctypes.c_int, ctypes.c_double, _i32p, _i32p,
                                          ctypes.c_uint64, ctypes.c_int, ctypes.c_int, _dp,
                                          ctypes.c_int]
        _lib = L
    return _lib


def _d(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def _c(a, dtype=np.float64) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=dtype)


def wavenumber(lam: float) -> float:
    return lib().oracle_wavenumber(lam)


def phasor(amp: float, phase: float, u, v, sign: int, lam: float) -> complex:
    u = _c(u)
    v = _c(v)
    out = np.zeros(2)
    lib().oracle_phasor(amp, phase, _d(u), _d(v), int(sign), wavenumber(lam), _d(out))
    return complex(out[0], out[1])


def transform(amp, phase, u, v, sign: int, lam: float, threads: int | None = None) -> np.ndarray:
    """Brute-force FP64 sum; returns complex128 array of M targets."""
    amp, phase, u, v = _c(amp), _c(phase), _c(u).reshape(-1), _c(v).reshape(-1)
    N, M = amp.size, v.size // 3
    y = np.zeros(2 * M)
    rc = lib().oracle_transform(N, _d(amp), _d(phase), _d(u), M, _d(v), int(sign), lam, _d(y),
                                threads or os.cpu_count() or 1)
    if rc != 0:
        raise ValueError("oracle_transform: bad arguments")
    return y.view(np.complex128)


def transform_subset(amp, phase, u, v, idx, sign: int, lam: float,
                     threads: int | None = None) -> np.ndarray:
    amp, phase, u, v = _c(amp), _c(phase), _c(u).reshape(-1), _c(v).reshape(-1)
    idx = _c(idx, np.int64)
    y = np.zeros(2 * idx.size)
    rc = lib().oracle_transform_subset(amp.size, _d(amp), _d(phase), _d(u), _d(v),
                                       idx.ctypes.data_as(_i64p), idx.size, int(sign), lam,
                                       _d(y), threads or os.cpu_count() or 1)
    if rc != 0:
        raise ValueError("oracle_transform_subset: bad arguments")
    return y.view(np.complex128)


def normalize_amp(y: np.ndarray) -> tuple[np.ndarray, float]:
    y2 = _c(y.view(np.float64) if y.dtype == np.complex128 else y).copy()
    mx = lib().oracle_normalize_amp(_d(y2), y2.size // 2)
    return y2.view(np.complex128), mx


def to_polar(y: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    y2 = _c(y.view(np.float64) if y.dtype == np.complex128 else y)
    M = y2.size // 2
    a, p = np.zeros(M), np.zeros(M)
    lib().oracle_to_polar(_d(y2), M, _d(a), _d(p))
    return a, p


def philox(ctr, key) -> np.ndarray:
    c = _c(ctr, np.uint32)
    k = _c(key, np.uint32)
    out = np.zeros(4, np.uint32)
    lib().oracle_philox4x32_10(c.ctypes.data_as(_u32p), k.ctypes.data_as(_u32p),
                               out.ctypes.data_as(_u32p))
    return out


def transform_mc(amp, phase, u, v, sign: int, lam: float, src_order, tgt_order, seed: int,
                 sub: int, block: int, threads: int | None = None) -> np.ndarray:
    amp, phase, u, v = _c(amp), _c(phase), _c(u).reshape(-1), _c(v).reshape(-1)
    so, to = _c(src_order, np.int32), _c(tgt_order, np.int32)
    M = v.size // 3
    y = np.zeros(2 * M)
    rc = lib().oracle_transform_mc(amp.size, _d(amp), _d(phase), _d(u), M, _d(v), int(sign), lam,
                                   so.ctypes.data_as(_i32p), to.ctypes.data_as(_i32p),
                                   ctypes.c_uint64(seed), sub, block, _d(y),
                                   threads or os.cpu_count() or 1)
    if rc != 0:
        raise ValueError("oracle_transform_mc: bad arguments")
    return y.view(np.complex128)


def reference_probe(lam_tag: str = "6328") -> ctypes.CDLL | None:
    """The reference's own host phasor_displacement, compiled under oracle/_ref
    (present only where the reference sources were available at build time)."""
    p = os.path.join(REF_DIR, f"libref_probe_{lam_tag}.so")
    if not os.path.exists(p):
        return None
    L = ctypes.CDLL(p)
    L.ref_lambda.restype = ctypes.c_double
    L.ref_two_pi_over_lambda.restype = ctypes.c_double
    L.ref_phasor.restype = None
    L.ref_phasor.argtypes = [ctypes.c_double, ctypes.c_double, _dp, _dp, ctypes.c_int, _dp]
    L.ref_transform.restype = None
    L.ref_transform.argtypes = [ctypes.c_size_t, _dp, _dp, _dp, ctypes.c_size_t, _dp,
                                ctypes.c_int, _dp]
    return L
