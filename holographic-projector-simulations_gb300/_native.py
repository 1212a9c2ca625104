"""ctypes binding of libholo.so (the C ABI declared in include/holo.h).

The library is built in-tree by ``build.py``.  Loading fails loudly when it is
missing: there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libholo.so")

OK = 0
ERR_INVALID = -1
ERR_CUDA = -2
ERR_ALLOC = -3
ERR_NONFINITE = -4
ERR_TIMEOUT = -5
ERR_UNSUPPORTED = -6
ERR_NO_DEVICE = -7

FP64 = 0
SPLIT32 = 1
FORWARDS = 1
BACKWARDS = -1
FLAG_CONST_PHASE = 0x1
TILE_HILBERT = 0  # tilings of holo_tile_order / holo_plan_tiling
TILE_PACKED = 1

_c = ctypes
_dp = _c.c_void_p  # device or host pointer
_sz = _c.c_size_t
_i = _c.c_int
_d = _c.c_double
_vp = _c.c_void_p


class HoloProblem(_c.Structure):
    """holo_problem of include/holo.h (device pointers)."""
    _fields_ = [("amp", _vp), ("phase", _vp), ("u_xyz", _vp), ("N", _sz), ("v_xyz", _vp),
                ("M", _sz), ("sign", _i), ("lambda_", _d), ("y_re_im", _vp)]


# name: (restype, argtypes)
SIGNATURES = {
    "holo_abi_version": (_i, []),
    "holo_last_error_string": (_c.c_char_p, []),
    "holo_create": (_i, [_i, _c.POINTER(_vp)]),
    "holo_destroy": (_i, [_vp]),
    "holo_device_status": (_i, [_vp, _vp]),
    "holo_transform": (_i, [_vp, _i, _d, _dp, _dp, _dp, _sz, _dp, _sz, _dp, _i, _vp]),
    "holo_transform_variant": (_i, [_vp, _i, _d, _dp, _dp, _dp, _sz, _dp, _sz, _dp, _i, _i, _vp]),
    "holo_plan_create": (_i, [_vp, _dp, _sz, _dp, _sz, _i, _vp, _c.POINTER(_vp)]),
    "holo_plan_destroy": (_i, [_vp]),
    "holo_plan_execute": (_i, [_vp, _i, _d, _dp, _dp, _dp, _vp]),
    "holo_plan_execute_flags": (_i, [_vp, _i, _d, _dp, _dp, _dp, _i, _vp]),
    "holo_plan_get_order": (_i, [_vp, _i, _vp]),
    "holo_plan_tiling": (_i, [_vp, _c.POINTER(_i), _c.POINTER(_i)]),
    "holo_tile_order": (_i, [_vp, _dp, _sz, _i, _vp, _vp]),
    "holo_plan_info": (_i, [_vp, _c.POINTER(_i), _c.POINTER(_i), _c.POINTER(_i), _c.POINTER(_i)]),
    "holo_plan_error_bound": (_i, [_vp, _c.POINTER(_d)]),
    "holo_transform_mc": (_i, [_vp, _i, _d, _dp, _dp, _dp, _sz, _dp, _sz, _dp, _c.c_uint64, _i,
                               _i, _vp]),
    "holo_plan_execute_mc": (_i, [_vp, _i, _d, _dp, _dp, _dp, _c.c_uint64, _i, _i, _vp]),
    "holo_plan_adjoint": (_i, [_vp, _i, _d, _dp, _dp, _dp, _dp, _dp, _vp]),
    "holo_adjoint": (_i, [_vp, _i, _d, _dp, _dp, _dp, _sz, _dp, _sz, _dp, _dp, _dp, _i, _vp]),
    "holo_normalize_polar": (_i, [_vp, _dp, _sz, _dp, _dp, _c.POINTER(_d), _vp]),
    "holo_project": (_i, [_vp, _d, _dp, _dp, _dp, _sz, _dp, _sz, _dp, _sz, _dp, _dp, _dp, _dp,
                          _i, _i, _d, _vp]),
    "holo_batch_create": (_i, [_vp, _c.POINTER(HoloProblem), _i, _i, _vp, _c.POINTER(_vp)]),
    "holo_batch_execute": (_i, [_vp, _vp]),
    "holo_batch_destroy": (_i, [_vp]),
    "holo_batch_pairs": (_i, [_vp, _c.POINTER(_c.c_longlong)]),
    "holo_transform_batched": (_i, [_vp, _c.POINTER(HoloProblem), _i, _i, _vp]),
    "holo_variant_count": (_i, [_i]),
    "holo_variant_describe": (_i, [_i, _i, _c.POINTER(_i), _c.POINTER(_i), _c.POINTER(_i),
                                   _c.POINTER(_i), _c.POINTER(_i), _c.POINTER(_i)]),
    "holo_set_variant": (_i, [_vp, _i, _i, _i]),
    "holo_get_variant": (_i, [_vp, _i, _i, _c.POINTER(_i)]),
    "holo_size_bucket": (_i, [_sz, _sz]),
    "holo_autotune": (_i, [_vp, _i, _sz, _sz, _i, _vp, _c.POINTER(_i), _c.POINTER(_d)]),
    "holo_kernel_launches": (_i, [_c.POINTER(_c.c_longlong)]),
    "holo_profile_begin": (_i, [_vp]),
    "holo_profile_end": (_i, [_vp, _c.POINTER(_d), _c.POINTER(_i)]),
    "holo_probe_peak": (_i, [_vp, _i, _c.POINTER(_d)]),
    "holo_selftest_bounded_wait": (_i, [_vp, _c.c_longlong, _vp]),
    "holo_transform_noalloc": (_i, [_i, _i, _d, _dp, _dp, _dp, _sz, _dp, _sz, _dp, _vp]),
}

_lib = None


class HoloError(RuntimeError):
    """A libholo entry point returned a negative status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load libholo.so and declare every entry point of include/holo.h."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"libholo.so is not built ({path}); run build.build() first -- "
                          "the library has no CPU fallback")
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(rc: int) -> None:
    if rc != OK:
        msg = load().holo_last_error_string()
        raise HoloError(rc, msg.decode() if msg else "unknown error")
