"""GB300-native Huygens superposition (x -> y -> z) for holographic projectors.

The package directory name is not a Python identifier; load it with
``__graft_entry__.load_package()`` (it registers the module as ``holo_gb300``)
or any importlib file-location loader.

Submodules:
  _native    ctypes binding of libholo.so (include/holo.h)
  api        Handle / Plan / Batch, transform, transform_mc, adjoint, project,
             normalize_polar, tile_order, the reference's names (transform_full, ...)
  torch_ops  autograd Function over the adjoint kernel, phase-only optimiser
  io         the reference's .dat / out.json file interface
  build      in-tree nvcc build of libholo.so and the holo CLI
"""
from . import _native, io  # noqa: F401
from ._native import (BACKWARDS, FLAG_CONST_PHASE, FORWARDS, FP64, SPLIT32,  # noqa: F401
                      TILE_HILBERT, TILE_PACKED, HoloError)
from .api import (Batch, Handle, Plan, Problem, adjoint, autotune, handle,  # noqa: F401
                  map_sum_kernel, normalize_polar, phasor_displacement, project,
                  projector_setup, size_bucket, tile_order, time_transform, transform,
                  transform_full, transform_mc, variants)

__all__ = ["Batch", "Handle", "Plan", "Problem", "HoloError", "adjoint", "autotune", "handle",
           "normalize_polar", "project", "transform", "transform_full", "transform_mc",
           "time_transform", "variants", "size_bucket", "map_sum_kernel",
           "phasor_displacement", "projector_setup", "FORWARDS", "BACKWARDS", "FP64",
           "SPLIT32", "FLAG_CONST_PHASE", "TILE_HILBERT", "TILE_PACKED", "tile_order"]
