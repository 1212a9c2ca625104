"""The reference's file interface in Python: raw little-endian FP64 ``.dat``
arrays and ``out.json`` (one JSON object per line), as written by
cuda/util.h:296-444 and read by py/util.py:685-751.
"""
from __future__ import annotations

import json
import os

import numpy as np


def read_dat(path: str) -> np.ndarray:
    """read_bytes<double> (cuda/util.h:249-283)."""
    data = np.fromfile(path, dtype="<f8")
    if data.size == 0:
        raise ValueError(f"{path}: empty or missing data")
    return data


def write_dat(path: str, data) -> None:
    np.ascontiguousarray(data, dtype="<f8").tofile(path)


def read_inputs(directory: str, projection: bool = False) -> dict:
    """x0_amp, x0_phase, u0, v0 (and w0_0, falling back to w0) of a -f directory."""
    d = {k: read_dat(os.path.join(directory, f"{k}.dat"))
         for k in ("x0_amp", "x0_phase", "u0", "v0")}
    if projection:
        for name in ("w0_0", "w0"):
            p = os.path.join(directory, f"{name}.dat")
            if os.path.exists(p):
                d["w0_0"] = read_dat(p)
                break
        else:
            raise FileNotFoundError(f"{directory}: neither w0_0.dat nor w0.dat")
    n = d["x0_amp"].size
    if d["x0_phase"].size != n or d["u0"].size != 3 * n or d["v0"].size % 3:
        raise ValueError("inconsistent input sizes")
    return d


def write_inputs(directory: str, x_amp, x_phase, u, v, w=None) -> None:
    """Write the reference's input files (matlab/projector.m:63-75 layout)."""
    os.makedirs(directory, exist_ok=True)
    write_dat(os.path.join(directory, "x0_amp.dat"), x_amp)
    write_dat(os.path.join(directory, "x0_phase.dat"), x_phase)
    write_dat(os.path.join(directory, "u0.dat"), u)
    write_dat(os.path.join(directory, "v0.dat"), v)
    if w is not None:
        write_dat(os.path.join(directory, "w0_0.dat"), w)


def parse_out_json(path: str) -> list[dict]:
    """Every metadata line of out.json (py/util.py:685-700)."""
    out = []
    with open(path) as f:
        for line in f:
            line = line.strip()
            if line:
                out.append(json.loads(line))
    return out
