"""Generate the golden fixtures under tests/golden/ from the reference itself.

Run in a container where the reference sources are mounted (default
/root/reference, override with HOLO_REFERENCE).  It

1. compiles the reference's own host-side ``phasor_displacement``
   (cuda/superposition.cu:35-51) through ``oracle/ref_probe.cu`` into
   ``oracle/_ref/`` (``make -C oracle ref``), once per wavelength;
2. imports the reference's NumPy prototype ``py/util.py`` with the smallest
   shims that make it importable (``numba.jit`` -> identity, a ``pandas`` stub,
   ``util.f = util.phasor_displacement``: the prototype calls an undefined ``f``
   at py/util.py:114);
3. writes the fixtures below.  The GPU machine has no reference sources: the tests
   there read only these committed files.

Fixtures
  pairs_6328.npz / pairs_650.npz  random single terms, reference host function
  known_answer.json               py/test_util.py:49-64 unit source at distance lambda
  transform_small.npz             x->y (Backwards) and y->z (Forwards) sums of the
                                  reference's own terms on a small grid, plus the
                                  prototype's polar output for the same x->y sum
  generators.npz                  the reference's own init::plane lattices (without
                                  -r) and init::sparse_plane object shapes for the
                                  planes of the holo CLI runs in
                                  tests/test_gpu_generators.py

``python make_golden.py generators`` writes generators.npz alone.
"""
from __future__ import annotations

import ctypes
import json
import os
import subprocess
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("HOLO_REFERENCE", "/root/reference")
sys.path.insert(0, os.path.join(REPO, "oracle"))
import oracle  # noqa: E402


def import_prototype(lam: float):
    """Import py/util.py from the reference with the minimal shims."""
    numba = types.ModuleType("numba")

    def jit(*args, **kwargs):
        if len(args) == 1 and callable(args[0]) and not kwargs:
            return args[0]
        return lambda f: f

    numba.jit = jit
    pandas = types.ModuleType("pandas")
    pandas.DataFrame = object
    sys.modules.setdefault("numba", numba)
    sys.modules.setdefault("pandas", pandas)
    sys.path.insert(0, os.path.join(REF, "py"))
    import util  # type: ignore

    util.f = util.phasor_displacement
    util.LAMBDA = lam
    return util


def grid(nx: int, ny: int, pitch: float, z: float) -> np.ndarray:
    """Centred square lattice, x slow / y fast (matlab/projector.m:31-39 order)."""
    xs = (np.arange(nx) - (nx - 1) / 2.0) * pitch
    ys = (np.arange(ny) - (ny - 1) / 2.0) * pitch
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), np.full(nx * ny, z)], axis=1)


# Planes of the generated-mode runs in tests/test_gpu_generators.py (holo -x 16 -y 4096
# -z 1024 -a 1.5 -A 0.8 -l 3e-3 -n 1.2e-3 -o 2e-4 -O 4e-4 -u 1e-4 -U 3e-4 -v -2e-4 -w 0.3
# -X 2 --shape S): per object plane i (ratio i), the object's width and offset, the
# projector lattice and the projection lattice, as the reference derives them
# (cuda/main.cu:125-181: lerp of the ranges, gerp of z; z offset fixed here).
GEN_PLANES = [
    # (object width, object offset xyz, modulate)
    (2e-4, (1e-4, -2e-4, 0.3), 0.0),
    (4e-4, (3e-4, -2e-4, 0.3), 0.5),
]
GEN_SHAPES = {"line": 0, "log-line": 1, "circle": 2, "dotted-circle": 3}


def generators() -> None:
    """The reference's own generators through the probe (host code: no GPU needed)."""
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "all", f"REF={REF}"],
                   check=True)
    R = oracle.reference_probe("650")
    assert R is not None
    dp = oracle._dp
    R.ref_plane.restype = None
    R.ref_plane.argtypes = [ctypes.c_size_t] + [ctypes.c_double] * 5 + [dp]
    R.ref_sparse_plane.restype = None
    R.ref_sparse_plane.argtypes = [ctypes.c_size_t, ctypes.c_int] + [ctypes.c_double] * 5 + [dp]

    def plane(n, width, off, aspect):
        out = np.zeros(3 * n)
        R.ref_plane(n, width, off[0], off[1], off[2], aspect, out.ctypes.data_as(dp))
        return out

    out = {}
    # the projector (-y 4096 -a 1.5 -l 3e-3, at the origin) and the projection plane
    # (-z 1024 -A 0.8 -n 1.2e-3, at the object's offset) of each object plane
    for i, (_, off, _) in enumerate(GEN_PLANES):
        out[f"v{i}"] = plane(4096, 3e-3, (0.0, 0.0, 0.0), 1.5)
        out[f"w{i}_0"] = plane(1024, 1.2e-3, off, 0.8)
    # the default projector of a plain run (-y 4096, width 512 x 7 um, square)
    out["v_default"] = plane(4096, 512 * 7e-6, (0.0, 0.0, 0.0), 1.0)
    # object shapes: 16 points, the array carried from plane to plane as the CLI does
    for name, code in GEN_SHAPES.items():
        u = np.zeros(3 * 16)
        for i, (width, off, mod) in enumerate(GEN_PLANES):
            R.ref_sparse_plane(16, code, width, off[0], off[1], off[2], mod,
                               u.ctypes.data_as(dp))
            out[f"u{i}_{name}"] = u.copy()
    # one point (the n == 1 branch)
    u1 = np.zeros(3)
    R.ref_sparse_plane(1, 2, 2e-4, 1e-4, -2e-4, 0.3, 0.0, u1.ctypes.data_as(dp))
    out["u_single"] = u1
    np.savez_compressed(os.path.join(HERE, "generators.npz"), **out)
    print("generators.npz written to", HERE)


def main() -> None:
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "all", f"REF={REF}"],
                   check=True)
    dp = oracle._dp
    rng = np.random.default_rng(20240601)

    # 1. single terms through the reference's own host function
    for tag, lam in (("6328", 632.8e-9), ("650", 0.65e-6)):
        R = oracle.reference_probe(tag)
        assert R is not None and abs(R.ref_lambda() - lam) < 1e-20
        n = 2048
        u = np.empty((n, 3))
        v = np.empty((n, 3))
        u[:, :2] = rng.uniform(-4e-3, 4e-3, (n, 2))
        u[:, 2] = 0.35 + rng.uniform(-2e-3, 2e-3, n)
        v[:, :2] = rng.uniform(-6e-3, 6e-3, (n, 2))
        v[:, 2] = rng.uniform(-1e-3, 1e-3, n)
        # a few near-field and far-field pairs as edge cases
        v[:16, 2] = u[:16, 2] - rng.uniform(1e-6, 1e-4, 16)
        u[16:32, 2] = rng.uniform(0.5, 2.0, 16)
        amp = rng.uniform(0.0, 1.0, n)
        phase = rng.uniform(-np.pi, 3 * np.pi, n)
        sign = np.where(rng.uniform(size=n) < 0.5, 1, -1).astype(np.int32)
        out = np.zeros((n, 2))
        for i in range(n):
            ui, vi, oi = (np.ascontiguousarray(a) for a in (u[i], v[i], out[i]))
            R.ref_phasor(amp[i], phase[i], ui.ctypes.data_as(dp), vi.ctypes.data_as(dp),
                         int(sign[i]), oi.ctypes.data_as(dp))
            out[i] = oi
        np.savez_compressed(os.path.join(HERE, f"pairs_{tag}.npz"), u=u, v=v, amp=amp,
                            phase=phase, sign=sign, lam=lam, ref=out)

    # 2. known answer of py/test_util.py:49-64 (lambda = 0.65e-6)
    util = import_prototype(0.65e-6)
    x = np.zeros((1, 2))
    x[:, 0] = 1.0
    u0 = np.zeros((1, 3))
    v0 = u0.copy()
    v0[0, 2] = util.LAMBDA
    c = np.sum(util.f(x[:, 0], x[:, 1], u0, v0[0], direction=1))
    a, phi = util.from_polar(c)
    known = {"lambda": 0.65e-6, "amp": float(a), "phase": float(phi),
             "amp_asserted": 1538461.5384615385, "phase_asserted": 2.4492935982947064e-16,
             "source": "py/test_util.py:63-64", "direction_py": 1, "sign_cuda": -1}
    with open(os.path.join(HERE, "known_answer.json"), "w") as f:
        json.dump(known, f, indent=1)

    # 3. small x->y->z through the reference's own terms (lambda = 632.8 nm)
    lam = 632.8e-9
    util = import_prototype(lam)
    R = oracle.reference_probe("6328")
    xg = grid(16, 16, 10e-6, 0.35)
    vg = grid(32, 32, 7.56e-6, 0.0)
    srng = np.random.default_rng(0)
    amp = srng.uniform(0.0, 1.0, xg.shape[0])
    phase = srng.uniform(0.0, 2 * np.pi, xg.shape[0])

    def ref_sum(a, p, u, v, sign):
        a, p, u, v = (np.ascontiguousarray(t, dtype=np.float64) for t in (a, p, u, v))
        y = np.zeros(2 * (v.size // 3))
        R.ref_transform(a.size, a.ctypes.data_as(dp), p.ctypes.data_as(dp),
                        u.ctypes.data_as(dp), v.size // 3, v.ctypes.data_as(dp), sign,
                        y.ctypes.data_as(dp))
        return y.view(np.complex128)

    y = ref_sum(amp, phase, xg, vg, -1)
    yn, _ = oracle.normalize_amp(y)
    y_amp, y_phase = oracle.to_polar(yn)
    z = ref_sum(y_amp, y_phase, vg, xg, +1)
    zn, _ = oracle.normalize_amp(z)
    z_amp, z_phase = oracle.to_polar(zn)

    # the prototype's own x->y sum: map_sum_kernel with direction=+1 is phase - k r
    proto = np.zeros((vg.shape[0], 2))
    util.map_sum_kernel(np.stack([amp, phase], axis=1), proto, xg, vg, direction=1)
    np.savez_compressed(os.path.join(HERE, "transform_small.npz"), lam=lam, u=xg, v=vg, w=xg,
                        amp=amp, phase=phase, y=y, y_amp=y_amp, y_phase=y_phase, z=z,
                        z_amp=z_amp, z_phase=z_phase, proto_y_amp=proto[:, 0],
                        proto_y_phase=proto[:, 1])
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    if sys.argv[1:] == ["generators"]:
        generators()
    else:
        main()
        generators()
