"""The generated-data mode's planes against the reference's own generators.

tests/golden/generators.npz holds the output of the reference's host functions
init::plane (lattice without -r, cuda/init.h:89-158) and init::sparse_plane (object
shapes, cuda/init.h:160-234), compiled here from its sources (oracle/ref_probe.cu,
tests/golden/make_golden.py).  The holo CLI builds the same planes with device kernels
(csrc/gen.cu); lattices and line objects must equal the reference bit for bit.  Shapes
that call sin, cos, pow or log10 may differ in the last places (CUDA's math library
against the C library): at most 2 ulps of the largest coordinate of the plane (an
offset added to a sine can cancel leading digits, so ulps of the result itself would
overstate the difference); their heights are exact.

The -r jitter (cuda/init.h:19-34, 120-141) is compared bit for bit with cuRAND's XORWOW
device generator driven from the test (seed 1235 for the first lattice, 1236 for the
next), called the reference's way: per lattice row, x + y uniforms into a buffer, then
(x + y) / 8 more into the start of the same buffer, which the row then reads.  (cuRAND's
host-side generator does not reproduce the device generator's sequence.)
"""
import ctypes
import ctypes.util
import glob
import math
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

GEN_FLAGS = ["-x", "16", "-y", "4096", "-z", "1024", "-a", "1.5", "-A", "0.8", "-l", "3e-3",
             "-n", "1.2e-3", "-o", "2e-4", "-O", "4e-4", "-u", "1e-4", "-U", "3e-4", "-v",
             "-2e-4", "-w", "0.3", "-X", "2"]


def _cli(holo):
    return os.path.join(os.path.dirname(holo.__file__), "holo")


def _run(holo, out, *flags):
    r = subprocess.run([_cli(holo), *flags, "--out", str(out), "--precision", "split32"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return lambda name: holo.io.read_dat(str(out / f"{name}.dat"))


def _xy_ulps(u, ref):
    """Largest difference of the x, y coordinates in ulps of the plane's largest one."""
    a, b = u.reshape(-1, 3)[:, :2], ref.reshape(-1, 3)[:, :2]
    return float(np.max(np.abs(a - b)) / np.spacing(np.max(np.abs(b))))


@pytest.mark.parametrize("shape", ["line", "log-line", "circle", "dotted-circle"])
def test_planes_match_the_reference_generators(holo, tmp_path, shape):
    g = np.load(os.path.join(GOLDEN, "generators.npz"))
    rd = _run(holo, tmp_path, *GEN_FLAGS, "--shape", shape)
    for i in range(2):
        # the projector lattice (aspect 1.5: 78 x 52 cells, 40 points repeating point 0)
        # and the projection lattice (aspect 0.8) of each object plane: bit for bit
        assert np.array_equal(rd(f"v{i}"), g[f"v{i}"]), i
        assert np.array_equal(rd(f"w{i}_0"), g[f"w{i}_0"]), i
        u, ref = rd(f"u{i}"), g[f"u{i}_{shape}"]
        if shape == "line":
            assert np.array_equal(u, ref), i
        else:
            assert np.array_equal(u.reshape(-1, 3)[:, 2], ref.reshape(-1, 3)[:, 2]), i
            assert _xy_ulps(u, ref) <= 2, (i, _xy_ulps(u, ref))


def test_single_object_point_and_default_projector(holo, tmp_path):
    g = np.load(os.path.join(GOLDEN, "generators.npz"))
    rd = _run(holo, tmp_path, "-x", "1", "-y", "4096", "-z", "256", "-o", "2e-4", "-u", "1e-4",
              "-v", "-2e-4", "-w", "0.3")
    assert np.array_equal(rd("u0"), g["u_single"])
    assert np.array_equal(rd("v0"), g["v_default"])  # 512 x 7 um wide, square


def _curand():
    names = [os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64", "libcurand.so")]
    names += sorted(glob.glob("/usr/local/cuda*/targets/*/lib/libcurand.so*"))
    found = ctypes.util.find_library("curand")
    if found:
        names.append(found)
    for n in names:
        try:
            return ctypes.CDLL(n)
        except OSError:
            continue
    pytest.skip("libcurand not found")


def _xorwow_rows(seed, rows, n_random):
    """The reference's numbers for one randomised lattice (cuda/init.h:19-34): one XORWOW
    device generator; per row, n_random uniforms into the buffer, then n_random * 4 / 32
    into its start; the row reads the buffer."""
    import torch
    L = _curand()
    gen = ctypes.c_void_p()
    assert L.curandCreateGenerator(ctypes.byref(gen), 101) == 0  # CURAND_RNG_PSEUDO_XORWOW
    buf = torch.zeros(n_random, dtype=torch.float32, device="cuda:0")
    rows_out = np.zeros((rows, n_random), np.float32)
    try:
        assert L.curandSetPseudoRandomGeneratorSeed(gen, ctypes.c_ulonglong(seed)) == 0
        for i in range(rows):
            assert L.curandGenerateUniform(gen, ctypes.c_void_p(buf.data_ptr()),
                                           ctypes.c_size_t(n_random)) == 0
            assert L.curandGenerateUniform(gen, ctypes.c_void_p(buf.data_ptr()),
                                           ctypes.c_size_t(n_random * 4 // 32)) == 0
            torch.cuda.synchronize()
            rows_out[i] = buf.cpu().numpy()
    finally:
        L.curandDestroyGenerator(gen)
    return rows_out


def _lattice(n, width, off, aspect, rnd=None):
    """init::plane (cuda/init.h:89-158) in NumPy, every operation rounded on its own."""
    x = int(math.sqrt(n * aspect))
    y = n // x
    height = width / aspect
    dx, dy = width / x, height / y
    x_half, y_half = (width - dx) / 2.0, (height - dy) / 2.0
    i, j = np.divmod(np.arange(x * y), y)
    px = (i * dx - x_half) + off[0]
    py = (j * dy - y_half) + off[1]
    if rnd is not None:
        x_range = dx - 0.5 * (0.05 * dx)
        y_range = dy - 0.5 * (0.05 * dy)
        r = rnd.astype(np.float64)
        px = px + x_range * (r[i, (2 * j) % (x + y)] - 0.5)
        py = py + y_range * (r[i, (2 * j + 1) % (x + y)] - 0.5)
    v = np.empty((n, 3))
    v[: x * y, 0], v[: x * y, 1], v[:, 2] = px, py, off[2]
    v[x * y:] = v[0]
    return v.ravel(), x, y


def test_randomised_lattice_matches_host_curand(holo, tmp_path):
    rd = _run(holo, tmp_path, "-x", "4", "-y", "4096", "-z", "1024", "-a", "1.5", "-r")
    width = 512 * 7e-6
    _, x, y = _lattice(4096, width, (0.0, 0.0, 0.0), 1.5)
    rnd = _xorwow_rows(1235, x, x + y)  # the first randomised lattice of the run
    v, _, _ = _lattice(4096, width, (0.0, 0.0, 0.0), 1.5, rnd)
    assert np.array_equal(rd("v0"), v)
    # the projection lattice draws from the next seed; its height is the object plane's
    # (gerp of the default z range, taken from the file)
    w_width, w_aspect = 1e-3 * 1.2, 1.0  # the reference's defaults (cuda/input.h:48-79)
    got = rd("w0_0")
    off = (0.0, 0.0, float(got[2]))
    _, xw, yw = _lattice(1024, w_width, off, w_aspect)
    rw = _xorwow_rows(1236, xw, xw + yw)
    w, _, _ = _lattice(1024, w_width, off, w_aspect, rw)
    assert np.array_equal(got, w)
