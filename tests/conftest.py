import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))

import __graft_entry__ as entry  # noqa: E402

GOLDEN = os.path.join(REPO, "tests", "golden")
LAM = 632.8e-9


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _cuda_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _cuda_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def built():
    """Build libholo.so, the CLI and the oracle once per session (nvcc, no GPU needed)."""
    entry._load_build_module().build()
    import oracle
    oracle.build()
    return True


@pytest.fixture(scope="session")
def holo(built):
    return entry.load_package()


@pytest.fixture(scope="session")
def orc(built):
    import oracle
    return oracle


def grid(n: int, pitch: float, z: float, ny: int | None = None) -> np.ndarray:
    """Centred square (or n x ny) lattice at height z, xyz rows."""
    ny = ny or n
    xs = (np.arange(n) - (n - 1) / 2.0) * pitch
    ys = (np.arange(ny) - (ny - 1) / 2.0) * pitch
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), np.full(n * ny, z)], axis=1)


def chain64(seed: int = 0):
    """64x64 source grid (10 um, z = 0.35 m), 256x256 projector (7.56 um, z = 0)."""
    rng = np.random.default_rng(seed)
    u = grid(64, 10e-6, 0.35)
    v = grid(256, 7.56e-6, 0.0)
    amp = rng.uniform(0.0, 1.0, len(u))
    phase = rng.uniform(0.0, 2 * np.pi, len(u))
    return amp, phase, u, v, u.copy()


def gaussian_blobs(n: int, rng, count: int = 8) -> np.ndarray:
    """Sum of `count` isotropic Gaussian blobs on an n x n grid, normalised to max 1."""
    yy, xx = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    img = np.zeros((n, n))
    for _ in range(count):
        cx, cy = rng.uniform(0, n, 2)
        sigma = rng.uniform(5, 40)
        peak = rng.uniform(0.2, 1.0)
        img += peak * np.exp(-((xx - cx) ** 2 + (yy - cy) ** 2) / (2 * sigma ** 2))
    return (img / img.max()).ravel()


def chain512(seed: int = 0):
    """512x512 sources (Gaussian-blob amplitudes), 1024x1024 projector, z = 512x512."""
    rng = np.random.default_rng(seed)
    u = grid(512, 10e-6, 0.35)
    v = grid(1024, 7.56e-6, 0.0)
    amp = gaussian_blobs(512, rng)
    phase = rng.uniform(0.0, 2 * np.pi, len(u))
    return amp, phase, u, v, u.copy()


def rel_l2(a, b) -> float:
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def max_phase_err(a, b) -> float:
    return float(np.max(np.abs(np.angle(np.asarray(a) / np.asarray(b)))))
