"""The device tilings (csrc/tiler.cu) against NumPy models of the same algorithms.

The tile order decides which points share a tile and so the split kernels' error
bound; the models below restate both tilings step by step -- the Hilbert order of a
64 x 64 cell grid, and strip packing into super tiles of 8192 by stable sorts of
quantised coordinates followed by recursive bisection with 64-bit keys -- and the
library's orders must equal them exactly.  This is test infrastructure: the library
never calls it.
"""
import math

import numpy as np
import pytest

from conftest import LAM, grid, rel_l2

pytestmark = pytest.mark.gpu

CELLS, SUPER, LEAF = 4096, 8192, 256


def _widest_axes(lo, hi):
    ext = hi - lo
    x, y, z = 0, 1, 2
    if ext[y] > ext[x]:
        x, y = y, x
    if ext[z] > ext[y]:
        y, z = z, y
    if ext[y] > ext[x]:
        x, y = y, x
    return x, y


def _axis_keys(p, lo, hi, a):
    ext = hi[a] - lo[a]
    sc = CELLS / ext if ext > 0 else 0.0
    return np.clip(((p[:, a] - lo[a]) * sc).astype(np.int64), 0, CELLS - 1)


def _strip_points(lo, hi, n):
    a0, a1 = _widest_axes(lo, hi)
    e0, e1 = hi[a0] - lo[a0], hi[a1] - lo[a1]
    nsup = (n + SUPER - 1) // SUPER
    aspect = max(e1 / e0, 1e-9) if e0 > 0 else 1.0
    strips = math.floor(math.sqrt(nsup / aspect) + 0.5)
    strips = max(1, min(strips, min(nsup, CELLS)))
    return (nsup + strips - 1) // strips * SUPER


def _ordered_bits(f32):
    b = f32.view(np.uint32).astype(np.uint64)
    return np.where(b & 0x80000000, (~b) & 0xFFFFFFFF, b | 0x80000000)


def _segment(i, nl, level):
    s, l = 0, nl
    for _ in range(level):
        if l <= LEAF:
            break
        unit = 1 << ((l - 1).bit_length() - 1)
        if i < s + unit:
            l = unit
        else:
            s, l = s + unit, l - unit
    return s, l


def _local_bisect(p, idx):
    nl = len(idx)
    ref = p[idx[0]]
    for level in range(5):
        segs = [_segment(i, nl, level) for i in range(nl)]
        rel = (p[idx] - ref).astype(np.float32)
        keys = np.zeros(nl, dtype=np.uint64)
        by_start = {}
        for i, (st, ln) in enumerate(segs):
            by_start.setdefault((st, ln), []).append(i)
        for (st, ln), members in by_start.items():
            members = np.array(members)
            c = np.zeros(len(members), dtype=np.uint64)
            if ln > LEAF:
                q = rel[members]
                ext = q.max(0) - q.min(0)
                a, e = 0, np.float32(-1)
                for d in range(3):
                    if ext[d] > e:
                        a, e = d, ext[d]
                c = _ordered_bits(np.ascontiguousarray(q[:, a]))
            keys[members] = (np.uint64(st) << np.uint64(45)) | (c << np.uint64(13)) | \
                members.astype(np.uint64)
        idx = idx[np.argsort(keys, kind="stable")]
    return idx


def model_order(p):
    n = len(p)
    if n <= SUPER:
        order = np.arange(n)
    else:
        lo, hi = p.min(0), p.max(0)
        a0, a1 = _widest_axes(lo, hi)
        ox = np.argsort(_axis_keys(p, lo, hi, a0), kind="stable")
        strip = np.empty(n, dtype=np.int64)
        strip[ox] = np.arange(n) // _strip_points(lo, hi, n)
        oy = np.argsort(_axis_keys(p, lo, hi, a1), kind="stable")
        order = oy[np.argsort(strip[oy], kind="stable")]
    out = [_local_bisect(p, order[b:b + SUPER]) for b in range(0, n, SUPER)]
    return np.concatenate(out)


def _hilbert_d(n, x, y):
    d = np.zeros_like(x)
    s = n // 2
    while s > 0:
        rx = ((x & s) > 0).astype(np.int64)
        ry = ((y & s) > 0).astype(np.int64)
        d += s * s * ((3 * rx) ^ ry)
        flip = (ry == 0) & (rx == 1)
        x = np.where(flip, n - 1 - x, x)
        y = np.where(flip, n - 1 - y, y)
        swap = ry == 0
        x, y = np.where(swap, y, x), np.where(swap, x, y)
        s //= 2
    return d


def hilbert_model_order(p, cells=64):
    lo, hi = p.min(0), p.max(0)
    a0, a1 = _widest_axes(lo, hi)
    e0, e1 = hi[a0] - lo[a0], hi[a1] - lo[a1]
    s0 = cells / e0 if e0 > 0 else 0.0
    s1 = cells / e1 if e1 > 0 else 0.0
    cx = np.clip(((p[:, a0] - lo[a0]) * s0).astype(np.int64), 0, cells - 1)
    cy = np.clip(((p[:, a1] - lo[a1]) * s1).astype(np.int64), 0, cells - 1)
    return np.argsort(_hilbert_d(cells, cx, cy), kind="stable")


def _point_sets():
    rng = np.random.default_rng(3)
    s = rng.uniform(-1.5e-3, 1.5e-3, (30000, 2))
    yield "grid 203x203 (odd)", grid(203, 10e-6, 0.3)
    yield "grid 97x97, 8192 points (one super tile)", grid(97, 10e-6, 0.3)[:8192]
    yield "grid 50x50 (a partial super tile)", grid(50, 10e-6, 0.3)
    yield "grid 40000 of 200x200", grid(200, 7.56e-6, 0.0)
    yield "random cloud", np.column_stack([s, np.full(len(s), 0.3)])
    yield "tilted 3-D", np.column_stack([s[:20000, 0], s[:20000, 1],
                                          0.25 + 0.3 * s[:20000, 0]])
    dup = grid(64, 10e-6, 0.3)
    yield "duplicated points", np.concatenate([dup, dup, dup, dup])[:15000]
    yield "wide strip", np.column_stack([rng.uniform(-8e-3, 8e-3, 24000),
                                         rng.uniform(-2e-4, 2e-4, 24000), np.full(24000, 0.2)])
    yield "8193 points (a one-point super tile)", grid(91, 10e-6, 0.3)[:8193]
    yield "10000 identical points", np.tile([[1e-4, -2e-4, 0.3]], (10000, 1))


def _fastest_build(holo, variant):
    """The planner's first choice: the tensor-core phase (pair model 3) on 1024-source
    tiles."""
    v = next(x for x in holo.variants("split32") if x["variant"] == variant)
    return v["pair_model"] == 3 and v["source_tile"] == 1024


@pytest.mark.parametrize("name,pts", list(_point_sets()),
                         ids=lambda x: x if isinstance(x, str) else "")
def test_tile_orders_match_models(holo, name, pts):
    for tiling, model in (("packed", model_order), ("hilbert", hilbert_model_order)):
        order = holo.tile_order(pts, tiling)
        assert np.array_equal(np.sort(order), np.arange(len(pts))), (tiling, "not a permutation")
        np.testing.assert_array_equal(order, model(pts), err_msg=tiling)


def test_packed_tiles_are_compact(holo):
    """On a 203 x 203 grid (10 um) every packed tile of 1024 / 512 / 256 points spans at
    most 1.4 / 1.5 / 1.4 times the side of a square of that many points (1.28 / 1.33 /
    1.25 here; the Hilbert runs reach 1.7 for the tiles of 1024)."""
    pts = grid(203, 10e-6, 0.3)
    ps = pts[holo.tile_order(pts, "packed")]
    for cs, lim in ((1024, 1.4), (512, 1.5), (256, 1.4)):
        side = math.sqrt(cs) * 10e-6
        worst = max(np.max(ps[i:i + cs, :2].max(0) - ps[i:i + cs, :2].min(0))
                    for i in range(0, len(ps) - cs + 1, cs))
        assert worst <= lim * side, (cs, worst / side)


def test_planner_retiles_where_hilbert_tiles_fail(holo, orc):
    """15838 sources 0.355 m above a 128^2 grid: on Hilbert tiles the bound rules out the
    1024-source tensor-core build (it takes the 512-source one), on packed tiles it holds,
    so the plan keeps the packed tiling and the faster build.  The 64^2 chain's planes keep
    the Hilbert tiles."""
    u = grid(126, 10e-6, 0.355)[:15838]
    v = grid(128, 7.56e-6, 0.0)
    with holo.Plan(u, v, "split32") as pl:
        info, tiling = pl.info(), pl.tiling()
        order = pl.order(0)
    assert tiling == {"sources": "packed", "targets": "packed"}, tiling
    assert _fastest_build(holo, info["variant"]) and info["path_error_bound_m"] <= 3.2e-13, info
    np.testing.assert_array_equal(order, model_order(u))
    # and the transform on those tiles meets the split path's tolerance
    rng = np.random.default_rng(5)
    amp, phase = rng.uniform(0, 1, len(u)), rng.uniform(0, 2 * np.pi, len(u))
    idx = np.arange(0, len(v), 41)
    for sign in (-1, 1):
        with holo.Plan(u, v, "split32") as pl:
            y = pl.execute(amp, phase, sign, LAM)
        y = y.cpu().numpy() if hasattr(y, "cpu") else np.asarray(y)
        ref = orc.transform_subset(amp, phase, u, v, idx, sign, LAM)
        assert rel_l2(y[idx], ref) < 1e-5, sign
    with holo.Plan(grid(64, 10e-6, 0.35), grid(256, 7.56e-6, 0.0), "split32") as pl:
        assert pl.tiling() == {"sources": "hilbert", "targets": "hilbert"}
        assert _fastest_build(holo, pl.info()["variant"])
    with holo.Plan(grid(64, 10e-6, 0.35), grid(64, 7.56e-6, 0.0), "fp64") as pl:
        assert pl.tiling() == {"sources": "none", "targets": "none"}
