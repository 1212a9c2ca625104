"""The builder-warp tensor-core kernel (operands, carries and results by warps of their own,
blocks source block outer, no block-wide barrier between tile pairs) against the same build
in the kernel that stops between tile pairs to build their operands.  Both run the same
tile pairs, MMAs and pair loop; the builder-warp kernel adds each block's sums into the
partial sums on their own, so the fields agree to float32 rounding.  The cases give every
work item many tile pairs (the hand-offs run through the item) and several items per CTA
(they run across item boundaries), single problems and a batch drained by a work queue."""
import math

import numpy as np
import pytest

from conftest import LAM, grid, rel_l2

pytestmark = pytest.mark.gpu

# builder-warp variant -> the same build in the other kernel (1024-, 768-, 512-, 256-source
# tiles)
PAIRS = {73: 58, 74: 71, 75: 67, 76: 69}


def _variants(holo):
    return {v["variant"]: v for v in holo.variants("split32")}


def test_pairs_differ_only_in_the_kernel(holo):
    vs = _variants(holo)
    for a, b in PAIRS.items():
        va, vb = dict(vs[a]), dict(vs[b])
        assert va.pop("variant") == a and vb.pop("variant") == b
        assert va == vb, (va, vb)  # the kernel flag is not among the described fields
        assert va["pair_loop"] == 3


def test_planner_prefers_the_builder_warp_kernel(holo):
    # 512^2 sources 0.35 m above 1024^2 targets: 1024-source tiles hold the bound
    u = grid(512, 10e-6, 0.35)
    v = grid(1024, 7.56e-6, 0.0)
    with holo.Plan(u, v, "split32") as pl:
        assert pl.info()["variant"] == 73


@pytest.mark.parametrize("var,base", sorted(PAIRS.items()))
def test_builder_warps_on_long_items(holo, orc, var, base):
    rng = np.random.default_rng(var)
    u = grid(192, 10e-6, 0.35)  # 36864 sources: 36 tiles of 1024 .. 144 of 256
    v = grid(512, 7.56e-6, 0.0)  # 262144 targets: 512 tiles of 512
    amp, phase = rng.uniform(0, 1, len(u)), rng.uniform(0, 2 * np.pi, len(u))
    sign = -1 if var % 2 else 1
    h = holo.handle(0)
    bucket = holo.size_bucket(len(u), len(v))
    saved = h.get_variant("split32", bucket)
    try:
        h.set_variant("split32", bucket, var)
        with holo.Plan(u, v, "split32") as pl:
            info = pl.info()
    finally:
        h.set_variant("split32", bucket, saved)
    assert info["variant"] == var, info
    cs = _variants(holo)[var]["source_tile"]
    # the work items run over many source tiles each
    assert math.ceil(len(u) / cs) / info["splits"] >= 8, info
    y = {k: holo.transform(amp, phase, u, v, sign, LAM, precision="split32", variant=k)
         for k in (var, base)}
    assert rel_l2(y[var], y[base]) < 2e-6
    idx = np.arange(0, len(v), 211)
    assert rel_l2(y[var][idx], orc.transform_subset(amp, phase, u, v, idx, sign, LAM)) < 1e-5


def test_builder_warps_on_short_items(holo, orc):
    """One to six source tiles per item, several items per CTA (1500 sources -> 300000
    targets)."""
    rng = np.random.default_rng(5)
    u = grid(40, 10e-6, 0.3)[:1500]
    v = grid(548, 7.56e-6, 0.0)[:300000]
    amp, phase = rng.uniform(0, 1, len(u)), rng.uniform(0, 2 * np.pi, len(u))
    idx = np.arange(0, len(v), 97)
    ref = orc.transform_subset(amp, phase, u, v, idx, 1, LAM)
    for var, base in sorted(PAIRS.items()):
        ya = holo.transform(amp, phase, u, v, 1, LAM, precision="split32", variant=var)
        yb = holo.transform(amp, phase, u, v, 1, LAM, precision="split32", variant=base)
        assert rel_l2(ya, yb) < 2e-6, var
        assert rel_l2(ya[idx], ref) < 1e-5, var


def test_builder_warps_batched(holo):
    """A batch of uneven problems through the work-queue kernel, with the builder-warp build
    and with the other kernel (chosen through the handle's variant table for every size
    bucket)."""
    import torch
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(17)
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a).reshape(-1), device=dev)
    cases = []
    for i, ns in enumerate((3000, 20000, 65536, 9000)):
        u = grid(int(math.ceil(math.sqrt(ns))), 10e-6, 0.4 + 0.05 * i)[:ns]
        v = grid((128, 256, 384, 200)[i], 7.56e-6, 0.0)
        cases.append((rng.uniform(0, 1, ns), rng.uniform(0, 2 * np.pi, ns), u, v,
                      -1 if i % 2 else 1))
    h = holo.handle(0)
    saved = [h.get_variant("split32", b) for b in range(8)]
    out = {}
    try:
        for var in (73, 58):
            for b in range(8):
                h.set_variant("split32", b, var)
            for _, _, u, v, _ in cases:
                with holo.Plan(u, v, "split32") as pl:
                    assert pl.info()["variant"] == var
            probs = [holo.Problem(T(a), T(p), T(u), T(v), s, LAM,
                                  torch.zeros(2 * len(v), dtype=torch.float64, device=dev))
                     for a, p, u, v, s in cases]
            with holo.Batch(probs, "split32") as bt:
                bt.execute()
                torch.cuda.synchronize()
                bt.execute()  # replay of the captured graph
                torch.cuda.synchronize()
            out[var] = [pb.y.cpu().numpy().view(np.complex128) for pb in probs]
    finally:
        for b, s in enumerate(saved):
            h.set_variant("split32", b, s)
    for ya, yb in zip(out[73], out[58]):
        assert rel_l2(ya, yb) < 2e-6
    holo.handle(0).status()
