"""Host-side arithmetic behind bench.py's roofline line: the per-pair pipe work of a
variant (MUFU ops on the XU pipe, FP32 lane-ops on the FMA pipe) from its pair model and
its sin/cos split, and the pipe bound that follows at 16 XU and 128 FMA lanes per clock.
The counts follow the kernels' pair loops: model 3 takes the phase from the tensor cores
(2 MUFU + 3 FP32 per MUFU pair, +13 FP32 and -2 MUFU per pair on the half-turn
polynomial); the CUDA-core model 2 computes it (2 + 8, +16 / -2 on the full-turn one)."""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)

import bench  # noqa: E402


def _variant(holo, v):
    return next(x for x in holo.variants("split32") if x["variant"] == v)


def test_tensor_core_variant_ops_per_pair(holo):
    mufu, fp32 = bench.pipe_ops_per_pair(_variant(holo, 34))  # 6 of 16 pairs polynomial
    assert mufu == pytest.approx(2.0 - 2.0 * 6 / 16)
    assert fp32 == pytest.approx(3.0 + 13.0 * 6 / 16)
    # the XU pipe binds: 16 / 1.25 = 12.8 pairs per clock per SM against 128 / 7.875
    assert 16.0 / mufu == pytest.approx(12.8) and 128.0 / fp32 > 16.0 / mufu


def test_cuda_core_variant_ops_per_pair(holo):
    mufu, fp32 = bench.pipe_ops_per_pair(_variant(holo, 23))  # 1 of 4 targets polynomial
    assert (mufu, fp32) == pytest.approx((1.5, 12.0))
    assert 16.0 / mufu == pytest.approx(128.0 / fp32)  # both pipes bind at once


def test_every_split_variant_has_a_pipe_model(holo):
    for v in holo.variants("split32"):
        mufu, fp32 = bench.pipe_ops_per_pair(v)
        assert 0.0 <= mufu <= 3.0 and 2.0 <= fp32 <= 28.0, v


def test_profile_commands_use_committed_files_and_live_flags():
    """Every command quoted in profiles/ runs bench.py with options it still has."""
    import glob
    import re
    import subprocess
    help_text = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--help"],
                               capture_output=True, text=True, check=True).stdout
    flags = set(re.findall(r"(--[a-z][a-z0-9-]*)", help_text))
    seen = 0
    for path in glob.glob(os.path.join(REPO, "profiles", "*.md")):
        text = open(path).read()
        assert "ncu " in text and "--clock-control none" in text, path
        for cmd in re.findall(r"python (\S+\.py)((?: --?[a-z0-9-]+(?: [0-9]+)?)*)", text):
            script, args = cmd
            assert os.path.exists(os.path.join(REPO, script)), (path, script)
            for flag in re.findall(r"--[a-z][a-z0-9-]*", args):
                assert flag in flags, (path, flag)
            seen += 1
    assert seen >= 4
