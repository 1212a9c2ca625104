"""The reference's file interface on the CPU (io.py): raw little-endian FP64 .dat arrays
(cuda/util.h:249-283, 296-322), the input set of a -f directory with w0_0.dat or the
reference's w0.dat, and out.json as one JSON object per line (py/util.py:685-700)."""
import json
import os

import numpy as np
import pytest


def test_dat_is_raw_little_endian_fp64(holo, tmp_path):
    p = str(tmp_path / "a.dat")
    holo.io.write_dat(p, [1.0, -2.5])
    assert open(p, "rb").read() == np.array([1.0, -2.5], dtype="<f8").tobytes()
    assert open(p, "rb").read()[:8] == b"\x00\x00\x00\x00\x00\x00\xf0\x3f"
    rng = np.random.default_rng(0)
    x = rng.standard_normal(1001)
    holo.io.write_dat(p, x)
    assert np.array_equal(holo.io.read_dat(p), x)  # bit for bit
    empty = str(tmp_path / "e.dat")
    open(empty, "wb").close()
    with pytest.raises(ValueError):
        holo.io.read_dat(empty)
    with pytest.raises(FileNotFoundError):
        holo.io.read_dat(str(tmp_path / "missing.dat"))


def test_input_set_round_trip_and_w_fallback(holo, tmp_path):
    rng = np.random.default_rng(1)
    n, m, p = 7, 11, 5
    amp, phase = rng.uniform(0, 1, n), rng.uniform(0, 2 * np.pi, n)
    u, v, w = (rng.standard_normal((k, 3)) for k in (n, m, p))
    d = str(tmp_path / "in")
    holo.io.write_inputs(d, amp, phase, u, v, w)
    got = holo.io.read_inputs(d, projection=True)
    for key, ref in (("x0_amp", amp), ("x0_phase", phase), ("u0", u), ("v0", v), ("w0_0", w)):
        assert np.array_equal(got[key], np.ravel(ref)), key
    # the reference's own name for the projection points, used when w0_0.dat is absent
    os.remove(os.path.join(d, "w0_0.dat"))
    holo.io.write_dat(os.path.join(d, "w0.dat"), w[:2])
    assert np.array_equal(holo.io.read_inputs(d, projection=True)["w0_0"], np.ravel(w[:2]))
    # w0_0.dat wins when both exist
    holo.io.write_dat(os.path.join(d, "w0_0.dat"), w)
    assert holo.io.read_inputs(d, projection=True)["w0_0"].size == 3 * p
    os.remove(os.path.join(d, "w0_0.dat"))
    os.remove(os.path.join(d, "w0.dat"))
    with pytest.raises(FileNotFoundError):
        holo.io.read_inputs(d, projection=True)
    assert "w0_0" not in holo.io.read_inputs(d)


def test_input_set_rejects_inconsistent_sizes(holo, tmp_path):
    rng = np.random.default_rng(2)
    d = str(tmp_path / "bad")
    holo.io.write_inputs(d, np.ones(4), np.zeros(4), rng.standard_normal((4, 3)),
                         rng.standard_normal((6, 3)))
    holo.io.write_dat(os.path.join(d, "x0_phase.dat"), np.zeros(3))  # 3 phases, 4 amplitudes
    with pytest.raises(ValueError):
        holo.io.read_inputs(d)
    holo.io.write_dat(os.path.join(d, "x0_phase.dat"), np.zeros(4))
    holo.io.write_dat(os.path.join(d, "v0.dat"), np.zeros(10))  # not xyz triples
    with pytest.raises(ValueError):
        holo.io.read_inputs(d)


def test_out_json_one_object_per_line(holo, tmp_path):
    p = tmp_path / "out.json"
    rows = [{"phasor": "x0", "n": 4}, {"phasor": "y0", "dt": 0.5, "flops": 1.2e12}]
    p.write_text("\n".join(json.dumps(r) for r in rows[:1]) + "\n\n" + json.dumps(rows[1]) + "\n")
    assert holo.io.parse_out_json(str(p)) == rows
