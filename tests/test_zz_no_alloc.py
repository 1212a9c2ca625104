"""holo_transform_noalloc: the split-precision transform for callers that cannot
allocate GPU memory (a host that owns the device memory budget, a plugin inside
someone else's allocator, a real-time loop that must not hit cudaMalloc's
implicit synchronisation).  Its scratch is one fixed 64 MiB array in the
library's device code.

Checked through the C ABI on two calls in a row with different problems, against
the allocating entry point (holo_transform, HOLO_SPLIT32) and against the FP64
oracle at the same targets, within the split path's tolerance (rel-L2 <= 1e-5);
the second call must not change the device's free memory.  This file is
collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from conftest import LAM, chain64, rel_l2

pytestmark = pytest.mark.gpu


def _call(lib, amp, phase, u, v, sign, y, stream, device=0):
    return lib.holo_transform_noalloc(device, sign, LAM, amp.data_ptr(), phase.data_ptr(),
                                      u.data_ptr(), amp.numel(), v.data_ptr(), v.numel() // 3,
                                      y.data_ptr(), ctypes.c_void_p(stream))


def test_noalloc_matches_allocating_entry_point_and_oracle(holo, orc):
    import torch
    lib = holo._native.load()
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev).cuda_stream
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a).reshape(-1), device=dev)
    free = []
    rng = np.random.default_rng(5)
    for seed, m, sign in ((0, 65536, -1), (1, 30000, +1)):  # two calls in a row
        amp, phase, u, v, _ = chain64(seed)
        v = v[:m]
        ta, tp, tu, tv = T(amp), T(phase), T(u), T(v)
        y = torch.full((2 * m,), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info(dev)[0])
        rc = _call(lib, ta, tp, tu, tv, sign, y, stream)
        assert rc == 0, lib.holo_last_error_string()
        free.append(torch.cuda.mem_get_info(dev)[0])
        got = y.cpu().numpy().view(np.complex128)
        ref = holo.transform(amp, phase, u, v, sign, LAM, precision="split32")
        assert rel_l2(got, ref) < 1e-5
        idx = np.sort(rng.choice(m, 1024, replace=False))
        exact = orc.transform_subset(amp, phase, u, v, idx, sign, LAM, 8)
        assert rel_l2(got[idx], exact) < 1e-5
    assert free[2] == free[3]  # the second call allocated nothing


def test_noalloc_rejects_problems_beyond_its_scratch(holo):
    import torch
    lib = holo._native.load()
    dev = torch.device("cuda:0")
    small = torch.zeros(12, dtype=torch.float64, device=dev)
    # sizes checked on the host before any device work: 4M x 4M needs > 64 MiB
    rc = lib.holo_transform_noalloc(0, -1, LAM, small.data_ptr(), small.data_ptr(),
                                    small.data_ptr(), 4 << 20, small.data_ptr(), 4 << 20,
                                    small.data_ptr(), None)
    assert rc == -1 and b"no-alloc scratch" in lib.holo_last_error_string()
    host = np.zeros(12)
    rc = lib.holo_transform_noalloc(0, -1, LAM, host.ctypes.data, host.ctypes.data,
                                    host.ctypes.data, 1, host.ctypes.data, 1, host.ctypes.data,
                                    None)
    assert rc == -1 and b"device pointers" in lib.holo_last_error_string()


def test_noalloc_rejects_memory_of_another_device(holo):
    """Device memory of GPU 0 handed to a call on GPU 1 is refused before any work
    (the path enables no peer access).  Needs two GPUs."""
    import torch
    if torch.cuda.device_count() < 2:
        pytest.skip("needs two GPUs")
    lib = holo._native.load()
    small = torch.zeros(12, dtype=torch.float64, device="cuda:0")
    rc = lib.holo_transform_noalloc(1, -1, LAM, small.data_ptr(), small.data_ptr(),
                                    small.data_ptr(), 1, small.data_ptr(), 1, small.data_ptr(),
                                    None)
    assert rc == -1 and b"device pointers of device 1" in lib.holo_last_error_string()


def test_noalloc_refuses_a_stream_under_capture(holo):
    """The call waits for its stream partway, so a stream being captured into a graph is
    refused before anything is queued (the capture then ends empty)."""
    import torch
    lib = holo._native.load()
    dev = torch.device("cuda:0")
    amp, phase, u, v, _ = chain64(0)
    v = v[:4096]
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a).reshape(-1), device=dev)
    ta, tp, tu, tv = T(amp), T(phase), T(u), T(v)
    y = torch.zeros(2 * len(v), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    s = torch.cuda.Stream(dev)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        rc = _call(lib, ta, tp, tu, tv, -1, y, s.cuda_stream)
    assert rc == -1 and b"captured" in lib.holo_last_error_string()
    # the stream is usable afterwards: the same call outside the capture succeeds
    rc = _call(lib, ta, tp, tu, tv, -1, y, torch.cuda.current_stream(dev).cuda_stream)
    assert rc == 0, lib.holo_last_error_string()
    assert torch.count_nonzero(y).item() > 0
