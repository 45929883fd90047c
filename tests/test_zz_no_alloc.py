"""bora_scan_u32_noalloc: the prefix sum for callers that cannot allocate device memory
(fixed-budget plugin hosts, graph-recorded code, real-time callbacks). Its per-block
scratch is a static device array shared by all calls, so this test calls it twice in a
row - a large input, then a smaller one over the first call's leftovers - and compares
each result with the allocating entry point bora_scan_u32 on the same input (integer
results: exact). Collected last so that a failure here leaves every other test run."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scan(lib, fn, d_in, n):
    import torch
    d_out = torch.full((max(n, 1),), -7, dtype=torch.int32, device="cuda")
    d_tot = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    status = getattr(lib, fn)(ctypes.c_void_p(d_in.data_ptr()), ctypes.c_void_p(d_out.data_ptr()), n,
                              ctypes.c_void_p(d_tot.data_ptr()), ctypes.c_void_p(st))
    torch.cuda.synchronize()
    return status, d_out.cpu().numpy()[:n], int(d_tot.cpu().numpy()[0])


def test_noalloc_scan_matches_allocating_scan(gpu):
    import torch
    lib = gpu.load()
    rng = np.random.default_rng(20261203)
    for n in (3_000_001, 4097):  # second call smaller: stale block sums must not leak in
        host = rng.integers(0, 500, size=n).astype(np.int32)
        d_in = torch.from_numpy(host).cuda()
        s_ref, out_ref, tot_ref = _scan(lib, "bora_scan_u32", d_in, n)
        s_new, out_new, tot_new = _scan(lib, "bora_scan_u32_noalloc", d_in, n)
        assert s_ref == 0 and s_new == 0
        np.testing.assert_array_equal(out_new, out_ref)
        assert tot_new == tot_ref == int(host.astype(np.int64).sum())


def test_noalloc_scan_rejects_oversize(gpu):
    lib = gpu.load()
    # checked before any pointer is touched
    assert lib.bora_scan_u32_noalloc(ctypes.c_void_p(16), ctypes.c_void_p(16), (1 << 28) + 1, None, None) == -6
