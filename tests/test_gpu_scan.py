"""bora_scan_u32: the device exclusive prefix sum of the sparse-frame rebuild, through
the C ABI, against numpy."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [0, 1, 7, 2047, 2048, 2049, 100003, 5_000_000])
def test_scan_matches_numpy(gpu, n):
    import torch
    lib = gpu.load()
    rng = np.random.default_rng(n)
    host = rng.integers(0, 1000, size=n, dtype=np.uint32)
    d_in = torch.from_numpy(host.astype(np.int64)).to(torch.int32).cuda() if n else torch.zeros(1, dtype=torch.int32, device="cuda")
    d_out = torch.full((max(n, 1),), -1, dtype=torch.int32, device="cuda")
    d_tot = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    assert lib.bora_scan_u32(ctypes.c_void_p(d_in.data_ptr()), ctypes.c_void_p(d_out.data_ptr()), n,
                             ctypes.c_void_p(d_tot.data_ptr()), ctypes.c_void_p(st)) == 0
    torch.cuda.synchronize()
    expect = np.concatenate([[0], np.cumsum(host.astype(np.uint64))[:-1]]).astype(np.uint32) if n else np.zeros(0)
    got = d_out.cpu().numpy().astype(np.uint32)[:n]
    np.testing.assert_array_equal(got, expect)
    assert int(d_tot.cpu().numpy().astype(np.uint32)[0]) == int(host.astype(np.uint64).sum() & 0xFFFFFFFF)


def test_scan_in_place_and_no_total(gpu):
    import torch
    lib = gpu.load()
    host = np.arange(1, 4097, dtype=np.int32)
    d = torch.from_numpy(host).cuda()
    assert lib.bora_scan_u32(ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(d.data_ptr()), host.size, None,
                             ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)) == 0
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d.cpu().numpy(), np.concatenate([[0], np.cumsum(host)[:-1]]))


def test_scan_rejects_null(gpu):
    lib = gpu.load()
    assert lib.bora_scan_u32(None, None, 10, None, None) == -1
