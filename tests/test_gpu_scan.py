"""The device exclusive scan against exact integer sums (``gpu.py:65-91``)."""

import ctypes as ct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run_scan(lib, torch, values):
    n = len(values)
    src = torch.tensor(values.astype(np.int64), dtype=torch.int64).to(torch.int32).cuda()
    out = torch.zeros(max(n, 1), dtype=torch.int32, device="cuda")
    total = torch.zeros(1, dtype=torch.int32, device="cuda")
    partials = torch.zeros(lib.sdg_scan_partials(), dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    rc = lib.sdg_exclusive_scan(ct.c_void_p(src.data_ptr()), ct.c_void_p(out.data_ptr()), n,
                                ct.c_void_p(total.data_ptr()), ct.c_void_p(partials.data_ptr()),
                                ct.c_void_p(stream.cuda_stream))
    assert rc == 0, lib.sdg_last_error()
    torch.cuda.synchronize()
    return out.cpu().numpy().view(np.uint32)[:n], int(total.cpu().numpy().view(np.uint32)[0])


@pytest.mark.parametrize("n", [1, 777, 256 * 608 + 5, 3_000_001])
def test_exclusive_scan_matches_cumsum(gpu_library, n):
    import torch

    values = (np.arange(n, dtype=np.uint64) % 17).astype(np.uint32)
    out, total = run_scan(gpu_library, torch, values)
    expected = np.cumsum(values.astype(np.uint64)) - values
    np.testing.assert_array_equal(out, expected.astype(np.uint32))
    assert total == int(values.astype(np.uint64).sum())
