"""The allocation-free scan entry point against the caller-scratch scan.

``sdg_exclusive_scan_static`` keeps its block partials in a fixed device array
of the library; two calls in a row must each give exactly what
``sdg_exclusive_scan`` gives on the same input.  Collected last so that it
also runs after every other test has used the library.
"""

import ctypes as ct

import numpy as np
import pytest

from sand_atlas_dem_gb300 import native

pytestmark = pytest.mark.gpu


def _p(t):
    return ct.c_void_p(t.data_ptr())


def _scan(lib, torch, values, static):
    n = len(values)
    src = torch.from_numpy(values.view(np.int32).copy()).cuda()
    out = torch.full((max(n, 1),), -1, dtype=torch.int32, device="cuda")
    total = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    if static:
        rc = lib.sdg_exclusive_scan_static(_p(src), _p(out), n, _p(total), ct.c_void_p(stream.cuda_stream))
    else:
        partials = torch.zeros(lib.sdg_scan_partials(), dtype=torch.int32, device="cuda")
        rc = lib.sdg_exclusive_scan(_p(src), _p(out), n, _p(total), _p(partials), ct.c_void_p(stream.cuda_stream))
    assert rc == 0, lib.sdg_last_error()
    torch.cuda.synchronize()
    return out.cpu().numpy().view(np.uint32)[:n].copy(), int(total.cpu().numpy().view(np.uint32)[0])


def test_static_scan_matches_scratch_scan_twice(gpu_library):
    import torch

    rng = np.random.default_rng(11)
    first = rng.integers(0, 1000, 3_000_001).astype(np.uint32)
    second = rng.integers(0, 70_000, 155_651).astype(np.uint32)  # a smaller scan right after a larger one
    for values in (first, second):
        got, got_total = _scan(gpu_library, torch, values, static=True)
        want, want_total = _scan(gpu_library, torch, values, static=False)
        np.testing.assert_array_equal(got, want)
        assert got_total == want_total == int(values.astype(np.uint64).sum() & 0xFFFFFFFF)
        np.testing.assert_array_equal(got, (np.cumsum(values.astype(np.uint64)) - values).astype(np.uint32))


def test_static_scan_of_nothing_has_total_zero(gpu_library):
    import torch

    got, total = _scan(gpu_library, torch, np.zeros(0, np.uint32), static=True)
    assert got.size == 0 and total == 0


def test_static_scan_rejects_oversized_input(gpu_library):
    lib = native.load()
    rc = lib.sdg_exclusive_scan_static(ct.c_void_p(16), ct.c_void_p(16), (1 << 30) + 1, None, None)
    assert rc == 1
    assert b"exceeds the limit" in lib.sdg_last_error()
