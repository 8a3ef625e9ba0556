"""The allocation-free Morton argsort, checked against the allocating one.

bhut_morton_argsort_noalloc is for callers that cannot call cudaMalloc --
their GPU memory belongs to another allocator, or they run a step loop in
which an allocation would synchronize the device.  It keeps its scratch in
one static device array, so this test calls it twice in a row (the second
call finds the first call's leftovers in the array) and compares both
results with bhut_morton_argsort, bit for bit (keys and permutation are
integers).  The file name sorts last so that a run stopping at the first
failure has run every other test before this one.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_POINTS = 1 << 20


def _cases():
    from bhut_gb300 import workloads
    yield workloads.plummer(100_003, seed=21)[0]
    yield workloads.gaussian(4097, seed=22, dim=2)[0]
    yield workloads.plummer(MAX_POINTS, seed=23)[0]
    # one key (the sort returns at once: keys and perm are written by the
    # Morton kernel), two keys, one short of a 4096-key sort tile
    yield workloads.gaussian(1, seed=24)[0]
    yield workloads.gaussian(2, seed=25)[0]
    yield workloads.gaussian(4095, seed=26)[0]


def _call(L, pos, stream=None):
    import torch
    n, dim = pos.shape
    pos_d = torch.from_numpy(pos).cuda()
    keys_d = torch.empty(n, dtype=torch.int64, device="cuda")
    perm_d = torch.empty(n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = L.bhut_morton_argsort_noalloc(pos_d.data_ptr(), n, dim, keys_d.data_ptr(),
                                       perm_d.data_ptr(),
                                       None if stream is None else stream.cuda_stream)
    torch.cuda.synchronize()
    return rc, keys_d.cpu().numpy().view(np.uint64), perm_d.cpu().numpy().astype(np.int64)


def test_noalloc_argsort_matches_allocating_entry_point(engine_lib):
    import torch

    import bhut_gb300 as bh
    from bhut_gb300 import _lib

    L = _lib.load()
    cases = list(_cases())
    side = torch.cuda.Stream()
    for call in range(2):
        for pos in cases:
            n, dim = pos.shape
            # second round on a non-default stream
            rc, got_keys, got_perm = _call(L, pos, side if call else None)
            assert rc == _lib.BHUT_OK, _lib.last_error()
            ref_keys, ref_perm = bh.morton_argsort(pos)
            assert np.array_equal(got_keys, ref_keys), (call, n, dim)
            assert np.array_equal(got_perm, ref_perm), (call, n, dim)


def test_noalloc_argsort_reports_nonfinite_then_recovers(engine_lib):
    import bhut_gb300 as bh
    from bhut_gb300 import _lib, workloads

    L = _lib.load()
    pos = workloads.plummer(5000, seed=27)[0]
    bad = pos.copy()
    bad[1234, 1] = np.nan
    rc, _, _ = _call(L, bad)
    assert rc == _lib.BHUT_EINVAL and "finite" in _lib.last_error()
    # the error word lives in the shared static array: the next call clears it
    rc, keys, perm = _call(L, pos)
    assert rc == _lib.BHUT_OK, _lib.last_error()
    ref_keys, ref_perm = bh.morton_argsort(pos)
    assert np.array_equal(keys, ref_keys) and np.array_equal(perm, ref_perm)


def test_noalloc_argsort_rejects_oversize_and_host_pointers(engine_lib):
    import torch

    from bhut_gb300 import _lib

    L = _lib.load()
    n = MAX_POINTS + 1
    pos_d = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    keys_d = torch.empty(n, dtype=torch.int64, device="cuda")
    perm_d = torch.empty(n, dtype=torch.int32, device="cuda")
    rc = L.bhut_morton_argsort_noalloc(pos_d.data_ptr(), n, 3, keys_d.data_ptr(),
                                       perm_d.data_ptr(), None)
    assert rc == _lib.BHUT_EINVAL and "limit" in _lib.last_error()
    host = np.zeros((16, 3))
    rc = L.bhut_morton_argsort_noalloc(host.ctypes.data, 16, 3, keys_d.data_ptr(),
                                       perm_d.data_ptr(), None)
    assert rc == _lib.BHUT_EINVAL and "device pointers" in _lib.last_error()


def test_noalloc_argsort_rejects_memory_of_another_device(engine_lib):
    """Memory of a second GPU is refused on the host, before any launch."""
    import torch

    from bhut_gb300 import _lib

    if torch.cuda.device_count() < 2:
        pytest.skip("needs two GPUs")
    L = _lib.load()
    n = 64
    pos_other = torch.zeros((n, 3), dtype=torch.float64, device="cuda:1")
    keys_d = torch.empty(n, dtype=torch.int64, device="cuda:0")
    perm_d = torch.empty(n, dtype=torch.int32, device="cuda:0")
    with torch.cuda.device(0):
        rc = L.bhut_morton_argsort_noalloc(pos_other.data_ptr(), n, 3, keys_d.data_ptr(),
                                           perm_d.data_ptr(), None)
    assert rc == _lib.BHUT_EINVAL and "current device" in _lib.last_error()
