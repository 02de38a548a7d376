"""GPU test of evoc_knn_to_csr_noalloc, the entry point that allocates nothing.

It serves callers that must not allocate device memory while they run, for
example services that reserve their device-memory budget up front, or host
frameworks that own the device heap and forbid operators to call cudaMalloc.
Its scratch lives in one fixed device array inside the library. The caller
passes inputs, outputs and a stream.

The result must equal, bit for bit, the weighted directed graph of the
allocating entry point (evoc_fuzzy_set_device with symmetrise = 0). Three
calls in a row (A, B, A) check that the shared scratch keeps no state between
calls that changes a result. This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(seed: int, n: int, k: int):
    rng = np.random.default_rng(seed)
    idx = rng.integers(0, n, size=(n, k)).astype(np.uint32)
    idx[:, 0] = np.arange(n)                     # self loops are dropped
    idx[::5, 3] = idx[::5, 2]                    # duplicates are kept
    lens = rng.integers(1, k + 1, size=n)
    for i in range(0, n, 3):
        idx[i, lens[i]:] = 0xFFFFFFFF            # ragged rows
    dist = np.sort(rng.uniform(0.0, 2.0, size=(n, k)).astype(np.float32), axis=1)
    return idx, dist


def _noalloc(lib, d_idx, d_dist, n, k, eff, capacity):
    import torch
    indptr = torch.empty(n + 1, dtype=torch.int64, device="cuda")
    indices = torch.empty(max(capacity, 1), dtype=torch.int32, device="cuda")
    weights = torch.empty(max(capacity, 1), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    nnz = C.c_int64(-1)
    rc = lib.evoc_knn_to_csr_noalloc(d_idx.data_ptr(), d_dist.data_ptr(), n, k, eff,
                                     indptr.data_ptr(), indices.data_ptr(), weights.data_ptr(),
                                     capacity, C.byref(nnz), None)
    return rc, nnz.value, indptr, indices, weights


def test_noalloc_matches_allocating_entry_point(ctx):
    import torch
    import evoc_gb300 as E
    lib = E.load_library()
    cases = [(11, 3000, 16, 16.0), (12, 1777, 9, 7.5), (11, 3000, 16, 16.0)]
    for seed, n, k, eff in cases:
        idx, dist = _inputs(seed, n, k)
        d_idx = torch.from_numpy(idx.view(np.int32)).cuda()
        d_dist = torch.from_numpy(dist).cuda()
        ref = ctx.fuzzy_set_device(d_idx.data_ptr(), d_dist.data_ptr(), n, k, eff,
                                   symmetrise=False)
        rip, rix, rw = ref.export()
        rc, nnz, indptr, indices, weights = _noalloc(lib, d_idx, d_dist, n, k, eff, n * k)
        assert rc == E.EVOC_OK, lib.evoc_last_error(None).decode()
        assert nnz == len(rix)
        assert np.array_equal(indptr.cpu().numpy(), rip)
        assert np.array_equal(indices[:nnz].cpu().numpy().view(np.uint32), rix)
        assert np.array_equal(weights[:nnz].cpu().numpy().view(np.uint32), rw.view(np.uint32))


def test_noalloc_call_allocates_no_device_memory(ctx):
    """After a first call (which loads the code and places the scratch array),
    a call with fresh inputs leaves the device's free memory unchanged."""
    import torch
    import evoc_gb300 as E
    lib = E.load_library()
    n, k = 2500, 12
    bufs = []
    for seed in (31, 32):
        idx, dist = _inputs(seed, n, k)
        bufs.append((torch.from_numpy(idx.view(np.int32)).cuda(), torch.from_numpy(dist).cuda()))
    indptr = torch.empty(n + 1, dtype=torch.int64, device="cuda")
    indices = torch.empty(n * k, dtype=torch.int32, device="cuda")
    weights = torch.empty(n * k, dtype=torch.float32, device="cuda")
    nnz = C.c_int64(-1)

    def call(d_idx, d_dist):
        return lib.evoc_knn_to_csr_noalloc(d_idx.data_ptr(), d_dist.data_ptr(), n, k, float(k),
                                           indptr.data_ptr(), indices.data_ptr(),
                                           weights.data_ptr(), n * k, C.byref(nnz), None)

    assert call(*bufs[0]) == E.EVOC_OK
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    assert call(*bufs[1]) == E.EVOC_OK
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before


def test_noalloc_rejects_oversize_and_small_capacity(ctx):
    import torch
    import evoc_gb300 as E
    lib = E.load_library()
    idx, dist = _inputs(3, 500, 8)
    d_idx = torch.from_numpy(idx.view(np.int32)).cuda()
    d_dist = torch.from_numpy(dist).cuda()
    too_many = (E.NOALLOC_SCRATCH_BYTES - 256) // 16 + 1
    rc, *_ = _noalloc(lib, d_idx, d_dist, too_many, 1, 1.0, 1)  # rejected before any access
    assert rc == E.EVOC_ERR_UNSUPPORTED
    assert b"no-allocation limit" in lib.evoc_last_error(None)
    rc, nnz, *_ = _noalloc(lib, d_idx, d_dist, 500, 8, 8.0, 10)
    assert rc == E.EVOC_ERR_INVALID_ARGUMENT
    rc, nnz, *_ = _noalloc(lib, d_idx, d_dist, 500, 8, 8.0, 500 * 8)
    assert rc == E.EVOC_OK and nnz > 10
