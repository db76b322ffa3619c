"""fe_scan_counts_noalloc, the allocation-free row-pointer scan, against the scan
behind fe_export_csr.

Who this entry point is for: callers that may not allocate device memory themselves
-- their buffers come from another owner's pool, or a cudaMalloc on their path would
synchronise the device.  They pass their own counts and offsets buffers; the scan's
per-tile sums use an array compiled into the library.  Here the buffers come from
torch (the test may allocate; the entry point must not), and the result must equal,
bit for bit, the row pointers fe_export_csr returns for the same matrices, on two
calls in a row (the second reuses the array the first one left behind).

The file name sorts last so that a run stopping at the first failure has already
run every other test.
"""
import ctypes

import numpy as np
import pytest

import golden_cases as gc

pytestmark = pytest.mark.gpu


def _noalloc_scan(lib, torch, counts):
    c = torch.from_numpy(np.ascontiguousarray(counts, dtype=np.int32)).to("cuda")
    out = torch.full((counts.size + 1,), -7, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    status = lib.fe_scan_counts_noalloc(ctypes.c_void_p(c.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                        counts.size, ctypes.c_void_p(stream))
    assert status == 0, lib.fe_last_error()
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _row_pointers(prob):
    """Row pointers from the existing entry point (fe_export_csr): the augmented
    K of create_matrix and the CSC K of k_matrix_sparse."""
    from finite_elements_gb300.engine import GpuSystem
    s = GpuSystem(prob)
    aug = s.create_matrix().indptr.astype(np.int64)
    csc = s.k_matrix_sparse().indptr.astype(np.int64)
    s.close()
    return aug, csc


def test_noalloc_scan_matches_the_export_row_pointers(gpu_lib):
    torch = pytest.importorskip("torch")
    from finite_elements_gb300 import meshgen
    problems = [gc.load("c1_cantilever")[0], gc.load("quirks_magnetic")[0],
                meshgen.plane_strain_random(600, 300, seed=5)]   # 362k rows: 177 tiles
    for prob in problems:
        for indptr in _row_pointers(prob):
            counts = np.diff(indptr)
            first = _noalloc_scan(gpu_lib, torch, counts)
            second = _noalloc_scan(gpu_lib, torch, counts)
            np.testing.assert_array_equal(first, indptr)
            np.testing.assert_array_equal(second, indptr)


def test_noalloc_scan_empty_and_oversize(gpu_lib):
    torch = pytest.importorskip("torch")
    out = _noalloc_scan(gpu_lib, torch, np.zeros(0, np.int32))
    np.testing.assert_array_equal(out, [0])
    # a total beyond int32 is flagged by offsets[n] = -1 (the earlier offsets that still
    # fit are exact)
    out = _noalloc_scan(gpu_lib, torch, np.full(3, 1 << 30, np.int32))
    assert out[3] == -1 and out[0] == 0 and out[1] == 1 << 30
    limit = (1 << 15) * 2048
    # rejected before any GPU work: the null buffers are never touched
    status = gpu_lib.fe_scan_counts_noalloc(None, None, limit + 1, None)
    assert status == 4
    assert b"exceed" in gpu_lib.fe_last_error()
