"""pwmgpu_mv_csr_device_noalloc: y = A x on caller-owned device CRS arrays
without allocating device memory.

It serves callers that cannot allocate at call time (an allocator that owns
all device memory, a serving loop that must not call cudaMalloc / cudaFree,
a plug-in handed device pointers only); its scratch is a fixed array in
device memory shared by every call.  The GPU test checks it through the C ABI
against the handle-based entry point (pwmgpu_load_csr + pwmgpu_mv) on two
calls in a row -- the second after the shared scratch holds the first call's
contents -- within the per-row bound the other SpMV tests use.

This file is collected last (test_zz_*), so a run that stops at the first
failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import pyoracle as O


def _lib():
    import thesis_spmv_gb300 as t
    return t.lib()


def _random_csr(n, mean_len, seed, empty_frac=0.0, dense_rows=0, dense_len=0):
    rng = np.random.default_rng(seed)
    lens = rng.poisson(mean_len, size=n)
    lens[rng.random(n) < empty_frac] = 0
    if dense_rows:
        lens[rng.choice(n, size=dense_rows, replace=False)] = dense_len
    lens = np.minimum(lens, n)
    rs = np.zeros(n + 1, np.int32)
    rs[1:] = np.cumsum(lens)
    cols = [np.sort(rng.choice(n, size=l, replace=False)) for l in lens if l]
    cols = np.concatenate(cols).astype(np.int32) if cols else np.zeros(0, np.int32)
    return O.CRSArrays(n, n, rs, cols, rng.uniform(-1, 1, int(lens.sum())))


def test_rejects_sizes_beyond_its_scratch():
    """Sizes beyond the fixed scratch are refused before any device work."""
    L = _lib()
    rc = L.pwmgpu_mv_csr_device_noalloc(100_000_000, 100_000_000, 40_000_000, None, None, None, None, None, None)
    assert rc == 1  # PWMGPU_ERR_INVALID
    assert "scratch" in L.pwmgpu_last_error().decode()
    assert L.pwmgpu_mv_csr_device_noalloc(-1, 3, 0, None, None, None, None, None, None) == 1


@pytest.mark.gpu
def test_noalloc_matches_handle_entry_point_twice():
    torch = pytest.importorskip("torch")
    import thesis_spmv_gb300 as t
    L = t.lib()
    stream = torch.cuda.Stream()
    matrices = [_random_csr(60000, 6, 3, empty_frac=0.1, dense_rows=3, dense_len=20000), O.fill_poisson(300, 170)]
    for call, A in enumerate(matrices):  # two calls in a row on the shared scratch
        x = np.random.default_rng(10 + call).uniform(-1, 1, A.noc)
        ref_mat = t.CRSCuda(1)
        ref_mat.loadCSR(A.nor, A.noc, A.row_start, A.col_ind, A.data)
        y_ref = np.zeros(A.nor)
        ref_mat.mv(x, y_ref)

        d_rs = torch.tensor(A.row_start, dtype=torch.int32, device="cuda")
        d_ci = torch.tensor(A.col_ind, dtype=torch.int32, device="cuda")
        d_v = torch.tensor(A.data, dtype=torch.float64, device="cuda")
        d_x = torch.tensor(x, dtype=torch.float64, device="cuda")
        d_y = torch.full((A.nor,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = L.pwmgpu_mv_csr_device_noalloc(A.nor, A.noc, A.nnz, C.c_void_p(d_rs.data_ptr()),
                                            C.c_void_p(d_ci.data_ptr()), C.c_void_p(d_v.data_ptr()),
                                            C.c_void_p(d_x.data_ptr()), C.c_void_p(d_y.data_ptr()),
                                            C.c_void_p(stream.cuda_stream))
        assert rc == 0, L.pwmgpu_last_error()
        stream.synchronize()
        y = d_y.cpu().numpy()
        bound = O.row_error_bound(A, x)
        assert np.all(np.abs(y - y_ref) <= 2 * bound), call
        assert np.all(np.abs(y - O.crs_mv(A, x)) <= bound), call


def _noalloc(L, torch, stream, A, x):
    d_rs = torch.tensor(A.row_start, dtype=torch.int32, device="cuda")
    d_ci = torch.tensor(A.col_ind if A.nnz else np.zeros(1, np.int32), dtype=torch.int32, device="cuda")
    d_v = torch.tensor(A.data if A.nnz else np.zeros(1), dtype=torch.float64, device="cuda")
    d_x = torch.tensor(x, dtype=torch.float64, device="cuda")
    d_y = torch.full((A.nor,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = L.pwmgpu_mv_csr_device_noalloc(A.nor, A.noc, A.nnz, C.c_void_p(d_rs.data_ptr()),
                                        C.c_void_p(d_ci.data_ptr()), C.c_void_p(d_v.data_ptr()),
                                        C.c_void_p(d_x.data_ptr()), C.c_void_p(d_y.data_ptr()),
                                        C.c_void_p(stream.cuda_stream))
    assert rc == 0, L.pwmgpu_last_error()
    stream.synchronize()
    return d_y.cpu().numpy()


@pytest.mark.gpu
def test_noalloc_empty_matrix_and_empty_edge_rows():
    """nnz = 0 writes every row of y as 0 (from a NaN-filled buffer); a matrix
    whose first and last 700 rows are empty (whole sub-tiles of row ends with
    no nonzeros at both ends of the merge path) matches the oracle."""
    torch = pytest.importorskip("torch")
    L = _lib()
    stream = torch.cuda.Stream()
    n = 5000
    Z = O.CRSArrays(n, n, np.zeros(n + 1, np.int32), np.zeros(0, np.int32), np.zeros(0))
    assert np.array_equal(_noalloc(L, torch, stream, Z, np.ones(n)), np.zeros(n))
    A = _random_csr(n, 7, 21)
    lens = np.diff(A.row_start)
    lens[:700] = 0
    lens[-700:] = 0
    rs = np.zeros(n + 1, np.int32)
    rs[1:] = np.cumsum(lens)
    keep = np.repeat(np.arange(n), np.diff(A.row_start))
    mask = (keep >= 700) & (keep < n - 700)
    E = O.CRSArrays(n, n, rs, A.col_ind[mask], A.data[mask])
    x = np.random.default_rng(5).uniform(-1, 1, n)
    for _ in range(2):  # twice: the second call finds the first call's scratch contents
        y = _noalloc(L, torch, stream, E, x)
        assert np.all(np.abs(y - O.crs_mv(E, x)) <= O.row_error_bound(E, x))
        assert np.all(y[:700] == 0) and np.all(y[-700:] == 0)
