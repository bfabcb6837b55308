"""CSB and CO-H formats: the library's builders against the oracle (bit for
bit, on the CPU: pwmgpu_csb_build_host / pwmgpu_coh_build_host need no
device), then the GPU kernels (pwmgpu_create with PWMGPU_FMT_CSB / _COH)
against the oracle's CRS::mv within 2*nnz_row*u*sum|a_ij x_j| and the power
method at equal iteration counts within 1e-10.

Reference: SOA_Implementations/CSB.hpp:96-113,147-173,464-567 and
BlockCOH.hpp:79-114,119-132,319-455 (restated in oracle/oracle.c, pinned
against the compiled reference by test_oracle_vs_ref)."""
import ctypes as C

import numpy as np
import pytest

from golden_cases import boost_close, case_ids, cases, triplets_for
from oracle import pyoracle as O


def _lib():
    import thesis_spmv_gb300 as t
    return t, t.lib()


def _random_coo(n, mean_len, seed, noc=None, empty_frac=0.0):
    noc = noc or n
    rng = np.random.default_rng(seed)
    lens = rng.poisson(mean_len, size=n)
    lens[rng.random(n) < empty_frac] = 0
    lens = np.minimum(lens, noc)
    rows = np.repeat(np.arange(n), lens).astype(np.int32)
    cols = np.concatenate([np.sort(rng.choice(noc, size=l, replace=False)) for l in lens if l]).astype(np.int32) \
        if lens.sum() else np.zeros(0, np.int32)
    vals = rng.uniform(-1, 1, rows.size)
    return n, noc, rows, cols, vals


def _banded_coo(n, offsets, seed, keep=0.9, dup=0.0):
    """Entries on the given diagonals (col - row = offset), each kept with
    probability `keep`: banded tiles whose diagonals are partly empty.  A
    fraction `dup` of the entries appears twice (CRS keeps both)."""
    rng = np.random.default_rng(seed)
    rows, cols = [], []
    for d in offsets:
        r = np.arange(max(0, -d), min(n, n - d))
        r = r[rng.random(r.size) < keep]
        r = np.concatenate([r, r[rng.random(r.size) < dup]])
        rows.append(r)
        cols.append(r + d)
    rows = np.concatenate(rows).astype(np.int32)
    cols = np.concatenate(cols).astype(np.int32)
    order = np.lexsort((cols, rows))
    rows, cols = rows[order], cols[order]
    return n, n, rows, cols, rng.uniform(-1, 1, rows.size)


def _crs_of(nor, noc, rows, cols, vals):
    return O.triplet_to_crs(nor, noc, rows.copy(), cols.copy(), vals.copy())


MATS = {
    "poisson_3x3": lambda: (9, 9) + O.triplet_poisson(3, 3),
    "poisson_40x23": lambda: (920, 920) + O.triplet_poisson(40, 23),
    "poisson_300x300": lambda: (90000, 90000) + O.triplet_poisson(300, 300),
    "random_5000": lambda: _random_coo(5000, 7, 1),
    "random_empty_rows": lambda: _random_coo(3000, 3, 2, empty_frac=0.3),
    "random_rect": lambda: _random_coo(700, 5, 3, noc=1300),
    # banded tiles: split per diagonal (4 diagonals) or kept whole (5)
    "banded_4diag": lambda: _banded_coo(40000, (-2, 0, 1, 3), 5),
    "banded_5diag": lambda: _banded_coo(30000, (-3, -1, 0, 2, 5), 6),
    # a tridiagonal band with repeated coordinates: its tiles are not split
    "banded_dups": lambda: _banded_coo(30000, (-1, 0, 1), 7, dup=0.02),
}


def _csb_lib(A):
    t, L = _lib()
    beta, bits = C.c_int32(), C.c_int32()
    assert L.pwmgpu_csb_params(A.nor, A.noc, C.byref(beta), C.byref(bits)) == 0
    hb = -(-A.noc // beta.value)
    vb = -(-A.nor // beta.value)
    ind = np.zeros(max(A.nnz, 1), np.uint32)
    data = np.zeros(max(A.nnz, 1), np.float64)
    blk = np.zeros(hb * vb + 1, np.int32)
    rc = L.pwmgpu_csb_build_host(A.nor, A.noc, A.nnz, A.row_start.ctypes.data, A.col_ind.ctypes.data,
                                 A.data.ctypes.data, ind.ctypes.data, data.ctypes.data, blk.ctypes.data)
    assert rc == 0, L.pwmgpu_last_error()
    return dict(ind=ind[:A.nnz], data=data[:A.nnz], blk_ptr=blk, beta=beta.value, block_bits=bits.value)


def _coh_lib(A, threads):
    t, L = _lib()
    cap = max(A.nnz, 1)
    part = np.zeros(9 * max(threads, 1), np.int32)
    rj = np.zeros(cap, np.uint16)
    cj = np.zeros(cap, np.uint16)
    d = np.zeros(cap, np.float64)
    bn = np.zeros(cap, np.int32)
    rjb = np.zeros(cap, np.int16)
    cjb = np.zeros(cap, np.int16)
    T, nrj, nblk, nrjb = C.c_int32(), C.c_int64(), C.c_int64(), C.c_int64()
    rc = L.pwmgpu_coh_build_host(A.nor, A.noc, A.nnz, A.row_start.ctypes.data, A.col_ind.ctypes.data,
                                 A.data.ctypes.data, threads, C.byref(T), C.byref(nrj), C.byref(nblk), C.byref(nrjb),
                                 part.ctypes.data, rj.ctypes.data, cj.ctypes.data, d.ctypes.data, bn.ctypes.data,
                                 rjb.ctypes.data, cjb.ctypes.data)
    assert rc == 0, L.pwmgpu_last_error()
    return dict(threads=T.value, part_info=part[:9 * T.value], row_jump=rj[:nrj.value], col_jump=cj[:A.nnz],
                data=d[:A.nnz], block_nnz=bn[:nblk.value], row_jump_block=rjb[:nrjb.value],
                col_jump_block=cjb[:nblk.value])


@pytest.mark.parametrize("name", sorted(MATS))
def test_csb_builder_bitexact(name):
    nor, noc, r, c, v = MATS[name]()
    A = _crs_of(nor, noc, r, c, v)
    got = _csb_lib(A)
    ref = O.csb_build(nor, noc, r.copy(), c.copy(), v.copy())
    assert got["beta"] == ref["beta"] and got["block_bits"] == ref["block_bits"]
    assert np.array_equal(got["blk_ptr"], ref["blk_ptr"])
    assert np.array_equal(got["ind"], ref["ind"])
    assert np.array_equal(got["data"].view(np.uint64), ref["data"].view(np.uint64))


@pytest.mark.parametrize("threads", [1, 4, 13, 64])
@pytest.mark.parametrize("name", sorted(MATS))
def test_coh_builder_bitexact(name, threads):
    nor, noc, r, c, v = MATS[name]()
    A = _crs_of(nor, noc, r, c, v)
    got = _coh_lib(A, threads)
    ref = O.coh_build(nor, noc, r.copy(), c.copy(), v.copy(), threads)
    assert got["threads"] == ref["threads"]
    for k in ("part_info", "block_nnz", "row_jump_block", "col_jump_block", "row_jump", "col_jump"):
        n = got[k].size
        assert np.array_equal(got[k], ref[k][:n]), k
    assert np.array_equal(got["data"].view(np.uint64), ref["data"][:A.nnz].view(np.uint64))


# ---------------------------------------------------------------- GPU
FORMATS = {"csb": "CSBCuda", "coh": "COHCuda"}


def _gpu(fmt, A, threads=1):
    t, _ = _lib()
    M = getattr(t, FORMATS[fmt])(threads)
    M.loadCSR(A.nor, A.noc, A.row_start, A.col_ind, A.data)
    return t, M


@pytest.mark.gpu
@pytest.mark.parametrize("fmt", sorted(FORMATS))
@pytest.mark.parametrize("name", sorted(MATS))
def test_format_spmv_row_bound(fmt, name):
    nor, noc, r, c, v = MATS[name]()
    A = _crs_of(nor, noc, r, c, v)
    t, M = _gpu(fmt, A, threads=16)
    x = np.random.default_rng(4).uniform(-1, 1, A.noc)
    y = np.full(A.nor, np.nan)
    M.mv(x, y)
    bound = O.row_error_bound(A, x)
    assert np.all(np.abs(y - O.crs_mv(A, x)) <= bound)
    rs, ci, d = M.getCSR()
    assert np.array_equal(rs, A.row_start) and np.array_equal(ci, A.col_ind)


@pytest.mark.gpu
@pytest.mark.parametrize("fmt", sorted(FORMATS))
def test_format_arrays_on_device_bitexact(fmt):
    nor, noc, r, c, v = MATS["poisson_300x300"]()
    A = _crs_of(nor, noc, r, c, v)
    t, M = _gpu(fmt, A, threads=8)
    if fmt == "csb":
        got, ref = M.getCSB(), O.csb_build(nor, noc, r.copy(), c.copy(), v.copy())
        keys = ("ind", "blk_ptr")
    else:
        got, ref = M.getCOH(), O.coh_build(nor, noc, r.copy(), c.copy(), v.copy(), 8)
        keys = ("part_info", "row_jump", "col_jump", "block_nnz", "row_jump_block", "col_jump_block")
    for k in keys:
        assert np.array_equal(got[k], ref[k][:got[k].size]), k
    assert np.array_equal(got["data"].view(np.uint64), ref["data"][:A.nnz].view(np.uint64))


@pytest.mark.gpu
@pytest.mark.parametrize("fmt", sorted(FORMATS))
@pytest.mark.parametrize("case", cases(), ids=case_ids())
def test_format_reference_known_answers(fmt, case):
    """Tests/poisson.cpp and Tests/input.cpp run every format; so do these."""
    t, _ = _lib()
    M = getattr(t, FORMATS[fmt])(4)
    tr = triplets_for(case)
    if tr is None:
        M.generatePoissonMatrix(case["input"]["m"], case["input"]["n"], 4)
        n = case["input"]["m"] * case["input"]["n"]
    else:
        nor, noc, r, c, v = tr
        M.loadFromTriplets(t.Triplet(nor, noc, r, c, v), 4)
        n = noc
    golden = np.array(case["golden"])
    x = np.ones(n)
    y = np.zeros(golden.size)
    if case["op"]["kind"] == "mv":
        M.mv(x, y)
        out = y
    else:
        M.powerIteration(x, y, case["op"]["iterations"])
        out = x
    assert boost_close(out, golden, case["tolerance"]).all()


@pytest.mark.gpu
@pytest.mark.parametrize("fmt", sorted(FORMATS))
@pytest.mark.parametrize("it", [1, 2, 11, 40])
def test_format_power_equal_counts(fmt, it):
    nor, noc, r, c, v = _random_coo(4000, 6, 8)
    v = np.abs(v) + 0.01
    A = _crs_of(nor, noc, r, c, v)
    t, M = _gpu(fmt, A, threads=32)
    x0 = np.random.default_rng(1).random(A.nor)
    xg, yg = x0.copy(), np.zeros(A.nor)
    M.powerIteration(xg, yg, it)
    xr, yr = O.power(A, x0, it)
    np.testing.assert_allclose(xg, xr, rtol=1e-10, atol=1e-13)
    np.testing.assert_allclose(yg, yr, rtol=1e-10, atol=1e-13)


@pytest.mark.gpu
def test_format_large_poisson_and_unsupported_calls():
    """A 1024^2 Poisson grid (CSB beta 8192, 4 block rows; CO-H beta 2^13) in
    both formats; the merge-only entry points refuse cleanly."""
    t, _ = _lib()
    A = O.fill_poisson(1024, 1024)
    x = np.random.default_rng(0).uniform(-1, 1, A.noc)
    ref = O.crs_mv(A, x)
    bound = O.row_error_bound(A, x)
    for fmt in sorted(FORMATS):
        M = getattr(t, FORMATS[fmt])(608)
        M.generatePoissonMatrix(1024, 1024, 608)
        y = np.zeros(A.nor)
        M.mv(x, y)
        assert np.all(np.abs(y - ref) <= bound), fmt
        with pytest.raises(t.PwmGpuError):
            M.solve(x.copy(), 10, 1e-10)
