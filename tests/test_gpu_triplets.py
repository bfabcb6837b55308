"""GPU triplet -> CRS (Util/TripletToCRS.hpp:135-172) through the C ABI:
pwmgpu_load_triplets (host arrays, sorted in place like the reference) and
pwmgpu_load_triplets_device (device arrays, left unchanged).

Bit-exact: row_start / col_ind / data against the oracle's TripletToCRS
restatement for unique coordinates, and against a stable (row, col) numpy
sort for any input (entries with equal coordinates keep their input order).
"""
import numpy as np
import pytest

from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pwm():
    import thesis_spmv_gb300 as t
    t.lib()
    return t


def _stable_crs(nor, rows, cols, vals):
    p = np.lexsort((cols, rows))  # stable: rows, then columns, then input order
    rs = np.zeros(nor + 1, np.int64)
    np.add.at(rs, rows.astype(np.int64) + 1, 1)
    return np.cumsum(rs).astype(np.int32), rows[p], cols[p], vals[p]


def _load_host(pwm, nor, noc, r, c, v):
    M = pwm.CRSCuda(1)
    t = pwm.Triplet(nor, noc, r.copy(), c.copy(), v.copy())
    M.loadFromTriplets(t, 1)
    return M, t


def _check(pwm, nor, noc, r, c, v):
    rs, rr, cc, vv = _stable_crs(nor, r, c, v)
    M, t = _load_host(pwm, nor, noc, r, c, v)
    grs, gci, gv = M.getCSR()
    assert np.array_equal(grs, rs)
    assert np.array_equal(gci, cc)
    assert np.array_equal(gv.view(np.uint64), vv.view(np.uint64))
    # the caller's triplet comes back sorted, as in the reference
    assert np.array_equal(t.row_coord, rr) and np.array_equal(t.col_coord, cc)
    assert np.array_equal(t.data.view(np.uint64), vv.view(np.uint64))
    return M


def _unique_triplets(rng, nor, noc, nnz):
    flat = rng.choice(nor * noc, size=nnz, replace=False)
    return (flat // noc).astype(np.int32), (flat % noc).astype(np.int32), rng.uniform(-1, 1, nnz)


@pytest.mark.parametrize("nor,noc,nnz,seed", [(1000, 700, 50_000, 1), (97, 5000, 4096, 2), (4097, 3, 9000, 3),
                                              (70_000, 70_000, 300_000, 4)])
def test_unique_matches_oracle(pwm, nor, noc, nnz, seed):
    rng = np.random.default_rng(seed)
    r, c, v = _unique_triplets(rng, nor, noc, nnz)
    ref = O.triplet_to_crs(nor, noc, r.copy(), c.copy(), v.copy())
    M = _check(pwm, nor, noc, r, c, v)
    grs, gci, gv = M.getCSR()
    assert np.array_equal(grs, ref.row_start)
    assert np.array_equal(gci, ref.col_ind)
    assert np.array_equal(gv, ref.data)


@pytest.mark.parametrize("seed", [5, 6])
def test_duplicates_keep_input_order(pwm, seed):
    rng = np.random.default_rng(seed)
    nor, noc, nnz = 300, 40, 60_000  # ~5 entries per coordinate
    r = rng.integers(0, nor, nnz).astype(np.int32)
    c = rng.integers(0, noc, nnz).astype(np.int32)
    v = rng.uniform(-1, 1, nnz)
    _check(pwm, nor, noc, r, c, v)


def test_sorted_and_column_major_inputs(pwm):
    rng = np.random.default_rng(7)
    nor, noc = 5000, 6000
    r, c, v = _unique_triplets(rng, nor, noc, 200_000)
    p = np.lexsort((c, r))
    _check(pwm, nor, noc, r[p], c[p], v[p])  # already CRS order: copied as is
    q = np.lexsort((r, c))
    _check(pwm, nor, noc, r[q], c[q], v[q])  # Matrix Market order: only the row digits sort


def test_poisson_shuffled(pwm):
    m, n = 37, 29
    r, c, v = O.triplet_poisson(m, n)
    p = np.random.default_rng(8).permutation(r.size)
    M = _check(pwm, m * n, m * n, r[p], c[p], v[p])
    A = O.fill_poisson(m, n)
    grs, gci, gv = M.getCSR()
    assert np.array_equal(grs, A.row_start) and np.array_equal(gci, A.col_ind) and np.array_equal(gv, A.data)


@pytest.mark.parametrize("shape", ["empty", "one_entry", "one_row", "one_col", "dense_row", "wide_keys"])
def test_edge_shapes(pwm, shape):
    rng = np.random.default_rng(9)
    if shape == "empty":
        nor, noc, nnz = 5, 5, 0
    elif shape == "one_entry":
        nor, noc, nnz = 3, 4, 1
    elif shape == "one_row":
        nor, noc, nnz = 1, 100_000, 30_000
    elif shape == "one_col":
        nor, noc, nnz = 100_000, 1, 30_000
    elif shape == "dense_row":  # one row holds most entries, the rest sparse
        nor, noc, nnz = 1000, 200_000, 0
    else:  # 27-bit rows and columns: four digits each
        nor, noc, nnz = 1 << 27, (1 << 27) - 3, 100_000
    if shape == "dense_row":
        cd = rng.permutation(noc)[:150_000].astype(np.int32)
        rd = np.full(cd.size, 17, np.int32)
        rs_, cs_, vs_ = _unique_triplets(rng, nor, noc, 20_000)
        keep = rs_ != 17
        r = np.concatenate([rd, rs_[keep]])
        c = np.concatenate([cd, cs_[keep]])
        v = rng.uniform(-1, 1, r.size)
        p = rng.permutation(r.size)
        r, c, v = r[p], c[p], v[p]
    elif shape == "wide_keys":
        r = rng.integers(0, nor, nnz).astype(np.int32)
        c = rng.integers(0, noc, nnz).astype(np.int32)
        v = rng.uniform(-1, 1, nnz)
    else:
        r, c, v = _unique_triplets(rng, nor, noc, nnz) if nnz else (np.zeros(0, np.int32),) * 2 + (np.zeros(0),)
    _check(pwm, nor, noc, r, c, v)


def test_device_entry_leaves_inputs(pwm):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(10)
    nor, noc = 20_000, 15_000
    r, c, v = _unique_triplets(rng, nor, noc, 120_000)
    dr, dc, dv = (torch.from_numpy(a).cuda() for a in (r, c, v))
    M = pwm.CRSCuda(1)
    M.loadFromDeviceTriplets(nor, noc, r.size, dr.data_ptr(), dc.data_ptr(), dv.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(dr.cpu().numpy(), r) and np.array_equal(dc.cpu().numpy(), c)
    assert np.array_equal(dv.cpu().numpy(), v)
    Mh, _ = _load_host(pwm, nor, noc, r, c, v)
    for a, b in zip(M.getCSR(), Mh.getCSR()):
        assert np.array_equal(a, b)
    # and the matrix computes: SpMV against the oracle
    x = rng.random(noc)
    y = np.zeros(nor)
    M.mv(x, y)
    A = O.triplet_to_crs(nor, noc, r.copy(), c.copy(), v.copy())
    assert np.all(np.abs(y - O.crs_mv(A, x)) <= O.row_error_bound(A, x))


@pytest.mark.parametrize("where", ["row", "col", "negative", "row_before_col"])
def test_out_of_range_entries(pwm, where):
    rng = np.random.default_rng(11)
    nor, noc = 50, 60
    r, c, v = _unique_triplets(rng, nor, noc, 900)
    good = pwm.CRSCuda(1)
    good.loadFromTriplets(pwm.Triplet(nor, noc, r.copy(), c.copy(), v.copy()), 1)
    x = rng.random(noc)
    y0 = np.zeros(nor)
    good.mv(x, y0)
    r2, c2 = r.copy(), c.copy()
    if where == "row":
        r2[700] = nor
        want = "row %d at entry 700" % nor
    elif where == "col":
        c2[333] = noc + 5
        want = "column %d at entry 333" % (noc + 5)
    elif where == "negative":
        c2[12] = -1
        want = "column -1 at entry 12"
    else:  # two bad entries: the first one is reported, its row before its column
        r2[400], c2[400] = -7, noc
        c2[401] = noc
        want = "row -7 at entry 400"
    with pytest.raises(RuntimeError, match=want):
        good.loadFromTriplets(pwm.Triplet(nor, noc, r2, c2, v.copy()), 1)
    # the previous matrix is still loaded and unchanged
    y1 = np.zeros(nor)
    good.mv(x, y1)
    assert np.array_equal(y0, y1)
