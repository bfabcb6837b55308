"""Pin the C oracle against the unmodified reference classes compiled from the
reference tree (oracle/_ref).  Runs only where that tree is present (the
development container); elsewhere the recorded outputs in
tests/golden/ref_outputs.npz stand in (tests/test_oracle_golden.py)."""
import numpy as np
import pytest

from oracle import pyoracle as O
from oracle import pyref as R

pytestmark = pytest.mark.skipif(not R.available(), reason="reference tree not present")


def _rand_triplets(n, nnz_per_row, seed):
    rng = np.random.default_rng(seed)
    rows, cols = [], []
    for i in range(n):
        k = rng.integers(1, 2 * nnz_per_row)
        cs = np.unique(rng.integers(0, n, size=k))
        rows += [i] * cs.size
        cols += cs.tolist()
    r = np.array(rows, np.int32)
    c = np.array(cols, np.int32)
    p = rng.permutation(r.size)
    return r[p].copy(), c[p].copy(), rng.random(r.size)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_random_crs_merge_csb_coh(seed):
    n = 300 + 50 * seed
    r, c, v = _rand_triplets(n, 6, seed)
    A = O.triplet_to_crs(n, n, r.copy(), c.copy(), v.copy())
    M = R.Matrix(R.METHOD_CRS).load(R.Triplet().set(n, n, r, c, v))
    rs, ci, d = M.crs()
    assert np.array_equal(rs, A.row_start) and np.array_equal(ci, A.col_ind) and np.array_equal(d, A.data)
    x = np.random.default_rng(seed + 10).random(n)
    assert np.array_equal(O.crs_mv(A, x), M.mv(x))
    for T in (1, 2, 5, 16):
        MM = R.Matrix(R.METHOD_MERGE, T).load(R.Triplet().set(n, n, r, c, v))
        P = O.merge_partition(A, T)
        tot = A.nor + A.nnz
        ipt = -(-tot // T)
        assert [tuple(p) for p in P] == [MM.merge_search(min(ipt * t, tot)) for t in range(T + 1)]
        assert np.array_equal(O.merge_mv(A, x, T), MM.mv(x))
    csb_ref = R.Matrix(R.METHOD_CSB, 2).load(R.Triplet().set(n, n, r, c, v)).csb()
    csb = O.csb_build(n, n, r.copy(), c.copy(), v.copy())
    for k in ("ind", "data", "blk_ptr"):
        assert np.array_equal(csb[k], csb_ref[k])
    for T in (1, 2, 4):
        ref = R.Matrix(R.METHOD_COH, T).load(R.Triplet().set(n, n, r, c, v)).coh()
        got = O.coh_build(n, n, r.copy(), c.copy(), v.copy(), T)
        assert got["threads"] == len(ref)
        cat = lambda k: np.concatenate([p[k] for p in ref])
        for k in ("row_jump", "col_jump", "data", "block_nnz", "row_jump_block", "col_jump_block"):
            assert np.array_equal(got[k][:cat(k).size], cat(k)), k


def test_power_matches_reference_bitwise():
    A = O.fill_poisson(33, 17)
    M = R.Matrix(R.METHOD_CRS).generate_poisson(33, 17)
    x = np.random.default_rng(5).random(A.nor)
    for it in (1, 2, 9, 40):
        xo, yo = O.power(A, x, it)
        xr, yr = M.power(x, it)
        assert np.array_equal(xo, xr) and np.array_equal(yo, yr)


@pytest.mark.parametrize("n,seed", [(777, 1), (3000, 2), (70000, 3)])
def test_calc_stats_matches_reference(n, seed):
    """Random square triplets (duplicates included) through the reference's
    calc_stats and the oracle: the same doubles."""
    rng = np.random.default_rng(seed)
    nnz = n * 7
    r = rng.integers(0, n, nnz).astype(np.int32)
    c = np.where(rng.random(nnz) < 0.5, r, rng.integers(0, n, nnz)).astype(np.int32)
    v = rng.random(nnz)
    got = O.calc_stats(n, r, c)
    want = R.calc_stats(n, n, r, c, v)
    for k, w in want.items():
        assert got[k] == w, (k, got[k], w)
