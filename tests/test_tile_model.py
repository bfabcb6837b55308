"""CPU model of the merge kernel's tile and TMA-window arithmetic
(thesis_spmv_gb300/csrc/merge.cuh issue_tile / process_tile), checked against
the buffers it touches before any of it runs on a GPU:

* tile end points are merge-path coordinates of the oracle's
  searchPathOnDiag restatement (CRS_Merge.hpp:42-62) at diagonals t*TM;
* every staged window starts 16-byte aligned, has a size that is a multiple of
  16 bytes, fits its shared-memory capacity and stays inside the array plus
  its kArrayPad padding;
* the row window covers every row_start entry the consume phase reads;
* the per-thread search restricted to the tile finds the global answer.
"""
import numpy as np
import pytest

from oracle import pyoracle as O

PAD = 16


def layout(NT, IPT, vsize):
    TM = NT * IPT
    VE = 16 // vsize
    return dict(TM=TM, VE=VE, VAL_CAP=TM + 2 * VE, COL_CAP=TM + 8, ROW_CAP=TM + 12)


def windows(c0, c1, nor, L):
    r0, k0 = c0
    r1, k1 = c1
    nk = k1 - k0
    rlast = min(r1, nor - 1)
    VE = L["VE"]
    k0a = k0 & ~(VE - 1)
    k1a = ((k1 + VE - 1) & ~(VE - 1)) if nk else k0a
    k0c = k0 & ~3
    k1c = ((k1 + 3) & ~3) if nk else k0c
    rs = r0 & ~3
    re = (rlast + 2 + 3) & ~3
    return (k0a, k1a), (k0c, k1c), (rs, re)


def check_matrix(A, NT, IPT, vsize):
    L = layout(NT, IPT, vsize)
    TM = L["TM"]
    nor, nnz = A.nor, A.nnz
    total = nor + nnz
    nt = -(-total // TM)
    coords = [O.merge_search(A, min(t * TM, total)) for t in range(nt + 1)]
    assert coords[0] == (0, 0) and coords[-1] == (nor, nnz)
    for t in range(nt):
        (r0, k0), (r1, k1) = coords[t], coords[t + 1]
        assert r0 <= nor - 1, "a non-empty tile starts before the last row"
        assert (r1 - r0) + (k1 - k0) <= TM
        (va, vb), (ca, cb), (ra, rb) = windows(coords[t], coords[t + 1], nor, L)
        # alignment (elements -> bytes) and sizes
        assert (va * vsize) % 16 == 0 and ((vb - va) * vsize) % 16 == 0
        assert (ca * 4) % 16 == 0 and ((cb - ca) * 4) % 16 == 0
        assert (ra * 4) % 16 == 0 and ((rb - ra) * 4) % 16 == 0 and rb > ra
        # capacities
        assert vb - va <= L["VAL_CAP"] and cb - ca <= L["COL_CAP"] and rb - ra <= L["ROW_CAP"]
        # inside allocation + padding
        assert vb <= nnz + PAD and cb <= nnz + PAD and rb <= nor + 1 + PAD
        # covers what the tile reads
        if k1 > k0:
            assert va <= k0 and vb >= k1 and ca <= k0 and cb >= k1
        rlast = min(r1, nor - 1)
        assert ra <= r0 and rb >= rlast + 2
        # per-thread searches inside the tile reproduce the global search
        d0, d1 = r0 + k0, r1 + k1
        for tid in range(0, NT, max(1, NT // 16)):
            d = d0 + tid * IPT
            if d >= d1:
                continue
            lo, hi = max(r0, d - k1), min(r1, d - k0)
            while lo < hi:
                p = (lo + hi) >> 1
                assert r0 <= p + 1 <= rlast + 1  # staged row_start index
                if A.row_start[p + 1] <= d - p - 1:
                    lo = p + 1
                else:
                    hi = p
            assert (lo, d - lo) == O.merge_search(A, d)


def _random_csr(n, mean_len, seed, empty_frac=0.0, dense_rows=0, dense_len=0):
    rng = np.random.default_rng(seed)
    lens = rng.poisson(mean_len, size=n)
    lens[rng.random(n) < empty_frac] = 0
    for r in rng.choice(n, size=dense_rows, replace=False) if dense_rows else []:
        lens[r] = dense_len
    lens = np.minimum(lens, n)
    rs = np.zeros(n + 1, np.int32)
    rs[1:] = np.cumsum(lens)
    cols = np.concatenate([np.sort(rng.choice(n, size=l, replace=False)) for l in lens]) if lens.sum() else \
        np.zeros(0, np.int64)
    return O.CRSArrays(n, n, rs, cols.astype(np.int32), rng.random(int(lens.sum())))


CONFIGS = [(256, 7, 8), (128, 11, 8), (256, 7, 4), (256, 7, 2)]


@pytest.mark.parametrize("cfg", CONFIGS)
def test_windows_poisson(cfg):
    for m, n in [(1, 1), (2, 3), (37, 29), (256, 200)]:
        check_matrix(O.fill_poisson(m, n), *cfg)


@pytest.mark.parametrize("cfg", CONFIGS)
def test_windows_irregular(cfg):
    check_matrix(_random_csr(3000, 5, 1, empty_frac=0.3), *cfg)       # many empty rows
    check_matrix(_random_csr(2500, 3, 2, dense_rows=3, dense_len=2400), *cfg)  # rows spanning tiles
    check_matrix(_random_csr(700, 0, 3), *cfg)                         # nnz == 0
    check_matrix(O.CRSArrays(5, 5, np.array([0, 0, 0, 0, 0, 0], np.int32), np.zeros(0, np.int32), np.zeros(0)),
                 *cfg)


def test_poisson_row_start_closed_form():
    """The device generator's closed form for row_start (merge.cu
    poisson_row_start) equals fillPoisson's running count."""
    def closed(row, m, n):
        mn = m * n
        below = row - m if row > m else 0
        left = row - (row + m - 1) // m
        right = row - row // m
        above = row if row < mn - m else max(mn - m, 0)
        return below + left + row + right + above
    for m, n in [(1, 1), (1, 5), (5, 1), (3, 3), (9, 3), (10, 5), (17, 13)]:
        A = O.fill_poisson(m, n)
        assert [closed(r, m, n) for r in range(m * n + 1)] == A.row_start.tolist()
