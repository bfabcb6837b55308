"""CPU model of the merge kernel (thesis_spmv_gb300/csrc/merge.cuh and
merge.cu), checked before any of it runs on a GPU:

* geometry: sub-tile ends are merge-path coordinates of the oracle's
  searchPathOnDiag restatement (CRS_Merge.hpp:42-62) at diagonals s*WM; a
  tile is W consecutive sub-tiles;
* TMA windows: every staged window starts 16-byte aligned, has a size that is
  a multiple of 16 bytes, fits its shared-memory capacity and stays inside
  the array plus its kArrayPad padding; the row window covers every
  row_start entry the lanes read;
* algorithm: a step-by-step simulation of process_subtile (nonzero split over
  32 lanes, row completion, the run-leader carry merge, the a < rw1 rule) and
  of k_merge_fixup reproduces the oracle's y = A x within the row bound.
"""
import numpy as np
import pytest

from oracle import pyoracle as O

PAD = 16


def geometry(NT, IPT, vsize):
    W = NT // 32
    WM = 32 * IPT
    TM = W * WM
    VE = 16 // vsize
    return dict(W=W, WM=WM, TM=TM, VE=VE, VAL_CAP=TM + 2 * VE, COL_CAP=TM + 8, ROW_CAP=TM + 12)


def sub_coords(A, WM):
    total = A.nor + A.nnz
    ns = -(-total // WM)
    return [O.merge_search(A, min(s * WM, total)) for s in range(ns + 1)]


def windows(r0, k0, r1, k1, nor, G):
    nk = k1 - k0
    rlast = min(r1, nor - 1)
    VE = G["VE"]
    k0a = k0 & ~(VE - 1)
    k1a = ((k1 + VE - 1) & ~(VE - 1)) if nk else k0a
    k0c = k0 & ~3
    k1c = ((k1 + 3) & ~3) if nk else k0c
    rs = r0 & ~3
    re = (rlast + 2 + 3) & ~3
    return (k0a, k1a), (k0c, k1c), (rs, re)


def check_windows(A, NT, IPT, vsize):
    G = geometry(NT, IPT, vsize)
    nor, nnz = A.nor, A.nnz
    sc = sub_coords(A, G["WM"])
    ns = len(sc) - 1
    assert sc[0] == (0, 0) and sc[-1] == (nor, nnz)
    nt = -(-ns // G["W"])
    for t in range(nt):
        s0, s1 = t * G["W"], min((t + 1) * G["W"], ns)
        (r0, k0), (r1, k1) = sc[s0], sc[s1]
        assert r0 <= nor - 1
        assert (r1 - r0) + (k1 - k0) <= G["TM"]
        (va, vb), (ca, cb), (ra, rb) = windows(r0, k0, r1, k1, nor, G)
        assert (va * vsize) % 16 == 0 and ((vb - va) * vsize) % 16 == 0
        assert (ca * 4) % 16 == 0 and ((cb - ca) * 4) % 16 == 0
        assert (ra * 4) % 16 == 0 and ((rb - ra) * 4) % 16 == 0 and rb > ra
        assert vb - va <= G["VAL_CAP"] and cb - ca <= G["COL_CAP"] and rb - ra <= G["ROW_CAP"]
        assert vb <= nnz + PAD and cb <= nnz + PAD and rb <= nor + 1 + PAD
        if k1 > k0:
            assert va <= k0 and vb >= k1 and ca <= k0 and cb >= k1
        rlast = min(r1, nor - 1)
        assert ra <= r0 and rb >= rlast + 2  # row_start[r0 .. rlast+1] staged
        for w in range(s1 - s0):
            (rw0, kw0), (rw1, kw1) = sc[s0 + w], sc[s0 + w + 1]
            assert r0 <= rw0 <= rw1 <= r1 and (rw1 - rw0) + (kw1 - kw0) <= G["WM"]


def simulate(A, x, IPT):
    """process_subtile for every sub-tile, then k_merge_fixup.  Returns y and
    how many times each row's square entered the power method's ||y||^2
    (must be exactly once)."""
    WM = 32 * IPT
    sc = sub_coords(A, WM)
    ns = len(sc) - 1
    rs = A.row_start
    nor = A.nor
    BIG = 2 ** 31 - 1
    y = np.full(nor, np.nan)
    counted = np.zeros(nor, np.int64)
    carries = np.zeros(ns)
    # k_mark_empty_rows: sub-tiles holding the end item of an empty row
    slow = np.zeros(ns + 1, bool)
    for r in range(nor):
        if rs[r + 1] == rs[r]:
            slow[(rs[r + 1] + r) // WM] = True
    for s in range(ns):
        (rw0, kw0), (rw1, kw1) = sc[s], sc[s + 1]
        nkw = kw1 - kw0
        q = (nkw + 31) >> 5
        assert q <= IPT
        lane_a, lane_acc, lane_b0 = [], [], []
        for lane in range(32):
            b0 = kw0 + lane * q
            qe = min(max(kw1 - b0, 0), q)
            a, rend = rw1, BIG
            if qe > 0:
                lo, hi = rw0, rw1
                while lo < hi:
                    mid = (lo + hi + 1) >> 1
                    if rs[mid] <= b0:
                        lo = mid
                    else:
                        hi = mid - 1
                a = lo
                assert rs[a] <= b0 < rs[a + 1] or a == rw1
                rend = rs[a + 1] if a < rw1 else BIG
            lane_a.append(a)
            lane_b0.append((b0, qe, rend))
        # rows [rw0, a_lane0) carry no nonzeros here
        for r in range(rw0, lane_a[0]):
            y[r] = 0.0
        crow, cval, hval = [], [], [None] * 32
        for lane in range(32):
            b0, qe, rend = lane_b0[lane]
            a = lane_a[lane]
            head_open = qe > 0 and rs[a] < b0
            acc, first = 0.0, True
            if not slow[s]:
                mask = 0
                r = a
                while r < rw1:
                    rr = rs[r + 1]
                    if rr > b0 + qe:
                        break
                    assert 0 <= rr - b0 - 1 < IPT and not (mask >> (rr - b0 - 1)) & 1
                    mask |= 1 << (rr - b0 - 1)
                    r += 1
                to_head = head_open and lane > 0
                count = not head_open
                for j in range(IPT):
                    if j < q:
                        if j < qe:
                            acc = acc + A.data[b0 + j] * x[A.col_ind[b0 + j]]
                        if (mask >> j) & 1:
                            if to_head:
                                hval[lane] = acc
                                to_head = False
                            else:
                                y[a] = acc
                                if count:
                                    counted[a] += 1
                            count = True
                            acc = 0.0
                            a += 1
                crow.append(a)
                cval.append(acc)
                continue
            for j in range(IPT):
                if j < q:
                    if j < qe:
                        acc = acc + A.data[b0 + j] * x[A.col_ind[b0 + j]]
                    bn = b0 + j + 1
                    if j < qe and bn == rend:
                        if first and head_open and lane > 0:
                            hval[lane] = acc
                        else:
                            y[a] = acc
                            if not (first and head_open):
                                counted[a] += 1
                        acc, first = 0.0, False
                        a += 1
                        rend = rs[a + 1] if a < rw1 else BIG
                        while rend == bn:
                            y[a] = 0.0
                            counted[a] += 1  # an empty row's square (0) is final here
                            a += 1
                            rend = rs[a + 1] if a < rw1 else BIG
            crow.append(a)
            cval.append(acc)
        assert crow[31] == rw1
        for lane in range(32):
            a = crow[lane]
            if lane == 0 or crow[lane - 1] != a:
                tot = cval[lane]
                u = lane + 1
                while u < 32 and crow[u] == a:
                    tot += cval[u]
                    u += 1
                if a < rw1:
                    if rs[a] < kw0 + u * q:
                        assert hval[u] is not None
                        y[a] = hval[u] + tot
                        if rs[a] >= kw0:
                            counted[a] += 1
                    else:
                        assert tot == 0.0
                elif a < nor:
                    carries[s] = tot
    # empty rows zeroed before lane 0's first row are final there too
    # (k_merge_fixup counts the open row rw0 of a sub-tile instead)
    for t in range(ns):
        r = sc[t + 1][0]
        if r >= nor or (t > 0 and sc[t][0] == r):
            continue
        tot = carries[t]
        n = t + 1
        while n < ns and sc[n + 1][0] == r:
            tot += carries[n]
            n += 1
        if sc[n][1] > rs[r]:
            y[r] = y[r] + tot
            counted[r] += 1
    return y, counted


def _random_csr(n, mean_len, seed, noc=None, empty_frac=0.0, dense_rows=0, dense_len=0):
    noc = noc or n
    rng = np.random.default_rng(seed)
    lens = rng.poisson(mean_len, size=n)
    lens[rng.random(n) < empty_frac] = 0
    if dense_rows:
        lens[rng.choice(n, size=dense_rows, replace=False)] = dense_len
    lens = np.minimum(lens, noc)
    rs = np.zeros(n + 1, np.int32)
    rs[1:] = np.cumsum(lens)
    cols = [np.sort(rng.choice(noc, size=l, replace=False)) for l in lens if l]
    cols = np.concatenate(cols).astype(np.int32) if cols else np.zeros(0, np.int32)
    return O.CRSArrays(n, noc, rs, cols, rng.uniform(-1, 1, int(lens.sum())))


CONFIGS = [(128, 12, 8), (128, 8, 8), (128, 12, 4), (128, 12, 2)]
MATRICES = {
    "poisson1x1": lambda: O.fill_poisson(1, 1),
    "poisson2x3": lambda: O.fill_poisson(2, 3),
    "poisson37x29": lambda: O.fill_poisson(37, 29),
    "empty_rows": lambda: _random_csr(3000, 5, 1, empty_frac=0.3),
    "dense_rows": lambda: _random_csr(2500, 3, 2, dense_rows=3, dense_len=2400),
    "nnz0": lambda: _random_csr(700, 0, 3),
    "all_empty": lambda: O.CRSArrays(5, 5, np.zeros(6, np.int32), np.zeros(0, np.int32), np.zeros(0)),
    "wide": lambda: _random_csr(300, 40, 4, noc=5000),
    "long_rows_exact": lambda: _random_csr(400, 224, 5, noc=600),
}


@pytest.mark.parametrize("cfg", CONFIGS)
@pytest.mark.parametrize("name", sorted(MATRICES))
def test_windows(cfg, name):
    check_windows(MATRICES[name](), *cfg)


@pytest.mark.parametrize("IPT", [8, 12])
@pytest.mark.parametrize("name", sorted(MATRICES))
def test_algorithm_simulation(IPT, name):
    A = MATRICES[name]()
    x = np.random.default_rng(1).uniform(-1, 1, A.noc)
    y, counted = simulate(A, x, IPT)
    ref = O.crs_mv(A, x)
    assert not np.isnan(y).any()
    assert np.all(np.abs(y - ref) <= O.row_error_bound(A, x) + 1e-300)
    # every nonempty-or-open row's square is summed exactly once; rows with no
    # nonzeros at all may be counted 0 or 1 times (their square is 0)
    nz = np.diff(A.row_start) > 0
    assert np.all(counted[nz] == 1), np.nonzero(counted[nz] != 1)[0][:10]
    assert np.all(counted <= 1)


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
