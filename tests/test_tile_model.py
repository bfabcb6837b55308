"""CPU model of the merge-path kernel (thesis_spmv_gb300/csrc/merge.cuh,
merge.cu), checked before any of it runs on a GPU.

Layout ("lane-interleaved merge-path CRS"): the merge path is cut into
sub-tiles of WM = 32*IPT items, one per warp; sub-tile s spans the nonzeros
[kw0, kw1) and hands lane l the contiguous range [kw0 + start_l, + cnt_l)
(qm = nkw // 32, rem = nkw % 32, cnt_l = qm + (l < rem)).  Each array is
stored per sub-tile at an 8-element-aligned base so that element j of lane l
sits at mli_pos(l, j, qm, V) with V = 2 (the kernel's lane_vec): 2-element
vector blocks consecutive across the warp, then a scalar tail of at most two
slots (the partial last slot for lanes < rem only).  Other V are checked too.

Checks: the permutation is a bijection into [base, base + nkw) and vector
slots are 16-byte aligned; bases never overlap and stay inside the
allocation; row-end masks, first rows and flags reproduce the CRS structure;
a step-by-step simulation of the kernel (fast and general paths, carries,
k_merge_fixup) reproduces the oracle's y = A x within the row bound.
"""
import numpy as np
import pytest

from oracle import pyoracle as O

BIG = 2 ** 31 - 1
LANE_VEC = 2  # merge.cuh lane_vec<T>()


def mli_pos(lane, j, qm, V):
    B = qm // V
    if j < V * B:
        return (j // V) * 32 * V + lane * V + (j % V)
    return 32 * V * B + (j - V * B) * 32 + lane


def mli_base(kw0, s):
    return 8 * ((kw0 + 7 * s + 7) // 8)


def sub_coords(A, WM):
    total = A.nor + A.nnz
    ns = -(-total // WM)
    return [O.merge_search(A, min(s * WM, total)) for s in range(ns + 1)]


def lane_range(kw0, kw1, lane):
    nkw = kw1 - kw0
    qm, rem = nkw >> 5, nkw & 31
    start = lane * qm + min(lane, rem)
    cnt = qm + (1 if lane < rem else 0)
    return kw0 + start, cnt, qm, rem


def row_of(rs, b, lo, hi):
    """largest a in [lo, hi] with row_start[a] <= b"""
    while lo < hi:
        mid = (lo + hi + 1) >> 1
        if rs[mid] <= b:
            lo = mid
        else:
            hi = mid - 1
    return lo


def plan(A, IPT):
    """k_mli_plan: permuted arrays, per-lane row-end masks, per-sub-tile meta."""
    WM = 32 * IPT
    rs = A.row_start
    sc = sub_coords(A, WM)
    ns = len(sc) - 1
    size = A.nnz + 7 * ns + 16
    valp = np.full(size, np.nan)
    colp = np.full(size, -1, np.int64)
    masks = np.zeros((ns, 32), np.int64)
    meta = []
    for s in range(ns):
        (rw0, kw0), (rw1, kw1) = sc[s], sc[s + 1]
        nkw = kw1 - kw0
        base = mli_base(kw0, s)
        fr = row_of(rs, kw0, rw0, rw1) if nkw > 0 else rw1
        has_empty = any(rs[r] == rs[r + 1] for r in range(rw0, rw1))
        open0 = nkw > 0 and rs[fr] < kw0
        for lane in range(32):
            b0, cnt, qm, rem = lane_range(kw0, kw1, lane)
            if cnt == 0:
                continue
            a = row_of(rs, b0, rw0, rw1)
            m = 0
            for j in range(cnt):
                b = b0 + j
                while a < rw1 and rs[a + 1] <= b:  # row a ends before b (empty rows)
                    a += 1
                if a < rw1 and b + 1 == rs[a + 1]:
                    m |= 1 << j
                pv, pc = mli_pos(lane, j, qm, LANE_VEC), mli_pos(lane, j, qm, LANE_VEC)
                assert np.isnan(valp[base + pv]) and colp[base + pc] == -1
                valp[base + pv] = A.data[b]
                colp[base + pc] = A.col_ind[b]
            masks[s, lane] = m
        meta.append((fr, int(has_empty), int(open0), base))
    return sc, valp, colp, masks, meta


def simulate(A, x, IPT):
    """The kernel (fast path unless the sub-tile holds an empty row) and
    k_merge_fixup; returns y."""
    sc, valp, colp, masks, meta = plan(A, IPT)
    rs, nor = A.row_start, A.nor
    ns = len(sc) - 1
    y = np.full(nor, np.nan)
    carries = np.zeros(ns)
    for s in range(ns):
        (rw0, kw0), (rw1, kw1) = sc[s], sc[s + 1]
        fr, has_empty, open0, base = meta[s]
        nkw = kw1 - kw0
        qm, rem = nkw >> 5, nkw & 31
        q = qm + (1 if rem else 0)
        # per lane: values / gathers, row-end masks
        lanes = []
        for lane in range(32):
            b0, cnt, _, _ = lane_range(kw0, kw1, lane)
            vv = [valp[base + mli_pos(lane, j, qm, LANE_VEC)] if j < cnt else 0.0 for j in range(IPT)]
            xv = [x[colp[base + mli_pos(lane, j, qm, LANE_VEC)]] if j < cnt else 0.0 for j in range(IPT)]
            lanes.append((b0, cnt, vv, xv, int(masks[s, lane])))
        # rows [rw0, fr) carry no nonzeros in this sub-tile
        for r in range(rw0, fr):
            y[r] = 0.0
        # first rows: exclusive prefix of popcounts (fast) or search (general)
        pc = [bin(l[4]).count("1") for l in lanes]
        crow, cval, hval = [], [], [None] * 32
        for lane in range(32):
            b0, cnt, vv, xv, m = lanes[lane]
            if not has_empty:
                a = fr + sum(pc[:lane])
                if cnt:
                    assert rs[a] <= b0 < rs[a + 1] or a == rw1
                if lane == 0:
                    head_open = bool(open0)
                else:
                    pb, pcnt = lanes[lane - 1][0], lanes[lane - 1][1]
                    head_open = cnt > 0 and not ((lanes[lane - 1][4] >> (pcnt - 1)) & 1)
                assert head_open == (cnt > 0 and rs[a] < b0)
            else:
                a = row_of(rs, b0, rw0, rw1) if cnt else rw1
                head_open = cnt > 0 and rs[a] < b0
            to_head = head_open and lane > 0
            acc = 0.0
            for j in range(IPT):
                if j < q:
                    acc = acc + vv[j] * xv[j]
                    if (m >> j) & 1:
                        if to_head:
                            hval[lane] = acc
                            to_head = False
                        else:
                            y[a] = acc
                        acc = 0.0
                        a += 1
                        if has_empty:  # general path: pass empty rows
                            while a < rw1 and rs[a + 1] == rs[a]:
                                y[a] = 0.0
                                a += 1
            if cnt == 0:
                a = rw1
            crow.append(a)
            cval.append(acc)
        assert crow[31] == rw1, (crow, rw1)
        for lane in range(32):
            a = crow[lane]
            if lane == 0 or crow[lane - 1] != a:
                tot = cval[lane]
                u = lane + 1
                while u < 32 and crow[u] == a:
                    tot += cval[u]
                    u += 1
                if a < rw1:
                    b0u = lanes[u][0]
                    if rs[a] < b0u:
                        assert hval[u] is not None
                        y[a] = hval[u] + tot
                    else:
                        assert tot == 0.0
                elif a < nor:
                    carries[s] = tot
    for t in range(ns):  # k_merge_fixup
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
    return y


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


MATRICES = {
    "poisson1x1": lambda: O.fill_poisson(1, 1),
    "poisson2x3": lambda: O.fill_poisson(2, 3),
    "poisson37x29": lambda: O.fill_poisson(37, 29),
    "empty_rows": lambda: _random_csr(3000, 5, 1, empty_frac=0.3),
    "dense_rows": lambda: _random_csr(2500, 3, 2, dense_rows=3, dense_len=2400),
    "nnz0": lambda: _random_csr(700, 0, 3),
    "all_empty": lambda: O.CRSArrays(5, 5, np.zeros(6, np.int32), np.zeros(0, np.int32), np.zeros(0)),
    "wide": lambda: _random_csr(300, 40, 4, noc=5000),
    "long_rows": lambda: _random_csr(400, 224, 5, noc=600),
    "short_rows": lambda: _random_csr(3000, 1, 6),
}


@pytest.mark.parametrize("IPT", [8, 10, 12])
@pytest.mark.parametrize("name", sorted(MATRICES))
def test_layout(IPT, name):
    A = MATRICES[name]()
    sc, valp, colp, masks, meta = plan(A, IPT)
    ns = len(sc) - 1
    size = A.nnz + 7 * ns + 16
    for s in range(ns):
        (rw0, kw0), (rw1, kw1) = sc[s], sc[s + 1]
        nkw = kw1 - kw0
        base = meta[s][3]
        assert base % 8 == 0 and base + nkw <= size
        if s + 1 < ns:
            assert mli_base(sc[s + 1][1], s + 1) >= base + nkw  # no overlap
        qm = nkw >> 5
        assert (nkw + 31) >> 5 <= IPT
        for V in (1, 2, 4, 8):
            pos = sorted(mli_pos(l, j, qm, V) for l in range(32) for j in range(lane_range(kw0, kw1, l)[1]))
            assert pos == list(range(nkw))  # bijection onto [0, nkw)
            for l in range(32):
                for blk in range(qm // V):  # V-element vector slots start at multiples of V: 16 bytes
                    assert (base + mli_pos(l, blk * V, qm, V)) % V == 0
    # all nonzeros placed exactly once
    assert np.count_nonzero(~np.isnan(valp)) == A.nnz and np.count_nonzero(colp >= 0) == A.nnz


@pytest.mark.parametrize("IPT", [8, 10, 12])
@pytest.mark.parametrize("name", sorted(MATRICES))
def test_algorithm_simulation(IPT, name):
    A = MATRICES[name]()
    x = np.random.default_rng(1).uniform(-1, 1, A.noc)
    y = simulate(A, x, IPT)
    ref = O.crs_mv(A, x)
    assert not np.isnan(y).any()
    assert np.all(np.abs(y - ref) <= O.row_error_bound(A, x) + 1e-300)


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
