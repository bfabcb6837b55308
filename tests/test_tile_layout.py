"""The device copy the CSB / CO-H tile kernel reads, checked on the CPU
(pwmgpu_tile_layout_host builds it with no device work).

For every unit: its range lies inside the arrays; a row-major or flat unit
(read 4 elements at a time) starts on a multiple of 4; a dense unit's x window starts on a multiple of the window side
and every element's column lies inside the matrix; a one-element-per-row
unit (kind 2, whose elements the kernel spreads over the lanes with no
atomics) has strictly ascending rows.  The elements are exactly the
matrix's (row, column, value) triples, each once, and the kernel's
arithmetic replayed on the copy (each element's product added to its row of
the window) matches CRS::mv (Matrix/CRS.hpp:99-109, restated in the oracle)
within the row error bound."""
import ctypes as C

import numpy as np
import pytest

from oracle import pyoracle as O
from test_autotune import _long_row_matrix
from test_formats import MATS, _crs_of

FMT_CSB, FMT_COH = 1, 2


def _layout(fmt, A, window, partitions=16):
    import thesis_spmv_gb300 as t
    L = t.lib()
    sizes = (C.c_int64 * 3)()
    args = (fmt, A.nor, A.noc, A.nnz, A.row_start.ctypes.data, A.col_ind.ctypes.data, A.data.ctypes.data,
            partitions, window, sizes)
    assert L.pwmgpu_tile_layout_host(*args, None, None, None, None, None) == 0, L.pwmgpu_last_error()
    wp = np.zeros(sizes[0], np.int32)
    un = np.zeros(max(sizes[1], 4), np.int32)
    ind = np.zeros(sizes[2], np.uint32)
    data = np.zeros(sizes[2], np.float64)
    col = np.zeros(sizes[2], np.int32)
    assert L.pwmgpu_tile_layout_host(*args, wp.ctypes.data, un.ctypes.data, ind.ctypes.data, data.ctypes.data,
                                     col.ctypes.data) == 0, L.pwmgpu_last_error()
    return wp, un[:sizes[1]].reshape(-1, 4), ind, data, col


def _check(A, S, wp, units, ind, data, col, x):
    """Invariants of every unit, the element multiset, and y = A x replayed
    on the copy.  Returns the count of units per kind."""
    nwin = -(-A.nor // S)
    assert wp.size == 2 * nwin + 1 and wp[0] == 0 and wp[-1] == units.shape[0]
    assert np.all(np.diff(wp) >= 0)
    y = np.zeros(A.nor)
    rows, cols, vals = [], [], []
    kinds = {0: 0, 2: 0, "flat": 0}
    for w in range(nwin):
        us, ud, ue = wp[2 * w], wp[2 * w + 1], wp[2 * w + 2]
        assert ud - us <= 1
        ys = np.zeros(S)
        for u in range(us, ue):
            lo, hi, c0, kind = (int(v) for v in units[u])
            assert 0 <= lo <= hi and hi + 8 <= ind.size
            assert kind != 0 or lo % 4 == 0
            idv = ind[lo:hi]
            if u < ud:  # the window's flat unit: global columns
                assert c0 == -1 and kind == 0
                kinds["flat"] += 1
                r = (idv >> 16).astype(np.int64) & (S - 1)
                g = col[lo:hi].astype(np.int64)
                v = data[lo:hi]
            else:
                assert 0 <= c0 < A.noc and c0 % S == 0 and kind in (0, 2)
                kinds[kind] += 1
                v = data[lo:hi]
                r = (idv >> 16).astype(np.int64) & (S - 1)
                g = c0 + (idv.astype(np.int64) & (S - 1))
                if kind == 2:
                    assert np.all(np.diff(r) > 0)
                if kind == 0:
                    assert np.all(np.diff(r) >= 0)
            assert np.all((g >= 0) & (g < A.noc))
            assert np.all(w * S + r < A.nor)
            np.add.at(ys, r, v * x[g])
            rows.append(w * S + r)
            cols.append(g)
            vals.append(v)
        n = min(S, A.nor - w * S)
        y[w * S:w * S + n] = ys[:n]
    rows, cols, vals = np.concatenate(rows), np.concatenate(cols), np.concatenate(vals)
    crs_rows = np.repeat(np.arange(A.nor), np.diff(A.row_start))
    got = np.lexsort((vals, cols, rows))
    ref = np.lexsort((A.data[:A.nnz], A.col_ind[:A.nnz], crs_rows))
    assert rows.size == A.nnz
    assert np.array_equal(rows[got], crs_rows[ref]) and np.array_equal(cols[got], A.col_ind[:A.nnz][ref])
    assert np.array_equal(vals[got].view(np.uint64), A.data[:A.nnz][ref].view(np.uint64))
    assert np.all(np.abs(y - O.crs_mv(A, x)) <= O.row_error_bound(A, x))
    return kinds


CASES = dict(MATS)
CASES["long_rows_and_duplicates"] = None
CASES["poisson_1024x256"] = lambda: (262144, 262144) + O.triplet_poisson(1024, 256)
CASES["random_tall"] = None  # more rows than columns


def _tall(nor=5000, noc=700, seed=9):
    rng = np.random.default_rng(seed)
    lens = np.minimum(rng.poisson(4, size=nor), noc)
    rows = np.repeat(np.arange(nor), lens).astype(np.int32)
    cols = np.concatenate([np.sort(rng.choice(noc, size=l, replace=False)) for l in lens if l]).astype(np.int32)
    return nor, noc, rows, cols, rng.uniform(-1, 1, rows.size)


def _matrix(name):
    if name == "long_rows_and_duplicates":
        return _long_row_matrix(20000, 21)
    nor, noc, r, c, v = _tall() if name == "random_tall" else CASES[name]()
    return _crs_of(nor, noc, r, c, v)


@pytest.mark.parametrize("window", [64, 256, 1024])
@pytest.mark.parametrize("fmt", [FMT_CSB, FMT_COH])
@pytest.mark.parametrize("name", sorted(CASES))
def test_tile_layout(name, fmt, window):
    A = _matrix(name)
    import thesis_spmv_gb300 as t
    beta = C.c_int32()
    t.lib().pwmgpu_csb_params(A.nor, A.noc, C.byref(beta), C.byref(C.c_int32()))
    if A.nor < 64:
        pytest.skip("fewer rows than the smallest window")
    if fmt == FMT_CSB and window > min(beta.value, 1024):
        pytest.skip("window larger than the CSB block")
    x = np.random.default_rng(3).uniform(-1, 1, A.noc)
    kinds = _check(A, window, *_layout(fmt, A, window), x)
    if name == "poisson_1024x256" and window >= 256:
        # a stencil whose grid width is a multiple of the window: every dense
        # unit is one diagonal of a tile
        assert kinds[0] == 0 and kinds[2] > 0
    if name == "banded_dups" and window >= 256:
        # a repeated coordinate keeps its tile whole (row-major; at 64 rows
        # the tiles are below the dense-unit size and go to the flat unit)
        assert kinds[0] > 0


def test_tile_layout_rejects_bad_windows():
    import thesis_spmv_gb300 as t
    L = t.lib()
    A = _matrix("poisson_300x300")
    sizes = (C.c_int64 * 3)()
    base = (A.nor, A.noc, A.nnz, A.row_start.ctypes.data, A.col_ind.ctypes.data, A.data.ctypes.data, 4)
    for fmt, window in ((FMT_CSB, 48), (FMT_CSB, 96), (FMT_CSB, 2048), (FMT_COH, 32), (0, 256)):
        assert L.pwmgpu_tile_layout_host(fmt, *base, window, sizes, None, None, None, None, None) == 1
