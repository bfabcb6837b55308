"""pwmgpu_stats (Util_Scripts/calc_stats.cpp figures on the device) against
the oracle, whose restatement is pinned to the reference's own script
(tests/golden/ref_stats.json).

Exact: size, nnz, rows_avg, block_bits, whole blocks, balanced, longest row.
Tolerance for the sums (the script adds its terms sequentially, the device
in a fixed parallel order; the terms are the same): rows_var within
2 (n + 1) u relative; block_avg (the device divides the exact total once)
within 2 (nb^2 + 1) u; block_var within 4 (nb^2 + 1) u relative plus four
times the square of the block means' difference; u = 2^-53.
"""
import numpy as np
import pytest

from golden_cases import stats_cases
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

U = 2.0 ** -53


@pytest.fixture(scope="module")
def pwm():
    import thesis_spmv_gb300 as t
    t.lib()
    return t


def _check(got, want, n, longest):
    for k in ("size", "nnz", "rows_avg", "balanced", "block_bits", "nb_blocks"):
        assert got[k] == want[k], (k, got[k], want[k])
    assert got["max_row_nnz"] == longest
    nb2 = float(want["nb_blocks"]) ** 2
    assert abs(got["rows_var"] - want["rows_var"]) <= 2 * (n + 1) * U * abs(want["rows_var"])
    d_avg = abs(got["block_avg"] - want["block_avg"])
    assert d_avg <= 2 * (nb2 + 1) * U * abs(want["block_avg"])
    assert abs(got["block_var"] - want["block_var"]) <= 4 * (nb2 + 1) * U * abs(want["block_var"]) + 4 * d_avg ** 2


def _load(pwm, n, r, c, v, cls=None):
    M = (cls or pwm.CRSCuda)(1)
    M.loadFromTriplets(pwm.Triplet(n, n, r.copy(), c.copy(), v.copy()), 1)
    return M


def _longest(r):
    return int(np.unique(r, return_counts=True)[1].max()) if r.size else 0


@pytest.mark.parametrize("case", stats_cases(), ids=lambda c: c[0])
def test_stats_cases(pwm, case):
    name, n, r, c, v = case
    M = _load(pwm, n, r, c, v)
    _check(M.stats(), O.calc_stats(n, r, c), n, _longest(r))


def test_stats_generated_matrices(pwm):
    M = pwm.CRSCuda(1)
    M.generatePoissonMatrix(1024, 1024, 1)
    r, c, _ = O.triplet_poisson(1024, 1024)
    _check(M.stats(), O.calc_stats(1024 * 1024, r, c), 1024 * 1024, 5)
    n = 300_000
    M.generateRandom(n, 17, mean_len=16.0, max_len=5000)
    A = O.random_crs(n, 17, mean=16.0, max_len=5000)
    rows = np.repeat(np.arange(n, dtype=np.int32), np.diff(A.row_start))
    _check(M.stats(), O.calc_stats(n, rows, A.col_ind), n, int(np.diff(A.row_start).max()))


def test_stats_other_formats_same(pwm):
    name, n, r, c, v = stats_cases()[-1]
    base = _load(pwm, n, r, c, v).stats()
    for cls in (pwm.CSBCuda, pwm.COHCuda):
        assert _load(pwm, n, r, c, v, cls).stats() == base


def test_stats_wide_block_grid(pwm):
    """More than 4096 whole blocks per side: counts go straight to global memory."""
    n = 4100 * 65536 + 123
    rng = np.random.default_rng(5)
    nnz = 400_000
    r = rng.integers(0, n, nnz).astype(np.int32)
    c = np.where(rng.random(nnz) < 0.3, r, rng.integers(0, n, nnz)).astype(np.int32)
    v = np.ones(nnz)
    M = _load(pwm, n, r, c, v)
    got = M.stats()
    assert got["nb_blocks"] == 4100 and got["block_bits"] == 16
    _check(got, O.calc_stats(n, r, c), n, _longest(r))


def test_stats_empty_matrix_rejected(pwm):
    M = pwm.CRSCuda(1)
    with pytest.raises(RuntimeError, match="statistics need"):
        M.stats()
