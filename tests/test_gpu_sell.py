"""SELL-32 layout of the FP32 / BF16 iterations against the oracle.

A matrix whose columns all lie within 32768 rows of their 32-row slice and
whose padding stays within a quarter of its nonzeros (stencils, banded
matrices) runs its low-precision iterations on the SELL-32 copy (one row per
lane, the row's products summed left to right in CRS order); any other
matrix, or a handle set to LOWFMT_MERGE, runs them on the merge layout.

Tolerances: FP32 SpMV rows within (2*nnz_row + 3) * 2^-24 * sum|a_ij x_j| of
the FP64 oracle (FP32 rounding of a and x, products and sums: the same bound
for both layouts); mixed solves: the oracle's residual of the returned u
within 2*tol and lambda within 1e-10 relative of the FP64 solve and of the
analytic Poisson lambda_max = 4 + 4 cos(pi/(m+1)).
"""
import math

import numpy as np
import pytest

from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

FORMATS = ["auto", "merge"]


@pytest.fixture(scope="module")
def pwm():
    import thesis_spmv_gb300 as t
    t.lib()
    return t


def _load(pwm, A, fmt):
    M = pwm.CRSCuda(1)
    M.loadCSR(A.nor, A.noc, A.row_start, A.col_ind, A.data)
    M.set_low_format(pwm.LOWFMT_AUTO if fmt == "auto" else pwm.LOWFMT_MERGE)
    return M


def _banded(n, offsets, seed, empty_every=0, spike=0.0):
    """Rows i with columns i + o (o in offsets, inside [0, n)), values in
    (0, 1]; every empty_every-th row empty; `spike` added to the diagonal
    entry of row n // 2 (a dominant, well separated eigenvalue)."""
    rng = np.random.default_rng(seed)
    rs = [0]
    cols, vals = [], []
    for i in range(n):
        if empty_every and i % empty_every == empty_every - 1:
            rs.append(rs[-1])
            continue
        c = sorted({i + o for o in offsets if 0 <= i + o < n})
        v = rng.uniform(0.0, 1.0, len(c)) + 1e-3
        if i == n // 2 and i in c:
            v[c.index(i)] += spike
        cols.extend(c)
        vals.extend(v.tolist())
        rs.append(rs[-1] + len(c))
    return O.CRSArrays(n, n, np.array(rs, np.int32), np.array(cols, np.int32), np.array(vals))


def _f32_rows_ok(pwm, M, A, seed):
    torch = pytest.importorskip("torch")
    x = np.random.default_rng(seed).uniform(-1, 1, A.noc)
    dx = torch.tensor(x, dtype=torch.float32, device="cuda")
    dy = torch.full((A.nor,), float("nan"), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    M.mv_device_f32(dx.data_ptr(), dy.data_ptr())
    torch.cuda.synchronize()
    y = dy.cpu().numpy().astype(np.float64)
    ref = O.crs_mv(A, x)
    s = O.crs_mv(O.CRSArrays(A.nor, A.noc, A.row_start, A.col_ind, np.abs(A.data)), np.abs(x))
    bound = (2 * np.diff(A.row_start) + 3) * 2.0 ** -24 * s
    return bool(np.all(np.abs(y - ref) <= bound)), y


@pytest.mark.parametrize("fmt", FORMATS)
@pytest.mark.parametrize("case", ["poisson_37x29", "poisson_300x200", "band_wide_offsets", "band_empty_rows",
                                  "band_too_wide", "one_long_row", "tiny"])
def test_f32_spmv_rows(pwm, case, fmt):
    """FP32 SpMV on both layouts: matrices that fit SELL (partial last
    slice, empty rows, offsets up to +-32767) and matrices that do not
    (offsets past 32768 rows, one long row: too much padding)."""
    A = {
        "poisson_37x29": lambda: O.fill_poisson(37, 29),
        "poisson_300x200": lambda: O.fill_poisson(300, 200),
        "band_wide_offsets": lambda: _banded(70001, (-32000, -7, 0, 5, 32700), 1),
        "band_empty_rows": lambda: _banded(5000, (-3, -1, 0, 1, 2), 2, empty_every=7),
        "band_too_wide": lambda: _banded(90000, (-40000, 0, 40000), 3),
        "one_long_row": lambda: O.CRSArrays(2000, 2000, *(_one_long_row(2000))),
        "tiny": lambda: O.fill_poisson(1, 3),
    }[case]()
    M = _load(pwm, A, fmt)
    ok, y = _f32_rows_ok(pwm, M, A, 7)
    assert ok
    ok2, y2 = _f32_rows_ok(pwm, M, A, 7)
    assert ok2 and np.array_equal(y, y2)  # deterministic


def _one_long_row(n):
    rs = [0]
    cols, vals = [], []
    for i in range(n):
        c = list(range(n)) if i == 5 else sorted({i, (i + 1) % n})
        cols.extend(c)
        vals.extend([1.0 + 0.001 * (k % 7) for k in range(len(c))])
        rs.append(rs[-1] + len(c))
    return np.array(rs, np.int32), np.array(cols, np.int32), np.array(vals)


@pytest.mark.parametrize("fmt", FORMATS)
@pytest.mark.parametrize("m", [14, 61])
def test_mixed_solve_poisson(pwm, m, fmt):
    """BF16 values (the stencil is exact in BF16), FP32 vectors, then the
    FP64 refinement: the oracle confirms the residual; lambda within 1e-10 of
    the FP64 solve and of the analytic lambda_max."""
    A = O.fill_poisson(m, m)
    M = _load(pwm, A, fmt)
    M.set_power_mode(pwm.POWER_MULTI)
    x0 = np.random.default_rng(5).random(A.nor)
    tol = 1e-10
    u64 = x0.copy()
    i64 = M.solve(u64, 40000, tol, pwm.PREC_F64)
    umx = x0.copy()
    imx = M.solve(umx, 40000, tol, pwm.PREC_MIXED)
    assert i64.converged == 1 and imx.converged == 1
    assert 0 < imx.iterations_low < imx.iterations
    lam_r, res_r = O.rayleigh(A, umx)
    assert res_r <= 2 * tol
    exact = 4.0 + 4.0 * math.cos(math.pi / (m + 1))
    for lam in (imx.lambda_, lam_r):
        assert abs(lam - i64.lambda_) <= 1e-10 * abs(i64.lambda_)
        assert abs(lam - exact) <= 1e-10 * exact


@pytest.mark.parametrize("fmt", FORMATS)
def test_f32_solve_banded(pwm, fmt):
    """FP32 values and vectors throughout (a banded positive matrix with a
    dominant diagonal entry): residual and lambda against the oracle."""
    A = _banded(20000, (-900, -1, 0, 1, 2, 900), 4, spike=8.0)
    M = _load(pwm, A, fmt)
    M.set_power_mode(pwm.POWER_MULTI)
    u = np.random.default_rng(2).random(A.nor)
    info = M.solve(u, 4000, 1e-5, pwm.PREC_F32)
    assert info.converged == 1 and info.iterations_low == info.iterations
    lam_r, res_r = O.rayleigh(A, u)
    assert res_r <= 1e-4
    assert abs(info.lambda_ - lam_r) <= 1e-5 * lam_r


def test_layouts_agree_on_a_large_poisson_grid(pwm):
    """60 mixed steps on a 600^2 grid with each layout: the low-precision
    iterates differ only by FP32 rounding, so lambda agrees closely."""
    g = 600
    M = pwm.CRSCuda(1)
    M.generatePoissonMatrix(g, g, 1)
    M.set_power_mode(pwm.POWER_MULTI)
    x0 = np.random.default_rng(4).random(g * g)
    lam = {}
    for fmt in FORMATS:
        M.set_low_format(pwm.LOWFMT_AUTO if fmt == "auto" else pwm.LOWFMT_MERGE)
        u = x0.copy()
        info = M.solve(u, 60, 0.0, pwm.PREC_MIXED)
        assert info.iterations == 60
        lam[fmt] = info.lambda_
    assert abs(lam["auto"] - lam["merge"]) <= 1e-6 * abs(lam["merge"])


def test_low_format_argument_check(pwm):
    M = pwm.CRSCuda(1)
    with pytest.raises(pwm.PwmGpuError):
        M.set_low_format(5)
