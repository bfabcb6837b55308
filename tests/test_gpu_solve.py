"""GPU power solve (pwmgpu_solve) and FP32 SpMV against the oracle.

The solve adds what the reference's powerIteration lacks (CRS.hpp:118-130
returns no eigenvalue): the Rayleigh quotient lambda of the normalised
iterate, the relative eigen-residual ||A u - lambda u|| / |lambda| and a
stopping test, all inside the persistent power kernel.

Tolerances: at equal iteration counts lambda and u within 1e-10 relative of
the oracle (power method + Rayleigh quotient in FP64 with CRS::mv); converged
Poisson solves within 1e-10 of the analytic lambda_max = 4 + 4 cos(pi/(m+1));
mixed-precision solves: the oracle's residual of the returned u within 2*tol
and lambda within 1e-10 relative of the FP64 solve; FP32 SpMV rows within
(2*nnz_row + 3) * 2^-24 * sum|a_ij x_j| (FP32 rounding of a and x, products
and sums).
"""
import math

import numpy as np
import pytest

from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pwm():
    import thesis_spmv_gb300 as t
    t.lib()
    return t


def _positive_random(n, mean_len, seed):
    """Random square matrix with positive values, a diagonal and a cycle
    (irreducible and aperiodic: a simple dominant Perron eigenvalue)."""
    rng = np.random.default_rng(seed)
    rows = []
    for i in range(n):
        k = int(rng.poisson(mean_len))
        c = set(rng.integers(0, n, size=k).tolist()) | {i, (i + 1) % n}
        rows.append(np.array(sorted(c), np.int32))
    rs = np.zeros(n + 1, np.int32)
    rs[1:] = np.cumsum([r.size for r in rows])
    cols = np.concatenate(rows)
    return O.CRSArrays(n, n, rs, cols, rng.uniform(0.0, 1.0, cols.size) + 1e-3)


def _load(pwm, A):
    M = pwm.CRSCuda(1)
    M.loadCSR(A.nor, A.noc, A.row_start, A.col_ind, A.data)
    return M


POWER_MODES = ["fused", "multi"]


def _set_mode(pwm, M, mode):
    """fused: the persistent kernel runs each chunk; multi: SpMV, fix-up and
    norm kernels per iteration plus the result pass."""
    M.set_power_mode(pwm.POWER_FUSED if mode == "fused" else pwm.POWER_MULTI)


@pytest.mark.parametrize("mode", POWER_MODES)
@pytest.mark.parametrize("kind,it", [("poisson", 2), ("poisson", 37), ("random", 2), ("random", 24),
                                     ("poisson", 301)])
def test_solve_equal_counts_matches_oracle(pwm, kind, it, mode):
    """tol = 0: exactly `it` SpMVs; lambda and u are those of the oracle's
    iterate after it - 1 steps of powerIteration."""
    A = O.fill_poisson(37, 23) if kind == "poisson" else _positive_random(3000, 7, 5)
    M = _load(pwm, A)
    _set_mode(pwm, M, mode)
    x0 = np.random.default_rng(8).random(A.nor)
    u = x0.copy()
    info = M.solve(u, it, 0.0, pwm.PREC_F64)
    assert info.iterations == it and info.iterations_low == 0 and info.converged == 0
    ur = O.power_result(A, x0, it - 1) if it > 1 else x0 / O.norm2(x0)
    lam_r, res_r = O.rayleigh(A, ur)
    assert abs(info.lambda_ - lam_r) <= 1e-10 * abs(lam_r)
    assert abs(info.residual - res_r) <= 1e-8 * res_r + 1e-14
    assert np.max(np.abs(u - ur)) <= 1e-10 * np.max(np.abs(ur))


@pytest.mark.parametrize("m", [5, 8, 12])
def test_solve_poisson_analytic_lambda_max(pwm, m):
    """Converged Poisson solves agree with lambda_max = 4 + 4 cos(pi/(m+1))."""
    A = O.fill_poisson(m, m)
    M = _load(pwm, A)
    u = np.random.default_rng(m).random(A.nor)
    info = M.solve(u, 20000, 1e-10, pwm.PREC_F64)
    assert info.converged == 1 and info.residual <= 1e-10
    exact = 4.0 + 4.0 * math.cos(math.pi / (m + 1))
    assert abs(info.lambda_ - exact) <= 1e-10 * exact
    lam_r, res_r = O.rayleigh(A, u)
    assert res_r <= 2e-10 and abs(lam_r - exact) <= 1e-10 * exact
    assert abs(np.linalg.norm(u) - 1.0) <= 1e-12


@pytest.mark.parametrize("mode", POWER_MODES)
@pytest.mark.parametrize("kind", ["poisson", "random"])
def test_solve_mixed_reaches_tolerance(pwm, kind, mode):
    """FP32 (BF16 values for the exactly representable Poisson stencil) bulk
    phase, FP64 refinement: the oracle confirms the residual, and lambda
    matches the FP64 solve."""
    A = O.fill_poisson(14, 14) if kind == "poisson" else _positive_random(20000, 8, 9)
    M = _load(pwm, A)
    _set_mode(pwm, M, mode)
    x0 = np.random.default_rng(3).random(A.nor)
    tol = 1e-10
    u64 = x0.copy()
    i64 = M.solve(u64, 20000, tol, pwm.PREC_F64)
    umx = x0.copy()
    imx = M.solve(umx, 20000, tol, pwm.PREC_MIXED)
    assert i64.converged == 1 and imx.converged == 1
    assert 0 < imx.iterations_low < imx.iterations
    lam_r, res_r = O.rayleigh(A, umx)
    assert res_r <= 2 * tol
    assert abs(imx.lambda_ - i64.lambda_) <= 1e-10 * abs(i64.lambda_)
    assert abs(lam_r - i64.lambda_) <= 1e-10 * abs(i64.lambda_)
    if kind == "poisson":
        exact = 4.0 + 4.0 * math.cos(math.pi / 15)
        assert abs(imx.lambda_ - exact) <= 1e-10 * exact


def test_solve_f32_only(pwm):
    A = _positive_random(20000, 8, 11)
    M = _load(pwm, A)
    u = np.random.default_rng(1).random(A.nor)
    info = M.solve(u, 2000, 1e-5, pwm.PREC_F32)
    assert info.converged == 1 and info.iterations_low == info.iterations
    lam_r, res_r = O.rayleigh(A, u)
    assert res_r <= 1e-4
    assert abs(info.lambda_ - lam_r) <= 1e-5 * lam_r


def test_solve_argument_checks(pwm):
    A = O.fill_poisson(6, 6)
    M = _load(pwm, A)
    u = np.ones(A.nor)
    with pytest.raises(pwm.PwmGpuError):
        M.solve(u, 1, 1e-10)  # max_it < 2
    with pytest.raises(pwm.PwmGpuError):
        M.solve(u, 10, -1.0)
    with pytest.raises(pwm.PwmGpuError):
        M.solve(u, 10, 1e-10, 7)
    R = pwm.CRSCuda(1)
    R.loadCSR(3, 4, np.array([0, 1, 2, 3]), np.array([0, 1, 3]), np.ones(3))
    with pytest.raises(pwm.PwmGpuError) as e:
        R.solve(np.ones(4), 10, 1e-10)
    assert e.value.code == 6  # PWMGPU_ERR_NOT_SQUARE
    z = pwm.CRSCuda(1)
    z.loadCSR(4, 4, np.zeros(5), np.zeros(0), np.zeros(0))  # A = 0: zero iterate
    with pytest.raises(pwm.PwmGpuError) as e:
        z.solve(np.ones(4), 10, 1e-10)
    assert e.value.code == 8  # PWMGPU_ERR_NUMERIC


@pytest.mark.parametrize("kind", ["poisson", "random"])
def test_mv_device_f32_row_bound(pwm, kind):
    torch = pytest.importorskip("torch")
    A = O.fill_poisson(300, 200) if kind == "poisson" else _positive_random(30000, 9, 4)
    M = _load(pwm, A)
    x = np.random.default_rng(6).uniform(-1, 1, A.noc)
    dx = torch.tensor(x, dtype=torch.float32, device="cuda")
    dy = torch.full((A.nor,), float("nan"), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    M.mv_device_f32(dx.data_ptr(), dy.data_ptr())
    torch.cuda.synchronize()
    y = dy.cpu().numpy().astype(np.float64)
    ref = O.crs_mv(A, x)
    nnz_row = np.diff(A.row_start)
    s = O.crs_mv(O.CRSArrays(A.nor, A.noc, A.row_start, A.col_ind, np.abs(A.data)), np.abs(x))
    bound = (2 * nnz_row + 3) * 2.0 ** -24 * s
    assert np.all(np.abs(y - ref) <= bound)


def test_solve_modes_agree_on_a_large_poisson_grid(pwm):
    """Large enough that AUTO takes the separate kernels: 60 steps in both
    forms give the same iterates (the SpMV bits do not depend on how the
    norms were summed), so lambda agrees to rounding; FP64 and mixed each."""
    g = 600
    M = pwm.CRSCuda(1)
    M.generatePoissonMatrix(g, g, 1)
    M.set_low_format(pwm.LOWFMT_MERGE)  # both modes on the merge layout (the SELL layout is another SpMV)
    x0 = np.random.default_rng(4).random(g * g)
    lam = {}
    for mode in POWER_MODES:
        _set_mode(pwm, M, mode)
        for prec in (pwm.PREC_F64, pwm.PREC_MIXED):
            u = x0.copy()
            info = M.solve(u, 60, 0.0, prec)
            assert info.iterations == 60
            lam[(mode, prec)] = info.lambda_
    for prec, tol in ((pwm.PREC_F64, 1e-12), (pwm.PREC_MIXED, 1e-9)):
        a, b = lam[("fused", prec)], lam[("multi", prec)]
        assert abs(a - b) <= tol * abs(a)
