"""Parity at the benchmark workloads' full sizes, through the C ABI.

C1: the 512^2 Poisson matrix, 100 power iterations and the SpMV against the
oracle's CRS::mv / powerIteration.  C2: the 4096^2 Poisson matrix (N =
16,777,216, nnz = 83,869,696): CRS arrays bit for bit against the oracle's
fillPoisson (Util/Poisson.hpp:32-83), the SpMV on a seeded uniform vector
within the per-row bound, and size-independent properties -- x = 1 gives the
exact row sums, A(2x) = 2(Ax) bit for bit (scaling by 2 is exact), 20 power
iterations within 1e-10 of the oracle; the same matrix in the CSB and CO-H
formats.  C3: the irregular lognormal-row
matrix (N = 4,194,304): the device generator's arrays bit for bit against
the oracle's restatement, the SpMV within the bound, and FP64 and mixed
solves to 1e-10 relative eigen-residual whose eigenvalues agree to 1e-10
and whose eigenvectors the oracle's Rayleigh quotient confirms.

Tolerances: rows within 2*nnz_row*u*sum|a_ij*x_j| (u = 2^-53); iterates at
equal iteration counts within 1e-10 relative.
"""
import numpy as np
import pytest

from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

SEED = 20261203
IRREGULAR = dict(n=4194304, seed=20261203, length_dist=0, mean_len=16.0, sigma=1.2, max_len=20000,
                 band_permille=300, band_half=4096)


@pytest.fixture(scope="module")
def pwm():
    import thesis_spmv_gb300 as t
    t.lib()
    return t


def _mv(M, x):
    y = np.zeros(x.size)
    M.mv(x, y)
    return y


def test_c1_poisson512_spmv_and_100_power_iterations(pwm):
    A = O.fill_poisson(512, 512)
    M = pwm.CRSCuda(1)
    M.generatePoissonMatrix(512, 512, 1)
    x = np.random.default_rng(SEED).random(A.noc)
    y = _mv(M, x)
    assert np.all(np.abs(y - O.crs_mv(A, x)) <= O.row_error_bound(A, x))
    xr, yr = O.power(A, x, 100)
    xg, yg = x.copy(), np.zeros(A.nor)
    M.powerIteration(xg, yg, 100)
    np.testing.assert_allclose(xg, xr, rtol=1e-10, atol=1e-15)
    lam_g, _ = O.rayleigh(A, xg)
    lam_r, _ = O.rayleigh(A, xr)
    assert abs(lam_g - lam_r) <= 1e-10 * abs(lam_r)


def test_c2_poisson4096_arrays_spmv_and_properties(pwm):
    A = O.fill_poisson(4096, 4096)
    assert A.nor == 16777216 and A.row_start[-1] == 83869696
    M = pwm.CRSCuda(1)
    M.generatePoissonMatrix(4096, 4096, 1)
    rs, ci, dv = M.getCSR()
    assert np.array_equal(rs, A.row_start) and np.array_equal(ci, A.col_ind) and np.array_equal(dv, A.data)
    del rs, ci, dv
    x = np.random.default_rng(SEED).random(A.noc)
    y = _mv(M, x)
    assert np.all(np.abs(y - O.crs_mv(A, x)) <= O.row_error_bound(A, x))
    # exact properties: row sums for x = 1 (integers), linearity under an exact scaling
    ones = np.ones(A.noc)
    assert np.array_equal(_mv(M, ones), O.crs_mv(A, ones))
    assert np.array_equal(_mv(M, 2.0 * x), 2.0 * y)
    # 20 power iterations (reference powerIteration semantics) against the oracle
    xr, yr = O.power(A, x, 20)
    xg, yg = x.copy(), np.zeros(A.nor)
    M.powerIteration(xg, yg, 20)
    np.testing.assert_allclose(xg, xr, rtol=1e-10, atol=1e-15)


def test_c3_irregular_arrays_spmv_and_solves(pwm):
    B = O.random_crs(IRREGULAR["n"], IRREGULAR["seed"], IRREGULAR["length_dist"], IRREGULAR["mean_len"],
                     IRREGULAR["sigma"], IRREGULAR["max_len"], IRREGULAR["band_permille"], IRREGULAR["band_half"])
    M = pwm.CRSCuda(1)
    M.generateRandom(**IRREGULAR)
    rs, ci, dv = M.getCSR()
    assert np.array_equal(rs, B.row_start) and np.array_equal(ci, B.col_ind) and np.array_equal(dv, B.data)
    del rs, ci, dv
    x = np.random.default_rng(SEED).random(B.noc)
    assert np.all(np.abs(_mv(M, x) - O.crs_mv(B, x)) <= O.row_error_bound(B, x))
    lams = {}
    for prec in (pwm.PREC_F64, pwm.PREC_MIXED):
        u = np.random.default_rng(SEED).random(B.noc)
        info = M.solve(u, 2000, 1e-10, prec)
        assert info.converged and info.residual <= 1e-10
        lam, res = O.rayleigh(B, u)  # the oracle's FP64 check of the returned eigenpair
        assert res <= 1.01e-10 and abs(lam - info.lambda_) <= 1e-10 * abs(lam)
        lams[prec] = info.lambda_
    assert abs(lams[pwm.PREC_MIXED] - lams[pwm.PREC_F64]) <= 1e-10 * abs(lams[pwm.PREC_F64])


@pytest.mark.parametrize("fmt", ["csb", "coh"])
def test_c2_poisson4096_other_formats(pwm, fmt):
    """The 4096^2 matrix in the CSB format (load-time variant choice) and
    the CO-H format (24 partitions per SM, as the bench runs it): SpMV within
    the row bound, and the exact row sums for x = 1."""
    import ctypes as C
    sm = C.c_int()
    pwm.lib().pwmgpu_device_info(C.byref(sm), None, None)
    A = O.fill_poisson(4096, 4096)
    M = pwm.CSBCuda(1) if fmt == "csb" else pwm.COHCuda(24 * sm.value)
    M.generatePoissonMatrix(4096, 4096, 1)
    x = np.random.default_rng(SEED + 1).random(A.noc)
    assert np.all(np.abs(_mv(M, x) - O.crs_mv(A, x)) <= O.row_error_bound(A, x))
    ones = np.ones(A.noc)
    assert np.array_equal(_mv(M, ones), O.crs_mv(A, ones))


@pytest.fixture(scope="module")
def irregular():
    """The irregular matrix's CRS arrays (oracle restatement of the device
    generator) and a seeded start vector, shared by the format tests."""
    B = O.random_crs(IRREGULAR["n"], IRREGULAR["seed"], IRREGULAR["length_dist"], IRREGULAR["mean_len"],
                     IRREGULAR["sigma"], IRREGULAR["max_len"], IRREGULAR["band_permille"], IRREGULAR["band_half"])
    x = np.random.default_rng(SEED + 2).random(B.noc)
    return B, x, O.crs_mv(B, x), O.row_error_bound(B, x), O.power(B, x, 10)


@pytest.mark.parametrize("fmt", ["csb", "coh"])
def test_c3_irregular_other_formats(pwm, irregular, fmt):
    """The irregular matrix (N = 4,194,304, lognormal row lengths up to 20,000,
    70 % of the columns uniform over [0, N)) in the CSB format (the variant its
    load-time tuner picks: flat units of sparse sub-squares with x gathered by
    global column) and the CO-H format (24 partitions per SM): each SpMV row
    within the bound of the oracle's CRS::mv, and 10 power iterations
    (SOA_Implementations/CSB.hpp:651-663, BlockCOH.hpp:519-531) within 1e-10
    of the oracle's CRS::powerIteration."""
    import ctypes as C
    B, x, ref, bound, (xr, yr) = irregular
    sm = C.c_int()
    pwm.lib().pwmgpu_device_info(C.byref(sm), None, None)
    M = pwm.CSBCuda(1) if fmt == "csb" else pwm.COHCuda(24 * sm.value)
    M.generateRandom(**IRREGULAR)
    assert np.all(np.abs(_mv(M, x) - ref) <= bound)
    xg, yg = x.copy(), np.zeros(B.nor)
    M.powerIteration(xg, yg, 10)
    np.testing.assert_allclose(xg, xr, rtol=1e-10, atol=1e-15)
