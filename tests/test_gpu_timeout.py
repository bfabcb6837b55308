"""Failure detection without a GPU fault: the persistent power kernel's grid
barriers are bounded waits.  A test-only setting (pwmgpu_test_grid_wait) asks
every barrier for one CTA more than the grid has, with a budget of 1e5 clock
cycles (about 50 us), so no barrier can open: every CTA gives up, records
PWMGPU_ERR_TIMEOUT in the handle's status word and returns.  The call must
report that status, and the same handle, back on the default budget, must run
the next power iteration to the oracle's result (status word and barrier
words reset by the host).  Nothing faults or traps; every wait ends."""
import ctypes as C

import numpy as np
import pytest

from oracle import pyoracle as O


def _lib():
    import thesis_spmv_gb300 as t
    return t, t.lib()


def test_grid_wait_arguments_are_checked():
    t, L = _lib()
    assert L.pwmgpu_test_grid_wait(None, 100000, 1) == 1  # null handle: PWMGPU_ERR_INVALID


@pytest.mark.gpu
@pytest.mark.parametrize("grid", [(16, 16), (120, 100)])
def test_grid_barrier_timeout_is_reported_and_the_handle_recovers(grid):
    t, L = _lib()
    m, n = grid
    A = O.fill_poisson(m, n)
    M = t.CRSCuda(1)
    M.generatePoissonMatrix(m, n, 1)
    M.set_power_mode(t.POWER_FUSED)  # the persistent kernel, whose grid barriers are under test
    for bad in ((5000, 1), (100000, 2), (10 ** 10, 0)):
        assert L.pwmgpu_test_grid_wait(M.handle, *bad) == 1
    assert L.pwmgpu_test_grid_wait(M.handle, 100000, 1) == 0
    x = np.random.default_rng(3).random(A.nor)
    with pytest.raises(t.PwmGpuError) as err:
        M.powerIteration(x.copy(), np.zeros(A.nor), 6)
    assert err.value.code == 4, str(err.value)  # PWMGPU_ERR_TIMEOUT
    assert "timed out" in str(err.value)
    # a solve on the persistent kernel reports the timeout too
    with pytest.raises(t.PwmGpuError) as err:
        M.solve(x.copy(), 40, 0.0, t.PREC_F64)
    assert err.value.code == 4
    # back to the default budget: the same handle gives the oracle's result
    assert L.pwmgpu_test_grid_wait(M.handle, 0, 0) == 0
    xg, yg = x.copy(), np.zeros(A.nor)
    M.powerIteration(xg, yg, 6)
    xr, yr = O.power(A, x, 6)
    np.testing.assert_allclose(xg, xr, rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(yg, yr, rtol=1e-12, atol=1e-15)
