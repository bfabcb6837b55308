"""Format autotuner (PWMGPU_FMT_AUTO handles, selectType method 15) and the
CSB kernel variants it chooses among.

CPU: the class key (features of Util_Scripts/calc_stats.cpp:45-98) and the
class table's record / list / reset.  GPU: every CSB kernel variant against
the oracle's CRS::mv (rows within 2*nnz_row*u*sum|a_ij*x_j|, u = 2^-53); an
AUTO handle times the candidates on the first matrix of a class and takes
the recorded choice on the next; recorded CSB / CO-H choices run those
kernels; mv and powerIteration of every AUTO handle match the oracle.
"""
import numpy as np
import pytest

from oracle import pyoracle as O

POISSON_STATS = dict(size=16777216, nnz=83869696, rows_avg=4.9990234375, rows_var=0.000976, block_avg=319.94,
                     block_var=47270312.5, balanced=1, block_bits=15, nb_blocks=512, max_row_nnz=5)
IRREGULAR_STATS = dict(size=4194304, nnz=67127838, rows_avg=16.0045, rows_var=819.84, block_avg=1024.29,
                       block_var=18626179.6, balanced=1, block_bits=14, nb_blocks=256, max_row_nnz=3578)


@pytest.fixture(scope="module")
def pwm():
    import thesis_spmv_gb300 as t
    t.lib()
    return t


def test_class_key_features(pwm):
    """size, mean row length, row-length spread, block spread, balance, longest
    row and SM count, each bucketed on a log scale."""
    assert pwm.class_key(POISSON_STATS, 152) == [24, 4, 0, 4, 1, 2, 152]
    assert pwm.class_key(IRREGULAR_STATS, 152) == [22, 8, 3, 2, 1, 11, 152]
    # the same class up to a bucket edge; another SM count is another class
    near = dict(POISSON_STATS, size=16777216 + 1000, nnz=83869696 + 5000)
    assert pwm.class_key(near, 152) == pwm.class_key(POISSON_STATS, 152)
    assert pwm.class_key(POISSON_STATS, 148)[6] == 148


def test_tuner_table_record_and_reset(pwm):
    pwm.tuner_reset()
    assert pwm.tuner_size() == 0
    pwm.tuner_record([1, 2, 3, 4, 1, 5, 152], "csb", 3, 1)
    pwm.tuner_record([1, 2, 3, 4, 1, 5, 152], "coh")  # replaces the entry
    pwm.tuner_record([9, 2, 3, 4, 1, 5, 152], "merge", 0, 5)
    pwm.tuner_record([5, 2, 3, 4, 1, 5, 152], "coh", 0, 0, 8)
    assert sorted(pwm.tuner_entries()) == [([1, 2, 3, 4, 1, 5, 152], "coh", 0, 0, 24),
                                            ([5, 2, 3, 4, 1, 5, 152], "coh", 0, 0, 8),
                                            ([9, 2, 3, 4, 1, 5, 152], "merge", 0, 5, 24)]
    with pytest.raises(pwm.PwmGpuError):
        pwm.tuner_record([0] * 7, "csb", 4, 0)
    with pytest.raises(pwm.PwmGpuError):
        pwm.tuner_record([0] * 7, "merge", 0, 2)
    with pytest.raises(pwm.PwmGpuError):
        pwm.tuner_record([0] * 7, "coh", 0, 0, 65)
    pwm.tuner_reset()
    assert pwm.tuner_entries() == []


# ---- GPU -------------------------------------------------------------------

# 1400^2 Poisson grid: 1.96 M rows, 9.8 M nonzeros, above the size from which
# the merge tuner (and so the format tuner) times candidates
GRID = 1400


def _check_mv(M, A, seed):
    x = np.random.default_rng(seed).random(A.noc)
    y = np.zeros(A.nor)
    M.mv(x, y)
    ref = O.crs_mv(A, x)
    assert np.all(np.abs(y - ref) <= O.row_error_bound(A, x))


@pytest.fixture(scope="module")
def poisson():
    return O.fill_poisson(GRID, GRID)


@pytest.mark.gpu
@pytest.mark.parametrize("variant", [0, 1, 2, 3])
def test_csb_variants_match_oracle(pwm, variant):
    """CSB with 4 / 8 elements per lane and 128 / 256 threads per CTA, on a
    stencil (all sub-squares dense) and a random matrix (mostly sparse
    sub-squares, a few long rows crossing warp chunks)."""
    A = O.fill_poisson(300, 200)
    M = pwm.CSBCuda(1)
    M.generatePoissonMatrix(300, 200, 1)
    M.set_csb_variant(variant)
    _check_mv(M, A, 1)
    B = O.random_crs(50000, seed=11, mean=24.0, sigma=1.2, max_len=5000, band_permille=600, band_half=300)
    R = pwm.CSBCuda(1)
    R.loadCSR(B.nor, B.noc, B.row_start, B.col_ind, B.data)
    R.set_csb_variant(variant)
    _check_mv(R, B, 2)


@pytest.mark.gpu
def test_auto_times_then_reuses_class(pwm, poisson):
    pwm.tuner_reset()
    M = pwm.selectType(15, 1)
    M.generatePoissonMatrix(GRID, GRID, 1)
    t = M.tuning()
    assert t["timed"] and not t["cache_hit"]
    assert t["format"] in ("merge", "csb", "coh")
    assert t["merge_ms"] > 0 and all(v > 0 for v in t["coh_ms"]) and all(v > 0 for v in t["csb_ms"])
    best = min([t["merge_ms"]] + t["coh_ms"] + t["csb_ms"])
    chosen = {"merge": t["merge_ms"], "coh": t["coh_ms"][t["csb_variant"]],
              "csb": t["csb_ms"][t["csb_variant"]]}[t["format"]]
    assert chosen == best
    assert pwm.tuner_size() == 1
    _check_mv(M, poisson, 3)
    # a second matrix of the class: the recorded choice, no timing
    M2 = pwm.AutoCuda(1)
    M2.generatePoissonMatrix(GRID, GRID, 1)
    t2 = M2.tuning()
    assert t2["cache_hit"] and not t2["timed"]
    assert (t2["format"], t2["csb_variant"], t2["class_key"]) == (t["format"], t["csb_variant"], t["class_key"])
    _check_mv(M2, poisson, 4)
    # powerIteration through the chosen format, against the oracle
    x0 = np.random.default_rng(5).random(poisson.noc)
    xr, yr = O.power(poisson, x0, 6)
    xg, yg = x0.copy(), np.zeros(poisson.nor)
    M2.powerIteration(xg, yg, 6)
    np.testing.assert_allclose(xg, xr, rtol=1e-10, atol=1e-14)


@pytest.mark.gpu
@pytest.mark.parametrize("fmt,variant,pps", [("csb", 0, 0), ("csb", 3, 0), ("coh", 0, 0), ("coh", 2, 8),
                                             ("merge", 0, 0)])
def test_auto_recorded_choice_runs_that_format(pwm, poisson, fmt, variant, pps):
    """A recorded class choice (as a tuning carried from another process)
    makes the AUTO handle run that format's kernel; results match the oracle
    and the merge-only paths (the solve) still work."""
    pwm.tuner_reset()
    probe = pwm.CRSCuda(1)
    probe.generatePoissonMatrix(GRID, GRID, 1)
    import ctypes as C
    sm = C.c_int()
    pwm.lib().pwmgpu_device_info(C.byref(sm), None, None)
    key = pwm.class_key(probe.stats(), sm.value)
    pwm.tuner_record(key, fmt, variant, 0, pps)
    M = pwm.AutoCuda(1)
    M.generatePoissonMatrix(GRID, GRID, 1)
    t = M.tuning()
    assert t["cache_hit"] and (t["format"], t["csb_variant"]) == (fmt, variant if fmt != "merge" else 0)
    assert t["coh_partitions"] == ((pps or 24) * sm.value if fmt == "coh" else 0)
    _check_mv(M, poisson, 6)
    x0 = np.random.default_rng(7).random(poisson.noc)
    xr, yr = O.power(poisson, x0, 5)
    xg, yg = x0.copy(), np.zeros(poisson.nor)
    M.powerIteration(xg, yg, 5)
    np.testing.assert_allclose(yg, yr, rtol=1e-10, atol=1e-14)
    info = M.solve(np.random.default_rng(8).random(poisson.noc), 20, 1e-10)
    assert 0 < info.iterations <= 20
    pwm.tuner_reset()


@pytest.mark.gpu
def test_auto_small_matrix_runs_merge(pwm):
    A = O.fill_poisson(40, 30)
    M = pwm.AutoCuda(1)
    M.generatePoissonMatrix(40, 30, 1)
    t = M.tuning()
    assert t["format"] == "merge" and not t["timed"] and not t["cache_hit"]
    _check_mv(M, A, 9)


def _long_row_matrix(n, seed):
    """Rows of very different lengths inside dense sub-squares: most rows hold
    a few entries near the diagonal, every 97th row 200-900 entries within
    +-30 columns, so mostly repeated coordinates (CRS keeps duplicates): in a
    dense sub-square such a row is a chain over many lanes (the
    segmented-scan branch) and longer than a warp's chunk (the atomic
    branch); some rows are empty."""
    rng = np.random.default_rng(seed)
    rows, cols = [], []
    for r in range(n):
        if r % 13 == 5:
            continue  # empty row
        if r % 97 == 0:
            k = int(rng.integers(200, 900))
            lo, hi = max(0, r - 30), min(n, r + 31)
            c = np.sort(rng.integers(lo, hi, k))  # with repeats
        else:
            c = np.unique(np.clip(r + rng.integers(-3, 4, int(rng.integers(1, 6))), 0, n - 1))
        rows.append(np.full(c.size, r))
        cols.append(c)
    r = np.concatenate(rows).astype(np.int32)
    c = np.concatenate(cols).astype(np.int32)
    rs = np.zeros(n + 1, np.int32)
    np.add.at(rs, r + 1, 1)
    rs = np.cumsum(rs).astype(np.int32)
    return O.CRSArrays(n, n, rs, c, rng.uniform(-1, 1, c.size))


@pytest.mark.gpu
@pytest.mark.parametrize("variant", [0, 1, 2, 3])
def test_csb_long_rows_and_duplicates(pwm, variant):
    A = _long_row_matrix(60000, 21)
    M = pwm.CSBCuda(1)
    M.loadCSR(A.nor, A.noc, A.row_start, A.col_ind, A.data)
    M.set_csb_variant(variant)
    for seed in (1, 2):
        _check_mv(M, A, 30 + seed)


@pytest.mark.gpu
def test_csb_handle_picks_variant_at_load(pwm, poisson):
    """A CSB handle on a matrix large enough to time picks one of the four
    variants at load time; the result matches the oracle; the variant can be
    overridden."""
    M = pwm.CSBCuda(1)
    M.generatePoissonMatrix(GRID, GRID, 1)
    assert M.csb_variant() in (0, 1, 2, 3)
    _check_mv(M, poisson, 41)
    M.set_csb_variant(3)
    assert M.csb_variant() == 3
    _check_mv(M, poisson, 42)


@pytest.mark.gpu
def test_service_precision_tuner_per_matrix_class():
    """The service's precision tuner: a mixed request runs one FP64 probe
    round, then keeps matrices that would finish within a few rounds in FP64
    (the random Poisson(8)-row class of the batch workload) and moves slowly
    converging ones (Poisson grids) to the FP32 / BF16 bulk phase.  Every
    result is confirmed by the oracle; the same requests in FP64 take the
    same number of steps where the tuner kept FP64."""
    from oracle import pyoracle as O
    from thesis_spmv_gb300 import service as S
    import thesis_spmv_gb300 as t
    rand = [dict(n=n, seed=1000 + i, length_dist=1, mean_len=8.0, sigma=0.0, max_len=64, band_permille=0,
                 band_half=0) for i, n in enumerate((3000, 40000, 200000))]
    grids = [(40, 40), (96, 64)]
    out = {}
    for prec in (t.PREC_MIXED, t.PREC_F64):
        svc = S.Service(round_iterations=8)
        ids = [svc.submit_random(max_it=2000, tol=1e-10, precision=prec, x0_seed=11, keep_vector=True, **kw)
               for kw in rand]
        ids += [svc.submit_poisson(m, n, max_it=2000, tol=1e-10, precision=prec, x0_seed=11, keep_vector=True)
                for m, n in grids]
        svc.run_until_idle()
        out[prec] = [svc.result(i, want_vector=True) for i in ids]
        svc.close()
    for j, kw in enumerate(rand):
        (rm, um), (r64, _) = out[t.PREC_MIXED][j], out[t.PREC_F64][j]
        assert rm.converged and rm.iterations_low == 0 and rm.iterations == r64.iterations
        lam, res = O.rayleigh(O.random_crs(kw["n"], kw["seed"], 1, 8.0, 0.0, 64, 0, 0), um)
        assert res <= 2e-10 and abs(lam - rm.lambda_) <= 1e-10 * abs(lam)
    for j, (m, n) in enumerate(grids):
        rm, um = out[t.PREC_MIXED][len(rand) + j]
        assert rm.iterations_low > 0
        lam, res = O.rayleigh(O.fill_poisson(m, n), um)
        assert abs(lam - rm.lambda_) <= 1e-10 * abs(lam) and abs(res - rm.residual) <= 1e-12
