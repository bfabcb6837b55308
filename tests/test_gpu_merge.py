"""GPU parity of the merge-path CRS path (K1 partition, K2 SpMV + fix-up,
power method) against the oracle, through the C ABI.

Tolerances: SpMV rows within 2*nnz_row*u*sum|a_ij*x_j| (u = 2^-53)
of the oracle's CRS::mv; builders and merge-path coordinates bit-exact; power
iterates at equal iteration counts within 1e-10 relative (eigenvalue
estimates likewise); the reference's own known answers at its tolerances.
"""
import numpy as np
import pytest

from golden_cases import boost_close, case_ids, cases, triplets_for
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

CASES = cases()


@pytest.fixture(scope="module")
def pwm():
    import thesis_spmv_gb300 as t
    t.lib()
    return t


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


def _gpu_matrix(pwm, A):
    M = pwm.CRSCuda(1)
    M.loadCSR(A.nor, A.noc, A.row_start, A.col_ind, A.data)
    return M


def _case_matrix(pwm, case):
    M = pwm.CRSCuda(1)
    t = triplets_for(case)
    if t is None:
        M.generatePoissonMatrix(case["input"]["m"], case["input"]["n"], 1)
        return M, case["input"]["m"] * case["input"]["n"]
    nor, noc, r, c, v = t
    M.loadFromTriplets(pwm.Triplet(nor, noc, r, c, v), 1)
    return M, noc


@pytest.mark.parametrize("case", CASES, ids=case_ids())
def test_reference_known_answers(pwm, case):
    """Tests/poisson.cpp and Tests/input.cpp, all 24 cases, at their tolerances."""
    M, n = _case_matrix(pwm, case)
    golden = np.array(case["golden"])
    x = np.ones(n)
    y = np.zeros(golden.size)
    if case["op"]["kind"] == "mv":
        M.mv(x, y)
        out = y
    else:
        M.powerIteration(x, y, case["op"]["iterations"])
        out = x  # 100 iterations: result in x (CRS.hpp:121-129)
    assert boost_close(out, golden, case["tolerance"]).all()


@pytest.mark.parametrize("mn", [(1, 1), (1, 7), (7, 1), (3, 3), (9, 3), (64, 33), (512, 512)])
def test_device_poisson_generator_bitexact(pwm, mn):
    M = pwm.CRSCuda(1)
    M.generatePoissonMatrix(*mn, 1)
    rs, ci, d = M.getCSR()
    A = O.fill_poisson(*mn)
    assert np.array_equal(rs, A.row_start) and np.array_equal(ci, A.col_ind) and np.array_equal(d, A.data)


@pytest.mark.parametrize("name", ["arc130.mtx", "gre_1107.mtx", "G38.mtx"])
def test_triplet_to_crs_bitexact(pwm, name):
    c = [c for c in CASES if c["input"].get("file") == name][0]
    nor, noc, r, cc, v = triplets_for(c)
    T = pwm.Triplet(nor, noc, r.copy(), cc.copy(), v.copy())
    M = pwm.CRSCuda(1)
    M.loadFromTriplets(T, 1)
    A = O.triplet_to_crs(nor, noc, r, cc, v)
    rs, ci, d = M.getCSR()
    assert np.array_equal(rs, A.row_start) and np.array_equal(ci, A.col_ind) and np.array_equal(d, A.data)
    # the caller's triplet is left sorted, as TripletToCRS leaves it (TripletToCRS.hpp:139-142)
    assert np.array_equal(T.row_coord, r) and np.array_equal(T.col_coord, cc) and np.array_equal(T.data, v)


@pytest.mark.parametrize("parts", [1, 2, 3, 7, 8, 31, 152, 1000])
def test_merge_partition_bitexact(pwm, parts):
    for A in (O.fill_poisson(37, 29), _random_csr(3000, 4, 5, empty_frac=0.2, dense_rows=2, dense_len=2500)):
        M = _gpu_matrix(pwm, A)
        assert np.array_equal(M.merge_partition(parts), O.merge_partition(A, parts))


def test_partition_kernel_many_parts(pwm):
    A = _random_csr(20000, 6, 9, empty_frac=0.1, dense_rows=4, dense_len=15000)
    M = _gpu_matrix(pwm, A)
    tm, nt, grid = M.tile_info()
    total = A.nor + A.nnz
    assert nt == -(-total // tm)
    # the tile ends are the merge path at diagonals t*TM; K1 with ipt = TM
    parts = M.merge_partition(nt)
    want = [O.merge_search(A, min(t * (-(-total // nt)), total)) for t in range(nt + 1)]
    assert [tuple(p) for p in parts] == want


def _check_spmv(pwm, A, seed=0):
    M = _gpu_matrix(pwm, A)
    x = np.random.default_rng(seed).uniform(-1, 1, A.noc)
    y = np.full(A.nor, np.nan)
    M.mv(x, y)
    ref = O.crs_mv(A, x)
    bound = O.row_error_bound(A, x)
    bad = np.abs(y - ref) > bound
    assert not bad.any(), (np.nonzero(bad)[0][:10], y[bad][:5], ref[bad][:5])
    return M, x, y


@pytest.mark.parametrize("kind", ["poisson_small", "poisson_c1", "random", "empty_rows", "dense_rows",
                                  "rectangular_wide", "rectangular_tall", "nnz0", "single", "one_dense_row"])
def test_spmv_row_bound(pwm, kind):
    A = {
        "poisson_small": lambda: O.fill_poisson(37, 29),
        "poisson_c1": lambda: O.fill_poisson(512, 512),
        "random": lambda: _random_csr(50000, 8, 1),
        "empty_rows": lambda: _random_csr(30000, 3, 2, empty_frac=0.5),
        "dense_rows": lambda: _random_csr(20000, 4, 3, dense_rows=5, dense_len=19000),
        "rectangular_wide": lambda: _random_csr(3000, 9, 4, noc=70000),
        "rectangular_tall": lambda: _random_csr(70000, 2, 5, noc=300),
        "nnz0": lambda: _random_csr(5000, 0, 6),
        "single": lambda: O.CRSArrays(1, 1, np.array([0, 1], np.int32), np.array([0], np.int32), np.array([2.5])),
        "one_dense_row": lambda: O.CRSArrays(1, 40000, np.array([0, 40000], np.int32),
                                             np.arange(40000, dtype=np.int32),
                                             np.random.default_rng(8).random(40000)),
    }[kind]()
    _check_spmv(pwm, A)


def test_spmv_deterministic(pwm):
    A = _random_csr(40000, 7, 11, dense_rows=3, dense_len=30000)
    M, x, y = _check_spmv(pwm, A)
    y2 = np.zeros_like(y)
    for _ in range(3):
        M.mv(x, y2)
        assert np.array_equal(y, y2)


def test_spmv_device_pointers_and_stream(pwm):
    torch = pytest.importorskip("torch")
    A = O.fill_poisson(300, 200)
    M = _gpu_matrix(pwm, A)
    x = np.random.default_rng(3).random(A.noc)
    dx = torch.tensor(x, device="cuda", dtype=torch.float64)
    dy = torch.zeros(A.nor, device="cuda", dtype=torch.float64)
    s = torch.cuda.Stream()
    M.set_stream(s.cuda_stream)
    with torch.cuda.stream(s):
        M.mv_device(dx.data_ptr(), dy.data_ptr())
    s.synchronize()
    ref = O.crs_mv(A, x)
    assert np.all(np.abs(dy.cpu().numpy() - ref) <= O.row_error_bound(A, x))


@pytest.mark.parametrize("mode", ["fused", "multi"])
@pytest.mark.parametrize("it", [1, 2, 3, 10, 55])
def test_power_iteration_equal_counts(pwm, it, mode):
    """x / y placement and values of powerIteration (CRS.hpp:118-130), with
    the persistent kernel (fused) and with two kernels per iteration."""
    A = _random_csr(5000, 6, 21)
    A.data = np.abs(A.data) + 0.01  # positive: a dominant Perron eigenvalue
    M = _gpu_matrix(pwm, A)
    M.set_power_mode(pwm.POWER_FUSED if mode == "fused" else pwm.POWER_MULTI)
    x0 = np.random.default_rng(4).random(A.nor)
    xg, yg = x0.copy(), np.zeros(A.nor)
    M.powerIteration(xg, yg, it)
    xr, yr = O.power(A, x0, it)
    np.testing.assert_allclose(xg, xr, rtol=1e-10, atol=1e-13)
    np.testing.assert_allclose(yg, yr, rtol=1e-10, atol=1e-13)
    if it == 1:
        assert np.array_equal(xg, x0)  # untouched input, as in the reference


def test_power_poisson_eigenvalue_estimate(pwm):
    """Norm-ratio eigenvalue estimate after equal counts agrees to 1e-10."""
    m = 40
    A = O.fill_poisson(m, m)
    M = _gpu_matrix(pwm, A)
    x0 = np.random.default_rng(2).random(A.nor)
    for it in (50, 51):
        xg, yg = x0.copy(), np.zeros(A.nor)
        M.powerIteration(xg, yg, it)
        xr, yr = O.power(A, x0, it)
        ug = xg if it % 2 == 0 else yg
        ur = xr if it % 2 == 0 else yr
        lam_g = O.norm2(O.crs_mv(A, ug))
        lam_r = O.norm2(O.crs_mv(A, ur))
        assert abs(lam_g - lam_r) <= 1e-10 * abs(lam_r)


def test_power_rejects_rectangular(pwm):
    A = _random_csr(100, 3, 1, noc=120)
    M = _gpu_matrix(pwm, A)
    with pytest.raises(pwm.PwmGpuError):
        M.powerIteration(np.ones(120), np.zeros(120), 3)


def test_invalid_csr_rejected(pwm):
    M = pwm.CRSCuda(1)
    with pytest.raises(pwm.PwmGpuError):
        M.loadCSR(3, 3, np.array([0, 1, 2, 3]), np.array([0, 5, 1]), np.ones(3))  # column out of range
    with pytest.raises(pwm.PwmGpuError):
        M.loadCSR(3, 3, np.array([0, 2, 1, 3]), np.array([0, 1, 1]), np.ones(3))  # decreasing row_start
    with pytest.raises(pwm.PwmGpuError):
        M.mv(np.ones(3), np.zeros(3))  # nothing loaded


@pytest.mark.parametrize("scale", [1e150, 1e-150, 1e30])
@pytest.mark.parametrize("mode", ["fused", "multi"])
def test_power_extreme_scales(pwm, scale, mode):
    """Entries of size 1e150 / 1e-150: the iterate's norm leaves the rescale
    window within an iteration or two, so the exact power-of-two rescale must
    keep it finite; results equal the oracle's, which normalises every
    iteration (CRS.hpp:118-130)."""
    A = _random_csr(3000, 5, 17)
    A.data = (np.abs(A.data) + 0.01) * scale
    M = _gpu_matrix(pwm, A)
    M.set_power_mode(pwm.POWER_FUSED if mode == "fused" else pwm.POWER_MULTI)
    x0 = np.random.default_rng(3).random(A.nor)
    for it in (7, 30):
        xg, yg = x0.copy(), np.zeros(A.nor)
        M.powerIteration(xg, yg, it)
        xr, yr = O.power(A, x0, it)
        assert np.all(np.isfinite(xg)) and np.all(np.isfinite(yg))
        np.testing.assert_allclose(xg, xr, rtol=1e-10, atol=1e-13)
        np.testing.assert_allclose(yg, yr, rtol=1e-10, atol=1e-13)


@pytest.mark.parametrize("kind", ["poisson", "random"])
def test_launch_tuner_variants_same_bits(pwm, kind):
    """The load-time tuner times the launch variants of the merge kernels on
    a matrix large enough to tune; all give the same SpMV bits (a sub-tile is
    computed the same whichever warp takes it and whichever cache path its x
    gathers take); the power method's norms are summed in grid-dependent
    order, so its iterates agree to rounding."""
    M = pwm.CRSCuda(1)
    if kind == "poisson":
        M.generatePoissonMatrix(2048, 2048, 1)
    else:
        M.generateRandom(1_500_000, 77, mean_len=16.0)
    l1, grid, pgrid, ms = M.launch_config()
    assert ms[0] > 0 and ms[1] > 0 and l1 in (0, 1) and grid > 0 and pgrid > 0
    assert M.launch_variant() in range(8)
    n = M.dims()[0]
    x = np.random.default_rng(2).uniform(-1, 1, n)
    ys, ps = [], []
    for v in (0, 1, 4, 5):
        M.set_launch_variant(v)
        assert M.launch_variant() & ~2 == v
        y = np.zeros(n)
        M.mv(x, y)
        ys.append(y)
        xp, yp = x.copy(), np.zeros(n)
        M.powerIteration(xp, yp, 3)
        ps.append(yp)
    for y in ys[1:]:
        assert np.array_equal(ys[0], y)
    for p in ps[1:]:
        np.testing.assert_allclose(ps[0], p, rtol=1e-13, atol=1e-15)
    rs, ci, d = M.getCSR()
    A = O.CRSArrays(n, n, rs, ci, d)
    assert np.all(np.abs(ys[0] - O.crs_mv(A, x)) <= O.row_error_bound(A, x))
    with pytest.raises(RuntimeError):
        M.set_launch_variant(2)


@pytest.mark.parametrize("offset", [0, 1])
def test_pipelined_host_mv_pageable_and_pinned(pwm, offset):
    """Host arrays that are pinned go through the copy engines; pageable ones
    (where the GPU reaches pageable memory) through SM copy kernels -- both at
    any 8-byte offset, with the same bits as the device-resident path."""
    torch = pytest.importorskip("torch")
    M = pwm.CRSCuda(1)
    M.generatePoissonMatrix(701, 899, 1)
    n = M.dims()[0]
    x = np.random.default_rng(8).uniform(-1, 1, n)
    dx = torch.tensor(x, device="cuda")
    dy = torch.zeros(n, dtype=torch.float64, device="cuda")
    M.mv_device(dx.data_ptr(), dy.data_ptr())
    torch.cuda.synchronize()
    want = dy.cpu().numpy()
    # pageable, shifted by `offset` doubles (8-byte phase of a 16-byte boundary)
    xb = np.empty(n + 1)
    yb = np.full(n + 1, np.nan)
    xa, ya = xb[offset:offset + n], yb[1 - offset:1 - offset + n]
    xa[:] = x
    for _ in range(2):
        ya[:] = np.nan
        M.mv(xa, ya)
        assert np.array_equal(ya, want)
    # pinned
    xp = torch.tensor(x).pin_memory()
    yp = torch.full((n,), float("nan"), dtype=torch.float64).pin_memory()
    M.mv(xp.numpy(), yp.numpy())
    assert np.array_equal(yp.numpy(), want)


@pytest.mark.parametrize("kind", ["poisson", "random", "long_rows"])
def test_pipelined_host_mv_same_bits(pwm, kind):
    """pwmgpu_mv on host arrays runs pipelined (x up in pieces, the SpMV in
    chunks, y down per chunk) for matrices large enough; it must give the
    same bits as the device-resident path."""
    torch = pytest.importorskip("torch")
    M = pwm.CRSCuda(1)
    if kind == "poisson":
        M.generatePoissonMatrix(700, 900, 1)
    elif kind == "random":
        M.generateRandom(600_000, 5, mean_len=12.0)
    else:  # lognormal rows up to 20000 long: runs of sub-tiles cross chunks
        M.generateRandom(120_000, 9, mean_len=60.0, sigma=1.6, max_len=20000)
    n = M.dims()[0]
    x = np.random.default_rng(7).uniform(-1, 1, n)
    y = np.full(n, np.nan)
    M.mv(x, y)
    dx = torch.tensor(x, device="cuda")
    dy = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    M.mv_device(dx.data_ptr(), dy.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(y, dy.cpu().numpy())
    rs, ci, d = M.getCSR()
    A = O.CRSArrays(n, n, rs, ci, d)
    assert np.all(np.abs(y - O.crs_mv(A, x)) <= O.row_error_bound(A, x))


def test_sixteen_bit_columns_where_spans_fit(pwm):
    """Stencil / banded matrices stream 16-bit column offsets (2 bytes per
    nonzero less); a matrix with columns spread over 4M does not; both give
    the oracle's SpMV, and the merge, CSB and CO-H formats agree on Poisson."""
    M = pwm.CRSCuda(1)
    M.generatePoissonMatrix(1500, 1300, 1)
    assert M.column_bytes() == 2
    n = M.dims()[0]
    x = np.random.default_rng(3).uniform(-1, 1, n)
    y = np.zeros(n)
    M.mv(x, y)
    rs, ci, d = M.getCSR()
    A = O.CRSArrays(n, n, rs, ci, d)
    assert np.all(np.abs(y - O.crs_mv(A, x)) <= O.row_error_bound(A, x))
    xs, ys = x.copy(), np.zeros(n)
    M.powerIteration(xs, ys, 5)
    xr, yr = O.power(A, x.copy(), 5)
    assert np.allclose(ys, yr, rtol=1e-12, atol=1e-14)
    R = pwm.CRSCuda(1)
    R.generateRandom(300_000, 4, mean_len=10.0)
    assert R.column_bytes() == 4
    # a span of exactly 65535 fits, 65536 does not
    for span, want in ((65535, 2), (65536, 4)):
        nn = 70_000
        rows = np.arange(nn, dtype=np.int32)  # the identity plus (0, span)
        B = pwm.CRSCuda(1)
        B.loadFromTriplets(pwm.Triplet(nn, nn, np.concatenate([rows, [0]]).astype(np.int32),
                                       np.concatenate([rows, [span]]).astype(np.int32), np.ones(nn + 1)), 1)
        assert B.column_bytes() == want
        xb = np.random.default_rng(5).random(nn)
        yb = np.zeros(nn)
        B.mv(xb, yb)
        want_y = xb.copy()
        want_y[0] += xb[span]
        assert np.allclose(yb, want_y, rtol=1e-15, atol=0)
