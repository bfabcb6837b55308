"""Seeded random matrices (the irregular and batch benchmark inputs).

CPU: the oracle's restatement has the stated shape -- sorted duplicate-free
columns, values in (0, 1], the row-length distribution's mean and the band
fraction.  GPU: the device generator reproduces it bit for bit."""
import numpy as np
import pytest

from oracle import pyoracle as O

PARAMS = [
    # n, seed, kind, mean, sigma, max_len, band_permille, band_half
    (20000, 20261203, 0, 16.0, 1.2, 20000, 300, 4096),
    (5000, 7, 0, 16.0, 1.2, 20000, 300, 4096),
    (30000, 11, 1, 8.0, 0.0, 64, 0, 0),
    (1, 3, 1, 8.0, 0.0, 64, 0, 0),
    (7, 5, 0, 4.0, 1.0, 50, 500, 2),
    (3000, 99, 0, 40.0, 0.5, 2000, 1000, 10),
]


def test_length_tables():
    t = O.random_table(0, 16.0, 1.2, 20000)
    assert t[0] == 0 and t[-1] == 2 ** 53 and np.all(np.diff(t.astype(np.float64)) >= 0)
    p = O.random_table(1, 8.0, 0.0, 64)
    assert p[0] > 0 and p[-1] == 2 ** 53 and np.all(np.diff(p.astype(np.float64)) >= 0)


@pytest.mark.parametrize("prm", PARAMS[:3] + PARAMS[4:])
def test_oracle_random_matrix_shape(prm):
    n, seed, kind, mean, sigma, max_len, bp, bh = prm
    A = O.random_crs(n, seed, kind, mean, sigma, max_len, bp, bh)
    rs, ci, d = A.row_start, A.col_ind, A.data
    assert rs[0] == 0 and np.all(np.diff(rs) >= 0) and rs[-1] == ci.size
    assert np.all((ci >= 0) & (ci < n))
    rows = np.repeat(np.arange(n), np.diff(rs))
    # strictly ascending within each row
    same = rows[1:] == rows[:-1]
    assert np.all(ci[1:][same] > ci[:-1][same])
    assert np.all((d > 0) & (d <= 1))
    if n >= 20000:
        lens = np.diff(rs)
        assert abs(lens.mean() - mean) < 0.05 * mean
    if bp == 300 and n >= 20000:
        band = np.abs(ci - rows) <= bh
        # 30 % drawn from the band, plus the uniform draws that land in it
        i = np.arange(n)
        wb = np.minimum(n - 1, i + bh) - np.maximum(0, i - bh) + 1
        expect = 0.3 + 0.7 * wb.mean() / n
        assert abs(band.mean() - expect) < 0.03


def test_oracle_random_matrix_deterministic():
    a = O.random_crs(4000, 5)
    b = O.random_crs(4000, 5)
    c = O.random_crs(4000, 6)
    assert np.array_equal(a.col_ind, b.col_ind) and np.array_equal(a.data, b.data)
    assert not np.array_equal(a.row_start, c.row_start)


@pytest.mark.gpu
@pytest.mark.parametrize("prm", PARAMS)
def test_device_generator_bitexact(prm):
    import thesis_spmv_gb300 as t
    n, seed, kind, mean, sigma, max_len, bp, bh = prm
    M = t.CRSCuda(1)
    M.generateRandom(n, seed, kind, mean, sigma, max_len, bp, bh)
    rs, ci, d = M.getCSR()
    A = O.random_crs(n, seed, kind, mean, sigma, max_len, bp, bh)
    assert np.array_equal(rs, A.row_start)
    assert np.array_equal(ci, A.col_ind)
    assert np.array_equal(d.view(np.uint64), A.data.view(np.uint64))


@pytest.mark.gpu
def test_device_generator_spmv_and_invalid_args():
    import thesis_spmv_gb300 as t
    M = t.CRSCuda(1)
    M.generateRandom(50000, 1234)
    A = O.random_crs(50000, 1234)
    x = np.random.default_rng(0).uniform(-1, 1, A.noc)
    y = np.zeros(A.nor)
    M.mv(x, y)
    assert np.all(np.abs(y - O.crs_mv(A, x)) <= O.row_error_bound(A, x))
    for bad in [dict(n=0), dict(length_dist=5), dict(mean_len=-1.0), dict(sigma=0.0), dict(max_len=0),
                dict(band_permille=1001), dict(band_half=-1)]:
        kw = dict(n=10, seed=1, length_dist=0, mean_len=16.0, sigma=1.2, max_len=100, band_permille=300,
                  band_half=4)
        kw.update(bad)
        with pytest.raises(t.PwmGpuError):
            M.generateRandom(**kw)
