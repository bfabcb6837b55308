"""numpy front end of the C oracle (oracle/oracle.c).  Test infrastructure only.

Every function maps one-to-one onto an ``orc_*`` function of oracle.h, which
cites the reference function it restates.
"""
import ctypes as C
import os

import numpy as np

from .build import build_oracle

_lib = None

I32P = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
U32P = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
U16P = np.ctypeslib.ndpointer(np.uint16, flags="C_CONTIGUOUS")
I16P = np.ctypeslib.ndpointer(np.int16, flags="C_CONTIGUOUS")
F64P = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


def lib():
    global _lib
    if _lib is None:
        path = build_oracle()
        L = C.CDLL(path)
        L.orc_poisson_nnz.restype = C.c_int64
        L.orc_poisson_nnz.argtypes = [C.c_int32, C.c_int32]
        L.orc_fill_poisson.argtypes = [C.c_int32, C.c_int32, I32P, I32P, F64P]
        L.orc_triplet_poisson.argtypes = [C.c_int32, C.c_int32, I32P, I32P, F64P]
        L.orc_triplet_to_crs.argtypes = [C.c_int32, C.c_int32, I32P, I32P, F64P, I32P, I32P, F64P]
        L.orc_crs_mv.argtypes = [C.c_int32, I32P, I32P, F64P, F64P, F64P]
        L.orc_row_blocks.argtypes = [C.c_int32, C.c_int32, I32P, I32P]
        L.orc_triplet_to_multi_crs.argtypes = [C.c_int32, C.c_int32, C.c_int32, I32P, I32P, F64P, I32P, I32P, I32P,
                                               I32P, F64P]
        L.orc_fill_poisson_rows.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_int32, I32P, I32P, F64P]
        L.orc_power_rows.argtypes = [C.c_int32, C.c_int32, I32P, I32P, F64P, F64P, C.c_int32]
        L.orc_crs_omp_mv.argtypes = [C.c_int32, I32P, I32P, F64P, F64P, F64P, C.c_int]
        L.orc_merge_search.argtypes = [C.c_int32, C.c_int32, C.c_int32, I32P, C.POINTER(C.c_int32),
                                       C.POINTER(C.c_int32)]
        L.orc_merge_partition.argtypes = [C.c_int32, C.c_int32, I32P, C.c_int32, I32P]
        L.orc_merge_mv.argtypes = [C.c_int32, C.c_int32, I32P, I32P, F64P, F64P, F64P, C.c_int32]
        L.orc_merge_omp_mv.argtypes = [C.c_int32, C.c_int32, I32P, I32P, F64P, F64P, F64P, C.c_int32]
        L.orc_norm2.restype = C.c_double
        L.orc_norm2.argtypes = [F64P, C.c_int64]
        L.orc_normalize.argtypes = [F64P, C.c_int64]
        L.orc_power.argtypes = [C.c_int, C.c_int32, C.c_int32, I32P, I32P, F64P, F64P, F64P, C.c_int32, C.c_int]
        L.orc_rayleigh.argtypes = [C.c_int32, I32P, I32P, F64P, F64P, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_random_table.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int32, C.c_void_p]
        L.orc_random_crs.argtypes = [C.c_int32, C.c_uint64, C.c_int, C.c_double, C.c_double, C.c_int32, C.c_int32,
                                     C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_random_crs.restype = C.c_int64
        L.orc_uniform_vector.argtypes = [C.c_int32, C.c_uint64, C.c_void_p]
        L.orc_csb_params.argtypes = [C.c_int32, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
        L.orc_csb_build.restype = C.c_int
        L.orc_csb_build.argtypes = [C.c_int32, C.c_int32, C.c_int32, I32P, I32P, F64P, U32P, F64P, I32P]
        L.orc_csb_mv.argtypes = [C.c_int32, C.c_int32, U32P, F64P, I32P, F64P, F64P]
        L.orc_hilbert.restype = C.c_int32
        L.orc_hilbert.argtypes = [C.c_int32, C.c_int32, C.c_int32]
        L.orc_coh_sizes.restype = C.c_int
        L.orc_coh_sizes.argtypes = [C.c_int32, C.c_int32, C.c_int32, I32P, I32P, C.c_int32,
                                    C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.orc_coh_build.restype = C.c_int
        L.orc_coh_build.argtypes = [C.c_int32, C.c_int32, C.c_int32, I32P, I32P, F64P, C.c_int32, I32P, U16P,
                                    U16P, F64P, I32P, I16P, I16P]
        L.orc_coh_mv.argtypes = [C.c_int32, C.c_int32, I32P, U16P, U16P, F64P, I32P, I16P, I16P, F64P, F64P]
        L.orc_load_mm.restype = C.c_int64
        L.orc_load_mm.argtypes = [C.c_char_p, C.c_int, C.c_int, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64]
        L.orc_load_bin.restype = C.c_int64
        L.orc_load_bin.argtypes = [C.c_char_p, C.c_int32, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64]
        L.orc_calc_stats.restype = C.c_int
        L.orc_calc_stats.argtypes = [C.c_int64, C.c_int32, C.c_void_p, C.c_void_p, F64P]
        _lib = L
    return _lib


class CRSArrays:
    """Plain CRS arrays (row_start[nor+1], col_ind[nnz], data[nnz])."""

    def __init__(self, nor, noc, row_start, col_ind, data):
        self.nor, self.noc = int(nor), int(noc)
        self.row_start = np.ascontiguousarray(row_start, dtype=np.int32)
        self.col_ind = np.ascontiguousarray(col_ind, dtype=np.int32)
        self.data = np.ascontiguousarray(data, dtype=np.float64)

    @property
    def nnz(self):
        return int(self.col_ind.size)


def poisson_nnz(m, n):
    return int(lib().orc_poisson_nnz(m, n))


def fill_poisson(m, n):
    nnz = poisson_nnz(m, n)
    rs = np.zeros(m * n + 1, np.int32)
    ci = np.zeros(max(nnz, 1), np.int32)
    d = np.zeros(max(nnz, 1), np.float64)
    lib().orc_fill_poisson(m, n, rs, ci, d)
    return CRSArrays(m * n, m * n, rs, ci[:nnz], d[:nnz])


def triplet_poisson(m, n):
    nnz = poisson_nnz(m, n)
    r = np.zeros(max(nnz, 1), np.int32)
    c = np.zeros(max(nnz, 1), np.int32)
    v = np.zeros(max(nnz, 1), np.float64)
    lib().orc_triplet_poisson(m, n, r, c, v)
    return r[:nnz].copy(), c[:nnz].copy(), v[:nnz].copy()


def triplet_to_crs(nor, noc, rows, cols, vals):
    """Returns CRSArrays; rows/cols/vals (numpy arrays) are sorted in place."""
    nnz = rows.size
    rs = np.zeros(nor + 1, np.int32)
    ci = np.zeros(max(nnz, 1), np.int32)
    d = np.zeros(max(nnz, 1), np.float64)
    if nnz:
        lib().orc_triplet_to_crs(nnz, nor, rows, cols, vals, rs, ci, d)
    return CRSArrays(nor, noc, rs, ci[:nnz], d[:nnz])


def row_blocks(nor, parts):
    """(first_rows, thread_rows) of the reference's 1D row split."""
    f = np.zeros(parts, np.int32)
    t = np.zeros(parts, np.int32)
    lib().orc_row_blocks(int(nor), int(parts), f, t)
    return f, t


def triplet_to_multi_crs(nor, noc, rows, cols, vals, parts):
    """TripletToMultipleCRS: list of CRSArrays (local rows, global columns),
    one per row block, and the blocks' first rows; the triplet arrays are
    sorted in place."""
    nnz = rows.size
    f = np.zeros(parts, np.int32)
    t = np.zeros(parts, np.int32)
    rs = np.zeros(nor + parts, np.int32)
    ci = np.zeros(max(nnz, 1), np.int32)
    d = np.zeros(max(nnz, 1), np.float64)
    lib().orc_triplet_to_multi_crs(nnz, nor, parts, _nz(rows, np.int32), _nz(cols, np.int32), _nz(vals), f, t, rs,
                                   ci, d)
    out, base, k0 = [], 0, 0
    for p in range(parts):
        r = rs[base:base + t[p] + 1].copy()
        n = int(r[-1])
        out.append(CRSArrays(t[p], noc, r, ci[k0:k0 + n].copy(), d[k0:k0 + n].copy()))
        base += t[p] + 1
        k0 += n
    return out, f


def fill_poisson_rows(m, n, first_row, last_row):
    """Rows [first_row, last_row) of the m x n Poisson matrix (local row
    starts, global columns): CRSArrays."""
    rows = last_row - first_row
    rs = np.zeros(rows + 1, np.int32)
    ci = np.zeros(max(5 * rows, 1), np.int32)
    d = np.zeros(max(5 * rows, 1), np.float64)
    lib().orc_fill_poisson_rows(m, n, first_row, last_row, rs, ci, d)
    k = int(rs[-1])
    return CRSArrays(rows, m * n, rs, ci[:k], d[:k])


def power_rows(blocks, x, it):
    """MPI_driver_poisson.cpp's row-sharded power method over the blocks (a
    list of CRSArrays in rank order, as triplet_to_multi_crs returns them):
    the normalised full iterate after `it` iterations."""
    nor = sum(b.nor for b in blocks)
    rs = np.concatenate([b.row_start for b in blocks]).astype(np.int32)
    ci = np.concatenate([b.col_ind for b in blocks] + [np.zeros(1, np.int32)]).astype(np.int32)
    d = np.concatenate([b.data for b in blocks] + [np.zeros(1)])
    x = np.array(x, dtype=np.float64, copy=True)
    lib().orc_power_rows(nor, len(blocks), rs, ci, d, x, int(it))
    return x


def crs_mv(A, x):
    y = np.zeros(A.nor, np.float64)
    lib().orc_crs_mv(A.nor, A.row_start, _nz(A.col_ind, np.int32), _nz(A.data), np.ascontiguousarray(x, np.float64), y)
    return y


def crs_omp_mv(A, x, threads):
    y = np.zeros(A.nor, np.float64)
    lib().orc_crs_omp_mv(A.nor, A.row_start, _nz(A.col_ind, np.int32), _nz(A.data),
                         np.ascontiguousarray(x, np.float64), y, threads)
    return y


def merge_search(A, diagonal):
    a, b = C.c_int32(), C.c_int32()
    lib().orc_merge_search(diagonal, A.nor, A.nnz, np.ascontiguousarray(A.row_start[1:]), C.byref(a), C.byref(b))
    return a.value, b.value


def merge_partition(A, parts):
    out = np.zeros(2 * (parts + 1), np.int32)
    lib().orc_merge_partition(A.nor, A.nnz, A.row_start, parts, out)
    return out.reshape(parts + 1, 2)


def merge_mv(A, x, threads):
    y = np.zeros(A.nor, np.float64)
    lib().orc_merge_mv(A.nor, A.nnz, A.row_start, _nz(A.col_ind, np.int32), _nz(A.data),
                       np.ascontiguousarray(x, np.float64), y, threads)
    return y


def merge_omp_mv(A, x, threads):
    """CRS_Merge::mv with one partition per OpenMP thread (timing path)."""
    y = np.zeros(A.nor, np.float64)
    lib().orc_merge_omp_mv(A.nor, A.nnz, A.row_start, _nz(A.col_ind, np.int32), _nz(A.data),
                           np.ascontiguousarray(x, np.float64), y, threads)
    return y


def norm2(x):
    return float(lib().orc_norm2(np.ascontiguousarray(x, np.float64), x.size))


def power(A, x, it, kind=0, threads=1):
    """Reference powerIteration: returns (x, y) after `it` iterations; the
    result is x when `it` is even and y when it is odd."""
    x = np.array(x, dtype=np.float64, copy=True)
    y = np.zeros(A.nor, np.float64)
    lib().orc_power(kind, A.nor, A.nnz, A.row_start, _nz(A.col_ind, np.int32), _nz(A.data), x, y, it, threads)
    return x, y


def power_result(A, x, it, kind=0, threads=1):
    xo, yo = power(A, x, it, kind, threads)
    return xo if it % 2 == 0 else yo


def rayleigh(A, u):
    """(lambda, relative eigen-residual) of u: lambda = u.(Au)/u.u with Au
    from CRS::mv, residual = ||Au - lambda u|| / (|lambda| ||u||)."""
    u = np.ascontiguousarray(u, np.float64)
    lam, res = C.c_double(), C.c_double()
    lib().orc_rayleigh(A.nor, A.row_start, _nz(A.col_ind, np.int32), _nz(A.data), u, C.byref(lam), C.byref(res))
    return lam.value, res.value


def random_table(kind, mean, sigma, max_len):
    thr = np.zeros(max_len + 1, np.uint64)
    lib().orc_random_table(kind, mean, sigma, max_len, thr.ctypes.data)
    return thr


def random_crs(n, seed, kind=0, mean=16.0, sigma=1.2, max_len=20000, band_permille=300, band_half=4096):
    """The seeded random matrix of the library's device generator
    (pwmgpu_generate_random), restated on the host: CRSArrays."""
    L = lib()
    nnz = L.orc_random_crs(n, seed, kind, mean, sigma, max_len, band_permille, band_half, None, None, None)
    rs = np.zeros(n + 1, np.int32)
    ci = np.zeros(max(nnz, 1), np.int32)
    d = np.zeros(max(nnz, 1), np.float64)
    L.orc_random_crs(n, seed, kind, mean, sigma, max_len, band_permille, band_half, rs.ctypes.data, ci.ctypes.data,
                     d.ctypes.data)
    return CRSArrays(n, n, rs, ci[:nnz], d[:nnz])


def uniform_vector(n, seed):
    """The service's seeded start vector (x0_seed): uniform in [0, 1)."""
    x = np.zeros(n, np.float64)
    lib().orc_uniform_vector(n, seed & (2 ** 64 - 1), x.ctypes.data)
    return x


def csb_params(nor, noc):
    b, bits = C.c_int32(), C.c_int32()
    lib().orc_csb_params(nor, noc, C.byref(b), C.byref(bits))
    return b.value, bits.value


def csb_build(nor, noc, rows, cols, vals):
    """Returns dict(ind, data, blk_ptr, beta, block_bits, hb, vb, balanced)."""
    beta, bits = csb_params(nor, noc)
    hb = -(-noc // beta)
    vb = -(-nor // beta)
    nnz = rows.size
    ind = np.zeros(max(nnz, 1), np.uint32)
    data = np.zeros(max(nnz, 1), np.float64)
    blk = np.zeros(hb * vb + 1, np.int32)
    bal = lib().orc_csb_build(nor, noc, nnz, rows, cols, vals, ind, data, blk)
    return dict(ind=ind[:nnz], data=data[:nnz], blk_ptr=blk, beta=beta, block_bits=bits, hb=hb, vb=vb,
                balanced=int(bal))


def csb_mv(nor, noc, csb, x):
    y = np.zeros(nor, np.float64)
    lib().orc_csb_mv(nor, noc, _nz(csb["ind"], np.uint32), _nz(csb["data"]), csb["blk_ptr"],
                     np.ascontiguousarray(x, np.float64), y)
    return y


def hilbert(size, row, col):
    return int(lib().orc_hilbert(size, row, col))


def coh_build(nor, noc, rows, cols, vals, threads):
    """Flat CO-H description (see orc_coh_build)."""
    nnz = rows.size
    trj, tb = C.c_int64(), C.c_int64()
    T = lib().orc_coh_sizes(nor, noc, nnz, rows, cols, threads, C.byref(trj), C.byref(tb))
    cap = max(nnz, 1)
    part = np.zeros(9 * T, np.int32)
    rj = np.zeros(cap, np.uint16)
    cj = np.zeros(cap, np.uint16)
    d = np.zeros(cap, np.float64)
    bn = np.zeros(cap, np.int32)
    rjb = np.zeros(cap, np.int16)
    cjb = np.zeros(cap, np.int16)
    T2 = lib().orc_coh_build(nor, noc, nnz, rows, cols, vals, threads, part, rj, cj, d, bn, rjb, cjb)
    assert T2 == T
    info = part.reshape(T, 9)
    nrj = int(info[:, 7].sum())
    nblk = int(info[:, 6].sum())
    nrjb = int(info[:, 8].sum())
    return dict(threads=T, part_info=part, row_jump=rj[:max(nrj, 1)].copy(), col_jump=cj[:max(nnz, 1)].copy(),
                data=d[:max(nnz, 1)].copy(), block_nnz=bn[:max(nblk, 1)].copy(),
                row_jump_block=rjb[:max(nrjb, 1)].copy(), col_jump_block=cjb[:max(nblk, 1)].copy())


def coh_mv(nor, coh, x):
    y = np.zeros(nor, np.float64)
    lib().orc_coh_mv(nor, coh["threads"], coh["part_info"], coh["row_jump"], coh["col_jump"], coh["data"],
                     coh["block_nnz"], coh["row_jump_block"], coh["col_jump_block"],
                     np.ascontiguousarray(x, np.float64), y)
    return y


def load_mm(path, has_data, symmetric):
    nor, noc = C.c_int32(), C.c_int32()
    cap = lib().orc_load_mm(path.encode(), int(has_data), int(symmetric), C.byref(nor), C.byref(noc),
                            None, None, None, 0)
    if cap < 0:
        raise IOError(path)
    r = np.zeros(max(cap, 1), np.int32)
    c = np.zeros(max(cap, 1), np.int32)
    v = np.zeros(max(cap, 1), np.float64)
    n = lib().orc_load_mm(path.encode(), int(has_data), int(symmetric), C.byref(nor), C.byref(noc),
                          r.ctypes.data, c.ctypes.data, v.ctypes.data, cap)
    if n < 0:
        raise IOError(path)
    return nor.value, noc.value, r[:n].copy(), c[:n].copy(), v[:n].copy()


def load_bin(path, mat_size, symmetric):
    cap = lib().orc_load_bin(path.encode(), mat_size, int(symmetric), None, None, None, 0)
    if cap < 0:
        raise IOError(path)
    r = np.zeros(max(cap, 1), np.int32)
    c = np.zeros(max(cap, 1), np.int32)
    v = np.zeros(max(cap, 1), np.float64)
    n = lib().orc_load_bin(path.encode(), mat_size, int(symmetric), r.ctypes.data, c.ctypes.data,
                           v.ctypes.data, cap)
    return mat_size, mat_size, r[:n].copy(), c[:n].copy(), v[:n].copy()


def _nz(a, dtype=np.float64):
    """ctypes needs a non-empty buffer even when nnz == 0."""
    a = np.ascontiguousarray(a, dtype=dtype)
    return a if a.size else np.zeros(1, dtype)


def row_error_bound(A, x, u=2.0 ** -53):
    """Per-row bound 2*nnz_row*u*sum|a_ij*x_j| used by the parity tests."""
    rl = np.diff(A.row_start).astype(np.float64)
    absx = np.abs(np.asarray(x, np.float64))
    prod = np.abs(A.data) * absx[A.col_ind]
    rows = np.repeat(np.arange(A.nor), np.diff(A.row_start))
    s = np.bincount(rows, weights=prod, minlength=A.nor)
    return 2.0 * rl * u * s


STAT_KEYS = ("size", "nnz", "rows_avg", "rows_var", "block_avg", "block_var", "balanced", "block_bits",
             "nb_blocks")


def calc_stats(nor, rows, cols):
    """Util_Scripts/calc_stats.cpp:45-98 on a square triplet: dict of STAT_KEYS."""
    r = np.ascontiguousarray(rows, np.int32)
    c = np.ascontiguousarray(cols, np.int32)
    out = np.zeros(9)
    rc = lib().orc_calc_stats(r.size, nor, r.ctypes.data if r.size else None, c.ctypes.data if c.size else None,
                              out)
    if rc != 0:
        raise ValueError("calc_stats: column block out of range or allocation failed")
    d = dict(zip(STAT_KEYS, out.tolist()))
    for k in ("size", "nnz", "balanced", "block_bits", "nb_blocks"):
        d[k] = int(d[k])
    return d
