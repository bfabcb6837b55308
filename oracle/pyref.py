"""ctypes front end of oracle/_ref/libpwmref.so: the UNMODIFIED reference
classes compiled from the reference tree (development container only).

Used to pin the C oracle (tests/test_oracle_vs_ref.py) and to generate the
golden fixtures (tests/golden/make_golden.py).  ``available()`` is False on a
machine without the reference tree; callers skip then.
"""
import ctypes as C
import os

import numpy as np

from .build import build_ref, REF_LIB

_lib = None

I32P = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
F64P = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")

METHOD_CRS, METHOD_CRSOMP, METHOD_MERGE, METHOD_CSB, METHOD_COH = 1, 2, 8, 9, 10


def available():
    try:
        return lib() is not None
    except Exception:
        return False


def lib():
    global _lib
    if _lib is None:
        path = build_ref()
        if path is None or not os.path.exists(path):
            return None
        try:
            L = C.CDLL(path)
        except OSError:
            return None
        vp = C.c_void_p
        L.ref_triplet_new.restype = vp
        L.ref_triplet_delete.argtypes = [vp]
        L.ref_triplet_load_mm.argtypes = [vp, C.c_char_p, C.c_int, C.c_int, C.c_int]
        L.ref_triplet_load_bin.argtypes = [vp, C.c_char_p, C.c_int, C.c_int, C.c_int]
        L.ref_triplet_poisson.argtypes = [vp, C.c_int, C.c_int]
        L.ref_triplet_set.argtypes = [vp, C.c_int, C.c_int, C.c_int, I32P, I32P, F64P]
        L.ref_triplet_info.restype = C.c_int
        L.ref_triplet_info.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.ref_triplet_get.argtypes = [vp, I32P, I32P, F64P]
        L.ref_matrix_new.restype = vp
        L.ref_matrix_new.argtypes = [C.c_int, C.c_int]
        L.ref_matrix_delete.argtypes = [vp]
        L.ref_generate_poisson.argtypes = [vp, C.c_int, C.c_int, C.c_int]
        L.ref_load_triplets.argtypes = [vp, vp, C.c_int]
        L.ref_mv.argtypes = [vp, F64P, F64P]
        L.ref_power.argtypes = [vp, F64P, F64P, C.c_int]
        L.ref_dims.restype = C.c_int
        L.ref_dims.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.ref_crs_get.argtypes = [vp, C.c_int, I32P, I32P, F64P]
        L.ref_merge_search.argtypes = [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.ref_csb_info.argtypes = [vp] + [C.POINTER(C.c_int)] * 5
        L.ref_csb_get.argtypes = [vp, np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS"), F64P, I32P]
        L.ref_coh_threads.restype = C.c_int
        L.ref_coh_threads.argtypes = [vp]
        L.ref_coh_thread_info.argtypes = [vp, C.c_int] + [C.POINTER(C.c_int)] * 9
        L.ref_coh_thread_get.argtypes = [vp, C.c_int, np.ctypeslib.ndpointer(np.uint16, flags="C_CONTIGUOUS"),
                                         C.c_int, np.ctypeslib.ndpointer(np.uint16, flags="C_CONTIGUOUS"), F64P,
                                         I32P, np.ctypeslib.ndpointer(np.int16, flags="C_CONTIGUOUS"), C.c_int,
                                         np.ctypeslib.ndpointer(np.int16, flags="C_CONTIGUOUS")]
        L.ref_hilbert.restype = C.c_int
        L.ref_hilbert.argtypes = [C.c_int, C.c_int, C.c_int]
        L.ref_set_threads.argtypes = [C.c_int]
        L.ref_multi_crs.argtypes = [C.c_int, C.c_int, C.c_int, I32P, I32P, F64P, I32P, I32P, I32P, I32P, F64P]
        L.ref_fill_poisson_rows.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, I32P, I32P, F64P]
        L.ref_max_threads.restype = C.c_int
        L.ref_srand.argtypes = [C.c_uint]
        _lib = L
    return _lib


class Triplet:
    """pwm::Triplet<double,int> (Matrix/Triplet.hpp)."""

    def __init__(self):
        self.h = lib().ref_triplet_new()

    def __del__(self):
        try:
            lib().ref_triplet_delete(self.h)
        except Exception:
            pass

    def load_mm(self, path, has_data, symmetric, random_fill=False):
        lib().ref_triplet_load_mm(self.h, path.encode(), int(has_data), int(symmetric), int(random_fill))
        return self

    def load_bin(self, path, size, symmetric, random_vals=False):
        lib().ref_triplet_load_bin(self.h, path.encode(), size, int(symmetric), int(random_vals))
        return self

    def poisson(self, m, n):
        lib().ref_triplet_poisson(self.h, m, n)
        return self

    def set(self, nor, noc, r, c, v):
        lib().ref_triplet_set(self.h, nor, noc, r.size, np.ascontiguousarray(r, np.int32),
                              np.ascontiguousarray(c, np.int32), np.ascontiguousarray(v, np.float64))
        return self

    def get(self):
        nor, noc = C.c_int(), C.c_int()
        nnz = lib().ref_triplet_info(self.h, C.byref(nor), C.byref(noc))
        r = np.zeros(max(nnz, 1), np.int32)
        c = np.zeros(max(nnz, 1), np.int32)
        v = np.zeros(max(nnz, 1), np.float64)
        lib().ref_triplet_get(self.h, r, c, v)
        return nor.value, noc.value, r[:nnz].copy(), c[:nnz].copy(), v[:nnz].copy()


class Matrix:
    """A reference SparseMatrix subclass chosen by method number."""

    def __init__(self, method, threads=1):
        self.method = method
        self.h = lib().ref_matrix_new(method, threads)
        assert self.h

    def __del__(self):
        try:
            lib().ref_matrix_delete(self.h)
        except Exception:
            pass

    def generate_poisson(self, m, n, partitions=1):
        lib().ref_generate_poisson(self.h, m, n, partitions)
        return self

    def load(self, trip, partitions=1):
        lib().ref_load_triplets(self.h, trip.h, partitions)
        return self

    def dims(self):
        nor, noc = C.c_int(), C.c_int()
        nnz = lib().ref_dims(self.h, C.byref(nor), C.byref(noc))
        return nor.value, noc.value, nnz

    def mv(self, x):
        nor, _, _ = self.dims()
        y = np.zeros(nor, np.float64)
        lib().ref_mv(self.h, np.ascontiguousarray(x, np.float64), y)
        return y

    def power(self, x, it):
        x = np.array(x, np.float64, copy=True)
        y = np.zeros_like(x)
        lib().ref_power(self.h, x, y, it)
        return x, y

    def crs(self):
        nor, noc, nnz = self.dims()
        rs = np.zeros(nor + 1, np.int32)
        ci = np.zeros(max(nnz, 1), np.int32)
        d = np.zeros(max(nnz, 1), np.float64)
        lib().ref_crs_get(self.h, self.method, rs, ci, d)
        return rs, ci[:nnz], d[:nnz]

    def merge_search(self, diagonal):
        a, b = C.c_int(), C.c_int()
        lib().ref_merge_search(self.h, diagonal, C.byref(a), C.byref(b))
        return a.value, b.value

    def csb(self):
        vals = [C.c_int() for _ in range(5)]
        lib().ref_csb_info(self.h, *[C.byref(v) for v in vals])
        beta, bits, hb, vb, bal = [v.value for v in vals]
        nor, noc, nnz = self.dims()
        ind = np.zeros(max(nnz, 1), np.uint32)
        d = np.zeros(max(nnz, 1), np.float64)
        blk = np.zeros(hb * vb + 1, np.int32)
        lib().ref_csb_get(self.h, ind, d, blk)
        return dict(ind=ind[:nnz], data=d[:nnz], blk_ptr=blk, beta=beta, block_bits=bits, hb=hb, vb=vb,
                    balanced=bal)

    def coh(self):
        T = lib().ref_coh_threads(self.h)
        parts = []
        for p in range(T):
            vals = [C.c_int() for _ in range(9)]
            lib().ref_coh_thread_info(self.h, p, *[C.byref(v) for v in vals])
            rs, beta, bits, hb, vb, tn, tb, nrj, nrjb = [v.value for v in vals]
            rj = np.zeros(max(nrj, 1), np.uint16)
            cj = np.zeros(max(tn, 1), np.uint16)
            d = np.zeros(max(tn, 1), np.float64)
            bn = np.zeros(max(tb, 1), np.int32)
            rjb = np.zeros(max(nrjb, 1), np.int16)
            cjb = np.zeros(max(tb, 1), np.int16)
            lib().ref_coh_thread_get(self.h, p, rj, nrj, cj, d, bn, rjb, nrjb, cjb)
            parts.append(dict(row_start=rs, beta=beta, block_bits=bits, hb=hb, vb=vb, nnz=tn, blocks=tb,
                              row_jump=rj[:nrj], col_jump=cj[:tn], data=d[:tn], block_nnz=bn[:tb],
                              row_jump_block=rjb[:nrjb], col_jump_block=cjb[:tb]))
        return parts


def hilbert(size, row, col):
    return int(lib().ref_hilbert(size, row, col))


def calc_stats(nor, noc, rows, cols, vals):
    """Run the reference's calc_stats (oracle/_ref/calc_stats) on a triplet;
    returns the printed figures (17 significant digits) as a dict with the
    keys of pyoracle.STAT_KEYS (without block_bits / nb_blocks)."""
    import subprocess
    import tempfile
    from .build import REF_STATS
    if lib() is None or not os.path.exists(REF_STATS):
        raise RuntimeError("reference calc_stats not built")
    r = np.ascontiguousarray(rows, np.int32)
    c = np.ascontiguousarray(cols, np.int32)
    v = np.ascontiguousarray(vals, np.float64)
    tmpdir = os.path.join(os.path.dirname(REF_STATS), "tmp")
    os.makedirs(tmpdir, exist_ok=True)
    with tempfile.NamedTemporaryFile(dir=tmpdir, suffix=".trip", delete=False) as f:
        np.array([nor, noc, r.size], np.int32).tofile(f)
        r.tofile(f)
        c.tofile(f)
        v.tofile(f)
        path = f.name
    try:
        out = subprocess.run([REF_STATS, path], capture_output=True, text=True, check=True).stdout
    finally:
        os.remove(path)
    keys = {"Size:": "size", "Nonzeros:": "nnz", "Average nnz per row:": "rows_avg",
            "Variance of nnz per row:": "rows_var", "Average nnz per block:": "block_avg",
            "Variance of nnz per block:": "block_var"}
    d = {}
    for line in out.splitlines():
        for label, key in keys.items():
            if line.startswith(label):
                d[key] = float(line[len(label):])
        if "balanced for CSB" in line:
            d["balanced"] = 0 if "unbalanced" in line else 1
    d["size"], d["nnz"] = int(d["size"]), int(d["nnz"])
    return d


def multi_crs(nor, rows, cols, vals, parts):
    """The reference's TripletToMultipleCRS on copies of the triplet arrays:
    (first_rows, thread_rows, concatenated row starts, columns, values)."""
    L = lib()
    r = np.ascontiguousarray(rows, np.int32).copy()
    c = np.ascontiguousarray(cols, np.int32).copy()
    v = np.ascontiguousarray(vals, np.float64).copy()
    f = np.zeros(parts, np.int32)
    t = np.zeros(parts, np.int32)
    rs = np.zeros(nor + parts, np.int32)
    ci = np.zeros(max(r.size, 1), np.int32)
    d = np.zeros(max(r.size, 1), np.float64)
    L.ref_multi_crs(nor, r.size, parts, r, c, v, f, t, rs, ci, d)
    return f, t, rs, ci[:r.size], d[:r.size]


def fill_poisson_rows(m, n, first_row, last_row):
    """The reference's fillPoisson over rows [first_row, last_row)."""
    L = lib()
    rows = last_row - first_row
    rs = np.zeros(rows + 1, np.int32)
    ci = np.zeros(max(5 * rows, 1), np.int32)
    d = np.zeros(max(5 * rows, 1), np.float64)
    L.ref_fill_poisson_rows(m, n, first_row, last_row, rs, ci, d)
    return rs, ci[:rs[-1]], d[:rs[-1]]
