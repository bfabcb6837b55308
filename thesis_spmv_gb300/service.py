"""Python binding of the batched power-method service (include/pwmsvc.h).

    svc = Service(hbm_budget_bytes=150 << 30, round_iterations=8)
    rid = svc.submit_poisson(512, 512, tol=1e-10, max_it=2000, precision=PREC_MIXED)
    svc.run_until_idle()
    res, u = svc.result(rid, want_vector=True)
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import PREC_F64, check

SRC_CSR, SRC_POISSON, SRC_RANDOM, SRC_TRIPLETS = 0, 1, 2, 3
QUEUED, RUNNING, DONE, FAILED = 0, 1, 2, 3


class Config(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_size_t), ("max_live", C.c_int32), ("round_iterations", C.c_int32),
                ("use_graph", C.c_int32)]


class Request(C.Structure):
    _fields_ = [("source", C.c_int32), ("nor", C.c_int32), ("nnz", C.c_int32), ("row_start", C.c_void_p),
                ("col_ind", C.c_void_p), ("vals", C.c_void_p), ("grid_m", C.c_int32), ("grid_n", C.c_int32),
                ("n", C.c_int32), ("seed", C.c_uint64), ("length_dist", C.c_int32), ("mean_len", C.c_double),
                ("sigma", C.c_double), ("max_len", C.c_int32), ("band_permille", C.c_int32),
                ("band_half", C.c_int32), ("x0", C.c_void_p), ("x0_seed", C.c_uint64), ("max_it", C.c_int32),
                ("tol", C.c_double), ("precision", C.c_int32), ("keep_vector", C.c_int32),
                ("row_ind", C.c_void_p)]


class Result(C.Structure):
    _fields_ = [("state", C.c_int32), ("n", C.c_int32), ("iterations", C.c_int32), ("iterations_low", C.c_int32),
                ("converged", C.c_int32), ("precision", C.c_int32), ("error", C.c_int32), ("pad", C.c_int32),
                ("lambda_", C.c_double), ("residual", C.c_double), ("t_submit", C.c_double),
                ("t_admit", C.c_double), ("t_done", C.c_double)]


class Stats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("finished", C.c_int64), ("failed", C.c_int64), ("rounds", C.c_int64),
                ("live", C.c_int32), ("queued", C.c_int32), ("hbm_in_use", C.c_size_t),
                ("hbm_budget", C.c_size_t), ("gpu_round_ms", C.c_double)]


vp = C.c_void_p
SIGNATURES = {
    "pwmsvc_create": (C.c_int, [C.POINTER(Config), C.POINTER(vp)]),
    "pwmsvc_destroy": (C.c_int, [vp]),
    "pwmsvc_submit": (C.c_int, [vp, C.POINTER(Request), C.POINTER(C.c_int64)]),
    "pwmsvc_step": (C.c_int, [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "pwmsvc_result": (C.c_int, [vp, C.c_int64, C.POINTER(Result), vp]),
    "pwmsvc_release": (C.c_int, [vp, C.c_int64]),
    "pwmsvc_stats": (C.c_int, [vp, C.POINTER(Stats)]),
}

_bound = False


def lib():
    global _bound
    L = _lib.lib()
    if not _bound:
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _bound = True
    return L


class Service:
    """The serving loop: submit solves, step rounds, read results."""

    def __init__(self, hbm_budget_bytes=0, max_live=1024, round_iterations=8, use_graph=True):
        self._h = C.c_void_p()
        cfg = Config(int(hbm_budget_bytes), int(max_live), int(round_iterations), 1 if use_graph else 0)
        check(lib().pwmsvc_create(C.byref(cfg), C.byref(self._h)), "pwmsvc_create")
        self._keep = {}

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().pwmsvc_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _submit(self, req, x0, keep):
        if x0 is not None:
            x0 = np.ascontiguousarray(x0, np.float64)
            req.x0 = x0.ctypes.data
        rid = C.c_int64()
        check(lib().pwmsvc_submit(self._h, C.byref(req), C.byref(rid)), "pwmsvc_submit")
        return rid.value

    @staticmethod
    def _common(req, max_it, tol, precision, x0_seed, keep_vector):
        req.max_it = int(max_it)
        req.tol = float(tol)
        req.precision = int(precision)
        req.x0_seed = int(x0_seed) & (2 ** 64 - 1)
        req.keep_vector = 1 if keep_vector else 0

    def submit_poisson(self, m, n, max_it=2000, tol=1e-10, precision=PREC_F64, x0=None, x0_seed=0,
                       keep_vector=False):
        req = Request()
        req.source = SRC_POISSON
        req.grid_m, req.grid_n = int(m), int(n)
        self._common(req, max_it, tol, precision, x0_seed, keep_vector)
        return self._submit(req, x0, keep_vector)

    def submit_random(self, n, seed, length_dist=0, mean_len=16.0, sigma=1.2, max_len=20000, band_permille=300,
                      band_half=4096, max_it=2000, tol=1e-10, precision=PREC_F64, x0=None, x0_seed=0,
                      keep_vector=False):
        req = Request()
        req.source = SRC_RANDOM
        req.n, req.seed, req.length_dist = int(n), int(seed) & (2 ** 64 - 1), int(length_dist)
        req.mean_len, req.sigma, req.max_len = float(mean_len), float(sigma), int(max_len)
        req.band_permille, req.band_half = int(band_permille), int(band_half)
        self._common(req, max_it, tol, precision, x0_seed, keep_vector)
        return self._submit(req, x0, keep_vector)

    def submit_csr(self, A, max_it=2000, tol=1e-10, precision=PREC_F64, x0=None, x0_seed=0, keep_vector=False):
        """A: any object with nor, row_start, col_ind, data (square)."""
        rs = np.ascontiguousarray(A.row_start, np.int32)
        ci = np.ascontiguousarray(A.col_ind, np.int32)
        d = np.ascontiguousarray(A.data, np.float64)
        req = Request()
        req.source = SRC_CSR
        req.nor, req.nnz = int(A.nor), int(ci.size)
        req.row_start, req.col_ind, req.vals = rs.ctypes.data, ci.ctypes.data, d.ctypes.data
        self._common(req, max_it, tol, precision, x0_seed, keep_vector)
        return self._submit(req, x0, keep_vector)

    def submit_triplets(self, n, rows, cols, vals, max_it=2000, tol=1e-10, precision=PREC_F64, x0=None, x0_seed=0,
                        keep_vector=False):
        """An n x n matrix as triplets (any entry order), sorted into CRS on the device at admission."""
        ri = np.ascontiguousarray(rows, np.int32)
        ci = np.ascontiguousarray(cols, np.int32)
        d = np.ascontiguousarray(vals, np.float64)
        if not (ri.size == ci.size == d.size):
            raise ValueError("rows, cols and vals differ in length")
        req = Request()
        req.source = SRC_TRIPLETS
        req.nor, req.nnz = int(n), int(ci.size)
        req.row_ind, req.col_ind, req.vals = ri.ctypes.data, ci.ctypes.data, d.ctypes.data
        self._common(req, max_it, tol, precision, x0_seed, keep_vector)
        return self._submit(req, x0, keep_vector)

    def step(self):
        """One round; returns (live, queued, finished_this_round)."""
        a, b, c = C.c_int32(), C.c_int32(), C.c_int32()
        check(lib().pwmsvc_step(self._h, C.byref(a), C.byref(b), C.byref(c)), "pwmsvc_step")
        return a.value, b.value, c.value

    def run_until_idle(self, max_rounds=10 ** 7):
        for _ in range(max_rounds):
            live, queued, _ = self.step()
            if live == 0 and queued == 0:
                return
        raise RuntimeError("service did not drain")

    def result(self, rid, want_vector=False):
        r = Result()
        check(lib().pwmsvc_result(self._h, int(rid), C.byref(r), None), "pwmsvc_result")
        if not want_vector:
            return r
        u = np.zeros(r.n, np.float64)
        check(lib().pwmsvc_result(self._h, int(rid), C.byref(r), u.ctypes.data), "pwmsvc_result")
        return r, u

    def release(self, rid):
        check(lib().pwmsvc_release(self._h, int(rid)), "pwmsvc_release")

    def stats(self):
        s = Stats()
        check(lib().pwmsvc_stats(self._h, C.byref(s)), "pwmsvc_stats")
        return s
