"""Python mirror of the reference's operator interface, backed by libpwmgpu.so.

``Triplet`` mirrors pwm::Triplet<T,int_type> (Matrix/Triplet.hpp:26-279) and
``CRSCuda`` / ``CSBCuda`` / ``COHCuda`` mirror a pwm::SparseMatrix<T,int_type>
subclass (Matrix/SparseMatrix.hpp:13-68): same method names, argument meaning
and in-place behaviour (loadFromTriplets sorts the triplet; mv fills y;
powerIteration leaves the result in x for an even and in y for an odd
iteration count).  Every compute call goes through the C ABI; a failing call
raises PwmGpuError.
"""
import ctypes as C
import os

import numpy as np

from . import _lib
from ._lib import (FMT_AUTO, FMT_COH, FMT_CSB, FMT_MERGE, LOWFMT_AUTO, LOWFMT_MERGE, POWER_AUTO, POWER_FUSED, POWER_MULTI, PREC_F32,  # noqa: F401
                   PREC_F64, PREC_MIXED, SolveInfo, check)

_I32 = np.int32
_F64 = np.float64


def _ptr(a):
    return a.ctypes.data if a is not None and a.size else None


class Triplet:
    """COO matrix: row_coord, col_coord, data, row_size, col_size, nnz."""

    def __init__(self, row_size=0, col_size=0, rows=None, cols=None, vals=None):
        self.row_size = int(row_size)
        self.col_size = int(col_size)
        self.row_coord = np.ascontiguousarray(rows if rows is not None else np.zeros(0), dtype=_I32)
        self.col_coord = np.ascontiguousarray(cols if cols is not None else np.zeros(0), dtype=_I32)
        self.data = np.ascontiguousarray(vals if vals is not None else np.zeros(0), dtype=_F64)

    @property
    def nnz(self):
        return int(self.row_coord.size)

    def generatePoisson(self, m, n):
        """Matrix/Triplet.hpp:226-278: diagonal, super/sub, then the two far diagonals per row."""
        m, n = int(m), int(n)
        size = m * n
        i = np.arange(size, dtype=np.int64)
        parts_r, parts_c, parts_v = [i], [i], [np.full(size, 4.0)]
        sup = (i < size - 1) & (i % m != m - 1)
        sub = (i < size - 1) & ((i + 1) % m != 0)
        far = i < size - m
        # interleave in the reference's per-row emission order
        order_r, order_c, order_v, key = [], [], [], []
        slots = [(i, i, 4.0, np.ones(size, bool)), (i, i + 1, -1.0, sup), (i + 1, i, -1.0, sub),
                 (i + m, i, -1.0, far), (i, i + m, -1.0, far)]
        for s, (r, c, v, mask) in enumerate(slots):
            idx = np.nonzero(mask)[0]
            order_r.append(r[idx])
            order_c.append(c[idx])
            order_v.append(np.full(idx.size, v))
            key.append(idx * 5 + s)
        k = np.concatenate(key)
        p = np.argsort(k, kind="stable")
        self.row_size = self.col_size = size
        self.row_coord = np.concatenate(order_r)[p].astype(_I32)
        self.col_coord = np.concatenate(order_c)[p].astype(_I32)
        self.data = np.concatenate(order_v)[p].astype(_F64)
        return self

    def loadFromMM(self, filename, has_data, symmetric, random_fill=False):
        """Matrix/Triplet.hpp:75-154 (random_fill is not supported)."""
        if random_fill:
            raise NotImplementedError("random_fill needs Boost's uniform_real_distribution stream")
        rows, cols, vals = [], [], []
        with open(filename) as f:
            for line in f:
                if not line.startswith("%"):
                    hdr = line.split()
                    self.row_size, self.col_size = int(hdr[0]), int(hdr[1])
                    break
            for line in f:
                t = line.split()
                if not t:
                    break
                r, c = int(t[0]) - 1, int(t[1]) - 1
                v = float(t[2]) if has_data else 1.0
                if has_data and v == 0.0:
                    continue
                rows.append(r); cols.append(c); vals.append(v)
                if symmetric and r != c:
                    rows.append(c); cols.append(r); vals.append(v)
        self.row_coord = np.array(rows, _I32)
        self.col_coord = np.array(cols, _I32)
        self.data = np.array(vals, _F64)
        return self

    def loadFromBin(self, filename, mat_size, symmetric, random_vals=False):
        """Matrix/Triplet.hpp:164-216: uint32 (row, col) pairs, value 1."""
        if random_vals:
            raise NotImplementedError("random_vals needs Boost's uniform_real_distribution stream")
        rc = np.fromfile(filename, dtype=np.uint32).reshape(-1, 2).astype(np.int64)
        r, c = rc[:, 0], rc[:, 1]
        if symmetric:
            off = r != c
            # entry, then its transpose right after it when off-diagonal
            idx = np.repeat(np.arange(r.size), np.where(off, 2, 1))
            first = np.concatenate([[True], idx[1:] != idx[:-1]])
            rr = np.where(first, r[idx], c[idx])
            cc = np.where(first, c[idx], r[idx])
            r, c = rr, cc
        self.row_size = self.col_size = int(mat_size)
        self.row_coord = r.astype(_I32)
        self.col_coord = c.astype(_I32)
        self.data = np.ones(r.size, _F64)
        return self


class CudaSparseMatrix:
    """A pwm::SparseMatrix on the GPU; `format` selects the storage."""

    FORMAT = FMT_MERGE

    def __init__(self, threads=1):
        self._h = C.c_void_p()
        check(_lib.lib().pwmgpu_create(self.FORMAT, int(threads) if threads else 1, C.byref(self._h)),
              "pwmgpu_create")
        self.threads = threads

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.lib().pwmgpu_destroy(h)
            except Exception:
                pass
            self._h = C.c_void_p()

    @property
    def handle(self):
        return self._h

    # ---- SparseMatrix.hpp:41 ----
    def generatePoissonMatrix(self, m, n, partitions=1):
        check(_lib.lib().pwmgpu_generate_poisson(self._h, int(m), int(n)), "generatePoissonMatrix")

    def generateRandom(self, n, seed, length_dist=0, mean_len=16.0, sigma=1.2, max_len=20000, band_permille=300,
                       band_half=4096):
        """Seeded random n x n matrix generated on the device (lognormal
        (length_dist 0) or Poisson (1) row lengths, band_permille / 1000 of
        the columns within +-band_half of the diagonal, values in (0, 1])."""
        check(_lib.lib().pwmgpu_generate_random(self._h, int(n), int(seed) & (2 ** 64 - 1), int(length_dist),
                                                float(mean_len), float(sigma), int(max_len), int(band_permille),
                                                int(band_half)), "generateRandom")

    # ---- SparseMatrix.hpp:48 ----
    def loadFromTriplets(self, triplet, partitions_am=1):
        for name in ("row_coord", "col_coord", "data"):
            a = getattr(triplet, name)
            want = _F64 if name == "data" else _I32
            if not (isinstance(a, np.ndarray) and a.dtype == want and a.flags.c_contiguous):
                setattr(triplet, name, np.ascontiguousarray(a, dtype=want))
        check(_lib.lib().pwmgpu_load_triplets(self._h, triplet.row_size, triplet.col_size, triplet.nnz,
                                              _ptr(triplet.row_coord), _ptr(triplet.col_coord),
                                              _ptr(triplet.data)), "loadFromTriplets")

    def loadFromDeviceTriplets(self, nor, noc, nnz, rows_ptr, cols_ptr, vals_ptr):
        """CRS from triplet arrays already on the device (int32 rows / cols,
        float64 values, e.g. torch tensors' data_ptr()); they stay unchanged."""
        check(_lib.lib().pwmgpu_load_triplets_device(self._h, int(nor), int(noc), int(nnz), rows_ptr, cols_ptr,
                                                     vals_ptr), "loadFromDeviceTriplets")

    def loadCSR(self, nor, noc, row_start, col_ind, data):
        rs = np.ascontiguousarray(row_start, _I32)
        ci = np.ascontiguousarray(col_ind, _I32)
        d = np.ascontiguousarray(data, _F64)
        check(_lib.lib().pwmgpu_load_csr(self._h, int(nor), int(noc), int(ci.size), _ptr(rs), _ptr(ci), _ptr(d)),
              "pwmgpu_load_csr")

    def dims(self):
        nor, noc, nnz = C.c_int32(), C.c_int32(), C.c_int64()
        check(_lib.lib().pwmgpu_dims(self._h, C.byref(nor), C.byref(noc), C.byref(nnz)), "pwmgpu_dims")
        return nor.value, noc.value, nnz.value

    def stats(self):
        """Util_Scripts/calc_stats.cpp figures of the loaded matrix, computed on
        the device: dict with size, nnz, rows_avg, rows_var, block_avg,
        block_var, balanced, block_bits, nb_blocks, max_row_nnz."""
        st = _lib.MatrixStats()
        check(_lib.lib().pwmgpu_stats(self._h, C.byref(st)), "pwmgpu_stats")
        return {name: getattr(st, name) for name, _ in st._fields_}

    def getCSR(self):
        """The device CRS arrays (row_start, col_ind, data) copied to the host."""
        nor, noc, nnz = self.dims()
        rs = np.zeros(nor + 1, _I32)
        ci = np.zeros(max(nnz, 1), _I32)
        d = np.zeros(max(nnz, 1), _F64)
        check(_lib.lib().pwmgpu_get_csr(self._h, _ptr(rs), _ptr(ci), _ptr(d)), "pwmgpu_get_csr")
        return rs, ci[:nnz], d[:nnz]

    # ---- SparseMatrix.hpp:57 ----
    def mv(self, x, y):
        """y = A x on host arrays (y filled in place)."""
        nor, noc, _ = self.dims()
        assert x.dtype == _F64 and y.dtype == _F64 and x.size >= noc and y.size >= nor
        assert x.flags.c_contiguous and y.flags.c_contiguous
        check(_lib.lib().pwmgpu_mv(self._h, _ptr(x), _ptr(y)), "mv")

    # ---- SparseMatrix.hpp:66 ----
    def powerIteration(self, x, y, it):
        nor, _, _ = self.dims()
        assert x.dtype == _F64 and y.dtype == _F64 and x.size >= nor and y.size >= nor
        check(_lib.lib().pwmgpu_power(self._h, _ptr(x), _ptr(y), int(it)), "powerIteration")

    # ---- device-resident and extended entry points ----
    def mv_device(self, dx_ptr, dy_ptr):
        check(_lib.lib().pwmgpu_mv_device(self._h, C.c_void_p(dx_ptr), C.c_void_p(dy_ptr)), "mv_device")

    def mv_device_f32(self, dx_ptr, dy_ptr):
        check(_lib.lib().pwmgpu_mv_device_f32(self._h, C.c_void_p(dx_ptr), C.c_void_p(dy_ptr)), "mv_device_f32")

    def power_device(self, dx_ptr, dy_ptr, it):
        check(_lib.lib().pwmgpu_power_device(self._h, C.c_void_p(dx_ptr), C.c_void_p(dy_ptr), int(it)),
              "power_device")

    def set_stream(self, stream_ptr):
        check(_lib.lib().pwmgpu_set_stream(self._h, C.c_void_p(stream_ptr)), "set_stream")

    def set_power_mode(self, mode):
        """POWER_AUTO / POWER_FUSED (one persistent kernel) / POWER_MULTI
        (two kernels per iteration)."""
        check(_lib.lib().pwmgpu_set_power_mode(self._h, int(mode)), "set_power_mode")

    def set_low_format(self, fmt):
        """LOWFMT_AUTO (SELL-32 for the FP32 / BF16 iterations where the
        matrix fits it) / LOWFMT_MERGE (always the merge-path layout)."""
        check(_lib.lib().pwmgpu_set_low_format(self._h, int(fmt)), "set_low_format")

    def solve(self, x, max_it, tol, precision=PREC_F64):
        """Power solve to ||A u - lambda u|| / |lambda| <= tol (or max_it
        SpMVs); x: start vector in, normalised eigenvector estimate out.
        Returns the SolveInfo (iterations, iterations_low, converged,
        precision, lambda_, residual)."""
        assert x.dtype == _F64 and x.flags.c_contiguous
        info = SolveInfo()
        check(_lib.lib().pwmgpu_solve(self._h, _ptr(x), int(max_it), float(tol), int(precision), C.byref(info)),
              "solve")
        return info

    def merge_partition(self, parts):
        out = np.zeros(2 * (parts + 1), _I32)
        check(_lib.lib().pwmgpu_merge_partition(self._h, int(parts), _ptr(out)), "merge_partition")
        return out.reshape(parts + 1, 2)

    def launch_config(self):
        """(prefer_l1, grid, power_grid, (ms variant 0, ms variant 1)) chosen
        by the load-time tuner."""
        a, b, c = C.c_int32(), C.c_int32(), C.c_int32()
        ms = (C.c_float * 2)()
        check(_lib.lib().pwmgpu_launch_config(self._h, C.byref(a), C.byref(b), C.byref(c), ms), "launch_config")
        return a.value, b.value, c.value, (ms[0], ms[1])

    def column_bytes(self):
        """2 when the merge kernels stream 16-bit column offsets, else 4."""
        return self.plan_info()[0]

    def plan_info(self):
        """(bytes per streamed column index, 1 if the x gathers bypass L1)."""
        b, g = C.c_int32(), C.c_int32()
        check(_lib.lib().pwmgpu_plan_info(self._h, C.byref(b), C.byref(g)), "pwmgpu_plan_info")
        return b.value, g.value

    def launch_variant(self):
        """The merge kernels' launch variant bits (pwmgpu_launch_variant)."""
        v = C.c_int32()
        check(_lib.lib().pwmgpu_launch_variant(self._h, C.byref(v)), "pwmgpu_launch_variant")
        return v.value

    def set_launch_variant(self, variant):
        """Override the load-time tuner: 0 / 1 (shared-memory carveout), 4 / 5
        (the same, x gathers around L1)."""
        check(_lib.lib().pwmgpu_set_launch_variant(self._h, int(variant)), "set_launch_variant")

    def tile_info(self):
        a, b, c = C.c_int32(), C.c_int32(), C.c_int32()
        check(_lib.lib().pwmgpu_tile_info(self._h, C.byref(a), C.byref(b), C.byref(c)), "tile_info")
        return a.value, b.value, c.value


    def set_csb_variant(self, variant):
        """CSB kernel variant (CSB handles): bit 0 = 8 elements per lane, bit 1 = 256 threads per CTA."""
        check(_lib.lib().pwmgpu_set_csb_variant(self._h, int(variant)), "pwmgpu_set_csb_variant")

    def csb_variant(self):
        """The CSB kernel variant in use (picked at load time on large matrices)."""
        v = C.c_int32()
        check(_lib.lib().pwmgpu_get_csb_variant(self._h, C.byref(v)), "pwmgpu_get_csb_variant")
        return v.value

    def getCSB(self):
        """The CSB arrays (CSB.hpp:464-567) of a CSBCuda handle: dict(ind,
        data, blk_ptr, beta, block_bits, hb, vb)."""
        L = _lib.lib()
        beta, bits, hb, vb, nnz = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32(), C.c_int64()
        check(L.pwmgpu_csb_info(self._h, C.byref(beta), C.byref(bits), C.byref(hb), C.byref(vb), C.byref(nnz)),
              "pwmgpu_csb_info")
        ind = np.zeros(max(nnz.value, 1), np.uint32)
        data = np.zeros(max(nnz.value, 1), _F64)
        blk = np.zeros(hb.value * vb.value + 1, _I32)
        check(L.pwmgpu_get_csb(self._h, _ptr(ind), _ptr(data), _ptr(blk)), "pwmgpu_get_csb")
        return dict(ind=ind[:nnz.value], data=data[:nnz.value], blk_ptr=blk, beta=beta.value,
                    block_bits=bits.value, hb=hb.value, vb=vb.value)

    def getCOH(self):
        """The CO-H arrays (BlockCOH.hpp:319-455) of a COHCuda handle."""
        L = _lib.lib()
        T, nrj, nblk, nrjb, nnz = C.c_int32(), C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        check(L.pwmgpu_coh_info(self._h, C.byref(T), C.byref(nrj), C.byref(nblk), C.byref(nrjb), C.byref(nnz)),
              "pwmgpu_coh_info")
        part = np.zeros(9 * T.value, _I32)
        rj = np.zeros(max(nrj.value, 1), np.uint16)
        cj = np.zeros(max(nnz.value, 1), np.uint16)
        d = np.zeros(max(nnz.value, 1), _F64)
        bn = np.zeros(max(nblk.value, 1), _I32)
        rjb = np.zeros(max(nrjb.value, 1), np.int16)
        cjb = np.zeros(max(nblk.value, 1), np.int16)
        check(L.pwmgpu_get_coh(self._h, _ptr(part), _ptr(rj), _ptr(cj), _ptr(d), _ptr(bn), _ptr(rjb), _ptr(cjb)),
              "pwmgpu_get_coh")
        return dict(threads=T.value, part_info=part, row_jump=rj[:nrj.value], col_jump=cj[:nnz.value],
                    data=d[:nnz.value], block_nnz=bn[:nblk.value], row_jump_block=rjb[:nrjb.value],
                    col_jump_block=cjb[:nblk.value])


class CRSCuda(CudaSparseMatrix):
    """Merge-path CRS on the GPU (drop-in beside CRS_Merge, method 12)."""
    FORMAT = FMT_MERGE


class CSBCuda(CudaSparseMatrix):
    """CSB on the GPU (drop-in beside CSB, method 13)."""
    FORMAT = FMT_CSB


class COHCuda(CudaSparseMatrix):
    """Block CO-H on the GPU (drop-in beside BlockCOH, method 14)."""
    FORMAT = FMT_COH


class AutoCuda(CudaSparseMatrix):
    """Format-autotuned GPU matrix (method 15, no counterpart in the
    reference): the merge-path plan plus whichever of merge, CSB or CO-H (and
    kernel variant) the class-keyed tuner found fastest for mv /
    powerIteration."""
    FORMAT = FMT_AUTO

    def tuning(self):
        """dict of pwmgpu_tuning_info: chosen format and variants, cache hit,
        class key and the timings (ms per SpMV) of every candidate."""
        t = _lib.Tuning()
        check(_lib.lib().pwmgpu_tuning_info(self._h, C.byref(t)), "pwmgpu_tuning_info")
        return dict(format={FMT_MERGE: "merge", FMT_CSB: "csb", FMT_COH: "coh"}[t.format],
                    csb_variant=t.csb_variant, merge_variant=t.merge_variant, cache_hit=bool(t.cache_hit),
                    timed=bool(t.timed), class_key=list(t.class_key), coh_partitions=t.coh_partitions,
                    merge_ms=t.merge_ms, csb_ms=list(t.csb_ms), coh_ms=list(t.coh_ms),
                    tune_seconds=t.tune_seconds)


def tuner_reset():
    """Forget the autotuner's recorded class choices."""
    check(_lib.lib().pwmgpu_tuner_reset(), "pwmgpu_tuner_reset")


def tuner_size():
    """Number of matrix classes the autotuner has recorded."""
    return int(_lib.lib().pwmgpu_tuner_size())


def tuner_record(key, fmt, csb_variant=0, merge_variant=0, coh_parts_per_sm=0):
    """Record a class choice (fmt "merge" / "csb" / "coh") in the autotuner's table."""
    k = (C.c_int32 * 7)(*[int(v) for v in key])
    f = {"merge": FMT_MERGE, "csb": FMT_CSB, "coh": FMT_COH}[fmt]
    check(_lib.lib().pwmgpu_tuner_record(k, f, int(csb_variant), int(merge_variant), int(coh_parts_per_sm)),
          "pwmgpu_tuner_record")


def tuner_entries():
    """The autotuner's table: list of (class key, format, csb_variant,
    merge_variant, coh_parts_per_sm)."""
    n = tuner_size()
    keys = (C.c_int32 * (7 * max(n, 1)))()
    ch = (C.c_int32 * (4 * max(n, 1)))()
    got = _lib.lib().pwmgpu_tuner_entries(n, keys, ch)
    if got < 0:
        check(-got, "pwmgpu_tuner_entries")
    names = {FMT_MERGE: "merge", FMT_CSB: "csb", FMT_COH: "coh"}
    return [(list(keys[7 * i:7 * i + 7]), names[ch[4 * i]], ch[4 * i + 1], ch[4 * i + 2], ch[4 * i + 3])
            for i in range(got)]


def class_key(stats, sm_count):
    """The autotuner's class key of a statistics dict (CudaSparseMatrix.stats())."""
    st = _lib.MatrixStats(**{k: stats[k] for k in (f[0] for f in _lib.MatrixStats._fields_)})
    key = (C.c_int32 * 7)()
    check(_lib.lib().pwmgpu_class_key(C.byref(st), int(sm_count), key), "pwmgpu_class_key")
    return list(key)


def selectType(method, threads=1):
    """Util/DriverUtil.hpp:38-84 selectType for the GPU method numbers
    (12 merge-path CRS, 13 CSB, 14 CO-H, 15 autotuned); None for any other
    number, like the reference's NULL."""
    return {12: CRSCuda, 13: CSBCuda, 14: COHCuda, 15: AutoCuda}.get(int(method), lambda t: None)(threads)
