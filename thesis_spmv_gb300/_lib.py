"""ctypes binding of libpwmgpu.so (include/pwmgpu.h).

The library is the only compute path: if it is missing or fails to load,
every entry raises.  There is no CPU fallback.
"""
import ctypes as C
import os
import threading

from .build import LIB

_lock = threading.Lock()
_lib = None

PWMGPU_OK = 0
STATUS_NAMES = {0: "OK", 1: "ERR_INVALID", 2: "ERR_CUDA", 3: "ERR_NOMEM", 4: "ERR_TIMEOUT", 5: "ERR_STATE",
                6: "ERR_NOT_SQUARE", 7: "ERR_BUDGET", 8: "ERR_NUMERIC", 9: "ERR_UNSUPPORTED"}

FMT_MERGE, FMT_CSB, FMT_COH, FMT_AUTO = 0, 1, 2, 3
PREC_F64, PREC_F32, PREC_MIXED = 0, 1, 2
POWER_AUTO, POWER_FUSED, POWER_MULTI = 0, 1, 2
LOWFMT_AUTO, LOWFMT_MERGE = 0, 1
RAND_LOGNORMAL, RAND_POISSON = 0, 1


class PwmGpuError(RuntimeError):
    def __init__(self, code, where):
        self.code = code
        msg = "%s: %s (%s)" % (where, STATUS_NAMES.get(code, str(code)), last_error())
        super().__init__(msg)


class MatrixStats(C.Structure):
    _fields_ = [("size", C.c_int64), ("nnz", C.c_int64), ("rows_avg", C.c_double), ("rows_var", C.c_double),
                ("block_avg", C.c_double), ("block_var", C.c_double), ("balanced", C.c_int32),
                ("block_bits", C.c_int32), ("nb_blocks", C.c_int32), ("max_row_nnz", C.c_int32)]


class Tuning(C.Structure):
    """pwmgpu_tuning: what the format autotuner chose for a PWMGPU_FMT_AUTO handle."""
    _fields_ = [("format", C.c_int32), ("csb_variant", C.c_int32), ("merge_variant", C.c_int32),
                ("cache_hit", C.c_int32), ("timed", C.c_int32), ("class_key", C.c_int32 * 7),
                ("coh_partitions", C.c_int32), ("merge_ms", C.c_float), ("csb_ms", C.c_float * 4),
                ("coh_ms", C.c_float * 4),
                ("tune_seconds", C.c_double)]


class SolveInfo(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("iterations_low", C.c_int32), ("converged", C.c_int32),
                ("precision", C.c_int32), ("lambda_", C.c_double), ("residual", C.c_double)]


vp = C.c_void_p
i32 = C.c_int32
i64 = C.c_int64

# name -> (restype, argtypes); every symbol declared in include/pwmgpu.h
SIGNATURES = {
    "pwmgpu_last_error": (C.c_char_p, []),
    "pwmgpu_device_info": (C.c_int, [C.POINTER(C.c_int), C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
    "pwmgpu_create": (C.c_int, [C.c_int, C.c_int, C.POINTER(vp)]),
    "pwmgpu_destroy": (C.c_int, [vp]),
    "pwmgpu_set_stream": (C.c_int, [vp, vp]),
    "pwmgpu_generate_poisson": (C.c_int, [vp, i32, i32]),
    "pwmgpu_generate_random": (C.c_int, [vp, i32, C.c_uint64, C.c_int, C.c_double, C.c_double, i32, i32, i32]),
    "pwmgpu_load_csr": (C.c_int, [vp, i32, i32, i32, vp, vp, vp]),
    "pwmgpu_load_triplets": (C.c_int, [vp, i32, i32, i32, vp, vp, vp]),
    "pwmgpu_load_triplets_device": (C.c_int, [vp, i32, i32, i32, vp, vp, vp]),
    "pwmgpu_dims": (C.c_int, [vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i64)]),
    "pwmgpu_stats": (C.c_int, [vp, C.POINTER(MatrixStats)]),
    "pwmgpu_tuning_info": (C.c_int, [vp, C.POINTER(Tuning)]),
    "pwmgpu_class_key": (C.c_int, [C.POINTER(MatrixStats), i32, C.POINTER(i32)]),
    "pwmgpu_tuner_reset": (C.c_int, []),
    "pwmgpu_tuner_size": (C.c_int, []),
    "pwmgpu_tuner_record": (C.c_int, [C.POINTER(i32), i32, i32, i32, i32]),
    "pwmgpu_tuner_entries": (C.c_int, [i32, C.POINTER(i32), C.POINTER(i32)]),
    "pwmgpu_set_csb_variant": (C.c_int, [vp, i32]),
    "pwmgpu_get_csb_variant": (C.c_int, [vp, C.POINTER(i32)]),
    "pwmgpu_get_csr": (C.c_int, [vp, vp, vp, vp]),
    "pwmgpu_mv": (C.c_int, [vp, vp, vp]),
    "pwmgpu_mv_device": (C.c_int, [vp, vp, vp]),
    "pwmgpu_mv_device_f32": (C.c_int, [vp, vp, vp]),
    "pwmgpu_power": (C.c_int, [vp, vp, vp, i32]),
    "pwmgpu_power_device": (C.c_int, [vp, vp, vp, i32]),
    "pwmgpu_set_power_mode": (C.c_int, [vp, C.c_int]),
    "pwmgpu_test_grid_wait": (C.c_int, [vp, i64, i32]),
    "pwmgpu_row_blocks": (C.c_int, [i32, i32, vp, vp]),
    "pwmgpu_generate_poisson_rows": (C.c_int, [vp, i32, i32, i32, i32]),
    "pwmgpu_load_triplets_rows": (C.c_int, [vp, i32, i32, i32, vp, vp, vp, i32, i32]),
    "pwmgpu_rows_step_device": (C.c_int, [vp, vp, vp, vp]),
    "pwmgpu_rows_normalize_device": (C.c_int, [vp, vp, vp]),
    "pwmgpu_set_low_format": (C.c_int, [vp, C.c_int]),
    "pwmgpu_solve": (C.c_int, [vp, vp, i32, C.c_double, C.c_int, C.POINTER(SolveInfo)]),
    "pwmgpu_merge_partition": (C.c_int, [vp, i32, vp]),
    "pwmgpu_tile_info": (C.c_int, [vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)]),
    "pwmgpu_csb_info": (C.c_int, [vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32), C.POINTER(i32),
                                  C.POINTER(i64)]),
    "pwmgpu_get_csb": (C.c_int, [vp, vp, vp, vp]),
    "pwmgpu_coh_info": (C.c_int, [vp, C.POINTER(i32), C.POINTER(i64), C.POINTER(i64), C.POINTER(i64),
                                  C.POINTER(i64)]),
    "pwmgpu_get_coh": (C.c_int, [vp, vp, vp, vp, vp, vp, vp, vp]),
    "pwmgpu_csb_params": (C.c_int, [i32, i32, C.POINTER(i32), C.POINTER(i32)]),
    "pwmgpu_launch_config": (C.c_int, [vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32), C.POINTER(C.c_float)]),
    "pwmgpu_set_launch_variant": (C.c_int, [vp, i32]),
    "pwmgpu_launch_variant": (C.c_int, [vp, C.POINTER(i32)]),
    "pwmgpu_plan_info": (C.c_int, [vp, C.POINTER(i32), C.POINTER(i32)]),
    "pwmgpu_csb_build_host": (C.c_int, [i32, i32, i64, vp, vp, vp, vp, vp, vp]),
    "pwmgpu_coh_build_host": (C.c_int, [i32, i32, i64, vp, vp, vp, i32, C.POINTER(i32), C.POINTER(i64),
                                        C.POINTER(i64), C.POINTER(i64), vp, vp, vp, vp, vp, vp, vp]),
    "pwmgpu_mv_csr_device_noalloc": (C.c_int, [i32, i32, i32, vp, vp, vp, vp, vp, vp]),
    "pwmgpu_tile_layout_host": (C.c_int, [i32, i32, i32, i64, vp, vp, vp, i32, i32, C.POINTER(i64), vp, vp, vp, vp,
                                          vp]),
}


def lib_path():
    return LIB


def lib():
    """Load libpwmgpu.so (built by __graft_entry__.build()); raise if absent."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB):
                raise RuntimeError("libpwmgpu.so is not built (%s); run __graft_entry__.build()" % LIB)
            L = C.CDLL(LIB)
            for name, (res, args) in SIGNATURES.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
    return _lib


def last_error():
    try:
        s = lib().pwmgpu_last_error()
        return s.decode() if s else ""
    except Exception:
        return ""


def check(code, where):
    if code != PWMGPU_OK:
        raise PwmGpuError(code, where)
