"""C ABI checks that need no GPU: the library builds and loads, exports every
symbol include/*.h declares, and fails with a status (never a crash) when no
device is present."""
import ctypes
import glob
import os
import re

import pytest

from conftest import ROOT


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[\w\s\*]+?\b((?:pwmgpu|pwmsvc)_\w+)\s*\(", src, re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("pwmgpu_create", "pwmgpu_destroy", "pwmgpu_load_csr", "pwmgpu_load_triplets",
                 "pwmgpu_generate_poisson", "pwmgpu_mv", "pwmgpu_mv_device", "pwmgpu_power",
                 "pwmgpu_last_error", "pwmgpu_merge_partition"):
        assert must in names


def test_library_exports_every_declared_symbol():
    import thesis_spmv_gb300 as t
    L = t.lib()
    missing = [n for n in declared_symbols() if not hasattr(L, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from thesis_spmv_gb300 import _lib
    declared = set(declared_symbols())
    bound = set(_lib.SIGNATURES)
    # every pwmgpu_ symbol has a ctypes signature; the service's pwmsvc_ ones
    # are bound in service.py
    assert {n for n in declared if n.startswith("pwmgpu_")} <= bound
    from thesis_spmv_gb300 import service
    assert {n for n in declared if n.startswith("pwmsvc_")} <= set(service.SIGNATURES)
    service.lib()  # binds every pwmsvc_ signature


def _cuda_present():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_cuda_present(), reason="checks the no-device error path")
def test_no_device_returns_status_not_crash():
    import thesis_spmv_gb300 as t
    L = t.lib()
    h = ctypes.c_void_p()
    rc = L.pwmgpu_create(0, 1, ctypes.byref(h))
    assert rc != 0 and not h.value
    assert t._lib.last_error()
    with pytest.raises(t.PwmGpuError):
        t.CRSCuda(1)


def test_null_arguments_are_rejected():
    import thesis_spmv_gb300 as t
    L = t.lib()
    assert L.pwmgpu_create(0, 1, None) == 1          # PWMGPU_ERR_INVALID
    assert L.pwmgpu_mv(None, None, None) == 1
    assert L.pwmgpu_power(None, None, None, 3) == 1
    assert L.pwmgpu_destroy(None) == 0
    assert L.pwmgpu_create(7, 1, ctypes.byref(ctypes.c_void_p())) == 1  # unknown format
    v = ctypes.c_int32()
    assert L.pwmgpu_launch_variant(None, ctypes.byref(v)) == 1
    assert L.pwmgpu_set_launch_variant(None, 0) == 1
    assert L.pwmgpu_set_launch_variant(None, 12) == 1


def test_host_builders_reject_malformed_crs():
    """The host-side builders (CSB, CO-H, the tile layout) index the caller's
    CRS arrays: row_start not running from 0 to nnz, a decreasing row_start
    or a column outside [0, noc) give PWMGPU_ERR_INVALID, not a crash."""
    import numpy as np
    import thesis_spmv_gb300 as t
    L = t.lib()
    nor, noc = 4, 5
    good_rs = np.array([0, 2, 3, 3, 5], np.int32)
    good_ci = np.array([0, 4, 1, 2, 3], np.int32)
    bad = [
        (np.array([1, 2, 3, 3, 5], np.int32), good_ci),    # does not start at 0
        (np.array([0, 2, 3, 3, 4], np.int32), good_ci),    # does not end at nnz
        (np.array([0, 3, 2, 3, 5], np.int32), good_ci),    # decreases
        (good_rs, np.array([0, 5, 1, 2, 3], np.int32)),    # column == noc
        (good_rs, np.array([0, -1, 1, 2, 3], np.int32)),   # negative column
    ]
    vals = np.ones(5)
    ind = np.zeros(5, np.uint32)
    data = np.zeros(5)
    blk = np.zeros(64, np.int32)
    part = np.zeros(9 * 2, np.int32)
    T, nrj, nblk, nrjb = ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    sizes = (ctypes.c_int64 * 3)()
    for rs, ci in [(good_rs, good_ci)] + bad:
        want = 0 if rs is good_rs and ci is good_ci else 1
        args = (nor, noc, 5, rs.ctypes.data, ci.ctypes.data, vals.ctypes.data)
        assert L.pwmgpu_csb_build_host(*args, ind.ctypes.data, data.ctypes.data, blk.ctypes.data) == want
        assert L.pwmgpu_coh_build_host(*args, 2, ctypes.byref(T), ctypes.byref(nrj), ctypes.byref(nblk),
                                       ctypes.byref(nrjb), part.ctypes.data, None, None, None, None, None,
                                       None) == want
        if want:
            assert t._lib.last_error()
    # the tile layout needs at least a 64-row window: same checks on a taller matrix
    n = 128
    rs = np.arange(n + 1, dtype=np.int32)
    ci = np.arange(n, dtype=np.int32)
    ci_bad = ci.copy()
    ci_bad[7] = n
    for c, want in ((ci, 0), (ci_bad, 1)):
        assert L.pwmgpu_tile_layout_host(1, n, n, n, rs.ctypes.data, c.ctypes.data, np.ones(n).ctypes.data, 1, 64,
                                         sizes, None, None, None, None, None) == want
