"""The header-only C++ drop-in classes (include/pwmgpu/CudaSparseMatrix.hpp):
pwm::CRSCuda / CSBCuda / BlockCOHCuda / AutoCuda derive from the reference's
pwm::SparseMatrix and are used through that interface by a driver in the
shape of the reference's drivers (tests/cpp/dropin_driver.cpp).

CPU: the header and the driver compile against the real reference interface
(Matrix/SparseMatrix.hpp, Matrix/Triplet.hpp) where the reference tree is
present.  GPU: the driver, built against the interface stand-in, runs all
four methods (15: the format autotuner); its outputs match the oracle (mv rows within the row bound,
powerIteration within 1e-10, the triplet sorted like TripletToCRS)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from oracle import pyoracle as O

CPP = os.path.join(ROOT, "tests", "cpp")


def _gxx():
    g = shutil.which("g++")
    if not g:
        pytest.skip("g++ not found")
    return g


def test_header_compiles_against_reference_interface(tmp_path):
    from oracle.build import build_ref, reference_dir
    build_ref()
    REF = reference_dir()
    if REF is None:
        pytest.skip("reference tree not present")
    cmd = [_gxx(), "-std=c++17", "-fsyntax-only", "-fopenmp", "-DNTBB", "-include", "cstring", "-include", "climits",
           "-I" + os.path.join(ROOT, "oracle", "ref_shim"), "-I" + REF, "-I" + os.path.join(ROOT, "include"),
           os.path.join(CPP, "dropin_driver.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def _build_driver(tmp_path):
    import thesis_spmv_gb300 as t
    lib = t.lib_path()
    exe = str(tmp_path / "dropin_driver")
    cmd = [_gxx(), "-std=c++17", "-O2", "-I" + os.path.join(CPP, "stand_in"), "-I" + os.path.join(ROOT, "include"),
           os.path.join(CPP, "dropin_driver.cpp"), "-o", exe, "-L" + os.path.dirname(lib), "-lpwmgpu",
           "-Wl,-rpath," + os.path.dirname(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def test_driver_builds_against_stand_in(tmp_path):
    t = pytest.importorskip("thesis_spmv_gb300")
    t.lib()
    _build_driver(tmp_path)


@pytest.mark.gpu
@pytest.mark.parametrize("itype", ["u32", "int", "unsigned"])
@pytest.mark.parametrize("method", [12, 13, 14, 15])
def test_driver_runs_through_the_interface(tmp_path, method, itype):
    """Every method with the index types the reference instantiates:
    uint32_t (drivers), int and unsigned int (Tests/poisson.cpp:28,146)."""
    exe = _build_driver(tmp_path)
    m, n, it = 37, 23, 9
    out = str(tmp_path / "out.bin")
    r = subprocess.run([exe, str(method), str(m), str(n), str(it), out, itype], capture_output=True, text=True)
    assert r.returncode == 0, (r.stdout, r.stderr)
    assert "threw=1" in r.stdout
    N = m * n
    raw = open(out, "rb").read()
    y = np.frombuffer(raw, np.float64, N, 0)
    p = np.frombuffer(raw, np.float64, N, 8 * N)
    A = O.fill_poisson(m, n)
    x = np.ones(N)
    assert np.all(np.abs(y - O.crs_mv(A, x)) <= O.row_error_bound(A, x))
    np.testing.assert_allclose(p, O.power_result(A, x, it), rtol=1e-10, atol=1e-14)
    # the random triplet: the driver's LCG, restated here
    R, nnz = 501, 4000
    s = 12345
    rows, cols, vals, seen = [], [], [], set()

    def nxt():
        nonlocal s
        s = (s * 6364136223846793005 + 1442695040888963407) % 2 ** 64
        return s >> 33
    while len(rows) < nnz:
        rr, cc = nxt() % R, nxt() % R
        if (rr, cc) in seen:
            continue
        seen.add((rr, cc))
        rows.append(rr)
        cols.append(cc)
        vals.append((nxt() % 2000) / 1000.0 - 1.0)
    B = O.triplet_to_crs(R, R, np.array(rows, np.int32), np.array(cols, np.int32), np.array(vals))
    xb = 1.0 + (np.arange(R) % 7)
    off = 16 * N
    yb = np.frombuffer(raw, np.float64, R, off)
    assert np.all(np.abs(yb - O.crs_mv(B, xb)) <= O.row_error_bound(B, xb))
    off += 8 * R
    idt = np.int32 if itype == "int" else np.uint32
    srows = np.frombuffer(raw, idt, nnz, off)
    scols = np.frombuffer(raw, idt, nnz, off + 4 * nnz)
    order = np.lexsort((np.array(cols), np.array(rows)))
    assert np.array_equal(srows, np.array(rows)[order]) and np.array_equal(scols, np.array(cols)[order])
