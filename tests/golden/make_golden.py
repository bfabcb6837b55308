"""Generate the golden fixtures in tests/golden/ from the reference tree.

Run in the development container (needs the reference tree and a C++
compiler):  python tests/golden/make_golden.py [reference_dir]

Writes
  reference_cases.json  -- the 24 known-answer cases of the reference's
                           Boost.Test suite (Tests/poisson.cpp, Tests/input.cpp):
                           input, operation, tolerance and the golden vector
                           ("precomputed using matlab"), read as text.
  matrices/             -- the six input fixtures of Test_input/, as files.
  ref_stats.json        -- what the reference's Util_Scripts/calc_stats.cpp
                           prints for the matrices of
                           tests/golden_cases.stats_cases() (--stats: only these).
  ref_outputs.npz       -- outputs of the UNMODIFIED reference classes
                           (oracle/_ref) on small seeded inputs: CRS arrays,
                           merge-path coordinates, CSB and CO-H arrays, mv and
                           power results.  These let the GPU-box tests pin the
                           oracle without the reference tree.
  ref_multi_crs.npz     -- the reference's TripletToMultipleCRS blocks and its
                           row-range fillPoisson (--multi: only these).
"""
import json
import os
import re
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def parse_cases(path):
    """Extract each BOOST_AUTO_TEST_CASE of a reference test file."""
    src = open(path).read()
    suites = [(m.start(), m.group(1)) for m in re.finditer(r"BOOST_AUTO_TEST_SUITE\((\w+)\)", src)]
    cases = []
    for m in re.finditer(r"BOOST_AUTO_TEST_CASE\((\w+),\s*\*\s*boost::unit_test::tolerance\(std::pow\(10,\s*(-?\d+)\)\)\)",
                         src):
        start = m.end()
        nxt = src.find("BOOST_AUTO_TEST_CASE(", start)
        body = src[start:nxt if nxt > 0 else len(src)]
        line = src.count("\n", 0, m.start()) + 1
        suite = [s for pos, s in suites if pos < m.start()][-1]
        case = dict(name=m.group(1), suite=suite, line=line, tolerance=10.0 ** int(m.group(2)),
                    index_type="unsigned" if "unsigned" in suite or "<double, unsigned" in body else "int")
        sol = re.search(r"double real_sol\[\]\s*=\s*\{(.*?)\};", body, re.S)
        if sol is None:
            continue  # a case without a golden vector has nothing to pin
        nums = [float(t) for t in re.split(r"[,\s]+", sol.group(1).strip()) if t]
        case["golden"] = nums
        pm = re.search(r"generatePoissonMatrix\((\d+),\s*(\d+),", body)
        mm = re.search(r'loadFromMM\("Test_input/([\w.]+)",\s*(true|false),\s*(true|false)(?:,\s*(true|false))?\)', body)
        bm = re.search(r'loadFromBin\("Test_input/([\w.]+)",\s*(std::pow\(\d+,\s*\d+\)|\d+),\s*(true|false),\s*(true|false)\)',
                       body)
        if pm:
            case["input"] = dict(kind="poisson", m=int(pm.group(1)), n=int(pm.group(2)))
        elif mm:
            case["input"] = dict(kind="mm", file=mm.group(1), has_data=mm.group(2) == "true",
                                 symmetric=mm.group(3) == "true")
        elif bm:
            size_expr = bm.group(2).strip()
            size = int(eval(size_expr.replace("std::pow", "pow"), {"pow": pow}))
            case["input"] = dict(kind="bin", file=bm.group(1), size=size, symmetric=bm.group(3) == "true",
                                 random_vals=bm.group(4) == "true")
        it = re.search(r"powerIteration\(x,\s*y,\s*(\d+)\)", body)
        if it:
            case["op"] = dict(kind="power", iterations=int(it.group(1)), result="x")
        else:
            case["op"] = dict(kind="mv")
        case["x"] = "ones"
        cases.append(case)
    return cases


def main(ref_dir):
    from oracle import pyref as R
    assert R.available(), "oracle/_ref could not be built"
    cases = parse_cases(os.path.join(ref_dir, "Tests", "poisson.cpp"))
    cases += parse_cases(os.path.join(ref_dir, "Tests", "input.cpp"))
    for c in cases:
        c["source"] = "Tests/%s:%d" % ("poisson.cpp" if c["input"]["kind"] == "poisson" else "input.cpp", c["line"])
    with open(os.path.join(HERE, "reference_cases.json"), "w") as f:
        json.dump(dict(generated_by="tests/golden/make_golden.py", cases=cases), f, indent=1)
    print("cases:", len(cases))

    mdir = os.path.join(HERE, "matrices")
    os.makedirs(mdir, exist_ok=True)
    for fn in sorted(os.listdir(os.path.join(ref_dir, "Test_input"))):
        shutil.copyfile(os.path.join(ref_dir, "Test_input", fn), os.path.join(mdir, fn))

    out = {}
    rng = np.random.default_rng(20261203)
    # CRS arrays + mv + power of the reference's sequential CRS on Poisson grids
    for (m, n) in [(3, 3), (9, 3), (5, 5), (10, 5), (37, 29)]:
        M = R.Matrix(R.METHOD_CRS).generate_poisson(m, n)
        rs, ci, d = M.crs()
        x = rng.random(m * n)
        key = "poisson_%dx%d" % (m, n)
        out[key + "_row_start"], out[key + "_col_ind"], out[key + "_data"] = rs, ci, d
        out[key + "_x"] = x
        out[key + "_mv"] = M.mv(x)
        xp, yp = M.power(x, 7)
        out[key + "_power7"] = yp
        # merge-path coordinates for several partition counts (CRS_Merge.hpp:42-62)
        for T in (1, 3, 8, 31):
            MM = R.Matrix(R.METHOD_MERGE, T).generate_poisson(m, n)
            tot = m * n + d.size
            ipt = -(-tot // T)
            out[key + "_merge%d" % T] = np.array([MM.merge_search(min(ipt * t, tot)) for t in range(T + 1)],
                                                 np.int32)
            out[key + "_merge%d_mv" % T] = MM.mv(x)
    # CSB and CO-H arrays on a Poisson triplet and on two fixture matrices
    sets = []
    T = R.Triplet().poisson(40, 24)
    sets.append(("poisson40x24",) + T.get())
    for fn, hd, sym in [("gre_1107.mtx", True, False), ("G38.mtx", False, True)]:
        sets.append((fn.split(".")[0],) + R.Triplet().load_mm(os.path.join(ref_dir, "Test_input", fn), hd, sym).get())
    for name, nor, noc, r, c, v in sets:
        out["trip_%s_rows" % name], out["trip_%s_cols" % name], out["trip_%s_vals" % name] = r, c, v
        out["trip_%s_dims" % name] = np.array([nor, noc], np.int32)
        x = rng.random(noc)
        out["trip_%s_x" % name] = x
        csb = R.Matrix(R.METHOD_CSB, 2).load(R.Triplet().set(nor, noc, r, c, v))
        cs = csb.csb()
        for k in ("ind", "data", "blk_ptr"):
            out["csb_%s_%s" % (name, k)] = cs[k]
        out["csb_%s_info" % name] = np.array([cs["beta"], cs["block_bits"], cs["hb"], cs["vb"], cs["balanced"]],
                                             np.int32)
        out["csb_%s_mv" % name] = csb.mv(x)
        for T in (1, 3):
            coh = R.Matrix(R.METHOD_COH, T).load(R.Triplet().set(nor, noc, r, c, v))
            parts = coh.coh()
            out["coh%d_%s_nparts" % (T, name)] = np.array([len(parts)], np.int32)
            for p, P in enumerate(parts):
                pre = "coh%d_%s_p%d_" % (T, name, p)
                out[pre + "info"] = np.array([P["row_start"], P["beta"], P["block_bits"], P["hb"], P["vb"],
                                              P["nnz"], P["blocks"]], np.int32)
                for k in ("row_jump", "col_jump", "data", "block_nnz", "row_jump_block", "col_jump_block"):
                    out[pre + k] = P[k]
            out["coh%d_%s_mv" % (T, name)] = coh.mv(x)
    # Hilbert indices (BlockCOH.hpp:103-114)
    hs = []
    for size in (1, 2, 4, 8, 16, 64):
        for r in range(min(size, 16)):
            for c in range(min(size, 16)):
                hs.append((size, r, c, R.hilbert(size, r, c)))
    out["hilbert"] = np.array(hs, np.int32)
    np.savez_compressed(os.path.join(HERE, "ref_outputs.npz"), **out)
    print("ref_outputs keys:", len(out), "bytes:", os.path.getsize(os.path.join(HERE, "ref_outputs.npz")))


def make_stats():
    """ref_stats.json: the figures the reference's Util_Scripts/calc_stats.cpp
    prints (built unmodified into oracle/_ref/calc_stats, 17 significant
    digits) for tests/golden_cases.stats_cases()."""
    from oracle import pyref as R
    sys.path.insert(0, os.path.dirname(HERE))
    from golden_cases import stats_cases
    res = {}
    for name, n, r, c, v in stats_cases():
        res[name] = R.calc_stats(n, n, r, c, v)
    with open(os.path.join(HERE, "ref_stats.json"), "w") as f:
        json.dump(dict(generated_by="tests/golden/make_golden.py --stats", cases=res), f, indent=1)
    print("stats cases:", len(res))


def make_multi(ref_dir):
    """ref_multi_crs.npz: the reference's TripletToMultipleCRS
    (Util/TripletToCRS.hpp:309-385) on three triplets for 1, 2, 3 and 5 row
    blocks, and its fillPoisson over row ranges (Util/Poisson.hpp:33-83)."""
    from oracle import pyref as R
    assert R.available(), "oracle/_ref could not be built"
    out = {}
    sets = [("poisson40x24",) + R.Triplet().poisson(40, 24).get()]
    for fn, hd, sym in [("gre_1107.mtx", True, False), ("G38.mtx", False, True)]:
        sets.append((fn.split(".")[0],) + R.Triplet().load_mm(os.path.join(ref_dir, "Test_input", fn), hd, sym).get())
    for name, nor, noc, r, c, v in sets:
        out["trip_%s_rows" % name], out["trip_%s_cols" % name], out["trip_%s_vals" % name] = r, c, v
        out["trip_%s_dims" % name] = np.array([nor, noc], np.int32)
        for parts in (1, 2, 3, 5):
            f, t, rs, ci, d = R.multi_crs(nor, r, c, v, parts)
            pre = "multi%d_%s_" % (parts, name)
            out[pre + "first"], out[pre + "rows"], out[pre + "row_start"] = f, t, rs
            out[pre + "col_ind"], out[pre + "data"] = ci, d
    # (last_row = 0 means "every row" to the reference, so an empty range is not asked for)
    for (m, n, a, b) in [(7, 5, 0, 35), (7, 5, 3, 20), (10, 10, 50, 100), (33, 17, 100, 101), (33, 17, 560, 561)]:
        rs, ci, d = R.fill_poisson_rows(m, n, a, b)
        pre = "poisson_rows_%d_%d_%d_%d_" % (m, n, a, b)
        out[pre + "row_start"], out[pre + "col_ind"], out[pre + "data"] = rs, ci, d
    np.savez_compressed(os.path.join(HERE, "ref_multi_crs.npz"), **out)
    print("ref_multi_crs keys:", len(out))


if __name__ == "__main__":
    if "--stats" in sys.argv:
        make_stats()
    elif "--multi" in sys.argv:
        make_multi(os.environ["PWM_REFERENCE_DIR"] if len(sys.argv) < 3 else sys.argv[-1])
    else:
        if len(sys.argv) < 2 and not os.environ.get("PWM_REFERENCE_DIR"):
            sys.exit("usage: make_golden.py REFERENCE_TREE (or set PWM_REFERENCE_DIR)")
        main(sys.argv[1] if len(sys.argv) > 1 else os.environ["PWM_REFERENCE_DIR"])
        make_stats()
        make_multi(sys.argv[1] if len(sys.argv) > 1 else os.environ["PWM_REFERENCE_DIR"])
