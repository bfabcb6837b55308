"""Pin the C oracle against the reference's own known answers.

1. The 24 Boost.Test cases of Tests/poisson.cpp and Tests/input.cpp (golden
   vectors "precomputed using matlab"), at the reference's tolerances, for the
   sequential CRS path and the merge path at several partition counts.
2. Outputs of the unmodified reference classes recorded in
   tests/golden/ref_outputs.npz (CRS arrays, merge coordinates, CSB / CO-H
   arrays, mv / power results).
"""
import numpy as np
import pytest

from oracle import pyoracle as O
from golden_cases import boost_close, case_ids, cases, ref_outputs, triplets_for

CASES = cases()


def _matrix(case):
    t = triplets_for(case)
    if t is None:
        return O.fill_poisson(case["input"]["m"], case["input"]["n"])
    nor, noc, r, c, v = t
    return O.triplet_to_crs(nor, noc, r, c, v)


@pytest.mark.parametrize("case", CASES, ids=case_ids())
def test_known_answers(case):
    A = _matrix(case)
    x = np.ones(A.noc)
    golden = np.array(case["golden"])
    tol = case["tolerance"]
    if case["op"]["kind"] == "mv":
        outs = [O.crs_mv(A, x)] + [O.merge_mv(A, x, t) for t in (1, 2, 3, 7)] + [O.crs_omp_mv(A, x, 4)]
    else:
        it = case["op"]["iterations"]
        outs = [O.power(A, x, it, kind=k, threads=t)[0] for k, t in ((0, 1), (1, 4), (2, 3))]
    for y in outs:
        assert y.shape == golden.shape
        assert boost_close(y, golden, tol).all()


def test_reference_count():
    assert len(CASES) == 24


REF = ref_outputs()


@pytest.mark.parametrize("mn", [(3, 3), (9, 3), (5, 5), (10, 5), (37, 29)])
def test_poisson_against_reference_outputs(mn):
    m, n = mn
    key = "poisson_%dx%d" % mn
    A = O.fill_poisson(m, n)
    assert np.array_equal(A.row_start, REF[key + "_row_start"])
    assert np.array_equal(A.col_ind, REF[key + "_col_ind"])
    assert np.array_equal(A.data, REF[key + "_data"])
    x = REF[key + "_x"]
    assert np.array_equal(O.crs_mv(A, x), REF[key + "_mv"])
    assert np.array_equal(O.power(A, x, 7)[1], REF[key + "_power7"])
    # COO generator + triplet->CRS gives the same arrays (Triplet.hpp:226-278)
    r, c, v = O.triplet_poisson(m, n)
    B = O.triplet_to_crs(m * n, m * n, r, c, v)
    assert np.array_equal(B.row_start, A.row_start) and np.array_equal(B.col_ind, A.col_ind)
    for T in (1, 3, 8, 31):
        assert np.array_equal(O.merge_partition(A, T), REF[key + "_merge%d" % T])
        assert np.array_equal(O.merge_mv(A, x, T), REF[key + "_merge%d_mv" % T])


@pytest.mark.parametrize("name", ["poisson40x24", "gre_1107", "G38"])
def test_csb_coh_against_reference_outputs(name):
    nor, noc = [int(v) for v in REF["trip_%s_dims" % name]]
    r = REF["trip_%s_rows" % name].copy()
    c = REF["trip_%s_cols" % name].copy()
    v = REF["trip_%s_vals" % name].copy()
    x = REF["trip_%s_x" % name]
    csb = O.csb_build(nor, noc, r.copy(), c.copy(), v.copy())
    info = REF["csb_%s_info" % name]
    assert [csb["beta"], csb["block_bits"], csb["hb"], csb["vb"], csb["balanced"]] == list(info)
    for k in ("ind", "data", "blk_ptr"):
        assert np.array_equal(csb[k], REF["csb_%s_%s" % (name, k)])
    np.testing.assert_allclose(O.csb_mv(nor, noc, csb, x), REF["csb_%s_mv" % name], rtol=1e-13, atol=1e-13)
    for T in (1, 3):
        coh = O.coh_build(nor, noc, r.copy(), c.copy(), v.copy(), T)
        nparts = int(REF["coh%d_%s_nparts" % (T, name)][0])
        assert coh["threads"] == nparts
        info = coh["part_info"].reshape(nparts, 9)
        o = dict(rj=0, nz=0, b=0, rjb=0)
        for p in range(nparts):
            pre = "coh%d_%s_p%d_" % (T, name, p)
            assert list(info[p, :7]) == list(REF[pre + "info"])
            nrj, nz, nb, nrjb = info[p, 7], info[p, 5], info[p, 6], info[p, 8]
            assert np.array_equal(coh["row_jump"][o["rj"]:o["rj"] + nrj], REF[pre + "row_jump"])
            assert np.array_equal(coh["col_jump"][o["nz"]:o["nz"] + nz], REF[pre + "col_jump"])
            assert np.array_equal(coh["data"][o["nz"]:o["nz"] + nz], REF[pre + "data"])
            assert np.array_equal(coh["block_nnz"][o["b"]:o["b"] + nb], REF[pre + "block_nnz"])
            assert np.array_equal(coh["col_jump_block"][o["b"]:o["b"] + nb], REF[pre + "col_jump_block"])
            assert np.array_equal(coh["row_jump_block"][o["rjb"]:o["rjb"] + nrjb], REF[pre + "row_jump_block"])
            o["rj"] += nrj; o["nz"] += nz; o["b"] += nb; o["rjb"] += nrjb
        np.testing.assert_allclose(O.coh_mv(nor, coh, x), REF["coh%d_%s_mv" % (T, name)], rtol=1e-13, atol=1e-13)


def test_hilbert_against_reference_outputs():
    for size, r, c, h in REF["hilbert"]:
        assert O.hilbert(int(size), int(r), int(c)) == int(h)


def test_oracle_plants_a_mistake_is_caught():
    """A planted error in an oracle output must fail the golden comparison."""
    case = CASES[0]
    A = _matrix(case)
    y = O.crs_mv(A, np.ones(A.noc))
    y[3] += 1e-9
    assert not boost_close(y, np.array(case["golden"]), case["tolerance"]).all()


def test_calc_stats_against_reference_outputs():
    """The oracle's Util_Scripts/calc_stats.cpp restatement prints the same
    doubles as the reference's own script (tests/golden/ref_stats.json)."""
    from golden_cases import ref_stats, stats_cases
    ref = ref_stats()
    names = set()
    for name, n, r, c, v in stats_cases():
        got = O.calc_stats(n, r, c)
        want = ref[name]
        for k in ("size", "nnz", "rows_avg", "rows_var", "block_avg", "block_var", "balanced"):
            assert got[k] == want[k], (name, k, got[k], want[k])
        names.add(name)
    assert names == set(ref)
    assert any(w["balanced"] == 0 for w in ref.values()) and any(w["balanced"] == 1 for w in ref.values())


def test_merge_omp_matches_sequential_partitions():
    """The OpenMP CRS_Merge restatement (the CPU baseline's timing path) gives
    the sequential-partition restatement's bits, which the compiled reference
    pins (ref_outputs.npz)."""
    for mn in [(37, 29), (10, 5)]:
        A = O.fill_poisson(*mn)
        x = REF["poisson_%dx%d_x" % mn]
        for T in (1, 3, 8, 31):
            assert np.array_equal(O.merge_omp_mv(A, x, T), O.merge_mv(A, x, T))
            assert np.array_equal(O.merge_omp_mv(A, x, T), REF["poisson_%dx%d_merge%d_mv" % (mn + (T,))])
