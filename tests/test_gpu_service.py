"""The batched power-method service (include/pwmsvc.h) against the oracle.

Each round advances every live solve in one launch per power step (their
merge-path sub-tiles form the block-diagonal merge path of the live
matrices).  Tolerances as for pwmgpu_solve: at equal step counts lambda and u
within 1e-10 relative of the oracle; converged results confirmed by the
oracle's residual (within 2 tol) and, for Poisson grids, the analytic
lambda_max = 4 + 4 cos(pi/(m+1)) within 1e-10.  A solve gives the same bits
alone and in a mix (sums run over each solve's own sub-tiles in a fixed
order); the test asserts bit equality, which implies the stated tolerance.
"""
import math

import numpy as np
import pytest

from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def svc_mod():
    import thesis_spmv_gb300 as t
    from thesis_spmv_gb300 import service
    t.lib()
    service.lib()
    return t, service


def _positive_random(n, mean_len, seed):
    rng = np.random.default_rng(seed)
    rows = []
    for i in range(n):
        c = set(rng.integers(0, n, size=int(rng.poisson(mean_len))).tolist()) | {i, (i + 1) % n}
        rows.append(np.array(sorted(c), np.int32))
    rs = np.zeros(n + 1, np.int32)
    rs[1:] = np.cumsum([r.size for r in rows])
    cols = np.concatenate(rows)
    return O.CRSArrays(n, n, rs, cols, rng.uniform(0.0, 1.0, cols.size) + 1e-3)


def test_service_poisson_analytic(svc_mod):
    t, S = svc_mod
    svc = S.Service(round_iterations=8)
    m = 8
    rid = svc.submit_poisson(m, m, max_it=20000, tol=1e-10, precision=t.PREC_F64, x0_seed=3, keep_vector=True)
    svc.run_until_idle()
    r, u = svc.result(rid, want_vector=True)
    assert r.state == S.DONE and r.converged == 1 and r.residual <= 1e-10
    exact = 4.0 + 4.0 * math.cos(math.pi / (m + 1))
    assert abs(r.lambda_ - exact) <= 1e-10 * exact
    lam_r, res_r = O.rayleigh(O.fill_poisson(m, m), u)
    assert res_r <= 2e-10 and abs(lam_r - exact) <= 1e-10 * exact
    assert r.iterations % 8 == 0


@pytest.mark.parametrize("seeded", [True, False])
def test_service_equal_counts_match_oracle(svc_mod, seeded):
    """tol = 0: exactly max_it steps (3 rounds of 8); lambda and u are those
    of the oracle's iterate after 23 powerIteration steps."""
    t, S = svc_mod
    A = O.fill_poisson(29, 31)
    svc = S.Service(round_iterations=8)
    if seeded:
        x0 = O.uniform_vector(A.nor, 77)
        rid = svc.submit_poisson(29, 31, max_it=24, tol=0.0, x0_seed=77, keep_vector=True)
    else:
        x0 = np.random.default_rng(5).random(A.nor)
        rid = svc.submit_csr(A, max_it=24, tol=0.0, x0=x0, keep_vector=True)
    svc.run_until_idle()
    r, u = svc.result(rid, want_vector=True)
    assert r.state == S.DONE and r.iterations == 24 and r.converged == 0
    ur = O.power_result(A, x0, 23)
    lam_r, res_r = O.rayleigh(A, ur)
    assert abs(r.lambda_ - lam_r) <= 1e-10 * abs(lam_r)
    assert abs(r.residual - res_r) <= 1e-8 * res_r
    assert np.max(np.abs(u - ur)) <= 1e-10 * np.max(np.abs(ur))


def _run_target(S, t, others, use_graph=True, poisson=False):
    """The target solve (a fast-converging random matrix, or a 14 x 14
    Poisson grid whose slow convergence makes the mixed solve take its
    low-precision phase), submitted between other requests over several
    rounds; returns its result and vector."""
    svc = S.Service(round_iterations=8, use_graph=use_graph)
    for o in others[: len(others) // 2]:
        o(svc)
    if others:
        svc.step()
        svc.step()
    if poisson:
        rid = svc.submit_poisson(14, 14, max_it=4000, tol=1e-10, precision=t.PREC_MIXED, x0_seed=9,
                                 keep_vector=True)
    else:
        rid = svc.submit_random(6000, 42, mean_len=12.0, max_it=4000, tol=1e-10, precision=t.PREC_MIXED,
                                x0_seed=9, keep_vector=True)
    for o in others[len(others) // 2:]:
        svc.step()
        o(svc)
    svc.run_until_idle()
    return svc.result(rid, want_vector=True)


@pytest.mark.parametrize("poisson", [False, True])
def test_service_alone_equals_mix(svc_mod, poisson):
    """The same request alone and among others (sizes, sources and
    precisions mixed, arriving before and after it) gives identical bits --
    in FP64 throughout (the precision tuner's choice for the fast random
    matrix) and through the FP32 / BF16 bulk phase (the Poisson grid)."""
    t, S = svc_mod
    A = _positive_random(2000, 6, 1)
    others = [
        lambda s: s.submit_poisson(40, 25, max_it=300, tol=1e-10, precision=t.PREC_F64),
        lambda s: s.submit_random(50000, 7, length_dist=1, mean_len=8.0, max_len=64, band_permille=0, band_half=0,
                                  max_it=400, tol=1e-10, precision=t.PREC_MIXED),
        lambda s: s.submit_csr(A, max_it=200, tol=1e-12, precision=t.PREC_F32),
        lambda s: s.submit_poisson(128, 128, max_it=160, tol=1e-10, precision=t.PREC_MIXED),
        lambda s: s.submit_random(20000, 3, max_it=400, tol=1e-10, precision=t.PREC_F64),
        lambda s: s.submit_random(1000, 5, mean_len=4.0, max_it=64, tol=0.0, precision=t.PREC_F64),
    ]
    r1, u1 = _run_target(S, t, [], poisson=poisson)
    r2, u2 = _run_target(S, t, others, poisson=poisson)
    assert r1.state == S.DONE and r1.converged == 1
    assert (r1.iterations_low > 0) if poisson else (r1.iterations_low == 0)
    for f in ("iterations", "iterations_low", "converged"):
        assert getattr(r1, f) == getattr(r2, f), f
    assert r1.lambda_ == r2.lambda_ and r1.residual == r2.residual
    assert np.array_equal(u1.view(np.uint64), u2.view(np.uint64))
    # and the oracle confirms the result
    B = O.fill_poisson(14, 14) if poisson else O.random_crs(6000, 42, 0, 12.0, 1.2, 20000, 300, 4096)
    lam_r, res_r = O.rayleigh(B, u1)
    assert res_r <= 2e-10 and abs(lam_r - r1.lambda_) <= 1e-10 * abs(lam_r)


def test_service_graph_equals_direct_launches(svc_mod):
    t, S = svc_mod
    r1, u1 = _run_target(S, t, [], use_graph=True)
    r2, u2 = _run_target(S, t, [], use_graph=False)
    assert r1.iterations == r2.iterations and r1.lambda_ == r2.lambda_
    assert np.array_equal(u1, u2)


def test_service_budget_admission(svc_mod):
    t, S = svc_mod
    n = 200_000
    # each request is charged about 31 MB (plan, CRS during the build,
    # vectors, for 1.1 nnz estimated per unit of mean row length): two fit
    svc = S.Service(hbm_budget_bytes=80 << 20, round_iterations=4)
    with pytest.raises(t.PwmGpuError) as e:
        svc.submit_random(50 * n, 1, mean_len=16.0, max_it=10, tol=0.0)
    assert e.value.code == 7  # PWMGPU_ERR_BUDGET
    ids = [svc.submit_random(n, s, length_dist=1, mean_len=5.0, max_len=64, band_permille=0, band_half=0,
                             max_it=8, tol=0.0) for s in range(6)]
    saw_queue = False
    for _ in range(1000):
        live, queued, _ = svc.step()
        st = svc.stats()
        assert st.hbm_in_use <= st.hbm_budget
        saw_queue |= live > 0 and queued > 0
        if live == 0 and queued == 0:
            break
    assert saw_queue
    for rid in ids:
        r = svc.result(rid)
        assert r.state == S.DONE and r.iterations == 8
        assert r.t_submit <= r.t_admit <= r.t_done


def test_service_mixed_and_f32_against_oracle(svc_mod):
    t, S = svc_mod
    A = _positive_random(20000, 8, 9)
    svc = S.Service(round_iterations=8)
    x0 = np.random.default_rng(2).random(A.nor)
    ids = {p: svc.submit_csr(A, max_it=2000, tol=tol, precision=p, x0=x0, keep_vector=True)
           for p, tol in ((t.PREC_F64, 1e-10), (t.PREC_MIXED, 1e-10), (t.PREC_F32, 1e-5))}
    svc.run_until_idle()
    res = {p: svc.result(rid, want_vector=True) for p, rid in ids.items()}
    (r64, u64), (rmx, umx), (r32, u32) = res[t.PREC_F64], res[t.PREC_MIXED], res[t.PREC_F32]
    assert r64.converged == rmx.converged == r32.converged == 1
    # this matrix converges within a few rounds: the precision tuner keeps the
    # mixed solve in FP64 after its probe round
    assert rmx.iterations_low == 0 and r32.iterations_low == r32.iterations
    for u, tol in ((u64, 1e-10), (umx, 1e-10)):
        lam_r, res_r = O.rayleigh(A, u)
        assert res_r <= 2 * tol and abs(lam_r - r64.lambda_) <= 1e-10 * abs(lam_r)
    lam_r, res_r = O.rayleigh(A, u32)
    assert res_r <= 1e-4 and abs(lam_r - r64.lambda_) <= 1e-5 * abs(lam_r)


def test_service_triplet_source_equals_csr(svc_mod):
    """PWMSVC_SRC_TRIPLETS: shuffled triplets of a matrix, sorted into CRS on
    the device at admission, give the same bits as the CSR request of it."""
    t, S = svc_mod
    A = _positive_random(3000, 6.0, 21)
    rows = np.repeat(np.arange(A.nor, dtype=np.int32), np.diff(A.row_start))
    p = np.random.default_rng(22).permutation(rows.size)
    svc = S.Service(round_iterations=8)
    a = svc.submit_csr(A, max_it=400, tol=1e-12, x0_seed=4, keep_vector=True)
    b = svc.submit_triplets(A.nor, rows[p], A.col_ind[p], A.data[p], max_it=400, tol=1e-12, x0_seed=4,
                            keep_vector=True)
    svc.run_until_idle()
    ra, ua = svc.result(a, want_vector=True)
    rb, ub = svc.result(b, want_vector=True)
    assert ra.state == rb.state == S.DONE and ra.iterations == rb.iterations
    assert ra.lambda_ == rb.lambda_ and ra.residual == rb.residual
    assert np.array_equal(ua, ub)
    with pytest.raises(ValueError):
        svc.submit_triplets(10, np.zeros(3), np.zeros(2), np.zeros(3))
    # an entry out of range fails at admission, as a failed request
    bad = svc.submit_triplets(4, np.array([0, 1, 9]), np.array([0, 1, 2]), np.ones(3), max_it=10)
    svc.run_until_idle()
    assert svc.result(bad).state == S.FAILED


@pytest.mark.parametrize("precision", ["f64", "mixed"])
def test_service_batch_classes_confirmed_by_oracle(svc_mod, precision):
    """A seeded sub-batch shaped like the benchmark's 256-matrix batch and
    serving stream (Poisson grids; random matrices with Poisson(8) rows and
    uniform columns; lognormal-row matrices with a band), solved together to
    1e-10 or 2,000 steps: every returned eigenpair is checked by the FP64
    oracle's Rayleigh quotient -- lambda within 1e-10 relative, the oracle's
    residual within 2 tol for converged solves and equal to the reported one
    within 1e-12 absolute for the capped ones."""
    t, S = svc_mod
    prec = t.PREC_F64 if precision == "f64" else t.PREC_MIXED
    specs = [("poisson", dict(m=37, n=41)), ("poisson", dict(m=64, n=64)),
             ("random", dict(n=3000, seed=1001, length_dist=1, mean_len=8.0, sigma=0.0, max_len=64,
                             band_permille=0, band_half=0)),
             ("random", dict(n=40000, seed=1002, length_dist=1, mean_len=8.0, sigma=0.0, max_len=64,
                             band_permille=0, band_half=0)),
             ("random", dict(n=20000, seed=5001, length_dist=0, mean_len=16.0, sigma=1.2, max_len=20000,
                             band_permille=300, band_half=4096))]
    svc = S.Service(round_iterations=8)
    ids = []
    for kind, kw in specs:
        if kind == "poisson":
            ids.append(svc.submit_poisson(kw["m"], kw["n"], max_it=2000, tol=1e-10, precision=prec, x0_seed=11,
                                          keep_vector=True))
        else:
            ids.append(svc.submit_random(max_it=2000, tol=1e-10, precision=prec, x0_seed=11, keep_vector=True, **kw))
    svc.run_until_idle()
    for (kind, kw), rid in zip(specs, ids):
        r, u = svc.result(rid, want_vector=True)
        assert r.state == S.DONE
        A = O.fill_poisson(kw["m"], kw["n"]) if kind == "poisson" else O.random_crs(
            kw["n"], kw["seed"], kw["length_dist"], kw["mean_len"], kw["sigma"], kw["max_len"], kw["band_permille"],
            kw["band_half"])
        lam_o, res_o = O.rayleigh(A, u)
        assert abs(r.lambda_ - lam_o) <= 1e-10 * abs(lam_o), (kind, kw)
        if r.converged:
            assert res_o <= 2e-10, (kind, kw, res_o)
        else:
            assert r.iterations >= 2000 and abs(r.residual - res_o) <= 1e-12, (kind, kw, r.residual, res_o)
    assert svc.result(ids[2]).converged and svc.result(ids[4]).converged  # the random classes converge
    svc.close()


def test_service_burst_built_beside_a_round(svc_mod):
    """Requests that arrive while solves are live are built beside the
    running round, several matrices at a time on host threads, and then join
    the next round: each result equals the same request served alone, bit
    for bit, in every source and precision."""
    t, S = svc_mod
    A = _positive_random(3000, 6, 11)
    reqs = [
        lambda s: s.submit_poisson(60, 40, max_it=96, tol=0.0, precision=t.PREC_F64, x0_seed=1, keep_vector=True),
        lambda s: s.submit_random(40000, 3, max_it=96, tol=0.0, precision=t.PREC_MIXED, x0_seed=2,
                                  keep_vector=True),
        lambda s: s.submit_csr(A, max_it=96, tol=0.0, precision=t.PREC_F32, x0_seed=3, keep_vector=True),
        lambda s: s.submit_poisson(90, 90, max_it=96, tol=0.0, precision=t.PREC_MIXED, x0_seed=4,
                                   keep_vector=True),
        lambda s: s.submit_random(20000, 8, mean_len=6.0, max_it=96, tol=0.0, precision=t.PREC_F64, x0_seed=5,
                                  keep_vector=True),
    ]

    def alone(i):
        svc = S.Service(round_iterations=8)
        rid = reqs[i](svc)
        svc.run_until_idle()
        out = svc.result(rid, want_vector=True)
        svc.close()
        return out

    svc = S.Service(round_iterations=8)
    first = svc.submit_poisson(200, 200, max_it=400, tol=0.0, precision=t.PREC_F64, x0_seed=9)
    svc.step()  # admits the first request with nothing live
    svc.step()  # its round runs
    ids = [f(svc) for f in reqs]  # a burst while it is live
    svc.run_until_idle()
    assert svc.result(first).state == S.DONE
    for i, rid in enumerate(ids):
        r, u = svc.result(rid, want_vector=True)
        ra, ua = alone(i)
        assert r.state == S.DONE and r.iterations == ra.iterations == 96
        assert r.lambda_ == ra.lambda_ and r.residual == ra.residual
        assert np.array_equal(u.view(np.uint64), ua.view(np.uint64))
    svc.close()
