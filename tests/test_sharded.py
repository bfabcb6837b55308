"""Partitioned CRS and the row-sharded power method.

The reference's TripletToMultipleCRS (Util/TripletToCRS.hpp:309-385) and its
row-range fillPoisson (Util/Poisson.hpp:33-83) are restated in the oracle and
pinned to the reference's own outputs (tests/golden/ref_multi_crs.npz, made
by tests/golden/make_golden.py --multi).  The library builds the same blocks
on the device (pwmgpu_generate_poisson_rows, pwmgpu_load_triplets_rows), bit
for bit.  The distributed power method of MPI_driver_poisson.cpp:38-63 runs
in thesis_spmv_gb300.sharded over torch.distributed:

* on the CPU, two and three gloo ranks run the host logic (row split,
  allreduce of the squared norms, allgather of the blocks) with the oracle's
  block arithmetic plugged in as the per-rank work; with two ranks the result
  is bit for bit the oracle's single-process restatement of the MPI driver
  (a sum of two doubles does not depend on the order), and every case is
  within 1e-10 of the reference's one-process CRS::powerIteration;
* on the GPU, two gloo ranks (processes sharing the one GPU; no kernel of one
  rank waits on the other) run their blocks through the CUDA kernels, within
  1e-10 of the oracle at equal iteration counts.
"""
import os
import socket
import sys

import numpy as np
import pytest

from conftest import GOLDEN, ROOT
from oracle import pyoracle as O

MULTI = np.load(os.path.join(GOLDEN, "ref_multi_crs.npz"))


def _golden_triplet(name):
    nor, noc = [int(v) for v in MULTI["trip_%s_dims" % name]]
    return (nor, noc, MULTI["trip_%s_rows" % name].copy(), MULTI["trip_%s_cols" % name].copy(),
            MULTI["trip_%s_vals" % name].copy())


@pytest.mark.parametrize("name", ["poisson40x24", "gre_1107", "G38"])
@pytest.mark.parametrize("parts", [1, 2, 3, 5])
def test_oracle_multi_crs_against_reference_outputs(name, parts):
    nor, noc, r, c, v = _golden_triplet(name)
    blocks, first = O.triplet_to_multi_crs(nor, noc, r, c, v, parts)
    pre = "multi%d_%s_" % (parts, name)
    assert np.array_equal(first, MULTI[pre + "first"])
    assert np.array_equal([b.nor for b in blocks], MULTI[pre + "rows"])
    assert np.array_equal(np.concatenate([b.row_start for b in blocks]), MULTI[pre + "row_start"])
    assert np.array_equal(np.concatenate([b.col_ind for b in blocks]), MULTI[pre + "col_ind"])
    assert np.array_equal(np.concatenate([b.data for b in blocks]), MULTI[pre + "data"])


@pytest.mark.parametrize("mnab", [(7, 5, 0, 35), (7, 5, 3, 20), (10, 10, 50, 100), (33, 17, 100, 101),
                                  (33, 17, 560, 561)])
def test_oracle_poisson_rows_against_reference_outputs(mnab):
    B = O.fill_poisson_rows(*mnab)
    pre = "poisson_rows_%d_%d_%d_%d_" % mnab
    assert np.array_equal(B.row_start, MULTI[pre + "row_start"])
    assert np.array_equal(B.col_ind, MULTI[pre + "col_ind"])
    assert np.array_equal(B.data, MULTI[pre + "data"])


@pytest.mark.parametrize("nor,parts", [(960, 1), (960, 7), (1107, 5), (3, 5), (0, 2), (1, 1)])
def test_row_blocks_library_and_host_split_match_oracle(nor, parts):
    from thesis_spmv_gb300 import sharded
    f, t = O.row_blocks(nor, parts)
    fl, tl = sharded.row_blocks(nor, parts)
    fh, th = sharded.row_blocks_host(nor, parts)
    assert np.array_equal(f, fl) and np.array_equal(t, tl)
    assert np.array_equal(f, fh) and np.array_equal(t, th)
    assert t.sum() == nor


def test_oracle_power_rows_is_the_power_method():
    """The MPI driver's iteration equals CRS::powerIteration up to the
    summation order of the norm."""
    A = O.fill_poisson(30, 20)
    x = np.random.default_rng(4).random(A.nor)
    for parts in (1, 2, 4):
        blocks = [O.fill_poisson_rows(30, 20, int(a), int(a + n)) for a, n in zip(*O.row_blocks(A.nor, parts))]
        np.testing.assert_allclose(O.power_rows(blocks, x, 9), O.power_result(A, x, 9), rtol=1e-13, atol=1e-16)


class OracleRowOps:
    """The per-rank block arithmetic of MPI_driver_poisson.cpp done by the
    oracle (test-only stand-in for the CUDA kernels, so the collectives can
    run on CPU ranks)."""

    def __init__(self):
        import torch
        self.torch = torch
        self.B = None

    def generate_poisson_rows(self, m, n, a, b):
        self.B = O.fill_poisson_rows(m, n, a, b)

    def load_triplets_rows(self, t, a, b):
        A = O.triplet_to_crs(t.row_size, t.col_size, t.row_coord.copy(), t.col_coord.copy(), t.data.copy())
        rs = A.row_start[a:b + 1] - A.row_start[a]
        k0, k1 = A.row_start[a], A.row_start[b]
        self.B = O.CRSArrays(b - a, t.col_size, rs, A.col_ind[k0:k1], A.data[k0:k1])

    def vector(self, host):
        return self.torch.tensor(np.asarray(host, np.float64))

    def spmv_sumsq(self, x):
        y = O.crs_mv(self.B, x.numpy())
        nsq = float(np.cumsum(y * y)[-1]) if y.size else 0.0  # rank's sum in row order (:44-47)
        return self.torch.tensor(y), self.torch.tensor([nsq], dtype=self.torch.float64)

    def normalize(self, y, nsq_total):
        return y / np.sqrt(float(nsq_total[0]))  # a true divide (:53-57)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q, kind, it, device):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import torch.distributed as dist
    from thesis_spmv_gb300 import Triplet, sharded
    try:
        dist.init_process_group("gloo", rank=rank, world_size=world)
        if device:
            import torch
            torch.cuda.set_device(0)
            ops = sharded.DeviceRowOps()
        else:
            from test_sharded import OracleRowOps
            ops = OracleRowOps()
        P = sharded.RowShardedPower(ops=ops)
        if kind[0] == "poisson":
            P.generatePoissonMatrix(kind[1], kind[2])
            n = kind[1] * kind[2]
        else:
            nor, noc, r, c, v = _golden_triplet(kind[1])
            P.loadFromTriplets(Triplet(nor, noc, r, c, v))
            n = nor
        x = np.random.default_rng(17).random(n)
        out = P.powerIteration(x, it)
        q.put((rank, out))
        dist.destroy_process_group()
    except Exception as e:  # reported to the parent, which fails the test
        q.put((rank, repr(e)))


def _run_ranks(world, kind, it, device=False):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q, kind, it, device)) for r in range(world)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for r in range(world):
        assert not isinstance(out[r], str), out[r]
    return out


def _reference_inputs(kind):
    if kind[0] == "poisson":
        A = O.fill_poisson(kind[1], kind[2])
        blocks_of = lambda parts: [O.fill_poisson_rows(kind[1], kind[2], int(a), int(a + n))
                                   for a, n in zip(*O.row_blocks(A.nor, parts))]
    else:
        nor, noc, r, c, v = _golden_triplet(kind[1])
        A = O.triplet_to_crs(nor, noc, r.copy(), c.copy(), v.copy())
        blocks_of = lambda parts: O.triplet_to_multi_crs(nor, noc, r.copy(), c.copy(), v.copy(), parts)[0]
    return A, blocks_of


@pytest.mark.parametrize("world", [2, 3])
@pytest.mark.parametrize("kind", [("poisson", 30, 20), ("triplet", "G38")])
def test_sharded_power_gloo_ranks_match_oracle(world, kind):
    pytest.importorskip("torch")
    it = 12
    out = _run_ranks(world, kind, it)
    A, blocks_of = _reference_inputs(kind)
    x = np.random.default_rng(17).random(A.nor)
    want_mpi = O.power_rows(blocks_of(world), x, it)
    want = O.power_result(A, x, it)
    for r in range(world):
        assert np.array_equal(out[r], out[0])  # every rank holds the same x
        if world == 2:
            assert np.array_equal(out[r], want_mpi)
        else:
            np.testing.assert_allclose(out[r], want_mpi, rtol=1e-14, atol=1e-17)
        np.testing.assert_allclose(out[r], want, rtol=1e-10, atol=1e-15)


@pytest.mark.gpu
@pytest.mark.parametrize("kind,parts", [(("poisson", 40, 24), 3), (("triplet", "gre_1107"), 5), (("triplet", "G38"), 2)])
def test_row_blocks_on_device_bitexact(kind, parts):
    """Every block the library builds equals the oracle's (and so the
    reference's) block bit for bit; its SpMV is within the row bound."""
    import thesis_spmv_gb300 as t
    L = t.lib()
    A, blocks_of = _reference_inputs(kind)
    blocks = blocks_of(parts)
    first, rows = O.row_blocks(A.nor, parts)
    x = np.random.default_rng(2).random(A.noc)
    for p, B in enumerate(blocks):
        M = t.CRSCuda(1)
        a, b = int(first[p]), int(first[p] + rows[p])
        if kind[0] == "poisson":
            t.check(L.pwmgpu_generate_poisson_rows(M.handle, kind[1], kind[2], a, b), "poisson rows")
        else:
            nor, noc, r, c, v = _golden_triplet(kind[1])
            M2 = t.Triplet(nor, noc, r, c, v)
            t.check(L.pwmgpu_load_triplets_rows(M.handle, nor, noc, M2.nnz, M2.row_coord.ctypes.data,
                                                M2.col_coord.ctypes.data, M2.data.ctypes.data, a, b), "rows")
            assert np.array_equal(M2.row_coord, r)  # the caller's triplet is left as it was
        rs, ci, d = M.getCSR()
        assert np.array_equal(rs, B.row_start) and np.array_equal(ci, B.col_ind) and np.array_equal(d, B.data)
        y = np.zeros(B.nor)
        M.mv(x, y)
        assert np.all(np.abs(y - O.crs_mv(B, x)) <= O.row_error_bound(B, x))


@pytest.mark.gpu
@pytest.mark.parametrize("kind", [("poisson", 64, 48), ("triplet", "G38")])
def test_sharded_power_two_ranks_on_gpu(kind):
    """Two gloo ranks, each running its row block through the CUDA kernels
    (pwmgpu_rows_step_device, pwmgpu_rows_normalize_device): 12 iterations
    within 1e-10 of the oracle's CRS::powerIteration."""
    pytest.importorskip("torch")
    it = 12
    out = _run_ranks(2, kind, it, device=True)
    A, _ = _reference_inputs(kind)
    x = np.random.default_rng(17).random(A.nor)
    want = O.power_result(A, x, it)
    for r in range(2):
        np.testing.assert_allclose(out[r], want, rtol=1e-10, atol=1e-15)
