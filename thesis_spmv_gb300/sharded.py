"""Row-sharded power method: one rank per GPU, each holding a block of rows.

Host mirror of the reference's distributed power method
(MPI_driver_poisson.cpp:38-63, 84-101) and of its partitioned CRS
(Util/TripletToCRS.hpp:309-385 TripletToMultipleCRS): the rows are split
into `world` consecutive blocks by the reference's rule (nor // world rows per
block, the last block takes the rest); rank r holds block r as a
(rows_r x N) CRS matrix with global columns on its GPU.  One iteration is

    y_r = A_r x                       (pwmgpu_rows_step_device, with ||y_r||^2)
    s   = allreduce(||y_r||^2)        (MPI_Allreduce, :50)
    y_r = y_r / sqrt(s)               (pwmgpu_rows_normalize_device, :53-57)
    x   = allgather(y_0, ..., y_{P-1}) (MPI_Allgatherv, :61)

The collectives run through torch.distributed: NCCL on device tensors when
the process group's backend is "nccl", host tensors otherwise (gloo).  The
blocks have unequal sizes (the last one is larger), so the allgather moves
blocks padded to the largest one and x is assembled from their prefixes.

`RowShardedPower(ops=...)` takes the per-rank device work as an object with
`spmv_sumsq(x) -> (y, nsq)` and `normalize(y, nsq_total) -> y`; the default
is `DeviceRowOps` (the CUDA kernels through the C ABI).  The host logic --
blocks, collectives, assembly -- is the same whatever the ops.
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import check
from .matrix import CRSCuda, Triplet


def row_blocks(nor, parts):
    """(first_rows, thread_rows) of the reference's 1D split."""
    f = np.zeros(parts, np.int32)
    t = np.zeros(parts, np.int32)
    check(_lib.lib().pwmgpu_row_blocks(int(nor), int(parts), f.ctypes.data, t.ctypes.data), "pwmgpu_row_blocks")
    return f, t


def row_blocks_host(nor, parts):
    """The same split computed in Python (for ranks without the library
    loaded, e.g. host-only tests of the collectives)."""
    if parts < 1 or nor < 0:
        raise ValueError("parts >= 1 and nor >= 0")
    am = nor // parts
    first = np.array([i * am for i in range(parts)], np.int32)
    rows = np.array([am] * (parts - 1) + [nor - am * (parts - 1)], np.int32)
    return first, rows


class DeviceRowOps:
    """A rank's block on its GPU: CRS (merge-path plan) built by the library,
    the step and the normalisation as CUDA kernels on torch device tensors."""

    def __init__(self, device=None):
        import torch
        self.torch = torch
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else device
        self.M = CRSCuda(1)
        self.stream = torch.cuda.current_stream(self.device)
        self.M.set_stream(self.stream.cuda_stream)
        self.rows = 0

    def generate_poisson_rows(self, m, n, first_row, last_row):
        check(_lib.lib().pwmgpu_generate_poisson_rows(self.M.handle, int(m), int(n), int(first_row), int(last_row)),
              "pwmgpu_generate_poisson_rows")
        self.rows = int(last_row - first_row)

    def load_triplets_rows(self, triplet, first_row, last_row):
        t = triplet
        check(_lib.lib().pwmgpu_load_triplets_rows(
            self.M.handle, t.row_size, t.col_size, t.nnz, t.row_coord.ctypes.data if t.nnz else None,
            t.col_coord.ctypes.data if t.nnz else None, t.data.ctypes.data if t.nnz else None,
            int(first_row), int(last_row)), "pwmgpu_load_triplets_rows")
        self.rows = int(last_row - first_row)

    def vector(self, host):
        return self.torch.as_tensor(np.ascontiguousarray(host, np.float64)).to(self.device)

    def spmv_sumsq(self, x):
        torch = self.torch
        y = torch.empty(max(self.rows, 1), dtype=torch.float64, device=self.device)
        nsq = torch.empty(1, dtype=torch.float64, device=self.device)
        check(_lib.lib().pwmgpu_rows_step_device(self.M.handle, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                                                 C.c_void_p(nsq.data_ptr())), "pwmgpu_rows_step_device")
        return y[:self.rows], nsq

    def normalize(self, y, nsq_total):
        check(_lib.lib().pwmgpu_rows_normalize_device(self.M.handle, C.c_void_p(y.data_ptr()),
                                                      C.c_void_p(nsq_total.data_ptr())),
              "pwmgpu_rows_normalize_device")
        return y


class RowShardedPower:
    """The distributed power method over a torch.distributed process group
    (one rank per GPU): generatePoissonMatrix / loadFromTriplets build this
    rank's row block, powerIteration runs the iterations on every rank."""

    def __init__(self, group=None, ops=None):
        import torch.distributed as dist
        self.dist = dist
        self.group = group
        self.world = dist.get_world_size(group)
        self.rank = dist.get_rank(group)
        self.ops = ops if ops is not None else DeviceRowOps()
        self.nor = 0
        self.first = self.rows = None

    def _blocks(self, nor):
        try:
            f, t = row_blocks(nor, self.world)
        except (RuntimeError, OSError):
            f, t = row_blocks_host(nor, self.world)
        self.nor = int(nor)
        self.first, self.rows = f, t
        return int(f[self.rank]), int(f[self.rank] + t[self.rank])

    def generatePoissonMatrix(self, m, n):
        """This rank's rows of the m x n Poisson matrix (the MPI driver's
        fillPoisson(first_row, last_row), MPI_driver_poisson.cpp:91-101)."""
        a, b = self._blocks(int(m) * int(n))
        self.ops.generate_poisson_rows(m, n, a, b)

    def loadFromTriplets(self, triplet):
        """This rank's block of TripletToMultipleCRS (every rank passes the
        whole triplet; square matrices, as the power method needs)."""
        if not isinstance(triplet, Triplet):
            raise TypeError("a Triplet")
        if triplet.row_size != triplet.col_size:
            raise ValueError("the power method needs a square matrix")
        a, b = self._blocks(triplet.row_size)
        self.ops.load_triplets_rows(triplet, a, b)

    def powerIteration(self, x, it):
        """`it` iterations from the full start vector x (host, length N);
        returns the normalised full iterate (numpy) on every rank."""
        import torch
        if self.first is None:
            raise RuntimeError("no matrix loaded")
        dist = self.dist
        on_device = dist.get_backend(self.group) == "nccl"
        width = max(int(self.rows.max()), 1)
        mine = int(self.rows[self.rank])
        xd = self.ops.vector(np.asarray(x, np.float64))
        for _ in range(int(it)):
            y, nsq = self.ops.spmv_sumsq(xd)
            s = nsq.clone() if on_device else nsq.to("cpu")
            dist.all_reduce(s, op=dist.ReduceOp.SUM, group=self.group)
            y = self.ops.normalize(y, s.to(nsq.device))
            comm = y.device if on_device else torch.device("cpu")
            blk = torch.zeros(width, dtype=torch.float64, device=comm)
            blk[:mine] = y[:mine].to(comm)
            outs = [torch.empty(width, dtype=torch.float64, device=comm) for _ in range(self.world)]
            dist.all_gather(outs, blk, group=self.group)
            xd = torch.cat([outs[p][:int(self.rows[p])] for p in range(self.world)]).to(nsq.device)
        return xd.cpu().numpy()
