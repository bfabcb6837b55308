"""Benchmark: FP64 merge-path SpMV and power method on the 4096x4096-grid
2D Poisson matrix (N = 16,777,216, nnz = 83,869,696), GB300.

One step = one SpMV y = A x over the whole matrix (the plain FP64
merge-path SpMV, reported as GB/s against the HBM roofline).  Inputs are
larger than L2 (1.34 GB of matrix and vectors per pass), so no flush is
needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  N > 1 runs independent replicas, one per GPU
(the path does not shard on this single-GPU pool): value = all ranks' bytes /
max time over ranks.

--impl reference times the reference's CPU path (CRSOMP::mv and
CRS_Merge::mv restated in the C oracle, OpenMP over all host cores; the faster
is the value) on the same workload.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SpMV GB/s vs HBM peak; power-method solves/s, p50/p99 @1e-10, mixed vs FP64"
GRID = 4096
NOMINAL_HBM_GBS = 8000.0


def algorithmic_bytes(N, nnz, vbytes=8, xbytes=8):
    """12 B per nonzero (value + int32 column), int32 row_start, x read once,
    y written once."""
    return (vbytes + 4) * nnz + 4 * (N + 1) + xbytes * N + xbytes * N


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def profile_traffic():
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        try:
            with open(p) as f:
                return json.load(f)
        except Exception:
            return {}
    return {}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(n_gpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        import torch
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return world, rank, local


def max_over_ranks(v, world, device="cuda"):
    """The slowest rank's time (replicas: the job ends with its last rank)."""
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_gbs(bytes_per_rank, ms_max, world):
    """Whole-job throughput of N independent replicas: every rank's bytes over
    the slowest rank's time (weak scaling: each rank does a full SpMV)."""
    return bytes_per_rank * world / (ms_max * 1e-3) / 1e9


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def cpu_baseline_sample(A, x, threads, seconds=10.0, method="crsomp", max_reps=50):
    """One of the reference's CPU SpMVs (restated in the oracle) on the host
    cores: "crsomp" (CRSOMP::mv, OpenMP over rows, method 2), "crs_merge"
    (CRS_Merge::mv, one merge-path partition per thread, method 8) or "crs"
    (sequential CRS::mv, method 1, one core).  Returns (s per SpMV, reps)."""
    from oracle import pyoracle as O
    fn = {"crsomp": lambda: O.crs_omp_mv(A, x, threads), "crs_merge": lambda: O.merge_omp_mv(A, x, threads),
          "crs": lambda: O.crs_mv(A, x)}[method]
    fn()  # warm
    t0 = time.perf_counter()
    reps = 0
    while True:
        fn()
        reps += 1
        el = time.perf_counter() - t0
        if el > seconds or reps >= max_reps:
            break
    return el / reps, reps


def cpu_methods(A, x, threads, B, seconds):
    """GB/s of the reference's three CPU SpMVs (methods 1, 2, 8 of its
    selectType) on the same matrix and x."""
    out = {}
    for method, cores in (("crs", 1), ("crsomp", threads), ("crs_merge", threads)):
        s, reps = cpu_baseline_sample(A, x, threads, seconds=seconds, method=method,
                                      max_reps=10 if method == "crs" else 50)
        out[method] = {"gb_s": round(B / s / 1e9, 3), "ms": round(s * 1e3, 3), "cores": cores, "reps": reps}
    return out


def run_reference(args, world, rank):
    """--impl reference: the reference's CPU SpMV on the host cores -- its two
    parallel methods, CRSOMP::mv (method 2) and CRS_Merge::mv (method 8),
    restated in the oracle, each timed over --steps SpMVs; the value is the
    faster one (the sequential CRS::mv is reported beside them)."""
    if rank != 0:
        return
    from oracle import pyoracle as O
    threads = os.cpu_count() or 1
    A = O.fill_poisson(GRID, GRID)
    x = np.random.default_rng(20261203).random(A.noc)
    timed = {}
    for name, fn in (("crsomp", lambda: O.crs_omp_mv(A, x, threads)),
                     ("crs_merge", lambda: O.merge_omp_mv(A, x, threads))):
        for _ in range(max(args.warmup, 1)):
            fn()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            fn()
        timed[name] = (time.perf_counter() - t0) / args.steps * 1e3
    best = min(timed, key=timed.get)
    ms = timed[best]
    B = algorithmic_bytes(A.nor, A.nnz)
    gbs = B / (ms * 1e-3) / 1e9
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": round(gbs, 3), "unit": "GB/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "poisson2d_4096x4096_fp64_spmv", "N": A.nor, "nnz": A.nnz,
                   "l2": "inputs larger than L2"},
        "cpu_baseline": {"value": round(gbs, 3), "unit": "GB/s", "cores": threads, "kind": "port",
                         "methods": cpu_methods(A, x, threads, B, 2.0), "value_method": best,
                         "timed_ms": {k: round(v, 4) for k, v in timed.items()},
                         "sample": "%d full SpMVs per method (CRSOMP::mv, OpenMP dynamic,512, and CRS_Merge::mv, "
                                   "one merge-path partition per thread, restated in oracle/oracle.c); value = "
                                   "the faster" % args.steps},
        "e2e": {"value": round(gbs, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def coh_partitions(n, nnz, sm_count):
    """CO-H partition count (the reference's thread count) for the GPU: 24
    per SM.  The partitions split the rows by nonzero count as the
    reference's threads do; the tile kernel runs their Hilbert-ordered blocks
    window by window, so the count only moves partition boundaries (beta
    depends on the column count for square matrices); n and nnz are
    unused."""
    return 24 * sm_count


IRREGULAR = dict(n=4194304, seed=20261203, length_dist=0, mean_len=16.0, sigma=1.2, max_len=20000,
                 band_permille=300, band_half=4096)


def autotune_report(pwm, torch, stream, load, load_same_class, x, y, B):
    """The format autotuner (PWMGPU_FMT_AUTO, selectType method 15) on one
    matrix: the first load of its class times every candidate (merge launch
    variants, CSB lanes x threads variants, CO-H) and records the fastest;
    a second matrix of the same class takes the recorded choice.  Reports the
    choice, the candidates' ms per SpMV, the load + tuning wall time of both
    loads, and the SpMV through the tuned handle."""
    out = {}
    for tag, fn in (("first_of_class", load), ("same_class", load_same_class)):
        A = pwm.AutoCuda(1)
        A.set_stream(stream.cuda_stream)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn(A)
        wall = time.perf_counter() - t0
        t = A.tuning()
        rec = {"load_and_tune_s": round(wall, 3), "format": t["format"], "csb_variant": t["csb_variant"],
               "merge_variant": t["merge_variant"], "cache_hit": t["cache_hit"], "timed": t["timed"],
               "class_key": t["class_key"]}
        if t["timed"]:
            rec["candidates_ms"] = {"merge": round(t["merge_ms"], 5),
                                    **{"csb_v%d" % v: round(t["csb_ms"][v], 5) for v in range(4)},
                                    **{"coh_v%d" % v: round(t["coh_ms"][v], 5) for v in range(4)}}
        if tag == "first_of_class":
            for _ in range(3):
                A.mv_device(x.data_ptr(), y.data_ptr())
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(50):
                A.mv_device(x.data_ptr(), y.data_ptr())
            e1.record(stream)
            e1.synchronize()
            ms = e0.elapsed_time(e1) / 50
            rec["spmv_ms"] = round(ms, 5)
            rec["gb_s_crs_bytes"] = round(B / (ms * 1e-3) / 1e9, 2)
        out[tag] = rec
        del A
    return out


def poisson512(pwm, torch, dev, stream):
    """The 512 x 512-grid Poisson workload (N = 262,144, nnz = 1,308,672, the
    reference's CPU-runnable case): 100 timed SpMVs after 10 warm-ups and a
    100-iteration power method (reference powerIteration semantics).  Its
    21 MB of matrix and vectors stay in the 129 MB L2 between SpMVs, so the
    GB/s here are L2 figures, not HBM ones."""
    M = pwm.CRSCuda(1)
    M.set_stream(stream.cuda_stream)
    M.generatePoissonMatrix(512, 512, 1)
    N, _, nnz = M.dims()
    B = algorithmic_bytes(N, nnz)
    x = torch.rand(N, dtype=torch.float64, generator=torch.Generator().manual_seed(3)).to(dev)
    y = torch.zeros_like(x)
    for _ in range(10):
        M.mv_device(x.data_ptr(), y.data_ptr())
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(100):
        M.mv_device(x.data_ptr(), y.data_ptr())
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / 100
    px = x.clone()
    M.power_device(px.data_ptr(), y.data_ptr(), 10)
    px.copy_(x)
    e0.record(stream)
    M.power_device(px.data_ptr(), y.data_ptr(), 100)
    e1.record(stream)
    e1.synchronize()
    pms = e0.elapsed_time(e1)
    return {"workload": "poisson2d_512x512_fp64", "N": N, "nnz": nnz, "spmv_ms": round(ms, 5),
            "spmv_gb_s_l2_resident": round(B / (ms * 1e-3) / 1e9, 2),
            "power_100_iterations_ms": round(pms, 4), "power_ms_per_iteration": round(pms / 100, 5),
            "note": "21 MB of matrix and vectors: L2-resident between SpMVs"}


def irregular_and_solves(pwm, torch, dev, stream, args):
    """The irregular lognormal-row matrix (N = 4,194,304, generated on the
    device): FP64 SpMV GB/s, then power solves to 1e-10 relative
    eigen-residual in FP64 and in mixed precision (FP32 bulk + FP64
    refinement), each solve end to end through pwmgpu_solve (host vector in,
    eigenvector out): solves/s, p50/p99 latency."""
    M = pwm.CRSCuda(1)
    M.set_stream(stream.cuda_stream)
    M.generateRandom(**IRREGULAR)
    N, _, nnz = M.dims()
    B = algorithmic_bytes(N, nnz)
    x = torch.rand(N, dtype=torch.float64, generator=torch.Generator().manual_seed(5), device="cpu").to(dev)
    y = torch.zeros_like(x)
    for _ in range(5):
        M.mv_device(x.data_ptr(), y.data_ptr())
    steps = 200
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        M.mv_device(x.data_ptr(), y.data_ptr())
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / steps
    out = {"irregular": {"workload": "lognormal_rows_n4194304_mean16_sigma1.2_band30pct", "N": N, "nnz": nnz,
                         "spmv_ms": round(ms, 5), "spmv_gb_s": round(B / (ms * 1e-3) / 1e9, 2),
                         "spmv_gflop_s": round(2.0 * nnz / (ms * 1e-3) / 1e9, 2),
                         "frac_of_measured_hbm": round(B / (ms * 1e-3) / 1e9 / measured_peaks()[0], 4)}}
    # the same matrix in the CSB and CO-H formats (the reference's methods 9 and
    # 10): device SpMV time, GB/s on the CRS algorithmic bytes
    rs, ci, dv = M.getCSR()
    fm = {}
    for name, cls in (("csb", pwm.CSBCuda), ("coh", pwm.COHCuda)):
        F = cls(coh_partitions(N, nnz, torch.cuda.get_device_properties(dev).multi_processor_count))
        F.set_stream(stream.cuda_stream)
        F.loadCSR(N, N, rs, ci, dv)
        for _ in range(3):
            F.mv_device(x.data_ptr(), y.data_ptr())
        e0.record(stream)
        for _ in range(50):
            F.mv_device(x.data_ptr(), y.data_ptr())
        e1.record(stream)
        e1.synchronize()
        fms = e0.elapsed_time(e1) / 50
        fm[name] = {"spmv_ms": round(fms, 5), "gb_s_crs_bytes": round(B / (fms * 1e-3) / 1e9, 2)}
        if name == "csb":
            fm[name]["variant"] = F.csb_variant()
        del F
    out["irregular"]["formats"] = fm
    out["irregular"]["stats"] = M.stats()
    out["irregular"]["autotuner"] = autotune_report(
        pwm, torch, stream, lambda A: A.generateRandom(**IRREGULAR),
        lambda A: A.generateRandom(**dict(IRREGULAR, seed=IRREGULAR["seed"] + 1)), x, y, B)
    x0 = np.random.default_rng(20261203).random(N)
    solves = {}
    lam = {}
    for name, prec in (("fp64", pwm.PREC_F64), ("mixed", pwm.PREC_MIXED)):
        u = x0.copy()
        M.solve(u, 2000, 1e-10, prec)  # warm (value copies, buffers)
        lat = []
        info = None
        for _ in range(args.solves):
            u = x0.copy()
            t0 = time.perf_counter()
            info = M.solve(u, 2000, 1e-10, prec)
            lat.append(time.perf_counter() - t0)
        lat = np.array(lat) * 1e3
        lam[name] = info.lambda_
        solves[name] = {"solves_per_s": round(1e3 / lat.mean(), 3), "p50_ms": round(float(np.percentile(lat, 50)), 3),
                        "p99_ms": round(float(np.percentile(lat, 99)), 3), "iterations": info.iterations,
                        "iterations_low_precision": info.iterations_low, "converged": bool(info.converged),
                        "residual": info.residual, "lambda": info.lambda_}
    solves["mixed"]["lambda_rel_diff_vs_fp64"] = abs(lam["mixed"] - lam["fp64"]) / abs(lam["fp64"])
    solves["speedup_mixed_vs_fp64"] = round(solves["mixed"]["solves_per_s"] / solves["fp64"]["solves_per_s"], 3)
    out["solve_irregular_1e-10"] = solves
    return out


def _batch_specs(rng, count=128):
    """The 256-matrix batch: 128 Poisson grids with side uniform in
    [32, 1024] and 128 random matrices with N log-uniform in [1e3, 1e6],
    Poisson(8) row lengths, uniform columns, values in (0, 1]."""
    specs = []
    for i in range(count):
        side = int(rng.integers(32, 1025))
        specs.append(("poisson", dict(m=side, n=side)))
    for i in range(count):
        n = int(round(10 ** rng.uniform(3, 6)))
        specs.append(("random", dict(n=n, seed=1000 + i, length_dist=1, mean_len=8.0, sigma=0.0, max_len=64,
                                     band_permille=0, band_half=0)))
    return specs


def _stream_specs(rng, count):
    """Serving stream requests: N log-uniform in [1e4, 4e6]; half Poisson
    grids (side = round(sqrt(N))), half lognormal-row random matrices."""
    specs = []
    for i in range(count):
        n = int(round(10 ** rng.uniform(4, math.log10(4e6))))
        if i % 2 == 0:
            side = max(2, int(round(math.sqrt(n))))
            specs.append(("poisson", dict(m=side, n=side)))
        else:
            specs.append(("random", dict(n=n, seed=5000 + i, length_dist=0, mean_len=16.0, sigma=1.2,
                                         max_len=20000, band_permille=300, band_half=4096)))
    return specs


def _submit(svc, kind, kw, precision, max_it, tol, keep=False):
    if kind == "poisson":
        return svc.submit_poisson(kw["m"], kw["n"], max_it=max_it, tol=tol, precision=precision, x0_seed=11,
                                  keep_vector=keep)
    return svc.submit_random(max_it=max_it, tol=tol, precision=precision, x0_seed=11, keep_vector=keep, **kw)


def seeded_uniform(n, seed):
    """The service's seeded start vector (x0_seed): x[i] = (mix(seed +
    g (i + 1)) >> 11) 2^-53 with the splitmix64 finaliser, in numpy."""
    z = np.uint64(seed) + np.uint64(0x9e3779b97f4a7c15) * np.arange(1, n + 1, dtype=np.uint64)
    z ^= z >> np.uint64(30)
    z *= np.uint64(0xbf58476d1ce4e5b9)
    z ^= z >> np.uint64(27)
    z *= np.uint64(0x94d049bb133111eb)
    z ^= z >> np.uint64(31)
    return (z >> np.uint64(11)).astype(np.float64) * 2.0 ** -53


def _one_at_a_time(pwm, kind, kw, max_it, tol):
    """The plain FP64 merge-path path on one request: a fresh handle, the
    matrix built on the device, pwmgpu_solve.  Returns (SolveInfo,
    eigenvector)."""
    M = pwm.CRSCuda(1)
    if kind == "poisson":
        M.generatePoissonMatrix(kw["m"], kw["n"], 1)
    else:
        M.generateRandom(**kw)
    x = seeded_uniform(M.dims()[0], 11)  # the service's start vector for x0_seed = 11
    return M.solve(x, max_it, tol, pwm.PREC_F64), x


def _oracle_matrix(kind, kw):
    from oracle import pyoracle as O
    if kind == "poisson":
        return O.fill_poisson(kw["m"], kw["n"])
    return O.random_crs(kw["n"], kw["seed"], kw["length_dist"], kw["mean_len"], kw["sigma"], kw["max_len"],
                        kw["band_permille"], kw["band_half"])


def _oracle_checks(rows):
    """The FP64 oracle's check of returned eigenpairs: for each (kind, kw,
    lambda, residual, converged, u) the oracle's Rayleigh quotient of u
    (CRS::mv and sequential FP64 dots) gives lambda_o and the relative
    eigen-residual res_o.  Reports the largest |lambda - lambda_o| /
    |lambda_o|, the largest res_o over converged solves (the stopping target
    is 1e-10), and the largest gap |res - res_o| between the residual the
    GPU reported and the oracle's (both are FP64 sums of rounded terms, so a
    residual near 1e-13 agrees to a few digits only)."""
    from oracle import pyoracle as O
    lam_err, res_conv, res_gap, n_conv = 0.0, 0.0, 0.0, 0
    for kind, kw, lam, res, conv, u in rows:
        lo, ro = O.rayleigh(_oracle_matrix(kind, kw), u)
        lam_err = max(lam_err, abs(lam - lo) / abs(lo))
        res_gap = max(res_gap, abs(res - ro))
        if conv:
            n_conv += 1
            res_conv = max(res_conv, ro)
    return {"checked": len(rows), "checked_converged": n_conv, "max_lambda_rel_err_vs_oracle": lam_err,
            "max_residual_vs_oracle_converged": res_conv if n_conv else None,
            "max_residual_abs_diff_gpu_vs_oracle": res_gap}


def _check_set(specs, per_class=3, max_n=400000):
    """Indices of the requests whose eigenpairs the oracle checks: the first
    `per_class` Poisson grids and random matrices with at most max_n rows."""
    out, seen = [], {"poisson": 0, "random": 0}
    for i, (k, kw) in enumerate(specs):
        n = kw["m"] * kw["n"] if k == "poisson" else kw["n"]
        if n <= max_n and seen[k] < per_class:
            out.append(i)
            seen[k] += 1
    return set(out)


def _class_counts(specs, conv, iters, max_it, low=None):
    """Per matrix class: requests, converged to the tolerance, stopped at the
    iteration cap, and (mixed precision) the share of steps run in FP32 /
    BF16 -- the service's precision tuner's choice for the class."""
    out = {}
    for cls in ("poisson", "random"):
        idx = [i for i, (k, _) in enumerate(specs) if k == cls]
        out[cls] = {"requests": len(idx), "converged": int(sum(bool(conv[i]) for i in idx)),
                    "capped_at_max_it": int(sum((not conv[i]) and iters[i] >= max_it for i in idx))}
        if low is not None:
            steps = sum(iters[i] for i in idx)
            out[cls]["low_precision_step_share"] = round(sum(low[i] for i in idx) / max(steps, 1), 4)
            out[cls]["solves_kept_in_fp64"] = int(sum(low[i] == 0 for i in idx))
    return out


def _stream_run(submit_fn, arrivals, step_fn, idle_fn):
    """Drive arrivals on the wall clock; returns per-request latency (s)."""
    t0 = time.perf_counter()
    i = 0
    while True:
        now = time.perf_counter() - t0
        while i < len(arrivals) and arrivals[i] <= now:
            submit_fn(i, t0)
            i += 1
        busy = step_fn()
        if not busy:
            if i >= len(arrivals):
                break
            wait = arrivals[i] - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(min(wait, 0.01))
    return idle_fn(t0)


def _service_batch(pwm, S, specs, prec, max_it, tol, check):
    """All requests submitted at once to a fresh service, run until idle."""
    svc = S.Service(hbm_budget_bytes=150 << 30, round_iterations=8)
    t0 = time.perf_counter()
    ids = [_submit(svc, k, kw, prec, max_it, tol, keep=i in check) for i, (k, kw) in enumerate(specs)]
    svc.run_until_idle()
    el = time.perf_counter() - t0
    res = [svc.result(i) for i in ids]
    vecs = {i: svc.result(ids[i], want_vector=True)[1] for i in check}
    st = svc.stats()
    svc.close()
    return el, res, vecs, st


def serving(pwm, args):
    """Batch (256 uneven matrices) and serving-stream workloads: the batched
    service in mixed precision and in FP64 (one launch per power step for all
    live solves, graph-captured rounds) against the plain FP64 merge-path
    path solving one request at a time (pwmgpu_solve per matrix).  Every
    figure is split by matrix class (Poisson grids, random matrices); solves
    that reach the 1e-10 residual are counted apart from solves stopped at the
    2,000-step cap; a seeded subset of the returned eigenpairs is checked by
    the FP64 oracle's Rayleigh quotient (outside the timed runs)."""
    from thesis_spmv_gb300 import service as S
    tol, max_it = 1e-10, 2000
    out = {}

    # ---- the 256-matrix batch, all submitted at once ----
    specs = _batch_specs(np.random.default_rng(20261203), args.batch_count)
    check = _check_set(specs)
    batch = {}
    arms = (("service_mixed", pwm.PREC_MIXED), ("service_fp64", pwm.PREC_F64))
    if args.batch_only:
        arms = ((("service_mixed", pwm.PREC_MIXED),) if args.batch_precision == "mixed"
                else (("service_fp64", pwm.PREC_F64),))
    lam = {}
    for name, prec in arms:
        el, res, vecs, st = _service_batch(pwm, S, specs, prec, max_it, tol, check)
        conv = [r.converged for r in res]
        rec = {"seconds": round(el, 3), "solves_per_s": round(len(res) / el, 2),
               "converged": int(sum(conv)), "converged_solves_per_s": round(sum(conv) / el, 2),
               "capped_at_max_it": int(sum((not r.converged) and r.iterations >= max_it for r in res)),
               "steps_total": int(sum(r.iterations for r in res)),
               "steps_low_precision": int(sum(r.iterations_low for r in res)),
               "max_reported_residual_converged": max([r.residual for r in res if r.converged], default=None),
               "rounds": int(st.rounds), "gpu_round_ms": round(st.gpu_round_ms, 1),
               "by_class": _class_counts(specs, conv, [r.iterations for r in res], max_it,
                                         [r.iterations_low for r in res])}
        if not args.batch_only:
            rec["oracle_check"] = _oracle_checks([(specs[i][0], specs[i][1], res[i].lambda_, res[i].residual,
                                                   res[i].converged, vecs[i]) for i in sorted(check)])
        lam[name] = [r.lambda_ for r in res]
        batch[name] = rec
    if args.batch_only:
        return {"batch_256": batch}
    # the plain FP64 path, one request at a time (sequential: each class's
    # solves/s is its requests over the time its own solves took)
    t_req, one, vecs = [], [], {}
    t0 = time.perf_counter()
    for i, (k, kw) in enumerate(specs):
        ts = time.perf_counter()
        info, u = _one_at_a_time(pwm, k, kw, max_it, tol)
        t_req.append(time.perf_counter() - ts)
        one.append(info)
        if i in check:
            vecs[i] = u
    el = time.perf_counter() - t0
    conv = [r.converged for r in one]
    batch["one_at_a_time_fp64"] = {
        "seconds": round(el, 3), "solves_per_s": round(len(specs) / el, 2), "converged": int(sum(conv)),
        "converged_solves_per_s": round(sum(conv) / el, 2),
        "capped_at_max_it": int(sum((not r.converged) and r.iterations >= max_it for r in one)),
        "steps_total": int(sum(r.iterations for r in one)),
        "by_class": _class_counts(specs, conv, [r.iterations for r in one], max_it),
        "oracle_check": _oracle_checks([(specs[i][0], specs[i][1], one[i].lambda_, one[i].residual,
                                         one[i].converged, vecs[i]) for i in sorted(check)])}
    diffs = [abs(a - b) / abs(b) for a, b in zip(lam["service_mixed"], lam["service_fp64"])]
    batch["lambda_rel_diff_mixed_vs_fp64"] = {"max": max(diffs), "median": float(np.median(diffs))}
    batch["speedup_service_mixed_vs_one_at_a_time_fp64"] = round(
        batch["service_mixed"]["solves_per_s"] / batch["one_at_a_time_fp64"]["solves_per_s"], 3)
    # per class: each class alone through the service arms; the one-at-a-time
    # time of a class is the sum of its own solves' times
    per_class = {}
    for cls in ("poisson", "random"):
        sub = [(k, kw) for k, kw in specs if k == cls]
        row = {}
        for name, prec in arms:
            el, res, _, _ = _service_batch(pwm, S, sub, prec, max_it, tol, set())
            row[name] = {"solves_per_s": round(len(sub) / el, 2),
                         "converged": int(sum(r.converged for r in res)),
                         "converged_solves_per_s": round(sum(r.converged for r in res) / el, 2)}
        t_cls = sum(t for t, (k, _) in zip(t_req, specs) if k == cls)
        n_conv = sum(bool(r.converged) for r, (k, _) in zip(one, specs) if k == cls)
        row["one_at_a_time_fp64"] = {"solves_per_s": round(len(sub) / t_cls, 2), "converged": n_conv,
                                     "converged_solves_per_s": round(n_conv / t_cls, 2)}
        row["speedup_service_mixed_vs_one_at_a_time_fp64"] = round(
            row["service_mixed"]["solves_per_s"] / row["one_at_a_time_fp64"]["solves_per_s"], 3)
        row["speedup_service_mixed_vs_service_fp64"] = round(
            row["service_mixed"]["solves_per_s"] / row["service_fp64"]["solves_per_s"], 3)
        row["target_2x_vs_one_at_a_time_fp64_met"] = row["speedup_service_mixed_vs_one_at_a_time_fp64"] >= 2.0
        per_class[cls] = row
    batch["per_class"] = per_class
    out["batch_256"] = dict(workload="128 Poisson grids (side U[32,1024]) + 128 random (N log-uniform [1e3,1e6], "
                                     "Poisson(8) rows); tol 1e-10 or 2000 steps", **batch)

    # ---- serving stream: Poisson arrivals at a few rates ----
    stream = {}
    R = args.stream_requests
    specs = _stream_specs(np.random.default_rng(7), R)
    check = _check_set(specs, per_class=2, max_n=300000)
    kinds = np.array([k for k, _ in specs])

    def lat_stats(lat, conv, span):
        rec = {"p50_ms": round(float(np.percentile(lat, 50)) * 1e3, 2),
               "p99_ms": round(float(np.percentile(lat, 99)) * 1e3, 2),
               "solves_per_s": round(R / span, 2), "converged": int(np.sum(conv)),
               "converged_solves_per_s": round(float(np.sum(conv)) / span, 2)}
        for cls in ("poisson", "random"):
            sel = kinds == cls
            rec[cls] = {"p50_ms": round(float(np.percentile(lat[sel], 50)) * 1e3, 2),
                        "p99_ms": round(float(np.percentile(lat[sel], 99)) * 1e3, 2),
                        "requests": int(sel.sum()), "converged": int(np.sum(conv[sel]))}
        return rec

    for rate in args.stream_rates:
        arr = np.cumsum(np.random.default_rng(int(rate)).exponential(1.0 / rate, R))
        arr -= arr[0]
        row = {}
        for name, prec in (("service_mixed", pwm.PREC_MIXED), ("service_fp64", pwm.PREC_F64)):
            svc = S.Service(hbm_budget_bytes=150 << 30, round_iterations=8)
            t_create = time.perf_counter()
            ids = {}

            def submit_fn(i, t0, svc=svc, ids=ids, prec=prec):
                k, kw = specs[i]
                ids[i] = _submit(svc, k, kw, prec, max_it, tol, keep=i in check)

            def step_fn(svc=svc):
                live, queued, _ = svc.step()
                return live > 0 or queued > 0

            def idle_fn(t0, svc=svc, ids=ids, arr=arr, t_create=t_create):
                lat = np.zeros(R)
                for i, rid in ids.items():
                    r = svc.result(rid)
                    lat[i] = r.t_done + (t_create - t0) - arr[i]
                return lat

            lat = _stream_run(submit_fn, arr, step_fn, idle_fn)
            res = [svc.result(ids[i]) for i in range(R)]
            rec = lat_stats(lat, np.array([r.converged for r in res], bool), max(float(np.max(lat + arr)), 1e-9))
            st = svc.stats()
            rec["rounds"] = int(st.rounds)
            rec["gpu_round_ms"] = round(st.gpu_round_ms, 1)
            rec["oracle_check"] = _oracle_checks([(specs[i][0], specs[i][1], res[i].lambda_, res[i].residual,
                                                   res[i].converged, svc.result(ids[i], want_vector=True)[1])
                                                  for i in sorted(check)])
            row[name] = rec
            svc.close()
        # plain FP64 path, one request at a time in arrival order
        done_t, one, vecs = [], [], {}
        t0 = time.perf_counter()
        for i, (k, kw) in enumerate(specs):
            now = time.perf_counter() - t0
            if arr[i] > now:
                time.sleep(arr[i] - now)
            info, u = _one_at_a_time(pwm, k, kw, max_it, tol)
            done_t.append(time.perf_counter() - t0)
            one.append(info)
            if i in check:
                vecs[i] = u
        lat = np.array(done_t) - arr
        rec = lat_stats(lat, np.array([r.converged for r in one], bool), max(done_t[-1], 1e-9))
        rec["oracle_check"] = _oracle_checks([(specs[i][0], specs[i][1], one[i].lambda_, one[i].residual,
                                               one[i].converged, vecs[i]) for i in sorted(check)])
        row["one_at_a_time_fp64"] = rec
        row["speedup_service_mixed_vs_one_at_a_time_fp64"] = round(
            row["service_mixed"]["solves_per_s"] / row["one_at_a_time_fp64"]["solves_per_s"], 3)
        stream["rate_%g_per_s" % rate] = row
    out["serving_stream"] = dict(workload="%d requests per rate, N log-uniform [1e4, 4e6], half Poisson grids, half "
                                          "lognormal-row random; Poisson arrivals; tol 1e-10 or 2000 steps; HBM "
                                          "budget 150 GB" % R, **stream)
    return out


def triplet_load(pwm, torch, dev, M, N, cpu=True):
    """Triplet -> CRS on the device (pwmgpu_load_triplets_device) for the
    entries of the matrix M holds in a seeded shuffled order; the result must
    be M's CRS bit for bit.  CPU leg: the oracle's TripletToCRS restatement
    (one thread) on a shuffled 1024 x 1024 Poisson triplet."""
    rs, ci, v = M.getCSR()
    nnz = ci.size
    counts = torch.from_numpy(np.diff(rs).astype(np.int64)).to(dev)
    rows = torch.repeat_interleave(torch.arange(N, dtype=torch.int32, device=dev), counts)
    g = torch.Generator(device=dev).manual_seed(11)
    perm = torch.randperm(nnz, device=dev, generator=g)
    dr = rows[perm].contiguous()
    dc = torch.from_numpy(ci).to(dev)[perm].contiguous()
    dv = torch.from_numpy(v).to(dev)[perm].contiguous()
    del rows, perm, counts
    T = pwm.CRSCuda(1)
    times = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        T.loadFromDeviceTriplets(N, N, nnz, dr.data_ptr(), dc.data_ptr(), dv.data_ptr())
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    trs, tci, tv = T.getCSR()
    same = bool(np.array_equal(trs, rs) and np.array_equal(tci, ci) and np.array_equal(tv, v))
    ms = 1e3 * sorted(times)[1]
    out = {"workload": "%d shuffled triplets of the Poisson matrix above" % nnz,
           "api": "pwmgpu_load_triplets_device (includes the merge-path plan build)",
           "ms": round(ms, 3), "entries_per_s": round(nnz / (ms * 1e-3), 1), "same_crs_as_generated": same}
    del dr, dc, dv, T
    if cpu:
        from oracle import pyoracle as O
        r0, c0, v0 = O.triplet_poisson(1024, 1024)
        p = np.random.default_rng(11).permutation(r0.size)
        r0, c0, v0 = r0[p].copy(), c0[p].copy(), v0[p].copy()
        t0 = time.perf_counter()
        O.triplet_to_crs(1024 * 1024, 1024 * 1024, r0, c0, v0)
        cs = time.perf_counter() - t0
        out["cpu_baseline"] = {"entries_per_s": round(r0.size / cs, 1), "cores": 1, "kind": "port",
                               "sample": "%d shuffled triplets of the 1024x1024 Poisson matrix "
                                         "(TripletToCRS restated in oracle/oracle.c)" % r0.size}
    return out


def run_case(args):
    """--case: one kernel on one matrix, for profiling (a small launch count
    before the timed ones): the irregular lognormal-row matrix with
    --case-n rows or the Poisson grid --grid, in the format --case-format
    (merge, csb, coh with 24 partitions per SM, or "power": --steps
    iterations of the power method in one pwmgpu_power_device call, AUTO
    mode).  Prints ms per SpMV / iteration and GB/s of CRS algorithmic
    bytes."""
    import torch
    import thesis_spmv_gb300 as pwm
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    sm = torch.cuda.get_device_properties(dev).multi_processor_count
    fmt = args.case_format
    cls = {"merge": pwm.CRSCuda, "power": pwm.CRSCuda, "csb": pwm.CSBCuda, "coh": pwm.COHCuda}[fmt]
    M = cls(coh_partitions(0, 0, sm) if fmt == "coh" else 1)
    stream = torch.cuda.Stream(device=dev)
    M.set_stream(stream.cuda_stream)
    if args.case == "irregular":
        M.generateRandom(**dict(IRREGULAR, n=args.case_n))
        workload = "lognormal_rows_n%d_mean16_sigma1.2_band30pct" % args.case_n
    else:
        M.generatePoissonMatrix(args.grid, args.grid, 1)
        workload = "poisson2d_%dx%d" % (args.grid, args.grid)
    N, _, nnz = M.dims()
    B = algorithmic_bytes(N, nnz)
    x = torch.rand(N, dtype=torch.float64, generator=torch.Generator().manual_seed(5)).to(dev)
    y = torch.zeros_like(x)

    if fmt == "power":
        M.power_device(x.data_ptr(), y.data_ptr(), max(args.warmup, 1))
    else:
        for _ in range(args.warmup):
            M.mv_device(x.data_ptr(), y.data_ptr())
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    if fmt == "power":
        M.power_device(x.data_ptr(), y.data_ptr(), args.steps)
    else:
        for _ in range(args.steps):
            M.mv_device(x.data_ptr(), y.data_ptr())
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    print(json.dumps({"case": args.case, "format": fmt, "workload": workload, "N": N, "nnz": nnz,
                      "ms_per_launch": round(ms, 5), "gb_s_crs_bytes": round(B / (ms * 1e-3) / 1e9, 2)}))


def run_ours(args, world, rank, local):
    import torch
    import thesis_spmv_gb300 as pwm

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    if args.batch_only:
        print(json.dumps(serving(pwm, args)))
        return
    grid_side = args.grid
    M = pwm.CRSCuda(1)
    M.generatePoissonMatrix(grid_side, grid_side, 1)
    N, _, nnz = M.dims()
    B = algorithmic_bytes(N, nnz)
    tm, ntiles, grid = M.tile_info()

    stream = torch.cuda.Stream(device=dev)
    M.set_stream(stream.cuda_stream)
    g = torch.Generator(device="cpu").manual_seed(20261203)
    x_host = torch.rand(N, dtype=torch.float64, generator=g)
    dx = x_host.to(dev)
    dy = torch.zeros(N, dtype=torch.float64, device=dev)

    # ---- device-resident SpMV (value) ----
    for _ in range(args.warmup):
        M.mv_device(dx.data_ptr(), dy.data_ptr())
    stream.synchronize()
    barrier(world)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            M.mv_device(dx.data_ptr(), dy.data_ptr())
        ev1.record(stream)
        ev1.synchronize()
        torch.cuda.synchronize()
    ms_total = ev0.elapsed_time(ev1)
    barrier(world)
    ms_total = max_over_ranks(ms_total, world)
    ms = ms_total / args.steps
    value = replica_gbs(B, ms, world)

    # ---- the same Poisson matrix in the CSB and CO-H formats ----
    formats = {}
    if not args.no_extra:
        for name, cls in (("csb", pwm.CSBCuda), ("coh", pwm.COHCuda)):
            F = cls(coh_partitions(N, nnz, torch.cuda.get_device_properties(dev).multi_processor_count))
            F.set_stream(stream.cuda_stream)
            F.generatePoissonMatrix(grid_side, grid_side, 1)
            for _ in range(3):
                F.mv_device(dx.data_ptr(), dy.data_ptr())
            f0 = torch.cuda.Event(enable_timing=True)
            f1 = torch.cuda.Event(enable_timing=True)
            f0.record(stream)
            for _ in range(50):
                F.mv_device(dx.data_ptr(), dy.data_ptr())
            f1.record(stream)
            f1.synchronize()
            fms = f0.elapsed_time(f1) / 50
            formats[name] = {"spmv_ms": round(fms, 5), "gb_s_crs_bytes": round(B / (fms * 1e-3) / 1e9, 2)}
            if name == "csb":
                formats[name]["variant"] = F.csb_variant()
            del F
        # the autotuner on this class: the 4096^2 grid, then a 4200 x 4096 grid
        formats["autotuner"] = autotune_report(
            pwm, torch, stream, lambda A: A.generatePoissonMatrix(grid_side, grid_side, 1),
            lambda A: A.generatePoissonMatrix(grid_side + 104, grid_side, 1), dx, dy, B)
        formats_load = triplet_load(pwm, torch, dev, M, N, cpu=rank == 0 and world == 1 and not args.no_cpu)

    # ---- power method: 500 iterations (reference powerIteration semantics),
    #      fused persistent kernel and two kernels per iteration ----
    p_it = args.power_iters
    px = dx.clone()
    py = torch.zeros_like(dx)
    power_ms = {}
    for mode, name in ((pwm.POWER_FUSED, "fused"), (pwm.POWER_MULTI, "multi")):
        M.set_power_mode(mode)
        M.power_device(px.data_ptr(), py.data_ptr(), 4)
        stream.synchronize()
        px.copy_(dx)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        M.power_device(px.data_ptr(), py.data_ptr(), p_it)
        e1.record(stream)
        e1.synchronize()
        power_ms[name] = e0.elapsed_time(e1)
    M.set_power_mode(pwm.POWER_AUTO)

    # ---- end to end through the C ABI with host buffers (pinned) ----
    e2e_s = float("nan")
    e2e_steps = 0 if args.no_e2e else max(3, min(args.steps, 50))
    if e2e_steps:
        xh = x_host.pin_memory()
        yh = torch.zeros(N, dtype=torch.float64).pin_memory()
        xn = xh.numpy()
        yn_ = yh.numpy()
        M.mv(xn, yn_)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            M.mv(xn, yn_)  # H2D x, SpMV, D2H y, synchronous
        e2e_s = (time.perf_counter() - t0) / e2e_steps
        # the same call on pageable arrays (what the reference's drivers pass:
        # new[] buffers)
        xq = x_host.numpy().copy()
        yq = np.zeros(N)
        M.mv(xq, yq)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            M.mv(xq, yq)
        e2e_pageable_s = (time.perf_counter() - t0) / e2e_steps
    e2e_gbs = B * world / e2e_s / 1e9 if e2e_steps else None

    extra = None if args.no_extra else irregular_and_solves(pwm, torch, dev, stream, args)
    if extra is not None:
        extra["poisson512"] = poisson512(pwm, torch, dev, stream)
    if not args.no_serving and rank == 0:
        extra = dict(extra or {}, **serving(pwm, args))

    peak, peak_kind = measured_peaks()
    traffic = profile_traffic().get("k_merge_spmv_f64_poisson4096")
    result = {
        "metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 5), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "poisson2d_%dx%d_fp64_spmv" % (grid_side, grid_side), "N": N, "nnz": nnz,
                   "l2": "inputs larger than L2 (1.34 GB per pass)", "items_per_tile": tm, "tiles": ntiles,
                   "grid": grid, "launch_variant": dict(zip(("prefer_l1", "grid", "power_grid", "tuned_ms"),
                                                            M.launch_config()),
                                                        column_bytes=M.plan_info()[0],
                                                        gathers_bypass_l1=M.plan_info()[1]),
                   "parallelism": "replicas" if world > 1 else "single"},
        "roofline": {"bound": "hbm", "achieved": round(B / (ms * 1e-3) / 1e9, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(B / (ms * 1e-3) / 1e9 / peak, 4), "traffic": traffic,
                     "peak_source": peak_kind, "frac_of_nominal_8TBs": round(B / (ms * 1e-3) / 1e9 / NOMINAL_HBM_GBS, 4),
                     "algorithmic_bytes_per_launch": B, "timed": "k_merge_spmv + k_fix_runs (one SpMV)"},
        "gflop_s": round(2.0 * nnz * world / (ms * 1e-3) / 1e9, 2),
        "e2e": ({"value": round(e2e_gbs, 3), "unit": "GB/s", "h2d_bytes_per_step": 8 * N,
                 "d2h_bytes_per_step": 8 * N, "ms_per_step": round(e2e_s * 1e3, 4),
                 "api": "pwmgpu_mv (host arrays, pinned)",
                 "pageable": {"ms_per_step": round(e2e_pageable_s * 1e3, 4),
                              "gb_s": round(B * world / e2e_pageable_s / 1e9, 3)}} if e2e_steps else None),
        "gpu_launches": 2 * args.steps,
        "power": {"iterations": p_it,
                  "fused": {"ms_per_iteration": round(power_ms["fused"] / p_it, 5),
                            "gb_s": round(B / (power_ms["fused"] / p_it * 1e-3) / 1e9, 2),
                            "kernels": "k_power_persistent (1 launch for all iterations; SpMV pass, barrier, "
                                       "fix-up pass, barrier per iteration)"},
                  "multi": {"ms_per_iteration": round(power_ms["multi"] / p_it, 5),
                            "gb_s": round(B / (power_ms["multi"] / p_it * 1e-3) / 1e9, 2),
                            "kernels": "k_merge_spmv + k_fix_runs per iteration (the rescale from the "
                                       "largest magnitude key; the last two iterations sum ||y||^2 in the "
                                       "same two kernels)"}},
        "clocks": clk.summary(),
    }
    if formats:
        result["formats_poisson"] = formats
        result["triplet_to_crs"] = formats_load
        result["poisson_stats"] = M.stats()
    if extra:
        result.update(extra)
    if rank == 0 and world == 1 and not args.no_cpu:
        from oracle import pyoracle as O
        A = O.fill_poisson(grid_side, grid_side)
        threads = os.cpu_count() or 1
        meth = cpu_methods(A, x_host.numpy(), threads, B, 3.0)
        best = max(("crsomp", "crs_merge"), key=lambda k: meth[k]["gb_s"])
        result["cpu_baseline"] = {"value": meth[best]["gb_s"], "unit": "GB/s", "cores": threads, "kind": "port",
                                  "sample": "%d full SpMVs of the same matrix (%s restated in oracle/oracle.c)"
                                            % (meth[best]["reps"], {"crsomp": "CRSOMP::mv",
                                                                    "crs_merge": "CRS_Merge::mv"}[best]),
                                  "methods": meth,
                                  "note": "methods: the reference's sequential CRS (1), CRSOMP (2) and CRS_Merge (8) "
                                          "restated in oracle/oracle.c; value = the faster parallel one"}
    if rank == 0:
        print(json.dumps(result))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--power-iters", type=int, default=500)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer end-to-end leg")
    ap.add_argument("--grid", type=int, default=GRID, help="Poisson grid side (default 4096)")
    ap.add_argument("--no-extra", action="store_true", help="skip the irregular matrix and the solves")
    ap.add_argument("--solves", type=int, default=20, help="timed solves per precision")
    ap.add_argument("--no-serving", action="store_true", help="skip the batch and serving-stream workloads")
    ap.add_argument("--batch-count", type=int, default=128,
                    help="Poisson grids and random matrices in the batch (128 each)")
    ap.add_argument("--batch-only", action="store_true",
                    help="only the 256-matrix batch through the service (a profiling case)")
    ap.add_argument("--batch-precision", choices=["fp64", "mixed"], default="fp64",
                    help="the service precision of --batch-only")
    ap.add_argument("--stream-requests", type=int, default=300)
    ap.add_argument("--stream-rates", type=float, nargs="+", default=[50.0, 100.0, 200.0, 500.0, 1000.0, 2000.0])
    ap.add_argument("--case", choices=["irregular", "poisson"],
                    help="profiling case: one kernel on one matrix (see run_case)")
    ap.add_argument("--case-n", type=int, default=1 << 21, help="rows of the irregular matrix of --case irregular")
    ap.add_argument("--case-format", default="merge", choices=["merge", "csb", "coh", "power"])
    args = ap.parse_args()
    if args.case:
        run_case(args)
        return
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        world = int(os.environ.get("WORLD_SIZE", "1"))
        rank = int(os.environ.get("RANK", "0"))
        run_reference(args, world, rank)
        return
    world, rank, local = dist_setup(args.gpus)
    run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
