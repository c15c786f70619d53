#!/usr/bin/env python
"""Benchmark of the tiled dense Cholesky task graph on the GB300 executor.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one step): solve A X = B to backward error ≤ 1e-14 per column with
A = G·Gᵀ/N + αI (N = 32768, tile 512, 45,760 tasks, α = 1e-4, seed 2) and 16
right-hand sides, through ttg_chol_posv: the mixed-precision tiled Cholesky
(BF16 trailing updates on the tensor cores — by default split into three BF16
terms per operand, six products, for FP32-level updates (--mixed-kind 2) —
FP32 TRSM, FP64 diagonal POTRF;
one persistent-kernel launch of the task graph captured from the Taskflow<K>
drop-in) followed by iterative refinement (classic steps x += M⁻¹r while
each gains 10×, then GMRES; every residual an FP64-accurate product on the
tensor cores).  The same step with split-FP16 updates (--mixed-kind 3: two
FP16 terms per operand, three products) is reported beside it.
Inputs (4.4 GB of FP64 lower tiles) are resident in HBM and larger than L2.
`value` is N³/3 / time to solution (effective Cholesky TFLOP/s); solves/s is
reported beside it.  `e2e` runs the same step through the C ABI with pinned
host buffers (tiles and B in, X out).  The plain FP64 device path on the same
input, the three conditionings α ∈ {1, 1e-4, 1e-8}, and the forward error of
the mixed solution against the FP64 one are reported in the same line.

With torchrun (N > 1 GPUs) every rank factorises its own matrix ("replicas
only": the path has no exchange step) and `value` sums the ranks' work over
the slowest rank's time.  `--impl reference` times the reference's algorithm
on the host cores instead (the oracle port: restated Taskflow/Threadpool with
OpenBLAS, one BLAS thread per task) on a bounded sample of the workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Cholesky TFLOP/s & solves/s, p50/p99: mixed+IR vs FP64 on GB300 at bwd err≤1e-14"


class ClockSampler:
    """nvidia-smi clock / throttle samples while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
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
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sms, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sms.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sms) if sms else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sms)}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl" if os.environ.get("TTG_BENCH_GLOO") is None else "gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(world, v):
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _tasks(nb):
    return nb + nb * (nb - 1) // 2 + (nb - 1) * nb * (nb + 1) // 6


def workload_config(args):
    """The workload both arms report (the same dict: same matrix, tiles,
    right-hand sides and conditioning)."""
    nb = args.n // args.block
    N = nb * args.block
    elems = nb * (nb + 1) // 2 * args.block ** 2
    return {"workload": "tiled Cholesky + solve of A X = B to backward error <= %g, A = G*G^T/N + alpha*I" % args.tol,
            "gpu_variant": "mixed precision: BF16 tensor-core updates (%s), FP32 TRSM, FP64 diagonal POTRF, GMRES-IR" % (
                {0: "plain BF16 first", 1: "FP32 updates", 2: "split into three BF16 terms",
                 3: "split into two FP16 terms"}[args.mixed_kind]),
            "mixed_kind": args.mixed_kind, "matrix_size": N, "block_size": args.block, "nrhs": args.nrhs,
            "alpha": args.alpha, "seed": args.seed, "priority_kind": args.kind, "tasks": _tasks(nb),
            "l2": "inputs larger than L2 (%.1f GB of FP64 tiles)" % (elems * 8 / 1e9)}


def cpu_factor_sample(tiles, args, steps, warmup):
    """The reference's algorithm on the host cores: the oracle port (the
    Taskflow/Threadpool_shared graph of 2d_cholesky at one rank, OpenBLAS with
    one BLAS thread per task, one worker per host core), FP64, on the given
    packed lower tiles of the workload's matrix.  A bounded sample: only the
    tasks of the first `args.cpu_panels` panel steps run (their exact flops
    are counted), timed from seeding to join like 2d_cholesky.cpp:612-619.
    Returns (TFLOP/s median, cores, blas, sample seconds median, sample
    flops, fraction of N^3/3)."""
    from oracle import oracle as orc
    orc.lib(use_blas=True)
    if orc.blas_name() == "loops":
        raise RuntimeError("the CPU sample needs the host OpenBLAS (oracle loaded without it)")
    cores = os.cpu_count() or 1
    nb = args.n // args.block
    N = nb * args.block
    rates, times = [], []
    for i in range(warmup + steps):
        r = orc.cholesky(block_size=args.block, num_blocks=nb, n_threads=cores, kind=args.kind, want_L=False, tiles=tiles,
                         panel_limit=args.cpu_panels)
        if r["info"] != 0 or r["errors"] != 0:
            raise RuntimeError("oracle factorisation sample failed (info %d)" % r["info"])
        if i >= warmup:
            rates.append(r["flops"] / r["time_s"] / 1e12)
            times.append(r["time_s"])
    return (statistics.median(rates), cores, r["blas"], statistics.median(times), r["flops"],
            r["flops"] / (N ** 3 / 3.0))


def _cpu_sample_text(args, cores, blas, frac, tail):
    nb = args.n // args.block
    return ("FP64 tiled Cholesky of the same matrix (N=%d, tile %d, alpha=%g, seed %d): the tasks of the first %d of %d "
            "panel steps (%.1f%% of N^3/3, where the task graph is widest), oracle port of 2d_cholesky at one rank "
            "(Taskflow/Threadpool_shared restated, OpenBLAS %s one thread per task), %d worker threads; the triangular "
            "solves (2*N^2*nrhs flops, <0.2%% of N^3/3) are not timed; %s" % (
                args.n, args.block, args.alpha, args.seed, args.cpu_panels, nb, 100 * frac, os.path.basename(blas),
                cores, tail))


def gram_tiles_host(args):
    """The workload's matrix as packed lower FP64 tiles in host memory.  Up to
    N = 4096 the host restatement of the generator makes it (G*G^T as an
    exact FP64 product of the integer G); above, the device generator does (G*G^T
    at N=32768 takes minutes on the host cores) and a few entries are checked
    against the host restatement's exact integer formula."""
    import ctypes
    import numpy as np
    from oracle import oracle as orc
    orc.lib(use_blas=True)  # the first load decides: the CPU samples use OpenBLAS
    nb = args.n // args.block
    N = nb * args.block
    b = args.block
    if N <= 4096:
        G = orc.qnormals(0, N * N, args.seed, 0).astype(np.float64).reshape(N, N, order="F")
        A = G @ G.T / (256.0 * N) + args.alpha * np.eye(N)
        return np.concatenate([A[i * b:(i + 1) * b, j * b:(j + 1) * b].reshape(-1, order="F")
                               for j in range(nb) for i in range(j, nb)])
    import torch
    import tasktorrent_gb300 as t
    ctx = t.Context(device=0, timeout_s=60.0)
    bs = np.full(nb, args.block, np.int32)
    elems = nb * (nb + 1) // 2 * args.block ** 2
    d = torch.empty(elems, dtype=torch.float64, device="cuda")
    t.check(t.lib().ttg_gen_gram_tiles(ctx.h, nb * args.block, bs.ctypes.data, nb, args.alpha, args.seed,
                                       ctypes.c_void_p(d.data_ptr()), None), "gram tiles")
    torch.cuda.synchronize()
    h = d.cpu().numpy()
    del d
    ctx.close()
    torch.cuda.empty_cache()
    # Spot check: entry (i, j) of A from the host generator's definition.
    rng = np.random.default_rng(0)
    for _ in range(4):
        i, j = sorted(rng.integers(0, N, 2).tolist(), reverse=True)
        ti, tj = i // b, j // b
        o = sum((nb - c) * b * b for c in range(tj)) + (ti - tj) * b * b + (i - ti * b) + (j - tj * b) * b
        v = orc.gram_entry(N, i, j, args.alpha, args.seed)
        if h[o] != v:
            raise RuntimeError("device input differs from the host generator at (%d, %d)" % (i, j))
    return h


def run_reference(args, world, rank):
    if rank != 0:
        return
    tiles = gram_tiles_host(args)
    v, cores, blas, t, flops, frac = cpu_factor_sample(tiles, args, args.steps, args.warmup)
    sample = _cpu_sample_text(args, cores, blas, frac, "median of %d steps after %d warm-up" % (args.steps, args.warmup))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic: the same seeded matrix as the GPU arm",
            "config": workload_config(args),
            "cpu_baseline": {"value": v, "unit": "TFLOP/s", "cores": cores, "kind": "port", "sample": sample,
                             "sample_flops": flops, "kind_note": "the reference's runtime cannot be built on the "
                             "measuring host (its sources are not shipped there); the oracle restates it"},
            "e2e": {"value": v, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_batched(ctx, args):
    """cfg4: many independent SPD systems (N log-uniform in [32, 2048], A_i from
    seed 3 + i, one right-hand side each) in one executor launch replayed as a
    CUDA graph; tile size and worker count from the autotuner; FP64 plain and
    FP32 factor + in-launch refinement."""
    import numpy as np
    import tasktorrent_gb300 as t
    rng = np.random.default_rng(3)
    sizes = np.exp(rng.uniform(np.log(32), np.log(2048), args.batch_n)).astype(np.int32)
    out = {"systems": int(args.batch_n), "sizes": "log-uniform [32, 2048] (numpy default_rng(3))",
           "flops_total": float(np.sum(sizes.astype(np.float64) ** 3) / 3.0)}
    for name, prec in (("fp64", t.PREC_F64), ("mixed", t.PREC_MIXED)):
        tile, workers, _ = t.batch_autotune(ctx, sizes, [64, 128, 256], [0, t.lib().ttg_workers(ctx.h) // 2],
                                            precision=prec, ir_steps=2, max_sample=300)
        b = t.Batch(ctx, sizes, tile, precision=prec, nrhs=1, ir_steps=2, seed=3, alpha=1.0)
        b.run()
        ms = []
        for _ in range(3):
            st, rep = b.run()
            if st != t.TTG_OK:
                raise RuntimeError("batch run failed: %s" % t.strerror(st))
            ms.append(rep.run.elapsed_ms)
        errs = b.backward_errors()
        best = min(ms)
        out[name] = {"tile": tile, "workers": workers, "ms_per_batch": ms, "systems_per_s": args.batch_n / (best * 1e-3),
                     "tflops": rep.flops / (best * 1e-3) / 1e12, "tasks": int(rep.tasks), "worst_bwd_err": float(errs.max()),
                     "ir_steps": 2 if prec == t.PREC_MIXED else 0}
        b.close()
        t.check(t.lib().ttg_set_workers(ctx.h, 0), "reset workers")
    out["speedup_mixed_vs_fp64"] = min(out["fp64"]["ms_per_batch"]) / min(out["mixed"]["ms_per_batch"])
    return out


def run_serving(args, local):
    """cfg5: a Poisson stream of factor-and-solve requests (N log-uniform in
    [64, 8192], A = G·Gᵀ/N + 1e-4·I, 30% follow-up right-hand sides on a
    resident factor) over executor lanes sharing the GPU (four for mixed, the
    best of 2, 4 and 8 measured; two for FP64, which saturates at ~92
    solves/s on two lanes and ~67 on four), admission by an
    180 GB HBM budget; p50/p99 latency and solves/s per arrival rate, mixed
    (FP32 factor, split-BF16 tensor-core updates for tiles of 128 and 256, and
    three rounds of FP64-residual refinement in the launch — a request above
    the tolerance solves again with twice the rounds) and plain FP64."""
    import tasktorrent_gb300 as t
    out = {"requests_per_rate": {"mixed": args.serve_n, "fp64": args.serve_n_fp64}, "n_range": [64, 8192], "alpha": 1e-4,
           "followup_frac": 0.3,
           "hbm_budget_gb": 180.0, "lanes": {"mixed": 4, "fp64": 2}, "mixed_ir_steps": 3}
    for name, prec in (("mixed", t.PREC_MIXED), ("fp64", t.PREC_F64)):
        rows = []
        for rate in args.serve_rates:
            n_req = args.serve_n if prec == t.PREC_MIXED else args.serve_n_fp64
            s = t.Serve(n_req, rate=rate, n_min=64, n_max=8192, alpha=1e-4, seed=2, followup_frac=0.3, precision=prec,
                        ir_steps=3, lanes=4 if prec == t.PREC_MIXED else 2, max_batch=16, hbm_budget_gb=180.0,
                        device=local)
            st, rep, _ = s.run()
            s.close()
            if st != t.TTG_OK:
                raise RuntimeError("serving failed: %s" % t.strerror(st))
            d = rep.as_dict()
            d["rate"] = rate
            rows.append(d)
        out[name] = rows
    return out


def run_small_configs(ctx, args, world):
    """The two smaller workloads, device and host side by side: tiled Cholesky
    N=2048 tile 128 (A = G*G^T/N + I, seed 0; FP64) and the 2D block GEMM DAG
    N=8192 block 512 (A, B iid U[-1,1], seed 1; FP64).  Device: executor
    kernel time, median of 5 after 1 warm-up.  Host: the oracle port on all
    cores (OpenBLAS, one thread per task), median of 5 after 1 warm-up."""
    import numpy as np
    import tasktorrent_gb300 as t
    from oracle import oracle as orc
    out = {}
    # Cholesky N=2048 tile 128.
    p = t.CholPlan(ctx, 128, 16, n_threads=16, kind=args.kind, matrix=1, alpha=1.0, seed=0)
    ms = []
    for i in range(6):
        st, rep = p.factor()
        if st != t.TTG_OK:
            raise RuntimeError("N=2048 factorisation failed: %s" % t.strerror(st))
        if i:
            ms.append(rep.elapsed_ms)
    L = p.factor_L()
    A = p.input_A()
    p.close()
    err = float(np.linalg.norm(L @ L.T - A) / np.linalg.norm(A))
    flops = 2048.0 ** 3 / 3
    out["cholesky_n2048_b128"] = {"gpu_ms": statistics.median(ms), "gpu_tflops": flops / statistics.median(ms) / 1e9,
                                  "rel_err_LLt": err, "tasks": 816}
    # 2D block GEMM N=8192 block 512.
    g = t.GemmPlan(ctx, 8192, 512, n_threads=16, inputs=1, seed=1)
    ms = []
    for i in range(6):
        st, rep = g.run()
        if st != t.TTG_OK:
            raise RuntimeError("N=8192 block GEMM failed: %s" % t.strerror(st))
        if i:
            ms.append(rep.elapsed_ms)
    host = world == 1 and not args.no_cpu_baseline
    C = g.C() if host else None
    g.close()
    gflops = 2 * 8192.0 ** 3
    out["gemm_n8192_b512"] = {"gpu_ms": statistics.median(ms), "gpu_tflops": gflops / statistics.median(ms) / 1e9,
                              "tasks": 4608}
    if host:
        orc.lib(use_blas=True)
        cores = os.cpu_count() or 1
        ts = []
        for i in range(6):
            r = orc.cholesky(block_size=128, num_blocks=16, n_threads=cores, kind=args.kind, matrix=1, alpha=1.0, seed=0,
                             want_L=(i == 5))
            if i:
                ts.append(r["time_s"])
        out["cholesky_n2048_b128"].update(
            {"cpu_ms": statistics.median(ts) * 1e3, "cpu_tflops": flops / statistics.median(ts) / 1e12, "cpu_cores": cores,
             "rel_diff_vs_oracle": float(np.linalg.norm(L - r["L"]) / np.linalg.norm(r["L"]))})
        ts = []
        for i in range(6):
            r = orc.gemm(8192, 512, n_threads=cores, inputs=1, seed=1, want_C=(i == 5))
            if i:
                ts.append(r["time_s"])
        out["gemm_n8192_b512"].update(
            {"cpu_ms": statistics.median(ts) * 1e3, "cpu_tflops": gflops / statistics.median(ts) / 1e12, "cpu_cores": cores,
             "rel_diff_vs_oracle": float(np.linalg.norm(C - r["C"]) / np.linalg.norm(r["C"]))})
        out["cpu_note"] = "oracle port (%s, one BLAS thread per task), median of 5 after 1 warm-up" % os.path.basename(r["blas"])
    return out


def run_ours(args, world, rank, local):
    import ctypes
    import numpy as np
    import torch
    import tasktorrent_gb300 as t
    torch.cuda.set_device(local)
    ctx = t.Context(device=local, timeout_s=120.0)
    nb = args.n // args.block
    N = nb * args.block
    nrhs = args.nrhs
    flops = N ** 3 / 3.0
    lib = t.lib()

    # Right-hand sides: iid N(0,1) from seed, on the device.
    B = torch.empty(nrhs, N, dtype=torch.float64, device="cuda")  # column-major N×nrhs
    X = torch.empty_like(B)
    t.check(lib.ttg_gen_normal(ctx.h, N * nrhs, args.seed + 100, 1, ctypes.c_void_p(B.data_ptr()), None), "rhs")
    torch.cuda.synchronize()

    def opts():
        return t.SolveOpts(nrhs, args.tol, 12, 30, 0, 0.0)

    def posv(plan):
        """One time-to-solution step through ttg_chol_posv on the resident
        input: restore the in-place input tiles (one device copy), factor,
        solve and refine.  Returns (ms, report)."""
        rep = t.SolveReport()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        st = lib.ttg_chol_posv(plan.h, ctypes.c_void_p(B.data_ptr()), ctypes.c_void_p(X.data_ptr()), ctypes.byref(opts()),
                               ctypes.byref(rep), None)
        e1.record()
        torch.cuda.synchronize()
        if st != t.TTG_OK:
            raise RuntimeError("posv failed: %s (%s)" % (t.strerror(st), rep.as_dict()))
        return e0.elapsed_time(e1), rep

    # Headline: mixed precision (BF16 tensor-core updates, split into three
    # BF16 terms by default) + GMRES-IR at alpha.
    plan = t.CholPlan(ctx, args.block, nb, n_threads=16, kind=args.kind, matrix=1, alpha=args.alpha,
                      seed=args.seed, precision=t.PREC_MIXED, mixed_kind=args.mixed_kind)
    n_tasks, capture_s = plan.tasks()
    for _ in range(args.warmup):
        posv(plan)
    barrier(world)
    times, reps, kernel_ms = [], [], []
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        launches0 = lib.ttg_kernel_launches()
        w0 = time.perf_counter()
        for _ in range(args.steps):
            ms, rep = posv(plan)
            times.append(ms)
            reps.append(rep)
            kernel_ms.append(rep.factor_ms)
        torch.cuda.synchronize()
        wall = time.perf_counter() - w0
        gpu_launches = int(lib.ttg_kernel_launches() - launches0)
    barrier(world)
    step_ms = allmax(world, statistics.mean(times))
    value = world * flops / (step_ms * 1e-3) / 1e12
    X_mixed = X.clone()

    # e2e through the C ABI: pinned host tiles of A and host B in, host X out.
    elems = plan.tile_elems()
    e2e = None
    if not args.no_e2e:
        hin = torch.empty(elems, dtype=torch.float64, pin_memory=True)
        hB = torch.empty(nrhs * N, dtype=torch.float64, pin_memory=True)
        hX = torch.empty(nrhs * N, dtype=torch.float64, pin_memory=True)
        plan.copy_tiles(1, hin.data_ptr())
        hB.copy_(B.reshape(-1).cpu())
        o = opts()
        rep = t.SolveReport()
        t.check(lib.ttg_chol_posv_host(plan.h, ctypes.c_void_p(hin.data_ptr()), ctypes.c_void_p(hB.data_ptr()),
                                       ctypes.c_void_p(hX.data_ptr()), ctypes.byref(o), ctypes.byref(rep), None), "e2e warm")
        barrier(world)
        ts = []
        # At least five timed calls: the host copy shares the host's memory
        # system with other work, and single calls have seen stalls.
        e2e_steps = max(args.steps, 5)
        phases = {k: [] for k in ("h2d_ms", "compute_ms", "factor_ms", "solve_ms", "d2h_ms", "total_ms")}
        for _ in range(e2e_steps):
            s0 = time.perf_counter()
            st = lib.ttg_chol_posv_host(plan.h, ctypes.c_void_p(hin.data_ptr()), ctypes.c_void_p(hB.data_ptr()),
                                        ctypes.c_void_p(hX.data_ptr()), ctypes.byref(o), ctypes.byref(rep), None)
            ts.append(time.perf_counter() - s0)
            if st != t.TTG_OK:
                raise RuntimeError("e2e failed: %s" % t.strerror(st))
            for k in phases:
                phases[k].append(getattr(rep, k))
        e2e_s = allmax(world, statistics.mean(ts))
        e2e = {"value": world * flops / e2e_s / 1e12, "unit": "TFLOP/s", "solves_per_s": world * nrhs / e2e_s,
               "h2d_bytes_per_step": elems * 8 + N * nrhs * 8, "d2h_bytes_per_step": N * nrhs * 8,
               "steps": e2e_steps, "ms_per_step": e2e_s * 1e3,
               "phases_ms": {k: statistics.mean(v) for k, v in phases.items()},
               "phases_note": "per call, mean: h2d (the input tiles streaming in on a copy stream while the "
                              "factorisation runs, events), compute (factor + solve + refinement, events), factor (executor "
                              "kernels), solve (host clock), d2h (X, events), total (host clock)"}
        if world == 1 and not args.no_cpu_baseline:
            host_tiles = hin.numpy().copy()
        del hin, hB, hX
    plan.close()

    # Roofline of the dominant kernel (the mixed executor: BF16 tensor-core
    # updates, FP32 TRSM, FP64 diagonal POTRF) against the measured dense BF16
    # tensor peak.
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except Exception:
        pass
    bf16_peak = peaks.get("bf16_tflops", 1900.0)
    kms = statistics.mean(kernel_ms)
    achieved = flops / (kms * 1e-3) / 1e12

    extra = {}
    if not args.quick:
        # The plain FP64 device path on the same input (time to solution).
        p64 = t.CholPlan(ctx, args.block, nb, n_threads=16, kind=args.kind, matrix=1, alpha=args.alpha, seed=args.seed + rank)
        posv(p64)
        ms64, rep64 = posv(p64)
        X64 = X.clone()
        fwd = float(torch.linalg.norm(X_mixed - X64) / torch.linalg.norm(X64))
        extra["fp64"] = {"ms_per_solve": ms64, "tflops": flops / (ms64 * 1e-3) / 1e12, "factor_ms": rep64.factor_ms,
                         "bwd_err": rep64.bwd_err, "fp64_peak_tflops": ctx.fp64_peak(200.0)}
        extra["speedup_mixed_vs_fp64"] = ms64 / step_ms
        extra["fwd_err_vs_fp64"] = fwd
        p64.close()
        # The three conditionings of the workload (one step each).
        # mixed_kind 0: plain BF16 first (remedies on loss of definiteness);
        # 2: split BF16 (FP32-level updates on the tensor cores); 3: split FP16.
        per_alpha = []
        for mk in (0, 2, 3):
            for a in (1.0, 1e-4, 1e-8):
                pa = t.CholPlan(ctx, args.block, nb, n_threads=16, kind=args.kind, matrix=1, alpha=a, seed=args.seed + rank,
                                precision=t.PREC_MIXED, mixed_kind=mk)
                posv(pa)
                msa, ra = posv(pa)
                per_alpha.append({"mixed_kind": mk, "alpha": a, "ms": msa, "factor_ms": ra.factor_ms, "outer": ra.outer,
                                  "inner": ra.inner, "gmres_prec": ra.gmres_prec, "remedy": ra.remedy, "bwd_err": ra.bwd_err})
                pa.close()
        extra["mixed_per_alpha"] = per_alpha
        # The same step with split-FP16 updates (two FP16 slices per operand,
        # three products; the split-BF16 factor replaces it when its first
        # refinement step gains less than 10x), timed like the headline.
        alt = 3 if args.mixed_kind != 3 else 2
        pf = t.CholPlan(ctx, args.block, nb, n_threads=16, kind=args.kind, matrix=1, alpha=args.alpha, seed=args.seed + rank,
                        precision=t.PREC_MIXED, mixed_kind=alt)
        for _ in range(args.warmup):
            posv(pf)
        fm, fr = [], None
        for _ in range(args.steps):
            msf, fr = posv(pf)
            fm.append(msf)
        pf.close()
        extra["mixed_kind_%d" % alt] = {"ms_per_step": statistics.mean(fm), "tflops": flops / (statistics.mean(fm) * 1e-3) / 1e12,
                                        "factor_ms": fr.factor_ms, "bwd_err": fr.bwd_err, "outer": fr.outer, "inner": fr.inner,
                                        "remedy": fr.remedy, "steps": args.steps}
    if not args.quick and not args.no_batched:
        extra["batched"] = run_batched(ctx, args)
    if not args.quick and not args.no_serving:
        extra["serving"] = run_serving(args, local)

    if not args.quick and not args.no_configs:
        extra["configs"] = run_small_configs(ctx, args, world)

    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        if args.no_e2e:
            host_tiles = gram_tiles_host(args)
        v, cores, blas, tcpu, sflops, frac = cpu_factor_sample(host_tiles, args, 2, 1)
        del host_tiles
        cpu = {"value": v, "unit": "TFLOP/s", "cores": cores, "kind": "port",
               "sample": _cpu_sample_text(args, cores, blas, frac, "median of 2 after 1 warm-up"), "sample_flops": sflops}

    if rank == 0:
        last = reps[-1]
        line = {"metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "bf16",
                "data": "synthetic: A = G*G^T/N + alpha*I, G quantised N(0,1) (Philox-4x32-10, seed %d); B iid N(0,1)" % args.seed,
                "config": workload_config(args), "tasks": n_tasks, "capture_s": capture_s, "wall_s_timed": wall,
                "solves_per_s": world * nrhs / (step_ms * 1e-3),
                "bwd_err": last.bwd_err, "refinement": {"outer": last.outer, "inner": last.inner, "gmres_prec": last.gmres_prec,
                                                          "remedy": last.remedy, "factor_ms": last.factor_ms},
                "roofline": {"bound": "tensor", "achieved": achieved, "peak": bf16_peak, "unit": "TFLOP/s",
                             "frac": achieved / bf16_peak,
                             # ncu capture of one N=16384 factorisation of this kernel: 15.28 GB of
                             # DRAM traffic, 13.63 GB of it growing with the update-task count
                             # (C tiles and operand slices) and 1.65 GB with N^2 (input conversion).
                             "traffic": 13.63e9 * ((nb - 1) * nb * (nb + 1) / 6) / 5456.0 + 1.65e9 * (N / 16384.0) ** 2,
                             "traffic_note": "DRAM bytes per factorisation launch: an N=16384 ncu capture (15.28 GB) "
                                             "scaled by the update-task count and N^2",
                             "kernel": "exec_kernel_mixed (launches of one factorisation, all remedy attempts); "
                                       "achieved = N^3/3 / their duration",
                             "peak_source": "measured: MEASURED_PEAKS.json bf16_tflops (burst)"},
                "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": gpu_launches, "clocks": clk.summary()}
        line.update(extra)
        print(json.dumps(line))
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=32768)
    ap.add_argument("--block", type=int, default=512)
    ap.add_argument("--alpha", type=float, default=1e-4)
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--kind", type=int, default=2)
    ap.add_argument("--mixed-kind", dest="mixed_kind", type=int, default=2,
                    help="0: BF16 updates (remedies on loss of definiteness); 2: split BF16; 3: split FP16; 1: FP32")
    ap.add_argument("--cpu-panels", dest="cpu_panels", type=int, default=2,
                    help="panel steps of the factorisation in the CPU samples")
    ap.add_argument("--no-configs", dest="no_configs", action="store_true",
                    help="skip the N=2048 Cholesky and N=8192 block-GEMM comparisons")
    ap.add_argument("--no-e2e", dest="no_e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", dest="no_cpu_baseline", action="store_true")
    ap.add_argument("--nrhs", type=int, default=16)
    ap.add_argument("--tol", type=float, default=1e-14)
    ap.add_argument("--quick", action="store_true", help="skip the FP64, per-alpha, batched and serving runs")
    ap.add_argument("--no-batched", dest="no_batched", action="store_true")
    ap.add_argument("--no-serving", dest="no_serving", action="store_true")
    ap.add_argument("--batch-n", dest="batch_n", type=int, default=10000)
    ap.add_argument("--serve-n", dest="serve_n", type=int, default=10000,
                    help="requests per arrival rate of the mixed serving stream")
    ap.add_argument("--serve-n-fp64", dest="serve_n_fp64", type=int, default=2000,
                    help="requests per arrival rate of the plain FP64 serving stream (saturates near 90 solves/s)")
    ap.add_argument("--serving-only", dest="serving_only", action="store_true",
                    help="run only the serving stream and print its section")
    ap.add_argument("--serve-rates", dest="serve_rates", type=lambda s: [float(x) for x in s.split(",")],
                    default=[100.0, 1000.0, 10000.0])
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    world, rank, local = dist_init()
    if args.serving_only:
        # The serving stream alone (e.g. --serve-n 10000): one JSON object.
        import torch
        torch.cuda.set_device(local)
        out = run_serving(args, local)
        if rank == 0:
            print(json.dumps({"serving": out}))
        return
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
