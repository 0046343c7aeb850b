"""Benchmark: time to a 1e-10 relative residual on the 512^3 Poisson problem.

Workload (one step): a complete mixed-precision solve -- FP32 V(2,2)-cycles inside FP64
defect correction, RBGS smoother (omega 1.0), 8 levels down to 2^3, stop at
sqrt(|r|^2/|r0|^2) < 1e-10 -- of the seeded 512^3 Gaussian-blob problem (sum of 8
Gaussians, sigma 0.05, plus 1e-3 uniform noise, PCG64(3)) from x0 = 0.  Inputs are
resident in HBM for `value`; `e2e` is the same solve through the C-ABI with pinned
host buffers (host<->device copies inside the timed region).  The plain FP64 path
(bitwise the reference arithmetic) is timed once for the mixed/FP64 ratio.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

With N > 1 (torchrun) every rank solves its own replica (the solve does not shard on
one node: replicas only).  `--impl reference` times the CPU restatement of the
reference (oracle/, OpenMP over all host cores) on the same workload and prints the
same JSON line with "impl": "reference".
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_DEFAULT = 512
LEVELS = {512: 8, 384: 7, 256: 7, 128: 6, 96: 5, 64: 4}
TOL = 1e-10
MAXIT = 2
OMEGA = 1.0
METRIC = "time_to_1e-10_rel_residual_512cubed_mixed"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=N_DEFAULT)
    p.add_argument("--inner", type=int, default=4, help="FP32 V-cycles per FP64 correction (4 is fastest at 512^3)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--quick", action="store_true",
                   help="time the mixed solve only (no FP64 comparison, e2e or CPU baseline); for profiling")
    p.add_argument("--precision", default="mixed", choices=["mixed", "fp64"],
                   help="with --quick: the precision of the timed solve")
    p.add_argument("--workload", default="solve", choices=["solve", "batch"],
                   help="batch: the 128-problem batched solve (sizes from {32..192}, PCG64(4)); prints "
                        "its own JSON line (cells per second)")
    p.add_argument("--batch", type=int, default=128, help="problems of --workload batch")
    return p.parse_args()


def max_over_ranks(value, world, device):
    """The job's time: the maximum of a per-rank value over all ranks (replicas)."""
    if world <= 1:
        return value
    import torch
    t = torch.tensor([value], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(cells_per_rank, ms, world):
    """Whole-job cells per second of `world` replicas that each solved `cells_per_rank`
    cells in (the slowest rank's) `ms` milliseconds."""
    return cells_per_rank * world / (ms * 1e-3)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        """Starts sampling every 20 ms and returns once the first sample has arrived (at most
        5 s), so the samples cover the timed region that follows."""
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.time()
            while not self.lines and time.time() - t0 < 5.0 and self.proc.poll() is None:
                time.sleep(0.01)
            self.first = len(self.lines)
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def ncu_traffic():
    """Per-launch DRAM bytes of the profiled kernel classes, from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return {}


def cpu_baseline(mesh, rhs, n_levels, cycles_needed, threads, sample_cycles=1):
    """Time the oracle (CPU restatement of the reference, OpenMP) on a bounded sample of
    the same workload: `sample_cycles` FP64 V-cycles after the initial residual; the
    time to solution is extrapolated to the cycle count the FP64 solve needs."""
    from oracle import oracle as O
    O.set_threads(threads)
    n = len(mesh[0][0]) - 2
    t0 = time.perf_counter()
    omg = O.OracleMG(mesh, n_levels, sample_cycles, 0, 0, 0, omp=True)
    t_setup = time.perf_counter() - t0
    sol, rsd = O.field(n, n, n), O.field(n, n, n)
    t0 = time.perf_counter()
    omg.solve(sol, rsd, rhs, MAXIT, TOL, OMEGA)
    t_sample = time.perf_counter() - t0
    omg.close()
    per_cycle = t_sample / sample_cycles
    return {"value": per_cycle * cycles_needed * 1e3, "unit": "ms", "cores": threads, "kind": "port",
            "sample": "%d FP64 V(2,2) cycle(s) of the %d^3 solve (%.2f s, setup %.1f s excluded) x %d cycles "
                      "to 1e-10" % (sample_cycles, n, t_sample, t_setup, cycles_needed)}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    from peps_mg_gb300 import problems
    n = args.n
    mesh, rhs = problems.gaussian_blobs(n)
    rhs = np.asfortranarray(rhs)
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    t0 = time.perf_counter()
    omg = O.OracleMG(mesh, LEVELS[n], 1, 0, 0, 0, omp=True)
    setup = time.perf_counter() - t0
    # cycles to convergence of the reference algorithm: one full FP64 solve (untimed)
    full = O.OracleMG(mesh, LEVELS[n], 100, 0, 0, 0, omp=True)
    sol, rsd = O.field(n, n, n), O.field(n, n, n)
    t0 = time.perf_counter()
    cycles, hist, _ = full.solve(sol, rsd, rhs, MAXIT, TOL, OMEGA)
    t_full = time.perf_counter() - t0
    full.close()
    per = []
    for s in range(args.warmup + args.steps):
        sol[...] = 0.0
        t0 = time.perf_counter()
        omg.solve(sol, rsd, rhs, MAXIT, TOL, OMEGA)        # one V-cycle after the initial residual
        dt = time.perf_counter() - t0
        if s >= args.warmup:
            per.append(dt)
    value = statistics.mean(per) * cycles * 1e3
    line = {"metric": METRIC, "value": round(value, 3), "unit": "ms", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(value, 3), "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Gaussian blobs, PCG64(3))",
            "impl": "reference",
            "config": {"workload": "512^3 Poisson, FP64 V(2,2) RBGS cycles of the reference algorithm to 1e-10",
                       "n": n, "levels": LEVELS[n], "cycles_to_tolerance": int(cycles),
                       "full_solve_s": round(t_full, 3), "setup_s": round(setup, 3)},
            "cpu_baseline": {"value": round(value, 3), "unit": "ms", "cores": threads, "kind": "port",
                             "sample": "one FP64 V-cycle per step x %d cycles to 1e-10 (a full solve took %.2f s)"
                                       % (cycles, t_full)},
            "e2e": {"value": round(value, 3), "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    import peps_mg_gb300 as pmg
    from peps_mg_gb300 import problems

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", torch.cuda.current_device())
    n = args.n
    nl = LEVELS[n]
    mesh, rhs = problems.gaussian_blobs(n)
    rhs = np.asfortranarray(rhs)
    d_rhs = torch.from_numpy(rhs.T.copy()).to(dev)
    d_sol = torch.zeros_like(d_rhs)
    d_rsd = torch.zeros_like(d_rhs)
    stream = torch.cuda.current_stream(dev)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
            torch.cuda.synchronize()

    prec = args.precision if args.quick else "mixed"
    mg = pmg.Multigrid(mesh, nl, 100, "cgs", precision=prec, mixed_inner_cycles=args.inner,
                       stream=stream.cuda_stream)

    def step():
        d_sol.zero_()
        return mg.solve_vcycle(d_sol, d_rsd, d_rhs, MAXIT, TOL, OMEGA)

    for _ in range(max(args.warmup, 3)):
        rep = step()
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    l0 = pmg.launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.nvtx.range_push("timed")
    e0.record(stream)
    reps = [step() for _ in range(args.steps)]
    e1.record(stream)
    torch.cuda.nvtx.range_pop()
    barrier()
    launches = pmg.launch_count() - l0
    ms = e0.elapsed_time(e1) / args.steps
    clk = clocks.stop()
    # per-kernel-class breakdown from separate solves with the library's event profiler on
    # (its events are not inside the timed region)
    mg.profile(True)
    for _ in range(args.steps):
        step()
    prof = {pmg.PROF_CLASSES[c]: mg.profile_read(c) for c in pmg.PROF_CLASSES}
    mg.profile(False)
    ms = max_over_ranks(ms, world, dev)
    rep = reps[-1]
    assert rep.converged and rep.final_ratio < TOL, "solve did not converge"

    if args.quick:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": round(ms, 3), "unit": "ms", "quick": True, "n": n,
                              "precision": prec, "cycles": rep.cycles,
                              "ratios": [float(v) for v in rep.history[:, 2]],
                              "coarse_iterations": [int(v) for v in rep.coarse_iterations],
                              "kernels": {k: v for k, v in prof.items() if v[1]}, "gpu_launches": launches}))
        mg.destroy()
        return

    # error of the mixed solution against the plain FP64 solution
    mg64 = pmg.Multigrid(mesh, nl, 100, "cgs", precision="fp64", stream=stream.cuda_stream)
    s64 = torch.zeros_like(d_rhs)
    r64 = torch.zeros_like(d_rhs)
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    barrier()
    f0.record(stream)
    rep64 = mg64.solve_vcycle(s64, r64, d_rhs, MAXIT, TOL, OMEGA)
    f1.record(stream)
    barrier()
    fp64_ms = f0.elapsed_time(f1)
    diff = (d_sol - s64).abs().max().item()
    scale = s64.abs().max().item()
    l2 = ((d_sol - s64).norm() / s64.norm()).item()
    mg64.destroy()
    del s64, r64

    # end to end through the C-ABI with pinned host buffers (copies inside the timed region)
    h_rhs = torch.from_numpy(rhs.T.copy()).pin_memory()
    h_sol = torch.zeros_like(h_rhs).pin_memory()
    h_rsd = torch.zeros_like(h_rhs).pin_memory()
    a_rhs, a_sol, a_rsd = h_rhs.numpy(), h_sol.numpy(), h_rsd.numpy()
    mg.solve_vcycle(a_sol, a_rsd, a_rhs, MAXIT, TOL, OMEGA)
    barrier()
    e2e, e2e_stream = [], []
    for _ in range(args.steps):
        a_sol[...] = 0.0
        t0 = time.perf_counter()
        rep_e = mg.solve_vcycle(a_sol, a_rsd, a_rhs, MAXIT, TOL, OMEGA)
        e2e.append((time.perf_counter() - t0) * 1e3)
        e2e_stream.append(rep_e.elapsed_ms)
    e2e_ms = statistics.mean(e2e)
    nbytes = a_rhs.nbytes

    # roofline of the dominant kernel class
    peak, peak_kind = measured_peaks()
    dom = max((k for k in prof if prof[k][2] > 0), key=lambda k: prof[k][0])
    t_tot, n_l, b_l = prof[dom]
    achieved = b_l / (t_tot / n_l * 1e-3) / 1e9
    traffic = ncu_traffic().get(dom)
    cells = float(n) ** 3
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            cpu = cpu_baseline(mesh, rhs, nl, rep64.cycles, os.cpu_count() or 1)
        except Exception as exc:  # report, do not hide
            cpu = {"value": None, "error": str(exc)}
    if rank == 0:
        line = {
            "metric": METRIC, "value": round(ms, 3), "unit": "ms", "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": round(ms, 3), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic (seeded Gaussian blobs, PCG64(3))",
            "config": {"workload": "512^3 Poisson, mixed FP32 V(2,2) in FP64 defect correction to 1e-10 "
                                   "(replicas only across GPUs)",
                       "n": n, "levels": nl, "inner_cycles_per_correction": args.inner,
                       "outer_corrections": rep.cycles, "fp32_vcycles": rep.inner_cycles,
                       "l2": "inputs larger than L2 (8.7 GB of FP64/FP32 arrays per solve)",
                       "fp64_ms": round(fp64_ms, 3), "fp64_cycles": rep64.cycles,
                       "speedup_mixed_vs_fp64": round(fp64_ms / ms, 3),
                       "mixed_vs_fp64_max_abs_err_rel": diff / scale, "mixed_vs_fp64_l2_rel": l2},
            "roofline": {"kernel": dom, "bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4),
                         "traffic": traffic},
            "kernels": {k: {"ms_total": round(v[0], 3), "launches": v[1],
                            "gbs": round(v[2] / (v[0] / v[1] * 1e-3) / 1e9, 1) if v[1] and v[0] > 0 and v[2] > 0
                            else None} for k, v in prof.items() if v[1]},
            "cpu_baseline": cpu,
            "e2e": {"value": round(e2e_ms, 3), "unit": "ms", "h2d_bytes_per_step": 2 * nbytes,
                    "d2h_bytes_per_step": 2 * nbytes,
                    "stream_ms": round(statistics.mean(e2e_stream), 3)},
            "gpu_launches": launches,
            "clocks": clk,
            "cells_per_s": round(replica_throughput(cells, ms, world), 1),
        }
        print(json.dumps(line), flush=True)
    mg.destroy()
    if world > 1:
        torch.distributed.destroy_process_group()


def run_batch(args):
    """The batched configuration: one solve of every problem to 1e-10 (mixed precision,
    depth-synchronous persistent launches, graph-captured corrections), timed with CUDA
    events on the batch's stream; value = interior cells of all problems / solve time."""
    import torch
    from peps_mg_gb300 import problems
    from peps_mg_gb300.batch import BatchSolver

    rank, world, local = dist_env()
    if world > 1:
        torch.cuda.set_device(local)
    dims = problems.batch_dims(args.batch)
    with BatchSolver(dims, mixed_inner_cycles=args.inner) as bs:
        rhs = bs.field()
        for p, vals in enumerate(problems.batch_rhs(dims)):
            bs.view(rhs, p)[1:-1, 1:-1, 1:-1] = torch.from_numpy(vals).cuda()
        sol = bs.field()
        for _ in range(max(args.warmup, 3)):
            sol.zero_()
            cycles, ratio, _ = bs.solve(sol, rhs, MAXIT, TOL, OMEGA, max_cycles=100)
        times = []
        torch.cuda.nvtx.range_push("timed")
        for _ in range(args.steps):
            sol.zero_()
            torch.cuda.synchronize()
            cycles, ratio, ms = bs.solve(sol, rhs, MAXIT, TOL, OMEGA, max_cycles=100)
            times.append(ms)
        torch.cuda.nvtx.range_pop()
        assert np.all(ratio < TOL), "batched solve did not converge"
        cells = int(np.prod(dims, axis=1).sum())
        ms = statistics.mean(times)
        if rank == 0:
            print(json.dumps({"metric": "batched_solve_cells_per_s", "value": round(cells / (ms * 1e-3), 1),
                              "unit": "cells/s", "ms_per_step": round(ms, 3), "steps": args.steps,
                              "higher_is_better": True, "dtype": "f32+f64", "data": "synthetic (U[-1,1], PCG64)",
                              "config": {"workload": "%d independent problems, axis sizes from {32..192} "
                                                     "(PCG64(4)), mixed precision to 1e-10" % args.batch,
                                         "problems": args.batch, "cells": cells,
                                         "inner_cycles_per_correction": args.inner,
                                         "corrections_max": int(cycles.max()),
                                         "corrections_mean": round(float(cycles.mean()), 2)}}))


def main():
    args = parse()
    if args.workload == "batch":
        run_batch(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
