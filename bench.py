"""Benchmark: time to a 1e-10 relative residual on the 512^3 Poisson problem.

Workload (one step): a complete mixed-precision solve -- FP32 V(2,2)-cycles inside FP64
defect correction, RBGS smoother (omega 1.0), 8 levels down to 2^3, stop at
sqrt(|r|^2/|r0|^2) < 1e-10 -- of the seeded 512^3 Gaussian-blob problem (sum of 8
Gaussians, sigma 0.05, plus 1e-3 uniform noise, PCG64(3)) from x0 = 0.  Inputs are
resident in HBM for `value`; `e2e` is the same solve through the C-ABI with pinned
host buffers (host<->device copies inside the timed region; `e2e.pageable_ms` with
ordinary pageable arrays, `e2e.cold_ms` adding create, the first solve's autotuning and
destroy, the parts the reference's own timer spans).  The plain FP64 path (bitwise the
reference arithmetic) is timed as the mean of three warm solves for the mixed/FP64
ratio.  `cpu_baseline` is one complete FP64 solve by the oracle on all host cores; its
solution is the one the GPU solutions are compared with (`config.*_vs_oracle_*`).
`batch` adds the 128-problem batched workload (a few timed solves).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

With N > 1 (torchrun) every rank solves its own replica (the solve does not shard on
one node: replicas only).  `--impl reference` times the CPU restatement of the
reference (oracle/, OpenMP over all host cores) on the same workload, one complete
solve per step, and prints the same JSON line with "impl": "reference".
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


def metric_for(n, prec="mixed"):
    """The metric's name for an n^3 problem (METRIC at the default size)."""
    return "time_to_1e-10_rel_residual_%dcubed_%s" % (n, prec)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=N_DEFAULT)
    p.add_argument("--inner", type=int, default=4, help="FP32 V-cycles per FP64 correction (4 is fastest at 512^3)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-batch", action="store_true", help="leave the batched workload out of the bench line")
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


def cpu_model():
    """The host CPU's model name and the number of cores this process may use."""
    name = None
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                if ln.lower().startswith(("model name", "cpu model")):
                    name = ln.split(":", 1)[1].strip()
                    break
    except OSError:
        pass
    if name is None:
        try:
            out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
            for ln in out.splitlines():
                if ln.startswith("Model name:"):
                    name = ln.split(":", 1)[1].strip()
                    break
        except (OSError, subprocess.SubprocessError):
            pass
    return name or "unknown", os.cpu_count() or 1


def oracle_solve(mesh, rhs, n_levels, threads):
    """One complete FP64 solve by the oracle (CPU restatement of the reference, OpenMP over
    `threads` host threads), timed the way the reference times it (src/main_peps.f90:167-183:
    multigrid_create, multigrid_solve_vcycle and multigrid_destroy inside the timer) from
    x0 = 0.  Returns (seconds, solution, cycles, history)."""
    from oracle import oracle as O
    O.set_threads(threads)
    n = len(mesh[0][0]) - 2
    sol, rsd = O.field(n, n, n), O.field(n, n, n)
    t0 = time.perf_counter()
    omg = O.OracleMG(mesh, n_levels, 100, 0, 0, 0, omp=True)
    cycles, hist, _ = omg.solve(sol, rsd, rhs, MAXIT, TOL, OMEGA)
    omg.close()
    dt = time.perf_counter() - t0
    return dt, sol, int(cycles), hist


def cpu_baseline(mesh, rhs, n_levels):
    """The oracle timed on one complete solve of the same workload (about 10 s on 16 Grace
    cores at 512^3): no extrapolation.  Also returns the oracle's solution, against which the
    GPU solutions are compared."""
    name, cores = cpu_model()
    dt, sol, cycles, _ = oracle_solve(mesh, rhs, n_levels, cores)
    n = len(mesh[0][0]) - 2
    return {"value": round(dt * 1e3, 3), "unit": "ms", "cores": cores, "cpu": name, "kind": "port",
            "sample": "one complete FP64 solve of the %d^3 problem to 1e-10 from x0 = 0 (%d V(2,2) cycles; "
                      "create + solve + destroy timed, as src/main_peps.f90:167-183 times it)" % (n, cycles)}, sol


def run_reference(args):
    """The reference's CPU path (its restatement, oracle/) on the same workload: every step
    (warm-up and timed) is one complete FP64 solve to 1e-10 from x0 = 0, timed from
    multigrid_create to multigrid_destroy; value = the mean over the timed steps."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from peps_mg_gb300 import problems
    n = args.n
    mesh, rhs = problems.gaussian_blobs(n)
    rhs = np.asfortranarray(rhs)
    name, threads = cpu_model()
    per, cycles = [], None
    for s in range(args.warmup + args.steps):
        dt, _, cycles, _ = oracle_solve(mesh, rhs, LEVELS[n], threads)
        if s >= args.warmup:
            per.append(dt)
    value = statistics.mean(per) * 1e3
    line = {"metric": metric_for(n), "value": round(value, 3), "unit": "ms", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(value, 3), "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Gaussian blobs, PCG64(3))",
            "impl": "reference",
            "config": {"workload": "%d^3 Poisson, FP64 V(2,2) RBGS cycles of the reference algorithm to 1e-10" % n,
                       "n": n, "levels": LEVELS[n], "cycles_to_tolerance": cycles,
                       "step_s_min": round(min(per), 3), "step_s_max": round(max(per), 3)},
            "cpu_baseline": {"value": round(value, 3), "unit": "ms", "cores": threads, "cpu": name, "kind": "port",
                             "sample": "one complete FP64 solve per step (%d cycles; create + solve + destroy "
                                       "timed), %d timed steps after %d warm-up steps"
                                       % (cycles, args.steps, args.warmup)},
            "e2e": {"value": round(value, 3), "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def batch_algorithmic_bytes(levels_per_problem, dims, corrections, inner):
    """Algorithmic bytes of one batched solve, counted like the single-grid profiler counts
    them (each array once per launch, FP32 V-cycle work on the grid levels of every problem):
    per FP32 V(2,2)-cycle and grid level, four smoother iterations at 12 B/cell (8 B/cell for
    an iteration from e = 0: the first of each coarse level and of a correction's first cycle
    on the finest level), the fused residual-restriction and the prolongation at 8.5 B/cell
    each; per correction, the FP64 x += e with the residual update (40 B/cell) or the FP64
    residual (28 B/cell), here counted as the update; plus the first residual (28 B/cell)."""
    total = 0.0
    for p, nl in enumerate(levels_per_problem):
        n = [int(v) for v in dims[p]]
        cells0 = float(n[0] * n[1] * n[2])
        per_cycle_first = per_cycle = 0.0
        sizes = [n]
        for _ in range(int(nl)):
            sizes.append([(v // 2 if v % 2 == 0 else v) for v in sizes[-1]])
        for l, s in enumerate(sizes[:-1]):
            c = float(s[0] * s[1] * s[2])
            if c <= 4096:
                break
            first_it = 8.0
            smooth_first = (first_it + 12.0 + 24.0) * c
            smooth_later = ((12.0 if l == 0 else 8.0) + 12.0 + 24.0) * c
            xfer = 17.0 * c
            per_cycle_first += smooth_first + xfer
            per_cycle += smooth_later + xfer
        per_corr = per_cycle_first + (inner - 1) * per_cycle + 40.0 * cells0
        total += 28.0 * cells0 + corrections[p] * per_corr
    return total


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
    # set-up cost, first context of the process: multigrid_create, the first solve (it
    # autotunes the smoother per level and captures the V-cycle graphs) and, at the end,
    # multigrid_destroy -- the parts of the reference's timed region outside the solve
    barrier()
    t0 = time.perf_counter()
    mg = pmg.Multigrid(mesh, nl, 100, "cgs", precision=prec, mixed_inner_cycles=args.inner,
                       stream=stream.cuda_stream)
    torch.cuda.synchronize()
    create_ms = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    mg.solve_vcycle(d_sol, d_rsd, d_rhs, MAXIT, TOL, OMEGA)
    torch.cuda.synchronize()
    first_solve_ms = (time.perf_counter() - t0) * 1e3

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
    peak, peak_kind = measured_peaks()

    def kernel_table(p, solves):
        out = {}
        for k, v in p.items():
            if not v[1]:
                continue
            gbs = v[2] / (v[0] / v[1] * 1e-3) / 1e9 if v[0] > 0 and v[2] > 0 else None
            out[k] = {"ms_total": round(v[0], 3), "launches": v[1], "ms_per_solve": round(v[0] / solves, 3),
                      "gbs": round(gbs, 1) if gbs else None, "frac": round(gbs / peak, 4) if gbs else None}
        return out

    if args.quick:
        if rank == 0:
            print(json.dumps({"metric": metric_for(n, prec), "value": round(ms, 3), "unit": "ms", "quick": True, "n": n,
                              "precision": prec, "cycles": rep.cycles,
                              "ratios": [float(v) for v in rep.history[:, 2]],
                              "coarse_iterations": [int(v) for v in rep.coarse_iterations],
                              "kernels": kernel_table(prof, args.steps), "gpu_launches": launches,
                              "setup": {"create_ms": round(create_ms, 1), "first_solve_ms": round(first_solve_ms, 1)}}))
        mg.destroy()
        return

    # the plain FP64 path (bitwise the reference's arithmetic): one warm-up solve, then the
    # mean of three
    mg64 = pmg.Multigrid(mesh, nl, 100, "cgs", precision="fp64", stream=stream.cuda_stream)
    s64 = torch.zeros_like(d_rhs)
    r64 = torch.zeros_like(d_rhs)
    mg64.solve_vcycle(s64, r64, d_rhs, MAXIT, TOL, OMEGA)
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    fp64_steps = 3
    barrier()
    f0.record(stream)
    for _ in range(fp64_steps):
        s64.zero_()
        rep64 = mg64.solve_vcycle(s64, r64, d_rhs, MAXIT, TOL, OMEGA)
    f1.record(stream)
    barrier()
    fp64_ms = f0.elapsed_time(f1) / fp64_steps
    mg64.profile(True)
    s64.zero_()
    mg64.solve_vcycle(s64, r64, d_rhs, MAXIT, TOL, OMEGA)
    prof64 = {pmg.PROF_CLASSES[c]: mg64.profile_read(c) for c in pmg.PROF_CLASSES}
    mg64.profile(False)
    # the fused CG iteration of the lower API (cg_iterator) on the 512^3 level: the time of
    # 20 iterations from the difference of a 25- and a 5-iteration call (set-up, the first
    # residual and the final read cancel); 88 algorithmic bytes per cell and iteration
    # (A p with Ap.p: read p, write Ap; x/r update with r.r: read x, r, p, Ap, write x, r;
    # p = r + beta p: read r, p, write p)
    xcg = torch.zeros_like(d_rhs)
    mg64.cg_iterator(0, xcg, d_rhs, 2)
    cg_ms = {}
    for its in (5, 25):
        c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        xcg.zero_()
        barrier()
        c0.record(stream)
        mg64.cg_iterator(0, xcg, d_rhs, its)
        c1.record(stream)
        barrier()
        cg_ms[its] = c0.elapsed_time(c1)
    cg_it_ms = (cg_ms[25] - cg_ms[5]) / 20.0
    cg_gbs = 88.0 * float(n) ** 3 / (cg_it_ms * 1e-3) / 1e9
    del xcg
    mg64.destroy()
    sol64_host = s64.cpu().numpy().T        # (0:n+1)^3 in Fortran order, as the oracle holds it
    sol_mixed_host = d_sol.cpu().numpy().T
    # the FP64 performance mode (FMA, stored omega/c0, normalised transfer weights): the
    # fastest FP64 V-cycle this library has, the comparator for the mixed path's speed-up
    mgf = pmg.Multigrid(mesh, nl, 100, "cgs", precision="fp64_fast", stream=stream.cuda_stream)
    s64.zero_()
    mgf.solve_vcycle(s64, r64, d_rhs, MAXIT, TOL, OMEGA)
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    barrier()
    f0.record(stream)
    for _ in range(fp64_steps):
        s64.zero_()
        repf = mgf.solve_vcycle(s64, r64, d_rhs, MAXIT, TOL, OMEGA)
    f1.record(stream)
    barrier()
    fast_ms = f0.elapsed_time(f1) / fp64_steps
    mgf.profile(True)
    s64.zero_()
    mgf.solve_vcycle(s64, r64, d_rhs, MAXIT, TOL, OMEGA)
    proff = {pmg.PROF_CLASSES[c]: mgf.profile_read(c) for c in pmg.PROF_CLASSES}
    mgf.profile(False)
    mgf.destroy()
    sol_fast_host = s64.cpu().numpy().T
    del s64, r64

    # end to end through the C-ABI with host buffers (copies inside the timed region):
    # pinned (page-locked) buffers, then ordinary pageable numpy arrays as a Fortran caller
    # would pass them
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
    del h_rhs, h_sol, h_rsd, a_rhs, a_sol, a_rsd
    # allocated and initialised on the host, as a Fortran caller's arrays are (np.zeros maps
    # untouched pages, which the GPU would then be the first to write)
    p_rhs = np.ascontiguousarray(rhs.T)
    p_sol, p_rsd = np.empty_like(p_rhs), np.empty_like(p_rhs)
    p_sol[...] = 0.0
    p_rsd[...] = 0.0
    mg.solve_vcycle(p_sol, p_rsd, p_rhs, MAXIT, TOL, OMEGA)
    pageable, pageable_stream = [], []
    for _ in range(min(args.steps, 3)):
        p_sol[...] = 0.0
        t0 = time.perf_counter()
        rep_p = mg.solve_vcycle(p_sol, p_rsd, p_rhs, MAXIT, TOL, OMEGA)
        pageable.append((time.perf_counter() - t0) * 1e3)
        pageable_stream.append(rep_p.elapsed_ms)
    del p_sol, p_rsd, p_rhs
    barrier()
    t0 = time.perf_counter()
    mg.destroy()
    torch.cuda.synchronize()
    destroy_ms = (time.perf_counter() - t0) * 1e3

    # the batched workload (128 problems of uneven sizes), a few timed solves
    batch = None
    if not args.no_batch:
        batch = batch_summary(args, peak)

    # roofline of the dominant kernel class
    dom = max((k for k in prof if prof[k][2] > 0), key=lambda k: prof[k][0])
    t_tot, n_l, b_l = prof[dom]
    achieved = b_l / (t_tot / n_l * 1e-3) / 1e9
    traffic = ncu_traffic().get(dom)
    cells = float(n) ** 3
    cpu, errors = None, {}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            cpu, osol = cpu_baseline(mesh, rhs, nl)
            inner = (slice(1, -1),) * 3
            o = osol[inner]
            scale = float(np.abs(o).max())
            errors = {
                "fp64_gpu_equals_oracle_bitwise": bool(np.array_equal(sol64_host, osol)),
                "fp64_gpu_vs_oracle_max_abs": float(np.abs(sol64_host[inner] - o).max()),
                "mixed_vs_oracle_max_abs_err_rel": float(np.abs(sol_mixed_host[inner] - o).max()) / scale,
                "mixed_vs_oracle_l2_rel": float(np.linalg.norm(sol_mixed_host[inner] - o) / np.linalg.norm(o)),
                "fp64_fast_vs_oracle_max_abs_err_rel": float(np.abs(sol_fast_host[inner] - o).max()) / scale,
            }
        except Exception as exc:  # report, do not hide
            cpu = {"value": None, "error": str(exc)}
    if rank == 0:
        line = {
            "metric": metric_for(n), "value": round(ms, 3), "unit": "ms", "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": round(ms, 3), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic (seeded Gaussian blobs, PCG64(3))",
            "config": {"workload": "%d^3 Poisson, mixed FP32 V(2,2) in FP64 defect correction to 1e-10 " % n +
                                   "(replicas only across GPUs)",
                       "n": n, "levels": nl, "inner_cycles_per_correction": args.inner,
                       "outer_corrections": rep.cycles, "fp32_vcycles": rep.inner_cycles,
                       "l2": "inputs larger than L2 (8.7 GB of FP64/FP32 arrays per solve)",
                       "fp64_ms": round(fp64_ms, 3), "fp64_steps": fp64_steps, "fp64_cycles": rep64.cycles,
                       "speedup_mixed_vs_fp64": round(fp64_ms / ms, 3),
                       "fp64_fast_ms": round(fast_ms, 3), "fp64_fast_cycles": repf.cycles,
                       "speedup_mixed_vs_fp64_fast": round(fast_ms / ms, 3), **errors},
            "setup": {"create_ms": round(create_ms, 1), "first_solve_ms": round(first_solve_ms, 1),
                      "destroy_ms": round(destroy_ms, 1),
                      "note": "first context of the process; the first solve autotunes the smoother per level "
                              "and captures the V-cycle graphs"},
            "roofline": {"kernel": dom, "bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4),
                         "traffic": traffic},
            "kernels": kernel_table(prof, args.steps),
            "kernels_fp64": kernel_table(prof64, 1),
            "kernels_fp64_fast": kernel_table(proff, 1),
            "cg_fp64": {"ms_per_iteration": round(cg_it_ms, 4), "gbs": round(cg_gbs, 1),
                        "frac": round(cg_gbs / peak, 4), "bytes_per_cell": 88,
                        "workload": "fused CG iterations (cg_iterator) on the 512^3 level, FP64 bitwise"},
            "cpu_baseline": cpu,
            # host to device: the right-hand side; the initial guess (x0 = 0 here) is scanned on
            # the host and not sent.  Device to host: the solution and the residual.
            "e2e": {"value": round(e2e_ms, 3), "unit": "ms", "h2d_bytes_per_step": nbytes,
                    "d2h_bytes_per_step": 2 * nbytes, "initial_guess": "zero (scanned on the host, not copied)",
                    "stream_ms": round(statistics.mean(e2e_stream), 3),
                    "median_ms": round(statistics.median(e2e), 3),
                    "steps_ms": [round(v, 2) for v in e2e],
                    "host_buffers": "pinned",
                    "pageable_ms": round(statistics.mean(pageable), 3),
                    "pageable_stream_ms": round(statistics.mean(pageable_stream), 3),
                    "cold_ms": round(create_ms + first_solve_ms + destroy_ms + e2e_ms - ms, 1)},
            "gpu_launches": launches,
            "clocks": clk,
            "cells_per_s": round(replica_throughput(cells, ms, world), 1),
        }
        if batch:
            line["batch"] = batch
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def batch_summary(args, peak):
    """The batched workload inside the main bench line: create, first solve (autotune and
    graph capture), then the mean of a few timed solves; throughput in cells per second and
    the algorithmic bytes of a solve over its time against the HBM peak."""
    import torch
    from peps_mg_gb300 import problems
    from peps_mg_gb300.batch import BatchSolver

    dims = problems.batch_dims(args.batch)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    bs = BatchSolver(dims, mixed_inner_cycles=args.inner)
    torch.cuda.synchronize()
    create_ms = (time.perf_counter() - t0) * 1e3
    try:
        rhs = bs.field()
        for p, vals in enumerate(problems.batch_rhs(dims)):
            bs.view(rhs, p)[1:-1, 1:-1, 1:-1] = torch.from_numpy(vals).cuda()
        sol = bs.field()
        t0 = time.perf_counter()
        bs.solve(sol, rhs, MAXIT, TOL, OMEGA, max_cycles=100)
        first_ms = (time.perf_counter() - t0) * 1e3
        times = []
        for _ in range(3):
            sol.zero_()
            torch.cuda.synchronize()
            cycles, ratio, ms = bs.solve(sol, rhs, MAXIT, TOL, OMEGA, max_cycles=100)
            times.append(ms)
        assert np.all(ratio < TOL), "batched solve did not converge"
        cells = int(np.prod(dims, axis=1).sum())
        ms = statistics.mean(times)
        abytes = batch_algorithmic_bytes(bs.levels, dims, cycles, args.inner)
        gbs = abytes / (ms * 1e-3) / 1e9
        return {"metric": "batched_solve_cells_per_s", "value": round(cells / (ms * 1e-3), 1), "unit": "cells/s",
                "ms_per_solve": round(ms, 3), "problems": args.batch, "cells": cells,
                "corrections_max": int(cycles.max()), "create_ms": round(create_ms, 1),
                "first_solve_ms": round(first_ms, 1),
                "roofline": {"bound": "hbm", "achieved": round(gbs, 1), "peak": peak, "unit": "GB/s",
                             "frac": round(gbs / peak, 4), "algorithmic_bytes_per_solve": abytes}}
    finally:
        bs.destroy()


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
