"""Benchmark: FDTD TM Yee loop (400x400, 2000 steps, float32) on the GPU, with
the FDFD solve throughput reported beside it.

One "step" = one full 2000-time-step FDTD run of the 400x400 rod-lattice
workload (Gaussian-pulse point source), inputs resident in HBM.  The 400x400
state (~4.5 MB) is L2-resident, so L2 is flushed (a 512 MB write) before every
timed step; the flush is outside the timed events.

Beside the headline the line carries, measured after the timed region:
`fdfd` (config-1 solves/s, plain and direct-preconditioned), `fdfd_1e6`
(solves/s at 1e-6 FP64 residual for the 256-problem 256x256 batch and the
2048x2048 x 16-omega batch, Ez and Hz: direct-preconditioned vs plain GMRES,
host SuperLU beside), `fdtd_scaled` (4096^2) and `fdfd_learned_vs_plain`
(config 4: the learned preconditioner, trained here on the GPU, against plain
GMRES at equal iteration counts and to a common residual).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Under torchrun each rank runs an independent replica (the path has no
exchange); rank 0 prints one JSON line with the max time over ranks.
"""
import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time
import warnings

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "FDTD Gcell-updates/s (400x400 TM, 2000 steps)"
UNIT = "Gcell-updates/s"
BYTES_PER_CELL_UPDATE = 28  # read+write Hx, Hy, Dz + read 1/eps (float32)
# dram__bytes_read.sum + dram__bytes_write.sum of one k_tm_strip launch (the
# whole 2000-step run) on this workload (ncu capture summarised in
# profiles/fdtd_tm_400x400_strip_kernel.md)
STRIP400_DRAM_BYTES_PER_LAUNCH = 4358912 + 653824


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampler during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.idx = device_index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True,
                                     text=True, timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4)
                          if len(s) > 5 + k and s[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _barrier_max(value, ws):
    """Max of a per-rank value over the replicas (the slowest rank's time)."""
    if ws == 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank, seconds_max, ws):
    """Whole-job rate of N independent replicas: the units all ranks processed
    divided by the slowest rank's time (weak scaling)."""
    return units_per_rank * ws / seconds_max


# ------------------------------------------------------------------ CPU arm
def _cpu_worker(args):
    steps, seed = args
    from ceviche_gb300.workloads import config2
    from oracle import fdtd as oft
    p = config2()
    F = oft.FDTD2D(p["eps"], p["dL"], p["npml"])
    t0 = time.perf_counter()
    for t in range(steps):
        F.forward(Jz=p["src"] * p["amps"][t])
    return time.perf_counter() - t0, p["eps"].size * steps


def cpu_baseline(time_steps=300, procs=1):
    """The FP64 numpy restatement of ceviche's fdtd.forward (oracle port) on a
    bounded sample: `procs` independent 400x400 runs of `time_steps` steps."""
    t0 = time.perf_counter()
    if procs == 1:
        res = [_cpu_worker((time_steps, 0))]
    else:
        with mp.get_context("spawn").Pool(procs) as pool:
            res = pool.map(_cpu_worker, [(time_steps, k) for k in range(procs)])
    wall = time.perf_counter() - t0
    cells = sum(r[1] for r in res)
    per_core = [r[1] / r[0] for r in res]
    return cells / wall / 1e9, float(np.mean(per_core)) / 1e9, wall, cells


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return
    # all host cores (CEV_CPU_PROCS=<n> caps the worker processes)
    procs = int(os.environ.get("CEV_CPU_PROCS", "0")) or max(1, len(os.sched_getaffinity(0)))
    ts = 60  # time steps per process per bench step (bounded sample)
    for _ in range(args.warmup if args.warmup < 1 else 1):
        cpu_baseline(10, 1)
    vals, walls = [], []
    for _ in range(args.steps):
        v, _, wall, cells = cpu_baseline(ts, procs)
        vals.append(v)
        walls.append(wall)
    value = float(np.median(vals))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * float(np.median(walls)), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "fdtd_tm_400x400_2000steps (sampled: %d procs x %d time steps per step)"
                   % (procs, ts), "grid": [400, 400], "npml": [20, 20, 0]},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": "port",
                         "sample": f"{procs} independent 400x400 runs x {ts} FDTD steps, numpy FP64"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GPU arm
def _flush_l2(buf):
    buf.zero_()


def fdfd_numbers():
    """Config-1 FDFD Ez solve throughput (plain GMRES, 1e-6 FP64 true residual)
    through the public API: one problem (the fused single-launch cycle), a
    batch of 16 frequencies in one solve, and the reference's own method
    (scipy SuperLU spsolve of the assembled matrix, via the oracle) on one
    host core for comparison."""
    import torch
    from ceviche_gb300 import primitives as P
    from ceviche_gb300.workloads import config1
    from oracle import fdfd as ofd
    p = config1()
    kw = dict(tol=1e-6, max_iters=40000, max_stall=200)
    plan = P.get_plan("ez", p["eps"].shape, p["dL"], p["omega"], p["npml"])
    eps = torch.as_tensor(p["eps"], device="cuda")
    b = (1j * p["omega"] * torch.as_tensor(p["src"], device="cuda")).to(torch.complex128)
    x, info = P.solve(plan, eps, b, **kw)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    n = 3
    for _ in range(n):
        x, info = P.solve(plan, eps, b, **kw)
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / n
    out = {"workload": "fdfd_ez_200x200 (plain restarted GMRES(30), 1e-6 FP64 residual)",
           "solves_per_s": 1.0 / dt, "iterations": info[0]["iterations"],
           "us_per_iteration": 1e6 * dt / info[0]["iterations"],
           "residual": info[0]["residual"], "status": info[0]["status"],
           "path": "fused single-launch restart cycle"}
    # the same solve preconditioned by the nested-dissection factorisation
    # (factorisation inside the timed region)
    def direct():
        dp = P.DirectPrecond(plan, eps)
        return P.solve(plan, eps, b, precond="direct", direct=dp, **kw)[1]
    direct()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(n):
        infod = direct()
    torch.cuda.synchronize()
    dtd = (time.perf_counter() - t0) / n
    out["direct"] = {"solves_per_s": 1.0 / dtd, "iterations": infod[0]["iterations"],
                     "residual": infod[0]["residual"],
                     "path": "FGMRES(30) + complex64 nested-dissection factors (factorisation timed)"}
    # 16 frequencies (lambda 1.50-1.60 um) solved as one batch
    lams = np.linspace(1.50e-6, 1.60e-6, 16)
    oms = 2 * np.pi * 299792458.0 / lams
    planb = P.get_plan("ez", p["eps"].shape, p["dL"], oms, p["npml"])
    bb = torch.stack([(1j * w * torch.as_tensor(p["src"], device="cuda")).to(torch.complex128)
                      for w in oms])
    xb, infob = P.solve(planb, eps, bb, **kw)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    xb, infob = P.solve(planb, eps, bb, **kw)
    torch.cuda.synchronize()
    dtb = time.perf_counter() - t0
    out["batch16"] = {"solves_per_s": 16 / dtb,
                      "max_iterations": max(i["iterations"] for i in infob),
                      "worst_residual": max(i["residual"] for i in infob),
                      "converged": sum(i["code"] == 0 for i in infob)}
    # reference method on the host: assemble + SuperLU, 1 core
    A = ofd.make_A_ez(p["omega"], p["dL"], p["eps"], p["npml"])
    rhs = 1j * p["omega"] * p["src"].ravel()
    t0 = time.perf_counter()
    ofd.spsolve(A, rhs)
    t_lu = time.perf_counter() - t0
    out["cpu_spsolve"] = {"solves_per_s": 1.0 / t_lu, "cores": 1, "kind": "port",
                          "sample": "one 200x200 Ez solve, scipy SuperLU of the assembled matrix"}
    return out


def _timed(fn):
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = fn()
    torch.cuda.synchronize()
    return out, time.perf_counter() - t0


def _solve_record(info, wall, n):
    its = sorted(i["iterations"] for i in info)
    conv = int(sum(i["code"] == 0 and i["residual"] <= 1e-6 for i in info))
    return {"wall_s": wall, "problems": n, "converged_1e-6": conv,
            "solves_per_s_at_1e-6": conv / wall,
            "median_iterations": float(np.median(its)), "max_iterations": int(its[-1]),
            "worst_residual": float(max(i["residual"] for i in info))}


def fdfd_1e6_numbers(plain_cap4=2000, plain_cap5=300):
    """The metric's FDFD half: solves/s at 1e-6 FP64 true residual through
    the public primitives, inputs resident on the device.
      config 4: 256 problems of 256x256 (binary eps, lambda 1.3-1.8 um) in one
        batch; config 5: 2048x2048 with 16 omegas in one batch, Ez and Hz.
    direct: flexible GMRES(30) preconditioned by the complex64
    nested-dissection factorisation; the wall time counts the factorisation
    (every problem has its own eps or omega) and the solve.  plain: restarted
    GMRES(30) capped at `plain_cap` iterations (it does not reach 1e-6 on
    these configurations); its residual is reported.  cpu_spsolve: the
    reference's method (assembly + SuperLU) for one config-4 problem on one
    host core."""
    import torch
    from ceviche_gb300 import primitives as P
    from ceviche_gb300.workloads import config4_problem, config5
    from oracle import fdfd as ofd
    out = {}
    probs = [config4_problem(i) for i in range(256)]
    oms = np.array([q["omega"] for q in probs])
    eps4 = torch.as_tensor(np.stack([q["eps"] for q in probs]), device="cuda")
    b4 = torch.as_tensor(np.stack([1j * q["omega"] * q["src"] for q in probs]), device="cuda")
    c4 = {}
    for pol in ("ez", "hz"):
        plan = P.Plan(pol, (256, 256), probs[0]["dL"], oms, probs[0]["npml"])

        def direct():
            dp = P.DirectPrecond(plan, eps4)
            return P.solve(plan, eps4, b4, precond="direct", direct=dp, tol=1e-6)[1]
        direct()  # grid analysis (cached per grid) and first-call costs
        info, wall = _timed(direct)
        rec = {"direct": _solve_record(info, wall, 256)}
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            info, wall = _timed(lambda: P.solve(plan, eps4, b4, tol=1e-6, max_iters=plain_cap4,
                                                max_stall=10 ** 6)[1])
        rec["plain"] = dict(_solve_record(info, wall, 256), iteration_cap=plain_cap4,
                            median_residual=float(np.median([i["residual"] for i in info])))
        c4[pol] = rec
        del plan
    q = probs[0]
    A = ofd.make_A_ez(q["omega"], q["dL"], q["eps"], q["npml"])
    t0 = time.perf_counter()
    ofd.spsolve(A, 1j * q["omega"] * q["src"].ravel())
    t_lu = time.perf_counter() - t0
    c4["cpu_spsolve"] = {"solves_per_s": 1 / t_lu, "cores": 1, "kind": "port",
                         "sample": "one 256x256 Ez problem, scipy SuperLU of the assembled matrix"}
    out["config4_256x256_batch256"] = c4
    del eps4, b4
    torch.cuda.empty_cache()
    q5 = config5()
    n5 = q5["eps"].shape[0]
    e5 = torch.as_tensor(q5["eps"], device="cuda")
    b5 = torch.as_tensor(np.stack([1j * w * q5["src"] for w in q5["omegas"]]), device="cuda")
    c5 = {}
    for pol in ("ez", "hz"):
        plan = P.Plan(pol, (n5, n5), q5["dL"], q5["omegas"], q5["npml"])
        holder = {}

        def direct():
            holder["dp"] = P.DirectPrecond(plan, e5)
            return P.solve(plan, e5, b5, precond="direct", direct=holder["dp"], tol=1e-6)[1]
        direct()  # grid analysis (cached) and first-call costs
        holder.clear()
        torch.cuda.empty_cache()
        info, wall = _timed(direct)
        dp = holder.pop("dp")
        _, t_fac = _timed(lambda: P.DirectPrecond(plan, e5))
        r = torch.randn(16, n5, n5, dtype=torch.complex64, device="cuda")
        _, t_app = _timed(lambda: dp.apply(r))
        rec = {"direct": dict(_solve_record(info, wall, 16), factor_s=t_fac,
                              factor_GB=dp.factor_bytes / 1e9,
                              factor_TFMAs=4 * dp.factor_cmacs / t_fac / 1e12,
                              apply_ms=1e3 * t_app, apply_GBps=dp.factor_bytes / t_app / 1e9)}
        del dp, holder
        torch.cuda.empty_cache()
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            info, wall = _timed(lambda: P.solve(plan, e5, b5, tol=1e-6, max_iters=plain_cap5,
                                                max_stall=10 ** 6)[1])
        rec["plain"] = dict(_solve_record(info, wall, 16), iteration_cap=plain_cap5,
                            median_residual=float(np.median([i["residual"] for i in info])))
        c5[pol] = rec
        del plan
        torch.cuda.empty_cache()
    c5["cpu_spsolve"] = {"note": "not timed here: one 1024x1024 SuperLU solve took 63 s on one "
                                 "core of the build machine; 2048x2048 is several hundred s"}
    out["config5_2048x2048_16omega"] = c5
    return out


def fdtd_te_numbers(steps=2000):
    """The TE polarisation (Hz, Dx, Dy with Jx, Jy point sources carrying the
    config-2 pulse) on the config-2 grid through the time-blocked TE runner,
    beside the TM headline."""
    import torch
    import ceviche_gb300 as cev
    from ceviche_gb300.workloads import config2
    p = config2()
    F = cev.fdtd(p["eps"], p["dL"], p["npml"], precision="float32")
    sx, sy = p["src"], -0.5 * p["src"]
    F.run_te(steps, sx, sy, p["amps"])
    stream = torch.cuda.current_stream()
    ts = []
    for _ in range(3):
        F.initialize_fields()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        F.run_te(steps, sx, sy, p["amps"])
        e1.record(stream)
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1) / 1e3)
    t = min(ts)
    cells = p["eps"].size * steps
    return {"workload": "fdtd_te_400x400_2000steps (k_te_tile, 8 steps per launch)",
            "value": cells / t / 1e9, "unit": UNIT,
            "algorithmic_GBps": cells * 36 / t / 1e9,
            "note": "36 B/cell-update algorithmic (Hz, Dx, Dy r+w, 1/eps_xx, 1/eps_yy r)"}


def fdtd_scaled_numbers(steps=256, n=4096):
    """Builder addition: the TM runner on an n x n grid (config-2 generator
    scaled by area; 4096^2 and 8192^2), where the state (> 400 MB) does not
    fit in L2, so the roofline fraction measures HBM bandwidth."""
    import torch
    import ceviche_gb300 as cev
    from ceviche_gb300.workloads import config2
    p = config2(N=n, steps=steps)
    F = cev.fdtd(p["eps"], p["dL"], p["npml"], precision="float32")
    amps = p["amps"][:steps]
    F.run(steps, p["src"], amps)
    stream = torch.cuda.current_stream()
    ts = []
    for _ in range(3):
        F.initialize_fields()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        F.run(steps, p["src"], amps)
        e1.record(stream)
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1) / 1e3)
    t = min(ts)
    cells = n * n * steps
    peak, kind = _peaks()
    gbs = cells * BYTES_PER_CELL_UPDATE / t / 1e9
    return {"workload": f"fdtd_tm_{n}x{n}_{steps}steps (config-2 generator scaled by area)",
            "value": cells / t / 1e9, "unit": UNIT,
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s",
                         "frac": gbs / peak, "peak_kind": kind}}


def run_ours(args):
    import torch
    import ceviche_gb300 as cev
    from ceviche_gb300.workloads import config2

    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.cuda.current_device()
    p = config2()
    steps_t = p["steps"]
    N = p["eps"].size
    F = cev.fdtd(p["eps"], p["dL"], p["npml"], precision="float32")
    flush = torch.empty(512 * 2 ** 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()

    def one_run():
        F.initialize_fields()
        F.run(steps_t, p["src"], p["amps"])

    for _ in range(max(args.warmup, 3)):
        one_run()
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    times = []
    with Clocks(dev) as clk:
        for _ in range(args.steps):
            _flush_l2(flush)
            F.initialize_fields()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            F.run(steps_t, p["src"], p["amps"])
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    total = _barrier_max(sum(times), ws)
    value = aggregate_rate(N * steps_t * args.steps, total, ws) / 1e9
    ms_per_step = 1e3 * total / args.steps

    # end to end through the public API with host buffers
    eps_host = torch.as_tensor(p["eps"]).pin_memory()
    amps_host = torch.as_tensor(p["amps"].astype(np.float32)).pin_memory()
    e2e_times = []
    for k in range(max(2, args.steps // 2) + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        G = cev.fdtd(eps_host, p["dL"], p["npml"], precision="float32")
        G.run(steps_t, p["src"], amps_host)
        ez = G.fields["Ez"].cpu()
        torch.cuda.synchronize()
        if k > 0:
            e2e_times.append(time.perf_counter() - t0)
        del G
    e2e_t = _barrier_max(float(np.median(e2e_times)), ws)
    e2e_val = aggregate_rate(N * steps_t, e2e_t, ws) / 1e9

    line = None
    if rank == 0:
        peak, peak_kind = _peaks()
        achieved = N * BYTES_PER_CELL_UPDATE * steps_t / (total / args.steps) / 1e9
        launches_per_run = 1  # one cooperative k_tm_strip launch advances all 2000 steps
        cpu_v, cpu_core, cpu_wall, _ = cpu_baseline(int(os.environ.get("CEV_CPU_STEPS", "500")), 1)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "fdtd_tm_400x400_2000steps", "grid": [400, 400],
                       "npml": [20, 20, 0], "time_steps": steps_t, "rods": 30,
                       "l2": "flushed (512 MB write) before every timed step",
                       "parallelism": f"replicas x{ws}"},
            "gpu_launches": launches_per_run * args.steps,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": STRIP400_DRAM_BYTES_PER_LAUNCH,
                         "traffic_unit": "bytes per launch (the whole 2000-step run)",
                         "algorithmic_bytes_per_launch": N * BYTES_PER_CELL_UPDATE * steps_t,
                         "kernel": "k_tm_strip<float,14,3,8,persistent>", "peak_kind": peak_kind,
                         "note": "algorithmic 28 B/cell-update; one cooperative launch keeps the "
                                 "400x400 state in registers across all 2000 steps and exchanges "
                                 "8-cell rings between tiles through L2 every 8 steps, so DRAM "
                                 "traffic is 0.06% of the algorithmic bytes: the kernel is bound "
                                 "by the ring exchange latency and the on-chip stencil work"},
            "cpu_baseline": {"value": cpu_v, "unit": UNIT, "cores": 1, "kind": "port",
                             "sample": "400x400 x %s FDTD steps, numpy FP64 oracle port"
                                       % os.environ.get("CEV_CPU_STEPS", "500")},
            "e2e": {"value": e2e_val, "unit": UNIT,
                    "h2d_bytes_per_step": int(p["eps"].size * 8 + steps_t * 4 + 16),
                    "d2h_bytes_per_step": int(N * 4)},
            "clocks": clk.summary(),
        }
        if not args.no_fdfd:
            try:
                line["fdfd"] = fdfd_numbers()
            except Exception as e:  # reported, never hidden
                line["fdfd"] = {"error": repr(e)}
            try:
                line["fdfd_1e6"] = fdfd_1e6_numbers()
            except Exception as e:
                line["fdfd_1e6"] = {"error": repr(e)}
            try:
                line["fdtd_te"] = fdtd_te_numbers()
            except Exception as e:
                line["fdtd_te"] = {"error": repr(e)}
            try:
                line["fdtd_scaled"] = fdtd_scaled_numbers()
            except Exception as e:
                line["fdtd_scaled"] = {"error": repr(e)}
            try:
                line["fdtd_scaled_8192"] = fdtd_scaled_numbers(steps=128, n=8192)
            except Exception as e:
                line["fdtd_scaled_8192"] = {"error": repr(e)}
            try:
                # the metric's "learned vs plain" part on config 4 (a shorter
                # training schedule than --configs: 64 problems, 3000 + 1500 steps)
                line["fdfd_learned_vs_plain"] = learned_numbers(train_problems=64, steps=3000,
                                                                iter_cap=300)
            except Exception as e:
                line["fdfd_learned_vs_plain"] = {"error": repr(e)}
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def learned_numbers(train_problems=128, steps=6000, eval_batch=16, iter_cap=900):
    """Config 4 with the learned preconditioner: build training residuals
    with the plain solver on `train_problems` problems, train the network on
    the GPU (Adam, physics loss through the stencil), then solve `eval_batch`
    held-out problems with FGMRES(30)+network and with plain GMRES(30), both
    capped at `iter_cap` iterations; plus the network's own throughput."""
    import torch
    from ceviche_gb300 import primitives as P
    from ceviche_gb300.learned import LearnedPreconditioner, on_policy_samples, residual_samples
    from ceviche_gb300.workloads import config4_problem

    def group(ids):
        pr = [config4_problem(i) for i in ids]
        om = np.array([q["omega"] for q in pr])
        pl = P.get_plan("ez", (256, 256), pr[0]["dL"], om, pr[0]["npml"])
        ep = torch.as_tensor(np.stack([q["eps"] for q in pr])).cuda()
        bb = torch.stack([torch.as_tensor(1j * q["omega"] * q["src"]) for q in pr]).cuda()
        return pl, ep, bb

    iters = (0, 10, 30, 90, 270, 810)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    samples = []
    for g0 in range(0, train_problems, 16):
        pl, ep, bb = group(range(g0, g0 + 16))
        samples += [(pl, ep, r) for r in residual_samples(pl, ep, bb, iters=iters)]
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    net = LearnedPreconditioner(256, 256, max_batch=16, c0=32, seed=0)
    t0 = time.perf_counter()
    net.fit(samples, steps=steps, lr=5e-4)
    # one on-policy round: add the residuals where FGMRES with the network stalls
    extra = []
    for g0 in range(0, train_problems, 16):
        pl, ep, bb = group(range(g0, g0 + 16))
        extra += [(pl, ep, r) for r in on_policy_samples(net, pl, ep, bb)]
    net.fit(samples + 2 * extra, steps=steps // 2, lr=2e-4, seed=1)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    pl, ep, bb = group(range(256, 256 + eval_batch))
    held = [float(net.loss_and_grad(pl, ep, r)[0]) for r in residual_samples(pl, ep, bb, iters=iters)]
    res = {}
    for name, kw in (("plain", {}), ("learned", dict(precond="learned", learned=net))):
        for k in sorted({30, 90, 300, iter_cap}):
            with warnings.catch_warnings():
                warnings.simplefilter("ignore")
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                _, info = P.solve(pl, ep, bb, tol=1e-6, max_iters=k, max_stall=10 ** 6, **kw)
                torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            res[f"{name}_at_{k}"] = {
                "median_residual": float(np.median([i["residual"] for i in info])),
                "converged": int(sum(i["code"] == 0 for i in info)), "wall_s": dt,
                "ms_per_iteration": 1e3 * dt / k}
    # wall time to the residual the learned solver reaches in one restart cycle
    target = res["learned_at_30"]["median_residual"]
    to_target = {}
    for name, kw, cap in (("plain", {}, 20000), ("learned", dict(precond="learned", learned=net), 900)):
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            _, info = P.solve(pl, ep, bb, tol=target, max_iters=cap, max_stall=10 ** 6, **kw)
            torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        to_target[name] = {"wall_s": dt, "solves_per_s": eval_batch / dt,
                           "converged": int(sum(i["code"] == 0 for i in info)),
                           "median_iterations": float(np.median([i["iterations"] for i in info]))}
    res["to_learned_30_iteration_residual"] = dict(tol=target, **to_target)
    # network throughput: forward on a 16-problem batch
    r = bb.to(torch.complex64)
    for _ in range(3):
        net.forward(pl, ep, r)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(20):
        net.forward(pl, ep, r)
    torch.cuda.synchronize()
    tf = (time.perf_counter() - t0) / 20
    c = 32
    macs_px = (8 * c + 2 * c * c / 4 + 8 * c * c / 16 + (32 + 64 + 32) * c * c / 64
               + (16 + 8) * c * c / 16 + (4 + 2) * c * c / 4 + c * c) * 9
    flops = 2 * macs_px * eval_batch * 256 * 256
    return {"train_problems": train_problems, "train_steps": steps, "data_s": t_data,
            "train_s": t_train, "heldout_loss_by_plain_iterate": dict(zip(map(str, iters), held)),
            "eval_batch": eval_batch, "solves": res,
            "network_forward_ms_batch16": 1e3 * tf, "network_forward_tflops": flops / tf / 1e12,
            "note": "tol 1e-6 FP64 true residual: neither method reaches it within the cap; "
                    "compared: median residual at equal iteration counts, and wall time to "
                    "the residual the learned solver reaches in 30 iterations"}


def learned_forward_numbers(conv_impl=1, steps=5, warmup=3, batch=16):
    """Network forward of the learned preconditioner on `batch` config-4
    problems of 256x256 (random-init weights; the cost does not depend on
    them): time per forward and FLOP rate, for the tcgen05 or mma.sync conv."""
    import torch
    from ceviche_gb300 import _lib
    from ceviche_gb300 import primitives as P
    from ceviche_gb300.learned import LearnedPreconditioner
    from ceviche_gb300.workloads import config4_problem
    lib = _lib.load()
    _lib.check(lib.cev_learned_set_conv_impl(conv_impl), "set_conv_impl")
    probs = [config4_problem(i) for i in range(batch)]
    oms = np.array([q["omega"] for q in probs])
    plan = P.get_plan("ez", (256, 256), probs[0]["dL"], oms, probs[0]["npml"])
    eps = torch.as_tensor(np.stack([q["eps"] for q in probs])).cuda()
    r = torch.stack([torch.as_tensor(1j * q["omega"] * q["src"]) for q in probs]).cuda()
    r = r.to(torch.complex64)
    net = LearnedPreconditioner(256, 256, max_batch=batch, c0=32)
    for _ in range(max(1, warmup)):
        net.forward(plan, eps, r)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    start.record()
    for _ in range(steps):
        net.forward(plan, eps, r)
    end.record()
    torch.cuda.synchronize()
    ms = start.elapsed_time(end) / steps
    flops = 2 * 66816 * batch * 256 * 256  # 7424 MACs x 9 taps per full-resolution pixel
    return {"metric": "learned preconditioner forward", "conv_impl": ["mma.sync", "tcgen05"][conv_impl],
            "batch": batch, "grid": [256, 256], "ms_per_forward": ms,
            "tflops": flops / ms / 1e9, "steps": steps}


def config_numbers(max_iters5=1500):
    """The other FDFD configurations with the plain GPU Krylov path (one JSON
    line, not part of the default run):
      3: 600x600 adjoint gradient (forward + transposed solve + gradient kernel)
         beside the host SuperLU forward solve of the same matrix;
      4: 256 problems of 256x256 (binary eps, lambda 1.3-1.8 um, dL =
         lambda0/20) solved as one batch;
      5: 2048x2048 Ez, 16 frequencies as one batch, capped at max_iters5
         Arnoldi iterations (plain GMRES(30) does not reach 1e-6 here): the
         residual reached, time per iteration and the algorithmic bytes moved."""
    import torch
    import ceviche_gb300 as cev
    from ceviche_gb300 import primitives as P
    from ceviche_gb300.workloads import config3, config4_problem, config5
    from oracle import fdfd as ofd
    out = {}
    # config 3
    p = config3()
    kw = dict(tol=1e-6, max_iters=200000, max_stall=100000)
    F = cev.fdfd_ez(p["omega"], p["dL"], p["eps"], p["npml"], **kw)
    probe = torch.as_tensor(p["probe"], device="cuda")
    src = torch.as_tensor(p["src"], device="cuda")

    def grad_once(scale):
        eps = torch.tensor(p["eps"] * scale, device="cuda", requires_grad=True)
        F.eps_r = eps
        _, _, ez = F.solve(src)
        J = ((ez * probe.conj()).sum().abs() ** 2)
        J.backward()
        return eps.grad

    # two warm-up gradients carry the one-time costs (symbolic analysis,
    # workspace, first kernel use); the timed one has a new eps, as an
    # optimisation step would, so both factorisations are in the time
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    grad_once(1.0)
    grad_once(1.0 + 1e-3)
    torch.cuda.synchronize()
    t_first = time.perf_counter() - t0
    t0 = time.perf_counter()
    grad_once(1.0 + 2e-3)
    torch.cuda.synchronize()
    t_grad = time.perf_counter() - t0
    A = ofd.make_A_ez(p["omega"], p["dL"], p["eps"], p["npml"])
    t0 = time.perf_counter()
    ofd.spsolve(A, 1j * p["omega"] * p["src"].ravel())
    t_lu = time.perf_counter() - t0
    out["config3_adjoint_gradient_600x600"] = {
        "gpu_gradient_s": t_grad, "gpu_gradients_per_s": 1 / t_grad,
        "gpu_first_two_gradients_s": t_first,
        "cpu_spsolve_forward_s": t_lu, "cpu_cores": 1,
        "note": "GPU: forward + transposed FGMRES(30) solves to 1e-6 with the direct "
                "preconditioner (the drop-in class default; factorisations timed) and the "
                "gradient kernel; CPU: one SuperLU forward solve (the adjoint needs a second)"}
    # config 3b: FDTD reverse-time adjoint, 400x400, 4000 steps, checkpoints every 64
    from ceviche_gb300.workloads import config2
    p2 = config2(steps=4000)
    probes = [(300, 200), (200, 300), (120, 120)]
    for rep in range(2):  # second run timed (first one builds the plan)
        eps_t = torch.tensor(p2["eps"], device="cuda", requires_grad=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        series = cev.fdtd_probe_series(eps_t, p2["dL"], p2["npml"], 4000, p2["src"], p2["amps"],
                                       probes, precision="float32", ckpt_every=64)
        torch.cuda.synchronize()
        t_fwd = time.perf_counter() - t0
        series.sum().backward()
        torch.cuda.synchronize()
        t_all = time.perf_counter() - t0
    cells = p2["eps"].size * 4000
    out["config3b_fdtd_adjoint_400x400_4000steps"] = {
        "forward_s": t_fwd, "forward_plus_adjoint_s": t_all,
        "forward_gcell_per_s": cells / t_fwd / 1e9,
        "adjoint_gcell_per_s": cells / (t_all - t_fwd) / 1e9, "ckpt_every": 64,
        "precision": "float32"}
    # config 4
    probs = [config4_problem(i) for i in range(256)]
    n4 = probs[0]["eps"].shape[0]
    oms = np.array([q["omega"] for q in probs])
    plan = P.get_plan("ez", (n4, n4), probs[0]["dL"], oms, probs[0]["npml"])
    eps4 = torch.as_tensor(np.stack([q["eps"] for q in probs]))
    b4 = torch.stack([torch.as_tensor(1j * q["omega"] * q["src"]) for q in probs])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _, info = P.solve(plan, eps4, b4, tol=1e-6, max_iters=20000, max_stall=100000)
    torch.cuda.synchronize()
    t4 = time.perf_counter() - t0
    conv = sum(i["code"] == 0 for i in info)
    its = [i["iterations"] for i in info]
    out["config4_batch256_256x256"] = {
        "solves_per_s": len(probs) / t4, "wall_s": t4, "converged": conv, "batch": len(probs),
        "median_iterations": float(np.median(its)), "max_iterations": int(max(its)),
        "worst_residual": float(max(i["residual"] for i in info))}
    out["config4_learned_vs_plain_256x256"] = learned_numbers()
    # config 5: Ez and Hz
    q = config5()
    n5 = q["eps"].shape[0]
    b5 = torch.stack([torch.as_tensor(1j * w * q["src"]) for w in q["omegas"]])
    e5 = torch.as_tensor(q["eps"])
    cells = n5 * n5 * len(q["omegas"])
    for pol in ("ez", "hz"):
        plan = P.get_plan(pol, (n5, n5), q["dL"], q["omegas"], q["npml"])
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            _, info = P.solve(plan, e5, b5, tol=1e-6, max_iters=max_iters5, max_stall=100000)
            torch.cuda.synchronize()
        t5 = time.perf_counter() - t0
        it5 = max(i["iterations"] for i in info)
        key = "config5_2048x2048_16omega" + ("" if pol == "ez" else "_hz")
        out[key] = {
            "pol": pol, "iterations": it5, "wall_s": t5, "ms_per_iteration": 1e3 * t5 / it5,
            "converged": sum(i["code"] == 0 for i in info),
            "best_residual": float(min(i["residual"] for i in info)),
            "worst_residual": float(max(i["residual"] for i in info)),
            "algorithmic_GBps": cells * 292 * it5 / t5 / 1e9,
            "note": "292 B/cell per GMRES(30) iteration (stencil 20 + Gram-Schmidt 16j + 24, "
                    "averaged over j = 1..30); plain Krylov does not converge here"}
        del plan
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-fdfd", action="store_true")
    ap.add_argument("--configs", action="store_true",
                    help="measure the other FDFD configurations (plain GPU Krylov) instead")
    ap.add_argument("--learned-forward", action="store_true",
                    help="time the learned preconditioner's network on 16 problems of 256x256")
    ap.add_argument("--conv-impl", type=int, default=1, choices=[0, 1],
                    help="with --learned-forward: 1 tcgen05 conv (default), 0 mma.sync conv")
    args = ap.parse_args()
    if args.learned_forward:
        print(json.dumps(learned_forward_numbers(args.conv_impl, args.steps, args.warmup)), flush=True)
    elif args.configs:
        print(json.dumps(config_numbers()), flush=True)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
