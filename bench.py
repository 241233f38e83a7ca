"""Benchmark of the GB300 SunlightLB update step.

Workload (the packed-bed permeability case): periodic 128^3 lattice, seeded
random sequential addition of non-overlapping spheres with radius uniform in
[4, 8] up to lattice solid fraction 0.30, fixed objects with link
bounce-back, body force 1e-6 along x, tau = 1 (viscosity 1/6), Stokes flow,
FP32 populations.  A step is one lattice Boltzmann update (bounce-back,
streaming and collision of every node) of the whole lattice.

Metric: million lattice updates per second (all nodes, fluid and solid, as
the reference's own fwrstats counts them, src/lbmisc.c:264-274).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl mine|reference]

Under torchrun each rank advances its own replica of the lattice (the single
lattice is not split across GPUs); value is the sum over ranks of the nodes
updated divided by the slowest rank's time.

The JSON line carries:
  value      device-resident throughput, CUDA events around each step on the
             lattice's stream, L2 flushed (256 MiB write) between steps;
  e2e        the same metric through the public C API with host buffers:
             populations, geometry and body force uploaded from the host, the
             steps run as check intervals (98 lbstep + measure, which reads
             the mean flow and the drag back), populations read back at the end;
  roofline   achieved HBM GB/s of the fused step kernel against the measured
             copy bandwidth (120 algorithmic bytes per FP32 node update);
  cpu_baseline  the CPU oracle (a restatement of the reference's C code) on
             one host core, on a time-bounded sample of steps.
"""

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_SIDE = 128
PHI = 0.30
RMIN, RMAX = 4.0, 8.0
FORCE = 1e-6
TAU = 1.0
SEED = 1
# state bytes per node update (the 2-byte flag word read by every step is
# left out): FP64/FP32 read and write 15 populations; BF16 paired-deviation
# storage reads and writes one float4 of moments and one 16-byte vector of
# deviations
BYTES_PER_UPDATE = {0: 240, 1: 120, 2: 64}
CHECK = 100                           # check interval of the e2e run (98 steps + measure)


def config(prec_name, l2):
    return {"workload": f"packed-bed permeability, periodic {N_SIDE}^3, RSA spheres r~U[{RMIN:g},{RMAX:g}] "
                        f"to solid fraction {PHI}, body force {FORCE:g} along x, tau {TAU:g}, Stokes",
            "lattice": [N_SIDE, N_SIDE, N_SIDE], "populations": prec_name, "seed": SEED,
            "velocity_set": "D3Q15", "l2": l2, "parallelism": "replicas"}


def dist_env():
    return int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0"))


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                for line in out.stdout.strip().splitlines():
                    self.samples.append([c.strip() for c in line.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *exc):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no nvidia-smi samples"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 5 + i and s[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(self.samples)}


def aggregate(total_ms, nodes, steps, world, dist=None, device=None):
    """Replica throughput over ranks: every rank advanced its own lattice of
    `nodes` nodes by `steps` steps in total_ms; the job's time is the
    slowest rank's.  Returns (MLUPS of the whole job, ms per step)."""
    if world > 1 and dist is not None:
        import torch
        t = torch.tensor([float(total_ms)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_per_step = total_ms / steps
    return world * nodes / (ms_per_step * 1e-3) / 1e6, ms_per_step


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic(prec_name):
    """DRAM bytes per launch of the fused step (mean of the odd and even
    step) from the committed ncu summary profiles/lb_step_128.md, line
    'traffic_per_launch_<precision>: <bytes>'."""
    p = os.path.join(ROOT, "profiles", "lb_step_128.md")
    try:
        with open(p) as f:
            for line in f:
                key = f"traffic_per_launch_{prec_name}:"
                if line.strip().startswith(key):
                    return int(float(line.split(":", 1)[1].split()[0]))
    except Exception:
        pass
    return None


def build_lattice(L, precision, spheres, solid):
    from sunlightlb_gb300 import workloads as W
    lb, _, _ = W.packed_bed(L, n=N_SIDE, phi=PHI, rmin=RMIN, rmax=RMAX, seed=SEED, force=FORCE, tau=TAU,
                            precision=precision, spheres=spheres)
    return lb


class Flusher:
    """L2 flush between timed steps: write a 256 MiB buffer (larger than the
    129 MB L2), then read it back so the lines left in L2 are clean and no
    write-back of flush data lands inside the next timed step."""

    def __init__(self, torch):
        self.buf = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def __call__(self):
        self.buf.zero_()
        self.buf.sum()


def time_steps(torch, L, lb, steps, warmup, flusher=None):
    """Per-step device times (ms) of `steps` lbstep calls, CUDA events on
    the lattice's own stream, optional L2 flush before each timed step."""
    stream = torch.cuda.ExternalStream(L.lbgetstream(lb))
    for _ in range(warmup):
        L.lbstep(lb)
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    with torch.cuda.stream(stream):
        for s in range(steps):
            if flusher is not None:
                flusher()
            starts[s].record(stream)
            L.lbstep(lb)
            ends[s].record(stream)
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in zip(starts, ends)]


def tuning(L, lb):
    import ctypes
    cfg = (ctypes.c_int * 4)()
    state = L.lbtuning(lb, ctypes.addressof(cfg))
    st = {1: "tuned", -1: "default", 0: "none"}.get(state, state)
    if lb.precision == 2:  # one update kernel: planes per block (32 x 8 threads)
        return {"state": st, "planes_per_block": cfg[0]}
    return {"state": st, "even": {"rows_per_thread": cfg[0], "threads_k": cfg[1]},
            "odd": {"rows_per_thread": cfg[2], "threads_k": cfg[3]}}


def variant_line(torch, L, name, n, solid, precision, steps, flush):
    from sunlightlb_gb300 import workloads as W
    lb = L.newlb(n, n, n, "null")
    lb.precision = precision
    lb.tau = TAU
    lb.stokes_flow = 1
    W.insert_solid(L, lb, solid)
    L.flattenobj(lb)
    L.syncobjs(lb)
    L.addbf(lb, FORCE, 0.0, 0.0)
    L.lbsteps(lb, 2)
    ms = time_steps(torch, L, lb, steps, 3, Flusher(torch) if flush else None)
    mean = sum(ms) / len(ms)
    nodes = lb.nnodes
    peak, kind = measured_peak()
    gbs = BYTES_PER_UPDATE[precision] * nodes / (mean * 1e-3) / 1e9
    out = {"lattice": n, "populations": {0: "fp64", 1: "fp32", 2: "fp32 moments + bf16 paired deviations"}[precision],
           "MLUPS": round(nodes / (mean * 1e-3) / 1e6, 1), "bytes_per_update": BYTES_PER_UPDATE[precision],
           "ms_per_step": round(mean, 5), "hbm_gbs": round(gbs, 1), "frac_of_measured_hbm": round(gbs / peak, 4),
           "l2": "flushed" if flush else "lattice larger than L2", "tuning": tuning(L, lb)}
    L.freelb(lb)
    return name, out


def permeability_run(torch, L, solid, precision, tol, maxsteps):
    """Packed bed to convergence (checks every 100 steps until the relative
    change of the mean flow is below tol): update steps, wall time and the
    Darcy constant k = vmeanx * eta / b."""
    from sunlightlb_gb300 import workloads as W
    lb = L.newlb(N_SIDE, N_SIDE, N_SIDE, "null")
    lb.precision = precision
    lb.tau = TAU
    lb.stokes_flow = 1
    W.insert_solid(L, lb, solid)
    L.flattenobj(lb)
    L.syncobjs(lb)
    L.addbf(lb, FORCE, 0.0, 0.0)
    L.lbsteps(lb, 2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    steps = L.lbconverge(lb, CHECK, tol, maxsteps)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    k = W.permeability(lb, FORCE)
    objs = lb.objects()
    drag = objs[0].frcx if objs else None
    L.freelb(lb)
    return {"steps": steps + 2, "wall_s": round(dt, 3), "k": k, "drag_x": drag, "converged": steps < maxsteps}


def run_mine(args):
    import numpy as np
    import torch
    import sunlightlb_gb300
    from sunlightlb_gb300 import workloads as W

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    L = sunlightlb_gb300.library()
    precision = {"fp64": 0, "fp32": 1, "bf16dev": 2}[args.precision]
    prec_name = args.precision
    spheres, solid = W.rsa_packing(N_SIDE, PHI, RMIN, RMAX, SEED)
    lb = build_lattice(L, precision, spheres, solid)
    nodes = lb.nnodes

    # -------- device-resident throughput: one step per timed iteration --------
    L.lbsteps(lb, 2)  # first device call: upload, autotune
    flusher = Flusher(torch)
    for _ in range(args.warmup):
        L.lbstep(lb)
    torch.cuda.synchronize()
    k0 = L.lbkernelcount()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        t0 = time.perf_counter()
        step_ms = time_steps(torch, L, lb, args.steps, 0, flusher)
        wall = time.perf_counter() - t0
    launches = L.lbkernelcount() - k0
    total_ms = sum(step_ms)
    value, ms_per_step = aggregate(total_ms, nodes, args.steps, world,
                                   torch.distributed if world > 1 else None, "cuda")
    if world > 1:
        torch.distributed.barrier()
    peak, peak_kind = measured_peak()
    achieved = BYTES_PER_UPDATE[precision] * nodes / (ms_per_step * 1e-3) / 1e9
    tune = tuning(L, lb)

    # -------- end-to-end through the public API with host buffers -------------
    e2e = run_e2e(L, precision, spheres, solid, args)

    # -------- other precisions and sizes of the same packing ------------------
    variants = {}
    if not args.no_variants and rank == 0:
        big = np.tile(solid, (2, 2, 2))  # 256^3, the 128^3 packing repeated periodically
        for name, n, sol, prec, flush in (("fp32_256", 256, big, 1, False),
                                          ("bf16dev_128", N_SIDE, solid, 2, True),
                                          ("bf16dev_256", 256, big, 2, False),
                                          ("fp64_128", N_SIDE, solid, 0, True)):
            k, v = variant_line(torch, L, name, n, sol, prec, min(args.steps, 30), flush)
            variants[k] = v

    perm = {}
    if not args.no_convergence and rank == 0:
        for name, prec in (("fp64", 0), ("fp32", 1), ("bf16dev", 2)):
            perm[name] = permeability_run(torch, L, solid, prec, 1e-8, args.max_converge_steps)
        if "fp64" in perm and perm["fp64"]["k"]:
            for name in perm:
                perm[name]["k_rel_error_vs_fp64"] = abs(perm[name]["k"] - perm["fp64"]["k"]) / abs(perm["fp64"]["k"])

    if rank != 0:
        return
    line = {
        "metric": "MLUPS (million lattice updates per second, all nodes), packed-bed lattice Boltzmann step",
        "value": round(value, 1),
        "unit": "MLUPS",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_per_step, 5),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": {0: "f64", 1: "f32", 2: "f32 arithmetic, bf16 paired-deviation storage"}[precision],
        "data": "synthetic seeded RSA sphere packing (the reference publishes no benchmark data set)",
        "config": dict(config(prec_name, "flushed between timed steps (256 MiB write, then read)"), autotune=tune),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                     "traffic": profile_traffic(prec_name),
                     "bytes_per_update": BYTES_PER_UPDATE[precision],
                     "kernel": "k_step_pair (paired-deviation update)" if precision == 2 else "k_step (fused AA update)"},
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "wall_s_timed": round(wall, 4),
        "variants": variants,
        "permeability": dict(perm, criterion="|d vmeanx| / vmeanx < 1e-8 between 100-step checks"),
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(spheres, solid, budget_s=args.cpu_seconds)
    print(json.dumps(line), flush=True)


def run_e2e(L, precision, spheres, solid, args):
    """MLUPS of check intervals run through the public API, host buffers:
    a fresh lattice whose populations come from the host (lbpush uploads
    them with the geometry and body force), intervals of 98 lbstep + measure
    (mean flow and drag read back each interval), populations read back."""
    import numpy as np
    import torch
    lb = build_lattice(L, precision, spheres, solid)
    n = lb.nnodes
    intervals = max(1, args.e2e_intervals)
    L.lbpull(lb)  # allocates the host mirror (zero populations)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    L.lbpush(lb)
    h2d = 15 * 8 * n + 4 * n + 3 * 8 * n  # populations (FP64), object map, body force arrays
    d2h = 0
    for _ in range(intervals):
        L.lbsteps(lb, CHECK - 2)
        L.measure(lb)
        _ = (lb.vmeanx, lb.step)
        d2h += 5 * 8 * 3 + 6 * 8  # three mean-flow sums and the object force/torque
    L.lbpull(lb)  # populations into the host buffer lb->a (FP64, reference order)
    pops = lb.array("a")
    d2h += pops.nbytes
    dt = time.perf_counter() - t0
    steps = intervals * CHECK
    return {"value": round(n * steps / dt / 1e6, 1), "unit": "MLUPS",
            "h2d_bytes_per_step": int(h2d / steps), "d2h_bytes_per_step": int(d2h / steps),
            "steps": steps, "note": "public C API: lbpush, lbsteps + measure per 100 steps, lbpull"}


def oracle_lib():
    from sunlightlb_gb300 import build as b
    from sunlightlb_gb300.binding import Library
    path = os.path.join(ROOT, "oracle", "liboracle.so")
    if not os.path.exists(path):
        b.build_oracle(with_reference=False)
    return Library(path, extended=True)


def _cpu_worker(spheres, solid, budget_s, out, slot):
    L = oracle_lib()
    from sunlightlb_gb300 import workloads as W
    lb = L.newlb(N_SIDE, N_SIDE, N_SIDE, "null")
    lb.tau = TAU
    lb.stokes_flow = 1
    W.insert_solid(L, lb, solid)
    L.flattenobj(lb)
    L.syncobjs(lb)
    L.addbf(lb, FORCE, 0.0, 0.0)
    L.lbstep(lb)
    steps = 0
    t0 = time.perf_counter()
    while steps < 2 or time.perf_counter() - t0 < budget_s:
        L.lbstep(lb)
        steps += 1
    out[slot] = (steps, time.perf_counter() - t0, lb.nnodes)


def cpu_baseline(spheres, solid, budget_s=10.0, threads=1):
    """The CPU oracle (restatement of the reference's single-threaded C
    update, strict FP64) on host cores; one lattice per thread."""
    out = [None] * threads
    ts = [threading.Thread(target=_cpu_worker, args=(spheres, solid, budget_s, out, s)) for s in range(threads)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    total = sum(s * n for s, _, n in out) / max(dt for _, dt, _ in out) / 1e6
    steps = [s for s, _, _ in out]
    return {"value": round(total, 3), "unit": "MLUPS", "cores": threads, "kind": "port",
            "sample": f"{min(steps)}-{max(steps)} FP64 update steps per thread of the same {N_SIDE}^3 packing "
                      f"({threads} lattice(s), about {budget_s:g} s of CPU time each)"}


def run_reference(args):
    """The reference's CPU implementation of the path (the oracle port of its
    C code: a build of the reference needs its sources, which this machine
    may not hold) on every host core: one lattice per thread, aggregate MLUPS
    per step."""
    from sunlightlb_gb300 import workloads as W
    world, rank, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    spheres, solid = W.rsa_packing(N_SIDE, PHI, RMIN, RMAX, SEED)
    budget = max(5.0, min(60.0, args.cpu_seconds * 2))
    cb = cpu_baseline(spheres, solid, budget_s=budget, threads=threads)
    line = {
        "impl": "reference",
        "metric": "MLUPS (million lattice updates per second, all nodes), packed-bed lattice Boltzmann step",
        "value": cb["value"], "unit": "MLUPS", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic seeded RSA sphere packing",
        "config": config("fp64 (CPU reference code)", "n/a (CPU)"),
        "cpu_baseline": cb,
        "e2e": {"value": cb["value"], "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---- flow + passive scalar in a large packed bed ----------------------------

TRACER_PHI, TRACER_RMIN, TRACER_RMAX, TRACER_SEED = 0.35, 6.0, 12.0, 4
TRACER_ALPHA, TRACER_ADPROB = 0.5, 0.01
# bytes per tracer update: 15 FP32 populations + p in, rho, p out
# bytes per tracer update on the frozen flow: FP32 tracers apply 15 FP32
# stencil coefficients per node and read and write p as two FP32 words
# (high and low part; the coefficients are built once from the flow); FP64
# tracers read 15 FP32 populations, p and rho (FP64) and write p
TRACER_BYTES = {1: 60 + 4 * 4, 0: 60 + 3 * 8}


def time_tracer(torch, L, lb, mp, steps):
    """Device time (ms) of `steps` mpstep calls, CUDA events on the
    lattice's stream."""
    stream = torch.cuda.ExternalStream(L.lbgetstream(lb))
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        a.record(stream)
        for _ in range(steps):
            L.mpstep(mp)
        b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b)


def cpu_tracer_baseline(budget_s):
    """The oracle's FP64 tracer update (restatement of the reference's
    mpstep) on one host core, on a 64^3 crop of the same kind of packing."""
    from sunlightlb_gb300 import workloads as W
    L = oracle_lib()
    lb, _ = W.large_bed(L, 64, TRACER_PHI, TRACER_RMIN, TRACER_RMAX, TRACER_SEED, precision=0)
    L.addbf(lb, 1e-5, 0.0, 0.0)
    for _ in range(20):
        L.lbstep(lb)
    mp = L.newmp(lb, "null")
    mp.alpha = TRACER_ALPHA
    mp.adprob = TRACER_ADPROB
    L.mpinit(mp)
    L.adall(mp)
    steps, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < budget_s:
        L.mpwall(mp, "x", 0, 1.0)
        L.mpstep(mp)
        steps += 1
    dt = time.perf_counter() - t0
    return {"value": round(lb.nnodes * steps / dt / 1e6, 3), "unit": "MLUPS", "cores": 1, "kind": "port",
            "sample": f"{steps} FP64 tracer updates (with the source plane) of a 64^3 packing of the same kind"}


def run_tracer(args):
    """Large packed bed, flow at pore Reynolds number about 1, then a passive
    scalar with partial adsorption carried through the frozen flow."""
    import torch
    import sunlightlb_gb300
    from sunlightlb_gb300 import workloads as W

    world, rank, local = dist_env()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    L = sunlightlb_gb300.library()
    n = args.side
    t0 = time.perf_counter()
    lb, spheres = W.large_bed(L, n, TRACER_PHI, TRACER_RMIN, TRACER_RMAX, TRACER_SEED, precision=1)
    t_build = time.perf_counter() - t0
    diameter = 2.0 * statistics.mean(r for r, _, _, _ in spheres)
    nodes = lb.nnodes
    L.lbsteps(lb, 2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    flow = W.calibrated_flow(L, lb, diameter, re_target=1.0, maxsteps=args.max_converge_steps)
    torch.cuda.synchronize()
    flow["wall_s"] = round(time.perf_counter() - t0, 2)
    flow["fluid_fraction"] = L.countfluid(lb) / nodes
    peak, peak_kind = measured_peak()
    with Clocks(local) as clk:
        ms = time_steps(torch, L, lb, 60, 3)
    step_ms = statistics.mean(ms)
    flow_kernel = {"MLUPS": round(nodes / (step_ms * 1e-3) / 1e6, 1), "ms_per_step": round(step_ms, 4),
                   "hbm_gbs": round(BYTES_PER_UPDATE[1] * nodes / (step_ms * 1e-3) / 1e9, 1),
                   "frac_of_measured_hbm": round(BYTES_PER_UPDATE[1] * nodes / (step_ms * 1e-3) / 1e9 / peak, 4),
                   "bytes_per_update": BYTES_PER_UPDATE[1], "clocks": clk.summary()}
    tracers = {}
    for name, prec, nsteps in (("fp32", 1, args.tracer_steps), ("fp64", 0, args.fp64_tracer_steps)):
        if nsteps <= 0:
            continue
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        mp, curve, bals = W.tracer_breakthrough(L, lb, nsteps, precision=prec, alpha=TRACER_ALPHA,
                                                adprob=TRACER_ADPROB, sample_every=args.sample_every)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        kms = time_tracer(torch, L, lb, mp, 50) / 50
        gbs = TRACER_BYTES[prec] * nodes / (kms * 1e-3) / 1e9
        _, fl, ad, al, inj = bals[-1]
        tracers[name] = {
            "steps": nsteps, "wall_s": round(wall, 2),
            "MLUPS_with_planes_and_samples": round(nodes * nsteps / wall / 1e6, 1),
            "kernel": {"MLUPS": round(nodes / (kms * 1e-3) / 1e6, 1), "ms_per_step": round(kms, 4),
                       "hbm_gbs": round(gbs, 1), "frac_of_measured_hbm": round(gbs / peak, 4),
                       "bytes_per_update": TRACER_BYTES[prec],
                       "update": "stencil coefficients of the frozen flow" if prec == 1 else
                                 "terms from the populations, the reference's summation order"},
            "balance": {"fluid": fl, "adsorbed": ad, "all": al, "injected": inj,
                        "rel_error": (al - inj) / inj if inj else None},
            "breakthrough": curve,
            "balances": bals,
        }
        L.freemp(mp)
    if "fp32" in tracers and "fp64" in tracers:
        c32 = dict(tracers["fp32"]["breakthrough"])
        c64 = dict(tracers["fp64"]["breakthrough"])
        b32 = {b[0]: b for b in tracers["fp32"]["balances"]}
        b64 = {b[0]: b for b in tracers["fp64"]["balances"]}
        common = sorted(set(c32) & set(c64))
        last = common[-1] if common else None
        tracers["fp32_vs_fp64"] = {
            "compared_at_steps": [common[0], last] if common else None,
            "breakthrough_max_abs_diff": max(abs(c32[s] - c64[s]) for s in common) if common else None,
            "adsorbed_rel_diff": abs(b32[last][2] - b64[last][2]) / max(abs(b64[last][2]), 1e-300) if last else None,
            "held_rel_diff": abs(b32[last][3] - b64[last][3]) / max(abs(b64[last][3]), 1e-300) if last else None}
    line = {
        "workload": f"flow and passive scalar, periodic {n}^3 packed bed",
        "metric": "MLUPS of the flow and tracer kernels; breakthrough and tracer mass balance",
        "config": {"lattice": [n, n, n], "solid_fraction_target": TRACER_PHI,
                   "radii": [TRACER_RMIN, TRACER_RMAX], "seed": TRACER_SEED, "spheres": len(spheres),
                   "mean_diameter": diameter, "tau": 1.0, "flow": "Navier-Stokes (stokes_flow = 0), FP32 populations",
                   "tracer_alpha": TRACER_ALPHA, "adsorption_probability": TRACER_ADPROB,
                   "source": "mpwall x = 0, p = 1, and absorbing mpwall x = side - 1, p = 0, re-set before every update",
                   "breakthrough_plane": "x = side - 2 (mean over its fluid nodes)"},
        "build_s": round(t_build, 1), "flow": flow, "flow_kernel": flow_kernel, "tracer": tracers,
        "measured_peak_gbs": peak, "peak_kind": peak_kind,
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_tracer_baseline(args.cpu_seconds)
    print(json.dumps(line), flush=True)
    L.freelb(lb)


# ---- batched ensemble of small moving-sphere domains ------------------------

BATCH_SIDES = (24, 32, 40, 48, 56, 64)
BATCH_RMIN, BATCH_RMAX, BATCH_SPEED, BATCH_SEED = 3.0, 6.0, 1e-3, 2


def batch_domains(ndom, seed=BATCH_SEED):
    """Seeded domains: (side, radius, centre, velocity)."""
    from sunlightlb_gb300 import workloads as W
    rng = W.SplitMix64(seed)
    out = []
    for _ in range(ndom):
        side = BATCH_SIDES[min(len(BATCH_SIDES) - 1, int(rng.uniform(0.0, len(BATCH_SIDES))))]
        rad = rng.uniform(BATCH_RMIN, BATCH_RMAX)
        centre = [rng.uniform(0.0, side) for _ in range(3)]
        vel = [BATCH_SPEED * c for c in rng.unit_vector()]
        out.append((side, rad, centre, vel))
    return out


def build_domain(L, side, rad, centre, vel, precision=1):
    """Periodic cube with one sphere (and its periodic images, merged into
    one object) translating at vel: fixed node map, wall velocity spread to
    the solid nodes (vspread), Stokes flow, tau = 1."""
    from sunlightlb_gb300 import workloads as W
    lb = L.newlb(side, side, side, "null")
    if L.extended:
        lb.precision = precision
    lb.tau = 1.0
    lb.stokes_flow = 1
    lb.objects_moving = 1
    for c in W.images((side, side, side), rad, centre):
        L.insertsph(lb, rad, c[0], c[1], c[2])
    obj = L.flattenobj(lb)
    obj.velx, obj.vely, obj.velz = vel
    L.syncobjs(lb)
    L.vspread(lb)
    return lb


def drag(lb):
    o = lb.objects()[0]
    return [o.frcx, o.frcy, o.frcz]


def _oracle_domain(spec, steps, out, slot):
    L = oracle_lib()
    lb = build_domain(L, *spec, precision=0)
    for _ in range(steps):
        L.lbstep(lb)
    L.measure(lb)
    out[slot] = drag(lb)


def run_batch(args):
    """Many independent moving-sphere domains: one persistent launch for
    all of them (batchsteps) against the same domains one at a time
    (lbsteps per domain), per-domain drag compared; a seeded subset against
    the CPU oracle (FP64)."""
    import torch
    import sunlightlb_gb300

    world, rank, local = dist_env()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    L = sunlightlb_gb300.library()
    specs = batch_domains(args.domains)
    nodes = sum(s[0] ** 3 for s in specs)
    steps = args.batch_steps
    t0 = time.perf_counter()
    batch = [build_domain(L, *sp) for sp in specs]
    alone = [build_domain(L, *sp) for sp in specs]
    t_build = time.perf_counter() - t0
    for lb in batch + alone:  # upload, first device use
        L.lbsteps(lb, 2)
    torch.cuda.synchronize()
    b = L.newbatch()
    for lb in batch:
        L.batchadd(b, lb)
    L.batchsteps(b, 2)  # set-up, warm-up
    for lb in alone:
        L.lbsteps(lb, 2)  # the same step count
    torch.cuda.synchronize()
    k0 = L.lbkernelcount()
    with Clocks(local) as clk:
        t0 = time.perf_counter()
        L.batchsteps(b, steps)
        torch.cuda.synchronize()
        t_batch = time.perf_counter() - t0
    launches = L.lbkernelcount() - k0
    t0 = time.perf_counter()
    for lb in alone:
        L.lbsteps(lb, steps)
        torch.cuda.synchronize()  # one domain at a time
    t_alone = time.perf_counter() - t0
    worst = 0.0
    drags = []
    for lb1, lb2 in zip(batch, alone):
        L.measure(lb1)
        L.measure(lb2)
        d1, d2 = drag(lb1), drag(lb2)
        drags.append(d1)
        worst = max(worst, max(abs(x - y) for x, y in zip(d1, d2)))
    # the other batch mode (one persistent launch, blocks owning whole
    # lattices), timed on the same lattices after the drag comparison
    psteps = max(2, steps // 10)
    L.batchmode(b, 1)
    L.batchsteps(b, 2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    L.batchsteps(b, psteps)
    torch.cuda.synchronize()
    t_pers = time.perf_counter() - t0
    peak, peak_kind = measured_peak()
    gbs = BYTES_PER_UPDATE[1] * nodes * steps / t_batch / 1e9
    line = {
        "workload": f"batched ensemble: {args.domains} periodic moving-sphere domains, sides {list(BATCH_SIDES)}",
        "metric": "MLUPS of all domains together, batched vs one domain at a time",
        "config": {"domains": args.domains, "cells": nodes, "steps": steps, "radii": [BATCH_RMIN, BATCH_RMAX],
                   "speed": BATCH_SPEED, "seed": BATCH_SEED, "tau": 1.0, "flow": "Stokes",
                   "populations": "fp32", "boundary": "moving-wall link bounce-back on the fixed node map (vspread)"},
        "build_s": round(t_build, 1),
        "batched": {"mode": "packed tiles, one launch per step, CUDA graph", "wall_s": round(t_batch, 3), "MLUPS": round(nodes * steps / t_batch / 1e6, 1),
                    "hbm_gbs": round(gbs, 1), "frac_of_measured_hbm": round(gbs / peak, 4),
                    "gpu_launches": launches, "clocks": clk.summary()},
        "batched_persistent_mode": {"steps": psteps, "wall_s": round(t_pers, 3),
                                    "MLUPS": round(nodes * psteps / t_pers / 1e6, 1)},
        "one_at_a_time": {"wall_s": round(t_alone, 3), "MLUPS": round(nodes * steps / t_alone / 1e6, 1)},
        "speedup": round(t_alone / t_batch, 2),
        "drag_max_abs_diff_batched_vs_one_at_a_time": worst,
        "measured_peak_gbs": peak, "peak_kind": peak_kind,
    }
    if args.cpu_subset > 0:
        # the smallest domains, FP64 on the CPU oracle, one thread each
        sub = sorted(range(len(specs)), key=lambda d: (specs[d][0], d))[:args.cpu_subset]
        out = [None] * len(sub)
        t0 = time.perf_counter()
        ts = [threading.Thread(target=_oracle_domain, args=(specs[d], steps + 4, out, n)) for n, d in enumerate(sub)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        t_cpu = time.perf_counter() - t0
        # the drag decays as the periodic fluid picks up the sphere's motion,
        # so differences are scaled by the Stokes drag 6 pi eta a |v|
        eta = 72.0 * (1.0 - 0.5) / 3.0
        rel = []
        for n, d in enumerate(sub):
            ref = out[n]
            scale = 6.0 * math.pi * eta * specs[d][1] * BATCH_SPEED
            rel.append(max(abs(x - y) for x, y in zip(drags[d], ref)) / scale)
        line["cpu_subset"] = {"domains": sub, "steps": steps + 4, "wall_s": round(t_cpu, 2), "cores": len(sub),
                              "MLUPS": round(sum(specs[d][0] ** 3 for d in sub) * (steps + 4) / t_cpu / 1e6, 2),
                              "kind": "port", "drag_max_diff_over_stokes_drag_gpu_fp32_vs_cpu_fp64": max(rel)}
    print(json.dumps(line), flush=True)
    L.freebatch(b)


# ---- learned warm start ------------------------------------------------------

WARM_SEED, WARM_FORCE = 3, 1e-6
WARM_CHECKS = (100, 50)  # permeability check intervals of the time-to-accuracy comparison
WARM_VARIANTS = ("velocity_only", "state_whole_force_shift")


def run_warmstart(args):
    """Train the encoder-decoder on converged flows of seeded 64^3 packings
    (labels from the solver's own batched lattices), then compare warm-started
    and plain permeability runs on held-out 128^3 packings."""
    import numpy as np
    import torch
    import sunlightlb_gb300
    from sunlightlb_gb300 import warmstart as WS

    world, rank, local = dist_env()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    L = sunlightlb_gb300.library()
    side, ev_side, force = args.warm_side, args.eval_side, WARM_FORCE
    specs = WS.packing_specs(args.train + args.eval, WARM_SEED)
    tr_specs, ev_specs = specs[:args.train], specs[args.train:]
    t0 = time.perf_counter()
    solids = [WS.packing(side, phi, sd) for phi, sd in tr_specs]
    t_pack = time.perf_counter() - t0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    fields, lsteps = WS.converged_flows(L, solids, force=force, tol=args.label_tol, maxsteps=args.label_maxsteps,
                                        density=True)
    torch.cuda.synchronize()
    t_labels = time.perf_counter() - t0
    masks = torch.as_tensor(np.stack(solids).astype(np.uint8), device="cuda")
    labels = torch.stack([WS.to_labels(f, (side, side, side)) for f in fields])
    del fields
    net = WS.UNet(L, side, side, side, batch=args.batch, seed=1)
    iters = max(1, args.epochs * args.train // args.batch)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    # each sample's loss relative to its own label energy (labels span more
    # than an order of magnitude with the solid fraction)
    sample_w = 1.0 / labels.pow(2).mean(dim=(1, 2, 3, 4)).clamp_min(1e-12)
    hist = WS.train(net, masks, labels, iters, lr=args.lr, seed=2, log_every=max(1, iters // 20), sample_w=sample_w,
                    lr_min=args.lr * 0.01)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    tc_status = net.status()
    # held-out packings at the evaluation size
    inf = WS.UNet(L, ev_side, ev_side, ev_side, batch=1, params=net.params)
    rows = []
    for phi, sd in ev_specs:
        solid = WS.packing(ev_side, phi, sd)
        traj = WS.permeability_run(L, solid, force)
        k_conv = traj[-1][1]
        sdev = torch.as_tensor(solid.astype(np.uint8), device="cuda")
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        u, drho = WS.predict_state(inf, sdev, force, WS.ETA_TAU1)
        torch.cuda.synchronize()
        t_inf = time.perf_counter() - t0
        row = {"phi": round(phi, 4), "k": k_conv, "plain_converged_steps": traj[-1][0], "inference_s": round(t_inf, 4)}
        # time to k within 1e-4, the permeability measured every `check` steps
        # in both arms (the plain arm from rest, the warm arm from the
        # prediction, inference included)
        for check in WARM_CHECKS:
            tp = traj if check == 100 else WS.permeability_run(L, solid, force, k_ref=k_conv, check=check)
            plain = WS.first_within(tp, k_conv, 1e-4)
            trajw = WS.permeability_run(L, solid, force, k_ref=k_conv, warm_u=u, warm_drho=drho, check=check)
            hitw = WS.first_within(trajw, k_conv, 1e-4)
            row[f"check{check}"] = {"plain_steps": plain[0] if plain else None,
                                    "plain_wall_s": round(plain[1], 4) if plain else None,
                                    "warm_steps": hitw[0] if hitw else None,
                                    "warm_wall_s": round(hitw[1] + t_inf, 4) if hitw else None}
            if check == 100:
                row["warm_k_error_first_check"] = abs(trajw[0][1] - k_conv) / abs(k_conv)
                row["plain_k_error_first_check"] = abs(traj[0][1] - k_conv) / abs(k_conv)
        # the same network set without its density (rho = rho0, u - F / rho0,
        # the best shift without a density) and with its density but the
        # whole-force shift (the warm start sets u - F / (2 rho0) and rho)
        for name in WARM_VARIANTS:
            if name == "velocity_only":
                vs, ds = WS.predict_velocity(inf, sdev, force, WS.ETA_TAU1, force_shift=1.0), None
            else:
                vs, ds = WS.predict_state(inf, sdev, force, WS.ETA_TAU1, force_shift=1.0)
            hs = WS.first_within(WS.permeability_run(L, solid, force, k_ref=k_conv, warm_u=vs, warm_drho=ds, check=50),
                                 k_conv, 1e-4)
            row[f"check50_{name}"] = {"warm_steps": hs[0] if hs else None,
                                      "warm_wall_s": round(hs[1] + t_inf, 4) if hs else None}
        rows.append(row)

    def summary(check):
        ok = [r[f"check{check}"] for r in rows if r[f"check{check}"]["plain_wall_s"] and r[f"check{check}"]["warm_wall_s"]]
        speed = [r["plain_wall_s"] / r["warm_wall_s"] for r in ok]
        steps_ratio = [r["plain_steps"] / r["warm_steps"] for r in ok]
        return {"check_every": check, "samples": len(ok),
                "wall_speedup_mean": float(np.mean(speed)) if speed else None,
                "wall_speedup_median": float(np.median(speed)) if speed else None,
                "steps_ratio_mean": float(np.mean(steps_ratio)) if steps_ratio else None,
                "warm_faster_fraction": float(np.mean([s > 1 for s in speed])) if speed else None,
                "plain_wall_total_s": round(float(sum(r["plain_wall_s"] for r in ok)), 3),
                "warm_wall_total_s": round(float(sum(r["warm_wall_s"] for r in ok)), 3)}

    line = {
        "workload": f"learned warm start: U-Net trained on {args.train} converged {side}^3 packings, "
                    f"evaluated on {args.eval} held-out {ev_side}^3 packings",
        "metric": "wall time and steps to permeability within 1e-4 of the plain converged value, warm vs plain",
        "config": {"train_side": side, "eval_side": ev_side, "train_samples": args.train, "eval_samples": args.eval,
                   "phi": [0.1, 0.5], "radii": [3.0, 8.0], "spheres_overlap": True, "force": force, "tau": 1.0,
                   "widths": list(net.widths), "batch": args.batch, "iterations": iters,
                   "lr": f"{args.lr:g} -> {args.lr * 0.01:g} (half cosine)",
                   "input": "solid mask + periodic wall distance d/5 and (d/5)^2 (d capped at 5)",
                   "output": "velocity and density deviation; set with u - F / (2 rho0) and rho0 + drho",
                   "labels": f"FP32 populations, converged to |d vmeanx|/vmeanx < {args.label_tol:g} per 200 steps",
                   "precision": "BF16 weights/activations, FP32 accumulation (tcgen05)"},
        "packing_s": round(t_pack, 1), "labels_s": round(t_labels, 1),
        "label_steps": {"mean": float(np.mean(lsteps)), "max": int(np.max(lsteps))},
        "train_s": round(t_train, 1), "train_ms_per_iteration": round(1e3 * t_train / iters, 2),
        "loss": hist, "tc_status": tc_status,
        "eval": rows,
        "summary": summary(WARM_CHECKS[-1]),
        "summary_by_check": [summary(c) for c in WARM_CHECKS],
        "variants_at_check50": {
            name: {"wall_speedup_mean": float(np.mean([r["check50"]["plain_wall_s"] / r[f"check50_{name}"]["warm_wall_s"]
                                                       for r in rows if r[f"check50_{name}"]["warm_wall_s"]])),
                   "steps_ratio_mean": float(np.mean([r["check50"]["plain_steps"] / r[f"check50_{name}"]["warm_steps"]
                                                      for r in rows if r[f"check50_{name}"]["warm_steps"]]))}
            for name in WARM_VARIANTS},
    }
    print(json.dumps(line), flush=True)
    if args.save_weights:
        torch.save({n: {k: v.cpu() for k, v in p.items() if k in ("w", "b")} for n, p in net.params.items()},
                   args.save_weights)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="mine", choices=["mine", "reference"])
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64", "bf16dev"])
    ap.add_argument("--e2e-intervals", type=int, default=20)
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--no-convergence", action="store_true")
    ap.add_argument("--max-converge-steps", type=int, default=60000)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="packed", choices=["packed", "tracer", "batch", "warmstart"],
                    help="packed: the 128^3 packed-bed step (default); tracer: large bed, flow + passive "
                         "scalar; batch: many small moving-sphere domains in one launch")
    ap.add_argument("--domains", type=int, default=512, help="batch workload: number of domains")
    ap.add_argument("--batch-steps", type=int, default=20000)
    ap.add_argument("--cpu-subset", type=int, default=8, help="batch workload: domains checked on the CPU oracle")
    ap.add_argument("--train", type=int, default=2000, help="warmstart workload: training packings")
    ap.add_argument("--eval", type=int, default=100, help="warmstart workload: held-out packings")
    ap.add_argument("--epochs", type=int, default=10)
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--warm-side", type=int, default=64)
    ap.add_argument("--eval-side", type=int, default=128)
    ap.add_argument("--label-tol", type=float, default=1e-7)
    ap.add_argument("--label-maxsteps", type=int, default=20000)
    ap.add_argument("--save-weights", default="")
    ap.add_argument("--side", type=int, default=512, help="tracer workload: lattice side")
    ap.add_argument("--tracer-steps", type=int, default=50000)
    ap.add_argument("--fp64-tracer-steps", type=int, default=10000)
    ap.add_argument("--sample-every", type=int, default=500)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "tracer":
        run_tracer(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "warmstart":
        run_warmstart(args)
    else:
        run_mine(args)


if __name__ == "__main__":
    main()
