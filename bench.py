"""Benchmark of the GB300 SunlightLB update step.

Headline workload (the large packed bed): periodic 512^3 lattice, seeded
random sequential addition of non-overlapping spheres with radius uniform in
[6, 12] up to lattice solid fraction 0.35 (23,309 spheres), fixed objects
with link bounce-back, Navier-Stokes collision (stokes_flow = 0), tau = 1
(viscosity 1/6), body force 1e-6 along x, FP32 populations.  A step is one
lattice Boltzmann update (bounce-back, streaming and collision of every
node) of the whole lattice.

Metric: million lattice updates per second (all nodes, fluid and solid, as
the reference's own fwrstats counts them, src/lbmisc.c:264-274).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl mine|reference]

Under torchrun each rank advances its own replica of the lattice (the single
lattice is not split across GPUs); value is the sum over ranks of the nodes
updated divided by the slowest rank's time.

The JSON line carries:
  value      device-resident throughput, CUDA events around each step on the
             lattice's stream (the populations, 8 GB, are larger than L2);
  e2e        the same metric through the public C API with host buffers:
             populations, geometry and body force uploaded from the host, the
             steps run as check intervals (98 lbstep + measure, which reads
             the mean flow and the drag back), populations read back at the
             end; e2e_fp64 the same with FP64 populations (the reference's
             own precision);
  roofline   achieved HBM GB/s of the fused step kernel against the measured
             copy bandwidth (120 algorithmic bytes per FP32 node update);
  variants   other precisions and sizes (128^3 / 256^3 packings, FP64,
             BF16 paired deviations) and the permeability of the 128^3
             packing to convergence in FP64, FP32 and BF16;
  legs       compact runs of the other workloads: batched vs one-at-a-time
             moving-sphere domains, flow + passive scalar with partial
             adsorption on a 256^3 bed, and the learned warm start against
             the plain start on held-out 128^3 packings;
  cpu_baseline  the CPU restatement of the reference's update (the oracle,
             compiled with the reference's shipped -O3 -ffast-math flags,
             FP32 = the reference's -D_SINGLE build and FP64 = its default)
             on every host core, one 128^3 block of the same packing per
             core, on a time-bounded sample of steps.

--impl reference times that CPU restatement alone on the same workload
(FP32, and FP64 beside it), one 128^3 block of the 512^3 packing per host
core, W warm-up and K timed steps per core.  --workload tracer / batch /
warmstart run the full-size forms of the legs.
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

# headline: the large packed bed
HEAD_N, HEAD_PHI, HEAD_RMIN, HEAD_RMAX, HEAD_SEED = 512, 0.35, 6.0, 12.0, 4
HEAD_STOKES = 0
# the 128^3 packed bed of the permeability runs and of the smaller variants
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
CPU_BLOCK = 128                       # side of the block of the packing one CPU core advances


def head_workload():
    return (f"packed bed, periodic {HEAD_N}^3, RSA spheres r~U[{HEAD_RMIN:g},{HEAD_RMAX:g}] to solid fraction "
            f"{HEAD_PHI}, Navier-Stokes, body force {FORCE:g} along x, tau {TAU:g}")


def config(prec_name, l2):
    return {"workload": head_workload(), "lattice": [HEAD_N] * 3, "populations": prec_name, "seed": HEAD_SEED,
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


def profile_traffic(prec_name, n=None):
    """DRAM bytes per launch of the fused step (mean of the odd and even
    step) at an n^3 lattice from the committed ncu summary
    profiles/lb_step_<n>.md, line 'traffic_per_launch_<precision>: <bytes>'."""
    p = os.path.join(ROOT, "profiles", f"lb_step_{n or HEAD_N}.md")
    try:
        with open(p) as f:
            for line in f:
                key = f"traffic_per_launch_{prec_name}:"
                if line.strip().startswith(key):
                    return int(float(line.split(":", 1)[1].split()[0]))
    except Exception:
        pass
    return None


def make_lattice(L, solid, precision, stokes=1, force=FORCE, tau=TAU):
    """A periodic lattice whose solid nodes are `solid` (one object), body
    force along x."""
    from sunlightlb_gb300 import workloads as W
    n = solid.shape
    lb = L.newlb(n[0], n[1], n[2], "null")
    lb.precision = precision
    lb.tau = tau
    lb.stokes_flow = stokes
    W.insert_solid(L, lb, solid)
    L.flattenobj(lb)
    L.syncobjs(lb)
    L.addbf(lb, force, 0.0, 0.0)
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


def time_steps(torch, L, lb, steps, warmup, flusher=None, kinds=None):
    """Per-step device times (ms) of `steps` lbstep calls, CUDA events on
    the lattice's own stream, optional L2 flush before each timed step.
    With a list `kinds`, appends per step whether it was the pull-and-push
    update (the layout before it was the one an even update leaves)."""
    stream = torch.cuda.ExternalStream(L.lbgetstream(lb))
    for _ in range(warmup):
        L.lbstep(lb)
    torch.cuda.synchronize()
    if kinds is not None:
        first = L.lblayout(lb) == 1
        kinds.extend((first if s % 2 == 0 else not first) for s in range(steps))
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


PREC_NAMES = {0: "fp64", 1: "fp32", 2: "fp32 moments + bf16 paired deviations"}


def variant_line(torch, L, n, solid, precision, steps, flush, stokes=1):
    lb = make_lattice(L, solid, precision, stokes=stokes)
    L.lbsteps(lb, 2)
    kinds = []
    ms = time_steps(torch, L, lb, steps, 3, Flusher(torch) if flush else None, kinds)
    mean = sum(ms) / len(ms)
    split = {}
    for name, want in (("pull_push", True), ("local", False)):
        sel = [m for m, k in zip(ms, kinds) if k == want]
        if sel:
            split[name] = round(statistics.mean(sel), 5)
    nodes = lb.nnodes
    peak, _ = measured_peak()
    gbs = BYTES_PER_UPDATE[precision] * nodes / (mean * 1e-3) / 1e9
    out = {"lattice": n, "populations": PREC_NAMES[precision], "collision": "Stokes" if stokes else "Navier-Stokes",
           "MLUPS": round(nodes / (mean * 1e-3) / 1e6, 1), "bytes_per_update": BYTES_PER_UPDATE[precision],
           "ms_per_step": round(mean, 5), "ms_per_step_by_update": split if precision != 2 else None,
           "hbm_gbs": round(gbs, 1), "frac_of_measured_hbm": round(gbs / peak, 4),
           "l2": "flushed" if flush else "lattice larger than L2", "tuning": tuning(L, lb)}
    L.freelb(lb)
    return out


def permeability_run(torch, L, solid, precision, tol, maxsteps):
    """Packed bed to convergence (checks every 100 steps until the relative
    change of the mean flow is below tol): update steps, wall time and the
    Darcy constant k = vmeanx * eta / b."""
    from sunlightlb_gb300 import workloads as W
    lb = make_lattice(L, solid, precision, stokes=1)
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
    t0 = time.perf_counter()
    _, solid = W.rsa_packing(HEAD_N, HEAD_PHI, HEAD_RMIN, HEAD_RMAX, HEAD_SEED)
    t_pack = time.perf_counter() - t0
    lb = make_lattice(L, solid, precision, stokes=HEAD_STOKES)
    nodes = lb.nnodes

    # -------- device-resident throughput: one step per timed iteration --------
    L.lbsteps(lb, 2)  # first device call: upload, autotune
    for _ in range(args.warmup):
        L.lbstep(lb)
    torch.cuda.synchronize()
    k0 = L.lbkernelcount()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    kinds = []
    with Clocks(local) as clk:
        t0 = time.perf_counter()
        step_ms = time_steps(torch, L, lb, args.steps, 0, None, kinds)
        wall = time.perf_counter() - t0
    by_kind = {"pull_push": [m for m, k in zip(step_ms, kinds) if k],
               "local": [m for m, k in zip(step_ms, kinds) if not k]}
    launches = L.lbkernelcount() - k0
    total_ms = sum(step_ms)
    value, ms_per_step = aggregate(total_ms, nodes, args.steps, world,
                                   torch.distributed if world > 1 else None, "cuda")
    if world > 1:
        torch.distributed.barrier()
    peak, peak_kind = measured_peak()
    achieved = BYTES_PER_UPDATE[precision] * nodes / (ms_per_step * 1e-3) / 1e9
    tune = tuning(L, lb)
    L.freelb(lb)

    # -------- end-to-end through the public API with host buffers -------------
    e2e = run_e2e(L, precision, solid, args.e2e_intervals)
    e2e64 = run_e2e(L, 0, solid, args.e2e_fp64_intervals) if precision != 0 and args.e2e_fp64_intervals > 0 else None

    # -------- other precisions and sizes --------------------------------------
    variants = {}
    perm = {}
    legs = {}
    if rank == 0:
        _, small = W.rsa_packing(N_SIDE, PHI, RMIN, RMAX, SEED)
        if not args.no_variants:
            big = np.tile(small, (2, 2, 2))  # 256^3, the 128^3 packing repeated periodically
            nv = min(args.steps, 30)
            for name, n, sol, prec, flush, stokes, k in (
                    ("fp32_128", N_SIDE, small, 1, True, 1, nv),
                    ("fp32_256", 256, big, 1, False, 1, nv),
                    ("bf16dev_128", N_SIDE, small, 2, True, 1, nv),
                    ("bf16dev_256", 256, big, 2, False, 1, nv),
                    ("bf16dev_512", HEAD_N, solid, 2, False, HEAD_STOKES, nv),
                    ("fp64_128", N_SIDE, small, 0, True, 1, nv),
                    ("fp64_512", HEAD_N, solid, 0, False, HEAD_STOKES, 5)):
                variants[name] = variant_line(torch, L, n, sol, prec, k, flush, stokes=stokes)
        if not args.no_convergence:
            for name, prec in (("fp64", 0), ("fp32", 1), ("bf16dev", 2)):
                perm[name] = permeability_run(torch, L, small, prec, 1e-8, args.max_converge_steps)
            if "fp64" in perm and perm["fp64"]["k"]:
                for name in perm:
                    perm[name]["k_rel_error_vs_fp64"] = abs(perm[name]["k"] - perm["fp64"]["k"]) / abs(perm["fp64"]["k"])
        if not args.no_legs:
            legs["batch"] = batch_leg(torch, L, args)
            legs["tracer"] = tracer_leg(torch, L, args)
            legs["warmstart"] = warm_leg(torch, L, args)

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
        "config": dict(config(prec_name, f"not flushed: the populations ({BYTES_PER_UPDATE[precision] // 2 * nodes / 1e9:.1f} GB) "
                                         "are larger than L2"), autotune=tune, packing_s=round(t_pack, 2)),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                     "traffic": profile_traffic(prec_name),
                     "bytes_per_update": BYTES_PER_UPDATE[precision],
                     "kernel": "k_step_pair (paired-deviation update)" if precision == 2 else "k_step (fused AA update)"},
        "e2e": e2e,
        "e2e_fp64": e2e64,
        "ms_per_step_by_update": {k: round(statistics.mean(v), 5) for k, v in by_kind.items() if v},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "wall_s_timed": round(wall, 4),
        "variants": variants,
        "permeability": dict(perm, lattice=N_SIDE, criterion="|d vmeanx| / vmeanx < 1e-8 between 100-step checks"),
        "legs": legs,
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(solid, budget_s=args.cpu_seconds)
    print(json.dumps(line), flush=True)


def run_e2e(L, precision, solid, intervals):
    """MLUPS of check intervals run through the public API, host buffers:
    a fresh lattice whose populations come from the host (lbpush uploads
    them with the geometry and body force), intervals of 98 lbstep + measure
    (mean flow and drag read back each interval), populations read back."""
    import torch
    lb = make_lattice(L, solid, precision, stokes=HEAD_STOKES)
    n = lb.nnodes
    intervals = max(1, intervals)
    # device set-up and the autotuner's one-off timing of launch shapes (per
    # lattice shape and precision, once per process) before the timed region;
    # lbpush below makes the next call upload every host array again
    L.lbsteps(lb, 2)
    L.lbpull(lb)  # allocates the host mirror
    lb.array("a")[:] = 0.0  # a fresh state: every population at rest
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    L.lbpush(lb)
    h2d = 15 * 8 * n + 4 * n + 3 * 8 * n  # populations (FP64), object map, body force arrays
    d2h = 0
    t_first = None
    for it in range(intervals):
        L.lbsteps(lb, CHECK - 2)
        L.measure(lb)
        _ = (lb.vmeanx, lb.step)
        if it == 0:
            t_first = time.perf_counter() - t0  # upload + the first interval
        d2h += 5 * 8 * 3 + 6 * 8  # three mean-flow sums and the object force/torque
    t_steps = time.perf_counter() - t0
    L.lbpull(lb)  # populations into the host buffer lb->a (FP64, reference order)
    pops = lb.array("a")
    d2h += pops.nbytes
    dt = time.perf_counter() - t0
    steps = intervals * CHECK
    L.freelb(lb)
    return {"value": round(n * steps / dt / 1e6, 1), "unit": "MLUPS",
            "h2d_bytes_per_step": int(h2d / steps), "d2h_bytes_per_step": int(d2h / steps),
            "steps": steps, "populations": PREC_NAMES[precision], "wall_s": round(dt, 3),
            "wall_breakdown_s": {"upload_and_first_interval": round(t_first, 3),
                                 "other_intervals": round(t_steps - t_first, 3),
                                 "download": round(dt - t_steps, 3)},
            "note": "public C API: lbpush, lbsteps + measure per 100 steps, lbpull"}


def oracle_lib():
    from sunlightlb_gb300 import build as b
    from sunlightlb_gb300.binding import Library
    path = os.path.join(ROOT, "oracle", "liboracle.so")
    if not os.path.exists(path):
        b.build_oracle(with_reference=False)
    return Library(path, extended=True)


def timing_lib(bits):
    """The oracle's timing build (reference shipped flags), LBReal of `bits`."""
    import ctypes as C
    from sunlightlb_gb300 import build as b
    path = os.path.join(ROOT, "oracle", f"liboracle_time{bits}.so")
    if not os.path.exists(path):
        b.build_oracle(with_reference=False)
    lib = C.CDLL(path)
    f = lib.orc_time_steps
    f.restype = C.c_double
    f.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_double, C.c_int, C.c_int,
                  C.c_void_p]
    return f


def cpu_blocks(solid, count):
    """`count` distinct CPU_BLOCK^3 blocks of the packing (k fastest), each a
    periodic lattice of its own."""
    import numpy as np
    per = solid.shape[0] // CPU_BLOCK
    out = []
    for b in range(count):
        b %= per ** 3  # more cores than blocks: blocks repeat
        i, j, k = (b // (per * per)) % per, (b // per) % per, b % per
        out.append(np.ascontiguousarray(solid[i * CPU_BLOCK:(i + 1) * CPU_BLOCK, j * CPU_BLOCK:(j + 1) * CPU_BLOCK,
                                              k * CPU_BLOCK:(k + 1) * CPU_BLOCK], dtype=np.uint8))
    return out


def cpu_run(solid, bits, threads, warmup, steps):
    """Every thread advances its own block of the packing by warmup, then
    `steps` timed update steps (the oracle's timing build; ctypes releases
    the interpreter lock, so the threads run on separate cores).  Returns
    (MLUPS of all threads over the slowest thread's time, steps)."""
    import ctypes as C
    f = timing_lib(bits)
    blocks = cpu_blocks(solid, threads)
    out = [None] * threads

    def work(t):
        cs = C.c_double()
        out[t] = f(blocks[t].ctypes.data, CPU_BLOCK, CPU_BLOCK, CPU_BLOCK, TAU, HEAD_STOKES, FORCE, warmup, steps,
                   C.byref(cs))

    ts = [threading.Thread(target=work, args=(t,)) for t in range(threads)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    if any(v is None or v <= 0 for v in out):
        raise RuntimeError("CPU baseline failed")
    return threads * CPU_BLOCK ** 3 * steps / max(out) / 1e6


def cpu_steps_for(solid, bits, budget_s):
    """Steps per thread that take about budget_s (one calibration step)."""
    import ctypes as C
    f = timing_lib(bits)
    blk = cpu_blocks(solid, 1)[0]
    cs = C.c_double()
    dt = f(blk.ctypes.data, CPU_BLOCK, CPU_BLOCK, CPU_BLOCK, TAU, HEAD_STOKES, FORCE, 0, 1, C.byref(cs))
    return max(2, int(budget_s / max(dt, 1e-3)))


def cpu_baseline(solid, budget_s=10.0):
    """The CPU restatement of the reference's update under its shipped flags
    on every host core, FP32 (-D_SINGLE) and FP64, one 128^3 block of the
    packing per core, about budget_s of steps per core each."""
    threads = os.cpu_count() or 1
    res = {}
    for bits, name in ((32, "fp32"), (64, "fp64")):
        steps = cpu_steps_for(solid, bits, budget_s)
        res[name] = (round(cpu_run(solid, bits, threads, 1, steps), 3), steps)
    v32, s32 = res["fp32"]
    v64, s64 = res["fp64"]
    return {"value": v32, "unit": "MLUPS", "cores": threads, "kind": "port",
            "build": "oracle restatement of the reference's update, -O3 -ffast-math (the reference's shipped "
                     "flags), -D_SINGLE for FP32",
            "sample": f"{s32} FP32 / {s64} FP64 update steps per core of a distinct {CPU_BLOCK}^3 block of the "
                      f"same {HEAD_N}^3 packing (periodic), {threads} cores",
            "fp64": {"value": v64, "unit": "MLUPS", "cores": threads}}


def run_reference(args):
    """The reference's CPU implementation of the path (the oracle port of
    its C code under the reference's shipped flags: a build of the reference
    itself needs its sources, which this machine may not hold) on every host
    core, FP32 (the reference's -D_SINGLE build) as the value and FP64 (its
    default build) beside it; one 128^3 block of the headline packing per
    core, W warm-up and K timed steps per core."""
    from sunlightlb_gb300 import workloads as W
    world, rank, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    _, solid = W.rsa_packing(HEAD_N, HEAD_PHI, HEAD_RMIN, HEAD_RMAX, HEAD_SEED)
    v32 = cpu_run(solid, 32, threads, args.warmup, args.steps)
    v64 = cpu_run(solid, 64, threads, args.warmup, args.steps)
    sample = (f"{args.warmup} warm-up + {args.steps} timed update steps per core, each core a distinct "
              f"{CPU_BLOCK}^3 block of the {HEAD_N}^3 packing (periodic), {threads} cores")
    line = {
        "impl": "reference",
        "metric": "MLUPS (million lattice updates per second, all nodes), packed-bed lattice Boltzmann step",
        "value": round(v32, 3), "unit": "MLUPS", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic seeded RSA sphere packing",
        "config": config("fp32 (the reference's -D_SINGLE build, on the CPU)", "n/a (CPU)"),
        "cpu_baseline": {"value": round(v32, 3), "unit": "MLUPS", "cores": threads, "kind": "port",
                         "build": "oracle restatement of the reference's update, -O3 -ffast-math, -D_SINGLE",
                         "sample": sample},
        "fp64": {"value": round(v64, 3), "unit": "MLUPS", "cores": threads,
                 "build": "the same restatement, LBReal double (the reference's default build)"},
        "e2e": {"value": round(v32, 3), "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
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


def tracer_result(torch, L, n, fp32_steps, fp64_steps, sample_every, maxsteps, kernel_steps=50):
    """Large packed bed, flow at pore Reynolds number about 1, then a passive
    scalar with partial adsorption carried through the frozen flow, in FP32
    and FP64 tracers; kernel rates, breakthrough and mass balance."""
    from sunlightlb_gb300 import workloads as W
    local = dist_env()[2]
    t0 = time.perf_counter()
    lb, spheres = W.large_bed(L, n, TRACER_PHI, TRACER_RMIN, TRACER_RMAX, TRACER_SEED, precision=1)
    t_build = time.perf_counter() - t0
    diameter = 2.0 * statistics.mean(r for r, _, _, _ in spheres)
    nodes = lb.nnodes
    L.lbsteps(lb, 2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    flow = W.calibrated_flow(L, lb, diameter, re_target=1.0, maxsteps=maxsteps)
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
    for name, prec, nsteps in (("fp32", 1, fp32_steps), ("fp64", 0, fp64_steps)):
        if nsteps <= 0:
            continue
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        mp, curve, bals = W.tracer_breakthrough(L, lb, nsteps, precision=prec, alpha=TRACER_ALPHA,
                                                adprob=TRACER_ADPROB, sample_every=sample_every)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        kms = time_tracer(torch, L, lb, mp, kernel_steps) / kernel_steps
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
    out = {
        "workload": f"flow and passive scalar, periodic {n}^3 packed bed",
        "config": {"lattice": [n, n, n], "solid_fraction_target": TRACER_PHI,
                   "radii": [TRACER_RMIN, TRACER_RMAX], "seed": TRACER_SEED, "spheres": len(spheres),
                   "mean_diameter": diameter, "tau": 1.0, "flow": "Navier-Stokes (stokes_flow = 0), FP32 populations",
                   "tracer_alpha": TRACER_ALPHA, "adsorption_probability": TRACER_ADPROB,
                   "source": "mpwall x = 0, p = 1, and absorbing mpwall x = side - 1, p = 0, re-set before every update",
                   "breakthrough_plane": "x = side - 2 (mean over its fluid nodes)"},
        "build_s": round(t_build, 1), "flow": flow, "flow_kernel": flow_kernel, "tracer": tracers,
        "measured_peak_gbs": peak, "peak_kind": peak_kind,
    }
    L.freelb(lb)
    return out


def run_tracer(args):
    import torch
    import sunlightlb_gb300
    world, rank, local = dist_env()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    L = sunlightlb_gb300.library()
    line = {"metric": "MLUPS of the flow and tracer kernels; breakthrough and tracer mass balance"}
    line.update(tracer_result(torch, L, args.side, args.tracer_steps, args.fp64_tracer_steps, args.sample_every,
                              args.max_converge_steps))
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_tracer_baseline(args.cpu_seconds)
    print(json.dumps(line), flush=True)


def tracer_leg(torch, L, args):
    """Compact form for the default line: 256^3 bed, 2000 FP32 and 2000
    FP64 tracer updates (mass balance and FP32 vs FP64)."""
    out = tracer_result(torch, L, args.leg_tracer_side, args.leg_tracer_steps, args.leg_tracer_steps, 500,
                        args.max_converge_steps)
    for t in ("fp32", "fp64"):
        if t in out["tracer"]:
            out["tracer"][t].pop("balances", None)
    return out


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
    obj.posx, obj.posy, obj.posz = centre  # flattenobj leaves the centroid of the (wrapped) nodes
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


def translate_all(L, lbs, specs, every):
    """Move every domain's sphere on by its velocity times `every` steps
    (lbtranslate: the node set re-rasterised on the GPU)."""
    for lb, (side, rad, centre, vel) in zip(lbs, specs):
        obj = lb.objects()[0]
        c = [(getattr(obj, a) + v * every) % side for a, v in zip(("posx", "posy", "posz"), vel)]
        L.lbtranslate(lb, obj, rad, *c)


def advance(L, lbs, specs, steps, every, batch=None):
    """steps update steps of the domains (one batch, or one domain at a
    time), the spheres translated every `every` steps (0: fixed nodes)."""
    import torch
    done = 0
    while done < steps:
        n = steps - done if every <= 0 else min(every, steps - done)
        if batch is not None:
            L.batchsteps(batch, n)
        else:
            for lb in lbs:
                L.lbsteps(lb, n)
                torch.cuda.synchronize()  # one domain at a time
        done += n
        if every > 0 and n == every:
            translate_all(L, lbs, specs, every)


def batch_result(torch, L, ndom, steps, cpu_subset=0, persistent=True, clocks=True, translate_every=0):
    """Many independent moving-sphere domains advanced together (batchsteps,
    packed tiles, one launch per step from a CUDA graph) against the same
    domains one at a time (lbsteps per domain), per-domain drag compared;
    optionally the other batch mode and a seeded subset against the CPU
    oracle (FP64).  With translate_every > 0 the spheres really move: every
    that many steps each is re-rasterised at its new centre (lbtranslate),
    in both arms (the CPU subset keeps fixed nodes)."""
    local = dist_env()[2]
    specs = batch_domains(ndom)
    nodes = sum(s[0] ** 3 for s in specs)
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
    clk = Clocks(local) if clocks else None
    if clk:
        clk.__enter__()
    t0 = time.perf_counter()
    advance(L, batch, specs, steps, translate_every, batch=b)
    torch.cuda.synchronize()
    t_batch = time.perf_counter() - t0
    if clk:
        clk.__exit__(None, None, None)
    launches = L.lbkernelcount() - k0
    t0 = time.perf_counter()
    advance(L, alone, specs, steps, translate_every)
    torch.cuda.synchronize()
    t_alone = time.perf_counter() - t0
    worst = 0.0
    drags = []
    for lb1, lb2 in zip(batch, alone):
        L.measure(lb1)
        L.measure(lb2)
        d1, d2 = drag(lb1), drag(lb2)
        drags.append(d1)
        worst = max(worst, max(abs(x - y) for x, y in zip(d1, d2)))
    peak, peak_kind = measured_peak()
    gbs = BYTES_PER_UPDATE[1] * nodes * steps / t_batch / 1e9
    out = {
        "config": {"domains": ndom, "sides": list(BATCH_SIDES), "cells": nodes, "steps": steps,
                   "radii": [BATCH_RMIN, BATCH_RMAX], "speed": BATCH_SPEED, "seed": BATCH_SEED, "tau": 1.0,
                   "flow": "Stokes", "populations": "fp32",
                   "boundary": "moving-wall link bounce-back (vspread)" +
                               (f", spheres re-rasterised at their new centres every {translate_every} steps "
                                "(lbtranslate)" if translate_every > 0 else " on the fixed node map")},
        "build_s": round(t_build, 1),
        "batched": {"mode": "packed tiles, one launch per step, CUDA graph", "wall_s": round(t_batch, 3),
                    "MLUPS": round(nodes * steps / t_batch / 1e6, 1), "hbm_gbs": round(gbs, 1),
                    "frac_of_measured_hbm": round(gbs / peak, 4), "gpu_launches": launches,
                    "clocks": clk.summary() if clk else None},
        "one_at_a_time": {"wall_s": round(t_alone, 3), "MLUPS": round(nodes * steps / t_alone / 1e6, 1)},
        "speedup": round(t_alone / t_batch, 2),
        "drag_max_abs_diff_batched_vs_one_at_a_time": worst,
        "measured_peak_gbs": peak, "peak_kind": peak_kind,
    }
    if persistent:
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
        out["batched_persistent_mode"] = {"steps": psteps, "wall_s": round(t_pers, 3),
                                          "MLUPS": round(nodes * psteps / t_pers / 1e6, 1)}
    if cpu_subset > 0 and translate_every <= 0:
        # the smallest domains, FP64 on the CPU oracle, one thread each
        sub = sorted(range(len(specs)), key=lambda d: (specs[d][0], d))[:cpu_subset]
        res = [None] * len(sub)
        t0 = time.perf_counter()
        ts = [threading.Thread(target=_oracle_domain, args=(specs[d], steps + 4, res, n)) for n, d in enumerate(sub)]
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
            scale = 6.0 * math.pi * eta * specs[d][1] * BATCH_SPEED
            rel.append(max(abs(x - y) for x, y in zip(drags[d], res[n])) / scale)
        out["cpu_subset"] = {"domains": sub, "steps": steps + 4, "wall_s": round(t_cpu, 2), "cores": len(sub),
                             "MLUPS": round(sum(specs[d][0] ** 3 for d in sub) * (steps + 4) / t_cpu / 1e6, 2),
                             "kind": "port", "drag_max_diff_over_stokes_drag_gpu_fp32_vs_cpu_fp64": max(rel)}
    L.freebatch(b)
    for lb in batch + alone:
        L.freelb(lb)
    return out


def run_batch(args):
    import torch
    import sunlightlb_gb300
    world, rank, local = dist_env()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    L = sunlightlb_gb300.library()
    out = batch_result(torch, L, args.domains, args.batch_steps, cpu_subset=args.cpu_subset,
                       translate_every=args.translate_every)
    line = {"workload": f"batched ensemble: {args.domains} periodic moving-sphere domains, sides {list(BATCH_SIDES)}",
            "metric": "MLUPS of all domains together, batched vs one domain at a time"}
    line.update(out)
    print(json.dumps(line), flush=True)


def batch_leg(torch, L, args):
    """Compact form for the default line: 64 domains, 2000 steps."""
    out = batch_result(torch, L, args.leg_domains, args.leg_batch_steps, cpu_subset=2, persistent=False,
                       clocks=False)
    out["workload"] = f"batched ensemble, {args.leg_domains} moving-sphere domains"
    return out


# ---- learned warm start ------------------------------------------------------



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
    side, ev_side, force = args.warm_side, args.eval_side, WS.PACKING_FORCE
    # held-out packings: the ones after the training set, or from --eval-offset
    # (to evaluate networks trained on different sets on the same packings)
    ev_off = args.train if args.eval_offset is None else args.eval_offset
    if ev_off < args.train:
        raise SystemExit("--eval-offset must not reach into the training packings")
    specs = WS.packing_specs(ev_off + args.eval, WS.PACKING_SEED)
    tr_specs, ev_specs = specs[:args.train], specs[ev_off:ev_off + args.eval]
    train_now = args.epochs > 0 or not args.init_weights
    t0 = time.perf_counter()
    solids = [WS.packing(side, phi, sd) for phi, sd in tr_specs] if train_now else []
    t_pack = time.perf_counter() - t0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lsteps = [0]
    if train_now:
        fields, lsteps = WS.converged_flows(L, solids, force=force, tol=args.label_tol, maxsteps=args.label_maxsteps,
                                            density=True)
    torch.cuda.synchronize()
    t_labels = time.perf_counter() - t0
    if train_now:
        masks = torch.as_tensor(np.stack(solids).astype(np.uint8), device="cuda")
        labels = torch.stack([WS.to_labels(f, (side, side, side)) for f in fields])
        del fields
    init_meta = None
    if args.init_weights:  # fine-tune a saved network (same widths and input encoding)
        params, widths, features, init_meta = WS.load_weights(args.init_weights)
        net = WS.UNet(L, side, side, side, batch=args.batch, widths=widths, features=features,
                      params=WS.with_adam_state(params))
        args.features = features
    else:
        net = WS.UNet(L, side, side, side, batch=args.batch, seed=1, features=args.features)
    iters = max(1, args.epochs * args.train // args.batch) if train_now else 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hist = []
    if train_now:
        # each sample's loss relative to its own label energy (labels span more
        # than an order of magnitude with the solid fraction)
        sample_w = 1.0 / labels.pow(2).mean(dim=(1, 2, 3, 4)).clamp_min(1e-12)
        hist = WS.train(net, masks, labels, iters, lr=args.lr, seed=2, log_every=max(1, iters // 20),
                        sample_w=sample_w, lr_min=args.lr * 0.01, warmup=100 if not args.init_weights else 20,
                        proj_weight=args.proj_weight)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    tc_status = net.status()
    # held-out packings at the evaluation size
    inf = WS.UNet(L, ev_side, ev_side, ev_side, batch=1, params=net.params, features=args.features)
    rows = []
    checks = tuple(int(c) for c in args.warm_checks.split(",") if c)
    variants = tuple(v for v in args.warm_variants.split(",") if v)
    corrections = tuple(int(c) for c in args.warm_correct.split(",") if c)
    for phi, sd in ev_specs:
        solid = WS.packing(ev_side, phi, sd)
        pstats = {}
        traj = WS.permeability_run(L, solid, force, stats=pstats)
        k_conv = traj[-1][1]
        sdev = torch.as_tensor(solid.astype(np.uint8), device="cuda")
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        u, drho = WS.predict_state(inf, sdev, force, WS.ETA_TAU1)
        torch.cuda.synchronize()
        t_inf = time.perf_counter() - t0
        pinfo = {}
        WS.predict_state(inf, sdev, force, WS.ETA_TAU1, info=pinfo)  # the same again, for the flux spread
        row = {"phi": round(phi, 4), "k": k_conv, "plain_converged_steps": traj[-1][0], "inference_s": round(t_inf, 4),
               "plain_final_force_imbalance": pstats["imbalance_final"],
               "plane_flux_spread": pinfo.get("plane_flux_spread")}
        if args.warm_probe:
            row["warm_probe"] = WS.permeability_run(L, solid, force, k_ref=k_conv, warm_u=u, warm_drho=drho,
                                                    probe=args.warm_probe)
        # time to k within 1e-4, the permeability measured every `check` steps
        # in both arms (the plain arm from rest, the warm arm from the
        # prediction, inference included)
        for check in checks:
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
                row["warm_k_signed_error_checks"] = [(st, (kk - k_conv) / k_conv) for st, kk, _ in trajw[:6]]
                row["plain_k_error_first_check"] = abs(traj[0][1] - k_conv) / abs(k_conv)
        # the same network set without its density (rho = rho0, u - F / rho0,
        # the best shift without a density) and with its density but the
        # whole-force shift (the warm start sets u - F / (2 rho0) and rho)
        for n in corrections:  # the force-balance correction `n` steps after the warm state
            hs = WS.first_within(WS.permeability_run(L, solid, force, k_ref=k_conv, warm_u=u, warm_drho=drho, check=50,
                                                     correct=n), k_conv, 1e-4)
            row[f"check50_correct{n}"] = {"warm_steps": hs[0] if hs else None,
                                          "warm_wall_s": round(hs[1] + t_inf, 4) if hs else None}
        for name in variants:
            if name == "velocity_only":
                vs, ds = WS.predict_velocity(inf, sdev, force, WS.ETA_TAU1, force_shift=1.0), None
            elif name == "no_plane_flux":  # the state as decoded, without the plane-flux correction
                vs, ds = WS.predict_state(inf, sdev, force, WS.ETA_TAU1, plane_flux=False)
            elif name == "cross_flux":  # the warm state with its y and z plane fluxes made uniform too
                vs, ds = WS.predict_state(inf, sdev, force, WS.ETA_TAU1, cross_flux=True)
            elif name == "plane_flux_velocity":  # the plane-flux velocity scaling without its pressure
                vs, ds = WS.predict_state(inf, sdev, force, WS.ETA_TAU1, plane_flux=False)
                work = torch.empty(3 * ev_side + 1, device="cuda", dtype=torch.float64)
                inf.k.nn_plane_flux(vs.data_ptr(), None, sdev.data_ptr(), ev_side, ev_side, ev_side, force, 1.0,
                                    work.data_ptr(), inf.stream)
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
                   "loss": "relative MSE per sample" + (f" + {args.proj_weight:g} x (projection of the velocity error "
                                                        "on the label)^2" if args.proj_weight > 0 else ""),
                   "input": {0: "solid mask", 1: "solid mask + periodic wall distance d/5 and (d/5)^2 (d capped at 5)",
                             2: "solid mask + periodic wall distance d/12, (d/12)^2 (capped at 12) and min(d,5)/5"}[
                                 args.features],
                   "output": "velocity and density deviation; set with u - F / (2 rho0) and rho0 + drho",
                   "labels": f"FP32 populations, converged to |d vmeanx|/vmeanx < {args.label_tol:g} per 200 steps",
                   "precision": "BF16 weights/activations, FP32 accumulation (tcgen05)"},
        "packing_s": round(t_pack, 1), "labels_s": round(t_labels, 1),
        "label_steps": {"mean": float(np.mean(lsteps)), "max": int(np.max(lsteps))},
        "train_s": round(t_train, 1), "train_ms_per_iteration": round(1e3 * t_train / iters, 2) if iters else None,
        "loss": hist, "tc_status": tc_status,
        "eval": rows,
        "summary": summary(checks[-1]),
        "summary_by_check": [summary(c) for c in checks],
        "variants_at_check50": {
            name: {"wall_speedup_mean": float(np.mean([r["check50"]["plain_wall_s"] / r[f"check50_{name}"]["warm_wall_s"]
                                                       for r in rows if r[f"check50_{name}"]["warm_wall_s"]])),
                   "steps_ratio_mean": float(np.mean([r["check50"]["plain_steps"] / r[f"check50_{name}"]["warm_steps"]
                                                      for r in rows if r[f"check50_{name}"]["warm_steps"]])),
                   "plain_wall_total_s": round(float(sum(r["check50"]["plain_wall_s"] for r in rows
                                                         if r[f"check50_{name}"]["warm_wall_s"])), 3),
                   "warm_wall_total_s": round(float(sum(r[f"check50_{name}"]["warm_wall_s"] for r in rows
                                                        if r[f"check50_{name}"]["warm_wall_s"])), 3)}
            for name in variants + tuple(f"correct{n}" for n in corrections)} if 50 in checks else None,
    }
    print(json.dumps(line), flush=True)
    if args.save_weights:
        WS.save_weights(net, args.save_weights,
                        meta={"train_samples": args.train, "train_side": side, "epochs": args.epochs,
                              "iterations": iters, "seed": WS.PACKING_SEED, "label_tol": args.label_tol,
                              "final_loss": hist[-1] if hist else None, "lr": args.lr,
                              "proj_weight": args.proj_weight,
                              "fine_tuned_from": init_meta})


def warm_leg(torch, L, args):
    """Compact form for the default line: the committed network
    (sunlightlb_gb300/data/warm_unet.npz, trained by --workload warmstart
    --save-weights on the GPU) against the plain start on the first
    `--leg-warm-eval` held-out 128^3 packings of the warmstart workload;
    steps and wall time to permeability within 1e-4 of the plain converged
    value, checks every 50 steps in both arms, inference timed
    (warmstart.held_out_comparison)."""
    import numpy as np
    from sunlightlb_gb300 import warmstart as WS
    if not os.path.exists(WS.WEIGHTS):
        return {"skipped": "no trained weights in sunlightlb_gb300/data/warm_unet.npz"}
    rows, meta = WS.held_out_comparison(L, args.leg_warm_eval, side=args.eval_side, check=50)
    _, widths, _, _ = WS.load_weights()
    ok = [r for r in rows if r["plain_wall_s"] and r["warm_wall_s"]]
    tot_p = sum(r["plain_wall_s"] for r in ok)
    tot_w = sum(r["warm_wall_s"] for r in ok)
    return {"workload": f"learned warm start, {len(rows)} held-out {args.eval_side}^3 packings",
            "network": {"widths": list(widths), "trained": meta},
            "criterion": "permeability within 1e-4 of the plain converged value, checks every 50 steps",
            "samples": len(ok), "plain_wall_total_s": round(tot_p, 3), "warm_wall_total_s": round(tot_w, 3),
            "total_wall_ratio": round(tot_p / tot_w, 3) if tot_w else None,
            "wall_speedup_mean": round(float(np.mean([r["plain_wall_s"] / r["warm_wall_s"] for r in ok])), 3) if ok else None,
            "steps_ratio_total": round(sum(r["plain_steps"] for r in ok) / sum(r["warm_steps"] for r in ok), 3) if ok else None,
            "rows": rows}


def main():
    global HEAD_N
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="mine", choices=["mine", "reference"])
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64", "bf16dev"])
    ap.add_argument("--e2e-intervals", type=int, default=20)
    ap.add_argument("--e2e-fp64-intervals", type=int, default=2)
    ap.add_argument("--head-side", type=int, default=HEAD_N,
                    help="side of the headline packed bed (smaller sides for profiling runs only)")
    ap.add_argument("--no-legs", action="store_true", help="default workload: skip the batch, tracer and "
                                                         "warm-start legs")
    ap.add_argument("--leg-domains", type=int, default=64)
    ap.add_argument("--leg-batch-steps", type=int, default=2000)
    ap.add_argument("--leg-tracer-side", type=int, default=256)
    ap.add_argument("--leg-tracer-steps", type=int, default=2000)
    ap.add_argument("--leg-warm-eval", type=int, default=10)
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--no-convergence", action="store_true")
    ap.add_argument("--max-converge-steps", type=int, default=60000)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="packed", choices=["packed", "tracer", "batch", "warmstart"],
                    help="packed: the 512^3 packed-bed step with its variants and legs (default); tracer: "
                         "large bed, flow + passive scalar; batch: many small moving-sphere domains in one "
                         "launch; warmstart: train and evaluate the learned warm start")
    ap.add_argument("--domains", type=int, default=512, help="batch workload: number of domains")
    ap.add_argument("--batch-steps", type=int, default=20000)
    ap.add_argument("--cpu-subset", type=int, default=8, help="batch workload: domains checked on the CPU oracle")
    ap.add_argument("--translate-every", type=int, default=0,
                    help="batch workload: move the spheres (re-rasterise them) every this many steps; 0 keeps "
                         "the node map fixed")
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
    ap.add_argument("--init-weights", default="", help="warmstart workload: start from a saved network (fine-tune; "
                                                         "with --epochs 0 only evaluate it)")
    ap.add_argument("--eval-offset", type=int, default=None,
                    help="warmstart workload: index of the first held-out packing (default: after the training set)")
    ap.add_argument("--proj-weight", type=float, default=0.0,
                    help="warmstart workload: weight of the squared projection of the velocity error on the label")
    ap.add_argument("--warm-checks", default="100,50",
                    help="warmstart workload: permeability check intervals of the time-to-accuracy comparison")
    ap.add_argument("--warm-variants", default="velocity_only,state_whole_force_shift,no_plane_flux",
                    help="warmstart workload: other ways of setting the prediction, timed at 50-step checks")
    ap.add_argument("--warm-correct", default="",
                    help="warmstart workload: force-balance corrections of the mean flow, after these steps")
    ap.add_argument("--warm-probe", type=int, default=0,
                    help="warmstart workload: record the force imbalance and permeability error of this many "
                         "measures in a row after the warm state")
    ap.add_argument("--features", type=int, default=1, choices=[0, 1, 2],
                    help="warmstart workload: input encoding (wall distance searched to 5 or 12)")
    ap.add_argument("--side", type=int, default=512, help="tracer workload: lattice side")
    ap.add_argument("--tracer-steps", type=int, default=50000)
    ap.add_argument("--fp64-tracer-steps", type=int, default=10000)
    ap.add_argument("--sample-every", type=int, default=500)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    HEAD_N = args.head_side
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
