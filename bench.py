"""Benchmark of the GB300 MUSCL-Hancock hydro step (one JSON line on rank 0).

Default workload: 3-D 256^3 periodic box with 32 spheres and a harmonic
density ripple (superbee, courant 0.3, gamma 5/3), in the mixed FP32/FP64
form, with the plain FP64 path timed on the same box beside it and the
per-field L1 / Linf difference between the two after 300 steps: the
configuration the mixed-vs-FP64 metric is quoted on. A step is one driver
iteration (dt -> ghost fill -> solve) over the box. Every arm first advances
the box untimed to the middle of its run (--advance, default half the
workload's step count: step 150 of the 300-step sphere run), so the timed
window sees the developed flow rather than the nearly uniform start.

  value   cell-updates/s with the state resident in HBM, timed with CUDA
          events on the library's stream around each step; L2 is flushed
          (a 512 MiB write) between timed steps, outside the events.
  e2e     the same metric through the reference-facing C-ABI with the state
          in host memory: per step host->device upload, dt (read back),
          ghost fill, solve and device->host download (the drop-in loop
          with host write-back), wall-clock timed; the median of 5 windows
          of --e2e-steps steps, each window reported.
  roofline  HBM roofline of the dominant kernel: the step's algorithmic
          bytes (U^n read + U^{n+1} written, (NDIM+2) FP64 fields per cell)
          over that kernel's event-timed duration per step.
  cpu_baseline  the CPU oracle (a restatement of the reference's
          memory-intensive solver with OpenMP over the outer loop) on a
          bounded sample of the same workload, all host threads
          (--cpu-threads N for fewer).

Other workloads (--workload): slab2d (2-D 256^2 shear slab, plain FP64,
500 steps), riemann1d (1-D 512 cells, 100 steps), spheres3d<N>, batch4096
(4096 uneven 3-D boxes stepped as one batch; use --steps 10), serve (a
seeded Poisson stream of 512 requests served by the continuous-batching
server, against one-at-a-time plain FP64 on its first 48, with per-request
errors of the served mixed results against FP64) and rates (the GPU's FP64
and FP32 arithmetic rates for the operations this path is bound by).

--impl reference times the CPU implementation alone on the same config and
window: the whole box, advanced by the CPU itself (with --cpu-threads N, on
N OpenMP threads).
Under torchrun the single-box workloads run as one box in slabs along the
outermost axis, a slab per rank, with the halo rows exchanged device to
device over NCCL (strong scaling; --replicas: an independent replica per
rank instead); batch4096 shards its boxes over the ranks and serve runs a
stream per rank (weak scaling, value summed over ranks).
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

METRIC = "cell-updates/s"
L2_FLUSH_BYTES = 512 << 20
DEFAULT_WORKLOAD = "spheres3d256"
SERVE_REQUESTS = 512      # p99 over a stream of this many requests
BATCH_STEPS = 200         # timed steps of the many-box workload
SERVE_FP64_PREFIX = 48    # the one-at-a-time FP64 baseline serves this prefix
SERVE_ERR_REQUESTS = 24   # served results replayed alone in FP64 for the error
E2E_WINDOWS = 5


def workload(name, precision=None):
    """(cells, dx, params, config dict) of a named single-box workload;
    precision None takes the workload's own."""
    from rhyme_gb300.params import FP64, MIXED
    cells, dx, p, cfg = _workload(name)
    prec = precision or cfg["precision"]
    p = dict(p, precision=MIXED if prec == "mixed" else FP64)
    form = "mixed FP32/FP64" if prec == "mixed" else "plain FP64"
    cfg = dict(cfg, workload="%s, %s" % (cfg["workload"], form), precision=prec)
    return cells, dx, p, cfg


def _workload(name):
    from rhyme_gb300 import ic
    if name == "slab2d":
        cells, dx, p = ic.slab_2d(n=256, seed=0)
        cfg = {"workload": "2-D 256x256 periodic shear slab, minmod, courant 0.8",
               "ndim": 2, "cells": 256 * 256, "steps_in_run": 500, "precision": "fp64"}
    elif name == "riemann1d":
        cells, dx, p = ic.riemann_1d(n=512, seed=0)
        cfg = {"workload": "1-D 512-cell seeded Riemann problem, van Leer, courant 0.8",
               "ndim": 1, "cells": 512, "steps_in_run": 100, "precision": "fp64"}
    elif name.startswith("spheres3d"):
        n = int(name[len("spheres3d"):] or 256)
        cells, dx, p = ic.spheres_3d(n=n, seed=0)
        cfg = {"workload": "3-D %d^3 periodic, 32 spheres + harmonic density, superbee, courant %.2g"
                           % (n, p["courant"]), "ndim": 3, "cells": n ** 3, "steps_in_run": 300,
               "precision": "mixed"}
    else:
        raise SystemExit("unknown workload %s" % name)
    return cells, dx, p, cfg


def algorithmic_bytes_per_cell(ndim):
    # U^n read once + U^{n+1} written once, NDIM+2 FP64 fields
    return 2 * (ndim + 2) * 8


def dtype_name(prec):
    return "f64" if prec == "fp64" else "f32+f64"


class ClockSampler:
    """nvidia-smi SM clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append((time.time(), line.strip()))

    def summary(self, t_begin, t_end):
        """Median SM clock and active throttle reasons between two times."""
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = [r for t, r in self.rows if t_begin - 0.15 <= t <= t_end + 0.15] or [r for _, r in self.rows[-3:]]
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            f = [x.strip() for x in r.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}

    def stop(self):
        if self.proc is None:
            return
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        return float(pk["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic(workload_name, kernel):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary
    (profiles/ncu_traffic.txt lines: workload kernel bytes_per_launch)."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    try:
        for line in open(path):
            f = line.split()
            if len(f) >= 3 and not line.startswith("#") and f[0] == workload_name and f[1] == kernel:
                return float(f[2])
    except OSError:
        pass
    return None


def cpu_sample(cells, dx, p, steps_cap, budget_s, nthreads):
    """Oracle cell-updates/s stepping `cells` (bounded by steps_cap steps and
    about budget_s seconds; the first step, which allocates the workspace,
    is untimed)."""
    import oracle
    c = cells.copy()
    interior = int(np.prod([s - 4 for s in c.shape[1:]]))
    t0 = time.perf_counter()
    oracle.run(p, c, dx, 1, nthreads=nthreads)  # warm (allocates the workspace)
    first = time.perf_counter() - t0
    done, t = 0, 0.0
    chunk = 1
    while done < steps_cap and t + first < budget_s:
        t0 = time.perf_counter()
        oracle.run(p, c, dx, chunk, nthreads=nthreads)
        t += time.perf_counter() - t0
        done += chunk
        chunk = min(chunk * 2, steps_cap - done) if done < steps_cap else 0
        if chunk <= 0:
            break
    if done == 0:  # a single step is already beyond the budget
        return interior / first, 1, first
    return interior * done / t, done, t


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend="nccl")
    return rank, local, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(x, world):
    from rhyme_gb300.shard import reduce_scalar
    return reduce_scalar(x, world, "max", device="cuda")


def allsum(x, world):
    from rhyme_gb300.shard import reduce_scalar
    return reduce_scalar(x, world, "sum", device="cuda")


def launches_per_step(prec, ndim, fused_xy=False):
    """Kernels of this library launched per single-box step: FP64 cfl, ghost
    fill, faces, fluxes, update; mixed cfl (carried, or the whole pass that
    also writes the FP32 mirror), ghost fill (of the FP64 state and of the
    mirror, in one kernel), one sweep per axis (one kernel for x and y of a
    3-D box where fused_xy) and the FP64 fix-up of the queued interfaces."""
    if prec == "fp64":
        return 5
    return 3 + ndim - (1 if fused_xy else 0)


def advance_steps(args, cfg):
    """Untimed steps before the warm-up: half the workload's run by default."""
    return cfg["steps_in_run"] // 2 if args.advance is None else args.advance


def window_text(adv, W, K, cfg):
    return "steps %d-%d of the %d-step run (advanced %d steps untimed, then %d warm-up steps)" % (
        adv + W + 1, adv + W + K, cfg["steps_in_run"], adv, W)


REF_BATCH_BOXES = 64


def run_reference_batch(args):
    """The reference arm on the many-box workload: the CPU implementation
    steps the first REF_BATCH_BOXES boxes of the same seeded list (the list
    is drawn box by box from one generator, so these are the batch's own
    first boxes), box after box as the reference's driver loop does, each
    with its own dt. Boxes are independent, so the subset changes the
    sample's size, not its work per cell."""
    from rhyme_gb300 import ic
    from rhyme_gb300.params import FP64
    import oracle
    nthreads = args.cpu_threads or os.cpu_count() or 1
    nb = min(args.nboxes, REF_BATCH_BOXES)
    items = ic.batch_boxes(nb, seed=0)
    states = [c.copy() for c, _, _ in items]
    n = sum(int(np.prod([s - 4 for s in c.shape[1:]])) for c, _, _ in items)

    def steps(k):
        for _ in range(k):
            for st, (_, dx, p) in zip(states, items):
                oracle.run(dict(p, precision=FP64), st, dx, 1, nthreads=nthreads)

    steps(args.warmup)
    t0 = time.perf_counter()
    steps(args.steps)
    t = time.perf_counter() - t0
    v = n * args.steps / t
    sample = ("%d timed steps after %d warm-up steps; the first %d of the %d boxes (%d cells), one box "
              "after another; OpenMP over each box's outer cell loop" % (args.steps, args.warmup, nb,
                                                                           args.nboxes, n))
    cfg = {"workload": "%d uneven 3-D boxes (edges 8..64 per axis), Riemann or sphere ICs, van Albada, "
                       "courant 0.3, plain FP64" % args.nboxes, "cells": n, "boxes": nb,
           "l2": "the sample's state (%.2f GB of FP64) is stepped box by box" % (n * 40 / 1e9),
           "parallelism": "one CPU process"}
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": METRIC, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": cfg,
            "cpu_baseline": {"value": v, "unit": METRIC, "cores": nthreads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_reference(args, rank, world):
    if rank != 0:
        return
    from rhyme_gb300.params import FP64
    if args.workload == "serve":
        raise SystemExit("--impl reference covers the box workloads")
    if args.workload == "batch4096":
        return run_reference_batch(args)
    cells, dx, p, cfg = workload(args.workload, "fp64")
    p = dict(p, precision=FP64)  # the CPU implementation is FP64
    import oracle
    nthreads = args.cpu_threads or os.cpu_count() or 1
    c, n = cells.copy(), cfg["cells"]
    adv = advance_steps(args, cfg)
    if adv:
        oracle.run(p, c, dx, adv, nthreads=nthreads)
    if args.warmup:
        oracle.run(p, c, dx, args.warmup, nthreads=nthreads)
    t0 = time.perf_counter()
    oracle.run(p, c, dx, args.steps, nthreads=nthreads)
    t = time.perf_counter() - t0
    v = n * args.steps / t
    sample = "the whole box (%d cells), %s; OpenMP over the outer cell loop" % (
        n, window_text(adv, args.warmup, args.steps, cfg))
    cfg = dict(cfg, window=window_text(adv, args.warmup, args.steps, cfg))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": METRIC, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": dict(cfg, workload=cfg["workload"].replace("mixed FP32/FP64", "plain FP64")),
            "cpu_baseline": {"value": v, "unit": METRIC, "cores": nthreads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def time_steps(ctx, box, dx, K, flush, stream):
    """K single steps, each bracketed by CUDA events on the library's stream,
    with an L2 flush between them outside the events; ms per step."""
    import torch
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    for k in range(K):
        with torch.cuda.stream(stream):
            flush.zero_()
        starts[k].record(stream)
        ctx.run(box, dx, 1, trace=False)
        ends[k].record(stream)
    ctx.synchronize()
    torch.cuda.synchronize()
    return [s.elapsed_time(e) for s, e in zip(starts, ends)]


def run_gpu(args, rank, local, world):
    import torch
    from rhyme_gb300 import gpu
    from rhyme_gb300.metrics import field_errors
    from rhyme_gb300.params import FP64
    torch.cuda.set_device(local)
    cells, dx, p, cfg = workload(args.workload, args.precision)
    prec = cfg["precision"]
    ndim = p["ndim"]
    interior = cfg["cells"]
    K, W = args.steps, args.warmup
    compare = prec == "mixed" and not args.no_compare
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    # the host array of the end-to-end loop, allocated (and first touched)
    # before the other runs, as a caller's state array would be
    host = cells.copy()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)

    adv = advance_steps(args, cfg)

    # headline form, advanced untimed to the window
    ctx = gpu.Context(p)
    state = cells.copy()
    box = ctx.register_box(state)
    stream = torch.cuda.ExternalStream(ctx.stream)
    if adv:
        ctx.run(box, dx, adv, trace=False)
        ctx.sync_to_host(box)
        np.copyto(host, state)  # the end-to-end loop starts from the same state
    ctx.run(box, dx, W, trace=False)
    ctx.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    t_begin = time.time()
    per_step = time_steps(ctx, box, dx, K, flush, stream)
    barrier(world)
    t_end = time.time()
    clk = clocks.summary(t_begin, t_end)
    ms = allmax(sum(per_step), world)
    value = world * interior * K / (ms * 1e-3)

    # plain FP64 on the same box, and the difference after the run's steps
    cmp = None
    cpu_state = cells  # the CPU baseline's starting state (the window's)
    if compare:
        pc = dict(p, precision=FP64)
        ctx_c = gpu.Context(pc)
        state_c = cells.copy()
        box_c = ctx_c.register_box(state_c)
        stream_c = torch.cuda.ExternalStream(ctx_c.stream)
        ctx_c.run(box_c, dx, adv + W, trace=False)
        ctx_c.sync_to_host(box_c)
        # the FP64 path is bit-identical to the CPU oracle, so this is the
        # oracle's own state at the timed window
        cpu_state = state_c.copy()
        ctx_c.synchronize()
        barrier(world)
        tc0 = time.time()
        per_c = time_steps(ctx_c, box_c, dx, K, flush, stream_c)
        barrier(world)
        tc1 = time.time()
        ms_c = allmax(sum(per_c), world)
        value_c = world * interior * K / (ms_c * 1e-3)
        n_acc = max(cfg["steps_in_run"], adv + W + K)
        for c_, b_ in ((ctx, box), (ctx_c, box_c)):
            if n_acc > adv + W + K:
                c_.run(b_, dx, n_acc - (adv + W + K), trace=False)
            c_.sync_to_host(b_)
        fb = ctx.fallback_count(box)
        errs = field_errors(state, state_c, ndim)
        names = ["rho"] + ["rho_v%s" % "xyz"[a] for a in range(ndim)] + ["e_tot"]
        cmp = {"fp64_value": value_c, "fp64_ms_per_step": ms_c / K, "mixed_over_fp64": value / value_c,
               "fp64_clocks": clocks.summary(tc0, tc1),
               "errors_vs_fp64": {"after_steps": n_acc, "definition": "relative L1 = sum|d|/sum|f64|, "
                                  "relative Linf = max|d|/max|f64| over the interior",
                                  "l1": dict(zip(names, [e[0] for e in errs])),
                                  "linf": dict(zip(names, [e[1] for e in errs]))},
               "fp64_interfaces_redone_in_run": fb}
        ctx_c.close()
        # the headline box continues from its own state for the profile below
    clocks.stop()

    # phase timing of the same step (direct launches, events between kernels)
    phases = ctx.profile_steps(box, dx, max(5, min(50, K)))
    dom = max(phases, key=phases.get)
    bpc = algorithmic_bytes_per_cell(ndim)
    peak, peak_kind = measured_peaks()
    achieved = interior * bpc / (phases[dom] * 1e-3) / 1e9
    traffic = ncu_traffic("%s-%s" % (args.workload, prec), dom)
    ctx.close()

    # end to end through the C-ABI with the state in host memory
    ctx2 = gpu.Context(p)
    b2 = ctx2.register_box(host)
    # the drop-in mode: each solve copies its result back while it runs
    ctx2.set_host_writeback(b2)
    hydro_bytes = (ndim + 2) * int(np.prod(host.shape[1:])) * 8
    ke = max(1, min(K, args.e2e_steps))

    def e2e_step():
        ctx2.sync_to_device(b2)
        dt = ctx2.cfl_time_step(b2, dx)
        ctx2.set_boundaries(b2)
        ctx2.muscl_hancock_solve(b2, dx, dt)
        ctx2.sync_to_host(b2)

    for _ in range(min(W, 3)):
        e2e_step()
    # E2E_WINDOWS windows of ke steps each (the host link is shared with the
    # machine's other jobs, whose traffic comes and goes): the median window
    # is the figure, every window is reported
    windows = []
    for _ in range(E2E_WINDOWS):
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(ke):
            e2e_step()
        te = allmax(time.perf_counter() - t0, world)
        windows.append(world * interior * ke / te)
    barrier(world)
    e2e = statistics.median(windows)
    ctx2.close()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        nthreads = args.cpu_threads or os.cpu_count() or 1
        start = adv + W
        if cpu_state is cells:
            # no FP64 run on the GPU: the oracle advances the box itself
            cpu_state = cells.copy()
            import oracle
            oracle.run(dict(p, precision=FP64), cpu_state, dx, start, nthreads=nthreads)
        v, n, t = cpu_sample(cpu_state, dx, dict(p, precision=FP64), max(1, cfg["steps_in_run"] - start),
                             args.cpu_budget, nthreads)
        cpu = {"value": v, "unit": METRIC, "cores": nthreads, "kind": "port",
               "sample": "the whole box, %d timed steps after step %d of the same workload (%.1f s), CPU "
                         "oracle (FP64), OpenMP" % (n, start + 1, t)}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": K,
                "warmup": W, "ms_per_step": ms / K, "ms_per_step_median": statistics.median(per_step),
                "ms_per_step_max": max(per_step), "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": dtype_name(prec), "data": "synthetic",
                "config": dict(cfg, l2="flushed (512 MiB write) between timed steps, outside the events",
                               parallelism="replicas" if world > 1 else "single box",
                               window=window_text(adv, W, K, cfg)),
                "e2e": {"value": e2e, "unit": METRIC, "h2d_bytes_per_step": hydro_bytes + 8,
                        "d2h_bytes_per_step": hydro_bytes + 8 + 4, "steps": ke,
                        "windows": windows, "statistic": "median of %d windows of %d steps" % (E2E_WINDOWS, ke)},
                "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                             "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                             "traffic": traffic, "bytes_per_cell_update": bpc,
                             "step_achieved": value / world * bpc / 1e9,
                             "note": "compute-bound: FP64 pipe (plain) / FP32 issue (mixed), not HBM; the "
                                     "step's 80 B per cell charged to its longest kernel" +
                                     (", which runs the x and y sweeps of the step" if dom == "sweep_xy" else "")},
                "phases_ms": phases, "clocks": clk,
                "gpu_launches": launches_per_step(prec, ndim, "sweep_xy" in phases) * K,
                "cpu_baseline": cpu}
        if cmp is not None:
            line["vs_fp64"] = cmp
        print(json.dumps(line), flush=True)


def run_slabs(args, rank, local, world):
    """One box decomposed into slabs along its outermost axis, one slab per
    rank (rhyme_gb300.slabs.run_rank: dt minimum by all-reduce, the two halo
    rows per face exchanged device to device over NCCL). value: the whole
    box's cell updates per second over the slowest rank's wall clock
    (strong scaling: the box is the same at every N). e2e: the drop-in loop
    per rank (slab upload from host memory, dt read back, ghost fill, halo
    exchange, solve with host write-back)."""
    import torch
    from rhyme_gb300 import gpu, slabs
    from rhyme_gb300.params import PERIODIC
    torch.cuda.set_device(local)
    cells, dx, p, cfg = workload(args.workload, args.precision)
    ndim = p["ndim"]
    K, W = args.steps, args.warmup
    adv = advance_steps(args, cfg)
    rows = slabs.split_rows(cells.shape[1] - 4, world)
    a, c = rows[rank]
    arr = slabs.slab_cells(cells, a, c)
    lo_f, hi_f = 2 * (ndim - 1), 2 * (ndim - 1) + 1
    periodic = p["bc"][lo_f] == PERIODIC and p["bc"][hi_f] == PERIODIC
    ops = slabs.GpuOps(dx)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    ctx = gpu.Context(p)
    b = ctx.register_box(arr)
    ctx.set_box_params(b, bc=slabs.slab_bc(p["bc"], ndim, rank, world), limiter=p["limiter"], omega=p["omega"])
    sl = (ctx, b)
    slabs.run_rank(sl, c, adv + W, ops, periodic, rank, world)
    ctx.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    t_begin = time.time()
    t0 = time.perf_counter()
    slabs.run_rank(sl, c, K, ops, periodic, rank, world)
    ctx.synchronize()
    torch.cuda.synchronize()
    el = allmax(time.perf_counter() - t0, world)
    barrier(world)
    clk = clocks.summary(t_begin, time.time())
    clocks.stop()
    value = cfg["cells"] * K / el
    # the drop-in form: the slab's state in host memory between steps
    ctx.sync_to_host(b)
    ctx.set_host_writeback(b)
    hydro_bytes = (ndim + 2) * int(np.prod(arr.shape[1:])) * 8

    class DropInOps(slabs.GpuOps):
        def dt(self, s):
            s[0].sync_to_device(s[1])
            return s[0].cfl_time_step(s[1], self.dx)

        def solve(self, s, dt):
            s[0].muscl_hancock_solve(s[1], self.dx, dt)
            s[0].sync_to_host(s[1])

    ke = max(1, min(K, args.e2e_steps))
    slabs.run_rank(sl, c, min(W, 3), DropInOps(dx), periodic, rank, world)
    windows = []
    for _ in range(E2E_WINDOWS):
        barrier(world)
        t0 = time.perf_counter()
        slabs.run_rank(sl, c, ke, DropInOps(dx), periodic, rank, world)
        te = allmax(time.perf_counter() - t0, world)
        windows.append(cfg["cells"] * ke / te)
    ctx.close()
    if rank == 0:
        prec = cfg["precision"]
        line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": K, "warmup": W,
                "ms_per_step": 1e3 * el / K, "higher_is_better": True, "scaling": "strong",
                "vs_baseline": None, "dtype": dtype_name(prec), "data": "synthetic",
                "config": dict(cfg, parallelism="one box in %d slabs along its outermost axis, one per GPU; "
                                                "halo rows device to device over NCCL" % world,
                               window=window_text(adv, W, K, cfg), slab_rows=[r[1] for r in rows],
                               l2="inputs larger than L2 (%.2f GB of FP64 state per slab)" % (hydro_bytes / 1e9)),
                "e2e": {"value": statistics.median(windows), "unit": METRIC, "h2d_bytes_per_step": hydro_bytes,
                        "d2h_bytes_per_step": hydro_bytes, "windows": windows,
                        "statistic": "median of %d windows of %d steps; bytes per rank" % (E2E_WINDOWS, ke)},
                "clocks": clk, "gpu_launches": launches_per_step(prec, ndim) * K}
        print(json.dumps(line), flush=True)


def trace_mixed_only(items, idx, nsteps, physical):
    """Each box that ends unphysical in mixed precision only, stepped alone in
    FP64 (the batch's FP64 result bit for bit) and in mixed precision with
    the state checked after every step: the first unphysical step of each,
    and how many such boxes stay physical at every FP64 step (a mixed-only
    loss) or pass through an unphysical FP64 state that later recovers."""
    from rhyme_gb300 import gpu
    from rhyme_gb300.params import FP64, MIXED
    first = {"fp64": [], "mixed": []}
    for i in idx:
        c0, dx, p = items[i]
        for name, prec in (("fp64", FP64), ("mixed", MIXED)):
            c = c0.copy()
            step = None
            with gpu.Context(dict(p, precision=prec)) as ctx:
                b = ctx.register_box(c)
                for s in range(nsteps):
                    ctx.run(b, dx, 1)
                    ctx.sync_to_host(b)
                    if not physical(c[:, 2:-2, 2:-2, 2:-2]):
                        step = s + 1
                        break
            first[name].append(step)
    lost = sum(1 for f in first["fp64"] if f is None)
    return {"boxes": len(idx), "fp64_physical_at_every_step": lost,
            "fp64_unphysical_at_some_step": len(idx) - lost,
            "mixed_unphysical_before_fp64": sum(1 for f, m in zip(first["fp64"], first["mixed"])
                                                if m is not None and (f is None or m < f)),
            "first_unphysical_step": {"fp64": first["fp64"], "mixed": first["mixed"]}}


def run_batch(args, rank, local, world):
    """4096 uneven 3-D boxes (edges from {8..64} per axis, Riemann or sphere
    ICs, reflective/outflow faces, van Albada) stepped as one batch: a
    work-queue launch per pass, the step captured in a CUDA graph, each box
    with its own dt. Mixed form headline, plain FP64 beside it, errors of
    mixed against FP64 after the run. Ranks take cost-balanced shares of the
    boxes (rhyme_gb300.shard)."""
    import torch
    from rhyme_gb300 import gpu, ic
    from rhyme_gb300.params import FP64, MIXED
    torch.cuda.set_device(local)
    from rhyme_gb300 import shard
    items = ic.batch_boxes(args.nboxes, seed=0)
    items = shard.my_share(items, [shard.box_cost(c) for c, _, _ in items], rank, world)
    interior = sum(int(np.prod([s - 4 for s in c.shape[1:]])) for c, _, _ in items)
    K, W = args.steps, args.warmup
    prec = args.precision or "mixed"
    order = [prec] + ([] if args.no_compare else ["fp64" if prec == "mixed" else "mixed"])
    # the FP64 leg's timed run is one stream wait of K x 2.3 s; the library's
    # wait limit (600 s by default) is a guard against a hung stream
    os.environ.setdefault("RHYME_GPU_TIMEOUT_S", str(max(600, 10 * K)))
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    res, finals = {}, {}
    for pr in order:
        base = dict(items[0][2], precision=MIXED if pr == "mixed" else FP64)
        states = [c.copy() for c, _, _ in items]
        ctx = gpu.Context(base)
        boxes = []
        for st, (_, dx, p) in zip(states, items):
            b = ctx.register_box(st)
            ctx.set_box_params(b, bc=p["bc"], limiter=p["limiter"], omega=p["omega"])
            boxes.append(b)
        bt = ctx.batch(boxes, [dx for _, dx, _ in items])
        stream = torch.cuda.ExternalStream(ctx.stream)
        bt.run(W)
        ctx.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier(world)
        t_begin = time.time()
        ev0.record(stream)
        bt.run(K)
        ev1.record(stream)
        ctx.synchronize()
        torch.cuda.synchronize()
        barrier(world)
        t_end = time.time()
        ms = allmax(ev0.elapsed_time(ev1), world)
        res[pr] = {"value": allsum(interior, world) * K / (ms * 1e-3), "ms_per_step": ms / K,
                   "clocks": clocks.summary(t_begin, t_end)}
        for b in boxes:
            ctx.sync_to_host(b)
        bt.close()
        ctx.close()
        finals[pr] = states
    clocks.stop()
    cmp = None
    if len(order) == 2:
        a, b = finals["mixed"], finals["fp64"]
        d1 = np.zeros(5)
        s1 = np.zeros(5)
        dm = np.zeros(5)
        sm = np.zeros(5)
        bad64, bad_mixed_only, used = 0, 0, 0
        def physical(c):
            # finite, positive density and positive pressure (gamma 5/3)
            if not np.isfinite(c).all() or c[0].min() <= 0:
                return False
            ke = 0.5 * (c[1] ** 2 + c[2] ** 2 + c[3] ** 2) / c[0]
            return bool(((c[4] - ke) * (2.0 / 3.0)).min() > 0)

        mixed_only = []
        for i, (x, y) in enumerate(zip(a, b)):
            xi, yi = x[:, 2:-2, 2:-2, 2:-2], y[:, 2:-2, 2:-2, 2:-2]
            ok64 = physical(yi)
            okm = physical(xi)
            if not ok64:
                bad64 += 1
                continue
            if not okm:
                bad_mixed_only += 1
                mixed_only.append(i)
                continue
            used += 1
            d = np.abs(xi - yi).reshape(5, -1)
            r = np.abs(yi).reshape(5, -1)
            d1 += d.sum(1)
            s1 += r.sum(1)
            dm = np.maximum(dm, d.max(1))
            sm = np.maximum(sm, r.max(1))
        names = ["rho", "rho_vx", "rho_vy", "rho_vz", "e_tot"]
        traces = trace_mixed_only(items, mixed_only, W + K, physical)
        cmp = {"after_steps": W + K, "definition": "relative L1 = sum|d|/sum|f64|, relative Linf = "
               "max|d|/max|f64| over the interiors of the boxes whose FP64 state after the run is "
               "physical (finite, positive density and pressure)", "boxes_compared": used,
               "boxes_failing_in_fp64": bad64, "boxes_failing_in_mixed_only": bad_mixed_only,
               "mixed_only_boxes_traced": traces,
               "l1": dict(zip(names, (d1 / s1).tolist())), "linf": dict(zip(names, (dm / sm).tolist()))}
    if rank == 0:
        h = res[prec]
        line = {"metric": METRIC, "value": h["value"], "unit": METRIC, "n_gpus": world, "steps": K,
                "warmup": W, "ms_per_step": h["ms_per_step"], "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": dtype_name(prec), "data": "synthetic",
                "config": {"workload": "%d uneven 3-D boxes (edges 8..64 per axis), Riemann or sphere ICs, "
                                       "van Albada, courant 0.3, one batch, %s" % (args.nboxes, prec),
                           "cells": interior, "boxes": len(items),
                           "l2": "inputs larger than L2 (%.1f GB of FP64 state)" % (interior * 40 / 1e9),
                           "parallelism": "boxes sharded over ranks" if world > 1 else "one batch"},
                "e2e": None, "clocks": h["clocks"],
                "gpu_launches": launches_per_step(prec, 3) * K, "forms": res, "mixed_vs_fp64": cmp}
        if "fp64" in res and "mixed" in res:
            line["mixed_over_fp64"] = res["mixed"]["value"] / res["fp64"]["value"]
        print(json.dumps(line), flush=True)


def run_serve(args, rank, local, world):
    """A seeded Poisson stream of requests served by the continuous-batching
    server (mixed precision, max 256 active, 150 GB budget; initial states
    uploaded, and painted on the device) and the same stream served one
    request at a time in plain FP64; p50/p99 latency (submission to result
    in host memory) and cell-updates/s over the makespan of each."""
    import torch
    from rhyme_gb300 import serving
    from rhyme_gb300.params import FP64, MIXED, hydro_params
    torch.cuda.set_device(local)
    nreq = args.requests if args.requests is not None else SERVE_REQUESTS
    stream = serving.make_stream(n=nreq, rate=args.rate, seed=rank)
    out = {}
    served = None
    for name, prec, cap, paint, reqs in (("continuous_mixed", MIXED, 256, False, stream),
                                         ("continuous_mixed_painted", MIXED, 256, True, stream),
                                         ("one_at_a_time_fp64", FP64, 1, False, stream[:SERVE_FP64_PREFIX])):
        r = serving.replay(reqs, hydro_params(3, precision=prec), hbm_budget=150 << 30, max_active=cap,
                           paint=paint)
        lat = r["latencies"]
        out[name] = {"value": r["cell_updates"] / r["makespan"], "p50_s": float(np.percentile(lat, 50)),
                     "p99_s": float(np.percentile(lat, 99)), "makespan_s": r["makespan"],
                     "cell_updates": r["cell_updates"], "peak_active": r["peak_active"], "requests": len(reqs)}
        if name == "continuous_mixed":
            served = r["results"]
    out["one_at_a_time_fp64"]["note"] = ("the first %d requests of the stream, at their arrival times"
                                         % min(SERVE_FP64_PREFIX, nreq))
    # per-request error of the served (mixed) results against each request
    # replayed alone in FP64, over a seeded subset
    from rhyme_gb300.metrics import field_errors
    pick = sorted(np.random.default_rng(1).choice(nreq, size=min(SERVE_ERR_REQUESTS, nreq), replace=False))
    per = []
    names = ["rho", "rho_v1", "rho_v2", "rho_v3", "e_tot"]
    for i in pick:
        q = stream[i]
        ref = serving.run_alone(q, hydro_params(3), FP64)
        e = field_errors(served[i], ref, q["ndim"])
        fields = [names[0]] + names[1:1 + q["ndim"]] + [names[4]]
        per.append({"request": int(i), "ndim": q["ndim"], "dims": q["dims"], "steps": q["nsteps"],
                    "fp64_finite": bool(np.isfinite(ref).all()), "served_finite": bool(np.isfinite(served[i]).all()),
                    "l1": dict(zip(fields, [x[0] for x in e])), "linf": dict(zip(fields, [x[1] for x in e]))})
    finite = [x for x in per if all(np.isfinite(v) for v in x["l1"].values())]
    errs = {"requests": len(per), "definition": "per request and field: relative L1 = sum|d|/sum|f64|, "
            "relative Linf = max|d|/max|f64| over the interior; the served mixed result against the "
            "request replayed alone in plain FP64",
            "max_l1": {f: max((x["l1"].get(f, 0.0) for x in finite), default=None) for f in names},
            "max_linf": {f: max((x["linf"].get(f, 0.0) for x in finite), default=None) for f in names},
            "median_l1_rho": float(np.median([x["l1"]["rho"] for x in finite])) if finite else None,
            "requests_over_1e-6_l1_rho": sum(1 for x in finite if x["l1"]["rho"] > 1e-6),
            "requests_nonfinite_in_fp64": sum(1 for x in per if not x["fp64_finite"]),
            "requests_nonfinite_in_mixed_only": sum(1 for x in per if x["fp64_finite"] and not x["served_finite"]),
            "per_request": per}
    # capacity: the same requests all submitted at once (painted on the device)
    burst = [dict(q, arrival=0.0) for q in stream]
    r = serving.replay(burst, hydro_params(3, precision=MIXED), hbm_budget=150 << 30, max_active=256, paint=True)
    out["capacity_mixed_all_at_once"] = {"value": r["cell_updates"] / r["makespan"], "makespan_s": r["makespan"],
                                         "p50_s": float(np.percentile(r["latencies"], 50)),
                                         "p99_s": float(np.percentile(r["latencies"], 99)),
                                         "peak_active": r["peak_active"]}
    h = out["continuous_mixed"]
    value = allsum(h["value"], world)
    if rank == 0:
        cu = sum(int(np.prod([s - 4 for s in q["cells"].shape[1:]])) * q["nsteps"] for q in stream)
        line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": nreq,
                "warmup": 0, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
                "config": {"workload": "Poisson stream, %d requests at %.3g/s, seed 0; 1-/2-/3-D equiprobable, "
                                       "cells log-uniform in [256, 128^3], 50-500 steps; 150 GB budget"
                                       % (nreq, args.rate), "cell_updates": cu},
                "latency_s": {"p50": h["p50_s"], "p99": h["p99_s"], "requests": nreq},
                "errors_vs_fp64": errs,
                "e2e": {"value": value, "unit": METRIC, "note": "host arrays in, results drained to host"},
                "forms": out,
                "throughput_over_one_at_a_time": h["value"] / out["one_at_a_time_fp64"]["value"]}
        print(json.dumps(line), flush=True)


def run_rates(args, rank, local, world):
    """Arithmetic rates of this GPU for the operations the path is bound by
    (rhyme_gpu_rate_probe: FP64 FMA, division, square root, the restated
    C-library pow; FP32 FMA, approximate division, exp2f(y log2f(x)); the
    FP64 add and FP64 <-> FP32 conversions of the mixed state update),
    CUDA events, SM clock sampled during the launches. No clock control."""
    import torch
    from rhyme_gb300 import gpu
    torch.cuda.set_device(local)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    rates = {}
    t0 = time.time()
    for k, name in enumerate(gpu.RATE_KINDS):
        iters = 20000 if ("fma" in name or "add" in name or "conversions" in name) else 2000
        r, ms = gpu.rate_probe(k, iters)
        rates[name] = {"per_s": r, "ms": ms}
    t1 = time.time()
    clk = clocks.summary(t0, t1)
    clocks.stop()
    if rank == 0:
        per = lambda n: rates[n]["per_s"]
        line = {"metric": "operations/s", "workload": "rates", "n_gpus": 1, "rates": rates,
                "fp32_over_fp64_fma": per("fp32_fma_flops") / per("fp64_fma_flops"),
                "fp32_pow_over_fp64_pow": per("fp32_pow_exp2_log2") / per("fp64_pow"),
                "clocks": clk,
                "how": "8 independent chains per thread, 8 CTAs of 256 threads per SM, fastest of 3 launches "
                       "after a warm-up; FMA counted as 2 flops"}
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 300; 200 for batch4096, whose FP64 leg takes 2.3 s a step)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD)
    ap.add_argument("--precision", default=None, choices=["fp64", "mixed"])
    ap.add_argument("--no-compare", action="store_true", help="skip the other precision")
    ap.add_argument("--slabs", action="store_true",
                    help="the slab-decomposed form also on one GPU (one slab: the whole box)")
    ap.add_argument("--replicas", action="store_true",
                    help="under torchrun, step a replica of the box per rank instead of one box in slabs")
    ap.add_argument("--advance", type=int, default=None,
                    help="untimed steps before the warm-up (default: half the workload's run)")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-budget", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-threads", type=int, default=0,
                    help="OpenMP threads of the CPU oracle legs (default: every core)")
    ap.add_argument("--nboxes", type=int, default=4096)
    ap.add_argument("--requests", type=int, default=None,
                    help="requests of the serve workload (default %d)" % SERVE_REQUESTS)
    ap.add_argument("--rate", type=float, default=8.0)
    args = ap.parse_args()
    if args.steps is None:
        args.steps = BATCH_STEPS if args.workload == "batch4096" else 300
    if args.warmup < 3 and args.workload != "serve":
        raise SystemExit("at least 3 warm-up steps")
    rank, local, world = dist_init()
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.workload == "batch4096":
        run_batch(args, rank, local, world)
    elif args.workload == "serve":
        run_serve(args, rank, local, world)
    elif args.workload == "rates":
        run_rates(args, rank, local, world)
    elif args.slabs or (world > 1 and not args.replicas):
        run_slabs(args, rank, local, world)
    else:
        run_gpu(args, rank, local, world)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
