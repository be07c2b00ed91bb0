"""Benchmark of the GB300 MUSCL-Hancock hydro step (one JSON line on rank 0).

Default workload: 2-D 256x256 periodic shear slab (minmod, courant 0.8,
gamma 5/3), plain FP64, the configuration the plain GPU path is quoted on.
A step is one driver iteration (dt -> ghost fill -> solve) over the box.

  value   cell-updates/s with the state resident in HBM, timed with CUDA
          events on the library's stream around each step; L2 is flushed
          (a 512 MiB write) between timed steps, outside the events.
  e2e     the same metric through the reference-facing C-ABI with the state
          in host memory: per step host->device upload, dt (read back),
          ghost fill, solve and device->host download, wall-clock timed.
  roofline  HBM roofline of the dominant kernel (the interface-flux pass),
          from algorithmic bytes per step over its event-timed duration.
  cpu_baseline  the CPU oracle (a restatement of the reference's
          memory-intensive solver with OpenMP over the outer loop) on a
          bounded sample of the same workload, all host threads.

--impl reference times that CPU implementation alone on the same config.
Under torchrun each rank runs an independent replica (the path shards by
box; a single box is replicated) and value is the sum over ranks.
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


def workload(name, precision="fp64"):
    """(cells, dx, params, config dict) of a named workload."""
    from rhyme_gb300 import ic
    cells, dx, p, cfg = _workload(name)
    if precision == "mixed":
        from rhyme_gb300.params import MIXED
        p = dict(p, precision=MIXED)
        cfg = dict(cfg, workload=cfg["workload"].replace("plain FP64", "mixed FP32/FP64"))
    return cells, dx, p, cfg


def _workload(name):
    from rhyme_gb300 import ic
    if name == "slab2d":
        cells, dx, p = ic.slab_2d(n=256, seed=0)
        cfg = {"workload": "2-D 256x256 periodic shear slab, minmod, courant 0.8, plain FP64",
               "ndim": 2, "cells": 256 * 256, "steps_in_run": 500}
    elif name == "riemann1d":
        cells, dx, p = ic.riemann_1d(n=512, seed=0)
        cfg = {"workload": "1-D 512-cell seeded Riemann problem, van Leer, courant 0.8, plain FP64",
               "ndim": 1, "cells": 512, "steps_in_run": 100}
    elif name.startswith("spheres3d"):
        n = int(name[len("spheres3d"):] or 256)
        cells, dx, p = ic.spheres_3d(n=n, seed=0)
        cfg = {"workload": "3-D %d^3 periodic, 32 spheres + harmonic density, superbee, courant %.2g, plain FP64"
                           % (n, p["courant"]), "ndim": 3, "cells": n ** 3, "steps_in_run": 300}
    else:
        raise SystemExit("unknown workload %s" % name)
    return cells, dx, p, cfg


def algorithmic_bytes_per_cell(ndim):
    # U^n read once + U^{n+1} written once, NDIM+2 FP64 fields
    return 2 * (ndim + 2) * 8


class ClockSampler:
    """nvidia-smi SM clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None
        self.t0 = None

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

    def mark(self):
        return time.time()

    def stop(self, t_begin, t_end):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
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
    """Oracle cell-updates/s on the first steps of the workload (bounded)."""
    import oracle
    c = cells.copy()
    interior = int(np.prod([s - 4 for s in c.shape[1:]]))
    oracle.run(p, c, dx, 1, nthreads=nthreads)  # warm (allocates the workspace)
    done, t = 0, 0.0
    chunk = 1
    while done < steps_cap and t < budget_s:
        t0 = time.perf_counter()
        oracle.run(p, c, dx, chunk, nthreads=nthreads)
        t += time.perf_counter() - t0
        done += chunk
        chunk = min(chunk * 2, steps_cap - done) if done < steps_cap else 0
        if chunk <= 0:
            break
    return interior * done / t, done, t


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl"
        dist.init_process_group(backend=backend)
    return rank, local, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args, rank, world):
    if rank != 0:
        return
    cells, dx, p, cfg = workload(args.workload)
    p = dict(p, precision=0)  # the CPU implementation is FP64
    import oracle
    nthreads = os.cpu_count() or 1
    interior = cfg["cells"]
    c = cells.copy()
    if args.warmup:
        oracle.run(p, c, dx, args.warmup, nthreads=nthreads)
    t0 = time.perf_counter()
    oracle.run(p, c, dx, args.steps, nthreads=nthreads)
    t = time.perf_counter() - t0
    v = interior * args.steps / t
    sample = "%d timed steps of the workload after %d warm-up steps, OpenMP over the outer cell loop" % (
        args.steps, args.warmup)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": METRIC, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": cfg,
            "cpu_baseline": {"value": v, "unit": METRIC, "cores": nthreads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gpu(args, rank, local, world):
    import torch
    from rhyme_gb300 import gpu
    torch.cuda.set_device(local)
    cells, dx, p, cfg = workload(args.workload, args.precision)
    ndim = p["ndim"]
    interior = cfg["cells"]
    K, W = args.steps, args.warmup

    ctx = gpu.Context(p)
    state = cells.copy()
    box = ctx.register_box(state)
    stream = torch.cuda.ExternalStream(ctx.stream)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    ctx.run(box, dx, W, trace=False)
    ctx.synchronize()

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    barrier(world)
    torch.cuda.synchronize()
    ctx.synchronize()
    t_begin = time.time()
    for k in range(K):
        with torch.cuda.stream(stream):
            flush.zero_()
        starts[k].record(stream)
        ctx.run(box, dx, 1, trace=False)
        ends[k].record(stream)
    ctx.synchronize()
    torch.cuda.synchronize()
    barrier(world)
    t_end = time.time()
    clk = clocks.stop(t_begin, t_end)
    per_step = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms = allmax(sum(per_step), world)
    value = world * interior * K / (ms * 1e-3)

    # phase timing of the same step (direct launches, events between kernels)
    phases = ctx.profile_steps(box, dx, max(5, min(50, K)))
    dom = max(phases, key=phases.get)
    bpc = algorithmic_bytes_per_cell(ndim)
    peak, peak_kind = measured_peaks()
    achieved = interior * bpc / (phases[dom] * 1e-3) / 1e9
    traffic = ncu_traffic(args.workload, dom)

    # end to end through the C-ABI with the state in host memory
    host = cells.copy()
    ctx2 = gpu.Context(p)
    b2 = ctx2.register_box(host)
    hydro_bytes = (ndim + 2) * int(np.prod(host.shape[1:])) * 8
    ke = max(1, min(K, args.e2e_steps))
    for _ in range(min(W, 3)):
        ctx2.sync_to_device(b2)
        dt = ctx2.cfl_time_step(b2, dx)
        ctx2.set_boundaries(b2)
        ctx2.muscl_hancock_solve(b2, dx, dt)
        ctx2.sync_to_host(b2)
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(ke):
        ctx2.sync_to_device(b2)
        dt = ctx2.cfl_time_step(b2, dx)
        ctx2.set_boundaries(b2)
        ctx2.muscl_hancock_solve(b2, dx, dt)
        ctx2.sync_to_host(b2)
    te = allmax(time.perf_counter() - t0, world)
    barrier(world)
    e2e = world * interior * ke / te

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        nthreads = os.cpu_count() or 1
        v, n, t = cpu_sample(cells, dx, p, cfg["steps_in_run"], args.cpu_budget, nthreads)
        cpu = {"value": v, "unit": METRIC, "cores": nthreads, "kind": "port",
               "sample": "first %d steps of the same workload (%.1f s), CPU oracle, OpenMP" % (n, t)}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": K,
                "warmup": W, "ms_per_step": ms / K, "ms_per_step_median": statistics.median(per_step),
                "ms_per_step_max": max(per_step), "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64",
                "data": "synthetic",
                "config": dict(cfg, l2="flushed (512 MiB write) between timed steps, outside the events",
                               parallelism="replicas" if world > 1 else "single box"),
                "e2e": {"value": e2e, "unit": METRIC, "h2d_bytes_per_step": hydro_bytes + 8,
                        "d2h_bytes_per_step": hydro_bytes + 8 + 4, "steps": ke},
                "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                             "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                             "traffic": traffic, "bytes_per_cell_update": bpc,
                             "note": "the plain FP64 path is bound by the FP64 pipe, not HBM"},
                "phases_ms": phases, "clocks": clk,
                "gpu_launches": (5 if args.precision == "fp64" else 3 + ndim) * K,
                "cpu_baseline": cpu}
        print(json.dumps(line), flush=True)
    ctx2.close()
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="slab2d")
    ap.add_argument("--e2e-steps", type=int, default=200)
    ap.add_argument("--cpu-budget", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    args = ap.parse_args()
    if args.warmup < 3:
        raise SystemExit("at least 3 warm-up steps")
    rank, local, world = dist_init()
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gpu(args, rank, local, world)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
