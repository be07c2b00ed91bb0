"""Full-length parity of the 3-D 256^3 sphere workload against the CPU oracle.

Not a pytest module (the oracle needs about five minutes per 300-step run on
16 cores); run it by hand on a GPU machine:

    python tests/parity_full.py [--n 256] [--steps 300]

It steps the box on the GPU in plain FP64 and in mixed precision, and on the
CPU with the oracle, whose powers are the C library's pow (the arithmetic of
the compiled reference); the GPU's FP64 kernels raise powers with a
restatement of that pow, so the FP64 run must be bit-identical. It prints
one JSON object: per field relative L1 / Linf of each GPU form against the
oracle, the largest relative dt difference, whether the FP64 GPU run is
bit-identical to the oracle, and mixed against FP64 on the GPU.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle  # noqa: E402
from parity import field_errors  # noqa: E402
from rhyme_gb300 import gpu, ic  # noqa: E402
from rhyme_gb300.params import FP64, MIXED  # noqa: E402

NAMES = ["rho", "rho_vx", "rho_vy", "rho_vz", "e_tot"]


def on_gpu(cells, dx, p, steps, precision):
    c = cells.copy()
    with gpu.Context(dict(p, precision=precision)) as ctx:
        b = ctx.register_box(c)
        dts = ctx.run(b, dx, steps)
        ctx.sync_to_host(b)
    return c, np.asarray(dts)


def on_cpu(cells, dx, p, steps, mode):
    c = cells.copy()
    t0 = time.time()
    with oracle.pow_mode(mode):
        dts = oracle.run(dict(p, precision=FP64), c, dx, steps, nthreads=os.cpu_count() or 1)
    return c, np.asarray(dts), time.time() - t0


def compare(a, b, da, db):
    errs = field_errors(a, b, 3)
    return {"l1": dict(zip(NAMES, [e[0] for e in errs])), "linf": dict(zip(NAMES, [e[1] for e in errs])),
            "dt_max_rel": float(np.max(np.abs(da - db) / np.abs(db)))}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--steps", type=int, default=300)
    args = ap.parse_args()
    cells, dx, p = ic.spheres_3d(n=args.n, seed=0)
    f64, d64 = on_gpu(cells, dx, p, args.steps, FP64)
    mix, dmx = on_gpu(cells, dx, p, args.steps, MIXED)
    out = {"workload": "3-D %d^3 spheres (seed 0), %d steps" % (args.n, args.steps),
           "oracle_threads": os.cpu_count()}
    ref, dref, secs = on_cpu(cells, dx, p, args.steps, 0)
    out["oracle_libc_pow"] = {"seconds": secs, "fp64_gpu": compare(f64, ref, d64, dref),
                              "mixed_gpu": compare(mix, ref, dmx, dref),
                              "fp64_gpu_bit_identical": bool(np.array_equal(f64, ref) and np.array_equal(d64, dref))}
    out["mixed_vs_fp64_gpu"] = compare(mix, f64, dmx, d64)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
