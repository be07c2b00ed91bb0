"""Callers of the library other than the Python tests, run on the GPU.

- tests/c_abi_driver.c: the driver loop of src/main.f90:106-177 in C99
  against include/rhyme_gpu.h alone, compiled, linked and run; its Sod tube
  conserves mass (outflow faces, no flow through them in 50 steps) and its
  last dt is positive.
- bench.py's slab-decomposed form (the multi-GPU layout of one box) on one
  GPU, where the single slab is the whole box and the device-to-device halo
  path has no neighbour: one JSON line with the contract's keys.
"""
import json
import os
import shutil
import subprocess
import sys

import pytest

from rhyme_gb300 import build

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_c_driver_runs_on_the_gpu(tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not found")
    exe = str(tmp_path / "driver")
    out = subprocess.run(["gcc", "-std=c99", "-O2", "-I", os.path.join(ROOT, "include"),
                          os.path.join(ROOT, "tests", "c_abi_driver.c"), "-L", build.OUT_DIR, "-lrhyme_gpu",
                          "-Wl,-rpath," + build.OUT_DIR, "-o", exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    run = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stderr
    # "mass M0 -> M1, last dt DT"
    words = run.stdout.replace(",", " ").split()
    m0, m1, dt = float(words[1]), float(words[3]), float(words[6])
    assert abs(m1 - m0) <= 1e-13 * m0 and dt > 0.0


@pytest.mark.timeout(600)
def test_bench_slab_form_on_one_gpu():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--slabs", "--workload", "spheres3d64",
                          "--steps", "3", "--warmup", "3", "--advance", "2", "--e2e-steps", "2"],
                         cwd=ROOT, capture_output=True, text=True, timeout=580)
    assert out.returncode == 0, out.stderr[-3000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "e2e", "config", "clocks", "gpu_launches"):
        assert k in d, k
    assert d["value"] > 0 and d["e2e"]["value"] > 0 and d["scaling"] == "strong"
