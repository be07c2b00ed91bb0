"""Build recipe for librhyme_gpu.so (sm_103a), in-tree under rhyme_gb300/_build.

Each .cu translation unit is compiled in parallel with nvcc for
`-gencode arch=compute_103a,code=sm_103a`, then linked into one shared
library exporting the C-ABI of include/rhyme_gpu.h. The plain-FP64 units
are compiled with --fmad=false so the double arithmetic matches the
reference operation by operation; host code is compiled with
-ffp-contract=off for the same reason (aarch64 compilers contract by default).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "librhyme_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# translation unit -> extra nvcc flags
# (object name, source, extra flags). The plain FP64 units are compiled
# without FMA contraction (--fmad=false) so that their arithmetic matches the
# CPU oracle operation for operation; the mixed-precision units keep it.
# The FP32 arithmetic of the mixed form (sweeps, CFL) uses the hardware's
# approximate FP32 division and square root (<= 2 ulp) instead of the
# IEEE-exact sequences, with FP32 subnormals flushed to zero (the state's
# FP32 values are far above 1e-38; mirrors are flushed alike in every unit,
# rgpu_internal.h mirror_of); FP64 arithmetic is unaffected by these flags.
FP32_SWEEP_FLAGS = ["-prec-div=false", "-prec-sqrt=false", "-ftz=true"]

UNITS = [
    ("kernels_box", "kernels_box.cu", ["--fmad=false"]),
    ("kernels_elem", "kernels_elem.cu", ["--fmad=false"]),
    ("rhyme_gpu", "rhyme_gpu.cu", ["--fmad=false"]),
    ("kernels_mixed", "kernels_mixed.cu", FP32_SWEEP_FLAGS),
    ("sweeps_1d", "sweeps.cu", ["-DSWEEP_D=1"] + FP32_SWEEP_FLAGS),
    ("sweeps_2d", "sweeps.cu", ["-DSWEEP_D=2"] + FP32_SWEEP_FLAGS),
    ("sweeps_3d", "sweeps.cu", ["-DSWEEP_D=3"] + FP32_SWEEP_FLAGS),
    ("noalloc", "noalloc.cu", ["--fmad=false"]),
    ("kernels_batch", "kernels_batch.cu", ["--fmad=false"]),
    ("kernels_output", "kernels_output.cu", []),
    ("kernels_sanity", "kernels_sanity.cu", ["--fmad=false"]),
    ("kernels_paint", "kernels_paint.cu", ["--fmad=false"]),
    ("kernels_probe", "kernels_probe.cu", FP32_SWEEP_FLAGS),
]
HEADERS = ["hydro.cuh", "rgpu_internal.h", "detmath.h", "libm_pow.h", "libm_pow_tables.h", "box_elems.cuh", "sweep.cuh"]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build librhyme_gpu.so")


def _deps():
    deps = sorted({os.path.join(CSRC, src) for _, src, _ in UNITS}) + [os.path.join(CSRC, h) for h in HEADERS]
    deps.append(os.path.join(ROOT, "include", "rhyme_gpu.h"))
    deps.append(os.path.abspath(__file__))
    return deps


def needs_build():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in _deps() if os.path.exists(p))


def _compile(name, unit, flags, verbose):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(OUT_DIR, name + ".o")
    cmd = [nvcc()] + ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                             "-I", os.path.join(ROOT, "include"), "-c", src, "-o", obj] + flags
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (unit, r.stdout, r.stderr))
    return obj


def build(force=False, verbose=False):
    """Compile and link librhyme_gpu.so if missing or stale; return its path."""
    if not force and not needs_build():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda u: _compile(u[0], u[1], u[2], verbose), UNITS))
    tmp = LIB + ".tmp.%d" % os.getpid()
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
