"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle_capi.cpp (the restatement in rhyme_oracle.hpp) into
oracle/_build/liboracle.so with -O2 -ffp-contract=off -fopenmp, so that no
multiply-add is contracted and the outermost cell loop of each solver pass is
shared among OpenMP threads as in the reference. Host-portable: no
-march flags, builds the same on x86-64 and aarch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SOURCES = [os.path.join(HERE, "oracle_capi.cpp")]
DEPS = SOURCES + [os.path.join(HERE, "rhyme_oracle.hpp"),
                  os.path.join(os.path.dirname(HERE), "rhyme_gb300", "csrc", "libm_pow.h"),
                  os.path.join(os.path.dirname(HERE), "rhyme_gb300", "csrc", "libm_pow_tables.h")]


def needs_build():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in DEPS)


def build(force=False, verbose=False):
    """Compile liboracle.so if missing or stale; return its path."""
    if not force and not needs_build():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp.%d" % os.getpid()
    cmd = ["g++", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
           "-fPIC", "-shared", "-std=c++17", "-o", tmp] + SOURCES
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
