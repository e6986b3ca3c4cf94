"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/*.c into oracle/_build/liboracle.so with gcc.  FMA
contraction is disabled (-ffp-contract=off) so every rounding happens where
the source says; the explicit fma() calls in detmath.h stay fused.  The same
flags are used on x86-64 and aarch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SOURCES = ["oracle_physics.c", "oracle_sampler.c", "oracle_solve.c"]
HEADERS = ["oracle.h", "oracle_internal.h", "oracle_sampler.h",
           os.path.join("..", "etraj.jl_gb300", "csrc", "detmath.h"),
           os.path.join("..", "include", "etraj.h")]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = SOURCES + HEADERS + [os.path.basename(__file__)]
    return any(os.path.getmtime(os.path.join(HERE, d)) > t for d in deps)


def build(force=False, verbose=False):
    """Compile the oracle if any source is newer than the library; return its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp.%d" % os.getpid()
    cmd = ["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wno-unused-function",
           "-o", tmp] + [os.path.join(HERE, s) for s in SOURCES] + ["-lm"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
