"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/*.c into oracle/_build/liboracle.so with gcc.  FMA
contraction is disabled (-ffp-contract=off) so every rounding happens where
the source says; the explicit fma() calls in detmath.h stay fused.  The same
flags are used on x86-64 and aarch64.
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SOURCES = ["oracle_physics.c", "oracle_sampler.c", "oracle_solve.c", "oracle_spa_ref.c", "oracle_mol_ref.c"]


def _headers():
    """Every header the sources reach through quoted #includes (the oracle's own
    and those it shares with the device code), so that an edit to any of them
    rebuilds the library."""
    seen, todo = set(), [os.path.join(HERE, s) for s in SOURCES]
    while todo:
        path = todo.pop()
        for inc in re.findall(r'^\s*#\s*include\s+"([^"]+)"', open(path).read(), flags=re.M):
            dep = os.path.normpath(os.path.join(os.path.dirname(path), inc))
            if dep not in seen and os.path.exists(dep):
                seen.add(dep)
                todo.append(dep)
    return sorted(seen)


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(HERE, s) for s in SOURCES] + _headers() + [os.path.abspath(__file__)]
    return any(os.path.getmtime(d) > t for d in deps)


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
