"""Build recipe of libetraj_gb300.so (sm_103a only).

Each .cu file is compiled by nvcc in parallel and linked into
etraj.jl_gb300/lib/libetraj_gb300.so.  The FP64 translation units use
--fmad=false (every fused multiply-add is an explicit fma(), which is what
makes them bit-compatible with the CPU oracle); host code is compiled with
-ffp-contract=off for the same reason.  The FP32 bulk integrator keeps FMA
contraction on.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
ROOT = os.path.dirname(PKG)
LIB_DIR = os.path.join(PKG, "lib")
OBJ_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(LIB_DIR, "libetraj_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
          "-I" + HERE, "-I" + os.path.join(ROOT, "include"), "--expt-relaxed-constexpr"]
UNITS = {
    "api.cu": ["--fmad=false"],
    "job.cu": ["--fmad=false"],
    "pipeline.cu": ["--fmad=false"],
    "tune.cu": ["--fmad=false"],
    "batch.cu": ["--fmad=false"],
    "server.cu": ["--fmad=false"],
    "sampler.cu": ["--fmad=false"],
    "integrate_fp64.cu": ["--fmad=false"],
    "deposit.cu": ["--fmad=false"],
    "integrate_fp32.cu": ["--fmad=true"],
    "integrate_df.cu": ["--fmad=false"],
    "sampler_fp32.cu": ["--fmad=true"],
}
HEADERS = sorted(f for f in os.listdir(HERE) if f.endswith((".h", ".cuh")))


def nvcc():
    for c in (os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc"), "nvcc"):
        if os.path.sep not in c or os.path.exists(c):
            return c
    return "nvcc"


def _deps_time():
    paths = [os.path.join(HERE, h) for h in HEADERS] + [os.path.join(ROOT, "include", "etraj.h"),
                                                        os.path.abspath(__file__)]
    return max(os.path.getmtime(p) for p in paths)


def _compile(src, extra, verbose):
    obj = os.path.join(OBJ_DIR, os.path.splitext(src)[0] + ".o")
    srcp = os.path.join(HERE, src)
    if os.path.exists(obj) and os.path.getmtime(obj) > max(os.path.getmtime(srcp), _deps_time()):
        return obj
    cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", srcp, "-o", obj + ".tmp"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose=False, ptxas_verbose=False):
    os.makedirs(LIB_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    extra_v = ["-Xptxas", "-v"] if ptxas_verbose else []
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        futs = [ex.submit(_compile, src, flags + extra_v, verbose) for src, flags in UNITS.items()]
        objs = [f.result() for f in futs]
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        tmp = LIB + ".tmp.%d" % os.getpid()
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, ptxas_verbose="-v" in sys.argv))
