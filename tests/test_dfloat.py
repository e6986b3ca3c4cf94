"""The double-float arithmetic of the FP32-pipe integrator (csrc/dfloat.h),
built for the host with g++ (no contraction, as the device build) and checked
against FP64: every operation within 2^-44 relative of the FP64 result of the
same inputs (a double-float carries a ~48-bit significand), exp down to e^-87
(relative to e^-69, absolute below), 2^x and log2, and the 2^(j/256) table
within 2^-47."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "etraj.jl_gb300", "csrc")
TOL = 2.0 ** -44


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("dfloat") / "libdfprobe.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
                    "-I" + CSRC, os.path.join(HERE, "dfloat_probe.cpp"), "-o", out], check=True)
    lib = C.CDLL(out)
    FP = C.POINTER(C.c_float)
    lib.probe_op.argtypes = [C.c_int, C.c_long, FP, FP, FP]
    lib.probe_exp2_table.argtypes = [FP]
    return lib


def split(v):
    hi = v.astype(np.float32)
    lo = (v - hi.astype(np.float64)).astype(np.float32)
    return np.stack([hi, lo], axis=1).ravel()


def join(p):
    p = p.reshape(-1, 2).astype(np.float64)
    return p[:, 0] + p[:, 1]


def run(lib, op, a, b=None):
    pa = split(a)
    pb = split(a if b is None else b)
    out = np.zeros_like(pa)
    fp = C.POINTER(C.c_float)
    lib.probe_op(op, a.size, pa.ctypes.data_as(fp), pb.ctypes.data_as(fp), out.ctypes.data_as(fp))
    # the exact values of the double-float inputs, for the FP64 references
    return join(out), join(pa), join(pb)


def rel(got, want):
    return np.max(np.abs(got - want) / np.maximum(np.abs(want), 1e-300))


rng = np.random.default_rng(11)
X = rng.uniform(-1, 1, 20000) * 10.0 ** rng.uniform(-6, 6, 20000)
Y = rng.uniform(-1, 1, 20000) * 10.0 ** rng.uniform(-6, 6, 20000)


def test_add_mul_fma_sqr(probe):
    r, a, b = run(probe, 0, X, Y)
    # the sloppy add: error relative to the larger operand
    assert np.max(np.abs(r - (a + b)) / np.maximum(np.abs(a), np.abs(b))) <= TOL
    r, a, b = run(probe, 1, X, Y)
    assert rel(r, a * b) <= TOL
    r, a, b = run(probe, 6, X, Y)
    assert np.max(np.abs(r - (a * b + a)) / np.maximum(np.abs(a * b), np.abs(a))) <= TOL
    r, a, _ = run(probe, 7, X)
    assert rel(r, a * a) <= TOL


def test_div_rcp_sqrt_rsqrt(probe):
    r, a, b = run(probe, 2, X, Y)
    assert rel(r, a / b) <= TOL
    r, a, _ = run(probe, 8, X)
    assert rel(r, 1.0 / a) <= TOL
    P = np.abs(X) + 1e-30
    r, a, _ = run(probe, 3, P)
    assert rel(r, np.sqrt(a)) <= TOL
    r, a, _ = run(probe, 4, P)
    assert rel(r, 1.0 / np.sqrt(a)) <= TOL


def test_exp_neg(probe):
    x = -np.concatenate([rng.uniform(0, 1e-3, 5000), rng.uniform(0, 1, 5000), rng.uniform(0, 86.9, 20000),
                         np.arange(0, 86, 0.25)])
    r, a, _ = run(probe, 5, x)
    # below e^-69 the low float is subnormal: the relative bound holds above, an
    # absolute one of 2^-44 e^-69 below (the integrator drops terms below e^-50)
    big = a >= -69.0
    assert rel(r[big], np.exp(a[big])) <= TOL
    assert np.max(np.abs(r[~big] - np.exp(a[~big]))) <= TOL * np.exp(-69.0)
    r, _, _ = run(probe, 5, np.array([-87.5, -200.0]))
    assert np.all(r == 0.0)


def test_exp2_log2(probe):
    # (below 2^-100 the low float of the result is subnormal)
    x = np.concatenate([rng.uniform(-100, 126, 20000), rng.uniform(-1, 1, 5000), rng.uniform(-1e-3, 1e-3, 5000)])
    r, a, _ = run(probe, 9, x)
    assert rel(r, np.exp2(a)) <= TOL
    v = np.concatenate([10.0 ** rng.uniform(-37, 37, 20000), rng.uniform(0.5, 2.0, 20000),
                        1.0 + rng.uniform(-1e-6, 1e-6, 100)])
    r, a, _ = run(probe, 10, v)
    # error of log2 relative to max(1, |log2 x|) (the step controller's powers see the absolute one)
    want = np.log2(a)
    assert np.max(np.abs(r - want) / np.maximum(1.0, np.abs(want))) <= TOL


def test_exp2_table(probe):
    t = np.zeros(512, dtype=np.float32)
    probe.probe_exp2_table(t.ctypes.data_as(C.POINTER(C.c_float)))
    v = join(t)
    want = np.exp2(np.arange(256, dtype=np.longdouble) / 256)
    assert np.max(np.abs((v.astype(np.longdouble) - want) / want)) <= 2.0 ** -47
    assert np.all(np.abs(t[1::2]) <= np.spacing(t[0::2]) / 2)  # normalized pairs
