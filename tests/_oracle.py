"""ctypes wrapper of the CPU oracle (oracle/_build/liboracle.so) for the tests.

The oracle is the checker: tests call it to produce the expected values and
compare the CUDA library's results against them.
"""
import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import build as _oracle_build  # noqa: E402  (oracle/build.py)

sys.path.pop(0)

from etraj_gb300 import abi  # noqa: E402

_DP = C.POINTER(C.c_double)
_I32P = C.POINTER(C.c_int32)
_I64P = C.POINTER(C.c_int64)
_JP = C.POINTER(abi.Job)
_lib = None

SCALARS = ["ion_prob", "ion_prob_uncollected", "num_effective", "num_failed", "num_ionized",
           "num_steps"]


def lib():
    global _lib
    if _lib is None:
        path = _oracle_build.build()
        L = C.CDLL(path)
        sig = {
            "oracle_validate": (C.c_int, [_JP, C.c_char_p, C.c_int]),
            "oracle_batch_info": (C.c_int, [_JP, _I64P, _I64P]),
            "oracle_t_samples": (C.c_int, [_JP, _DP]),
            "oracle_sample_batch": (C.c_int, [_JP, C.c_int64, _DP, C.c_int64, _I64P]),
            "oracle_sample_all": (C.c_int, [_JP, _DP, C.c_int64, _I64P, C.c_int]),
            "oracle_integrate": (C.c_int, [_JP, C.c_int64, _DP, _DP, _I32P, _I32P, C.c_int]),
            "oracle_integrate_rmin": (C.c_int, [_JP, C.c_int64, _DP, _DP, _I32P, _I32P, _DP, C.c_int]),
            "oracle_collect": (C.c_int, [_JP, C.c_int64, _DP, _DP, _I32P, _I32P, _DP, _DP, _DP, _DP, _I32P]),
            "oracle_run": (C.c_int, [_JP, _DP, _DP, _DP, C.c_int]),
            "oracle_contributions": (C.c_int, [_JP, C.c_int64, _DP, _DP, _I32P, C.c_void_p, _DP, _DP]),
            "oracle_laser_eval": (None, [C.POINTER(abi.Laser), C.c_int64, _DP, _DP, _DP, _DP, _DP, _DP, _DP, _DP]),
            "oracle_laser_eval_complex": (None, [C.POINTER(abi.Laser), C.c_int64, _DP, _DP, _DP, _DP, _DP, _DP]),
            "oracle_target_eval": (None, [C.POINTER(abi.Target), C.c_int64, _DP, _DP, _DP]),
            "oracle_hartree_asymp_coeff": (C.c_double, [C.c_int, C.c_double, C.c_int]),
            "oracle_mol_wfat_G": (None, [C.POINTER(abi.Target), C.c_int, C.c_int, C.c_double, C.c_double, _DP]),
            "oracle_mol_wfat_G_ref": (None, [C.POINTER(abi.Target), C.c_int, C.c_int, C.c_double, C.c_double,
                                             _DP]),
            "oracle_set_mol_independent": (None, [C.c_int]),
            "oracle_rhs": (None, [_JP, C.c_double, _DP, _DP]),
            "oracle_sae_skip_exact": (C.c_int, [C.c_void_p]),
            "oracle_set_sae_skip": (None, [C.c_int]),
            "oracle_set_spa_independent": (None, [C.c_int]),
            "oracle_detmath": (None, [C.c_int, C.c_int64, _DP, _DP, _DP]),
            "oracle_tsit5_tableau": (None, [_DP, _DP, _DP]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(_DP)


def nthreads():
    return max(1, os.cpu_count() or 1)


def validate(job):
    buf = C.create_string_buffer(256)
    st = lib().oracle_validate(C.byref(job), buf, 256)
    return st, buf.value.decode()


def batch_info(job):
    nb, mx = C.c_int64(), C.c_int64()
    lib().oracle_batch_info(C.byref(job), C.byref(nb), C.byref(mx))
    return nb.value, mx.value


def t_samples(job):
    t = np.zeros(job.sample_t_num)
    lib().oracle_t_samples(C.byref(job), _p(t))
    return t


def sample_batch(job, batch_id):
    _, mx = batch_info(job)
    buf = np.zeros(job.rows * max(mx, 1))
    n = C.c_int64()
    st = lib().oracle_sample_batch(C.byref(job), batch_id, _p(buf), mx, C.byref(n))
    assert st == 0, st
    if n.value == 0:
        return None
    return buf[: job.rows * n.value].reshape(n.value, job.rows).T


def sample_all(job):
    nb, mx = batch_info(job)
    cap = nb * mx
    buf = np.zeros(job.rows * max(cap, 1))
    n = C.c_int64()
    st = lib().oracle_sample_all(C.byref(job), _p(buf), cap, C.byref(n), nthreads())
    assert st == 0, st
    return buf[: job.rows * n.value].reshape(n.value, job.rows).copy()


def integrate(job, init):
    init = np.ascontiguousarray(init, dtype=np.float64)
    n = init.shape[0]
    fin = np.zeros((n, job.state_size))
    status = np.zeros(n, dtype=np.int32)
    steps = np.zeros(n, dtype=np.int32)
    lib().oracle_integrate(C.byref(job), n, _p(init), _p(fin), status.ctypes.data_as(_I32P),
                           steps.ctypes.data_as(_I32P), nthreads())
    return fin, status, steps


def integrate_rmin(job, init):
    """integrate() plus each trajectory's least |r| over its accepted steps."""
    init = np.ascontiguousarray(init, dtype=np.float64)
    n = init.shape[0]
    fin = np.zeros((n, job.state_size))
    status = np.zeros(n, dtype=np.int32)
    steps = np.zeros(n, dtype=np.int32)
    rmin = np.zeros(n)
    lib().oracle_integrate_rmin(C.byref(job), n, _p(init), _p(fin), status.ctypes.data_as(_I32P),
                                steps.ctypes.data_as(_I32P), _p(rmin), nthreads())
    return fin, status, steps, rmin


def collect(job, init, fin, status, steps=None):
    n = init.shape[0]
    G = job.grid_size
    spec = np.zeros(G)
    amp = np.zeros(2 * G)
    sc = np.zeros(6)
    pinf = np.zeros((n, 3))
    binv = np.zeros(n, dtype=np.int32)
    st = np.ascontiguousarray(status, dtype=np.int32)
    sp = None if steps is None else np.ascontiguousarray(steps, dtype=np.int32)
    lib().oracle_collect(C.byref(job), n, _p(np.ascontiguousarray(init)), _p(np.ascontiguousarray(fin)),
                         st.ctypes.data_as(_I32P), None if sp is None else sp.ctypes.data_as(_I32P),
                         _p(spec), _p(amp), _p(sc), _p(pinf), binv.ctypes.data_as(_I32P))
    return spec, amp, dict(zip(SCALARS, sc)), pinf, binv


def contributions(job, init, fin, status):
    n = init.shape[0]
    key = np.zeros(n, dtype=np.uint32)
    cre = np.zeros(n)
    cim = np.zeros(n)
    st = np.ascontiguousarray(status, dtype=np.int32)
    lib().oracle_contributions(C.byref(job), n, _p(np.ascontiguousarray(init)), _p(np.ascontiguousarray(fin)),
                               st.ctypes.data_as(_I32P), key.ctypes.data, _p(cre), _p(cim))
    return key, cre, cim


def run(job):
    G = job.grid_size
    spec = np.zeros(G)
    amp = np.zeros(2 * G)
    sc = np.zeros(6)
    st = lib().oracle_run(C.byref(job), _p(spec), _p(amp), _p(sc), nthreads())
    assert st == 0, st
    return spec, amp, dict(zip(SCALARS, sc))


def laser_eval(laser_c, t):
    t = np.ascontiguousarray(t, dtype=np.float64)
    n = t.size
    out = {k: np.zeros(n) for k in ("Fx", "Fy", "Ax", "Ay", "dFx", "dFy", "env")}
    lib().oracle_laser_eval(C.byref(laser_c), n, _p(t), *[_p(out[k]) for k in ("Fx", "Fy", "Ax", "Ay", "dFx", "dFy", "env")])
    return out


def laser_eval_complex(laser_c, t):
    t = np.ascontiguousarray(t, dtype=np.complex128)
    n = t.size
    tr, ti = np.ascontiguousarray(t.real), np.ascontiguousarray(t.imag)
    out = {k: np.zeros(2 * n) for k in ("Ax", "Ay", "Fx", "Fy")}
    lib().oracle_laser_eval_complex(C.byref(laser_c), n, _p(tr), _p(ti), *[_p(out[k]) for k in ("Ax", "Ay", "Fx", "Fy")])
    return {k: v[0::2] + 1j * v[1::2] for k, v in out.items()}


def target_eval(target_c, xyz):
    xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    n = xyz.shape[0]
    V = np.zeros(n)
    F = np.zeros((n, 3))
    lib().oracle_target_eval(C.byref(target_c), n, _p(xyz), _p(V), _p(F))
    return V, F


def sae_skip_exact(target_c):
    return bool(lib().oracle_sae_skip_exact(C.byref(target_c)))


def set_sae_skip(enable):
    lib().oracle_set_sae_skip(1 if enable else 0)


class spa_independent:
    """Within the block the oracle's SPA candidates come from the independent
    restatement (oracle_spa_ref.c) instead of the device's twin."""

    def __enter__(self):
        lib().oracle_set_spa_independent(1)

    def __exit__(self, *a):
        lib().oracle_set_spa_independent(0)


def rhs(job, t, u):
    u = np.ascontiguousarray(u, dtype=np.float64)
    du = np.zeros_like(u)
    lib().oracle_rhs(C.byref(job), t, _p(u), _p(du))
    return du


DETMATH = {"exp": 0, "expm1": 1, "log": 2, "log1p": 3, "sin": 4, "cos": 5, "tanh": 6, "atan": 7,
           "atan2": 8, "asinh": 9, "pow": 10}


def detmath(fn, x, y=None):
    x = np.ascontiguousarray(x, dtype=np.float64)
    yy = np.ascontiguousarray(y if y is not None else np.zeros_like(x), dtype=np.float64)
    out = np.zeros_like(x)
    lib().oracle_detmath(DETMATH[fn], x.size, _p(x), _p(yy), _p(out))
    return out


def tsit5_tableau():
    c = np.zeros(7)
    a = np.zeros(42)
    bt = np.zeros(7)
    lib().oracle_tsit5_tableau(_p(c), _p(a), _p(bt))
    return c, a.reshape(7, 6), bt


def mol_wfat_G(target, nxi, m, theta, chi, independent=False):
    """G_{n_xi m}(theta, chi) from the device's twin (mol.h) or, with independent,
    from oracle_mol_ref.c."""
    out = np.zeros(2)
    f = lib().oracle_mol_wfat_G_ref if independent else lib().oracle_mol_wfat_G
    f(C.byref(target), nxi, m, theta, chi, _p(out))
    return complex(out[0], out[1])


class mol_independent:
    """Within the block the oracle's molecular prefactor numerators and WFAT
    rates come from the independent restatement (oracle_mol_ref.c)."""

    def __enter__(self):
        lib().oracle_set_mol_independent(1)

    def __exit__(self, *a):
        lib().oracle_set_mol_independent(0)
