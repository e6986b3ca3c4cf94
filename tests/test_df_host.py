"""The double-float integrator's per-electron solve (csrc/df_solve.cuh, the code
its kernel runs), built for the host with g++ and checked on the CPU against the
FP64 oracle on the oracle's own sampled electrons.

Bar, set by how far the FP64 solve itself moves when its rounding changes: in
an electron's first steps its error estimate is a sum that cancels to ~1e-11
of its terms, so FP64's own rounding moves it by ~1e-5 and the step sizes after
it by ~1e-6.  Run with the double-float table's field in place of its own (as
accurate, rounded differently), the oracle's asymptotic momenta move by a
median of 2e-10 on the elliptical argon job below and 4e-11 on the circular
one.  So: the same status for every electron; step attempts equal for all but
a few in 1e4; median relative difference of the asymptotic momenta below
1e-9; momentum distribution within 1e-5 relative L2 (on the full headline job,
4.0e6 electrons, the same comparison gives 3.7e-6)."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

import _oracle as O
import etraj_gb300 as et

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "etraj.jl_gb300", "csrc")
CUDA_INC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
T800 = 2 * np.pi / (45.563352525 / 800.0)


@pytest.fixture(scope="module")
def dfhost(tmp_path_factory):
    if not os.path.isfile(os.path.join(CUDA_INC, "cuda_runtime.h")):
        pytest.skip("CUDA headers (vector types) not found")
    out = str(tmp_path_factory.mktemp("dfhost") / "libdfhost.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
                    "-I" + CSRC, "-I" + os.path.join(ROOT, "include"), "-I" + CUDA_INC,
                    os.path.join(HERE, "df_host.cpp"), "-o", out], check=True)
    lib = C.CDLL(out)
    DP, IP = C.POINTER(C.c_double), C.POINTER(C.c_int32)
    lib.dfhost_integrate.argtypes = [C.c_void_p, C.c_int64, DP, C.c_double, DP, IP, IP]
    return lib


def host_integrate(lib, job, init, tmin=None):
    """The host build's solve of init's electrons; tmin (default: the job's first time
    sample) places the field table as the library does for the job."""
    if tmin is None:
        tmin = float(O.t_samples(job).min())
    n = init.shape[0]
    fin = np.zeros((n, job.state_size))
    st = np.zeros(n, np.int32)
    steps = np.zeros(n, np.int32)
    DP, IP = C.POINTER(C.c_double), C.POINTER(C.c_int32)
    lib.dfhost_integrate(C.addressof(job), n, np.ascontiguousarray(init).ctypes.data_as(DP),
                         tmin, fin.ctypes.data_as(DP), st.ctypes.data_as(IP),
                         steps.ctypes.data_as(IP))
    return fin, st, steps


def jobs():
    ar_cp = et.Cos2Laser(peak_int=1.2e14, wave_len=800.0, cyc_num=2, ellip=1.0)
    bich = et.BichromaticLaser(et.Cos4Laser(peak_int=5e13, wave_len=800.0, cyc_num=8, ellip=1.0),
                               et.Cos4Laser(peak_int=5e13, wave_len=400.0, cyc_num=16, ellip=-1.0), delay=0.0)
    common = dict(final_p_max=(2.0, 2.0), final_p_num=(400, 400))
    return {
        "ar-spane-scts-2d": et.make_job(init_cond_method="SPANE", laser=ar_cp, target=et.get_atom("Ar"), dimension=2,
                                        sample_t_intv=(-T800, T800), sample_t_num=60, traj_t_final=3 * T800,
                                        sample_monte_carlo=True, mc_kt_num=500, mc_kd_max=1.0,
                                        traj_phase_method="SCTS", seed=1, **common),
        "ar-adk-qtmc-3d": et.make_job(init_cond_method="ADK", target=et.get_atom("Ar"), dimension=3,
                                      laser=et.Cos2Laser(peak_int=1e14, wave_len=800.0, cyc_num=2, ellip=0.5, cep=0.3,
                                                         azi=0.4),
                                      sample_t_intv=(-T800, T800), sample_t_num=40, traj_t_final=3 * T800,
                                      ss_kd_max=1.0, ss_kd_num=15, ss_kz_max=1.0, ss_kz_num=9,
                                      final_p_max=(2.0, 2.0, 2.0), final_p_num=(64, 64, 64), traj_phase_method="QTMC"),
        "h-adk-ctmc-3d": et.make_job(init_cond_method="ADK", target=et.get_atom("H"), dimension=3,
                                     laser=et.Cos4Laser(peak_int=1e14, wave_len=800.0, cyc_num=2, ellip=0.0),
                                     sample_t_intv=(-T800, T800), sample_t_num=60, traj_t_final=3 * T800,
                                     ss_kd_max=1.0, ss_kd_num=21, ss_kz_max=1.0, ss_kz_num=11,
                                     final_p_max=(1.5, 1.5, 1.0), final_p_num=(200, 200, 1), traj_phase_method="CTMC"),
        "h-spa-qtmc-3d-bichromatic": et.make_job(init_cond_method="SPA", laser=bich, target=et.get_atom("H"),
                                                 dimension=3, sample_t_intv=(-4 * T800, 4 * T800), sample_t_num=100,
                                                 traj_t_final=6 * T800, final_p_max=(2.0, 2.0, 2.0),
                                                 final_p_num=(64, 64, 64), sample_monte_carlo=True, mc_kt_num=200,
                                                 mc_kd_max=1.0, mc_kz_max=1.0, traj_phase_method="QTMC", seed=2),
        "xe-adk-qtmc-2d-gauss": et.make_job(init_cond_method="ADK", target=et.get_atom("Xe"), dimension=2,
                                            laser=et.GaussianLaser(peak_int=1e14, wave_len=800.0, spread_cyc_num=1.0,
                                                                   ellip=1.0),
                                            sample_t_intv=(-2 * T800, 2 * T800), sample_t_num=100,
                                            traj_t_final=4 * T800, ss_kd_max=1.0, ss_kd_num=101,
                                            traj_phase_method="QTMC", **common),
    }


@pytest.mark.parametrize("name", sorted(jobs()))
def test_double_float_solve_tracks_the_oracle(dfhost, name):
    job = jobs()[name]
    init = O.sample_all(job)
    fin, st, steps = O.integrate(job, init)
    spec, _, _, p, _ = O.collect(job, init, fin, st, steps)
    f2, s2, k2 = host_integrate(dfhost, job, init)
    spec2, _, _, p2, _ = O.collect(job, init, f2, s2, k2)
    n = init.shape[0]
    assert n > 500
    assert np.array_equal(s2, st)
    assert np.sum(k2 != steps) <= 2 + n // 10000
    ion = (np.linalg.norm(p, axis=1) > 0) & (np.linalg.norm(p2, axis=1) > 0)
    rel = np.linalg.norm(p2[ion] - p[ion], axis=1) / np.linalg.norm(p[ion], axis=1)
    assert np.median(rel) <= 1e-9
    assert np.linalg.norm(spec2 - spec) / np.linalg.norm(spec) <= 1e-5
