"""The FP32-bulk integrator against the FP64 plain path on the same sampled
electrons (through the C ABI).

Tolerances: the bulk path integrates with FP32 stages, compensated
(double-float) state and an FP32 field table, so per-trajectory final momenta
agree with FP64 to ~1e-6 relative (the integration tolerance), and the
momentum distribution of a large ensemble to <= 1e-3 relative L2.
"""
import numpy as np
import pytest

import _oracle as O
import etraj_gb300 as et
from etraj_gb300 import abi
from test_gpu_parity import job_of, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    e = et.Engine(device=0)
    yield e
    e.close()


def bulk(job):
    j = job.copy()
    j.precision = abi.PRECISION_FP32_BULK
    return j


CASES = [(d, p, t) for d in (2, 3) for p in ("CTMC", "QTMC", "SCTS") for t in ("H", "Ar")]


@pytest.mark.parametrize("dim,phase,target", CASES)
def test_bulk_final_states_close_to_fp64(eng, dim, phase, target):
    job = job_of(method="SPANE", dim=dim, phase=phase, target=target, nt=30, nkd=21, nkz=9,
                 laser="cos2", ellip=1.0 if dim == 2 else 0.5)
    init = O.sample_all(job)
    f64, s64, n64 = eng.integrate(job, init)
    f32, s32, n32 = eng.integrate(bulk(job), init)
    ok = (s64 == 0) & (s32 == 0)
    assert ok.mean() > 0.99
    nq = 2 * dim
    p64 = f64[ok][:, dim:nq]
    p32 = f32[ok][:, dim:nq]
    err = np.abs(p32 - p64).max(axis=1) / np.maximum(np.abs(p64).max(axis=1), 1e-3)
    assert np.median(err) < 1e-5, np.median(err)
    assert np.mean(err < 1e-3) > 0.98
    if phase != "CTMC":
        dphi = np.abs(f32[ok][:, -1] - f64[ok][:, -1])
        assert np.median(dphi) < 1e-4
    # same controller: step counts agree to within a few attempts for most electrons
    assert np.median(np.abs(n32[ok] - n64[ok])) <= 2


@pytest.mark.parametrize("phase", ["CTMC", "SCTS"])
def test_bulk_pmd_close_to_fp64(eng, phase):
    job = job_of(method="SPANE", dim=2, phase=phase, target="Ar", laser="cos2", ellip=1.0, mc=True,
                 nt=2000, nkd=100, nkz=1, pnum=(200, 200), pmax=2.0)
    r64, s64, a64 = eng.run(job, want_amplitude=True)
    r32, s32, a32 = eng.run(bulk(job), want_amplitude=True)
    assert r32.num_effective_traj == r64.num_effective_traj > 50000
    assert abs(r32.ion_prob - r64.ion_prob) <= 1e-6 * r64.ion_prob
    assert rel_l2(s32, s64) <= 1e-3, rel_l2(s32, s64)


def test_bulk_deterministic(eng):
    job = bulk(job_of(method="ADK", dim=3, phase="QTMC", target="H", nt=40, nkd=15, nkz=9))
    _, s1, a1 = eng.run(job, want_amplitude=True)
    _, s2, a2 = eng.run(job, want_amplitude=True)
    assert np.array_equal(s1, s2) and np.array_equal(a1, a2)
