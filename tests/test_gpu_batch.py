"""Multi-instance batches: many FP32-bulk jobs in one integrator launch.

The batch shares one work-stealing launch across all instances, but every
electron's integration depends only on its own instance's parameters and the
deposit is deterministic, so each instance must equal its job run alone, bit
for bit, and the weighted sum must equal the sum of the instance spectra in
instance order.
"""
import numpy as np
import pytest

import etraj_gb300 as et
from etraj_gb300 import abi
from test_gpu_parity import job_of

pytestmark = pytest.mark.gpu


def scan_jobs(n=8, seed=4):
    """A focal-volume intensity scan: Ar, Gaussian 800 nm linearly polarized,
    ADK Monte-Carlo in 3D (kd, kz), SCTS, 120 x 120 x 1 grid; intensities and
    sample counts log-uniform."""
    rng = np.random.default_rng(seed)
    jobs, ints = [], []
    for i in range(n):
        inten = float(np.exp(rng.uniform(np.log(5e13), np.log(4e14))))
        t_num = int(np.exp(rng.uniform(np.log(10), np.log(200))))
        laser = et.GaussianLaser(peak_int=inten, wave_len=800.0, spread_cyc_num=1.0, ellip=0.0)
        T = laser.Period()
        jobs.append(et.make_job(init_cond_method="ADK", laser=laser, target=et.get_atom("Ar"), dimension=3,
                                sample_t_intv=(-2 * T, 2 * T), sample_t_num=t_num, traj_t_final=4 * T,
                                final_p_max=(1.5, 1.5, 1.0), final_p_num=(120, 120, 1),
                                sample_monte_carlo=True, mc_kt_num=400, mc_kd_max=1.0, mc_kz_max=1.0,
                                traj_phase_method="SCTS", seed=100 + i, precision="fp32_bulk"))
        ints.append(inten)
    return jobs, np.array(ints)


def same(a, b):
    return (a is None and b is None) or np.array_equal(a.view(np.uint64), b.view(np.uint64))


def scalars(r):
    return (r.ion_prob, r.ion_prob_uncollected, r.num_effective_traj, r.num_failed_traj,
            r.num_ionized_traj, r.num_steps)


@pytest.fixture(scope="module")
def eng():
    e = et.Engine(device=0)
    yield e
    e.close()


def test_intensity_scan_equals_alone(eng):
    jobs, ints = scan_jobs()
    w = (ints / ints.max()) ** -1.5
    outs, wsum = eng.run_batch(jobs, want_spectrum=True, want_amplitude=True, weights=w)
    ref = 0.0
    for i, (job, (r, s, a)) in enumerate(zip(jobs, outs)):
        r0, s0, a0 = eng.run(job, want_spectrum=True, want_amplitude=True)
        assert r0.num_effective_traj > 0
        assert scalars(r) == scalars(r0), i
        assert same(s, s0) and same(a, a0), i
        ref = ref + w[i] * s0
    assert np.array_equal(wsum.view(np.uint64), np.asarray(ref).view(np.uint64))


def test_mixed_lasers_and_samplers_equal_alone(eng):
    kw = dict(dim=2, phase="QTMC", ellip=1.0, pnum=(96, 96))
    jobs = [job_of(method="ADK", nt=40, nkd=31, **kw),
            job_of(method="SPANE", laser="cos2", nt=60, nkd=41, **kw),
            job_of(method="SPA", laser="bichrom", nt=12, nkd=21, **kw),
            job_of(method="ADK", laser="gauss", mc=True, nt=50, nkd=30, nkz=1, **kw)]
    for j in jobs:
        j.precision = abi.PRECISION_FP32_BULK
    outs, wsum = eng.run_batch(jobs, want_spectrum=True, want_amplitude=True)
    assert wsum is None
    for job, (r, s, a) in zip(jobs, outs):
        r0, s0, a0 = eng.run(job, want_spectrum=True, want_amplitude=True)
        assert scalars(r) == scalars(r0)
        assert same(s, s0) and same(a, a0)


def test_batch_rejects_incompatible_jobs(eng):
    jobs, _ = scan_jobs(3)
    bad = jobs[1].copy()
    bad.final_p_num[0] = 121
    with pytest.raises(et.EtrajError) as e:
        eng.run_batch([jobs[0], bad])
    assert e.value.status == abi.ERR_INVALID_ARGUMENT
    fp64 = jobs[2].copy()
    fp64.precision = abi.PRECISION_FP64
    with pytest.raises(et.EtrajError):
        eng.run_batch([jobs[0], fp64])
    many = [jobs[0]] * 65
    with pytest.raises(et.EtrajError):
        eng.run_batch(many)
    # 64 small instances are accepted; identical jobs give identical results
    small = job_of(method="ADK", dim=2, nt=8, nkd=11, ellip=1.0, pnum=(32, 32))
    small.precision = abi.PRECISION_FP32_BULK
    outs, _ = eng.run_batch([small] * 64)
    for r, s, _ in outs[1:]:
        assert scalars(r) == scalars(outs[0][0]) and same(s, outs[0][1])
