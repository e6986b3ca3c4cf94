"""The Gaussian transverse-momentum proposal (etraj_mc_proposal ADK_GAUSS, not in
the reference; a Gaussian of the ADK width for the transverse momenta), checked on
the CPU with the oracle: the checks of the job, and that it estimates the same
rate integral as the reference's uniform draws -- the sum of the sampled rates,
each carrying its dkdt -- over the same (seeded) time samples, while it keeps
more of its candidates."""
import ctypes as C

import numpy as np
import pytest

import _oracle as O
import etraj_gb300 as et
from etraj_gb300 import abi

T800 = 2 * np.pi / (45.563352525 / 800.0)


def job(method="ADK", dim=2, proposal="uniform", seed=0, nkt=4000, nt=40, mc=True):
    laser = et.Cos4Laser(peak_int=1e14, wave_len=800.0, cyc_num=2, ellip=0.3)
    kw = dict(init_cond_method=method, laser=laser, target=et.get_atom("H"), dimension=dim,
              sample_t_intv=(-T800 / 2, T800 / 2), sample_t_num=nt, traj_t_final=2 * T800,
              final_p_max=(1.5,) * dim, final_p_num=(50,) * dim, traj_phase_method="CTMC", seed=seed,
              mc_kt_proposal=proposal)
    if mc:
        kw.update(sample_monte_carlo=True, mc_kt_num=nkt, mc_kd_max=1.2, mc_kz_max=1.0)
    else:
        kw.update(ss_kd_max=1.2, ss_kd_num=11, ss_kz_max=1.0, ss_kz_num=5)
    return et.make_job(**kw)


def test_proposal_checks():
    lib = abi.load_library()
    buf = C.create_string_buffer(256)
    for bad in (job(mc=False, proposal="adk_gauss"), job(method="SPA", proposal="adk_gauss")):
        assert lib.etraj_validate(C.byref(bad), buf, 256) == abi.ERR_INVALID_ARGUMENT
        assert b"ADK_GAUSS" in buf.value
        st, msg = O.validate(bad)
        assert st == abi.ERR_INVALID_ARGUMENT and "ADK_GAUSS" in msg
    good = job(proposal="adk_gauss")
    assert lib.etraj_validate(C.byref(good), buf, 256) == abi.OK
    with pytest.raises(ValueError):
        job(proposal="cauchy")


def rate_sum(j):
    """Sum of the kept rates, its Monte-Carlo error (sqrt of the sum of squares)
    and the number kept."""
    w = O.sample_all(j)[:, 2 * j.dimension + 1]
    return w.sum(), np.sqrt((w * w).sum()), w.size


@pytest.mark.parametrize("method,dim", [("ADK", 2), ("ADK", 3), ("SPANE", 2)])
def test_gaussian_proposal_estimates_the_same_rate_integral(method, dim):
    # the time samples depend on the seed alone, so each seed pairs the two proposals
    # on the same times and their difference is the transverse-momentum sampling's
    u = np.array([rate_sum(job(method, dim, "uniform", seed=s)) for s in range(6)])
    g = np.array([rate_sum(job(method, dim, "adk_gauss", seed=s)) for s in range(6)])
    z = (g[:, 0] - u[:, 0]) / np.hypot(g[:, 1], u[:, 1])
    assert np.abs(z).max() <= 4.0
    assert abs(g[:, 0].sum() / u[:, 0].sum() - 1) <= 0.02
    assert (g[:, 2] > u[:, 2]).all()  # more candidates kept above the cutoff


def test_gaussian_draws_follow_the_adk_width():
    j = job("ADK", 2, "adk_gauss", nkt=20000, nt=4)
    init = O.sample_all(j)
    assert init.shape[0] > 1000
    # kd is the transverse momentum along (-sin phi, cos phi): |k0| = |kd|
    kd = np.hypot(init[:, 2], init[:, 3])
    assert kd.max() <= 1.2 + 1e-12
