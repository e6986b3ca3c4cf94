"""The SPA sampler's saddle-point solve and quadratures against an independent
restatement (oracle/oracle_spa_ref.c: the C library's complex functions, its
own trust-region solve and adaptive Gauss-Kronrod, the laser written out from
the reference's formulas) instead of the code the device and the oracle's twin
share (csrc/spa.h).

Bar: the same electrons (a candidate within 1e-9 of the cutoff may fall either
way); exit points, momenta and times within 1e-9 relative (of the largest
magnitude in the column); rates within 1e-8 relative (the finite-difference
Jacobian of :280-292 divides solve residuals by 0.02); phases within 1e-8 rad.
The reference's own survivor counts (test/ElectronSamplers_test.jl) hold for
the independent restatement too."""
import json
import math
import os

import numpy as np
import pytest

import _oracle as O
import etraj_gb300 as et
from test_oracle_pins import SURV, survivor_job

T800 = 2 * np.pi / (45.563352525 / 800.0)


def jobs():
    bich = et.BichromaticLaser(et.Cos4Laser(peak_int=5e13, wave_len=800.0, cyc_num=8, ellip=1.0),
                               et.Cos4Laser(peak_int=5e13, wave_len=400.0, cyc_num=16, ellip=-1.0), delay=3.0)
    out = {
        "h-bichromatic-3d-qtmc-mc": et.make_job(
            init_cond_method="SPA", laser=bich, target=et.get_atom("H"), dimension=3,
            sample_t_intv=(-4 * T800, 4 * T800), sample_t_num=40, traj_t_final=6 * T800,
            final_p_max=(2.0, 2.0, 2.0), final_p_num=(16, 16, 16), sample_monte_carlo=True, mc_kt_num=60,
            mc_kd_max=1.0, mc_kz_max=1.0, traj_phase_method="QTMC", seed=3),
        "ar-cos2-ep-azi-scts-grid-prejac": et.make_job(
            init_cond_method="SPA", target=et.get_atom("Ar"), dimension=2,
            laser=et.Cos2Laser(peak_int=1.2e14, wave_len=800.0, cyc_num=4, ellip=0.6, azi=0.7, cep=0.4,
                               t_shift=5.0),
            sample_t_intv=(-1.5 * T800, 1.5 * T800), sample_t_num=40, traj_t_final=3 * T800,
            final_p_max=(2.0, 2.0), final_p_num=(16, 16), ss_kd_max=1.2, ss_kd_num=41,
            traj_phase_method="SCTS", rate_prefix=["Pre", "Jac"]),
        "xe-gauss-lp-qtmc-precc": et.make_job(
            init_cond_method="SPA", target=et.get_atom("Xe"), dimension=3,
            laser=et.GaussianLaser(peak_int=8e13, wave_len=1200.0, spread_cyc_num=1.5, ellip=0.0),
            sample_t_intv=(-2 * T800, 2 * T800), sample_t_num=30, traj_t_final=4 * T800,
            final_p_max=(2.0, 2.0, 2.0), final_p_num=(16, 16, 16), ss_kd_max=1.0, ss_kd_num=15,
            ss_kz_max=1.0, ss_kz_num=7, traj_phase_method="QTMC", rate_prefix="PreCC"),
    }
    return out


def sample_both(job):
    a = O.sample_all(job)
    with O.spa_independent():
        b = O.sample_all(job)
    return a, b


def compare(a, b, job):
    """Matches the rows of the two samples by (time, kd-ordering) position; both
    keep the reference's order, so a candidate dropped by one of them shows up
    as a shift, which the cutoff check below accounts for."""
    rate_col = 2 * job.dimension + 1
    ph = job.traj_phase_method != 0
    if a.shape != b.shape:
        # the two keep different sets: only candidates at the cutoff may differ
        cut = job.sample_cutoff_limit
        near = lambda s: np.sum(np.abs(s[:, rate_col] / cut - 1.0) < 1e-6)  # noqa: E731
        assert abs(a.shape[0] - b.shape[0]) <= near(a) + near(b), (a.shape, b.shape)
        return None
    cols = rate_col  # x, y[, z], kx, ky[, kz], t
    for c in range(cols):
        scale = max(np.max(np.abs(a[:, c])), 1e-300)
        assert np.max(np.abs(a[:, c] - b[:, c])) <= 1e-9 * scale, c
    rel = np.abs(a[:, rate_col] - b[:, rate_col]) / a[:, rate_col]
    assert rel.max() <= 1e-8
    if ph:
        d = np.angle(np.exp(1j * (a[:, rate_col + 1] - b[:, rate_col + 1])))
        assert np.abs(d).max() <= 1e-8
    return rel.max()


@pytest.mark.parametrize("name", sorted(jobs()))
def test_spa_twin_matches_independent_restatement(name):
    job = jobs()[name]
    a, b = sample_both(job)
    assert a.shape[0] > 50
    compare(a, b, job)


SPA_CASES = [c for c in SURV["cases"] if "spa" in c["modifiers"] and "mol" not in c["modifiers"]
             and "mol_rot" not in c["modifiers"]]


@pytest.mark.parametrize("case", SPA_CASES, ids=["-".join(c["modifiers"]) for c in SPA_CASES])
def test_independent_spa_meets_the_reference_survivor_counts(case):
    job = survivor_job(case["modifiers"])
    with O.spa_independent():
        r = O.sample_batch(job, SURV["batch_id"])
    if case["expected"] is None:
        assert r is not None and r.shape[1] > 0
    else:
        assert r is not None and list(r.shape) == case["expected"]
    a = O.sample_batch(job, SURV["batch_id"])
    compare(a.T, r.T, job)
