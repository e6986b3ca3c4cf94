"""The molecular rate pieces the device and the oracle's twin share (csrc/mol.h:
the MO-ADK prefactor numerator and the WFAT rate, with their Euler angles,
Wigner matrices, solid harmonics and structure factors) against an independent
restatement (oracle/oracle_mol_ref.c, C library functions and C99 complex).

Bar: the structure factor's pinned |G|^2 (test/Targets_test.jl:119-120) within
1e-12; G on every channel within 1e-12 of the twin's; sampled electrons the
same, their exit points, momenta and times identical (no molecular code enters
them), rates within 1e-10 relative and phases within 1e-10 rad; the reference's
molecular survivor counts hold through the independent pieces."""
import math

import numpy as np
import pytest

import _oracle as O
import etraj_gb300 as et
from _mol import hydrogen
from test_molecules import PINS
from test_oracle_pins import SURV, survivor_job

T800 = 2 * np.pi / (45.563352525 / 800.0)


@pytest.mark.parametrize("key,theta", [("G2_theta0", 0.0), ("G2_theta_pi2", math.pi / 2)])
def test_independent_structure_factor_meets_the_pins(key, theta):
    t, keep = hydrogen().to_c(0, wfat=True)
    G = O.mol_wfat_G(t, 0, 0, theta, 0.0, independent=True)
    assert math.isclose(abs(G) ** 2, PINS[key]["value"], rel_tol=1e-12)


def test_structure_factor_twin_matches_independent():
    t, keep = hydrogen().to_c(0, wfat=True)
    for nxi in range(t.wfat_nxi_max + 1):
        for m in range(-t.wfat_m_max, t.wfat_m_max + 1):
            for theta, chi in ((0.0, 0.0), (0.7, 1.3), (2.1, -0.4), (math.pi, 2.5)):
                a = O.mol_wfat_G(t, nxi, m, theta, chi)
                b = O.mol_wfat_G(t, nxi, m, theta, chi, independent=True)
                assert abs(a - b) <= 1e-12 * max(1.0, abs(a)), (nxi, m, theta, chi)


def jobs():
    ep = et.Cos4Laser(peak_int=2e14, wave_len=800.0, cyc_num=3, ellip=0.5, azi=0.3)
    common = dict(sample_t_intv=(-1.5 * T800, 1.5 * T800), sample_t_num=24, traj_t_final=3 * T800,
                  final_p_max=(2.0, 2.0, 2.0), final_p_num=(16, 16, 16), dimension=3, ss_kd_max=1.2,
                  ss_kd_num=21, ss_kz_max=1.0, ss_kz_num=9)
    rot = hydrogen(rot_α=0.4, rot_β=1.1, rot_γ=-0.6)
    return {
        "moadk-rotated-qtmc": et.make_job(init_cond_method="MOADK", laser=ep, target=rot, traj_phase_method="QTMC",
                                          **common),
        "mospane-ctmc": et.make_job(init_cond_method="MOSPANE", laser=ep, target=hydrogen(), **common),
        "mospa-rotated-scts": et.make_job(init_cond_method="MOSPA", laser=ep, target=rot, traj_phase_method="SCTS",
                                          **dict(common, ss_kd_num=9, ss_kz_num=5)),
        "wfat-rotated": et.make_job(init_cond_method="WFAT", laser=ep, target=rot, **common),
    }


def compare(a, b, job):
    rc = 2 * job.dimension + 1
    assert a.shape == b.shape
    np.testing.assert_array_equal(a[:, :rc], b[:, :rc])
    rel = np.abs(a[:, rc] - b[:, rc]) / a[:, rc]
    assert rel.max() <= 1e-10
    if a.shape[1] > rc + 1:
        d = np.angle(np.exp(1j * (a[:, rc + 1] - b[:, rc + 1])))
        assert np.abs(d).max() <= 1e-10


@pytest.mark.parametrize("name", sorted(jobs()))
def test_molecular_rates_twin_match_independent(name):
    job = jobs()[name]
    a = O.sample_all(job)
    with O.mol_independent():
        b = O.sample_all(job)
    assert a.shape[0] > 50
    compare(a, b, job)


MOL_CASES = [c for c in SURV["cases"] if "mol" in c["modifiers"] or "mol_rot" in c["modifiers"]]


@pytest.mark.parametrize("case", MOL_CASES, ids=["-".join(c["modifiers"]) for c in MOL_CASES])
def test_independent_molecular_pieces_meet_the_reference_survivor_counts(case):
    job = survivor_job(case["modifiers"])
    with O.mol_independent():
        r = O.sample_batch(job, SURV["batch_id"])
    if case["expected"] is None:
        assert r is not None and r.shape[1] > 0
    else:
        assert r is not None and list(r.shape) == case["expected"]
    compare(O.sample_batch(job, SURV["batch_id"]).T, r.T, job)
