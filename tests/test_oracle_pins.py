"""Pins the CPU oracle against the reference's own known-answer tests (CPU only).

- sampler survivor counts: test/ElectronSamplers_test.jl:53-292 (tests/golden/sampler_survivors.json)
- A' = -F for every laser:   test/Lasers_test.jl:42-54, 88-100
- F = -grad V, potential values and the He asymptotic coefficient:
  test/Targets_test.jl:31-36, 56-64
- the Tsit5 tableau satisfies the order conditions of a 5(4) pair
- detmath agrees with glibc to a few ulp
"""
import json
import math
import os

import numpy as np
import pytest

import _oracle as O
import etraj_gb300 as et
from etraj_gb300 import abi
from _mol import hydrogen

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
with open(os.path.join(GOLDEN, "sampler_survivors.json")) as f:
    SURV = json.load(f)
with open(os.path.join(GOLDEN, "physics_pins.json")) as f:
    PINS = json.load(f)

BUILT_METHODS = {"ADK", "SPANE", "SPA", "WFAT"}


def survivor_job(modifiers):
    """The sampler of an `init_sampler(; merge(params, ...)...)` test case; the
    molecule is get_mol("Hydrogen") (rotated by rot_β=π/2, rot_γ=π/2 for mol_rot)."""
    p = dict(SURV["common"])
    for m in modifiers:
        p.update(SURV["modifiers"][m])
    L = p.pop("laser")
    p.pop("target")
    laser = et.Cos4Laser(peak_int=L["peak_int"], wave_len=L["wave_len"], cyc_num=L["cyc_num"],
                         ellip=L["ellip"])
    if "mol_rot" in modifiers:
        target = hydrogen(rot_β=math.pi / 2, rot_γ=math.pi / 2)
    elif "mol" in modifiers:
        target = hydrogen()
    else:
        target = et.get_atom("H")
    dim = p["dimension"]
    return et.make_job(laser=laser, target=target, traj_t_final=200.0,
                       final_p_max=(2.0,) * dim, final_p_num=(10,) * dim, **p)


def _case_id(c):
    return "-".join(c["modifiers"]) or "adk"


@pytest.mark.parametrize("case", SURV["cases"], ids=[_case_id(c) for c in SURV["cases"]])
def test_sampler_survivor_counts(case):
    job = survivor_job(case["modifiers"])
    if O.validate(job)[0] == 2:
        pytest.skip("sampler not built yet")
    r = O.sample_batch(job, SURV["batch_id"])
    if case["expected"] is None:
        # Monte-Carlo cases: the reference only asserts a non-empty batch
        assert r is not None and r.shape[1] > 0
    else:
        assert r is not None and list(r.shape) == case["expected"], (case, None if r is None else r.shape)


def test_hartree_coefficient_he():
    p = PINS["he_asymp_coeff"]
    c = O.lib().oracle_hartree_asymp_coeff(p["Z"], p["Ip"], p["l"])
    assert c == pytest.approx(p["value"], rel=1e-14)
    assert et.hartree_asymp_coeff(p["Z"], p["Ip"], p["l"]) == pytest.approx(p["value"], rel=1e-14)
    assert et.get_atom("He").asymp_coeff == pytest.approx(p["value"], rel=1e-14)


def test_potential_values():
    # Julia's `≈` is rtol = sqrt(eps); the soft core 1e-10 shifts the value by 1.7e-11
    V, _ = O.target_eval(et.get_atom("H").to_c(), [1.0, 1.0, 1.0])
    assert V[0] == pytest.approx(PINS["h_potential_111"]["value"], rel=1.5e-8)
    he = et.get_atom("He").to_c()
    V, _ = O.target_eval(he, [1.0, 1.0, 1.0])
    r = 1.73205081
    expect = -(1.0 + 1.230723 * math.exp(-0.6620055 * r) - 1.325040 * r * math.exp(-1.236224 * r)
               - 0.2307230 * math.exp(-0.4804286 * r)) / r
    assert V[0] == pytest.approx(expect, rel=1e-7)


@pytest.mark.parametrize("atom", ["H", "He", "Ar", "Xe"])
def test_force_is_minus_gradient(atom):
    tc = et.get_atom(atom).to_c()
    h = 1e-6
    for p in PINS["gradient_points"]:
        p = np.array(p, dtype=float)
        _, F = O.target_eval(tc, p)
        grad = np.zeros(3)
        for k in range(3):
            e = np.zeros(3)
            e[k] = h
            Vp, _ = O.target_eval(tc, p + e)
            Vm, _ = O.target_eval(tc, p - e)
            grad[k] = (Vp[0] - Vm[0]) / (2 * h)
        np.testing.assert_allclose(-grad, F[0], rtol=1e-7, atol=1e-9)


def _lasers():
    l6 = PINS["laser_l6"]
    l7 = PINS["laser_l7"]
    kw6 = {k: l6[k] for k in ("peak_int", "wave_len", "cyc_num", "ellip", "azi", "cep", "t_shift")}
    kw7 = {k: l7[k] for k in ("peak_int", "wave_len", "cyc_num", "ellip", "azi", "cep", "t_shift")}
    g6 = dict(kw6)
    g6["spread_cyc_num"] = g6.pop("cyc_num")
    g7 = dict(kw7)
    g7["spread_cyc_num"] = g7.pop("cyc_num")
    out = [et.Cos2Laser(**kw6), et.Cos2Laser(**kw7), et.Cos4Laser(**kw6), et.Cos4Laser(**kw7),
           et.GaussianLaser(**g6), et.GaussianLaser(**g7)]
    out.append(et.BichromaticLaser(et.Cos4Laser(peak_int=1e15, wave_len=800, cyc_num=10, ellip=1),
                                   et.Cos4Laser(peak_int=1e15, wave_len=400, cyc_num=20, ellip=-1),
                                   delay=20.67))
    return out


@pytest.mark.parametrize("laser", _lasers(), ids=lambda l: repr(l)[:40])
def test_vector_potential_derivative_is_minus_field(laser):
    """A'(t) = -F(t) at t = 0 and t = 10 (test/Lasers_test.jl:42-54)."""
    lc = laser.to_c()
    h = 1e-4
    for t in PINS["laser_derivative_times"]:
        ts = np.array([t - 2 * h, t - h, t + h, t + 2 * h, t])
        v = O.laser_eval(lc, ts)
        for A, F in (("Ax", "Fx"), ("Ay", "Fy")):
            a = v[A]
            dA = (a[0] - 8 * a[1] + 8 * a[2] - a[3]) / (12 * h)
            scale = max(abs(v[F][4]), 1e-3 * laser_f0(laser))
            assert abs(dA + v[F][4]) <= 1e-7 * scale, (t, A, dA, v[F][4])


def laser_f0(laser):
    if isinstance(laser, et.BichromaticLaser):
        return laser[1].LaserF0() + laser[2].LaserF0()
    return laser.LaserF0()


@pytest.mark.parametrize("laser", _lasers(), ids=lambda l: repr(l)[:40])
def test_field_derivative_matches_finite_difference(laser):
    """The forward-mode derivative SPANE needs (SPANESampler.jl:168-169)."""
    lc = laser.to_c()
    h = 1e-4
    for t in (-40.0, 0.0, 10.0, 35.5):
        ts = np.array([t - 2 * h, t - h, t + h, t + 2 * h, t])
        v = O.laser_eval(lc, ts)
        for F, dF in (("Fx", "dFx"), ("Fy", "dFy")):
            f = v[F]
            fd = (f[0] - 8 * f[1] + 8 * f[2] - f[3]) / (12 * h)
            assert abs(fd - v[dF][4]) <= 1e-7 * laser_f0(laser), (t, F, fd, v[dF][4])


@pytest.mark.parametrize("laser", _lasers()[:6], ids=lambda l: repr(l)[:40])
def test_complex_time_field_matches_real(laser):
    """The complex-time evaluation used by SPA reduces to the real one on the real axis
    and is analytic (Cauchy-Riemann) off it, except for the real(t) window."""
    lc = laser.to_c()
    t = np.array([-30.0, 0.0, 12.5, 40.0])
    vr = O.laser_eval(lc, t)
    vc = O.laser_eval_complex(lc, t + 0j)
    for k in ("Ax", "Ay", "Fx", "Fy"):
        np.testing.assert_allclose(vc[k].real, vr[k], rtol=1e-13, atol=1e-15)
        np.testing.assert_allclose(vc[k].imag, 0.0, atol=1e-15)
    # dA/d(i tau) = -F at t + i tau, away from the window edges
    tau, h = 3.0, 1e-4
    zp = O.laser_eval_complex(lc, t + 1j * (tau + h))
    zm = O.laser_eval_complex(lc, t + 1j * (tau - h))
    z0 = O.laser_eval_complex(lc, t + 1j * tau)
    for A, F in (("Ax", "Fx"), ("Ay", "Fy")):
        dA = (zp[A] - zm[A]) / (2j * h)
        np.testing.assert_allclose(dA, -z0[F], rtol=1e-6, atol=1e-9)


def test_laser_getters():
    """Getter identities of test/Lasers_test.jl:29-39 and the unit-free constructors."""
    l1 = et.Cos2Laser(peak_int=4e14, wave_len=800.0, cyc_num=2.0, ellip=1.0, azi=math.pi / 2,
                      cep=math.pi, t_shift=10.0)
    l2 = et.Cos2Laser(peak_int=4e14, ang_freq=0.05695419065625, cyc_num=2.0, ellip=1.0,
                      azi=math.pi / 2, cep=math.pi, t_shift=10.0)
    l3 = et.Cos2Laser(peak_int=4e14, wave_len=800.0, duration=220.63996467273427, ellip=1.0,
                      azi=math.pi / 2, cep=math.pi, t_shift=10.0)
    assert l1 == l2
    assert l1.CycNum() == pytest.approx(l3.CycNum(), rel=1e-14)
    assert l1.AngFreq() == 45.563352525 / l1.WaveLen()
    assert l1.Period() == 2 * math.pi / l1.AngFreq()
    assert l1.LaserF0() == math.sqrt(l1.PeakInt() / (1.0 + l1.Ellipticity() ** 2) / 3.50944521e16)
    assert l1.LaserA0() == l1.LaserF0() / l1.AngFreq()
    g = et.GaussianLaser(peak_int=4e14, wave_len=800.0, spread_cyc_num=2.0, ellip=1.0)
    g2 = et.GaussianLaser(peak_int=4e14, wave_len=800.0, FWHM_duration=g.FWHM_Duration(), ellip=1.0)
    assert g2.SpreadCycNum() == pytest.approx(2.0, rel=1e-14)


def test_tsit5_order_conditions():
    c, A, bt = O.tsit5_tableau()
    b = np.append(A[6], 0.0)  # FSAL: the 7th stage has weight 0
    AA = np.zeros((7, 7))
    AA[:, :6] = A
    assert np.max(np.abs(AA.sum(1) - c)) < 1e-15
    Ac = AA @ c

    def conds(w):
        return [w.sum() - 1, w @ c - 0.5, w @ c ** 2 - 1 / 3, w @ Ac - 1 / 6, w @ c ** 3 - 0.25,
                w @ (c * Ac) - 1 / 8, w @ (AA @ c ** 2) - 1 / 12, w @ (AA @ Ac) - 1 / 24]

    order5 = conds(b) + [b @ c ** 4 - 0.2, b @ (c * c * Ac) - 0.1, b @ (Ac * Ac) - 0.05,
                         b @ (c * (AA @ c ** 2)) - 1 / 15, b @ (AA @ c ** 3) - 0.05,
                         b @ (c * (AA @ Ac)) - 1 / 30, b @ (AA @ (c * Ac)) - 1 / 40,
                         b @ (AA @ (AA @ c ** 2)) - 1 / 60, b @ (AA @ (AA @ Ac)) - 1 / 120]
    assert max(abs(x) for x in order5) < 1e-14
    assert max(abs(x) for x in conds(b - bt)) < 1e-14
    assert abs(bt.sum()) < 1e-16


def test_least_radius_of_the_oracle():
    """The least |r| of a trajectory is at most its initial radius and at most
    its final radius, and matches a plain integrate() step for step."""
    T = 2 * math.pi / (45.563352525 / 800.0)
    job = et.make_job(init_cond_method="ADK", laser=et.Cos4Laser(peak_int=1e14, wave_len=800.0, cyc_num=2, ellip=0.0),
                      target=et.get_atom("H"), dimension=2, sample_t_intv=(-T, T), sample_t_num=6,
                      traj_t_final=2 * T, final_p_max=(1.5, 1.5), final_p_num=(32, 32), ss_kd_max=1.0,
                      ss_kd_num=9, ss_kz_num=0, ss_kz_max=0.0, traj_phase_method="CTMC")
    init = O.sample_all(job)
    assert init.shape[0] > 10
    fin, st, steps, rmin = O.integrate_rmin(job, init)
    fin0, st0, steps0 = O.integrate(job, init)
    assert np.array_equal(fin, fin0) and np.array_equal(st, st0) and np.array_equal(steps, steps0)
    r0 = np.hypot(init[:, 0], init[:, 1])
    rf = np.hypot(fin[:, 0], fin[:, 1])
    assert np.all(rmin > 0.0) and np.all(rmin <= r0) and np.all(rmin[st == 0] <= rf[st == 0])


def _ulp_err(got, ref):
    ref = np.asarray(ref, dtype=np.float64)
    sp = np.spacing(np.abs(ref))
    return np.max(np.abs(got - ref) / np.where(sp > 0, sp, 5e-324))


@pytest.mark.parametrize("fn,lo,hi,bound", [
    ("exp", -700, 700, 2), ("exp", -1, 1, 2), ("expm1", -30, 30, 2), ("expm1", -0.3, 0.3, 2),
    ("log", 1e-300, 1e300, 2), ("log", 0.5, 2.0, 2), ("log1p", -0.5, 10, 3),
    ("sin", -1000, 1000, 2), ("cos", -1000, 1000, 2), ("tanh", -25, 25, 3), ("tanh", -0.5, 0.5, 3),
    ("atan", -50, 50, 4), ("asinh", -100, 100, 4), ("asinh", -2, 2, 4)])
def test_detmath_accuracy(fn, lo, hi, bound):
    rng = np.random.default_rng(1)
    if fn == "log" and lo > 0 and hi / lo > 1e10:
        x = np.exp(rng.uniform(math.log(lo), math.log(hi), 20000))
    else:
        x = rng.uniform(lo, hi, 20000)
    got = O.detmath(fn, x)
    ref = getattr(np, {"asinh": "arcsinh", "atan": "arctan"}.get(fn, fn))(x)
    assert _ulp_err(got, ref) <= bound


def test_detmath_atan2_and_pow():
    rng = np.random.default_rng(2)
    y, x = rng.uniform(-3, 3, 20000), rng.uniform(-3, 3, 20000)
    assert _ulp_err(O.detmath("atan2", y, x), np.arctan2(y, x)) <= 6
    for a, b in ((0.0, 1.0), (-0.0, 1.0), (0.0, -1.0), (-0.0, -1.0), (1.0, 0.0), (-1.0, 0.0)):
        assert O.detmath("atan2", np.array([a]), np.array([b]))[0] == math.atan2(a, b)
    xb, yb = rng.uniform(0.01, 10, 20000), rng.uniform(-3, 3, 20000)
    np.testing.assert_allclose(O.detmath("pow", xb, yb), xb ** yb, rtol=2e-15)


def test_validation_messages():
    job = survivor_job([])
    assert O.validate(job)[0] == 0
    bad = job.copy()
    bad.sample_t_intv[0], bad.sample_t_intv[1] = 5.0, 1.0
    st, msg = O.validate(bad)
    assert st == 1 and "sample_t_intv" in msg
    bad = job.copy()
    bad.rate_prefix = 3
    st, msg = O.validate(bad)
    assert st == 1 and "conflict" in msg
    bad = job.copy()
    bad.ss_kd_num = 1
    st, msg = O.validate(bad)
    assert st == 1 and "endpoints differ" in msg
    bad.ss_kd_num, bad.init_cond_method = 0, abi.SAMPLER_SPA
    st, msg = O.validate(bad)
    assert st == 1 and msg.startswith("[SPASampler] Invalid kd sample number")
    with pytest.raises(ValueError):
        et.rate_prefix_bits(["Pre", "PreCC"])
    with pytest.raises(AssertionError):
        et.make_job(**{**_kw(), "traj_t_final": 50.0})


def _kw():
    l = et.Cos4Laser(peak_int=1e14, wave_len=800.0, cyc_num=2, ellip=0.0)
    return dict(init_cond_method="ADK", laser=l, target=et.get_atom("H"), dimension=2,
                sample_t_intv=(-100, 100), sample_t_num=10, traj_t_final=300,
                final_p_max=(1.5, 1.5), final_p_num=(50, 50), ss_kd_max=1.0, ss_kd_num=11)


def test_grid_time_samples_match_julia_range():
    """range(-100, 100; length=400) elements are the rationals (200 i - 40100)/399, rounded."""
    job = survivor_job([])
    t = O.t_samples(job)
    from fractions import Fraction
    for i in (1, 2, 199, 200, 398, 400):
        assert t[i - 1] == float(Fraction(-100 * (400 - i) + 100 * (i - 1), 399))


def test_mc_time_samples_sorted_and_seeded():
    job = survivor_job(["mc2d"])
    t1 = O.t_samples(job)
    assert np.all(np.diff(t1) >= 0) and t1[0] >= -100 and t1[-1] < 100
    job.seed = 7
    t2 = O.t_samples(job)
    assert not np.array_equal(t1, t2)
