"""The exp(-b r) skip of the SAE potential changes no bit of any result.

The kernels and the oracle drop exp(-b r) when b r > 60 for targets that pass
etraj_sae_skip_exact (csrc/sae_skip.h).  These CPU tests check the decision
on the preset table of AtomDatabase.jl, reject a target whose negative term
could cancel the nuclear charge, and compare potential, force, right-hand
side and whole oracle runs with the skip switched on and off.
"""
import numpy as np
import pytest

import _oracle as O
import etraj_gb300 as et


@pytest.fixture
def skip_off():
    O.set_sae_skip(False)
    try:
        yield
    finally:
        O.set_sae_skip(True)


def test_presets_pass_the_exactness_check():
    for name in et.get_available_atoms():
        t = et.get_atom(name)
        if isinstance(t, et.SAEAtom):
            assert O.sae_skip_exact(t.to_c()), name


def test_cancelling_or_slow_terms_are_rejected():
    # a negative a1 e^{-r/2} that is still far below -Z where e^{-3 r} is dropped (r > 20)
    bad = et.SAEAtom(Ip=0.5, Z=1, a1=-1e6, b1=0.5, a3=1.0, b3=3.0)
    assert not O.sae_skip_exact(bad.to_c())
    # a term that never decays (b = 0) with a negative weight
    assert not O.sae_skip_exact(et.SAEAtom(Ip=0.5, Z=1, a1=-0.5, b1=0.0, a2=1.0, b2=2.0).to_c())
    # a decay constant so small that exp(-b r) is dropped at r where 1/r^3 is subnormal
    assert not O.sae_skip_exact(et.SAEAtom(Ip=0.5, Z=1, a1=1.0, b1=1e-9).to_c())
    # a huge weight
    assert not O.sae_skip_exact(et.SAEAtom(Ip=0.5, Z=1, a1=1e10, b1=1.0).to_c())


def _points(rng, n):
    r = np.exp(rng.uniform(np.log(1e-3), np.log(1e7), n))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return d * r[:, None]


@pytest.mark.parametrize("atom", ["He", "Ne", "Ar", "Xe", "Ta", "Kr"])
def test_potential_and_force_identical(atom, skip_off):
    tc = et.get_atom(atom).to_c()
    xyz = _points(np.random.default_rng(5), 20000)
    V0, F0 = O.target_eval(tc, xyz)
    O.set_sae_skip(True)
    V1, F1 = O.target_eval(tc, xyz)
    assert V0.tobytes() == V1.tobytes()
    assert F0.tobytes() == F1.tobytes()


def _job(atom, dim, phase, method="ADK", t_num=24, kd_num=16):
    laser = et.Cos4Laser(peak_int=1.2e14, wave_len=800.0, cyc_num=2, ellip=1.0 if dim == 2 else 0.5)
    kw = dict(init_cond_method=method, laser=laser, target=et.get_atom(atom), dimension=dim,
              sample_t_intv=(-100.0, 100.0), sample_t_num=t_num, traj_t_final=160.0,
              final_p_max=(1.5,) * dim, final_p_num=(24,) * dim, ss_kd_max=1.0, ss_kd_num=kd_num,
              traj_phase_method=phase, traj_rtol=1e-6)
    if dim == 3:
        kw.update(ss_kz_max=1.0, ss_kz_num=5)
    return et.make_job(**kw)


@pytest.mark.parametrize("dim,phase", [(2, "SCTS"), (2, "QTMC"), (3, "SCTS"), (3, "CTMC")])
def test_rhs_identical(dim, phase, skip_off):
    job = _job("Ar", dim, phase)
    rng = np.random.default_rng(11)
    n = {(2, "SCTS"): 5, (2, "QTMC"): 5, (3, "SCTS"): 7, (3, "CTMC"): 6}[(dim, phase)]
    us = []
    for _ in range(3000):
        u = rng.normal(size=n)
        u[:dim] *= np.exp(rng.uniform(-3, 9))
        us.append(u)
    d0 = [O.rhs(job, 12.5, u) for u in us]
    O.set_sae_skip(True)
    d1 = [O.rhs(job, 12.5, u) for u in us]
    assert all(a.tobytes() == b.tobytes() for a, b in zip(d0, d1))


@pytest.mark.parametrize("atom,dim,phase,method", [("Ar", 2, "SCTS", "SPANE"), ("Xe", 3, "QTMC", "ADK")])
def test_whole_run_identical(atom, dim, phase, method, skip_off):
    job = _job(atom, dim, phase, method)
    s0, a0, c0 = O.run(job)
    O.set_sae_skip(True)
    s1, a1, c1 = O.run(job)
    assert c0["num_effective"] > 0
    assert s0.tobytes() == s1.tobytes() and a0.tobytes() == a1.tobytes()
    assert c0 == c1
