"""Molecular targets on the CPU: the JLD2 reader, GenericMolecule's accessors,
the shared WFAT structure factor and the target checks.

Pins: test/Targets_test.jl:100-155 (tests/golden/molecule_pins.json) and the
molecular sampler counts of test/ElectronSamplers_test.jl (test_oracle_pins).
"""
import ctypes as C
import json
import math
import os

import numpy as np
import pytest

import _oracle as O
import etraj_gb300 as et
from _mol import GOLDEN, hydrogen
from etraj_gb300 import abi

with open(os.path.join(GOLDEN, "molecule_pins.json"), encoding="utf-8") as f:
    PINS = json.load(f)

from conftest import REFERENCE_DB as REF_DB  # noqa: E402

need_db = pytest.mark.skipif(not (REF_DB and os.path.isdir(REF_DB)),
                             reason="set ETRAJ_REFERENCE_DIR to a reference checkout (its molecule database)")


def close(a, b):
    return math.isclose(a, b, rel_tol=1e-12, abs_tol=0.0)


def test_hydrogen_accessors_match_pins():
    m = hydrogen()
    assert m.MolAtoms() == ["H", "H"]
    assert np.array_equal(m.MolAtomCoords(), [[0.0, 0.0, -0.37072], [0.0, 0.0, 0.37072]])
    assert m.MolCharge() == 0 and m.MolEnergyDataAvailable()
    assert close(m.MolEnergyLevels()[0], PINS["homo_energy"]["value"])
    assert close(m.MolHOMOEnergy(), PINS["homo_energy"]["value"])
    assert m.MolWFATAvailableIndices() == {0} and m.MolAsympCoeffAvailableIndices() == {0}
    mu, I = m.MolWFATData(0)
    assert np.all(np.abs(mu) <= 1e-10)
    assert close(I[0, 0, 0, 0].real, PINS["intdata_1111"]["value"])
    assert close(m.MolAsympCoeff(0)[0, 0].real, PINS["asymp_coeff_11"]["value"])
    assert m.MolExportAtomInfo() == PINS["atom_info"]["value"]
    assert m.IonPotential() == -m.MolHOMOEnergy() and m.IonPotential(0) == -m.MolHOMOEnergy()
    assert m.AsympNuclCharge() == PINS["asymp_charge"]["value"]
    assert m.TargetName() == PINS["name"]["value"]
    assert m.TargetPotential()(1.0, 1.0, 1.0) == PINS["potential_111"]["value"]
    assert m.TargetForce()(1.0, 1.0, 1.0) == tuple(PINS["force_111"]["value"])
    m.SetMolRotation(math.pi, math.pi / 2, math.pi / 3)
    assert m.MolRotation() == (math.pi, math.pi / 2, math.pi / 3)
    m.SetMolRotation((math.pi / 2, math.pi / 3, math.pi / 4))
    assert m.MolRotation() == (math.pi / 2, math.pi / 3, math.pi / 4)


@pytest.mark.parametrize("key,theta", [("G2_theta0", 0.0), ("G2_theta_pi2", math.pi / 2)])
def test_structure_factor_matches_pins(key, theta):
    m = hydrogen()
    want = PINS[key]["value"]
    # the host accessor and the shared device/oracle implementation (mol.h)
    assert math.isclose(abs(m.MolWFATStructureFactor_G(0, 0, 0, theta, 0.0)) ** 2, want, rel_tol=1e-13)
    t, keep = m.to_c(0, wfat=True)
    G = O.mol_wfat_G(t, 0, 0, theta, 0.0)
    assert math.isclose(abs(G) ** 2, want, rel_tol=1e-13)
    # both agree on every channel and at an oblique orientation
    for nxi in range(3):
        for mm in (-2, 0, 1):
            a = m.MolWFATStructureFactor_G(0, nxi, mm, 0.7, 1.3)
            b = O.mol_wfat_G(t, nxi, mm, 0.7, 1.3)
            assert abs(a - b) <= 1e-13 * max(1.0, abs(a))


def test_molecule_target_is_the_soft_core_coulomb_tail():
    """GenericMolecule.jl:444-445: V = -(charge+1)/sqrt(r^2+1), F = -(charge+1) r/(r^2+1)^1.5,
    through the oracle's target evaluation of the molecular etraj_target."""
    m = hydrogen()
    t, _ = m.to_c(0)
    xyz = np.array([[1.0, 1.0, 1.0], [0.3, -2.0, 0.5], [0.0, 0.0, 0.0]])
    V, F = O.target_eval(t, xyz)
    assert V[0] == PINS["potential_111"]["value"]
    assert tuple(F[0]) == tuple(PINS["force_111"]["value"])
    for i, p in enumerate(xyz):
        assert math.isclose(V[i], m.TargetPotential()(*p), rel_tol=1e-15)
        assert np.allclose(F[i], m.TargetForce()(*p), rtol=1e-15, atol=0)


def test_molecule_trajectories_equal_the_hydrogen_like_ones():
    """A molecule's ODE is the hydrogen-like one with Z = charge+1, soft core 1.0
    and Ip = IonPotential(mol): the oracle integrates both to the same bits."""
    m = hydrogen()
    L = et.Cos2Laser(peak_int=2e14, wave_len=800.0, cyc_num=2, ellip=1.0)
    kw = dict(init_cond_method="ADK", laser=L, dimension=2, sample_t_intv=(-50.0, 50.0), sample_t_num=20,
              traj_t_final=300.0, final_p_max=(2.0, 2.0), final_p_num=(50, 50), ss_kd_max=1.0, ss_kd_num=21,
              traj_phase_method="QTMC")
    jm = et.make_job(target=m, **kw)
    h = et.HydrogenLikeAtom(Ip=m.IonPotential(), Z=1, soft_core=1.0)
    jh = et.make_job(target=h, **kw)
    init = O.sample_all(jm)
    assert init.shape[0] > 10
    fm, sm, nm = O.integrate(jm, init)
    fh, sh, nh = O.integrate(jh, init)
    assert np.array_equal(fm, fh) and np.array_equal(sm, sh) and np.array_equal(nm, nh)


def _check(job):
    st, msg = O.validate(job)
    buf = C.create_string_buffer(256)
    st_lib = abi.load_library().etraj_validate(C.byref(job), buf, 256)
    assert st_lib == st, (st, st_lib, msg, buf.value)
    return st, msg


def test_molecular_checks():
    m = hydrogen()
    L = et.Cos4Laser(peak_int=1e15, wave_len=800.0, cyc_num=2, ellip=1.0)
    kw = dict(laser=L, dimension=2, sample_t_intv=(-100, 100), sample_t_num=10, traj_t_final=200.0,
              final_p_max=(2.0, 2.0), final_p_num=(10, 10), ss_kd_max=2.0, ss_kd_num=20)
    assert _check(et.make_job(init_cond_method="WFAT", target=m, **kw))[0] == abi.OK
    assert _check(et.make_job(init_cond_method="MOADK", target=m, **kw))[0] == abi.OK
    with pytest.raises(ValueError):
        et.make_job(init_cond_method="WFAT", target=m, traj_phase_method="QTMC", **kw)
    with pytest.raises(TypeError):
        et.make_job(init_cond_method="WFAT", target=et.get_atom("H"), **kw)
    # the same checks in the C validation
    j = et.make_job(init_cond_method="WFAT", target=m, **kw)
    j.traj_phase_method = abi.PHASE_QTMC
    assert _check(j)[0] == abi.ERR_INVALID_ARGUMENT
    j = et.make_job(init_cond_method="ADK", target=et.get_atom("H"), **kw)
    j.init_cond_method = abi.SAMPLER_WFAT
    assert _check(j)[0] == abi.ERR_INVALID_ARGUMENT
    # an orbital without data needs the molecular calculator: unsupported here
    bare = hydrogen()
    bare.asymp_coeff, bare.wfat_intdata = {}, {}
    assert _check(et.make_job(init_cond_method="ADK", target=bare, **kw))[0] == abi.ERR_UNSUPPORTED
    assert _check(et.make_job(init_cond_method="WFAT", target=bare, **kw))[0] == abi.ERR_UNSUPPORTED
    with pytest.raises(IndexError):
        m.IonPotential(-1)  # H2 has no HOMO-1
    j = et.make_job(init_cond_method="WFAT", target=m, **kw)
    j.target.wfat_lmax = 7
    assert _check(j)[0] == abi.ERR_UNSUPPORTED
    j = et.make_job(init_cond_method="ADK", target=m, **kw)
    j.target.Ip = -0.1
    assert _check(j)[0] == abi.ERR_INVALID_ARGUMENT


def test_job_keeps_the_molecular_tables_alive():
    j = et.make_job(init_cond_method="WFAT", target=hydrogen(), laser=et.Cos4Laser(peak_int=1e15, wave_len=800.0,
                    cyc_num=2, ellip=1.0), dimension=2, sample_t_intv=(-100, 100), sample_t_num=10,
                    traj_t_final=200.0, final_p_max=(2.0, 2.0), final_p_num=(10, 10), ss_kd_max=2.0, ss_kd_num=20)
    c = j.copy()
    assert c._keep is j._keep
    assert c.target.wfat_intdata[0] == j._keep[0][0]


@need_db
def test_jld2_reader_matches_the_fixture():
    m = et.LoadMolecule(os.path.join(REF_DB, "Molecule_Hydrogen.jld2"))
    h = hydrogen()
    assert m.atoms == h.atoms and m.name == h.name and m.charge == h.charge
    assert np.array_equal(m.energy_levels, h.energy_levels) and np.array_equal(m.orbit_occ, h.orbit_occ)
    assert np.array_equal(m.wfat_intdata[0], h.wfat_intdata[0])
    assert np.array_equal(m.asymp_coeff[0], h.asymp_coeff[0])


@need_db
def test_every_database_molecule_loads():
    for name in et.get_available_mols():
        m = et.get_mol(name, database_dir=REF_DB)
        assert m.MolEnergyDataAvailable() and m.IonPotential() > 0
        for idx in m.MolWFATAvailableIndices():
            nxi, mmax = m.MolWFATMaxChannels(idx)
            assert nxi <= abi.MOL_MAX_L and mmax <= abi.MOL_MAX_L and m.IonPotential(idx) > 0
        for idx in m.MolAsympCoeffAvailableIndices():
            assert m.MolAsympCoeff_lMax(idx) <= abi.MOL_MAX_L
    o = et.get_mol("Oxygen", rot_α=math.pi / 4, rot_β=math.pi, rot_γ=2 * math.pi, database_dir=REF_DB)
    assert o.TargetName() == PINS["oxygen_name"]["value"] and o.MolAtoms() == ["O", "O"]
    assert o.MolRotation() == (math.pi / 4, math.pi, 2 * math.pi)
    # open shell: orbitals are (spin, index) pairs
    assert all(isinstance(k, tuple) and k[0] in (1, 2) for k in o.MolWFATAvailableIndices())
