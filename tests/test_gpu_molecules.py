"""Molecular targets on the GPU: MO-ADK / MO-SPANE / MO-SPA prefactors, the
WFAT sampler and GenericMolecule trajectories, against the CPU oracle.

The device sampler evaluates the shared mol.h in the same order as the
oracle, so sampled rows, final states and spectra are compared bit for bit.
The molecule is the reference database's Hydrogen (tests/golden fixture);
the molecular survivor counts of the reference's own tests run on the GPU in
test_gpu_parity.test_gpu_sampler_survivor_counts.
"""
import numpy as np
import pytest

import _oracle as O
import etraj_gb300 as et
from _mol import hydrogen
from etraj_gb300 import abi
from test_gpu_parity import same_bits, rel_l2, period

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    e = et.Engine(device=0)
    yield e
    e.close()


def mol_job(method="MOADK", dim=2, phase="CTMC", rot=(0.0, 0.0, 0.0), laser="cos4", mc=False, nt=24, nkd=31,
            nkz=7, pnum=None, prefix="Full", ellip=1.0, intensity=3e14, precision="fp64", seed=5):
    T = period()
    if laser == "cos4":
        L = et.Cos4Laser(peak_int=intensity, wave_len=800.0, cyc_num=2, ellip=ellip)
    elif laser == "cos2":
        L = et.Cos2Laser(peak_int=intensity, wave_len=800.0, cyc_num=2, ellip=ellip, cep=0.3, azi=0.4)
    else:
        L = et.BichromaticLaser(et.Cos4Laser(peak_int=intensity, wave_len=800.0, cyc_num=2, ellip=1.0),
                                et.Cos4Laser(peak_int=intensity, wave_len=400.0, cyc_num=4, ellip=-1.0),
                                delay=3.0)
    kw = dict(init_cond_method=method, laser=L, target=hydrogen(*rot), dimension=dim, sample_t_intv=(-T, T),
              sample_t_num=nt, traj_t_final=3.0 * T, final_p_max=(1.5,) * dim,
              final_p_num=pnum or (64,) * dim, traj_phase_method=phase, rate_prefix=prefix,
              sample_cutoff_limit=1e-16, seed=seed, precision=precision)
    if mc:
        kw.update(sample_monte_carlo=True, mc_kt_num=nkd * nkz, mc_kd_max=1.0, mc_kz_max=1.0 if dim == 3 else 0.0)
    else:
        kw.update(ss_kd_max=1.0, ss_kd_num=nkd, ss_kz_max=1.0, ss_kz_num=nkz if dim == 3 else 0)
    return et.make_job(**kw)


ROT = (0.4, 1.1, -0.7)
SAMPLE_CASES = [
    dict(method="MOADK", dim=2),
    dict(method="MOADK", dim=3, phase="QTMC", rot=ROT),
    dict(method="MOADK", dim=2, phase="SCTS", prefix="Pre", mc=True, rot=ROT, laser="cos2", ellip=0.5),
    dict(method="MOSPANE", dim=2, phase="SCTS", laser="cos2"),
    dict(method="MOSPANE", dim=3, mc=True, rot=ROT, prefix=["Pre", "Jac"], laser="bichrom"),
    dict(method="MOSPA", dim=2, phase="QTMC", nt=12, nkd=21),
    dict(method="MOSPA", dim=3, rot=ROT, nt=8, nkd=9, nkz=5),
    dict(method="WFAT", dim=2),
    dict(method="WFAT", dim=3, rot=ROT),
    dict(method="WFAT", dim=2, mc=True, rot=ROT, laser="bichrom"),
    dict(method="WFAT", dim=3, mc=True, laser="cos2", ellip=0.3),
]


@pytest.mark.parametrize("kw", SAMPLE_CASES, ids=lambda k: "-".join(str(v) for v in k.values()))
def test_molecular_sampling_bit_exact(eng, kw):
    job = mol_job(**kw)
    got = eng.sample_all(job)
    ref = O.sample_all(job)
    assert got.shape == ref.shape and got.shape[0] > 0
    assert same_bits(got, ref)


RUN_CASES = [
    dict(method="WFAT", dim=2, rot=ROT),
    dict(method="MOADK", dim=3, phase="QTMC", pnum=(32, 32, 16), nkd=15, nkz=5),
    dict(method="MOSPANE", dim=2, phase="SCTS", mc=True, laser="cos2", ellip=1.0),
]


@pytest.mark.parametrize("kw", RUN_CASES, ids=lambda k: "-".join(str(v) for v in k.values()))
def test_molecular_run_matches_oracle(eng, kw):
    job = mol_job(**kw)
    res, spec, amp = eng.run(job, want_spectrum=True, want_amplitude=True)
    rspec, ramp, rsc = O.run(job)
    assert res.num_effective_traj == int(rsc["num_effective"]) > 0
    assert res.num_failed_traj == int(rsc["num_failed"])
    assert res.num_ionized_traj == int(rsc["num_ionized"])
    assert res.num_steps == int(rsc["num_steps"])
    assert rel_l2(spec, rspec) <= 1e-10
    assert same_bits(spec, rspec)
    assert res.ion_prob == rsc["ion_prob"]
    if job.traj_phase_method != abi.PHASE_CTMC:
        assert same_bits(amp, ramp)


@pytest.mark.parametrize("phase", ["CTMC", "SCTS"])
def test_molecular_bulk_path_within_fp64_band(eng, phase):
    """The FP32-bulk integrator on a molecule (hydrogen-like equations, soft core
    1.0): the same sampled electrons (FP64 sampler), the ionization yield, and
    the PMD inside FP64's own tolerance band (FP64 at rtol against rtol/10),
    at full resolution and coarse-grained."""
    job = mol_job(method="MOADK", dim=2, phase=phase, laser="cos2", mc=True, nt=400, nkd=500, nkz=1,
                  pnum=(200, 200))
    r64, s64, _ = eng.run(job)
    tight = job.copy()
    tight.traj_rtol = job.traj_rtol / 10
    r64b, s64b, _ = eng.run(tight)
    b = job.copy()
    b.precision = abi.PRECISION_FP32_BULK
    r32, s32, _ = eng.run(b)
    assert r64.num_effective_traj > 100000
    assert abs(r32.num_effective_traj - r64.num_effective_traj) <= 1e-4 * r64.num_effective_traj + 1
    assert abs(r32.ion_prob - r64.ion_prob) <= 1e-4 * r64.ion_prob
    band = rel_l2(s64b, s64)
    assert rel_l2(s32, s64) <= 1.5 * band, (rel_l2(s32, s64), band)
    c32, c64, c64b = (s.reshape(40, 5, 40, 5).sum(axis=(1, 3)) for s in (s32, s64, s64b))
    assert rel_l2(c32, c64) <= max(1.5 * rel_l2(c64b, c64), 2e-3), (rel_l2(c32, c64), rel_l2(c64b, c64))


@pytest.mark.parametrize("kw", [dict(method="MOADK", dim=3, phase="QTMC", rot=ROT, nkd=21, nkz=9),
                                dict(method="MOSPANE", dim=2, phase="SCTS", mc=True, laser="cos2", nkd=400),
                                dict(method="WFAT", dim=3, rot=ROT, nkd=21, nkz=9)],
                         ids=["moadk-3d", "mospane-2d-mc", "wfat-3d"])
def test_molecular_bulk_sampler_tracks_fp64(eng, kw):
    """The bulk path samples molecules in FP32 from the FP64 per-time-sample
    tables: the same electrons but for any within ~1e-6 of the cutoff, with
    rates and phases to FP32 accuracy."""
    job = mol_job(nt=60, **kw)
    a64 = eng.sample_all(job)
    b = job.copy()
    b.precision = abi.PRECISION_FP32_BULK
    a32 = eng.sample_all(b)
    assert len(a64) > 500 and abs(len(a32) - len(a64)) <= 1e-3 * len(a64) + 1
    n = min(len(a32), len(a64))
    rc = 7 if job.dimension == 3 else 5
    if len(a32) == len(a64):
        np.testing.assert_allclose(a32[:, :rc], a64[:, :rc], rtol=1e-5, atol=1e-6)
        np.testing.assert_allclose(a32[:, rc], a64[:, rc], rtol=2e-4)
        if job.traj_phase_method != abi.PHASE_CTMC:
            assert np.abs(np.angle(np.exp(1j * (a32[:, -1] - a64[:, -1])))).max() < 1e-4
    assert abs(a32[:n, rc].sum() - a64[:n, rc].sum()) <= 1e-4 * a64[:, rc].sum()


def test_batches_reject_molecules(eng):
    job = mol_job(method="MOADK", precision="fp32_bulk")
    with pytest.raises(et.EtrajError) as e:
        eng.run_batch([job, job])
    assert e.value.status == abi.ERR_UNSUPPORTED
