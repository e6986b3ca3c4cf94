"""GPU parity of the FP64 path against the CPU oracle, through the C ABI.

Bar of this path: per-trajectory final momenta within 1e-9 relative and the
momentum distribution within 1e-10 relative L2 of the CPU path on the same
sampled inputs.  The FP64 kernels use the same
elementary-function implementation and operation order as the oracle, so
these tests also assert bit-exact equality where the arithmetic is
identical (sampled rows, final states, spectra).
"""
import json
import os

import numpy as np
import pytest

import _oracle as O
import etraj_gb300 as et
from etraj_gb300 import abi

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def eng():
    e = et.Engine(device=0)
    yield e
    e.close()


def period(wave_len=800.0):
    return 2 * np.pi / (45.563352525 / wave_len)


def job_of(method="ADK", dim=2, phase="CTMC", target="H", laser="cos4", mc=False, nt=24,
           nkd=15, nkz=7, pnum=None, pmax=1.5, prefix="Full", cutoff=1e-16, seed=3, ellip=0.0,
           intensity=1e14, t_final_periods=3.0, rtol=1e-6, proposal="uniform"):
    T = period()
    if laser == "cos4":
        L = et.Cos4Laser(peak_int=intensity, wave_len=800.0, cyc_num=2, ellip=ellip)
    elif laser == "cos2":
        L = et.Cos2Laser(peak_int=intensity, wave_len=800.0, cyc_num=2, ellip=ellip, cep=0.3, azi=0.4)
    elif laser == "gauss":
        L = et.GaussianLaser(peak_int=intensity, wave_len=800.0, spread_cyc_num=0.6, ellip=ellip)
    else:
        L = et.BichromaticLaser(et.Cos4Laser(peak_int=intensity, wave_len=800.0, cyc_num=2, ellip=1.0),
                                et.Cos4Laser(peak_int=intensity, wave_len=400.0, cyc_num=4, ellip=-1.0),
                                delay=3.0)
    tgt = et.get_atom(target)
    if pnum is None:
        pnum = (64,) * dim
    kw = dict(init_cond_method=method, laser=L, target=tgt, dimension=dim, sample_t_intv=(-T, T),
              sample_t_num=nt, traj_t_final=t_final_periods * T, final_p_max=(pmax,) * dim,
              final_p_num=pnum, traj_phase_method=phase, rate_prefix=prefix,
              sample_cutoff_limit=cutoff, seed=seed, traj_rtol=rtol, mc_kt_proposal=proposal)
    if mc:
        kw.update(sample_monte_carlo=True, mc_kt_num=nkd * nkz, mc_kd_max=1.0,
                  mc_kz_max=1.0 if dim == 3 else 0.0)
    else:
        kw.update(ss_kd_max=1.0, ss_kd_num=nkd, ss_kz_max=1.0, ss_kz_num=nkz if dim == 3 else 0)
    return et.make_job(**kw)


def same_bits(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint64) if a.dtype == np.float64 else a,
                                                 b.view(np.uint64) if b.dtype == np.float64 else b)


# ---- sampler ----------------------------------------------------------------------

with open(os.path.join(GOLDEN, "sampler_survivors.json")) as f:
    SURV = json.load(f)

from test_oracle_pins import survivor_job  # noqa: E402


@pytest.mark.parametrize("case", [c for c in SURV["cases"]],
                         ids=["-".join(c["modifiers"]) or "adk" for c in SURV["cases"]])
def test_gpu_sampler_survivor_counts(eng, case):
    """gen_electron_batch(sp, 200) on the GPU: the reference's pinned shapes, and the
    same columns as the oracle bit for bit."""
    job = survivor_job(case["modifiers"])
    if job is None:
        pytest.skip("molecular targets are outside the built path")
    if O.validate(job)[0] == 2:
        pytest.skip("sampler not built yet")
    got = eng.sample_batch(job, SURV["batch_id"])
    ref = O.sample_batch(job, SURV["batch_id"])
    if case["expected"] is not None:
        assert got is not None and list(got.shape) == case["expected"]
    assert same_bits(got, ref)


SAMPLE_CASES = [
    dict(method="ADK", dim=2), dict(method="ADK", dim=3, phase="QTMC"),
    dict(method="SPANE", dim=2, phase="SCTS", laser="cos2", ellip=0.7),
    dict(method="SPANE", dim=3, target="Ar", phase="QTMC"),
    # (Ar's m=0 orbital has a node in the polarization plane: 2D linear polarization
    # gives rates ~1e-47, so the 2D Ar cases use circular polarization)
    dict(method="ADK", dim=2, mc=True, target="Ar", laser="gauss", phase="SCTS", ellip=1.0),
    dict(method="SPANE", dim=3, mc=True, laser="bichrom", prefix="Pre", phase="QTMC"),
    dict(method="ADK", dim=3, target="Xe", prefix=["Pre", "Jac"]),
    dict(method="SPANE", dim=2, mc=True, target="He", prefix="Exp"),
    dict(method="SPA", dim=2, target="Ar", laser="cos2", phase="SCTS", ellip=1.0, nt=16, nkd=31),
    dict(method="SPA", dim=3, mc=True, laser="bichrom", phase="QTMC", nt=12, nkd=8, nkz=8),
    dict(method="SPA", dim=3, target="Xe", laser="gauss", prefix=["Pre", "Jac"], ellip=0.5, nt=12, nkd=9, nkz=5),
    dict(method="SPA", dim=2, prefix="Exp", ellip=1.0, nt=16, nkd=31),
    # the Gaussian transverse-momentum proposal (importance weights in dkdt)
    dict(method="ADK", dim=2, mc=True, proposal="adk_gauss", ellip=0.3),
    dict(method="ADK", dim=3, mc=True, target="Ar", laser="gauss", phase="SCTS", proposal="adk_gauss"),
    dict(method="SPANE", dim=3, mc=True, laser="bichrom", prefix="Pre", proposal="adk_gauss"),
    dict(method="SPANE", dim=2, mc=True, target="He", prefix="Exp", proposal="adk_gauss"),
]


@pytest.mark.parametrize("kw", SAMPLE_CASES, ids=lambda k: "-".join(str(v) for v in k.values()))
def test_gpu_sample_all_bit_exact(eng, kw):
    job = job_of(**kw)
    got = eng.sample_all(job)
    ref = O.sample_all(job)
    assert got.shape == ref.shape and got.shape[0] > 0
    assert same_bits(got, ref)


# ---- integrator ---------------------------------------------------------------------

INTEGRATE_CASES = [(d, p, t) for d in (2, 3) for p in ("CTMC", "QTMC", "SCTS") for t in ("H", "Ar")]


@pytest.mark.parametrize("dim,phase,target", INTEGRATE_CASES)
def test_gpu_integrate_bit_exact(eng, dim, phase, target):
    job = job_of(method="ADK", dim=dim, phase=phase, target=target, nt=16, nkd=9, nkz=5,
                 laser="cos2" if target == "Ar" else "cos4", ellip=0.5 if target == "Ar" else 0.0)
    init = O.sample_all(job)
    fin, st, steps = eng.integrate(job, init)
    rfin, rst, rsteps = O.integrate(job, init)
    assert np.array_equal(st, rst)
    assert np.array_equal(steps, rsteps)
    ok = rst == 0
    # the path's tolerance, then the stronger bit-exact claim
    np.testing.assert_allclose(fin[ok], rfin[ok], rtol=1e-9, atol=1e-12)
    assert same_bits(fin[ok], rfin[ok])


def test_gpu_integrate_other_lasers(eng):
    for laser in ("gauss", "bichrom"):
        job = job_of(method="SPANE", dim=3, phase="SCTS", laser=laser, nt=12, nkd=7, nkz=5)
        init = O.sample_all(job)
        fin, st, steps = eng.integrate(job, init)
        rfin, rst, rsteps = O.integrate(job, init)
        assert np.array_equal(st, rst) and np.array_equal(steps, rsteps)
        assert same_bits(fin[rst == 0], rfin[rst == 0])


# ---- whole job -------------------------------------------------------------------------

RUN_CASES = [
    dict(method="ADK", dim=2), dict(method="ADK", dim=2, phase="QTMC", ellip=1.0),
    dict(method="SPANE", dim=2, phase="SCTS", target="Ar", laser="cos2", ellip=1.0, mc=True),
    dict(method="ADK", dim=3, phase="SCTS", pnum=(32, 32, 16)),
    dict(method="SPANE", dim=3, phase="CTMC", laser="bichrom", mc=True, pnum=(40, 40, 1)),
    dict(method="ADK", dim=2, pnum=(1, 50)),
    dict(method="ADK", dim=2, pmax=0.3),  # many electrons land outside the grid
    dict(method="SPA", dim=2, phase="QTMC", ellip=1.0, nt=16, nkd=31),
    dict(method="ADK", dim=2, phase="SCTS", mc=True, ellip=0.3, proposal="adk_gauss"),
]


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / nb if nb > 0 else np.linalg.norm(a)


@pytest.mark.parametrize("kw", RUN_CASES, ids=lambda k: "-".join(str(v) for v in k.values()))
def test_gpu_run_matches_oracle(eng, kw):
    job = job_of(**kw)
    res, spec, amp = eng.run(job, want_spectrum=True, want_amplitude=True)
    rspec, ramp, rsc = O.run(job)
    assert res.num_effective_traj == int(rsc["num_effective"])
    assert res.num_failed_traj == int(rsc["num_failed"])
    assert res.num_ionized_traj == int(rsc["num_ionized"])
    assert res.num_steps == int(rsc["num_steps"])
    assert rel_l2(spec, rspec) <= 1e-10
    assert same_bits(spec, rspec)
    assert res.ion_prob == rsc["ion_prob"]
    assert res.ion_prob_uncollected == rsc["ion_prob_uncollected"]
    if job.traj_phase_method != abi.PHASE_CTMC:
        assert same_bits(amp, ramp)
    assert res.num_kernel_launches > 0
    if "pmax" in kw:
        assert res.ion_prob_uncollected > 0


def test_gpu_run_deterministic_and_stream_independent(eng):
    job = job_of(method="SPANE", dim=2, phase="QTMC", mc=True, nt=40, nkd=30, nkz=3)
    r1, s1, a1 = eng.run(job, want_amplitude=True)
    r2, s2, a2 = eng.run(job, want_amplitude=True)
    import torch
    st = torch.cuda.Stream()
    eng.set_stream(st.cuda_stream)
    r3, s3, a3 = eng.run(job, want_amplitude=True)
    eng.set_stream(None)
    assert same_bits(s1, s2) and same_bits(s1, s3) and same_bits(a1, a3)
    assert r1.ion_prob == r2.ion_prob == r3.ion_prob


def test_gpu_empty_job(eng):
    """Every candidate below the cutoff: the reference returns `nothing` for every
    batch (ADKSampler.jl:392-394) and the spectrum stays zero."""
    job = job_of(method="ADK", dim=2, cutoff=1e300)
    res, spec, _ = eng.run(job)
    assert res.num_effective_traj == 0 and res.ion_prob == 0.0
    assert not spec.any()
    assert eng.sample_batch(job, 1) is None


def test_gpu_async_submit_poll(eng):
    jobs = [job_of(method="ADK", dim=2, nt=10 + 3 * i) for i in range(3)]
    outs = []
    for j in jobs:
        res = abi.Result()
        spec = np.zeros(j.grid_size)
        res.momentum_spec = abi.dptr(spec)
        outs.append((eng.submit(j, res), res, spec, j))
    for tk, res, spec, j in outs:
        eng.wait(tk, res)
        rspec, _, rsc = O.run(j)
        assert same_bits(spec, rspec)
        assert res.num_effective_traj == int(rsc["num_effective"])


def test_gpu_perform_traj_simulation_api(eng):
    T = period()
    out = et.perform_traj_simulation(
        init_cond_method="ADK", laser=et.Cos4Laser(peak_int=1e14, wave_len=800.0, cyc_num=2, ellip=1.0),
        target=et.get_atom("H"), dimension=2, sample_t_intv=(-T, T), sample_t_num=30,
        traj_t_final=3 * T, final_p_max=(1.5, 1.5), final_p_num=(80, 60), ss_kd_max=1.0,
        ss_kd_num=20, traj_phase_method="SCTS", engine=eng)
    assert out["momentum_spec"].shape == (80, 60)
    assert out["px"].shape == (80,) and out["py"].shape == (60,)
    assert out["num_effective_traj"] > 0 and out["ion_prob"] > 0
    assert np.allclose(np.abs(out["amplitude"]) ** 2, out["momentum_spec"])


@pytest.mark.parametrize("fmt", [":jld2", ":h5"])
def test_gpu_perform_traj_simulation_writes_the_reference_file(eng, tmp_path, fmt):
    """write_output!'s datasets (TrajectorySimulation.jl:502-546), read back
    with the package's JLD2/HDF5 reader; a 3D grid keeps Julia's axis order."""
    T = period()
    path = str(tmp_path / "run")
    kw = dict(init_cond_method="ADK", laser=et.Cos4Laser(peak_int=1e14, wave_len=800.0, cyc_num=2, ellip=0.5),
              target=et.get_atom("H"), dimension=3, sample_t_intv=(-T, T), sample_t_num=20, traj_t_final=3 * T,
              final_p_max=(1.5, 1.2, 0.8), final_p_num=(40, 30, 6), ss_kd_max=1.0, ss_kd_num=15, ss_kz_max=1.0,
              ss_kz_num=5, traj_phase_method="QTMC", engine=eng, output_fmt=fmt, output_path=path)
    out = et.perform_traj_simulation(**kw)
    ext = "." + fmt[1:]
    assert out["output_path"] == path + ext
    d = et.jld2.load(out["output_path"])
    names = ["info", "params_text"] + (["params"] if fmt == ":jld2" else []) + [
        "px", "py", "pz", "momentum_spec", "ion_prob", "ion_prob_uncollected", "num_effective_traj"]
    assert list(d) == names
    if fmt == ":jld2":
        assert d["params"]["init_cond_method"] == "ADK" and d["params"]["laser"]["type"] == "Cos4Laser"
        assert tuple(d["params"]["final_p_num"]) == (40, 30, 6)
    assert np.array_equal(d["momentum_spec"], out["momentum_spec"]) and d["momentum_spec"].shape == (40, 30, 6)
    assert np.array_equal(d["px"], out["px"]) and np.array_equal(d["pz"], out["pz"])
    assert d["ion_prob"] == out["ion_prob"] and d["num_effective_traj"] == out["num_effective_traj"]
    assert d["params_text"] == out["params_text"]
    # an existing file is kept; the next run saves under another name
    with pytest.warns(UserWarning):
        out2 = et.perform_traj_simulation(**{**kw, "output_path": out["output_path"]})
    assert out2["output_path"] != out["output_path"]
    import os
    os.remove(out2["output_path"])


def test_gpu_budget_refusal():
    e = et.Engine(device=0, hbm_budget_bytes=1 << 20)
    job = job_of(method="ADK", dim=2, nt=400, nkd=200)
    with pytest.raises(et.EtrajError) as ei:
        e.run(job)
    assert ei.value.status == abi.ERR_OUT_OF_MEMORY
    e.close()


def test_gpu_h_adk_3d_full_size(eng):
    """The plain-path workload at full size (hydrogen, Cos4 1e14 W/cm^2 800 nm 2 cycles,
    ADK 2000 t x 21 x 21 in 3D, CTMC, 500 x 500 px-py grid): same spectrum as the oracle."""
    T = period()
    job = et.make_job(init_cond_method="ADK", laser=et.Cos4Laser(peak_int=1e14, wave_len=800.0,
                                                                   cyc_num=2, ellip=0.0),
                      target=et.HydrogenLikeAtom(Ip=0.5, Z=1), dimension=3, sample_t_intv=(-T, T),
                      sample_t_num=2000, traj_t_final=3 * T, final_p_max=(1.5, 1.5, 1.0),
                      final_p_num=(500, 500, 1), ss_kd_max=1.0, ss_kd_num=21, ss_kz_max=1.0,
                      ss_kz_num=21, traj_phase_method="CTMC")
    res, spec, _ = eng.run(job)
    rspec, _, rsc = O.run(job)
    # 2000 x 441 candidates; about 1.1e5 survive the default 1e-16 rate cutoff
    assert res.num_effective_traj == int(rsc["num_effective"]) > 100000
    assert rel_l2(spec, rspec) <= 1e-10
    assert same_bits(spec, rspec)
    assert res.ion_prob == rsc["ion_prob"]


# ---- per-trajectory final states (etraj_dump_final_states) -------------------------------

@pytest.mark.parametrize("phase", ["QTMC", "SCTS"])
def test_gpu_dump_final_states_match_oracle(eng, phase):
    """Per survivor, in the reference's column order: p_inf, status and step
    counts bit for bit; the QTMC phase is the ODE's last component, the SCTS
    phase reproduces the oracle's deposited amplitude sqrt(w) e^{i phase}."""
    job = job_of(method="ADK", dim=3, phase=phase, target="Ar", nt=16, nkd=9, nkz=5, laser="cos2", ellip=0.5)
    eng.keep_final_states(True)
    try:
        res, _, _ = eng.run(job)
        n = res.num_effective_traj
        p, ph, st = eng.dump_final_states(n)
        steps = eng.dump_step_counts(n)
    finally:
        eng.keep_final_states(False)
    init = O.sample_all(job)
    fin, rst, rsteps = O.integrate(job, init)
    _, _, sc, rp, _ = O.collect(job, init, fin, rst, rsteps)
    assert n == init.shape[0] > 0
    assert np.array_equal(st & 0xFF, rst) and np.array_equal(steps, rsteps)
    assert int(np.count_nonzero(st & 0x100)) == res.num_ionized_traj == int(sc["num_ionized"])
    ion = (st & 0x100) != 0
    assert same_bits(p[ion], rp[ion])
    ok = rst == 0
    if phase == "QTMC":
        assert same_bits(ph[ok], fin[ok, -1])
    else:
        key, cre, cim = O.contributions(job, init, fin, rst)
        dep = key < job.grid_size
        w = np.sqrt(init[dep, 7])
        np.testing.assert_allclose(w * np.cos(ph[dep]), cre[dep], rtol=1e-12, atol=1e-14 * w.max())
        np.testing.assert_allclose(w * np.sin(ph[dep]), cim[dep], rtol=1e-12, atol=1e-14 * w.max())


@pytest.mark.parametrize("dim", [2, 3])
def test_gpu_dump_min_radius_matches_oracle(eng, dim):
    """Each survivor's least |r| over its accepted steps, bit for bit; the bulk
    path does not track it."""
    job = job_of(method="ADK", dim=dim, phase="QTMC", target="Ar", nt=16, nkd=9, nkz=5, laser="cos2", ellip=0.5)
    eng.keep_final_states(True)
    try:
        res, _, _ = eng.run(job)
        n = res.num_effective_traj
        rmin = eng.dump_min_radius(n)
        b = job.copy()
        b.precision = abi.PRECISION_FP32_BULK
        eng.run(b)
        with pytest.raises(et.EtrajError) as e:
            eng.dump_min_radius(n)
        assert e.value.status == abi.ERR_UNSUPPORTED
    finally:
        eng.keep_final_states(False)
    init = O.sample_all(job)
    _, _, _, rref = O.integrate_rmin(job, init)
    assert n == init.shape[0] > 0
    assert same_bits(rmin, rref)
    assert rmin.min() < 5.0 < rmin.max()


def test_gpu_dump_final_states_bookkeeping(eng):
    job = job_of(method="ADK", dim=2, nt=8, nkd=11)
    eng.run(job)  # not kept
    with pytest.raises(et.EtrajError) as e:
        eng.dump_final_states(1)
    assert e.value.status == abi.ERR_NOT_FOUND
    eng.keep_final_states(True)
    try:
        r1 = abi.Result()
        t1 = eng.submit(job, r1)
        eng.wait(t1, r1)
        p1, _, s1 = eng.dump_final_states(r1.num_effective_traj, ticket=t1)
        p0, _, s0 = eng.dump_final_states(r1.num_effective_traj)  # ticket 0: the last job
        assert same_bits(p1, p0) and np.array_equal(s1, s0)
        eng.run(job_of(method="ADK", dim=2, nt=8, nkd=11, seed=4))
        with pytest.raises(et.EtrajError):  # overwritten by the next job
            eng.dump_final_states(r1.num_effective_traj, ticket=t1)
    finally:
        eng.keep_final_states(False)


def test_gpu_dump_final_states_bulk_path(eng):
    """The bulk path's per-survivor asymptotic momenta track FP64's."""
    job = job_of(method="SPANE", dim=2, phase="SCTS", target="Ar", laser="cos2", ellip=1.0, mc=True, nt=200,
                 nkd=100, nkz=1)
    eng.keep_final_states(True)
    try:
        r64, _, _ = eng.run(job)
        p64, _, s64 = eng.dump_final_states(r64.num_effective_traj)
        b = job.copy()
        b.precision = abi.PRECISION_FP32_BULK
        r32, _, _ = eng.run(b)
        p32, _, s32 = eng.dump_final_states(r32.num_effective_traj)
    finally:
        eng.keep_final_states(False)
    assert r32.num_effective_traj == r64.num_effective_traj
    both = ((s64 & 0x100) != 0) & ((s32 & 0x100) != 0)
    assert both.sum() > 0.95 * ((s64 & 0x100) != 0).sum()
    d = np.linalg.norm(p32[both] - p64[both], axis=1) / np.linalg.norm(p64[both], axis=1)
    assert np.median(d) < 1e-3
