"""The FP32-bulk path against the FP64 path (through the C ABI).

The bulk integrator is a different floating-point evaluation of the same
adaptive Tsit5 method (FP32 stages, double-float state, FP32 field table), so
it cannot match FP64 bit for bit, and an adaptive integrator's answer is only
defined to within its own tolerance band: at rtol 1e-6 the FP64 path itself
differs from a converged solution by ~1e-5..1e-4 per electron, and by more
for the few chaotic, Coulomb-focused ones.  The tests therefore measure both
paths against a converged FP64 reference (rtol 1e-9) and require the bulk
error to sit inside FP64's own band:

 * per electron: median and 90th-percentile momentum error <= 2x / 3x FP64's
   at the same rtol (plus a 2e-6 floor for FP32 resolution);
 * momentum distributions: relative L2 distance to FP64 at rtol <= 1.5x the
   distance between FP64 at rtol and at rtol/10, at full resolution and after
   summing 10x10 bins (or <= 2e-3 there).
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


def with_rtol(job, rtol):
    j = job.copy()
    j.traj_rtol = rtol
    return j


def rebin(spec, pnum, f):
    a = spec.reshape(pnum)
    for ax, n in enumerate(pnum):
        a = np.add.reduceat(a, np.arange(0, n, f), axis=ax)
    return a.ravel()


CASES = [(d, p, t) for d in (2, 3) for p in ("CTMC", "QTMC", "SCTS") for t in ("H", "Ar")]


@pytest.mark.parametrize("dim,phase,target", CASES)
def test_bulk_final_states_within_fp64_band(eng, dim, phase, target):
    job = job_of(method="SPANE", dim=dim, phase=phase, target=target, nt=30, nkd=21, nkz=9,
                 laser="cos2", ellip=1.0 if dim == 2 else 0.5)
    init = O.sample_all(job)
    f64, s64, n64 = eng.integrate(job, init)
    fref, sref, _ = eng.integrate(with_rtol(job, 1e-9), init)
    f32, s32, n32 = eng.integrate(bulk(job), init)
    ok = (s64 == 0) & (s32 == 0) & (sref == 0)
    assert ok.mean() > 0.99
    nq = 2 * dim
    pref = fref[ok][:, dim:nq]
    scale = np.maximum(np.abs(pref).max(axis=1), 1e-3)
    e64 = np.abs(f64[ok][:, dim:nq] - pref).max(axis=1) / scale
    e32 = np.abs(f32[ok][:, dim:nq] - pref).max(axis=1) / scale
    assert np.median(e32) <= 2.0 * np.median(e64) + 2e-6, (np.median(e32), np.median(e64))
    assert np.quantile(e32, 0.9) <= 3.0 * np.quantile(e64, 0.9) + 2e-6, (np.quantile(e32, 0.9),
                                                                        np.quantile(e64, 0.9))
    if phase != "CTMC":
        d64 = np.abs(f64[ok][:, -1] - fref[ok][:, -1])
        d32 = np.abs(f32[ok][:, -1] - fref[ok][:, -1])
        assert np.median(d32) <= 2.0 * np.median(d64) + 1e-5, (np.median(d32), np.median(d64))
    # same controller; the FP32 error estimate less its rounding-noise bound
    # takes a few percent fewer attempts, never many more
    assert 0.75 * np.median(n64[ok]) - 2 <= np.median(n32[ok]) <= 1.1 * np.median(n64[ok]) + 2


@pytest.mark.parametrize("phase", ["CTMC", "SCTS"])
def test_bulk_pmd_within_fp64_band(eng, phase):
    pnum = (200, 200)
    job = job_of(method="SPANE", dim=2, phase=phase, target="Ar", laser="cos2", ellip=1.0, mc=True,
                 nt=2000, nkd=100, nkz=1, pnum=pnum, pmax=2.0)
    r64, s64, _ = eng.run(job)
    r64b, s64b, _ = eng.run(with_rtol(job, job.traj_rtol / 10))
    r32, s32, _ = eng.run(bulk(job))
    # the FP32 sampler keeps the same electrons except ones within ~1e-7 of the cutoff
    assert r64.num_effective_traj > 50000
    assert abs(r32.num_effective_traj - r64.num_effective_traj) <= 1e-4 * r64.num_effective_traj
    assert abs(r32.ion_prob - r64.ion_prob) <= 1e-4 * r64.ion_prob
    band = rel_l2(s64b, s64)
    assert rel_l2(s32, s64) <= 1.5 * band, (rel_l2(s32, s64), band)
    c32, c64, c64b = (rebin(s, pnum, 10) for s in (s32, s64, s64b))
    assert rel_l2(c32, c64) <= max(1.5 * rel_l2(c64b, c64), 2e-3), (rel_l2(c32, c64), rel_l2(c64b, c64))


def test_bulk_sampler_keeps_the_fp64_electrons(eng):
    """Grid sampling (ADK, 3D, full prefix): the FP32 sampler's survivors and
    their summed rate agree with the FP64 sampler's."""
    job = job_of(method="ADK", dim=3, phase="QTMC", target="Ar", nt=200, nkd=41, nkz=21, ellip=0.5)
    r64, _, _ = eng.run(job)
    r32, _, _ = eng.run(bulk(job))
    assert r64.num_effective_traj > 10000
    assert abs(r32.num_effective_traj - r64.num_effective_traj) <= 1e-4 * r64.num_effective_traj + 1
    assert abs(r32.ion_prob - r64.ion_prob) <= 1e-4 * r64.ion_prob


def test_bulk_deterministic(eng):
    job = bulk(job_of(method="ADK", dim=3, phase="QTMC", target="H", nt=40, nkd=15, nkz=9))
    _, s1, a1 = eng.run(job, want_amplitude=True)
    _, s2, a2 = eng.run(job, want_amplitude=True)
    assert np.array_equal(s1, s2) and np.array_equal(a1, a2)


def test_autotuned_shape_changes_no_result():
    """The autotuner picks the bulk integrator's launch shape from timings; one
    electron per lane and the deterministic deposit make results independent of it."""
    job = bulk(job_of(method="SPANE", dim=2, phase="SCTS", target="Ar", laser="cos2", ellip=1.0, mc=True,
                      nt=700, nkd=400, nkz=1, pnum=(200, 200), pmax=2.0))
    tuned = et.Engine(device=0)
    fixed = et.Engine(device=0)
    fixed.set_autotune(False)
    r1, s1, a1 = tuned.run(job, want_amplitude=True)
    assert tuned.bulk_tile(2, abi.PHASE_SCTS, abi.TARGET_SAE)[3]  # 2.8e5 candidates: tuned on this run
    r2, s2, a2 = fixed.run(job, want_amplitude=True)
    assert fixed.bulk_tile(2, abi.PHASE_SCTS, abi.TARGET_SAE) == (256, 2, 4, False)
    assert r1.num_effective_traj == r2.num_effective_traj and r1.ion_prob == r2.ion_prob
    assert np.array_equal(s1, s2) and np.array_equal(a1, a2)
    tuned.close()
    fixed.close()


TILES = [(256, 2, 4), (256, 2, 16), (128, 4, 1), (64, 8, 32), (256, 3, 4), (128, 6, 8), (64, 12, 2), (64, 1, 4)]


@pytest.mark.parametrize("dim,pname", [(2, "SCTS"), (3, "QTMC")])
def test_every_launch_shape_gives_the_same_bits(dim, pname):
    """Launch shapes of both register budgets (16 and 24 warps per SM), tiny and
    wide refill thresholds, and a one-block-per-SM launch: one electron per lane
    and the warp-uniform far-field branch of the SAE force keep every bit."""
    phase = {"SCTS": abi.PHASE_SCTS, "QTMC": abi.PHASE_QTMC}[pname]
    job = bulk(job_of(method="SPANE", dim=dim, phase=pname, target="Ar", laser="cos2",
                      ellip=1.0, mc=True, nt=300, nkd=200, nkz=1 if dim == 2 else 4,
                      pnum=(120, 120) if dim == 2 else (48, 48, 16), pmax=2.0))
    eng = et.Engine(device=0)
    ref = None
    for th, bps, rf in TILES:
        eng.set_bulk_tile(dim, phase, abi.TARGET_SAE, th, bps, rf)
        assert eng.bulk_tile(dim, phase, abi.TARGET_SAE)[:3] == (th, bps, rf)
        out = eng.run(job, want_amplitude=phase != abi.PHASE_CTMC)
        if ref is None:
            ref = out
            assert out[0].num_effective_traj > 0
            continue
        assert out[0].num_effective_traj == ref[0].num_effective_traj and out[0].ion_prob == ref[0].ion_prob
        assert out[0].num_steps == ref[0].num_steps
        assert np.array_equal(out[1], ref[1]) and np.array_equal(out[2], ref[2])
    eng.close()


def test_set_bulk_tile_rejects_bad_shapes():
    eng = et.Engine(device=0)
    for th, bps, rf in [(96, 2, 4), (256, 4, 4), (128, 0, 4), (128, 2, 0), (128, 2, 33)]:
        with pytest.raises(et.EtrajError):
            eng.set_bulk_tile(2, abi.PHASE_SCTS, abi.TARGET_SAE, th, bps, rf)
    eng.close()



def test_rounds_with_parking_keep_every_bit():
    """The integrator's rounds park electrons past a step budget and resume them
    in other lanes, warps and launches; results stay the same bits (a long pulse
    at a long wavelength gives electrons past every budget)."""
    T = 2 * np.pi * 1600.0 / 45.563352525
    L = et.Cos2Laser(peak_int=1e14, wave_len=1600.0, cyc_num=6, ellip=0.3)
    job = et.make_job(init_cond_method="ADK", laser=L, target=et.get_atom("Ar"), dimension=2,
                      sample_t_intv=(-1.5 * T, 1.5 * T), sample_t_num=400, traj_t_final=5 * T,
                      final_p_max=(2.0, 2.0), final_p_num=(120, 120), sample_monte_carlo=True, mc_kt_num=500,
                      mc_kd_max=1.0, traj_phase_method="SCTS", seed=7, precision="fp32_bulk")
    on = et.Engine(device=0)
    off = et.Engine(device=0)
    off.set_straggler_repack(False)
    for e in (on, off):
        e.keep_final_states(True)
    r1, s1, a1 = on.run(job, want_amplitude=True)
    r2, s2, a2 = off.run(job, want_amplitude=True)
    n = r1.num_effective_traj
    assert n == r2.num_effective_traj > 0
    assert r1.num_steps == r2.num_steps and r1.ion_prob == r2.ion_prob and r1.num_failed_traj == r2.num_failed_traj
    assert np.array_equal(s1, s2) and np.array_equal(a1, a2)
    p1, f1, t1 = on.dump_final_states(n)
    p2, f2, t2 = off.dump_final_states(n)
    assert np.array_equal(p1, p2) and np.array_equal(f1, f2) and np.array_equal(t1, t2)
    st = on.dump_step_counts(n)
    assert np.array_equal(st, off.dump_step_counts(n))
    assert (st > 1024).sum() > 0 and (st > 16384).sum() > 0  # electrons went through later rounds
    on.close()
    off.close()


def test_step_chunk_keeps_every_bit():
    """The rounds' step chunk (the tuner's third dimension) moves where electrons
    run, not what they compute: a pinned chunk of 64 steps parks hundreds of
    electrons and gives the default's bits."""
    T = 2 * np.pi * 1600.0 / 45.563352525
    L = et.Cos2Laser(peak_int=1e14, wave_len=1600.0, cyc_num=4, ellip=0.3)
    job = et.make_job(init_cond_method="ADK", laser=L, target=et.get_atom("Ar"), dimension=2,
                      sample_t_intv=(-T, T), sample_t_num=200, traj_t_final=3 * T,
                      final_p_max=(2.0, 2.0), final_p_num=(100, 100), sample_monte_carlo=True, mc_kt_num=400,
                      mc_kd_max=1.0, traj_phase_method="SCTS", seed=3, precision="fp32_bulk")
    a = et.Engine(device=0)
    b = et.Engine(device=0)
    b.set_bulk_step_chunk(2, abi.PHASE_SCTS, abi.TARGET_SAE, 64)
    assert b.bulk_step_chunk(2, abi.PHASE_SCTS, abi.TARGET_SAE)[0] == 64
    r1, s1, a1 = a.run(job, want_amplitude=True)
    r2, s2, a2 = b.run(job, want_amplitude=True)
    assert r1.num_effective_traj == r2.num_effective_traj > 0 and r1.num_steps == r2.num_steps
    assert np.array_equal(s1, s2) and np.array_equal(a1, a2)
    with pytest.raises(et.EtrajError):
        b.set_bulk_step_chunk(2, abi.PHASE_SCTS, abi.TARGET_SAE, 8)
    a.close()
    b.close()


def test_static_assignment_keeps_every_bit():
    """One electron per lane with no work stealing and no rounds (the plain
    kernel's schedule) gives the same bits as the work-stealing schedule, on the
    uneven-step recollision workload (SPA, bichromatic, 3D, QTMC)."""
    from test_gpu_full_size import recollision_job
    job = recollision_job(t_num=300)
    job.precision = abi.PRECISION_FP32_BULK
    ws = et.Engine(device=0)
    st = et.Engine(device=0)
    st.set_static_assignment(True)
    for e in (ws, st):
        e.keep_final_states(True)
    r1, s1, a1 = ws.run(job, want_amplitude=True)
    r2, s2, a2 = st.run(job, want_amplitude=True)
    n = r1.num_effective_traj
    assert n == r2.num_effective_traj > 1000
    assert r1.num_steps == r2.num_steps and r1.ion_prob == r2.ion_prob
    assert np.array_equal(s1, s2) and np.array_equal(a1, a2)
    p1, f1, t1 = ws.dump_final_states(n)
    p2, f2, t2 = st.dump_final_states(n)
    assert np.array_equal(p1, p2) and np.array_equal(f1, f2) and np.array_equal(t1, t2)
    ws.close()
    st.close()


SPA_CASES = [
    dict(method="SPA", dim=3, mc=True, laser="bichrom", phase="QTMC", nt=40, nkd=12, nkz=12, prefix=["Pre", "Jac"]),
    dict(method="SPA", dim=2, target="Ar", laser="cos2", phase="SCTS", ellip=1.0, mc=True, nt=60, nkd=200, nkz=1),
]


@pytest.mark.parametrize("kw", SPA_CASES, ids=["H-bichrom-3d-prejac", "Ar-cos2-2d-full"])
def test_bulk_spa_sampler_tracks_fp64(eng, kw):
    """The bulk path's FP32 SPA candidates (saddle-point solve, quadratures and
    Jacobian at FP32 tolerances) keep the FP64 sampler's electrons: the same
    survivors but for a few near the cutoff or the solver's convergence edge,
    exit points and momenta to ~1e-4, rates to ~1e-3, phases to ~1e-3 rad."""
    job = job_of(**kw)
    a64 = eng.sample_all(job)
    a32 = eng.sample_all(bulk(job))
    dim = job.dimension
    tc, rc = (6, 7) if dim == 3 else (4, 5)
    n64, n32 = len(a64), len(a32)
    assert n64 > 200
    assert abs(n32 - n64) <= 0.01 * n64 + 2
    assert abs(a32[:, rc].sum() - a64[:, rc].sum()) <= 1e-3 * a64[:, rc].sum()
    kcols = [3, 4, 5] if dim == 3 else [2, 3]
    matched, close = 0, 0
    for t in np.unique(a64[:, tc]):
        r64 = a64[a64[:, tc] == t]
        r32 = a32[a32[:, tc] == t]
        if len(r32) == 0:
            continue
        d = np.linalg.norm(r32[:, None, kcols] - r64[None, :, kcols], axis=2)
        j = d.argmin(axis=1)
        ok = d[np.arange(len(r32)), j] < 1e-4
        matched += ok.sum()
        a, b = r32[ok], r64[j[ok]]
        good = (np.abs(a[:, rc] - b[:, rc]) <= 5e-3 * b[:, rc]) & (np.abs(a[:, 0] - b[:, 0]) <= 1e-3 * np.abs(b[:, 0]) + 1e-3)
        if job.traj_phase_method != abi.PHASE_CTMC:
            dph = np.angle(np.exp(1j * (a[:, -1] - b[:, -1])))
            good &= np.abs(dph) <= 1e-3
        close += good.sum()
    assert matched >= 0.999 * n32
    assert close >= 0.999 * matched


def test_bulk_spa_pmd_within_fp64_band(eng):
    """SPA electrons start closer to the core than ADK's, so the FP32 integrator
    moves a coherent PMD more; with 1.4e5 electrons it stays within FP64's own
    tolerance band (measured: 0.025 against 0.027 at full resolution, 1.3x the
    band after 10x10 rebinning)."""
    job = job_of(method="SPA", dim=2, target="Ar", laser="cos2", phase="SCTS", ellip=1.0, mc=True, nt=2000,
                 nkd=200, nkz=1, pnum=(100, 100), pmax=2.0)
    r64, s64, _ = eng.run(job)
    tight = job.copy()
    tight.traj_rtol = job.traj_rtol / 10
    r64b, s64b, _ = eng.run(tight)
    r32, s32, _ = eng.run(bulk(job))
    assert r64.num_effective_traj > 100000
    assert abs(r32.num_effective_traj - r64.num_effective_traj) <= 1e-3 * r64.num_effective_traj
    assert abs(r32.ion_prob - r64.ion_prob) <= 2e-3 * r64.ion_prob
    assert rel_l2(s32, s64) <= 1.5 * rel_l2(s64b, s64), (rel_l2(s32, s64), rel_l2(s64b, s64))
    c32, c64, c64b = (rebin(s, (100, 100), 10) for s in (s32, s64, s64b))
    assert rel_l2(c32, c64) <= max(2.0 * rel_l2(c64b, c64), 5e-3), (rel_l2(c32, c64), rel_l2(c64b, c64))


# ---- edge cases of the bulk path ---------------------------------------------------------

@pytest.mark.parametrize("method", ["ADK", "SPANE"])
def test_bulk_empty_job(eng, method):
    """No candidate survives the cutoff: no trajectory, zero spectrum and
    probabilities, as on the FP64 path (ADKSampler.jl:392-394)."""
    job = bulk(job_of(method=method, dim=2, phase="SCTS", target="Ar", cutoff=1e300))
    res, spec, amp = eng.run(job, want_amplitude=True)
    assert res.num_effective_traj == 0 and res.ion_prob == 0.0 and res.ion_prob_uncollected == 0.0
    assert not spec.any() and not amp.any()


def test_bulk_four_electrons(eng):
    """Eight candidates (kd = +-0.2 at t = -T, -T/3, T/3, T; the field vanishes
    at +-T): the bulk path keeps the FP64 path's four electrons and their weights."""
    job = job_of(method="ADK", dim=2, phase="QTMC", target="H", nt=4, nkd=2, nkz=1, intensity=4e14)
    job.ss_kd_max = 0.2
    r64, s64, _ = eng.run(job)
    r32, s32, _ = eng.run(bulk(job))
    assert r64.num_effective_traj == r32.num_effective_traj == 4
    assert r32.ion_prob == pytest.approx(r64.ion_prob, rel=1e-5)
    assert s32.sum() == pytest.approx(s64.sum(), rel=1e-4)


@pytest.mark.parametrize("pnum", [(1, 50), (50, 1)])
def test_bulk_single_bin_axis(eng, pnum):
    """final_p_num = 1 along an axis puts every electron in its one bin
    (TrajectorySimulation.jl:254-260, the index rule for num = 1)."""
    job = job_of(method="ADK", dim=2, phase="CTMC", target="H", nt=40, nkd=21, pnum=pnum)
    r64, s64, _ = eng.run(job)
    r32, s32, _ = eng.run(bulk(job))
    assert r32.num_effective_traj == r64.num_effective_traj > 0
    assert s32.sum() == pytest.approx(s64.sum(), rel=1e-4)
    assert rel_l2(s32, s64) <= 0.05
