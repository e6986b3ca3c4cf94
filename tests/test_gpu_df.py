"""The double-float integrator (ETRAJ_PRECISION_FP32_DF) on the GPU, through the
C ABI.

  * Against its host build (df_solve.cuh compiled by g++, tests/df_host.cpp):
    the same final states, status and step attempts bit for bit, so the warp
    interleaving, the shared-memory stage slots and the work stealing of the
    kernel change nothing in an electron's arithmetic.
  * Against the FP64 path on the same jobs: it samples with the FP64 sampler
    (the same electrons) and follows the FP64 step sequence.  Bar, set by how far
    the FP64 solve moves when its own rounding changes (test_df_host.py): the
    same electrons and failures, ionized electrons within a few, step attempts
    equal for all but a few in 1e4, median relative difference of the asymptotic
    momenta below 1e-9, momentum distribution within 1e-5 relative L2.
"""
import numpy as np
import pytest

import etraj_gb300 as et
from etraj_gb300 import abi
from test_df_host import dfhost, host_integrate, jobs  # noqa: F401  (dfhost: fixture)
from test_gpu_parity import job_of, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    e = et.Engine(device=0)
    yield e
    e.close()


def run_kept(eng, job):
    eng.keep_final_states(True)
    try:
        res, spec, _ = eng.run(job)
        n = res.num_effective_traj
        p, ph, st = eng.dump_final_states(n)
        steps = eng.dump_step_counts(n)
    finally:
        eng.keep_final_states(False)
    return res, spec, p, st, steps


def compare_df_fp64(eng, job):
    r64, s64, p64, st64, k64 = run_kept(eng, job)
    d = job.copy()
    d.precision = abi.PRECISION_FP32_DF
    rdf, sdf, pdf, stdf, kdf = run_kept(eng, d)
    n = r64.num_effective_traj
    assert rdf.num_effective_traj == n > 0
    assert rdf.num_failed_traj == r64.num_failed_traj
    assert abs(rdf.num_ionized_traj - r64.num_ionized_traj) <= 2 + n // 100000
    both = ((st64 & 0x100) != 0) & ((stdf & 0x100) != 0)
    rel = np.linalg.norm(pdf[both] - p64[both], axis=1) / np.maximum(np.linalg.norm(p64[both], axis=1), 1e-300)
    assert np.median(rel) <= 1e-9, np.median(rel)
    assert np.sum(kdf != k64) <= 2 + n // 10000, np.sum(kdf != k64)
    pmd = rel_l2(sdf, s64)
    assert pmd <= 1e-5, pmd
    assert abs(rdf.ion_prob - r64.ion_prob) <= 1e-9 * abs(r64.ion_prob)


CASES = [
    dict(method="ADK", dim=2, phase="CTMC", target="H", laser="cos4", nt=200, nkd=201),
    dict(method="SPANE", dim=2, phase="SCTS", target="Ar", laser="cos2", ellip=1.0, mc=True, nt=300, nkd=200,
         nkz=1, intensity=1.2e14),
    dict(method="ADK", dim=3, phase="QTMC", target="Ar", laser="cos2", ellip=0.5, nt=60, nkd=25, nkz=15),
    dict(method="ADK", dim=3, phase="SCTS", target="Ar", laser="cos4", nt=60, nkd=25, nkz=15, intensity=2e14),
    dict(method="ADK", dim=2, phase="SCTS", target="H", laser="gauss", nt=200, nkd=101),
    dict(method="SPANE", dim=3, phase="CTMC", target="H", laser="bichrom", mc=True, nt=100, nkd=30, nkz=30),
    dict(method="ADK", dim=2, phase="QTMC", target="Xe", laser="cos4", ellip=1.0, nt=200, nkd=101),
    dict(proposal="adk_gauss", method="SPANE", dim=2, phase="SCTS", target="Ar", laser="cos2", ellip=1.0,
         mc=True, nt=300, nkd=200, nkz=1, intensity=1.2e14),
    # SPA: the FP64 sampler over the candidates its FP32 pre-pass keeps at 0.8 x the cutoff
    dict(method="SPA", dim=2, phase="SCTS", target="Ar", laser="cos2", ellip=1.0, nt=64, nkd=61),
    dict(method="SPA", dim=3, phase="QTMC", target="H", laser="bichrom", mc=True, nt=40, nkd=20, nkz=20),
]


@pytest.mark.parametrize("kw", CASES, ids=lambda k: "-".join(str(v) for v in list(k.values())[:5]))
def test_df_tracks_fp64(eng, kw):
    compare_df_fp64(eng, job_of(**kw))


@pytest.mark.parametrize("name", sorted(jobs()))
def test_df_kernel_matches_its_host_build(eng, dfhost, name):  # noqa: F811
    job = jobs()[name].copy()
    job.precision = abi.PRECISION_FP32_DF
    init = eng.sample_all(job)  # the FP64 sampler
    fin, st, steps = eng.integrate(job, init)
    hfin, hst, hsteps = host_integrate(dfhost, job, init, tmin=float(init[:, 2 * job.dimension].min()))
    assert init.shape[0] > 500
    assert np.array_equal(st, hst) and np.array_equal(steps, hsteps)
    assert np.array_equal(fin.view(np.uint64), hfin.view(np.uint64))


def test_df_through_submit_and_server(eng):
    """The same job through the asynchronous entry points and a server slot gives
    the same bits as etraj_run."""
    job = job_of(method="SPANE", dim=2, phase="SCTS", target="Ar", laser="cos2", ellip=1.0, mc=True, nt=100,
                 nkd=100, nkz=1, intensity=1.2e14)
    job.precision = abi.PRECISION_FP32_DF
    r0, s0, _ = eng.run(job)
    r1 = abi.Result()
    s1 = np.zeros(job.grid_size)
    r1.momentum_spec = abi.dptr(s1)
    t = eng.submit(job, r1)
    eng.wait(t, r1)
    assert np.array_equal(s0, s1) and r1.ion_prob == r0.ion_prob
    srv = et.Server(device=0, slots=2)
    try:
        tk = srv.submit(job)
        r2, s2, _ = srv.wait(tk)
    finally:
        srv.close()
    assert np.array_equal(s0, s2) and r2.ion_prob == r0.ion_prob


def test_df_rejects_spans_beyond_its_clock(eng):
    job = job_of(method="ADK", dim=2, nt=4, nkd=5)
    job.precision = abi.PRECISION_FP32_DF
    job.traj_t_final = 2e4 * 2 * np.pi / (45.563352525 / 800.0)
    with pytest.raises(et.EtrajError) as e:
        eng.run(job)
    assert e.value.status == abi.ERR_UNSUPPORTED


def test_df_small_and_empty_jobs(eng):
    """The passes' warps go through the stages in step and a block leaves when all
    of its lanes are free: jobs of a few electrons (most warps of a block without
    work), of just over one block, and of none, against the FP64 path."""
    empty = job_of(method="ADK", dim=2, cutoff=1e300)
    empty.precision = abi.PRECISION_FP32_DF
    res, spec, _ = eng.run(empty)
    assert res.num_effective_traj == 0 and res.ion_prob == 0.0 and not spec.any()
    for kw in (dict(method="ADK", dim=2, nt=4, nkd=9),                # 4 electrons
               dict(method="ADK", dim=3, phase="QTMC", nt=6, nkd=9, nkz=5),  # a few tens
               dict(method="SPANE", dim=2, phase="SCTS", target="Ar", laser="cos2", ellip=1.0,
                    mc=True, nt=12, nkd=300, nkz=1, intensity=1.2e14)):  # 1329: two blocks of 1024 lanes' work
        job = job_of(**kw)
        r64, _, _ = eng.run(job)
        assert 0 < r64.num_effective_traj < 2048, r64.num_effective_traj
        compare_df_fp64(eng, job)
