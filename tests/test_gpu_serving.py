"""Asynchronous jobs and the serving loop (continuous batching on one GPU).

Every job is a pure function of its parameters: the server runs jobs on
separate contexts (own stream, own buffers) and the deposit is deterministic,
so each result must be bit-identical alone (etraj_run on a fresh context) and
in any mix of concurrently running jobs.
"""
import numpy as np
import pytest

import etraj_gb300 as et
from etraj_gb300 import abi
from test_gpu_parity import job_of

pytestmark = pytest.mark.gpu


def mix():
    """Jobs of different lasers, targets, samplers, phases, dimensions, grids and paths."""
    jobs = [
        job_of(method="ADK", dim=2, nt=60, nkd=41, ellip=0.5),
        job_of(method="SPANE", dim=2, phase="SCTS", target="Ar", laser="cos2", ellip=1.0, mc=True, nt=300,
               nkd=200, nkz=1, pnum=(256, 256), pmax=2.0),
        job_of(method="ADK", dim=3, phase="QTMC", laser="gauss", nt=40, nkd=15, nkz=9, pnum=(48, 48, 16)),
        job_of(method="SPANE", dim=3, phase="CTMC", laser="bichrom", mc=True, nt=30, nkd=20, nkz=10,
               pnum=(40, 40, 1)),
        job_of(method="SPA", dim=2, phase="QTMC", ellip=1.0, nt=16, nkd=31),
        job_of(method="ADK", dim=2, phase="SCTS", target="Ne", ellip=1.0, nt=80, nkd=61, pmax=1.0),
    ]
    bulk = []
    for j in (jobs[1], jobs[2]):
        b = j.copy()
        b.precision = abi.PRECISION_FP32_BULK
        bulk.append(b)
    return jobs + bulk


def same(a, b):
    return (a is None and b is None) or np.array_equal(a.view(np.uint64), b.view(np.uint64))


def scalars(r):
    return (r.ion_prob, r.ion_prob_uncollected, r.num_effective_traj, r.num_failed_traj,
            r.num_ionized_traj, r.num_steps)


@pytest.fixture(scope="module")
def alone():
    """Each job of the mix on a fresh context, one at a time."""
    out = []
    for job in mix():
        eng = et.Engine(device=0)
        out.append(eng.run(job, want_spectrum=True, want_amplitude=True))
        eng.close()
    return out


def test_async_submit_matches_run(alone):
    eng = et.Engine(device=0)
    jobs = mix()[:4]
    held = []
    for job in jobs:
        res = abi.Result()
        spec = np.zeros(job.grid_size)
        amp = np.zeros(2 * job.grid_size) if job.traj_phase_method != abi.PHASE_CTMC else None
        res.momentum_spec = abi.dptr(spec)
        res.amplitude = abi.dptr(amp)
        held.append((eng.submit(job, res), res, spec, amp))
    for (tk, res, spec, amp), (r0, s0, a0) in zip(held, alone):
        eng.wait(tk, res)
        assert scalars(res) == scalars(r0)
        assert same(spec, s0) and same(amp, a0)
    eng.close()


def test_server_mix_equals_alone(alone):
    srv = et.Server(device=0, slots=3)
    tickets = [srv.submit(job, want_spectrum=True, want_amplitude=True) for job in mix()]
    seen_running = srv.stats()[0]
    for tk, (r0, s0, a0) in zip(tickets, alone):
        r, s, a = srv.wait(tk, timeout=300.0)
        assert scalars(r) == scalars(r0)
        assert same(s, s0) and same(a, a0)
    assert seen_running >= 1
    assert srv.stats()[:2] == (0, 0)
    srv.close()


def test_server_queues_under_a_small_budget(alone):
    # room for about one of the larger jobs at a time: the rest wait in the queue
    srv = et.Server(device=0, slots=4, hbm_budget_bytes=24 << 20)
    jobs = mix()
    tickets = [srv.submit(job) for job in jobs]
    _, queued, _ = srv.stats()
    assert queued >= 1
    for tk, (r0, s0, _) in zip(tickets, alone):
        r, s, _ = srv.wait(tk, timeout=300.0)
        assert scalars(r) == scalars(r0) and same(s, s0)
    assert srv.stats()[2] <= 24 << 20
    srv.close()


def test_server_rejects_and_times_out():
    srv = et.Server(device=0, slots=2, hbm_budget_bytes=8 << 20)
    big = job_of(method="ADK", dim=2, nt=2000, nkd=401)
    tk = srv.submit(big)
    with pytest.raises(et.EtrajError) as e:
        srv.wait(tk, timeout=60.0)
    assert e.value.status == abi.ERR_OUT_OF_MEMORY
    bad = job_of(method="ADK", dim=2)
    bad.traj_t_final = -1.0
    with pytest.raises(et.EtrajError):
        srv.submit(bad)
    srv.close()
    srv = et.Server(device=0, slots=1)
    slow = job_of(method="SPANE", dim=2, phase="SCTS", target="Ar", laser="cos2", ellip=1.0, mc=True,
                  nt=4000, nkd=1000, nkz=1)
    tk = srv.submit(slow)
    with pytest.raises(et.EtrajError):
        srv.wait(tk, timeout=0.0)
    r, _, _ = srv.wait(tk, timeout=300.0)
    assert r.num_effective_traj > 0
    srv.close()
