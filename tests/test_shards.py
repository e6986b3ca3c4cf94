"""Sharding one job over ranks (etraj_gb300.shards), on the CPU.

The merge math is checked against the oracle (two grid shards of a job merge
to the whole job), and the collectives over two gloo ranks, as the multi-GPU
bench runs them with NCCL."""
import math
import os
import socket

import numpy as np
import pytest

import _oracle as O
import etraj_gb300 as et
from etraj_gb300 import shards


def _job(mc=False, phase="QTMC", nt=12, cutoff=0.0, dim=2):
    T = 2 * math.pi / (45.563352525 / 800.0)
    kw = dict(init_cond_method="ADK", laser=et.Cos4Laser(peak_int=1e14, wave_len=800.0, cyc_num=2, ellip=0.0),
              target=et.get_atom("H"), dimension=dim, sample_t_intv=(-T, T), sample_t_num=nt,
              traj_t_final=2 * T, final_p_max=(1.5,) * dim, final_p_num=(48, 48, 8)[:dim], traj_phase_method=phase,
              sample_cutoff_limit=cutoff, seed=5)
    if mc:
        kw.update(sample_monte_carlo=True, mc_kt_num=40, mc_kd_max=1.0, mc_kz_max=1.0 if dim == 3 else 0.0)
    else:
        kw.update(ss_kd_max=1.0, ss_kd_num=15, ss_kz_max=1.0 if dim == 3 else 0.0, ss_kz_num=5 if dim == 3 else 0)
    return et.make_job(**kw)


def test_grid_shards_cover_the_time_samples_once():
    job = _job(nt=23)
    t = np.linspace(job.sample_t_intv[0], job.sample_t_intv[1], job.sample_t_num)
    got, n = [], 0
    for r in range(3):
        j, w = shards.shard_job(job, r, 3)
        tr = np.linspace(j.sample_t_intv[0], j.sample_t_intv[1], j.sample_t_num)
        got.append(tr)
        n += j.sample_t_num
        step_full = (t[-1] - t[0]) / t.size
        assert w == pytest.approx(step_full / ((tr[-1] - tr[0]) / tr.size), rel=1e-14)
    assert n == job.sample_t_num
    np.testing.assert_allclose(np.concatenate(got), t, rtol=0, atol=1e-12 * abs(t).max())
    with pytest.raises(ValueError):
        shards.shard_job(_job(nt=5), 0, 3)


def test_monte_carlo_shards_differ_by_seed():
    job = _job(mc=True)
    js = [shards.shard_job(job, r, 4) for r in range(4)]
    assert [j.seed for j, _ in js] == [job.seed + r for r in range(4)]
    assert all(w == 0.25 for _, w in js)
    assert all(j.mc_kt_num == job.mc_kt_num and j.sample_t_num == job.sample_t_num for j, _ in js)


class _Res:
    def __init__(self, sc):
        self.ion_prob = sc["ion_prob"]
        self.ion_prob_uncollected = sc["ion_prob_uncollected"]
        self.num_effective_traj = int(sc["num_effective"])


@pytest.mark.parametrize("phase,dim", [("CTMC", 2), ("QTMC", 2), ("SCTS", 3)])
def test_grid_shards_merge_to_the_whole_job(phase, dim):
    """Two grid shards, each weighted by its step(t), sum to the whole job's
    spectrum, probabilities and trajectory count (the shards' time samples
    agree with the whole job's to rounding)."""
    job = _job(phase=phase, dim=dim)
    coherent = shards.is_coherent(job)
    spec, amp, sc = O.run(job)
    vec, tot = 0.0, 0.0
    for r in range(2):
        j, w = shards.shard_job(job, r, 2)
        s_r, a_r, sc_r = O.run(j)
        v, t = shards.weigh(_Res(sc_r), s_r, a_r, w, coherent)
        vec, tot = vec + v, tot + t
    mspec, ion, unc, neff = shards.finalize(vec, tot, coherent)
    assert neff == int(sc["num_effective"]) > 0
    assert ion == pytest.approx(sc["ion_prob"], rel=1e-9)
    assert unc == pytest.approx(sc["ion_prob_uncollected"], rel=1e-9, abs=1e-300)
    assert np.linalg.norm(mspec - spec) <= 1e-8 * np.linalg.norm(spec)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("coherent", [False, True])
def test_merge_over_two_gloo_ranks(tmp_path, coherent):
    import torch.multiprocessing as mp
    import _shard_worker as W
    world = 2
    mp.spawn(W.worker, args=(world, _free_port(), str(tmp_path), coherent), nprocs=world, join=True)
    vec, tot = 0.0, 0.0
    for r in range(world):
        res, spec, amp = W.rank_arrays(r, 64)
        v, t = shards.weigh(res, spec, amp, 1.0 / world, coherent)
        vec, tot = vec + v, tot + t
    want = shards.finalize(vec, tot, coherent)
    for r in range(world):
        got = np.load(os.path.join(tmp_path, "r%d.npz" % r))
        np.testing.assert_allclose(got["spec"], want[0], rtol=1e-14, atol=0)
        np.testing.assert_allclose(got["scal"], np.array(want[1:], dtype=np.float64), rtol=1e-14)
        assert tuple(got["agg"]) == (2001.0, 2.0, 2001.0 / 2.0)
