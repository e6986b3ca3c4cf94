"""One job over several GPUs: one shard per rank, merged by a single sum-reduce.

Trajectories are independent, so a job splits into shards that run with no
exchange at all; the reference's own reduction (`write_output!`,
TrajectorySimulation.jl:521-543: the per-thread spectra summed, then `abs2`
for the coherent modes, and ion_prob / ion_prob_uncollected / eff_trajs
summed) becomes one all-reduce over ranks of the complex amplitude grid
(before `abs2`) or the CTMC spectrum, plus three scalars.

Sharding keeps the reference's normalisation.  Every deposited weight
carries the sampler's cell size dkdt = step(t) step(kd) step(kz) (Monte
Carlo: the spans over mc_kt_num; ADKSampler.jl:267-276, step = (max - min) /
length), and the amplitude sqrt(dkdt):

- A Monte-Carlo job shards by seed: rank r runs the same job with seed + r,
  an independent estimate of the same spectrum.  The merge is their mean: a
  shard's weights count 1 / world and its amplitudes 1 / sqrt(world), as in
  one job of world x the time samples at dkdt / world.  (That job's step(t)
  would be the spread of all shards' random time samples over their number;
  each shard's own spread differs from it by O(1 / sample_t_num).)
- A grid job shards by contiguous ranges of its time samples (the points of
  range(t1, t2, length = n)); a shard's own step(t) is that of its range, so
  its weights count step_full / step_shard.  ADK's rate cutoff (ADKSampler.jl:
  332) compares rates that carry the shard's own dkdt, so a candidate within
  that factor of the cutoff can fall on the other side of it in a shard.

The collective uses whatever process group is given: gloo with CPU tensors,
NCCL with CUDA tensors.
"""
import math

import numpy as np

from . import abi


def shard_job(job, rank, world):
    """(job_r, weight_r): rank's shard of `job` and the factor its deposited
    weights carry in the merge (its amplitudes carry sqrt(weight_r))."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d of %d" % (rank, world))
    j = job.copy()
    if world == 1:
        return j, 1.0
    if job.sample_monte_carlo:
        j.seed = job.seed + rank
        return j, 1.0 / world
    n = int(job.sample_t_num)
    if n < 2 * world:
        raise ValueError("a grid job of %d time samples cannot give %d shards of two or more" % (n, world))
    t1, t2 = job.sample_t_intv[0], job.sample_t_intv[1]
    a, b = (rank * n) // world, ((rank + 1) * n) // world  # time samples a .. b-1

    def t_at(k):
        return t2 if k == n - 1 else t1 + (t2 - t1) * k / (n - 1)

    j.sample_t_intv[0], j.sample_t_intv[1] = t_at(a), t_at(b - 1)
    j.sample_t_num = b - a
    step_full = (t2 - t1) / n
    step_shard = (j.sample_t_intv[1] - j.sample_t_intv[0]) / (b - a)
    return j, step_full / step_shard


def weigh(res, spectrum, amplitude, weight, coherent):
    """A shard's contribution to the merge: (grid vector, scalars).  The vector
    is the amplitude grid (interleaved re, im) times sqrt(weight) for the
    coherent modes, the CTMC spectrum times weight otherwise; the scalars are
    ion_prob and ion_prob_uncollected times weight, and num_effective_traj."""
    if coherent:
        if amplitude is None:
            raise ValueError("a coherent shard needs its amplitude grid (want_amplitude=True)")
        vec = np.asarray(amplitude, dtype=np.float64) * math.sqrt(weight)
    else:
        vec = np.asarray(spectrum, dtype=np.float64) * weight
    sc = np.array([res.ion_prob * weight, res.ion_prob_uncollected * weight, float(res.num_effective_traj)])
    return vec, sc


def finalize(vec, scalars, coherent):
    """(momentum_spec, ion_prob, ion_prob_uncollected, num_effective_traj) of the
    summed contributions: abs2 of the summed amplitudes for the coherent modes."""
    if coherent:
        re, im = vec[0::2], vec[1::2]
        spec = re * re + im * im
    else:
        spec = vec.copy()
    return spec, float(scalars[0]), float(scalars[1]), int(round(scalars[2]))


def _device(group):
    import torch.distributed as dist
    return "cuda" if dist.get_backend(group) == "nccl" else "cpu"


def merge_shards(res, spectrum, amplitude, weight, coherent, group=None):
    """All ranks' shards merged (every rank gets the result): see `finalize`."""
    import torch
    import torch.distributed as dist
    vec, sc = weigh(res, spectrum, amplitude, weight, coherent)
    dev = _device(group)
    tv = torch.from_numpy(vec).to(dev)
    ts = torch.from_numpy(sc).to(dev)
    dist.all_reduce(tv, group=group)
    dist.all_reduce(ts, group=group)
    return finalize(tv.cpu().numpy(), ts.cpu().numpy(), coherent)


def aggregate_throughput(n_local, seconds_local, group=None):
    """(trajectories over all ranks, the slowest rank's time, their ratio): a
    weak-scaling run's whole-job rate."""
    import torch
    import torch.distributed as dist
    dev = _device(group)
    n = torch.tensor([float(n_local)], dtype=torch.float64, device=dev)
    t = torch.tensor([float(seconds_local)], dtype=torch.float64, device=dev)
    dist.all_reduce(n, group=group)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return n.item(), t.item(), n.item() / t.item()


def is_coherent(job):
    return job.traj_phase_method != abi.PHASE_CTMC
