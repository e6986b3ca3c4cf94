"""Rank body of the two-rank gloo test of etraj_gb300.shards (a spawned child
process imports this module only, so it loads the package itself)."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
import __graft_entry__  # noqa: E402

__graft_entry__.load_package()


def rank_arrays(rank, grid):
    """Deterministic stand-ins for one rank's result, spectrum and amplitude grid."""
    rng = np.random.default_rng(100 + rank)
    res = type("R", (), {})()
    res.ion_prob, res.ion_prob_uncollected, res.num_effective_traj = 0.3 + rank, 0.01 * (rank + 1), 1000 + rank
    return res, rng.random(grid), rng.standard_normal(2 * grid)


def worker(rank, world, port, out_dir, coherent):
    import torch.distributed as dist
    from etraj_gb300 import shards
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        res, spec, amp = rank_arrays(rank, 64)
        m = shards.merge_shards(res, spec, amp, 1.0 / world, coherent)
        agg = shards.aggregate_throughput(res.num_effective_traj, 1.0 + rank)
        np.savez(os.path.join(out_dir, "r%d.npz" % rank), spec=m[0], scal=np.array(m[1:], dtype=np.float64),
                 agg=np.array(agg))
    finally:
        dist.destroy_process_group()
