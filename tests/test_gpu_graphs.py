"""CUDA-graph replay of the per-job kernel sequence gives the same results."""
import numpy as np
import pytest

import etraj_gb300 as et
from etraj_gb300 import abi
from test_gpu_parity import job_of

pytestmark = pytest.mark.gpu


def test_graph_replay_matches_direct_launches():
    jobs = [job_of(method="ADK", dim=2, phase="QTMC", ellip=1.0, nt=40, nkd=31),
            job_of(method="SPANE", dim=2, phase="SCTS", target="Ar", laser="cos2", ellip=1.0, mc=True, nt=200,
                   nkd=200, nkz=1, pnum=(128, 128), pmax=2.0)]
    b = jobs[1].copy()
    b.precision = abi.PRECISION_FP32_BULK
    jobs.append(b)
    direct = et.Engine(device=0)
    direct.set_graphs(False)
    ref = [direct.run(j, want_amplitude=True) for j in jobs]
    direct.close()
    g = et.Engine(device=0)
    g.set_graphs(True)
    # capture, replay twice, interleave another job (recapture), come back
    for j, (r0, s0, a0) in list(zip(jobs, ref)) * 2 + [(jobs[0], ref[0])] * 3:
        r, s, a = g.run(j, want_amplitude=True)
        assert r.num_effective_traj == r0.num_effective_traj and r.ion_prob == r0.ion_prob
        assert np.array_equal(s, s0) and (a is None or np.array_equal(a, a0))
    import ctypes as C
    buf = (C.c_double * 8)()
    assert g.lib.etraj_stage_times(g.ctx, buf, 8) == 6 and buf[3] > 0.0
    g.close()


def test_batch_graph_replay_matches_direct_launches():
    """A multi-instance batch runs directly, is captured the second time and
    replayed the third, each time with the direct run's bits."""
    import bench
    jobs, w = bench.multi_instance_jobs(n=6, seed=3)
    direct = et.Engine(device=0)
    direct.set_graphs(False)
    ref, wref = direct.run_batch(jobs, want_spectrum=True, weights=w)
    direct.close()
    g = et.Engine(device=0)
    for _ in range(3):
        outs, wsum = g.run_batch(jobs, want_spectrum=True, weights=w)
        assert np.array_equal(wsum, wref)
        for (r, s, _), (r0, s0, _) in zip(outs, ref):
            assert r.num_effective_traj == r0.num_effective_traj and r.ion_prob == r0.ion_prob
            assert np.array_equal(s, s0)
    g.close()
