"""Shards of one job run through the engine (one after the other on one GPU)
and merged as the multi-GPU path merges them: the whole job's result."""
import numpy as np
import pytest

import etraj_gb300 as et
from etraj_gb300 import abi, shards
from test_gpu_parity import job_of, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    e = et.Engine(device=0)
    yield e
    e.close()


@pytest.mark.parametrize("phase,precision", [("CTMC", abi.PRECISION_FP64), ("SCTS", abi.PRECISION_FP64),
                                             ("QTMC", abi.PRECISION_FP32_BULK)])
def test_grid_shards_merge_to_the_whole_job(eng, phase, precision):
    job = job_of(method="ADK", dim=2, phase=phase, target="Ar", nt=60, nkd=31, laser="cos2", ellip=0.5,
                 cutoff=0.0)
    job.precision = precision
    coh = shards.is_coherent(job)
    r, spec, _ = eng.run(job)
    for world in (2, 3):
        vec, tot = 0.0, 0.0
        for k in range(world):
            j, w = shards.shard_job(job, k, world)
            rk, sk, ak = eng.run(j, want_spectrum=not coh, want_amplitude=coh)
            v, t = shards.weigh(rk, sk, ak, w, coh)
            vec, tot = vec + v, tot + t
        mspec, ion, unc, neff = shards.finalize(vec, tot, coh)
        assert neff == r.num_effective_traj > 0
        assert ion == pytest.approx(r.ion_prob, rel=1e-9)
        assert rel_l2(mspec, spec) <= (1e-8 if precision == abi.PRECISION_FP64 else 1e-2)
