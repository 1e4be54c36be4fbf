"""LibrarySweeper (umt_gb300/sharding.py) on the GPU: the directions split over
two library contexts (what two ranks would hold on two GPUs) sweep to partial
fluxes whose sum is the one-context flux."""
import numpy as np
import pytest

from umt_gb300 import capi, sharding
from umt_gb300.problems import synthetic_problem

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,tol", [(capi.UMT_FP64, 1e-13), (capi.UMT_FP32, 1e-6)])
def test_direction_shards_sum_to_full_sweep(umtlib, precision, tol):
    prob = synthetic_problem((3, 2, 2), 2, 2, 8, seed=5, time_dependent=True)
    m = prob.mesh
    STotal = sharding.scattering_source(prob, np.full((m.ncornr, prob.ngr), 0.3), prob.q_ext)
    full = sharding.LibrarySweeper(umtlib, prob, np.arange(len(prob.weight)), precision).sweep(STotal)
    ids, parts = [], []
    for dirs in sharding.direction_shards(len(prob.weight), 2):
        cid = umtlib.context_create()
        umtlib.context_select(cid)
        parts.append(sharding.LibrarySweeper(umtlib, prob, dirs, precision).sweep(STotal))
        ids.append(cid)
    umtlib.context_select(0)
    for cid in ids:
        umtlib.context_destroy(cid)
    total = parts[0] + parts[1]
    assert float(np.max(np.abs(total - full)) / np.max(np.abs(full))) < tol
