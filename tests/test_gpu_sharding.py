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


@pytest.mark.parametrize("precision,si_tol,tol", [(capi.UMT_FP64, 1e-11, 1e-12), (capi.UMT_FP32, 1e-6, 2e-5)])
def test_device_plane_two_shards_match_one_context(umtlib, precision, si_tol, tol):
    """Two library contexts (the direction blocks two ranks would hold on two
    GPUs) iterate with PhiTotal on the device: each builds its source and
    sweeps (umt103_si_step); their device PhiTotal buffers are summed in
    place through torch views of umt103_phi_device (standing in for the NCCL
    all-reduce, which needs two GPUs); the converged flux equals the
    one-context source iteration."""
    pytest.importorskip("torch")
    prob = synthetic_problem((3, 2, 2), 2, 2, 8, seed=5, c_range=(0.3, 0.8), time_dependent=True)
    m = prob.mesh
    umtlib.init(m, prob.omega, prob.weight, prob.ngr, flags=(1 if precision == capi.UMT_FP64 else 2) | 8)
    umtlib.set_materials(prob.sigt, prob.sigs, prob.tau)
    umtlib.set_psi(prob.psi0, None)
    r = umtlib.source_iterate(precision=precision, rel_tol=si_tol, q_ext=prob.q_ext, save_psi=False, max_iters=500)
    ref = umtlib.get_phi()
    ids, sws = [], []
    for dirs in sharding.direction_shards(len(prob.weight), 2):
        cid = umtlib.context_create()
        umtlib.context_select(cid)
        sws.append(sharding.DeviceSweeper(umtlib, prob, dirs, precision))
        ids.append(cid)

    class Pair:                                    # the two shards driven as one rank pair
        def __init__(self):
            self.t = []
            for cid, sw in zip(ids, sws):
                umtlib.context_select(cid)
                self.t.append(sw.phi_tensor())

        def phi_tensor(self):
            return self.t[0]

        def step(self):
            for cid, sw in zip(ids, sws):
                umtlib.context_select(cid)
                sw.step()

        def change(self):
            rel = []
            for cid, sw in zip(ids, sws):
                umtlib.context_select(cid)
                rel.append(sw.change())
            assert abs(rel[0] - rel[1]) <= 1e-12 * max(rel[0], 1e-300)   # atomic reduction order
            return rel[0]

    pair = Pair()

    def allreduce(_):
        s = pair.t[0] + pair.t[1]
        pair.t[0].copy_(s)
        pair.t[1].copy_(s)

    pair.t[1].zero_()
    it, conv = sharding.source_iterate_device(pair, allreduce, rel_tol=si_tol, max_iters=500)
    got = pair.t[0].cpu().numpy().reshape(m.ncornr, prob.ngr)
    umtlib.context_select(0)
    for cid in ids:
        umtlib.context_destroy(cid)
    assert conv and abs(it - r["iterations"]) <= 1          # summation order of the two shards
    assert float(np.max(np.abs(got - ref)) / np.max(np.abs(ref))) < tol
