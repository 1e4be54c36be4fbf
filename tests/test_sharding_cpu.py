"""Angle sharding over ranks (umt_gb300/sharding.py): host logic checked with
world_size-2 gloo process groups on the CPU.  Each rank sweeps its block of
directions with the oracle standing in for its GPU (the product uses
LibrarySweeper); one all-reduce of PhiTotal per source iteration must give the
single-rank result."""
import multiprocessing as mp
import os
import socket

import numpy as np
import pytest

from umt_gb300 import sharding
from umt_gb300.problems import synthetic_problem

PROBLEM = dict(tiles=(2, 2, 1), npolar=2, nazimuthal=2, ngr=4, seed=17, sigt_range=(1.0, 10.0),
               c_range=(0.5, 0.9), time_dependent=True)


def _problem():
    p = dict(PROBLEM)
    return synthetic_problem(p.pop("tiles"), p.pop("npolar"), p.pop("nazimuthal"), p.pop("ngr"), **p)


class OracleSweeper:
    """The oracle over a subset of directions (test stand-in for a rank's GPU)."""

    def __init__(self, prob, dirs):
        from oracle import pyoracle as po
        self.po, self.prob = po, prob
        m = prob.mesh
        self.geo = po.geometry(m)
        self.om = np.ascontiguousarray(prob.omega[dirs])
        self.w = np.ascontiguousarray(prob.weight[dirs])
        self.S = po.schedule(m, self.geo[0], self.geo[1], self.om)
        self.psi = np.ascontiguousarray(prob.psi0[dirs])

    def sweep(self, STotal, savePsi=False):
        p, m = self.prob, self.prob.mesh
        PsiB = np.zeros((len(self.w), m.nbelem, p.ngr))
        Phi, _, _ = self.po.set_sweep(m, self.geo, self.S, np.ascontiguousarray(p.sigt),
                                      np.ascontiguousarray(STotal), p.tau, self.om, self.w,
                                      self.psi.copy(), PsiB, savePsi=False)
        return Phi


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        prob = _problem()
        dirs = sharding.direction_shards(len(prob.weight), world)[rank]
        sw = OracleSweeper(prob, dirs)
        phi, it, conv = sharding.source_iterate(sw, prob, sharding.torch_allreduce(), q_ext=prob.q_ext,
                                                rel_tol=1e-10, max_iters=300)
        out.put((rank, phi, it, conv))
    finally:
        dist.destroy_process_group()


def test_direction_shards_cover_every_direction_once():
    for A, world in [(32, 1), (32, 2), (128, 3), (128, 8), (8, 8)]:
        sh = sharding.direction_shards(A, world)
        assert len(sh) == world
        allv = np.concatenate(sh)
        assert np.array_equal(np.sort(allv), np.arange(A))
        sizes = [len(s) for s in sh]
        assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        sharding.direction_shards(4, 8)


def test_sharded_source_iteration_matches_single_rank():
    prob = _problem()
    ref_phi, ref_it, ref_conv = sharding.source_iterate(OracleSweeper(prob, np.arange(len(prob.weight))), prob,
                                                        lambda x: x, q_ext=prob.q_ext, rel_tol=1e-10,
                                                        max_iters=300)
    assert ref_conv and ref_it > 5
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    for _ in procs:
        r, phi, it, conv = out.get(timeout=300)
        res[r] = (phi, it, conv)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # every rank holds the same flux, equal to the single-rank iteration up to
    # the summation order of the directions
    assert np.array_equal(res[0][0], res[1][0])
    assert res[0][1] == ref_it and res[0][2]
    assert float(np.max(np.abs(res[0][0] - ref_phi)) / np.max(np.abs(ref_phi))) < 1e-12


class FailingSweeper(OracleSweeper):
    """Raises on its n-th sweep: a rank failure made on the host."""

    def __init__(self, prob, dirs, fail_at):
        super().__init__(prob, dirs)
        self.calls, self.fail_at = 0, fail_at

    def sweep(self, STotal, savePsi=False):
        self.calls += 1
        if self.fail_at and self.calls == self.fail_at:
            raise RuntimeError("rank failure injected")
        return super().sweep(STotal, savePsi)


def _rank_fail_main(rank, world, port, out):
    import datetime
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=10))
    try:
        prob = _problem()
        dirs = sharding.direction_shards(len(prob.weight), world)[rank]
        sw = FailingSweeper(prob, dirs, fail_at=3 if rank == 1 else 0)
        try:
            sharding.source_iterate(sw, prob, sharding.torch_allreduce(), q_ext=prob.q_ext, rel_tol=1e-10,
                                    max_iters=300)
            out.put((rank, "finished", sw.calls))
        except Exception as e:  # the failure this test makes, or the peer's report of it
            out.put((rank, f"{type(e).__name__}: {e}"[:300], sw.calls))
    finally:
        try:
            dist.destroy_process_group()
        except Exception:
            pass


def test_rank_failure_ends_the_other_ranks_collective():
    """One rank raises in its third sweep and leaves; the other rank's next
    all-reduce ends with an error (peer gone or the process group's 10 s
    timeout) instead of waiting forever, and both processes exit."""
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_fail_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    for _ in procs:
        r, msg, calls = out.get(timeout=120)
        res[r] = (msg, calls)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode is not None
    assert res[1][0].startswith("RuntimeError: rank failure injected")
    assert res[0][0] != "finished"                   # the survivor learned of the failure
    assert res[0][1] == 3                            # in the iteration the failing rank left


class OracleBufferSweeper(OracleSweeper):
    """The device data plane's interface (DeviceSweeper) over the oracle: the
    rank's PhiTotal lives in one persistent buffer (a host tensor here, the
    library's device buffer on a GPU), the step builds the source from it and
    overwrites it with this rank's partial flux, the change is taken against
    the previous iterate."""

    def __init__(self, prob, dirs):
        import torch
        super().__init__(prob, dirs)
        m = prob.mesh
        self.buf = torch.zeros(m.ncornr * prob.ngr, dtype=torch.float64)
        self.prev = np.zeros(m.ncornr * prob.ngr)

    def phi_tensor(self):
        return self.buf

    def step(self):
        import torch
        p, m = self.prob, self.prob.mesh
        phi = self.buf.numpy().reshape(m.ncornr, p.ngr)
        part = OracleSweeper.sweep(self, sharding.scattering_source(p, phi, p.q_ext))
        self.buf.copy_(torch.from_numpy(part.ravel()))

    def change(self):
        cur = self.buf.numpy().copy()
        d = np.linalg.norm(cur - self.prev)
        n = np.linalg.norm(cur)
        self.prev = cur
        return d / n if n > 0 else 0.0


def _rank_device_plane_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        prob = _problem()
        dirs = sharding.direction_shards(len(prob.weight), world)[rank]
        sw = OracleBufferSweeper(prob, dirs)
        it, conv = sharding.source_iterate_device(sw, sharding.torch_allreduce_inplace(), rel_tol=1e-10,
                                                  max_iters=300)
        out.put((rank, sw.buf.numpy().copy(), it, conv))
    finally:
        dist.destroy_process_group()


def test_device_plane_sharded_iteration_matches_single_rank():
    """source_iterate_device (in-place all-reduce of each rank's PhiTotal
    buffer) over two gloo ranks gives the single-rank iteration."""
    prob = _problem()
    ref_phi, ref_it, ref_conv = sharding.source_iterate(OracleSweeper(prob, np.arange(len(prob.weight))), prob,
                                                        lambda x: x, q_ext=prob.q_ext, rel_tol=1e-10,
                                                        max_iters=300)
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_device_plane_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    for _ in procs:
        r, phi, it, conv = out.get(timeout=300)
        res[r] = (phi, it, conv)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert np.array_equal(res[0][0], res[1][0])
    assert res[0][2] and res[0][1] == ref_it
    got = res[0][0].reshape(ref_phi.shape)
    assert float(np.max(np.abs(got - ref_phi)) / np.max(np.abs(ref_phi))) < 1e-12
