"""Angle-set sharding of the sweep across ranks, one GPU per rank.

On one spatial domain every direction's sweep is independent; the directions
couple only through the scalar flux: the tally PhiTotal = sum_a w_a psi_a, the
scattering source built from it, and the convergence test.  Teton expresses
this with MPI all-reduces of the flux (snac/SetSweep.F90:199,
rt/scat_prod.F90:81).  Here each rank owns a contiguous block of the
quadrature's directions in its own library context, sweeps them, and one
sum all-reduce of PhiTotal (nc x G, FP64) per source iteration gives every
rank the full flux; the energy edits' boundary powers are all-reduced the
same way.

The collective is passed in as a callable, so the same host logic runs over
NCCL between GPUs (torch.distributed with device tensors) or over gloo on
host tensors.

Two data planes: `LibrarySweeper` + `source_iterate` move PhiTotal through
the host each iteration (any collective, any device count); `DeviceSweeper`
+ `source_iterate_device` keep it on the GPU: the library builds the
scattering source from PhiTotal on the device and sweeps (umt103_si_step),
the collective sums the library's own PhiTotal buffer in place (a torch
view of umt103_phi_device, no copy), and the change norm is taken on the
device (umt103_si_change).
"""
from __future__ import annotations

from typing import Callable, Optional

import numpy as np

FOUR_PI = 4.0 * np.pi


def direction_shards(A: int, world: int) -> list[np.ndarray]:
    """Contiguous blocks of the A directions, sizes differing by at most one."""
    if world < 1 or A < world:
        raise ValueError(f"cannot split {A} directions over {world} ranks")
    bounds = np.linspace(0, A, world + 1).round().astype(int)
    return [np.arange(bounds[r], bounds[r + 1]) for r in range(world)]


def torch_allreduce(group=None, device=None) -> Callable[[np.ndarray], np.ndarray]:
    """Sum all-reduce of an FP64 array with torch.distributed (NCCL when the
    process group lives on GPUs, then pass device='cuda'; gloo on host)."""
    import torch
    import torch.distributed as dist

    def reduce(x: np.ndarray) -> np.ndarray:
        t = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64))
        if device is not None:
            t = t.to(device)
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        return t.cpu().numpy()

    return reduce


class LibrarySweeper:
    """This rank's directions, resident on this rank's GPU through the C-ABI."""

    def __init__(self, lib, prob, directions: np.ndarray, precision: int, flags: int = 8):
        from . import capi
        self.lib, self.prob, self.dirs = lib, prob, np.asarray(directions)
        self.precision = precision
        m = prob.mesh
        need = capi.UMT_FP32 if precision == capi.UMT_FP32 else capi.UMT_FP64
        lib.init(m, prob.omega[self.dirs], prob.weight[self.dirs], prob.ngr,
                 flags=flags | (2 if need == capi.UMT_FP32 else 1))
        lib.set_materials(prob.sigt, prob.sigs, prob.tau)
        if prob.psi0 is not None:
            lib.set_psi(prob.psi0[self.dirs], None)

    def sweep(self, STotal: np.ndarray, savePsi: bool = False) -> np.ndarray:
        """PhiTotal summed over this rank's directions only."""
        return self.lib.sweep(STotal, savePsi=savePsi, precision=self.precision)


def scattering_source(prob, phi: np.ndarray, q_ext: Optional[np.ndarray]) -> np.ndarray:
    """STotal = (sigma_s phi + q) / (4 pi) per corner (isotropic scattering)."""
    m = prob.mesh
    s = prob.sigs[m.cToZone] * phi
    if q_ext is not None:
        s = s + q_ext[m.cToZone]
    return s / FOUR_PI


def tally(lib, allreduce: Callable[[np.ndarray], np.ndarray], siga=None, precision=None) -> dict:
    """Energy edits of a sharded sweep: every edit is a sum over directions
    (or linear in PhiTotal, which each rank holds for its own directions), so
    the rank-local edits are summed."""
    t = lib.tally(siga, precision=precision)
    keys = ("EnergyRadiation", "PowerEscape", "PowerIncident", "PowerAbsorbed")
    tot = allreduce(np.array([t[k] for k in keys], np.float64))
    return dict(zip(keys, (float(v) for v in tot)))


def source_iterate(sweeper, prob, allreduce: Callable[[np.ndarray], np.ndarray], q_ext=None,
                   rel_tol: float = 1e-8, max_iters: int = 200):
    """Source iteration with the directions sharded over ranks (rt/rtmainsn.F90
    outer loop): every rank sweeps its directions, one all-reduce forms the
    full PhiTotal, every rank tests convergence on the same vector.

    Returns (PhiTotal, iterations, converged)."""
    m = prob.mesh
    phi = np.zeros((m.ncornr, prob.ngr))
    for it in range(1, max_iters + 1):
        partial = sweeper.sweep(scattering_source(prob, phi, q_ext))
        new = allreduce(partial)
        norm = np.linalg.norm(new)
        rel = np.linalg.norm(new - phi) / norm if norm > 0 else 0.0
        phi = new
        if rel < rel_tol:
            return phi, it, True
    return phi, max_iters, False


class CudaBuffer:
    """A library-owned device buffer of FP64 values, exposed through the CUDA
    array interface so that torch (or any consumer of the interface) can view
    it without copying."""

    def __init__(self, ptr: int, count: int):
        self.__cuda_array_interface__ = {"shape": (int(count),), "typestr": "<f8", "data": (int(ptr), False),
                                         "version": 3, "strides": None}


def torch_allreduce_inplace(group=None):
    """In-place sum all-reduce of a tensor (NCCL for CUDA tensors, gloo for
    host tensors)."""
    import torch.distributed as dist

    def reduce(t):
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        return t

    return reduce


class DeviceSweeper:
    """This rank's directions with PhiTotal kept on this rank's GPU."""

    def __init__(self, lib, prob, directions: np.ndarray, precision: int, flags: int = 8):
        from . import capi
        self.lib, self.prob, self.dirs, self.precision = lib, prob, np.asarray(directions), precision
        m = prob.mesh
        need = 2 if precision == capi.UMT_FP32 else 1
        lib.init(m, prob.omega[self.dirs], prob.weight[self.dirs], prob.ngr, flags=flags | need)
        lib.set_materials(prob.sigt, prob.sigs, prob.tau)
        if prob.psi0 is not None:
            lib.set_psi(prob.psi0[self.dirs], None)
        lib.set_external_source(prob.q_ext)

    def phi_tensor(self):
        import torch
        return torch.as_tensor(CudaBuffer(*self.lib.phi_device()), device="cuda")

    def step(self):
        self.lib.si_step(self.precision)

    def change(self) -> float:
        return self.lib.si_change()


def source_iterate_device(sweeper, allreduce_inplace, rel_tol: float = 1e-8, max_iters: int = 200):
    """Source iteration with the directions sharded over ranks and PhiTotal
    on the device: step (source + sweep of this rank's directions), sum
    PhiTotal over ranks in place, change norm.  Returns (iterations,
    converged); the full PhiTotal is left in sweeper.phi_tensor()."""
    import torch
    phi = sweeper.phi_tensor()
    sync = torch.cuda.synchronize if phi.is_cuda else (lambda: None)
    phi.zero_()
    sync()                                         # torch's stream before the library's
    sweeper.change()                               # previous iterate := 0
    for it in range(1, max_iters + 1):
        sweeper.step()                             # returns with the library's stream drained
        allreduce_inplace(phi)
        sync()
        if sweeper.change() < rel_tol:
            return it, True
    return max_iters, False
