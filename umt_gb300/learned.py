"""Training driver of the learned source-iteration correction.

The network and its forward, backward and Adam kernels live in the CUDA
library (umt_gb300/csrc/learn.cu, umt103_mlp_*); this module drives them:

* `converged_phi` solves a problem's scattering equation to a tight
  tolerance with the library's FP64 sweep as the operator: PhiTotal is the
  fixed point of T(phi) = sweep(STotal(phi)), STotal = (sigma_s phi + q)/4pi
  (source iteration's map), found by restarted GMRES on (I - K) phi = T(0)
  with K phi = T(phi) - T(0).  Every application of K is one FP64 sweep.
* `collect` runs plain FP64 source iteration from zero and stores the zone
  features at chosen iterations (umt103_mlp_collect); once the converged
  PhiTotal is known, `umt103_mlp_set_targets` turns the stored iterates into
  targets (converged minus current, per zone and group).
* `train_on_problems` does both for a list of seeded problems and then runs
  Adam on the device (umt103_mlp_train).

No counterpart in the reference: Teton accelerates source iteration only
with grey transport (rt/GTASolver.F90).
"""
from __future__ import annotations

import time

import numpy as np

from . import capi
from .quadrature import WTISO_XYZ


def strongly_scattering_problem(tiles, seed, G=32, P=4, Az=4):
    """The strongly scattering distribution (total opacity log-uniform on
    [1, 1e3] per zone and group, scattering ratio uniform on [0.95, 0.999],
    q = 1, tau = 1/(c dt)) on `tiles` tiles per axis."""
    from .problems import synthetic_problem
    t = tiles if isinstance(tiles, tuple) else (tiles,) * 3
    return synthetic_problem(t, P, Az, G, seed=seed, sigt_range=(1.0, 1e3), c_range=(0.95, 0.999), q=1.0,
                             time_dependent=True)


def load_problem(lib, prob, flags=1 | 8):
    lib.init(prob.mesh, prob.omega, prob.weight, prob.ngr, flags=flags)
    lib.set_materials(prob.sigt, prob.sigs, prob.tau)
    lib.set_psi(prob.psi0, None)


def _source(prob, phi):
    m = prob.mesh
    return WTISO_XYZ * (prob.sigs[m.cToZone] * phi + prob.q_ext[m.cToZone])


def converged_phi(lib, prob, tol=1e-10, restart=60, max_sweeps=4000, precision=capi.UMT_FP64):
    """PhiTotal of the loaded problem solved to a relative residual `tol`
    (restarted GMRES, one sweep per operator application).  Returns
    (phi, sweeps)."""
    m = prob.mesh
    shape = (m.ncornr, prob.ngr)

    def T(phi):
        lib.set_source(_source(prob, phi))
        lib.sweep_resident(False, precision)
        return lib.get_phi(m.ncornr, prob.ngr)

    b = T(np.zeros(shape)).ravel()
    sweeps = 1

    def A(x):
        nonlocal sweeps
        sweeps += 1
        return x - (T(x.reshape(shape)).ravel() - b)

    x = b.copy()                                   # one source iteration from zero
    bn = np.linalg.norm(b)
    while sweeps < max_sweeps:
        r = b - A(x)
        beta = np.linalg.norm(r)
        if beta <= tol * bn:
            break
        V = np.zeros((restart + 1, b.size))
        Hm = np.zeros((restart + 1, restart))
        V[0] = r / beta
        g = np.zeros(restart + 1)
        g[0] = beta
        cs, sn = np.zeros(restart), np.zeros(restart)
        k_used = 0
        for k in range(restart):
            wv = A(V[k])
            for j in range(k + 1):
                Hm[j, k] = V[j] @ wv
                wv -= Hm[j, k] * V[j]
            Hm[k + 1, k] = np.linalg.norm(wv)
            if Hm[k + 1, k] > 0:
                V[k + 1] = wv / Hm[k + 1, k]
            for j in range(k):
                t = cs[j] * Hm[j, k] + sn[j] * Hm[j + 1, k]
                Hm[j + 1, k] = -sn[j] * Hm[j, k] + cs[j] * Hm[j + 1, k]
                Hm[j, k] = t
            den = np.hypot(Hm[k, k], Hm[k + 1, k])
            cs[k], sn[k] = Hm[k, k] / den, Hm[k + 1, k] / den
            Hm[k, k] = den
            Hm[k + 1, k] = 0.0
            g[k + 1] = -sn[k] * g[k]
            g[k] = cs[k] * g[k]
            k_used = k + 1
            if abs(g[k + 1]) <= tol * bn or sweeps >= max_sweeps:
                break
        y = np.linalg.solve(np.triu(Hm[:k_used, :k_used]), g[:k_used])
        x = x + V[:k_used].T @ y
    return x.reshape(shape), sweeps


def collect(lib, prob, iterations=(3, 5, 8, 12, 18, 26), precision=capi.UMT_FP64):
    """Plain source iteration from zero; the zone features of the iterate at
    each listed iteration go into the training set.  Returns rows added."""
    rows, done = 0, 0
    for k in iterations:
        lib.source_iterate(precision=precision, max_iters=k - done, rel_tol=0.0, q_ext=prob.q_ext,
                           save_psi=False, allow_notconv=True, warm_start=done > 0)
        done = k
        rows += lib.mlp_collect()
    return rows


def train_on_problems(lib, problems, steps=1500, batch=4096, lr=2e-3, seed=0, log=None):
    """Generate training data from each problem (FP64 sweeps) and train the
    library's network on it.  Returns a summary dict."""
    G = problems[0].ngr
    lib.mlp_init(G, seed)
    t0 = time.perf_counter()
    sweeps = 0
    for prob in problems:
        load_problem(lib, prob)
        phi_star, n = converged_phi(lib, prob)
        sweeps += n
        collect(lib, prob)
        lib.mlp_set_targets(phi_star)
        if log:
            log(f"problem {prob.name}: converged in {n} FP64 sweeps")
    t_data = time.perf_counter() - t0
    t1 = time.perf_counter()
    loss = lib.mlp_train(steps, batch, lr)
    t_train = time.perf_counter() - t1
    return {"problems": len(problems), "rows": lib.mlp_rows(), "fp64_sweeps": sweeps, "data_s": t_data,
            "train_s": t_train, "steps": steps, "batch": batch, "loss_first": loss[0], "loss_last": loss[1]}


def iterate_to(lib, prob, phi_ref, target=1e-6, precision=capi.UMT_FP32, learn_every=0, learn_start=3,
               max_iters=5000, use_gta=False):
    """Source iteration from zero until PhiTotal is within `target` relative
    L2 of phi_ref (checked on the device after every iteration).  Returns
    the result dict of umt103_source_iterate plus the host wall time."""
    t0 = time.perf_counter()
    r = lib.source_iterate(precision=precision, max_iters=max_iters, rel_tol=target, q_ext=prob.q_ext,
                           save_psi=False, allow_notconv=True, learn_every=learn_every, learn_start=learn_start,
                           phi_ref=phi_ref, use_gta=use_gta)
    r["wall_s"] = time.perf_counter() - t0
    r["error"] = float(np.linalg.norm(lib.get_phi(prob.mesh.ncornr, prob.ngr) - phi_ref) / np.linalg.norm(phi_ref))
    return r
