"""Shared set-up for the parity tests: run the oracle on a problem."""
import numpy as np

from oracle import pyoracle as po


def oracle_sweep(prob, savePsi=True, STotal=None, Psi=None, PsiB=None, nthreads=1):
    m = prob.mesh
    geo = po.geometry(m)
    S = po.schedule(m, geo[0], geo[1], prob.omega)
    A, G = len(prob.weight), prob.ngr
    Psi = np.zeros((A, m.ncornr, G)) if Psi is None else Psi.copy()
    PsiB = np.zeros((A, m.nbelem, G)) if PsiB is None else PsiB.copy()
    STotal = np.zeros((m.ncornr, G)) if STotal is None else np.ascontiguousarray(STotal)
    sigt = np.ascontiguousarray(prob.sigt)
    Phi, Psi1, _ = po.set_sweep(m, geo, S, sigt, STotal, prob.tau, prob.omega, prob.weight,
                                Psi, PsiB, savePsi=savePsi, nthreads=nthreads)
    return dict(Phi=Phi, Psi=Psi, PsiB=PsiB, geo=geo, sched=S)


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
