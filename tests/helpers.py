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


def oracle_cycles(prob, ncycles):
    """The mini-app cycle (radtr: 2 sweeps + savePsi sweep, rtedit) on the oracle."""
    from umt_gb300.problems import SPEED_LIGHT
    m = prob.mesh
    geo = po.geometry(m)
    S = po.schedule(m, geo[0], geo[1], prob.omega)
    A, G = len(prob.weight), prob.ngr
    Psi = prob.psi0.copy()
    PsiB = np.zeros((A, m.nbelem, G))
    STotal = np.zeros((m.ncornr, G))
    sigt = np.ascontiguousarray(prob.sigt)
    vol, A_bdy = geo[2], geo[4]
    phi_tot = np.einsum("a,acg->cg", prob.weight, Psi)
    out = []
    for _ in range(ncycles):
        erad_boc = (vol[:, None] * phi_tot).sum() / SPEED_LIGHT
        for save in (False, False, True):
            phi_tot, _, _ = po.set_sweep(m, geo, S, sigt, STotal, prob.tau, prob.omega, prob.weight,
                                         Psi, PsiB, savePsi=save)
        erad = (vol[:, None] * phi_tot).sum() / SPEED_LIGHT
        pabs = (vol[:, None] * phi_tot * prob.siga[m.cToZone]).sum()
        pesc = 0.0
        for a in range(A):
            d = A_bdy @ prob.omega[a]
            sel = d > 0
            pesc += prob.weight[a] * (d[sel] * Psi[a][m.bdyToC[sel]].sum(1)).sum()
        out.append(dict(PhiTotal=phi_tot.copy(), EnergyRadiation=erad, PowerEscape=pesc, PowerAbsorbed=pabs,
                        EnergyCheck=prob.dt * (-pesc) - (erad - erad_boc),
                        EnergyCheckClosed=prob.dt * (-pesc - pabs) - (erad - erad_boc)))
    return out
