"""CPU restatement of the grey transport acceleration step (test
infrastructure only: the GPU tests use it as the checker of
umt103_gta_correction; nothing in the product imports it).

It restates, in numpy float64 with the oracle's C++ sweep (orc_set_sweep,
the restatement of snac/SweepUCBxyz.F90) as the grey S2 sweep:

* the grey opacities of rt/setGTAOpacity.F90:176-232 (spectrum-weighted
  harmonic means, greysigs floored to zero below a ratio of 1e-10, the
  stretched-TSA eps = 1/sqrt(1 - sigma_s/sigma_t) and opacity sigma_t/eps);
* the grey operator of rt/GreySweep.F90 (GreySweep: a grey S2 sweep of
  wtiso (sigma_s P + R), then a stretched sweep of wtiso sigma_s eps (P1 - P)
  added to it) with snac/GTASweep.F90's sources;
* the BiCGStab loop of rt/GTASolver.F90:219-402, inner products weighted by
  sigma_s V (rt/scat_prod.F90) and the shadow product their plain sum
  (rt/scat_prod1.F90), stopping on the zone-averaged correction change.

The spectrum chi, which the reference takes from its material-coupling
solver (not in the reference tree), is the library's own choice: per zone,
the shape of the scattering residual |sigma_s,g (phi_g - phi_g_prev)|
summed over the zone's corners (umt_gb300/csrc/si.cu, k_gta_spectrum); it is
restated here from that definition.
"""
from __future__ import annotations

import numpy as np

from . import pyoracle as po

WTISO = 1.0 / (4.0 * np.pi)


def s2_quadrature():
    """Level-symmetric S2: 8 directions (+-1, +-1, +-1)/sqrt(3), weights 4pi/8."""
    s = 0.57735026918962576451
    sg = [(1, 1, 1), (-1, 1, 1), (-1, -1, 1), (1, -1, 1), (1, 1, -1), (-1, 1, -1), (-1, -1, -1), (1, -1, -1)]
    omega = np.array(sg, dtype=np.float64) * s
    weight = np.full(8, 4.0 * np.pi / 8.0)
    return omega, weight


def spectrum(m, vol, sigt, sigs, tau, phi, prev):
    """chi [nz, G] and the grey sigma_t, sigma_s [nz] (k_gta_spectrum, mode 0)."""
    nz, G = sigt.shape
    chi = np.zeros((nz, G))
    gt = np.zeros(nz)
    gs = np.zeros(nz)
    for z in range(nz):
        c0, nC = m.cOffSet[z], m.numCorner[z]
        cs = slice(c0, c0 + nC)
        r = (vol[cs, None] * np.abs(sigs[z][None, :] * (phi[cs] - prev[cs]))).sum(0)
        rsum = r.sum()
        x = r / rsum if rsum > 0.0 else np.full(G, 1.0 / G)
        si = 1.0 / sigt[z]
        sa = sigt[z] - sigs[z] - tau
        inv = (x * si).sum()
        inv2 = (x * si * si).sum()
        aav = (x * sa * si).sum()
        chi[z] = x * si
        if inv > 0.0:
            chi[z] /= inv
            t = inv / inv2
            ga = tau + aav / inv
            s = t - ga
            if s / t <= 1.0e-10:
                s, t = 0.0, ga
        else:
            t, s = (tau if tau > 0.0 else 1.0), 0.0
        gt[z], gs[z] = t, s
    return chi, gt, gs


class GreyProblem:
    def __init__(self, m):
        self.m = m
        self.geo = po.geometry(m)
        self.omega, self.weight = s2_quadrature()
        self.S = po.schedule(m, self.geo[0], self.geo[1], self.omega)

    def sweep(self, sigt_zone, source_corner):
        m = self.m
        Psi = np.zeros((8, m.ncornr, 1))
        PsiB = np.zeros((8, m.nbelem, 1))
        Phi, _, _ = po.set_sweep(m, self.geo, self.S, np.ascontiguousarray(sigt_zone[:, None]),
                                 np.ascontiguousarray(source_corner[:, None]), 0.0, self.omega, self.weight,
                                 Psi, PsiB)
        return Phi[:, 0]


def gta_correction(m, sigt, sigs, tau, phi, prev, maxit=10, tol=1e-4):
    """(correction [nc], chi [nz, G], grey sweeps) of one GTA step."""
    gp = GreyProblem(m)
    vol = gp.geo[2]
    cz = m.cToZone
    chi, gt, gs = spectrum(m, vol, sigt, sigs, tau, phi, prev)
    eps = 1.0 / np.sqrt(1.0 - gs / gt)
    gt2 = gt / eps
    R = (sigs[cz] * (phi - prev)).sum(1)
    svol = gs[cz] * vol
    sweeps = [0]

    def M(P, with_source):
        src = WTISO * (gs[cz] * (P if P is not None else 0.0) + (R if with_source else 0.0))
        p1 = gp.sweep(gt, src)
        p0 = P if P is not None else 0.0
        p2 = gp.sweep(gt2, WTISO * gs[cz] * eps[cz] * (p1 - p0))
        sweeps[0] += 2
        return p1 + p2

    vz = np.zeros(m.nzones)
    np.add.at(vz, cz, vol)
    radE = np.zeros(m.nzones)
    np.add.at(radE, cz, vol * phi.sum(1))
    radE /= vz
    pzOld = np.zeros(m.nzones)
    small = 1.0e-150
    x = np.zeros(m.ncornr)
    r = M(None, True)
    d = r.copy()
    rrOld = (r * svol).sum()
    nGrey = 1
    it = 0
    while True:
        if abs(rrOld) < small:
            if nGrey <= 2:
                x = r.copy()
            break
        nGrey += 2
        Ad = d - M(d, False)
        dAd = (Ad * svol).sum()
        if abs(dAd) < small:
            break
        alpha = rrOld / dAd
        r = r - alpha * Ad
        As = r - M(r, False)
        num, den = (As * r * svol).sum(), (As * As * svol).sum()
        if abs(den) < small or abs(num) < small:
            x = x + alpha * d
            break
        omega = num / den
        x = x + alpha * d + omega * r
        r = r - omega * As
        rr = (r * svol).sum()
        beta = (rr * alpha) / (rrOld * omega)
        d = r + beta * (d - omega * Ad)
        pz = np.zeros(m.nzones)
        np.add.at(pz, cz, vol * x)
        pz /= vz
        err = pz - pzOld
        phiNew = radE + pz
        l2 = np.sqrt(abs((vz * err * err).sum() / (vz * phiNew * phiNew).sum()))
        pt = np.max(np.abs(err[phiNew != 0] / phiNew[phiNew != 0])) if np.any(phiNew != 0) else 0.0
        pzOld = pz
        it += 1
        if max(pt, l2) < tol or it >= maxit:
            break
        rrOld = rr
    return x, chi, sweeps[0]
