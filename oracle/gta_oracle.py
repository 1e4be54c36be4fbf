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


# ---------------------------------------------------------------------------
# The reference's newer grey solver (Size%useNewGTASolver; driver option
# gta_kernel = 2, driver/test_driver.cc:1527-1530): the stretched-TSA sweep
# is replaced by a direct per-zone solve of the zone-local scattering.
#   * init_grey_tt      snac/InitSweepGreyUCBxyz.F90:10-253 (TT per zone)
#   * grey_sweep_new    snac/GTASweep.F90 (GTA%ID = 1) with
#                       snac/SweepGreyUCBxyz.F90 SweepGreyUCBxyzKernelNew:
#                       the sweep also accumulates PhiInc, the part of the
#                       scalar flux carried in by upwind flux
#   * zone_decompose /  snac/UpdateScalarIntensity.F90: A = I - TT wtiso
#     zone_solve        sigma_s per zone, LU in place, then L y = S, U x = y
#   * gta_correction_new  rt/GTASolver.F90:158-402 with GreySweepNEW
#                       (rt/GreySweep.F90:12-47)
# Written as literal loops (small meshes only).
# ---------------------------------------------------------------------------

def init_grey_tt(gp, gt_corner):
    """TT [nc, 8]: TT[c0+c, cc] = sum_a w_a d psi_a(c) / d TsaSource(cc) within
    the zone (TT(cc, c0+c) of the reference)."""
    m = gp.m
    nc = m.ncornr
    Afp = gp.geo[0].reshape(nc, 3, 3)
    Aez = gp.geo[1].reshape(nc, 3, 3)
    V = gp.geo[2]
    TT = np.zeros((nc, 8))
    for z in range(m.nzones):
        c0, nC = int(m.cOffSet[z]), int(m.numCorner[z])
        for a in range(len(gp.weight)):
            om, w = gp.omega[a], gp.weight[a]
            nxez = [[] for _ in range(nC)]
            need = [0] * nC
            Pvv = np.zeros((nC, nC))                  # Pvv[col, row] as the reference's Pvv(column,row)
            for c in range(nC):
                Pvv[c, c] = V[c0 + c]
            sig = [gt_corner[c0 + c] for c in range(nC)]
            denom = [0.0] * nC
            for c in range(nC):
                cc = c0 + c
                sigv = V[cc] * sig[c]
                denom[c] = sigv
                ncf = int(m.nCFaces[cc])
                afp = [float(om @ Afp[cc, f]) for f in range(ncf)]
                for f in range(ncf):
                    if afp[f] > 0.0:
                        denom[c] += afp[f]
                for f in range(ncf):
                    aez = float(om @ Aez[cc, f])
                    cez = int(m.cEZ[cc, f])
                    if cez > c:
                        if aez > 0.0:
                            need[cez] += 1
                            nxez[c].append((cez, aez))
                        elif aez < 0.0:
                            need[c] += 1
                            nxez[cez].append((c, -aez))
                    if aez > 0.0:
                        denom[c] += aez
                        area_opp = 0.0
                        if ncf == 3:
                            ifp = (f + 1) % ncf
                            if afp[ifp] < 0.0:
                                area_opp = -afp[ifp]
                        else:
                            ifp = f
                            for _ in range(ncf - 2):
                                ifp = (ifp + 1) % ncf
                                if afp[ifp] < 0.0:
                                    area_opp -= afp[ifp]
                        if area_opp > 0.0:
                            sigv2 = sigv * sigv
                            gnum = aez * aez * (1.82 * sigv2 + aez * (4.0 * sigv + 3.0 * aez))
                            gtau = gnum / (gnum + 4.0 * sigv2 * sigv2 +
                                           aez * sigv * (6.0 * sigv2 + 2.0 * aez * (2.0 * sigv + aez)))
                            B0 = 0.5 * aez * (1.0 - gtau)
                            B1 = (B0 - gtau * sigv) / sig[c]
                            B2 = B0 / sig[cez]
                        else:
                            B1 = 0.5 * aez / sig[c]
                            B2 = 0.5 * aez / sig[cez]
                        Pvv[c, c] += B1
                        Pvv[cez, c] -= B2
                        Pvv[c, cez] -= B1
                        Pvv[cez, cez] += B2
            for _ in range(nC):
                c = int(np.argmin(need))               # minloc: first index of the minimum
                dInv = 1.0 / denom[c]
                Pvv[:, c] *= dInv
                for cez, coef in nxez[c]:
                    need[cez] -= 1
                    Pvv[:, cez] += coef * Pvv[:, c]
                need[c] = 99
            for c1 in range(nC):
                for c in range(nC):
                    TT[c0 + c1, c] += w * Pvv[c, c1]
    return TT


def grey_sweep_new(gp, gt_corner, tsa):
    """(tPhi, PhiInc) [nc] of one grey S2 sweep with the corner source tsa
    (TsaSource, already times wtiso), vacuum boundaries."""
    m = gp.m
    nc, nb = m.ncornr, m.nbelem
    Afp = gp.geo[0].reshape(nc, 3, 3)
    Aez = gp.geo[1].reshape(nc, 3, 3)
    V = gp.geo[2]
    tphi = np.zeros(nc)
    phi_inc = np.zeros(nc)
    S = gp.S
    for a in range(len(gp.weight)):
        om, w = gp.omega[a], gp.weight[a]
        tpsi = np.zeros(nc + nb)
        pinc = np.zeros(nc)
        pos = 0
        for h in range(int(S.nHyperPlanes[a])):
            for ii in range(int(S.zonesInPlane[a][h])):
                zv = int(S.nextZ[a][pos + ii])
                z = zv if zv >= 0 else -zv - 1
                c0, nC = int(m.cOffSet[z]), int(m.numCorner[z])
                Q = [tsa[c0 + c] / gt_corner[c0 + c] for c in range(nC)]
                src = [V[c0 + c] * tsa[c0 + c] for c in range(nC)]
                nxez = [[] for _ in range(nC)]
                denom = [0.0] * nC
                for c in range(nC):
                    cc = c0 + c
                    sigv = V[cc] * gt_corner[cc]
                    denom[c] = sigv
                    ncf = int(m.nCFaces[cc])
                    afp = [float(om @ Afp[cc, f]) for f in range(ncf)]
                    psifp = [0.0] * ncf
                    for f in range(ncf):
                        if afp[f] > 0.0:
                            denom[c] += afp[f]
                        elif afp[f] < 0.0:
                            psifp[f] = tpsi[int(m.cFP[cc, f])]
                            src[c] -= afp[f] * psifp[f]
                            pinc[cc] -= afp[f] * psifp[f]
                    for f in range(ncf):
                        aez = float(om @ Aez[cc, f])
                        cez = int(m.cEZ[cc, f])
                        if cez > c:
                            if aez > 0.0:
                                nxez[c].append((cez, aez))
                            elif aez < 0.0:
                                nxez[cez].append((c, -aez))
                        if aez > 0.0:
                            psi_opp = 0.0
                            area_opp = 0.0
                            denom[c] += aez
                            ifp = (f + 1) % ncf
                            if afp[ifp] < 0.0:
                                area_opp = -afp[ifp]
                                psi_opp = -afp[ifp] * psifp[ifp]
                            for _ in range(ncf - 3):
                                ifp = (ifp + 1) % ncf
                                if afp[ifp] < 0.0:
                                    area_opp -= afp[ifp]
                                    psi_opp -= afp[ifp] * psifp[ifp]
                            if area_opp > 0.0:
                                psi_opp /= area_opp
                                sigv2 = sigv * sigv
                                gnum = aez * aez * (1.82 * sigv2 + aez * (4.0 * sigv + 3.0 * aez))
                                gtau = gnum / (gnum + 4.0 * sigv2 * sigv2 +
                                               aez * sigv * (6.0 * sigv2 + 2.0 * aez * (2.0 * sigv + aez)))
                                sez = gtau * sigv * (psi_opp - Q[c]) + 0.5 * aez * (1.0 - gtau) * (Q[c] - Q[cez])
                                src[c] += sez
                                src[cez] -= sez
                                pinc[c0 + c] += gtau * sigv * psi_opp
                                pinc[c0 + cez] -= gtau * sigv * psi_opp
                            else:
                                sez = 0.5 * aez * (Q[c] - Q[cez])
                                src[c] += sez
                                src[cez] -= sez
                for i in range(nC):
                    c = int(S.nextC[a][c0 + i])
                    tpsi[c0 + c] = src[c] / denom[c]
                    pinc[c0 + c] /= denom[c]
                    for cez, coef in nxez[c]:
                        src[cez] += coef * tpsi[c0 + c]
                        pinc[c0 + cez] += coef * pinc[c0 + c]
            pos += int(S.zonesInPlane[a][h])
        tphi += w * tpsi[:nc]
        phi_inc += w * pinc
    return tphi, phi_inc


def zone_decompose(m, TT, gs_corner, z):
    """A = I - TT diag(wtiso sigma_s) of zone z, LU in place (the reference's
    order); returns LU [nC, nC] with LU[i, j] = A[i][j] factors."""
    c0, nC = int(m.cOffSet[z]), int(m.numCorner[z])
    # T[col][row] as the reference's TT(col, c0+row)
    T = [[-WTISO * gs_corner[c0 + cc] * TT[c0 + c, cc] for c in range(nC)] for cc in range(nC)]
    for c in range(nC):
        T[c][c] = 1.0 + T[c][c]
    for i in range(nC):
        t = 0.0
        for k in range(i):
            t += T[k][i] * T[i][k]
        T[i][i] -= t
        diagInv = 1.0 / T[i][i]
        for j in range(i + 1, nC):
            t = 0.0
            v = 0.0
            for k in range(i):
                t += T[k][i] * T[j][k]
                v += T[k][j] * T[i][k]
            T[j][i] -= t
            T[i][j] = diagInv * (T[i][j] - v)
    return T


def zone_solve(T, phi):
    nC = len(phi)
    phi = list(phi)
    for j in range(1, nC):
        t = 0.0
        for i in range(j):
            t -= T[i][j] * phi[i]
        phi[j] += t
    phi[nC - 1] /= T[nC - 1][nC - 1]
    for k in range(nC - 2, -1, -1):
        t = 0.0
        for i in range(k + 1, nC):
            t += phi[i] * T[i][k]
        phi[k] = (phi[k] - t) / T[k][k]
    return phi


def gta_correction_new(m, sigt, sigs, tau, phi, prev, maxit=10, tol=1e-4):
    """(correction [nc], chi [nz, G], grey sweeps) of one GTA step with the
    newer solver."""
    gp = GreyProblem(m)
    vol = gp.geo[2]
    cz = m.cToZone
    chi, gt, gs = spectrum(m, vol, sigt, sigs, tau, phi, prev)
    gtc, gsc = gt[cz], gs[cz]
    R = (sigs[cz] * (phi - prev)).sum(1)
    svol = gsc * vol
    TT = init_grey_tt(gp, gtc)
    LU = [None] * m.nzones
    sweeps = [0]

    def M(P, with_source):
        p = P if P is not None else np.zeros(m.ncornr)
        src = WTISO * (gsc * p + (R if with_source else 0.0))
        _, phi_inc = grey_sweep_new(gp, gtc, src)
        sweeps[0] += 1
        out = np.zeros(m.ncornr)
        for z in range(m.nzones):
            c0, nC = int(m.cOffSet[z]), int(m.numCorner[z])
            rhs = [phi_inc[c0 + c] for c in range(nC)]
            if with_source:
                for c in range(nC):
                    for cc in range(nC):
                        rhs[c] += TT[c0 + c, cc] * WTISO * R[c0 + cc]
                LU[z] = zone_decompose(m, TT, gsc, z)
            out[c0:c0 + nC] = zone_solve(LU[z], rhs)
        return out

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
