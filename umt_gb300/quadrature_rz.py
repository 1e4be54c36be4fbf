"""RZ product quadrature and its angular-derivative coefficients.

Restates, for Teton's 2-D cylindrical (RZ) geometry:
  * rt/quadrz.F90:127-219 (product branch): per polar cosine xi (from the
    product tables), a level with xi < 0 and one with xi > 0; each level is a
    zero-weight starting direction (mu = -sqrt(1 - xi^2)), the azimuthal
    directions in increasing mu, and a zero-weight finishing direction;
  * rt/rtquad.F90:101-126: weights scaled so that sum w = 1/wtiso = 2 pi
    (mods/Size_mod.F90:278), and the starting / finishing flags from the
    zero weights;
  * rt/AngleCoef2D.F90: alpha and tau of every direction of a level;
  * mods/AngleSet_mod.F90:335-346: angDerivFac, quadTauW1, quadTauW2.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import quadrature_data as Q

WTISO_RZ = 1.0 / (2.0 * math.pi)
ADQT_EPSILON = np.finfo(np.float64).eps


@dataclass
class QuadRZ:
    omega: np.ndarray        # [A, 2] (mu, xi)
    weight: np.ndarray       # [A]
    starting: np.ndarray     # [A] bool
    finishing: np.ndarray    # [A] bool
    level: np.ndarray        # [A] level (bin) of each direction
    alpha: np.ndarray
    tau: np.ndarray
    angDerivFac: np.ndarray
    quadTauW1: np.ndarray
    quadTauW2: np.ndarray


def product_quadrature_rz(npolar: int, nazimuthal: int) -> QuadRZ:
    if not (1 <= npolar <= 32 and 1 <= nazimuthal <= 32):
        raise ValueError("npolar and nazimuthal must be in 1..32")
    th1, th2 = Q.first[npolar - 1], Q.last[npolar - 1]
    ph1, ph2 = Q.first[nazimuthal - 1], Q.last[nazimuthal - 1]
    om, w = [], []
    for jth in range(th2, th1 - 1, -1):
        xi = Q.cosTheta[jth - 1]
        st = math.sqrt(1.0 - xi * xi)
        wt = Q.weightTheta[jth - 1]
        for sgn in (-1.0, 1.0):
            om.append((-math.sqrt(1.0 - xi * xi), sgn * xi)); w.append(0.0)
            for iph in range(ph2, ph1 - 1, -1):
                om.append((-st * Q.cosPhiRZ[iph - 1], sgn * xi)); w.append(wt * Q.weightPhiRZ[iph - 1])
            for iph in range(ph1, ph2 + 1):
                om.append((st * Q.cosPhiRZ[iph - 1], sgn * xi)); w.append(wt * Q.weightPhiRZ[iph - 1])
            om.append((math.sqrt(1.0 - xi * xi), sgn * xi)); w.append(0.0)
    omega = np.array(om)
    weight = np.array(w)
    weight *= 1.0 / (WTISO_RZ * weight.sum())
    A = len(weight)
    starting = np.zeros(A, bool)
    finishing = np.zeros(A, bool)
    iang = -1
    for a in range(A):
        if weight[a] < ADQT_EPSILON:
            if iang == -1:
                starting[a] = True
            else:
                finishing[a] = True
            iang = -iang
    level = np.cumsum(starting) - 1
    alpha = np.zeros(A)
    tau = np.zeros(A)
    for lev in range(level.max() + 1):
        idx = np.nonzero(level == lev)[0]
        wl = weight[idx].sum()
        phimh, mumh = math.pi, omega[0, 0]
        for a in idx:
            if starting[a]:
                alpha[a] = 0.0; tau[a] = 0.0
                phimh, mumh = math.pi, omega[a, 0]
            elif finishing[a]:
                alpha[a] = 0.0; tau[a] = 0.0
            else:
                alpha[a] = alpha[a - 1] - weight[a] * omega[a, 0]
                phiph = phimh - weight[a] * math.pi / wl
                muph = math.sqrt(1.0 - omega[a, 1] * omega[a, 1]) * math.cos(phiph)
                if omega[a, 0] < mumh or omega[a, 0] > muph:
                    raise ValueError("mu not between the cell-edge limits (AngleCoef2D)")
                tau[a] = (omega[a, 0] - mumh) / (muph - mumh)
                phimh, mumh = phiph, muph
    sf = starting | finishing
    with np.errstate(divide="ignore", invalid="ignore"):
        adf = np.where(sf, 0.0, omega[:, 0] + alpha / (weight * tau))
        w1 = np.where(sf, 1.0, 1.0 / tau)
        w2 = np.where(sf, 0.0, (1.0 - tau) / tau)
    return QuadRZ(omega, weight, starting, finishing, level.astype(np.int32), alpha, tau, adf, w1, w2)
