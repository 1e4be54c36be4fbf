"""Product quadrature for 3-D xyz geometry.

Restates rt/quadProduct.F90:21-186 (ordinate construction per polar axis and
octant numbering) and the weight normalisation of rt/rtquad.F90:101-112
(sum of weights = 1/wtiso = 4*pi).  Directions are numbered consecutively
within an octant block of 8, exactly as Teton numbers them, so angle indices
are interchangeable with the reference's.
"""
from __future__ import annotations

import math
import numpy as np

from . import quadrature_data as Q

WTISO_XYZ = 1.0 / (4.0 * math.pi)      # mods/Size_mod.F90:281

# octant sign pattern (quadProduct.F90:126-178)
_OCT = np.array([[1, 1, 1], [-1, 1, 1], [-1, -1, 1], [1, -1, 1],
                 [1, 1, -1], [-1, 1, -1], [-1, -1, -1], [1, -1, -1]], np.float64)


def product_quadrature(npolar: int, nazimuthal: int, polaraxis: int = 1):
    """Return (omega[A,3], weight[A]) with A = 8*npolar*nazimuthal."""
    if not (1 <= npolar <= 32 and 1 <= nazimuthal <= 32 and 1 <= polaraxis <= 3):
        raise ValueError("npolar, nazimuthal must be in 1..32 and polaraxis in 1..3")
    phi1, phi2 = Q.first[nazimuthal - 1], Q.last[nazimuthal - 1]
    th1, th2 = Q.first[npolar - 1], Q.last[npolar - 1]
    ox, oy, oz, w = [], [], [], []
    for iphi in range(phi1, phi2 + 1):
        cphi = Q.cosPhiXYZ[iphi - 1]
        for jth in range(th2, th1 - 1, -1):
            ct = Q.cosTheta[jth - 1]
            st = math.sqrt(1.0 - ct * ct)
            if polaraxis == 1:
                x = ct; y = st * cphi; z = math.sqrt(1.0 - x * x - y * y)
            elif polaraxis == 2:
                y = ct; z = st * cphi; x = math.sqrt(1.0 - y * y - z * z)
            else:
                z = ct; x = st * cphi; y = math.sqrt(1.0 - x * x - z * z)
            ox.append(x); oy.append(y); oz.append(z)
            w.append(Q.weightTheta[jth - 1] * Q.weightPhiXYZ[iphi - 1])
    n = len(w)
    omega = np.zeros((8 * n, 3))
    weight = np.zeros(8 * n)
    for i in range(n):
        for o in range(8):
            omega[8 * i + o] = _OCT[o] * (ox[i], oy[i], oz[i])
            weight[8 * i + o] = w[i]
    s = 0.0
    for a in range(8 * n):
        s = s + weight[a]
    fac = 1.0 / (WTISO_XYZ * s)
    weight = fac * weight
    return omega, weight
