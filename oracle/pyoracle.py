"""ctypes bindings to the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs import
this module; the product never does.
"""
from __future__ import annotations

import ctypes as C
import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(_build.build())
        for name in ("orc_geometry", "orc_schedule", "orc_sweep_angle", "orc_set_sweep", "orc_geometry_rz",
                     "orc_set_sweep_rz"):
            getattr(_lib, name).restype = C.c_int
        _lib.orc_planck_groups.restype = None
    return _lib


def _p(a, dtype):
    assert a.dtype == dtype and a.flags.c_contiguous, (a.dtype, a.flags)
    return a.ctypes.data_as(C.c_void_p)


def _i(a):
    return _p(a, np.int32)


def _d(a):
    return _p(a, np.float64)


def geometry(m):
    """orc_geometry: A_fp, A_ez [nc,3,3], Volume [nc], VolumeZone [nz], A_bdy [nb,3]."""
    nc, nz, nb = m.ncornr, m.nzones, m.nbelem
    A_fp = np.zeros((nc, 3, 3)); A_ez = np.zeros((nc, 3, 3))
    vol = np.zeros(nc); volz = np.zeros(nz); A_bdy = np.zeros((nb, 3))
    rc = lib().orc_geometry(nz, nc, nb, 3, m.zoneOpp.shape[1], _i(m.numCorner), _i(m.cOffSet),
                            _i(m.zoneFaces), _i(m.zoneOpp), _i(m.nCFaces), _i(m.cFP), _i(m.cEZ),
                            _i(m.CToFace), _d(m.px), _d(A_fp), _d(A_ez), _d(vol), _d(volz), _d(A_bdy))
    assert rc == 0
    return A_fp, A_ez, vol, volz, A_bdy


class Schedule:
    """Per-angle sweep schedules packed like the C-ABI's device schedule."""

    def __init__(self, nz, nc, A):
        self.nextZ = np.zeros((A, nz), np.int32)
        self.nextC = np.zeros((A, nc), np.int32)
        self.zonesInPlane = np.zeros((A, nz), np.int32)
        self.nHyperPlanes = np.zeros(A, np.int32)
        self.numCycles = np.zeros(A, np.int32)
        self.cycleOffSet = np.zeros(A, np.int32)
        self.cycleList = np.zeros(0, np.int32)


def schedule(m, A_fp, A_ez, omega):
    """Per-direction schedules; the number of corner faces per corner is taken
    from the mesh (3 for the 3-D meshes, 2 for RZ)."""
    maxcf = int(m.cFP.shape[1])
    A = omega.shape[0]
    nz, nc = m.nzones, m.ncornr
    S = Schedule(nz, nc, A)
    cyc = []
    off = 0
    for a in range(A):
        cl = np.zeros(nc + 1, np.int32)
        ncyc = np.zeros(1, np.int32)
        om = np.ascontiguousarray(omega[a], np.float64)
        nzr = np.ascontiguousarray(S.nextZ[a]); ncr = np.ascontiguousarray(S.nextC[a])
        zip_ = np.ascontiguousarray(S.zonesInPlane[a])
        nh = lib().orc_schedule(nz, nc, maxcf, m.zoneOpp.shape[1], _i(m.numCorner), _i(m.cOffSet),
                                _i(m.zoneFaces), _i(m.zoneOpp), _i(m.faceOpp), _i(m.nCFaces),
                                _i(m.CToFace), _i(m.cEZ), _d(A_fp), _d(A_ez), _d(om),
                                _i(nzr), _i(ncr), _i(zip_), _i(cl), _i(ncyc))
        if nh <= 0:
            raise RuntimeError(f"orc_schedule failed for angle {a}: {nh}")
        S.nextZ[a] = nzr; S.nextC[a] = ncr; S.zonesInPlane[a] = zip_
        S.nHyperPlanes[a] = nh
        S.numCycles[a] = ncyc[0]
        S.cycleOffSet[a] = off
        off += int(ncyc[0])
        cyc.append(cl[:ncyc[0]])
    S.cycleList = np.ascontiguousarray(np.concatenate(cyc) if cyc else np.zeros(0, np.int32), np.int32)
    return S


def set_sweep(m, geo, S, Sigt, STotal, tau, omega, weight, Psi, PsiB, Psi1=None,
              cyclePsi=None, savePsi=False, nthreads=1):
    """orc_set_sweep over all angles; returns (Phi, Psi1, cyclePsi). Psi/PsiB updated in place."""
    A_fp, A_ez, vol = geo[0], geo[1], geo[2]
    A, nc, G = Psi.shape
    nb = m.nbelem
    if Psi1 is None:
        Psi1 = np.zeros((nc + nb, G))
    if cyclePsi is None:
        cyclePsi = np.zeros((max(len(S.cycleList), 1), G))
    Phi = np.zeros((nc, G))
    rc = lib().orc_set_sweep(m.nzones, nc, nb, 3, G, A, _i(m.numCorner), _i(m.cOffSet),
                             _i(m.nCFaces), _i(m.cFP), _i(m.cEZ), _d(A_fp), _d(A_ez), _d(vol),
                             _d(Sigt), _d(STotal), C.c_double(tau), _d(omega), _d(weight),
                             _i(S.nHyperPlanes), _i(S.zonesInPlane), _i(S.nextZ), _i(S.nextC),
                             _i(S.numCycles), _i(S.cycleOffSet), _i(S.cycleList), _d(cyclePsi),
                             _d(Psi1), _d(Phi), _d(PsiB), _d(Psi), int(savePsi), int(nthreads))
    if rc != 0:
        raise RuntimeError(f"orc_set_sweep failed: {rc}")
    return Phi, Psi1, cyclePsi


def planck_groups(T, k, Bnorm, gnu):
    gnu = np.ascontiguousarray(gnu, np.float64)
    B = np.zeros(len(gnu) - 1)
    lib().orc_planck_groups(C.c_double(T), C.c_double(k), C.c_double(Bnorm), len(B), _d(gnu), _d(B))
    return B


def geometry_rz(m):
    """orc_geometry_rz: A_fp, A_ez [nc,2,3] (third component 0), Area, Volume [nc],
    RadiusFP, RadiusEZ [nc,2], A_bdy [nb,3]."""
    nc = m.ncornr
    A_fp = np.zeros((nc, 2, 3)); A_ez = np.zeros((nc, 2, 3))
    area = np.zeros(nc); vol = np.zeros(nc); rfp = np.zeros((nc, 2)); rez = np.zeros((nc, 2))
    px = np.ascontiguousarray(m.px, np.float64)
    rc = lib().orc_geometry_rz(m.nzones, nc, _i(m.numCorner), _i(m.cOffSet), _i(m.cEZ), _i(m.cFP), _d(px),
                               _d(A_fp), _d(A_ez), _d(area), _d(vol), _d(rfp), _d(rez))
    assert rc == 0
    A_bdy = np.zeros((m.nbelem, 3))
    for cc in range(nc):
        for f in range(2):
            v = int(m.cFP[cc, f])
            if v >= nc:
                A_bdy[v - nc] = A_fp[cc, f]
    return dict(A_fp=A_fp, A_ez=A_ez, Area=area, Volume=vol, RadiusFP=rfp, RadiusEZ=rez, A_bdy=A_bdy)


def set_sweep_rz(m, geo, S, Sigt, STotal, tau, omega3, q, Psi, PsiB, savePsi=False):
    """orc_set_sweep_rz over all directions; returns Phi.  Psi/PsiB updated in place."""
    A, nc, G = Psi.shape
    Phi = np.zeros((nc, G))
    i32 = lambda x: np.ascontiguousarray(x, np.int32)
    d64 = lambda x: np.ascontiguousarray(x, np.float64)
    rc = lib().orc_set_sweep_rz(
        m.nzones, nc, m.nbelem, G, A, _i(m.numCorner), _i(m.cOffSet), _i(m.cFP), _i(m.cEZ),
        _d(geo["A_fp"]), _d(geo["A_ez"]), _d(geo["Area"]), _d(geo["Volume"]), _d(geo["RadiusFP"]),
        _d(geo["RadiusEZ"]), _d(d64(Sigt)), _d(d64(STotal)), C.c_double(tau), _d(d64(omega3)),
        _d(d64(q.weight)), _d(d64(q.angDerivFac)), _d(d64(q.quadTauW1)), _d(d64(q.quadTauW2)),
        _i(i32(q.starting)), _i(i32(q.finishing)), _i(S.nHyperPlanes), _i(S.zonesInPlane), _i(S.nextZ),
        _i(S.nextC), _d(geo["A_bdy"]), _i(m.bdyToC), _d(Phi), _d(PsiB), _d(Psi), int(savePsi))
    if rc != 0:
        raise RuntimeError(f"orc_set_sweep_rz failed: {rc}")
    return Phi
