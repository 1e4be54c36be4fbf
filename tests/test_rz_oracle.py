"""The RZ restatements on the CPU: mesh, geometry (rt/geometryUCBrz.F90),
quadrature (rt/quadrz.F90, rt/rtquad.F90, rt/AngleCoef2D.F90) and the
oracle's RZ sweep."""
import math

import numpy as np
import pytest

from oracle import pyoracle as po
from umt_gb300.mesh_rz import build_rz_mesh
from umt_gb300.quadrature_rz import product_quadrature_rz, WTISO_RZ


@pytest.mark.parametrize("distort", [0.0, 0.2])
def test_rz_geometry_invariants(distort):
    m = build_rz_mesh(5, 4, distort=distort, seed=3)
    geo = po.geometry_rz(m)
    nz = m.nzones
    for z in range(nz):
        p = m.px[4 * z:4 * z + 4]
        shoelace = 0.5 * abs(np.dot(p[:, 0], np.roll(p[:, 1], -1)) - np.dot(p[:, 1], np.roll(p[:, 0], -1)))
        assert abs(geo["Area"][4 * z:4 * z + 4].sum() - shoelace) < 1e-14
        # the corner volumes are r-weighted areas: between r_min*area and r_max*area
        assert p[:, 0].min() * shoelace <= geo["Volume"][4 * z:4 * z + 4].sum() <= p[:, 0].max() * shoelace
    # face vectors: EZ and FP faces shared by two corners are exact negations,
    # and every zone's FP faces close
    for c in range(m.ncornr):
        z = c // 4
        for f in range(2):
            n = 4 * z + m.cEZ[c, f]
            assert np.array_equal(geo["A_ez"][c, f], -geo["A_ez"][n, 1 - f])
            v = m.cFP[c, f]
            if v < m.ncornr:
                assert np.array_equal(geo["A_fp"][c, f], -geo["A_fp"][v, 1 - f])
    assert np.abs(geo["A_fp"].reshape(nz, 4, 2, 3).sum(axis=(1, 2))).max() < 1e-15
    assert (geo["A_fp"][..., 2] == 0).all() and (geo["A_ez"][..., 2] == 0).all()


def test_rz_polygon_builder_reproduces_the_grid():
    from umt_gb300.mesh_rz import build_rz_polygon_mesh, _grid
    m = build_rz_mesh(4, 3, distort=0.1, seed=3)
    R, Z = _grid(4, 3, 0.2, 1.2, 0.0, 1.0, 0.1, 3)
    vix = lambda i, j: i * 4 + j
    polys = [[vix(i, j), vix(i + 1, j), vix(i + 1, j + 1), vix(i, j + 1)] for i in range(4) for j in range(3)]
    m2 = build_rz_polygon_mesh(np.stack([R.ravel(), Z.ravel()], 1), polys)
    for k in ("numCorner", "cOffSet", "zoneFaces", "zoneOpp", "faceOpp", "cFP", "cEZ", "CToFace", "px", "bdyToC"):
        assert np.array_equal(getattr(m, k), getattr(m2, k)), k


def test_rz_mixed_mesh_geometry():
    """Triangles, quadrilaterals and hexagons: corner areas close to the zone's
    shoelace area, shared faces are exact negations, every zone closes."""
    from umt_gb300.mesh_rz import build_rz_mixed_mesh
    m = build_rz_mixed_mesh(6, 5, distort=0.15, seed=7)
    assert set(np.unique(m.numCorner)) == {3, 4, 6}
    geo = po.geometry_rz(m)
    for z in range(m.nzones):
        c0, n = m.cOffSet[z], m.numCorner[z]
        p = m.px[c0:c0 + n]
        shoelace = 0.5 * (np.dot(p[:, 0], np.roll(p[:, 1], -1)) - np.dot(p[:, 1], np.roll(p[:, 0], -1)))
        assert shoelace > 0
        assert abs(geo["Area"][c0:c0 + n].sum() - shoelace) < 1e-14
        assert abs(geo["A_fp"][c0:c0 + n].sum(axis=(0, 1))).max() < 1e-15
    for c in range(m.ncornr):
        for f in range(2):
            v = m.cFP[c, f]
            if v < m.ncornr:
                assert np.array_equal(geo["A_fp"][c, f], -geo["A_fp"][v, 1 - f])
                assert np.array_equal(m.px[v], m.px[c])
    with pytest.raises(ValueError):
        from umt_gb300.mesh_rz import build_rz_polygon_mesh
        build_rz_polygon_mesh(np.array([[0.2, 0.0], [1.0, 0.0], [0.2, 1.0]]), [[0, 2, 1]])   # clockwise


@pytest.mark.parametrize("P,Az", [(1, 1), (2, 2), (4, 4), (8, 6)])
def test_rz_quadrature(P, Az):
    q = product_quadrature_rz(P, Az)
    A = len(q.weight)
    assert A == 2 * P * (2 * Az + 2)
    assert abs(q.weight.sum() * WTISO_RZ - 1.0) < 1e-14
    assert np.allclose(np.linalg.norm(q.omega, axis=1) <= 1.0 + 1e-15, True)
    assert q.starting.sum() == q.finishing.sum() == 2 * P
    for lev in range(2 * P):
        idx = np.nonzero(q.level == lev)[0]
        assert q.starting[idx[0]] and q.finishing[idx[-1]]
        mu = q.omega[idx, 0]
        assert (np.diff(mu) > 0).all()                               # mu increases along a level
        inner = idx[1:-1]
        assert ((q.tau[inner] > 0) & (q.tau[inner] < 1)).all()
        # alpha telescopes to zero across the level (the angular redistribution
        # moves particles between directions without creating any)
        assert abs(q.alpha[inner[-1]]) < 1e-15
    sf = q.starting | q.finishing
    assert (q.angDerivFac[sf] == 0).all() and (q.quadTauW1[sf] == 1).all() and (q.quadTauW2[sf] == 0).all()


def test_rz_oracle_sweep_is_deterministic_and_positive():
    m = build_rz_mesh(4, 4, distort=0.1, seed=5)
    q = product_quadrature_rz(2, 3)
    geo = po.geometry_rz(m)
    om3 = np.zeros((len(q.weight), 3)); om3[:, :2] = q.omega
    S = po.schedule(m, geo["A_fp"], geo["A_ez"], om3)
    G = 3
    rng = np.random.default_rng(2)
    sigt = rng.uniform(0.5, 5.0, size=(m.nzones, G)); STotal = rng.uniform(0.1, 1.0, size=(m.ncornr, G))
    out = []
    for _ in range(2):
        Psi = np.full((len(q.weight), m.ncornr, G), 0.05); PsiB = np.zeros((len(q.weight), m.nbelem, G))
        out.append(po.set_sweep_rz(m, geo, S, sigt, STotal, 0.2, om3, q, Psi, PsiB, savePsi=True))
    assert np.array_equal(out[0], out[1])
    assert (out[0] > 0).all() and np.isfinite(out[0]).all()
