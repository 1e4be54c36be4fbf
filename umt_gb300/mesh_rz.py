"""2-D RZ mesh (quadrilateral zones in the (r, z) half-plane) with Teton's
corner connectivity for the RZ UCB sweep.

Conventions (as rt/geometryUCBrz.F90:48-150 reads them; 0-based here):
  * a zone's corners are its vertices in counter-clockwise order in (r, z);
  * cEZ[c, 0] is the previous corner of the zone, cEZ[c, 1] the next one;
  * corner face 0 is the half of edge (c, next) at c, corner face 1 the half
    of edge (previous, c) at c; cFP[c, f] is the corner at the same vertex in
    the zone across that edge, or ncornr + b for boundary element b;
  * zone face k is the edge from vertex k to vertex k+1, so corner face 0 of
    corner k lies on zone face k and corner face 1 on zone face k-1;
  * boundary elements are corner faces on the mesh boundary, ordered by zone,
    zone face, corner.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class MeshRZ:
    nzones: int
    ncornr: int
    nbelem: int
    numCorner: np.ndarray   # [nz] int32
    cOffSet: np.ndarray     # [nz] int32
    zoneFaces: np.ndarray   # [nz] int32
    zoneOpp: np.ndarray     # [nz, 4] int32, -1 on the boundary
    faceOpp: np.ndarray     # [nz, 4] int32
    nCFaces: np.ndarray     # [nc] int32 (2)
    cFP: np.ndarray         # [nc, 2] int32
    cEZ: np.ndarray         # [nc, 2] int32
    CToFace: np.ndarray     # [nc, 2] int32
    px: np.ndarray          # [nc, 2] (r, z) of each corner's vertex
    bdyToC: np.ndarray      # [nb] int32
    cToZone: np.ndarray     # [nc] int32


def build_rz_polygon_mesh(verts: np.ndarray, polys: list[list[int]]) -> MeshRZ:
    """A conforming mesh of polygons (3 to 6 vertices each, listed
    counter-clockwise in (r, z)) with the conventions of the module
    docstring; neighbours are found by matching edges."""
    verts = np.asarray(verts, np.float64)
    nz = len(polys)
    numCorner = np.array([len(p) for p in polys], np.int32)
    if nz == 0 or numCorner.min() < 3 or numCorner.max() > 6:
        raise ValueError("RZ polygons need 3 to 6 vertices")
    for p in polys:
        q = verts[p]
        if 0.5 * (np.dot(q[:, 0], np.roll(q[:, 1], -1)) - np.dot(q[:, 1], np.roll(q[:, 0], -1))) <= 0.0:
            raise ValueError("RZ polygons must be counter-clockwise")
    cOffSet = np.concatenate([[0], np.cumsum(numCorner)[:-1]]).astype(np.int32)
    nc = int(numCorner.sum())
    maxF = int(numCorner.max())
    vid = np.concatenate([np.asarray(p, np.int64) for p in polys])
    px = verts[vid]
    edge_owner = {}                                      # (v_from, v_to) -> (zone, face)
    for z, p in enumerate(polys):
        n = len(p)
        for k in range(n):
            e = (p[k], p[(k + 1) % n])
            if e in edge_owner:
                raise ValueError("edge used twice in the same direction: polygons overlap or are not CCW")
            edge_owner[e] = (z, k)
    zoneOpp = np.full((nz, maxF), -1, np.int32)
    faceOpp = np.full((nz, maxF), -1, np.int32)
    for z, p in enumerate(polys):
        n = len(p)
        for k in range(n):
            other = edge_owner.get((p[(k + 1) % n], p[k]))
            if other is not None:
                zoneOpp[z, k], faceOpp[z, k] = other
    cEZ = np.zeros((nc, 2), np.int32)
    CToFace = np.zeros((nc, 2), np.int32)
    cFP = np.full((nc, 2), -1, np.int64)
    cToZone = np.repeat(np.arange(nz, dtype=np.int32), numCorner)
    for z, p in enumerate(polys):
        n = len(p)
        for k in range(n):
            c = cOffSet[z] + k
            cEZ[c] = ((k + n - 1) % n, (k + 1) % n)
            CToFace[c] = (k, (k + n - 1) % n)
            for f, edge in enumerate((k, (k + n - 1) % n)):
                zo = zoneOpp[z, edge]
                if zo >= 0:
                    hit = np.nonzero(vid[cOffSet[zo]:cOffSet[zo] + numCorner[zo]] == vid[c])[0]
                    assert len(hit) == 1
                    cFP[c, f] = cOffSet[zo] + hit[0]
    bdy = []
    for z, p in enumerate(polys):
        n = len(p)
        for edge in range(n):
            if zoneOpp[z, edge] < 0:
                c_a, c_b = cOffSet[z] + edge, cOffSet[z] + (edge + 1) % n
                for c, f in ((c_a, 0), (c_b, 1)):
                    cFP[c, f] = nc + len(bdy)
                    bdy.append(c)
    assert (cFP >= 0).all()
    return MeshRZ(nz, nc, len(bdy), numCorner, cOffSet, numCorner.copy(), zoneOpp, faceOpp,
                  np.full(nc, 2, np.int32), cFP.astype(np.int32), cEZ, CToFace, px,
                  np.asarray(bdy, np.int32), cToZone)


def build_rz_mixed_mesh(nr: int, nzr: int, r0: float = 0.2, r1: float = 1.2, z0: float = 0.0, z1: float = 1.0,
                        distort: float = 0.0, seed: int = 0, p_triangle: float = 0.25,
                        p_hexagon: float = 0.25) -> MeshRZ:
    """The nr x nzr grid of build_rz_mesh with, seeded, some quadrilaterals
    split into two triangles along a diagonal and some pairs of neighbours in
    r merged into one hexagon (whose shared edge's vertices become 180-degree
    vertices of the hexagon).  `distort` moves interior vertices that belong
    to no hexagon, so every zone stays convex."""
    R, Z = _grid(nr, nzr, r0, r1, z0, z1, 0.0, seed)
    rng = np.random.Generator(np.random.Philox(seed + 1))
    vix = lambda i, j: i * (nzr + 1) + j
    polys, pinned = [], set()
    j_rows = range(nzr)
    for j in j_rows:
        i = 0
        while i < nr:
            u = rng.uniform()
            if u < p_hexagon and i + 1 < nr:
                polys.append([vix(i, j), vix(i + 1, j), vix(i + 2, j), vix(i + 2, j + 1), vix(i + 1, j + 1),
                              vix(i, j + 1)])
                pinned.update({(i + di, j + dj) for di in range(3) for dj in range(2)})
                i += 2
                continue
            q = [vix(i, j), vix(i + 1, j), vix(i + 1, j + 1), vix(i, j + 1)]
            if u < p_hexagon + p_triangle:
                polys += [[q[0], q[1], q[2]], [q[0], q[2], q[3]]]
            else:
                polys.append(q)
            i += 1
    if distort > 0.0:
        drng = np.random.Generator(np.random.Philox(seed))
        dr, dz = (r1 - r0) / nr, (z1 - z0) / nzr
        for i in range(1, nr):
            for j in range(1, nzr):
                a, b = drng.uniform(-1, 1, size=2)
                if (i, j) not in pinned:
                    R[i, j] += distort * dr * a
                    Z[i, j] += distort * dz * b
    verts = np.stack([R.ravel(), Z.ravel()], axis=1)
    return build_rz_polygon_mesh(verts, polys)


def _grid(nr, nzr, r0, r1, z0, z1, distort, seed):
    if nr < 1 or nzr < 1 or not (0.0 < r0 < r1) or not (z0 < z1) or not (0.0 <= distort < 0.3):
        raise ValueError("bad RZ mesh parameters")
    rr = np.linspace(r0, r1, nr + 1)
    zz = np.linspace(z0, z1, nzr + 1)
    R, Z = np.meshgrid(rr, zz, indexing="ij")             # vertex (i, j)
    if distort > 0.0:
        rng = np.random.Generator(np.random.Philox(seed))
        dr, dz = (r1 - r0) / nr, (z1 - z0) / nzr
        R[1:-1, 1:-1] += distort * dr * rng.uniform(-1, 1, size=(nr - 1, nzr - 1))
        Z[1:-1, 1:-1] += distort * dz * rng.uniform(-1, 1, size=(nr - 1, nzr - 1))
    return R, Z


def build_rz_mesh(nr: int, nzr: int, r0: float = 0.2, r1: float = 1.2, z0: float = 0.0, z1: float = 1.0,
                  distort: float = 0.0, seed: int = 0) -> MeshRZ:
    """nr x nzr quadrilaterals over [r0, r1] x [z0, z1] (r0 > 0: no axis);
    interior vertices moved by up to `distort` of a cell width (seeded)."""
    R, Z = _grid(nr, nzr, r0, r1, z0, z1, distort, seed)
    nz = nr * nzr
    zid = lambda i, j: i * nzr + j
    # vertex (i, j) offsets of the 4 corners, counter-clockwise
    off = [(0, 0), (1, 0), (1, 1), (0, 1)]
    numCorner = np.full(nz, 4, np.int32)
    cOffSet = (4 * np.arange(nz)).astype(np.int32)
    nc = 4 * nz
    px = np.zeros((nc, 2))
    vid = np.zeros(nc, np.int64)
    zoneOpp = np.full((nz, 4), -1, np.int32)
    faceOpp = np.full((nz, 4), -1, np.int32)
    for i in range(nr):
        for j in range(nzr):
            z = zid(i, j)
            for k, (di, dj) in enumerate(off):
                px[4 * z + k] = (R[i + di, j + dj], Z[i + di, j + dj])
                vid[4 * z + k] = (i + di) * (nzr + 1) + (j + dj)
            # edges: 0 bottom (j-1), 1 right (i+1), 2 top (j+1), 3 left (i-1)
            nb = [(i, j - 1, 2), (i + 1, j, 3), (i, j + 1, 0), (i - 1, j, 1)]
            for k, (ii, jj, fo) in enumerate(nb):
                if 0 <= ii < nr and 0 <= jj < nzr:
                    zoneOpp[z, k] = zid(ii, jj)
                    faceOpp[z, k] = fo
    cEZ = np.zeros((nc, 2), np.int32)
    CToFace = np.zeros((nc, 2), np.int32)
    cFP = np.full((nc, 2), -1, np.int64)
    cToZone = np.repeat(np.arange(nz, dtype=np.int32), 4)
    for z in range(nz):
        for k in range(4):
            c = 4 * z + k
            cEZ[c] = ((k + 3) % 4, (k + 1) % 4)
            CToFace[c] = (k, (k + 3) % 4)
            for f, edge in enumerate((k, (k + 3) % 4)):
                zo = zoneOpp[z, edge]
                if zo >= 0:
                    hit = np.nonzero(vid[4 * zo:4 * zo + 4] == vid[c])[0]
                    assert len(hit) == 1
                    cFP[c, f] = 4 * zo + hit[0]
    # boundary elements: zone order, zone face, corner (corner face 0 of the
    # edge's first vertex, corner face 1 of its second)
    bdy = []
    for z in range(nz):
        for edge in range(4):
            if zoneOpp[z, edge] < 0:
                c_a, c_b = 4 * z + edge, 4 * z + (edge + 1) % 4
                for c, f in ((c_a, 0), (c_b, 1)):
                    cFP[c, f] = nc + len(bdy)
                    bdy.append(c)
    assert (cFP >= 0).all()
    return MeshRZ(nz, nc, len(bdy), numCorner, cOffSet, np.full(nz, 4, np.int32), zoneOpp, faceOpp,
                  np.full(nc, 2, np.int32), cFP.astype(np.int32), cEZ, CToFace, px,
                  np.asarray(bdy, np.int32), cToZone)
