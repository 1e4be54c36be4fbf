"""Tiled polyhedral mesh and its Teton corner connectivity.

The reference driver builds its 3-D test mesh by repeating one 2-D tile
(squares, quadrilaterals and triangles) over an nx x ny grid and extruding
each tile one zone-layer thick in z, nz times (test_driver.cc:1758-1817, tile
shown in img/tile.jpg).  The tile generator itself lives in a third-party
library that is not part of the reference, so this module defines its own
24-zone tile with the same make-up (8 squares, 8 convex quadrilaterals,
8 triangles) and the same conforming tile boundary on all four sides.

Connectivity follows the conventions `teton_setzone` consumes and builds
(aux/setTetonZone.F90:10-202):

* a corner is a (zone, vertex) pair; corners of a zone are contiguous and
  numbered from ``cOffSet[zone]``;
* per corner, its corner faces are ordered by chaining around the vertex:
  the next corner face is the zone face whose counter-clockwise neighbour of
  the corner equals the clockwise neighbour on the previous face
  (setTetonZone.F90:161-181);
* ``cEZ[c, i]`` is the zone-local index of the corner across edge-zone face
  i, ``cFP[c, i]`` the global corner across the zone face (or
  ``ncornr + b`` for boundary element b), ``CToFace[c, i]`` the zone face;
* face vertex lists are ordered so that the right-hand normal points INTO
  the zone; with that ordering the area-vector formula of
  rt/geometryUCBxyz.F90:110-141 yields outward normals.

Every array here is 0-based (``cFP >= ncornr`` marks a boundary element).
The C-ABI accepts 0-based or 1-based input through ``UmtMesh.index_base``.
"""
from __future__ import annotations

import dataclasses
import numpy as np

MAXCF = 3          # corner faces per corner (vertex degree 3 in extruded meshes)
MAXCORNER = 8      # hexahedron
MAXFACES = 6       # hexahedron
TILE_UNITS = 8     # tile coordinates live on an 8 x 8 integer lattice


def _tile_polygons() -> list[list[tuple[int, int]]]:
    """The 24 polygons of one tile, counter-clockwise, on the 8x8 lattice."""
    sq = lambda x0, y0, s: [(x0, y0), (x0 + s, y0), (x0 + s, y0 + s), (x0, y0 + s)]
    polys = []
    # centre block split into 2x2 squares, then the four corner squares
    polys += [sq(3, 3, 1), sq(4, 3, 1), sq(4, 4, 1), sq(3, 4, 1)]
    polys += [sq(0, 0, 1), sq(7, 0, 1), sq(7, 7, 1), sq(0, 7, 1)]
    # one quadrant of the remaining region: two quads and two triangles
    quadrant = [
        [(1, 0), (4, 0), (3, 3), (1, 1)],
        [(4, 0), (4, 3), (3, 3)],
        [(0, 1), (1, 1), (3, 3), (0, 4)],
        [(0, 4), (3, 3), (3, 4)],
    ]
    for mx, my in [(False, False), (True, False), (True, True), (False, True)]:
        for p in quadrant:
            q = [((8 - x) if mx else x, (8 - y) if my else y) for (x, y) in p]
            if mx != my:          # a single reflection flips orientation
                q = q[::-1]
            polys.append(q)
    return polys


TILE_POLYGONS = _tile_polygons()
ZONES_PER_TILE = len(TILE_POLYGONS)


def _zone_faces(n: int) -> list[list[int]]:
    """Local face -> local corner list of an extruded n-gon, inward RH normal.

    Corners 0..n-1 are the bottom ring (polygon order), n..2n-1 the top ring.
    """
    faces = [list(range(n)), [n + i for i in range(n - 1, -1, -1)]]
    for e in range(n):
        faces.append([e, n + e, n + (e + 1) % n, (e + 1) % n])
    return faces


def _chain_corner_faces(nc: int, faces: list[list[int]]):
    """Per-corner corner-face ordering of one zone (setTetonZone.F90:143-181).

    Returns (nCFaces[nc], cEZ[nc,3], CToFace[nc,3], pos[nc,3]) where pos is the
    position of the corner in the face list (used to look up the opposite
    corner across the face).
    """
    lists = [[] for _ in range(nc)]          # (cw, ccw, face, pos)
    for f, fl in enumerate(faces):
        m = len(fl)
        for i, c in enumerate(fl):
            lists[c].append((fl[(i + 1) % m], fl[(i - 1) % m], f, i))
    ncf = np.zeros(nc, np.int32)
    cez = np.full((nc, MAXCF), -1, np.int32)
    ctf = np.full((nc, MAXCF), -1, np.int32)
    pos = np.full((nc, MAXCF), -1, np.int32)
    for c in range(nc):
        L = lists[c]
        k = len(L)
        assert k <= MAXCF, "vertex of degree > 3"
        ncf[c] = k
        cw, ccw, f, p = L[0]
        cez[c, 0], ctf[c, 0], pos[c, 0] = ccw, f, p
        last = cw
        for i in range(1, k):
            for ii in range(1, k):
                if L[ii][1] == last:
                    cw, ccw, f, p = L[ii]
                    cez[c, i], ctf[c, i], pos[c, i] = ccw, f, p
                    last = cw
                    break
            else:
                raise ValueError("corner faces do not close around the vertex")
    return ncf, cez, ctf, pos


@dataclasses.dataclass
class Mesh:
    """Teton-style corner mesh (0-based indices)."""
    nzones: int
    ncornr: int
    nbelem: int
    numCorner: np.ndarray     # [nz] int32
    cOffSet: np.ndarray       # [nz] int32
    zoneFaces: np.ndarray     # [nz] int32
    zoneOpp: np.ndarray       # [nz, MAXFACES] int32, -1 = problem boundary
    faceOpp: np.ndarray       # [nz, MAXFACES] int32
    nCFaces: np.ndarray       # [nc] int32
    cFP: np.ndarray           # [nc, MAXCF] int32  (>= ncornr: boundary element)
    cEZ: np.ndarray           # [nc, MAXCF] int32  zone-local corner
    CToFace: np.ndarray       # [nc, MAXCF] int32  zone-local face
    px: np.ndarray            # [nc, 3] float64 corner vertex coordinates
    bdyToC: np.ndarray        # [nbelem] int32 global corner of boundary element
    cToZone: np.ndarray       # [nc] int32
    tiles: tuple = (0, 0, 0)
    tile_of_zone: np.ndarray | None = None   # [nz] int32 tile index (x fastest)

    @property
    def maxCorner(self) -> int:
        return int(self.numCorner.max())

    def corner_to_zone(self):
        return self.cToZone


def build_tiled_mesh(nx: int, ny: int, nz: int, perturb: float = 0.0, seed: int = 0) -> Mesh:
    """Unit-cube mesh of nx x ny x nz tiles, one zone layer per tile.

    Zones are numbered tile by tile (x fastest, then y, then z) and by the
    fixed polygon order inside a tile, which keeps neighbours close in memory
    (the role of the reference's k-d tree zone reordering).

    perturb > 0 moves every interior lattice vertex by a seeded random
    displacement of up to `perturb` lattice spacings along each axis
    (boundary vertices stay on their boundary planes).  The faces then stop
    being planar, and for some directions a zone face is partly incoming and
    partly outgoing, a zone's corners cannot be ordered, or zones depend on
    one another in a loop: the mesh cycles that Teton's cycle list handles.
    """
    U = TILE_UNITS
    LX, LY = U * nx + 1, U * ny + 1
    ntile = nx * ny * nz
    nP = ZONES_PER_TILE

    # ---- zone templates (one per tile polygon) ------------------------------
    tmpl = []
    for poly in TILE_POLYGONS:
        n = len(poly)
        faces = _zone_faces(n)
        ncf, cez, ctf, pos = _chain_corner_faces(2 * n, faces)
        tmpl.append(dict(n=n, poly=poly, faces=faces, ncf=ncf, cez=cez, ctf=ctf, pos=pos))
    nC_t = np.array([2 * t["n"] for t in tmpl], np.int32)          # corners / zone
    nF_t = np.array([2 + t["n"] for t in tmpl], np.int32)          # faces / zone

    # ---- zone numbering ------------------------------------------------------
    tiles_idx = np.arange(ntile)
    ti = tiles_idx % nx
    tj = (tiles_idx // nx) % ny
    tk = tiles_idx // (nx * ny)
    nzones = ntile * nP
    zone_tile = np.repeat(tiles_idx, nP)
    zone_poly = np.tile(np.arange(nP), ntile)
    numCorner = nC_t[zone_poly]
    cOffSet = np.zeros(nzones, np.int64)
    cOffSet[1:] = np.cumsum(numCorner)[:-1]
    ncornr = int(numCorner.sum())
    corners_per_tile = int(nC_t.sum())
    tile_c0 = np.concatenate([[0], np.cumsum(nC_t)[:-1]]).astype(np.int64)

    # ---- per-corner 3-D lattice vertex id -----------------------------------
    # corner template: for polygon p, local corner l -> (dx, dy, dz)
    c_lx, c_ly, c_lz, c_poly, c_loc = [], [], [], [], []
    for p, t in enumerate(tmpl):
        n = t["n"]
        for l in range(2 * n):
            x, y = t["poly"][l % n]
            c_lx.append(x); c_ly.append(y); c_lz.append(l // n)
            c_poly.append(p); c_loc.append(l)
    c_lx = np.array(c_lx, np.int64); c_ly = np.array(c_ly, np.int64)
    c_lz = np.array(c_lz, np.int64)
    gx = (ti[:, None] * U + c_lx[None, :]).ravel()
    gy = (tj[:, None] * U + c_ly[None, :]).ravel()
    gz = (tk[:, None] + c_lz[None, :]).ravel()
    vid = (gz * LY + gy) * LX + gx                                  # [ncornr]
    px = np.stack([gx / (U * nx), gy / (U * ny), gz / float(nz)], axis=1)
    if perturb > 0.0:
        LZ = nz + 1
        rng = np.random.Generator(np.random.Philox(seed))
        d = rng.uniform(-perturb, perturb, size=(LZ * LY * LX, 3))
        lx = np.arange(LZ * LY * LX) % LX
        ly = (np.arange(LZ * LY * LX) // LX) % LY
        lz = np.arange(LZ * LY * LX) // (LX * LY)
        d[(lx == 0) | (lx == LX - 1), 0] = 0.0
        d[(ly == 0) | (ly == LY - 1), 1] = 0.0
        d[(lz == 0) | (lz == LZ - 1), 2] = 0.0
        px = px + d[vid] * np.array([1.0 / (U * nx), 1.0 / (U * ny), 1.0 / nz])

    # ---- per-corner template connectivity ------------------------------------
    ncf_t = np.concatenate([t["ncf"] for t in tmpl])
    cez_t = np.concatenate([t["cez"] for t in tmpl])
    ctf_t = np.concatenate([t["ctf"] for t in tmpl])
    pos_t = np.concatenate([t["pos"] for t in tmpl])
    nCFaces = np.tile(ncf_t, ntile).astype(np.int32)
    cEZ = np.tile(cez_t, (ntile, 1)).astype(np.int32)
    CToFace = np.tile(ctf_t, (ntile, 1)).astype(np.int32)
    cToZone = np.repeat(np.arange(nzones, dtype=np.int32), numCorner)

    # ---- zone faces: key every face by its sorted vertex ids ----------------
    zoneFaces = nF_t[zone_poly].astype(np.int32)
    face_z, face_f, face_key = [], [], []
    # vertex ids of face (zone, f): gather through template face lists
    maxfv = 4
    fz_all, ff_all, fv_all = [], [], []
    for p, t in enumerate(tmpl):
        zs = np.arange(p, nzones, nP)                                # zones with this polygon
        c0 = cOffSet[zs]
        for f, fl in enumerate(t["faces"]):
            v = np.full((len(zs), maxfv), -1, np.int64)
            for i, lc in enumerate(fl):
                v[:, i] = vid[c0 + lc]
            fz_all.append(zs); ff_all.append(np.full(len(zs), f)); fv_all.append(v)
    fz = np.concatenate(fz_all); ff = np.concatenate(ff_all); fv = np.concatenate(fv_all)
    fvs = np.sort(np.where(fv < 0, np.iinfo(np.int64).max, fv), axis=1)
    order = np.lexsort(tuple(fvs[:, k] for k in range(maxfv - 1, -1, -1)))
    fvs_o = fvs[order]
    same = np.all(fvs_o[1:] == fvs_o[:-1], axis=1)
    zoneOpp = np.full((nzones, MAXFACES), -1, np.int32)
    faceOpp = np.full((nzones, MAXFACES), -1, np.int32)
    a = order[:-1][same]; b = order[1:][same]
    zoneOpp[fz[a], ff[a]] = fz[b]; faceOpp[fz[a], ff[a]] = ff[b]
    zoneOpp[fz[b], ff[b]] = fz[a]; faceOpp[fz[b], ff[b]] = ff[a]

    # ---- cFP: corner across each corner face ---------------------------------
    cFP = np.full((ncornr, MAXCF), -1, np.int64)
    zc = cToZone.astype(np.int64)
    cidx = np.arange(ncornr)
    for i in range(MAXCF):
        f = CToFace[:, i].astype(np.int64)
        zo = zoneOpp[zc, f].astype(np.int64)
        fo = faceOpp[zc, f].astype(np.int64)
        inner = zo >= 0
        # find the corner of zone zo on face fo with the same vertex id
        cand = np.full(ncornr, -1, np.int64)
        cc = cidx[inner]; zoi = zo[inner]; foi = fo[inner]
        pz = zone_poly[zoi]
        myv = vid[cc]
        for p, t in enumerate(tmpl):
            selp = pz == p
            if not selp.any():
                continue
            for f2, fl in enumerate(t["faces"]):
                sel = selp & (foi == f2)
                if not sel.any():
                    continue
                c0o = cOffSet[zoi[sel]]
                mv = myv[sel]
                res = np.full(sel.sum(), -1, np.int64)
                for lc in fl:
                    hit = vid[c0o + lc] == mv
                    res[hit] = c0o[hit] + lc
                cand[cc[sel]] = res
        cFP[inner, i] = cand[inner]
    assert (cFP[np.arange(MAXCF)[None, :] < nCFaces[:, None]][
        (zoneOpp[zc[:, None].repeat(MAXCF, 1), CToFace] >= 0)[np.arange(MAXCF)[None, :] < nCFaces[:, None]]] >= 0).all()

    # ---- boundary elements: zone order, face order, corner order on face ----
    # for each zone face on the boundary, its corners in face order
    rows = []
    for p, t in enumerate(tmpl):
        zs = np.arange(p, nzones, nP)
        for f, fl in enumerate(t["faces"]):
            onb = zoneOpp[zs, f] < 0
            if not onb.any():
                continue
            zb = zs[onb]
            for i, lc in enumerate(fl):
                rows.append(np.stack([zb, np.full(len(zb), f), np.full(len(zb), i),
                                      cOffSet[zb] + lc], axis=1))
    rows = np.concatenate(rows) if rows else np.zeros((0, 4), np.int64)
    order = np.lexsort((rows[:, 2], rows[:, 1], rows[:, 0]))
    rows = rows[order]
    nbelem = len(rows)
    bdyToC = rows[:, 3].astype(np.int32)
    # corner face (c, i) on a boundary face -> ncornr + b
    key_b = (rows[:, 3] * MAXFACES + rows[:, 1])
    srt = np.argsort(key_b)
    key_sorted = key_b[srt]
    for i in range(MAXCF):
        f = CToFace[:, i].astype(np.int64)
        valid = i < nCFaces
        onb = valid & (zoneOpp[zc, np.where(f < 0, 0, f)] < 0)
        k = cidx[onb] * MAXFACES + f[onb]
        loc = np.searchsorted(key_sorted, k)
        assert (key_sorted[loc] == k).all()
        cFP[onb, i] = ncornr + srt[loc]

    return Mesh(nzones=nzones, ncornr=ncornr, nbelem=nbelem,
                numCorner=numCorner.astype(np.int32), cOffSet=cOffSet.astype(np.int32),
                zoneFaces=zoneFaces, zoneOpp=zoneOpp, faceOpp=faceOpp,
                nCFaces=nCFaces, cFP=cFP.astype(np.int32), cEZ=cEZ, CToFace=CToFace,
                px=np.ascontiguousarray(px), bdyToC=bdyToC, cToZone=cToZone,
                tiles=(nx, ny, nz), tile_of_zone=zone_tile.astype(np.int32))
