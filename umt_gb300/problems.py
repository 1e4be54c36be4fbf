"""Problem set-ups: the reference driver's uniform-material problem and the
seeded synthetic multigroup problems the benchmarks run.

Uniform problem (test_driver.cc:1163-1286, 1822-1841): sigma_a = 10 in every
group, sigma_s = 0, radiation temperature 0.05 (initial intensity is the
group-integrated Planck function at Tr, aux/InitTeton.F90:101-115), electron
temperature 0.5, density 1.31, specific heat 0.501, group bounds
log-spaced on [1e-6, 1e2], vacuum on all six sides, product quadrature with
polar axis x, dt = 1e-3 (tau = 1/(c dt), control/initializeSets.F90:81).

Synthetic problems: per-zone per-group total opacity log-uniform on a stated
range, scattering ratio uniform on a stated range, isotropic source q, all
drawn from numpy's Philox generator with the stated seed.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from .mesh import Mesh, build_tiled_mesh
from .quadrature import WTISO_XYZ, product_quadrature

SPEED_LIGHT = 299.792458               # mods/radconstant_mod.F90 (mini-app)
RAD_CONSTANT = 0.013720169264801055


def group_bounds(ngr: int) -> np.ndarray:
    """test_driver.cc:1174-1183."""
    lo, hi = math.log(1.0e-6), math.log(1.0e2)
    d = (hi - lo) / ngr
    gnu = np.array([math.exp(lo + g * d) for g in range(ngr + 1)])
    gnu[ngr] = 1.0e2
    return gnu


def _clark_cumulative(e: float) -> float:
    # Clark, J. Comput. Phys. 70 (1987) 311: eq. 32 (small argument) and the
    # rational fit of eq. 48, as normalised by 15/pi^4.
    if e < 0.01:
        return e * e * e * (0.05132991127342032 - 0.01924871672753262 * e)
    num = 1.0 + e * (1.2807339766120354 + e * (0.8578722513311724 + e * (
        0.33288908614428098 + e * (0.079984931563508915 + e * 0.011878558806454416))))
    den = 1.0 + e * (0.2807339758744 + e * 0.07713864107538)
    return 1.0 - math.exp(-e) * num / den


def planck_groups(T: float, k: float, bnorm: float, gnu: np.ndarray) -> np.ndarray:
    """Group integrals of the Planck function (integrateBlackBodyGroups)."""
    ngr = len(gnu) - 1
    B = np.zeros(ngr)
    kT = k * T
    if not kT > 0.0:
        return B
    full = bnorm * (T * T) * (T * T)
    lo = 0.0
    for g in range(ngr - 1):
        hi = _clark_cumulative(gnu[g + 1] / kT)
        B[g] = full * (hi - lo)
        lo = hi
    B[ngr - 1] = full * (1.0 - lo)
    return B


@dataclasses.dataclass
class Problem:
    name: str
    mesh: Mesh
    omega: np.ndarray
    weight: np.ndarray
    ngr: int
    siga: np.ndarray          # [nz, G]
    sigs: np.ndarray          # [nz, G]
    tau: float
    psi0: np.ndarray | None   # [A, nc, G] initial (previous-cycle) angular flux
    q_ext: np.ndarray | None  # [nz, G] isotropic external source (per steradian-integrated)
    seed: int | None = None
    dt: float = 1.0e-3

    @property
    def sigt(self) -> np.ndarray:
        """Sigt = SigA + SigS + tau (control/setTotalOpacity.F90:52)."""
        return self.siga + self.sigs + self.tau

    @property
    def units(self) -> int:
        return self.mesh.ncornr * len(self.weight) * self.ngr


def uniform_problem(tiles=(10, 10, 10), npolar=2, nazimuthal=2, ngr=2, dt=1.0e-3) -> Problem:
    """The reference driver's built-in uniform material (test_driver.cc:1163-1286):
    sigma_a = 10 in every group, no scattering, Tr = 0.05 Planck initial intensity."""
    m = build_tiled_mesh(*tiles)
    omega, weight = product_quadrature(npolar, nazimuthal, 1)
    siga = np.full((m.nzones, ngr), 10.0)
    sigs = np.zeros((m.nzones, ngr))
    tau = 1.0 / (SPEED_LIGHT * dt)
    gnu = group_bounds(ngr)
    planck = planck_groups(0.05, 1.0, SPEED_LIGHT * RAD_CONSTANT, gnu)
    psi_g = np.maximum(WTISO_XYZ * planck, 0.0)
    psi0 = np.broadcast_to(psi_g, (len(weight), m.ncornr, ngr)).copy()
    return Problem("uniform", m, omega, weight, ngr, siga, sigs, tau, psi0, None, None, dt)


def synthetic_problem(tiles, npolar, nazimuthal, ngr, seed, sigt_range=(1e-2, 1e2),
                      c_range=(0.0, 0.5), q=1.0, n_materials=None, dt=1.0e-3,
                      time_dependent=False) -> Problem:
    """Seeded multigroup problem with scattering (the scattering workloads: 20^3
    and 30^3 tiles with 128 directions and 16 groups, batches of small problems).

    Opacities are drawn per zone (or per material, with a per-tile material
    index when n_materials is given) and per group; sigma_s = c*sigma_t and
    sigma_a = (1-c)*sigma_t.  With time_dependent the tau*psi term of
    Teton's time discretisation is kept with a flat initial intensity.
    """
    m = build_tiled_mesh(*tiles)
    omega, weight = product_quadrature(npolar, nazimuthal, 1)
    rng = np.random.Generator(np.random.Philox(seed))
    lo, hi = math.log(sigt_range[0]), math.log(sigt_range[1])
    if n_materials:
        mat_sigt = np.exp(rng.uniform(lo, hi, size=(n_materials, ngr)))
        mat_c = rng.uniform(c_range[0], c_range[1], size=(n_materials, ngr))
        ntile = m.tiles[0] * m.tiles[1] * m.tiles[2]
        tile_mat = rng.integers(0, n_materials, size=ntile)
        zmat = tile_mat[m.tile_of_zone]
        sigt = mat_sigt[zmat]
        cr = mat_c[zmat]
    else:
        sigt = np.exp(rng.uniform(lo, hi, size=(m.nzones, ngr)))
        cr = rng.uniform(c_range[0], c_range[1], size=(m.nzones, ngr))
    sigs = cr * sigt
    siga = sigt - sigs
    tau = 1.0 / (SPEED_LIGHT * dt) if time_dependent else 0.0
    psi0 = None
    if time_dependent:
        psi0 = np.full((len(weight), m.ncornr, ngr), WTISO_XYZ)
    q_ext = np.full((m.nzones, ngr), float(q))
    return Problem(f"synthetic{seed}", m, omega, weight, ngr, siga, sigs, tau, psi0, q_ext, seed, dt)


def zone_to_corner(m: Mesh, zarr: np.ndarray) -> np.ndarray:
    return zarr[m.cToZone]
