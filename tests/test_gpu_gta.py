"""Grey transport acceleration against the oracle's CPU restatement
(oracle/gta_oracle.py): the spectrum chi and the grey correction vector of
one GTA step, on the same iterate, previous iterate and materials.

Reference: rt/GTASolver.F90:42-425 (BiCGStab), rt/GreySweep.F90 (grey sweep
plus stretched-TSA sweep; or, with the newer solver, one grey sweep and a
per-zone direct solve: snac/InitSweepGreyUCBxyz.F90,
snac/UpdateScalarIntensity.F90), rt/setGTAOpacity.F90:176-232 (grey and
stretched opacities), rt/scat_prod.F90 / scat_prod1.F90 (inner products).  The
reference ships no GTA data, so this pins the device implementation to the
restatement, not to the reference's output.  Tolerances: chi 1e-12, the
correction 1e-9 (relative max norm): the grey sweeps agree to ~1e-15 and
BiCGStab carries that through a few iterations.
"""
import numpy as np
import pytest

from umt_gb300 import capi
from umt_gb300.problems import synthetic_problem
from oracle import gta_oracle as go
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("solver", [capi.UMT_GTA_TSA, capi.UMT_GTA_ZONE])
@pytest.mark.parametrize("tiles,G,crange,maxit", [((3, 2, 2), 4, (0.5, 0.95), 10), ((2, 2, 2), 8, (0.9, 0.999), 4)])
def test_gta_correction_matches_oracle(umtlib, tiles, G, crange, maxit, solver):
    prob = synthetic_problem(tiles, 2, 2, G, seed=41, sigt_range=(0.5, 50.0), c_range=crange, time_dependent=True)
    m = prob.mesh
    rng = np.random.default_rng(42)
    phi0 = rng.uniform(0.5, 1.5, size=(m.ncornr, G))
    umtlib.init(m, prob.omega, prob.weight, G, flags=1)
    umtlib.set_materials(prob.sigt, prob.sigs, prob.tau)
    umtlib.set_psi(prob.psi0, None)
    umtlib.set_gta(maxit, 1e-6, 0)
    umtlib.set_gta_solver(solver)
    STotal = (prob.sigs[m.cToZone] * phi0 + prob.q_ext[m.cToZone]) / (4 * np.pi)
    phi1 = umtlib.sweep(STotal, savePsi=False, precision=capi.UMT_FP64)
    x, chi, sweeps = umtlib.gta_correction(phi0)
    restated = go.gta_correction if solver == capi.UMT_GTA_TSA else go.gta_correction_new
    xr, chir, sweeps_r = restated(m, np.ascontiguousarray(prob.sigt), np.ascontiguousarray(prob.sigs),
                                  prob.tau, phi1, phi0, maxit=maxit, tol=1e-6)
    print(f"\nsolver {solver}: correction rel err {rel_err(x, xr):.2e}, chi rel err {rel_err(chi, chir):.2e}, "
          f"grey sweeps {sweeps} (oracle {sweeps_r})")
    assert sweeps == sweeps_r
    assert rel_err(chi, chir) < 1e-12
    assert rel_err(x, xr) < 1e-9
    assert np.abs(x).max() > 0
