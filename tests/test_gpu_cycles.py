"""Meshes with sweep cycles: the device schedule's cycle list against the
oracle's (snac/snneed.F90 mixed faces, snac/getDownStreamData.F90 + fixZone
lagged zones, snac/cyclebreaker.F90 + sccsearch.F90 zone cycles), and the
sweep with lagged corner fluxes (initFromCycleList / updateCycleList,
control/constructDynMemory.F90:111-214) against the oracle's SetSweep.

The tiled mesh with its interior vertices moved by a seeded 1% or 6% of a
lattice spacing has non-planar faces: for many of the 128 directions a zone
face is partly incoming and partly outgoing, zones depend on one another in
loops, and (at 6%) some zones' corners cannot be ordered.  FP64 to 1e-12,
FP32 to 1e-5 (PhiTotal) and 1e-4 (Psi, PsiB), over two sweeps in a row so
that the second reads the cycle values the first stored.
"""
import numpy as np
import pytest

from umt_gb300 import capi
from umt_gb300.mesh import build_tiled_mesh
from umt_gb300.quadrature import product_quadrature
from oracle import pyoracle as po
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("perturb,G", [(0.01, 4), (0.06, 3)])
def test_sweep_with_cycle_list_matches_oracle(umtlib, perturb, G):
    m = build_tiled_mesh(3, 3, 2, perturb=perturb, seed=7)
    omega, weight = product_quadrature(4, 4, 1)
    A = len(weight)
    rng = np.random.default_rng(11)
    sigt = np.exp(rng.uniform(np.log(0.5), np.log(50.0), size=(m.nzones, G)))
    tau = 2.0
    psi0 = rng.uniform(0.05, 0.2, size=(A, m.ncornr, G))
    STotal = rng.uniform(0.1, 1.0, size=(m.ncornr, G))
    geo = po.geometry(m)
    S = po.schedule(m, geo[0], geo[1], omega)
    assert S.numCycles.sum() > 0
    # the reference starts the cycle values from the saved flux
    cyc = np.zeros((max(len(S.cycleList), 1), G))
    for a in range(A):
        o = S.cycleOffSet[a]
        for k in range(S.numCycles[a]):
            cyc[o + k] = psi0[a, S.cycleList[o + k]]
    Psi_ref = psi0.copy()
    PsiB_ref = np.zeros((A, m.nbelem, G))
    outs = []
    for save in (False, True):
        Phi, _, cyc = po.set_sweep(m, geo, S, sigt, STotal, tau, omega, weight, Psi_ref, PsiB_ref,
                                   cyclePsi=cyc, savePsi=save, nthreads=1)
        outs.append((Phi.copy(), Psi_ref.copy(), PsiB_ref.copy()))

    umtlib.init(m, omega, weight, G, flags=3 | 8)
    # the cycle list: per direction the corners of every lagged zone
    for a in range(A):
        nh, ncyc = umtlib.schedule_info(a)
        o = S.cycleOffSet[a]
        assert ncyc == len(np.unique(S.cycleList[o:o + S.numCycles[a]])), a
    for prec, tphi, tpsi in ((capi.UMT_FP64, 1e-12, 1e-12), (capi.UMT_FP32, 1e-5, 1e-4)):
        umtlib.set_materials(sigt, None, tau)
        umtlib.set_psi(psi0, None)
        for k, save in enumerate((False, True)):
            PsiB = np.zeros((A, m.nbelem, G))
            Phi = umtlib.sweep(STotal, savePsi=save, PsiB=PsiB, precision=prec)
            ref_phi, ref_psi, ref_psib = outs[k]
            print(f"\nperturb {perturb} precision {prec} sweep {k}: phi err {rel_err(Phi, ref_phi):.2e}")
            assert rel_err(Phi, ref_phi) < tphi
            assert rel_err(PsiB, ref_psib) < tpsi
        Psi, _ = umtlib.get_psi(prec)
        assert rel_err(Psi, outs[1][1]) < tpsi


def test_persistent_mode_refuses_a_cycle_list(umtlib):
    m = build_tiled_mesh(2, 2, 1, perturb=0.06, seed=7)
    omega, weight = product_quadrature(4, 4, 1)
    umtlib.init(m, omega, weight, 2, flags=2 | 8)
    with pytest.raises(capi.UmtError) as e:
        umtlib.set_sweep_mode(1)
    assert e.value.code == capi.UMT_ERR_CYCLE
