"""2-D RZ sweep (snac/SweepUCBrz.F90 with SetSweep's RZ angle order) through
the C-ABI against the CPU oracle's restatement."""
import numpy as np
import pytest

from umt_gb300 import capi
from umt_gb300.mesh_rz import build_rz_mesh
from umt_gb300.quadrature_rz import product_quadrature_rz
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu


def _problem(nr, nzr, P, Az, G, seed, distort=0.15):
    m = build_rz_mesh(nr, nzr, distort=distort, seed=seed)
    q = product_quadrature_rz(P, Az)
    rng = np.random.default_rng(seed)
    sigt = rng.uniform(0.2, 20.0, size=(m.nzones, G))
    STotal = rng.uniform(0.05, 1.0, size=(m.ncornr, G))
    psi0 = rng.uniform(0.01, 0.2, size=(len(q.weight), m.ncornr, G))
    PsiB = rng.uniform(0.0, 0.05, size=(len(q.weight), m.nbelem, G))
    return m, q, sigt, STotal, psi0, PsiB


def _oracle(m, q, sigt, STotal, psi0, PsiB, tau):
    from oracle import pyoracle as po
    geo = po.geometry_rz(m)
    om3 = np.zeros((len(q.weight), 3)); om3[:, :2] = q.omega
    S = po.schedule(m, geo["A_fp"], geo["A_ez"], om3)
    assert S.numCycles.sum() == 0
    Psi = psi0.copy(); PB = PsiB.copy()
    Phi = po.set_sweep_rz(m, geo, S, sigt, STotal, tau, om3, q, Psi, PB, savePsi=True)
    return geo, Phi, Psi, PB


@pytest.mark.parametrize("nr,nzr,P,Az,G,index_base", [(4, 3, 2, 2, 4, 0), (6, 5, 4, 3, 8, 0), (3, 4, 1, 2, 1, 1)])
def test_rz_sweep_matches_oracle(umtlib, nr, nzr, P, Az, G, index_base):
    m, q, sigt, STotal, psi0, PsiB = _problem(nr, nzr, P, Az, G, seed=nr * 10 + G)
    tau = 0.7
    geo, Phi_ref, Psi_ref, PsiB_ref = _oracle(m, q, sigt, STotal, psi0, PsiB, tau)
    umtlib.init_rz(m, q, G, index_base=index_base)
    g = umtlib.geometry_rz()
    for k in ("Area", "Volume", "RadiusFP", "RadiusEZ"):
        assert np.array_equal(g[k], geo[k]), k
    umtlib.set_materials(sigt, np.zeros_like(sigt), tau)
    umtlib.set_psi(psi0, None)
    PB = PsiB.copy()
    Phi = umtlib.sweep_rz(STotal, savePsi=True, PsiB=PB)
    Psi, _ = umtlib.get_psi(capi.UMT_FP64)
    assert rel_err(Phi, Phi_ref) < 1e-12
    assert rel_err(Psi, Psi_ref) < 1e-12
    assert rel_err(PB, PsiB_ref) < 1e-12
    # finishing directions carry the level's last half-angle intensity
    fin = np.nonzero(q.finishing)[0]
    assert np.abs(Psi[fin]).max() > 0


def test_rz_repeated_sweeps_and_source_iteration(umtlib):
    """Several sweeps in a row (savePsi on and off) stay equal to the oracle's."""
    m, q, sigt, STotal, psi0, PsiB = _problem(5, 4, 2, 2, 4, seed=3)
    tau = 0.3
    from oracle import pyoracle as po
    geo = po.geometry_rz(m)
    om3 = np.zeros((len(q.weight), 3)); om3[:, :2] = q.omega
    S = po.schedule(m, geo["A_fp"], geo["A_ez"], om3)
    umtlib.init_rz(m, q, 4)
    umtlib.set_materials(sigt, np.zeros_like(sigt), tau)
    umtlib.set_psi(psi0, None)
    Psi_o = psi0.copy()
    for save in (False, True, True):
        PB_o = PsiB.copy(); PB_d = PsiB.copy()
        Phi_o = po.set_sweep_rz(m, geo, S, sigt, STotal, tau, om3, q, Psi_o, PB_o, savePsi=save)
        Phi_d = umtlib.sweep_rz(STotal, savePsi=save, PsiB=PB_d)
        assert rel_err(Phi_d, Phi_o) < 1e-12
        assert rel_err(PB_d, PB_o) < 1e-12


# FP32 RZ sweep: the flux is kept in FP32 (approximate reciprocals, the EZ
# closure divided through by aez^4) and the tallies in FP64.  Stated
# tolerance: 2e-5 relative (max-norm) on PhiTotal, 1e-4 on Psi and PsiB.
FP32_PHI_TOL, FP32_PSI_TOL = 2e-5, 1e-4


@pytest.mark.parametrize("nr,nzr,P,Az,G,index_base", [(6, 5, 4, 3, 8, 0), (7, 6, 2, 4, 16, 1), (3, 4, 1, 2, 3, 0),
                                                    (3, 3, 1, 2, 40, 0)])
def test_rz_fp32_sweep_matches_oracle(umtlib, nr, nzr, P, Az, G, index_base):
    m, q, sigt, STotal, psi0, PsiB = _problem(nr, nzr, P, Az, G, seed=nr * 7 + G)
    tau = 0.7
    geo, Phi_ref, Psi_ref, PsiB_ref = _oracle(m, q, sigt, STotal, psi0, PsiB, tau)
    umtlib.init_rz(m, q, G, index_base=index_base)
    umtlib.set_materials(sigt, np.zeros_like(sigt), tau)
    umtlib.set_psi(psi0, None)
    PB = PsiB.copy()
    Phi = umtlib.sweep_rz(STotal, savePsi=True, PsiB=PB, precision=capi.UMT_FP32)
    Psi, _ = umtlib.get_psi(capi.UMT_FP32)
    assert rel_err(Phi, Phi_ref) < FP32_PHI_TOL
    assert rel_err(Psi, Psi_ref) < FP32_PSI_TOL
    assert rel_err(PB, PsiB_ref) < FP32_PSI_TOL


@pytest.mark.parametrize("precision", [capi.UMT_FP64, capi.UMT_FP32])
def test_rz_mixed_polygons_match_oracle(umtlib, precision):
    """Triangles, quadrilaterals and hexagons in one mesh (the FP32 kernel's
    8-corner instantiation and 3-corner zones)."""
    from umt_gb300.mesh_rz import build_rz_mixed_mesh
    m = build_rz_mixed_mesh(7, 6, distort=0.15, seed=5)
    assert set(np.unique(m.numCorner)) == {3, 4, 6}
    q = product_quadrature_rz(2, 3)
    G = 8
    rng = np.random.default_rng(9)
    sigt = rng.uniform(0.2, 20.0, size=(m.nzones, G))
    STotal = rng.uniform(0.05, 1.0, size=(m.ncornr, G))
    psi0 = rng.uniform(0.01, 0.2, size=(len(q.weight), m.ncornr, G))
    PsiB = rng.uniform(0.0, 0.05, size=(len(q.weight), m.nbelem, G))
    tau = 0.4
    geo, Phi_ref, Psi_ref, PsiB_ref = _oracle(m, q, sigt, STotal, psi0, PsiB, tau)
    umtlib.init_rz(m, q, G)
    g = umtlib.geometry_rz()
    for k in ("Area", "Volume", "RadiusFP", "RadiusEZ"):
        assert np.array_equal(g[k], geo[k]), k
    umtlib.set_materials(sigt, np.zeros_like(sigt), tau)
    umtlib.set_psi(psi0, None)
    PB = PsiB.copy()
    Phi = umtlib.sweep_rz(STotal, savePsi=True, PsiB=PB, precision=precision)
    Psi, _ = umtlib.get_psi(precision)
    tol_phi, tol_psi = (1e-12, 1e-12) if precision == capi.UMT_FP64 else (FP32_PHI_TOL, FP32_PSI_TOL)
    assert rel_err(Phi, Phi_ref) < tol_phi
    assert rel_err(Psi, Psi_ref) < tol_psi
    assert rel_err(PB, PsiB_ref) < tol_psi


def test_rz_fp32_repeated_sweeps_and_tau_change(umtlib):
    """FP32 sweeps replayed from graphs of both buffer parities, and captured
    again after tau changes, stay within the FP32 tolerance of the oracle."""
    m, q, sigt, STotal, psi0, PsiB = _problem(5, 6, 2, 3, 16, seed=11)
    from oracle import pyoracle as po
    geo = po.geometry_rz(m)
    om3 = np.zeros((len(q.weight), 3)); om3[:, :2] = q.omega
    S = po.schedule(m, geo["A_fp"], geo["A_ez"], om3)
    umtlib.init_rz(m, q, 16)
    umtlib.set_psi(psi0, None)
    Psi_o = psi0.copy()
    for tau, save in ((0.3, True), (0.3, False), (0.3, True), (1.1, True), (1.1, True)):
        umtlib.set_materials(sigt, np.zeros_like(sigt), tau)
        PB_o = PsiB.copy(); PB_d = PsiB.copy()
        Phi_o = po.set_sweep_rz(m, geo, S, sigt, STotal, tau, om3, q, Psi_o, PB_o, savePsi=save)
        Phi_d = umtlib.sweep_rz(STotal, savePsi=save, PsiB=PB_d, precision=capi.UMT_FP32)
        assert rel_err(Phi_d, Phi_o) < FP32_PHI_TOL
        assert rel_err(PB_d, PB_o) < FP32_PSI_TOL
    Psi_d, _ = umtlib.get_psi(capi.UMT_FP32)
    assert rel_err(Psi_d, Psi_o) < FP32_PSI_TOL


@pytest.mark.parametrize("precision", [capi.UMT_FP64, capi.UMT_FP32])
def test_rz_sweep_writes_only_exiting_psib_rows(umtlib, precision):
    """The caller's PsiB changes only on the rows the sweep writes (exits,
    and a finishing direction's rows on its predecessor's exits): every row
    the oracle leaves unchanged keeps its FP64 input bit for bit."""
    m, q, sigt, STotal, psi0, PsiB = _problem(5, 4, 2, 3, 8, seed=21)
    tau = 0.6
    geo, Phi_ref, Psi_ref, PsiB_ref = _oracle(m, q, sigt, STotal, psi0, PsiB, tau)
    umtlib.init_rz(m, q, 8)
    umtlib.set_materials(sigt, np.zeros_like(sigt), tau)
    umtlib.set_psi(psi0, None)
    PB = PsiB.copy()
    umtlib.sweep_rz(STotal, savePsi=True, PsiB=PB, precision=precision)
    kept = np.all(PsiB_ref == PsiB, axis=2)
    assert kept.any() and (~kept).any()
    assert np.array_equal(PB[kept], PsiB[kept])
    tol = 1e-12 if precision == capi.UMT_FP64 else FP32_PSI_TOL
    assert rel_err(PB[~kept], PsiB_ref[~kept]) < tol


def test_rz_precision_refusals(umtlib):
    m, q, sigt, STotal, psi0, PsiB = _problem(2, 3, 1, 1, 2, seed=4)
    umtlib.init_rz(m, q, 2, flags=1)                     # FP64 flux only
    umtlib.set_materials(sigt, np.zeros_like(sigt), 0.5)
    with pytest.raises(capi.UmtError) as e:
        umtlib.sweep_rz(STotal, precision=capi.UMT_FP32)
    assert e.value.code == capi.UMT_ERR_STATE
    with pytest.raises(capi.UmtError) as e:
        umtlib.sweep_rz(STotal, precision=7)
    assert e.value.code == capi.UMT_ERR_ARG
    umtlib.init_rz(m, q, 2, flags=2)                     # FP32 flux only
    umtlib.set_materials(sigt, np.zeros_like(sigt), 0.5)
    with pytest.raises(capi.UmtError) as e:
        umtlib.sweep_rz(STotal, precision=capi.UMT_FP64)
    assert e.value.code == capi.UMT_ERR_STATE
    assert np.isfinite(umtlib.sweep_rz(STotal, precision=capi.UMT_FP32)).all()
    with pytest.raises(capi.UmtError) as e:              # the 3-D sweep refuses an RZ context
        umtlib.sweep(STotal, precision=capi.UMT_FP32)
    assert e.value.code == capi.UMT_ERR_STATE
    # the 3-D energy edits (3-D boundary projections) refuse an RZ context too
    with pytest.raises(capi.UmtError) as e:
        umtlib.tally(None, precision=capi.UMT_FP32)
    assert e.value.code == capi.UMT_ERR_STATE
    with pytest.raises(capi.UmtError) as e:
        umtlib.tally_noalloc(None, precision=capi.UMT_FP32)
    assert e.value.code == capi.UMT_ERR_STATE


def test_rz_errors(umtlib):
    m, q, sigt, STotal, psi0, PsiB = _problem(2, 2, 1, 1, 2, seed=1)
    bad = product_quadrature_rz(1, 1)
    bad.finishing = bad.finishing.copy(); bad.finishing[-1] = False       # last level never finishes
    with pytest.raises(capi.UmtError) as e:
        umtlib.init_rz(m, bad, 2)
    assert e.value.code == capi.UMT_ERR_ARG
    umtlib.init(*_tiny3d())
    with pytest.raises(capi.UmtError) as e:
        umtlib.sweep_rz(None)
    assert e.value.code == capi.UMT_ERR_STATE


def _tiny3d():
    from umt_gb300.problems import uniform_problem
    p = uniform_problem((1, 1, 1), 1, 1, 2)
    return p.mesh, p.omega, p.weight, p.ngr
