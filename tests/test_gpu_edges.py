"""Edge cases of the sweep through the C-ABI: one group, one tile, the Fortran
(1-based) index path, the largest direction set of the product quadrature,
zero inputs, extreme opacities, and argument / call-order errors."""
import numpy as np
import pytest

from umt_gb300 import capi
from umt_gb300.problems import synthetic_problem, uniform_problem
from tests.helpers import oracle_sweep, rel_err

pytestmark = pytest.mark.gpu


def _sweep(lib, prob, precision, STotal=None, index_base=0, flags=0):
    m = prob.mesh
    lib.init(m, prob.omega, prob.weight, prob.ngr, flags=flags, index_base=index_base)
    lib.set_materials(prob.sigt, prob.sigs, prob.tau)
    lib.set_psi(prob.psi0, None)
    PsiB = np.zeros((len(prob.weight), m.nbelem, prob.ngr))
    Phi = lib.sweep(STotal, savePsi=True, PsiB=PsiB, precision=precision)
    return Phi, PsiB


@pytest.mark.parametrize("precision,tol", [(capi.UMT_FP64, 1e-12), (capi.UMT_FP32, 1e-5)])
def test_one_group_one_tile(umtlib, precision, tol):
    prob = uniform_problem((1, 1, 1), 2, 2, 1)
    ref = oracle_sweep(prob, Psi=prob.psi0)
    Phi, PsiB = _sweep(umtlib, prob, precision)
    assert rel_err(Phi, ref["Phi"]) < tol
    assert rel_err(PsiB, ref["PsiB"]) < 10 * tol


def test_fortran_index_base_gives_identical_results(umtlib):
    prob = synthetic_problem((2, 1, 2), 2, 2, 4, seed=13, time_dependent=True)
    STotal = np.repeat(prob.q_ext, prob.mesh.numCorner, axis=0) / (4 * np.pi)
    out = [_sweep(umtlib, prob, capi.UMT_FP64, STotal, index_base=b) for b in (0, 1)]
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("precision,tol", [(capi.UMT_FP64, 1e-12), (capi.UMT_FP32, 1e-5)])
def test_512_directions(umtlib, precision, tol):
    """P = Az = 8: 512 directions (the product tables go up to 32 x 32)."""
    prob = synthetic_problem((1, 1, 1), 8, 8, 4, seed=14, time_dependent=True)
    assert len(prob.weight) == 512
    STotal = np.repeat(prob.q_ext, prob.mesh.numCorner, axis=0) / (4 * np.pi)
    ref = oracle_sweep(prob, STotal=STotal, Psi=prob.psi0)
    Phi, PsiB = _sweep(umtlib, prob, precision, STotal)
    assert rel_err(Phi, ref["Phi"]) < tol
    assert rel_err(PsiB, ref["PsiB"]) < 10 * tol


@pytest.mark.parametrize("precision", [capi.UMT_FP64, capi.UMT_FP32])
def test_zero_source_and_flux_give_zero(umtlib, precision):
    prob = synthetic_problem((2, 2, 1), 2, 2, 8, seed=15, time_dependent=True)
    prob.psi0 = np.zeros_like(prob.psi0)
    Phi, PsiB = _sweep(umtlib, prob, precision, STotal=None)
    assert not Phi.any() and not PsiB.any()
    t = umtlib.tally(prob.siga, precision=precision)
    assert t["EnergyRadiation"] == 0.0 and t["PowerEscape"] == 0.0 and t["PowerAbsorbed"] == 0.0


@pytest.mark.parametrize("sig_max,tol32", [(1e6, 1e-5), (1e12, 1e-4)])
def test_extreme_opacities(umtlib, sig_max, tol32):
    """Optically very thick zones: at sigma_t = 1e12 the FP32 closure's x is
    capped at 1e8; FP64 still matches the oracle to 1e-12."""
    prob = synthetic_problem((2, 2, 1), 2, 2, 8, seed=16, sigt_range=(1e-2, sig_max), time_dependent=True)
    STotal = np.repeat(prob.q_ext, prob.mesh.numCorner, axis=0) / (4 * np.pi)
    ref = oracle_sweep(prob, STotal=STotal, Psi=prob.psi0)
    Phi64, _ = _sweep(umtlib, prob, capi.UMT_FP64, STotal)
    assert rel_err(Phi64, ref["Phi"]) < 1e-12
    Phi32, PsiB32 = _sweep(umtlib, prob, capi.UMT_FP32, STotal)
    assert np.isfinite(Phi32).all() and np.isfinite(PsiB32).all()
    assert rel_err(Phi32, ref["Phi"]) < tol32


def test_argument_and_call_order_errors(umtlib):
    prob = synthetic_problem((1, 1, 1), 2, 2, 4, seed=18, time_dependent=True)
    m = prob.mesh
    umtlib.init(m, prob.omega, prob.weight, prob.ngr, flags=1 | 8)      # FP64 flux only
    umtlib.set_materials(prob.sigt, prob.sigs, prob.tau)
    with pytest.raises(capi.UmtError) as e:
        umtlib.sweep(None, precision=7)
    assert e.value.code == capi.UMT_ERR_ARG
    with pytest.raises(capi.UmtError) as e:
        umtlib.sweep(None, precision=capi.UMT_FP32)
    assert e.value.code == capi.UMT_ERR_STATE
    with pytest.raises(capi.UmtError) as e:
        umtlib.sweep_resident(False, 3)
    assert e.value.code == capi.UMT_ERR_ARG
    with pytest.raises(capi.UmtError) as e:
        umtlib.tally(prob.siga, precision=9)
    assert e.value.code == capi.UMT_ERR_ARG
    with pytest.raises(capi.UmtError) as e:
        umtlib.set_sweep_mode(9)
    assert e.value.code == capi.UMT_ERR_ARG
    with pytest.raises(capi.UmtError) as e:
        umtlib.set_group_tile(3, 1)                                    # 3 lanes do not cover 4 groups
    assert e.value.code == capi.UMT_ERR_ARG
    with pytest.raises(capi.UmtError) as e:
        umtlib.set_materials(-prob.sigt, prob.sigs, prob.tau)
    assert e.value.code == capi.UMT_ERR_ARG
    bad = prob.mesh
    cfp = bad.cFP.copy()
    bad.cFP[0, 0] = m.ncornr + m.nbelem + 5                            # out of range
    try:
        with pytest.raises(capi.UmtError) as e:
            umtlib.init(bad, prob.omega, prob.weight, prob.ngr)
        assert e.value.code == capi.UMT_ERR_ARG
    finally:
        bad.cFP[...] = cfp
    # the library stays usable after every refused call
    Phi, _ = _sweep(umtlib, prob, capi.UMT_FP64)
    assert np.isfinite(Phi).all()


@pytest.mark.parametrize("item", ["first", "last"])
def test_persistent_wait_times_out_and_context_recovers(umtlib, item):
    """Failure detection without a GPU fault: one work item is given an
    upwind dependency nothing satisfies (a host-side injection).  The
    persistent sweep's bounded wait gives up, the call returns
    UMT_ERR_TIMEOUT within about a second, and the next sweep of the same
    context gives the undisturbed result again."""
    import time
    prob = synthetic_problem((2, 2, 1), 2, 2, 8, seed=6, time_dependent=True)
    m = prob.mesh
    A = len(prob.weight)
    STotal = np.repeat(prob.q_ext, m.numCorner, axis=0) / (4 * np.pi)
    umtlib.init(m, prob.omega, prob.weight, prob.ngr, flags=2 | 8)
    umtlib.set_materials(prob.sigt, prob.sigs, prob.tau)
    umtlib.set_sweep_mode(1)
    umtlib.set_psi(prob.psi0, None)
    ref = umtlib.sweep(STotal, savePsi=False, precision=capi.UMT_FP32)
    umtlib.hold_item(0 if item == "first" else A * m.nzones - 1)
    t0 = time.perf_counter()
    with pytest.raises(capi.UmtError) as e:
        umtlib.sweep(STotal, savePsi=False, precision=capi.UMT_FP32)
    assert e.value.code == capi.UMT_ERR_TIMEOUT
    assert time.perf_counter() - t0 < 30
    again = umtlib.sweep(STotal, savePsi=False, precision=capi.UMT_FP32)
    assert np.array_equal(again, ref)
    with pytest.raises(capi.UmtError) as e:
        umtlib.hold_item(A * m.nzones)
    assert e.value.code == capi.UMT_ERR_ARG
    umtlib.set_sweep_mode(0)
