"""Size-independent properties at the full size of the multigroup scattering
workload: 20^3 tiles (192,000 zones, 1,408,000 corners), 128 directions,
16 groups.

The oracle cannot sweep this size in seconds, so the device sweep is checked
against an identity that holds at any size.  Summed over a zone's corners the
UCB equations conserve particles: EZ couplings cancel pairwise inside a zone,
FP fluxes across interior faces cancel between the two zones, and what is
left, weighted by direction and summed over groups, is

    sum_c V_c sum_g sigma_t,g phi_g  +  PowerEscape  -  PowerIncident
        =  sum_c V_c sum_g ( W * STotal_g + tau * phi_old_g ),   W = sum_a w_a

(rt/rtedit.F90 and control/BoundaryEdit.F90 give the escape and incident
powers; the tally's absorbed power with sigma_t in place of sigma_a gives the
first term).
"""
import numpy as np
import pytest

from umt_gb300 import capi
from umt_gb300.problems import synthetic_problem

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def workload():
    return synthetic_problem((20, 20, 20), 4, 4, 16, seed=2, sigt_range=(1e-2, 1e2), c_range=(0.0, 0.5),
                             time_dependent=True)


# FP32 flux: stated tolerance 1e-5 relative; FP64: 1e-11
@pytest.mark.parametrize("precision,tol", [(capi.UMT_FP32, 1e-5), (capi.UMT_FP64, 1e-11)])
def test_particle_balance_at_full_size(umtlib, workload, precision, tol):
    prob = workload
    m = prob.mesh
    A, G = len(prob.weight), prob.ngr
    flags = (2 if precision == capi.UMT_FP32 else 1) | 8          # one precision, no grey context
    umtlib.init(m, prob.omega, prob.weight, G, flags=flags)
    umtlib.set_materials(prob.sigt, prob.sigs, prob.tau)
    umtlib.set_psi(prob.psi0, None)
    rng = np.random.default_rng(7)
    STotal = rng.uniform(0.05, 1.0, size=(m.ncornr, G))
    PsiB = np.zeros((A, m.nbelem, G))
    Phi = umtlib.sweep(STotal, savePsi=True, PsiB=PsiB, precision=precision)
    t = umtlib.tally(prob.sigt, precision=precision)              # "absorbed" = sum V sigma_t phi
    _, _, vol = umtlib.geometry()
    W = prob.weight.sum()
    phi_old = np.einsum("a,acg->cg", prob.weight, prob.psi0)
    rhs = float((vol[:, None] * (W * STotal + prob.tau * phi_old)).sum())
    lhs = t["PowerAbsorbed"] + t["PowerEscape"] - t["PowerIncident"]
    assert t["PowerIncident"] == 0.0                              # vacuum boundaries
    assert t["PowerEscape"] > 0.0
    assert abs(lhs - rhs) <= tol * rhs, (lhs, rhs, (lhs - rhs) / rhs)
    # the same first term from the returned PhiTotal
    sig_c = prob.sigt[m.cToZone]
    first = float((vol[:, None] * sig_c * Phi).sum())
    assert abs(first - t["PowerAbsorbed"]) <= 1e-12 * abs(first)
    assert np.isfinite(Phi).all() and (Phi > 0).all()
