"""GPU: the reference driver's uniform problem, cycle by cycle, against the
oracle (PhiTotal, radiation energy and the energy balance of every cycle),
and source iteration with scattering."""
import numpy as np
import pytest

from umt_gb300 import capi
from umt_gb300.problems import uniform_problem, synthetic_problem
from umt_gb300.teton import Teton
from tests.helpers import oracle_cycles, oracle_sweep, rel_err

pytestmark = pytest.mark.gpu


def test_uniform_problem_cycles_fp64(umtlib):
    prob = uniform_problem((2, 2, 2), 2, 2, 2)
    ref = oracle_cycles(prob, 3)
    t = Teton(prob, capi.UMT_FP64, umtlib)
    for k in range(3):
        e = t.radtr()
        assert e["tempIters"] == 2                       # 2 outer iterations + savePsi sweep
        assert rel_err(t.PhiTotal, ref[k]["PhiTotal"]) < 1e-12
        assert abs(e["EnergyRadiation"] / ref[k]["EnergyRadiation"] - 1) < 1e-12
        assert abs(e["PowerEscape"] / ref[k]["PowerEscape"] - 1) < 1e-12
        assert abs(e["EnergyCheck"] - ref[k]["EnergyCheck"]) < 1e-12 * e["EnergyRadiation"]
        # closed balance including absorption: exact up to rounding
        assert abs(e["EnergyCheckClosed"]) < 1e-11 * e["EnergyRadiation"]


def test_config1_ten_cycles_fp64(umtlib):
    """The reference driver's uniform problem at its full size (10^3 tiles,
    24,000 zones, 32 directions, 2 groups) for 10 cycles, every cycle against
    the oracle: PhiTotal, radiation energy, escape and the energy check."""
    prob = uniform_problem((10, 10, 10), 2, 2, 2)
    ref = oracle_cycles(prob, 10)
    t = Teton(prob, capi.UMT_FP64, umtlib)
    for k in range(10):
        e = t.radtr()
        assert rel_err(t.PhiTotal, ref[k]["PhiTotal"]) < 1e-12, k
        assert abs(e["EnergyRadiation"] / ref[k]["EnergyRadiation"] - 1) < 1e-12, k
        assert abs(e["PowerEscape"] / ref[k]["PowerEscape"] - 1) < 1e-12, k
        assert abs(e["EnergyCheck"] - ref[k]["EnergyCheck"]) < 1e-12 * e["EnergyRadiation"], k


def test_uniform_problem_cycles_fp32(umtlib):
    prob = uniform_problem((2, 2, 2), 2, 2, 2)
    ref = oracle_cycles(prob, 2)
    t = Teton(prob, capi.UMT_FP32, umtlib)
    for k in range(2):
        e = t.radtr()
        assert rel_err(t.PhiTotal, ref[k]["PhiTotal"]) < 1e-5
        assert abs(e["EnergyRadiation"] / ref[k]["EnergyRadiation"] - 1) < 1e-5
        assert abs(e["EnergyCheckClosed"]) < 1e-4 * e["EnergyRadiation"]


def _oracle_si(prob, tol, max_iters=200):
    m = prob.mesh
    G = prob.ngr
    phi = np.zeros((m.ncornr, G))
    for it in range(max_iters):
        st = (prob.sigs[m.cToZone] * phi + prob.q_ext[m.cToZone]) / (4 * np.pi)
        r = oracle_sweep(prob, STotal=st, Psi=prob.psi0, savePsi=False)
        new = r["Phi"]
        rel = np.linalg.norm(new - phi) / np.linalg.norm(new)
        phi = new
        if rel < tol:
            return phi, it + 1
    return phi, max_iters


@pytest.mark.parametrize("precision,tol", [(capi.UMT_FP64, 1e-11), (capi.UMT_FP32, 2e-5)])
def test_source_iteration(umtlib, precision, tol):
    prob = synthetic_problem((2, 2, 1), 2, 2, 4, seed=9, c_range=(0.0, 0.5), time_dependent=True)
    phi_ref, it_ref = _oracle_si(prob, 1e-10)
    m = prob.mesh
    umtlib.init(m, prob.omega, prob.weight, prob.ngr)
    umtlib.set_materials(prob.sigt, prob.sigs, prob.tau)
    umtlib.set_psi(prob.psi0, None)
    res = umtlib.source_iterate(precision=precision, rel_tol=1e-10 if precision == 0 else 1e-6,
                                q_ext=prob.q_ext, save_psi=False, max_iters=200)
    phi = umtlib.get_phi()
    assert res["converged"]
    assert rel_err(phi, phi_ref) < tol


def test_gta_accelerates_and_agrees(umtlib):
    """Strong scattering: source iteration with the grey transport correction
    converges to the same PhiTotal as plain iteration, in fewer outer
    iterations.  (Groups here couple only through the grey correction, so one
    grey mode removes part of the error, not all of it.)"""
    prob = synthetic_problem((2, 2, 1), 2, 2, 4, seed=12, sigt_range=(1.0, 30.0), c_range=(0.9, 0.98),
                             time_dependent=True)
    phi_ref, it_ref = _oracle_si(prob, 1e-10, max_iters=2000)
    m = prob.mesh
    out = {}
    for gta in (False, True):
        umtlib.init(m, prob.omega, prob.weight, prob.ngr)
        umtlib.set_materials(prob.sigt, prob.sigs, prob.tau)
        umtlib.set_psi(prob.psi0, None)
        res = umtlib.source_iterate(precision=capi.UMT_FP64, rel_tol=1e-10, q_ext=prob.q_ext, save_psi=False,
                                    max_iters=2000, use_gta=gta)
        assert res["converged"]
        out[gta] = (res, umtlib.get_phi())
    assert rel_err(out[False][1], phi_ref) < 1e-8
    assert rel_err(out[True][1], phi_ref) < 1e-8
    assert out[True][0]["iterations"] < 0.85 * out[False][0]["iterations"]
    assert out[True][0]["grey_sweeps"] > 0


def test_fp32_converged_phi_matches_oracle_source_iteration(umtlib):
    """The time-to-converge comparison's accuracy bar, against the oracle
    itself: the config-2 distribution (sigma_t log-uniform on [1e-2, 1e2],
    c <= 0.5, q = 1, tau = 1/(c dt)) on 6^3 tiles with all 128 directions
    and 16 groups.  The oracle's FP64 source iteration to 1e-10 and the
    FP32 device iteration to 1e-7 relative change end within 1e-6 relative
    L2 of each other, and the FP64 device iteration within 1e-10."""
    import os
    prob = synthetic_problem((6, 6, 6), 4, 4, 16, seed=2, sigt_range=(1e-2, 1e2), c_range=(0.0, 0.5),
                             time_dependent=True)
    m = prob.mesh
    nth = os.cpu_count() or 1
    phi = np.zeros((m.ncornr, prob.ngr))
    for _ in range(200):
        st = (prob.sigs[m.cToZone] * phi + prob.q_ext[m.cToZone]) / (4 * np.pi)
        new = oracle_sweep(prob, STotal=st, Psi=prob.psi0, savePsi=False, nthreads=nth)["Phi"]
        rel = np.linalg.norm(new - phi) / np.linalg.norm(new)
        phi = new
        if rel < 1e-10:
            break
    assert rel < 1e-10
    umtlib.init(m, prob.omega, prob.weight, prob.ngr, flags=3 | 8)
    umtlib.set_materials(prob.sigt, prob.sigs, prob.tau)
    for prec, tol_si, bar in ((capi.UMT_FP32, 1e-7, 1e-6), (capi.UMT_FP64, 1e-10, 1e-10)):
        umtlib.set_psi(prob.psi0, None)
        res = umtlib.source_iterate(precision=prec, rel_tol=tol_si, q_ext=prob.q_ext, save_psi=False, max_iters=200)
        assert res["converged"]
        got = umtlib.get_phi()
        err = float(np.linalg.norm(got - phi) / np.linalg.norm(phi))
        print(f"\nprecision {prec}: converged phi vs oracle, relative L2 {err:.2e} "
              f"({res['iterations']} iterations)")
        assert err < bar
