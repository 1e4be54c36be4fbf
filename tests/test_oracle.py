"""CPU tests: the oracle against the reference's golden vectors and against
the conservation identities of the UCB discretisation; mesh, quadrature and
schedule invariants."""
import json
import os
import re

import numpy as np
import pytest

from oracle import pyoracle as po
from umt_gb300 import problems
from umt_gb300.mesh import build_tiled_mesh
from umt_gb300.quadrature import product_quadrature
from tests.helpers import oracle_sweep, rel_err

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_mesh_geometry_invariants():
    m = build_tiled_mesh(2, 2, 2)
    assert m.nzones == 192 and m.numCorner.max() == 8 and (m.nCFaces == 3).all()
    A_fp, A_ez, vol, volz, A_bdy = po.geometry(m)
    # corner surfaces close, volumes tile the unit cube, boundary closes
    assert np.abs(A_fp.sum(1) + A_ez.sum(1)).max() < 1e-15
    assert abs(vol.sum() - 1.0) < 1e-13 and (vol > 0).all()
    assert np.abs(A_bdy.sum(0)).max() < 1e-14
    # FP normals point out of the zone, EZ normals toward the neighbour corner
    zc = np.zeros((m.nzones, 3)); np.add.at(zc, m.cToZone, m.px); zc /= m.numCorner[:, None]
    assert ((A_fp * (m.px[:, None, :] - zc[m.cToZone][:, None, :])).sum(2) > 0).all()
    pc = m.px[m.cOffSet[m.cToZone][:, None] + m.cEZ]
    assert ((A_ez * (pc - m.px[:, None, :])).sum(2) > 0).all()
    # FP area vectors of shared faces are equal and opposite
    inner = m.cFP < m.ncornr
    ci, fi = np.nonzero(inner)
    for c, f in zip(ci[:500], fi[:500]):
        o = m.cFP[c, f]
        k = int(np.nonzero(m.cFP[o] == c)[0][0])
        assert np.array_equal(A_fp[c, f], -A_fp[o, k])


def test_tile_statistics():
    m = build_tiled_mesh(10, 10, 10)
    assert m.nzones == 24000
    assert abs(m.ncornr / m.nzones - 7.333) < 0.01


@pytest.mark.parametrize("P,Az", [(2, 2), (4, 4), (1, 3)])
def test_product_quadrature(P, Az):
    om, w = product_quadrature(P, Az)
    assert om.shape == (8 * P * Az, 3)
    assert abs(w.sum() - 4 * np.pi) < 1e-12
    assert np.abs(np.linalg.norm(om, axis=1) - 1).max() < 1e-15
    assert np.abs((w[:, None] * om).sum(0)).max() < 1e-13
    # octant blocks of 8 share a magnitude pattern (quadProduct.F90:122-182)
    blk = np.abs(om).reshape(-1, 8, 3)
    assert np.array_equal(blk, np.broadcast_to(blk[:, :1], blk.shape))


def test_planck_against_reference_golden():
    d = json.load(open(os.path.join(GOLDEN, "planck_nbb.json")))
    for case in d["cases"]:
        gnu = np.array(case["gnu"]); B = np.array(case["B"])
        mine = problems.planck_groups(case["T"], case["k"], case["bnorm"], gnu)
        orc = po.planck_groups(case["T"], case["k"], case["bnorm"], gnu)
        assert np.allclose(mine, B, rtol=1e-14, atol=0)
        assert np.allclose(orc, B, rtol=1e-14, atol=0)


def test_schedule_is_a_valid_topological_order():
    prob = problems.uniform_problem((3, 2, 2), 2, 2, 2)
    m = prob.mesh
    A_fp, A_ez, *_ = po.geometry(m)
    S = po.schedule(m, A_fp, A_ez, prob.omega)
    assert S.numCycles.sum() == 0
    for a in range(len(prob.weight)):
        lev = np.full(m.nzones, -1)
        pos = 0
        for h in range(S.nHyperPlanes[a]):
            n = S.zonesInPlane[a, h]
            lev[np.abs(S.nextZ[a, pos:pos + n])] = h
            pos += n
        assert (lev >= 0).all() and pos == m.nzones
        # every corner face with flow into the corner comes from an earlier plane
        afp = (A_fp * prob.omega[a]).sum(2)
        inflow = (afp < 0) & (m.cFP < m.ncornr)
        c, f = np.nonzero(inflow)
        up = m.cToZone[m.cFP[c, f]]
        assert (lev[up] < lev[m.cToZone[c]]).all()


def _balance(prob, res, STotal):
    """Per-direction particle balance of the UCB equations (exact identity)."""
    m = prob.mesh
    geo = res["geo"]
    A_fp, vol = geo[0], geo[2]
    A = len(prob.weight)
    sigt_c = prob.sigt[m.cToZone]
    out = 0.0; inc = 0.0; src = 0.0; rem = 0.0
    Psi_old = prob.psi0
    for a in range(A):
        afp = (A_fp * prob.omega[a]).sum(2)
        bd = m.cFP >= m.ncornr
        c, f = np.nonzero(bd & (afp > 0))
        w = prob.weight[a]
        out += w * (afp[c, f][:, None] * res["Psi"][a, c]).sum()
        src += w * (vol[:, None] * (STotal + prob.tau * Psi_old[a])).sum()
        rem += w * (sigt_c * vol[:, None] * res["Psi"][a]).sum()
    return out + rem - src - inc, src


def test_oracle_sweep_conserves():
    prob = problems.synthetic_problem((2, 2, 1), 2, 2, 4, seed=5, time_dependent=True)
    STotal = np.ones((prob.mesh.ncornr, 4)) * 0.3
    res = oracle_sweep(prob, STotal=STotal, Psi=prob.psi0)
    resid, scale = _balance(prob, res, STotal)
    assert abs(resid) / scale < 1e-13
    # the tally is the weighted sum of the saved angular flux
    phi = np.einsum("a,acg->cg", prob.weight, res["Psi"])
    assert rel_err(res["Phi"], phi) < 1e-14


def test_oracle_threads_match_serial():
    prob = problems.uniform_problem((2, 2, 2), 2, 2, 2)
    r1 = oracle_sweep(prob, Psi=prob.psi0, nthreads=1)
    r4 = oracle_sweep(prob, Psi=prob.psi0, nthreads=4)
    assert rel_err(r4["Phi"], r1["Phi"]) < 1e-14
    assert np.array_equal(r4["Psi"], r1["Psi"])


@pytest.mark.parametrize("name", ["uniform_1x1x2_a32_g4", "synthetic_2x1x1_a128_g8"])
def test_oracle_against_reference_cuda_kernel(name):
    """Golden outputs of the reference's own CUDA sweep (tests/golden/gen_ref_sweep.py)."""
    path = os.path.join(GOLDEN, f"ref_sweep_{name}.npz")
    if not os.path.exists(path):
        pytest.skip("golden file not generated")
    from tests.golden import gen_ref_sweep as gen
    prob, STotal, geo, S = gen.build_inputs(name)
    g = np.load(path)
    assert str(g["digest"]) == gen.input_digest(prob, STotal, geo, S)
    assert np.allclose(g["sums"], gen.input_sums(prob, STotal, geo), rtol=1e-13, atol=0)
    res = oracle_sweep(prob, STotal=STotal, Psi=prob.psi0)
    assert rel_err(res["Phi"], g["Phi"]) < 1e-13
    keep = g["keep"] if "keep" in g.files else np.arange(len(prob.weight))
    assert rel_err(res["Psi"][keep], g["Psi"]) < 1e-13
    assert rel_err(res["PsiB"][keep], g["PsiB"]) < 1e-13


def test_gta_restatement_properties():
    """The CPU grey step: no residual gives no correction; the grey operator
    is linear in P; S2 weights sum to 4 pi."""
    from oracle import gta_oracle as go
    from umt_gb300.problems import synthetic_problem
    om, w = go.s2_quadrature()
    assert abs(w.sum() - 4 * np.pi) < 1e-12 and np.allclose((om * om).sum(1), 1.0)
    prob = synthetic_problem((2, 1, 1), 1, 1, 3, seed=5, c_range=(0.5, 0.9), time_dependent=True)
    m = prob.mesh
    phi = np.random.default_rng(1).uniform(0.5, 1.5, size=(m.ncornr, 3))
    x, chi, n = go.gta_correction(m, np.ascontiguousarray(prob.sigt), np.ascontiguousarray(prob.sigs), prob.tau,
                                  phi, phi.copy())
    assert np.all(x == 0.0)
    assert np.allclose(chi.sum(1) * 0 + 1, 1)
    gp = go.GreyProblem(m)
    sig = np.full(m.nzones, 2.0)
    a = np.random.default_rng(2).uniform(size=m.ncornr)
    b = np.random.default_rng(3).uniform(size=m.ncornr)
    lhs = gp.sweep(sig, 2.0 * a + 3.0 * b)
    rhs = 2.0 * gp.sweep(sig, a) + 3.0 * gp.sweep(sig, b)
    assert np.abs(lhs - rhs).max() <= 1e-13 * np.abs(rhs).max()


def test_gta_zone_solver_restatement():
    """The restatement of the newer grey solver (InitSweepGreyUCBxyz,
    SweepGreyUCBxyzKernelNew, ScalarIntensityDecompose/Solve): its literal
    grey sweep equals the oracle's C++ sweep; the inflow part PhiInc it
    accumulates equals tPhi - TT TsaSource (the identity the device uses);
    the LU solve inverts A = I - TT wtiso sigma_s; and at a tight tolerance
    the newer and the older solver reach the same grey correction."""
    from oracle import gta_oracle as go
    from umt_gb300.problems import synthetic_problem
    prob = synthetic_problem((2, 2, 1), 2, 2, 4, seed=41, sigt_range=(0.5, 50.0), c_range=(0.5, 0.95),
                             time_dependent=True)
    m = prob.mesh
    rng = np.random.default_rng(42)
    phi = rng.uniform(0.5, 1.5, size=(m.ncornr, 4))
    prev = phi * rng.uniform(0.9, 1.1, size=phi.shape)
    gp = go.GreyProblem(m)
    _, gt, gs = go.spectrum(m, gp.geo[2], prob.sigt, prob.sigs, prob.tau, phi, prev)
    gtc, gsc = gt[m.cToZone], gs[m.cToZone]
    TT = go.init_grey_tt(gp, gtc)
    tsa = rng.uniform(0.1, 1.0, m.ncornr)
    tphi, pinc = go.grey_sweep_new(gp, gtc, tsa)
    ref = gp.sweep(gt, tsa)
    assert np.abs(tphi - ref).max() <= 1e-14 * np.abs(ref).max()
    alt = tphi.copy()
    for z in range(m.nzones):
        c0, nC = m.cOffSet[z], m.numCorner[z]
        alt[c0:c0 + nC] -= TT[c0:c0 + nC, :nC] @ tsa[c0:c0 + nC]
    assert np.abs(alt - pinc).max() <= 1e-13 * np.abs(pinc).max()
    z = 3
    c0, nC = m.cOffSet[z], m.numCorner[z]
    A = np.eye(nC) - TT[c0:c0 + nC, :nC] * (go.WTISO * gsc[c0:c0 + nC])[None, :]
    b = rng.uniform(size=nC)
    x = np.array(go.zone_solve(go.zone_decompose(m, TT, gsc, z), b))
    assert np.abs(A @ x - b).max() <= 1e-13 * np.abs(b).max()
    args = (m, np.ascontiguousarray(prob.sigt), np.ascontiguousarray(prob.sigs), prob.tau, phi, prev)
    xn, _, sn = go.gta_correction_new(*args, maxit=200, tol=1e-10)
    xo, _, so = go.gta_correction(*args, maxit=200, tol=1e-10)
    assert np.abs(xn - xo).max() <= 1e-9 * np.abs(xo).max()
    assert sn < so
