"""Golden sweep outputs from the reference's own CUDA sweep kernel.

The UMT repository ships a CUDA implementation of SweepUCBxyz
(src/teton/gpu/GPU_SweepUCBxyz.cu: compAfpKernel :141-160, CompSTotalTauPsi
:162-170, SweepUCBxyzKernel :172-516).  oracle/ref_build.py compiles its
device code, unmodified, into oracle/_ref/ref_sweep.cubin.  This script
plays the part of its host driver gpu_sweepucbxyz (:532-994) for one
direction after another -- Psi1 carried from direction to direction, tau*Psi
folded into the source, Phi accumulated over all directions, PsiB exits,
savePsi -- on inputs built from this repository's mesh, geometry and
schedule, and writes the results to tests/golden/ref_sweep_<case>.npz.

Runs on a GPU host (needs the cubin next to it and torch for device memory):

    python tests/golden/gen_ref_sweep.py OUTDIR

Every launch is checked on the host first: the kernel indexes groups in
blocks of 4 and corner-face projections with stride 3, so only G % 4 == 0,
maxcf == 3 and <= 8 corners per zone are run; the cycle-list kernels are not
needed because the meshes used have no mesh cycles.
"""
import ctypes as C
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

CASES = {
    # name: (tiles, npolar, nazimuthal, G, seed or None for the uniform problem, with STotal)
    "uniform_1x1x2_a32_g4": ((1, 1, 2), 2, 2, 4, None, False),
    "synthetic_2x1x1_a128_g8": ((2, 1, 1), 4, 4, 8, 11, True),
}


def build_inputs(name):
    from umt_gb300.problems import uniform_problem, synthetic_problem
    from oracle import pyoracle as po
    tiles, P, Az, G, seed, with_src = CASES[name]
    if seed is None:
        prob = uniform_problem(tiles, P, Az, G)
        STotal = np.zeros((prob.mesh.ncornr, G))
    else:
        prob = synthetic_problem(tiles, P, Az, G, seed=seed, time_dependent=True)
        rng = np.random.default_rng(seed)
        STotal = rng.uniform(0.05, 1.0, size=(prob.mesh.ncornr, G))
        prob.psi0 = prob.psi0 * rng.uniform(0.5, 1.5, size=prob.psi0.shape)
    m = prob.mesh
    geo = po.geometry(m)
    S = po.schedule(m, geo[0], geo[1], prob.omega)
    return prob, STotal, geo, S


def input_digest(prob, STotal, geo, S):
    """Hash of the integer inputs (connectivity and schedule)."""
    h = hashlib.sha256()
    for a in (S.nextZ, S.nextC, S.zonesInPlane, prob.mesh.cFP, prob.mesh.cEZ):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def input_sums(prob, STotal, geo):
    """Sums of the floating-point inputs (checked to a tolerance)."""
    return np.array([np.abs(x).sum() for x in (prob.omega, prob.weight, prob.sigt, STotal, prob.psi0,
                                               geo[0], geo[1], geo[2])])


def run(name, outdir):
    import torch
    prob, STotal, geo, S = build_inputs(name)
    m = prob.mesh
    A, G, nc, nb, nz = len(prob.weight), prob.ngr, m.ncornr, m.nbelem, m.nzones
    # ---- host-side checks of every index the kernels will use ----
    assert G % 4 == 0, "kernel handles groups in blocks of 4"
    assert int(m.numCorner.max()) <= 8 and (m.nCFaces == 3).all()
    assert int(S.numCycles.sum()) == 0, "no cycle list expected"
    assert (m.cFP >= 0).all() and (m.cFP < nc + nb).all()
    assert (m.cEZ >= 0).all() and (m.cEZ < m.numCorner[m.cToZone][:, None]).all()
    for a in range(A):
        assert S.zonesInPlane[a, :S.nHyperPlanes[a]].sum() == nz

    dev = torch.device("cuda:0")
    torch.zeros(1, device=dev)          # creates the primary context
    torch.cuda.synchronize()
    cuda = C.CDLL("libcuda.so.1")
    ctx = C.c_void_p()
    assert cuda.cuCtxGetCurrent(C.byref(ctx)) == 0 and ctx.value
    mod = C.c_void_p()
    cubin = os.path.join(ROOT, "oracle", "_ref", "ref_sweep.cubin")
    assert cuda.cuModuleLoad(C.byref(mod), cubin.encode()) == 0, "cuModuleLoad failed"

    def fn(nm):
        f = C.c_void_p()
        assert cuda.cuModuleGetFunction(C.byref(f), mod, nm.encode()) == 0, nm
        return f

    k_afp, k_tau, k_sweep = fn("compAfpKernel"), fn("CompSTotalTauPsi"), fn("SweepUCBxyzKernel")
    SMEM = 98304
    assert cuda.cuFuncSetAttribute(k_sweep, 8, SMEM) == 0   # MAX_DYNAMIC_SHARED_SIZE_BYTES

    def T(x, dt):
        return torch.as_tensor(np.ascontiguousarray(x, dtype=dt), device=dev)

    f64, i32 = np.float64, np.int32
    d_Afp = T(geo[0], f64); d_Aez = T(geo[1], f64); d_vol = T(geo[2], f64)
    d_sigt = T(prob.sigt, f64)
    d_ncf = T(m.nCFaces, i32)
    d_cFP = T(m.cFP + 1, i32); d_cEZ = T(m.cEZ + 1, i32)
    d_numC = T(m.numCorner, i32); d_coff = T(m.cOffSet, i32)
    d_psi1 = torch.zeros((nc + nb) * G, dtype=torch.float64, device=dev)
    d_phi = torch.zeros(nc * G, dtype=torch.float64, device=dev)
    d_afp = torch.zeros(nc * 3, dtype=torch.float64, device=dev)
    d_aez = torch.zeros(nc * 3, dtype=torch.float64, device=dev)
    nblocks = (G + 3) // 4
    d_bdy = torch.zeros(nblocks * 32 * 2 * 3 * 8, dtype=torch.int32, device=dev)
    Psi = np.ascontiguousarray(prob.psi0, f64).copy()
    PsiB = np.zeros((A, nb, G))
    d_ST = T(STotal, f64)

    def launch(f, grid, block, smem, args):
        holders = []
        for kind, v in args:
            if kind == "i":
                holders.append(C.c_int(int(v)))
            elif kind == "u":
                holders.append(C.c_uint(int(v)))
            elif kind == "d":
                holders.append(C.c_double(float(v)))
            else:
                holders.append(C.c_void_p(v.data_ptr()))
        params = (C.c_void_p * len(holders))(*[C.cast(C.pointer(h), C.c_void_p) for h in holders])
        rc = cuda.cuLaunchKernel(f, grid, 1, 1, block, 1, 1, smem, None, params, None)
        assert rc == 0, rc

    for a in range(A):
        nh = int(S.nHyperPlanes[a])
        nextZ = S.nextZ[a].astype(np.int64)
        nextZ1 = np.where(nextZ >= 0, nextZ + 1, nextZ).astype(i32)   # Fortran sign convention
        d_nextZ = T(nextZ1, i32)
        d_nextC = T(S.nextC[a] + 1, i32)
        d_zip = T(S.zonesInPlane[a, :nh], i32)
        d_om = T(prob.omega[a], f64)
        d_psib = T(PsiB[a].reshape(-1), f64)
        d_psi1[nc * G:] = d_psib
        d_src = d_ST.clone()
        d_psi = T(Psi[a], f64)
        launch(k_afp, 4, 512, 0, [("p", d_om), ("p", d_Afp), ("p", d_afp), ("p", d_Aez), ("p", d_aez),
                                  ("u", nc * 3), ("u", 3)])
        launch(k_tau, 4, 1024, 0, [("p", d_src), ("p", d_psi), ("d", prob.tau), ("i", nc * G)])
        launch(k_sweep, nblocks, 128, SMEM,
               [("i", a + 1), ("i", nh), ("p", d_zip), ("p", d_nextZ), ("p", d_nextC), ("p", d_src),
                ("d", prob.tau), ("i", G), ("p", d_vol), ("p", d_sigt), ("p", d_ncf), ("i", 3), ("i", 3),
                ("i", nc), ("p", d_om), ("p", d_cFP), ("p", d_bdy), ("p", d_psi1), ("p", d_cEZ),
                ("d", prob.weight[a]), ("p", d_phi), ("p", d_psib), ("i", 8), ("p", d_afp), ("p", d_aez),
                ("p", d_numC), ("p", d_coff)])
        torch.cuda.synchronize()
        PsiB[a] = d_psib.cpu().numpy().reshape(nb, G)
        Psi[a] = d_psi1[:nc * G].cpu().numpy().reshape(nc, G)       # savePsi
    Phi = d_phi.cpu().numpy().reshape(nc, G)
    os.makedirs(outdir, exist_ok=True)
    keep = np.arange(0, A, max(1, A // 16))          # a subset of directions keeps the file small
    np.savez_compressed(os.path.join(outdir, f"ref_sweep_{name}.npz"), Phi=Phi, PsiB=PsiB[keep],
                        Psi=Psi[keep], keep=keep, digest=np.array(input_digest(prob, STotal, geo, S)),
                        sums=input_sums(prob, STotal, geo))
    print(name, "Phi sum", Phi.sum())


if __name__ == "__main__":
    out = sys.argv[1] if len(sys.argv) > 1 else HERE
    for name in CASES:
        run(name, out)
