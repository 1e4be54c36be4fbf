"""Golden sweep outputs, and timings, from the reference's own CUDA sweep kernel.

The UMT repository ships a CUDA implementation of SweepUCBxyz
(src/teton/gpu/GPU_SweepUCBxyz.cu: compAfpKernel :141-160, CompSTotalTauPsi
:162-170, SweepUCBxyzKernel :172-516).  oracle/ref_build.py compiles its
device code, unmodified, into oracle/_ref/ref_sweep.cubin.  This script
plays the part of its host driver gpu_sweepucbxyz (:532-994) for one
direction after another -- Psi1 carried from direction to direction, tau*Psi
folded into the source, Phi accumulated over all directions, PsiB exits,
savePsi -- on inputs built from this repository's mesh, geometry and
schedule.

Runs on a GPU host (needs the cubin next to it and torch for device memory):

    python tests/golden/gen_ref_sweep.py OUTDIR
        writes tests/golden/ref_sweep_<case>.npz for the golden cases
    python tests/golden/gen_ref_sweep.py --time TILES STRIDE OUT.json
        times the reference kernel on the multigroup scattering workload
        (TILES^3 tiles, 128 directions, 16 groups, seed 2) for every
        STRIDE-th direction: kernel-only time with CUDA events, and the time
        with the per-direction host copies the shipped driver makes (Psi and
        PsiB to the device, Psi1, PsiB back), scaled to all directions.

Every launch is checked on the host first: the kernel indexes groups in
blocks of 4 and corner-face projections with stride 3, so only G % 4 == 0,
maxcf == 3 and <= 8 corners per zone are run; the cycle-list kernels are not
needed because the meshes used have no mesh cycles.
"""
import ctypes as C
import hashlib
import json
import os
import sys
import time

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


class RefSweep:
    """The reference kernels on one problem; sweep(a, ...) is one direction."""

    SMEM = 98304

    def __init__(self, prob, STotal, geo, S, omega=None):
        import torch
        self.torch = torch
        m = prob.mesh
        omega = prob.omega if omega is None else omega
        A, G, nc, nb, nz = len(omega), prob.ngr, m.ncornr, m.nbelem, m.nzones
        # ---- host-side checks of every index the kernels will use ----
        assert G % 4 == 0, "kernel handles groups in blocks of 4"
        assert int(m.numCorner.max()) <= 8 and (m.nCFaces == 3).all()
        assert int(S.numCycles.sum()) == 0, "no cycle list expected"
        assert (m.cFP >= 0).all() and (m.cFP < nc + nb).all()
        assert (m.cEZ >= 0).all() and (m.cEZ < m.numCorner[m.cToZone][:, None]).all()
        for a in range(A):
            assert S.zonesInPlane[a, :S.nHyperPlanes[a]].sum() == nz
        self.prob, self.S, self.omega = prob, S, omega
        self.A, self.G, self.nc, self.nb = A, G, nc, nb
        dev = self.dev = torch.device("cuda:0")
        torch.zeros(1, device=dev)          # creates the primary context
        torch.cuda.synchronize()
        cuda = self.cuda = C.CDLL("libcuda.so.1")
        ctx = C.c_void_p()
        assert cuda.cuCtxGetCurrent(C.byref(ctx)) == 0 and ctx.value
        mod = C.c_void_p()
        cubin = os.path.join(ROOT, "oracle", "_ref", "ref_sweep.cubin")
        assert cuda.cuModuleLoad(C.byref(mod), cubin.encode()) == 0, "cuModuleLoad failed"

        def fn(nm):
            f = C.c_void_p()
            assert cuda.cuModuleGetFunction(C.byref(f), mod, nm.encode()) == 0, nm
            return f

        self.k_afp, self.k_tau, self.k_sweep = fn("compAfpKernel"), fn("CompSTotalTauPsi"), fn("SweepUCBxyzKernel")
        assert cuda.cuFuncSetAttribute(self.k_sweep, 8, self.SMEM) == 0   # MAX_DYNAMIC_SHARED_SIZE_BYTES
        f64, i32 = np.float64, np.int32
        T = self.T
        self.d_Afp = T(geo[0], f64); self.d_Aez = T(geo[1], f64); self.d_vol = T(geo[2], f64)
        self.d_sigt = T(prob.sigt, f64)
        self.d_ncf = T(m.nCFaces, i32)
        self.d_cFP = T(m.cFP + 1, i32); self.d_cEZ = T(m.cEZ + 1, i32)
        self.d_numC = T(m.numCorner, i32); self.d_coff = T(m.cOffSet, i32)
        self.d_psi1 = torch.zeros((nc + nb) * G, dtype=torch.float64, device=dev)
        self.d_phi = torch.zeros(nc * G, dtype=torch.float64, device=dev)
        self.d_afp = torch.zeros(nc * 3, dtype=torch.float64, device=dev)
        self.d_aez = torch.zeros(nc * 3, dtype=torch.float64, device=dev)
        self.nblocks = (G + 3) // 4
        self.d_bdy = torch.zeros(self.nblocks * 32 * 2 * 3 * 8, dtype=torch.int32, device=dev)
        self.d_ST = T(STotal, f64)
        self.d_src = torch.empty_like(self.d_ST)
        self.d_psi = torch.empty(nc * G, dtype=torch.float64, device=dev)
        self.d_psib = torch.empty(nb * G, dtype=torch.float64, device=dev)

    def T(self, x, dt):
        return self.torch.as_tensor(np.ascontiguousarray(x, dtype=dt), device=self.dev)

    def launch(self, f, grid, block, smem, args):
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
        rc = self.cuda.cuLaunchKernel(f, grid, 1, 1, block, 1, 1, smem, None, params, None)
        assert rc == 0, rc

    def upload(self, a, psi_a, psib_a):
        """Per-direction host-to-device copies of the shipped driver."""
        self.d_psib.copy_(self.torch.as_tensor(np.ascontiguousarray(psib_a).reshape(-1)))
        self.d_psi.copy_(self.torch.as_tensor(np.ascontiguousarray(psi_a).reshape(-1)))

    def kernels(self, a):
        S, prob, nc, G = self.S, self.prob, self.nc, self.G
        nh = int(S.nHyperPlanes[a])
        nextZ = S.nextZ[a].astype(np.int64)
        nextZ1 = np.where(nextZ >= 0, nextZ + 1, nextZ).astype(np.int32)   # Fortran sign convention
        d_nextZ = self.T(nextZ1, np.int32)
        d_nextC = self.T(S.nextC[a] + 1, np.int32)
        d_zip = self.T(S.zonesInPlane[a, :nh], np.int32)
        d_om = self.T(self.omega[a], np.float64)
        return nh, d_nextZ, d_nextC, d_zip, d_om

    def run_kernels(self, a, nh, d_nextZ, d_nextC, d_zip, d_om, weight):
        nc, G = self.nc, self.G
        self.d_psi1[nc * G:] = self.d_psib
        self.d_src.copy_(self.d_ST)
        self.launch(self.k_afp, 4, 512, 0, [("p", d_om), ("p", self.d_Afp), ("p", self.d_afp), ("p", self.d_Aez),
                                            ("p", self.d_aez), ("u", nc * 3), ("u", 3)])
        self.launch(self.k_tau, 4, 1024, 0, [("p", self.d_src), ("p", self.d_psi), ("d", self.prob.tau),
                                             ("i", nc * G)])
        self.launch(self.k_sweep, self.nblocks, 128, self.SMEM,
                    [("i", a + 1), ("i", nh), ("p", d_zip), ("p", d_nextZ), ("p", d_nextC), ("p", self.d_src),
                     ("d", self.prob.tau), ("i", G), ("p", self.d_vol), ("p", self.d_sigt), ("p", self.d_ncf),
                     ("i", 3), ("i", 3), ("i", nc), ("p", d_om), ("p", self.d_cFP), ("p", self.d_bdy),
                     ("p", self.d_psi1), ("p", self.d_cEZ), ("d", weight), ("p", self.d_phi),
                     ("p", self.d_psib), ("i", 8), ("p", self.d_afp), ("p", self.d_aez), ("p", self.d_numC),
                     ("p", self.d_coff)])

    def download(self):
        nc, nb, G = self.nc, self.nb, self.G
        return (self.d_psib.cpu().numpy().reshape(nb, G), self.d_psi1[:nc * G].cpu().numpy().reshape(nc, G))


def run(name, outdir):
    prob, STotal, geo, S = build_inputs(name)
    m = prob.mesh
    A, G, nb = len(prob.weight), prob.ngr, m.nbelem
    ref = RefSweep(prob, STotal, geo, S)
    Psi = np.ascontiguousarray(prob.psi0, np.float64).copy()
    PsiB = np.zeros((A, nb, G))
    for a in range(A):
        args = ref.kernels(a)
        ref.upload(a, Psi[a], PsiB[a])
        ref.run_kernels(a, *args, prob.weight[a])
        ref.torch.cuda.synchronize()
        PsiB[a], Psi[a] = ref.download()                 # exits; savePsi
    Phi = ref.d_phi.cpu().numpy().reshape(m.ncornr, G)
    os.makedirs(outdir, exist_ok=True)
    keep = np.arange(0, A, max(1, A // 16))          # a subset of directions keeps the file small
    np.savez_compressed(os.path.join(outdir, f"ref_sweep_{name}.npz"), Phi=Phi, PsiB=PsiB[keep],
                        Psi=Psi[keep], keep=keep, digest=np.array(input_digest(prob, STotal, geo, S)),
                        sums=input_sums(prob, STotal, geo))
    print(name, "Phi sum", Phi.sum())


def time_workload(tiles, stride, out):
    """Reference kernel on the multigroup scattering workload, every stride-th direction."""
    from umt_gb300.problems import synthetic_problem
    from oracle import pyoracle as po
    prob = synthetic_problem((tiles,) * 3, 4, 4, 16, seed=2, sigt_range=(1e-2, 1e2), c_range=(0.0, 0.5),
                             time_dependent=True)
    m = prob.mesh
    G = prob.ngr
    sample = np.arange(0, len(prob.weight), stride)
    omega = np.ascontiguousarray(prob.omega[sample])
    geo = po.geometry(m)
    S = po.schedule(m, geo[0], geo[1], omega)
    STotal = np.repeat(prob.q_ext, m.numCorner, axis=0) / (4 * np.pi)
    ref = RefSweep(prob, STotal, geo, S, omega=omega)
    torch = ref.torch
    Psi = np.ascontiguousarray(prob.psi0[sample], np.float64)
    PsiB = np.zeros((len(sample), m.nbelem, G))
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    kern_ms, full_s = [], []
    for i in range(len(sample)):
        args = ref.kernels(i)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ref.upload(i, Psi[i], PsiB[i])
        ev0.record()
        ref.run_kernels(i, *args, prob.weight[sample[i]])
        ev1.record()
        PsiB[i], Psi[i] = ref.download()
        torch.cuda.synchronize()
        full_s.append(time.perf_counter() - t0)
        kern_ms.append(ev0.elapsed_time(ev1))
    A_all = len(prob.weight)
    units = m.ncornr * A_all * G
    kern_sweep_s = float(np.mean(kern_ms)) * 1e-3 * A_all
    full_sweep_s = float(np.mean(full_s)) * A_all
    res = {"workload": f"multigroup scattering sweep, {tiles}^3 tiles, {A_all} directions, {G} groups",
           "kernel": "reference SweepUCBxyzKernel (+compAfpKernel, CompSTotalTauPsi), FP64, unmodified",
           "directions_timed": int(len(sample)), "stride": int(stride),
           "kernel_ms_per_direction": kern_ms, "with_copies_s_per_direction": full_s,
           "kernel_sweep_s": kern_sweep_s, "with_copies_sweep_s": full_sweep_s,
           "ns_per_unit_kernel": kern_sweep_s * 1e9 / units, "ns_per_unit_with_copies": full_sweep_s * 1e9 / units,
           "units_per_sweep": units}
    with open(out, "w") as f:
        json.dump(res, f, indent=1)
    print(json.dumps({k: v for k, v in res.items() if not isinstance(v, list)}))


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "--time":
        time_workload(int(sys.argv[2]), int(sys.argv[3]), sys.argv[4])
    else:
        out = sys.argv[1] if len(sys.argv) > 1 else HERE
        for name in CASES:
            run(name, out)
