"""ctypes binding of libumt103.so (include/umt103.h).

This is the Python face of the C-ABI; a Fortran caller binds the same entry
points through an ISO_C_BINDING interface block.  Loading fails loudly when
the library has not been built: there is no fallback path.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libumt103.so")

UMT_FP64, UMT_FP32, UMT_MIXED = 0, 1, 2
UMT_GTA_TSA, UMT_GTA_ZONE = 1, 2
UMT_BATCH_MERGED, UMT_BATCH_GRAPHS = 0, 1
(UMT_OK, UMT_ERR_ARG, UMT_ERR_STATE, UMT_ERR_CUDA, UMT_ERR_CYCLE, UMT_ERR_TIMEOUT, UMT_ERR_BOUNDS,
 UMT_ERR_NOMEM, UMT_ERR_NOTCONV) = (0, -1, -2, -3, -4, -5, -6, -7, -8)

ERRORS = {0: "UMT_OK", -1: "UMT_ERR_ARG", -2: "UMT_ERR_STATE", -3: "UMT_ERR_CUDA",
          -4: "UMT_ERR_CYCLE", -5: "UMT_ERR_TIMEOUT", -6: "UMT_ERR_BOUNDS",
          -7: "UMT_ERR_NOMEM", -8: "UMT_ERR_NOTCONV"}

_ip = C.POINTER(C.c_int)
_dp = C.POINTER(C.c_double)


class UmtMesh(C.Structure):
    _fields_ = [("index_base", C.c_int), ("nzones", C.c_int), ("ncornr", C.c_int),
                ("nbelem", C.c_int), ("maxcf", C.c_int), ("maxFaces", C.c_int),
                ("numCorner", _ip), ("cOffSet", _ip), ("zoneFaces", _ip), ("zoneOpp", _ip),
                ("faceOpp", _ip), ("nCFaces", _ip), ("cFP", _ip), ("cEZ", _ip),
                ("CToFace", _ip), ("bdyToC", _ip), ("px", _dp), ("A_fp", _dp),
                ("A_ez", _dp), ("Volume", _dp)]


class UmtQuad(C.Structure):
    _fields_ = [("nangles", C.c_int), ("omega", _dp), ("weight", _dp)]


class UmtMeshRZ(C.Structure):
    _fields_ = [("index_base", C.c_int), ("nzones", C.c_int), ("ncornr", C.c_int), ("nbelem", C.c_int),
                ("maxFaces", C.c_int), ("numCorner", _ip), ("cOffSet", _ip), ("zoneFaces", _ip),
                ("zoneOpp", _ip), ("faceOpp", _ip), ("cFP", _ip), ("cEZ", _ip), ("CToFace", _ip),
                ("bdyToC", _ip), ("px", _dp)]


class UmtQuadRZ(C.Structure):
    _fields_ = [("nangles", C.c_int), ("omega", _dp), ("weight", _dp), ("angDerivFac", _dp),
                ("quadTauW1", _dp), ("quadTauW2", _dp), ("starting", _ip), ("finishing", _ip)]


class UmtSIParams(C.Structure):
    _fields_ = [("precision", C.c_int), ("max_iters", C.c_int), ("rel_tol", C.c_double),
                ("use_gta", C.c_int), ("q_ext", _dp), ("save_psi", C.c_int), ("warm_start", C.c_int),
                ("learn_every", C.c_int), ("learn_start", C.c_int), ("phi_ref", _dp),
                ("inner_tol", C.c_double), ("inner_max", C.c_int)]


class UmtSIResult(C.Structure):
    _fields_ = [("iterations", C.c_int), ("sweeps", C.c_int), ("rel_change", C.c_double),
                ("seconds", C.c_double), ("grey_sweeps", C.c_int), ("learned_kept", C.c_int),
                ("learned_rejected", C.c_int), ("fp64_sweeps", C.c_int)]


class UmtEnergyTally(C.Structure):
    _fields_ = [("EnergyRadiation", C.c_double), ("PowerEscape", C.c_double),
                ("PowerIncident", C.c_double), ("PowerAbsorbed", C.c_double),
                ("Balance", C.c_double)]


class UmtError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run `python -m umt_gb300.build` "
                              "(the CUDA library is required, there is no CPU path)")
        _lib = C.CDLL(LIB_PATH)
        _lib.umt103_error_string.restype = C.c_char_p
        _lib.umt103_last_sweep_ms.restype = C.c_double
        _lib.umt103_finalize.restype = None
        for n in ("umt103_init", "umt103_set_materials", "umt103_set_psi", "umt103_get_psi",
                  "umt103_sweep", "umt103_set_source", "umt103_sweep_resident",
                  "umt103_get_phi", "umt103_source_iterate", "umt103_tally",
                  "umt103_schedule_info", "umt103_get_schedule", "umt103_get_geometry",
                  "umt103_last_timing", "umt103_launches_per_sweep", "umt103_select_device",
                  "umt103_set_group_tile", "umt103_tally_precision", "umt103_set_sweep_mode",
                  "umt103_set_gta", "umt103_set_gta_solver", "umt103_tally_noalloc", "umt103_context_create",
                  "umt103_init_rz", "umt103_sweep_rz", "umt103_get_geometry_rz",
                  "umt103_context_select", "umt103_context_current", "umt103_context_destroy",
                  "umt103_batch_sweep", "umt103_psib_rows", "umt103_hold_item",
                  "umt103_mlp_init", "umt103_mlp_info", "umt103_mlp_get_params", "umt103_mlp_set_params",
                  "umt103_mlp_forward", "umt103_mlp_gradient", "umt103_mlp_collect", "umt103_mlp_set_targets",
                  "umt103_mlp_rows", "umt103_mlp_clear", "umt103_mlp_train", "umt103_autotune",
                  "umt103_autotune_contexts", "umt103_gta_correction", "umt103_phi_device",
                  "umt103_set_external_source", "umt103_si_step", "umt103_si_change", "umt103_set_batch_mode"):
            getattr(_lib, n).restype = C.c_int
        _lib.umt103_mlp_finalize.restype = None
        _fp = C.POINTER(C.c_float)
        _lib.umt103_mlp_init.argtypes = [C.c_int, C.c_uint]
        _lib.umt103_mlp_forward.argtypes = [_fp, C.c_int, _fp]
        _lib.umt103_mlp_gradient.argtypes = [_fp, _fp, C.c_int, _fp]
        _lib.umt103_mlp_train.argtypes = [C.c_int, C.c_int, C.c_float, _fp]
        _lib.umt103_set_materials.argtypes = [_dp, _dp, C.c_double]
        _lib.umt103_tally.argtypes = [_dp, C.c_double, C.POINTER(UmtEnergyTally)]
        _lib.umt103_tally_precision.argtypes = [_dp, C.c_double, C.c_int, C.POINTER(UmtEnergyTally)]
        _lib.umt103_tally_noalloc.argtypes = [C.c_void_p, C.c_double, C.c_int, C.POINTER(UmtEnergyTally)]
    return _lib


EXPORTED = ["umt103_init", "umt103_finalize", "umt103_set_materials", "umt103_set_psi",
            "umt103_get_psi", "umt103_sweep", "umt103_set_source", "umt103_sweep_resident",
            "umt103_get_phi", "umt103_source_iterate", "umt103_tally", "umt103_schedule_info",
            "umt103_get_schedule", "umt103_get_geometry", "umt103_last_sweep_ms",
            "umt103_error_string", "umt103_last_timing", "umt103_launches_per_sweep",
            "umt103_select_device", "umt103_set_group_tile", "umt103_tally_precision",
            "umt103_set_sweep_mode", "umt103_set_gta", "umt103_set_gta_solver", "umt103_tally_noalloc",
            "umt103_context_create", "umt103_context_select", "umt103_context_current",
            "umt103_context_destroy", "umt103_batch_sweep", "umt103_init_rz", "umt103_sweep_rz",
            "umt103_get_geometry_rz", "umt103_psib_rows", "umt103_hold_item",
            "umt103_mlp_init", "umt103_mlp_finalize", "umt103_mlp_info", "umt103_mlp_get_params",
            "umt103_mlp_set_params", "umt103_mlp_forward", "umt103_mlp_gradient", "umt103_mlp_collect",
            "umt103_mlp_set_targets", "umt103_mlp_rows", "umt103_mlp_clear", "umt103_mlp_train",
            "umt103_autotune", "umt103_autotune_contexts", "umt103_gta_correction", "umt103_phi_device",
            "umt103_set_external_source", "umt103_si_step", "umt103_si_change", "umt103_set_batch_mode"]


def check(rc):
    if rc != 0:
        raise UmtError(rc, load().umt103_error_string().decode())
    return rc


def _i(a):
    return a.ctypes.data_as(_ip) if a is not None else None


def _d(a):
    return a.ctypes.data_as(_dp) if a is not None else None


def _c(a, dt):
    return None if a is None else np.ascontiguousarray(a, dtype=dt)


class Library:
    """Thin object wrapper keeping the argument arrays alive across calls."""

    def __init__(self):
        self.lib = load()
        self._keep = []
        self.A = self.G = self.nz = self.nc = self.nb = 0

    def init(self, mesh, omega, weight, ngr, flags=0, with_geometry=None, index_base=0):
        m = mesh
        arrs = dict(numCorner=_c(m.numCorner, np.int32), cOffSet=_c(m.cOffSet, np.int32),
                    zoneFaces=_c(m.zoneFaces, np.int32), zoneOpp=_c(m.zoneOpp, np.int32),
                    faceOpp=_c(m.faceOpp, np.int32), nCFaces=_c(m.nCFaces, np.int32),
                    cFP=_c(m.cFP, np.int32), cEZ=_c(m.cEZ, np.int32),
                    CToFace=_c(m.CToFace, np.int32), bdyToC=_c(m.bdyToC, np.int32))
        if index_base == 1:
            for k in ("cFP", "cEZ", "CToFace", "bdyToC", "faceOpp"):
                arrs[k] = arrs[k] + 1
            zo = arrs["zoneOpp"].copy()
            zo[zo >= 0] += 1
            arrs["zoneOpp"] = zo
            fo = arrs["faceOpp"].copy()
            fo[arrs["zoneOpp"] < 1] = -1
            arrs["faceOpp"] = fo
        px = _c(m.px, np.float64)
        geo = [None, None, None]
        if with_geometry is not None:
            geo = [_c(x, np.float64) for x in with_geometry]
            px = None
        st = UmtMesh(index_base, m.nzones, m.ncornr, m.nbelem, 3, m.zoneOpp.shape[1],
                     _i(arrs["numCorner"]), _i(arrs["cOffSet"]), _i(arrs["zoneFaces"]),
                     _i(arrs["zoneOpp"]), _i(arrs["faceOpp"]), _i(arrs["nCFaces"]),
                     _i(arrs["cFP"]), _i(arrs["cEZ"]), _i(arrs["CToFace"]), _i(arrs["bdyToC"]),
                     _d(px), _d(geo[0]), _d(geo[1]), _d(geo[2]))
        om = _c(omega, np.float64); w = _c(weight, np.float64)
        q = UmtQuad(len(w), _d(om), _d(w))
        check(self.lib.umt103_init(C.byref(st), C.byref(q), int(ngr), int(flags)))
        self.A, self.G, self.nz, self.nc, self.nb = len(w), int(ngr), m.nzones, m.ncornr, m.nbelem
        return self

    def finalize(self):
        self.lib.umt103_finalize()

    def set_materials(self, sigt, sigs=None, tau=0.0):
        sigt = _c(sigt, np.float64); sigs = _c(sigs, np.float64)
        check(self.lib.umt103_set_materials(_d(sigt), _d(sigs), C.c_double(tau)))

    def set_psi(self, Psi=None, PsiB=None):
        Psi = _c(Psi, np.float64); PsiB = _c(PsiB, np.float64)
        check(self.lib.umt103_set_psi(_d(Psi), _d(PsiB)))

    def get_psi(self, precision=UMT_FP64):
        Psi = np.zeros((self.A, self.nc, self.G)); PsiB = np.zeros((self.A, self.nb, self.G))
        check(self.lib.umt103_get_psi(_d(Psi), _d(PsiB), int(precision)))
        return Psi, PsiB

    def sweep(self, STotal=None, savePsi=False, PsiB=None, precision=UMT_FP64, want_phi=True, Phi=None):
        """umt103_sweep; Phi, if given, is a C-contiguous float64 (nc, G)
        array the result is written into (e.g. a view of pinned memory)."""
        STotal = _c(STotal, np.float64)
        if Phi is not None:
            assert Phi.dtype == np.float64 and Phi.flags.c_contiguous and Phi.shape == (self.nc, self.G)
        elif want_phi:
            Phi = np.zeros((self.nc, self.G))
        if PsiB is not None:
            assert PsiB.dtype == np.float64 and PsiB.flags.c_contiguous
        check(self.lib.umt103_sweep(_d(STotal), int(bool(savePsi)), _d(Phi), _d(PsiB), int(precision)))
        return Phi

    def set_source(self, STotal=None):
        STotal = _c(STotal, np.float64)
        check(self.lib.umt103_set_source(_d(STotal)))

    def sweep_resident(self, savePsi=False, precision=UMT_FP64):
        check(self.lib.umt103_sweep_resident(int(bool(savePsi)), int(precision)))

    def get_phi(self, nc=None, G=None):
        Phi = np.zeros((nc or self.nc, G or self.G))
        check(self.lib.umt103_get_phi(_d(Phi)))
        return Phi

    def timing(self):
        out = np.zeros(3)
        check(self.lib.umt103_last_timing(_d(out)))
        return out

    def launches_per_sweep(self, precision):
        n = self.lib.umt103_launches_per_sweep(int(precision))
        if n < 0:
            check(n)
        return n

    def psib_rows(self):
        """(exiting, total) PsiB rows of the FP32 sweep (umt103_psib_rows)."""
        ex, tot = C.c_longlong(0), C.c_longlong(0)
        check(self.lib.umt103_psib_rows(C.byref(ex), C.byref(tot)))
        return ex.value, tot.value

    def source_iterate(self, precision=UMT_FP64, max_iters=50, rel_tol=1e-8, q_ext=None, save_psi=True,
                       use_gta=False, allow_notconv=False, warm_start=False, learn_every=0, learn_start=2,
                       phi_ref=None, inner_tol=0.0, inner_max=0):
        q = _c(q_ext, np.float64)
        ref = _c(phi_ref, np.float64)
        prm = UmtSIParams(int(precision), int(max_iters), float(rel_tol), int(bool(use_gta)), _d(q),
                          int(bool(save_psi)), int(bool(warm_start)), int(learn_every), int(learn_start), _d(ref),
                          float(inner_tol), int(inner_max))
        res = UmtSIResult()
        rc = self.lib.umt103_source_iterate(C.byref(prm), C.byref(res))
        if rc != 0 and not (allow_notconv and rc == -8):
            check(rc)
        return dict(iterations=res.iterations, sweeps=res.sweeps, rel_change=res.rel_change,
                    seconds=res.seconds, converged=(rc == 0), grey_sweeps=res.grey_sweeps,
                    learned_kept=res.learned_kept, learned_rejected=res.learned_rejected,
                    fp64_sweeps=res.fp64_sweeps)

    # ---- learned acceleration (umt103_mlp_*) ----
    def mlp_init(self, ngr, seed=0):
        check(self.lib.umt103_mlp_init(int(ngr), int(seed)))

    def mlp_finalize(self):
        self.lib.umt103_mlp_finalize()

    def mlp_info(self):
        f, h, n = C.c_int(0), C.c_int(0), C.c_longlong(0)
        check(self.lib.umt103_mlp_info(C.byref(f), C.byref(h), C.byref(n)))
        return f.value, h.value, n.value

    def mlp_get_params(self):
        p = np.zeros(self.mlp_info()[2], np.float32)
        check(self.lib.umt103_mlp_get_params(p.ctypes.data_as(C.POINTER(C.c_float))))
        return p

    def mlp_set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        check(self.lib.umt103_mlp_set_params(p.ctypes.data_as(C.POINTER(C.c_float))))

    def mlp_forward(self, X, G):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.zeros((X.shape[0], G), np.float32)
        fp = C.POINTER(C.c_float)
        check(self.lib.umt103_mlp_forward(X.ctypes.data_as(fp), X.shape[0], Y.ctypes.data_as(fp)))
        return Y

    def mlp_gradient(self, X, dY):
        X = np.ascontiguousarray(X, dtype=np.float32); dY = np.ascontiguousarray(dY, dtype=np.float32)
        g = np.zeros(self.mlp_info()[2], np.float32)
        fp = C.POINTER(C.c_float)
        check(self.lib.umt103_mlp_gradient(X.ctypes.data_as(fp), dY.ctypes.data_as(fp), X.shape[0],
                                           g.ctypes.data_as(fp)))
        return g

    def mlp_collect(self):
        n = C.c_int(0)
        check(self.lib.umt103_mlp_collect(C.byref(n)))
        return n.value

    def mlp_set_targets(self, PhiStar):
        PhiStar = _c(PhiStar, np.float64)
        check(self.lib.umt103_mlp_set_targets(_d(PhiStar)))

    def mlp_rows(self):
        n = C.c_longlong(0)
        check(self.lib.umt103_mlp_rows(C.byref(n)))
        return n.value

    def mlp_clear(self):
        check(self.lib.umt103_mlp_clear())

    def mlp_train(self, steps, batch=4096, lr=1e-3):
        loss = np.zeros(2, np.float32)
        check(self.lib.umt103_mlp_train(int(steps), int(batch), C.c_float(lr),
                                        loss.ctypes.data_as(C.POINTER(C.c_float))))
        return float(loss[0]), float(loss[1])

    def tally(self, siga=None, speed_light=299.792458, precision=None):
        siga = _c(siga, np.float64)
        t = UmtEnergyTally()
        if precision is None:
            check(self.lib.umt103_tally(_d(siga), C.c_double(speed_light), C.byref(t)))
        else:
            check(self.lib.umt103_tally_precision(_d(siga), C.c_double(speed_light), int(precision), C.byref(t)))
        return dict(EnergyRadiation=t.EnergyRadiation, PowerEscape=t.PowerEscape,
                    PowerIncident=t.PowerIncident, PowerAbsorbed=t.PowerAbsorbed)

    def tally_noalloc(self, siga_dev_ptr=None, speed_light=299.792458, precision=UMT_FP64):
        """Energy edits without device allocation; siga_dev_ptr is a device
        address (int) of Siga(G,nzones) in FP64, or None."""
        t = UmtEnergyTally()
        check(self.lib.umt103_tally_noalloc(C.c_void_p(siga_dev_ptr) if siga_dev_ptr else None,
                                            C.c_double(speed_light), int(precision), C.byref(t)))
        return dict(EnergyRadiation=t.EnergyRadiation, PowerEscape=t.PowerEscape,
                    PowerIncident=t.PowerIncident, PowerAbsorbed=t.PowerAbsorbed)

    def context_create(self):
        cid = C.c_int(0)
        check(self.lib.umt103_context_create(C.byref(cid)))
        return cid.value

    def context_select(self, cid):
        check(self.lib.umt103_context_select(int(cid)))

    def context_destroy(self, cid):
        check(self.lib.umt103_context_destroy(int(cid)))

    def batch_sweep(self, ids, precision=UMT_FP32):
        arr = (C.c_int * len(ids))(*ids)
        ms = C.c_double(0.0)
        check(self.lib.umt103_batch_sweep(arr, len(ids), int(precision), C.byref(ms)))
        return ms.value

    def set_batch_mode(self, mode):
        """umt103_set_batch_mode: UMT_BATCH_MERGED (one launch per dependency
        stage over the problems of a group tile) or UMT_BATCH_GRAPHS (each
        context's sweep graph nested)."""
        check(self.lib.umt103_set_batch_mode(int(mode)))

    def set_group_tile(self, lanes_per_zone, groups_per_lane):
        check(self.lib.umt103_set_group_tile(int(lanes_per_zone), int(groups_per_lane)))

    def autotune(self, reps=2):
        """umt103_autotune: ((lanes_per_zone, groups_per_lane), {tile: best ms})."""
        gt, gpl, nt = C.c_int(0), C.c_int(0), C.c_int(0)
        times = np.zeros((8, 3))
        check(self.lib.umt103_autotune(int(reps), C.byref(gt), C.byref(gpl), _d(times), 8, C.byref(nt)))
        return (gt.value, gpl.value), {(int(t[0]), int(t[1])): float(t[2]) for t in times[:nt.value]}

    def autotune_contexts(self, ids, reps=2):
        arr = (C.c_int * len(ids))(*ids)
        check(self.lib.umt103_autotune_contexts(arr, len(ids), int(reps)))

    def set_gta(self, max_krylov=10, tol=1e-4, spectrum=0):
        self.lib.umt103_set_gta.argtypes = [C.c_int, C.c_double, C.c_int]
        check(self.lib.umt103_set_gta(int(max_krylov), float(tol), int(spectrum)))

    def set_gta_solver(self, solver):
        """umt103_set_gta_solver: UMT_GTA_TSA (grey + stretched-TSA sweeps) or
        UMT_GTA_ZONE (grey sweep + per-zone direct solve)."""
        check(self.lib.umt103_set_gta_solver(int(solver)))

    def phi_device(self):
        """umt103_phi_device: (device address, element count) of PhiTotal."""
        p, n = C.c_void_p(0), C.c_longlong(0)
        check(self.lib.umt103_phi_device(C.byref(p), C.byref(n)))
        return p.value, n.value

    def set_external_source(self, q_ext=None):
        q = _c(q_ext, np.float64)
        check(self.lib.umt103_set_external_source(_d(q)))

    def si_step(self, precision=UMT_FP64):
        check(self.lib.umt103_si_step(int(precision)))

    def si_change(self):
        r = C.c_double(0.0)
        check(self.lib.umt103_si_change(C.byref(r)))
        return r.value

    def schedule_info(self, angle):
        """umt103_schedule_info: (hyperplanes, cycle-list corners) of one direction."""
        h, n = C.c_int(0), C.c_int(0)
        check(self.lib.umt103_schedule_info(int(angle), C.byref(h), C.byref(n)))
        return h.value, n.value

    def gta_correction(self, PhiPrev):
        """umt103_gta_correction: (grey correction [nc], chi [nz, G], grey sweeps)."""
        prev = _c(PhiPrev, np.float64)
        x = np.zeros(self.nc); chi = np.zeros((self.nz, self.G)); gs = C.c_int(0)
        check(self.lib.umt103_gta_correction(_d(prev), _d(x), _d(chi), C.byref(gs)))
        return x, chi, gs.value

    def set_sweep_mode(self, mode):
        check(self.lib.umt103_set_sweep_mode(int(mode)))

    def hold_item(self, item):
        """umt103_hold_item: failure-path test hook (see the header)."""
        check(self.lib.umt103_hold_item(int(item)))

    def select_device(self, device):
        check(self.lib.umt103_select_device(int(device)))

    def last_ms(self):
        return float(self.lib.umt103_last_sweep_ms())

    def schedule_info(self, angle):
        """umt103_schedule_info: (hyperplanes, cycle-list corners) of one direction."""
        h, n = C.c_int(0), C.c_int(0)
        check(self.lib.umt103_schedule_info(int(angle), C.byref(h), C.byref(n)))
        return h.value, n.value

    def schedule(self):
        level = np.zeros((self.A, self.nz), np.int32); nh = np.zeros(self.A, np.int32)
        check(self.lib.umt103_get_schedule(_i(level), _i(nh)))
        return level, nh

    def geometry(self):
        afp = np.zeros((self.nc, 3, 3)); aez = np.zeros((self.nc, 3, 3)); vol = np.zeros(self.nc)
        check(self.lib.umt103_get_geometry(_d(afp), _d(aez), _d(vol)))
        return afp, aez, vol

    # ---- 2-D RZ geometry ----
    def init_rz(self, mesh, quad, ngr, index_base=0, flags=0):
        """umt103_init_rz with a umt_gb300.mesh_rz.MeshRZ and a
        umt_gb300.quadrature_rz.QuadRZ; flags as for umt103_init (0: FP64
        and FP32 angular flux)."""
        m = mesh
        a = dict(numCorner=_c(m.numCorner, np.int32), cOffSet=_c(m.cOffSet, np.int32),
                 zoneFaces=_c(m.zoneFaces, np.int32), zoneOpp=_c(m.zoneOpp, np.int32),
                 faceOpp=_c(m.faceOpp, np.int32), cFP=_c(m.cFP, np.int32), cEZ=_c(m.cEZ, np.int32),
                 CToFace=_c(m.CToFace, np.int32), bdyToC=_c(m.bdyToC, np.int32))
        if index_base == 1:
            for k in ("cFP", "cEZ", "CToFace", "bdyToC"):      # cOffSet is an offset in both conventions
                a[k] = a[k] + 1
            zo = a["zoneOpp"].copy(); zo[zo >= 0] += 1; a["zoneOpp"] = zo
            fo = a["faceOpp"].copy(); fo[fo >= 0] += 1; a["faceOpp"] = fo
        px = _c(m.px, np.float64)
        st = UmtMeshRZ(index_base, m.nzones, m.ncornr, m.nbelem, m.zoneOpp.shape[1], _i(a["numCorner"]),
                       _i(a["cOffSet"]), _i(a["zoneFaces"]), _i(a["zoneOpp"]), _i(a["faceOpp"]), _i(a["cFP"]),
                       _i(a["cEZ"]), _i(a["CToFace"]), _i(a["bdyToC"]), _d(px))
        q = quad
        arrs = [_c(q.omega, np.float64), _c(q.weight, np.float64), _c(q.angDerivFac, np.float64),
                _c(q.quadTauW1, np.float64), _c(q.quadTauW2, np.float64), _c(q.starting, np.int32),
                _c(q.finishing, np.int32)]
        qs = UmtQuadRZ(len(q.weight), _d(arrs[0]), _d(arrs[1]), _d(arrs[2]), _d(arrs[3]), _d(arrs[4]),
                       _i(arrs[5]), _i(arrs[6]))
        self._keep = [a, px, arrs]
        check(self.lib.umt103_init_rz(C.byref(st), C.byref(qs), int(ngr), int(flags)))
        self.A, self.G, self.nz, self.nc, self.nb = len(q.weight), int(ngr), m.nzones, m.ncornr, m.nbelem
        return self

    def sweep_rz(self, STotal=None, savePsi=False, PsiB=None, precision=UMT_FP64, Phi=None):
        """umt103_sweep_rz; returns PhiTotal (written into Phi when given, a
        C-contiguous float64 (nc, G) array), PsiB is updated in place."""
        STotal = _c(STotal, np.float64)
        if Phi is not None:
            assert Phi.dtype == np.float64 and Phi.flags.c_contiguous and Phi.shape == (self.nc, self.G)
        else:
            Phi = np.zeros((self.nc, self.G))
        if PsiB is not None:
            assert PsiB.dtype == np.float64 and PsiB.flags.c_contiguous
        check(self.lib.umt103_sweep_rz(_d(STotal), int(bool(savePsi)), _d(Phi), _d(PsiB), int(precision)))
        return Phi

    def geometry_rz(self):
        area = np.zeros(self.nc); vol = np.zeros(self.nc); rfp = np.zeros((self.nc, 2)); rez = np.zeros((self.nc, 2))
        check(self.lib.umt103_get_geometry_rz(_d(area), _d(vol), _d(rfp), _d(rez)))
        return dict(Area=area, Volume=vol, RadiusFP=rfp, RadiusEZ=rez)
