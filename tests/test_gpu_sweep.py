"""GPU parity: the CUDA sweep through the C-ABI against the CPU oracle."""
import os

import numpy as np
import pytest

from umt_gb300 import capi
from umt_gb300.problems import uniform_problem, synthetic_problem
from tests.helpers import oracle_sweep, rel_err

pytestmark = pytest.mark.gpu


def _run_gpu(lib, prob, precision, STotal=None, savePsi=True, Psi=None):
    m = prob.mesh
    lib.init(m, prob.omega, prob.weight, prob.ngr)
    lib.set_materials(prob.sigt, prob.sigs, prob.tau)
    lib.set_psi(Psi if Psi is not None else prob.psi0, None)
    A, G = len(prob.weight), prob.ngr
    PsiB = np.zeros((A, m.nbelem, G))
    Phi = lib.sweep(STotal, savePsi=savePsi, PsiB=PsiB, precision=precision)
    Psi_out, _ = lib.get_psi(precision)
    return Phi, Psi_out, PsiB


def test_geometry_bitwise(umtlib):
    prob = uniform_problem((2, 2, 2))
    umtlib.init(prob.mesh, prob.omega, prob.weight, prob.ngr)
    afp, aez, vol = umtlib.geometry()
    ref = oracle_sweep(prob)["geo"]
    assert np.array_equal(afp, ref[0])
    assert np.array_equal(aez, ref[1])
    assert np.array_equal(vol, ref[2])


def test_schedule_levels_match_oracle_hyperplanes(umtlib):
    prob = uniform_problem((3, 2, 2), 2, 2, 2)
    umtlib.init(prob.mesh, prob.omega, prob.weight, prob.ngr)
    level, nh = umtlib.schedule()
    S = oracle_sweep(prob)["sched"]
    for a in range(len(prob.weight)):
        assert nh[a] == S.nHyperPlanes[a]
        zl = np.zeros(prob.mesh.nzones, np.int32)
        pos = 0
        for h in range(S.nHyperPlanes[a]):
            n = S.zonesInPlane[a, h]
            zl[np.abs(S.nextZ[a, pos:pos + n])] = h
            pos += n
        assert np.array_equal(zl, level[a])


@pytest.mark.parametrize("G", [2, 4, 16])
def test_fp64_sweep_parity(umtlib, G):
    prob = uniform_problem((2, 2, 2), 2, 2, G)
    ref = oracle_sweep(prob, Psi=prob.psi0)
    Phi, Psi, PsiB = _run_gpu(umtlib, prob, capi.UMT_FP64)
    assert rel_err(Phi, ref["Phi"]) < 1e-12
    assert rel_err(Psi, ref["Psi"]) < 1e-12
    assert rel_err(PsiB, ref["PsiB"]) < 1e-12


def test_fp64_sweep_parity_scattering_source(umtlib):
    prob = synthetic_problem((2, 2, 1), 4, 4, 8, seed=7, time_dependent=True)
    m = prob.mesh
    rng = np.random.default_rng(1)
    STotal = rng.uniform(0.1, 1.0, size=(m.ncornr, prob.ngr))
    ref = oracle_sweep(prob, STotal=STotal, Psi=prob.psi0)
    Phi, Psi, PsiB = _run_gpu(umtlib, prob, capi.UMT_FP64, STotal=STotal)
    assert rel_err(Phi, ref["Phi"]) < 1e-12
    assert rel_err(Psi, ref["Psi"]) < 1e-12


def test_fp32_sweep_tolerance(umtlib):
    prob = synthetic_problem((2, 2, 2), 2, 2, 16, seed=3, time_dependent=True)
    m = prob.mesh
    STotal = np.repeat(prob.q_ext, m.numCorner, axis=0) / (4 * np.pi)
    ref = oracle_sweep(prob, STotal=STotal, Psi=prob.psi0)
    Phi, Psi, PsiB = _run_gpu(umtlib, prob, capi.UMT_FP32, STotal=STotal)
    # FP32 sweep arithmetic: stated tolerance 1e-5 relative (max-norm) on phi
    assert rel_err(Phi, ref["Phi"]) < 1e-5
    assert rel_err(Psi, ref["Psi"]) < 1e-4


@pytest.mark.parametrize("mode", [0, 2])
@pytest.mark.parametrize("G,tile", [(16, (16, 1)), (16, (8, 2)), (16, (4, 4)), (2, (1, 2)),
                                    (2, (2, 1)), (8, (2, 4)), (32, (8, 4)), (64, (32, 2)),
                                    (4, (2, 2)), (32, (16, 2))])
def test_fp32_group_tiles(umtlib, G, tile, mode):
    """Every group tile of the FP32 zone-program kernel (mode 0) and of the
    corner-slot kernel (mode 2) agrees with the oracle."""
    prob = synthetic_problem((2, 2, 1), 2, 2, G, seed=4, time_dependent=True)
    m = prob.mesh
    STotal = np.repeat(prob.q_ext, m.numCorner, axis=0) / (4 * np.pi)
    ref = oracle_sweep(prob, STotal=STotal, Psi=prob.psi0)
    umtlib.init(m, prob.omega, prob.weight, G)
    umtlib.set_materials(prob.sigt, prob.sigs, prob.tau)
    umtlib.set_psi(prob.psi0, None)
    umtlib.set_group_tile(*tile)
    umtlib.set_sweep_mode(mode)
    PsiB = np.zeros((len(prob.weight), m.nbelem, G))
    Phi = umtlib.sweep(STotal, savePsi=True, PsiB=PsiB, precision=capi.UMT_FP32)
    Psi, _ = umtlib.get_psi(capi.UMT_FP32)
    assert rel_err(Phi, ref["Phi"]) < 1e-5
    assert rel_err(Psi, ref["Psi"]) < 1e-4
    assert rel_err(PsiB, ref["PsiB"]) < 1e-4


@pytest.mark.parametrize("mode", [0, 2])
def test_fp32_thick_strongly_scattering_32_groups(umtlib, mode):
    """The 32-group, strongly scattering workload's distribution (sigma_t
    log-uniform on [1, 1e3], c in [0.95, 0.999], 128 directions) on 3^3
    tiles: optically thick zones, where the FP32 EZ closure works near its
    cap, agree with the oracle, in the max norm and corner by corner."""
    prob = synthetic_problem((3, 3, 3), 4, 4, 32, seed=5, sigt_range=(1.0, 1e3), c_range=(0.95, 0.999),
                             q=1.0, time_dependent=True)
    m = prob.mesh
    rng = np.random.default_rng(55)
    phi = rng.uniform(0.5, 2.0, size=(m.ncornr, prob.ngr))
    STotal = (prob.sigs[m.cToZone] * phi + prob.q_ext[m.cToZone]) / (4 * np.pi)
    ref = oracle_sweep(prob, STotal=STotal, Psi=prob.psi0)
    umtlib.init(m, prob.omega, prob.weight, prob.ngr)
    umtlib.set_materials(prob.sigt, prob.sigs, prob.tau)
    umtlib.set_psi(prob.psi0, None)
    umtlib.set_sweep_mode(mode)
    PsiB = np.zeros((len(prob.weight), m.nbelem, prob.ngr))
    Phi = umtlib.sweep(STotal, savePsi=True, PsiB=PsiB, precision=capi.UMT_FP32)
    Psi, _ = umtlib.get_psi(capi.UMT_FP32)
    assert rel_err(Phi, ref["Phi"]) < 1e-5
    assert rel_err(Psi, ref["Psi"]) < 1e-4
    assert rel_err(PsiB, ref["PsiB"]) < 1e-4
    big = ref["Phi"] > 1e-3 * ref["Phi"].max()
    assert np.max(np.abs(Phi[big] / ref["Phi"][big] - 1.0)) < 1e-4


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_fp32_sweep_modes(umtlib, mode):
    """Per-stage launches of the zone-program (0) and corner-slot (2)
    kernels, and the persistent dependency-driven launch (1)."""
    prob = synthetic_problem((3, 2, 2), 4, 4, 16, seed=6, time_dependent=True)
    m = prob.mesh
    STotal = np.repeat(prob.q_ext, m.numCorner, axis=0) / (4 * np.pi)
    ref = oracle_sweep(prob, STotal=STotal, Psi=prob.psi0)
    umtlib.init(m, prob.omega, prob.weight, prob.ngr)
    umtlib.set_materials(prob.sigt, prob.sigs, prob.tau)
    umtlib.set_psi(prob.psi0, None)
    umtlib.set_sweep_mode(mode)
    for _ in range(3):                       # repeated sweeps reuse the captured graph
        PsiB = np.zeros((len(prob.weight), m.nbelem, prob.ngr))
        Phi = umtlib.sweep(STotal, savePsi=False, PsiB=PsiB, precision=capi.UMT_FP32)
        assert rel_err(Phi, ref["Phi"]) < 1e-5
        assert rel_err(PsiB, ref["PsiB"]) < 1e-4


def _config4_draws(n=12, seed=4):
    """The batched workload's problem mix: G in {4, 8, 16, 32, 64}, A in
    {32, 128} (P = Az in {2, 4}); tiles per axis from U{2..4} instead of
    U{4..16} so that the single-context runs stay short."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        t = int(rng.integers(2, 5))
        out.append(((t, t, t), int(rng.choice([2, 4])), int(rng.choice([4, 8, 16, 32, 64])), 400 + k))
    return out


@pytest.mark.parametrize("mode", [capi.UMT_BATCH_MERGED, capi.UMT_BATCH_GRAPHS], ids=["merged", "graphs"])
@pytest.mark.parametrize("specs", [[((2, 2, 1), 2, 4, 31), ((3, 2, 1), 4, 8, 32), ((2, 3, 2), 2, 16, 33)],
                                   _config4_draws()], ids=["three", "config4_draws"])
def test_batch_of_contexts_matches_single_runs(umtlib, specs, mode):
    """Several problems of different size, group and direction counts resident
    in separate contexts, swept from one graph launch, give each problem's
    single-context result bit for bit: with every dependency stage of the
    problems that share a group tile in one launch (merged), and with each
    context's own sweep graph nested (graphs)."""
    umtlib.set_batch_mode(mode)
    try:
        _batch_case(umtlib, specs)
    finally:
        umtlib.set_batch_mode(capi.UMT_BATCH_GRAPHS)


def _batch_case(umtlib, specs):
    from umt_gb300.problems import synthetic_problem as sp
    probs = [sp(t, P, P, G, seed=s, time_dependent=True) for (t, P, G, s) in specs]
    single = []
    for pr in probs:
        umtlib.init(pr.mesh, pr.omega, pr.weight, pr.ngr, flags=2 | 8)
        umtlib.set_materials(pr.sigt, pr.sigs, pr.tau)
        umtlib.set_psi(pr.psi0, None)
        st = np.repeat(pr.q_ext, pr.mesh.numCorner, axis=0) / (4 * np.pi)
        single.append(umtlib.sweep(st, precision=capi.UMT_FP32))
    ids = []
    for pr in probs:
        cid = umtlib.context_create()
        umtlib.context_select(cid)
        umtlib.init(pr.mesh, pr.omega, pr.weight, pr.ngr, flags=2 | 8)
        umtlib.set_materials(pr.sigt, pr.sigs, pr.tau)
        umtlib.set_psi(pr.psi0, None)
        umtlib.set_source(np.repeat(pr.q_ext, pr.mesh.numCorner, axis=0) / (4 * np.pi))
        ids.append(cid)
    umtlib.context_select(0)
    for _ in range(2):                       # the second launch replays the kept batch graph
        ms = umtlib.batch_sweep(ids, capi.UMT_FP32)
        assert ms > 0
        for cid, pr, ref in zip(ids, probs, single):
            umtlib.context_select(cid)
            phi = umtlib.get_phi(pr.mesh.ncornr, pr.ngr)
            assert np.array_equal(phi, ref)
        umtlib.context_select(0)
    # a changed context (new materials) is captured again, not replayed stale
    pr = probs[0]
    umtlib.context_select(ids[0])
    umtlib.set_materials(2.0 * pr.sigt, pr.sigs, pr.tau)
    umtlib.sweep_resident(False, capi.UMT_FP32)          # source as set for the batch
    want = umtlib.get_phi(pr.mesh.ncornr, pr.ngr)
    assert not np.array_equal(want, single[0])
    umtlib.context_select(0)
    umtlib.batch_sweep(ids, capi.UMT_FP32)
    umtlib.context_select(ids[0])
    assert np.array_equal(umtlib.get_phi(pr.mesh.ncornr, pr.ngr), want)
    # refused: a context listed twice, a context with a held work item
    umtlib.context_select(0)
    with pytest.raises(capi.UmtError) as e:
        umtlib.batch_sweep([ids[0], ids[0]], capi.UMT_FP32)
    assert e.value.code == capi.UMT_ERR_ARG
    umtlib.context_select(ids[-1])
    umtlib.hold_item(0)
    umtlib.context_select(0)
    with pytest.raises(capi.UmtError) as e:
        umtlib.batch_sweep(ids, capi.UMT_FP32)
    assert e.value.code == capi.UMT_ERR_STATE
    umtlib.context_select(ids[-1])
    umtlib.hold_item(-1)
    umtlib.context_select(0)
    umtlib.batch_sweep(ids, capi.UMT_FP32)
    for cid in ids:
        umtlib.context_destroy(cid)


@pytest.mark.parametrize("memory", ["pageable", "pinned", "pinned_unaligned"])
@pytest.mark.parametrize("G", [8, 3])
def test_fp32_sweep_writes_only_exiting_psib_rows(umtlib, memory, G):
    """An FP32 sweep writes the caller's PsiB only on exiting rows, as the
    reference writes PsiB only on the exit list: every row the oracle leaves
    unchanged keeps its FP64 input bit for bit, exiting rows agree with the
    oracle to the FP32 tolerance, and umt103_psib_rows counts them.  G = 3 runs
    the generic FP32 kernel (no zone programs), and a page-locked array that
    is not 16-byte aligned takes the row-kernel path instead of the stage
    kernels' FP64 stores."""
    prob = synthetic_problem((3, 2, 2), 2, 2, G, seed=4, time_dependent=True)
    m = prob.mesh
    A = len(prob.weight)
    rng = np.random.default_rng(5)
    PsiB0 = rng.uniform(0.0, 0.1, size=(A, m.nbelem, G))
    STotal = np.repeat(prob.q_ext, m.numCorner, axis=0) / (4 * np.pi)
    ref = oracle_sweep(prob, savePsi=False, STotal=STotal, Psi=prob.psi0, PsiB=PsiB0)
    umtlib.init(m, prob.omega, prob.weight, G)
    umtlib.set_materials(prob.sigt, prob.sigs, prob.tau)
    umtlib.set_psi(prob.psi0, None)
    if memory == "pageable":
        PsiB = np.empty((A, m.nbelem, G))
    else:
        torch = pytest.importorskip("torch")
        n = A * m.nbelem * G
        buf = torch.empty(n + 1, dtype=torch.float64, pin_memory=True).numpy()
        PsiB = (buf[1:] if memory == "pinned_unaligned" else buf[:n]).reshape(A, m.nbelem, G)
        assert (PsiB.ctypes.data % 16 != 0) == (memory == "pinned_unaligned")
    PsiB[...] = PsiB0
    Phi = umtlib.sweep(STotal, savePsi=False, PsiB=PsiB, precision=capi.UMT_FP32)
    kept = np.all(ref["PsiB"] == PsiB0, axis=2)                  # rows the oracle did not write
    assert kept.any() and (~kept).any()
    assert np.array_equal(PsiB[kept], PsiB0[kept])
    assert rel_err(PsiB[~kept], ref["PsiB"][~kept]) < 1e-4
    assert rel_err(Phi, ref["Phi"]) < 1e-5
    ex, tot = umtlib.psib_rows()
    assert tot == A * m.nbelem
    assert ex == (~kept).sum()                                  # the same exit rows as the oracle's
    # the device's FP32 copy (what the energy tallies read) holds the input
    # rows and the exits, however the rows travelled
    _, PsiB_dev = umtlib.get_psi(capi.UMT_FP32)
    assert np.array_equal(PsiB_dev[kept], PsiB0[kept].astype(np.float32).astype(np.float64))
    assert np.array_equal(PsiB_dev[~kept], PsiB[~kept])


def test_fp32_sweep_pinned_psib_matches_pageable(umtlib):
    """Page-locked and pageable host arrays give bit-identical sweeps, with
    incoming boundary fluxes set and exits returned (the bench passes
    page-locked buffers, whose STotal and PsiB rows arrive in stage-ordered
    chunks beside the stages); the source the call leaves on the device
    drives the next resident sweep identically."""
    torch = pytest.importorskip("torch")
    prob = synthetic_problem((3, 2, 2), 2, 2, 8, seed=9, time_dependent=True)
    m = prob.mesh
    A, G = len(prob.weight), prob.ngr
    rng = np.random.default_rng(3)
    PsiB0 = rng.uniform(0.0, 0.1, size=(A, m.nbelem, G))
    STotal0 = rng.uniform(0.05, 1.0, size=(m.ncornr, G))
    out = []
    for pinned in (False, True):
        umtlib.init(m, prob.omega, prob.weight, G, flags=2 | 8)
        umtlib.set_materials(prob.sigt, prob.sigs, prob.tau)
        umtlib.set_psi(prob.psi0, None)
        if pinned:
            PsiB = torch.empty((A, m.nbelem, G), dtype=torch.float64, pin_memory=True).numpy()
            Phi = torch.empty((m.ncornr, G), dtype=torch.float64, pin_memory=True).numpy()
            STotal = torch.empty((m.ncornr, G), dtype=torch.float64, pin_memory=True).numpy()
        else:
            PsiB = np.empty((A, m.nbelem, G))
            Phi = np.empty((m.ncornr, G))
            STotal = np.empty((m.ncornr, G))
        PsiB[...] = PsiB0
        STotal[...] = STotal0
        umtlib.sweep(STotal, savePsi=True, PsiB=PsiB, precision=capi.UMT_FP32, Phi=Phi)
        umtlib.sweep_resident(False, capi.UMT_FP32)
        out.append((Phi.copy(), PsiB.copy(), umtlib.get_phi(m.ncornr, G)))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    assert np.array_equal(out[0][2], out[1][2])
    assert not np.array_equal(out[1][1], PsiB0)                   # exits were written back


def test_fp32_sweep_source_chunks_follow_each_call(umtlib):
    """The host-facing sweep converts a page-locked STotal in stage-ordered
    chunks read straight from the caller's array, inside a graph that is
    captured once and replayed.  A sequence of calls whose sources differ in
    value and in how they arrive gives, call by call, the same PhiTotal, PsiB
    and device source as the same sequence from pageable arrays.  The
    sequence uses a new page-locked array, the same array refilled, no source
    (zero), a page-locked array that is not 16-byte aligned (copied whole),
    and a page-locked array again."""
    torch = pytest.importorskip("torch")
    prob = synthetic_problem((3, 3, 2), 2, 2, 8, seed=12, time_dependent=True)
    m = prob.mesh
    A, G = len(prob.weight), prob.ngr
    rng = np.random.default_rng(21)
    PsiB0 = rng.uniform(0.0, 0.1, size=(A, m.nbelem, G))
    sources = [rng.uniform(0.05, 1.0, size=(m.ncornr, G)) for _ in range(4)]
    kinds = ["new", "refill", "none", "unaligned", "new"]
    values = [sources[0], sources[1], None, sources[2], sources[3]]

    def pinned(shape, offset=0):
        n = int(np.prod(shape))
        buf = torch.empty(n + offset, dtype=torch.float64, pin_memory=True).numpy()
        return buf[offset:offset + n].reshape(shape)

    runs = []
    for use_pinned in (False, True):
        umtlib.init(m, prob.omega, prob.weight, G, flags=2 | 8)
        umtlib.set_materials(prob.sigt, prob.sigs, prob.tau)
        umtlib.set_psi(prob.psi0, None)
        PsiB = pinned((A, m.nbelem, G)) if use_pinned else np.empty((A, m.nbelem, G))
        Phi = pinned((m.ncornr, G)) if use_pinned else np.empty((m.ncornr, G))
        PsiB[...] = PsiB0
        src = None
        out = []
        for kind, val in zip(kinds, values):
            if val is None:
                S = None
            elif not use_pinned:
                S = val.copy()
            elif kind == "refill" and src is not None:
                src[...] = val
                S = src
            elif kind == "unaligned":
                S = pinned((m.ncornr, G), offset=1)
                assert S.ctypes.data % 16 != 0
                S[...] = val
            else:
                src = pinned((m.ncornr, G))
                src[...] = val
                S = src
            umtlib.sweep(S, savePsi=True, PsiB=PsiB, precision=capi.UMT_FP32, Phi=Phi)
            # the source the call left on the device drives a resident sweep
            umtlib.sweep_resident(False, capi.UMT_FP32)
            out.append((Phi.copy(), PsiB.copy(), umtlib.get_phi(m.ncornr, G)))
        runs.append(out)
    for k, (a, b) in enumerate(zip(*runs)):
        for x, y in zip(a, b):
            assert np.array_equal(x, y), kinds[k]
    # the calls differed: a zero source is not the first source
    assert not np.array_equal(runs[1][0][0], runs[1][2][0])


def test_host_facing_chunks_at_128_directions_match_resident_sweep(umtlib):
    """At 10^3 tiles, 128 directions and 16 groups, the host-facing call
    splits its row lists into many chunks: about 47 of incoming PsiB rows, 5
    of source rows and 47 of exiting rows, each waited for or copied at its
    own stage.  Two calls with page-locked buffers and different sources (the
    second a graph replay) give the PhiTotal and the exiting rows of the
    resident sweep, which converts everything before stage 0, bit for bit.
    Every other row of the caller's PsiB keeps its input."""
    torch = pytest.importorskip("torch")
    t, G = 10, 16
    prob = synthetic_problem((t,) * 3, 4, 4, G, seed=31, time_dependent=True)
    m = prob.mesh
    A = len(prob.weight)
    need = 3 * A * m.ncornr * G * 8                    # the device flux fetched as FP64, plus headroom
    try:
        avail = os.sysconf("SC_AVPHYS_PAGES") * os.sysconf("SC_PAGE_SIZE")
    except (ValueError, OSError, AttributeError):
        avail = None
    if avail is not None and avail < need:
        pytest.skip(f"needs ~{need / 1e9:.0f} GB of free host memory")
    rng = np.random.default_rng(32)
    PsiB0 = rng.uniform(0.0, 0.1, size=(A, m.nbelem, G))
    sources = [rng.uniform(0.05, 1.0, size=(m.ncornr, G)) for _ in range(2)]

    def pinned(shape):
        return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()

    # resident references: the whole source and PsiB converted before stage 0
    umtlib.init(m, prob.omega, prob.weight, G, flags=2 | 8)
    umtlib.set_materials(prob.sigt, prob.sigs, prob.tau)
    refs = []
    for S in sources:
        umtlib.set_psi(prob.psi0, PsiB0)
        umtlib.set_source(S)
        umtlib.sweep_resident(False, capi.UMT_FP32)
        _, PsiB_dev = umtlib.get_psi(capi.UMT_FP32)
        refs.append((umtlib.get_phi(m.ncornr, G), PsiB_dev))
    # host-facing calls on a fresh context
    umtlib.init(m, prob.omega, prob.weight, G, flags=2 | 8)
    umtlib.set_materials(prob.sigt, prob.sigs, prob.tau)
    umtlib.set_psi(prob.psi0, None)
    PsiB, Phi, Sh = pinned((A, m.nbelem, G)), pinned((m.ncornr, G)), pinned((m.ncornr, G))
    for S, (phi_ref, psib_ref) in zip(sources, refs):
        PsiB[...] = PsiB0
        Sh[...] = S
        umtlib.sweep(Sh, savePsi=False, PsiB=PsiB, precision=capi.UMT_FP32, Phi=Phi)
        assert np.array_equal(Phi, phi_ref)
        kept = np.all(PsiB == PsiB0, axis=2)
        assert np.array_equal(PsiB[~kept], psib_ref[~kept])
        ex, tot = umtlib.psib_rows()
        assert (~kept).sum() == ex and tot == A * m.nbelem
    umtlib.finalize()


def test_autotuner_picks_the_fastest_tile_and_keeps_results(umtlib):
    """umt103_autotune times every group tile, keeps the fastest, and the
    tuned sweep equals a sweep with that tile set by hand (bit for bit) and
    the FP64 sweep within the FP32 tolerance; contexts of the same shape in a
    batch take the cached tile."""
    from umt_gb300.problems import synthetic_problem as sp
    prob = sp((4, 4, 3), 4, 4, 16, seed=7, time_dependent=True)
    m = prob.mesh
    st = np.repeat(prob.q_ext, m.numCorner, axis=0) / (4 * np.pi)
    umtlib.init(m, prob.omega, prob.weight, prob.ngr, flags=3 | 8)
    umtlib.set_materials(prob.sigt, prob.sigs, prob.tau)
    umtlib.set_psi(prob.psi0, None)
    umtlib.set_source(st)
    best, times = umtlib.autotune(reps=2)
    assert set(times) == {(16, 1), (8, 2), (4, 4)}
    assert best == min(times, key=times.get)
    umtlib.sweep_resident(False, capi.UMT_FP32)
    tuned = umtlib.get_phi()
    umtlib.set_group_tile(*best)
    umtlib.sweep_resident(False, capi.UMT_FP32)
    assert np.array_equal(umtlib.get_phi(), tuned)
    umtlib.sweep_resident(False, capi.UMT_FP64)
    assert rel_err(tuned, umtlib.get_phi()) < 1e-5
    ids = []
    for _ in range(2):
        cid = umtlib.context_create()
        umtlib.context_select(cid)
        umtlib.init(m, prob.omega, prob.weight, prob.ngr, flags=2 | 8)
        umtlib.set_materials(prob.sigt, prob.sigs, prob.tau)
        umtlib.set_psi(prob.psi0, None)
        umtlib.set_source(st)
        ids.append(cid)
    umtlib.context_select(0)
    umtlib.autotune_contexts(ids)                     # the shape is cached: no timing
    umtlib.batch_sweep(ids, capi.UMT_FP32)
    for cid in ids:
        umtlib.context_select(cid)
        assert np.array_equal(umtlib.get_phi(m.ncornr, prob.ngr), tuned)
    umtlib.context_select(0)
    for cid in ids:
        umtlib.context_destroy(cid)
