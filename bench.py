"""Benchmark: ns per corner*angle*group of one full UCB sweep on GB300.

Workload (one "step" = one sweep of every direction and group, plus the
psi->phi tally, on inputs already resident in HBM): the multigroup
scattering problem of 20x20x20 tiles of the 24-zone tile (192,000 zones,
1,408,000 corners), 4 polar x 4 azimuthal angles per octant (128
directions), 16 groups, total opacity log-uniform on [1e-2, 1e2], scattering
ratio uniform on [0, 0.5], isotropic source 1.0, vacuum boundaries, seeded
(Philox, seed 2).  Synthetic inputs with the stated shapes and distributions
stand in for the reference's problem; there is no dataset.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--tiles T] [--precision fp32|fp64] [--config 2|3|4|5] [--rz]

--config 3 is the larger scattering problem: 30^3 tiles, four materials by
tile (seed 3), total opacity log-uniform on [1e-3, 1e3], scattering ratio up
to 0.9; its sweep is timed without the time-to-converge run, whose FP64
flux buffers (2 x 78 GB) would not fit beside the FP32 ones.  --config 5 is
the strongly scattering 32-group problem: 20^3 tiles, total opacity
log-uniform on [1, 1e3] per zone and group (seed 5), scattering ratio uniform
on [0.95, 0.999]; its sweep is timed, and its time-to-converge leg runs the
same distribution on --ttc-tiles tiles per axis: plain FP64 source iteration
against FP64 and mixed FP64/FP32 iteration with the learned correction
(trained first on seeded problems by the library's own kernels).  --config 4
sweeps all 64 independent problems of uneven size (tiles per axis U{4..16},
4 to 64 groups, 32 or 128 directions; seed 4) in sub-batches that fit in
--c4-budget GB of device memory, each sub-batch from one graph launch,
against the same contexts swept one after another.  --rz times the 2-D RZ
sweep instead (200 x 200 quadrilaterals, 144 directions, 16 groups).

Multi-GPU: by default N GPUs run N independent replicas of the sweep (one
process per GPU, launched by torchrun); value is aggregated over all
replicas (units of all ranks / max time over ranks).  --shard instead splits
one problem's directions over the ranks and times a source-iteration step
with PhiTotal all-reduced in place on the devices.

--impl reference times the reference algorithm on the host cores: the C++
restatement of SweepUCBxyz/SetSweep (oracle/), FP64, OpenMP over directions
with every host thread, on a bounded sample of the same workload (a subset
of directions on the full mesh), and prints the same JSON line.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ns per corner*angle*group sweep"
MEASURED = os.path.join(ROOT, "MEASURED_PEAKS.json")


def b_alg(G: int, A: int, s_psi: int, s_g: int, ncf: int = 3) -> float:
    """Algorithmic bytes per corner*angle*group: read psi_old, write psi_new,
    per (corner, angle) geometry amortised over G, per (corner, group) source
    read and phi write amortised over A."""
    return 2 * s_psi + (s_g * 6 * ncf + 4 * 2 * ncf + s_g) / G + 16.0 / A


# DRAM bytes (read + write) per corner*angle*group unit of the FP32 stage
# kernels, summed by ncu over every stage launch of one whole sweep of the
# bench workload itself (dram__bytes_read.sum + dram__bytes_write.sum, one
# pass, --cache-control none; the ncu summary is kept under profiles/), keyed
# by (tiles per axis, groups).  Traffic per unit grows with the mesh (13.1 B
# on 12^3 tiles at 16 groups), so it is reported only where it was measured.
TRAFFIC_B_PER_UNIT_FP32 = {(20, 16): 17.353, (20, 32): 15.749, (30, 16): 19.649}


def peaks():
    try:
        d = json.load(open(MEASURED))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm = [float(s[1]) for s in self.samples if len(s) > 8 and s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if len(s) > 8 and s[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            if len(s) > 8:
                for k, n in enumerate(names):
                    if s[5 + k].lower().startswith("active"):
                        reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


MATERIALS = {2: "sigma_t log-uniform on [1e-2, 1e2] per zone and group (seed 2), c ~ U[0, 0.5]",
             3: "4 materials by tile (seed 3), sigma_t log-uniform on [1e-3, 1e3], c ~ U[0, 0.9]",
             5: "sigma_t log-uniform on [1, 1e3] per zone and group (seed 5), c ~ U[0.95, 0.999]"}


def make_problem(tiles, config=2):
    """The scattering workloads: 128 directions (P = Az = 4), q = 1,
    tau = 1/(c dt) with dt = 1e-3; config 2 (16 groups) draws opacities per
    zone, config 3 (16 groups) per material with a per-tile material index,
    config 5 (32 groups) per zone with scattering ratios near 1."""
    from umt_gb300.problems import synthetic_problem
    if config == 5:
        return synthetic_problem((tiles,) * 3, 4, 4, 32, seed=5, sigt_range=(1.0, 1e3), c_range=(0.95, 0.999),
                                 q=1.0, time_dependent=True)
    if config == 3:
        return synthetic_problem((tiles,) * 3, 4, 4, 16, seed=3, sigt_range=(1e-3, 1e3), c_range=(0.0, 0.9),
                                 q=1.0, n_materials=4, time_dependent=True)
    return synthetic_problem((tiles,) * 3, 4, 4, 16, seed=2, sigt_range=(1e-2, 1e2), c_range=(0.0, 0.5),
                             q=1.0, time_dependent=True)


def source_from_phi(prob, phi):
    """STotal = (sigma_s * phi + q)/(4 pi) per corner (isotropic scattering source)."""
    from umt_gb300.quadrature import WTISO_XYZ
    m = prob.mesh
    return WTISO_XYZ * (prob.sigs[m.cToZone] * phi + prob.q_ext[m.cToZone])


def run_reference(args, world, rank):
    """Reference arm: the reference algorithm (oracle port) on the host cores."""
    if rank != 0:
        return
    from oracle import pyoracle as po
    prob = make_problem(args.tiles, args.config)
    m = prob.mesh
    A, G = len(prob.weight), prob.ngr
    nth = os.cpu_count() or 1
    sample_angles = min(A, max(nth, 16))
    sel = np.linspace(0, A - 1, sample_angles).round().astype(int)
    om = np.ascontiguousarray(prob.omega[sel]); w = np.ascontiguousarray(prob.weight[sel])
    geo = po.geometry(m)
    S = po.schedule(m, geo[0], geo[1], om)
    Psi = np.ascontiguousarray(prob.psi0[sel])
    PsiB = np.zeros((sample_angles, m.nbelem, G))
    STotal = np.ascontiguousarray(source_from_phi(prob, np.zeros((m.ncornr, G))))
    sigt = np.ascontiguousarray(prob.sigt)
    units = m.ncornr * sample_angles * G
    for _ in range(args.warmup):
        po.set_sweep(m, geo, S, sigt, STotal, prob.tau, om, w, Psi, PsiB, nthreads=nth)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        po.set_sweep(m, geo, S, sigt, STotal, prob.tau, om, w, Psi, PsiB, nthreads=nth)
        times.append(time.perf_counter() - t0)
    t = statistics.median(times)
    v = t * 1e9 / units
    line = {"metric": METRIC, "value": v, "unit": "ns", "impl": "reference", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"multigroup scattering, {args.tiles}^3 tiles, {A} directions, {G} groups",
                       "materials": MATERIALS[args.config], "tiles": args.tiles, "directions": A, "groups": G, "zones": m.nzones,
                       "corners": m.ncornr, "sample_directions": int(sample_angles)},
            "cpu_baseline": {"value": v, "unit": "ns", "cores": nth, "kind": "port",
                             "sample": f"{sample_angles} of {A} directions on the full mesh, all groups"},
            "e2e": {"value": v, "unit": "ns", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def cpu_baseline_sample(prob, budget_s=20.0):
    """Oracle FP64 sweep over a few directions on the full mesh (bounded)."""
    from oracle import pyoracle as po
    m = prob.mesh
    G = prob.ngr
    nth = os.cpu_count() or 1
    n_ang = max(1, min(len(prob.weight), nth))
    sel = np.linspace(0, len(prob.weight) - 1, n_ang).round().astype(int)
    om = np.ascontiguousarray(prob.omega[sel]); w = np.ascontiguousarray(prob.weight[sel])
    geo = po.geometry(m)
    S = po.schedule(m, geo[0], geo[1], om)
    Psi = np.ascontiguousarray(prob.psi0[sel]); PsiB = np.zeros((n_ang, m.nbelem, G))
    STotal = np.ascontiguousarray(source_from_phi(prob, np.zeros((m.ncornr, G))))
    sigt = np.ascontiguousarray(prob.sigt)
    t0 = time.perf_counter(); reps = 0
    while True:
        po.set_sweep(m, geo, S, sigt, STotal, prob.tau, om, w, Psi, PsiB, nthreads=nth)
        reps += 1
        if time.perf_counter() - t0 > budget_s / 2 or reps >= 3:
            break
    t = (time.perf_counter() - t0) / reps
    return {"value": t * 1e9 / (m.ncornr * n_ang * G), "unit": "ns", "cores": nth, "kind": "port",
            "sample": f"{n_ang} of {len(prob.weight)} directions on the full mesh, all groups, FP64"}


def fp64_sweep_figure(lib, prob, units, steps=3):
    """The same workload swept with the FP64 flux (the parity path, FP64
    arithmetic throughout): device time per sweep, so the FP32 figure has a
    same-precision companion beside the FP64 CPU arm."""
    from umt_gb300 import capi
    lib.sweep_resident(False, capi.UMT_FP64)
    ms = []
    for _ in range(steps):
        lib.sweep_resident(False, capi.UMT_FP64)
        ms.append(lib.timing()[0])
    t = statistics.median(ms)
    return {"value": t * 1e6 / units, "unit": "ns", "ms_per_step": t, "steps": steps, "dtype": "f64",
            "kernel": "k_sweep<double> (all dependency stages) + FP64 tally", "bound": "fp64 pipe"}


def time_to_converge(lib, prob, use_gta=False, tol64=1e-8, tol32=1e-7):
    """Second half of the metric: wall time of source iteration to convergence,
    plain FP64 GPU sweeps versus the FP32 sweep (FP64 tallies), and the FP32
    solution's relative L2 error against the FP64 one.  The FP64 GPU path is
    the reference here: it agrees with the CPU oracle to 1e-12 (tests)."""
    from umt_gb300 import capi
    m = prob.mesh
    out = {}
    for prec, tol in ((capi.UMT_FP64, tol64), (capi.UMT_FP32, tol32)):
        lib.set_psi(prob.psi0, None)
        t0 = time.perf_counter()
        r = lib.source_iterate(precision=prec, rel_tol=tol, q_ext=prob.q_ext, save_psi=False, max_iters=400,
                               use_gta=(use_gta and prec == capi.UMT_FP32), allow_notconv=True)
        wall = time.perf_counter() - t0
        out[prec] = (r, wall, lib.get_phi())
    r64, w64, phi64 = out[capi.UMT_FP64]
    r32, w32, phi32 = out[capi.UMT_FP32]
    err = float(np.linalg.norm(phi32 - phi64) / np.linalg.norm(phi64))
    return {"fp64_plain_s": w64, "fp64_iterations": r64["iterations"], "fp64_device_s": r64["seconds"],
            "fp32_s": w32, "fp32_iterations": r32["iterations"], "fp32_device_s": r32["seconds"],
            "fp32_gta": bool(use_gta), "speedup": w64 / w32, "rel_l2_err_fp32_vs_fp64": err,
            "tolerance_fp64": tol64, "tolerance_fp32": tol32}


def run_shard(args, world, rank, local):
    """--shard: one source-iteration step of the config-2 problem with its
    directions split over the ranks (one GPU each): every rank builds the
    scattering source on its device and sweeps its block of directions
    (umt103_si_step), the device PhiTotal is summed over ranks in place by an
    NCCL all-reduce (a torch view of umt103_phi_device), and the change norm
    is taken on the device.  The problem's total work is fixed (strong
    scaling); value = units of the whole problem / max step time over ranks."""
    import torch
    from umt_gb300 import build, capi, sharding
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    build.build()
    lib = capi.Library()
    lib.select_device(local)
    prec = capi.UMT_FP32 if args.precision == "fp32" else capi.UMT_FP64
    prob = make_problem(args.tiles, args.config)
    m = prob.mesh
    A, G = len(prob.weight), prob.ngr
    dirs = sharding.direction_shards(A, world)[rank]
    sw = sharding.DeviceSweeper(lib, prob, dirs, prec)
    phi = sw.phi_tensor()
    reduce = sharding.torch_allreduce_inplace() if dist else (lambda t: t)
    phi.zero_()
    torch.cuda.synchronize()
    sw.change()

    def step():
        sw.step()
        reduce(phi)
        torch.cuda.synchronize()
        return sw.change()

    for _ in range(args.warmup):
        step()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    times = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            rel = step()
            times.append(time.perf_counter() - t0)
    t = sum(times) / len(times)
    if dist:
        tt = torch.tensor([t], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t = float(tt.item())
        dist.barrier()
    units = m.ncornr * A * G
    if rank == 0:
        line = {"metric": METRIC + " (angle-sharded source iteration step)", "value": t * 1e9 / units, "unit": "ns",
                "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
                "higher_is_better": False, "scaling": "strong", "vs_baseline": None,
                "dtype": "f32" if prec == capi.UMT_FP32 else "f64", "data": "synthetic",
                "config": {"workload": f"multigroup scattering, {args.tiles}^3 tiles, {A} directions, {G} groups",
                           "materials": MATERIALS[args.config],
                           "directions_per_rank": [len(d) for d in sharding.direction_shards(A, world)],
                           "parallelism": f"angle{world}",
                           "collective": "NCCL all-reduce of PhiTotal in place (%d FP64 values) per step" % (m.ncornr * G),
                           "l2": "inputs larger than L2"},
                "last_rel_change": rel, "timing": "host wall time of each step (it ends with a device sync)",
                "clocks": clk.summary()}
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def ttc_learned(args, lib):
    """Time to converge on the strongly scattering distribution (config 5:
    sigma_t log-uniform on [1, 1e3], c in [0.95, 0.999], 32 groups, 128
    directions), on a reduced mesh of --ttc-tiles tiles per axis, where plain
    FP64 source iteration still finishes in about a minute.  The learned
    correction is first trained on the device from seeded problems of 3 and
    4 tiles per axis (each solved by FP64 sweeps under GMRES); then every
    method iterates from zero until PhiTotal is within 1e-6 relative L2 of
    the FP64 GMRES answer (checked on the device after each iteration)."""
    from umt_gb300 import capi, learned
    t0 = time.perf_counter()
    train = [learned.strongly_scattering_problem(3 + (k % 2), seed=5000 + k) for k in range(args.train_problems)]
    summary = learned.train_on_problems(lib, train, steps=args.train_steps, batch=4096, lr=2e-3)
    summary["wall_s"] = time.perf_counter() - t0
    prob = learned.strongly_scattering_problem(args.ttc_tiles, seed=5)
    learned.load_problem(lib, prob, flags=3)          # with the grey (GTA) context
    t1 = time.perf_counter()
    phi_star, n_ref = learned.converged_phi(lib, prob)
    ref_s = time.perf_counter() - t1
    runs = {}
    lib.set_gta_solver(capi.UMT_GTA_ZONE)
    lib.set_gta(10, 1e-4, 0)
    for name, prec, le, gta in (("fp64_plain", capi.UMT_FP64, 0, False), ("fp64_learned", capi.UMT_FP64, 5, False),
                                ("fp64_gta", capi.UMT_FP64, 0, True),
                                ("fp32_plain", capi.UMT_FP32, 0, False), ("mixed_plain", capi.UMT_MIXED, 0, False),
                                ("mixed_learned", capi.UMT_MIXED, 5, False)):
        r = learned.iterate_to(lib, prob, phi_star, precision=prec, learn_every=le, learn_start=3,
                               max_iters=4000 if prec != capi.UMT_MIXED else 60, use_gta=gta)
        runs[name] = {k: r[k] for k in ("iterations", "sweeps", "fp64_sweeps", "seconds", "wall_s", "error",
                                         "converged", "learned_kept", "learned_rejected", "grey_sweeps")}
    base = runs["fp64_plain"]["seconds"]
    best = runs["mixed_learned"]
    heldout = heldout_eval(args, lib) if args.eval_seeds > 0 else None
    return {"heldout": heldout,"workload": f"strongly scattering, {args.ttc_tiles}^3 tiles ({prob.mesh.nzones} zones), 128 directions, "
                        f"32 groups, seed 5", "target": "1e-6 relative L2 of PhiTotal vs FP64 GMRES (1e-10)",
            "reference_fp64_sweeps": n_ref, "reference_s": ref_s, "training": summary, "runs": runs,
            "speedup_mixed_learned_vs_fp64_plain": base / best["seconds"] if best["converged"] else None,
            "speedup_fp64_learned_vs_fp64_plain": base / runs["fp64_learned"]["seconds"],
            "speedup_fp64_gta_vs_fp64_plain": base / runs["fp64_gta"]["seconds"],
            "gta": "newer solver (per-zone transfer matrices), 10 BiCGStab iterations at most, tolerance 1e-4",
            "time": "device seconds of umt103_source_iterate (CUDA events); wall_s is the host time of the call"}


def heldout_eval(args, lib):
    """The trained network on --eval-seeds held-out seeds (none used in
    training) of the same distribution on --eval-tiles tiles per axis: each
    problem is solved by FP64 GMRES (1e-10), then iterated from zero to 1e-6
    relative L2 of that answer in FP64 and in the mixed form, each without and
    with the learned step.  Reports the distribution over the seeds."""
    from umt_gb300 import capi, learned
    meth = (("fp64_plain", capi.UMT_FP64, 0), ("fp64_learned", capi.UMT_FP64, 5),
            ("mixed_plain", capi.UMT_MIXED, 0), ("mixed_learned", capi.UMT_MIXED, 5))
    rec = {m[0]: [] for m in meth}
    t0 = time.perf_counter()
    for k in range(args.eval_seeds):
        prob = learned.strongly_scattering_problem(args.eval_tiles, seed=900000 + k)
        learned.load_problem(lib, prob, flags=3 | 8)
        phi_star, _ = learned.converged_phi(lib, prob)
        for name, prec, le in meth:
            r = learned.iterate_to(lib, prob, phi_star, precision=prec, learn_every=le, learn_start=3,
                                   max_iters=4000 if prec != capi.UMT_MIXED else 60)
            rec[name].append((r["iterations"], r["sweeps"], r["fp64_sweeps"], r["seconds"], bool(r["converged"]),
                              r["learned_kept"], r["learned_rejected"]))

    def stats(v):
        v = sorted(v)
        q = lambda f: v[min(len(v) - 1, int(f * (len(v) - 1) + 0.5))]
        return {"min": v[0], "median": q(0.5), "p90": q(0.9), "max": v[-1], "mean": sum(v) / len(v)}

    out = {"seeds": args.eval_seeds, "tiles": args.eval_tiles, "seed_range": [900000, 900000 + args.eval_seeds - 1],
           "wall_s": time.perf_counter() - t0}
    for name in rec:
        rs = rec[name]
        out[name] = {"converged": sum(r[4] for r in rs), "sweeps": stats([r[1] for r in rs]),
                     "fp64_sweeps": stats([r[2] for r in rs]), "seconds": stats([r[3] for r in rs]),
                     "learned_kept": sum(r[5] for r in rs), "learned_rejected": sum(r[6] for r in rs)}
    ratio = lambda a, b, i: [x[i] / y[i] for x, y in zip(rec[a], rec[b])]
    out["fp64_sweep_ratio_plain_over_learned"] = stats(ratio("fp64_plain", "fp64_learned", 1))
    out["mixed_sweep_ratio_plain_over_learned"] = stats(ratio("mixed_plain", "mixed_learned", 1))
    out["time_ratio_fp64_plain_over_mixed_learned"] = stats(ratio("fp64_plain", "mixed_learned", 3))
    out["learned_helps_fp64"] = sum(1 for r in ratio("fp64_plain", "fp64_learned", 1) if r > 1.0)
    out["learned_helps_mixed"] = sum(1 for r in ratio("mixed_plain", "mixed_learned", 1) if r > 1.0)
    return out


def run_rz(args):
    """2-D RZ sweep (--precision, FP32 by default): nr x nz quadrilaterals,
    RZ product quadrature P = 4, Az = 8 (144 directions), 16 groups.  Device
    time of the whole sweep (stage kernels + tally) with CUDA events; end to
    end through umt103_sweep_rz with host buffers; the oracle's FP64 RZ sweep
    on two whole xi-levels of the same mesh as the single-thread CPU
    baseline."""
    import torch
    from umt_gb300 import build, capi
    from umt_gb300.mesh_rz import build_rz_mesh
    from umt_gb300.quadrature_rz import product_quadrature_rz
    build.build()
    lib = capi.Library()
    nr = nzr = args.rz_cells
    m = build_rz_mesh(nr, nzr, distort=0.1, seed=2)
    q = product_quadrature_rz(4, 8)
    G = 16
    A = len(q.weight)
    rng = np.random.Generator(np.random.Philox(2))
    sigt = np.exp(rng.uniform(np.log(1e-2), np.log(1e2), size=(m.nzones, G)))
    STotal = rng.uniform(0.05, 1.0, size=(m.ncornr, G))
    prec = capi.UMT_FP32 if args.precision == "fp32" else capi.UMT_FP64
    lib.init_rz(m, q, G, flags=2 if prec == capi.UMT_FP32 else 1)
    lib.set_materials(sigt, np.zeros_like(sigt), 1.0 / (299.792458 * 1e-3))
    lib.set_psi(np.full((A, m.ncornr, G), 0.5 / np.pi), None)
    # inputs and results in page-locked host memory, allocated once
    def pinned(shape):
        return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()

    STotal_h = pinned((m.ncornr, G))
    STotal_h[...] = STotal
    STotal = STotal_h
    PsiB = pinned((A, m.nbelem, G))
    PsiB[...] = 0.0
    Phi = pinned((m.ncornr, G))
    units = m.ncornr * A * G
    for _ in range(args.warmup):
        lib.sweep_rz(STotal, savePsi=False, PsiB=PsiB, precision=prec, Phi=Phi)
    torch.cuda.synchronize()
    ms = []
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()                # the sampler's start and stop stay outside the window
        for _ in range(args.steps):
            lib.sweep_rz(STotal, savePsi=False, PsiB=PsiB, precision=prec, Phi=Phi)
            ms.append(lib.last_ms())
        t_e2e = (time.perf_counter() - t0) / args.steps
    t_dev = sum(ms) / len(ms)
    line = {"metric": METRIC + " (RZ)", "value": t_dev * 1e6 / units, "unit": "ns", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_dev, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if prec == capi.UMT_FP32 else "f64",
            "data": "synthetic",
            "config": {"workload": f"RZ sweep, {nr}x{nzr} quadrilaterals, 144 directions, 16 groups",
                       "zones": m.nzones, "corners": m.ncornr, "directions": A, "groups": G,
                       "units_per_step": units, "psi": args.precision, "tallies": "fp64",
                       "l2": "angular flux %.2f GB per buffer" % (units * (4 if prec == capi.UMT_FP32 else 8) / 1e9)},
            "e2e": {"value": t_e2e * 1e9 / units, "unit": "ns",
                    "h2d_bytes_per_step": STotal.nbytes + PsiB.nbytes, "d2h_bytes_per_step": Phi.nbytes + PsiB.nbytes,
                    "host_memory": "pinned"},
            "clocks": clk.summary()}
    if not args.no_cpu_baseline:
        from oracle import pyoracle as po
        geo = po.geometry_rz(m)
        keep = np.nonzero(q.level < 2)[0]                      # two whole xi-levels
        sub = product_quadrature_rz(4, 8)
        for k in ("omega", "weight", "starting", "finishing", "level", "alpha", "tau", "angDerivFac",
                  "quadTauW1", "quadTauW2"):
            setattr(sub, k, getattr(sub, k)[keep])
        om3 = np.zeros((len(keep), 3)); om3[:, :2] = sub.omega
        S = po.schedule(m, geo["A_fp"], geo["A_ez"], om3)
        Psi = np.full((len(keep), m.ncornr, G), 0.5 / np.pi); PB = np.zeros((len(keep), m.nbelem, G))
        t0 = time.perf_counter()
        po.set_sweep_rz(m, geo, S, sigt, STotal, 1.0 / (299.792458 * 1e-3), om3, sub, Psi, PB)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": dt * 1e9 / (m.ncornr * len(keep) * G), "unit": "ns", "cores": 1,
                                "kind": "port", "sample": f"{len(keep)} of {A} directions (two xi-levels), FP64"}
    print(json.dumps(line), flush=True)


def config4_draws(n=64, seed=4, tiles=(4, 16)):
    """The batched workload's problems: tiles per axis U{4..16} (or the given
    range), P = Az in {2, 4} (32 or 128 directions), G in {4, 8, 16, 32, 64}."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        t = int(rng.integers(tiles[0], tiles[1] + 1))
        out.append((t, int(rng.choice([2, 4])), int(rng.choice([4, 8, 16, 32, 64])), 400 + k))
    return out


def config4_device_bytes(t, P, G):
    """Device bytes of one FP32 context, estimated with a 10% margin: flux
    (two buffers), corner records, zone programs and headers, FP64
    projections; 7.33 corners per zone."""
    A, nz = 8 * P * P, 24 * t ** 3
    nc = nz * 22 / 3
    return 1.1 * (2 * nc * A * G * 4 + 32 * A * nc + 371 * A * nz + 48 * A * nc)


def run_config4(args):
    """Config 4: independent problems of uneven size resident in separate
    contexts, swept from one graph launch per batch (umt103_batch_sweep),
    against the same contexts swept one after another.  The 64 draws hold
    about 430 GB in FP32, more than one GPU, so they are taken in order in
    sub-batches whose estimated device memory stays within --c4-budget GB;
    each sub-batch is one graph launch, timed, then released before the
    next is built.  The group tile of each problem shape is tuned once
    (umt103_autotune_contexts) and applied in the batch.  Reported: the
    aggregate over all draws (sum of units / sum of sub-batch times)."""
    import gc
    from umt_gb300 import build, capi
    from umt_gb300.problems import synthetic_problem
    build.build()
    lib = capi.Library()
    draws = config4_draws(tiles=tuple(args.c4_tiles))
    batches, cur, used = [], [], 0.0
    for d in draws:
        est = config4_device_bytes(*d[:3])
        if cur and used + est > args.c4_budget * 1e9:
            batches.append(cur)
            cur, used = [], 0.0
        cur.append(d)
        used += est
    if cur:
        batches.append(cur)
    if args.c4_max_batches:
        batches = batches[:args.c4_max_batches]
    tot_units, tot_balg = 0, 0.0
    tb_ms = ts_ms = wb_ms = ws_ms = tn_ms = 0.0
    per_batch = []
    with ClockSampler(0) as clk:
        for taken in batches:
            ids, units, balg_units = [], 0, 0.0
            for (t, P, G, seed) in taken:
                pr = synthetic_problem((t,) * 3, P, P, G, seed=seed, time_dependent=True)
                cid = lib.context_create()
                lib.context_select(cid)
                lib.init(pr.mesh, pr.omega, pr.weight, G, flags=2 | 8)
                lib.set_materials(pr.sigt, pr.sigs, pr.tau)
                lib.set_psi(pr.psi0, None)
                lib.set_source(np.repeat(pr.q_ext, pr.mesh.numCorner, axis=0) / (4 * np.pi))
                u = pr.mesh.ncornr * len(pr.weight) * G
                units += u
                balg_units += b_alg(G, len(pr.weight), 4, 4) * u
                ids.append(cid)
                del pr
                gc.collect()
            lib.context_select(0)
            if not args.c4_no_tune:
                lib.autotune_contexts(ids, reps=1)
            for _ in range(args.warmup):
                lib.batch_sweep(ids, capi.UMT_FP32)
            for cid in ids:
                lib.context_select(cid)
                for _ in range(args.warmup):
                    lib.sweep_resident(False, capi.UMT_FP32)
            lib.context_select(0)
            batch_ms, batch_wall = [], []
            for _ in range(args.steps):
                t0 = time.perf_counter()
                batch_ms.append(lib.batch_sweep(ids, capi.UMT_FP32))
                batch_wall.append((time.perf_counter() - t0) * 1e3)
            # the same batch with every dependency stage of the problems of a group tile in one launch
            lib.set_batch_mode(capi.UMT_BATCH_MERGED)
            for _ in range(args.warmup):
                lib.batch_sweep(ids, capi.UMT_FP32)
            merged_ms = [lib.batch_sweep(ids, capi.UMT_FP32) for _ in range(args.steps)]
            lib.set_batch_mode(capi.UMT_BATCH_GRAPHS)
            seq_ms, seq_wall = [], []
            for _ in range(args.steps):
                tot = 0.0
                t0 = time.perf_counter()
                for cid in ids:
                    lib.context_select(cid)
                    lib.sweep_resident(False, capi.UMT_FP32)
                    tot += lib.timing()[0]
                seq_wall.append((time.perf_counter() - t0) * 1e3)
                seq_ms.append(tot)
            lib.context_select(0)
            for cid in ids:
                lib.context_destroy(cid)
            b, sq = statistics.median(batch_ms), statistics.median(seq_ms)
            wb, ws = statistics.median(batch_wall), statistics.median(seq_wall)
            nb = statistics.median(merged_ms)
            tb_ms += b; ts_ms += sq; wb_ms += wb; ws_ms += ws; tn_ms += nb
            tot_units += units
            tot_balg += balg_units
            per_batch.append({"problems": len(taken), "units": units, "batch_ms": b, "merged_stages_ms": nb,
                              "sequential_ms": sq,
                              "batch_wall_ms": wb, "sequential_wall_ms": ws,
                              "draws": [list(d[:3]) for d in taken]})
    peak, src = peaks()
    achieved = tot_balg / (tb_ms * 1e-3) / 1e9
    ndraws = sum(len(t) for t in batches)
    line = {"metric": METRIC, "value": tb_ms * 1e6 / tot_units, "unit": "ns", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tb_ms, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "batch of independent problems (tiles per axis U{%d..%d}, G in {4..64}, "
                                   "32 or 128 directions; seed 4), one graph launch per sub-batch "
                                   "(each problem's sweep graph nested)" % tuple(args.c4_tiles),
                       "problems": ndraws, "of_draws": len(draws), "sub_batches": len(batches),
                       "device_budget_gb": args.c4_budget, "units_per_step": tot_units,
                       "autotuned": not args.c4_no_tune, "l2": "inputs larger than L2"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": None, "peak_source": src,
                         "kernel": "whole batch (stage kernels and tallies of every problem)",
                         "bytes_per_unit": tot_balg / tot_units},
            "sequential": {"value": ts_ms * 1e6 / tot_units, "unit": "ns", "ms_per_step": ts_ms,
                           "how": "the same contexts swept one after another (umt103_sweep_resident)"},
            "merged_stages": {"value": tn_ms * 1e6 / tot_units, "unit": "ns", "ms_per_step": tn_ms,
                              "how": "the same batch with every dependency stage of the problems that share a "
                                     "group tile in one kernel launch (umt103_set_batch_mode(UMT_BATCH_MERGED))"},
            "wall_clock": {"batch_ms": wb_ms, "sequential_ms": ws_ms, "ratio": ws_ms / wb_ms,
                           "how": "host time of each whole call (launch, wait, status checks); the batch "
                                  "graph is instantiated once and replayed (kept by umt103_batch_sweep)"},
            "sub_batches": per_batch,
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--tiles", type=int, default=None, help="tiles per axis (default 20, or 30 for --config 3)")
    ap.add_argument("--c4-budget", type=float, default=160.0,
                    help="--config 4: device memory (GB) the batch of draws may take")
    ap.add_argument("--c4-max-batches", type=int, default=0, help="--config 4: time only the first N sub-batches")
    ap.add_argument("--c4-no-tune", action="store_true", help="--config 4: skip the per-shape autotuning")
    ap.add_argument("--c4-tiles", type=int, nargs=2, default=(4, 16), metavar=("LO", "HI"),
                    help="--config 4: range of tiles per axis of the draws (default 4 16)")
    ap.add_argument("--config", type=int, default=2, choices=(2, 3, 4, 5),
                    help="2: opacities per zone (default); 3: four materials by tile, c up to 0.9; "
                         "5: 32 groups, c in [0.95, 0.999] (3 and 5: no time-to-converge run)")
    ap.add_argument("--precision", default="fp32")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ttc", action="store_true", help="skip the time-to-converge measurement")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 same-workload sweep figure")
    ap.add_argument("--no-learned", action="store_true", help="--config 5: skip the learned time-to-converge leg")
    ap.add_argument("--shard", action="store_true",
                    help="time the angle-sharded source-iteration step (directions split over the ranks)")
    ap.add_argument("--ttc-tiles", type=int, default=6, help="--config 5: tiles per axis of the time-to-converge mesh")
    ap.add_argument("--train-problems", type=int, default=8, help="--config 5: training problems (3 and 4 tiles per axis)")
    ap.add_argument("--train-steps", type=int, default=1500, help="--config 5: Adam steps")
    ap.add_argument("--eval-seeds", type=int, default=0,
                    help="--config 5: also evaluate the trained network on this many held-out seeds")
    ap.add_argument("--eval-tiles", type=int, default=3, help="--config 5: tiles per axis of the held-out problems")
    ap.add_argument("--gta", action="store_true", help="grey acceleration in the FP32 time-to-converge run")
    ap.add_argument("--gta-solver", type=int, default=1, choices=(1, 2),
                    help="with --gta: 1 grey + stretched-TSA sweeps, 2 grey sweep + per-zone direct solve")
    ap.add_argument("--rz", action="store_true", help="time the 2-D RZ sweep instead (precision as --precision)")
    ap.add_argument("--rz-cells", type=int, default=200, help="RZ mesh: cells per direction")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.tiles is None:
        args.tiles = 30 if args.config == 3 else 20
    if args.config in (3, 5):
        args.no_ttc = True
    world, rank, local = dist_setup()
    if args.config == 4:
        if rank == 0:
            if args.impl == "reference":
                print(json.dumps({"impl": "reference", "unavailable": "config 4 is timed on the GPU arm only"}))
            else:
                run_config4(args)
        return
    if args.rz:
        if rank == 0:
            run_rz(args)
        return
    if args.shard:
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "--shard is timed on the GPU arm only"}))
            return
        run_shard(args, world, rank, local)
        return

    if args.impl == "reference":
        run_reference(args, world, rank)
        return

    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from umt_gb300 import build, capi
    build.build()
    lib = capi.Library()
    lib.select_device(local)
    prec = capi.UMT_FP32 if args.precision == "fp32" else capi.UMT_FP64
    prob = make_problem(args.tiles, args.config)
    m = prob.mesh
    A, G = len(prob.weight), prob.ngr
    # the FP64 flux too (same-precision figure and time to converge) where it fits beside the FP32 one
    # (config 2 unless --no-ttc, config 5 unless --no-fp64; config 3's FP64 flux would not fit)
    fp64_ok = world == 1 and not args.no_fp64 and ((args.config == 2 and not args.no_ttc) or args.config == 5)
    lib.init(m, prob.omega, prob.weight, G, flags=3 if (fp64_ok or (world == 1 and not args.no_ttc)) else
             (2 if prec == capi.UMT_FP32 else 1))
    lib.set_materials(prob.sigt, prob.sigs, prob.tau)
    lib.set_psi(prob.psi0, None)
    STotal = np.ascontiguousarray(source_from_phi(prob, np.zeros((m.ncornr, G))))
    lib.set_source(STotal)
    units = prob.units

    def barrier():
        if dist:
            dist.barrier()

    # ---- device-resident timed region ----
    for _ in range(args.warmup):
        lib.sweep_resident(False, prec)
    barrier()
    kern_ms, tally_ms, step_ms = [], [], []
    launches_per_step = lib.launches_per_sweep(prec)
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            lib.sweep_resident(False, prec)
            t = lib.timing()
            step_ms.append(t[0]); kern_ms.append(t[1]); tally_ms.append(t[2])
    barrier()
    t_step = sum(step_ms) / len(step_ms)
    if dist:
        tt = torch.tensor([t_step], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_step = float(tt.item())
    value = t_step * 1e6 / (units * world)

    # ---- end to end through the public API with host buffers ----
    # inputs and results in page-locked host memory, allocated once
    def pinned(shape):
        return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()

    STotal_h = pinned((m.ncornr, G))
    STotal_h[...] = STotal
    STotal = STotal_h
    Phi = pinned((m.ncornr, G))
    PsiB = pinned((A, m.nbelem, G))
    PsiB[...] = 0.0
    for _ in range(2):
        lib.sweep(STotal, savePsi=False, PsiB=PsiB, precision=prec, Phi=Phi)
    barrier()
    e2e_steps = max(3, min(args.steps, 10))
    call_ms = []
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        tc = time.perf_counter()
        lib.sweep(STotal, savePsi=False, PsiB=PsiB, precision=prec, Phi=Phi)
        call_ms.append((time.perf_counter() - tc) * 1e3)
    t_e2e = (time.perf_counter() - t0) / e2e_steps
    barrier()
    if dist:
        tt = torch.tensor([t_e2e], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_e2e = float(tt.item())
    if prec == capi.UMT_FP32:
        # the FP32 call moves the PsiB rows the sweep reads in and the rows it writes out
        ex_rows, all_rows = lib.psib_rows()
        row_bytes = G * 8
        h2d = STotal.nbytes + (all_rows - ex_rows) * row_bytes
        d2h = Phi.nbytes + ex_rows * row_bytes
    else:
        h2d = STotal.nbytes + PsiB.nbytes
        d2h = Phi.nbytes + PsiB.nbytes

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    s = 4 if prec == capi.UMT_FP32 else 8
    balg = b_alg(G, A, s, s)
    k_avg = sum(kern_ms) / len(kern_ms)
    peak, src = peaks()
    achieved = balg * units / (k_avg * 1e-3) / 1e9
    tpu = TRAFFIC_B_PER_UNIT_FP32.get((args.tiles, G)) if s == 4 else None
    traffic = tpu * units if tpu else None
    line = {
        "metric": METRIC, "value": value, "unit": "ns", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if prec == capi.UMT_FP32 else "f64", "data": "synthetic",
        "config": {"workload": f"multigroup scattering sweep, {args.tiles}^3 tiles (24-zone tile), "
                               f"{A} directions, {G} groups",
                   "materials": MATERIALS[args.config],
                   "tiles": args.tiles, "zones": m.nzones, "corners": m.ncornr, "directions": A,
                   "groups": G, "units_per_step": units, "parallelism": f"replicas{world}",
                   "l2": "inputs larger than L2 (angular flux %.1f GB)" % (A * m.ncornr * G * s / 1e9),
                   "psi": "fp32" if s == 4 else "fp64", "tallies": "fp64"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "traffic_unit": "bytes per sweep",
                     "peak_source": src,
                     "kernel": ("k_sweep32p" if s == 4 else "k_sweep<double>") +
                               " (all dependency stages of one sweep)",
                     "bytes_per_unit": balg, "kernel_ms": k_avg, "tally_ms": sum(tally_ms) / len(tally_ms)},
        "e2e": {"value": t_e2e * 1e9 / (units * world), "unit": "ns", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "host_memory": "pinned",
                "call": "umt103_sweep(STotal, savePsi=0, PhiTotal, PsiB inout, %s)" %
                        ("FP32" if prec == capi.UMT_FP32 else "FP64"),
                "psib": ("rows the sweep reads in, rows it writes out (FP64 host array)"
                         if prec == capi.UMT_FP32 else "whole array both ways"),
                "call_ms": {"min": min(call_ms), "median": statistics.median(call_ms), "max": max(call_ms),
                            "calls": len(call_ms)}},
        "gpu_launches": launches_per_step * args.steps,
        "clocks": clk.summary(),
    }
    if world == 1 and prec == capi.UMT_FP32 and fp64_ok:
        line["fp64"] = fp64_sweep_figure(lib, prob, units)
    if world == 1 and not args.no_ttc:
        if args.gta:
            lib.set_gta_solver(args.gta_solver)
        line["time_to_converge"] = time_to_converge(lib, prob, use_gta=args.gta)
        if args.gta:
            line["time_to_converge"]["gta_solver"] = args.gta_solver
    if world == 1 and args.config == 5 and not args.no_learned:
        line["time_to_converge"] = ttc_learned(args, lib)
    if not args.no_cpu_baseline and world == 1:
        line["cpu_baseline"] = cpu_baseline_sample(prob)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
