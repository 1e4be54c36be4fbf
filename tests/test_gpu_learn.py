"""Learned source-iteration correction: the tensor-core (tcgen05) forward
and backward kernels against the float64 CPU restatement, and what the
trained network gains over source iteration without it.

Tolerances: the kernels accumulate in FP32 where the CPU accumulates in
float64, so a hidden activation can round to a neighbouring BF16 value
(2^-8 relative) on one side and not the other.  Outputs and gradients are
therefore compared as relative L2 norms per tensor: 1e-2 against the CPU
with the kernels' BF16 rounding points, 5e-2 against the exact float64
gradient of the same forward pass.
"""
import numpy as np
import pytest

from umt_gb300 import capi
from umt_gb300 import learned
from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _random_inputs(rows, G, seed):
    rng = np.random.default_rng(seed)
    return rng.normal(0.0, 0.7, size=(rows, mo.features(G))).astype(np.float32)


def _params_with_active_output(umtlib, G, seed):
    """Library-initialised weights with a larger output layer, so that the
    outputs (and their gradients) are not dominated by the biases."""
    p = umtlib.mlp_get_params().astype(np.float64)
    d = mo.unpack(p, G)
    rng = np.random.default_rng(seed)
    d["W4"] = rng.normal(0.0, 0.1, size=d["W4"].shape)
    d["b1"] = rng.normal(0.0, 0.05, size=d["b1"].shape)
    d["b4"] = rng.normal(0.0, 0.1, size=d["b4"].shape)
    p = mo.pack(d).astype(np.float32)
    umtlib.mlp_set_params(p)
    return p


@pytest.mark.parametrize("G,rows", [(32, 300), (16, 128), (4, 77), (60, 256)])
def test_mlp_forward_matches_cpu(umtlib, G, rows):
    umtlib.mlp_init(G, seed=G)
    f, h, n = umtlib.mlp_info()
    assert (f, h) == (mo.features(G), 128)
    p = _params_with_active_output(umtlib, G, seed=G + 1)
    assert n == p.size
    X = _random_inputs(rows, G, seed=G + 2)
    Y = umtlib.mlp_forward(X, G)
    ref, _ = mo.forward(p, X, G)
    err = _rel(Y, ref)
    print(f"\nG={G} rows={rows}: forward relative L2 error {err:.2e}")
    assert err < 1e-2
    # a row's outputs depend on that row only (partial last tile included)
    Y1 = umtlib.mlp_forward(X[-1:], G)
    assert _rel(Y1[0], Y[-1]) < 1e-6


@pytest.mark.parametrize("G,rows", [(32, 256), (16, 512), (4, 128)])
def test_mlp_gradient_matches_cpu(umtlib, G, rows):
    umtlib.mlp_init(G, seed=3 * G)
    p = _params_with_active_output(umtlib, G, seed=3 * G + 1)
    X = _random_inputs(rows, G, seed=3 * G + 2)
    rng = np.random.default_rng(3 * G + 3)
    dY = rng.normal(0.0, 1.0, size=(rows, G)).astype(np.float32)
    g = umtlib.mlp_gradient(X, dY).astype(np.float64)
    ref = mo.gradient(p, X, dY, G)
    exact = mo.gradient(p, X, dY, G, exact=True)
    gd, rd, ed = mo.unpack(g, G), mo.unpack(ref, G), mo.unpack(exact, G)
    for k in ("W1", "b1", "W2", "b2", "W3", "b3", "W4", "b4"):
        e1, e2 = _rel(gd[k], rd[k]), _rel(gd[k], ed[k])
        print(f"G={G} {k}: vs CPU (BF16 points) {e1:.2e}, vs exact float64 {e2:.2e}")
        assert e1 < 1e-2, k
        assert e2 < 5e-2, k
    # the gradient is linear in dY
    g2 = umtlib.mlp_gradient(X, 2.0 * dY).astype(np.float64)
    assert _rel(g2, 2.0 * g) < 1e-6


def test_learned_correction_trains_and_accelerates(umtlib):
    """Trained on strongly scattering problems (sigma_t log-uniform on
    [1, 1e3], c in [0.95, 0.999], 32 groups, 128 directions) of 3^3 tiles
    solved to 1e-10 by FP64 sweeps, the network cuts the source iterations
    needed to reach 1e-6 relative L2 of the converged answer on held-out
    seeds, with the residual guard on: in FP64 source iteration, and in the
    mixed iteration (FP64 residual sweeps, FP32 correction sweeps), which
    also reaches 1e-6 where plain FP32 iteration stalls near it."""
    train = [learned.strongly_scattering_problem(3, seed=1000 + k) for k in range(8)]
    summary = learned.train_on_problems(umtlib, train, steps=1500, batch=4096, lr=2e-3)
    print("\n", summary)
    # training happened; what the network gains is asserted below
    assert summary["loss_last"] < 0.7 * summary["loss_first"]
    assert summary["loss_last"] < 0.2
    for seed in (2000, 2001):
        prob = learned.strongly_scattering_problem(3, seed=seed)
        learned.load_problem(umtlib, prob, flags=3 | 8)
        phi_star, _ = learned.converged_phi(umtlib, prob)
        out = {}
        for prec in (capi.UMT_FP64, capi.UMT_MIXED):
            for le in (0, 5):
                r = learned.iterate_to(umtlib, prob, phi_star, precision=prec, learn_every=le, learn_start=3)
                print(f"seed {seed} precision {prec} learn_every {le}: {r['iterations']} iterations, "
                      f"{r['sweeps']} sweeps ({r['fp64_sweeps']} FP64), {r['seconds']:.3f} s, error {r['error']:.2e}, "
                      f"corrections kept {r['learned_kept']}, undone {r['learned_rejected']}")
                assert r["converged"] and r["error"] < 1e-6
                out[prec, le] = r
        assert out[capi.UMT_FP64, 5]["learned_kept"] >= 1
        assert out[capi.UMT_FP64, 5]["sweeps"] < out[capi.UMT_FP64, 0]["sweeps"] / 1.8
        assert out[capi.UMT_MIXED, 5]["sweeps"] < out[capi.UMT_MIXED, 0]["sweeps"] / 1.5
        # the mixed form with the learned step against plain FP64 iteration, device time
        assert out[capi.UMT_MIXED, 5]["seconds"] < out[capi.UMT_FP64, 0]["seconds"] / 3


def test_mixed_iteration_without_model_matches_fp64(umtlib):
    """UMT_MIXED alone (no learned step) on a moderately scattering problem:
    converges to the FP64 iteration's answer to 1e-9 with a few FP64 sweeps."""
    from umt_gb300.problems import synthetic_problem
    prob = synthetic_problem((3, 2, 2), 2, 2, 8, seed=31, c_range=(0.5, 0.95), time_dependent=True)
    learned.load_problem(umtlib, prob, flags=3 | 8)
    r64 = umtlib.source_iterate(precision=capi.UMT_FP64, rel_tol=1e-12, q_ext=prob.q_ext, save_psi=False,
                                max_iters=2000)
    phi64 = umtlib.get_phi()
    rm = umtlib.source_iterate(precision=capi.UMT_MIXED, rel_tol=1e-11, q_ext=prob.q_ext, save_psi=False,
                               max_iters=30, inner_tol=1e-3)
    phim = umtlib.get_phi()
    err = float(np.linalg.norm(phim - phi64) / np.linalg.norm(phi64))
    print(f"\nFP64 {r64['iterations']} iterations; mixed {rm['iterations']} outer, {rm['sweeps']} sweeps "
          f"({rm['fp64_sweeps']} FP64); difference {err:.2e}")
    assert rm["converged"] and err < 1e-9
    assert rm["fp64_sweeps"] <= 8
