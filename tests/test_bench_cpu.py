"""The benchmark's own arithmetic and contract, on the CPU: algorithmic bytes
per unit, the synthetic workloads' stated distributions, and the JSON line of
the reference arm (the reference algorithm on the host cores)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

import bench

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("G,A,s,expect", [(16, 128, 4, 14.375), (32, 128, 4, 11.25), (16, 128, 8, 27.125)])
def test_algorithmic_bytes_per_unit(G, A, s, expect):
    """B_alg = 2 s_psi + (6 nCF s_g + 8 nCF + s_g)/G + 16/A with nCF = 3."""
    assert bench.b_alg(G, A, s, s) == pytest.approx(expect, abs=1e-12)


@pytest.mark.parametrize("config,G,sig_range,c_range", [
    (2, 16, (1e-2, 1e2), (0.0, 0.5)),
    (3, 16, (1e-3, 1e3), (0.0, 0.9)),
    (5, 32, (1.0, 1e3), (0.95, 0.999)),
])
def test_workload_distributions(config, G, sig_range, c_range):
    """Each workload has its stated groups, directions, opacity and
    scattering-ratio ranges (on 2^3 tiles; the draws do not depend on size
    beyond their count)."""
    p = bench.make_problem(2, config)
    assert p.ngr == G and len(p.weight) == 128
    assert p.tau == pytest.approx(1.0 / (299.792458 * 1e-3))
    sig = p.siga + p.sigs                      # material opacity, without tau
    assert sig.min() >= sig_range[0] * (1 - 1e-12) and sig.max() <= sig_range[1] * (1 + 1e-12)
    c = p.sigs / sig
    assert c.min() >= c_range[0] - 1e-12 and c.max() <= c_range[1] + 1e-12
    if config == 3:                            # four materials by tile
        assert len(np.unique(sig[:, 0])) <= 4
    assert np.allclose(p.sigt, sig + p.tau)


def test_reference_arm_json_line():
    """`bench.py --impl reference` prints one JSON line with the keys the
    benchmark contract asks for (2^3 tiles here, so it runs in seconds)."""
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--tiles", "2", "--steps", "1",
                        "--warmup", "3"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["higher_is_better"] is False and d["warmup"] >= 3
    assert d["value"] > 0 and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["config"]["groups"] == 16 and d["config"]["directions"] == 128


def test_config4_draws_and_memory_budget():
    """The batched workload's draws have the stated ranges; all 64 need more
    device memory than one GPU holds, so the bench takes the prefix that fits
    its budget; the estimate errs high (the 20^3-tile, 128-direction,
    16-group context holds about 48 GB)."""
    d = bench.config4_draws()
    assert len(d) == 64 and d == bench.config4_draws()
    assert all(4 <= t <= 16 and P in (2, 4) and G in (4, 8, 16, 32, 64) for t, P, G, _ in d)
    est = [bench.config4_device_bytes(t, P, G) for t, P, G, _ in d]
    assert sum(est) > 280e9
    n, used = 0, 0.0
    while n < len(est) and used + est[n] <= 160e9:
        used += est[n]; n += 1
    assert n == 11
    assert 48e9 < bench.config4_device_bytes(20, 4, 16) < 56e9
    small = bench.config4_draws(tiles=(2, 4))
    assert all(2 <= t <= 4 for t, _, _, _ in small)
