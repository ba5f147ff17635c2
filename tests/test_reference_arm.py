"""CPU checks of the benchmark's reference arm and of the oracle it times: the arm never loads the
product library, runs small configurations whole and large ones as a bounded sample that says
so, and the oracle's blocked LU solve of the fit system agrees with numpy's LAPACK solve."""
import json
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import oracle

ROOT = Path(__file__).resolve().parent.parent


def run_reference_arm(*args):
    code = ("import runpy, sys, json\n"
            f"sys.argv = ['bench.py', '--impl', 'reference', *{list(args)!r}]\n"
            "runpy.run_path('bench.py', run_name='__main__')\n"
            "print(json.dumps({'product_loaded': any(m.startswith('polatory_gb300') "
            "for m in sys.modules)}))\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    return lines[0], lines[-1]["product_loaded"]


def test_reference_arm_samples_large_configs():
    # c2 at 0.01 scale: 30,000 data points (above the dense limit) -> 12,000 of them and every
    # one of the 20,000 queries per step, labelled as a sample that does not carry over.
    line, loaded = run_reference_arm("--workload", "c2", "--scale", "0.01", "--steps", "1",
                                     "--warmup", "0")
    assert not loaded
    assert "unavailable" not in line and line["value"] > 0
    cb = line["cpu_baseline"]
    assert cb["comparable"] is False and "12000 of the 30000 data points" in cb["sample"]
    assert "does not carry over" in cb["sample"]


def test_reference_arm_samples_batched_fits():
    line, loaded = run_reference_arm("--workload", "c4", "--scale", "0.004", "--steps", "1",
                                     "--warmup", "0")
    assert not loaded
    assert line["value"] > 0 and "first" in line["cpu_baseline"]["sample"]


def test_reference_arm_reports_serving_unavailable():
    line, loaded = run_reference_arm("--workload", "c5")
    assert line["impl"] == "reference"
    assert "unavailable" in line and "cannot be built" in line["unavailable"]
    assert not loaded


def test_reference_arm_runs_a_small_config_in_full():
    # c2 at 0.001 scale: 3,000 data points + 2,000 queries, the whole (scaled) configuration.
    line, loaded = run_reference_arm("--workload", "c2", "--scale", "0.001", "--steps", "1",
                                     "--warmup", "0")
    assert not loaded
    assert "unavailable" not in line
    assert line["value"] > 0 and line["steps"] == 1
    assert line["config"]["n_fit"] == 3000 and line["config"]["n_eval"] == 2000
    assert line["e2e"]["value"] == line["value"]


def saddle_matrix(pts, nugget=0.0):
    """[A + nugget I, P; P^T, 0] of biharmonic3d (-r) with a degree-1 polynomial."""
    n = pts.shape[0]
    d = np.linalg.norm(pts[:, None, :] - pts[None, :, :], axis=2)
    p = np.concatenate([np.ones((n, 1)), pts], axis=1)
    a = np.zeros((n + 4, n + 4))
    a[:n, :n] = -d + nugget * np.eye(n)
    a[:n, n:] = p
    a[n:, :n] = p.T
    return a


@pytest.mark.parametrize("n", [5, 63, 64, 130, 257])
def test_oracle_blocked_lu_matches_lapack(n):
    g = np.random.Generator(np.random.PCG64(n))
    pts = g.random((n, 3))
    vals = g.standard_normal(n)
    model = oracle.model("bh3", [1.0], 1)
    got = oracle.fit_exact(model, pts, vals)
    want = np.linalg.solve(saddle_matrix(pts), np.concatenate([vals, np.zeros(4)]))
    assert np.max(np.abs(got - want)) <= 1e-9 * max(1.0, np.max(np.abs(want)))
