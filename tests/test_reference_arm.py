"""CPU checks of the benchmark's reference arm and of the oracle it times: the arm never loads the
product library, reports the configurations it cannot run in full as unavailable (with the
reason), and the oracle's blocked LU solve of the fit system agrees with numpy's LAPACK solve."""
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


@pytest.mark.parametrize("workload", ["c2", "c3", "c4", "c5"])
def test_reference_arm_reports_oversized_configs_unavailable(workload):
    line, loaded = run_reference_arm("--workload", workload, "--scale", "0.05")
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
