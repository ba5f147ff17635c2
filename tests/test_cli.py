"""The command-line front end (polatory-gpu fit / evaluate, the reference's cli/fit_command.cpp
and cli/evaluate_command.cpp on the GPU library): on CPU its usage and argument errors; on the
GPU a fit from a table file and an evaluation from the saved interpolant file, compared with the
library's own fit and the oracle."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
CLI = ROOT / "polatory_gb300" / "polatory-gpu"


def run(*args):
    return subprocess.run([str(CLI), *map(str, args)], capture_output=True, text=True, timeout=600)


def test_usage_and_argument_errors(tmp_path):
    r = run("--help")
    assert r.returncode == 0 and "polatory-gpu fit" in r.stdout
    assert run().returncode == 1
    r = run("fit", "--in", tmp_path / "none.csv", "--dim", "2", "--rbf", "bh3", "--tol", "1e-3",
            "--out", tmp_path / "o.bin")
    assert r.returncode == 1 and "only --dim 3" in r.stderr
    r = run("fit", "--in", tmp_path / "none.csv", "--dim", "3", "--rbf", "bh3", "--tol", "1e-3",
            "--out", tmp_path / "o.bin")
    assert r.returncode == 1 and "cannot open file" in r.stderr
    (tmp_path / "t.csv").write_text("0 0 0 1\n")
    r = run("fit", "--in", tmp_path / "t.csv", "--dim", "3", "--rbf", "xyz", "1", "--tol", "1e-3",
            "--out", tmp_path / "o.bin")
    assert r.returncode == 1 and "unknown RBF" in r.stderr


@pytest.mark.gpu
def test_fit_and_evaluate_round_trip(tmp_path):
    import oracle
    import polatory_gb300 as pg
    from polatory_gb300 import workloads

    g = np.random.Generator(np.random.PCG64(81))
    pts = g.random((3000, 3))
    vals = workloads.f_c1(pts)
    lines = ["# x y z value"] + [",".join(f"{float(c):.17g}" for c in (*p, v)) for p, v in zip(pts, vals)]
    (tmp_path / "in.csv").write_text("\n".join(lines) + "\n")
    q = g.random((500, 3))
    (tmp_path / "q.txt").write_text("\n".join(" ".join(f"{float(c):.17g}" for c in p) for p in q) + "\n")
    r = run("fit", "--in", tmp_path / "in.csv", "--dim", "3", "--rbf", "bh3", "1.0", "--deg", "1",
            "--tol", "1e-6", "--out", tmp_path / "model.bin")
    assert r.returncode == 0, r.stderr
    r = run("evaluate", "--in", tmp_path / "model.bin", "--points", tmp_path / "q.txt", "--dim", "3",
            "--out", tmp_path / "out.txt")
    assert r.returncode == 0, r.stderr
    out = np.loadtxt(tmp_path / "out.txt")
    assert out.shape == (500, 4)
    assert np.array_equal(out[:, :3], q)
    it = pg.Interpolant.load(str(tmp_path / "model.bin"))
    model = pg.Model(pg.Biharmonic3D([1.0]), 1)
    want = oracle.direct_evaluate(model, it.centers, it.weights, q)
    assert np.max(np.abs(out[:, 3] - want)) <= 1e-9
    # The residual of the command-line fit at the data points, recomputed by the oracle.
    fit_vals = oracle.direct_evaluate(model, it.centers, it.weights, pts)
    assert np.max(np.abs(fit_vals - vals)) <= 1e-6
    # Values and gradients (--grads): seven columns.
    r = run("evaluate", "--in", tmp_path / "model.bin", "--points", tmp_path / "q.txt", "--dim", "3",
            "--grads", "--out", tmp_path / "outg.txt")
    assert r.returncode == 0, r.stderr
    outg = np.loadtxt(tmp_path / "outg.txt")
    assert outg.shape == (500, 7)
    assert np.max(np.abs(outg[:, 3] - want)) <= 1e-9
