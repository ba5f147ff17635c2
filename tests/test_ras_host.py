"""CPU test of the RAS host set-up (domain division, coarse points): compiles
tests/ras_host_check.cpp against polatory_gb300/csrc/ras_host.cpp with g++ and runs it.
Restates test/preconditioner/test_domain_divider.cpp:18-90 and
test/polynomial/test_lagrange_basis.cpp:16-31, and checks the level-parallel coarse-point
selection against a sequential priority-queue restatement."""
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_domain_divider_and_coarse_points(tmp_path):
    exe = tmp_path / "ras_host_check"
    cmd = ["g++", "-O2", "-std=c++20", "-fopenmp", "-ffp-contract=off", f"-I{ROOT / 'include'}",
           f"-I{ROOT / 'polatory_gb300' / 'csrc'}", "-I/usr/local/cuda/include",
           str(ROOT / "tests" / "ras_host_check.cpp"),
           str(ROOT / "polatory_gb300" / "csrc" / "ras_host.cpp"), "-o", str(exe)]
    subprocess.run(cmd, check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ok" in r.stdout
