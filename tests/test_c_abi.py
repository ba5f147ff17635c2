"""The boundary from the caller's side: a plain C program compiled against include/polatory_gpu.h,
and the C++ binding of INTEGRATION.md (the reference-side wrapper a maintainer would add)
compiled against minimal stand-ins of the reference's types. On CPU both must compile; on the
GPU both are linked against libpolatory_gpu.so and run a fit + evaluation."""
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HERE = Path(__file__).resolve().parent / "c_abi"
LIBDIR = ROOT / "polatory_gb300"


def extract_binding(tmp_path) -> Path:
    text = (ROOT / "INTEGRATION.md").read_text()
    block = re.search(r"```cpp\n(.*?)```", text, flags=re.S).group(1)
    out = tmp_path / "gpu_interpolant.hpp"
    out.write_text("#pragma once\n" + block)
    return tmp_path


def c_cmd(out, syntax_only):
    cmd = ["gcc", "-std=c11", "-Wall", "-Werror", f"-I{ROOT / 'include'}", str(HERE / "fit_evaluate.c")]
    if syntax_only:
        return cmd + ["-fsyntax-only"]
    return cmd + [f"-L{LIBDIR}", "-lpolatory_gpu", f"-Wl,-rpath,{LIBDIR}", "-lm", "-o", str(out)]


def cpp_cmd(inc, out, syntax_only):
    cmd = ["g++", "-std=c++20", "-Wall", "-Werror", f"-I{inc}", f"-I{HERE / 'stub'}",
           f"-I{ROOT / 'include'}", str(HERE / "cpp_binding_main.cpp")]
    if syntax_only:
        return cmd + ["-fsyntax-only"]
    return cmd + [f"-L{LIBDIR}", "-lpolatory_gpu", f"-Wl,-rpath,{LIBDIR}", "-o", str(out)]


def test_c_program_and_cpp_binding_compile(tmp_path):
    subprocess.run(c_cmd(None, True), check=True)
    inc = extract_binding(tmp_path)
    subprocess.run(cpp_cmd(inc, None, True), check=True)


@pytest.mark.gpu
def test_c_program_runs_against_the_library(tmp_path):
    exe = tmp_path / "fit_evaluate"
    subprocess.run(c_cmd(exe, False), check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "max_error" in r.stdout


@pytest.mark.gpu
def test_cpp_binding_runs_against_the_library(tmp_path):
    inc = extract_binding(tmp_path)
    exe = tmp_path / "cpp_binding"
    subprocess.run(cpp_cmd(inc, exe, False), check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
