"""Builds the oracle (test infrastructure only) into oracle/_build/liboracle.so with gcc."""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
OUT = HERE / "_build" / "liboracle.so"


def build() -> Path:
    src = HERE / "oracle.c"
    OUT.parent.mkdir(exist_ok=True)
    if OUT.exists() and OUT.stat().st_mtime > max(src.stat().st_mtime,
                                                   (ROOT / "include" / "polatory_gpu.h").stat().st_mtime):
        return OUT
    tmp = OUT.with_suffix(".so.tmp")
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", f"-I{ROOT / 'include'}",
           str(src), "-o", str(tmp), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build())
