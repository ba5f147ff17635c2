"""Builds libpolatory_gpu.so in-tree for sm_103a (nvcc) and the host objects (g++).

Usage: python polatory_gb300/build.py   (or __graft_entry__.build())
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libpolatory_gpu.so"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found")


def _headers_digest() -> str:
    h = hashlib.sha256()
    for p in sorted(list(CSRC.glob("*.hpp")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))):
        h.update(p.name.encode())
        h.update(p.read_bytes())
    return h.hexdigest()[:16]


def _compile(src: Path, obj: Path, cuda: Path, flags_key: str) -> str:
    stamp = obj.with_suffix(".stamp")
    common = ["-std=c++20", "-O3", f"-I{INCLUDE}", f"-I{CSRC}"]
    if src.suffix == ".cu":
        cmd = [str(cuda / "bin" / "nvcc"), *common, *ARCH, "-lineinfo", "--expt-relaxed-constexpr",
               "-Xcompiler", "-fPIC,-fopenmp,-ffp-contract=off", "-c", str(src), "-o", str(obj)]
    else:
        cmd = ["g++", *common, "-fPIC", "-fopenmp", "-ffp-contract=off", f"-I{cuda / 'include'}",
               "-c", str(src), "-o", str(obj)]
    digest = (hashlib.sha256(src.read_bytes()).hexdigest()[:16] + flags_key +
              hashlib.sha256(" ".join(cmd).encode()).hexdigest()[:8])
    if obj.exists() and stamp.exists() and stamp.read_text() == digest:
        return f"cached {src.name}"
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    stamp.write_text(digest)
    return f"built {src.name}"


def build(verbose: bool = False) -> Path:
    cuda = _cuda_home()
    BUILD.mkdir(exist_ok=True)
    key = _headers_digest()
    sources = sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))
    objs = [BUILD / (s.name + ".o") for s in sources]
    jobs = min(len(sources), max(2, os.cpu_count() or 2))
    with cf.ThreadPoolExecutor(jobs) as ex:
        futs = [ex.submit(_compile, s, o, cuda, key) for s, o in zip(sources, objs)]
        for f in futs:
            msg = f.result()
            if verbose:
                print(msg, file=sys.stderr)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [str(cuda / "bin" / "nvcc"), "-shared", *ARCH, "-o", str(tmp), *map(str, objs),
           "-Xcompiler", "-fopenmp", "-lcudart", "-lgomp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    # The command-line front end (fit / evaluate) over the C ABI.
    cli = PKG / "polatory-gpu"
    cmd = ["g++", "-std=c++20", "-O2", f"-I{INCLUDE}", str(PKG / "cli" / "polatory_gpu_cli.cpp"),
           f"-L{PKG}", "-lpolatory_gpu", "-Wl,-rpath,$ORIGIN", "-o", str(cli)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"cli build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
