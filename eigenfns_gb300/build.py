"""Build the CUDA library in-tree: eigenfns_gb300/_lib/libeigenfns_gb300.so.

Each csrc/*.cu translation unit is compiled for sm_103a in parallel with nvcc and
linked into one shared library against the shared CUDA runtime (the one PyTorch
loads), so streams and device pointers from torch are valid inside it.

    python -m eigenfns_gb300.build          # or __graft_entry__.build()
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_lib"
LIB = OUT / "libeigenfns_gb300.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", f"-I{INCLUDE}"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build eigenfns_gb300")


def _sources():
    return sorted(CSRC.glob("*.cu"))


def _deps():
    return sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.inc")) + \
        sorted(INCLUDE.glob("*.h"))


def _stale(obj: Path, src: Path, dep_mtime: float) -> bool:
    return not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, dep_mtime)


def build(verbose: bool = False, jobs: int | None = None, force: bool = False) -> Path:
    nvcc = _nvcc()
    objdir = OUT / "obj"
    objdir.mkdir(parents=True, exist_ok=True)
    dep_mtime = max(p.stat().st_mtime for p in _deps())
    srcs = _sources()
    todo = [s for s in srcs if force or _stale(objdir / (s.stem + ".o"), s, dep_mtime)]

    def compile_one(src: Path):
        obj = objdir / (src.stem + ".o")
        cmd = [nvcc, *ARCH, *FLAGS, "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
        return obj

    if todo:
        with ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            list(ex.map(compile_one, todo))
    objs = [objdir / (s.stem + ".o") for s in srcs]
    if force or todo or not LIB.exists() or LIB.stat().st_mtime < max(o.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc, *ARCH, "-shared", "-cudart", "shared", "-o", str(tmp), *map(str, objs),
               "-Xlinker", "-rpath,/usr/local/cuda/lib64"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        tmp.replace(LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
