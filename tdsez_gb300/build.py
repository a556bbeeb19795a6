"""Build libtdz.so in-tree for sm_103a (nvcc for .cu, g++ through nvcc for
.cpp), one object per source compiled in parallel, then linked.

    python -m tdsez_gb300.build        # or __graft_entry__.build()
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT = HERE / "libtdz.so"
BUILD = HERE / "_build"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libtdz")
    return cand


def sources():
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _flags(src: Path):
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "-I", str(CSRC), "-I", str(HERE.parent / "include")]
    if src.suffix == ".cu":
        return ARCH + ["-lineinfo", "-Xptxas", "-O3"] + common
    return common


def _digest() -> str:
    h = hashlib.sha256()
    for p in sources() + sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [HERE.parent / "include" / "tdz.h"]:
        h.update(p.name.encode())
        h.update(p.read_bytes())
    h.update(" ".join(ARCH).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False) -> Path:
    stamp = BUILD / "stamp"
    dig = _digest()
    if OUT.exists() and stamp.exists() and stamp.read_text() == dig and not force:
        return OUT
    BUILD.mkdir(exist_ok=True)
    cc = nvcc()
    jobs = []
    for src in sources():
        obj = BUILD / (src.name + ".o")
        cmd = [cc, "-c", str(src), "-o", str(obj)] + _flags(src)
        jobs.append((src, obj, cmd))

    def run(job):
        src, obj, cmd = job
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compiling {src.name} failed:\n{r.stdout}\n{r.stderr}")
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(run, jobs))
    link = [cc, "-shared", "-o", str(OUT)] + ARCH + [str(o) for o in objs] + ["-lcudart"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"linking libtdz.so failed:\n{r.stdout}\n{r.stderr}")
    stamp.write_text(dig)
    return OUT


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose=True)
    print(p)
