"""Build recipe for the in-tree CUDA library (sm_103a only).

``python -m tecs_gb300.build`` or ``tecs_gb300.build.build()`` compiles
``csrc/tecs_gpu.cu`` into ``tecs_gb300/_build/libtecs_gb300.so`` with nvcc.
Host code is portable C++17 (x86_64 here, aarch64 on Grace machines).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libtecs_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: no multiply-add contraction, so the pair predicates and the
# force sums keep the reference's rounding (Serial backend, no FMA).
NVCC_FLAGS = ["-O3", "-std=c++20", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC", "-shared"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


DEVICE_HEADERS = PKG.parent / "include" / "tecs" / "device"


def sources():
    return (sorted(CSRC.glob("*.cu")) + sorted(DEVICE_HEADERS.glob("*.cuh")) +
            sorted(DEVICE_HEADERS.glob("*.inc")) + [PKG.parent / "include" / "tecs_gpu.h"])


def build(force: bool = False, verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    newest = max(p.stat().st_mtime for p in sources())
    if LIB.exists() and not force and LIB.stat().st_mtime >= newest:
        return LIB
    # one object per translation unit, compiled in parallel, then one shared library
    units = sorted(CSRC.glob("*.cu"))
    objs, procs = [], []
    for u in units:
        obj = BUILD / (u.stem + ".o")
        cmd = [nvcc(), *ARCH, *NVCC_FLAGS[:-1], "-c", str(u), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append(subprocess.Popen(cmd))
        objs.append(obj)
    failed = [p.wait() for p in procs]
    if any(failed):
        raise subprocess.CalledProcessError(max(failed), "nvcc")
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", *map(str, objs), "-o", str(tmp)]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
