"""In-tree build of libg5gpu.so (sm_103a) with nvcc.

Six translation units compiled in parallel:
  g5_fp64.cu   FP64 kernels, --fmad=false (bit-reproducible reference arithmetic)
  g5_mixed.cu  FP32-bulk 2D kernels and the FP32-bulk dispatch, --use_fast_math
  g5_mixed3d.cu FP32-bulk 3D kernels, --use_fast_math
  g5_capi.cu   the C ABI (include/g5gpu.h)
  g5_static.cu the allocation-free g5_step_static and its fixed scratch array
  g5_forest.cpp the host block forest of the dynamic AMR cycle
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libg5gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

UNITS = {
    "g5_fp64.cu": ["--fmad=false"],
    "g5_mixed.cu": ["--use_fast_math"],
    "g5_mixed3d.cu": ["--use_fast_math"],
    "g5_capi.cu": [],
    "g5_static.cu": [],
    "g5_forest.cpp": [],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HERE, "..", "include", "g5gpu.h")]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    procs = []
    objs = []
    for unit, flags in UNITS.items():
        obj = os.path.join(BUILD, os.path.splitext(unit)[0] + ".o")
        objs.append(obj)
        cmd = [cc, *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-c", os.path.join(CSRC, unit), "-o", obj, *flags]
        if extra:
            cmd += extra
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((unit, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = []
    for unit, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((unit, out))
        elif verbose and out.strip():
            print(out, file=sys.stderr)
    if failed:
        msg = "\n".join(f"--- {u}\n{o}" for u, o in failed)
        raise RuntimeError(f"nvcc failed:\n{msg}")
    tmp = LIB + ".tmp"
    subprocess.run([cc, *ARCH, "-shared", "-o", tmp, *objs], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else None)
    print(LIB)
