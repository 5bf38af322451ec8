"""In-tree build of libspgpu.so (nvcc, sm_103a only, no CMake).

``python -m spatialpy_gb300.build`` compiles every translation unit of
``csrc/`` in parallel and links ``_build/libspgpu.so``.  The NSM and
neighbour-search units are compiled with ``-fmad=false`` so their double
precision arithmetic rounds exactly as written; the SDPD unit likewise, in
both precisions, so it rounds like the CPU oracle.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libspgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
UNITS = {
    "engine.cu": [],
    "nsm.cu": ["-fmad=false"],
    "nsm_batch.cu": ["-fmad=false"],
    "nsm_batchw.cu": ["-fmad=false"],
    "neighbors.cu": ["-fmad=false"],
    "sdpd.cu": ["-fmad=false"],
    "chem.cu": ["-fmad=false"],
    "fno.cu": [],
}


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _compile(unit: str, extra: list, verbose: bool) -> str:
    obj = os.path.join(OUT, unit.replace(".cu", ".o"))
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-I", os.path.join(PKG, "..", "include"), *extra, "-c", os.path.join(SRC, unit),
           "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{r.stdout}\n{r.stderr}")
    if verbose:
        sys.stderr.write(r.stderr)
    return obj


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    srcs = [os.path.join(SRC, f) for f in os.listdir(SRC)]
    srcs.append(os.path.join(PKG, "..", "include", "spgpu.h"))
    return any(os.path.getmtime(s) > t for s in srcs)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    with cf.ThreadPoolExecutor(len(UNITS)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1], verbose), UNITS.items()))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
