"""Builds libgridoxide_gb300.so in-tree (sm_103a), no cmake, parallel compile.

    python -m gridoxide_gb300.build        # or gridoxide_gb300.build.build()
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libgridoxide_gb300.so")
OBJ = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["gox_symbolic.cpp", "gox_engine.cpp", "gox_stream.cpp", "gox_api.cu"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _compile(src: str, nvcc: str, extra: list[str]) -> str:
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    path = os.path.join(CSRC, src)
    if src.endswith(".cu"):
        cmd = [nvcc, "-c", path, "-o", obj, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
               "--expt-relaxed-constexpr"] + ARCH + extra
    else:
        cmd = [nvcc, "-c", path, "-o", obj, "-O2", "-std=c++17", "-Xcompiler", "-fPIC",
               "-Xcompiler", "-ffp-contract=off"]
    subprocess.run(cmd, check=True)
    return obj


def _stale() -> bool:
    if not os.path.exists(OUT):
        return True
    t = os.path.getmtime(OUT)
    for d, _, files in os.walk(CSRC):
        for f in files:
            if os.path.getmtime(os.path.join(d, f)) > t:
                return True
    inc = os.path.join(os.path.dirname(HERE), "include")
    for f in os.listdir(inc):
        if os.path.getmtime(os.path.join(inc, f)) > t:
            return True
    return False


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    if not force and not _stale():
        return OUT
    os.makedirs(OBJ, exist_ok=True)
    nvcc = _nvcc()
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, nvcc, extra), SOURCES))
    tmp = OUT + ".tmp"
    subprocess.run([nvcc, "-shared", "-o", tmp] + objs + ARCH + ["-lcudart_static", "-lrt",
                   "-lpthread", "-ldl"], check=True)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
