"""Build the closure engine in-tree (no cmake): libgrg.so and the `comp` CLI.

    python graspan-g_gb300/build.py

Outputs go to graspan-g_gb300/_build/. CUDA code is compiled for sm_103a only.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.environ.get("GRG_BUILD_DIR") or os.path.join(HERE, "_build")
INC = os.path.join(ROOT, "include")
LIB = os.path.join(OUT, "libgrg.so")
COMP = os.path.join(OUT, "comp")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INC, "-I", CSRC]
# tuning overrides of the join kernel, e.g. GRG_NVCC_DEFS="-DGRG_WIN2=16 -DGRG_WIN2_LO=8"
NVCC_FLAGS += os.environ.get("GRG_NVCC_DEFS", "").split()
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-I", INC]
CUDA_INC = ["-I", os.path.join(os.path.dirname(os.path.dirname(shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")), "include")]

CU_SOURCES = ["grg_engine.cu", "grg_format.cu"]
CXX_SOURCES = ["grg_parse.cpp", "grg_part.cpp"]


def _nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    # objects built with other GRG_NVCC_DEFS overrides are stale too
    defs_file = os.path.join(OUT, "nvcc_defs.txt")
    defs = " ".join(NVCC_FLAGS)
    if not os.path.exists(defs_file) or open(defs_file).read() != defs:
        force = True
    nvcc = _nvcc()
    headers = [os.path.join(INC, "grg.h")] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    jobs = []
    objs = []
    for f in CU_SOURCES:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT, f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc] + NVCC_FLAGS + ["-Xptxas", "-v", "-c", src, "-o", obj])
    for f in CXX_SOURCES:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT, f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append(["g++"] + CXX_FLAGS + CUDA_INC + ["-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        logs = list(ex.map(_run, jobs))
    if verbose:
        for line in logs:
            print(line)
    if force or jobs or _stale(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    comp_src = os.path.join(CSRC, "comp.cpp")
    if os.path.exists(comp_src) and (force or _stale(COMP, [comp_src, LIB] + headers)):
        _run(["g++"] + CXX_FLAGS + [comp_src, "-o", COMP, "-L", OUT, "-lgrg", "-Wl,-rpath,$ORIGIN"])
    with open(defs_file, "w") as f:
        f.write(defs)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
