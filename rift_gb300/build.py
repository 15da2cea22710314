"""In-tree build of the CUDA engine (sm_103a) into rift_gb300/_lib/."""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIB_DIR, "librift_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-use_fast_math", "-lineinfo", "-Xcompiler", "-fPIC", "-shared"]
SOURCES = ["rift_engine.cu"]
DEPS = ["rift_engine.cu", "rift_kernels.cuh", "rift_march.cuh", "rift_persist.cuh", "rift_grow.cuh", "rift_device.cuh"]


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(LIB_DIR, exist_ok=True)
    deps = [os.path.join(SRC, d) for d in DEPS]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "rift_gb300.h"))
    if force or _stale(LIB, deps):
        cmd = ["nvcc", *ARCH, *FLAGS, "-o", LIB, *[os.path.join(SRC, s) for s in SOURCES]]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
