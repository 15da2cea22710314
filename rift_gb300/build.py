"""In-tree build into rift_gb300/_lib/: the CUDA engine (sm_103a,
librift_gb300.so), the host drop-in layer above its C ABI (librift_host.so)
and the command-line driver (rift-sim)."""
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
DEPS = ["rift_engine.cu", "rift_kernels.cuh", "rift_march.cuh", "rift_persist.cuh", "rift_grow.cuh",
        "rift_device.cuh", "rift_ensemble.cuh", "rift_update1.cuh"]


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


HOST_SRC = os.path.join(HERE, "host")
HOST_LIB = os.path.join(LIB_DIR, "librift_host.so")
HOST_CLI = os.path.join(LIB_DIR, "rift-sim")
HOST_SOURCES = ["host_io.cpp", "grid_series.cpp", "simulator.cpp"]
HOST_DEPS = HOST_SOURCES + ["host_internal.hpp", "grid_series.hpp", "rift_sim_main.cpp"]
HOST_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{cmd[0]} failed:\n{r.stdout}\n{r.stderr}")
    return r


def build_host(force: bool = False) -> str:
    """librift_host.so (linked to the engine, found next to it at run time)
    and the rift-sim driver."""
    build(force=force)
    inc = os.path.join(os.path.dirname(HERE), "include")
    deps = [os.path.join(HOST_SRC, d) for d in HOST_DEPS]
    deps += [os.path.join(inc, "rift_host.h"), os.path.join(inc, "rift_gb300.h"), LIB]
    rpath = ["-Wl,-rpath,$ORIGIN", f"-L{LIB_DIR}", "-lrift_gb300"]
    if force or _stale(HOST_LIB, deps):
        _run(["g++", *HOST_FLAGS, "-shared", "-o", HOST_LIB,
              *[os.path.join(HOST_SRC, s) for s in HOST_SOURCES], *rpath])
    if force or _stale(HOST_CLI, deps + [HOST_LIB]):
        _run(["g++", *HOST_FLAGS, "-o", HOST_CLI, os.path.join(HOST_SRC, "rift_sim_main.cpp"),
              f"-L{LIB_DIR}", "-lrift_host", "-lrift_gb300", "-Wl,-rpath,$ORIGIN"])
    return HOST_LIB


CLOSURE_LIB = os.path.join(LIB_DIR, "librift_closure.so")
CLOSURE_DEPS = ["rift_closure.cu", "rift_device.cuh"]


def build(force: bool = False, verbose: bool = False) -> str:
    """The engine and the closure library, compiled side by side."""
    os.makedirs(LIB_DIR, exist_ok=True)
    inc = os.path.join(os.path.dirname(HERE), "include")
    jobs = []
    deps = [os.path.join(SRC, d) for d in DEPS] + [os.path.join(inc, "rift_gb300.h")]
    if force or _stale(LIB, deps):
        jobs.append(["nvcc", *ARCH, *FLAGS, "-o", LIB, *[os.path.join(SRC, s) for s in SOURCES]])
    cdeps = [os.path.join(SRC, d) for d in CLOSURE_DEPS]
    cdeps += [os.path.join(inc, "rift_closure.h"), os.path.join(inc, "rift_gb300.h")]
    if force or _stale(CLOSURE_LIB, cdeps):
        jobs.append(["nvcc", *ARCH, *FLAGS, "-o", CLOSURE_LIB, os.path.join(SRC, "rift_closure.cu")])
    if verbose:
        for cmd in jobs:
            cmd.insert(1, "-Xptxas=-v")
    procs = [subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
             for cmd in jobs]
    errors = []
    for cmd, p in zip(jobs, procs):
        out, err = p.communicate()
        if p.returncode != 0:
            errors.append(f"{cmd[0]} failed:\n{out}\n{err}")
        elif verbose:
            print(err)
    if errors:
        raise RuntimeError("\n".join(errors))
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
    print(build_host(force=True))
