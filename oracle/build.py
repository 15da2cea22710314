"""Build recipe for the test oracle (test infrastructure).

- librift_oracle.so : the FP64 CPU restatement (oracle/rift_oracle.cpp), g++.
- rift_ref_sm103a.fatbin : the reference's own grid.cu compiled for sm_103a
  with the reference's --use_fast_math, from the sources where they lie in
  the reference tree.  Built only where that tree is present; the output goes
  to oracle/_ref/ (git-ignored) and goes with the repository to the machine
  that has the GPU.
- refrun : the driver-API host runner for that fatbin (oracle/refkit/refrun.cu),
  built on whichever machine runs it.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BIN = os.path.join(HERE, "_bin")
REF_OUT = os.path.join(HERE, "_ref")
# Read-only reference sources, present only where the fatbin is built: the
# RIFT_REFERENCE_TREE environment variable, else a "reference" directory beside
# this repository's root.
REFERENCE_TREE = os.environ.get(
    "RIFT_REFERENCE_TREE",
    os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def _newer(out, srcs):
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(s) <= t for s in srcs)


def oracle_lib_path():
    return os.path.join(BIN, "librift_oracle.so")


def build_oracle(force=False):
    os.makedirs(BIN, exist_ok=True)
    src = os.path.join(HERE, "rift_oracle.cpp")
    out = oracle_lib_path()
    deps = [src, os.path.join(HERE, "rift_oracle.h"),
            os.path.join(os.path.dirname(HERE), "include", "rift_gb300.h")]
    if force or not _newer(out, deps):
        # -ffp-contract=off: no FMA contraction, so x86 and aarch64 hosts
        # produce identical oracle results.
        _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
              "-o", out, src])
    return out


def fatbin_path():
    return os.path.join(REF_OUT, "rift_ref_sm103a.fatbin")


def build_ref_fatbin(force=False):
    """Compile the reference's grid.cu (device code only) where the reference
    tree exists; a no-op elsewhere (the prebuilt fatbin is used)."""
    if not os.path.isdir(REFERENCE_TREE) or shutil.which("nvcc") is None:
        return fatbin_path() if os.path.exists(fatbin_path()) else None
    os.makedirs(REF_OUT, exist_ok=True)
    src = os.path.join(HERE, "refkit", "ref_device.cu")
    out = fatbin_path()
    deps = [src, os.path.join(REFERENCE_TREE, "grid.cu")]
    if force or not _newer(out, deps):
        _run(["nvcc", "-fatbin", *ARCH, "--use_fast_math", "-std=c++17",
              "-I", os.path.join(HERE, "refkit", "shim"), "-I", REFERENCE_TREE, src, "-o", out])
    return out


def refrun_path():
    return os.path.join(BIN, "refrun")


def build_refrun(force=False):
    if shutil.which("nvcc") is None:
        return None
    os.makedirs(BIN, exist_ok=True)
    src = os.path.join(HERE, "refkit", "refrun.cu")
    out = refrun_path()
    if force or not _newer(out, [src]):
        # host float arithmetic without FMA contraction (the series
        # interpolation must round like the x86 host build of the reference)
        _run(["nvcc", "-O2", "-std=c++17", *ARCH, "-Xcompiler", "-ffp-contract=off", "-o", out,
              src, "-lcuda"])
    return out


def build_all(force=False):
    return dict(oracle=build_oracle(force), fatbin=build_ref_fatbin(force),
                refrun=build_refrun(force))


if __name__ == "__main__":
    print(build_all(force=True))
