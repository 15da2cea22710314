"""The integer dt division (rift_gb300/csrc/rift_divdf.h) returns the FP64
quotient bit for bit: compiled for the host with g++ and checked against
the hardware FP64 division on 27 million operand pairs."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_divdf_matches_fp64_division(tmp_path):
    exe = tmp_path / "divdf_check"
    src = os.path.join(HERE, "native", "divdf_check.cpp")
    try:
        subprocess.run(["g++", "-O2", "-std=c++17", "-o", str(exe), src], check=True,
                       capture_output=True, text=True)
    except FileNotFoundError:
        pytest.skip("no g++")
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    n, bad = map(int, r.stdout.split()[-2:])
    assert r.returncode == 0 and bad == 0 and n > 20_000_000, r.stdout
