"""Generate the golden fixtures by running the REFERENCE's own kernels.

Runs on a GB300 machine (after __graft_entry__.build()), through
oracle/_bin/refrun and the reference device fatbin oracle/_ref/
rift_ref_sm103a.fatbin.  Writes one .npz per case into --out; the committed
copies live in tests/golden/.  Every input array is stored in the fixture so
the tests never depend on regenerating the same random numbers.

    python tests/golden/make_golden.py --out <output directory>
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from rift_gb300 import synth  # noqa: E402
import refcase  # noqa: E402

FATBIN = os.path.join(ROOT, "oracle", "_ref", "rift_ref_sm103a.fatbin")
REFRUN = os.path.join(ROOT, "oracle", "_bin", "refrun")


def probe_table():
    """Limiter inputs covering the low-word signf cases: exact zeros, values
    whose low 31 mantissa bits are zero (+-1, +-2.5, 0.5, ...), generic
    values of both signs, and values differing only in mantissa bit 31."""
    rng = np.random.default_rng(11)
    short = np.array([0.0, -0.0, 1.0, -1.0, 2.5, -2.5, 0.5, -0.25, 3.0, 1e-3, -7.125])
    gen = rng.normal(0, 1, 60) * 10.0 ** rng.integers(-8, 2, 60)
    bit31 = []
    for v in rng.normal(0, 1, 10):
        b = np.float64(v).view(np.uint64)
        bit31.append(np.uint64(b | np.uint64(0x80000000)).view(np.float64))
        bit31.append(np.uint64(b & ~np.uint64(0x80000000)).view(np.float64))
    vals = np.concatenate([short, gen, np.array(bit31)])
    a = rng.choice(vals, 400)
    b = rng.choice(vals, 400)
    c = rng.choice(vals, 400)
    # hand-picked rows
    rows = [(-0.3, -0.2, -0.1), (0.3, -0.2, 0.1), (0.0, 1.0, 2.0), (1.0, 2.0, 3.0),
            (0.123, 0.456, 0.789), (-0.123, -0.456, -0.789), (1e-9, 2e-9, 3e-9)]
    a[: len(rows)] = [r[0] for r in rows]
    b[: len(rows)] = [r[1] for r in rows]
    c[: len(rows)] = [r[2] for r in rows]
    return a, b, c


def run_ref(case_dir, out_dir):
    os.makedirs(out_dir, exist_ok=True)
    r = subprocess.run([REFRUN, FATBIN, case_dir, out_dir], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"refrun failed ({r.returncode}): {r.stderr}\n{r.stdout}")
    return r.stdout


def case_inputs(case):
    BX, BY = case.faces()
    d = dict(BX=BX, BY=BY, n=case.n, flags=case.flags, cell=case.cell, kappa=case.kappa,
             courant=case.courant, psi=case.psi, dtheta=case.dtheta, t0=case.t0, B=case.B)
    if case.K is not None:
        d["K"] = case.K
    if case.h0 is not None:
        d["h0"] = case.h0
    for w, (t, r) in case.series.items():
        d[f"series{w}_t"] = t
        d[f"series{w}_r"] = r
    if case.src_idx is not None:
        d["src_idx"] = case.src_idx
    return d


def golden_cases():
    cases = []
    # A: uniform rain on a bumpy plane, tile acceleration on
    a = synth.small_case(40, 36, seed=7)
    cases.append(("rain", a, 60, (1, 2, 5, 20, 60), None, None))
    # B: initial depth, infiltration, point source, uniform drain, max/arrival maps
    b = synth.small_case(44, 30, seed=3, h0_depth=0.4)
    b.flags |= (synth.INFILTRATION | synth.POINT_SOURCE | synth.DRAIN_UNIFORM | synth.SAVE_MAX
                | synth.SAVE_ARRIVAL)
    rng = np.random.default_rng(5)
    b.K = np.zeros_like(b.n)
    b.K[2:-2, 2:-2] = np.exp(np.log(5.0) + 0.8 * rng.standard_normal((30, 44))) / 3.6e6
    b.psi, b.dtheta = 0.11, 0.3
    b.src_idx = np.array([(12 + 2) * b.h_nx + (10 + 2), (12 + 2) * b.h_nx + (11 + 2)], np.int32)
    b.series[2] = synth.csv_series([0, 0.05, 0.2], [0, 300, 0])
    b.series[1] = synth.csv_series([0, 1], [20, 20])
    cases.append(("h0_infil_src", b, 40, (1, 10, 40), None, None))
    # C: dry domain, wet front from a point source (activity grows)
    c = synth.small_case(64, 56, seed=9, rain_mmhr=0.0)
    c.flags = synth.POINT_SOURCE | synth.TILE_ACCEL | synth.SAVE_MAX | synth.SAVE_ARRIVAL
    c.series = {2: synth.csv_series([0, 0.1, 1.0], [0, 400, 0])}
    c.src_idx = np.array([(30 + 2) * c.h_nx + (20 + 2)], np.int32)
    cases.append(("front", c, 150, (1, 50, 150), None, None))
    # D: gridded rain (hold) on part of a dry domain + interpolated surge strip
    d = synth.small_case(64, 56, seed=13, rain_mmhr=0.0)
    d.flags = synth.RAIN_GRID | synth.SURGE_GRID | synth.TILE_ACCEL
    d.series = {}
    rain = np.zeros_like(d.n)
    rain[2 + 30:2 + 50, 2 + 36:2 + 60] = 60.0 / 3.6e6
    s0 = np.full_like(d.n, -9999.0)
    s1 = np.full_like(d.n, -9999.0)
    s0[2:-2, 2:5] = 0.2
    s1[2:-2, 2:5] = 0.6
    maps = {"rain": (1, rain, None, 0.0), "surge": (2, s0, s1, 0.35)}
    cases.append(("gridrain_surge", d, 60, (1, 30, 60), maps, None))
    # E: Euler integration with max/arrival maps
    e = synth.small_case(40, 36, seed=21)
    e.flags |= synth.EULER | synth.SAVE_MAX | synth.SAVE_ARRIVAL
    cases.append(("euler", e, 40, (1, 40), None, None))
    # F: tile acceleration off
    f = synth.small_case(40, 36, seed=22)
    f.flags &= ~synth.TILE_ACCEL
    cases.append(("noaccel", f, 20, (1, 20), None, None))
    return cases


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--work", default="/tmp/rift_golden_work")
    args = ap.parse_args()
    os.makedirs(args.out, exist_ok=True)
    if os.path.exists(args.work):
        shutil.rmtree(args.work)

    # 1. limiter probe on the GPU
    a, b, c = probe_table()
    pd = os.path.join(args.work, "probe")
    os.makedirs(pd, exist_ok=True)
    for nm, v in (("a", a), ("b", b), ("c", c)):
        v.astype(np.float64).tofile(os.path.join(pd, f"probe_{nm}.bin"))
    kap = synth.kappa_for(10.0, 10.0)
    with open(os.path.join(pd, "params.txt"), "w") as f:
        f.write(f"mode probe\nn {len(a)}\nkappa {kap!r}\n")
    po = os.path.join(args.work, "probe_out")
    print(run_ref(pd, po).strip())
    res = {k: np.fromfile(os.path.join(po, f"probe_{k}.bin"), dtype=np.float64)
           for k in ("signf", "minmod", "limiter", "velocity")}
    np.savez_compressed(os.path.join(args.out, "probe.npz"), a=a, b=b, c=c, kappa=kap, **res)

    # 2. reference runs
    for name, case, nsteps, dumps, maps, rates in golden_cases():
        cd = os.path.join(args.work, name)
        od = os.path.join(args.work, name + "_out")
        refcase.write_case(case, cd, nsteps, dump=dumps, maps=maps, rates=rates)
        print(name, run_ref(cd, od).strip())
        fx = case_inputs(case)
        fx["nsteps"] = nsteps
        fx["dumps"] = np.array(dumps)
        for k, (mode, t0, t1, factor) in (maps or {}).items():
            fx[f"map_{k}_mode"] = mode
            fx[f"map_{k}_t0"] = t0
            if t1 is not None:
                fx[f"map_{k}_t1"] = t1
            fx[f"map_{k}_factor"] = factor
        nBX = -(-case.h_nx // 16)
        nBY = -(-case.h_ny // 14)
        log = np.loadtxt(os.path.join(od, "steps.txt"), ndmin=2)
        fx["steps_log"] = log
        names = ("w", "hu", "hv", "F", "hmax", "qmax", "twet")
        for s in dumps:
            r = refcase.read_dump(od, s, case.h_nx, case.h_ny, nBX * nBY, names=names)
            for k, v in r.items():
                fx[f"s{s}_{k}"] = v
        np.savez_compressed(os.path.join(args.out, f"{name}.npz"), **fx)
    print("golden ok")


if __name__ == "__main__":
    main()
