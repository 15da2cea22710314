"""Write a workload in the format oracle/refkit/refrun.cu reads, and read back
its dumps.  Test infrastructure: used by make_golden.py (run on a GB300 machine)
and by the parity tests."""
from __future__ import annotations

import os

import numpy as np


def write_case(case, d, nsteps, dump=(), timing=False, maps=None, rates=None, src_rate=None,
               map_times=None, extra=None):
    """case: rift_gb300.synth.Case.  maps: {name: (mode, t0, t1, factor)} with
    name in rain/drain/surge and mode 1 = hold, 2 = interpolate.
    rates: (rain_mps, drain_mps) fixed uniform rates when no series is set.
    map_times: {name: (t0, t1)}: the interpolation factor of that map follows
    the simulated time, (t - t0) / (t1 - t0).  extra: further refrun
    parameters (t_stop, dump_final, timed_steps, dump_bc)."""
    os.makedirs(d, exist_ok=True)
    BX, BY = case.faces()
    BX.astype(np.float64).tofile(os.path.join(d, "BX.bin"))
    BY.astype(np.float64).tofile(os.path.join(d, "BY.bin"))
    case.n.astype(np.float64).tofile(os.path.join(d, "n.bin"))
    if case.K is not None:
        case.K.astype(np.float64).tofile(os.path.join(d, "K.bin"))
    if case.h0 is not None:
        case.h0.astype(np.float64).tofile(os.path.join(d, "h0.bin"))
    p = dict(nx=case.h_nx, ny=case.h_ny, flags=case.flags, dx=repr(case.cell), dy=repr(case.cell),
             kappa=repr(case.kappa), nodata="-9999", courant=repr(case.courant), psi=repr(case.psi),
             dtheta=repr(case.dtheta), t0=repr(case.t0), nsteps=nsteps, timing=int(timing))
    if dump:
        p["dump"] = ",".join(str(s) for s in dump)
    for which, (t, r) in case.series.items():
        p[f"series{which}"] = len(t)
        np.asarray(t, np.float32).tofile(os.path.join(d, f"series{which}_t.bin"))
        np.asarray(r, np.float32).tofile(os.path.join(d, f"series{which}_r.bin"))
    if case.src_idx is not None:
        p["nsrc"] = len(case.src_idx)
        np.asarray(case.src_idx, np.int32).tofile(os.path.join(d, "src_idx.bin"))
        if src_rate is not None:
            np.asarray(src_rate, np.float64).tofile(os.path.join(d, "src_rate.bin"))
    if rates is not None:
        p["rain_rate"] = repr(float(rates[0]))
        p["drain_rate"] = repr(float(rates[1]))
    for name, (mode, t0, t1, factor) in (maps or {}).items():
        p[f"map_{name}"] = mode
        p[f"factor_{name}"] = repr(float(factor))
        np.asarray(t0, np.float64).tofile(os.path.join(d, f"{name}_t0.bin"))
        if t1 is not None:
            np.asarray(t1, np.float64).tofile(os.path.join(d, f"{name}_t1.bin"))
    for name, (a, b) in (map_times or {}).items():
        p[f"map_times_{name}"] = f"{float(a)!r} {float(b)!r}"
    for k, v in (extra or {}).items():
        p[k] = repr(float(v)) if isinstance(v, float) else v
    with open(os.path.join(d, "params.txt"), "w") as f:
        for k, v in p.items():
            f.write(f"{k} {v}\n")


def write_state(d, snap):
    """A hotstart-like state (reference representation) for refrun."""
    for k in ("w", "hu", "hv", "F"):
        if k in snap and snap[k] is not None:
            np.asarray(snap[k], np.float64).tofile(os.path.join(d, f"state_{k}.bin"))
    np.asarray(snap["wet"], np.uint8).tofile(os.path.join(d, "state_wet.bin"))
    np.asarray(snap["active"], np.int32).tofile(os.path.join(d, "state_active.bin"))
    np.asarray(snap["mx"], np.float64).tofile(os.path.join(d, "state_mx.bin"))
    np.asarray(snap["my"], np.float64).tofile(os.path.join(d, "state_my.bin"))
    with open(os.path.join(d, "params.txt"), "a") as f:
        f.write(f"state 1\nstate_nactive {len(snap['active'])}\n")
        f.write(f"t0 {float(snap['t'])!r}\ndt0 {float(snap['dt'])!r}\n")


def read_dump(out, step, nx, ny, grid_size, names=("w", "hu", "hv")):
    pre = os.path.join(out, f"s{step:05d}_")
    r = {}
    for nm in names:
        fn = pre + nm + ".bin"
        if os.path.exists(fn):
            r[nm] = np.fromfile(fn, dtype=np.float64).reshape(ny, nx)
    r["wet"] = np.fromfile(pre + "wet.bin", dtype=np.uint8)
    r["active"] = np.fromfile(pre + "active.bin", dtype=np.int32)
    r["mx"] = np.fromfile(pre + "mx.bin", dtype=np.float64)
    r["my"] = np.fromfile(pre + "my.bin", dtype=np.float64)
    t = np.fromfile(pre + "t.bin", dtype=np.float64)
    r["t"], r["dt"] = float(t[0]), float(t[1])
    return r


def run(case, nsteps, dump=(), maps=None, map_times=None, extra=None, state=None, workdir=None):
    """Run the reference's own kernels (oracle/refkit/refrun with the prebuilt
    fatbin) on `case`; returns (the runner's JSON record, {step: dump},
    steps.txt rows).  `state`: a snapshot (reference representation) to start
    from.  Raises RuntimeError when the runner or the fatbin is missing."""
    import json
    import shutil
    import subprocess
    import tempfile

    from oracle import build as ob
    fat = ob.fatbin_path()
    if not os.path.exists(fat):
        raise RuntimeError("reference fatbin missing")
    exe = ob.build_refrun()
    if exe is None:
        raise RuntimeError("no nvcc to build the runner")
    d = tempfile.mkdtemp(prefix="rift_ref_", dir=workdir)
    try:
        write_case(case, d, nsteps, dump=dump, maps=maps, map_times=map_times, extra=extra)
        if state is not None:
            write_state(d, state)
        out = os.path.join(d, "out")
        os.makedirs(out)
        r = subprocess.run([exe, fat, d, out], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"refrun rc={r.returncode}: {r.stderr[-500:]}")
        rec = json.loads(r.stdout.strip().splitlines()[-1])
        nbx, nby = -(-case.h_nx // 16), -(-case.h_ny // 14)
        steps = sorted(set(dump) | ({rec["steps"]} if (extra or {}).get("dump_final") else set()))
        dumps = {s: read_dump(out, s, case.h_nx, case.h_ny, nbx * nby,
                              names=("w", "hu", "hv", "F", "hmax", "twet")) for s in steps}
        log = np.loadtxt(os.path.join(out, "steps.txt"), ndmin=2)
        return rec, dumps, log
    finally:
        shutil.rmtree(d, ignore_errors=True)
