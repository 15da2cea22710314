"""Benchmark of the GB300 RIFT step (one JSON line on stdout).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--config 1|2|3|4|5]
                    [--impl ours|reference]

A step is one full RK2 time step (both stages, Grow, dt) of the whole domain
with only active tiles computed, as the reference does.  Workloads are the
seeded synthetic configs of rift_gb300.synth (no datasets are involved):
  1: 512^2 bumpy plane, uniform rain           (the reference's small case)
  2: 2048^2 fractal + channel, point-source hydrograph, Green-Ampt (default)
  3: 8192^2 urban fractal with buildings, uniform drain, interpolated rain maps
  4: the learned flux closure: training patches from fine runs of seeded
     1024^2 scenarios, Adam on the tensor-core kernels, then held-out
     scenarios run fine (N^2 at 2 m) and coarse ((N/2)^2 at 4 m, plain and
     with the closure); metric the fine/closure wall-time ratio, with the
     peak-depth RMSE and arrival-time error against the fine run
  5: a batched ensemble (--members, --side-min/--side-max, --tf) run to tf in
     one persistent kernel; metric members/hour, per-member p50/p99, and the
     same members run one after another for comparison
The state is spun up (untimed) to --spinup seconds of simulated time so the
timed steps see a developed flood, then W warm-up and K timed steps run.

value  = domain cell-updates/s = interior cells x K / device time (CUDA
         events on the engine's stream around the K steps: one persistent
         launch, or K step-graph launches);
e2e    = the same metric through the C ABI with host buffers: the state
         uploaded from host arrays, one rift_run call over the K steps (as a
         caller of RunSimulation makes it), the depth map read back, all
         inside the timed region; e2e.per_step_calls repeats it with one
         rift_step call per step (t and dt returned to the host each step);
roofline: HBM bytes per active cell-update (algorithmic, FP32 words of the
         reference data model) x active cell-updates / device time, against
         the measured copy bandwidth.
--impl reference times the FP64 CPU restatement of the reference step on all
host cores over a bounded sample of the same state (the reference has no CPU
path of its own; its CUDA build, run through oracle/refkit, is reported
beside it when the prebuilt fatbin is present).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from rift_gb300 import capi, synth  # noqa: E402

# algorithmic FP32 words per active cell-update (both stages):
# plain core 23 words; Green-Ampt +7; interpolated map +4; gridded hold +2
WORDS = {1: 23, 2: 23 + 7, 3: 23 + 4}


def make_case(cfg, N=None):
    if cfg == 1:
        return synth.config1(N=N or 512)
    if cfg == 2:
        return synth.config2(N=N or 2048)
    if cfg == 3:
        return synth.config3(N=N or 8192)
    raise ValueError(cfg)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def bf16_peak():
    """Dense BF16 burst rate (TFLOP/s) of MEASURED_PEAKS.json, else the fallback."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return {"bf16_tflops": float(json.load(f)["bf16_tflops"]), "kind": "measured"}
    except Exception:
        return {"bf16_tflops": 1900.0, "kind": "fallback"}


class ClockSampler:
    """SM clock and clock-event reasons sampled during the timed region:
    NVML through ctypes every millisecond (a timed region of a few ms still
    gets samples), else nvidia-smi every 100 ms.  Reads only."""

    # nvmlClocksEventReason* bits (nvml.h)
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self):
        self.samples = []  # (sm_mhz, reason bits)
        self.sm_max = None
        self._stop = threading.Event()
        self._thread = None
        self._proc = None

    def _nvml(self):
        nv = ctypes.CDLL("libnvidia-ml.so.1")
        if nv.nvmlInit_v2() != 0:
            raise OSError("nvmlInit")
        idx = os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]
        dev = ctypes.c_void_p()
        if not idx.isdigit() or nv.nvmlDeviceGetHandleByIndex_v2(int(idx), ctypes.byref(dev)) != 0:
            if nv.nvmlDeviceGetHandleByIndex_v2(0, ctypes.byref(dev)) != 0:
                raise OSError("nvmlDeviceGetHandleByIndex")
        mx = ctypes.c_uint()
        if nv.nvmlDeviceGetMaxClockInfo(dev, 1, ctypes.byref(mx)) == 0:  # NVML_CLOCK_SM
            self.sm_max = float(mx.value)
        reasons = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            nv.nvmlDeviceGetCurrentClocksThrottleReasons
        return nv, dev, reasons

    def start(self):
        try:
            nv, dev, reasons = self._nvml()

            def loop():
                clk, bits = ctypes.c_uint(), ctypes.c_ulonglong()
                while not self._stop.is_set():
                    if nv.nvmlDeviceGetClockInfo(dev, 1, ctypes.byref(clk)) == 0 and \
                            reasons(dev, ctypes.byref(bits)) == 0:
                        self.samples.append((float(clk.value), int(bits.value)))
                    time.sleep(0.001)

            self._thread = threading.Thread(target=loop, daemon=True)
            self._thread.start()
        except Exception:
            self._start_smi()
        return self

    def _start_smi(self):
        q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self._proc = subprocess.Popen(
                ["nvidia-smi", "-i", "0", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read_smi, daemon=True).start()
        except Exception:
            self._proc = None

    def _read_smi(self):
        bits = (0x8, 0x40, 0x20, 0x4)
        for line in self._proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 6 and parts[0].replace(".", "").isdigit():
                if parts[1].replace(".", "").isdigit():
                    self.sm_max = float(parts[1])
                b = sum(bit for bit, v in zip(bits, parts[2:6]) if v.lower() == "active")
                self.samples.append((float(parts[0]), b))

    def stop(self):
        self._stop.set()
        if self._thread:
            self._thread.join(timeout=2)
        if self._proc:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=2)
            except Exception:
                pass
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": self.sm_max, "reasons": ["unsampled"]}
        reasons = sorted({name for _, b in self.samples for bit, name in self.REASONS.items()
                          if b & bit})
        return {"sm_mhz": float(np.median([c for c, _ in self.samples])),
                "sm_max_mhz": self.sm_max, "reasons": reasons, "samples": len(self.samples)}


def spin_up(sim, t_target, chunk=2000):
    t = sim.time()[0]
    while t < t_target:
        t, _, done = sim.run(chunk, t_target)
        if done == 0:
            break
    return t


def device_timed_run(sim, steps):
    """K graph launches bracketed by CUDA events on the engine stream."""
    lib = sim.lib
    D = ctypes.POINTER(ctypes.c_double)
    lib.rift_bench_run.restype = ctypes.c_int
    lib.rift_bench_run.argtypes = [ctypes.c_void_p, ctypes.c_int32, D, D, D, D, D]
    out = [ctypes.c_double() for _ in range(5)]
    rc = lib.rift_bench_run(sim.h, steps, *[ctypes.byref(o) for o in out])
    if rc != 0:
        raise RuntimeError(f"rift_bench_run rc={rc}")
    ms, act_total, done, stage_ms, stage_act = (o.value for o in out)
    return ms, act_total, done, stage_ms, stage_act


def run_ours(args, device=0, sync=None):
    """One replica's bench line.  `sync` (multi-rank runs) is called on both
    sides of the device-timed region: a barrier over the ranks plus a device
    synchronize."""
    cfg = args.config
    case = make_case(cfg, args.N)
    interior = (case.h_nx - 4) * (case.h_ny - 4)
    spin = args.spinup if args.spinup is not None else {1: 600.0, 2: 3600.0, 3: 120.0}[cfg]

    # ---- e2e through the C ABI with host buffers ----------------------------
    t0 = time.perf_counter()
    sim = capi.Sim(case, device=device).set_schedule(args.schedule).set_persistent(args.persistent)
    sim.set_march_rows(args.march_rows)
    sim.setup()
    t_setup = time.perf_counter() - t0
    spin_up(sim, spin)
    snap = sim.snapshot()
    for _ in range(args.warmup):
        sim.step()
    e2e_steps = args.steps
    h2d = sum(snap[k].nbytes for k in ("w", "hu", "hv", "wet", "active", "mx", "my"))
    if "F" in snap:
        h2d += snap["F"].nbytes
    # one rift_run call over the steps, as a caller of RunSimulation makes it
    t0 = time.perf_counter()
    sim.load_snapshot(snap)  # host arrays -> device (state upload)
    sim.run(e2e_steps)
    depth = sim.field("H")
    t_e2e = time.perf_counter() - t0
    e2e_value = interior * e2e_steps / t_e2e
    d2h = depth.nbytes + 24
    # one rift_step call per step (state mirror synchronised after each)
    call_steps = min(args.steps, 200)
    t0 = time.perf_counter()
    sim.load_snapshot(snap)
    for _ in range(call_steps):
        sim.step()
    sim.field("H")
    t_calls = time.perf_counter() - t0
    e2e_calls = {"value": interior * call_steps / t_calls, "steps": call_steps,
                 "us_per_call": 1e6 * t_calls / call_steps}

    # ---- device-timed run (inputs resident) --------------------------------
    sim.load_snapshot(snap)
    tuned = None
    if args.autotune > 0:
        choice, ms = sim.autotune(args.autotune)
        tuned = {"choice": capi.Sim.AUTOTUNE_CANDIDATES[choice],
                 "ms_per_step": {n: (None if np.isnan(x) else float(x))
                                 for n, x in zip(capi.Sim.AUTOTUNE_CANDIDATES, ms)}}
    for _ in range(args.warmup):
        sim.step()
    clocks = ClockSampler().start()
    if sync:
        sync()
    p0, g0 = sim.path_stats()
    ms, active_cells, done, stage_ms, stage_cells = device_timed_run(sim, args.steps)
    p1, g1 = sim.path_stats()
    if sync:
        sync()
    clk = clocks.stop()
    persist_steps, graph_steps = p1 - p0, g1 - g0
    steps = int(done)
    value = interior * steps / (ms * 1e-3)
    active_rate = active_cells / (ms * 1e-3)
    peak, peak_kind = peaks()
    bytes_per = 4 * WORDS[cfg]
    if persist_steps > 0 and graph_steps == 0:
        # one cooperative launch ran every timed step: the kernel is the step
        kernel = ("k_persist (whole step in one cooperative launch: grow, speeds + dt, "
                  "RK stages 1+2)")
        achieved = active_cells * bytes_per / (ms * 1e-3) / 1e9
        launches = 1
    else:
        kernel = ("RK stages 1+2 (k_march<1>, k_update1, k_march<2> or k_stage<1>, k_stage<2>; one "
                  "schedule runs, the other exits at entry)")
        achieved = stage_cells * bytes_per / (stage_ms * 1e-3) / 1e9 if stage_ms > 0 else None
        launches = graph_steps * launches_per_step(case.flags) + (1 if persist_steps else 0)
    # DRAM bytes (read + write) of the reported kernel per launch, from the
    # ncu capture summarised under profiles/ (per step there)
    traffic = None
    prof = os.path.join(ROOT, "profiles", f"traffic_config{cfg}.json")
    if os.path.exists(prof) and args.N is None:
        try:
            rec = json.load(open(prof))
            if rec.get("kernel") == ("k_persist" if launches == 1 else "stages"):
                traffic = rec["bytes_per_step"] * (steps if launches == 1 else 1)
        except Exception:
            traffic = None
    line = {
        "metric": "cell-updates/s",
        "value": value,
        "unit": "cell-updates/s",
        "n_gpus": args.gpus,
        "steps": steps,
        "warmup": args.warmup,
        "ms_per_step": ms / max(steps, 1),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": case.name, "cells": interior, "spinup_s": spin,
                   "active_cell_updates_per_s": active_rate,
                   "active_fraction": active_cells / max(steps, 1) / interior,
                   "l2": "inputs larger than L2 (state + statics > 129 MB)" if interior > 2e6
                   else "inputs smaller than L2; steps are back to back",
                   "parallelism": "replicas only"},
        "e2e": {"value": e2e_value, "unit": "cell-updates/s", "h2d_bytes_per_step": h2d / e2e_steps,
                "d2h_bytes_per_step": d2h / e2e_steps, "setup_s": t_setup,
                "per_step_calls": e2e_calls},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                     "peak_kind": peak_kind, "bytes_per_active_cell_update": bytes_per,
                     "kernel": kernel},
        "clocks": clk,
        "gpu_launches": launches,
        "path": {"persistent_steps": persist_steps, "graph_steps": graph_steps,
                 "autotune": tuned, "march_rows": sim.march_rows()},
    }
    if args.cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(case, snap, args)
    sim.close()
    return line


def launches_per_step(flags):
    """Kernels one step's graph launches: k_track (gridded rain or surge),
    k_grow, the speed/dt kernel and the stage kernels of both schedules (the
    schedule not chosen for the step exits at entry), k_commit in Euler
    mode."""
    n = 1 + 2 + 2 + (1 if flags & synth.EULER else 2)
    if flags & (synth.RAIN_GRID | synth.SURGE_GRID):
        n += 1
    return n


def combine_replicas(line, world, allreduce_max):
    """Whole-job line of a replicas-only run from this rank's line.  Every rank
    ran the same workload on its own GPU: the job's time is the slowest rank's
    (max over ranks) and the value counts the cell updates of all ranks.
    `allreduce_max` maps a list of floats to their element-wise max over ranks."""
    ms_max, inv_e2e = allreduce_max([line["ms_per_step"], 1.0 / line["e2e"]["value"]])
    out = dict(line)
    cells = line["config"]["cells"]
    out["ms_per_step"] = ms_max
    out["value"] = world * cells / (ms_max * 1e-3)
    out["e2e"] = dict(line["e2e"], value=world / inv_e2e)
    out["n_gpus"] = world
    out["gpu_launches"] = line["gpu_launches"] * world
    return out


def cpu_baseline(case, snap, args, seconds=15.0):
    """The FP64 oracle (REF mode) on all host cores, stepped for `seconds`
    from the spun-up state `snap` (reference representation)."""
    from oracle import build as ob
    lib = ctypes.CDLL(ob.build_oracle())
    threads = lib.rift_oracle_set_threads(os.cpu_count() or 1)
    api = (lib, capi.bind(lib, "rift_oracle_", create_has_mode=True))
    sim = capi.Sim(case, api=api, create_mode=0).setup()
    sim.load_snapshot(snap)
    interior = (case.h_nx - 4) * (case.h_ny - 4)
    steps = 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        sim.step()
        steps += 1
    el = time.perf_counter() - t0
    return {"value": interior * steps / el, "unit": "cell-updates/s", "cores": int(threads),
            "kind": "port",
            "sample": f"{steps} steps of {case.name} from the spun-up state ({el:.1f} s)"}


def reference_kernels_run(case, spin, timed_steps):
    """The reference's own CUDA kernels (grid.cu compiled for sm_103a, driven
    in RunSimulation order by oracle/refkit/refrun) on the workload: spun up
    from t0 to `spin` seconds, the state dumped, then `timed_steps` more steps
    timed.  Returns (timing record, spun-up state in the reference
    representation).  No code of this repository's engine runs here."""
    import shutil
    import tempfile

    from oracle import build as ob
    fat = ob.fatbin_path()
    if not os.path.exists(fat):
        raise RuntimeError("reference fatbin oracle/_ref/rift_ref_sm103a.fatbin is absent")
    run = ob.build_refrun()
    if run is None:
        raise RuntimeError("no nvcc to build the reference-kernel runner")
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import refcase
    d = tempfile.mkdtemp(prefix="rift_refbench_")
    try:
        maps = mt = None
        if case.rain_maps is not None:
            maps = {"rain": (2, case.rain_maps[0], case.rain_maps[1], 0.0)}
            if case.map_times is not None:
                mt = {"rain": case.map_times}
        refcase.write_case(case, d, 2 ** 31 - 1, maps=maps, map_times=mt,
                           extra={"t_stop": float(spin), "dump_final": 1,
                                  "timed_steps": int(timed_steps), "dump_bc": 0})
        out = os.path.join(d, "out")
        os.makedirs(out)
        r = subprocess.run([run, fat, d, out], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"refrun rc={r.returncode}: {r.stderr.strip()[-300:]}")
        rec = json.loads(r.stdout.strip().splitlines()[-1])
        nBX, nBY = -(-case.h_nx // 16), -(-case.h_ny // 14)
        snap = refcase.read_dump(out, rec["spinup_steps"], case.h_nx, case.h_ny, nBX * nBY,
                                 names=("w", "hu", "hv", "F"))
        if "F" not in snap:
            snap["F"] = None
        return rec, snap
    finally:
        shutil.rmtree(d, ignore_errors=True)


def run_reference(args):
    """The reference arm.  The reference has no CPU implementation of the
    step, so `value` is the FP64 CPU restatement of it (oracle, REF mode) on
    all host cores; the reference's own CUDA kernels on this GPU are reported
    beside it (`reference_cuda_gb300`).  The spun-up state both time from is
    made by the reference's own kernels, not by this repository's engine."""
    case = make_case(args.config, args.N)
    spin = args.spinup if args.spinup is not None else {1: 600.0, 2: 3600.0, 3: 120.0}[args.config]
    interior = (case.h_nx - 4) * (case.h_ny - 4)
    try:
        # the reference kernels' own rate over at most 200 steps (a side figure:
        # 0.31 s per step on config 3), so the arm ends within a few minutes
        rec, snap = reference_kernels_run(case, spin, min(max(args.steps, 20), 200))
    except Exception as e:  # the reference kernels cannot run here
        return {"impl": "reference", "unavailable": f"reference kernels: {e}"[:300]}
    cb = cpu_baseline(case, snap, args, seconds=args.ref_seconds)
    line = {"metric": "cell-updates/s", "value": cb["value"], "unit": "cell-updates/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": case.name, "cells": interior, "spinup_s": spin,
                       "spinup": "reference kernels (oracle/refkit) from t0"},
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "cell-updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "reference_cuda_gb300": rec}
    return line


def run_ensemble(args):
    """Config 5: a batched ensemble run to tf in one persistent kernel
    (rift_ensemble_run), timed on the host around the synchronous call, then
    the same members run one after another for comparison."""
    cases = synth.config5(members=args.members, side=(args.side_min, args.side_max), tf=args.tf)
    model = None
    if args.closure:
        # members coarsened 2x (10 m cells) with the learned closure, trained
        # on scenarios at the members' fine resolution (5 m -> 10 m)
        from rift_gb300 import closure
        ds = closure.generate(list(range(args.closure_seeds)), N=args.closure_train_N, cell=5.0,
                              log=lambda m: print(m, file=sys.stderr, flush=True))
        model, _ = closure.train(ds, steps=args.train_steps, batch=256)
        del ds
        cases = [closure.coarse_case(closure.even_side(c)) for c in cases]

    def setup():
        return [capi.Sim(c).setup() for c in cases]

    if model is not None:
        args.sequential = False  # the one-after-another comparison runs members without it
    members = setup()
    ens = capi.Ensemble(members)
    ens.set_solo_cells(args.solo_cells)
    ens.run(max_steps=args.warmup)  # warm-up steps (counted in t, not timed)
    runner = None
    if model is not None:
        runner = closure.EnsembleClosure(ens, members, model, every=args.closure_every,
                                         gain=args.closure_gain)
    clocks = ClockSampler().start()
    l0 = ens.launch_count()
    t0 = time.perf_counter()
    if runner is None:
        t_end, k = ens.run(t_stop=args.tf)
    else:
        t_end, k = runner.run(args.tf)
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    # ensemble kernels plus the kernels of the members run on their own
    launches = ens.launch_count() - l0
    cells = np.array([(c.h_nx - 4) * (c.h_ny - 4) for c in cases], dtype=float)
    iters = int(k.max())
    # each member's completion time, measured: the device clock at the end of
    # its last step (one kernel), or the host clock at the end of the chunk in
    # which it reached tf (with the closure between chunks)
    if runner is None:
        per_member = ens.member_times()
        completion = "device globaltimer at each member's last step (from the kernel start)"
    else:
        per_member = runner.finish_wall
        completion = "host clock at the end of the chunk in which each member reached tf"
    ens.close()
    for s in members:
        s.close()
    seq = 0.0
    if args.sequential:
        solo = setup()
        for s in solo:
            s.run(args.warmup)
        for s in solo:
            ts = time.perf_counter()
            s.run(2 ** 31 - 1, args.tf)
            seq += time.perf_counter() - ts
            s.close()
    line = {"metric": "members/hour", "value": len(cases) / wall * 3600.0, "unit": "members/hour",
            "n_gpus": 1, "steps": iters, "warmup": args.warmup, "ms_per_step": wall / iters * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "config5", "members": len(cases),
                       "side_cells": [args.side_min, args.side_max], "tf_s": args.tf,
                       "total_cells": int(cells.sum()), "iterations": iters,
                       "solo_cells": args.solo_cells,
                       "solo_members": int(np.sum(cells >= args.solo_cells)) if args.solo_cells else 0,
                       "member_steps_min_max": [int(k.min()), int(k.max())]},
            "per_member_s": {"p50": float(np.percentile(per_member, 50)),
                             "p99": float(np.percentile(per_member, 99)),
                             "max": float(np.max(per_member)), "measured": completion},
            "domain_cell_updates_per_s": float((cells * k).sum() / wall),
            "clocks": clk, "gpu_launches": launches}
    if args.sequential:
        line["sequential_s"] = seq
        line["ensemble_speedup_vs_sequential"] = seq / wall
    if runner is not None:
        ev, fbk = 0, 0
        for r in runner.runs:
            a, b = r.block_counts()
            ev, fbk = ev + a, fbk + b
        line["gpu_launches"] = launches + 2 * sum(r.applies for r in runner.runs)
        line["config"]["closure"] = {"grid": "members coarsened 2x (10 m cells)",
                                     "every_steps": args.closure_every, "gain": args.closure_gain,
                                     "train_scenarios": args.closure_seeds,
                                     "blocks_evaluated": ev, "blocks_fallen_back": fbk}
    return line


def _timed_chunks(run_to, tf, every_s, depth):
    """Run to tf in chunks of every_s simulated seconds; returns the wall time
    of the runs alone and the first time each interior cell's depth exceeded
    ARRIVAL_DEPTH at a chunk end (inf where it never did)."""
    import torch
    wall, t = 0.0, 0.0
    arrival = None
    while t < tf:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        t = run_to(min(t + every_s, tf))
        torch.cuda.synchronize()
        wall += time.perf_counter() - t0
        h = depth()
        if arrival is None:
            arrival = np.full(h.shape, np.inf)
        arrival[(h > ARRIVAL_DEPTH) & np.isinf(arrival)] = t
    return wall, arrival


ARRIVAL_DEPTH = 0.05  # m: a cell has "arrived" once its depth passes 5 cm


def closure_step_rate(cc, model, args, t_spin=1800.0, reps=20):
    """Tensor-core rate of the closure step (k_closure + k_apply) on a wet
    state: the coarse case spun up to t_spin by the engine alone, then one
    untimed and `reps` timed applications, CUDA events on the engine's
    stream.  Algorithmic FLOPs: 2 x 14,144 multiply-adds per output cell of
    every evaluated 16 x 16 block."""
    import torch

    from rift_gb300 import closure

    sim = capi.Sim(cc).setup()
    sim.run(2 ** 31 - 1, min(args.tf, t_spin))
    cr = closure.ClosureRun(sim, model, every=args.closure_every, gain=args.closure_gain)
    st = torch.cuda.ExternalStream(cr.view.stream)
    t = sim.time()[0]
    cr.apply(1e-3, t)
    torch.cuda.synchronize()
    b0 = cr.block_counts()[0]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        cr.apply(1e-3, t)
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    blocks = (cr.block_counts()[0] - b0) / reps
    sim.close()
    flops = blocks * 256 * 2 * (150 * 32 + 288 * 32 + 32 * 4)
    pk = bf16_peak()
    achieved = flops / (ms * 1e-3) / 1e12
    return {"bound": "tensor", "achieved": achieved, "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
            "frac": achieved / pk["bf16_tflops"], "traffic": None, "peak_kind": pk["kind"],
            "kernel": "k_closure + k_apply (one closure step)", "ms_per_apply": ms,
            "blocks_per_apply": blocks, "coarse_cells": (cc.h_nx - 4) * (cc.h_ny - 4)}


def run_closure(args):
    """Config 4: train the closure on fine runs of --closure-seeds scenarios
    (1024^2 at 2 m), then run held-out scenarios fine (N^2 at 2 m) and
    coarse ((N/2)^2 at 4 m, plain and with the closure) to --tf."""
    import torch

    from rift_gb300 import closure

    def log(m):
        print(m, file=sys.stderr, flush=True)

    N = args.N or 4096
    if args.closure_profile:
        # the closure step alone on a wet coarse state (ncu target): untrained
        # weights, unit scales
        cc = closure.coarse_case(closure.scenario(100_001, N=N, cell=2.0, tf=args.tf))
        model = closure.Model(closure.init_params(0), np.ones(6, np.float32), np.full(4, 1e-4, np.float32))
        return {"workload": "config4 closure step", "roofline": closure_step_rate(cc, model, args)}
    t0 = time.perf_counter()
    ds = closure.generate(list(range(args.closure_seeds)), N=args.closure_train_N, cell=2.0, log=log)
    t_gen = time.perf_counter() - t0
    log(f"{len(ds.feats)} patches in {t_gen:.1f} s")
    t0 = time.perf_counter()
    model, loss = closure.train(ds, steps=args.train_steps, batch=256, log=log)
    t_train = time.perf_counter() - t0
    n_patches = len(ds.feats)
    del ds
    clocks = ClockSampler().start()
    evals = []
    for k in range(args.eval_seeds):
        seed = 100_001 + k  # scenario 100000 chose the correction gain
        fc = closure.scenario(seed, N=N, cell=2.0, tf=args.tf)
        cc = closure.coarse_case(fc)
        res = {"seed": seed, "generator": "config1" if seed % 2 == 0 else "config2"}

        def interior_depth(sim):
            return (sim.field("W") - bc_of[id(sim)])[2:-2, 2:-2]

        bc_of = {}
        fine = capi.Sim(fc).setup()
        bc_of[id(fine)] = fine.field("BC")
        w_f, arr_f = _timed_chunks(lambda t: fine.run(2 ** 31 - 1, t)[0], args.tf, 120.0,
                                   lambda: interior_depth(fine))
        hmax_f = closure.restrict(fine.field("HMAX")[2:-2, 2:-2])
        fine.close()
        n2 = arr_f.shape[0] // 2
        arr_f = arr_f.reshape(n2, 2, n2, 2).min(axis=(1, 3))
        wet = hmax_f > 0.01
        for mode in ("plain", "closure"):
            sim = capi.Sim(cc).setup()
            bc_of[id(sim)] = sim.field("BC")
            if mode == "closure":
                cr = closure.ClosureRun(sim, model, every=args.closure_every, gain=args.closure_gain,
                                        fine=fc if args.fine_fallback else None,
                                        fine_batch=args.fine_batch)
                w, arr = _timed_chunks(cr.run, args.tf, 120.0, lambda: interior_depth(sim))
                res["closure_blocks"], res["closure_fallback_blocks"] = cr.block_counts()
                res["closure_applies"] = cr.applies
                if cr.fallback is not None:
                    res["fine_resolved_blocks"] = cr.fallback.refined
                    cr.fallback.close()
            else:
                w, arr = _timed_chunks(lambda t: sim.run(2 ** 31 - 1, t)[0], args.tf, 120.0,
                                       lambda: interior_depth(sim))
            hmax = sim.field("HMAX")[2:-2, 2:-2]
            both = np.isfinite(arr) & np.isfinite(arr_f)
            res[mode] = {"wall_s": w,
                         "peak_depth_rmse_m": float(np.sqrt(np.mean((hmax - hmax_f)[wet] ** 2))),
                         "arrival_mae_s": float(np.mean(np.abs(arr[both] - arr_f[both]))) if both.any() else None,
                         "arrival_missed_frac": float(np.mean(np.isinf(arr) & np.isfinite(arr_f)))}
            sim.close()
        res["fine_wall_s"] = w_f
        res["wet_cells"] = int(wet.sum())
        res["speedup_closure"] = w_f / res["closure"]["wall_s"]
        res["speedup_plain"] = w_f / res["plain"]["wall_s"]
        evals.append(res)
        log(json.dumps(res))
    clk = clocks.stop()
    roof = closure_step_rate(cc, model, args)
    sp = float(np.mean([r["speedup_closure"] for r in evals]))
    line = {"metric": "closure vs fine-grid wall-time ratio", "value": sp, "unit": "x",
            "n_gpus": 1, "steps": None, "warmup": 0, "ms_per_step": None,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16 net / f32 solver",
            "data": "synthetic",
            "config": {"workload": "config4", "fine": f"{N}^2 at 2 m", "coarse": f"{N // 2}^2 at 4 m",
                       "tf_s": args.tf, "train_scenarios": args.closure_seeds,
                       "train_grid": f"{args.closure_train_N}^2 at 2 m", "train_patches": n_patches,
                       "train_steps": args.train_steps, "batch": 256, "closure_every_steps": args.closure_every,
                       "closure_gain": args.closure_gain,
                       "fallback_batched": args.fine_fallback and args.fine_batch,
                       "fallback": "fine-grid re-solve of the block" if args.fine_fallback
                       else "plain coarse solve of the block",
                       "eval_scenarios": args.eval_seeds},
            "peak_depth_rmse_m": {"closure": float(np.mean([r["closure"]["peak_depth_rmse_m"] for r in evals])),
                                  "plain_coarse": float(np.mean([r["plain"]["peak_depth_rmse_m"] for r in evals]))},
            "speedup_plain_coarse": float(np.mean([r["speedup_plain"] for r in evals])),
            "evals": evals,
            "training": {"generate_s": t_gen, "train_s": t_train, "loss_first": float(loss[:20].mean()),
                         "loss_last": float(loss[-20:].mean())},
            "roofline": roof,
            "clocks": clk, "gpu_launches": None}
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--config", type=int, default=3, choices=(1, 2, 3, 4, 5))
    ap.add_argument("--closure-seeds", type=int, default=32, help="config 4: training scenarios")
    ap.add_argument("--closure-train-N", type=int, default=1024, help="config 4: training grid side")
    ap.add_argument("--train-steps", type=int, default=1500, help="config 4: Adam steps")
    ap.add_argument("--eval-seeds", type=int, default=2, help="config 4: held-out scenarios")
    ap.add_argument("--closure-every", type=int, default=8,
                    help="config 4: coarse steps between closure applications")
    ap.add_argument("--closure", action="store_true",
                    help="config 5: members coarsened 2x with the learned closure")
    ap.add_argument("--closure-profile", action="store_true",
                    help="config 4: time only the closure step on a wet coarse state")
    ap.add_argument("--no-fine-fallback", dest="fine_fallback", action="store_false",
                    help="config 4: blocks that fall back keep the plain coarse solve instead of "
                         "a fine-grid re-solve")
    ap.add_argument("--no-fine-batch", dest="fine_batch", action="store_false",
                    help="config 4: re-solve fallen-back blocks one patch run after another "
                         "instead of one ensemble launch per interval")
    ap.add_argument("--closure-gain", type=float, default=0.25,
                    help="config 4: strength of the applied corrections (chosen on scenario 100000)")
    ap.add_argument("--members", type=int, default=32, help="config 5: ensemble members")
    ap.add_argument("--solo-cells", type=int, default=1 << 20,
                    help="config 5: members of at least this many cells run on their own per-step "
                         "graphs (the march) after the ensemble kernel; 0 puts all in the kernel")
    ap.add_argument("--side-min", type=int, default=128, help="config 5: smallest side (cells)")
    ap.add_argument("--side-max", type=int, default=512, help="config 5: largest side (cells)")
    ap.add_argument("--tf", type=float, default=3600.0, help="config 5: end time (s)")
    ap.add_argument("--no-sequential", dest="sequential", action="store_false",
                    help="config 5: skip the one-after-another comparison")
    ap.add_argument("--N", type=int, default=None, help="override the grid size (cells per side)")
    ap.add_argument("--impl", default="ours", choices=("ours", "reference"))
    ap.add_argument("--spinup", type=float, default=None)
    ap.add_argument("--ref-seconds", type=float, default=20.0)
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--schedule", type=int, default=-1,
                    help="march kernels from this many active strips up (-1: engine default)")
    ap.add_argument("--autotune", type=int, default=0,
                    help="before the timed region, time each schedule for this many steps "
                         "from the spun-up state and keep the fastest (0: off)")
    ap.add_argument("--march-rows", type=int, default=2, choices=(1, 2, 4),
                    help="column march work items of this many 16 x 14 tile rows")
    ap.add_argument("--persistent", type=int, default=-1,
                    help="persistent step loop while at most this many tiles are active "
                         "(-1: engine default, 0: off)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.config == 5 and args.impl != "reference":
        if rank == 0:
            print(json.dumps(run_ensemble(args)))
        return
    if args.config == 4 and args.impl != "reference":
        if rank == 0:
            print(json.dumps(run_closure(args)))
        return
    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(run_reference(args)))
        return
    if world > 1:
        # replicas only: every rank runs the same workload on its own GPU
        import torch
        import torch.distributed as dist
        local = int(os.environ.get("LOCAL_RANK", "0"))
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        args.cpu_baseline = args.cpu_baseline and rank == 0

        def sync():
            dist.barrier()
            torch.cuda.synchronize()

        def allreduce_max(vals):
            t = torch.tensor(vals, dtype=torch.float64, device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            return t.tolist()

        line = combine_replicas(run_ours(args, device=local, sync=sync), world, allreduce_max)
        if rank == 0:
            print(json.dumps(line))
        dist.destroy_process_group()
        return
    print(json.dumps(run_ours(args)))


if __name__ == "__main__":
    main()
