"""Parity of the CUDA engine with the reference's own kernels (golden
fixtures run on the GB300) and with the FP64 oracle, through the C ABI.

Bars: tile wet flags and active-tile lists bit-exact at every dumped step;
surface elevation within 1e-6 m of the reference on 99% of the cells and
within 5e-5 m everywhere (the wet/dry-correction knife edge, where the
rounding order of two codes picks the branch, also separates the reference
from its own FP64 restatement by 1.4e-5 m in the noaccel run); simulated
time within 1e-5 relative (the same knife edge moves dt by 1e-6 relative).
"""
import numpy as np
import pytest

import fixture as FX
from rift_gb300 import capi

pytestmark = pytest.mark.gpu

Q99_TOL = 1e-6
MAX_TOL = 5e-5


def _close(a, b, what):
    d = np.abs(FX.interior(a - b))
    assert np.quantile(d, 0.99) <= Q99_TOL, f"{what}: q99 {np.quantile(d, 0.99)}"
    assert d.max() <= MAX_TOL, f"{what}: max {d.max()}"


# (march threshold in strips, persistent-loop threshold in tiles, march
# work-item height in tile rows)
SCHEDULES = {"auto": (-1, -1, 2), "tiles": (1 << 30, 0, 2), "march": (0, 0, 2),
             "march1": (0, 0, 1), "march4": (0, 0, 4), "persist": (1 << 30, 1 << 30, 2)}


def _scheduled(sim, schedule):
    march, persist, rows = SCHEDULES[schedule]
    return sim.set_schedule(march).set_persistent(persist).set_march_rows(rows)


def _run_against_golden(engine_api, name, schedule="auto"):
    fx, case = FX.load(name)
    eng = FX.start(_scheduled(capi.Sim(case, api=engine_api), schedule), fx)
    step = 0
    log = fx["steps_log"]
    for s in FX.dumps(fx):
        while step < s:
            t, dt = eng.step()
            step += 1
            wet, act = eng.tiles()
            assert len(act) == int(log[step - 1][3]), f"{name}: active count at step {step}"
        ref = FX.ref_state(fx, s)
        wet, act = eng.tiles()
        assert np.array_equal(wet, ref["wet"]), f"{name}: wet tiles differ at step {s}"
        assert np.array_equal(act, ref["active"]), f"{name}: active tiles differ at step {s}"
        assert abs(t - ref["t"]) <= 1e-5 * max(1.0, abs(ref["t"])), f"{name}: t {t} vs {ref['t']}"
        _close(eng.field("W"), ref["w"], f"{name} w step {s}")
        if "F" in ref:
            _close(eng.field("F"), ref["F"], f"{name} F step {s}")
        if "hmax" in ref:
            _close(eng.field("HMAX"), ref["hmax"], f"{name} hmax step {s}")
        if "twet" in ref:
            tw = eng.field("TWET")
            assert np.array_equal(FX.interior(tw) < 0, FX.interior(ref["twet"]) < 0), name
    return eng


def test_persistent_runs_match_reference_kernels(engine_api, name_run):
    """Multi-step persistent launches (rift_run between the dumped steps: the
    loop's tile table and split barriers run) against the reference kernels."""
    name = name_run
    fx, case = FX.load(name)
    eng = FX.start(_scheduled(capi.Sim(case, api=engine_api), "persist"), fx)
    step = 0
    for s in FX.dumps(fx):
        if s > step:
            eng.run(s - step)
            step = s
        ref = FX.ref_state(fx, s)
        wet, act = eng.tiles()
        t = eng.time()[0]
        assert np.array_equal(wet, ref["wet"]), f"{name}: wet tiles differ at step {s}"
        assert np.array_equal(act, ref["active"]), f"{name}: active tiles differ at step {s}"
        assert abs(t - ref["t"]) <= 1e-5 * max(1.0, abs(ref["t"])), f"{name}: t {t} vs {ref['t']}"
        _close(eng.field("W"), ref["w"], f"{name} w step {s}")
        if "F" in ref:
            _close(eng.field("F"), ref["F"], f"{name} F step {s}")
        if "hmax" in ref:
            _close(eng.field("HMAX"), ref["hmax"], f"{name} hmax step {s}")
    persist_steps, graph_steps = eng.path_stats()
    assert graph_steps == 0 and persist_steps == step


@pytest.fixture(params=FX.CASES)
def name_run(request):
    return request.param


@pytest.mark.parametrize("schedule", ["tiles", "march", "march1", "march4", "persist"])
@pytest.mark.parametrize("name", FX.CASES)
def test_engine_matches_reference_kernels(engine_api, name, schedule):
    """Every kernel schedule (per-tile kernels, column march on work items of
    2, 1 and 4 tile rows, persistent cooperative loop) against the reference
    kernels."""
    eng = _run_against_golden(engine_api, name, schedule)
    persist_steps, graph_steps = eng.path_stats()
    if schedule == "persist":
        assert graph_steps == 0 and persist_steps > 0
    else:
        assert persist_steps == 0 and graph_steps > 0


def _scheduled_count(sim):
    """Active tiles that hold interior cells (the persistent loop's count)."""
    _, act = sim.tiles()
    bx, by = act % sim.nBX, act // sim.nBX
    return int(np.sum((bx * 16 + 2 <= sim.nx - 3) & (by * 14 + 2 <= sim.ny - 3)))


def test_persistent_hands_over_to_graph(engine_api):
    """A persistent threshold at the active count of step 2 (21 tiles) runs
    the loop until the wet front grows the set past it (24 tiles at step 5);
    the per-step graph then finishes the run, with the results of the graph
    alone."""
    fx, case = FX.load("front")
    runs = []
    for persist in (True, False):
        eng = FX.start(_scheduled(capi.Sim(case, api=engine_api), "tiles").set_persistent(0), fx)
        eng.run(2)
        if persist:
            eng.set_persistent(_scheduled_count(eng))
        eng.run(12)
        runs.append((eng.tiles(), eng.field("W"), eng.time(), eng.path_stats()))
    (w1, a1), W1, t1, st1 = runs[0]
    (w0, a0), W0, t0, st0 = runs[1]
    assert st1[0] >= 1 and st1[1] >= 3 and st1[0] + st1[1] == 14, st1
    assert np.array_equal(w1, w0) and np.array_equal(a1, a0)
    assert abs(t1[0] - t0[0]) <= 1e-6 * max(1.0, t0[0])
    _close(W1, W0, "persistent then graph vs graph")


def test_single_steps_switching_paths(engine_api):
    """rift_step calls (the one-step persistent graph) interleaved with
    changes of the persistent bound and runs match one run of the same
    length."""
    fx, case = FX.load("gridrain_surge")
    a = FX.start(_scheduled(capi.Sim(case, api=engine_api), "persist"), fx)
    for k in range(12):
        if k % 4 == 2:
            a.set_persistent(0)
        elif k % 4 == 3:
            a.set_persistent(1 << 30)
        if k % 5 == 4:
            a.run(1)
        else:
            a.step()
    b = FX.start(_scheduled(capi.Sim(case, api=engine_api), "tiles"), fx)
    b.run(12)
    assert a.path_stats()[0] > 0 and a.path_stats()[1] > 0
    assert np.array_equal(a.tiles()[0], b.tiles()[0]) and np.array_equal(a.tiles()[1], b.tiles()[1])
    assert abs(a.time()[0] - b.time()[0]) <= 1e-6 * max(1.0, b.time()[0])
    _close(a.field("W"), b.field("W"), "single steps vs run")


@pytest.mark.parametrize("schedule", ["tiles", "march", "persist"])
@pytest.mark.parametrize("name", ["rain", "front", "gridrain_surge", "h0_infil_src", "euler"])
def test_one_step_from_identical_snapshot(engine_api, oracle_api, name, schedule):
    """From the reference's own state at a dumped step, one engine step and one
    oracle step give identical tile sets and depths within tolerance."""
    fx, case = FX.load(name)
    s = FX.dumps(fx)[-2] if len(FX.dumps(fx)) > 1 else FX.dumps(fx)[0]
    ref = FX.ref_state(fx, s)
    runs = []
    for api, mode in ((engine_api, None), (oracle_api, 0)):
        sim = capi.Sim(case, api=api, create_mode=mode)
        if mode is None:
            _scheduled(sim, schedule)
        sim = FX.start(sim, fx)
        sim.set_state(ref["t"], ref["dt"], ref["w"], ref["hu"], ref["hv"], ref.get("F"),
                      ref["wet"], ref["active"], ref["mx"], ref["my"])
        sim.step()
        runs.append((sim.tiles(), sim.field("W"), sim.time()))
    (we, ae), w_e, t_e = runs[0]
    (wo, ao), w_o, t_o = runs[1]
    assert np.array_equal(we, wo)
    assert np.array_equal(ae, ao)
    assert abs(t_e[0] - t_o[0]) <= 1e-6 * max(1.0, t_o[0])
    _close(w_e, w_o, f"{name} snapshot step")


def test_autotune_restores_state(engine_api):
    """The autotuner times the schedules and march item heights from the
    current state, puts the state back exactly and keeps the fastest; the run
    then goes on as if nothing had happened."""
    fx, case = FX.load("rain")
    a = FX.start(capi.Sim(case, api=engine_api), fx)
    b = FX.start(capi.Sim(case, api=engine_api), fx)
    a.run(6)
    b.run(6)
    choice, ms = b.autotune(8)
    assert choice in range(len(capi.Sim.AUTOTUNE_CANDIDATES))
    assert np.isfinite(ms).sum() >= 4
    if choice >= 2:
        assert b.march_rows() == (2, 1, 4)[choice - 2]
    assert np.isfinite(ms[choice]) and ms[choice] == np.nanmin(ms)
    assert np.array_equal(a.field("W"), b.field("W"))
    assert a.time() == b.time()
    (wa, aa), (wb, ab) = a.tiles(), b.tiles()
    assert np.array_equal(wa, wb) and np.array_equal(aa, ab)
    a.run(12)
    b.run(12)
    (wa, aa), (wb, ab) = a.tiles(), b.tiles()
    assert np.array_equal(wa, wb) and np.array_equal(aa, ab)
    _close(b.field("W"), a.field("W"), "after autotune")


@pytest.mark.parametrize("rows", [1, 4])
def test_march_item_heights_match_on_a_dense_grid(engine_api, rows):
    """On a 1024^2 grid under uniform rain (every tile active, 74 x 37 strips
    of 7 x 2 tiles), march items of 1 and 4 tile rows give the results of the
    default 2-row items: the same tile sets, and t and the state within the
    parity bars (each height is its own instantiation, so the compiler may
    round a few operations differently: measured 1.2e-8 relative in t after
    40 steps).  The golden runs above cover partial activity on every
    height."""
    from rift_gb300 import synth
    case = synth.config1(N=1024)
    runs = []
    for r in (2, rows):
        sim = capi.Sim(case, api=engine_api).set_schedule(0).set_persistent(0).set_march_rows(r).setup()
        sim.run(40)
        runs.append((sim.tiles(), sim.time(), sim.field("W"), sim.field("HU")))
        sim.close()
    (w0, a0), t0, W0, U0 = runs[0]
    (w1, a1), t1, W1, U1 = runs[1]
    assert np.array_equal(w0, w1) and np.array_equal(a0, a1)
    assert abs(t0[0] - t1[0]) <= 1e-6 * t0[0]
    _close(W1, W0, f"{rows}-row items vs 2-row items")
    assert np.abs(U1 - U0)[2:-2, 2:-2].max() <= 1e-4


def test_launch_count_counts_the_step_graph_kernels(engine_api):
    """rift_get_launch_count: on the per-step graph (persistent loop off) each
    step replays grow, speed, march and per-tile stage-1 kernels, the update,
    and the two stage-2 kernels; gridded rain adds the map tracker."""
    from rift_gb300 import synth
    for case, per_step in ((synth.config1(N=256), 7),
                           (synth.config3(N=512, nblocks=20), 8)):
        sim = capi.Sim(case, api=engine_api).set_persistent(0).setup()
        n0 = sim.launch_count()
        sim.run(70)
        assert sim.launch_count() - n0 == 70 * per_step, case.name
        sim.close()
