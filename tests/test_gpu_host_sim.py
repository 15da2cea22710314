"""The host drop-in layer end to end on the GPU: a config file with ESRI and
CSV inputs runs through rift_sim_* (ReadUserParams, InitSimulation,
RunSimulation, PrintData, WriteHotstart, ReadHotstart, CloseSimulation) and
its printed maps are checked against the FP64 oracle stepped over the same
inputs, the oracle fed by a restatement of the reference's rules for each
input (corner means, CSV series, Coord2Index, GridSeries map timing)."""
import ctypes as C
import math
import os

import numpy as np
import pytest

from rift_gb300 import build as eb
from rift_gb300 import capi, synth

pytestmark = pytest.mark.gpu

MAX_DH = 1e-4
CELL = 10.0
NODATA = -9999.0


def _esri(path, corners, xll=500.0, yll=700.0, cell=CELL, nodata=NODATA):
    ny, nx = corners.shape
    with open(path, "w") as f:
        f.write(f"ncols {nx}\nnrows {ny}\nxllcorner {xll}\nyllcorner {yll}\n"
                f"cellsize {cell}\nNODATA_value {nodata}\n")
        for j in range(ny - 1, -1, -1):
            f.write(" ".join("%.17g" % v for v in corners[j]) + "\n")


def _read_map(path):
    lines = open(path).read().splitlines()
    return np.array([[float(v) for v in ln.split()] for ln in lines[6:]])[::-1]


def _corner_mean(C4):
    """InitSimulation's 0.25 * (ur + lr + ll + ul) per interior cell."""
    out = np.zeros((C4.shape[0] + 3, C4.shape[1] + 3))
    ll, ul, ur, lr = C4[:-1, :-1], C4[1:, :-1], C4[1:, 1:], C4[:-1, 1:]
    out[2:-2, 2:-2] = 0.25 * (((ur + lr) + ll) + ul)
    return out


def _map_mean(C4, scale, allow_nodata):
    """GridSeries::p_interp: mean of the non-nodata corners where >= 3."""
    fill = NODATA if allow_nodata else 0.0
    out = np.full((C4.shape[0] + 3, C4.shape[1] + 3), fill)
    for j in range(2, out.shape[0] - 2):
        for i in range(2, out.shape[1] - 2):
            jt, it = j - 2, i - 2
            vals = [C4[jt + nj, it + ni] for ni in (0, 1) for nj in (0, 1)]
            good = [v for v in vals if v != NODATA]
            if len(good) > 2:
                s = 0.0
                for v in good:
                    s += v
                out[j, i] = (s / len(good)) * scale
    return out


class _Hold:
    """HyetographGridSeries timing (map k on [(k-1)dt, k dt), zeros after tf)."""

    def __init__(self, maps, dt, tmax, scale):
        self.maps, self.dt, self.tmax, self.scale = maps, float(int(dt)), tmax, scale
        self.tin, self.done, self.cur = -9999.0, False, None

    def update(self, t):
        changed = False
        if self.tin < 0:
            self.tin = t
            if self.tin < self.tmax:
                self.cur, changed = self.maps[int(math.trunc(self.tin / self.dt))], True
        if t >= self.tmax:
            if not self.done:
                self.cur, changed = np.zeros_like(self.maps[0]), True
            self.done = True
        elif t >= self.tin:
            self.tin += self.dt
            self.cur, changed = self.maps[int(math.trunc(self.tin / self.dt))], True
        return changed


class _Interp:
    """InterpolatedGridSeries timing (maps trunc(t/dt) and +1, last held)."""

    def __init__(self, maps, dt, tmax):
        self.maps, self.dt, self.tmax = maps, float(int(dt)), tmax
        self.tin, self.tnext, self.done = -9999.0, 0.0, False

    def update(self, t):
        if self.tin < 0:
            k = int(math.trunc(t / self.dt))
            self.m0, self.m1 = self.maps[k], self.maps[k + 1]
            self.tin, self.tnext = k * self.dt, k * self.dt + self.dt
            return True
        if t >= self.tmax:
            if not self.done:
                self.tin, self.tnext, self.m0 = self.tnext, self.tnext + self.dt, self.m1
                self.done = True
                return True
            return False
        if t >= self.tnext:
            self.m0, self.tin, self.tnext = self.m1, self.tnext, self.tnext + self.dt
            self.m1 = self.maps[int(math.trunc(self.tnext / self.dt))]
            return True
        return False


@pytest.fixture(scope="module")
def host():
    lib = C.CDLL(eb.build_host())
    lib.rift_host_last_error.restype = C.c_char_p
    lib.rift_sim_last_error.restype = C.c_char_p
    lib.rift_sim_engine.restype = C.c_void_p
    return lib


_NX, _NY = 48, 40


def _scene(tmp, nx=_NX, ny=_NY, seed=5):
    rng = np.random.default_rng(seed)
    xs = np.arange(nx + 1) * CELL
    ys = np.arange(ny + 1) * CELL
    X, Y = np.meshgrid(xs, ys)
    z = 30.0 - 0.004 * X + 0.002 * Y + synth.gaussian_bumps(X, Y, rng, 5, (0.5, 2), (30, 90),
                                                           nx * CELL)
    z[:2, :] += 40.0
    z[-2:, :] += 40.0
    z[:, :2] += 40.0
    z[:, -2:] += 40.0
    _esri(os.path.join(tmp, "dem.asc"), z)
    K = np.exp(np.log(8.0) + 0.5 * rng.standard_normal(z.shape))
    _esri(os.path.join(tmp, "K.asc"), K)
    with open(os.path.join(tmp, "rain.csv"), "w") as f:
        f.write("# hours, mm/hr\n0, 60\n0.02, 60\n0.02, 0\n0.04, 0\n")
    with open(os.path.join(tmp, "hydro.csv"), "w") as f:
        f.write("0, 0\n0.01, 40\n0.03, 0\n")
    return z, K


def _config(tmp, extra):
    base = {"DEM": "dem.asc", "t0": "0", "tf": "150", "projected": "1", "n": "0.035",
            "output": "out", "dt_print": "30", "h_print": "1"}
    base.update(extra)
    os.makedirs(os.path.join(tmp, base["output"]), exist_ok=True)
    path = os.path.join(tmp, "sim.cfg")
    with open(path, "w") as f:
        f.write("; drop-in test\n" + "".join(f"{k} = {v}\n" for k, v in base.items()))
    return path


def _oracle_case(z, flags, n_const=0.035, K=None, psi=0.0, dtheta=0.0, series=None, src=None):
    n = np.zeros((z.shape[0] + 3, z.shape[1] + 3))
    n[2:-2, 2:-2] = n_const
    case = synth.Case(name="dropin", B=z, cell=CELL, n=n, flags=flags, psi=psi, dtheta=dtheta,
                      tf=150.0)
    if K is not None:
        case.K = _corner_mean(K) / (3600.0 * 1000.0)
    case.series = series or {}
    if src is not None:
        case.src_idx = np.array(src, dtype=np.int32)
    return case


def _run_sim(host, cfg, cwd):
    """Open, run to tf, read the final surface through the engine handle,
    close.  Returns (t, steps, W)."""
    old = os.getcwd()
    os.chdir(cwd)
    try:
        sim = C.c_void_p()
        rc = host.rift_sim_open(cfg.encode(), C.byref(sim))
        assert rc == 0, host.rift_host_last_error()
        t, steps = C.c_double(), C.c_int64()
        rc = host.rift_sim_run(sim, C.c_double(1e30), C.byref(t), C.byref(steps))
        assert rc == 0, host.rift_sim_last_error(sim)
        eng = C.CDLL(eb.build())
        h = C.c_void_p(host.rift_sim_engine(sim))
        nbx, nby = C.c_int32(), C.c_int32()
        assert eng.rift_get_tile_grid(h, C.byref(nbx), C.byref(nby)) == 0
        W = np.zeros((_NY + 4, _NX + 4))
        assert eng.rift_get_field(h, 0, W.ctypes.data_as(C.POINTER(C.c_double)),
                                  C.c_size_t(_NX + 4)) == 0
        assert host.rift_sim_close(sim) == 0
        return t.value, steps.value, W
    finally:
        os.chdir(old)


def _oracle_prints(oracle_api, case, tf, dt_print, series_hooks=()):
    """Step the oracle like RunSimulation: outputs at the first step with
    t > t_print; returns the depth maps at those steps."""
    lib, _ = oracle_api
    lib.rift_oracle_set_threads(os.cpu_count() or 1)
    sim = capi.Sim(case, api=oracle_api, create_mode=0).upload()
    for hook in series_hooks:
        hook(sim, 0.0)
    sim.init()
    prints, t, t_print, steps = [], 0.0, 0.0, 0
    while t < tf:
        t, _ = sim.step()
        steps += 1
        for hook in series_hooks:
            hook(sim, t)
        if t > t_print:
            prints.append(sim.field("H"))
            t_print += dt_print
    return prints, t, steps


def _compare(tmp, prints, out="out"):
    for k, ref in enumerate(prints):
        got = _read_map(os.path.join(tmp, out, f"h{k}.txt"))
        dh = np.abs(got - ref[2:-2, 2:-2]).max()
        assert dh <= MAX_DH, f"h{k}.txt differs from the oracle by {dh:.3e} m"
    assert not os.path.exists(os.path.join(tmp, out, f"h{len(prints)}.txt"))


def test_dropin_rain_source_infiltration(host, oracle_api, tmp_path):
    tmp = str(tmp_path)
    z, K = _scene(tmp)
    # the hydrograph enters at the cell Coord2Index gives for this point:
    # 2 cells west / south of it (h_xll is the centre of h-cell 2)
    X, Y = 500.0 + 5.0 + 20 * CELL, 700.0 + 5.0 + 18 * CELL
    cfg = _config(tmp, {"hyetograph": "rain.csv", "hydrograph": "hydro.csv",
                        "source_pt": f"({X}, {Y})", "K": "K.asc", "psi": "0.11",
                        "dtheta": "0.3", "save_max": "1", "save_arrival": "1",
                        "check_volume": "1", "save_hotstart": "1", "q_print": "1",
                        "ws_print": "1", "b_print": "1", "n_print": "1"})
    t_end, steps, _ = _run_sim(host, cfg, tmp)
    h_nx = z.shape[1] + 3
    i, j = int((X - (500.0 + 5.0)) / CELL + 0.5), int((Y - (700.0 + 5.0)) / CELL + 0.5)
    flags = (synth.RAIN_UNIFORM | synth.POINT_SOURCE | synth.INFILTRATION | synth.TILE_ACCEL |
             synth.SAVE_MAX | synth.SAVE_ARRIVAL)
    series = {0: synth.csv_series([0, 0.02, 0.02, 0.04], [60, 60, 0, 0]),
              2: synth.csv_series([0, 0.01, 0.03], [0, 40, 0])}
    case = _oracle_case(z, flags, K=K, psi=0.11, dtheta=0.3, series=series, src=[j * h_nx + i])
    prints, t_o, steps_o = _oracle_prints(oracle_api, case, 150.0, 30.0)
    assert steps == steps_o and abs(t_end - t_o) <= 1e-5 * t_o
    _compare(tmp, prints)
    out = os.path.join(tmp, "out")
    for name in ("peak_flood_depth.txt", "peak_unit_flow.txt", "time_to_peak.txt",
                 "time_to_dry.txt", "flood_wave_arrival.txt", "bc.txt", "n.txt", "ws0.txt",
                 "q0.txt", "hot0.bin", f"hot{len(prints) - 1}.bin"):
        assert os.path.exists(os.path.join(out, name)), name
    n_map = _read_map(os.path.join(out, "n.txt"))
    assert np.all(n_map == 0.035)


def test_dropin_hotstart_restart(host, tmp_path):
    """A run restarted from hot<k>.bin ends where the continuous run ends."""
    tmp = str(tmp_path)
    _scene(tmp)
    cfg = _config(tmp, {"hyetograph": "rain.csv", "save_hotstart": "1", "output": "full"})
    t_full, _, W_full = _run_sim(host, cfg, tmp)
    hot = os.path.join(tmp, "full", "hot2.bin")
    assert os.path.exists(hot)
    t_hot = np.frombuffer(open(hot, "rb").read(8), "<f8")[0]
    assert 60.0 < t_hot < 90.0
    os.remove(cfg)
    cfg = _config(tmp, {"hyetograph": "rain.csv", "read_hotstart": hot, "output": "restart",
                        "t0": repr(float(t_hot))})
    t_re, _, W_re = _run_sim(host, cfg, tmp)
    assert t_re == t_full
    assert np.abs(W_full - W_re)[2:-2, 2:-2].max() <= 1e-6


@pytest.mark.parametrize("interp", [0, 1])
def test_dropin_gridded_rain_maps(host, oracle_api, tmp_path, interp):
    """hyetograph_prefix maps (held, or interpolated in time) and a drain
    CSV: the printed depths follow the oracle fed with the same map timing."""
    tmp = str(tmp_path)
    z, _ = _scene(tmp)
    rng = np.random.default_rng(11)
    corner_maps = []
    for k in range(8):
        m = np.clip(40.0 + 30.0 * rng.standard_normal(z.shape), 0.0, None) * (k % 3 != 2)
        corner_maps.append(m)
        _esri(os.path.join(tmp, f"rain-{k:03d}.txt"), m)
    with open(os.path.join(tmp, "drain.csv"), "w") as f:
        f.write("0, 5\n1, 5\n")
    cfg = _config(tmp, {"hyetograph_prefix": "rain", "hyetograph_dt": "40.7",
                        "hyetograph_tf": "120", "hyetograph_interp": str(interp),
                        "drain": "drain.csv"})
    _run_sim(host, cfg, tmp)
    scale = 1.0 / 3600.0 / 1000.0
    maps = [_map_mean(m, scale, False) for m in corner_maps]
    series = _Interp(maps, 40.7, 120.0) if interp else _Hold(maps, 40.7, 120.0, scale)

    def hook(sim, t):
        if series.update(t):
            if interp:
                sim.set_map(0, series.m0, series.m1, 0.0)
                sim.set_map_times(0, series.tin, series.tnext)
            else:
                sim.set_map(0, series.cur)

    flags = synth.RAIN_GRID | synth.DRAIN_UNIFORM | synth.TILE_ACCEL
    case = _oracle_case(z, flags, series={1: synth.csv_series([0, 1], [5, 5])})
    prints, _, _ = _oracle_prints(oracle_api, case, 150.0, 30.0, [hook])
    _compare(tmp, prints)


def test_coupling_hooks_drive_the_source(host, oracle_api, tmp_path):
    """The 1D-2D coupling calls (OpenSimulation with a flow rate,
    setSourceValue, updateSources): a configuration that places a source
    without a hydrograph, its discharge set by the caller before every step.
    The run matches the oracle stepped with the same per-cell rates, and the
    V_added bookkeeping is the reference's: rate x the dt current at the
    call, per source cell."""
    tmp = str(tmp_path)
    z, _ = _scene(tmp)
    X0, Y0 = 500.0 + 5.0 + 20 * CELL, 700.0 + 5.0 + 18 * CELL
    X1, Y1 = X0 + CELL, Y0 + CELL  # a 2 x 2 rectangle of source cells
    cfg = _config(tmp, {"source_rect_X": f"({X0}, {X1})", "source_rect_Y": f"({Y0}, {Y1})",
                        "check_volume": "1", "h_print": "0", "tf": "120"})

    def q_of(t):  # the coupled model's discharge, m^3/s
        return 6.0 * np.sin(np.pi * min(t, 100.0) / 100.0) ** 2

    old = os.getcwd()
    os.chdir(tmp)
    try:
        sim = C.c_void_p()
        rc = host.rift_sim_open_flow(cfg.encode(), C.c_double(2.5), C.byref(sim))
        assert rc == 0, host.rift_host_last_error()
        fr, ns = C.c_double(), C.c_int32()
        assert host.rift_sim_flow_rate(sim, C.byref(fr)) == 0 and fr.value == 2.5
        assert host.rift_sim_num_sources(sim, C.byref(ns)) == 0 and ns.value == 4
        t, dt, tf = C.c_double(), C.c_double(), C.c_double()
        rates, v_ref = [], 0.0
        while True:
            assert host.rift_sim_time(sim, C.byref(t), C.byref(dt), C.byref(tf)) == 0
            if t.value >= tf.value:
                break
            q = q_of(t.value)
            assert host.rift_sim_set_source_value(sim, C.c_double(q)) == 0
            assert host.rift_sim_update_sources(sim) == 0
            r = q / CELL / CELL / 4
            v_ref += 4 * (r * dt.value)
            rates.append(r)
            assert host.rift_sim_step(sim, C.byref(t)) == 0, host.rift_sim_last_error(sim)
        va = C.c_double()
        assert host.rift_sim_source_volume(sim, C.byref(va)) == 0
        assert abs(va.value - v_ref) <= 1e-12 * v_ref
        eng = C.CDLL(eb.build())
        h = C.c_void_p(host.rift_sim_engine(sim))
        W = np.zeros((_NY + 4, _NX + 4))
        assert eng.rift_get_field(h, 0, W.ctypes.data_as(C.POINTER(C.c_double)),
                                  C.c_size_t(_NX + 4)) == 0
        assert host.rift_sim_close(sim) == 0
    finally:
        os.chdir(old)
    h_nx = z.shape[1] + 3
    i0 = int((X0 - (500.0 + 5.0)) / CELL + 0.5)
    j0 = int((Y0 - (700.0 + 5.0)) / CELL + 0.5)
    src = [j * h_nx + i for i in (i0, i0 + 1) for j in (j0, j0 + 1)]
    case = _oracle_case(z, synth.POINT_SOURCE | synth.TILE_ACCEL, src=src)
    lib, _ = oracle_api
    lib.rift_oracle_set_threads(os.cpu_count() or 1)
    orc = capi.Sim(case, api=oracle_api, create_mode=0).setup()
    for r in rates:
        orc.set_point_sources(src, [r] * 4)
        orc.step()
    Wo = orc.field("W")
    dh = np.abs(W - Wo)[2:-2, 2:-2].max()
    assert dh <= MAX_DH, dh
    assert (Wo - orc.field("BC"))[2:-2, 2:-2].max() > 0.05  # the source filled cells
