"""ctypes binding of the C ABI declared in include/rift_gb300.h.

`Sim` drives any library that exports that ABI under a symbol prefix (the
CUDA engine exports it as "rift_*").  A library whose create call takes an
extra int32 mode argument is bound with `create_has_mode=True`.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "librift_gb300.so")

RIFT_OK = 0
ERRORS = {1: "bad argument", 2: "CUDA error", 3: "call out of order", 4: "numeric fault",
          5: "out of device memory", 6: "unsupported"}

FIELD = dict(W=0, HU=1, HV=2, F=3, H=4, Q=5, HMAX=6, QMAX=7, TPEAK=8, TDRY=9, TWET=10, BC=11)
MAP = dict(RAIN=0, DRAIN=1, SURGE=2)


class GridDesc(C.Structure):
    _fields_ = [("h_nx", C.c_int32), ("h_ny", C.c_int32), ("dx", C.c_double), ("dy", C.c_double),
                ("kappa", C.c_double), ("nodata", C.c_double), ("courant", C.c_double),
                ("psi", C.c_double), ("dtheta", C.c_double), ("flags", C.c_uint32),
                ("device", C.c_int32)]


class DeviceView(C.Structure):
    """rift_device_view: device pointers of a handle's state (include/rift_gb300.h)."""
    _fields_ = [("h", C.c_void_p), ("hu", C.c_void_p), ("hv", C.c_void_p), ("e", C.c_void_p),
                ("n", C.c_void_p), ("t", C.c_void_p), ("dt", C.c_void_p), ("stream", C.c_void_p),
                ("h_nx", C.c_int32), ("h_ny", C.c_int32), ("pitch", C.c_int32), ("rows", C.c_int32),
                ("dx", C.c_double), ("dy", C.c_double), ("kappa", C.c_double)]


class Ledger(C.Structure):
    """rift_ledger (include/rift_gb300.h)."""
    _fields_ = [(n, C.c_double) for n in ("volume", "soil", "volume0", "soil0", "added", "drained",
                                          "infiltrated", "clamped", "surge", "boundary")]


class RiftError(RuntimeError):
    pass


_P = C.c_void_p
_D = C.POINTER(C.c_double)
_F = C.POINTER(C.c_float)
_I = C.POINTER(C.c_int32)
_U8 = C.POINTER(C.c_uint8)


def _sig(lib, name, res, args):
    f = getattr(lib, name)
    f.restype = res
    f.argtypes = args
    return f


def exported_symbols():
    """Entry points of include/rift_gb300.h (without the prefix)."""
    return ["create", "upload_static", "init", "set_uniform_rates", "set_point_sources",
            "set_map", "set_map_factor", "set_map_times", "step", "run", "set_series", "get_field", "get_tiles",
            "get_tile_speeds", "set_state", "get_time", "volume", "mass_ledger", "get_tile_grid",
            "last_error", "destroy"]


def bind(lib, prefix: str, create_has_mode: bool = False):
    """Attach argtypes/restype for every ABI entry point; returns a namespace."""
    p = prefix
    ns = {}
    if create_has_mode:
        ns["create"] = _sig(lib, p + "create", C.c_int, [C.POINTER(GridDesc), C.c_int32, C.POINTER(_P)])
    else:
        ns["create"] = _sig(lib, p + "create", C.c_int, [C.POINTER(GridDesc), C.POINTER(_P)])
    ns["upload_static"] = _sig(lib, p + "upload_static", C.c_int, [_P, _D, _D, _D, _D, _D])
    ns["init"] = _sig(lib, p + "init", C.c_int, [_P, C.c_double])
    ns["set_uniform_rates"] = _sig(lib, p + "set_uniform_rates", C.c_int, [_P, C.c_double, C.c_double])
    ns["set_point_sources"] = _sig(lib, p + "set_point_sources", C.c_int, [_P, _I, _D, C.c_int32])
    ns["set_map"] = _sig(lib, p + "set_map", C.c_int, [_P, C.c_int32, _D, _D, C.c_double])
    ns["set_map_factor"] = _sig(lib, p + "set_map_factor", C.c_int, [_P, C.c_int32, C.c_double])
    ns["set_map_times"] = _sig(lib, p + "set_map_times", C.c_int,
                               [_P, C.c_int32, C.c_double, C.c_double])
    if hasattr(lib, p + "mass_ledger_terms"):
        ns["mass_ledger_terms"] = _sig(lib, p + "mass_ledger_terms", C.c_int, [_P, C.POINTER(Ledger)])
    if hasattr(lib, p + "set_point_rates"):
        ns["set_point_rates"] = _sig(lib, p + "set_point_rates", C.c_int, [_P, _D, C.c_int32])
    if hasattr(lib, p + "set_march_rows"):
        ns["set_march_rows"] = _sig(lib, p + "set_march_rows", C.c_int, [_P, C.c_int32])
        ns["get_march_rows"] = _sig(lib, p + "get_march_rows", C.c_int, [_P, _I])
    if hasattr(lib, p + "set_schedule"):
        ns["set_schedule"] = _sig(lib, p + "set_schedule", C.c_int, [_P, C.c_int32])
    if hasattr(lib, p + "ensemble_create"):
        ns["ensemble_create"] = _sig(lib, p + "ensemble_create", C.c_int,
                                     [C.POINTER(_P), C.c_int32, C.POINTER(_P)])
        ns["ensemble_run"] = _sig(lib, p + "ensemble_run", C.c_int,
                                  [_P, C.c_double, C.c_int32, _D, C.POINTER(C.c_int32)])
        ns["ensemble_last_error"] = _sig(lib, p + "ensemble_last_error", C.c_char_p, [_P])
        ns["ensemble_destroy"] = _sig(lib, p + "ensemble_destroy", None, [_P])
        if hasattr(lib, p + "ensemble_member_times"):
            ns["ensemble_member_times"] = _sig(lib, p + "ensemble_member_times", C.c_int, [_P, _D])
        if hasattr(lib, p + "ensemble_set_solo_cells"):
            ns["ensemble_set_solo_cells"] = _sig(lib, p + "ensemble_set_solo_cells", C.c_int,
                                                 [_P, C.c_int64])
        if hasattr(lib, p + "ensemble_launch_count"):
            ns["ensemble_launch_count"] = _sig(lib, p + "ensemble_launch_count", C.c_int,
                                               [_P, C.POINTER(C.c_int64)])
    if hasattr(lib, p + "autotune"):
        ns["autotune"] = _sig(lib, p + "autotune", C.c_int, [_P, C.c_int32, _I, _D])
    if hasattr(lib, p + "set_persistent"):
        ns["set_persistent"] = _sig(lib, p + "set_persistent", C.c_int, [_P, C.c_int32])
        ns["get_path_stats"] = _sig(lib, p + "get_path_stats", C.c_int,
                                    [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int64)])
        ns["get_table_steps"] = _sig(lib, p + "get_table_steps", C.c_int,
                                     [_P, C.POINTER(C.c_int64)])
    if hasattr(lib, p + "get_launch_count"):
        ns["get_launch_count"] = _sig(lib, p + "get_launch_count", C.c_int, [_P, C.POINTER(C.c_int64)])
    if hasattr(lib, p + "set_host_access"):
        ns["set_host_access"] = _sig(lib, p + "set_host_access", C.c_int, [_P, C.c_int32])
        ns["get_host_access"] = _sig(lib, p + "get_host_access", C.c_int, [_P, C.POINTER(C.c_int32)])
    if hasattr(lib, p + "get_device_view"):
        ns["get_device_view"] = _sig(lib, p + "get_device_view", C.c_int, [_P, C.POINTER(DeviceView)])
    ns["set_series"] = _sig(lib, p + "set_series", C.c_int, [_P, C.c_int32, _F, _F, C.c_int32])
    ns["step"] = _sig(lib, p + "step", C.c_int, [_P, _D, _D])
    ns["run"] = _sig(lib, p + "run", C.c_int, [_P, C.c_int32, C.c_double, _D, _D, _I])
    ns["get_field"] = _sig(lib, p + "get_field", C.c_int, [_P, C.c_int32, _D, C.c_size_t])
    ns["get_tiles"] = _sig(lib, p + "get_tiles", C.c_int, [_P, _U8, _I, _I])
    ns["get_tile_speeds"] = _sig(lib, p + "get_tile_speeds", C.c_int, [_P, _D, _D])
    ns["set_state"] = _sig(lib, p + "set_state", C.c_int,
                           [_P, C.c_double, C.c_double, _D, _D, _D, _D, _U8, _I, C.c_int32, _D, _D])
    ns["get_time"] = _sig(lib, p + "get_time", C.c_int, [_P, _D, _D])
    ns["volume"] = _sig(lib, p + "volume", C.c_int, [_P, _D])
    ns["mass_ledger"] = _sig(lib, p + "mass_ledger", C.c_int, [_P, _D, _D])
    ns["get_tile_grid"] = _sig(lib, p + "get_tile_grid", C.c_int, [_P, _I, _I])
    ns["last_error"] = _sig(lib, p + "last_error", C.c_char_p, [_P])
    ns["destroy"] = _sig(lib, p + "destroy", None, [_P])
    return ns


def _dp(a):
    if a is None:
        return None
    return a.ctypes.data_as(_D)


_product = None


def load_product():
    """Load the in-tree CUDA library.  Fails loudly when it is missing: there
    is no CPU fallback on the product path."""
    global _product
    if _product is None:
        if not os.path.exists(LIB_PATH):
            raise RiftError(f"CUDA extension not built: {LIB_PATH} missing (run build())")
        lib = C.CDLL(LIB_PATH)
        _product = (lib, bind(lib, "rift_"))
    return _product


class Sim:
    """One simulation handle behind the C ABI."""

    def __init__(self, case, api=None, create_mode=None, device=0):
        if api is None:
            api = load_product()
        self.lib, self.f = api
        self.case = case
        self.nx, self.ny = case.h_nx, case.h_ny
        d = GridDesc(case.h_nx, case.h_ny, case.cell, case.cell, case.kappa, -9999.0,
                     case.courant, case.psi, case.dtheta, case.flags, device)
        self._desc = d
        h = _P()
        if create_mode is None:
            rc = self.f["create"](C.byref(d), C.byref(h))
        else:
            rc = self.f["create"](C.byref(d), create_mode, C.byref(h))
        self._check(rc, "create", h)
        self.h = h
        nbx, nby = C.c_int32(), C.c_int32()
        self._check(self.f["get_tile_grid"](h, C.byref(nbx), C.byref(nby)), "get_tile_grid")
        self.nBX, self.nBY = nbx.value, nby.value
        self.grid_size = self.nBX * self.nBY

    def _check(self, rc, what, h=None):
        if rc != RIFT_OK:
            msg = ""
            hh = h if h is not None else getattr(self, "h", None)
            if hh:
                m = self.f["last_error"](hh)
                msg = m.decode() if m else ""
            raise RiftError(f"{what} failed: {ERRORS.get(rc, rc)} {msg}")

    def close(self):
        if getattr(self, "h", None):
            self.f["destroy"](self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- setup ------------------------------------------------------------
    def upload(self):
        c = self.case
        BX, BY = c.faces()
        BX = np.ascontiguousarray(BX, dtype=np.float64)
        BY = np.ascontiguousarray(BY, dtype=np.float64)
        n = np.ascontiguousarray(c.n, dtype=np.float64)
        K = None if c.K is None else np.ascontiguousarray(c.K, dtype=np.float64)
        h0 = None if c.h0 is None else np.ascontiguousarray(c.h0, dtype=np.float64)
        self._keep = (BX, BY, n, K, h0)
        self._check(self.f["upload_static"](self.h, _dp(BX), _dp(BY), _dp(n), _dp(K), _dp(h0)),
                    "upload_static")
        for which, (t, r) in c.series.items():
            self.set_series(which, t, r)
        if c.src_idx is not None:
            idx = np.ascontiguousarray(c.src_idx, dtype=np.int32)
            rate = np.zeros(len(idx))
            self.set_point_sources(idx, rate)
        if c.rain_maps is not None:
            m0, m1 = c.rain_maps
            self.set_map(0, m0, m1, 0.0)
            if c.map_times is not None:
                self.set_map_times(0, *c.map_times)
        return self

    def init(self, t0=None):
        self._check(self.f["init"](self.h, self.case.t0 if t0 is None else t0), "init")
        return self

    def setup(self):
        return self.upload().init()

    def set_series(self, which, times, rates):
        t = np.ascontiguousarray(times, dtype=np.float32)
        r = np.ascontiguousarray(rates, dtype=np.float32)
        self._check(self.f["set_series"](self.h, which, t.ctypes.data_as(_F), r.ctypes.data_as(_F),
                                         len(t)), "set_series")

    def set_uniform_rates(self, rain, drain):
        self._check(self.f["set_uniform_rates"](self.h, rain, drain), "set_uniform_rates")

    def set_point_sources(self, idx, rate):
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        rate = np.ascontiguousarray(rate, dtype=np.float64)
        self._check(self.f["set_point_sources"](self.h, idx.ctypes.data_as(_I), _dp(rate), len(idx)),
                    "set_point_sources")

    def set_map(self, which, t0, t1=None, factor=0.0):
        a0 = np.ascontiguousarray(t0, dtype=np.float64)
        a1 = None if t1 is None else np.ascontiguousarray(t1, dtype=np.float64)
        self._check(self.f["set_map"](self.h, which, _dp(a0), _dp(a1), factor), "set_map")

    def set_map_factor(self, which, factor):
        self._check(self.f["set_map_factor"](self.h, which, factor), "set_map_factor")

    def set_map_times(self, which, t0, t1):
        self._check(self.f["set_map_times"](self.h, which, t0, t1), "set_map_times")

    def set_schedule(self, march_min_strips):
        """Kernel schedule: march kernels from this many active strips up
        (-1 default, 0 always march, a huge value always per-tile)."""
        if "set_schedule" in self.f:
            self._check(self.f["set_schedule"](self.h, march_min_strips), "set_schedule")
        return self

    def set_march_rows(self, tile_rows):
        """Column march work items of 1, 2 or 4 tile rows."""
        if "set_march_rows" in self.f:
            self._check(self.f["set_march_rows"](self.h, tile_rows), "set_march_rows")
        return self

    def march_rows(self):
        r = C.c_int32()
        self._check(self.f["get_march_rows"](self.h, C.byref(r)), "get_march_rows")
        return r.value

    def set_persistent(self, max_active_tiles):
        """Persistent cooperative step loop while at most this many tiles are
        active (-1 default, 0 off)."""
        if "set_persistent" in self.f:
            self._check(self.f["set_persistent"](self.h, max_active_tiles), "set_persistent")
        return self

    AUTOTUNE_CANDIDATES = ("persistent", "graph+tiles", "graph+march 2 rows", "graph+march 1 row",
                           "graph+march 4 rows")

    def autotune(self, probe_steps=10):
        """Time each kernel schedule and march work-item height from the
        current state, restore the state, keep the fastest; returns (choice,
        ms per step of each candidate, AUTOTUNE_CANDIDATES order)."""
        choice = C.c_int32()
        ms = np.zeros(len(self.AUTOTUNE_CANDIDATES))
        self._check(self.f["autotune"](self.h, probe_steps, C.byref(choice), _dp(ms)), "autotune")
        return choice.value, ms

    def launch_count(self):
        """Kernels launched by rift_run / rift_step so far (rift_get_launch_count)."""
        n = C.c_int64()
        self._check(self.f["get_launch_count"](self.h, C.byref(n)), "get_launch_count")
        return int(n.value)

    def path_stats(self):
        """(steps run by the persistent launch, steps run by the per-step graph)."""
        a, b = C.c_int64(), C.c_int64()
        self._check(self.f["get_path_stats"](self.h, C.byref(a), C.byref(b)), "get_path_stats")
        return a.value, b.value

    def table_steps(self):
        """Persistent steps run from the loop's tile table (no grow phase)."""
        a = C.c_int64()
        self._check(self.f["get_table_steps"](self.h, C.byref(a)), "get_table_steps")
        return a.value

    # -- stepping ---------------------------------------------------------
    def step(self):
        t, dt = C.c_double(), C.c_double()
        self._check(self.f["step"](self.h, C.byref(t), C.byref(dt)), "step")
        return t.value, dt.value

    def run(self, nsteps, t_stop=float("inf")):
        t, dt, k = C.c_double(), C.c_double(), C.c_int32()
        self._check(self.f["run"](self.h, nsteps, t_stop, C.byref(t), C.byref(dt), C.byref(k)), "run")
        return t.value, dt.value, k.value

    # -- readback ---------------------------------------------------------
    def field(self, name):
        out = np.zeros((self.ny, self.nx))
        self._check(self.f["get_field"](self.h, FIELD[name], _dp(out), self.nx), f"get_field {name}")
        return out

    def tiles(self):
        wet = np.zeros(self.grid_size, dtype=np.uint8)
        act = np.zeros(self.grid_size, dtype=np.int32)
        n = C.c_int32()
        self._check(self.f["get_tiles"](self.h, wet.ctypes.data_as(_U8), act.ctypes.data_as(_I),
                                        C.byref(n)), "get_tiles")
        return wet, act[: n.value].copy()

    def tile_speeds(self):
        mx = np.zeros(self.grid_size)
        my = np.zeros(self.grid_size)
        self._check(self.f["get_tile_speeds"](self.h, _dp(mx), _dp(my)), "get_tile_speeds")
        return mx, my

    def host_access(self):
        """True when state uploads and field reads run as device kernels on
        the caller's host arrays (pageable memory through the host page tables)."""
        v = C.c_int32()
        self._check(self.f["get_host_access"](self.h, C.byref(v)), "get_host_access")
        return bool(v.value)

    def set_host_access(self, on):
        self._check(self.f["set_host_access"](self.h, 1 if on else 0), "set_host_access")
        return self

    def device_view(self):
        """Device pointers of U^n, the face offsets and n (DeviceView)."""
        v = DeviceView()
        self._check(self.f["get_device_view"](self.h, C.byref(v)), "get_device_view")
        return v

    def time(self):
        t, dt = C.c_double(), C.c_double()
        self._check(self.f["get_time"](self.h, C.byref(t), C.byref(dt)), "get_time")
        return t.value, dt.value

    def volume(self):
        v = C.c_double()
        self._check(self.f["volume"](self.h, C.byref(v)), "volume")
        return v.value

    def mass_ledger(self):
        """(volume, volume added by the sources since init), FP64."""
        v, a = C.c_double(), C.c_double()
        self._check(self.f["mass_ledger"](self.h, C.byref(v), C.byref(a)), "mass_ledger")
        return v.value, a.value

    def ledger(self):
        """The full volume ledger (rift_mass_ledger_terms) as a dict, with
        `residual` = (volume - volume0) - (added - drained - infiltrated -
        clamped + surge + boundary)."""
        L = Ledger()
        self._check(self.f["mass_ledger_terms"](self.h, C.byref(L)), "mass_ledger_terms")
        d = {n: getattr(L, n) for n, _ in Ledger._fields_}
        d["residual"] = (d["volume"] - d["volume0"]) - (d["added"] - d["drained"] - d["infiltrated"]
                                                        - d["clamped"] + d["surge"] + d["boundary"])
        return d

    def set_state(self, t, dt_prev, w, hu, hv, F=None, wet=None, active=None, mx=None, my=None):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) if a is not None else None
                for a in (w, hu, hv, F, mx, my)]
        w_, hu_, hv_, F_, mx_, my_ = arrs
        wet_ = None if wet is None else np.ascontiguousarray(wet, dtype=np.uint8)
        act_ = None if active is None else np.ascontiguousarray(active, dtype=np.int32)
        self._check(self.f["set_state"](
            self.h, t, dt_prev, _dp(w_), _dp(hu_), _dp(hv_), _dp(F_),
            None if wet_ is None else wet_.ctypes.data_as(_U8),
            None if act_ is None else act_.ctypes.data_as(_I),
            -1 if act_ is None else len(act_), _dp(mx_), _dp(my_)), "set_state")

    def snapshot(self):
        """Everything needed to restart the step bit-for-bit."""
        t, dt = self.time()
        wet, act = self.tiles()
        mx, my = self.tile_speeds()
        snap = dict(t=t, dt=dt, w=self.field("W"), hu=self.field("HU"), hv=self.field("HV"),
                    wet=wet, active=act, mx=mx, my=my)
        if self.case.flags & 16:
            snap["F"] = self.field("F")
        return snap

    def load_snapshot(self, s):
        self.set_state(s["t"], s["dt"], s["w"], s["hu"], s["hv"], s.get("F"), s["wet"],
                       s["active"], s["mx"], s["my"])


class Ensemble:
    """Members (Sim objects of one engine library) stepped together by one
    persistent kernel; each keeps its own dt and results."""

    def __init__(self, sims):
        self.sims = list(sims)
        self.f = self.sims[0].f
        arr = (_P * len(self.sims))(*[s.h for s in self.sims])
        self.h = _P()
        rc = self.f["ensemble_create"](arr, len(self.sims), C.byref(self.h))
        if rc != RIFT_OK:
            msg = self.f["ensemble_last_error"](self.h) if self.h else b""
            raise RiftError(f"ensemble_create failed: {ERRORS.get(rc, rc)} "
                            f"{(msg or b'').decode()}")

    def run(self, t_stop=float("inf"), max_steps=2**31 - 1):
        n = len(self.sims)
        t = np.zeros(n)
        k = np.zeros(n, dtype=np.int32)
        rc = self.f["ensemble_run"](self.h, t_stop, max_steps, _dp(t),
                                    k.ctypes.data_as(C.POINTER(C.c_int32)))
        if rc != RIFT_OK:
            raise RiftError(f"ensemble_run failed: {ERRORS.get(rc, rc)} "
                            f"{self.f['ensemble_last_error'](self.h).decode()}")
        return t, k

    def set_solo_cells(self, min_cells):
        """Members with at least min_cells interior cells run on their own
        per-step graphs after the ensemble kernel (0: none)."""
        rc = self.f["ensemble_set_solo_cells"](self.h, int(min_cells))
        if rc != RIFT_OK:
            raise RiftError(f"ensemble_set_solo_cells failed: {ERRORS.get(rc, rc)}")
        return self

    def launch_count(self):
        """Kernels launched by rift_ensemble_run so far (rift_ensemble_launch_count)."""
        n = C.c_int64()
        rc = self.f["ensemble_launch_count"](self.h, C.byref(n))
        if rc != RIFT_OK:
            raise RiftError(f"ensemble_launch_count failed: {ERRORS.get(rc, rc)}")
        return int(n.value)

    def member_times(self):
        """Device seconds from the last run's start to each member's end."""
        out = np.zeros(len(self.sims))
        rc = self.f["ensemble_member_times"](self.h, _dp(out))
        if rc != RIFT_OK:
            raise RiftError(f"ensemble_member_times failed: {ERRORS.get(rc, rc)}")
        return out

    def close(self):
        if getattr(self, "h", None):
            self.f["ensemble_destroy"](self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
