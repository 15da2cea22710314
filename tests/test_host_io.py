"""Host drop-in layer, file formats (CPU): keyword=value configuration
(config.h), ESRI ASCII rasters (io.cc), GridConfig (grid_config.cpp), CSV
series (source.cc) and hot<k>.bin (simulator.cu:912-1090), each against the
reference's rules restated here."""
import ctypes as C
import math
import os

import numpy as np
import pytest

from rift_gb300 import build as eb
from rift_gb300 import synth


class GridConfig(C.Structure):
    _fields_ = [("b_nx", C.c_int32), ("b_ny", C.c_int32), ("b_xll", C.c_double),
                ("b_yll", C.c_double), ("cellsize_original", C.c_double),
                ("h_nx", C.c_int32), ("h_ny", C.c_int32), ("h_xll", C.c_double),
                ("h_yll", C.c_double), ("cellsize", C.c_double), ("h_dx", C.c_double),
                ("h_dy", C.c_double), ("square_cells", C.c_uint8), ("projected", C.c_uint8)]


@pytest.fixture(scope="module")
def host():
    lib = C.CDLL(eb.build_host())
    lib.rift_host_last_error.restype = C.c_char_p
    lib.rift_hotstart_size.restype = C.c_int64
    lib.rift_grow_grid_size.restype = C.c_int32
    return lib


def _write_esri(path, data_south_first, xll=100.0, yll=200.0, cell=10.0, nodata=-9999):
    ny, nx = data_south_first.shape
    with open(path, "w") as f:
        f.write(f"ncols {nx}\nnrows {ny}\nxllcorner {xll}\nyllcorner {yll}\n"
                f"cellsize {cell}\nNODATA_value {nodata}\n")
        for j in range(ny - 1, -1, -1):  # north row first
            f.write(" ".join(repr(float(v)) for v in data_south_first[j]) + "\n")


# ---------------------------------------------------------------- config
def test_config_rules(host, tmp_path):
    p = tmp_path / "a.cfg"
    p.write_text("; comment line\n\nDEM = dem.asc ; trailing comment\n"
                 "\tn=0.035\nK  =   -0.5\nbig = 3e-2\nflag = 1\n"
                 "source_pt = (10.5, -3)\nname with space = x\n")
    cfg = C.c_void_p()
    assert host.rift_config_open(str(p).encode(), C.byref(cfg)) == 0
    buf = C.create_string_buffer(256)
    assert host.rift_config_get(cfg, b"DEM", buf, 256) == 0 and buf.value == b"dem.asc"
    assert host.rift_config_has(cfg, b"n") == 1
    # keyIsNumber: digits and '.' only
    assert host.rift_config_is_number(cfg, b"n") == 1
    assert host.rift_config_is_number(cfg, b"K") == 0
    assert host.rift_config_is_number(cfg, b"big") == 0
    v = C.c_double()
    assert host.rift_config_get_double(cfg, b"K", C.byref(v)) == 0 and v.value == -0.5
    # the key ends at its first blank
    assert host.rift_config_has(cfg, b"name") == 1
    assert host.rift_config_has(cfg, b"missing") == 0
    assert host.rift_config_get(cfg, b"missing", buf, 256) != 0
    host.rift_config_close(cfg)


@pytest.mark.parametrize("text", ["a = 1\na = 2\n", "no separator here\n", "= 3\n", "key =   \n"])
def test_config_errors_return_codes(host, tmp_path, text):
    """Malformed files fail with a status and a message, without exiting."""
    p = tmp_path / "bad.cfg"
    p.write_text(text)
    cfg = C.c_void_p()
    assert host.rift_config_open(str(p).encode(), C.byref(cfg)) != 0
    assert host.rift_host_last_error()


# ---------------------------------------------------------------- rasters
def test_esri_read_flips_rows(host, tmp_path):
    rng = np.random.default_rng(0)
    data = rng.uniform(0, 50, size=(7, 9))
    p = tmp_path / "dem.asc"
    _write_esri(p, data)
    nc, nr = C.c_int32(), C.c_int32()
    xll, yll, cs, nd = C.c_double(), C.c_double(), C.c_double(), C.c_double()
    assert host.rift_esri_read_header(str(p).encode(), C.byref(nc), C.byref(nr), C.byref(xll),
                                      C.byref(yll), C.byref(cs), C.byref(nd)) == 0
    assert (nc.value, nr.value, xll.value, yll.value, cs.value, nd.value) == \
        (9, 7, 100.0, 200.0, 10.0, -9999.0)
    out = np.zeros((7, 9))
    assert host.rift_esri_read(str(p).encode(), 9, 7, 0,
                               out.ctypes.data_as(C.POINTER(C.c_double))) == 0
    np.testing.assert_array_equal(out, data)
    # wrong expected size
    assert host.rift_esri_read(str(p).encode(), 8, 7, 0,
                               out.ctypes.data_as(C.POINTER(C.c_double))) != 0


def test_esri_nodata_policy(host, tmp_path):
    data = np.ones((3, 4))
    data[1, 2] = -1.0
    p = tmp_path / "m.asc"
    _write_esri(p, data, nodata=-1)
    out = np.zeros((3, 4))
    ptr = out.ctypes.data_as(C.POINTER(C.c_double))
    assert host.rift_esri_read(str(p).encode(), 4, 3, 0, ptr) != 0  # DEM, n, K: abort
    assert host.rift_esri_read(str(p).encode(), 4, 3, 1, ptr) == 0  # map series: nodata
    assert out[1, 2] == -9999.0 and out[0, 0] == 1.0


def test_gridconfig_and_write_hgrid(host, tmp_path):
    data = np.arange(6 * 5, dtype=float).reshape(6, 5)
    dem = tmp_path / "dem.asc"
    _write_esri(dem, data, xll=1000.0, yll=2000.0, cell=2.5)
    gc = GridConfig()
    assert host.rift_gridconfig_from_dem(str(dem).encode(), 1, 1, C.byref(gc)) == 0
    assert (gc.b_nx, gc.b_ny, gc.h_nx, gc.h_ny) == (5, 6, 8, 9)
    assert gc.h_xll == 1000.0 + 1.25 and gc.h_yll == 2000.0 + 1.25
    assert gc.h_dx == gc.h_dy == gc.cellsize == 2.5
    # degrees, square cells: cellsize * 6378137 * pi / 180
    gd = GridConfig()
    assert host.rift_gridconfig_from_dem(str(dem).encode(), 1, 0, C.byref(gd)) == 0
    assert gd.h_dx == 2.5 * 6378137.0 * math.pi / 180.0
    # Coord2Index: i = int((X - h_xll) / cs + 0.5), 2 cells west of the point
    i, j, ok = C.c_int32(), C.c_int32(), C.c_int32()
    host.rift_gridconfig_coord2index(C.byref(gc), C.c_double(1000.0 + 1.25 + 3 * 2.5),
                                     C.c_double(2000.0 + 1.25 + 4 * 2.5), C.byref(i), C.byref(j),
                                     C.byref(ok))
    assert (i.value, j.value, ok.value) == (3, 4, 1)
    # writeGrid: interior only, north row first, 15 significant digits
    x = np.random.default_rng(1).uniform(-5, 5, size=(gc.h_ny, gc.h_nx))
    out = tmp_path / "h0.txt"
    assert host.rift_esri_write_hgrid(str(out).encode(), x.ctypes.data_as(C.POINTER(C.c_double)),
                                      C.byref(gc)) == 0
    lines = out.read_text().splitlines()
    assert lines[0].split() == ["ncols", "4"] and lines[1].split() == ["nrows", "5"]
    assert lines[5].split() == ["NODATA_value", "-9999"]
    body = [[float(v) for v in ln.split()] for ln in lines[6:]]
    expect = x[2:-2, 2:-2][::-1]
    np.testing.assert_allclose(np.array(body), expect, rtol=1e-14)
    assert lines[6].split()[0] == "%.15g" % expect[0, 0]


# ---------------------------------------------------------------- CSV
@pytest.mark.parametrize("hours,rates", [([0, 0.5, 0.5, 1], [50, 50, 0, 0]),
                                         ([0, 1, 3], [0, 500, 0]),
                                         ([0, 0.25, 0.5], [12.5, 30, 7])])
def test_csv_matches_source_rules(host, tmp_path, hours, rates):
    p = tmp_path / "s.csv"
    p.write_text("# header comment\n" + "".join(f"{h}, {r}\n" for h, r in zip(hours, rates)))
    n = C.c_int32()
    t = np.zeros(16, dtype=np.float32)
    r = np.zeros(16, dtype=np.float32)
    assert host.rift_csv_read(str(p).encode(), t.ctypes.data_as(C.POINTER(C.c_float)),
                              r.ctypes.data_as(C.POINTER(C.c_float)), 16, C.byref(n)) == 0
    et, er = synth.csv_series(hours, rates)
    assert n.value == len(et)
    np.testing.assert_array_equal(t[:n.value], et)
    np.testing.assert_array_equal(r[:n.value], er)


# ---------------------------------------------------------------- hotstart
def _grow(h_nx, h_ny):
    nbx, nby = -(-h_nx // 16), -(-h_ny // 14)
    return (-(-nbx // 16) * 16) * (-(-nby // 14) * 14)


@pytest.mark.parametrize("has_F", [0, 1])
def test_hotstart_layout_and_round_trip(host, tmp_path, has_F):
    data = np.zeros((20, 33))
    dem = tmp_path / "dem.asc"
    _write_esri(dem, data, cell=5.0)
    gc = GridConfig()
    assert host.rift_gridconfig_from_dem(str(dem).encode(), 1, 1, C.byref(gc)) == 0
    G = _grow(gc.h_nx, gc.h_ny)
    assert host.rift_grow_grid_size(gc.h_nx, gc.h_ny) == G
    rng = np.random.default_rng(2)
    n = gc.h_nx * gc.h_ny
    fields = [rng.standard_normal(n) for _ in range(3 + has_F)]
    wet = rng.integers(0, 2, size=G).astype(np.uint8)
    act = rng.integers(-50, 50, size=G).astype(np.int32)
    p = tmp_path / "hot3.bin"
    D = C.POINTER(C.c_double)
    args = [f.ctypes.data_as(D) for f in fields] + ([None] if not has_F else [])
    assert host.rift_hotstart_write(str(p).encode(), C.c_double(12.5), C.c_double(0.25),
                                    C.byref(gc), *args, wet.ctypes.data_as(C.POINTER(C.c_uint8)),
                                    act.ctypes.data_as(C.POINTER(C.c_int32))) == 0
    raw = p.read_bytes()
    assert len(raw) == 98 + 8 * n * (3 + has_F) + 5 * G == host.rift_hotstart_size(C.byref(gc), has_F)
    # byte layout: t, dt, b_nx, b_ny, b_xll, b_yll, cs, h_nx, h_ny, h_xll, h_yll, cellsize,
    # h_dx, h_dy, square, projected, then the fields and tile arrays
    assert np.frombuffer(raw, "<f8", 2, 0).tolist() == [12.5, 0.25]
    assert np.frombuffer(raw, "<i4", 2, 16).tolist() == [33, 20]
    assert np.frombuffer(raw, "<i4", 2, 48).tolist() == [gc.h_nx, gc.h_ny]
    assert np.frombuffer(raw, "<f8", 1, 80)[0] == 5.0 and raw[96] == 1 and raw[97] == 1
    off = 98
    for f in fields:
        np.testing.assert_array_equal(np.frombuffer(raw, "<f8", n, off), f)
        off += 8 * n
    np.testing.assert_array_equal(np.frombuffer(raw, np.uint8, G, off), wet)
    np.testing.assert_array_equal(np.frombuffer(raw, "<i4", G, off + G), act)
    # read back
    t, dt, g2 = C.c_double(), C.c_double(), GridConfig()
    back = [np.zeros(n) for _ in range(4)]
    wb, ab = np.zeros(G, np.uint8), np.zeros(G, np.int32)
    assert host.rift_hotstart_read(str(p).encode(), C.byref(t), C.byref(dt), C.byref(g2), has_F,
                                   *[b.ctypes.data_as(D) for b in back],
                                   wb.ctypes.data_as(C.POINTER(C.c_uint8)),
                                   ab.ctypes.data_as(C.POINTER(C.c_int32))) == 0
    assert (t.value, dt.value, g2.h_nx, g2.b_ny) == (12.5, 0.25, gc.h_nx, 20)
    for f, b in zip(fields, back):
        np.testing.assert_array_equal(f, b)
    np.testing.assert_array_equal(wb, wet)
    np.testing.assert_array_equal(ab, act)
    # a truncated file is an error, not a crash
    (tmp_path / "short.bin").write_bytes(raw[:200])
    assert host.rift_hotstart_read(str(tmp_path / "short.bin").encode(), C.byref(t), C.byref(dt),
                                   C.byref(g2), has_F, *[b.ctypes.data_as(D) for b in back],
                                   wb.ctypes.data_as(C.POINTER(C.c_uint8)),
                                   ab.ctypes.data_as(C.POINTER(C.c_int32))) != 0


def test_sim_open_reports_config_errors(host, tmp_path):
    """A missing required key fails cleanly (the reference waits on stdin)."""
    p = tmp_path / "sim.cfg"
    p.write_text("t0 = 0\ntf = 10\n")
    sim = C.c_void_p()
    assert host.rift_sim_open(str(p).encode(), C.byref(sim)) != 0
    assert not sim.value
    assert b"DEM" in host.rift_host_last_error()
