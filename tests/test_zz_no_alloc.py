"""rift_volume_noalloc: the volume sum for callers that cannot allocate.

A caller that must not allocate device memory (a coupled model summing the
2D volume from inside its own time loop, with memory from its own pool)
passes its own depth buffer and its own one-double output; the library keeps
its scratch in a fixed device array.  These checks call it through the C ABI
on buffers the test owns and compare it with rift_volume, which sums the
same depth field held by an engine handle: two calls in a row, on different
fields, so a stale partial from the first call would show in the second.
Tolerance: 1e-12 relative (both are FP64 compensated sums of the same FP32
values, in different orders).

This file is collected last so that a failure here does not stop the rest
of a -x run.
"""
import ctypes

import numpy as np
import pytest

from rift_gb300 import capi, synth

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12


def _bind(lib):
    f = lib.rift_volume_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                  ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]
    return f


def _engine_volume(sim, bc, h32):
    """rift_volume of an engine handle whose state holds depth h32."""
    w = bc + h32.astype(np.float64)
    z = np.zeros_like(w)
    sim.set_state(0.0, 1e-3, w, z, z)
    return sim.volume()


def test_noalloc_volume_matches_engine_volume_twice(engine_api):
    torch = pytest.importorskip("torch")
    lib, _ = engine_api
    noalloc = _bind(lib)
    case = synth.small_case(70, 58, seed=31)
    sim = capi.Sim(case, api=engine_api).setup()
    bc = sim.field("BC")
    rng = np.random.default_rng(4)
    ny, nx = bc.shape
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        h32 = np.zeros((ny, nx), dtype=np.float32)
        h32[2:-2, 2:-2] = rng.uniform(0.0, 2.0 + call, size=(ny - 4, nx - 4)).astype(np.float32)
        expected = _engine_volume(sim, bc, h32)
        dev = torch.from_numpy(h32).cuda().contiguous()
        torch.cuda.synchronize()
        rc = noalloc(ctypes.c_void_p(dev.data_ptr()), None, nx, ny, nx,
                     ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream))
        assert rc == 0
        torch.cuda.synchronize()
        got = float(out.item())
        assert abs(got - expected) <= REL_TOL * abs(expected), (call, got, expected)
        # against the exact sum of the same float values
        exact = float(np.sum(h32[2:-2, 2:-2].astype(np.float64)))
        assert abs(got - exact) <= REL_TOL * exact
    sim.close()


@pytest.mark.parametrize("rows", [37, 2101, 32768])
def test_noalloc_volume_tall_grids(engine_api, rows):
    """Grids from a few rows (most of the combining warp's lanes get no rows)
    up to the scratch limit (every lane sums a block of 1,024 rows), with an
    infiltration field and a leading dimension wider than the grid."""
    torch = pytest.importorskip("torch")
    lib, _ = engine_api
    noalloc = _bind(lib)
    nx, ld = 21, 32
    rng = np.random.default_rng(rows)
    h = np.zeros((rows, ld), dtype=np.float32)
    F = np.zeros((rows, ld), dtype=np.float32)
    h[2:-2, 2:nx - 2] = rng.uniform(0.0, 3.0, size=(rows - 4, nx - 4)).astype(np.float32)
    F[2:-2, 2:nx - 2] = rng.uniform(0.0, 0.1, size=(rows - 4, nx - 4)).astype(np.float32)
    h[:, nx - 2:] = 1e6  # outside the interior: must not be summed
    exact = float(np.sum(h[2:-2, 2:nx - 2].astype(np.float64)) +
                  np.sum(F[2:-2, 2:nx - 2].astype(np.float64)))
    dh, dF = torch.from_numpy(h).cuda(), torch.from_numpy(F).cuda()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    for _ in range(2):
        torch.cuda.synchronize()
        rc = noalloc(ctypes.c_void_p(dh.data_ptr()), ctypes.c_void_p(dF.data_ptr()), nx, rows, ld,
                     ctypes.c_void_p(out.data_ptr()), None)
        assert rc == 0
        torch.cuda.synchronize()
        got = float(out.item())
        assert abs(got - exact) <= REL_TOL * exact, (rows, got, exact)


def test_noalloc_volume_rejects_grids_beyond_its_scratch(engine_api):
    torch = pytest.importorskip("torch")
    lib, _ = engine_api
    noalloc = _bind(lib)
    buf = torch.zeros(16, dtype=torch.float32, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    max_rows = 32768  # RIFT_NOALLOC_MAX_ROWS
    rc = noalloc(ctypes.c_void_p(buf.data_ptr()), None, 8, max_rows + 1, 8,
                 ctypes.c_void_p(out.data_ptr()), None)
    assert rc == 7  # RIFT_ERR_TOO_LARGE, nothing launched
