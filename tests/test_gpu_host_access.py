"""The host-array access path (state import and field export as device
kernels on the caller's pageable arrays, where the GPU reads host memory
through the host page tables) gives bit for bit what the staged host path
gives: every field after a run, and the steps that follow a state upload."""
import numpy as np
import pytest

from rift_gb300 import capi, synth

pytestmark = pytest.mark.gpu

FIELDS = ("W", "HU", "HV", "H", "F", "HMAX", "QMAX", "TWET", "Q", "BC")


def _sim(engine_api):
    flags = (synth.RAIN_UNIFORM | synth.TILE_ACCEL | synth.INFILTRATION | synth.SAVE_MAX
             | synth.SAVE_ARRIVAL)
    case = synth.small_case(nx_cells=70, ny_cells=52, seed=11, cell=5.0, flags=flags,
                            rain_mmhr=300.0)
    case.K = np.full_like(case.n, 2e-6)
    case.psi, case.dtheta = 0.11, 0.3
    return capi.Sim(case).setup()


def test_host_access_fields_and_uploads_match_the_staged_path(engine_api):
    sim = _sim(engine_api)
    try:
        sim.set_host_access(True)
    except capi.RiftError:
        pytest.skip("the device does not access pageable host memory")
    assert sim.host_access()
    sim.run(300)
    direct = {f: sim.field(f) for f in FIELDS}
    sim.set_host_access(False)
    staged = {f: sim.field(f) for f in FIELDS}
    for f in FIELDS:
        assert np.array_equal(direct[f], staged[f]), f
    snap = sim.snapshot()
    ends = []
    for on in (True, False):
        sim.set_host_access(on)
        sim.load_snapshot(snap)
        sim.run(50)
        sim.set_host_access(False)
        ends.append({f: sim.field(f) for f in ("W", "HU", "HV", "F")} | {"tiles": sim.tiles()})
    for f in ("W", "HU", "HV", "F"):
        assert np.array_equal(ends[0][f], ends[1][f]), f
    assert np.array_equal(ends[0]["tiles"][1], ends[1]["tiles"][1])
    sim.close()
