"""Stage fusion of the column march (k_march2f) on the GPU: stage 2 rebuilds
U* from U^n and the stored stage-1 divergence on the strips whose staged block
holds no ghost cell.  It must give the results of the unfused march (stage-1
update pass + stage 2 reading U*), which the parity tests pin against the
reference: the same rk1Core arithmetic runs in both, so tile sets, times and
states are compared exactly (a difference of one FP32 rounding would show as
a few ulp; the bar allows 1e-6 m and reports what it saw).

Workloads at 1024^2, large enough for strips that qualify and strips that do
not: the plain rain plane (uniform-rain instantiation), the channel flood with
Green-Ampt and a point source (its instantiation, F* rebuilt per cell), the
urban map-rain grid with a drain (its instantiation), and check_volume runs
(the generic instantiation, whose ledger terms must match too)."""
import numpy as np
import pytest

from rift_gb300 import capi, synth

pytestmark = pytest.mark.gpu

STEPS = 30


def _march(case, engine_api, fused):
    sim = capi.Sim(case, api=engine_api).set_schedule(0).set_persistent(0).set_stage_fusion(fused)
    return sim.setup()


def _cases():
    c1 = synth.config1(N=1024)
    c2 = synth.config2(N=1024)
    c3 = synth.config3(N=1024, nblocks=60)
    c3l = synth.config3(N=1024, nblocks=60)
    c3l.flags |= synth.CHECK_VOLUME
    c2l = synth.config2(N=1024)
    c2l.flags |= synth.CHECK_VOLUME
    return {"rain": c1, "channel_infiltration": c2, "map_rain_drain": c3, "generic_ledger_rain": c3l,
            "generic_ledger_infil": c2l}


@pytest.mark.parametrize("name", list(_cases()))
def test_fused_stage_two_matches_the_split_march(engine_api, name):
    case = _cases()[name]
    spin = {"channel_infiltration": 3600.0, "generic_ledger_infil": 3600.0}.get(name, 120.0)
    base = _march(case, engine_api, False)
    base.run(2 ** 31 - 1, spin)
    snap = base.snapshot()
    fused = _march(case, engine_api, True)
    fused.load_snapshot(snap)
    base.load_snapshot(snap)
    tb, _, kb = base.run(STEPS)
    tf, _, kf = fused.run(STEPS)
    assert kb == kf == STEPS and tb == tf, (tb, tf)
    wb, ab = base.tiles()
    wf, af = fused.tiles()
    assert np.array_equal(wb, wf) and np.array_equal(ab, af)
    for fld in ("W", "HU", "HV") + (("F",) if case.flags & synth.INFILTRATION else ()):
        d = np.abs(base.field(fld) - fused.field(fld))[2:-2, 2:-2]
        print(f"{name}: max |fused - split| {fld} = {d.max():.3e}")
        assert d.max() <= 1e-6, (fld, d.max())
    if case.flags & synth.CHECK_VOLUME:
        Lb, Lf = base.ledger(), fused.ledger()
        scale = abs(Lb["volume0"]) + abs(Lb["added"]) + abs(Lb["drained"]) + abs(Lb["infiltrated"])
        for k in ("added", "drained", "infiltrated", "clamped", "surge", "boundary", "volume"):
            assert abs(Lb[k] - Lf[k]) <= 1e-6 * scale, (k, Lb[k], Lf[k])
    base.close()
    fused.close()
