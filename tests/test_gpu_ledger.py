"""The engine's volume ledger (rift_mass_ledger_terms, check_volume runs) on
the GPU, against the oracle's FP64 ledger on the same inputs, on every
schedule of the step (persistent loop, per-tile kernels, column march).

Each engine term is accumulated from the FP32 quantities the step applies,
so it agrees with the oracle's FP64 term to FP32 accuracy (TERM_TOL of the
water moved).  The engine's closure residual is the FP32 state's own
rounding: every cell update rounds h to 24 bits, which no ledger term can
see; CLOSE_TOL bounds it and the printed value is the measured one."""
import numpy as np
import pytest

import fixture as FX
from rift_gb300 import capi, synth

pytestmark = pytest.mark.gpu

TERM_TOL = 1e-4   # |engine term - oracle term| / water moved
CLOSE_TOL = 1e-7  # |engine residual| / water moved (measured on GB300: at most 2.5e-8)
TERMS = ("added", "drained", "infiltrated", "clamped", "surge", "boundary")

SCHEDULES = {
    "default": lambda s: s,
    "tiles": lambda s: s.set_persistent(0).set_schedule(1 << 30),
    "march": lambda s: s.set_persistent(0).set_schedule(0),
}


def _scale(L):
    return (abs(L["volume0"]) + abs(L["added"]) + abs(L["drained"]) + abs(L["infiltrated"]) +
            abs(L["clamped"]) + abs(L["surge"]) + abs(L["boundary"]))


@pytest.mark.parametrize("schedule", list(SCHEDULES))
@pytest.mark.parametrize("name,steps", [("rain", 60), ("h0_infil_src", 40), ("gridrain_surge", 60),
                                        ("euler", 40), ("front", 150)])
def test_engine_ledger_matches_oracle(engine_api, oracle_api, name, steps, schedule):
    fx, case = FX.load(name)
    case.flags |= synth.CHECK_VOLUME
    eng = FX.start(SCHEDULES[schedule](capi.Sim(case, api=engine_api)), fx)
    orc = FX.start(capi.Sim(case, api=oracle_api, create_mode=0), fx)
    eng.run(steps)
    for _ in range(steps):
        orc.step()
    Le, Lo = eng.ledger(), orc.ledger()
    scale = _scale(Lo)
    worst = max(abs(Le[k] - Lo[k]) for k in TERMS + ("volume", "volume0")) / scale
    print(f"{name}/{schedule}: largest term difference {worst:.2e} of the water moved")
    for k in TERMS + ("volume", "volume0"):
        assert abs(Le[k] - Lo[k]) <= TERM_TOL * scale, (name, schedule, k, Le[k], Lo[k])
    print(f"{name}/{schedule}: engine residual {Le['residual'] / scale:.2e}, "
          f"oracle {Lo['residual'] / scale:.2e} of the water moved")
    assert abs(Le["residual"]) <= CLOSE_TOL * scale, (name, schedule, Le)
    eng.close()
    orc.close()


def test_ledger_off_without_check_volume(engine_api):
    """Without check_volume the per-cell terms are not kept (they read 0) and
    the step is the plain one."""
    fx, case = FX.load("h0_infil_src")
    eng = FX.start(capi.Sim(case, api=engine_api), fx)
    eng.run(20)
    L = eng.ledger()
    assert L["added"] > 0
    assert all(L[k] == 0.0 for k in ("drained", "infiltrated", "clamped", "surge", "boundary"))
    assert np.isnan(L["volume0"])


def test_ensemble_rejects_check_volume_members(engine_api):
    fx, case = FX.load("rain")
    case.flags |= synth.CHECK_VOLUME
    a = FX.start(capi.Sim(case, api=engine_api), fx)
    with pytest.raises(capi.RiftError):
        capi.Ensemble([a])
