"""The FP64 volume ledger of the oracle closes (CPU, no GPU).

Every way the reference's step adds or removes water is a ledger term:
rain and point sources (added), the drain and Green-Ampt withdrawals after
their h/dt caps (grid.cu:776-805), the epsilon clamps of ComputeFluxes_k and
the integrators (grid.cu:748-749, 914-915, 1083-1084), the surge condition
(grid.cu:894-904) and the flow through the critical-depth ghost cells
(grid.cu:1325-1406).  In FP64 the state change over a run equals the sum of
the terms to rounding:
    V - V0 = added - drained - infiltrated - clamped + surge + boundary
The bar is the north-star's 1e-9 of the water moved (initial volume plus the
magnitudes of every term); FP64 reaches ~1e-14.  Cases: the golden fixtures'
inputs (open and rimmed domains, infiltration with a point source and a
drain, gridded rain with a surge strip, Euler mode) and a closed rimmed
domain."""
import numpy as np
import pytest

import fixture as FX
from rift_gb300 import capi, synth

BAR = 1e-9


def _scale(L):
    return (abs(L["volume0"]) + abs(L["added"]) + abs(L["drained"]) + abs(L["infiltrated"]) +
            abs(L["clamped"]) + abs(L["surge"]) + abs(L["boundary"]))


def _oracle(case, oracle_api, fx=None):
    sim = capi.Sim(case, api=oracle_api, create_mode=1)  # PURE64: every rounding point in FP64
    return FX.start(sim, fx) if fx is not None else sim.setup()


@pytest.mark.parametrize("name,steps", [("rain", 60), ("h0_infil_src", 40), ("gridrain_surge", 60),
                                        ("euler", 40), ("noaccel", 20), ("front", 150)])
def test_oracle_ledger_closes_on_fixture_inputs(oracle_api, name, steps):
    fx, case = FX.load(name)
    sim = _oracle(case, oracle_api, fx)
    for _ in range(steps):
        sim.step()
    L = sim.ledger()
    scale = _scale(L)
    assert scale > 0
    assert abs(L["residual"]) <= BAR * scale, (name, L)
    if case.flags & synth.INFILTRATION:
        assert L["infiltrated"] > 0
        assert abs((L["soil"] - L["soil0"]) - L["infiltrated"]) <= BAR * scale
    sim.close()


def test_oracle_ledger_terms_are_exercised(oracle_api):
    """Each term is non-zero somewhere: the ledger is not closing on zeros."""
    seen = {}
    for name, steps in (("rain", 60), ("h0_infil_src", 40), ("gridrain_surge", 60)):
        fx, case = FX.load(name)
        sim = _oracle(case, oracle_api, fx)
        for _ in range(steps):
            sim.step()
        for k, v in sim.ledger().items():
            seen[k] = max(seen.get(k, 0.0), abs(v))
        sim.close()
    for k in ("added", "drained", "infiltrated", "clamped", "surge", "boundary"):
        assert seen[k] > 0, k


def test_oracle_ledger_closed_rimmed_domain_and_restart(oracle_api):
    """A rimmed domain (rain on the rim drains out through the edge, so the
    edge term is an outflow); a restart from a snapshot starts a new ledger
    that closes as well."""
    case = synth.small_case(48, 40, seed=5, rain_mmhr=80.0, rim=True)
    sim = _oracle(case, oracle_api)
    for _ in range(80):
        sim.step()
    L = sim.ledger()
    assert L["boundary"] < 0
    assert abs(L["residual"]) <= BAR * _scale(L)
    snap = sim.snapshot()
    sim.load_snapshot(snap)
    L0 = sim.ledger()
    assert L0["added"] == 0.0 and L0["volume0"] == L0["volume"]
    for _ in range(40):
        sim.step()
    L = sim.ledger()
    assert L["added"] > 0 and abs(L["residual"]) <= BAR * _scale(L)
    sim.close()
