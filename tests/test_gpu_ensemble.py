"""Ensembles on the GPU: members of different sizes and options stepped
together by one persistent kernel (rift_ensemble_*) give each member the
results of a run of its own."""
import numpy as np
import pytest

import fixture as FX
from rift_gb300 import capi

pytestmark = pytest.mark.gpu

Q99, MAX = 1e-6, 5e-5


def _members(engine_api, names):
    out = []
    for name in names:
        fx, case = FX.load(name)
        out.append(FX.start(capi.Sim(case, api=engine_api), fx))
    return out


def _same(a, b, what):
    (wa, aa), Wa, ta = a
    (wb, ab), Wb, tb = b
    assert np.array_equal(wa, wb), f"{what}: wet tiles"
    assert np.array_equal(aa, ab), f"{what}: active tiles"
    assert abs(ta - tb) <= 1e-6 * max(1.0, abs(tb)), f"{what}: t {ta} vs {tb}"
    d = np.abs(FX.interior(Wa - Wb))
    assert np.quantile(d, 0.99) <= Q99 and d.max() <= MAX, f"{what}: max |dw| {d.max()}"


def _state(sim):
    return sim.tiles(), sim.field("W"), sim.time()[0]


def test_ensemble_matches_members_run_alone(engine_api):
    names = list(FX.CASES)
    steps = 25
    solo = _members(engine_api, names)
    for s in solo:
        s.run(steps)
    ens_members = _members(engine_api, names)
    ens = capi.Ensemble(ens_members)
    t, k = ens.run(max_steps=steps)
    assert (k == steps).all()
    for name, a, b, tk in zip(names, ens_members, solo, t):
        assert tk == a.time()[0]
        _same(_state(a), _state(b), name)
    # a second call continues every member where it stopped
    for s in solo:
        s.run(10)
    t2, k2 = ens.run(max_steps=10)
    assert (k2 == 10).all()
    for name, a, b in zip(names, ens_members, solo):
        _same(_state(a), _state(b), name + " (continued)")
    ens.close()


def test_ensemble_stops_each_member_at_t_stop(engine_api):
    """Members of different dt reach t_stop after different step counts, as
    rift_run(…, t_stop) would stop them one by one."""
    names = ["rain", "front", "euler"]
    t_stop = 40.0
    solo = _members(engine_api, names)
    counts = [s.run(10 ** 6, t_stop)[2] for s in solo]
    ens_members = _members(engine_api, names)
    ens = capi.Ensemble(ens_members)
    t, k = ens.run(t_stop=t_stop)
    assert list(k) == counts
    assert all(tk >= t_stop for tk in t)
    for name, a, b in zip(names, ens_members, solo):
        _same(_state(a), _state(b), name)
    ens.close()


def test_ensemble_rejects_bad_members(engine_api):
    fx, case = FX.load("rain")
    a = capi.Sim(case, api=engine_api)  # not initialised
    with pytest.raises(capi.RiftError):
        capi.Ensemble([a])
    b = FX.start(capi.Sim(case, api=engine_api), fx)
    with pytest.raises(capi.RiftError):
        capi.Ensemble([b, b])
