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


def test_ensemble_members_match_the_reference_kernels(engine_api):
    """Every golden case stepped inside the ensemble kernel, all together,
    checked at its dump steps against the reference's own kernels (the
    golden dumps): tile sets bit-exact, t within 1e-5 relative, depths within
    the golden bars (1e-6 m on 99% of the cells, 5e-5 m everywhere)."""
    names = list(FX.CASES)
    fxs = [FX.load(n)[0] for n in names]
    members = _members(engine_api, names)
    ens = capi.Ensemble(members)
    done = [0] * len(names)
    targets = sorted({s for fx in fxs for s in FX.dumps(fx)})
    for s in targets:
        live = [m for m, fx in enumerate(fxs) if max(FX.dumps(fx)) >= s]
        # members past their last dump stay in the kernel; advance everyone to s
        steps = s - min(done[m] for m in live)
        t, k = ens.run(max_steps=steps)
        for m in range(len(names)):
            done[m] += int(k[m])
        for m in live:
            fx = fxs[m]
            if s not in FX.dumps(fx):
                continue
            assert done[m] == s, (names[m], done[m], s)
            ref = FX.ref_state(fx, s)
            wet, act = members[m].tiles()
            assert np.array_equal(wet, ref["wet"]), f"{names[m]}: wet tiles at step {s}"
            assert np.array_equal(act, ref["active"]), f"{names[m]}: active tiles at step {s}"
            tm = members[m].time()[0]
            assert abs(tm - ref["t"]) <= 1e-5 * max(1.0, abs(ref["t"])), (names[m], tm, ref["t"])
            d = np.abs(FX.interior(members[m].field("W") - ref["w"]))
            assert np.quantile(d, 0.99) <= Q99 and d.max() <= MAX, f"{names[m]} step {s}: {d.max()}"
    ens.close()


def test_ensemble_member_times_follow_completion(engine_api):
    """Members of different dt reach t_stop after different step counts: the
    device clock has each one finish no later than a member that ran more
    iterations of the shared loop, and every member that ran has a positive
    completion time inside the call's wall time."""
    import time
    names = ["rain", "front", "euler"]
    members = _members(engine_api, names)
    ens = capi.Ensemble(members)
    w0 = time.perf_counter()
    t, k = ens.run(t_stop=600.0)
    wall = time.perf_counter() - w0
    sec = ens.member_times()
    assert (sec > 0).all() and (sec <= wall).all(), (sec, wall)
    order = np.argsort(k, kind="stable")
    assert k[order[0]] < k[order[-1]], k  # the wet cases take smaller steps than the dry front
    assert sec[order[0]] <= sec[order[-1]]
    ens.close()


def test_ensemble_with_solo_members_matches_members_alone(engine_api):
    """Members above the solo threshold run on their own per-step graphs after
    the ensemble kernel; every member still ends where it ends alone, and the
    completion times are measured for all of them."""
    names = list(FX.CASES)
    steps = 25
    solo = _members(engine_api, names)
    for s in solo:
        s.run(steps)
    members = _members(engine_api, names)
    cells = np.array([(m.nx - 4) * (m.ny - 4) for m in members])
    thr = int(np.median(cells))
    ens = capi.Ensemble(members).set_solo_cells(thr)
    t, k = ens.run(max_steps=steps)
    assert (k == steps).all()
    sec = ens.member_times()
    assert (sec > 0).all()
    big = cells >= thr
    assert big.any() and (~big).any()
    assert sec[big].min() >= sec[~big].max()  # the solo members run after the kernel
    for name, a, b in zip(names, members, solo):
        _same(_state(a), _state(b), name)
    # launches: the one ensemble kernel plus every kernel the solo members ran
    solo_launches = sum(m.launch_count() for m, b_ in zip(members, big) if b_)
    assert solo_launches > 0
    assert ens.launch_count() == 1 + solo_launches
    ens.close()
