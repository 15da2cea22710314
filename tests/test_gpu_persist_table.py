"""The persistent loop's tile table on the GPU.

With one scheduled tile per CTA the loop keeps each tile on its CTA from
step to step: a CTA gives up a tile that went inactive, and a tile that
turns wet hands CTAs to its neighbours.  Runs of many steps in one launch
(rift_run) must give the tile sets and depths of the per-step graph, through
growth past the grid (the table is voided and the loop falls back to the
grow), drying (tiles given up, U* re-synced) and rebuilds.
"""
import numpy as np
import pytest

from rift_gb300 import capi, synth

pytestmark = pytest.mark.gpu

CELL = 10.0
Q99, MAX = 1e-6, 5e-5
PERSIST = (1 << 30, 1 << 30)   # march threshold (strips), persistent threshold (tiles)
GRAPH = (1 << 30, 0)


def _plane(N, slope=0.001, seed=0):
    rng = np.random.default_rng(seed)
    x = np.arange(N + 1) * CELL
    X, Y = np.meshgrid(x, x)
    z = 10.0 - slope * X + 0.05 * rng.standard_normal(X.shape)
    n = np.zeros((N + 4, N + 4))
    n[2:-2, 2:-2] = 0.03
    return z, n


def _mound(N, depth, radius_cells, at=None):
    h0 = np.zeros((N + 4, N + 4))
    cy, cx = at if at is not None else (N // 2, N // 2)
    jj, ii = np.meshgrid(np.arange(N), np.arange(N), indexing="ij")
    r2 = (jj - cy) ** 2 + (ii - cx) ** 2
    h0[2:-2, 2:-2] = np.where(r2 <= radius_cells ** 2, depth, 0.0)
    return h0


def _rain_front(N=256):
    """Uniform rain on a plane, water in one tile: every active tile is wet
    while it rains, so the active set grows by a ring of tiles per step and
    outgrows a one-wave grid within a few steps."""
    z, n = _plane(N)
    t, r = synth.csv_series([0, 1], [60, 60])
    case = synth.Case(name="rain_front", B=z, cell=CELL, n=n,
                      flags=synth.TILE_ACCEL | synth.RAIN_UNIFORM | synth.H_INIT,
                      series={0: (t, r)})
    case.h0 = _mound(N, 0.5, 4)
    return case


def _soak(N=192):
    """A dam-break mound on an infiltrating plane: the wet set spreads, then
    the soil takes the water and tiles dry and go inactive."""
    z, n = _plane(N, slope=0.0005, seed=1)
    case = synth.Case(name="soak", B=z, cell=CELL, n=n, psi=0.11, dtheta=0.3,
                      flags=synth.TILE_ACCEL | synth.INFILTRATION | synth.H_INIT)
    case.h0 = _mound(N, 0.05, 30)
    case.K = np.full((N + 4, N + 4), 2e-4)
    return case


def _channel():
    """The channel flood (hydrograph at the channel head, infiltration, n
    map) on a 256^2 grid: a slowly growing front."""
    return synth.config2(N=256, cell=5.0, tf=21600.0)


CASES = {"rain_front": _rain_front, "soak": _soak, "channel": _channel}


def _sim(engine_api, case, sched):
    return capi.Sim(case, api=engine_api).set_schedule(sched[0]).set_persistent(sched[1]).setup()


def _compare(a, b, what):
    (wa, aa), (wb, ab) = a.tiles(), b.tiles()
    assert np.array_equal(wa, wb), f"{what}: wet tiles"
    assert np.array_equal(aa, ab), f"{what}: active tiles"
    ta, tb = a.time()[0], b.time()[0]
    assert abs(ta - tb) <= 1e-6 * max(1.0, tb), f"{what}: t {ta} vs {tb}"
    d = np.abs(a.field("W") - b.field("W"))[2:-2, 2:-2]
    assert np.quantile(d, 0.99) <= Q99 and d.max() <= MAX, f"{what}: max |dw| {d.max()}"


@pytest.mark.parametrize("name", list(CASES))
def test_table_matches_graph(engine_api, name):
    case = CASES[name]()
    a = _sim(engine_api, case, PERSIST)
    b = _sim(engine_api, case, GRAPH)
    done = 0
    for chunk in (1, 9, 30, 60, 100):
        a.run(chunk)
        b.run(chunk)
        done += chunk
        _compare(a, b, f"{name} after {done} steps")
    persist, graph = a.path_stats()
    assert graph == 0 and persist == done
    assert a.table_steps() > 0, "the tile table never ran"


def test_table_voided_by_growth_then_rebuilt(engine_api):
    """The rain front outgrows the grid of its launch (claims run out of
    CTAs); the next launch, sized for the larger set, rebuilds the table."""
    case = _rain_front()
    a = _sim(engine_api, case, PERSIST)
    b = _sim(engine_api, case, GRAPH)
    a.run(3)
    b.run(3)
    first = a.table_steps()
    a.run(40)   # grid sized for the few tiles of step 3: the front outgrows it
    b.run(40)
    _compare(a, b, "after growth")
    grown = a.table_steps()
    assert grown - first < 40, "the table should have been voided during growth"
    a.run(20)   # a new launch sized for the grown set
    b.run(20)
    _compare(a, b, "after rebuild")
    assert a.table_steps() > grown
