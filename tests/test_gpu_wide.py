"""The wide path (one world spread over the whole GPU, cp_wide.cu) against
the oracle and against the one-block path, bit for bit.

cp_set_wide_bodies(1) sends every world, however small, through the wide
kernels, so the small scenes that reach every branch of World.step (edge
scenes, all three broadphases, constraints, sleeping, capacity regrowth)
check the wide path against the oracle step by step, with the sweeps on
the library's choice of schedule, on the slot schedule wherever it fits
(cp_set_sweep_schedule(1): early exits then roll back at every step that
stops early) and level by level.  The full-size box pile
(4097 bodies, SAP) and the mixed scene with chains (8193 bodies, grid,
sleeping) take the wide path by default; they are checked against the
oracle over horizons long enough for the pile to be in contact everywhere.
"""
import numpy as np
import pytest

from cannon_physics_gb300 import engine, scenes
from oracle import oracle_py as O

from tests.edge_scenes import EDGE_NAMES, edge_scene
from tests.parity import compare_step

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from cannon_physics_gb300 import build as B
    B.build()
    c = engine.Context()
    yield c
    c.close()


# The wide path's Gauss-Seidel sweeps run level by level or on a slot
# schedule across sweeps; every small-scene test runs with the library's
# choice, with the schedule forced wherever it fits, and with it off.
SCHEDULE_MODES = {"sched_auto": 0, "sched_forced": 1, "levels_only": -1}


@pytest.fixture(params=sorted(SCHEDULE_MODES))
def wide_ctx(ctx, request):
    ctx.set_wide_bodies(1)
    ctx.set_sweep_schedule(SCHEDULE_MODES[request.param])
    yield ctx
    ctx.set_sweep_schedule(0)
    ctx.set_wide_bodies(1024)


def run_parity(ctx, scene, steps, every=1, check_lists=True, oracle=None, start=0):
    engine.setup_scene(scene)
    gw = ctx.world(scene)
    ow = oracle or O.OracleWorld(scene)
    if start:
        gw.step(nsteps=start)
        ow.load_state(gw)
    done = 0
    while done < steps:
        k = min(every, steps - done)
        gw.step(nsteps=k)
        ow.step(nsteps=k)
        done += k
        errs = compare_step(gw, ow, check_lists=check_lists)
        assert not errs, f"{scene.name}: mismatch after step {start + done}:\n" + "\n".join(errs[:10])
    info = gw.info()
    gw.destroy()
    return info


@pytest.mark.parametrize("name", EDGE_NAMES)
def test_wide_edge_scenes(wide_ctx, name):
    run_parity(wide_ctx, edge_scene(name), 30)


def test_wide_small_box_pile_sap(wide_ctx):
    run_parity(wide_ctx, scenes.box_pile(6, 6, 4), 40)


def test_wide_small_grid_chains_sleep(wide_ctx):
    run_parity(wide_ctx, scenes.mixed_chains(8, 4, 4, chains=4, chain_len=8), 60, every=2)


@pytest.mark.parametrize("n,seed", [(60, 1002), (512, 1004)])
def test_wide_naive_columns(wide_ctx, n, seed):
    run_parity(wide_ctx, scenes.column_world(n, seed, "sphere_box"), 40, every=4)


def test_wide_dense_cluster_grows_capacities(wide_ctx):
    sc = scenes.spheres_on_plane(300)
    rng = scenes.SplitMix64(99)
    sc.bodies["position"][1:] = (rng.uniform(900).reshape(300, 3) * 1.2 + np.array([-0.6, 0.6, -0.6]))
    run_parity(wide_ctx, sc, 5)


def test_box_pile_full_size_in_contact(ctx):
    """The 4096-box SAP pile: 10 steps compared from the start, then from
    step 100 (every layer landed) the GPU world continues and is compared with
    the oracle continued from the same state, for 60 more steps."""
    run_parity(ctx, scenes.box_pile(), 10, every=5)
    info = run_parity(ctx, scenes.box_pile(), 60, every=10, start=100)
    assert info.num_contacts > 6000


@pytest.mark.parametrize("mode", [1, -1])
def test_box_pile_full_size_schedule_modes(ctx, mode):
    """The full-size pile from step 100 with the slot-scheduled sweeps forced
    on every step, and with them off."""
    ctx.set_sweep_schedule(mode)
    try:
        info = run_parity(ctx, scenes.box_pile(), 20, every=10, start=100)
    finally:
        ctx.set_sweep_schedule(0)
    assert info.num_contacts > 6000


def test_mixed_chains_full_size_thirty_steps(ctx):
    """8192 mixed shapes with 128 chains, GridBroadphase, sleeping on: 30
    steps from step 90 on."""
    info = run_parity(ctx, scenes.mixed_chains(), 30, every=10, start=90)
    assert info.num_rows > 5000


def test_wide_equals_one_block(ctx):
    """The same large world on the wide path and on one block."""
    sc = engine.setup_scene(scenes.column_world(1500, 8080, "mixed"))
    a = ctx.world(sc)
    a.step(nsteps=40)
    ctx.set_wide_bodies(0)
    try:
        b = ctx.world(sc)
        b.step(nsteps=40)
    finally:
        ctx.set_wide_bodies(1024)
    assert a.bodies().tobytes() == b.bodies().tobytes()
    pa, pb = a.pairs(), b.pairs()
    assert np.array_equal(pa[0], pb[0]) and np.array_equal(pa[1], pb[1])
    assert a.info().iterations == b.info().iterations
    a.destroy()
    b.destroy()


@pytest.mark.parametrize("tol", [1.0, 10.0])
def test_wide_sweeps_stop_early(wide_ctx, tol):
    """A loose solver tolerance ends the sweeps before the iteration limit
    (after the first sweep, at times); the exit test (order-free block sum,
    row-order sum inside the rounding band) takes the reference's decision:
    rows, bodies and iteration counts equal the oracle's at every step."""
    sc = engine.setup_scene(scenes.box_pile(8, 8, 4, seed=31))
    sc.tolerance = tol
    sc.iterations = 30
    gw = wide_ctx.world(sc)
    ow = O.OracleWorld(sc)
    its = []
    for s in range(40):
        gw.step(nsteps=1)
        ow.step(nsteps=1)
        errs = compare_step(gw, ow)
        assert not errs, f"step {s + 1}:\n" + "\n".join(errs[:10])
        its.append(gw.info().iterations)
    gw.destroy()
    assert min(its) < 30 and max(its) > min(its)


def test_wide_sweeps_long_chains(wide_ctx):
    """Tall stacks: long level chains, many sweeps; results stay the oracle's."""
    sc = scenes.box_pile(3, 3, 24, seed=32, pitch=1.05)
    sc.iterations = 25
    run_parity(wide_ctx, sc, 60)
