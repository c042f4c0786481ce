"""The event feed (cp_world_set_events / cp_world_get_events) against the
oracle's restatement of World's events.

The reference dispatches `collide` for every contact (its two collision
matrices are one object), then beginContact / endContact and
beginShapeContact / endShapeContact from its OverlapKeepers' sorted diffs,
where kinematic / static pairs whose shapes overlap count too
(lib/world/world_class.dart:593-610,703-770, narrow_phase.dart:712-715).
The oracle restates those structures as the reference has them (insertion
into sorted lists, a merge diff); the library builds the same event
sequences from each step's contact and pair lists with sorted key sets.
Sequences must be equal, event by event, every step.
"""
import numpy as np
import pytest

from cannon_physics_gb300 import engine, scenes
from oracle import oracle_py as O

from tests.edge_scenes import edge_scene

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from cannon_physics_gb300 import build as B
    B.build()
    c = engine.Context()
    yield c
    c.close()


def _run(ctx, sc, steps, body_ids=None, shape_ids=None):
    engine.setup_scene(sc)
    gw = ctx.world(sc)
    ow = O.OracleWorld(sc)
    gw.set_events(True, body_ids, shape_ids)
    ow.set_events(True, body_ids, shape_ids)
    counts = np.zeros(5, np.int64)
    for s in range(steps):
        gw.step(nsteps=1)
        ow.step(nsteps=1)
        ge, oe = gw.events(), ow.events()
        assert len(ge) == len(oe) and ge.tobytes() == oe.tobytes(), f"{sc.name}: events of step {s + 1} differ"
        for t in range(5):
            counts[t] += int((ge["type"] == t).sum())
    gw.destroy()
    return counts


@pytest.mark.parametrize("name", ["kinematic_trigger", "sleep_wake", "filters", "materials", "grid_spheres"])
def test_event_sequences_match_the_oracle(ctx, name):
    counts = _run(ctx, edge_scene(name), 60)
    assert counts[0] > 0 and counts[1] > 0


def test_event_order_follows_the_given_ids(ctx):
    """Body and shape ids in reverse index order: the overlap keys, and so
    the order of begin / end events within a step, follow the ids."""
    sc = scenes.column_world(40, 31, "mixed")
    nb, ns = sc.num_bodies, len(sc.shapes)
    counts = _run(ctx, sc, 50, body_ids=np.arange(nb)[::-1] + 100, shape_ids=np.arange(ns)[::-1] + 7)
    assert counts[1] > 5


def test_events_on_the_wide_path(ctx):
    ctx.set_wide_bodies(1)
    try:
        counts = _run(ctx, edge_scene("kinematic_trigger"), 40)
    finally:
        ctx.set_wide_bodies(1024)
    assert counts[1] > 0


def test_feed_off_records_nothing(ctx):
    sc = engine.setup_scene(scenes.spheres_on_plane(10))
    w = ctx.world(sc)
    w.step(nsteps=30)
    assert len(w.events()) == 0
    w.set_events(True)
    w.step(nsteps=30)
    assert len(w.events()) > 0
    w.set_events(False)
    w.step(nsteps=5)
    assert len(w.events()) == 0
    w.destroy()
