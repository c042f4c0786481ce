"""Compound bodies: a body with several shapes (Body.addShape with an offset
and an orientation, lib/objects/rigid_body.dart:348-369).

The reference's narrowphase runs every shape of a pair's first body against
every shape of its second (getContacts, narrow_phase.dart:654-721), each
shape at body position + body quaternion * offset and body quaternion *
orientation; the body's AABB is the first shape's world AABB extended by the
others' (rigid_body.dart:415-447) and its bounding radius the largest offset
length + shape radius (:395-412).  The GPU runs those shape pairs as
narrowphase jobs listed after the broadphase (pair-major, first body's shape
outer) and must give the oracle's contacts, rows and bodies bit for bit
through all three broadphases, on the one-block and the grid-wide paths,
with the event feed, and with friction reduction.
"""
import numpy as np
import pytest

from cannon_physics_gb300 import _abi as A
from cannon_physics_gb300 import engine, scenes
from oracle import oracle_py as O

from tests.parity import compare_step

BROADPHASES = {"naive": A.BROAD_NAIVE, "sap": A.BROAD_SAP, "grid": A.BROAD_GRID}


def test_oracle_compound_contacts_come_from_every_shape_pair():
    """In the oracle, a body pair of two compound bodies makes contacts from
    several of its shape pairs, the contacts of one pair stay together in
    shape-loop order, and the dynamic bodies' AABBs cover all their shapes."""
    sc = O.setup_scene(scenes.compound_pile(20, seed=5, kinematic=False))
    ow = O.OracleWorld(sc)
    multi = False
    for _ in range(70):
        ow.step(sc.dt, 1)
        ct = ow.contacts()
        for p in np.unique(ct["pair"]):
            sel = ct[ct["pair"] == p]
            if len(np.unique(np.stack([sel["si"], sel["sj"]], 1), axis=0)) > 1:
                multi = True
            # one pair's contacts are consecutive
            idx = np.flatnonzero(ct["pair"] == p)
            assert idx[-1] - idx[0] + 1 == len(idx)
    assert multi
    b = ow.bodies()
    ext = sc.bodies["extra_shapes_count"] > 0
    assert ext.sum() >= 10
    assert np.all(b["aabb_upper"][ext] >= b["aabb_lower"][ext])


def test_oracle_compound_pile_settles():
    """The pile comes to rest on the plane (no body falls through, none flies off)."""
    sc = O.setup_scene(scenes.compound_pile(20, seed=6, kinematic=False))
    ow = O.OracleWorld(sc)
    ow.step(sc.dt, 240)
    b = ow.bodies()
    assert np.all(b["position"][1:, 1] > -0.05)
    assert np.all(np.abs(b["velocity"][1:]) < 2.0)


# ---------------------------------------------------------------------------
# GPU parity


@pytest.fixture(scope="module")
def ctx():
    from cannon_physics_gb300 import build as B
    B.build()
    c = engine.Context()
    yield c
    c.close()


def _parity(ctx, sc, steps, events=False):
    engine.setup_scene(sc)
    gw = ctx.world(sc)
    ow = O.OracleWorld(sc)
    if events:
        gw.set_events(True)
        ow.set_events(True)
    n_events = 0
    for s in range(steps):
        gw.step(nsteps=1)
        ow.step(nsteps=1)
        errs = compare_step(gw, ow)
        assert not errs, f"{sc.name}: mismatch after step {s + 1}:\n" + "\n".join(errs[:10])
        if events:
            ge, oe = gw.events(), ow.events()
            assert len(ge) == len(oe) and ge.tobytes() == oe.tobytes(), f"events of step {s + 1} differ"
            n_events += len(ge)
    info = gw.info()
    gw.destroy()
    return info, n_events


@pytest.mark.gpu
@pytest.mark.parametrize("bp", sorted(BROADPHASES))
def test_compound_pile_matches_oracle(ctx, bp):
    _parity(ctx, scenes.compound_pile(30, seed=7, broadphase=BROADPHASES[bp]), 90)


@pytest.mark.gpu
@pytest.mark.parametrize("bp", sorted(BROADPHASES))
def test_compound_pile_wide_path_matches_oracle(ctx, bp):
    ctx.set_wide_bodies(1)
    try:
        _parity(ctx, scenes.compound_pile(30, seed=8, broadphase=BROADPHASES[bp]), 60)
    finally:
        ctx.set_wide_bodies(1024)


@pytest.mark.gpu
def test_compound_events_match_oracle(ctx):
    """A kinematic compound body sweeps through the pile: its shape pairs
    with static shapes take the justTest path, and the shape-pair events name
    the compound body's second and third shapes."""
    _, n = _parity(ctx, scenes.compound_pile(25, seed=9), 120, events=True)
    assert n > 0


@pytest.mark.gpu
def test_compound_friction_reduction_matches_oracle(ctx):
    sc = scenes.compound_pile(25, seed=10)
    sc.enable_friction_reduction = True
    _parity(ctx, sc, 80)


@pytest.mark.gpu
def test_compound_job_list_grows(ctx):
    """Tables (five shapes, 25 shape pairs per table pair) packed closely:
    their shape pairs outnumber the first job list (four per first-list
    pair), the step overflows it, the list grows and the step runs again,
    matching the oracle."""
    sc = scenes.compound_pile(40, seed=11, per_row=4, pitch=0.8, kinds=(2,))
    info, _ = _parity(ctx, sc, 40)
    assert info.num_pairs > 0
