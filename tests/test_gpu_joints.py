"""LockConstraint, ConeTwistConstraint and SpringConstraint, and the
ConvexPolyhedron subclasses with their own ShapeType (Capsule, Cone,
SizedPlane), on the GPU against the oracle, bit for bit.

Lock (lock_constraint.dart) keeps a point-to-point triple and three
rotational rows on the local frames its constructor stored; ConeTwist
(cone_twist_constraint.dart) adds a cone row (ConeEquation) and a twist row
on the second tangents of the local axes, both pushing one way
([-maxForce, 0]); Spring (spring_constraint.dart) is a contact row along the
bodies' centre line bounded by the stiffness.  The shapes take the convex
resolvers through the reference's resolver table, whose convex + sizedPlane
entry is never found (the scene drops pyramids through SizedPlane tiles).
"""
import pytest

from cannon_physics_gb300 import _abi as A
from cannon_physics_gb300 import engine, scenes
from oracle import oracle_py as O

from tests.parity import compare_step

pytestmark = pytest.mark.gpu

BROADPHASES = {"naive": A.BROAD_NAIVE, "sap": A.BROAD_SAP, "grid": A.BROAD_GRID}


@pytest.fixture(scope="module")
def ctx():
    from cannon_physics_gb300 import build as B
    B.build()
    c = engine.Context()
    yield c
    c.close()


def _parity(ctx, sc, steps):
    engine.setup_scene(sc)
    gw = ctx.world(sc)
    ow = O.OracleWorld(sc)
    kinds = set()
    for s in range(steps):
        gw.step(nsteps=1)
        ow.step(nsteps=1)
        errs = compare_step(gw, ow)
        assert not errs, f"{sc.name}: mismatch after step {s + 1}:\n" + "\n".join(errs[:10])
        ct = gw.contacts()
        kinds |= {(int(sc.shapes["type"][a]), int(sc.shapes["type"][b])) for a, b in zip(ct["si"], ct["sj"])}
    gw.destroy()
    return kinds


@pytest.mark.parametrize("bp", sorted(BROADPHASES))
def test_joints_and_hulls_match_oracle(ctx, bp):
    kinds = _parity(ctx, scenes.joints_and_hulls(broadphase=BROADPHASES[bp]), 150)
    # sized planes, cones and capsules all touched something
    flat = {t for k in kinds for t in k}
    assert {A.SHAPE_CAPSULE, A.SHAPE_CONE, A.SHAPE_SIZED_PLANE} <= flat


def test_joints_and_hulls_wide_path(ctx):
    ctx.set_wide_bodies(1)
    try:
        _parity(ctx, scenes.joints_and_hulls(n_chains=6, seed=43), 100)
    finally:
        ctx.set_wide_bodies(1024)


def test_joints_in_a_batch(ctx):
    """Worlds with the new joints and hulls stepped together by the batched
    kernels equal the oracle world by world."""
    scs = [engine.setup_scene(scenes.joints_and_hulls(n_chains=2 + k % 3, seed=50 + k)) for k in range(6)]
    gws = [ctx.world(sc) for sc in scs]
    ows = [O.OracleWorld(sc) for sc in scs]
    for _ in range(4):
        ctx.batch_step(gws, scs[0].dt, 10)
        for k, (gw, ow) in enumerate(zip(gws, ows)):
            ow.step(nsteps=10)
            errs = compare_step(gw, ow, check_lists=False)
            assert not errs, f"world {k}:\n" + "\n".join(errs[:10])
    for gw in gws:
        gw.destroy()
