"""Known-answer tests that pin the CPU oracle (no GPU).

The reference ships no tests or golden vectors, so the oracle is pinned by
restating the arithmetic of simple situations independently (numpy binary64
with binary32 stores) and by physical invariants.
"""
import math

import numpy as np
import pytest

from cannon_physics_gb300 import _abi as A
from cannon_physics_gb300 import scenes
from oracle import oracle_py as O

f32 = np.float32


def one_body_scene(shape_type=A.SHAPE_SPHERE, mass=1.0, pos=(0.0, 10.0, 0.0), vel=(0.0, 0.0, 0.0), gravity=(0.0, -9.82, 0.0), plane=False):
    n = 2 if plane else 1
    shapes = A.default_shapes(2)
    bodies = A.default_bodies(n)
    shapes[0]["type"] = shape_type
    shapes[0]["radius"] = 0.5
    shapes[0]["half_extents"] = (0.5, 0.5, 0.5)
    bodies[0]["mass"] = mass
    bodies[0]["position"] = pos
    bodies[0]["velocity"] = vel
    bodies[0]["shape"] = 0
    if plane:
        shapes[1]["type"] = A.SHAPE_PLANE
        bodies[1]["mass"] = 0.0
        bodies[1]["quaternion"] = scenes.euler_xyz(-math.pi / 2, 0, 0)
        bodies[1]["shape"] = 1
    sc = scenes.Scene("one", shapes, bodies, gravity=gravity, dt=1 / 60)
    return O.setup_scene(sc)


def test_free_fall_matches_closed_recurrence():
    """Body.integrate + damping + gravity (world_class.dart:460-471,648-673,
    rigid_body.dart:627-680) restated with numpy, one body, no contacts."""
    sc = one_body_scene(pos=(0.0, 100.0, 0.0))
    w = O.OracleWorld(sc)
    dt = 1 / 60
    g = float(f32(-9.82))
    ld = math.pow(1.0 - 0.01, dt)
    y, vy, fy = f32(100.0), f32(0.0), f32(0.0)
    for step in range(50):
        w.step(dt)
        fy = f32(float(fy) + 1.0 * g)                     # gravity add
        vy = f32(ld * float(vy))                          # damping
        vy = f32(float(vy) + float(fy) * (1.0 * dt) * 1.0)  # v += f * iMdt * linearFactor
        y = f32(float(y) + float(vy) * dt)                # x += v * dt
        fy = f32(0.0)                                     # clearForces
        b = w.bodies()
        assert b["position"][0, 1] == y
        assert b["velocity"][0, 1] == vy
    assert b["position"][0, 0] == 0.0 and b["position"][0, 2] == 0.0


def test_sphere_comes_to_rest_on_plane():
    sc = one_body_scene(pos=(0.0, 2.0, 0.0), plane=True)
    w = O.OracleWorld(sc)
    w.step(nsteps=300)
    b = w.bodies()
    assert abs(b["position"][0, 1] - 0.5) < 1e-3
    assert np.abs(b["velocity"][0]).max() < 1e-3
    assert w.info().num_contacts == 1
    rows = w.rows()
    # friction rows come first (world_class.dart:539-541), then the contact row
    assert list(rows["kind"]) == [A.ROW_FRICTION, A.ROW_FRICTION, A.ROW_CONTACT]
    # the contact multiplier carries the weight: lambda / dt ~ m g
    assert abs(rows["multiplier"][2] - 9.82) < 0.05


def test_box_rests_flat_with_four_symmetric_contacts():
    sc = one_body_scene(shape_type=A.SHAPE_BOX, pos=(0.0, 0.5, 0.0), plane=True)
    w = O.OracleWorld(sc)
    w.step(nsteps=120)
    c = w.contacts()
    assert len(c) == 4
    b = w.bodies()
    assert abs(b["position"][0, 1] - 0.5) < 2e-3
    rows = w.rows()
    lam = rows["multiplier"][rows["kind"] == A.ROW_CONTACT]
    assert abs(lam.sum() - 9.82) < 0.1


def test_head_on_spheres_conserve_momentum():
    shapes = A.default_shapes(1)
    shapes[0]["type"] = A.SHAPE_SPHERE
    shapes[0]["radius"] = 0.5
    bodies = A.default_bodies(2)
    bodies["mass"] = (1.0, 2.0)
    bodies["position"] = [(-1.0, 0, 0), (1.0, 0, 0)]
    bodies["velocity"] = [(3.0, 0, 0), (-1.0, 0, 0)]
    bodies["linear_damping"] = 0.0
    bodies["shape"] = 0
    sc = O.setup_scene(scenes.Scene("hit", shapes, bodies, gravity=(0, 0, 0), restitution=0.0))
    w = O.OracleWorld(sc)
    p0 = 1.0 * 3.0 + 2.0 * -1.0
    for _ in range(60):
        w.step()
    b = w.bodies()
    p1 = (b["mass"] * b["velocity"][:, 0]).sum()
    assert abs(p1 - p0) < 1e-4
    assert b["position"][1, 0] - b["position"][0, 0] >= 1.0 - 1e-2  # no interpenetration left


def _rotate(q, v):
    x, y, z, w = (float(c) for c in q)
    u = np.array([x, y, z])
    return v + 2.0 * np.cross(u, np.cross(u, v) + w * v)


def _pendulum(ctype):
    shapes = A.default_shapes(1)
    shapes[0]["radius"] = 0.25
    bodies = A.default_bodies(2)
    bodies["mass"] = (0.0, 1.0)
    bodies["position"] = [(0.0, 5.0, 0.0), (1.0, 5.0, 0.0)]
    bodies["shape"] = (-1, 0)
    cons = np.zeros(1, dtype=A.CONSTRAINT_DTYPE)
    cons["type"] = ctype
    cons["body_a"], cons["body_b"] = 0, 1
    cons["collide_connected"] = 1
    cons["pivot_a"] = (0.5, 0.0, 0.0)
    cons["pivot_b"] = (-0.5, 0.0, 0.0)
    cons["axis_a"] = (0.0, 0.0, 1.0)
    cons["axis_b"] = (0.0, 0.0, 1.0)
    cons["distance"] = -1.0
    cons["max_force"] = 1e6
    cons["spook_stiffness"], cons["spook_relaxation"], cons["spook_time_step"] = 1e7, 4.0, 1 / 60
    sc = O.setup_scene(scenes.Scene("pendulum", shapes, bodies, constraints=cons, dt=1 / 60))
    return sc


@pytest.mark.parametrize("ctype", [A.CON_P2P, A.CON_HINGE, A.CON_DISTANCE])
def test_pendulum_joint_holds(ctype):
    """A body hanging from a static anchor by PointToPoint / Hinge / Distance
    (point_to_point_constraint.dart, hinge_constraint.dart,
    distance_constraint.dart) swings down and keeps its joint."""
    sc = _pendulum(ctype)
    w = O.OracleWorld(sc)
    ymin = 10.0
    for _ in range(120):
        w.step()
        b = w.bodies()
        ymin = min(ymin, float(b["position"][1, 1]))
        pa, pb = b["position"][0].astype(np.float64), b["position"][1].astype(np.float64)
        if ctype == A.CON_DISTANCE:
            assert abs(np.linalg.norm(pa - pb) - 1.0) < 0.02
        else:
            wa = pa + _rotate(b["quaternion"][0], np.array([0.5, 0, 0]))
            wb = pb + _rotate(b["quaternion"][1], np.array([-0.5, 0, 0]))
            assert np.linalg.norm(wa - wb) < 0.02
    assert ymin < 4.6  # it swung down towards 5 - 0.5 (pivot 0.5 right of the anchor, arm 0.5)
    if ctype == A.CON_HINGE:  # rotation about z only
        q = b["quaternion"][1]
        assert abs(q[0]) < 1e-3 and abs(q[1]) < 1e-3


def test_grid_finds_the_naive_pair_set_and_sap_a_subset():
    """Grid (grid_broadphase.dart) finds the naive bounding-sphere pair set,
    except plane pairs: the plane sits only in the bins near it, while its
    infinite bounding radius pairs it with every body in the naive search.
    SAP (sap_broadphase.dart:138-166) finds a subset: it sorts by AABB lower
    bound but stops a scan on position - boundingRadius, so a later body with
    a looser sphere can be skipped; that is the reference's behaviour."""
    base = scenes.mixed_chains(8, 4, 4, chains=0)
    O.setup_scene(base)
    sets = {}
    for kind in (A.BROAD_NAIVE, A.BROAD_SAP, A.BROAD_GRID):
        sc = scenes.mixed_chains(8, 4, 4, chains=0)
        O.setup_scene(sc)
        sc.broadphase = kind
        w = O.OracleWorld(sc)
        w.step()
        p1, p2 = w.pairs()
        sets[kind] = {(min(a, b), max(a, b)) for a, b in zip(p1, p2)}
        assert len(sets[kind]) == len(p1)  # unique
    no_plane = lambda st: {p for p in st if 0 not in p}  # body 0 is the plane
    assert no_plane(sets[A.BROAD_NAIVE]) == no_plane(sets[A.BROAD_GRID])
    assert sets[A.BROAD_GRID] <= sets[A.BROAD_NAIVE]
    assert sets[A.BROAD_SAP] <= sets[A.BROAD_NAIVE]
    assert len(sets[A.BROAD_SAP]) > 0.8 * len(sets[A.BROAD_NAIVE])
    assert len(sets[A.BROAD_NAIVE]) > 10


def test_sap_order_is_stable_sorted_by_aabb_lower_x():
    sc = scenes.box_pile(4, 4, 2)
    O.setup_scene(sc)
    w = O.OracleWorld(sc)
    w.step()
    order = w.sap_order()
    lo = w.bodies()["aabb_lower"][order, 0]
    assert np.all(lo[:-1] <= lo[1:])
    assert sorted(order.tolist()) == list(range(sc.num_bodies))


def test_contacts_of_equal_shape_types_take_the_swapped_body_order():
    """For equal ShapeTypes the resolver is called with the pair swapped
    (narrow_phase.dart:706-710): sphere-sphere contacts have bi = p2."""
    shapes = A.default_shapes(1)
    shapes[0]["radius"] = 0.5
    bodies = A.default_bodies(2)
    bodies["mass"] = 1.0
    bodies["position"] = [(0.0, 0, 0), (0.9, 0, 0)]
    bodies["shape"] = 0
    sc = O.setup_scene(scenes.Scene("pair", shapes, bodies, gravity=(0, 0, 0)))
    w = O.OracleWorld(sc)
    w.step()
    p1, p2 = w.pairs()
    c = w.contacts()
    assert (p1[0], p2[0]) == (1, 0)
    assert (c["bi"][0], c["bj"][0]) == (0, 1)
    assert c["ni"][0][0] == 1.0


def test_sphere_inertia_comes_from_its_aabb():
    """updateMassProperties approximates every shape by its AABB box
    (rigid_body.dart:587-609): a sphere gets I = 2/3 m r^2, not 2/5."""
    sc = one_body_scene()
    b = sc.bodies[0]
    assert abs(1.0 / b["inv_inertia"][0] - 2.0 / 3.0 * 1.0 * 0.25) < 1e-6


def test_cylinder_hull_tables():
    shapes = A.default_shapes(1)
    shapes[0]["type"] = A.SHAPE_CYLINDER
    shapes[0]["radius_top"] = 0.5
    shapes[0]["radius_bottom"] = 0.5
    shapes[0]["height"] = 1.0
    shapes[0]["num_segments"] = 10
    v, n, e = O.shape_hull(shapes[0:1])
    assert v.shape == (20, 3) and n.shape == (12, 3)
    # +-y, and both directions of the 5 chord directions of an even 10-gon:
    # computeEdges does not merge an edge with its negation
    assert len(e) == 12
    assert np.allclose(np.linalg.norm(n, axis=1), 1.0, atol=1e-6)
