"""The binary32 filters in the regimes where their error bounds are tightest.

The narrowphase settles most pairs with binary32 arithmetic and a margin:
no-contact certificates for sphere-plane, sphere-box and plane-hull pairs,
and a bound on findSeparatingAxis (convex_polyhedron.dart:232-356) that
leaves out the axes that can neither separate the hulls nor be the first
minimum.  These scenes put hull pairs where those margins are thinnest:
thousands of metres from the origin, long thin boxes (aspect 50:1), boxes
meeting edge to face at 45 degrees so that a face axis and an edge axis tie,
and box pairs turned against each other by angles that bring edge cross
products next to the filter's near-parallel cut (0.05) and the reference's
almostZero cut (1e-6).  Each runs on the GPU against the oracle, bit for bit,
with the filter check on: every filtered decision is also taken the
unfiltered way, and the two must agree on every pair.
"""
import math

import numpy as np
import pytest

from cannon_physics_gb300 import _abi as A
from cannon_physics_gb300 import engine, scenes
from oracle import oracle_py as O

from tests.parity import compare_step

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from cannon_physics_gb300 import build as B
    B.build()
    c = engine.Context()
    c.set_filter_check(True)
    yield c
    c.set_filter_check(False)
    c.close()


def _quat_axis(axis, angle):
    ax = np.asarray(axis, np.float64)
    ax = ax / np.linalg.norm(ax)
    s = math.sin(angle / 2)
    return (ax[0] * s, ax[1] * s, ax[2] * s, math.cos(angle / 2))


def _boxes(name, he, pos, quat, **kw):
    n = len(pos)
    shapes = A.default_shapes(n + 1)
    bodies = A.default_bodies(n + 1)
    scenes._plane_body(bodies, shapes, 0, 0)
    for i in range(n):
        shapes[i + 1]["type"] = A.SHAPE_BOX
        shapes[i + 1]["half_extents"] = he[i]
        h = np.asarray(he[i], np.float64)
        bodies[i + 1]["mass"] = 8.0 * h[0] * h[1] * h[2]
        bodies[i + 1]["position"] = pos[i]
        bodies[i + 1]["quaternion"] = quat[i]
        bodies[i + 1]["shape"] = i + 1
    return scenes.Scene(name, shapes, bodies, **kw)


def far_from_origin():
    """A 4 x 4 x 3 box pile and loose spheres 5 km from the origin."""
    sc = scenes.box_pile(4, 4, 3, seed=21)
    sc.bodies["position"][1:, 0] += 3000.0
    sc.bodies["position"][1:, 2] -= 4000.0
    sc.name = "far_from_origin"
    return sc


def thin_boxes():
    """Rods of half extents (0.01, 0.5, 0.01) dropped across each other."""
    rng = scenes.SplitMix64(22)
    n = 36
    u = rng.uniform(4 * n).reshape(n, 4)
    pos = [((i % 6 - 2.5) * 0.35, 0.6 + 0.3 * (i // 6), ((i // 6) % 2 - 0.5) * 0.2 + 0.05 * u[i, 0]) for i in range(n)]
    quat = [scenes.shoemake(u[i:i + 1, 1], u[i:i + 1, 2], u[i:i + 1, 3])[0] for i in range(n)]
    he = [(0.01, 0.5, 0.01)] * n
    return _boxes("thin_boxes", he, pos, quat, friction=0.4)


def face_edge_ties():
    """Equal boxes turned 45 degrees about x or z resting edge-down on
    upright ones: the face axes of the upright box and the edge axes of the
    pair give equal depths."""
    pos, quat, he = [], [], []
    for k in range(8):
        x = (k - 3.5) * 1.6
        pos.append((x, 0.5, 0.0))
        quat.append((0.0, 0.0, 0.0, 1.0))
        he.append((0.5, 0.5, 0.5))
        pos.append((x, 1.0 + math.sqrt(0.5) + 0.002 * k, 0.0))
        quat.append(_quat_axis((1, 0, 0) if k % 2 else (0, 0, 1), math.pi / 4))
        he.append((0.5, 0.5, 0.5))
    return _boxes("face_edge_ties", he, pos, quat, iterations=20)


def near_parallel_edges():
    """Box pairs stacked with the upper box turned about y by angles around
    the two cuts on |edge x edge|: 0.05 (binary32 filter) and 1e-6
    (the reference's almostZero)."""
    angles = [0.05, 0.0501, 0.0499, 0.0505, 0.0495, 1e-6, 1.2e-6, 0.8e-6, 2e-6, 5e-7, 1e-4, 0.0]
    pos, quat, he = [], [], []
    for k, a in enumerate(angles):
        x = (k - 5.5) * 1.5
        pos.append((x, 0.4, 0.0))
        quat.append((0.0, 0.0, 0.0, 1.0))
        he.append((0.5, 0.4, 0.5))
        pos.append((x + 0.05, 1.2, 0.03))
        quat.append(_quat_axis((0, 1, 0), a))
        he.append((0.45, 0.4, 0.45))
    return _boxes("near_parallel_edges", he, pos, quat)


SCENES = {"far_from_origin": far_from_origin, "thin_boxes": thin_boxes, "face_edge_ties": face_edge_ties,
          "near_parallel_edges": near_parallel_edges}


def _run(ctx, sc, steps):
    engine.setup_scene(sc)
    gw = ctx.world(sc)
    ow = O.OracleWorld(sc)
    ctx.filter_check_counts(reset=True)
    for s in range(steps):
        gw.step(nsteps=1)
        ow.step(nsteps=1)
        errs = compare_step(gw, ow)
        assert not errs, f"{sc.name}: mismatch after step {s + 1}:\n" + "\n".join(errs[:10])
    checked, disagreed = ctx.filter_check_counts(reset=True)
    gw.destroy()
    return checked, disagreed


@pytest.mark.parametrize("name", sorted(SCENES))
def test_filters_agree_with_binary64_on_the_gpu(ctx, name):
    checked, disagreed = _run(ctx, SCENES[name](), 40)
    assert checked > 0
    assert disagreed == 0


@pytest.mark.parametrize("name", sorted(SCENES))
def test_filters_agree_on_the_wide_path(ctx, name):
    ctx.set_wide_bodies(1)
    try:
        checked, disagreed = _run(ctx, SCENES[name](), 20)
    finally:
        ctx.set_wide_bodies(1024)
    assert checked > 0
    assert disagreed == 0
