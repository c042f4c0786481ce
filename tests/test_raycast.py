"""World.raycastClosest / raycastAny / raycastAll over the resident state
(lib/world/world_class.dart:248-278, lib/collision/ray_class.dart).

CPU: the oracle's restatement against properties the reference's Ray has
(a sphere hit lies on the sphere and its normal points out of it; the
closest hit is the nearest of all hits; ANY hits exactly when CLOSEST does;
a grid world answers nothing).  GPU: every result field bit for bit against
the oracle, in all three modes, through all three broadphases, on compound
bodies, with collision filters, collisionResponse off and back faces
skipped or not; then the world keeps stepping in lockstep with the oracle,
since a raycast refreshes AABBs and re-sorts a SAP axis list as the
reference's aabbQuery does.
"""
import numpy as np
import pytest

from cannon_physics_gb300 import _abi as A
from cannon_physics_gb300 import engine, scenes
from oracle import oracle_py as O

from tests.parity import compare_step


def _rays(seed, n, lo, hi, down=True):
    rng = np.random.default_rng(seed)
    fr = np.column_stack([rng.uniform(lo[0], hi[0], n), rng.uniform(lo[1], hi[1], n), rng.uniform(lo[2], hi[2], n)])
    if down:
        to = fr + np.column_stack([rng.uniform(-2, 2, n), np.full(n, -(hi[1] - lo[1]) - 3.0), rng.uniform(-2, 2, n)])
    else:
        to = np.column_stack([rng.uniform(lo[0], hi[0], n), rng.uniform(lo[1], hi[1], n), rng.uniform(lo[2], hi[2], n)])
    return fr.astype(np.float32), to.astype(np.float32)


def _scene(kind, bp=A.BROAD_NAIVE):
    if kind == "column":
        sc = scenes.column_world(120, 77, "mixed")
        sc.broadphase = bp
        return sc
    if kind == "compound":
        return scenes.compound_pile(20, seed=13, broadphase=bp)
    return scenes.joints_and_hulls(broadphase=bp)


def _bounds(sc):
    p = sc.bodies["position"][1:]
    return p.min(axis=0) - 1.0, p.max(axis=0) + 1.5


# ---------------------------------------------------------------------------
# CPU: the oracle's restatement


def test_oracle_sphere_hits_lie_on_the_sphere():
    sc = O.setup_scene(scenes.spheres_on_plane(30, seed=4))
    ow = O.OracleWorld(sc)
    ow.step(sc.dt, 20)
    b = ow.bodies()
    lo, hi = _bounds(sc)
    fr, to = _rays(5, 400, lo, hi)
    h = ow.raycast(A.rays(fr, to), A.RAY_CLOSEST)
    hit_sphere = (h["has_hit"] == 1) & (h["body"] > 0)
    assert hit_sphere.sum() > 10
    r = sc.shapes["radius"][1]
    for k in np.flatnonzero(hit_sphere):
        c = b["position"][h["body"][k]].astype(np.float64)
        p = h["hit_point"][k].astype(np.float64)
        assert abs(np.linalg.norm(p - c) - r) < 1e-5
        assert np.dot(h["hit_normal"][k], p - c) > 0
    # a ray that starts above and ends below the plane always hits something
    assert h["has_hit"].all()


@pytest.mark.parametrize("kind", ["column", "compound"])
def test_oracle_closest_any_all_agree(kind):
    sc = O.setup_scene(_scene(kind))
    ow = O.OracleWorld(sc)
    ow.step(sc.dt, 30)
    lo, hi = _bounds(sc)
    fr, to = _rays(6, 300, lo, hi, down=False)
    rays = A.rays(fr, to, skip_backfaces=False)
    c = ow.raycast(rays, A.RAY_CLOSEST)
    a = ow.raycast(rays, A.RAY_ANY)
    hits, counts = ow.raycast(rays, A.RAY_ALL, 64)
    assert (counts <= 64).all()
    assert np.array_equal(c["has_hit"], a["has_hit"])
    assert np.array_equal(c["has_hit"], (counts > 0).astype(np.int32))
    for k in np.flatnonzero(counts):
        d = hits["distance"][k, :counts[k]]
        assert c["distance"][k] == d.min()
        # ANY reports the first hit of ALL
        assert a["distance"][k] == hits["distance"][k, 0]


def test_oracle_grid_world_answers_nothing():
    sc = O.setup_scene(scenes.compound_pile(12, seed=3, broadphase=A.BROAD_GRID))
    ow = O.OracleWorld(sc)
    ow.step(sc.dt, 5)
    fr, to = _rays(7, 50, *_bounds(sc))
    assert ow.raycast(A.rays(fr, to), A.RAY_CLOSEST)["has_hit"].sum() == 0


# ---------------------------------------------------------------------------
# GPU against the oracle


@pytest.fixture(scope="module")
def ctx():
    from cannon_physics_gb300 import build as B
    B.build()
    c = engine.Context()
    yield c
    c.close()


def _cmp(g, o, what):
    assert g.dtype == o.dtype
    bad = [f for f in g.dtype.names if g[f].tobytes() != o[f].tobytes()]
    if bad:
        f = bad[0]
        i = np.flatnonzero((g[f] != o[f]).reshape(len(g), -1).any(axis=1))[0]
        raise AssertionError(f"{what}: field {f} differs first at ray {i}: gpu {g[i]} oracle {o[i]}")


def _cast_and_compare(gw, ow, rays, max_hits=12):
    for mode in (A.RAY_CLOSEST, A.RAY_ANY):
        _cmp(gw.raycast(rays, mode), ow.raycast(rays, mode), f"mode {mode}")
    gh, gc = gw.raycast(rays, A.RAY_ALL, max_hits)
    oh, oc = ow.raycast(rays, A.RAY_ALL, max_hits)
    assert np.array_equal(gc, oc), "RAY_ALL hit counts differ"
    for k in range(len(rays)):
        m = min(gc[k], max_hits)
        if m:
            _cmp(gh[k, :m], oh[k, :m], f"RAY_ALL ray {k}")
    return gc


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["column", "compound", "joints"])
@pytest.mark.parametrize("bp", [A.BROAD_NAIVE, A.BROAD_SAP, A.BROAD_GRID])
def test_raycasts_match_oracle(ctx, kind, bp):
    sc = engine.setup_scene(_scene(kind, bp))
    gw = ctx.world(sc)
    ow = O.OracleWorld(sc)
    lo, hi = _bounds(sc)
    total = 0
    for rnd in range(4):
        gw.step(nsteps=10)
        ow.step(nsteps=10)
        fr, to = _rays(100 + rnd, 256, lo, hi, down=rnd % 2 == 0)
        variants = [A.rays(fr, to), A.rays(fr, to, skip_backfaces=False),
                    A.rays(fr, to, group=2, mask=1), A.rays(fr, to, check_collision_response=False)]
        for rays in variants:
            total += int(_cast_and_compare(gw, ow, rays).sum())
        # the raycast refreshed AABBs (and the SAP list) as the reference's
        # aabbQuery does: bodies, then the following steps, still agree
        errs = compare_step(gw, ow)
        assert not errs, "\n".join(errs[:10])
        assert np.array_equal(gw.bodies()["aabb_needs_update"], ow.bodies()["aabb_needs_update"])
    if bp == A.BROAD_GRID:
        assert total == 0
    else:
        assert total > 100
    gw.destroy()


@pytest.mark.gpu
def test_raycast_on_the_wide_path(ctx):
    """A world stepped by the grid-wide kernels answers the same rays."""
    ctx.set_wide_bodies(1)
    try:
        sc = engine.setup_scene(_scene("column", A.BROAD_SAP))
        gw = ctx.world(sc)
        ow = O.OracleWorld(sc)
        gw.step(nsteps=25)
        ow.step(nsteps=25)
        fr, to = _rays(9, 512, *_bounds(sc))
        _cast_and_compare(gw, ow, A.rays(fr, to))
        gw.step(nsteps=5)
        ow.step(nsteps=5)
        assert not compare_step(gw, ow)
        gw.destroy()
    finally:
        ctx.set_wide_bodies(1024)
