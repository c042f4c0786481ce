"""World.solver = SplitSolver(GSSolver) (lib/solver/split_solver.dart).

The SplitSolver cuts the equations into islands of non-static bodies and
solves each with the GSSolver on its own, its equations sorted by
Equation.id, highest first, with its own convergence test.  The order
therefore depends on the reference's equation ids, which come from a global
counter and from the narrowphase's last-in-first-out pools of contact and
friction equation objects (lib/world/world_class.dart:506-527,
narrow_phase.dart:492-586).  CPU tests check the oracle's id bookkeeping;
GPU tests compare every row (with its id), every body and the iteration
count with the oracle, step by step, on the one-block and batched paths.
"""
import numpy as np
import pytest

from cannon_physics_gb300 import _abi as A
from cannon_physics_gb300 import engine, scenes
from oracle import oracle_py as O

from tests.parity import compare_step


def _split(make):
    return scenes.use_split_solver(make())


SCENES = {
    "chains": lambda: scenes.mixed_chains(8, 4, 4, seed=3, chains=4, chain_len=8),
    "column": lambda: scenes.column_world(120, 77, "mixed"),
    "joints": scenes.joints_and_hulls,
    "compound": lambda: scenes.compound_pile(20, seed=14),
    "spheres": lambda: scenes.spheres_on_plane(40, seed=8),
}


def test_oracle_equation_ids_follow_the_pools():
    """Ids are distinct within a step and constraint ids are their
    constructors'.  spherePlane takes its equation object before its depth
    test and drops it when the sphere is clear of the plane
    (narrow_phase.dart:781-812), so while 40 spheres fall every step spends 40
    new ids; the first contacts then carry ids of the step they appear in."""
    sc = O.setup_scene(_split(SCENES["chains"]))
    ow = O.OracleWorld(sc)
    ncon = int(sc.equation_id_counter)
    for _ in range(40):
        ow.step(sc.dt, 1)
        rows = ow.rows()
        assert len(np.unique(rows["id"])) == len(rows)
        con = rows[rows["id"] < ncon]
        assert (con["kind"] != A.ROW_FRICTION).all()
    sc = O.setup_scene(_split(SCENES["spheres"]))
    n = len(sc.bodies) - 1
    ow = O.OracleWorld(sc)
    for s in range(1, 200):
        ow.step(sc.dt, 1)
        ct = ow.contacts()
        if len(ct):
            ids = ow.rows()["id"]
            assert ids.min() >= n * (s - 1) and ids.max() < n * s + 2 * len(ct)
            break
    else:
        raise AssertionError("no contact")


def test_oracle_split_islands_solve_apart():
    """Two far-apart copies of a pile settle like the copy alone.  Not bit for
    bit: the second pile's contacts take equation objects in between the
    first pile's (pairs come in body order, the plane's first), which changes
    the descending-id order inside the first pile's island."""
    one = scenes.column_world(40, 5, "sphere_box")
    two = scenes.column_world(40, 5, "sphere_box")
    n = len(one.bodies)
    # (np.concatenate would repack the padded record layouts)
    shapes = np.zeros(2 * len(one.shapes) - 1, dtype=A.SHAPE_DTYPE)
    shapes[:len(one.shapes)] = one.shapes
    shapes[len(one.shapes):] = one.shapes[1:]
    bodies = np.zeros(2 * n - 1, dtype=A.BODY_DTYPE)
    bodies[:n] = one.bodies
    bodies[n:] = one.bodies[1:]
    bodies["position"][n:, 0] += 500.0
    bodies["shape"][n:] = bodies["shape"][n:] + (len(one.shapes) - 1)
    both = scenes.Scene("two_piles", shapes, bodies, friction=one.friction, restitution=one.restitution,
                        iterations=one.iterations, broadphase=one.broadphase, dt=one.dt)
    a = O.OracleWorld(O.setup_scene(scenes.use_split_solver(two)))
    b = O.OracleWorld(O.setup_scene(scenes.use_split_solver(both)))
    for _ in range(40):
        a.step(one.dt, 1)
        b.step(one.dt, 1)
    pa, pb = a.bodies()["position"], b.bodies()["position"]
    assert np.abs(pa[1:] - pb[1:n]).max() < 0.1
    shifted = pb[n:].copy()
    shifted[:, 0] -= 500.0
    assert np.abs(shifted - pa[1:]).max() < 0.1


# ---------------------------------------------------------------------------
# GPU


@pytest.fixture(scope="module")
def ctx():
    from cannon_physics_gb300 import build as B
    B.build()
    c = engine.Context()
    yield c
    c.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(SCENES))
def test_split_solver_matches_oracle(ctx, name):
    sc = engine.setup_scene(_split(SCENES[name]))
    gw = ctx.world(sc)
    ow = O.OracleWorld(sc)
    for s in range(60):
        gw.step(nsteps=1)
        ow.step(nsteps=1)
        errs = compare_step(gw, ow)
        assert not errs, f"{name}: mismatch after step {s + 1}:\n" + "\n".join(errs[:10])
    assert (gw.rows()["id"] >= 0).all()
    gw.destroy()


@pytest.mark.gpu
@pytest.mark.parametrize("bp", [A.BROAD_SAP, A.BROAD_GRID])
def test_split_solver_broadphases(ctx, bp):
    sc = _split(lambda: scenes.compound_pile(24, seed=15, broadphase=bp))
    engine.setup_scene(sc)
    gw = ctx.world(sc)
    ow = O.OracleWorld(sc)
    for s in range(50):
        gw.step(nsteps=1)
        ow.step(nsteps=1)
        errs = compare_step(gw, ow)
        assert not errs, f"mismatch after step {s + 1}:\n" + "\n".join(errs[:10])
    gw.destroy()


@pytest.mark.gpu
def test_split_and_gs_worlds_in_one_batch(ctx):
    """SplitSolver worlds finish their step in the pre-step kernel; GSSolver
    worlds of the same batch go on to the solve kernel; both equal the oracle."""
    scs = []
    for k in range(8):
        sc = scenes.column_world(40 + 20 * k, 300 + k, "mixed")
        if k % 2 == 0:
            scenes.use_split_solver(sc)
        scs.append(engine.setup_scene(sc))
    gws = [ctx.world(sc) for sc in scs]
    ows = [O.OracleWorld(sc) for sc in scs]
    for _ in range(5):
        ctx.batch_step(gws, scs[0].dt, 8)
        for k, (gw, ow) in enumerate(zip(gws, ows)):
            ow.step(nsteps=8)
            errs = compare_step(gw, ow, check_lists=False)
            assert not errs, f"world {k}:\n" + "\n".join(errs[:10])
    for gw in gws:
        gw.destroy()


@pytest.mark.gpu
def test_split_pools_survive_list_growth(ctx):
    """A pile whose contact list outgrows its first capacity: the pools move
    to the larger allocation with their ids, and the ids stay the oracle's."""
    sc = _split(lambda: scenes.box_pile(6, 6, 3, seed=9))
    engine.setup_scene(sc)
    gw = ctx.world(sc)
    ow = O.OracleWorld(sc)
    for s in range(40):
        gw.step(nsteps=1)
        ow.step(nsteps=1)
        errs = compare_step(gw, ow)
        assert not errs, f"mismatch after step {s + 1}:\n" + "\n".join(errs[:10])
    gw.destroy()
