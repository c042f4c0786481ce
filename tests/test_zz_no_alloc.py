"""cp_world_step_static (the step with the static step scratch) against
cp_world_step.

Each scene is created twice; one copy is stepped with cp_world_step, the
other with cp_world_step_static, over two calls in a row.  After each call
the body records must be byte-identical, the tolerance every parity test
here uses, and so must the last step's pairs, contacts, solver rows and step
info that the getters return.  The file runs last so that it also covers a process in which
the other tests have already used the library; it creates its own context,
so it passes alone in a fresh process too.
"""
import ctypes as C

import pytest

from cannon_physics_gb300 import _abi as A
from cannon_physics_gb300 import engine, scenes

from tests.parity import CONTACT_FIELDS, ROW_FIELDS, diff_records

pytestmark = pytest.mark.gpu


def _lib():
    L = engine.lib()
    L.cp_world_step_static.argtypes = [C.c_void_p, C.c_int32, C.c_double, C.c_int32]
    return L


@pytest.fixture(scope="module")
def ctx():
    c = engine.Context(device=0)
    yield c
    c.close()


SCENES = [
    ("spheres_on_plane", lambda: scenes.spheres_on_plane(), 0),
    ("box_pile", lambda: scenes.box_pile(6, 6, 3), 0),
    ("mixed_column", lambda: scenes.column_world(300, 11, "mixed"), 0),
    # a GridBroadphase world with constraints and sleeping; both copies first
    # take 12 steps through cp_world_step, which grows the capacities its
    # first steps overflow (the static step never grows them)
    ("grid_chains", lambda: scenes.mixed_chains(8, 8, 4, seed=5, chains=4, chain_len=8), 12),
]


def _same_lists(ref, sta, what):
    errs = []
    rp, sp = ref.pairs(), sta.pairs()
    if not (len(rp[0]) == len(sp[0]) and (rp[0] == sp[0]).all() and (rp[1] == sp[1]).all()):
        errs.append(f"pairs differ: {len(rp[0])} vs {len(sp[0])}")
    errs += diff_records(ref.contacts(), sta.contacts(), CONTACT_FIELDS, "contacts")
    errs += diff_records(ref.rows(), sta.rows(), ROW_FIELDS, "rows")
    ri, si = ref.info(), sta.info()
    for f in ("stepnumber", "time", "num_pairs", "num_contacts", "num_rows", "iterations", "status", "num_levels"):
        if getattr(ri, f) != getattr(si, f):
            errs.append(f"info.{f}: {getattr(ri, f)} vs {getattr(si, f)}")
    assert not errs, f"{what}:\n" + "\n".join(errs[:10])


@pytest.mark.parametrize("name,make,grow", SCENES, ids=[n for n, _, _ in SCENES])
def test_static_step_matches_world_step(ctx, name, make, grow):
    sc = engine.setup_scene(make())
    ref = ctx.world(sc)
    sta = ctx.world(sc)
    if grow:
        ref.step(sc.dt, grow)
        sta.step(sc.dt, grow)
    L = _lib()
    for call in range(2):
        ref.step(sc.dt, 6)
        st = L.cp_world_step_static(ctx.h, sta.id, sc.dt, 6)
        assert st == A.CP_OK, L.cp_last_error().decode()
        assert ref.bodies().tobytes() == sta.bodies().tobytes(), f"{name}: call {call}"
        _same_lists(ref, sta, f"{name}: call {call}")
        assert sta.info().num_pairs > 0
    ref.destroy()
    sta.destroy()


def test_static_step_reports_overflow(ctx):
    """A grid world whose first step overflows its initial bin capacity: the
    static step cannot grow it, so it returns CP_ERR_CAPACITY, leaves the
    bodies as they were and clears the world's status; cp_world_step then
    takes the step, growing the capacity, exactly as it does for a world that
    was never given to the static step."""
    sc = engine.setup_scene(scenes.mixed_chains(8, 8, 4, seed=5, chains=4, chain_len=8))
    ref = ctx.world(sc)
    sta = ctx.world(sc)
    L = _lib()
    dynamic = ["position", "quaternion", "velocity", "angular_velocity", "force", "torque", "sleep_state"]
    before = [sta.bodies()[f].tobytes() for f in dynamic]
    st = L.cp_world_step_static(ctx.h, sta.id, sc.dt, 6)
    assert st == A.CP_ERR_CAPACITY, L.cp_last_error().decode()
    assert "overflowed" in L.cp_last_error().decode()
    # only the cached AABBs may have been refreshed
    after = sta.bodies()
    assert [after[f].tobytes() for f in dynamic] == before
    assert sta.info().stepnumber == 0
    assert sta.info().status == 0
    # the failed step's partial lists are not reported
    assert (sta.info().num_pairs, sta.info().num_contacts, sta.info().num_rows) == (0, 0, 0)
    assert len(sta.pairs()[0]) == 0 and len(sta.contacts()) == 0 and len(sta.rows()) == 0
    ref.step(sc.dt, 6)
    sta.step(sc.dt, 6)
    assert ref.bodies().tobytes() == sta.bodies().tobytes()
    ref.destroy()
    sta.destroy()


def test_static_step_rejects_worlds_beyond_its_size(ctx):
    sc = engine.setup_scene(scenes.spheres_on_plane(12000))
    w = ctx.world(sc)
    before = w.bodies().tobytes()
    L = _lib()
    st = L.cp_world_step_static(ctx.h, w.id, sc.dt, 1)
    assert st == A.CP_ERR_CAPACITY
    assert "static scratch" in L.cp_last_error().decode()
    assert w.bodies().tobytes() == before  # nothing ran
    w.destroy()
