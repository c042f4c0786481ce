"""cp_world_step_static (the step with the static step scratch) against
cp_world_step.

Each scene is created twice; one copy is stepped with cp_world_step, the
other with cp_world_step_static, over two calls in a row.  After each call
the body records must be byte-identical, the tolerance every parity test
here uses.  The file runs last so that it also covers a process in which
the other tests have already used the library; it creates its own context,
so it passes alone in a fresh process too.
"""
import ctypes as C

import pytest

from cannon_physics_gb300 import _abi as A
from cannon_physics_gb300 import engine, scenes

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
    ("spheres_on_plane", lambda: scenes.spheres_on_plane()),
    ("box_pile", lambda: scenes.box_pile(6, 6, 3)),
    ("mixed_column", lambda: scenes.column_world(300, 11, "mixed")),
]


@pytest.mark.parametrize("name,make", SCENES, ids=[n for n, _ in SCENES])
def test_static_step_matches_world_step(ctx, name, make):
    sc = engine.setup_scene(make())
    ref = ctx.world(sc)
    sta = ctx.world(sc)
    L = _lib()
    for call in range(2):
        ref.step(sc.dt, 6)
        st = L.cp_world_step_static(ctx.h, sta.id, sc.dt, 6)
        assert st == A.CP_OK, L.cp_last_error().decode()
        assert ref.info().stepnumber == sta.info().stepnumber
        assert ref.bodies().tobytes() == sta.bodies().tobytes(), f"{name}: call {call}"
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
