"""The World clock at the C ABI: World.step's interpolating form, the
internalStep entry a binding calls when World.step keeps the clock, and the
compact per-step body records.

The reference's World.step(dt, timeSinceLastCalled, maxSubSteps)
(lib/world/world_class.dart:400-430) runs internal steps while its
accumulator holds a whole dt, keeps the remainder, interpolates every body's
pose, and only then adds timeSinceLastCalled to World.time; sleepTick inside
the sub-steps reads the time from before the call.  These tests drive that
form through cp_world_step_interpolated and through the binding pattern
(cp_world_set_time, then cp_world_internal_step) with timeSinceLastCalled
values that are not multiples of dt and sleeping on, and compare with the
oracle's restatement step by step.  Every body field is compared bit for
bit except the interpolated quaternion, whose slerp calls acos and sin: the
device's and the C library's agree to within 2 ulp in binary64, so the
binary32 components may differ by one unit in the last place.
"""
import numpy as np
import pytest

from cannon_physics_gb300 import _abi as A
from cannon_physics_gb300 import engine, scenes
from oracle import oracle_py as O

from tests.parity import BODY_FIELDS, diff_records

pytestmark = pytest.mark.gpu

EXACT = BODY_FIELDS + ["interpolated_position", "sleep_state", "time_last_sleepy"]
# tail of a frame-time sequence a render loop sees: jitter around 1/60 s, a
# stall, and calls shorter than dt
SINCE = [0.0171, 0.0158, 0.0333, 0.004, 0.009, 0.0166, 0.0502, 0.0171, 0.0012, 0.0201] * 12


@pytest.fixture(scope="module")
def ctx():
    from cannon_physics_gb300 import build as B
    B.build()
    c = engine.Context()
    yield c
    c.close()


def _scene():
    sc = scenes.spheres_on_plane(24, seed=9)
    sc.allow_sleep = True
    return sc


def _ulps(a, b):
    ai = np.ascontiguousarray(a, np.float32).view(np.int32).astype(np.int64)
    bi = np.ascontiguousarray(b, np.float32).view(np.int32).astype(np.int64)
    ai = np.where(ai < 0, np.int64(-2 ** 31) - ai, ai)
    bi = np.where(bi < 0, np.int64(-2 ** 31) - bi, bi)
    return np.abs(ai - bi)


def _compare(gw, ow, what):
    gb, ob = gw.bodies(), ow.bodies()
    errs = diff_records(gb, ob, EXACT, "bodies")
    u = _ulps(gb["interpolated_quaternion"], ob["interpolated_quaternion"])
    if u.max(initial=0) > 1:
        errs.append(f"interpolated_quaternion: {int(u.max())} ulp")
    gi, oi = gw.info(), ow.info()
    for f in ("stepnumber", "time", "accumulator", "substeps", "num_pairs", "num_contacts", "num_rows", "iterations"):
        if getattr(gi, f) != getattr(oi, f):
            errs.append(f"info.{f}: gpu {getattr(gi, f)} oracle {getattr(oi, f)}")
    assert not errs, f"{what}:\n" + "\n".join(errs[:10])


def test_interpolated_step_matches_oracle(ctx):
    sc = engine.setup_scene(_scene())
    gw = ctx.world(sc)
    ow = O.OracleWorld(sc)
    dt = 1.0 / 60.0
    slept = False
    for k, since in enumerate(SINCE):
        n_gpu = gw.step_interpolated(dt, since, 3)
        n_orc = ow.step_interpolated(dt, since, 3)
        assert n_gpu == n_orc
        _compare(gw, ow, f"call {k} (timeSinceLastCalled {since})")
        slept |= bool((gw.bodies()["sleep_state"] == A.SLEEPING).any())
    # the sequence covers zero, one, several and clamped sub-steps, and bodies
    # fell asleep on the interpolated clock
    assert slept
    assert abs(gw.info().time - sum(SINCE)) < 1e-9
    gw.destroy()


def test_internal_step_leaves_the_clock_to_the_caller(ctx):
    """The binding pattern: the host World keeps time (World.step adds dt or
    timeSinceLastCalled itself); before each internalStep it pushes its time
    to the device world.  Equals the oracle's World.step in both forms."""
    sc = engine.setup_scene(_scene())
    gw = ctx.world(sc)
    ow = O.OracleWorld(sc)
    dt = 1.0 / 60.0
    host_time, host_acc, stepnumber = 0.0, 0.0, 0
    for k, since in enumerate(SINCE[:60]):
        # host side of World.step(dt, since, 3) with the GPU as internalStep
        t_before = host_time
        host_acc += since
        n = 0
        while host_acc >= dt and n < 3:
            gw.set_time(host_time, stepnumber)
            gw.internal_step(dt, 1)
            stepnumber += 1
            host_acc -= dt
            n += 1
        host_acc = host_acc % dt
        host_time += since
        ow.step_interpolated(dt, since, 3)
        gi = gw.info()
        assert gi.stepnumber == ow.info().stepnumber == stepnumber
        if n:
            assert gi.time == t_before  # internalStep never moves the clock
        # previousQuaternion is normalised by the host side of World.step
        # (the interpolation), which this loop leaves out; integrate
        # overwrites it before it is read again
        gb, ob = gw.bodies(), ow.bodies()
        fields = [f for f in BODY_FIELDS if f != "previous_quaternion"] + ["time_last_sleepy"]
        errs = diff_records(gb, ob, fields, "bodies")
        assert not errs, f"call {k}:\n" + "\n".join(errs[:10])
    gw.destroy()


def test_fixed_step_advances_time_by_dt(ctx):
    sc = engine.setup_scene(_scene())
    gw = ctx.world(sc)
    gw.set_time(2.5, 7)
    gw.step(1.0 / 60.0, 3)
    inf = gw.info()
    assert inf.stepnumber == 10
    assert inf.time == ((2.5 + 1.0 / 60.0) + 1.0 / 60.0) + 1.0 / 60.0
    gw.internal_step(1.0 / 60.0, 2)
    assert gw.info().stepnumber == 12 and gw.info().time == inf.time
    gw.destroy()


def test_states_round_trip_and_steer_the_step(ctx):
    """cp_world_get_states / set_states move only the per-step fields; a
    velocity set through them steers the next step exactly as the same change
    made through the full body records does."""
    sc = engine.setup_scene(scenes.column_world(40, 77, "mixed"))
    a = ctx.world(sc)
    b = ctx.world(sc)
    a.step(sc.dt, 5)
    b.step(sc.dt, 5)
    st = a.states()
    full = a.bodies()
    for f in ("position", "quaternion", "velocity", "angular_velocity", "previous_position", "previous_quaternion",
              "sleep_state", "time_last_sleepy", "aabb_needs_update"):
        assert np.array_equal(st[f], full[f]), f
    st["velocity"][1:] += np.float32(0.5)
    st["force"][3] = (1.0, 2.0, 3.0)
    a.set_states(st)
    full["velocity"][1:] += np.float32(0.5)
    full["force"][3] = (1.0, 2.0, 3.0)
    b.set_bodies(full)
    a.step(sc.dt, 4)
    b.step(sc.dt, 4)
    assert a.bodies().tobytes() == b.bodies().tobytes()
    a.destroy()
    b.destroy()
