"""ctypes binding of libcannon_gpu.so (include/cannon_gpu.h).

`Context` owns a CUDA stream and the device worlds; `GpuWorld` is one World
resident in HBM.  There is no CPU fallback: if the library is missing the
import of the engine fails with instructions to build it.
"""
import ctypes as C
import os

import numpy as np

from . import _abi as A

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libcannon_gpu.so")
_lib = None


class CannonError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"status {status}: {msg}")
        self.status = status


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(LIB_PATH)
        vp, i32, f64 = C.c_void_p, C.c_int32, C.c_double
        L.cp_last_error.restype = C.c_char_p
        L.cp_abi_version.restype = C.c_int
        L.cp_shape_setup.argtypes = [vp]
        L.cp_body_setup.argtypes = [vp, i32, vp, i32, vp, i32]
        L.cp_create.argtypes = [vp, vp]
        L.cp_destroy.argtypes = [vp]
        L.cp_world_create.argtypes = [vp, vp, vp]
        L.cp_world_destroy.argtypes = [vp, i32]
        L.cp_world_step.argtypes = [vp, i32, f64, i32]
        L.cp_world_internal_step.argtypes = [vp, i32, f64, i32]
        L.cp_world_step_interpolated.argtypes = [vp, i32, f64, f64, i32, vp]
        L.cp_world_set_time.argtypes = [vp, i32, f64, C.c_int64, f64]
        L.cp_world_get_states.argtypes = [vp, i32, vp, i32]
        L.cp_world_set_events.argtypes = [vp, i32, i32, vp, vp]
        L.cp_world_get_events.argtypes = [vp, i32, vp, i32, vp]
        L.cp_world_set_states.argtypes = [vp, i32, vp, i32]
        L.cp_world_get_bodies.argtypes = [vp, i32, vp, i32]
        L.cp_world_set_bodies.argtypes = [vp, i32, vp, i32]
        L.cp_world_get_pairs.argtypes = [vp, i32, vp, vp, i32, vp]
        L.cp_world_get_contacts.argtypes = [vp, i32, vp, i32, vp]
        L.cp_world_get_rows.argtypes = [vp, i32, vp, i32, vp]
        L.cp_world_get_info.argtypes = [vp, i32, vp]
        L.cp_world_get_sap_order.argtypes = [vp, i32, vp, i32]
        L.cp_world_raycast.argtypes = [vp, i32, vp, i32, i32, vp, i32, vp]
        L.cp_batch_step.argtypes = [vp, vp, i32, f64, i32]
        L.cp_batch_set_forces.argtypes = [vp, vp, i32, vp, C.c_int64]
        L.cp_batch_get_poses.argtypes = [vp, vp, i32, vp, C.c_int64]
        L.cp_kernel_launches.argtypes = [vp]
        L.cp_kernel_launches.restype = C.c_int64
        L.cp_get_stream.argtypes = [vp, vp]
        L.cp_batch_profile.argtypes = [vp, vp, vp]
        L.cp_phase_profile.argtypes = [vp, vp, i32]
        L.cp_set_resolver_profile.argtypes = [vp, i32]
        L.cp_autotune_info.argtypes = [vp, vp, vp, vp, i32]
        L.cp_set_variant.argtypes = [vp, i32]
        L.cp_set_group_bodies.argtypes = [vp, i32]
        L.cp_set_wide_bodies.argtypes = [vp, i32]
        L.cp_set_sweep_schedule.argtypes = [vp, i32]
        L.cp_set_filter_check.argtypes = [vp, i32]
        L.cp_filter_check_counts.argtypes = [vp, vp, vp, i32]
        _lib = L
    return _lib


def check(status, what=""):
    if status != A.CP_OK:
        raise CannonError(status, f"{what}: {lib().cp_last_error().decode()}")


def setup_scene(scene):
    """Run the Shape / Body constructor arithmetic (cp_shape_setup, cp_body_setup)
    over a scene in place; host-only, no GPU needed."""
    L = lib()
    for i in range(len(scene.shapes)):
        check(L.cp_shape_setup(scene.shapes[i:i + 1].ctypes.data), "cp_shape_setup")
    check(L.cp_body_setup(A.ptr(scene.shapes), len(scene.shapes), A.ptr(scene.body_shapes), len(scene.body_shapes),
                          A.ptr(scene.bodies), len(scene.bodies)), "cp_body_setup")
    return scene


class Context:
    def __init__(self, device=0):
        cfg = A.Config(device, 0, 0)
        h = C.c_void_p()
        check(lib().cp_create(C.byref(cfg), C.byref(h)), "cp_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().cp_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def launches(self):
        return int(lib().cp_kernel_launches(self.h))

    def stream_handle(self):
        s = C.c_void_p()
        check(lib().cp_get_stream(self.h, C.byref(s)), "cp_get_stream")
        return s.value

    PHASES = ("prepare", "broadphase", "narrowphase", "rows_wake_prep", "assemble", "levels", "gs_sweeps", "integrate")

    RESOLVERS = ("", "sphere_sphere", "sphere_plane", "sphere_box", "sphere_convex", "plane_box", "plane_convex", "box_box",
                 "box_convex", "convex_convex", "cert_sphere_plane", "cert_plane_hull", "cert_sphere_box")

    def phase_profile(self, resolvers=False):
        """SM cycles per step phase (summed over blocks) since the last call;
        with resolvers=True also {resolver: (thread cycles, calls)}."""
        out = np.zeros(40, np.float64)
        check(lib().cp_phase_profile(self.h, out.ctypes.data, len(out)), "cp_phase_profile")
        ph = dict(zip(self.PHASES, out[:8].tolist()))
        if not resolvers:
            return ph
        res = {name: (out[8 + i], out[24 + i]) for i, name in enumerate(self.RESOLVERS) if name and out[24 + i] > 0}
        return ph, res

    def resolver_profile(self, on=True):
        """Count per-resolver cycles and calls (off by default; per device)."""
        check(lib().cp_set_resolver_profile(self.h, int(bool(on))), "cp_set_resolver_profile")

    def set_filter_check(self, on=True):
        """Check every binary32 filter decision against the unfiltered binary64
        computation (slow; for tests and audits)."""
        check(lib().cp_set_filter_check(self.h, int(bool(on))), "cp_set_filter_check")

    def filter_check_counts(self, reset=False):
        """(pairs checked, disagreements) since the last reset."""
        a, b = C.c_int64(), C.c_int64()
        check(lib().cp_filter_check_counts(self.h, C.byref(a), C.byref(b), int(bool(reset))), "cp_filter_check_counts")
        return a.value, b.value

    def set_wide_bodies(self, n):
        """Single-world steps of worlds with at least n bodies spread over the
        whole GPU (0: never)."""
        check(lib().cp_set_wide_bodies(self.h, n), "cp_set_wide_bodies")

    def set_sweep_schedule(self, mode):
        """Sweeps of wide worlds: 0 on the slot schedule where it pays, 1
        wherever it fits, -1 always level by level (same bits)."""
        check(lib().cp_set_sweep_schedule(self.h, mode), "cp_set_sweep_schedule")

    def set_group_bodies(self, n):
        check(lib().cp_set_group_bodies(self.h, n), "cp_set_group_bodies")

    def autotune_info(self):
        v, t = C.c_int32(), C.c_int32()
        ms = np.zeros(64)
        n = lib().cp_autotune_info(self.h, C.byref(v), C.byref(t), ms.ctypes.data, 64)
        return {"variant": v.value, "threads": t.value, "ms_per_variant": ms[:n].round(3).tolist()}

    def set_variant(self, v):
        """Pin the batched kernel variant, or -1 to autotune."""
        check(lib().cp_set_variant(self.h, v), "cp_set_variant")

    def batch_profile(self):
        """(device ms, step launches) of batched graphs since the last call."""
        ms = C.c_double()
        n = C.c_int64()
        check(lib().cp_batch_profile(self.h, C.byref(ms), C.byref(n)), "cp_batch_profile")
        return ms.value, n.value

    def world(self, scene):
        return GpuWorld(self, scene)

    def batch_step(self, worlds, dt, nsteps):
        ids = np.array([w.id for w in worlds], dtype=np.int32)
        check(lib().cp_batch_step(self.h, ids.ctypes.data, len(ids), dt, nsteps), "cp_batch_step")


class Batch:
    """A fixed list of worlds stepped together, with packed host I/O."""

    def __init__(self, ctx, worlds):
        self.ctx = ctx
        self.worlds = list(worlds)
        self.ids = np.array([w.id for w in self.worlds], dtype=np.int32)
        self.total = int(sum(w.n for w in self.worlds))

    def step(self, dt, nsteps=1):
        check(lib().cp_batch_step(self.ctx.h, self.ids.ctypes.data, len(self.ids), dt, nsteps), "cp_batch_step")

    def set_forces(self, ft_ptr):
        """ft_ptr: address of total*6 float32 (force xyz, torque xyz per body)."""
        check(lib().cp_batch_set_forces(self.ctx.h, self.ids.ctypes.data, len(self.ids), ft_ptr, self.total), "set_forces")

    def get_poses(self, out_ptr):
        """out_ptr: address of total*13 float32 (pos, quat, vel, angular vel per body)."""
        check(lib().cp_batch_get_poses(self.ctx.h, self.ids.ctypes.data, len(self.ids), out_ptr, self.total), "get_poses")


class GpuWorld:
    def __init__(self, ctx, scene):
        self.ctx = ctx
        self.scene = scene
        self.n = scene.num_bodies
        desc = scene.world_desc()
        wid = C.c_int32()
        check(lib().cp_world_create(ctx.h, C.byref(desc), C.byref(wid)), "cp_world_create")
        self.id = wid.value

    def destroy(self):
        if self.id is not None and self.ctx.h:
            check(lib().cp_world_destroy(self.ctx.h, self.id), "cp_world_destroy")
            self.id = None

    def step(self, dt=None, nsteps=1):
        check(lib().cp_world_step(self.ctx.h, self.id, self.scene.dt if dt is None else dt, nsteps), "cp_world_step")

    def internal_step(self, dt=None, nsteps=1):
        """World.internalStep: stepnumber advances, time does not."""
        check(lib().cp_world_internal_step(self.ctx.h, self.id, self.scene.dt if dt is None else dt, nsteps), "internal_step")

    def step_interpolated(self, dt, time_since_last_called, max_sub_steps=10):
        """World.step(dt, timeSinceLastCalled, maxSubSteps); returns the sub-steps taken."""
        n = C.c_int32()
        check(lib().cp_world_step_interpolated(self.ctx.h, self.id, dt, time_since_last_called, max_sub_steps, C.byref(n)),
              "step_interpolated")
        return n.value

    def set_time(self, time, stepnumber, accumulator=0.0):
        check(lib().cp_world_set_time(self.ctx.h, self.id, time, stepnumber, accumulator), "set_time")

    def set_events(self, on=True, body_ids=None, shape_ids=None):
        """Record World's events (collide, begin/end contact, begin/end shape
        contact) every step; ids: the Body.id / Shape.id values (default: the
        indices)."""
        self._ids = (None if body_ids is None else np.ascontiguousarray(body_ids, np.int32),
                     None if shape_ids is None else np.ascontiguousarray(shape_ids, np.int32))
        bi, si = self._ids
        check(lib().cp_world_set_events(self.ctx.h, self.id, int(bool(on)), None if bi is None else bi.ctypes.data,
                                        None if si is None else si.ctypes.data), "set_events")

    def events(self):
        """The recorded events since the last call, oldest first."""
        cnt = C.c_int32()
        if lib().cp_world_get_events(self.ctx.h, self.id, None, 0, C.byref(cnt)) == A.CP_OK:
            return np.zeros(0, dtype=A.EVENT_DTYPE)
        out = np.zeros(cnt.value, dtype=A.EVENT_DTYPE)
        check(lib().cp_world_get_events(self.ctx.h, self.id, out.ctypes.data, len(out), C.byref(cnt)), "get_events")
        return out[:cnt.value]

    def raycast(self, rays, mode=A.RAY_CLOSEST, max_hits=16):
        """World.raycastClosest / Any (one RaycastResult per ray) or
        raycastAll (mode RAY_ALL: (hits of shape (n, max_hits), counts))."""
        rays = np.ascontiguousarray(rays, dtype=A.RAY_DTYPE)
        n = len(rays)
        if mode == A.RAY_ALL:
            hits = np.zeros(max(1, n * max_hits), dtype=A.RAY_HIT_DTYPE)
            counts = np.zeros(max(1, n), dtype=np.int32)
            check(lib().cp_world_raycast(self.ctx.h, self.id, rays.ctypes.data, n, mode, hits.ctypes.data, max_hits,
                                         counts.ctypes.data), "raycast")
            return hits[:n * max_hits].reshape(n, max_hits), counts[:n]
        hits = np.zeros(max(1, n), dtype=A.RAY_HIT_DTYPE)
        check(lib().cp_world_raycast(self.ctx.h, self.id, rays.ctypes.data, n, mode, hits.ctypes.data, 1, None), "raycast")
        return hits[:n]

    def states(self):
        out = np.zeros(self.n, dtype=A.BODY_STATE_DTYPE)
        check(lib().cp_world_get_states(self.ctx.h, self.id, out.ctypes.data, self.n), "get_states")
        return out

    def set_states(self, states):
        states = np.ascontiguousarray(states, dtype=A.BODY_STATE_DTYPE)
        check(lib().cp_world_set_states(self.ctx.h, self.id, states.ctypes.data, self.n), "set_states")

    def bodies(self):
        out = np.zeros(self.n, dtype=A.BODY_DTYPE)
        check(lib().cp_world_get_bodies(self.ctx.h, self.id, out.ctypes.data, self.n), "get_bodies")
        return out

    def set_bodies(self, bodies):
        bodies = np.ascontiguousarray(bodies, dtype=A.BODY_DTYPE)
        check(lib().cp_world_set_bodies(self.ctx.h, self.id, bodies.ctypes.data, self.n), "set_bodies")

    def info(self):
        inf = A.StepInfo()
        check(lib().cp_world_get_info(self.ctx.h, self.id, C.byref(inf)), "get_info")
        return inf

    def pairs(self):
        n = self.info().num_pairs
        p1 = np.zeros(max(n, 1), np.int32)
        p2 = np.zeros(max(n, 1), np.int32)
        cnt = C.c_int32()
        check(lib().cp_world_get_pairs(self.ctx.h, self.id, p1.ctypes.data, p2.ctypes.data, len(p1), C.byref(cnt)), "pairs")
        return p1[:cnt.value], p2[:cnt.value]

    def contacts(self):
        n = self.info().num_contacts
        out = np.zeros(max(n, 1), dtype=A.CONTACT_DTYPE)
        cnt = C.c_int32()
        check(lib().cp_world_get_contacts(self.ctx.h, self.id, out.ctypes.data, len(out), C.byref(cnt)), "contacts")
        return out[:cnt.value]

    def rows(self):
        n = self.info().num_rows
        out = np.zeros(max(n, 1), dtype=A.ROW_DTYPE)
        cnt = C.c_int32()
        check(lib().cp_world_get_rows(self.ctx.h, self.id, out.ctypes.data, len(out), C.byref(cnt)), "rows")
        return out[:cnt.value]

    def sap_order(self):
        out = np.zeros(self.n, np.int32)
        check(lib().cp_world_get_sap_order(self.ctx.h, self.id, out.ctypes.data, self.n), "sap order")
        return out
