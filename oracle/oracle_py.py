"""ctypes front end of the CPU oracle -- test infrastructure only.

Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs, to
compare the GPU path's results with and to time the CPU baseline.  The
cannon_physics_gb300 package never imports this module.
"""
import ctypes as C

import numpy as np

from cannon_physics_gb300 import _abi as A

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        vp, i32, f64 = C.c_void_p, C.c_int32, C.c_double
        L.orc_shape_setup.argtypes = [vp]
        L.orc_body_setup.argtypes = [vp, i32, vp, i32, vp, i32]
        L.orc_world_create.argtypes = [vp]
        L.orc_world_create.restype = vp
        L.orc_world_destroy.argtypes = [vp]
        L.orc_world_step.argtypes = [vp, f64, i32]
        L.orc_world_internal_step.argtypes = [vp, f64, i32]
        L.orc_world_step_interpolated.argtypes = [vp, f64, f64, i32, vp]
        L.orc_world_set_time.argtypes = [vp, f64, C.c_int64, f64]
        L.orc_world_set_bodies.argtypes = [vp, vp, i32]
        L.orc_world_set_events.argtypes = [vp, i32, vp, vp]
        L.orc_world_get_events.argtypes = [vp, vp, i32, vp]
        L.orc_world_set_sap_order.argtypes = [vp, vp, i32]
        L.orc_world_get_bodies.argtypes = [vp, vp, i32]
        L.orc_world_get_pairs.argtypes = [vp, vp, vp, i32, vp]
        L.orc_world_get_contacts.argtypes = [vp, vp, i32, vp]
        L.orc_world_get_rows.argtypes = [vp, vp, i32, vp]
        L.orc_world_get_info.argtypes = [vp, vp]
        L.orc_world_get_sap_order.argtypes = [vp, vp, i32]
        L.orc_world_raycast.argtypes = [vp, vp, i32, i32, vp, i32, vp]
        L.orc_worlds_step_parallel.argtypes = [vp, i32, f64, i32, i32]
        L.orc_shape_hull.argtypes = [vp, vp, i32, vp, vp, i32, vp, vp, i32, vp]
        _lib = L
    return _lib


def _check(st, what):
    if st != A.CP_OK:
        raise RuntimeError(f"oracle {what} failed with status {st}")


def setup_scene(scene):
    """Run the oracle's Shape/Body constructor restatement over a scene in place."""
    L = lib()
    for i in range(len(scene.shapes)):
        _check(L.orc_shape_setup(scene.shapes[i:i + 1].ctypes.data), "shape setup")
    _check(L.orc_body_setup(A.ptr(scene.shapes), len(scene.shapes), A.ptr(scene.body_shapes), len(scene.body_shapes),
                            A.ptr(scene.bodies), len(scene.bodies)), "body setup")
    return scene


class OracleWorld:
    def __init__(self, scene):
        self.scene = scene
        self.n = scene.num_bodies
        desc = scene.world_desc()
        self.h = lib().orc_world_create(C.byref(desc))
        if not self.h:
            raise RuntimeError("oracle world create failed")

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_world_destroy(self.h)
            self.h = None

    def step(self, dt=None, nsteps=1):
        _check(lib().orc_world_step(self.h, self.scene.dt if dt is None else dt, nsteps), "step")

    def internal_step(self, dt=None, nsteps=1):
        _check(lib().orc_world_internal_step(self.h, self.scene.dt if dt is None else dt, nsteps), "internal step")

    def step_interpolated(self, dt, time_since_last_called, max_sub_steps=10):
        n = C.c_int32()
        _check(lib().orc_world_step_interpolated(self.h, dt, time_since_last_called, max_sub_steps, C.byref(n)),
               "interpolated step")
        return n.value

    def set_time(self, time, stepnumber, accumulator=0.0):
        _check(lib().orc_world_set_time(self.h, time, stepnumber, accumulator), "set time")

    def bodies(self):
        out = np.zeros(self.n, dtype=A.BODY_DTYPE)
        _check(lib().orc_world_get_bodies(self.h, out.ctypes.data, self.n), "get bodies")
        return out

    def set_events(self, on=True, body_ids=None, shape_ids=None):
        self._ids = (None if body_ids is None else np.ascontiguousarray(body_ids, np.int32),
                     None if shape_ids is None else np.ascontiguousarray(shape_ids, np.int32))
        bi, si = self._ids
        _check(lib().orc_world_set_events(self.h, int(bool(on)), None if bi is None else bi.ctypes.data,
                                          None if si is None else si.ctypes.data), "set events")

    def events(self):
        cnt = C.c_int32()
        if lib().orc_world_get_events(self.h, None, 0, C.byref(cnt)) == A.CP_OK:
            return np.zeros(0, dtype=A.EVENT_DTYPE)
        out = np.zeros(cnt.value, dtype=A.EVENT_DTYPE)
        _check(lib().orc_world_get_events(self.h, out.ctypes.data, len(out), C.byref(cnt)), "events")
        return out[:cnt.value]

    def raycast(self, rays, mode=A.RAY_CLOSEST, max_hits=16):
        rays = np.ascontiguousarray(rays, dtype=A.RAY_DTYPE)
        n = len(rays)
        if mode == A.RAY_ALL:
            hits = np.zeros(max(1, n * max_hits), dtype=A.RAY_HIT_DTYPE)
            counts = np.zeros(max(1, n), dtype=np.int32)
            _check(lib().orc_world_raycast(self.h, rays.ctypes.data, n, mode, hits.ctypes.data, max_hits,
                                           counts.ctypes.data), "raycast")
            return hits[:n * max_hits].reshape(n, max_hits), counts[:n]
        hits = np.zeros(max(1, n), dtype=A.RAY_HIT_DTYPE)
        _check(lib().orc_world_raycast(self.h, rays.ctypes.data, n, mode, hits.ctypes.data, 1, None), "raycast")
        return hits[:n]

    def set_bodies(self, bodies):
        bodies = np.ascontiguousarray(bodies, dtype=A.BODY_DTYPE)
        _check(lib().orc_world_set_bodies(self.h, bodies.ctypes.data, self.n), "set bodies")

    def set_sap_order(self, order):
        order = np.ascontiguousarray(order, dtype=np.int32)
        _check(lib().orc_world_set_sap_order(self.h, order.ctypes.data, self.n), "set sap order")

    def load_state(self, gpu_world):
        """Continue from a GPU world's state (bodies, SAP order, time, step
        number): both then take the same next steps."""
        inf = gpu_world.info()
        self.set_bodies(gpu_world.bodies())
        self.set_sap_order(gpu_world.sap_order())
        self.set_time(inf.time, inf.stepnumber, inf.accumulator)

    def info(self):
        inf = A.StepInfo()
        _check(lib().orc_world_get_info(self.h, C.byref(inf)), "info")
        return inf

    def pairs(self):
        inf = self.info()
        n = inf.num_pairs
        p1 = np.zeros(max(n, 1), np.int32)
        p2 = np.zeros(max(n, 1), np.int32)
        cnt = C.c_int32()
        _check(lib().orc_world_get_pairs(self.h, p1.ctypes.data, p2.ctypes.data, len(p1), C.byref(cnt)), "pairs")
        return p1[:cnt.value], p2[:cnt.value]

    def contacts(self):
        inf = self.info()
        out = np.zeros(max(inf.num_contacts, 1), dtype=A.CONTACT_DTYPE)
        cnt = C.c_int32()
        _check(lib().orc_world_get_contacts(self.h, out.ctypes.data, len(out), C.byref(cnt)), "contacts")
        return out[:cnt.value]

    def rows(self):
        inf = self.info()
        out = np.zeros(max(inf.num_rows, 1), dtype=A.ROW_DTYPE)
        cnt = C.c_int32()
        _check(lib().orc_world_get_rows(self.h, out.ctypes.data, len(out), C.byref(cnt)), "rows")
        return out[:cnt.value]

    def sap_order(self):
        out = np.zeros(self.n, np.int32)
        _check(lib().orc_world_get_sap_order(self.h, out.ctypes.data, self.n), "sap order")
        return out


def step_parallel(worlds, dt, nsteps, threads):
    arr = (C.c_void_p * len(worlds))(*[w.h for w in worlds])
    _check(lib().orc_worlds_step_parallel(arr, len(worlds), dt, nsteps, threads), "parallel step")


def shape_hull(shape_rec):
    L = lib()
    v = np.zeros(3 * 256, np.float32)
    n = np.zeros(3 * 256, np.float32)
    e = np.zeros(3 * 256, np.float32)
    nv, nf, ne = C.c_int32(), C.c_int32(), C.c_int32()
    _check(L.orc_shape_hull(shape_rec.ctypes.data, v.ctypes.data, 256, C.byref(nv), n.ctypes.data, 256, C.byref(nf),
                            e.ctypes.data, 256, C.byref(ne)), "hull")
    return v[:3 * nv.value].reshape(-1, 3), n[:3 * nf.value].reshape(-1, 3), e[:3 * ne.value].reshape(-1, 3)
