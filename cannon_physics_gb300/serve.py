"""The served form: a continuous-batching request server (cp_serve_* in
include/cannon_gpu.h).

A request is one world and a horizon (`nsteps` steps at `dt`).  The server
keeps admitted worlds resident on the device, admits queued requests as the
HBM budget frees up, and steps every admitted world together, a few steps per
tick, so requests that arrive while others run share the device with them.
Each result is the same as stepping the world alone with `cp_world_step`.
"""
import ctypes as C

import numpy as np

from . import _abi as A
from .engine import check, lib

PENDING, ACTIVE, DONE, FAILED, CANCELLED = 0, 1, 2, 3, 4


class ServeConfig(C.Structure):
    _fields_ = [
        ("device", C.c_int32),
        ("steps_per_tick", C.c_int32),
        ("hbm_budget_bytes", C.c_int64),
        ("max_active_bodies", C.c_int64),
        ("variant", C.c_int32),
        ("group_bodies", C.c_int32),
        ("max_list_entries", C.c_int64),
        ("wide_bodies", C.c_int32),
        ("wide_lanes", C.c_int32),
    ]


class ServeStats(C.Structure):
    _fields_ = [(name, C.c_int64) for name in (
        "submitted", "admitted", "completed", "failed", "cancelled", "pending", "active", "ticks",
        "bytes_in_use", "bytes_peak", "bytes_budget", "body_steps")] + [
        (name, C.c_double) for name in ("span_s", "device_s", "p50_ms", "p99_ms", "mean_ms", "max_ms")]


def _bind(L):
    if getattr(L, "_serve_bound", False):
        return L
    vp, i32, i64, f64 = C.c_void_p, C.c_int32, C.c_int64, C.c_double
    L.cp_serve_start.argtypes = [vp, vp]
    L.cp_serve_stop.argtypes = [vp]
    L.cp_serve_submit.argtypes = [vp, vp, f64, i32, vp]
    L.cp_serve_poll.argtypes = [vp, i64, vp]
    L.cp_serve_wait.argtypes = [vp, i64, f64, vp]
    L.cp_serve_result.argtypes = [vp, i64, vp, i32, vp]
    L.cp_serve_cancel.argtypes = [vp, i64]
    L.cp_serve_get_stats.argtypes = [vp, vp, i32]
    L._serve_bound = True
    return L


class Server:
    """Request server on one device.

    hbm_budget: bytes of device memory that admitted worlds (state and step
    scratch) may hold at once; steps_per_tick: steps every admitted world
    advances per launch sequence; max_active_bodies: optional cap on the
    bodies stepping at once (0: only the budget limits admission)."""

    def __init__(self, device=0, hbm_budget=150e9, steps_per_tick=2, max_active_bodies=0, variant=-1, group_bodies=0,
                 max_list_entries=0, wide_bodies=0, wide_lanes=0):
        L = _bind(lib())
        cfg = ServeConfig(device, steps_per_tick, int(hbm_budget), int(max_active_bodies), variant, group_bodies,
                          int(max_list_entries), int(wide_bodies), int(wide_lanes))
        h = C.c_void_p()
        check(L.cp_serve_start(C.byref(cfg), C.byref(h)), "cp_serve_start")
        self.h = h
        self._sizes = {}

    def close(self):
        if getattr(self, "h", None):
            lib().cp_serve_stop(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def submit(self, scene, dt, nsteps):
        """Queue a rollout of `scene`; returns its ticket.  The scene's arrays
        are copied during the call."""
        desc = scene.world_desc()
        t = C.c_int64()
        check(lib().cp_serve_submit(self.h, C.byref(desc), dt, int(nsteps), C.byref(t)), "cp_serve_submit")
        self._sizes[t.value] = scene.num_bodies
        return t.value

    def poll(self, ticket):
        s = C.c_int32()
        check(lib().cp_serve_poll(self.h, ticket, C.byref(s)), "cp_serve_poll")
        return s.value

    def wait(self, ticket, timeout=-1.0):
        s = C.c_int32()
        check(lib().cp_serve_wait(self.h, ticket, float(timeout), C.byref(s)), "cp_serve_wait")
        return s.value

    def result(self, ticket):
        """Bodies after the rollout and the final step info; releases the
        request."""
        n = self._sizes.pop(ticket)
        out = np.zeros(n, dtype=A.BODY_DTYPE)
        info = A.StepInfo()
        check(lib().cp_serve_result(self.h, ticket, out.ctypes.data, n, C.byref(info)), "cp_serve_result")
        return out, info

    def cancel(self, ticket):
        check(lib().cp_serve_cancel(self.h, ticket), "cp_serve_cancel")

    def stats(self, reset=False):
        s = ServeStats()
        check(lib().cp_serve_get_stats(self.h, C.byref(s), int(reset)), "cp_serve_get_stats")
        return {name: getattr(s, name) for name, _ in ServeStats._fields_}
