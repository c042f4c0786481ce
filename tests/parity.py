"""Helpers shared by the parity tests: compare the GPU engine with the oracle."""
import numpy as np

from cannon_physics_gb300 import _abi as A

BODY_FIELDS = ["position", "quaternion", "velocity", "angular_velocity", "force", "torque", "inv_inertia_world",
               "aabb_lower", "aabb_upper", "previous_position", "previous_quaternion", "sleep_state", "time_last_sleepy",
               "type"]
CONTACT_FIELDS = ["bi", "bj", "si", "sj", "ni", "ri", "rj", "enabled", "pair", "restitution"]
ROW_FIELDS = ["kind", "bi", "bj", "B", "inv_c", "lambda_", "multiplier", "min_force", "max_force", "eps", "id"]


def diff_records(a, b, fields, what):
    """List of mismatch descriptions (bit-exact: equal values, -0 == +0)."""
    out = []
    if len(a) != len(b):
        return [f"{what}: count {len(a)} != {len(b)}"]
    for f in fields:
        x, y = a[f], b[f]
        eq = (x == y) | (np.isnan(x) & np.isnan(y)) if x.dtype.kind == "f" else (x == y)
        if not np.all(eq):
            bad = np.argwhere(~eq)
            i = tuple(bad[0])
            xf, yf = np.asarray(x, np.float64), np.asarray(y, np.float64)
            rel = np.max(np.abs(xf - yf) / np.maximum(np.abs(yf), 1e-30))
            out.append(f"{what}.{f}: {len(bad)} mismatches, first at {i}: {x[i]} vs {y[i]} (max rel {rel:.3g})")
    return out


def compare_step(gw, ow, check_lists=True):
    errs = []
    if check_lists:
        gp, op = gw.pairs(), ow.pairs()
        if len(gp[0]) != len(op[0]) or not (np.array_equal(gp[0], op[0]) and np.array_equal(gp[1], op[1])):
            errs.append(f"pairs differ: gpu {len(gp[0])} oracle {len(op[0])}")
        errs += diff_records(gw.contacts(), ow.contacts(), CONTACT_FIELDS, "contacts")
        errs += diff_records(gw.rows(), ow.rows(), ROW_FIELDS, "rows")
        gi, oi = gw.info(), ow.info()
        if gi.iterations != oi.iterations:
            errs.append(f"iterations {gi.iterations} != {oi.iterations}")
    errs += diff_records(gw.bodies(), ow.bodies(), BODY_FIELDS, "bodies")
    return errs
