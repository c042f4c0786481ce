"""Writes the golden step vectors under tests/golden/ from the oracle.

The reference (Dart, needs Flutter) cannot run in this environment and ships
no vectors of its own, so these vectors pin the oracle and the GPU path to
each other and to their own history: any change to either that alters a
single bit of a step shows up against them.  Each case is a small seeded
scene stepped by the oracle; after every step the counters (pairs, contacts,
rows, solver iterations) are recorded, and after the last step the body
state, the pair list, the contacts and the solver rows.

Run from the repository root:  python tests/golden/make_golden.py [case ...]
(with case names, only those cases are written again; the others' files and
manifest entries stay as they are)
"""
import json
import os
import platform
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from cannon_physics_gb300 import scenes  # noqa: E402
from oracle import build as OB  # noqa: E402
from oracle import oracle_py as O  # noqa: E402

# (name, scene builder, steps)
CASES = [
    ("spheres_naive", lambda: scenes.spheres_on_plane(64, seed=1), 90),
    ("boxes_sap", lambda: scenes.box_pile(4, 4, 3, seed=2), 40),
    ("mixed_grid_chains_sleep", lambda: scenes.mixed_chains(8, 4, 4, seed=3, chains=4, chain_len=8), 60),
    ("column_sphere_box", lambda: scenes.column_world(120, 1234, "sphere_box"), 50),
    ("column_mixed", lambda: scenes.column_world(80, 4321, "mixed"), 50),
    ("compound_naive", lambda: scenes.compound_pile(20, seed=12), 60),
    ("joints_hulls", lambda: scenes.joints_and_hulls(seed=44), 60),
    ("chains_split", lambda: scenes.use_split_solver(scenes.mixed_chains(8, 4, 4, seed=5, chains=4, chain_len=8)), 60),
]

BODY_FIELDS = ["position", "quaternion", "velocity", "angular_velocity", "inv_inertia_world", "sleep_state"]


def run_case(make, steps):
    sc = O.setup_scene(make())
    w = O.OracleWorld(sc)
    counters = np.zeros((steps, 4), np.int32)
    for s in range(steps):
        w.step(sc.dt, 1)
        inf = w.info()
        counters[s] = (inf.num_pairs, inf.num_contacts, inf.num_rows, inf.iterations)
    b = w.bodies()
    p1, p2 = w.pairs()
    ct = w.contacts()
    rows = w.rows()
    out = {f"body_{f}": np.ascontiguousarray(b[f]) for f in BODY_FIELDS}
    out.update(counters=counters, pair_a=p1, pair_b=p2,
               contact_bodies=np.stack([ct["bi"], ct["bj"]], 1).astype(np.int32) if len(ct) else np.zeros((0, 2), np.int32),
               contact_ni=np.ascontiguousarray(ct["ni"]), row_lambda=np.ascontiguousarray(rows["lambda_"]),
               row_kind=np.ascontiguousarray(rows["kind"]))
    return out


def main(only=()):
    OB.build()
    path = os.path.join(HERE, "manifest.json")
    manifest = {}
    if only and os.path.exists(path):
        with open(path) as f:
            manifest = json.load(f)["cases"]
    for name, make, steps in CASES:
        if only and name not in only:
            continue
        data = run_case(make, steps)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **data)
        manifest[name] = {"steps": steps, "bodies": int(len(data["body_position"])),
                          "final_pairs": int(data["counters"][-1, 0]), "final_contacts": int(data["counters"][-1, 1])}
    # libm and compiler differences between host architectures can move the
    # last bit of a few solver values; the machine that wrote the vectors is
    # recorded so that other machines compare floats with a tolerance
    manifest = {"machine": platform.machine(), "cases": manifest}
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)
    print(json.dumps(manifest, indent=1))


if __name__ == "__main__":
    main(tuple(sys.argv[1:]))
