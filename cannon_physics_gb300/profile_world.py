"""Steps one scene of `cannon_physics_gb300.scenes` for a profiler.

    python -m cannon_physics_gb300.profile_world box_pile --preroll 100 --steps 2

builds the library, creates the scene's world, takes `--preroll` untimed
steps, then `--steps` steps one call each, and prints one line: the kernel
launches the library made before the profiled steps (the `-s` to give
`ncu` so that it skips them), launches per profiled step, host-timed
milliseconds per step and the last step's list sizes.  `--wide-bodies`
sets the body count from which a world takes the grid-wide path (default:
the library's).
"""
import argparse
import json
import time

from cannon_physics_gb300 import build as B
from cannon_physics_gb300 import engine, scenes


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("scene", help="a scene builder of cannon_physics_gb300.scenes, e.g. box_pile or mixed_chains")
    ap.add_argument("--preroll", type=int, default=100)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--wide-bodies", type=int, default=None)
    a = ap.parse_args(argv)
    B.build()
    ctx = engine.Context(0)
    if a.wide_bodies is not None:
        ctx.set_wide_bodies(a.wide_bodies)
    sc = engine.setup_scene(getattr(scenes, a.scene)())
    w = ctx.world(sc)
    w.step(sc.dt, a.preroll)
    n0 = ctx.launches()
    t0 = time.perf_counter()
    for _ in range(a.steps):
        w.step(sc.dt, 1)
    sec = time.perf_counter() - t0
    inf = w.info()
    print(json.dumps({"scene": a.scene, "bodies": sc.num_bodies, "launches_before": n0,
                      "launches_per_step": (ctx.launches() - n0) / max(1, a.steps),
                      "ms_per_step": sec * 1e3 / max(1, a.steps), "pairs": inf.num_pairs, "contacts": inf.num_contacts,
                      "rows": inf.num_rows, "levels": inf.num_levels, "iterations": inf.iterations}), flush=True)
    w.destroy()
    ctx.close()


if __name__ == "__main__":
    main()
