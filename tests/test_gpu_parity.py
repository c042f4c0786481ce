"""CUDA path vs the CPU oracle, step by step, bit-exact.

Every comparison is exact: broadphase pairs (order and orientation),
contacts (bodies, shapes, normal, contact points, restitution), solver rows
(B, 1/C, lambda, multiplier, bounds), iteration counts and every body field.
The tolerance the parity contract allows for binary64 values (1e-9 relative)
is not needed: both sides round at the same points.
"""
import numpy as np
import pytest

from cannon_physics_gb300 import engine, scenes
from oracle import oracle_py as O

from tests.edge_scenes import EDGE_NAMES, edge_scene
from tests.parity import compare_step

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from cannon_physics_gb300 import build as B
    B.build()
    c = engine.Context()
    yield c
    c.close()


def run_parity(ctx, scene, steps, every=1, check_lists=True):
    engine.setup_scene(scene)
    gw = ctx.world(scene)
    ow = O.OracleWorld(scene)
    done = 0
    while done < steps:
        k = min(every, steps - done)
        gw.step(nsteps=k)
        ow.step(nsteps=k)
        done += k
        errs = compare_step(gw, ow, check_lists=check_lists)
        assert not errs, f"{scene.name}: mismatch after step {done}:\n" + "\n".join(errs[:10])
    info = gw.info()
    gw.destroy()
    return info


def test_spheres_on_plane_full_600_steps(ctx):
    """The 64-sphere scene (Naive, 10 iterations) over its whole 600-step horizon."""
    info = run_parity(ctx, scenes.spheres_on_plane(), 600, every=20)
    assert info.stepnumber == 600 and info.num_contacts >= 60


def test_box_pile_small(ctx):
    run_parity(ctx, scenes.box_pile(6, 6, 4), 40)


def test_box_pile_full_size_first_steps(ctx):
    """The 4096-box SAP pile (box-box SAT + clipping) for its first steps."""
    info = run_parity(ctx, scenes.box_pile(), 3)
    assert info.num_contacts > 1000


def test_mixed_chains_small(ctx):
    run_parity(ctx, scenes.mixed_chains(8, 4, 4, chains=4, chain_len=8), 60)


def test_mixed_chains_full_size_first_steps(ctx):
    """8192 mixed shapes with 128 chains, GridBroadphase, sleeping on."""
    info = run_parity(ctx, scenes.mixed_chains(), 2)
    assert info.num_rows > 5000


@pytest.mark.parametrize("n,seed", [(8, 1001), (60, 1002), (200, 1003), (512, 1004)])
def test_column_worlds(ctx, n, seed):
    run_parity(ctx, scenes.column_world(n, seed, "sphere_box"), 60, every=3)


@pytest.mark.parametrize("n,seed", [(16, 2001), (300, 2002)])
def test_mixed_request_worlds(ctx, n, seed):
    run_parity(ctx, scenes.column_world(n, seed, "mixed"), 40, every=2)


@pytest.mark.parametrize("name", EDGE_NAMES)
def test_edge_scenes(ctx, name):
    run_parity(ctx, edge_scene(name), 45)


def test_dense_cluster_grows_capacities(ctx):
    """300 spheres in a 1.2 m cube overlap far more than the initial pair and
    contact capacities; the step reports the overflow, the world's scratch is
    regrown and the step re-run, with results still equal to the oracle."""
    sc = scenes.spheres_on_plane(300)
    rng = scenes.SplitMix64(99)
    sc.bodies["position"][1:] = (rng.uniform(900).reshape(300, 3) * 1.2 + np.array([-0.6, 0.6, -0.6]))
    engine.setup_scene(sc)
    probe = ctx.world(sc)
    probe.step()
    assert probe.info().num_pairs > 4 * 301 + 64  # above the initial pair capacity
    probe.destroy()
    run_parity(ctx, sc, 5)


def test_batched_equals_plain_and_oracle(ctx):
    """cp_batch_step (persistent kernel, CUDA graph) gives each world exactly
    the result of stepping it alone."""
    worlds = [scenes.column_world(int(n), 3000 + i, "sphere_box") for i, n in enumerate(scenes.batch_sizes(48, 5000))]
    worlds += [scenes.column_world(40, 3100 + i, "mixed") for i in range(8)]
    for s in worlds:
        engine.setup_scene(s)
    batch = [ctx.world(s) for s in worlds]
    plain = [ctx.world(s) for s in worlds]
    ctx.batch_step(batch, 1 / 60, 25)
    ctx.batch_step(batch, 1 / 60, 25)  # graph replay
    for w in plain:
        w.step(1 / 60, 50)
    for b, p, s in zip(batch, plain, worlds):
        gb, gp = b.bodies(), p.bodies()
        assert gb.tobytes() == gp.tobytes(), s.name
    ow = O.OracleWorld(worlds[5])
    ow.step(1 / 60, 50)
    assert not compare_step(batch[5], ow, check_lists=True)
    for w in batch + plain:
        w.destroy()


def test_large_batch_equals_plain(ctx):
    """2048 worlds of the batched workload, 70 steps in two calls (the second
    replays the captured graph): a sample of worlds must match stepping each
    alone.  At this size every block of the persistent kernels handles many
    worlds in a row, which is where a missing barrier between phases shows."""
    scs = scenes.batch_worlds(2048, 1000)
    for s in scs:
        engine.setup_scene(s)
    ws = [ctx.world(s) for s in scs]
    ctx.batch_step(ws, 1 / 60, 35)
    ctx.batch_step(ws, 1 / 60, 35)
    sample = list(range(0, 2048, 97)) + [2047]
    for i in sample:
        p = ctx.world(scs[i])
        p.step(1 / 60, 70)
        assert p.bodies().tobytes() == ws[i].bodies().tobytes(), scs[i].name
        p.destroy()
    for w in ws:
        w.destroy()


def test_bench_batch_every_world_equals_plain(ctx):
    """The benchmark's own 4096-world batch: every world after 20 batched
    steps (two calls, the second replaying the captured graph, with the
    autotuner switching kernel variants) equals the same world stepped alone
    through cp_world_step, bit for bit."""
    scs = scenes.batch_worlds(4096, 1000)  # rank 0's worlds in bench.py
    for s in scs:
        engine.setup_scene(s)
    ws = [ctx.world(s) for s in scs]
    ctx.batch_step(ws, 1 / 60, 10)
    ctx.batch_step(ws, 1 / 60, 10)
    bad = []
    for i, s in enumerate(scs):
        p = ctx.world(s)
        p.step(1 / 60, 20)
        if p.bodies().tobytes() != ws[i].bodies().tobytes():
            bad.append(s.name)
        p.destroy()
    for w in ws:
        w.destroy()
    assert not bad, f"{len(bad)} worlds differ from the plain path, first {bad[:5]}"


def test_every_kernel_variant_gives_the_same_bits(ctx):
    """The autotuner may switch kernel variants between steps: every variant
    (block size, register budget) must produce identical state."""
    scs = [scenes.column_world(int(n), 4000 + i, "sphere_box") for i, n in enumerate(scenes.batch_sizes(24, 6000))]
    for s in scs:
        engine.setup_scene(s)
    results = []
    count = len(ctx.autotune_info()["ms_per_variant"])
    assert count >= 8
    for v in range(count):
        ws = [ctx.world(s) for s in scs]
        ctx.set_variant(v)
        ctx.batch_step(ws, 1 / 60, 12)
        results.append(b"".join(w.bodies().tobytes() for w in ws))
        for w in ws:
            w.destroy()
    ctx.set_variant(-1)
    assert all(r == results[0] for r in results[1:])


def test_bad_arguments_raise(ctx):
    sc = engine.setup_scene(scenes.spheres_on_plane(4))
    w = ctx.world(sc)
    with pytest.raises(engine.CannonError):
        w.step(dt=-1.0)
    with pytest.raises(engine.CannonError):
        ctx.batch_step([w], 0.0, 1)
    w.destroy()
    with pytest.raises(engine.CannonError):
        w.id = 12345
        w.step()
