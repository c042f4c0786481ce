"""The served form (cp_serve_*): continuous batching under an HBM budget.

A request's result must be the same alone, in a mix of requests that arrive
while others are on the device, and through the plain per-world path
(cp_world_step): bit for bit, the tolerance of every parity test here.
"""
import time

import pytest

from cannon_physics_gb300 import engine, scenes
from cannon_physics_gb300 import serve as S

pytestmark = pytest.mark.gpu


def _requests(n, seed, lo=16, hi=400, max_horizon=40):
    reqs = scenes.serve_requests(rate=1000.0, window=10.0, seed=seed, lo=lo, hi=hi, max_horizon=max_horizon)[:n]
    return [(r, engine.setup_scene(scenes.request_world(r))) for r in reqs]


def _plain(ctx, sc, horizon):
    w = ctx.world(sc)
    w.step(sc.dt, horizon)
    out = w.bodies()
    w.destroy()
    return out


@pytest.fixture(scope="module")
def ctx():
    c = engine.Context(device=0)
    yield c
    c.close()


def test_served_result_is_the_same_alone_in_the_mix_and_plain(ctx):
    reqs = _requests(40, seed=11)
    probe_req, probe = reqs[17]
    srv = S.Server(hbm_budget=8e9, steps_per_tick=3)
    # alone
    t = srv.submit(probe, probe.dt, probe_req.horizon)
    assert srv.wait(t, 120.0) == S.DONE
    alone, info = srv.result(t)
    assert info.stepnumber == probe_req.horizon
    # in a mix: half the requests first, the rest (the probe among them) once
    # the first ones are running on the device
    tickets = {}
    for i, (r, sc) in enumerate(reqs[:20]):
        tickets[i] = srv.submit(sc, sc.dt, r.horizon)
    deadline = time.time() + 60
    while not any(srv.poll(tickets[i]) == S.ACTIVE for i in range(20)):
        assert time.time() < deadline
        time.sleep(0.001)
    overlapped = any(srv.poll(tickets[i]) == S.ACTIVE for i in range(20))
    for i, (r, sc) in enumerate(reqs[20:], start=20):
        tickets[i] = srv.submit(sc, sc.dt, r.horizon)
    results = {}
    for i, t in tickets.items():
        assert srv.wait(t, 300.0) == S.DONE
        results[i], inf = srv.result(t)
        assert inf.stepnumber == reqs[i][0].horizon
    assert overlapped
    mixed = results[17]
    plain = _plain(ctx, probe, probe_req.horizon)
    assert alone.tobytes() == mixed.tobytes()
    assert plain.tobytes() == mixed.tobytes()
    for i in (0, 5, 33, 39):
        r, sc = reqs[i]
        assert _plain(ctx, sc, r.horizon).tobytes() == results[i].tobytes(), sc.name
    st = srv.stats()
    assert st["completed"] == 41 and st["failed"] == 0
    assert st["p99_ms"] >= st["p50_ms"] > 0
    steps = sum(sc.num_bodies * r.horizon for r, sc in reqs) + probe.num_bodies * probe_req.horizon
    assert st["body_steps"] == steps
    srv.close()


def test_admission_keeps_within_the_budget(ctx):
    reqs = _requests(12, seed=23, lo=250, hi=300, max_horizon=20)
    # room for about three of these worlds at a time
    srv = S.Server(hbm_budget=1e9, steps_per_tick=2)
    t0 = srv.submit(reqs[0][1], reqs[0][1].dt, 1)
    srv.wait(t0, 60.0)
    srv.result(t0)
    one = srv.stats(reset=True)["bytes_peak"]
    srv.close()
    budget = int(3.5 * one)
    srv = S.Server(hbm_budget=budget, steps_per_tick=2)
    tickets = [srv.submit(sc, sc.dt, r.horizon) for r, sc in reqs]
    for t in tickets:
        assert srv.wait(t, 300.0) == S.DONE
    out = [srv.result(t)[0] for t in tickets]
    st = srv.stats()
    assert 0 < st["bytes_peak"] <= budget
    assert st["bytes_in_use"] == 0 and st["active"] == 0 and st["pending"] == 0
    for i in (0, 7, 11):
        r, sc = reqs[i]
        assert _plain(ctx, sc, r.horizon).tobytes() == out[i].tobytes()
    srv.close()


def test_request_larger_than_the_budget_is_refused():
    (r, sc), = _requests(1, seed=31, lo=300, hi=301)
    srv = S.Server(hbm_budget=1 << 20)
    with pytest.raises(engine.CannonError) as e:
        srv.submit(sc, sc.dt, 5)
    assert e.value.status == 2  # CP_ERR_CAPACITY
    srv.close()


def test_cancel_pending_and_active_requests():
    reqs = _requests(4, seed=41, lo=200, hi=220, max_horizon=2)
    srv = S.Server(hbm_budget=8e9, steps_per_tick=1, max_active_bodies=1)
    # max_active_bodies=1 admits one world at a time: the others wait
    tickets = [srv.submit(sc, sc.dt, 200) for r, sc in reqs]
    deadline = time.time() + 60
    while srv.poll(tickets[0]) != S.ACTIVE:
        assert time.time() < deadline
        time.sleep(0.001)
    srv.cancel(tickets[2])  # still queued
    srv.cancel(tickets[0])  # running
    assert srv.wait(tickets[0], 60.0) == S.CANCELLED
    assert srv.wait(tickets[2], 60.0) == S.CANCELLED
    for t in (tickets[1], tickets[3]):
        assert srv.wait(t, 300.0) == S.DONE
        srv.result(t)
    with pytest.raises(engine.CannonError):
        srv.result(tickets[2])
    st = srv.stats()
    assert st["cancelled"] == 2 and st["completed"] == 2
    srv.close()


def _dense_cluster(seed=99, n=300):
    """300 spheres in a 1.2 m cube: far more pairs than a world of 301 bodies
    starts with room for (4 * 301 + 64), so its lists must grow."""
    sc = scenes.spheres_on_plane(n)
    rng = scenes.SplitMix64(seed)
    sc.bodies["position"][1:] = rng.uniform(3 * n).reshape(n, 3) * 1.2 + (-0.6, 0.6, -0.6)
    return engine.setup_scene(sc)


def test_a_world_that_cannot_grow_fails_alone(ctx):
    """With max_list_entries below what a dense cluster needs, that request
    fails with CP_ERR_CAPACITY; the requests stepped in the same ticks
    complete and equal their plain results."""
    reqs = _requests(10, seed=51, lo=16, hi=200, max_horizon=12)
    bad = _dense_cluster()
    srv = S.Server(hbm_budget=8e9, steps_per_tick=2, max_list_entries=2048)
    tickets = [srv.submit(sc, sc.dt, r.horizon) for r, sc in reqs[:5]]
    tb = srv.submit(bad, bad.dt, 6)
    tickets += [srv.submit(sc, sc.dt, r.horizon) for r, sc in reqs[5:]]
    assert srv.wait(tb, 120.0) == S.FAILED
    for t, (r, sc) in zip(tickets, reqs):
        assert srv.wait(t, 120.0) == S.DONE
        out, inf = srv.result(t)
        assert inf.stepnumber == r.horizon
        assert _plain(ctx, sc, r.horizon).tobytes() == out.tobytes(), sc.name
    st = srv.stats()
    assert st["failed"] == 1 and st["completed"] == len(reqs)
    srv.close()


def test_served_requests_of_the_full_size_range_match_the_oracle():
    """Requests drawn from the served workload's own distribution (16 to 4096
    bodies in the 40/40/20 sphere/box/cylinder mix), including worlds above
    the solve kernel's shared-memory group limit (640 bodies per 128 threads)
    next to small ones, each checked against the oracle at its horizon: once
    with every world in the ticks (the default), once with two wide lanes
    taking the worlds of 1024 bodies or more onto the grid-wide kernels."""
    from oracle import oracle_py as O
    reqs = scenes.serve_requests(rate=2000.0, window=1.0, seed=77)
    big = [r for r in reqs if r.n_bodies > 2000][:2]
    mid = [r for r in reqs if 640 < r.n_bodies <= 2000][:3]
    small = [r for r in reqs if r.n_bodies <= 200][:6]
    chosen = big + mid + small
    assert len(big) == 2 and len(mid) == 3
    built = []
    for r in chosen:
        r.horizon = min(r.horizon, 24)  # keeps the oracle's share of the test short
        built.append((r, engine.setup_scene(scenes.request_world(r))))
    expect = []
    for r, sc in built:
        ow = O.OracleWorld(O.setup_scene(scenes.request_world(r)))
        ow.step(sc.dt, r.horizon)
        expect.append(ow.bodies().tobytes())
    for lanes in (0, 2):
        srv = S.Server(hbm_budget=20e9, steps_per_tick=4, wide_lanes=lanes)
        tickets = [srv.submit(sc, sc.dt, r.horizon) for r, sc in built]
        for t, (r, sc), want in zip(tickets, built, expect):
            assert srv.wait(t, 600.0) == S.DONE
            out, inf = srv.result(t)
            assert out.tobytes() == want, f"lanes {lanes}: {sc.name} ({sc.num_bodies} bodies)"
        srv.close()
