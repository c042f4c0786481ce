#!/usr/bin/env python3
"""Batched World.step throughput on GB300: body-steps/s.

Workload (the batched form of cannon_physics' World.step): 4096 independent
worlds, body counts floor(exp(U[ln 8, ln 512])) plus a ground Plane each,
50/50 Sphere(0.5) / random Box, NaiveBroadphase, GSSolver 10 iterations,
dt 1/60, stepped together by one persistent launch per step (CUDA graph).
A step is one World.step of every world.  Body-steps count every body,
planes included.

Reported on one JSON line:
  value       device-timed body-steps/s (CUDA events on the library stream),
              state resident in HBM
  e2e         the same metric through the public C ABI with host buffers:
              per step cp_batch_set_forces (force/torque, pinned host -> device),
              cp_batch_step, cp_batch_get_poses (pose + velocities, device ->
              pinned host), timed by the host clock
  plain       the single-world drop-in path (cp_world_step) on a sample of the
              same worlds, and the batched/plain ratio
  roofline    HBM roofline of the step kernel (algorithmic bytes per body-step
              x body-steps / kernel time), peak from MEASURED_PEAKS.json
  cpu_baseline  the C++ oracle (a port of the reference) on the host cores,
              one world per thread, on a sample of the worlds

`--impl reference` times the reference algorithm on the CPU (the oracle port,
all host threads, one world per thread) on the same workload: the reference
is Dart + Flutter, neither of which exists on the box.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "body-steps/s batched vs plain on 1 GB300 at <=1e-9 rel; p50/p99 request latency"
UNIT = "body-steps/s"
ALG_BYTES_PER_BODY_STEP = 208  # binary32 state x,q,v,w and invInertiaWorld read+written, static per-body data read
DT = 1.0 / 60.0
# untimed steps before every arm's timed range: the columns have landed and
# the worlds are in contact by then (the autotuner's second round ends near
# call 62)
PREROLL = 80


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=120)
    ap.add_argument("--warmup", type=int, default=3, help="untimed steps before the autotuner's calls")
    ap.add_argument("--preroll", type=int, default=PREROLL,
                    help="every arm (GPU, e2e, plain, CPU baseline, reference) times steps preroll .. preroll+steps-1 "
                         "of the same worlds; the warm-up and autotuner calls are part of the GPU arm's pre-roll")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--worlds", type=int, default=4096)
    ap.add_argument("--plain-worlds", type=int, default=48)
    ap.add_argument("--cpu-sample", type=int, default=16, help="every k-th world goes into the CPU baseline sample")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-configs", action="store_true", help="skip the single-world configurations C1-C3")
    ap.add_argument("--serve-rate", type=float, default=2000.0, help="served form: Poisson arrival rate, requests/s")
    ap.add_argument("--serve-window", type=float, default=1.0, help="served form: seconds of arrivals")
    ap.add_argument("--serve-tick", type=int, default=4, help="served form: steps per tick")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--serve-lanes", type=int, default=0,
                    help="served form: wide lanes (threads stepping one large world each on the grid-wide path); 0 or -1: "
                         "none (the server's default)")
    ap.add_argument("--serve-wide-bodies", type=int, default=0,
                    help="served form: body count from which a request takes a wide lane; 0: the server's default")
    ap.add_argument("--variant", type=int, default=None,
                    help="pin the batched kernel variant (no autotuning): the step kernels then launch in a known order, "
                         "two per warm-up step, for profiling")
    return ap.parse_args()


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def rank_seed(rank, worlds):
    """Scene seed of a rank's world set: weak scaling, every rank steps its own
    `worlds` independent worlds and no data crosses ranks."""
    return 1000 + rank * worlds


def reduce_over_ranks(x, ws, op, device):
    """x reduced over the ranks ('max' for times, 'sum' for counts)."""
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


class Clocks:
    """nvidia-smi clock / throttle samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [ln.strip().split(",") for ln in self.f.read().splitlines() if ln.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except (ValueError, IndexError):
                continue
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic():
    """DRAM bytes per body-step of the two step kernels from the committed ncu
    summary (profiles/step_kernels_traffic.txt: 'dram_bytes_per_body_step: X')."""
    path = os.path.join(ROOT, "profiles", "step_kernels_traffic.txt")
    try:
        for ln in open(path):
            if ln.startswith("dram_bytes_per_body_step:"):
                return float(ln.split(":")[1])
    except OSError:
        pass
    return None


def profiled_fp64_ops():
    """Binary64 add, multiply and fused multiply-add thread-instructions per
    body-step of the two step kernels, from the committed ncu summary
    (profiles/step_kernels_fp64.txt: 'binary64_ops_per_body_step: X')."""
    path = os.path.join(ROOT, "profiles", "step_kernels_fp64.txt")
    try:
        for ln in open(path):
            if ln.startswith("binary64_ops_per_body_step:"):
                return float(ln.split(":")[1])
    except OSError:
        pass
    return None


# GB300's nominal binary64 rate: 1.25 TFLOP/s, i.e. 625 G fused multiply-adds
# (thread-instructions) per second
FP64_PEAK_G_PER_S = 625.0


def build_worlds(n, seed):
    from cannon_physics_gb300 import scenes
    return scenes.batch_worlds(n, seed)


def workload_config(n_worlds, total_bodies):
    return {"workload": f"batch_worlds: {n_worlds} independent worlds, bodies floor(exp(U[ln 8, ln 512])) + 1 Plane each "
                        f"({total_bodies} bodies), 50/50 Sphere(0.5)/Box(U[0.2,0.5]), NaiveBroadphase, GSSolver 10 iterations, "
                        "dt 1/60, one persistent launch per step (CUDA graph)",
            "worlds": n_worlds, "bodies": total_bodies, "arithmetic": "binary64 compute, binary32 vector storage (as Dart + vector_math)",
            "l2": "inputs larger than L2 (body state alone is ~240 MB)", "parity": "bit-exact vs oracle"}


def cpu_baseline(scenes_list, every, preroll, steps, threads=None):
    """The oracle port on the host cores, one world per thread, over the same
    step range as the timed GPU region (steps preroll .. preroll+steps-1)."""
    from oracle import oracle_py as O
    sample = scenes_list[::every]
    worlds = [O.OracleWorld(s) for s in sample]
    threads = threads or os.cpu_count() or 1
    bodies = sum(s.num_bodies for s in sample)
    O.step_parallel(worlds, DT, preroll, threads)
    t0 = time.perf_counter()
    O.step_parallel(worlds, DT, steps, threads)
    sec = time.perf_counter() - t0
    return {"value": bodies * steps / sec, "unit": UNIT, "cores": threads, "kind": "port",
            "timed_steps": [preroll, preroll + steps - 1],
            "sample": f"{len(sample)} of the worlds (every {every}th, {bodies} bodies), steps {preroll}..{preroll + steps - 1}, "
                      f"one world per thread, {threads} thread{'s' if threads > 1 else ''}"}


# The single-world configurations, each timed through the plain drop-in
# (one cp_world_step call per step, as GpuWorld.internalStep makes) and
# through the oracle on one host thread from the same state: name, scene,
# untimed pre-roll (mid-horizon, in contact), GPU steps timed, CPU steps timed
PLAIN_CONFIGS = [
    ("C1", "spheres_on_plane", "64 Sphere(0.5) on a Plane, NaiveBroadphase, GSSolver 10 iterations, dt 1/60", 300, 60, 60),
    ("C2", "box_pile", "4096 Box (half-extents U[0.2,0.5]) pile in a 16x16 footprint, SAPBroadphase x, GSSolver 20 iterations, "
                       "friction 0.4, dt 1/60", 150, 10, 3),
    ("C3", "mixed_chains", "8192 bodies 40/40/20 Sphere/Box/Cylinder(10), 128 chains of 16 (P2P/Hinge/Distance), "
                           "GridBroadphase cell 1, sleeping, GSSolver 15 iterations, dt 1/120", 120, 10, 3),
]


def plain_configs(ctx, only=None):
    from cannon_physics_gb300 import engine, scenes
    from oracle import oracle_py as O
    out = {}
    for name, make, desc, pre, k_gpu, k_cpu in PLAIN_CONFIGS:
        if only and name not in only:
            continue
        sc = engine.setup_scene(getattr(scenes, make)())
        w = ctx.world(sc)
        w.step(sc.dt, pre)
        t0 = time.perf_counter()
        for _ in range(k_gpu):
            w.step(sc.dt, 1)
        gsec = time.perf_counter() - t0
        inf = w.info()
        ow = O.OracleWorld(O.setup_scene(getattr(scenes, make)()))
        ow.load_state(w)
        t0 = time.perf_counter()
        ow.step(sc.dt, k_cpu)
        csec = time.perf_counter() - t0
        w.destroy()
        g = sc.num_bodies * k_gpu / gsec
        c = sc.num_bodies * k_cpu / csec
        out[name] = {"workload": desc, "bodies": sc.num_bodies, "ms_per_step": gsec * 1e3 / k_gpu, "value": g, "unit": UNIT,
                     "timed_steps": [pre, pre + k_gpu - 1], "pairs": inf.num_pairs, "contacts": inf.num_contacts,
                     "rows": inf.num_rows, "levels": inf.num_levels,
                     "cpu_1thread": {"ms_per_step": csec * 1e3 / k_cpu, "value": c, "kind": "port", "cores": 1,
                                     "timed_steps": [pre, pre + k_cpu - 1],
                                     "sample": "the oracle continued from the GPU world's state at the same step"},
                     "gpu_over_cpu_1thread": g / c}
    return out


SERVE_CLIENTS = 8


def serve_once(device, rate, window, seed, tick, lanes=0, wide_bodies=0, clients=SERVE_CLIENTS):
    """One served run: Poisson arrivals of rollout requests submitted on their
    arrival times to a fresh continuous-batching server (150 GB HBM budget)
    by `clients` client threads (request i from client i mod clients; a
    submission lays its world out on the client's thread, as a client
    process would); returns the request list, the scenes and the server's
    statistics."""
    import threading
    from cannon_physics_gb300 import engine, scenes
    from cannon_physics_gb300 import serve as S
    reqs = scenes.serve_requests(rate=rate, window=window, seed=seed)
    built = [engine.setup_scene(scenes.request_world(r)) for r in reqs]
    srv = S.Server(device=device, hbm_budget=150e9, steps_per_tick=tick, wide_lanes=lanes, wide_bodies=wide_bodies)
    warm = engine.setup_scene(scenes.request_world(scenes.Request(0.0, 64, 2, 5)))
    t = srv.submit(warm, warm.dt, 2)
    srv.wait(t)
    srv.result(t)
    srv.stats(reset=True)
    tickets = [None] * len(reqs)
    lag = [0.0]

    t0 = time.perf_counter() + 0.05

    def client(c):
        for i in range(c, len(reqs), clients):
            r, sc = reqs[i], built[i]
            delay = t0 + r.arrival - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            else:
                lag[0] = max(lag[0], -delay)
            tickets[i] = srv.submit(sc, sc.dt, r.horizon)

    clocks = Clocks(device)
    clocks.start()
    ths = [threading.Thread(target=client, args=(c,)) for c in range(clients)]
    for th in ths:
        th.start()
    for th in ths:
        th.join()
    for t in tickets:
        if srv.wait(t) != S.DONE:
            raise RuntimeError(f"served request {t} did not complete")
        srv.result(t)
    clk = clocks.stop()
    st = srv.stats()
    srv.close()
    offered = sum(sc.num_bodies * r.horizon for r, sc in zip(reqs, built))
    return reqs, built, {
        "rate_req_per_s": rate, "window_s": window, "requests": len(reqs), "completed": st["completed"],
        "value": st["body_steps"] / st["span_s"], "unit": UNIT,
        "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "mean_ms": st["mean_ms"], "max_ms": st["max_ms"],
        "offered_body_steps_per_s": offered / window, "span_s": st["span_s"], "clients": clients,
        "submit_lag_max_s": lag[0],
        "ticks": st["ticks"], "steps_per_tick": tick,
        "step_s": st["device_s"],  # time the server thread spent in step launches (the rest: admission, uploads, results)
        "bytes_peak_gb": st["bytes_peak"] / 1e9, "clocks": clk}


def run_served(args, device):
    """The served form: rollout requests (worlds of floor(exp(U[ln 16,
    ln 4096])) bodies in the 40/40/20 sphere/box/cylinder mix, horizons
    U{1..240}, dt 1/60) arriving as a Poisson process.  Two load points: the
    workload's own 2000 requests/s (about 40 times what one GB300 sustains, so
    its latency measures the queue) and 70 % of the throughput measured there
    (a sustainable load, whose latency measures the server).  Latency is
    submission to result ready; throughput is completed body-steps over the
    span from the first submission to the last completion."""
    from cannon_physics_gb300 import engine
    reqs, built, over = serve_once(device, args.serve_rate, args.serve_window, 77, args.serve_tick, args.serve_lanes,
                                   args.serve_wide_bodies)
    mean_req = over["offered_body_steps_per_s"] * args.serve_window / max(1, len(reqs))
    rate70 = 0.7 * over["value"] / mean_req
    window70 = max(4.0, 150.0 / rate70)
    _, _, sus = serve_once(device, rate70, window70, 78, args.serve_tick, args.serve_lanes, args.serve_wide_bodies)
    # the plain per-request path: a sample of the same requests, each alone
    # through cp_world_step
    ctx = engine.Context(device=device)
    sample = list(range(0, len(reqs), max(1, len(reqs) // 12)))[:12]
    t0 = time.perf_counter()
    plain_bs = 0
    for i in sample:
        w = ctx.world(built[i])
        w.step(built[i].dt, reqs[i].horizon)
        w.bodies()
        w.destroy()
        plain_bs += built[i].num_bodies * reqs[i].horizon
    plain_sec = time.perf_counter() - t0
    ctx.close()
    plain = plain_bs / plain_sec
    return dict(over, **{
        "workload": f"Poisson arrivals at {args.serve_rate:g} req/s for {args.serve_window:g} s ({len(reqs)} requests), "
                    "worlds floor(exp(U[ln 16, ln 4096])) bodies + Plane, 40/40/20 Sphere/Box/Cylinder(10), NaiveBroadphase, "
                    "GSSolver 10 iterations, dt 1/60, horizons U{1..240}; HBM budget 150 GB",
        "sustainable": dict(sus, note="70 % of the throughput measured at the overload point; latency here is the server's, "
                                      "not a queue's"),
        "plain_per_request": {"value": plain, "unit": UNIT,
                              "sample": f"{len(sample)} of the requests, each alone through cp_world_step ({plain_bs} body-steps)"},
        "served_over_plain": over["value"] / plain,
    })


def run_ours(args):
    import numpy as np
    import torch
    ws, rank, local = dist_info()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from cannon_physics_gb300 import build as B
    from cannon_physics_gb300 import engine

    B.build()
    scs = build_worlds(args.worlds, rank_seed(rank, args.worlds))
    for s in scs:
        engine.setup_scene(s)
    ctx = engine.Context(device=local)
    worlds = [ctx.world(s) for s in scs]
    batch = engine.Batch(ctx, worlds)
    total = batch.total
    ext = torch.cuda.ExternalStream(ctx.stream_handle())
    if args.variant is not None:
        ctx.set_variant(args.variant)

    for _ in range(args.warmup):
        batch.step(DT)
    calls = args.warmup
    # the autotuner times one kernel variant per batched call; it tunes again
    # once the worlds are in contact (call 48)
    while args.variant is None and (ctx.autotune_info()["variant"] < 0 or calls < 48) and calls < args.preroll:
        batch.step(DT)
        calls += 1
    if args.variant is None and ctx.autotune_info()["variant"] < 0:
        raise SystemExit(f"--preroll {args.preroll} ends before the autotuner has chosen a kernel variant")
    tune_calls = calls - args.warmup
    while calls < args.preroll:
        batch.step(DT)
        calls += 1
    timed = [args.preroll, args.preroll + args.steps - 1]
    # a second copy of the worlds for the end-to-end leg, at the same step
    e2e_worlds = [ctx.world(s) for s in scs]
    e2e_batch = engine.Batch(ctx, e2e_worlds)
    for _ in range(args.preroll):
        e2e_batch.step(DT)
    ctx.batch_profile()
    ctx.phase_profile()

    def barrier():
        if ws > 1:
            torch.distributed.barrier()

    # device-timed throughput, state resident
    clocks = Clocks(local)
    barrier()
    torch.cuda.synchronize()
    launches0 = ctx.launches()
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    for _ in range(args.steps):
        batch.step(DT)
    e1.record(ext)
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier()
    launches = ctx.launches() - launches0
    ms = e0.elapsed_time(e1)
    graph_ms, graph_steps = ctx.batch_profile()
    phases = ctx.phase_profile()
    ms = reduce_over_ranks(ms, ws, "max", "cuda")
    job_bodies = reduce_over_ranks(total, ws, "sum", "cuda")  # each rank its own worlds
    value = job_bodies * args.steps / (ms / 1e3)

    # end to end through the C ABI with pinned host buffers, on the second
    # copy of the worlds over the same steps
    ft = torch.zeros(total * 6, dtype=torch.float32, pin_memory=True)
    poses = torch.empty(total * 13, dtype=torch.float32, pin_memory=True)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_batch.set_forces(ft.data_ptr())
        e2e_batch.step(DT)
        e2e_batch.get_poses(poses.data_ptr())
    e2e_sec = time.perf_counter() - t0
    barrier()
    e2e_sec = reduce_over_ranks(e2e_sec, ws, "max", "cuda")
    e2e = {"value": job_bodies * args.steps / e2e_sec, "unit": UNIT, "h2d_bytes_per_step": total * 6 * 4,
           "d2h_bytes_per_step": total * 13 * 4, "steps": args.steps, "timed_steps": timed}
    assert np.isfinite(poses.numpy()).all()
    for w in e2e_worlds:
        w.destroy()

    # plain single-world path on a sample of the same worlds (fresh copies,
    # same pre-roll, same timed steps), one cp_world_step call per step as
    # GpuWorld.internalStep makes
    idx = np.linspace(0, len(scs) - 1, args.plain_worlds).astype(int)
    plain_worlds = [ctx.world(scs[i]) for i in idx]
    for w in plain_worlds:
        w.step(DT, args.preroll)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for w in plain_worlds:
        for _ in range(args.steps):
            w.step(DT, 1)
    plain_sec = time.perf_counter() - t0
    plain_bodies = sum(w.n for w in plain_worlds)
    plain = {"value": plain_bodies * args.steps / plain_sec, "unit": UNIT, "timed_steps": timed,
             "sample": f"{len(plain_worlds)} of the worlds ({plain_bodies} bodies), one cp_world_step call per step"}
    for w in plain_worlds:
        w.destroy()
    configs = plain_configs(ctx) if not args.no_configs else None

    if rank != 0:
        ctx.close()
        return
    peak, peak_kind = peaks()
    kernel_ms = graph_ms / max(graph_steps, 1)
    achieved = ALG_BYTES_PER_BODY_STEP * total / (kernel_ms / 1e3) / 1e9
    traffic_per_bs = profiled_traffic()
    fp64_per_bs = profiled_fp64_ops()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "timed_steps": timed,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded SplitMix64 scenes; the reference publishes no benchmark scenes)",
        "config": workload_config(args.worlds, total),
        "e2e": e2e,
        "plain": plain,
        "batched_over_plain": value / ws / plain["value"],
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "kernel": "k_step_pre + k_step_solve (one step)",
                     "alg_bytes_per_body_step": ALG_BYTES_PER_BODY_STEP, "kernel_ms": kernel_ms,
                     "traffic": None if traffic_per_bs is None else traffic_per_bs * total,
                     "note": "bound by binary64 issue (64 cycles per warp instruction per sub-partition on GB300), barriers and load latency, not HBM bandwidth; traffic is DRAM bytes of one step from the committed ncu capture, scaled by bodies"},
        "fp64": None if fp64_per_bs is None else {
            "ops_per_body_step": fp64_per_bs, "achieved": fp64_per_bs * value / ws / 1e9, "peak": FP64_PEAK_G_PER_S,
            "unit": "G binary64 thread-instructions/s per GPU", "frac": fp64_per_bs * value / ws / 1e9 / FP64_PEAK_G_PER_S,
            "peak_kind": "nominal (1.25 TFLOP/s)",
            "note": "add, multiply and fused multiply-add instructions per body-step from the committed ncu capture; "
                    "the binary64 pipe itself is 45-52 % busy because most binary64 warp instructions run with part of their lanes"},
        "gpu_launches": launches,
        "clocks": clk,
        "autotune": dict(ctx.autotune_info(), warmup_calls=args.warmup, tune_calls=tune_calls, preroll=args.preroll),
        "plain_configs": configs,
        "phase_share": {k: round(v / max(sum(phases.values()), 1.0), 4) for k, v in phases.items()},
    }
    ctx.close()
    if not args.no_serve:
        line["served"] = run_served(args, local)
        line["served"]["served_over_batched"] = line["served"]["value"] / (value / ws)
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(scs, args.cpu_sample, args.preroll, args.steps)
        line["cpu_baseline_1thread"] = cpu_baseline(scs, 4 * args.cpu_sample, args.preroll, args.steps, threads=1)
    print(json.dumps(line), flush=True)


def run_reference(args):
    ws, rank, local = dist_info()
    if rank != 0:
        return
    from oracle import oracle_py as O
    scs = build_worlds(args.worlds, 1000)
    for s in scs:
        O.setup_scene(s)
    worlds = [O.OracleWorld(s) for s in scs]
    threads = os.cpu_count() or 1
    total = sum(s.num_bodies for s in scs)
    O.step_parallel(worlds, DT, args.preroll, threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        O.step_parallel(worlds, DT, 1, threads)
    sec = time.perf_counter() - t0
    value = total * args.steps / sec
    timed = [args.preroll, args.preroll + args.steps - 1]
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "timed_steps": timed, "ms_per_step": sec * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": workload_config(args.worlds, total),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "timed_steps": timed,
                             "sample": f"all {args.worlds} worlds, steps {timed[0]}..{timed[1]} after {args.preroll} untimed "
                                       "steps; the Dart reference needs a Flutter SDK, absent here and on the GPU box, "
                                       "so its C++ port (oracle/) runs it"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
