"""The multi-rank host path of bench.py on CPU: two processes over gloo.

Worlds are independent, so ranks share no data: each rank steps its own
world set (its own seed), and the only cross-rank operations are the
barrier and the reductions of the bench's timing (max over ranks) and body
counts (sum over ranks).  The reference arm runs on rank 0 alone.
"""
import contextlib
import io
import json
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, out_dir):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    from cannon_physics_gb300 import scenes

    res = {"rank": rank}
    assert bench.dist_info() == (ws, rank, rank)
    # timing: the slowest rank; counts: the sum
    res["max"] = bench.reduce_over_ranks(1.5 + rank, ws, "max", "cpu")
    res["sum"] = bench.reduce_over_ranks(10.0 * (rank + 1), ws, "sum", "cpu")
    # each rank its own worlds
    seed = bench.rank_seed(rank, 4)
    worlds = scenes.batch_worlds(4, seed)
    res["seed"] = seed
    res["bodies"] = sum(w.num_bodies for w in worlds)
    res["first_pos"] = [float(v) for v in worlds[0].bodies["position"][1]]
    dist.barrier()
    # the reference arm: rank 0 alone works and prints
    buf = io.StringIO()
    if rank != 0:
        sys.argv = ["bench.py", "--impl", "reference", "--worlds", "2", "--steps", "1", "--warmup", "0"]
        with contextlib.redirect_stdout(buf):
            bench.run_reference(bench.parse())
    res["ref_output"] = buf.getvalue()
    dist.destroy_process_group()
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump(res, f)


def test_two_ranks_over_gloo(tmp_path):
    ws = 2
    mp.spawn(_rank_main, args=(ws, _free_port(), str(tmp_path)), nprocs=ws, join=True)
    r = [json.load(open(tmp_path / f"rank{i}.json")) for i in range(ws)]
    assert r[0]["max"] == r[1]["max"] == 2.5
    assert r[0]["sum"] == r[1]["sum"] == 30.0
    assert r[0]["seed"] != r[1]["seed"]
    assert r[0]["first_pos"] != r[1]["first_pos"]  # different world sets per rank
    assert r[1]["ref_output"] == ""  # rank 1 of the reference arm does no work


def test_single_rank_reductions_are_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_over_ranks(3.25, 1, "max", "cpu") == 3.25
    assert bench.reduce_over_ranks(7, 1, "sum", "cpu") == 7
    assert bench.rank_seed(0, 4096) == 1000 and bench.rank_seed(1, 4096) == 1000 + 4096
