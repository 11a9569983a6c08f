"""The benchmark's multi-rank path on CPU: two gloo ranks (127.0.0.1), as
torchrun launches them.  Each rank runs its own events (weak scaling, no
collective on the data path); the step time is the max over ranks and the
event count the sum."""
import json
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_dir):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    r, w, local, pg = bench.dist()
    bench.barrier(pg)
    res = {"rank": r, "world": w, "local": local,
           "max": bench.allmax(pg, 10.0 * (r + 1)), "sum": bench.allsum(pg, 64.0),
           "plan": bench.headline_plan(r, 128), "single": bench.single_plan(r, 4)}
    bench.barrier(pg)
    pg.destroy_process_group()
    with open(os.path.join(out_dir, "rank%d.json" % r), "w") as f:
        json.dump(res, f)


def test_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    res = [json.load(open(tmp_path / ("rank%d.json" % k))) for k in range(2)]
    for k, r in enumerate(res):
        assert r["rank"] == k and r["world"] == 2
        assert r["max"] == 20.0 and r["sum"] == 128.0
    seeds = [set(s for s, _ in r["plan"]) | set(s for s, _ in r["single"]) for r in res]
    assert len(seeds[0]) == 132 and len(seeds[1]) == 132 and not (seeds[0] & seeds[1])
    assert all(150.0 <= pu <= 300.0 for r in res for _, pu in r["plan"])
