"""The multi-GPU form on the host, without a GPU: `bench.py --gpus N` runs one
independent view per rank (replicas, no data-path collective), takes the
slowest rank's time, and only rank 0 prints.  Two gloo ranks on CPU."""
import json
import os
import socket
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(REPO))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ws, r, local = bench.dist_env()
    times = bench.max_over_ranks([10.0 + rank, 5.0 - rank])  # each rank's step time and e2e time
    view = bench.make_view("plain_small", r)
    Path(out_dir, "rank%d.json" % rank).write_text(json.dumps({
        "ws": ws, "rank": r, "local": local, "times": times,
        "light0": [float(x) for x in view.lights[0, :3]], "lights": int(view.light_count)}))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    port = _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = [json.loads((tmp_path / ("rank%d.json" % r)).read_text()) for r in range(2)]
    for r, d in enumerate(res):
        assert (d["ws"], d["rank"], d["local"]) == (2, r, r)
        assert d["times"] == [11.0, 5.0]  # MAX over ranks, every rank gets it
    # each replica culls its own view (weak scaling: per-GPU work is fixed)
    assert res[0]["lights"] == res[1]["lights"] and res[0]["light0"] != res[1]["light0"]


def test_reference_arm_prints_on_rank_zero_only(monkeypatch, capsys):
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")

    class Args:
        workload, steps, warmup = "plain_small", 1, 0
    assert bench.run_reference_arm(Args()) is None
    assert capsys.readouterr().out == ""
    assert bench.max_over_ranks([3.0, 4.0]) == [3.0, 4.0]  # no process group: the identity
