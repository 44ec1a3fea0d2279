"""The multi-rank path of bench.py on CPU: two gloo ranks, each timing its own
replica; the whole-job figure uses the slowest rank's time and all ranks'
agent-steps (no data-path collective, only the timing max-reduction)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, ws, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    assert bench.dist_env() == (ws, rank, rank)
    total_ms = 100.0 * (rank + 1)  # rank 1 is the slow one
    t_max, value = bench.whole_job(total_ms, 1000, 144, 10, ws, dist, "cpu")
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, t_max, value))


def test_two_gloo_ranks_take_the_slowest_time():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t_max, value in out:
        assert t_max == 200.0
        assert value == pytest.approx(1000 * 2 * 144 * 10 / 0.2)


def test_single_rank_needs_no_collective():
    import bench
    t_max, value = bench.whole_job(50.0, 2_000_000, 144, 4, 1)
    assert t_max == 50.0 and value == pytest.approx(2e6 * 144 * 4 / 0.05)


RANK_SCRIPT = r'''
import json, os, sys
sys.path.insert(0, {root!r})
import torch.distributed as dist
import bench
ws, rank, local = bench.dist_env()
dist.init_process_group("gloo")
t_max, value = bench.whole_job(100.0 * (rank + 1), 1000, 144, 10, ws, dist, "cpu")
if rank == 0:
    print(json.dumps({{"n_gpus": ws, "value": value, "ms": t_max, "local_ranks": ws}}))
with open(os.path.join({out!r}, "rank%d.json" % rank), "w") as f:
    json.dump({{"rank": rank, "local": local, "ws": ws}}, f)
dist.barrier()
dist.destroy_process_group()
'''


def test_launcher_starts_one_rank_per_gpu(tmp_path, capfd):
    """bench.launch_ranks (what `bench.py --gpus N` does outside torchrun) starts N
    ranks with RANK / LOCAL_RANK / WORLD_SIZE set; rank 0 prints the whole-job line."""
    import json
    import bench
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    script = tmp_path / "rank.py"
    script.write_text(RANK_SCRIPT.format(root=root, out=str(tmp_path)))
    env_ws = os.environ.pop("WORLD_SIZE", None)
    try:
        rc = bench.launch_ranks(2, [], script=str(script))
    finally:
        if env_ws is not None:
            os.environ["WORLD_SIZE"] = env_ws
    assert rc == 0
    ranks = sorted(json.loads((tmp_path / ("rank%d.json" % r)).read_text())["local"] for r in range(2))
    assert ranks == [0, 1]
    out = capfd.readouterr().out
    line = json.loads([x for x in out.splitlines() if x.startswith("{")][-1])
    assert line["n_gpus"] == 2 and line["ms"] == 200.0
    assert line["value"] == pytest.approx(1000 * 2 * 144 * 10 / 0.2)
