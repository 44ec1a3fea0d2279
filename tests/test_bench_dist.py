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
