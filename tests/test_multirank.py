"""The N > 1 path of bench.py on CPU: two gloo ranks (replicas, no collective
on the data path; the only collective is the max over ranks of the timed
region), and the reference arm's rank-0-only rule."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    # rank r "took" 100*(r+1) ms for 3 steps of 1e9 pixel-iterations each
    max_ms, value = bench.aggregate_over_ranks(100.0 * (rank + 1), 10 ** 9, 3, world)
    q.put((rank, max_ms, value))
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, max_ms, value in got:
        assert max_ms == 200.0
        assert abs(value - 2 * 3 * 1e9 / 0.2 / 1e9) < 1e-9  # both replicas' work over the slowest time


def test_reference_arm_only_on_rank_zero(monkeypatch, capsys):
    import sys
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class Args:
        gpus, steps, warmup = 2, 1, 1
    bench.run_reference(Args())
    assert capsys.readouterr().out == ""
