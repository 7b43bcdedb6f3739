"""View sharding over two gloo ranks on CPU: ownership, ordering of the all-gather, a rank with fewer views, and a
rank that fails between steps (detected by the others through the process group's timeout, no GPU involved)."""

from __future__ import annotations

import datetime
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from citrus_gb300.view_sharding import gather_signals, owned_views, sharded_scatter_stage


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _fake_view(v: int, angle: float) -> torch.Tensor:
    return torch.full((3, 4), float(v)) + angle


def _worker(rank: int, world: int, port: int, num_views: int, queue):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=30))
    angles = [0.1 * v for v in range(num_views)]
    out = sharded_scatter_stage(_fake_view, angles, (3, 4))
    queue.put((rank, out))
    dist.destroy_process_group()


def _failing_worker(rank: int, world: int, port: int, queue):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=3))
    angles = [0.0, 1.0, 2.0, 3.0]
    sharded_scatter_stage(_fake_view, angles, (3, 4))  # step 1 succeeds on both ranks
    if rank == 1:
        os._exit(0)  # leaves between steps, nothing in flight
    try:
        sharded_scatter_stage(_fake_view, angles, (3, 4))
        queue.put((rank, "no error"))
    except Exception as e:  # noqa: BLE001
        queue.put((rank, f"error: {type(e).__name__}"))


def test_owned_views_partition():
    for world in (1, 2, 3, 5):
        views = sorted(v for r in range(world) for v in owned_views(11, r, world))
        assert views == list(range(11))
    with pytest.raises(ValueError):
        owned_views(4, 2, 2)


@pytest.mark.parametrize("num_views", [4, 5, 1])
def test_two_rank_gather_is_in_view_order(num_views):
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, num_views, queue)) for r in range(2)]
    for p in procs:
        p.start()
    results = dict(queue.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    expected = torch.stack([_fake_view(v, 0.1 * v) for v in range(num_views)])
    for r in range(2):
        assert torch.equal(results[r], expected)


def test_a_rank_leaving_between_steps_is_reported_by_the_collective():
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_failing_worker, args=(r, 2, port, queue)) for r in range(2)]
    for p in procs:
        p.start()
    rank, message = queue.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        if p.is_alive():
            p.kill()
    assert rank == 0 and message.startswith("error")
