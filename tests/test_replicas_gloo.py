"""The multi-GPU form of the bench: N independent replicas combined on the
host (maximum step time over ranks, value counting every rank's work), run
here as two gloo processes on the CPU."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q) -> None:
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench._barrier()
    res = {"ms_per_step": 10.0 + 5.0 * rank, "value": 0.0,
           "config": {"edge_updates_per_step": 1000}}
    out = bench.combine_replicas(res, world, "cpu")
    q.put((rank, out["ms_per_step"], out["value"], out["n_gpus"]))
    dist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    got = sorted(q.get(timeout=5) for _ in range(world))
    for rank, ms, value, n in got:
        assert ms == 15.0 and n == world
        assert value == pytest.approx(world * 1000 / 0.015)
