"""bench.py's replica aggregation (--gpus N under torchrun): whole-job value is every
rank's particle-steps over the slowest rank's time.  world_size 2 over gloo on CPU."""
import os
import socket
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def test_combine_replicas_uses_slowest_rank():
    r = bench.combine_replicas([1000, 3000], [10.0, 20.0], steps=5)
    assert r["value"] == pytest.approx(4000 / 0.020)
    assert r["ms_per_step"] == pytest.approx(4.0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench.barrier()
    res = {"units": 100 * (rank + 1), "ms_per_step": 2.0 + rank, "steps": 10, "value": -1.0}
    bench.gather_replicas(res)
    out[rank] = (res["value"], res["ms_per_step"], res["n_gpus"])
    dist.destroy_process_group()


def test_gather_replicas_world2_gloo():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    # 300 particle-steps over the slower rank's 30 ms, identical on both ranks
    for r in range(2):
        v, ms, n = res[r]
        assert v == pytest.approx(300 / 0.030) and ms == pytest.approx(3.0) and n == 2
