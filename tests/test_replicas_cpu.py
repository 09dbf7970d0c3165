"""The N>1 path of bench.py on CPU: two gloo ranks, each running its own
model (the oracle on CPU, the GPU library on a GPU), with no data-path
collective; only the timing reduction crosses ranks."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    for p in (ROOT, os.path.join(ROOT, "hail-caesar_gb300"), os.path.join(ROOT, "oracle")):
        sys.path.insert(0, p)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    import oracle
    import synth
    case = synth.reach_case(imax=40, jmax=16, DX=10.0, hours=24, hydro_only=True, seed=rank + 1)
    o = oracle.Oracle(case)
    rec = o.iterate(50 + 25 * rank)  # ranks do different amounts of work
    ms = 10.0 * (rank + 1)
    got = bench.aggregate_replicas(ms, len(rec), dist)
    q.put((rank, got, float(rec[-1][1])))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replicas_gloo():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res = {r: (g, c) for r, g, c in out}
    # every rank sees the slowest rank's time and the total of both ranks' steps
    for r in range(world):
        assert res[r][0] == (20.0, 125.0)
    # the replicas are independent models (different seeds, different clocks)
    assert res[0][1] != res[1][1]
