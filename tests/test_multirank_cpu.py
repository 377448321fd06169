"""The benchmark's multi-rank plumbing (one process per GPU under torchrun)
on the CPU: two gloo ranks rendezvous on 127.0.0.1, meet at the barrier and
agree on the maximum of their step times (the time the JSON line reports).
The wavelet path has no data-path collective: ranks run independent
replicas (weak scaling), so this is all the exchange there is."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist()
    d.barrier()
    m = d.max(1.5 + rank)
    d.barrier()
    out.put((rank, d.rank, d.world, m))
    d.td.destroy_process_group()


def test_two_gloo_ranks_barrier_and_max():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 0, 2, 2.5), (1, 1, 2, 2.5)]
