"""CPU: the benchmark's multi-process host logic (barrier and maximum time over ranks)
with two gloo ranks, as torchrun runs it with one process per GPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, results):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    ranks = bench.Ranks()
    ranks.barrier()
    results[rank] = (ranks.world, ranks.device, ranks.max(10.0 + rank))
    ranks.close()


def test_two_gloo_ranks_agree_on_the_slowest_time():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    port = _free_port()
    with mp.Manager() as manager:
        results = manager.dict()
        procs = [mp.Process(target=_rank_main, args=(r, 2, port, results)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        assert dict(results) == {0: (2, 0, 11.0), 1: (2, 1, 11.0)}
