"""CPU: the replica path of the benchmark (one process per GPU, no collective on
the data path) aggregates correctly over two gloo ranks: the job's time is the
slowest rank's, its rate the units of every rank over that time."""
import os
import socket

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    dist, r, ws, local = bench._dist()
    assert (r, ws, local) == (rank, world, rank)
    ms = 100.0 + 50.0 * rank                      # rank 1 is the slow one
    ms_max, rate = bench.replica_rate(dist, ws, 1.0e6, ms)
    q.put((rank, ms_max, rate, dist.get_backend()))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_replicas_aggregate_on_the_slowest_rank():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    ps = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms_max, rate, backend in out:
        assert backend == "gloo"
        assert ms_max == 150.0
        assert rate == pytest.approx(2 * 1.0e6 / 0.150)


def test_single_process_needs_no_process_group():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench._dist() == (None, 0, 1, 0) or os.environ.get("WORLD_SIZE", "1") != "1"
    assert bench.replica_rate(None, 1, 5.0e5, 250.0) == (250.0, 2.0e6)
