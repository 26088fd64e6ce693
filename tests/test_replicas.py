"""The bench's multi-GPU form is replicas (the path has no exchange step):
world-size-2 gloo ranks on the CPU exercise its host logic -- process-group
set-up, the barrier before timing, the max of the ranks' times and the
whole-job rate -- without a GPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    r, w, local = bench.dist_env()
    bench.init_replicas(w, local, backend="gloo")
    bench.replica_barrier(w)
    mx = bench.max_over_ranks(times[r], w, device="cpu")
    rate = bench.replica_rate(1920 * 1080, 10, w, mx)
    import torch.distributed as dist
    dist.destroy_process_group()
    q.put((r, mx, rate))


def test_two_gloo_replicas():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    times = [12.5, 20.0]  # ms: rank 1 is the slow one
    procs = [mp.Process(target=_rank, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(r for r, _, _ in res) == [0, 1]
    for _, mx, rate in res:
        assert mx == 20.0  # every rank sees the slowest rank's time
        assert abs(rate - 1920 * 1080 * 10 * 2 / 0.020 / 1e6) < 1e-6


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    bench.init_replicas(1, 0)
    bench.replica_barrier(1)
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.replica_rate(100, 2, 1, 1000.0) == 100 * 2 / 1.0 / 1e6
