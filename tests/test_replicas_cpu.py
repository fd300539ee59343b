"""bench.py's N-replica aggregation on two gloo ranks (CPU): rays summed over ranks, time the
slowest rank's, so the whole-job throughput of independent replicas."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2")
    import bench

    d = bench.Dist(2, "gloo")
    value, ms_max, rays_all = bench.replica_throughput(d, 1000.0 * (rank + 1), 2.0 + rank)
    d.barrier()
    if rank == 0:
        with open(out, "w") as f:
            f.write("%r %r %r" % (value, ms_max, rays_all))
    d.close()


def test_two_replicas_sum_rays_over_slowest_time(tmp_path):
    out = str(tmp_path / "r.txt")
    mp.spawn(_rank, args=(_free_port(), out), nprocs=2, join=True)
    value, ms_max, rays_all = (float(x) for x in open(out).read().split())
    assert rays_all == 3000.0 and ms_max == 3.0
    assert value == pytest.approx(3000.0 / 3.0 / 1e3)
