"""The multi-GPU path of bench.py is replicas only: every rank steps its own
lattice, the job time is the slowest rank's, and the value counts the sites
of all ranks.  Checked here with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, REPO)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    assert bench.dist_env() == (ws, rank, rank)
    # rank r took 10 + r ms for 5 steps of 1,000 sites
    value, ms = bench.replica_throughput(10.0 + rank, 1000, 5, ws)
    bench.barrier(ws)
    q.put((rank, value, ms))
    dist.destroy_process_group()


def test_replica_throughput_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=180)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, value, ms in res:
        assert ms == 11.0  # the slower rank's time on every rank
        assert abs(value - 1000 * 2 * 5 / 11e-3 / 1e6) < 1e-12
