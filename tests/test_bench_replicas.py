"""bench.py --gpus N runs independent replicas: the host group (gloo, no GPU
collective) gives every rank the barrier, the slowest rank's time and the
whole job's voxel-iterations.  Two processes on CPU."""
import multiprocessing as mp
import os
import socket

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import bench
    r, w, local = bench.dist_env()
    grp = bench.Group(w)
    grp.barrier()
    # rank k did 1e9 * (k + 1) voxel-iterations in 100 * (k + 1) ms
    value, t_max, vi = bench.whole_job_rate(grp, 1e9 * (r + 1), 100.0 * (r + 1))
    grp.barrier()
    q.put((r, value, t_max, vi))
    grp.dist.destroy_process_group()


def test_replica_group_two_ranks_gloo():
    pytest.importorskip("torch")
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(k, world, port, q)) for k in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    out = sorted(q.get(timeout=10) for _ in range(world))
    for r, value, t_max, vi in out:
        assert t_max == 200.0 and vi == 3e9
        assert abs(value - 3e9 / 0.2) < 1e-3
