"""The multi-process path of bench.py on CPU (gloo, world size 2): replicas
only. Each rank runs its own analysis on its own GPU; the ranks meet at a
barrier around the timed region and reduce only the timings (max over
ranks), so the whole-job value is world x steps / max time."""
import multiprocessing as mp
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


def _rank(rank: int, world: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench
    w, r, local, pg = bench.dist_setup(world)
    bench.barrier(pg)
    t = bench.allmax(pg, 10.0 + 5.0 * r)  # rank 1 is the slower replica
    out.put((r, w, local, t))
    pg.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_gloo_replicas_reduce_the_max_time():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=90) for _ in ps)
    for p in ps:
        p.join(timeout=30)
        assert p.exitcode == 0
    assert [x[0] for x in res] == [0, 1]
    assert all(x[1] == 2 and x[2] == x[0] for x in res)
    assert all(x[3] == 15.0 for x in res)  # every rank sees the slowest replica's time
    # weak scaling: two replicas of 10 steps in max 15 ms -> 1333 steps/s for the job
    assert abs(2 * 10 / (15.0 / 1e3) - 1333.33) < 0.01
