"""The multi-rank path of bench.py on CPU: two gloo ranks, each advancing its
own replica box (the timestep does not shard: one domain per GPU, no halo
exchange), with the barrier and the max-over-ranks timing of the benchmark.
The CPU oracle stands in for the GPU step so this runs without a GPU."""
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench
    from guacho_gb300 import problems
    from oracle.oracle import Oracle
    d = bench.Dist()
    assert d.ws == world and d.rank == rank
    p, u0 = problems.orszag_tang(16, 16, 4)
    o = Oracle(p, threads=1)
    o.init(u0)
    d.barrier()
    import time
    t0 = time.perf_counter()
    o.run(1e30, 1e30, max_steps=3 + rank)   # uneven work per rank
    el = time.perf_counter() - t0
    tmax = d.max(el)
    out[rank] = (el, tmax, float(o.download()[2:-2, 2:-2, 2:-2, 0].sum()))
    d.close()


@pytest.mark.timeout(300)
def test_two_rank_replicas_max_time():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    procs = [ctx.Process(target=_worker, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(240)
        assert p.exitcode == 0
    el = [out[r][0] for r in range(world)]
    tmax = [out[r][1] for r in range(world)]
    # every rank sees the same max, equal to the slowest rank's time
    assert tmax[0] == tmax[1] == max(el)
    # replicas of the same periodic problem conserve the same mass
    np.testing.assert_allclose(out[0][2], out[1][2], rtol=1e-13)
