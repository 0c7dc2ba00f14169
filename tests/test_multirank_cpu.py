"""The multi-rank path of bench.py on CPU: two gloo ranks, each validating its
own replica of a small batch with the CPU oracle (the GPU path's stand-in
here), the barrier, the max-over-ranks time and the whole-job throughput."""
import os
import socket
import sys
from pathlib import Path

import numpy as np
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, str(ROOT))
    import time

    import bench
    import torch.distributed as dist
    import __graft_entry__ as ge
    from oracle import oracle as orc
    w, r, _ = bench.dist_setup("gloo")
    assert (w, r) == (world, rank)
    wl = ge.load_package().workloads.config2(n_edges=32, seed=5)
    bench.barrier(w)
    t = time.perf_counter()
    res = orc.validate(wl.scene, wl.bases, wl.q0, wl.q1, wl.granularity, wl.flags, threads=1)
    dt = time.perf_counter() - t + 0.01 * rank  # ranks of different speed
    slowest = bench.max_over_ranks(dt, w)
    value = bench.replica_throughput(32 * wl.granularity, 1, [dt], w)
    bench.barrier(w)
    out[rank] = (res["valid"].tobytes(), dt, slowest, value)
    dist.destroy_process_group()


def test_two_gloo_ranks_replicas():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    assert res[0][0] == res[1][0]                      # replicas give the same verdicts
    slowest = max(res[0][1], res[1][1])
    assert np.isclose(res[0][2], slowest) and np.isclose(res[1][2], slowest)  # every rank sees the max
    assert np.isclose(res[0][3], world * 32 * 32 / slowest)                # all ranks' units / slowest time
