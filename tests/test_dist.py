"""The multi-process path of bench.py on CPU: two gloo ranks rendezvous as
torchrun launches them (RANK / WORLD_SIZE / MASTER_* from the environment),
each integrates its own seed-rank instance draws (replicas, no data
exchange), and the job's time is the maximum over the ranks."""
import os
import socket

import numpy as np


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), BENCH_BACKEND="gloo")
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import torch
    import bench
    w, r, local = bench.dist_init()
    assert (w, r, local) == (world, rank, rank)
    bench.barrier(w)
    t = bench.max_over_ranks(torch, w, 1000.0 * (rank + 1))
    draws = bench.replica_draws(r)
    out.put((rank, t, draws[:4].copy(), bench.job_value(w, t)))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, t0, d0, v0), (r1, t1, d1, v1) = res
    assert t0 == t1 == 2000.0                  # the slowest rank's time
    assert not np.array_equal(d0, d1)          # each rank its own instances
    import bench
    assert np.array_equal(d0, bench.im_draws(4096, 0)[:4])
    assert np.array_equal(d1, bench.im_draws(4096, 1)[:4])
    assert v0 == v1 == 2 * 4096 / 2.0          # whole-job spectra/s
