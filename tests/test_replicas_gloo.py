"""The multi-GPU path is replicas only: under torchrun each rank serves its
own seeded stream and rank 0 reports the max-over-ranks time.  This runs
bench.py's distributed plumbing as two gloo ranks on the CPU."""
import os
import socket

import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import argparse

    import bench
    w, r = bench.dist_setup(argparse.Namespace())
    assert (w, r) == (world, rank)
    t = bench.max_over_ranks(1.0 + rank, w)
    specs, _ = bench.make_stream(argparse.Namespace(requests=3, req_steps=5), 5 + rank)
    bench.barrier(w)
    out.put((rank, t, tuple(s["seed"] for s in specs)))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][1] == res[1][1] == 2.0          # max over ranks
    assert res[0][2] != res[1][2]                  # each rank serves its own stream
