"""bench.py under torchrun: each rank advances its own replica (the path has
no exchange step), the line reports every replica's points over the slowest
rank's time, and the reference arm runs on rank 0 only.  Two gloo ranks on
the CPU (no GPU)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import argparse
    import torch.distributed as dist
    import bench
    args = argparse.Namespace(impl="reference")
    w, r, local, pg = bench.dist_setup(args)          # gloo for the reference arm
    assert (w, r, local) == (world, rank, rank) and pg is not None
    # replica times differ per rank; every rank gets the slowest
    slowest = bench.max_over_ranks(pg, 10.0 + 5.0 * rank)
    rate = bench.whole_job_rate(w, 1000, 4, slowest)
    # the reference arm: ranks other than 0 exit without work
    ref = bench.run_reference(argparse.Namespace(), w, r) if r != 0 else None
    pg.barrier()
    dist.destroy_process_group()
    q.put((rank, slowest, rate, ref))


def test_two_gloo_replicas():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [15.0, 15.0]
    assert out[0][2] == pytest.approx(2 * 1000 * 4 / 15.0 / 1e6)
    assert out[1][3] is None
