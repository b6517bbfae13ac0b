"""N > 1 is replicas only: whole-job throughput = all ranks' units over the
slowest rank's time.  world_size 2 on the gloo backend (CPU)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from grudon_gb300.replicas import job_throughput
    # rank r processed 100*(r+1) units in (r+1) seconds
    thr, secs, ws = job_throughput(100.0 * (rank + 1), float(rank + 1))
    q.put((rank, thr, secs, ws))
    dist.barrier()
    dist.destroy_process_group()


def test_job_throughput_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, thr, secs, ws in out:
        assert ws == 2 and secs == 2.0
        assert thr == pytest.approx(300.0 / 2.0)


def test_single_process_without_group():
    from grudon_gb300.replicas import job_throughput
    thr, secs, ws = job_throughput(50.0, 2.0)
    assert (thr, secs, ws) == (25.0, 2.0, 1)
