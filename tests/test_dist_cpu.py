"""The multi-GPU path of bench.py is replicas: every rank runs its own copy of
the workload, no collective on the data path; the job's time is the slowest
rank's and its throughput sums all ranks.  Checked here with two gloo ranks
on CPU, each running the CPU oracle as its replica: the max-over-ranks
reduction, the whole-job value, and that replicas of one scene agree bit for
bit (so the ranks' work is interchangeable)."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import time

    import bench
    from oracle import pyoracle as po
    from titan_gb300 import workloads as wl

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    assert bench.dist_env() == (rank, world, rank)
    sc = wl.falling_cube(contact=True)
    o = po.OracleSim(sc)
    t0 = time.perf_counter()
    o.step(200 + 100 * rank, po.ASCENDING, 1)  # unequal work: rank 1 is slower
    mine = time.perf_counter() - t0
    slowest = bench.max_over_ranks(mine, world, device="cpu")
    times = [torch.zeros(1, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(times, torch.tensor([mine], dtype=torch.float64))
    # replicas of the same scene and step count agree bit for bit
    o2 = po.OracleSim(sc)
    o2.step(300, po.ASCENDING, 1)
    digest = torch.tensor(np.frombuffer(o2.pos.tobytes(), np.int64)[:64].copy())
    digests = [torch.zeros_like(digest) for _ in range(world)]
    dist.all_gather(digests, digest)
    if rank == 0:
        out.put({"slowest": slowest, "times": [float(t.item()) for t in times],
                 "value": bench.replica_value(1036 * 300, world, slowest),
                 "same": all(torch.equal(digests[0], d) for d in digests)})
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = q.get(timeout=180)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res["slowest"] == max(res["times"])
    assert res["value"] == pytest.approx(2 * 1036 * 300 / res["slowest"])
    assert res["same"]
