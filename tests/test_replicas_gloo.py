"""The N > 1 path of bench.py on CPU: two gloo ranks on 127.0.0.1 run the
benchmark's barrier and max-over-ranks timing, the whole-job value of
independent replicas, and compile's refusal to shard (world size 1 only)."""
import os
import socket

import pytest
import torch
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import bench
    import easier_gb300 as esr
    from easier_gb300 import workloads
    from easier_gb300.utils import EasierJitException
    esr.init("gloo")
    try:
        w, r, _ = bench._dist()
        bench._barrier(w)
        ms = bench._max_over_ranks(w, 10.0 + 5.0 * r)  # each rank's own timed region
        refused = False
        try:
            esr.compile([workloads.make_swe(4)], "cuda")
        except EasierJitException as e:
            refused = "world size 1" in str(e)
        q.put((r, w, ms, refused))
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(240)
def test_two_replicas_gloo():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=200) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1] and all(o[1] == world for o in out)
    # every rank reports the slowest rank's time
    assert all(o[2] == 15.0 for o in out)
    assert all(o[3] for o in out)
    # whole-job value of replicas: all ranks' units over the slowest time
    units_per_rank, steps = 1000, 10
    value = world * units_per_rank * steps / (out[0][2] / 1e3)
    assert value == pytest.approx(2 * 1000 * 10 / 0.015)
