"""The N>1 path on CPU: two gloo ranks run the replica bookkeeping that
bench.py uses under torchrun (barrier, max-over-ranks time, summed units,
round-robin job shards) -- no GPU and no data-path collective involved."""
import os
import socket

import pytest
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
    from venusaur_gb300.replicas import Replicas

    r = Replicas(backend="gloo")
    r.barrier()
    units = 1000 * (rank + 1)        # rank-local segments
    secs = 0.5 + rank                # rank-local elapsed time
    tot, slow, rate = r.throughput(units, secs)
    jobs = r.shard(list(range(10)))
    q.put((rank, tot, slow, rate, jobs, r.backend))
    r.barrier()
    r.close()


def test_two_gloo_ranks():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(i, world, port, q)) for i in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    for rank, tot, slow, rate, jobs, backend in out:
        assert backend == "gloo"
        assert tot == 3000 and slow == 1.5 and rate == pytest.approx(2000.0)
    assert out[0][4] == [0, 2, 4, 6, 8] and out[1][4] == [1, 3, 5, 7, 9]


def test_single_process_is_identity():
    for k in ("WORLD_SIZE", "RANK"):
        os.environ.pop(k, None)
    from venusaur_gb300.replicas import Replicas

    r = Replicas()
    assert r.world == 1 and r.throughput(10, 2.0) == (10.0, 2.0, 5.0) and r.shard([1, 2]) == [1, 2]
