"""Multi-GPU replicas (one independent solve per rank, no data-path collective): the
cross-rank timing aggregation of bench.py on world_size-2 gloo process groups on CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from dirac_caspt2_gb300 import replicas
    replicas.barrier()
    # rank r timed its steps in (r + 1) seconds on the value leg and 2 (r + 1) on the e2e leg
    worst = replicas.max_over_ranks([1.0 * (rank + 1), 2.0 * (rank + 1)])
    thr = replicas.replica_throughput([1.0 * (rank + 1), 2.0 * (rank + 1)], steps=5, world=world)
    q.put((rank, worst, thr))
    dist.destroy_process_group()


def test_replica_throughput_two_ranks_gloo():
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, worst, thr in res:
        assert worst == (2.0, 4.0)               # the slowest rank bounds the job on every rank
        assert thr == pytest.approx((2 * 5 / 2.0, 2 * 5 / 4.0))   # whole-job solves/s


def test_replica_throughput_single_process():
    from dirac_caspt2_gb300 import replicas
    assert replicas.max_over_ranks([1.5, 3.0]) == (1.5, 3.0)
    assert replicas.replica_throughput([2.0], steps=4, world=1) == (2.0,)
