"""N>1 path of the benchmark on CPU: two gloo ranks, each a replica; the job's time is the
slowest rank's and its work the sum of the ranks' work."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "gpu-load-balance_gb300"))
    import replicas
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms, units, rate = replicas.whole_job(10.0 + 5.0 * rank, 1000 * (rank + 1))
    out.put((rank, ms, units, rate))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, units, rate in res:
        assert ms == 15.0 and units == 3000
        assert abs(rate - 3000 / 0.015) < 1e-6


def test_single_process_is_local():
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "gpu-load-balance_gb300"))
    import replicas
    assert replicas.whole_job(20.0, 500) == (20.0, 500, 500 / 0.02)
