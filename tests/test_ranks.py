"""The multi-rank master loop (ranks.build_ranks) on CPU: ranks whose services are the
oracle's own count and Hoare steps on their slabs, the per-cell counts summed in-process
and by a two-process gloo all-reduce. The heap, every rank's range map and every slab must
equal the oracle's T-rank mode (the reference's MDL semantics) bit for bit."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


class OracleRank:
    """One rank's services on its slab (src/services/count.cpp, countLeft.cpp,
    partition.cpp), computed by the oracle: the CPU stand-in for an engine context."""

    def __init__(self, oracle, x, y, z, heap_cells):
        self.O = oracle
        self.x, self.y, self.z = (np.array(a, np.float32, copy=True) for a in (x, y, z))
        self.rng = np.zeros((heap_cells, 2), np.uint32)
        self.rng[0] = (0, self.x.size)

    def count(self, cells):
        return np.array([self.rng[c["id"], 1] - self.rng[c["id"], 0] for c in cells], np.uint32)

    def count_left(self, cells, out):
        import ranks
        for i, c in enumerate(cells):
            if c["foundCut"]:
                continue
            a = max(int(c["cutAxis"]), 0)
            b, e = (int(v) for v in self.rng[c["id"]])
            out[i] = self.O.count_left((self.x, self.y, self.z)[a], float(ranks.get_cut(c)), b, e)
        return out

    def partition(self, cells):
        import ranks
        for c in cells:
            cid = int(c["id"])
            b, e = (int(v) for v in self.rng[cid])
            i, _ = self.O.hoare(self.x, self.y, self.z, max(int(c["cutAxis"]), 0),
                                float(ranks.get_cut(c)), begin=b, end=e)
            self.rng[2 * cid + 1] = (b, i)
            self.rng[2 * cid + 2] = (i, e)


def _compare(oracle, x, y, z, d, T, heap, rank_objs):
    ref = oracle.build_tree(x, y, z, d, nranks=T, make_axis=True)
    assert heap.tobytes() == ref.heap.tobytes()
    import ranks
    for r, ((off, cnt), ro) in enumerate(zip(ranks.slabs(x.size, T), rank_objs)):
        assert np.array_equal(ro.rng, ref.ranges[r])
        assert np.array_equal(ro.x, ref.x[off:off + cnt]) and np.array_equal(ro.z, ref.z[off:off + cnt])


@pytest.mark.parametrize("kind,n,d,T", [("uniform", 20000, 1 << 5, 3), ("plummer", 30000, 100, 2),
                                        ("uniform", 12345, 12, 4), ("uniform", 9000, 1 << 4, 1)])
def test_in_process_ranks_equal_the_mdl_oracle(oracle, kind, n, d, T):
    import ranks
    x, y, z = (oracle.gen_uniform if kind == "uniform" else oracle.gen_plummer)(n + T, n)
    objs = [OracleRank(oracle, x[o:o + c], y[o:o + c], z[o:o + c], 2 * d - 1)
            for o, c in ranks.slabs(n, T)]
    heap = ranks.build_ranks(objs, d, cell_dtype=oracle.CELL_DTYPE)
    _compare(oracle, x, y, z, d, T, heap, objs)


def test_arithmetic_matches_the_oracle(oracle):
    import ranks
    rng = np.random.default_rng(4)
    for _ in range(3000):
        c = int(rng.integers(0, 1 << 27))
        cl = int(rng.integers(0, c + 1))
        nl = int(rng.integers(1, 1 << 20))
        assert ranks.convergence(cl, c, nl) == oracle.convergence(cl, c, nl)[0]
    cell = np.zeros(1, oracle.CELL_DTYPE)[0]
    for _ in range(3000):
        a, b = np.sort(rng.uniform(-1, 1, 2).astype(np.float32))
        cell["cutMarginLeft"], cell["cutMarginRight"] = a, b
        assert ranks.get_cut(cell) == np.float32(oracle.get_cut(float(a), float(b)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _gloo_rank(rank, world, port, q):
    sys.path[:0] = [os.path.join(ROOT, "gpu-load-balance_gb300"), os.path.join(ROOT, "oracle"),
                    os.path.join(ROOT, "tests")]
    import torch
    import torch.distributed as dist
    import oracle as O
    import ranks
    from test_ranks import OracleRank
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    n, d = 24000, 1 << 6
    x, y, z = O.gen_plummer(17, n)
    off, cnt = ranks.slabs(n, world)[rank]
    me = OracleRank(O, x[off:off + cnt], y[off:off + cnt], z[off:off + cnt], 2 * d - 1)

    def allreduce(v):
        t = torch.from_numpy(v.astype(np.int64))
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        v[:] = t.numpy().astype(np.uint32)

    heap = ranks.build_ranks([me], d, allreduce=allreduce, cell_dtype=O.CELL_DTYPE)
    q.put((rank, heap.tobytes(), me.rng.copy(), me.x.copy()))
    dist.barrier()
    dist.destroy_process_group()


def test_two_process_gloo_allreduce_equals_the_mdl_oracle(oracle):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    import ranks
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_gloo_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=300) for _ in procs), key=lambda t: t[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    n, d = 24000, 1 << 6
    x, y, z = oracle.gen_plummer(17, n)
    ref = oracle.build_tree(x, y, z, d, nranks=2, make_axis=True)
    for r, heap_bytes, rng, xs in res:
        off, cnt = ranks.slabs(n, 2)[r]
        assert heap_bytes == ref.heap.tobytes()
        assert np.array_equal(rng, ref.ranges[r]) and np.array_equal(xs, ref.x[off:off + cnt])
