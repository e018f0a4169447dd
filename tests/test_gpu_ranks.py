"""Multi-rank builds on the GPU through the service entry points: T slabs, each in its own
engine context (orb_load_particles), counted with orb_count / orb_count_left and partitioned
with orb_partition, the per-cell uint32 counts summed over the ranks (the reference's MDL
Combine, src/services/countLeft.cpp:44-53) by ranks.build_ranks. The heap, every rank's
range map and every partitioned slab must equal the oracle's T-rank mode bit for bit."""
import numpy as np
import pytest

import ranks

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,n,d,T", [("uniform", 1 << 18, 1 << 8, 2), ("plummer", 300000, 1 << 7, 3),
                                        ("uniform", 200000, 100, 4), ("plummer", 1 << 17, 12, 2)])
def test_gpu_ranks_equal_the_mdl_oracle(engine, oracle, kind, n, d, T):
    x, y, z = (oracle.gen_uniform if kind == "uniform" else oracle.gen_plummer)(n % 97 + T, n)
    ctxs = [engine.Context(0) for _ in range(T)]
    try:
        for c, (off, cnt) in zip(ctxs, ranks.slabs(n, T)):
            c.load_particles(x[off:off + cnt].copy(), y[off:off + cnt].copy(), z[off:off + cnt].copy(),
                             2 * d - 1)
        heap = ranks.build_ranks(ctxs, d)
        ref = oracle.build_tree(x, y, z, d, nranks=T, make_axis=True)
        assert heap.tobytes() == ref.heap.tobytes()
        for r, (c, (off, cnt)) in enumerate(zip(ctxs, ranks.slabs(n, T))):
            assert np.array_equal(c.get_ranges(2 * d - 1), ref.ranges[r])
            sx, sy, sz, _ = c.store_particles()
            for got, want in ((sx, ref.x), (sy, ref.y), (sz, ref.z)):
                assert np.array_equal(got.view(np.uint32), want[off:off + cnt].view(np.uint32))
    finally:
        for c in ctxs:
            c.close()


def test_one_rank_is_the_plain_build(ctx, engine, oracle):
    """With one slab the service-level master loop is the reference's single-rank driver:
    its heap equals orb_build's."""
    n, d = 1 << 16, 1 << 6
    x, y, z = oracle.gen_uniform(3, n)
    ctx.load_particles(x, y, z, 2 * d - 1)
    heap = ranks.build_ranks([ctx], d)
    res = engine.Context(0)
    try:
        b = res.build(x.copy(), y.copy(), z.copy(), d)
    finally:
        res.close()
    assert heap.tobytes() == b.heap.tobytes()
    assert np.array_equal(ctx.get_ranges(2 * d - 1), b.ranges)
