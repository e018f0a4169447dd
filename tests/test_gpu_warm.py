"""Warm-started builds (orb_build_warm / orb_build_batch_warm / warm rebalances): a labelled
mode that starts every cell's bisection from the previous tree's cut. The trees are valid ORB
trees (children tile their parent, particles lie in their leaf boxes, every found cut passes
the reference's convergence test) but not bit-identical with a cold build; a hint that misses
restarts the cell cold, so when every hint misses the tree IS the cold tree."""
import numpy as np
import pytest

from helpers import tree_properties

pytestmark = pytest.mark.gpu
f32 = np.float32


def displaced(x, y, z, seed, sigma=1e-3):
    rng = np.random.default_rng(seed)
    out = []
    for a in (x, y, z):
        b = a + f32(sigma) * rng.standard_normal(a.shape[0]).astype(f32)
        out.append(np.clip(b, f32(-0.5), np.nextafter(f32(0.5), f32(0))).astype(f32))
    return out


def check_cuts(x, y, z, heap, ranges, levels):
    """Every split cell's recorded cut against its own particles: a found cut passes the
    reference's test (src/orbit.cpp:204-208), an unfound one used all 32 sweeps."""
    for cid in range((1 << levels) - 1):
        c = heap[cid]
        b, e = (int(v) for v in ranges[cid])
        n = e - b
        a = max(int(c["cutAxis"]), 0)
        cut = f32(f32(c["cutMarginRight"]) + f32(c["cutMarginLeft"])) * f32(0.5)
        cl = int(((x, y, z)[a][b:e] < cut).sum())
        diff = int(f32(cl) - f32(n) * f32(0.5))
        if c["foundCut"]:
            assert abs(diff) < 3, f"cell {cid}: cut does not pass the convergence test"


def test_warm_rebuild_is_a_valid_tree(ctx, oracle):
    n, d = 300000, 1 << 9
    x, y, z = oracle.gen_uniform(41, n)
    cold = ctx.build(x.copy(), y.copy(), z.copy(), d)
    xs, ys, zs = displaced(x, y, z, 7)
    wx, wy, wz = xs.copy(), ys.copy(), zs.copy()
    warm = ctx.build_warm(wx, wy, wz, d, cold.heap, 8.0)
    info = warm.info
    assert info["warm_cells"] > d // 2  # most split cells started from a hint
    assert info["warm_resets"] < info["warm_cells"] // 4
    tree_properties(wx, wy, wz, warm.heap, warm.ranges, n, d, 9)
    check_cuts(wx, wy, wz, warm.heap, warm.ranges, 9)
    assert np.array_equal(np.sort(warm.perm), np.arange(n, dtype=np.uint32))
    for got, src in ((wx, xs), (wy, ys), (wz, zs)):
        assert np.array_equal(got.view(np.uint32), src[warm.perm].view(np.uint32))


def test_missed_hints_restart_cold(ctx, oracle):
    n, d = 120000, 1 << 8
    x, y, z = oracle.gen_plummer(42, n)
    cold = ctx.build(x.copy(), y.copy(), z.copy(), d)
    # hints pinned to each cell's lower edge: no bracket holds the median
    prev = cold.heap.copy()
    for cid in range(d - 1):
        a = max(int(prev[cid]["cutAxis"]), 0)
        prev[cid]["cutMarginLeft"] = prev[cid]["lower"][a]
        prev[cid]["cutMarginRight"] = prev[cid]["lower"][a]
    r = ctx.build_warm(x.copy(), y.copy(), z.copy(), d, prev, 1e-4)
    assert r.info["warm_cells"] > 0 and r.info["warm_resets"] == r.info["warm_cells"]
    assert r.heap.tobytes() == cold.heap.tobytes()
    assert np.array_equal(r.ranges, cold.ranges)
    assert np.array_equal(r.perm, cold.perm)


def test_zero_width_is_cold(ctx, oracle):
    n, d = 50000, 64
    x, y, z = oracle.gen_uniform(43, n)
    cold = ctx.build(x.copy(), y.copy(), z.copy(), d)
    r = ctx.build_warm(x.copy(), y.copy(), z.copy(), d, cold.heap, 0.0)
    assert r.info["warm_cells"] == 0
    assert r.heap.tobytes() == cold.heap.tobytes() and np.array_equal(r.perm, cold.perm)


def test_batched_warm_equals_each_instance_alone(ctx, oracle):
    sizes = [(20000, 64), (3000, 16), (90000, 256), (500, 8)]
    xs, ys, zs, inst, prevs, widths, alone = [], [], [], [], [], [], []
    off = 0
    for i, (n, d) in enumerate(sizes):
        x, y, z = oracle.gen_uniform(60 + i, n)
        cold = ctx.build(x.copy(), y.copy(), z.copy(), d)
        dx, dy, dz = displaced(x, y, z, 90 + i)
        w = 0.0 if i == 1 else 8.0  # instance 1 builds cold inside the warm batch
        alone.append(ctx.build_warm(dx.copy(), dy.copy(), dz.copy(), d, cold.heap, w))
        xs.append(dx); ys.append(dy); zs.append(dz)
        inst.append({"offset": off, "n": n, "d": d})
        prevs.append(cold.heap)
        widths.append(w)
        off += n
    x, y, z = (np.concatenate(a) for a in (xs, ys, zs))
    parts, _, perm, info = ctx.build_batch_warm(x, y, z, inst, np.concatenate(prevs), widths)
    assert info["warm_cells"] > 0
    for (heap, ranges), ins, a in zip(parts, inst, alone):
        assert heap.tobytes() == a.heap.tobytes()
        assert np.array_equal(ranges, a.ranges)
        s = slice(ins["offset"], ins["offset"] + ins["n"])
        assert np.array_equal(perm[s], a.perm)


def test_server_warm_rebalance(engine, oracle):
    n, d = 40000, 128
    x, y, z = oracle.gen_uniform(71, n)
    with engine.Server(0, hbm_budget_bytes=1 << 28) as sv:
        inst = sv.submit_build(x, y, z, d)
        sv.wait(inst)
        assert sv.wait(sv.submit_rebalance(inst, 5, 1e-3, warm=8.0))["status"] == 0
        heap, ranges, x1, y1, z1, ident = sv.fetch(inst)
    tree_properties(x1, y1, z1, heap, ranges, n, d, 7)
    check_cuts(x1, y1, z1, heap, ranges, 7)
    assert np.array_equal(np.sort(ident), np.arange(n, dtype=np.uint32))
