"""Weighted ORB on the GPU (orb_build_weighted) against the oracle's weighted restatement:
integer weights moved with their particles, uint64 weight sums per cell, the reference's
bisection loop with the exact weighted test. Bit-exact on the heap, ranges, permutation,
coordinates and the reordered weights; with unit weights, equal to the unweighted build."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def check(ctx, oracle, x, y, z, w, d, levels=0, device=False):
    ref, wref = oracle.build_tree_weighted(x, y, z, w, d, levels=levels or None, threads=8)
    if device:
        torch = pytest.importorskip("torch")
        tx, ty, tz = (torch.from_numpy(a.copy()).cuda() for a in (x, y, z))
        tw = torch.from_numpy(w.view(np.int32).copy()).cuda()
        tp = torch.empty(x.size, dtype=torch.int32, device="cuda")
        res = ctx.build_weighted(tx, ty, tz, tw, d, levels=levels, perm=tp, device_pointers=True)
        gx, gw, perm = tx.cpu().numpy(), tw.cpu().numpy().view(np.uint32), tp.cpu().numpy().view(np.uint32)
        gy, gz = ty.cpu().numpy(), tz.cpu().numpy()
    else:
        gx, gy, gz, gw = x.copy(), y.copy(), z.copy(), w.copy()
        res = ctx.build_weighted(gx, gy, gz, gw, d, levels=levels)
        perm = res.perm
    assert res.heap.tobytes() == ref.heap.tobytes()
    assert np.array_equal(res.ranges, ref.ranges[0])
    assert np.array_equal(perm, ref.perm)
    assert np.array_equal(gw, wref)
    for a, b in ((gx, ref.x), (gy, ref.y), (gz, ref.z)):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert res.info["unfound_cells"] == ref.stats["unfound_cells"]
    return res, ref


@pytest.mark.parametrize("kind,n,d,wmax", [("uniform", 1 << 18, 1 << 9, 64), ("plummer", 300000, 1 << 10, 1000),
                                           ("uniform", 100000, 100, 16), ("plummer", 1 << 20, 1 << 12, 1 << 20)])
def test_weighted_matches_oracle(ctx, oracle, kind, n, d, wmax):
    x, y, z = (oracle.gen_uniform if kind == "uniform" else oracle.gen_plummer)(n % 101, n)
    w = np.random.default_rng(n).integers(0, wmax, n).astype(np.uint32)
    check(ctx, oracle, x, y, z, w, d)


def test_weighted_unit_weights_are_the_plain_build(ctx, oracle):
    n, d = 1 << 20, 1 << 10
    x, y, z = oracle.gen_plummer(31, n)
    res, _ = check(ctx, oracle, x, y, z, np.ones(n, np.uint32), d)
    plain = ctx.build(x.copy(), y.copy(), z.copy(), d)
    assert res.heap.tobytes() == plain.heap.tobytes() and np.array_equal(res.perm, plain.perm)


def test_weighted_device_pointers_and_edge_cases(ctx, oracle):
    x, y, z = oracle.gen_uniform(32, 70000)
    w = np.random.default_rng(2).integers(1, 9, 70000).astype(np.uint32)
    check(ctx, oracle, x, y, z, w, 1 << 8, device=True)
    check(ctx, oracle, x, y, z, np.zeros(70000, np.uint32), 1 << 4)  # no weight: found at once
    heavy = w.copy()
    heavy[::1000] = 4_000_000_000  # single particles outweigh their cells
    check(ctx, oracle, x, y, z, heavy, 1 << 6)
    check(ctx, oracle, x, y, z, w, 1 << 8, levels=5)
    for n in (0, 1, 5):
        e = np.zeros(n, np.float32) + np.float32(0.1)
        check(ctx, oracle, e, e.copy(), e.copy(), np.ones(n, np.uint32), 4)
