"""Builds from pinned host arrays: when the build finishes its last levels in subtree CTAs,
the subtree kernel reports each window of finished root cells and the host copies it back
into the caller's pinned arrays while later windows are built. Results must be bit-identical
to the oracle, whether the device takes the subtree path or refuses it (then the host copies
everything after the level kernels finish the tree)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def pinned_copy(a):
    """A pinned host array (numpy view of a pinned torch tensor) holding a copy of `a`."""
    t = torch.empty(a.shape[0], dtype=torch.float32 if a.dtype == np.float32 else torch.int32,
                    pin_memory=True)
    v = t.numpy().view(a.dtype)
    v[:] = a
    return t, v


def check(ctx, oracle, x, y, z, d, with_perm, offset=0):
    ref = oracle.build_tree(x, y, z, d)
    n = x.shape[0]
    keep, arrs = [], []
    for a in (x, y, z):
        # offset: the host arrays start `offset` floats into their pinned buffers (alignment
        # differs from the device arrays when offset is not a multiple of 4)
        t, v = pinned_copy(np.concatenate([np.zeros(offset, np.float32), a]))
        keep.append(t)
        arrs.append(v[offset:])
    perm = None
    if with_perm:
        t, perm = pinned_copy(np.zeros(n, np.uint32))
        keep.append(t)
    res = ctx.build(*arrs, d, perm=perm)
    assert res.heap.tobytes() == ref.heap.tobytes()
    assert np.array_equal(res.ranges, ref.ranges[0])
    for got, want in zip(arrs, (ref.x, ref.y, ref.z)):
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    if with_perm:
        assert np.array_equal(perm, ref.perm)
    return res


@pytest.mark.parametrize("kind,seed,logn,logd,with_perm,offset",
                         [("uniform", 90, 20, 10, True, 0), ("uniform", 91, 21, 12, False, 0),
                          ("plummer", 92, 20, 13, True, 1), ("plummer", 93, 19, 12, False, 3)])
def test_pinned_outputs_subtree_taken(ctx, oracle, kind, seed, logn, logd, with_perm, offset):
    gen = oracle.gen_uniform if kind == "uniform" else oracle.gen_plummer
    x, y, z = gen(seed, 1 << logn)
    check(ctx, oracle, x, y, z, 1 << logd, with_perm, offset)


def test_pinned_outputs_subtree_refused(ctx, oracle):
    # half of the particles on one point: their cell cannot be split, so at the level where
    # the host plans subtrees one cell still holds 2^20 particles and the device refuses the
    # subtree path (the level kernels finish the tree and the host copies the particles)
    n, d = 1 << 21, 1 << 12
    x, y, z = oracle.gen_uniform(94, n)
    for a in (x, y, z):
        a[: n // 2] = np.float32(0.125)
    res = check(ctx, oracle, x, y, z, d, True)
    assert res.info["degenerate_cells"] > 0 or res.info["unfound_cells"] > 0


def test_batch_subtree_refused(ctx, oracle):
    # a batch whose largest instance keeps a cell too large for one CTA at the planned
    # subtree level: the device refuses the subtree path for the whole batch, and the level
    # kernels finish every instance (each must still equal the oracle on its own)
    n0, d0 = 1 << 21, 1 << 12
    x0, y0, z0 = oracle.gen_uniform(95, n0)
    for a in (x0, y0, z0):
        a[: n0 // 2] = np.float32(-0.25)
    x1, y1, z1 = oracle.gen_plummer(96, 300000)
    inst = [{"offset": 0, "n": n0, "d": d0, "levels": 0},
            {"offset": n0, "n": 300000, "d": 1 << 9, "levels": 0}]
    bx, by, bz = (np.concatenate(p) for p in ((x0, x1), (y0, y1), (z0, z1)))
    parts, perm, _ = ctx.build_batch(bx, by, bz, inst)
    for (heap, ranges), ins, (ix, iy, iz) in zip(parts, inst, ((x0, y0, z0), (x1, y1, z1))):
        ref = oracle.build_tree(ix, iy, iz, ins["d"])
        a, b = ins["offset"], ins["offset"] + ins["n"]
        assert heap.tobytes() == ref.heap.tobytes()
        assert np.array_equal(ranges, ref.ranges[0])
        assert np.array_equal(perm[a:b], ref.perm)
        for got, want in ((bx, ref.x), (by, ref.y), (bz, ref.z)):
            assert np.array_equal(got[a:b].view(np.uint32), want.view(np.uint32))
