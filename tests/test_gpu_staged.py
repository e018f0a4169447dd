"""Staged builds from host arrays: x is copied first and level 1 (cut along x) runs on it
while y arrives; y then takes level 1's order through the permutation and level 2 runs on x
and y while z arrives. The cuts and swaps are the unstaged build's, so every output must be
bit-identical to the oracle (and to a build from device arrays, which is never staged). The
engine stages only boxes whose y side is at least as long as z's: level 2 can then only cut
along x or y."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def gathers(ctx):
    return ctx.profile().get("stage_gather", {}).get("launches", 0)


# ORB_NO_STAGE=1 (read when a context is created) turns staging off: the same results, no gathers
STAGED = 0 if os.environ.get("ORB_NO_STAGE", "0") not in ("", "0") else 2


def host_build(ctx, oracle, x, y, z, d, levels=0, lower=(-0.5,) * 3, upper=(0.5,) * 3, perm=True):
    ref = oracle.build_tree(x, y, z, d, levels=levels or None, lower=lower, upper=upper)
    hx, hy, hz = (np.array(a, copy=True) for a in (x, y, z))
    ctx.profile_reset()
    res = ctx.build(hx, hy, hz, d, levels=levels, lower=lower, upper=upper, perm=perm)
    assert res.heap.tobytes() == ref.heap.tobytes()
    assert np.array_equal(res.ranges, ref.ranges[0])
    for got, want in ((hx, ref.x), (hy, ref.y), (hz, ref.z)):
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    if perm is True:
        assert np.array_equal(res.perm, ref.perm)
    return gathers(ctx)


@pytest.mark.parametrize("kind,seed,n,d,levels,perm", [
    ("uniform", 300, 1 << 20, 1 << 10, 0, True),
    ("plummer", 301, 300001, 1000, 0, False),
    ("uniform", 302, 1 << 18, 1 << 4, 2, True),   # exactly the two staged levels
    ("plummer", 303, 1 << 19, 1 << 8, 3, False),
    ("uniform", 304, 5, 4, 0, True),              # fewer particles than leaves
])
def test_staged_host_build(ctx, oracle, kind, seed, n, d, levels, perm):
    gen = oracle.gen_uniform if kind == "uniform" else oracle.gen_plummer
    x, y, z = gen(seed, n)
    assert host_build(ctx, oracle, x, y, z, d, levels, perm=perm) == STAGED


def test_staged_level2_cuts_along_x(ctx, oracle):
    # x four times longer than y and z: level 2 cuts along x again, with y already moving
    x, y, z = oracle.gen_uniform(305, 1 << 20)
    x = x * np.float32(4)
    lo, hi = (-2.0, -0.5, -0.5), (2.0, 0.5, 0.5)
    assert host_build(ctx, oracle, x, y, z, 1 << 9, lower=lo, upper=hi) == STAGED


def test_staged_y_longest(ctx, oracle):
    # the root still cuts along x (src/orbit.cpp:75); level 2 cuts along y
    x, y, z = oracle.gen_plummer(306, 1 << 20)
    y = y * np.float32(2)
    assert host_build(ctx, oracle, x, y, z, 1 << 11, lower=(-0.5, -1.0, -0.5), upper=(0.5, 1.0, 0.5)) == STAGED


def test_unstaged_when_z_is_longer(ctx, oracle):
    # z longer than y: a level-2 cell may cut along z, so the build copies all three first
    x, y, z = oracle.gen_uniform(307, 1 << 20)
    z = z * np.float32(3)
    assert host_build(ctx, oracle, x, y, z, 1 << 10, lower=(-0.5, -0.5, -1.5), upper=(0.5, 0.5, 1.5)) == 0


def test_staged_equals_device_build(ctx, oracle):
    # a build from device arrays (never staged) against a staged one, at 2^23 particles
    x, y, z = oracle.gen_plummer(308, 1 << 23)
    d = 1 << 14
    hx, hy, hz = (np.array(a, copy=True) for a in (x, y, z))
    ctx.profile_reset()
    res_h = ctx.build(hx, hy, hz, d)
    assert gathers(ctx) == STAGED
    dx, dy, dz = (torch.from_numpy(a).cuda() for a in (x, y, z))
    perm = torch.empty(x.shape[0], dtype=torch.int32, device="cuda")
    res_d = ctx.build(dx, dy, dz, d, perm=perm, device_pointers=True)
    assert res_h.heap.tobytes() == res_d.heap.tobytes()
    assert np.array_equal(res_h.ranges, res_d.ranges)
    assert np.array_equal(res_h.perm, perm.cpu().numpy().view(np.uint32))
    for got, want in ((hx, dx), (hy, dy), (hz, dz)):
        assert np.array_equal(got.view(np.uint32), want.cpu().numpy().view(np.uint32))


# Builds from host arrays that finish their last levels in subtree CTAs copy the particles
# back in windows of consecutive root cells: the subtree kernel reports each window to the
# host once every cell of it is final, and the host copies it back while the kernel builds the
# next ones (16 windows by default; ORB_E2E_WINDOWS=0 copies everything after the build).

def context_with_windows(engine, k):
    import os
    old = os.environ.get("ORB_E2E_WINDOWS")
    os.environ["ORB_E2E_WINDOWS"] = str(k)
    try:
        return engine.Context(0)
    finally:
        if old is None:
            del os.environ["ORB_E2E_WINDOWS"]
        else:
            os.environ["ORB_E2E_WINDOWS"] = old


def pinned(a):
    t = torch.empty(a.shape[0], dtype=torch.float32 if a.dtype == np.float32 else torch.int32,
                    pin_memory=True)
    v = t.numpy().view(a.dtype)
    v[:] = a
    return t, v


def check_host_build(c, oracle, x, y, z, d, use_pinned):
    n = x.shape[0]
    ref = oracle.build_tree(x, y, z, d, threads=8)
    keep = []
    if use_pinned:
        arrs = []
        for a in (x, y, z, np.zeros(n, np.uint32)):
            t, v = pinned(a)
            keep.append(t)
            arrs.append(v)
        hx, hy, hz, perm = arrs
    else:
        hx, hy, hz = (np.array(a, copy=True) for a in (x, y, z))
        perm = np.zeros(n, np.uint32)
    res = c.build(hx, hy, hz, d, perm=perm)
    assert res.heap.tobytes() == ref.heap.tobytes()
    assert np.array_equal(res.ranges, ref.ranges[0])
    assert np.array_equal(perm, ref.perm)
    for got, want in ((hx, ref.x), (hy, ref.y), (hz, ref.z)):
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    return res


@pytest.mark.parametrize("kind,seed,n,d,use_pinned", [
    ("uniform", 310, (1 << 22) + 12345, 1 << 12, False),
    ("plummer", 311, 1 << 22, 1 << 14, True),
    ("uniform", 312, 1 << 23, 1 << 16, True),
    ("plummer", 315, 1 << 20, 1 << 10, True),
])
def test_windowed_host_build(ctx, oracle, kind, seed, n, d, use_pinned):
    gen = oracle.gen_uniform if kind == "uniform" else oracle.gen_plummer
    x, y, z = gen(seed, n)
    check_host_build(ctx, oracle, x, y, z, d, use_pinned)


@pytest.mark.parametrize("use_pinned", [False, True])
def test_windowed_subtree_refused(ctx, oracle, use_pinned):
    # a quarter of the particles on one point: a cell too large for one CTA remains at the
    # subtree level, so the device refuses the subtree path, reports no window, and the level
    # kernels finish the tree before everything is copied back
    n, d = 1 << 22, 1 << 12
    x, y, z = oracle.gen_uniform(313, n)
    for a in (x, y, z):
        a[: n // 4] = np.float32(0.3)
    res = check_host_build(ctx, oracle, x, y, z, d, use_pinned)
    assert res.info["degenerate_cells"] > 0 or res.info["unfound_cells"] > 0


def test_window_counts_agree(engine, oracle):
    # no windows, one, 8 and 64: the same tree and particle order
    x, y, z = oracle.gen_plummer(314, 1 << 22)
    d = 1 << 13
    for k in (0, 1, 8, 64):
        c = context_with_windows(engine, k)
        try:
            check_host_build(c, oracle, x, y, z, d, use_pinned=k % 2 == 0)
        finally:
            c.close()
