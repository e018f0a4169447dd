"""Bit-exact parity at the workload sizes, through the C ABI:

  - 2^27 uniform particles into 2^16 leaves (the headline build),
  - 2^26 clustered particles (64 Plummer spheres + 10% background) into 2^18 leaves,
  - the 128-instance batch (particles log-uniform 2^14..2^22, leaves 2^6..2^12, half
    uniform, half clustered), every instance against its own oracle build,

each under the default launch tuning and under the setting the autotuner chose for the
batch on GB300 (part 16 CTAs/SM, compaction threshold 256, one CTA per cell from 4096 cells,
6 subtree levels). The oracle is the single-rank restatement of the reference's CPU path
(src/orbit.cpp:102-275 with src/services/countLeft.cpp:33-36 and partition.cpp:33-52), run
with its cells in parallel (the same results as one thread). Heap, range map, permutation
and reordered coordinates are compared bit for bit."""
import os

import numpy as np
import pytest

import workloads as W

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1
TUNINGS = {
    "default": None,
    "autotuned": dict(hist_blocks_per_sm=6, part_blocks_per_sm=16, tile_blocks_per_sm=4,
                      sparse_keys_per_tile=256, cta_min_cells=4096, subtree_levels=6,
                      predict_sigmas=0),
}


def assert_bit_exact(res, ref, gx, gy, gz):
    if res.heap.tobytes() != ref.heap.tobytes():
        rows = np.any(res.heap.view(np.uint8).reshape(-1, 52) != ref.heap.view(np.uint8).reshape(-1, 52), 1)
        diff = np.nonzero(rows)[0]
        c = int(diff[0])
        raise AssertionError(f"heap differs at {len(diff)} cells, first {c}:\n gpu {res.heap[c]}\n"
                             f" cpu {ref.heap[c]}")
    assert np.array_equal(res.ranges, ref.ranges[0]), "range map differs"
    assert np.array_equal(res.perm, ref.perm), "particle order differs"
    for a, b in ((gx, ref.x), (gy, ref.y), (gz, ref.z)):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), "coordinates differ"


@pytest.fixture
def tuned_ctx(engine, request):
    c = engine.Context(0)
    if request.param is not None:
        c.set_tuning(**request.param)
    yield c
    c.close()


def _plain(oracle, kind, seed, n, d):
    gen = oracle.gen_uniform if kind == "uniform" else oracle.gen_plummer
    x, y, z = gen(seed, n, nthreads=THREADS)
    ref = oracle.build_tree(x, y, z, d, threads=THREADS)
    return x, y, z, ref


@pytest.fixture(scope="module")
def headline(oracle):
    return _plain(oracle, "uniform", 2027, 1 << 27, 1 << 16)


@pytest.fixture(scope="module")
def clustered(oracle):
    return _plain(oracle, "plummer", 2626, 1 << 26, 1 << 18)


def _check_plain(ctx, case):
    x, y, z, ref = case
    gx, gy, gz = x.copy(), y.copy(), z.copy()
    res = ctx.build(gx, gy, gz, len(ref.heap) // 2 + 1)
    assert_bit_exact(res, ref, gx, gy, gz)
    for k in ("degenerate_cells", "unfound_cells", "zero_volume_cells"):
        assert res.info[k] == ref.stats[k], k
    assert res.info["max_iterations"] == max(ref.stats["iterations"])
    return res


@pytest.mark.parametrize("tuned_ctx", list(TUNINGS.values()), ids=list(TUNINGS), indirect=True)
def test_headline_2p27_2p16_bit_exact(tuned_ctx, headline):
    """2^27 uniform / 2^16 leaves: the level-0 count uses the float roundings above 2^24 and
    the cells hold many keys per value of the 2^-24 grid (ties at the cuts)."""
    _check_plain(tuned_ctx, headline)


@pytest.mark.parametrize("tuned_ctx", list(TUNINGS.values()), ids=list(TUNINGS), indirect=True)
def test_clustered_2p26_2p18_bit_exact(tuned_ctx, clustered):
    """2^26 Plummer-clustered / 2^18 leaves: very uneven cells per level, 18 levels."""
    res = _check_plain(tuned_ctx, clustered)
    sizes = np.diff(res.ranges[(1 << 18) - 1:], axis=1).ravel()
    assert sizes.sum() == 1 << 26


@pytest.fixture(scope="module")
def batch128(oracle):
    specs = W.batched_instances(20270 + 77, 128)
    xs, ys, zs, inst, refs = [], [], [], [], []
    off = 0
    for sp in specs:
        x, y, z, ref = _plain(oracle, sp.kind, sp.seed, sp.n, sp.d)
        xs.append(x)
        ys.append(y)
        zs.append(z)
        inst.append({"offset": off, "n": sp.n, "d": sp.d})
        refs.append(ref)
        off += sp.n
    return np.concatenate(xs), np.concatenate(ys), np.concatenate(zs), inst, refs


@pytest.mark.parametrize("tuned_ctx", list(TUNINGS.values()), ids=list(TUNINGS), indirect=True)
def test_batch128_every_instance_bit_exact(tuned_ctx, batch128):
    x, y, z, inst, refs = batch128
    bx, by, bz = x.copy(), y.copy(), z.copy()
    parts, perm, _ = tuned_ctx.build_batch(bx, by, bz, inst)
    for i, ((heap, ranges), ins, ref) in enumerate(zip(parts, inst, refs)):
        a, b = ins["offset"], ins["offset"] + ins["n"]
        assert heap.tobytes() == ref.heap.tobytes(), f"instance {i}: heap differs"
        assert np.array_equal(ranges, ref.ranges[0]), f"instance {i}: ranges differ"
        assert np.array_equal(perm[a:b], ref.perm), f"instance {i}: permutation differs"
        for got, want in ((bx, ref.x), (by, ref.y), (bz, ref.z)):
            assert np.array_equal(got[a:b].view(np.uint32), want.view(np.uint32)), f"instance {i}"
