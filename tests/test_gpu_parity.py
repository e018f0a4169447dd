"""GPU parity of the engine (through the C ABI) against the CPU oracle.

Bit-exact on every output: the cell heap (cuts, margins, found flags, boxes, axes), the
range map, the permutation (particle -> position) and the reordered coordinates."""
import numpy as np
import pytest


pytestmark = pytest.mark.gpu


def first_heap_diff(a, b):
    for i in range(len(a)):
        if a[i].tobytes() != b[i].tobytes():
            return i, a[i], b[i]
    return None


def assert_same(res, ref, gx, gy, gz):
    d = first_heap_diff(res.heap, ref.heap)
    assert d is None, f"heap differs first at cell {d[0]}:\n gpu {d[1]}\n cpu {d[2]}"
    assert np.array_equal(res.ranges, ref.ranges[0]), "range map differs"
    assert np.array_equal(res.perm, ref.perm), "particle order differs"
    for a, b in ((gx, ref.x), (gy, ref.y), (gz, ref.z)):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), "coordinates differ"


def run_both(ctx, oracle, x, y, z, d, levels=0, **kw):
    ref = oracle.build_tree(x, y, z, d, levels=(levels or None), **kw)
    gx, gy, gz = x.copy(), y.copy(), z.copy()
    res = ctx.build(gx, gy, gz, d, levels=levels, **kw)
    assert_same(res, ref, gx, gy, gz)
    assert res.info["degenerate_cells"] == ref.stats["degenerate_cells"]
    assert res.info["unfound_cells"] == ref.stats["unfound_cells"]
    assert res.info["zero_volume_cells"] == ref.stats["zero_volume_cells"]
    return res, ref


@pytest.mark.parametrize("kind", ["uniform", "plummer"])
def test_generator_bit_exact(ctx, engine, oracle, kind):
    n = (1 << 20) + 37
    gen = oracle.gen_uniform if kind == "uniform" else oracle.gen_plummer
    x, y, z = gen(42, n)
    k = engine.ORB_GEN_UNIFORM if kind == "uniform" else engine.ORB_GEN_PLUMMER
    gx, gy, gz = ctx.generate_host(k, 42, n)
    assert np.array_equal(gx, x) and np.array_equal(gy, y) and np.array_equal(gz, z)


def test_reference_generator_stream(ctx, engine, oracle):
    """ORB_GEN_XORSHF96: the reference's own input stream (src/services/init.cu:11-25),
    generated on the device by jumps of the generator's linear map, bit for bit the
    sequential stream; `seed` skips draws."""
    n = (1 << 20) + 7
    x, y, z = oracle.gen_xorshf96(n)
    gx, gy, gz = ctx.generate_host(engine.ORB_GEN_XORSHF96, 0, n)
    assert np.array_equal(gx, x) and np.array_equal(gy, y) and np.array_equal(gz, z)
    k = 12345
    sx, sy, sz = ctx.generate_host(engine.ORB_GEN_XORSHF96, 3 * k, n - k)
    assert np.array_equal(sx, x[k:]) and np.array_equal(sz, z[k:])
    sx, sy, sz = ctx.generate_host(engine.ORB_GEN_XORSHF96, 1, 5)  # skip one draw: y_0 first
    assert sx[0] == y[0] and sy[0] == z[0] and sz[0] == x[1]


def test_reference_input_build(ctx, engine, oracle):
    """`orbit 20 10 0` on the reference's own input: 2^20 xorshf96 particles, 2^10 leaves,
    the reference's loop bound (9 levels), bit-exact."""
    n, d = 1 << 20, 1 << 10
    x, y, z = ctx.generate_host(engine.ORB_GEN_XORSHF96, 0, n)
    run_both(ctx, oracle, x, y, z, d, levels=9)


@pytest.mark.parametrize("n,d,seed", [(1 << 12, 1 << 4, 1), (1 << 16, 1 << 8, 2),
                                      ((1 << 16) + 123, 1 << 9, 3), (50000, 1 << 12, 4)])
def test_uniform_parity(any_ctx, oracle, n, d, seed):
    x, y, z = oracle.gen_uniform(seed, n)
    run_both(any_ctx, oracle, x, y, z, d)


def test_config1_parity(ctx, oracle):
    """2^20 uniform particles, 2^10 leaves (the reference's CPU-runnable case)."""
    x, y, z = oracle.gen_uniform(2024, 1 << 20)
    res, ref = run_both(ctx, oracle, x, y, z, 1 << 10)
    assert res.info["max_iterations"] == max(ref.stats["iterations"])


@pytest.mark.parametrize("n,d,seed", [(1 << 16, 1 << 10, 5), (1 << 18, 1 << 12, 6)])
def test_plummer_parity(any_ctx, oracle, n, d, seed):
    x, y, z = oracle.gen_plummer(seed, n)
    run_both(any_ctx, oracle, x, y, z, d)


def test_tie_heavy_parity(any_ctx, oracle):
    """Coordinates on a 64-value grid: most cuts land on keys, Hoare tie placement decides
    membership."""
    rng = np.random.default_rng(7)
    n = 1 << 17
    x, y, z = ((rng.integers(0, 64, n).astype(np.float32) / np.float32(64) - np.float32(0.5))
               for _ in range(3))
    res, ref = run_both(any_ctx, oracle, x, y, z, 1 << 10)
    assert ref.stats["unfound_cells"] > 0  # the grid defeats the bisection somewhere


def test_small_and_degenerate_cells(any_ctx, oracle):
    rng = np.random.default_rng(8)
    for n in (0, 1, 2, 3, 5, 7, 17, 100):
        for d in (1, 2, 4, 16):
            x, y, z = (rng.random(n).astype(np.float32) - np.float32(0.5) for _ in range(3))
            run_both(any_ctx, oracle, x, y, z, d)


def test_duplicates_nan_out_of_box(any_ctx, oracle):
    n = 4096
    same = np.full(n, 0.25, np.float32)
    run_both(any_ctx, oracle, same, same.copy(), same.copy(), 8)
    # a bracket that never shrinks below the shared list: repeated histogram passes
    big = np.full(40000, -0.125, np.float32)
    big[::7] = 0.3
    run_both(any_ctx, oracle, big, big.copy(), big[::-1].copy(), 4)
    rng = np.random.default_rng(9)
    x = rng.random(n).astype(np.float32) - np.float32(0.5)
    x[rng.integers(0, n, 200)] = np.nan
    y = rng.random(n).astype(np.float32) * np.float32(4) - np.float32(2)  # out of the box
    z = np.round(rng.random(n).astype(np.float32) * 8) / np.float32(8) - np.float32(0.5)
    run_both(any_ctx, oracle, x, y, z, 64)


def test_reference_level_bound(any_ctx, oracle):
    """levels = log2(d)-1 is the reference driver's own loop (d/2 leaves)."""
    x, y, z = oracle.gen_uniform(10, 1 << 15)
    run_both(any_ctx, oracle, x, y, z, 1 << 8, levels=7)


def test_custom_box(any_ctx, oracle):
    x, y, z = oracle.gen_uniform(12, 1 << 14)
    x = x * np.float32(3)
    run_both(any_ctx, oracle, x, y, z, 1 << 6, lower=(-1.5, -0.5, -0.5), upper=(1.5, 0.5, 0.5))


def test_device_pointers(ctx, oracle):
    torch = pytest.importorskip("torch")
    n, d = 1 << 18, 1 << 10
    x, y, z = oracle.gen_uniform(13, n)
    ref = oracle.build_tree(x, y, z, d)
    tx, ty, tz = (torch.from_numpy(a.copy()).cuda() for a in (x, y, z))
    tp = torch.empty(n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    res = ctx.build(tx, ty, tz, d, perm=tp, device_pointers=True)
    assert res.heap.tobytes() == ref.heap.tobytes()
    assert np.array_equal(res.ranges, ref.ranges[0])
    assert np.array_equal(tp.cpu().numpy().view(np.uint32), ref.perm)
    assert np.array_equal(tx.cpu().numpy().view(np.uint32), ref.x.view(np.uint32))


def test_service_layer(ctx, engine, oracle):
    """orb_count / orb_count_left / orb_partition reproduce the reference's services when
    driven by a host-side master loop (src/orbit.cpp:102-275)."""
    n, d = 1 << 15, 1 << 5
    x, y, z = oracle.gen_uniform(14, n)
    ref = oracle.build_tree(x, y, z, d)
    heap_cells = 2 * d - 1
    ctx.load_particles(x, y, z, heap_cells)
    heap = np.zeros(heap_cells, engine.CELL_DTYPE)
    heap[0]["nLeafCells"] = d
    heap[0]["prevCutAxis"] = -1
    heap[0]["cutAxis"] = 0
    heap[0]["lower"] = (-0.5, -0.5, -0.5)
    heap[0]["upper"] = (0.5, 0.5, 0.5)
    heap[0]["cutMarginLeft"], heap[0]["cutMarginRight"] = -0.5, 0.5
    levels = d.bit_length() - 1
    for l in range(1, levels + 1):
        a, b = (1 << (l - 1)) - 1, (1 << l) - 2
        cells = heap[a:b + 1].copy()
        counts = ctx.count(cells)
        left = np.zeros(len(cells), np.uint32)
        for _ in range(32):
            ctx.count_left(cells, left)
            done = True
            for i in range(len(cells)):
                if cells[i]["foundCut"]:
                    continue
                r, _ = oracle.convergence(int(left[i]), int(counts[i]), int(cells[i]["nLeafCells"]))
                cut = oracle.get_cut(float(cells[i]["cutMarginLeft"]), float(cells[i]["cutMarginRight"]))
                if r == 0:
                    cells[i]["foundCut"] = 1
                elif r > 0:
                    cells[i]["cutMarginRight"] = cut
                    done = False
                else:
                    cells[i]["cutMarginLeft"] = cut
                    done = False
            if done:
                break
        heap[a:b + 1] = cells
        # split on the host from the oracle's heap (the services do not split)
        for c in range(a, b + 1):
            heap[2 * c + 1] = ref.heap[2 * c + 1]
            heap[2 * c + 2] = ref.heap[2 * c + 2]
        ctx.partition(cells)
    assert heap.tobytes() == ref.heap.tobytes()
    assert np.array_equal(ctx.get_ranges(heap_cells), ref.ranges[0])
    sx, sy, sz, sp = ctx.store_particles()
    assert np.array_equal(sp, ref.perm) and np.array_equal(sx.view(np.uint32), ref.x.view(np.uint32))


def test_large_parity(ctx, oracle):
    """2^24 particles, 2^13 leaves: bit-exact against the oracle."""
    x, y, z = oracle.gen_uniform(99, 1 << 24)
    run_both(ctx, oracle, x, y, z, 1 << 13)


@pytest.mark.parametrize("d", [3, 5, 6, 7, 11, 12, 100, 1000])
def test_non_power_of_two_leaves(any_ctx, oracle, d):
    """d not a power of two, at the reference's own bound getNLevels()-1: the level slices
    of src/orbit.cpp:104-107 (partial or empty where getNCellsOnLastLevel() cuts them), the
    ceil(k/2) split of src/cell.h:79 and the ratio ceil(k/2)/k of src/orbit.cpp:204, which
    rounds in float32 for odd k (2/3 for k = 3)."""
    n = 1 << 16
    x, y, z = (oracle.gen_uniform if d % 2 else oracle.gen_plummer)(300 + d, n)
    res, ref = run_both(any_ctx, oracle, x, y, z, d)
    assert res.info["levels_built"] == oracle.max_levels(d)
    # the odd leaf counts really occur (not only at d itself)
    split = ref.heap[ref.heap["nLeafCells"] > 0]
    if d in (3, 7, 11, 100, 1000):
        assert (split["nLeafCells"] % 2 == 1).any()


def test_non_power_of_two_lower_levels_and_bounds(ctx, engine, oracle):
    x, y, z = oracle.gen_uniform(333, 50000)
    for d, levels in ((100, 3), (1000, 5), (6, 1)):
        run_both(ctx, oracle, x, y, z, d, levels=levels)
    with pytest.raises(engine.OrbError):
        ctx.build(x.copy(), y.copy(), z.copy(), 100, levels=7)  # beyond getNLevels()-1


@pytest.mark.parametrize("kind,seed,logn,logd", [("plummer", 501, 20, 15), ("uniform", 502, 21, 12),
                                                 ("plummer", 503, 19, 13)])
def test_subtree_levels_match_oracle(ctx, oracle, kind, seed, logn, logd):
    # deep trees whose last levels (cells of at most ~17K particles, up to 6 levels) are
    # finished by one CTA per cell
    gen = oracle.gen_uniform if kind == "uniform" else oracle.gen_plummer
    x, y, z = gen(seed, 1 << logn)
    ref = oracle.build_tree(x, y, z, 1 << logd)
    r = ctx.build(x.copy(), y.copy(), z.copy(), 1 << logd)
    assert r.heap.tobytes() == ref.heap.tobytes()
    assert np.array_equal(r.ranges, ref.ranges[0])
    assert np.array_equal(r.perm, ref.perm)
