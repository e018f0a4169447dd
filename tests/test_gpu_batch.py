"""Batched builds (orb_build_batch): every instance of a packed batch must equal its own
plain build and the oracle on that instance alone, bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_batch(oracle, specs, gap=0):
    """specs: list of (kind, seed, n, d, levels). Packs the instances (with `gap` unused
    particles between them) and returns the arrays, the descriptors and the inputs."""
    xs, ys, zs, inst, inputs = [], [], [], [], []
    off = 0
    for kind, seed, n, d, levels in specs:
        gen = oracle.gen_uniform if kind == "uniform" else oracle.gen_plummer
        x, y, z = gen(seed, n) if n else (np.zeros(0, np.float32),) * 3
        xs += [x, np.full(gap, 9.0, np.float32)]
        ys += [y, np.full(gap, 9.0, np.float32)]
        zs += [z, np.full(gap, 9.0, np.float32)]
        inst.append({"offset": off, "n": n, "d": d, "levels": levels})
        inputs.append((x, y, z))
        off += n + gap
    return (np.concatenate(xs), np.concatenate(ys), np.concatenate(zs), inst, inputs)


def check_batch(ctx, oracle, specs, gap=0):
    x, y, z, inst, inputs = make_batch(oracle, specs, gap)
    bx, by, bz = x.copy(), y.copy(), z.copy()
    parts, perm, info = ctx.build_batch(bx, by, bz, inst)
    for i, ((heap, ranges), ins, (ix, iy, iz)) in enumerate(zip(parts, inst, inputs)):
        levels = ins["levels"] or None
        ref = oracle.build_tree(ix, iy, iz, ins["d"], levels=levels)
        a, b = ins["offset"], ins["offset"] + ins["n"]
        assert heap.tobytes() == ref.heap.tobytes(), f"instance {i}: heap differs"
        assert np.array_equal(ranges, ref.ranges[0]), f"instance {i}: ranges differ"
        assert np.array_equal(perm[a:b], ref.perm), f"instance {i}: permutation differs"
        for got, want in ((bx, ref.x), (by, ref.y), (bz, ref.z)):
            assert np.array_equal(got[a:b].view(np.uint32), want.view(np.uint32))
    # particles between instances are untouched
    if gap:
        owned = np.zeros(len(x), bool)
        for ins in inst:
            owned[ins["offset"]:ins["offset"] + ins["n"]] = True
        assert np.all(bx[~owned] == 9.0)
    return parts, info


def test_batch_uneven_instances(any_ctx, oracle):
    rng = np.random.default_rng(21)
    specs = []
    for i in range(24):
        n = int(2 ** rng.uniform(10, 16))
        d = 1 << int(rng.integers(2, 9))
        specs.append(("uniform" if i % 2 == 0 else "plummer", 1000 + i, n, d, 0))
    check_batch(any_ctx, oracle, specs)


def test_batch_tiny_empty_and_reference_levels(any_ctx, oracle):
    specs = [("uniform", 1, 0, 4, 0), ("uniform", 2, 1, 2, 0), ("plummer", 3, 7, 8, 0),
             ("uniform", 4, 5000, 1 << 10, 0), ("uniform", 5, 3000, 64, 5),
             ("plummer", 6, 20000, 1 << 6, 0), ("uniform", 7, 300, 1, 0)]
    check_batch(any_ctx, oracle, specs, gap=3)


def test_batch_equals_plain_builds(ctx, oracle):
    specs = [("uniform", 40 + i, 1 << (12 + i % 5), 1 << (3 + i % 6), 0) for i in range(12)]
    x, y, z, inst, inputs = make_batch(oracle, specs)
    parts, perm, _ = ctx.build_batch(x.copy(), y.copy(), z.copy(), inst)
    for (heap, ranges), ins, (ix, iy, iz) in zip(parts, inst, inputs):
        px, py, pz = ix.copy(), iy.copy(), iz.copy()
        alone = ctx.build(px, py, pz, ins["d"])
        assert heap.tobytes() == alone.heap.tobytes()
        assert np.array_equal(ranges, alone.ranges)
        a, b = ins["offset"], ins["offset"] + ins["n"]
        assert np.array_equal(perm[a:b], alone.perm)


def test_batch_rejects_overlap(ctx, engine):
    x = np.zeros(100, np.float32)
    inst = [{"offset": 0, "n": 60, "d": 4}, {"offset": 50, "n": 50, "d": 4}]
    with pytest.raises(engine.OrbError):
        ctx.build_batch(x, x.copy(), x.copy(), inst)


def test_batch_non_power_of_two_instances(ctx, oracle):
    """Instances with leaf counts that are not powers of two, beside powers of two, at
    their default (most) levels and below."""
    specs = [("uniform", 41, 20000, 3, 0), ("plummer", 42, 30000, 100, 0),
             ("uniform", 43, 15000, 64, 0), ("plummer", 44, 40000, 1000, 0),
             ("uniform", 45, 9000, 12, 2), ("uniform", 46, 25000, 7, 0)]
    check_batch(ctx, oracle, specs, gap=5)
