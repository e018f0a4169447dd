"""Launch tuning and the autotuner: every setting builds the same trees (the parameters only
spread the work differently), out-of-range settings are refused, and the autotuner leaves
its inputs untouched and installs a setting under which builds still equal the oracle."""
import numpy as np
import pytest

from test_gpu_batch import make_batch

pytestmark = pytest.mark.gpu

EXTREMES = [
    dict(hist_blocks_per_sm=1, part_blocks_per_sm=1, tile_blocks_per_sm=1, sparse_keys_per_tile=1,
         cta_min_cells=0, subtree_levels=0, predict_sigmas=0),
    dict(hist_blocks_per_sm=8, part_blocks_per_sm=16, tile_blocks_per_sm=4,
         sparse_keys_per_tile=16384, cta_min_cells=0, subtree_levels=6, predict_sigmas=16),
    dict(hist_blocks_per_sm=3, part_blocks_per_sm=5, tile_blocks_per_sm=2, sparse_keys_per_tile=7,
         cta_min_cells=64, subtree_levels=2, predict_sigmas=1),
]


@pytest.fixture
def fresh(engine):
    c = engine.Context(0)
    yield c
    c.close()


def test_get_set_roundtrip_and_limits(fresh, engine):
    d = fresh.get_tuning()
    assert d == dict(hist_blocks_per_sm=6, part_blocks_per_sm=8, tile_blocks_per_sm=4,
                     sparse_keys_per_tile=64, cta_min_cells=0, subtree_levels=4, predict_sigmas=0)
    fresh.set_tuning(part_blocks_per_sm=12, sparse_keys_per_tile=100)
    assert fresh.get_tuning()["part_blocks_per_sm"] == 12
    assert fresh.get_tuning()["sparse_keys_per_tile"] == 100
    for bad in (dict(hist_blocks_per_sm=0), dict(hist_blocks_per_sm=9), dict(part_blocks_per_sm=17),
                dict(tile_blocks_per_sm=9), dict(sparse_keys_per_tile=0),
                dict(sparse_keys_per_tile=16385), dict(subtree_levels=7),
                dict(predict_sigmas=17)):
        with pytest.raises(engine.OrbError):
            fresh.set_tuning(**bad)
    assert fresh.get_tuning()["part_blocks_per_sm"] == 12  # a refused setting changes nothing


@pytest.mark.parametrize("setting", EXTREMES)
def test_settings_do_not_change_results(fresh, oracle, setting):
    x, y, z = oracle.gen_plummer(77, 200000)
    ref = oracle.build_tree(x, y, z, 1 << 9)
    fresh.set_tuning(**setting)
    r = fresh.build(x.copy(), y.copy(), z.copy(), 1 << 9)
    assert r.heap.tobytes() == ref.heap.tobytes()
    assert np.array_equal(r.ranges, ref.ranges[0])
    assert np.array_equal(r.perm, ref.perm)


def test_autotune_batch(fresh, oracle):
    specs = [("uniform" if i % 2 == 0 else "plummer", 300 + i, 3000 + 7919 * i, 1 << (4 + i % 6), 0)
             for i in range(16)]
    x, y, z, inst, inputs = make_batch(oracle, specs)
    keep = [a.copy() for a in (x, y, z)]
    best, ms = fresh.autotune_batch(x, y, z, inst, reps=2)
    assert ms > 0
    assert fresh.get_tuning() == best
    for a, b in zip((x, y, z), keep):  # inputs untouched
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    parts, perm, _ = fresh.build_batch(x, y, z, inst)
    for (heap, ranges), ins, (ix, iy, iz) in zip(parts, inst, inputs):
        ref = oracle.build_tree(ix, iy, iz, ins["d"])
        assert heap.tobytes() == ref.heap.tobytes()
        assert np.array_equal(ranges, ref.ranges[0])
