"""orb_count_left_static, the count-left that allocates nothing, against orb_count_left.

Callers that cannot allocate (a simulation that owns the whole device through its own
memory pool, or that cannot take the device-wide synchronisation of cudaMalloc/cudaFree
in its time step) use the static entry point. Its result must equal the context entry
point's bit for bit (integer counts), on consecutive calls that share its static scratch.
This file is collected last so a failure here leaves every other test already run.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cell_sets(oracle, heap):
    """Two disjoint-range cell sets from a finished oracle heap: level 6 with every second
    cell marked found, then level 7 with every third cell marked found."""
    a = heap[63:127].copy()
    a["foundCut"] = (np.arange(len(a)) % 2 == 1).astype(np.uint8)
    b = heap[127:255].copy()
    b["foundCut"] = (np.arange(len(b)) % 3 == 0).astype(np.uint8)
    return [a, b]


def test_count_left_static_matches_context(ctx, engine, oracle):
    torch = pytest.importorskip("torch")
    n, d = 1 << 18, 1 << 8
    x, y, z = oracle.gen_uniform(77, n)
    ref = oracle.build_tree(x, y, z, d)
    n_ranges = 2 * d - 1
    ranges = ref.ranges[0]
    ctx.load_particles(ref.x, ref.y, ref.z, n_ranges)
    ctx.set_ranges(ranges)
    dev = torch.device("cuda", 0)
    tx, ty, tz = (torch.from_numpy(a.copy()).to(dev) for a in (ref.x, ref.y, ref.z))
    tr = torch.from_numpy(ranges.reshape(-1).view(np.int32).copy()).to(dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for cells in _cell_sets(oracle, ref.heap):
        sentinel = np.uint32(0xA5A5A5A5)
        expect = ctx.count_left(cells, out=np.full(len(cells), sentinel, np.uint32))
        tc = torch.from_numpy(cells.view(np.uint8).copy()).to(dev)
        to = torch.full((len(cells),), int(np.int32(sentinel.view(np.int32))), dtype=torch.int32,
                        device=dev)
        engine.count_left_static(tx, ty, tz, n, tc, len(cells), tr, n_ranges, to, stream)
        torch.cuda.synchronize(dev)
        got = to.cpu().numpy().view(np.uint32)
        assert np.array_equal(got, expect)
        # found cells untouched, the others hold the oracle's count below the cut
        found = cells["foundCut"] == 1
        assert np.all(got[found] == sentinel)
        for i in np.nonzero(~found)[0][:8]:
            b, e = ranges[cells[i]["id"]]
            keys = (ref.x, ref.y, ref.z)[cells[i]["cutAxis"]]
            cut = oracle.get_cut(float(cells[i]["cutMarginLeft"]), float(cells[i]["cutMarginRight"]))
            assert got[i] == oracle.count_left(keys, cut, int(b), int(e))


def test_count_left_static_rejects_too_many_cells(engine):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    dummy = torch.zeros(16, dtype=torch.int32, device=dev)
    with pytest.raises(engine.OrbError) as e:
        engine.count_left_static(dummy, dummy, dummy, 16, dummy, engine.ORB_STATIC_MAX_CELLS + 1,
                                 dummy, 1, dummy)
    assert e.value.status == 4
