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


def test_count_left_static_at_capacity_with_bad_cells(ctx, engine, oracle):
    """ORB_STATIC_MAX_CELLS cells in one call (the plan kernel's threads then walk several
    cells each), twice in a row on the shared scratch: equal to orb_count_left; cells whose
    id lies outside the range map or whose range is corrupt count 0; a call where every cell
    is found leaves the output untouched."""
    torch = pytest.importorskip("torch")
    n, d = 1 << 20, 1 << 16
    x, y, z = oracle.gen_uniform(78, n)
    ref = oracle.build_tree(x, y, z, d)
    n_ranges = 2 * d - 1
    ranges = ref.ranges[0].copy()
    ctx.load_particles(ref.x, ref.y, ref.z, n_ranges)
    ctx.set_ranges(ranges)
    dev = torch.device("cuda", 0)
    tx, ty, tz = (torch.from_numpy(a.copy()).to(dev) for a in (ref.x, ref.y, ref.z))
    stream = torch.cuda.current_stream(dev).cuda_stream
    leaves = ref.heap[d - 1:].copy()  # 65536 cells with disjoint ranges
    assert len(leaves) == engine.ORB_STATIC_MAX_CELLS
    leaves["foundCut"] = (np.arange(len(leaves)) % 5 == 0).astype(np.uint8)
    expect = ctx.count_left(leaves, out=np.zeros(len(leaves), np.uint32))
    sentinel = 0xA5A5A5A5

    def static(cells, rng):
        tc = torch.from_numpy(cells.view(np.uint8).copy()).to(dev)
        tr = torch.from_numpy(rng.reshape(-1).view(np.int32).copy()).to(dev)
        to = torch.full((len(cells),), int(np.int32(np.uint32(sentinel).view(np.int32))),
                        dtype=torch.int32, device=dev)
        engine.count_left_static(tx, ty, tz, n, tc, len(cells), tr, n_ranges, to, stream)
        torch.cuda.synchronize(dev)
        return to.cpu().numpy().view(np.uint32)

    for _ in range(2):
        got = static(leaves, ranges)
        found = leaves["foundCut"] == 1
        assert np.array_equal(got[~found], expect[~found])
        assert np.all(got[found] == sentinel)
    # out-of-map ids and corrupt ranges count 0 (the context entry point rejects such calls)
    bad = leaves.copy()
    bad["foundCut"] = 0
    bad["id"][1:40:3] = n_ranges + np.arange(13)
    bad["id"][2:30:7] = -1 - np.arange(4)
    bad_rng = ranges.copy()
    corrupt = bad["id"][100:120].astype(np.int64)
    bad_rng[corrupt[:10], 0] = bad_rng[corrupt[:10], 1] + 1   # begin > end
    bad_rng[corrupt[10:], 1] = n + 7                          # end beyond n
    got = static(bad, bad_rng)
    zero = np.zeros(len(bad), bool)
    zero[1:40:3] = zero[2:30:7] = zero[100:120] = True
    assert np.all(got[zero] == 0)
    full = leaves.copy()
    full["foundCut"] = 0
    want = ctx.count_left(full, out=np.zeros(len(full), np.uint32))
    assert np.array_equal(got[~zero], want[~zero])
    # every cell found: nothing written
    done = leaves.copy()
    done["foundCut"] = 1
    assert np.all(static(done, ranges) == sentinel)
