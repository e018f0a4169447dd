"""The rule behind staged builds from host memory (CPU, oracle only). The engine copies x, y, z
one after another and runs level 1 on x alone and level 2 on x and y while z is in flight.
That is exact only if level 1 cuts along x, which the reference forces (src/orbit.cpp:75),
and no level-2 cell cuts along z: a level-2 cell keeps the root's y and z extents and at most
its x extent, so setCutAxis's first-longest rule (src/cell.h:102-121) picks x or y whenever
the box's y side is at least as long as its z side and longer than zero. The engine stages
only such boxes. Checked on the oracle's trees over random boxes and inputs, including cuts
at the box edge (all particles on one face) and boxes where the rule does not hold (there a
level-2 cell can cut along z, so those boxes are not staged)."""
import numpy as np
import pytest


def level2_axes(oracle, x, y, z, d, lower, upper):
    ref = oracle.build_tree(x, y, z, d, levels=2, lower=lower, upper=upper)
    assert ref.heap[0]["cutAxis"] == 0
    return {int(a) for a in ref.heap[1:3]["cutAxis"]}


def staged_rule(lower, upper):
    ye = np.float32(upper[1]) - np.float32(lower[1])
    ze = np.float32(upper[2]) - np.float32(lower[2])
    return ye > 0 and ye >= ze


@pytest.mark.parametrize("seed", range(12))
def test_level2_never_cuts_along_z_when_staged(oracle, seed):
    rng = np.random.default_rng(seed)
    n, d = 4000, 4
    for _ in range(8):
        lo = rng.uniform(-2, 0, 3).astype(np.float32)
        ext = rng.uniform(0.1, 3, 3).astype(np.float32)
        if rng.random() < 0.5:
            ext[2] = ext[1] * np.float32(rng.uniform(0.2, 1.0))  # y at least as long as z
        if rng.random() < 0.2:
            ext[2] = ext[1]  # ties go to y
        hi = lo + ext
        pts = [rng.uniform(lo[a], hi[a], n).astype(np.float32) for a in range(3)]
        if rng.random() < 0.25:
            pts[0][:] = lo[0]  # every particle on one face: level 1 cuts at the box edge
        axes = level2_axes(oracle, *pts, d, tuple(lo), tuple(hi))
        if staged_rule(lo, hi):
            assert axes <= {0, 1}, (lo, hi, axes)


def test_rule_is_needed(oracle):
    # z longer than y and x: level 2 cuts along z, so such a box must not be staged
    rng = np.random.default_rng(7)
    lo, hi = (-0.5, -0.5, -2.0), (0.5, 0.5, 2.0)
    pts = [rng.uniform(lo[a], hi[a], 4000).astype(np.float32) for a in range(3)]
    assert not staged_rule(lo, hi)
    assert 2 in level2_axes(oracle, *pts, 4, lo, hi)
