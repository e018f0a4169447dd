"""Shared checks for the parity tests."""
import numpy as np


def tree_properties(x, y, z, heap, ranges, n, d, levels):
    """Size-independent properties of a finished ORB build (no oracle needed)."""
    pts = np.stack([x, y, z], axis=1)
    first_leaf = (1 << levels) - 1
    leaves = np.arange(first_leaf, 2 * first_leaf + 1)
    # children of every split cell partition its range
    for cid in range(first_leaf):
        b, e = ranges[cid]
        lb, le = ranges[2 * cid + 1]
        rb, re = ranges[2 * cid + 2]
        assert lb == b and le == rb and re == e, f"cell {cid}: children do not tile the range"
    lr = ranges[leaves]
    assert lr[0, 0] == 0 and lr[-1, 1] == n
    assert np.all(lr[1:, 0] == lr[:-1, 1])
    # every particle lies in the closed box of its leaf
    for cid in leaves:
        b, e = ranges[cid]
        if e == b:
            continue
        p = pts[b:e]
        lo = heap[cid]["lower"]
        hi = heap[cid]["upper"]
        assert np.all(p >= lo) and np.all(p <= hi), f"leaf {cid}: particle outside its box"
