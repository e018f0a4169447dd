"""Multi-rank ORB build over the service ABI: the reference's MDL decomposition.

The reference runs one MDL rank per core: every rank owns a slab of the particles and its
own LocalData (src/services/pst.h:6-41); the master hands the cells of a level to every rank,
each rank counts on its slab (ServiceCount, ServiceCountLeft) and MDL sums the per-cell
uint32 counts over the ranks (Combine, src/services/countLeft.cpp:44-53,
src/services/TraversePST.cpp:37-44); the master tests the cuts (src/orbit.cpp:191-231),
splits the cells (src/orbit.cpp:235-250) and every rank Hoare-partitions its own slab
(ServicePartition).

Here each rank's slab lives in an engine context (orb_load_particles) and is counted and
partitioned on the GPU through the service entry points (orb_count, orb_count_left,
orb_partition). The per-cell count vectors are the only data exchanged: they are summed over
the ranks this process drives and then over processes by an all-reduce (torch.distributed,
gloo or nccl). The cut tests and splits are computed on every rank from the same summed
counts, with the reference's float32 arithmetic, so every rank holds the same heap without a
broadcast. With one slab this is the reference's single-rank driver; with T slabs its
result equals the oracle's T-rank mode (the reference's MDL semantics) bit for bit.
"""
from __future__ import annotations

import math

import numpy as np

f32 = np.float32


def get_cut(cell) -> np.float32:
    """Cell::getCut(), src/cell.h:74-76: the float sum, halved in double, back to float."""
    s = f32(f32(cell["cutMarginRight"]) + f32(cell["cutMarginLeft"]))
    return f32(np.float64(s) / 2.0)


def convergence(count_left: int, count: int, n_leaf: int) -> int:
    """src/orbit.cpp:204-230: 0 found, +1 the right margin moves to the cut, -1 the left."""
    ratio = f32(math.ceil(n_leaf / 2.0) / n_leaf)
    difference = int(f32(f32(count_left) - f32(f32(count) * ratio)))
    if abs(difference) < 3:
        return 0
    return 1 if difference > 0 else -1


def _eff_axis(cell) -> int:
    a = int(cell["cutAxis"])
    return 0 if a < 0 else a


def _set_cut_axis_and_margin(cell):
    """setCutAxis (src/cell.h:102-121, strict > over the float extents) and setCutMargin
    (src/cell.h:123-126); a box without extent keeps axis -1 and takes axis 0's margins."""
    max_d, max_size = -1, f32(0.0)
    for k in range(3):
        size = f32(f32(cell["upper"][k]) - f32(cell["lower"][k]))
        if size > max_size:
            max_size, max_d = size, k
    cell["cutAxis"] = max_d
    a = 0 if max_d < 0 else max_d
    cell["cutMarginLeft"] = cell["lower"][a]
    cell["cutMarginRight"] = cell["upper"][a]


def split(heap, cid: int):
    """Cell::cut() (src/cell.h:78-100), then the right child's and the left child's
    setCutAxis() and setCutMargin() (src/orbit.cpp:240-243)."""
    p = heap[cid]
    n_left = math.ceil(int(p["nLeafCells"]) / 2.0)
    cut = get_cut(p)
    a = _eff_axis(p)
    for child, n_leaf, side in ((2 * cid + 1, n_left, "upper"),
                                (2 * cid + 2, int(p["nLeafCells"]) - n_left, "lower")):
        c = heap[child]
        c["id"] = child
        c["nLeafCells"] = n_leaf
        c["prevCutAxis"] = p["cutAxis"]
        c["foundCut"] = 0
        c["lower"] = p["lower"]
        c["upper"] = p["upper"]
        c[side][a] = cut
    _set_cut_axis_and_margin(heap[2 * cid + 2])
    _set_cut_axis_and_margin(heap[2 * cid + 1])


def level_shape(d: int):
    """(getNLevels(), getNCellsOnLastLevel()) of a root of d leaves (src/cell.h:65-72)."""
    depth = (d - 1).bit_length()
    return depth, 2 * d - (1 << depth)


def max_levels(d: int) -> int:
    depth, _ = level_shape(d)
    return depth if d & (d - 1) == 0 else max(depth - 1, 0)


def slabs(n: int, nranks: int):
    """The reference's slab split (src/orbit.cpp:83: N/Threads() particles a rank; the last
    rank also takes the remainder, so every particle is owned): [(offset, count)]."""
    return [((n // nranks) * r, n - (n // nranks) * r if r == nranks - 1 else n // nranks)
            for r in range(nranks)]


def build_ranks(ranks, d: int, levels: int = 0, lower=(-0.5, -0.5, -0.5), upper=(0.5, 0.5, 0.5),
                allreduce=None, cell_dtype=None):
    """The master loop of src/orbit.cpp:74-275 over the ranks' services.

    ranks      the ranks this process drives: objects with count(cells), count_left(cells,
               out) and partition(cells) (engine contexts after load_particles with at least
               2d-1 range-map cells, or any object with the same service semantics)
    allreduce  sums a uint32 vector over the other processes in place (None: one process)
    Returns the heap (every rank's is the same) as an array of cell_dtype."""
    if cell_dtype is None:
        import orb_gb300 as E
        cell_dtype = E.CELL_DTYPE
    levels = levels or max_levels(d)
    if levels > max_levels(d):
        raise ValueError("levels beyond the most for d")
    heap = np.zeros(2 * d - 1, cell_dtype)
    root = heap[0]
    root["nLeafCells"] = d
    root["prevCutAxis"] = -1
    root["cutAxis"] = 0  # src/orbit.cpp:75
    root["lower"] = np.asarray(lower, f32)
    root["upper"] = np.asarray(upper, f32)
    root["cutMarginLeft"], root["cutMarginRight"] = f32(lower[0]), f32(upper[0])

    def summed(fn, cells):
        total = np.zeros(len(cells), np.uint32)
        for r in ranks:
            out = np.zeros(len(cells), np.uint32)
            fn(r, cells, out)
            total += out
        if allreduce is not None:
            allreduce(total)
        return total

    _, last = level_shape(d)
    for l in range(1, levels + 1):
        a = (1 << (l - 1)) - 1  # src/orbit.cpp:104-107
        b = min(last, 1 << l) - 2
        if b < a:
            continue  # an empty slice: a level without cells
        cells = heap[a:b + 1].copy()
        counts = summed(lambda r, c, o: o.__setitem__(slice(None), r.count(c)), cells)
        for _ in range(32):  # src/orbit.cpp:146-232
            left = summed(lambda r, c, o: r.count_left(c, o), cells)
            found_all = True
            for i in range(len(cells)):
                c = cells[i]
                if c["foundCut"]:
                    continue
                dirn = convergence(int(left[i]), int(counts[i]), int(c["nLeafCells"]))
                if dirn == 0:
                    c["foundCut"] = 1
                else:
                    found_all = False
                    c["cutMarginRight" if dirn > 0 else "cutMarginLeft"] = get_cut(c)
            if found_all:
                break
        heap[a:b + 1] = cells
        for cid in range(a, b + 1):
            split(heap, cid)
        for r in ranks:
            r.partition(cells)
    return heap
