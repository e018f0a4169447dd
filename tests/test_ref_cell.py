"""The oracle's cut and split arithmetic against the reference's own code: src/cell.h of
the reference, compiled unchanged into oracle/_ref/ (`make -C oracle ref`, where the
reference's sources are present; skipped elsewhere). Every split of the oracle's trees must
be the reference's cut() + setCutAxis() + setCutMargin() of the parent (src/orbit.cpp:
235-243), the root its Cell(0, d, lower, upper) with cutAxis 0 (src/orbit.cpp:74-76), and
getCut() the same float32 value."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libcellref.so")
f32 = np.float32


@pytest.fixture(scope="module")
def ref():
    # the recipe builds the library where the reference's sources are present, else nothing
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    if not os.path.exists(REF_LIB):
        pytest.skip("the reference's sources are not present")
    L = ctypes.CDLL(REF_LIB)
    L.ref_get_cut.restype = ctypes.c_float
    L.ref_get_cut.argtypes = [ctypes.c_float, ctypes.c_float]
    L.ref_split.restype = ctypes.c_int
    L.ref_split.argtypes = [ctypes.c_void_p] * 3
    L.ref_root.restype = None
    L.ref_root.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.ref_levels.restype = None
    L.ref_levels.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    assert ctypes.CDLL(REF_LIB).ref_cell_size() == 52
    return L


def same_f32(a, b):
    return np.asarray(a, f32).view(np.uint32) == np.asarray(b, f32).view(np.uint32)


def test_get_cut_is_the_references(ref, oracle):
    rng = np.random.default_rng(11)
    vals = np.concatenate([rng.uniform(-1, 1, 3000), rng.uniform(-1e30, 1e30, 500),
                           rng.uniform(-1e-38, 1e-38, 500)]).astype(f32)
    vals = np.concatenate([vals, np.array([0.0, -0.0, 1e-45, -1e-45, 0.5, -0.5], f32)])
    for _ in range(4000):
        a, b = (f32(v) for v in rng.choice(vals, 2))
        lo, hi = min(a, b), max(a, b)
        assert same_f32(ref.ref_get_cut(float(lo), float(hi)), oracle.get_cut(float(lo), float(hi)))


@pytest.mark.parametrize("kind,seed,n,d", [("uniform", 21, 1 << 14, 1 << 6),
                                           ("plummer", 22, 1 << 14, 1 << 8),
                                           ("grid", 23, 1 << 12, 1 << 6)])
def test_splits_are_the_references(ref, oracle, kind, seed, n, d):
    if kind == "grid":  # coordinates on a 16-value grid: ties, cuts on keys, unfound cells
        rng = np.random.default_rng(seed)
        x, y, z = ((rng.integers(0, 16, n).astype(f32) / f32(16) - f32(0.5)) for _ in range(3))
    else:
        x, y, z = (oracle.gen_uniform if kind == "uniform" else oracle.gen_plummer)(seed, n)
    lower, upper = np.full(3, -0.5, f32), np.full(3, 0.5, f32)
    heap = oracle.build_tree(x, y, z, d).heap
    fields = ("id", "nLeafCells", "prevCutAxis", "cutAxis", "lower", "upper")
    root = np.zeros(1, heap.dtype)
    ref.ref_root(d, lower.ctypes.data, upper.ctypes.data, root.ctypes.data)
    for f in fields + ("cutMarginLeft", "cutMarginRight"):
        if f in ("cutMarginLeft", "cutMarginRight"):
            continue  # the heap keeps the root's final margins
        assert np.array_equal(root[0][f], heap[0][f]), f"root {f}"
    leaves_from = d - 1
    checked = 0
    for cid in range(d - 1):
        parent = heap[cid:cid + 1].copy()
        if parent[0]["cutAxis"] < 0:
            continue  # no positive extent: the reference reads outside the box there
        left, right = np.zeros(1, heap.dtype), np.zeros(1, heap.dtype)
        undefined = ref.ref_split(parent.ctypes.data, left.ctypes.data, right.ctypes.data)
        for child, want in ((left, heap[2 * cid + 1]), (right, heap[2 * cid + 2])):
            for f in fields:
                if undefined and f == "cutAxis" and child[0]["cutAxis"] < 0:
                    continue
                assert np.all(same_f32(child[0][f], want[f])) if child[0][f].dtype == f32 \
                    else np.array_equal(child[0][f], want[f]), f"cell {cid}: child {f} differs"
            if want["id"] >= leaves_from and child[0]["cutAxis"] >= 0:
                # leaves keep the margins the split set (they are never bisected)
                assert same_f32(child[0]["cutMarginLeft"], want["cutMarginLeft"])
                assert same_f32(child[0]["cutMarginRight"], want["cutMarginRight"])
        checked += 1
    assert checked >= d // 2


def test_level_slices_are_the_references(ref, oracle):
    ds = [1 << y for y in range(0, 21)] + list(range(1, 1100)) + [12345, 99999, (1 << 20) + 3]
    for d in ds:
        nl, nc = ctypes.c_int(), ctypes.c_int()
        ref.ref_levels(d, ctypes.byref(nl), ctypes.byref(nc))
        assert (nl.value, nc.value) == oracle.level_shape(d), d
        if d & (d - 1) == 0:
            assert (nl.value, nc.value) == (d.bit_length() - 1, d)


@pytest.mark.parametrize("d", [3, 6, 7, 11, 12, 100, 1000])
def test_non_power_of_two_splits_are_the_references(ref, oracle, d):
    """Trees of d leaves not a power of two: every split (leaf counts ceil(k/2) and the rest,
    boxes, axes, margins) is the reference's cut() + setCutAxis() + setCutMargin()."""
    x, y, z = oracle.gen_plummer(d, 1 << 14)
    heap = oracle.build_tree(x, y, z, d).heap
    checked = 0
    for cid in range(len(heap)):
        if heap[cid]["nLeafCells"] == 0 or 2 * cid + 2 >= len(heap) or heap[2 * cid + 1]["nLeafCells"] == 0:
            continue
        parent = heap[cid:cid + 1].copy()
        left, right = np.zeros(1, heap.dtype), np.zeros(1, heap.dtype)
        ref.ref_split(parent.ctypes.data, left.ctypes.data, right.ctypes.data)
        for child, want in ((left, heap[2 * cid + 1]), (right, heap[2 * cid + 2])):
            for f in ("id", "nLeafCells", "prevCutAxis", "cutAxis", "lower", "upper"):
                assert np.array_equal(child[0][f], want[f]), f"d={d} cell {cid}: {f}"
        checked += 1
    assert checked >= 1
