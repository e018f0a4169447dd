"""Whole ORB trees of the oracle against the reference's own CPU services.

src/services/count.cpp, countLeft.cpp, makeAxis.cpp and partition.cpp of the reference, with
its src/cell.h, compiled unchanged into oracle/_ref/librefsvc.so (`make -C oracle ref`,
where the reference's sources are present; skipped elsewhere) against the shim headers in
oracle/refshim, and sequenced as the reference's master() sequences its MDL services for
orbit mode o=0 (oracle/ref_services.cpp). Every output is compared bit for bit: the cell
heap, every rank's range map and the partitioned coordinates, for the single-rank oracle and
for its multi-rank mode (slabs, per-rank services, counts summed by the services' own
Combine()). Inputs avoid the cells where the reference's Hoare scan leaves the cell (every
key below the cut) and boxes without extent, where the reference's code is undefined."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SVC_LIB = os.path.join(ROOT, "oracle", "_ref", "librefsvc.so")


@pytest.fixture(scope="module")
def refsvc():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    if not os.path.exists(SVC_LIB):
        pytest.skip("the reference's sources are not present")
    L = ctypes.CDLL(SVC_LIB)
    vp = ctypes.c_void_p
    L.refsvc_build.restype = ctypes.c_int
    L.refsvc_build.argtypes = [vp, vp, vp, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, vp, vp,
                               vp, vp, ctypes.c_int]
    assert L.refsvc_cell_size() == 52
    return L


def ref_build(L, oracle, x, y, z, d, levels=None, nranks=1, lower=(-0.5,) * 3, upper=(0.5,) * 3):
    x, y, z = (np.array(a, np.float32, copy=True) for a in (x, y, z))
    levels = oracle.max_levels(d) if levels is None else levels
    heap = np.zeros(2 * d - 1, oracle.CELL_DTYPE)
    rng = np.zeros((nranks, 2 * d - 1, 2), np.uint32)
    lo, hi = np.asarray(lower, np.float32), np.asarray(upper, np.float32)
    assert L.refsvc_build(x.ctypes.data, y.ctypes.data, z.ctypes.data, x.size, d, levels,
                          lo.ctypes.data, hi.ctypes.data, heap.ctypes.data, rng.ctypes.data,
                          nranks) == 0
    return x, y, z, heap, rng


def grid(seed, n, values):
    rng = np.random.default_rng(seed)
    return [(rng.integers(0, values, n).astype(np.float32) / np.float32(values) - np.float32(0.5))
            for _ in range(3)]


CASES = [
    ("uniform", 1 << 16, 1 << 8, 1), ("plummer", 1 << 16, 1 << 10, 1), ("uniform", 100000, 100, 1),
    ("plummer", 60000, 12, 1), ("grid", 1 << 15, 1 << 5, 1), ("uniform", 70000, 1000, 1),
    ("uniform", 1 << 15, 1 << 6, 4), ("plummer", 50000, 1 << 7, 3), ("uniform", 70000, 1000, 2),
    ("grid", 1 << 15, 1 << 4, 3), ("uniform", (1 << 20) + 7, 1 << 10, 1),
]


@pytest.mark.parametrize("kind,n,d,nranks", CASES)
def test_oracle_is_the_reference_services(refsvc, oracle, kind, n, d, nranks):
    if kind == "grid":
        x, y, z = grid(n + d, n, 1024)  # ties at most cuts, no cell left all below its cut
    else:
        x, y, z = (oracle.gen_uniform if kind == "uniform" else oracle.gen_plummer)(n % 89 + d, n)
    ora = oracle.build_tree(x, y, z, d, nranks=nranks, make_axis=nranks > 1)
    assert ora.stats["degenerate_cells"] == 0 and ora.stats["zero_volume_cells"] == 0
    rx, ry, rz, heap, rng = ref_build(refsvc, oracle, x, y, z, d, nranks=nranks)
    assert heap.tobytes() == ora.heap.tobytes()
    assert np.array_equal(rng, ora.ranges)
    for a, b in ((rx, ora.x), (ry, ora.y), (rz, ora.z)):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_reference_bound_and_custom_box(refsvc, oracle):
    x, y, z = oracle.gen_uniform(5, 40000)
    x = x * np.float32(3)
    for d, levels in ((1 << 8, 7), (1 << 6, 3), (100, 4)):
        ora = oracle.build_tree(x, y, z, d, levels=levels, lower=(-1.5, -0.5, -0.5), upper=(1.5, 0.5, 0.5))
        rx, _, _, heap, rng = ref_build(refsvc, oracle, x, y, z, d, levels=levels,
                                        lower=(-1.5, -0.5, -0.5), upper=(1.5, 0.5, 0.5))
        assert heap.tobytes() == ora.heap.tobytes() and np.array_equal(rng, ora.ranges)
        assert np.array_equal(rx, ora.x)
