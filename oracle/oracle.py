"""ctypes front end of the CPU oracle (test infrastructure only).

The oracle restates the reference's CPU-only ORB path (orbit mode o=0) in C++; see
orb_oracle.h for the reference files it follows. Only tests, the smoke check and the
benchmark's CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liborb_oracle.so")

CELL_DTYPE = np.dtype(
    [
        ("id", "<i4"),
        ("nLeafCells", "<i4"),
        ("prevCutAxis", "<i4"),
        ("cutAxis", "<i4"),
        ("foundCut", "u1"),
        ("pad_", "u1", (3,)),
        ("cutMarginLeft", "<f4"),
        ("cutMarginRight", "<f4"),
        ("lower", "<f4", (3,)),
        ("upper", "<f4", (3,)),
    ]
)
assert CELL_DTYPE.itemsize == 52

MAX_LEVELS = 40


class _Stats(ctypes.Structure):
    _fields_ = [
        ("levels_built", ctypes.c_uint32),
        ("iterations", ctypes.c_uint32 * MAX_LEVELS),
        ("cell_counts", ctypes.c_uint64),
        ("elements_counted", ctypes.c_uint64),
        ("degenerate_cells", ctypes.c_uint32),
        ("zero_volume_cells", ctypes.c_uint32),
        ("unfound_cells", ctypes.c_uint32),
        ("nranks", ctypes.c_uint32),
        ("t_make_axis_s", ctypes.c_double),
        ("t_count_s", ctypes.c_double),
        ("t_partition_s", ctypes.c_double),
        ("t_total_s", ctypes.c_double),
        ("elements_per_level", ctypes.c_uint64 * MAX_LEVELS),
    ]


def build() -> str:
    """Compile the oracle with its Makefile (idempotent)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        fp = ctypes.POINTER(ctypes.c_float)
        u32p = ctypes.POINTER(ctypes.c_uint32)
        L.oracle_draw.restype = ctypes.c_uint64
        L.oracle_draw.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        for name in ("oracle_gen_uniform", "oracle_gen_plummer"):
            f = getattr(L, name)
            f.restype = None
            f.argtypes = [ctypes.c_uint64, ctypes.c_uint64, fp, fp, fp, ctypes.c_int]
        L.oracle_gen_xorshf96.restype = None
        L.oracle_gen_xorshf96.argtypes = [ctypes.c_uint64, fp, fp, fp]
        L.oracle_plummer_clusters.restype = None
        L.oracle_plummer_clusters.argtypes = [ctypes.c_uint64, fp, ctypes.POINTER(ctypes.c_double)]
        L.oracle_get_cut.restype = ctypes.c_float
        L.oracle_get_cut.argtypes = [ctypes.c_float, ctypes.c_float]
        L.oracle_convergence.restype = ctypes.c_int
        L.oracle_convergence.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int32,
                                         ctypes.POINTER(ctypes.c_int32)]
        L.oracle_count_left.restype = ctypes.c_uint32
        L.oracle_count_left.argtypes = [fp, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_float]
        L.oracle_hoare.restype = ctypes.c_int64
        L.oracle_hoare.argtypes = [fp, fp, fp, u32p, ctypes.c_uint64, ctypes.c_uint64,
                                   ctypes.c_int, ctypes.c_float, ctypes.c_int,
                                   ctypes.POINTER(ctypes.c_int)]
        L.oracle_build.restype = ctypes.c_int
        L.oracle_build.argtypes = [fp, fp, fp, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32,
                                   fp, fp, ctypes.c_void_p, u32p, u32p,
                                   ctypes.POINTER(ctypes.c_uint8), ctypes.c_int, ctypes.c_int,
                                   ctypes.c_int, ctypes.POINTER(_Stats)]
        L.oracle_convergence_weighted.restype = ctypes.c_int
        L.oracle_convergence_weighted.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                                                  ctypes.c_int32]
        L.oracle_build_weighted.restype = ctypes.c_int
        L.oracle_build_weighted.argtypes = [fp, fp, fp, u32p, ctypes.c_uint64, ctypes.c_uint32,
                                            ctypes.c_uint32, fp, fp, ctypes.c_void_p, u32p, u32p,
                                            ctypes.POINTER(ctypes.c_uint8), ctypes.c_int,
                                            ctypes.POINTER(_Stats)]
        L.oracle_level_shape.restype = None
        L.oracle_level_shape.argtypes = [ctypes.c_uint32, u32p, u32p]
        L.oracle_max_levels.restype = ctypes.c_uint32
        L.oracle_max_levels.argtypes = [ctypes.c_uint32]
        _lib = L
    return _lib


def _f(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _u32(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))


def draw(seed: int, counter: int) -> int:
    return int(lib().oracle_draw(seed, counter))


def gen_uniform(seed: int, n: int, nthreads: int = 8):
    x, y, z = (np.empty(n, np.float32) for _ in range(3))
    lib().oracle_gen_uniform(seed, n, _f(x), _f(y), _f(z), nthreads)
    return x, y, z


def gen_plummer(seed: int, n: int, nthreads: int = 8):
    x, y, z = (np.empty(n, np.float32) for _ in range(3))
    lib().oracle_gen_plummer(seed, n, _f(x), _f(y), _f(z), nthreads)
    return x, y, z


def gen_xorshf96(n: int):
    """The reference's own input stream (src/services/init.cu:11-25), n particles."""
    x, y, z = (np.empty(n, np.float32) for _ in range(3))
    lib().oracle_gen_xorshf96(n, _f(x), _f(y), _f(z))
    return x, y, z


def plummer_clusters(seed: int):
    c = np.empty(64 * 3, np.float32)
    s = np.empty(64, np.float64)
    lib().oracle_plummer_clusters(seed, _f(c), s.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return c.reshape(64, 3), s


def get_cut(left: float, right: float) -> float:
    return float(lib().oracle_get_cut(left, right))


def convergence(count_left: int, count: int, n_leaf: int):
    d = ctypes.c_int32()
    r = lib().oracle_convergence(count_left, count, n_leaf, ctypes.byref(d))
    return int(r), int(d.value)


def count_left(keys: np.ndarray, cut: float, begin: int = 0, end: int | None = None) -> int:
    keys = np.ascontiguousarray(keys, np.float32)
    end = keys.size if end is None else end
    return int(lib().oracle_count_left(_f(keys), begin, end, cut))


def hoare(x, y, z, axis: int, cut: float, begin: int = 0, end: int | None = None,
          final_swap: bool = True, perm=None):
    """In-place Hoare partition of [begin, end); returns (split index, degenerate flag)."""
    end = x.size if end is None else end
    dg = ctypes.c_int()
    i = lib().oracle_hoare(_f(x), _f(y), _f(z), _u32(perm), begin, end, axis, cut,
                           1 if final_swap else 0, ctypes.byref(dg))
    return int(i), int(dg.value)


@dataclass
class OracleResult:
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    heap: np.ndarray       # CELL_DTYPE[2d-1]
    ranges: np.ndarray     # uint32[nranks, 2d-1, 2]
    perm: np.ndarray       # uint32[n]: original index of the particle at each position
    iters: np.ndarray      # uint8[2d-1]
    stats: dict


def level_shape(d: int):
    """(getNLevels(), getNCellsOnLastLevel()) of a root of d leaves (src/cell.h:65-72)."""
    a, b = ctypes.c_uint32(), ctypes.c_uint32()
    lib().oracle_level_shape(d, ctypes.byref(a), ctypes.byref(b))
    return int(a.value), int(b.value)


def max_levels(d: int) -> int:
    """Most split levels of a build of d leaves: log2(d) for a power of two, else the
    reference's own bound getNLevels() - 1."""
    return int(lib().oracle_max_levels(d))


def build_tree(x, y, z, d: int, levels: int | None = None, lower=(-0.5, -0.5, -0.5),
               upper=(0.5, 0.5, 0.5), nranks: int = 1, make_axis: bool = False,
               copy: bool = True, want_perm: bool = True, threads: int = 1) -> OracleResult:
    """Run the oracle ORB build. Inputs are copied unless copy=False (then permuted in place).
    levels=None runs max_levels(d). threads > 1 (single rank only) bisects and partitions the
    cells of a level in parallel, with the same results."""
    if copy:
        x, y, z = (np.array(a, dtype=np.float32, copy=True) for a in (x, y, z))
    n = x.size
    levels = max_levels(d) if levels is None else levels
    heap = np.zeros(2 * d - 1, CELL_DTYPE)
    ranges = np.zeros((nranks, 2 * d - 1, 2), np.uint32)
    perm = np.empty(n, np.uint32) if want_perm else None
    iters = np.zeros(2 * d - 1, np.uint8)
    lo = np.asarray(lower, np.float32)
    hi = np.asarray(upper, np.float32)
    st = _Stats()
    rc = lib().oracle_build(_f(x), _f(y), _f(z), n, d, levels, _f(lo), _f(hi),
                            heap.ctypes.data_as(ctypes.c_void_p), _u32(ranges), _u32(perm),
                            iters.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), nranks,
                            1 if make_axis else 0, threads, ctypes.byref(st))
    if rc != 0:
        raise ValueError(f"oracle_build rejected the arguments (code {rc})")
    stats = {
        "levels_built": st.levels_built,
        "iterations": list(st.iterations[: st.levels_built]),
        "cell_counts": st.cell_counts,
        "elements_counted": st.elements_counted,
        "elements_per_level": list(st.elements_per_level[: st.levels_built]),
        "degenerate_cells": st.degenerate_cells,
        "zero_volume_cells": st.zero_volume_cells,
        "unfound_cells": st.unfound_cells,
        "nranks": st.nranks,
        "t_make_axis_s": st.t_make_axis_s,
        "t_count_s": st.t_count_s,
        "t_partition_s": st.t_partition_s,
        "t_total_s": st.t_total_s,
    }
    return OracleResult(x, y, z, heap, ranges, perm, iters, stats)


def cut_of(heap: np.ndarray) -> np.ndarray:
    """getCut() of every heap cell, float32 exactly as src/cell.h:74-76 computes it."""
    s = (heap["cutMarginRight"] + heap["cutMarginLeft"]).astype(np.float32)
    return (s.astype(np.float64) / 2.0).astype(np.float32)


def convergence_weighted(w_left: int, w_cell: int, n: int, n_leaf: int) -> int:
    """The weighted test: 0 found, +1 right margin moves, -1 left (see orb_oracle.h)."""
    return int(lib().oracle_convergence_weighted(w_left, w_cell, n, n_leaf))


def build_tree_weighted(x, y, z, w, d: int, levels: int | None = None, lower=(-0.5, -0.5, -0.5),
                        upper=(0.5, 0.5, 0.5), threads: int = 1):
    """Weighted ORB build (uint32 weights, permuted with the particles). Returns
    (OracleResult, permuted weights)."""
    x, y, z = (np.array(a, dtype=np.float32, copy=True) for a in (x, y, z))
    w = np.array(w, dtype=np.uint32, copy=True)
    n = x.size
    levels = max_levels(d) if levels is None else levels
    heap = np.zeros(2 * d - 1, CELL_DTYPE)
    ranges = np.zeros((1, 2 * d - 1, 2), np.uint32)
    perm = np.empty(n, np.uint32)
    iters = np.zeros(2 * d - 1, np.uint8)
    lo = np.asarray(lower, np.float32)
    hi = np.asarray(upper, np.float32)
    st = _Stats()
    rc = lib().oracle_build_weighted(_f(x), _f(y), _f(z), _u32(w), n, d, levels, _f(lo), _f(hi),
                                     heap.ctypes.data_as(ctypes.c_void_p), _u32(ranges), _u32(perm),
                                     iters.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), threads,
                                     ctypes.byref(st))
    if rc != 0:
        raise ValueError(f"oracle_build_weighted rejected the arguments (code {rc})")
    stats = {"levels_built": st.levels_built, "iterations": list(st.iterations[: st.levels_built]),
             "degenerate_cells": st.degenerate_cells, "zero_volume_cells": st.zero_volume_cells,
             "unfound_cells": st.unfound_cells}
    return OracleResult(x, y, z, heap, ranges, perm, iters, stats), w
