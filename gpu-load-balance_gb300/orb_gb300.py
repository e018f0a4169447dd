"""Python front end of the GB300 ORB engine: builds liborb_gb300.so and binds its C ABI.

The engine itself is C++/CUDA behind the C ABI declared in include/orb/orb.h; this module
only compiles it (nvcc, sm_103a) and calls it through ctypes. There is no Python or CPU
compute path: every call fails with OrbError if the library cannot be loaded.
"""
from __future__ import annotations

import concurrent.futures as cf
import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_PATH = os.path.join(PKG_DIR, "liborb_gb300.so")
SOURCES = ["orb_kernels.cu", "orb_api.cu", "orb_static.cu", "orb_server.cu"]
HEADERS = ["orb_internal.cuh", "orb_leaf_ratio.h"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE,
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills",
              *os.environ.get("ORB_NVCC_FLAGS", "").split()]  # extra flags (build-time knobs)

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

ORB_DEVICE_POINTERS = 0x1
ORB_GEN_UNIFORM = 0
ORB_GEN_PLUMMER = 1
ORB_GEN_XORSHF96 = 2

STATUS = {
    0: "ok",
    1: "invalid argument",
    2: "CUDA error",
    3: "out of memory",
    4: "capacity exceeded",
    5: "no particles loaded",
    6: "timeout",
}

# Every symbol include/orb/orb.h declares (checked by the CPU tests).
EXPORTS = [
    "orb_abi_version", "orb_status_string", "orb_last_error", "orb_ctx_create",
    "orb_ctx_destroy", "orb_build", "orb_load_particles", "orb_store_particles", "orb_count",
    "orb_count_left", "orb_partition", "orb_get_ranges", "orb_set_ranges", "orb_generate",
    "orb_profile_reset", "orb_profile_read", "orb_count_left_static", "orb_build_batch",
    "orb_profile_kernel_index", "orb_server_create", "orb_server_destroy", "orb_server_submit_build",
    "orb_server_submit_generate", "orb_server_submit_rebalance", "orb_server_wait", "orb_server_poll",
    "orb_server_fetch", "orb_server_release", "orb_server_get_stats", "orb_get_tuning",
    "orb_set_tuning", "orb_autotune_batch", "orb_build_batch_warm", "orb_build_warm",
    "orb_server_submit_rebalance_warm", "orb_test_set_scan_wait", "orb_build_weighted",
]

ORB_STATIC_MAX_CELLS = 65536


class OrbError(RuntimeError):
    def __init__(self, status: int, msg: str = ""):
        self.status = status
        super().__init__(f"{STATUS.get(status, status)}: {msg}" if msg else STATUS.get(status, str(status)))


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS] + [os.path.join(INCLUDE, "orb", "orb.h")]
    return any(os.path.getmtime(p) > t for p in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile the CUDA sources for sm_103a (in parallel) and link liborb_gb300.so."""
    if not force and not _stale():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    objs = []

    def compile_one(src):
        obj = os.path.join(BUILD_DIR, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class Tuning(ctypes.Structure):
    """orb_tuning: launch parameters that never change a result."""
    _fields_ = [
        ("hist_blocks_per_sm", ctypes.c_uint32),
        ("part_blocks_per_sm", ctypes.c_uint32),
        ("tile_blocks_per_sm", ctypes.c_uint32),
        ("sparse_keys_per_tile", ctypes.c_uint32),
        ("cta_min_cells", ctypes.c_uint32),
        ("subtree_levels", ctypes.c_uint32),
        ("predict_sigmas", ctypes.c_uint32),
    ]

    def as_dict(self):
        return {f: int(getattr(self, f)) for f, _ in self._fields_}


class BuildInfo(ctypes.Structure):
    _fields_ = [
        ("levels_built", ctypes.c_uint32),
        ("degenerate_cells", ctypes.c_uint32),
        ("zero_volume_cells", ctypes.c_uint32),
        ("unfound_cells", ctypes.c_uint32),
        ("max_iterations", ctypes.c_uint32),
        ("count_passes", ctypes.c_uint32),
        ("device_ms", ctypes.c_float),
        ("h2d_ms", ctypes.c_float),
        ("d2h_ms", ctypes.c_float),
        ("warm_cells", ctypes.c_uint32),
        ("warm_resets", ctypes.c_uint32),
        ("sampled_cells", ctypes.c_uint32),
        ("sampled_misses", ctypes.c_uint32),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class BatchInstance(ctypes.Structure):
    _fields_ = [("offset", ctypes.c_uint64), ("n", ctypes.c_uint64), ("d", ctypes.c_uint32),
                ("levels", ctypes.c_uint32), ("lower", ctypes.c_float * 3),
                ("upper", ctypes.c_float * 3)]


class ServerOpts(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_uint64), ("max_batch", ctypes.c_uint32),
                ("lanes", ctypes.c_uint32)]


class RequestResult(ctypes.Structure):
    _fields_ = [("request_id", ctypes.c_uint64), ("instance_id", ctypes.c_uint64),
                ("status", ctypes.c_int32), ("kind", ctypes.c_int32), ("batch_size", ctypes.c_uint32),
                ("pad_", ctypes.c_uint32), ("submit_s", ctypes.c_double), ("start_s", ctypes.c_double),
                ("done_s", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "pad_"}


class ServerStats(ctypes.Structure):
    _fields_ = [(f, ctypes.c_uint64) for f in ("requests_submitted", "requests_done", "builds",
                                               "rebalances", "batches", "particles_built",
                                               "arena_particles", "arena_used")] + \
               [("max_batch_seen", ctypes.c_uint32), ("pending", ctypes.c_uint32)]


class KernelStat(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 32), ("launches", ctypes.c_uint64),
                ("total_ms", ctypes.c_double), ("bytes", ctypes.c_double)]


class Opts(ctypes.Structure):
    _fields_ = [("reserve_particles", ctypes.c_uint64), ("reserve_leaves", ctypes.c_uint32),
                ("flags", ctypes.c_uint32)]


_lib = None


def load(path: str | None = None):
    """Load the engine library (it must already be built; see build()). ORB_LIB may name
    another build of it (kernel-parameter experiments)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or os.environ.get("ORB_LIB") or LIB_PATH
    if not os.path.exists(path):
        raise OrbError(2, f"engine library not built: {path} (run __graft_entry__.build())")
    L = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    u32 = ctypes.c_uint32
    u64 = ctypes.c_uint64
    L.orb_abi_version.restype = ctypes.c_int
    L.orb_status_string.restype = ctypes.c_char_p
    L.orb_status_string.argtypes = [ctypes.c_int]
    L.orb_last_error.restype = ctypes.c_char_p
    L.orb_last_error.argtypes = [vp]
    L.orb_ctx_create.restype = ctypes.c_int
    L.orb_ctx_create.argtypes = [ctypes.c_int, ctypes.POINTER(Opts), ctypes.POINTER(vp)]
    L.orb_ctx_destroy.restype = ctypes.c_int
    L.orb_ctx_destroy.argtypes = [vp]
    L.orb_build.restype = ctypes.c_int
    L.orb_build.argtypes = [vp, vp, vp, vp, u64, u32, u32, vp, vp, vp, vp, vp, u32,
                            ctypes.POINTER(BuildInfo)]
    L.orb_build_weighted.restype = ctypes.c_int
    L.orb_build_weighted.argtypes = [vp, vp, vp, vp, vp, u64, u32, u32, vp, vp, vp, vp, vp, u32,
                                     ctypes.POINTER(BuildInfo)]
    L.orb_load_particles.restype = ctypes.c_int
    L.orb_load_particles.argtypes = [vp, vp, vp, vp, u64, u32, u32]
    L.orb_store_particles.restype = ctypes.c_int
    L.orb_store_particles.argtypes = [vp, vp, vp, vp, vp, u32]
    for name in ("orb_count", "orb_count_left"):
        f = getattr(L, name)
        f.restype = ctypes.c_int
        f.argtypes = [vp, vp, u32, vp]
    L.orb_partition.restype = ctypes.c_int
    L.orb_partition.argtypes = [vp, vp, u32]
    for name in ("orb_get_ranges", "orb_set_ranges"):
        f = getattr(L, name)
        f.restype = ctypes.c_int
        f.argtypes = [vp, vp, u32]
    L.orb_generate.restype = ctypes.c_int
    L.orb_generate.argtypes = [vp, ctypes.c_int, u64, u64, vp, vp, vp, u32]
    L.orb_profile_reset.restype = ctypes.c_int
    L.orb_profile_reset.argtypes = [vp, u32]
    L.orb_profile_kernel_index.restype = ctypes.c_int
    L.orb_profile_kernel_index.argtypes = [ctypes.c_char_p]
    L.orb_profile_read.restype = ctypes.c_int
    L.orb_profile_read.argtypes = [vp, ctypes.POINTER(KernelStat), ctypes.c_int]
    L.orb_get_tuning.restype = ctypes.c_int
    L.orb_get_tuning.argtypes = [vp, ctypes.POINTER(Tuning)]
    L.orb_set_tuning.restype = ctypes.c_int
    L.orb_set_tuning.argtypes = [vp, ctypes.POINTER(Tuning)]
    L.orb_autotune_batch.restype = ctypes.c_int
    L.orb_autotune_batch.argtypes = [vp, vp, vp, vp, u64, ctypes.POINTER(BatchInstance), u32, u32, u32,
                                     ctypes.POINTER(Tuning), ctypes.POINTER(ctypes.c_float)]
    L.orb_build_batch.restype = ctypes.c_int
    L.orb_build_batch.argtypes = [vp, vp, vp, vp, u64, ctypes.POINTER(BatchInstance), u32, vp, vp,
                                  vp, u32, ctypes.POINTER(BuildInfo)]
    L.orb_server_create.restype = ctypes.c_int
    L.orb_server_create.argtypes = [ctypes.c_int, ctypes.POINTER(ServerOpts), ctypes.POINTER(vp)]
    L.orb_server_destroy.restype = ctypes.c_int
    L.orb_server_destroy.argtypes = [vp]
    L.orb_server_submit_build.restype = ctypes.c_int
    L.orb_server_submit_build.argtypes = [vp, vp, vp, vp, u64, u32, u32, vp, vp, ctypes.POINTER(u64)]
    L.orb_server_submit_generate.restype = ctypes.c_int
    L.orb_server_submit_generate.argtypes = [vp, ctypes.c_int, u64, u64, u32, u32, ctypes.POINTER(u64)]
    L.orb_server_submit_rebalance_warm.restype = ctypes.c_int
    L.orb_server_submit_rebalance_warm.argtypes = [vp, u64, u64, ctypes.c_float, ctypes.c_float,
                                                   ctypes.POINTER(u64)]
    L.orb_build_warm.restype = ctypes.c_int
    L.orb_build_warm.argtypes = [vp, vp, vp, vp, u64, u32, u32, vp, vp, vp, ctypes.c_float, vp, vp, vp,
                                 u32, ctypes.POINTER(BuildInfo)]
    L.orb_build_batch_warm.restype = ctypes.c_int
    L.orb_build_batch_warm.argtypes = [vp, vp, vp, vp, u64, ctypes.POINTER(BatchInstance), u32, vp, vp,
                                       vp, vp, vp, u32, ctypes.POINTER(BuildInfo)]
    L.orb_server_submit_rebalance.restype = ctypes.c_int
    L.orb_server_submit_rebalance.argtypes = [vp, u64, u64, ctypes.c_float, ctypes.POINTER(u64)]
    L.orb_server_wait.restype = ctypes.c_int
    L.orb_server_wait.argtypes = [vp, u64, ctypes.POINTER(RequestResult)]
    L.orb_server_poll.restype = ctypes.c_int
    L.orb_server_poll.argtypes = [vp, ctypes.POINTER(RequestResult), u32, ctypes.POINTER(u32)]
    L.orb_server_fetch.restype = ctypes.c_int
    L.orb_server_fetch.argtypes = [vp, u64, vp, vp, vp, vp, vp, vp]
    L.orb_server_release.restype = ctypes.c_int
    L.orb_server_release.argtypes = [vp, u64]
    L.orb_server_get_stats.restype = ctypes.c_int
    L.orb_server_get_stats.argtypes = [vp, ctypes.POINTER(ServerStats)]
    L.orb_test_set_scan_wait.restype = ctypes.c_int
    L.orb_test_set_scan_wait.argtypes = [vp, u32, u32]
    L.orb_count_left_static.restype = ctypes.c_int
    L.orb_count_left_static.argtypes = [vp, vp, vp, u64, vp, u32, vp, u32, vp, vp]
    _lib = L
    return L


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if hasattr(a, "data_ptr"):  # torch tensor
        return a.data_ptr()
    return int(a)


def count_left_static(x, y, z, n: int, cells, n_cells: int, ranges, n_ranges: int, out,
                      stream=None):
    """orb_count_left_static: every argument is device memory (tensors or pointers); the
    call enqueues on `stream` (a raw cudaStream_t value, None = default stream)."""
    lib = load()
    st = lib.orb_count_left_static(_ptr(x), _ptr(y), _ptr(z), n, _ptr(cells), n_cells,
                                   _ptr(ranges), n_ranges, _ptr(out), stream)
    if st != 0:
        raise OrbError(st, "orb_count_left_static")


@dataclass
class BuildResult:
    heap: np.ndarray      # CELL_DTYPE[2d-1]
    ranges: np.ndarray    # uint32[2d-1, 2]
    perm: object          # uint32[n] (numpy) or the device tensor passed in
    info: dict


class Context:
    """One engine context on one CUDA device (owns a stream and device buffers)."""

    def __init__(self, device: int = 0, reserve_particles: int = 0, reserve_leaves: int = 0):
        self.lib = load()
        self.h = ctypes.c_void_p()
        o = Opts(reserve_particles, reserve_leaves, 0)
        self._check(self.lib.orb_ctx_create(device, ctypes.byref(o), ctypes.byref(self.h)))

    def _check(self, st):
        if st != 0:
            msg = self.lib.orb_last_error(self.h).decode() if self.h else ""
            raise OrbError(st, msg)

    def close(self):
        if self.h:
            self.lib.orb_ctx_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def build(self, x, y, z, d: int, levels: int = 0, lower=(-0.5, -0.5, -0.5),
              upper=(0.5, 0.5, 0.5), perm=True, device_pointers: bool = False,
              heap_out=None, ranges_out=None) -> BuildResult:
        """ORB build. Host numpy arrays are partitioned in place; with device_pointers the
        arguments are device tensors/pointers partitioned in place on the device. heap_out /
        ranges_out may supply (for instance pinned) host arrays for the results."""
        n = int(x.shape[0]) if hasattr(x, "shape") else int(x.size)
        heap = np.zeros(2 * d - 1, CELL_DTYPE) if heap_out is None else heap_out
        ranges = np.zeros((2 * d - 1, 2), np.uint32) if ranges_out is None else ranges_out
        if perm is True:
            perm = np.empty(n, np.uint32)
        lo = np.asarray(lower, np.float32)
        hi = np.asarray(upper, np.float32)
        info = BuildInfo()
        st = self.lib.orb_build(self.h, _ptr(x), _ptr(y), _ptr(z), n, d, levels, lo.ctypes.data,
                                hi.ctypes.data, heap.ctypes.data, ranges.ctypes.data, _ptr(perm),
                                ORB_DEVICE_POINTERS if device_pointers else 0, ctypes.byref(info))
        self._check(st)
        return BuildResult(heap, ranges, perm, info.as_dict())

    def build_weighted(self, x, y, z, w, d: int, levels: int = 0, lower=(-0.5, -0.5, -0.5),
                       upper=(0.5, 0.5, 0.5), perm=True, device_pointers: bool = False) -> BuildResult:
        """Weighted ORB build (orb_build_weighted): uint32 weights w, reordered in place with
        the particles."""
        n = int(x.shape[0]) if hasattr(x, "shape") else int(x.size)
        heap = np.zeros(2 * d - 1, CELL_DTYPE)
        ranges = np.zeros((2 * d - 1, 2), np.uint32)
        if perm is True:
            perm = np.empty(n, np.uint32)
        lo = np.asarray(lower, np.float32)
        hi = np.asarray(upper, np.float32)
        info = BuildInfo()
        st = self.lib.orb_build_weighted(self.h, _ptr(x), _ptr(y), _ptr(z), _ptr(w), n, d, levels,
                                         lo.ctypes.data, hi.ctypes.data, heap.ctypes.data,
                                         ranges.ctypes.data, _ptr(perm),
                                         ORB_DEVICE_POINTERS if device_pointers else 0, ctypes.byref(info))
        self._check(st)
        return BuildResult(heap, ranges, perm, info.as_dict())

    def build_warm(self, x, y, z, d: int, prev_heap, width: float, levels: int = 0,
                   lower=(-0.5, -0.5, -0.5), upper=(0.5, 0.5, 0.5), perm=True,
                   device_pointers: bool = False) -> BuildResult:
        """Warm-started build from a previous tree (orb_build_warm): a valid ORB tree, not
        bit-identical with build() on the same particles."""
        n = int(x.shape[0]) if hasattr(x, "shape") else int(x.size)
        heap = np.zeros(2 * d - 1, CELL_DTYPE)
        ranges = np.zeros((2 * d - 1, 2), np.uint32)
        prev = np.ascontiguousarray(prev_heap, dtype=CELL_DTYPE)
        if perm is True:
            perm = np.empty(n, np.uint32)
        lo = np.asarray(lower, np.float32)
        hi = np.asarray(upper, np.float32)
        info = BuildInfo()
        st = self.lib.orb_build_warm(self.h, _ptr(x), _ptr(y), _ptr(z), n, d, levels, lo.ctypes.data,
                                     hi.ctypes.data, prev.ctypes.data, width, heap.ctypes.data,
                                     ranges.ctypes.data, _ptr(perm),
                                     ORB_DEVICE_POINTERS if device_pointers else 0, ctypes.byref(info))
        self._check(st)
        return BuildResult(heap, ranges, perm, info.as_dict())

    def build_batch_warm(self, x, y, z, instances, prev_heaps, widths, perm=True,
                         device_pointers: bool = False):
        """Warm-started batched build (orb_build_batch_warm); prev_heaps laid out like the
        heaps build_batch returns back to back, widths one per instance (0 = cold)."""
        k = len(instances)
        arr, heap_cells, bases = self._instances(instances)
        n_total = int(x.shape[0]) if hasattr(x, "shape") else int(x.size)
        heaps = np.zeros(max(heap_cells, 1), CELL_DTYPE)
        ranges = np.zeros((max(heap_cells, 1), 2), np.uint32)
        prev = np.ascontiguousarray(prev_heaps, dtype=CELL_DTYPE)
        w = np.ascontiguousarray(widths, dtype=np.float32)
        if perm is True:
            perm = np.empty(n_total, np.uint32)
        info = BuildInfo()
        st = self.lib.orb_build_batch_warm(self.h, _ptr(x), _ptr(y), _ptr(z), n_total, arr, k,
                                           prev.ctypes.data, w.ctypes.data, heaps.ctypes.data,
                                           ranges.ctypes.data, _ptr(perm),
                                           ORB_DEVICE_POINTERS if device_pointers else 0,
                                           ctypes.byref(info))
        self._check(st)
        parts = []
        for i, ins in enumerate(instances):
            hc = 2 * int(ins["d"]) - 1
            parts.append((heaps[bases[i]:bases[i] + hc], ranges[bases[i]:bases[i] + hc]))
        return parts, heaps, perm, info.as_dict()

    @staticmethod
    def _instances(instances):
        k = len(instances)
        arr = (BatchInstance * max(k, 1))()
        heap_cells = 0
        bases = []
        for i, ins in enumerate(instances):
            b = arr[i]
            b.offset = int(ins["offset"])
            b.n = int(ins["n"])
            b.d = int(ins["d"])
            b.levels = int(ins.get("levels", 0))
            for a in range(3):
                b.lower[a] = ins.get("lower", (-0.5, -0.5, -0.5))[a]
                b.upper[a] = ins.get("upper", (0.5, 0.5, 0.5))[a]
            bases.append(heap_cells)
            heap_cells += 2 * b.d - 1
        return arr, heap_cells, bases

    def test_set_scan_wait(self, spin_limit: int = 0, ticket_start: int = 0):
        """Test hook of the tile scan's bounded look-back wait (orb_test_set_scan_wait)."""
        self._check(self.lib.orb_test_set_scan_wait(self.h, spin_limit, ticket_start))

    # launch tuning -----------------------------------------------------------------
    def get_tuning(self) -> dict:
        t = Tuning()
        self._check(self.lib.orb_get_tuning(self.h, ctypes.byref(t)))
        return t.as_dict()

    def set_tuning(self, **params):
        """Change some tuning parameters (the rest keep their current values)."""
        t = Tuning()
        self._check(self.lib.orb_get_tuning(self.h, ctypes.byref(t)))
        for k, v in params.items():
            setattr(t, k, int(v))
        self._check(self.lib.orb_set_tuning(self.h, ctypes.byref(t)))

    def autotune_batch(self, x, y, z, instances, reps: int = 3, device_pointers: bool = False):
        """Autotune the launch parameters on a batch (inputs are not modified). Returns
        (chosen tuning dict, its median build ms)."""
        arr, _, _ = self._instances(instances)
        n_total = int(x.shape[0]) if hasattr(x, "shape") else int(x.size)
        best = Tuning()
        ms = ctypes.c_float()
        self._check(self.lib.orb_autotune_batch(self.h, _ptr(x), _ptr(y), _ptr(z), n_total, arr,
                                                len(instances),
                                                ORB_DEVICE_POINTERS if device_pointers else 0,
                                                reps, ctypes.byref(best), ctypes.byref(ms)))
        return best.as_dict(), float(ms.value)

    def build_batch(self, x, y, z, instances, perm=True, device_pointers: bool = False):
        """Batched build. `instances`: list of dicts {offset, n, d, levels=0, lower, upper}.
        Returns (list of per-instance (heap, ranges) views, perm, info)."""
        k = len(instances)
        arr, heap_cells, bases = self._instances(instances)
        n_total = int(x.shape[0]) if hasattr(x, "shape") else int(x.size)
        heaps = np.zeros(max(heap_cells, 1), CELL_DTYPE)
        ranges = np.zeros((max(heap_cells, 1), 2), np.uint32)
        if perm is True:
            perm = np.empty(n_total, np.uint32)
        info = BuildInfo()
        st = self.lib.orb_build_batch(self.h, _ptr(x), _ptr(y), _ptr(z), n_total, arr, k,
                                      heaps.ctypes.data, ranges.ctypes.data, _ptr(perm),
                                      ORB_DEVICE_POINTERS if device_pointers else 0,
                                      ctypes.byref(info))
        self._check(st)
        parts = []
        for i, ins in enumerate(instances):
            hc = 2 * int(ins["d"]) - 1
            parts.append((heaps[bases[i]:bases[i] + hc], ranges[bases[i]:bases[i] + hc]))
        return parts, perm, info.as_dict()

    def generate(self, kind: int, seed: int, n: int, x, y, z, device_pointers: bool = False):
        self._check(self.lib.orb_generate(self.h, kind, seed, n, _ptr(x), _ptr(y), _ptr(z),
                                          ORB_DEVICE_POINTERS if device_pointers else 0))

    def generate_host(self, kind: int, seed: int, n: int):
        x, y, z = (np.empty(n, np.float32) for _ in range(3))
        self.generate(kind, seed, n, x, y, z)
        return x, y, z

    # profiling -----------------------------------------------------------------------
    def profile_reset(self, timing=False):
        """timing: False (counts only), True (time every kernel) or a list of kernel names."""
        if timing is True:
            mask = 0xFFFFFFFF
        elif not timing:
            mask = 0
        else:
            mask = 0
            for name in timing:
                k = self.lib.orb_profile_kernel_index(name.encode())
                if k < 0:
                    raise OrbError(1, f"unknown kernel {name}")
                mask |= 1 << k
        self._check(self.lib.orb_profile_reset(self.h, mask))

    def profile(self) -> dict:
        """{kernel name: {launches, total_ms, bytes}} since the last profile_reset."""
        n = self.lib.orb_profile_read(self.h, None, 0)
        arr = (KernelStat * max(n, 1))()
        n = self.lib.orb_profile_read(self.h, arr, n)
        return {arr[i].name.decode(): {"launches": int(arr[i].launches),
                                       "total_ms": float(arr[i].total_ms),
                                       "bytes": float(arr[i].bytes)} for i in range(n)}

    # service layer -------------------------------------------------------------------
    def load_particles(self, x, y, z, max_cells: int, device_pointers: bool = False):
        n = int(x.shape[0])
        self._check(self.lib.orb_load_particles(self.h, _ptr(x), _ptr(y), _ptr(z), n, max_cells,
                                                ORB_DEVICE_POINTERS if device_pointers else 0))
        self.loaded_n = n

    def store_particles(self):
        n = self.loaded_n
        x, y, z = (np.empty(n, np.float32) for _ in range(3))
        perm = np.empty(n, np.uint32)
        self._check(self.lib.orb_store_particles(self.h, x.ctypes.data, y.ctypes.data,
                                                 z.ctypes.data, perm.ctypes.data, 0))
        return x, y, z, perm

    def count(self, cells: np.ndarray) -> np.ndarray:
        out = np.zeros(len(cells), np.uint32)
        self._check(self.lib.orb_count(self.h, cells.ctypes.data, len(cells), out.ctypes.data))
        return out

    def count_left(self, cells: np.ndarray, out: np.ndarray | None = None) -> np.ndarray:
        out = np.zeros(len(cells), np.uint32) if out is None else out
        self._check(self.lib.orb_count_left(self.h, cells.ctypes.data, len(cells), out.ctypes.data))
        return out

    def partition(self, cells: np.ndarray):
        self._check(self.lib.orb_partition(self.h, cells.ctypes.data, len(cells)))

    def get_ranges(self, n_cells: int) -> np.ndarray:
        r = np.zeros((n_cells, 2), np.uint32)
        self._check(self.lib.orb_get_ranges(self.h, r.ctypes.data, n_cells))
        return r

    def set_ranges(self, ranges: np.ndarray):
        r = np.ascontiguousarray(ranges, np.uint32)
        self._check(self.lib.orb_set_ranges(self.h, r.ctypes.data, r.shape[0]))


class Server:
    """Continuous-batching ORB request server (orb_server_* of the C ABI)."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 4 << 30, max_batch: int = 0,
                 lanes: int = 2):
        self.lib = load()
        self.h = ctypes.c_void_p()
        o = ServerOpts(hbm_budget_bytes, max_batch, lanes)
        st = self.lib.orb_server_create(device, ctypes.byref(o), ctypes.byref(self.h))
        if st != 0:
            raise OrbError(st, "orb_server_create")
        self.d = {}

    def close(self):
        if self.h:
            self.lib.orb_server_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _chk(self, st, what):
        if st != 0:
            raise OrbError(st, what)

    def submit_build(self, x, y, z, d: int, levels: int = 0, lower=(-0.5, -0.5, -0.5),
                     upper=(0.5, 0.5, 0.5)) -> int:
        x, y, z = (np.ascontiguousarray(a, np.float32) for a in (x, y, z))
        lo = np.asarray(lower, np.float32)
        hi = np.asarray(upper, np.float32)
        rid = ctypes.c_uint64()
        self._chk(self.lib.orb_server_submit_build(self.h, x.ctypes.data, y.ctypes.data, z.ctypes.data,
                                                   x.size, d, levels, lo.ctypes.data, hi.ctypes.data,
                                                   ctypes.byref(rid)), "submit_build")
        self.d[rid.value] = (d, x.size)
        return rid.value

    def submit_generate(self, kind: int, seed: int, n: int, d: int, levels: int = 0) -> int:
        rid = ctypes.c_uint64()
        self._chk(self.lib.orb_server_submit_generate(self.h, kind, seed, n, d, levels,
                                                      ctypes.byref(rid)), "submit_generate")
        self.d[rid.value] = (d, n)
        return rid.value

    def submit_rebalance(self, instance: int, seed: int, sigma: float, warm: float = 0.0) -> int:
        """Rebalance: displace and rebuild. warm > 0 selects the warm-started rebuild with
        that bracket factor (orb_build_batch_warm; not bit-identical with a cold one)."""
        rid = ctypes.c_uint64()
        if warm > 0:
            st = self.lib.orb_server_submit_rebalance_warm(self.h, instance, seed, sigma, warm,
                                                           ctypes.byref(rid))
        else:
            st = self.lib.orb_server_submit_rebalance(self.h, instance, seed, sigma, ctypes.byref(rid))
        self._chk(st, "submit_rebalance")
        return rid.value

    def wait(self, request: int) -> dict:
        r = RequestResult()
        st = self.lib.orb_server_wait(self.h, request, ctypes.byref(r))
        out = r.as_dict()
        out["status"] = st
        return out

    def fetch(self, instance: int):
        d, n = self.d[instance]
        heap = np.zeros(2 * d - 1, CELL_DTYPE)
        ranges = np.zeros((2 * d - 1, 2), np.uint32)
        x, y, z = (np.empty(n, np.float32) for _ in range(3))
        ident = np.empty(n, np.uint32)
        self._chk(self.lib.orb_server_fetch(self.h, instance, heap.ctypes.data, ranges.ctypes.data,
                                            x.ctypes.data, y.ctypes.data, z.ctypes.data,
                                            ident.ctypes.data), "fetch")
        return heap, ranges, x, y, z, ident

    def release(self, instance: int):
        self._chk(self.lib.orb_server_release(self.h, instance), "release")

    def stats(self) -> dict:
        s = ServerStats()
        self._chk(self.lib.orb_server_get_stats(self.h, ctypes.byref(s)), "stats")
        return {k: getattr(s, k) for k, _ in s._fields_}
