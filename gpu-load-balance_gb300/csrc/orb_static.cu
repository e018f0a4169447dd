// orb_count_left_static: count-left for callers that may not allocate device memory.
//
// Simulation codes that call the ORB services from inside their time-step loop often own
// the whole device through their own memory pool, reserved at start-up: a cudaMalloc there
// either fails or fragments the pool, and cudaMalloc/cudaFree synchronise the device, which
// stalls the caller's other streams. orb_count_left needs a context whose buffers are
// allocated on first use; this entry point needs no context and allocates nothing. Its
// scratch (per-cell tile offsets and per-cell counters) is the file-scope device array
// below, ORB_STATIC_MAX_CELLS cells large; every GPU that loads the library holds it
// (2 * 65536 + 2 words, 512 KiB) until the process exits.
#include <cuda_runtime.h>

#include <mutex>

#include "orb_internal.cuh"

namespace {

constexpr uint32_t kMaxCells = ORB_STATIC_MAX_CELLS;
constexpr uint32_t kTileKeys = 8192;
constexpr int kMaxDevices = 64;

// [0, C]: exclusive prefix of tiles per cell (entry C = total tiles);
// [C+1, 2C+1): per-cell counts of keys below the cut.
static __device__ __align__(256) uint32_t g_count_scratch[2 * kMaxCells + 2];

struct DeviceSetup {
    bool done;
    uint32_t *scratch;  // device address of g_count_scratch on that device
    int sms;
};
std::mutex g_setup_mu;
DeviceSetup g_setup[kMaxDevices];

// Once per device, with that device current: resolve the array's device address. Host
// code must not pass `g_count_scratch` itself to a kernel: on the host that name is a
// host-side stand-in, not a device address. The address is kept for the life of the
// process, so the entry point must not be called on a device after cudaDeviceReset there
// (the module, and with it the array, is loaded again at another address).
cudaError_t setup_device(int dev, DeviceSetup *out) {
    std::lock_guard<std::mutex> g(g_setup_mu);
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    DeviceSetup &s = g_setup[dev];
    if (!s.done) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_count_scratch);
        if (e != cudaSuccess) return e;
        int sms = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return e;
        s.scratch = static_cast<uint32_t *>(p);
        s.sms = sms;
        s.done = true;
    }
    *out = s;
    return cudaSuccess;
}

// Range of a cell, or an empty range when its id or range is outside the caller's map.
__device__ __forceinline__ uint2 cell_range(const orb_cell_t &c, const uint32_t *ranges,
                                            uint32_t n_ranges, uint64_t n) {
    if (c.id < 0 || (uint32_t)c.id >= n_ranges) return make_uint2(0u, 0u);
    const uint32_t b = ranges[2 * c.id], e = ranges[2 * c.id + 1];
    if (b > e || (uint64_t)e > n) return make_uint2(0u, 0u);
    return make_uint2(b, e);
}

// One CTA: tiles per cell (none for found cells), exclusive scan into scratch[0..C],
// counters scratch[C+1 ..] cleared (they keep the previous call's values otherwise).
__global__ void __launch_bounds__(1024) k_static_plan(const orb_cell_t *cells, uint32_t C,
                                                      const uint32_t *ranges, uint32_t n_ranges,
                                                      uint64_t n, uint32_t *scratch) {
    __shared__ uint32_t warp_tot[32];
    const uint32_t tid = threadIdx.x, per = (C + blockDim.x - 1) / blockDim.x;
    const uint32_t c0 = min(C, tid * per), c1 = min(C, c0 + per);
    uint32_t mine = 0;
    for (uint32_t c = c0; c < c1; ++c) {
        scratch[C + 1 + c] = 0u;
        if (cells[c].foundCut) continue;
        const uint2 r = cell_range(cells[c], ranges, n_ranges, n);
        mine += (r.y - r.x + kTileKeys - 1) / kTileKeys;
    }
    // block exclusive scan of `mine`
    const int lane = tid & 31, warp = tid >> 5;
    uint32_t inc = mine;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) warp_tot[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const uint32_t w = warp_tot[lane];
        uint32_t s = w;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += t;
        }
        warp_tot[lane] = s - w;
    }
    __syncthreads();
    uint32_t off = warp_tot[warp] + inc - mine;
    for (uint32_t c = c0; c < c1; ++c) {
        scratch[c] = off;
        if (cells[c].foundCut) continue;
        const uint2 r = cell_range(cells[c], ranges, n_ranges, n);
        off += (r.y - r.x + kTileKeys - 1) / kTileKeys;
    }
    if (tid == blockDim.x - 1) scratch[C] = off;
}

__global__ void __launch_bounds__(256) k_static_count(const float *x, const float *y, const float *z,
                                                      const orb_cell_t *cells, uint32_t C,
                                                      const uint32_t *ranges, uint32_t n_ranges,
                                                      uint64_t n, uint32_t *scratch) {
    __shared__ uint32_t red[8];
    const uint32_t total = scratch[C];
    for (uint32_t t = blockIdx.x; t < total; t += gridDim.x) {
        uint32_t lo = 0, hi = C;  // largest c with scratch[c] <= t
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (scratch[mid] <= t) lo = mid; else hi = mid - 1;
        }
        const orb_cell_t &cell = cells[lo];
        const uint2 r = cell_range(cell, ranges, n_ranges, n);
        const uint32_t e0 = r.x + (t - scratch[lo]) * kTileKeys;
        const uint32_t e1 = min(r.y, e0 + kTileKeys);
        const int axis = cell.cutAxis < 0 ? 0 : cell.cutAxis;
        const float *keys = axis == 0 ? x : (axis == 1 ? y : z);
        const float cut = orb::mid_cut(cell.cutMarginLeft, cell.cutMarginRight);  // getCut()
        uint32_t cnt = 0;
        for (uint32_t i = e0 + threadIdx.x; i < e1; i += blockDim.x) cnt += __ldg(keys + i) < cut;
        for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = cnt;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t s = 0;
            for (int w = 0; w < 8; ++w) s += red[w];
            if (s) atomicAdd(&scratch[C + 1 + lo], s);
        }
        __syncthreads();
    }
}

__global__ void k_static_store(const orb_cell_t *cells, uint32_t C, uint32_t *out,
                               const uint32_t *scratch) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < C && !cells[c].foundCut) out[c] = scratch[C + 1 + c];
}

}  // namespace

extern "C" orb_status orb_count_left_static(const float *x, const float *y, const float *z,
                                            uint64_t n, const orb_cell_t *cells,
                                            uint32_t n_cells, const uint32_t *ranges,
                                            uint32_t n_ranges, uint32_t *out, void *stream) {
    if (n_cells == 0) return ORB_OK;
    if (n_cells > kMaxCells) return ORB_ERR_CAPACITY;  // more cells than the static scratch holds
    if (!cells || !ranges || !out || (n > 0 && (!x || !y || !z))) return ORB_ERR_INVALID_ARGUMENT;
    if (n >= (1ull << 31)) return ORB_ERR_CAPACITY;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return ORB_ERR_CUDA;
    DeviceSetup s;
    if (setup_device(dev, &s) != cudaSuccess) return ORB_ERR_CUDA;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    k_static_plan<<<1, 1024, 0, st>>>(cells, n_cells, ranges, n_ranges, n, s.scratch);
    k_static_count<<<s.sms * 8, 256, 0, st>>>(x, y, z, cells, n_cells, ranges, n_ranges, n, s.scratch);
    k_static_store<<<(n_cells + 255) / 256, 256, 0, st>>>(cells, n_cells, out, s.scratch);
    return cudaGetLastError() == cudaSuccess ? ORB_OK : ORB_ERR_CUDA;
}
