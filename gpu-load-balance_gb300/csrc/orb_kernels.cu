// ORB engine kernels for sm_103a.
//
// Per level of the tree (all cells of the level in every launch):
//   plan       per-cell tile and histogram offsets (one CTA scan)
//   hist       count-left: every key of an active cell is binned into a midpoint tree of
//              depth K over the cell's bracket [cutMarginLeft, cutMarginRight); keys below
//              the bracket are counted. One pass resolves up to K bisection iterations.
//   resolve    replays the reference's bisection (src/orbit.cpp:146-232) on the histogram:
//              the same cuts, the same integer counts, the same float32 test.
//   partition  the Hoare partition of src/services/partition.cpp:30-52 computed in
//              parallel: with L_k the k-th key >= cut from the left and R_k the k-th key
//              <= cut from the right, Hoare swaps exactly (L_k, R_k) for k <= s where
//              s = max_x min(#{>= cut in [0,x)}, #{<= cut in [x,n)}), stops at
//              i = min(L_{s+1}, R_s) and swaps (i, n-1). Counts, a per-cell scan, rank
//              tables and a swap pass reproduce the permutation exactly.
//   split      src/cell.h:78-126 and src/orbit.cpp:235-250 on the device.
#include <cuda_runtime.h>
#include <stdint.h>

#include "orb_internal.cuh"

namespace orb {

const char *const kKernelNames[kNumKernels] = {
    "init", "plan", "count_left_hist", "bisect_resolve", "part_count", "part_scan",
    "part_tables", "part_swap", "part_finish", "count_left", "generate"};

namespace {

__device__ __forceinline__ void add_bytes(const Level &v, Kernel k, unsigned long long b) {
    atomicAdd(&v.counters->bytes[k], b);
}

// ------------------------------------------------------------------------------------
// Block helpers
// ------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t warp_sum(uint32_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ uint32_t warp_max(uint32_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ __forceinline__ uint32_t warp_min(uint32_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Sum over the block; every thread gets the total. `sh` holds >= 32 words.
__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t *sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    uint32_t t = lane < nw ? sh[lane] : 0u;
    return warp_sum(t);
}

__device__ __forceinline__ uint32_t block_max(uint32_t v, uint32_t *sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_max(v);
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    uint32_t t = lane < nw ? sh[lane] : 0u;
    return warp_max(t);
}

__device__ __forceinline__ uint32_t block_min(uint32_t v, uint32_t *sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_min(v);
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    uint32_t t = lane < nw ? sh[lane] : 0xffffffffu;
    return warp_min(t);
}

// Exclusive scan of two counters over the block (thread order). Returns the exclusive
// prefix; *ta, *tb receive the block totals. `sh` holds >= 64 words.
__device__ __forceinline__ uint2 block_excl_scan2(uint32_t a, uint32_t b, uint32_t *sh,
                                                  uint32_t *ta, uint32_t *tb) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t ia = a, ib = b;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t xa = __shfl_up_sync(0xffffffffu, ia, o);
        uint32_t xb = __shfl_up_sync(0xffffffffu, ib, o);
        if (lane >= o) {
            ia += xa;
            ib += xb;
        }
    }
    __syncthreads();
    if (lane == 31) {
        sh[warp] = ia;
        sh[32 + warp] = ib;
    }
    __syncthreads();
    if (warp == 0) {
        uint32_t wa = lane < nw ? sh[lane] : 0u, wb = lane < nw ? sh[32 + lane] : 0u;
        uint32_t sa = wa, sb = wb;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t xa = __shfl_up_sync(0xffffffffu, sa, o);
            uint32_t xb = __shfl_up_sync(0xffffffffu, sb, o);
            if (lane >= o) {
                sa += xa;
                sb += xb;
            }
        }
        sh[lane] = sa - wa;  // exclusive warp offsets
        sh[32 + lane] = sb - wb;
        if (lane == 31) {
            sh[64] = sa;
            sh[65] = sb;
        }
    }
    __syncthreads();
    uint2 r = make_uint2(sh[warp] + ia - a, sh[32 + warp] + ib - b);
    *ta = sh[64];
    *tb = sh[65];
    __syncthreads();
    return r;
}

// Largest c in [0, C] with off[c] <= t (off non-decreasing, off[0] = 0).
__device__ __forceinline__ int find_cell(const uint32_t *off, int C, uint32_t t) {
    int lo = 0, hi = C;  // invariant: off[lo] <= t, answer in [lo, hi]
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= t)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// Visits every key of [e0, e1) once, float4 loads over the 16-byte aligned body.
template <class F>
__device__ __forceinline__ void for_keys(const float *__restrict__ keys, uint32_t e0, uint32_t e1,
                                         F &&f) {
    const uint32_t tid = threadIdx.x, nt = blockDim.x;
    const uintptr_t addr = reinterpret_cast<uintptr_t>(keys + e0);
    const uint32_t mis = (uint32_t)(((16u - (addr & 15u)) & 15u) >> 2);
    const uint32_t a0 = min(e1, e0 + mis);
    for (uint32_t i = e0 + tid; i < a0; i += nt) f(__ldg(keys + i));
    const uint32_t n4 = (e1 - a0) >> 2;
    const float4 *k4 = reinterpret_cast<const float4 *>(keys + a0);
#pragma unroll 4
    for (uint32_t j = tid; j < n4; j += nt) {
        float4 q = __ldg(k4 + j);
        f(q.x);
        f(q.y);
        f(q.z);
        f(q.w);
    }
    for (uint32_t i = a0 + (n4 << 2) + tid; i < e1; i += nt) f(__ldg(keys + i));
}

// Tile t of the level -> (cell, slot, key range). Block-uniform.
struct TileRef {
    int c;
    int slot;
    uint32_t e0, e1;   // absolute key range of the tile
    uint32_t local;    // tile index within the cell
};

__device__ __forceinline__ TileRef tile_ref(const Level &v, uint32_t t) {
    TileRef r;
    r.c = find_cell(v.tile_off, v.C, t);
    r.slot = level_slot(v, r.c);
    r.local = t - v.tile_off[r.c];
    const uint2 rg = v.ranges[r.slot];
    r.e0 = rg.x + r.local * (uint32_t)kTile;
    r.e1 = min(rg.y, r.e0 + (uint32_t)kTile);
    return r;
}

__device__ __forceinline__ int tree_depth(uint32_t n) {
    int lg = 31 - __clz(max(n, 1u));  // floor(log2 n)
    return max(4, min(kMaxBinsLog2, lg - 1));
}

// ------------------------------------------------------------------------------------
// Init: identity permutation, zeroed heap/ranges, root cell (src/orbit.cpp:74-81)
// ------------------------------------------------------------------------------------
__global__ void k_init(Level v, uint32_t n, float lo0, float lo1, float lo2, float hi0,
                       float hi1, float hi2, uint32_t d, int heap_cells) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v.idx)
        for (uint64_t i = g; i < n; i += stride) v.idx[i] = (uint32_t)i;
    uint32_t *hw = reinterpret_cast<uint32_t *>(v.heap);
    const uint64_t words = (uint64_t)heap_cells * 13;
    for (uint64_t i = g + 13; i < words; i += stride) hw[i] = 0u;
    for (uint64_t i = g + 1; i < (uint64_t)heap_cells; i += stride) v.ranges[i] = make_uint2(0u, 0u);
    if (g == 0) {
        orb_cell_t r;
        r.id = 0;
        r.nLeafCells = (int32_t)d;
        r.prevCutAxis = -1;
        r.cutAxis = 0;  // orbit.cpp:75
        r.foundCut = 0;
        r.pad_[0] = r.pad_[1] = r.pad_[2] = 0;
        r.lower[0] = lo0;
        r.lower[1] = lo1;
        r.lower[2] = lo2;
        r.upper[0] = hi0;
        r.upper[1] = hi1;
        r.upper[2] = hi2;
        r.cutMarginLeft = lo0;  // setCutMargin, orbit.cpp:76
        r.cutMarginRight = hi0;
        v.heap[0] = r;
        v.ranges[0] = make_uint2(0u, n);
        BuildCounters z = {};
        *v.counters = z;
    }
}

// ------------------------------------------------------------------------------------
// Plan: per-cell tile and histogram offsets (single CTA, any C).
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_plan(Level v) {
    __shared__ uint32_t sh[96];
    const int C = v.C, tid = threadIdx.x, nt = blockDim.x;
    const int per = (C + nt - 1) / nt;
    const int c0 = min(C, tid * per), c1 = min(C, c0 + per);
    uint32_t ta = 0, tb = 0;
    for (int c = c0; c < c1; ++c) {
        const uint2 rg = v.ranges[level_slot(v, c)];
        const uint32_t n = rg.y - rg.x;
        ta += (n + kTile - 1) / kTile;
        tb += 1u << tree_depth(n);
    }
    uint32_t tot_a, tot_b;
    uint2 p = block_excl_scan2(ta, tb, sh, &tot_a, &tot_b);
    for (int c = c0; c < c1; ++c) {
        const uint2 rg = v.ranges[level_slot(v, c)];
        const uint32_t n = rg.y - rg.x;
        const int k = tree_depth(n);
        v.tile_off[c] = p.x;
        v.hist_off[c] = p.y;
        v.hist_k[c] = (uint8_t)k;
        v.state[c] = kActive;
        v.iters[c] = 0;
        v.below[c] = 0;
        p.x += (n + kTile - 1) / kTile;
        p.y += 1u << k;
    }
    if (tid == 0) {
        v.tile_off[C] = tot_a;
        v.hist_off[C] = tot_b;
    }
}

// ------------------------------------------------------------------------------------
// Count-left histogram pass
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_hist(Level v) {
    __shared__ uint32_t s_hist[1 << kMaxBinsLog2];
    __shared__ uint32_t s_red[32];
    const uint32_t total = v.tile_off[v.C];
    for (uint32_t t = blockIdx.x; t < total; t += gridDim.x) {
        const TileRef tr = tile_ref(v, t);
        if (v.state[tr.c] != kActive) continue;
        const orb_cell_t &cell = v.heap[tr.slot];
        const float L = cell.cutMarginLeft, R = cell.cutMarginRight;
        const float *keys = axis_keys(v, eff_axis(cell.cutAxis));
        const int K = v.hist_k[tr.c];
        const uint32_t nb = 1u << K;
        for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) s_hist[b] = 0u;
        __syncthreads();
        uint32_t below = 0;
        for_keys(keys, tr.e0, tr.e1, [&](float k) {
            if (k < L) {
                ++below;
            } else if (k < R) {
                float lo = L, hi = R;
                uint32_t bin = 0;
                for (int s = 0; s < K; ++s) {
                    const float m = mid_cut(lo, hi);
                    const bool right = !(k < m);
                    bin = (bin << 1) | (uint32_t)right;
                    lo = right ? m : lo;
                    hi = right ? hi : m;
                }
                atomicAdd(&s_hist[bin], 1u);
            }
        });
        below = block_sum(below, s_red);
        if (threadIdx.x == 0) {
            if (below) atomicAdd(&v.below[tr.c], below);
            add_bytes(v, kKHist, 4ull * (tr.e1 - tr.e0));
        }
        uint32_t *g = v.hist + v.hist_off[tr.c];
        for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) {
            const uint32_t h = s_hist[b];
            if (h) atomicAdd(&g[b], h);
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------------------------
// Resolve: replay up to K bisection iterations per cell on its histogram (warp per cell).
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_resolve(Level v) {
    const int c = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (c >= v.C) return;
    if (v.state[c] != kActive) return;
    const int slot = level_slot(v, c);
    orb_cell_t &cell = v.heap[slot];
    const uint2 rg = v.ranges[slot];
    const uint32_t n = rg.y - rg.x;
    const int K = v.hist_k[c];
    uint32_t *g = v.hist + v.hist_off[c];
    float L = cell.cutMarginLeft, R = cell.cutMarginRight;
    uint32_t it = v.iters[c];
    uint32_t prefix = v.below[c];
    uint32_t pos = 0, width = 1u << K;
    uint8_t st = kActive;
    for (int step = 0; step < K; ++step) {
        if (it >= (uint32_t)kMaxIterations) {
            st = kCapped;
            break;
        }
        const uint32_t half = width >> 1;
        uint32_t sum = 0;
        for (uint32_t b = lane; b < half; b += 32) sum += g[pos + b];
        sum = warp_sum(sum);
        const uint32_t cl = prefix + sum;
        ++it;
        const int dir = convergence(cl, n);
        if (dir == 0) {
            st = kFound;
            break;
        }
        const float cut = mid_cut(L, R);
        if (dir > 0) {
            R = cut;
        } else {
            L = cut;
            prefix += sum;
            pos += half;
        }
        width = half;
    }
    if (st == kActive && it >= (uint32_t)kMaxIterations) st = kCapped;
    __syncwarp();
    for (uint32_t b = lane; b < (1u << K); b += 32) g[b] = 0u;
    if (lane == 0) {
        add_bytes(v, kKResolve, 8ull << K);  // bins read and cleared
        cell.cutMarginLeft = L;
        cell.cutMarginRight = R;
        cell.foundCut = st == kFound ? 1 : 0;
        v.iters[c] = (uint8_t)it;
        v.state[c] = st;
        v.below[c] = 0;
        atomicMax(&v.counters->max_iters, it);
        if (st == kCapped) atomicAdd(&v.counters->unfound, 1u);
        if (st == kActive) v.counters->any_active = 1u;
    }
}

// ------------------------------------------------------------------------------------
// Partition
// ------------------------------------------------------------------------------------
__device__ __forceinline__ float cell_cut(const orb_cell_t &c) {
    return mid_cut(c.cutMarginLeft, c.cutMarginRight);
}

// P1: keys >= cut and keys <= cut per tile.
__global__ void __launch_bounds__(kThreads) k_part_count(Level v) {
    __shared__ uint32_t s_red[32];
    const uint32_t total = v.tile_off[v.C];
    for (uint32_t t = blockIdx.x; t < total; t += gridDim.x) {
        const TileRef tr = tile_ref(v, t);
        const orb_cell_t &cell = v.heap[tr.slot];
        const float cut = cell_cut(cell);
        const float *keys = axis_keys(v, eff_axis(cell.cutAxis));
        uint32_t ge = 0, le = 0;
        for_keys(keys, tr.e0, tr.e1, [&](float k) {
            ge += !(k < cut);
            le += !(k > cut);
        });
        ge = block_sum(ge, s_red);
        le = block_sum(le, s_red);
        if (threadIdx.x == 0) {
            v.tile_ge_cnt[t] = ge;
            v.tile_le_cnt[t] = le;
            add_bytes(v, kKPartCount, 4ull * (tr.e1 - tr.e0) + 8ull);
        }
    }
}

constexpr int kSeg = kTile / kThreads;  // consecutive keys per thread in the ordered passes

// Loads one tile's keys into shared memory (coalesced) for an in-order walk.
__device__ __forceinline__ void load_tile(const float *keys, uint32_t e0, uint32_t e1, float *s_keys) {
    for (uint32_t i = threadIdx.x; i < e1 - e0; i += blockDim.x) s_keys[i] = __ldg(keys + e0 + i);
    __syncthreads();
}

// P1.5: per cell, prefix sums over its tiles and the swap count s.
__global__ void __launch_bounds__(kThreads) k_part_scan(Level v) {
    __shared__ uint32_t sh[96];
    __shared__ float s_keys[kTile];
    for (int c = blockIdx.x; c < v.C; c += gridDim.x) {
        const int slot = level_slot(v, c);
        const uint32_t t0 = v.tile_off[c], nt = v.tile_off[c + 1] - t0;
        uint32_t cg = 0, cl = 0;
        for (uint32_t b = 0; b < nt; b += blockDim.x) {
            const uint32_t i = b + threadIdx.x;
            const uint32_t a = i < nt ? v.tile_ge_cnt[t0 + i] : 0u;
            const uint32_t l = i < nt ? v.tile_le_cnt[t0 + i] : 0u;
            uint32_t ta, tl;
            const uint2 p = block_excl_scan2(a, l, sh, &ta, &tl);
            if (i < nt) {
                v.tile_ge[t0 + i] = cg + p.x;
                v.tile_le[t0 + i] = cl + p.y;
            }
            cg += ta;
            cl += tl;
        }
        const uint32_t ge_tot = cg, le_tot = cl;
        __syncthreads();  // prefixes visible to the whole block
        // First tile whose end boundary has f >= g (exists: f(n) >= 0 = g(n)).
        uint32_t cross = 0xffffffffu;
        for (uint32_t i = threadIdx.x; i < nt; i += blockDim.x) {
            const uint32_t f_end = v.tile_ge[t0 + i] + v.tile_ge_cnt[t0 + i];
            const uint32_t g_end = le_tot - (v.tile_le[t0 + i] + v.tile_le_cnt[t0 + i]);
            if (f_end >= g_end) cross = min(cross, i);
        }
        cross = block_min(cross, sh);
        uint32_t s = 0;
        if (nt > 0) {
            const uint32_t t = t0 + cross;
            const uint2 rg = v.ranges[slot];
            const uint32_t e0 = rg.x + cross * (uint32_t)kTile, e1 = min(rg.y, e0 + (uint32_t)kTile);
            const orb_cell_t &cell = v.heap[slot];
            const float cut = cell_cut(cell);
            load_tile(axis_keys(v, eff_axis(cell.cutAxis)), e0, e1, s_keys);
            const uint32_t m = e1 - e0;
            const uint32_t s0 = min(m, threadIdx.x * (uint32_t)kSeg), s1 = min(m, s0 + kSeg);
            uint32_t lg = 0, ll = 0;
            for (uint32_t i = s0; i < s1; ++i) {
                const float k = s_keys[i];
                lg += !(k < cut);
                ll += !(k > cut);
            }
            uint32_t ta, tl;
            const uint2 p = block_excl_scan2(lg, ll, sh, &ta, &tl);
            uint32_t f = v.tile_ge[t] + p.x;
            uint32_t gg = le_tot - v.tile_le[t] - p.y;
            uint32_t best = min(f, gg);
            for (uint32_t i = s0; i < s1; ++i) {
                const float k = s_keys[i];
                f += !(k < cut);
                gg -= !(k > cut);
                best = max(best, min(f, gg));
            }
            s = block_max(best, sh);
        }
        if (threadIdx.x == 0) {
            add_bytes(v, kKPartScan, 16ull * nt + (nt ? 4ull * min((uint32_t)kTile, v.ranges[slot].y - v.ranges[slot].x) : 0ull));
            v.part_s[c] = s;
            v.part_ge[c] = ge_tot;
            v.part_le[c] = le_tot;
        }
        __syncthreads();
    }
}

// P2: rank tables. tl[begin + k] = position of the (k+1)-th key >= cut for k <= s,
// tr[begin + k] = position of the (k+1)-th key <= cut from the right for k < s.
__global__ void __launch_bounds__(kThreads) k_part_tables(Level v) {
    __shared__ uint32_t sh[96];
    __shared__ float s_keys[kTile];
    const uint32_t total = v.tile_off[v.C];
    for (uint32_t t = blockIdx.x; t < total; t += gridDim.x) {
        const TileRef tr = tile_ref(v, t);
        const uint32_t s = v.part_s[tr.c], le_tot = v.part_le[tr.c];
        const uint32_t fpre = v.tile_ge[t], lpre = v.tile_le[t];
        const uint2 rg = v.ranges[tr.slot];
        // Nothing of this tile can enter the tables: every rank here is beyond s.
        const bool need_l = fpre <= s;
        const bool need_r = (le_tot - lpre) > 0 && (le_tot - lpre - v.tile_le_cnt[t]) < s;
        if (!need_l && !need_r) continue;
        const orb_cell_t &cell = v.heap[tr.slot];
        const float cut = cell_cut(cell);
        load_tile(axis_keys(v, eff_axis(cell.cutAxis)), tr.e0, tr.e1, s_keys);
        const uint32_t m = tr.e1 - tr.e0;
        const uint32_t s0 = min(m, threadIdx.x * (uint32_t)kSeg), s1 = min(m, s0 + kSeg);
        uint32_t lg = 0, ll = 0;
        for (uint32_t i = s0; i < s1; ++i) {
            const float k = s_keys[i];
            lg += !(k < cut);
            ll += !(k > cut);
        }
        uint32_t ta, tl;
        const uint2 p = block_excl_scan2(lg, ll, sh, &ta, &tl);
        uint32_t rk = fpre + p.x;   // 0-based left rank of the next key >= cut
        uint32_t lseen = lpre + p.y;  // keys <= cut before the current position
        const uint32_t pos0 = tr.e0 - rg.x;
        uint32_t written = 0;
        for (uint32_t i = s0; i < s1; ++i) {
            const float k = s_keys[i];
            if (!(k < cut)) {
                if (rk <= s) {
                    v.tl[rg.x + rk] = pos0 + i;
                    ++written;
                }
                ++rk;
            }
            if (!(k > cut)) {
                const uint32_t rr = le_tot - lseen - 1;  // 0-based right rank
                if (rr < s) {
                    v.tr[rg.x + rr] = pos0 + i;
                    ++written;
                }
                ++lseen;
            }
        }
        written = block_sum(written, sh);
        if (threadIdx.x == 0) add_bytes(v, kKPartTables, 4ull * m + 4ull * written);
        __syncthreads();
    }
}

__device__ __forceinline__ void swap_particles(const Level &v, uint32_t a, uint32_t b) {
    float t;
    t = v.x[a]; v.x[a] = v.x[b]; v.x[b] = t;
    t = v.y[a]; v.y[a] = v.y[b]; v.y[b] = t;
    t = v.z[a]; v.z[a] = v.z[b]; v.z[b] = t;
    if (v.idx) {
        uint32_t u = v.idx[a];
        v.idx[a] = v.idx[b];
        v.idx[b] = u;
    }
}

// P3: the s Hoare swaps of every cell; tile j of a cell swaps pairs [j*kTile, (j+1)*kTile).
__global__ void __launch_bounds__(kThreads) k_part_swap(Level v) {
    const uint32_t total = v.tile_off[v.C];
    for (uint32_t t = blockIdx.x; t < total; t += gridDim.x) {
        const int c = find_cell(v.tile_off, v.C, t);
        const uint32_t local = t - v.tile_off[c];
        const uint32_t s = v.part_s[c];
        const uint32_t k0 = local * (uint32_t)kTile;
        if (k0 >= s) continue;
        const uint32_t k1 = min(s, k0 + (uint32_t)kTile);
        const uint32_t b = v.ranges[level_slot(v, c)].x;
        for (uint32_t k = k0 + threadIdx.x; k < k1; k += blockDim.x)
            swap_particles(v, b + v.tl[b + k], b + v.tr[b + k]);
        // per pair: 2 x 16 B read + 2 x 16 B written (x,y,z,idx) + 8 B of rank tables
        if (threadIdx.x == 0) add_bytes(v, kKPartSwap, 72ull * (k1 - k0));
    }
}

__device__ void set_axis_and_margin(orb_cell_t &c, BuildCounters *ctr) {
    // setCutAxis (src/cell.h:102-121) then setCutMargin (src/cell.h:123-126)
    int max_d = -1;
    float max_size = 0.0f;
    for (int k = 0; k < 3; ++k) {
        const float size = __fsub_rn(c.upper[k], c.lower[k]);
        if (size > max_size) {
            max_size = size;
            max_d = k;
        }
    }
    c.cutAxis = max_d;
    if (max_d < 0) atomicAdd(&ctr->zero_volume, 1u);
    const int a = eff_axis(max_d);
    c.cutMarginLeft = c.lower[a];
    c.cutMarginRight = c.upper[a];
}

// P4: split index, final swap, children's ranges and (optionally) the children's cells.
__global__ void __launch_bounds__(kThreads) k_part_finish(Level v, int do_split) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= v.C) return;
    const int slot = level_slot(v, c);
    const orb_cell_t cell = v.heap[slot];
    const uint2 rg = v.ranges[slot];
    const uint32_t n = rg.y - rg.x;
    const uint32_t s = v.part_s[c], ge_tot = v.part_ge[c];
    uint32_t i = n;
    if (ge_tot > s) i = min(i, v.tl[rg.x + s]);
    if (s >= 1) i = min(i, v.tr[rg.x + s - 1]);
    if (i < n) {
        if (i != n - 1) swap_particles(v, rg.x + i, rg.x + n - 1);
    } else {
        atomicAdd(&v.counters->degenerate, 1u);
    }
    // children slots: slot - id is the instance's heap base
    const int lslot = slot + cell.id + 1, rslot = slot + cell.id + 2;
    v.ranges[lslot] = make_uint2(rg.x, rg.x + i);
    v.ranges[rslot] = make_uint2(rg.x + i, rg.y);
    if (!do_split) return;
    // Cell::cut (src/cell.h:78-100) and src/orbit.cpp:238-246
    const float cut = cell_cut(cell);
    const int a = eff_axis(cell.cutAxis);
    const int n_left = (cell.nLeafCells + 1) / 2;
    orb_cell_t lc, rc;
    lc.id = 2 * cell.id + 1;
    rc.id = 2 * cell.id + 2;
    lc.nLeafCells = n_left;
    rc.nLeafCells = cell.nLeafCells - n_left;
    lc.prevCutAxis = rc.prevCutAxis = cell.cutAxis;
    lc.foundCut = rc.foundCut = 0;
    lc.pad_[0] = lc.pad_[1] = lc.pad_[2] = 0;
    rc.pad_[0] = rc.pad_[1] = rc.pad_[2] = 0;
    for (int k = 0; k < 3; ++k) {
        lc.lower[k] = rc.lower[k] = cell.lower[k];
        lc.upper[k] = rc.upper[k] = cell.upper[k];
    }
    lc.upper[a] = cut;
    rc.lower[a] = cut;
    set_axis_and_margin(rc, v.counters);
    set_axis_and_margin(lc, v.counters);
    v.heap[lslot] = lc;
    v.heap[rslot] = rc;
}

// ------------------------------------------------------------------------------------
// Service count-left: one plain pass at getCut() per cell, found cells skipped.
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_count_left(Level v) {
    __shared__ uint32_t s_red[32];
    const uint32_t total = v.tile_off[v.C];
    for (uint32_t t = blockIdx.x; t < total; t += gridDim.x) {
        const TileRef tr = tile_ref(v, t);
        const orb_cell_t &cell = v.heap[tr.slot];
        if (cell.foundCut) continue;
        const float cut = cell_cut(cell);
        uint32_t cnt = 0;
        for_keys(axis_keys(v, eff_axis(cell.cutAxis)), tr.e0, tr.e1, [&](float k) { cnt += k < cut; });
        cnt = block_sum(cnt, s_red);
        if (threadIdx.x == 0) {
            if (cnt) atomicAdd(&v.out_counts[tr.c], cnt);
            add_bytes(v, kKCountLeft, 4ull * (tr.e1 - tr.e0));
        }
    }
}

// ------------------------------------------------------------------------------------
// Seeded generators (bit-identical with the CPU oracle's generator)
// ------------------------------------------------------------------------------------
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ uint64_t draw(uint64_t seed_mix, uint64_t counter) {
    return mix64(seed_mix + counter * 0xD1B54A32D192ED03ull);
}
__device__ __forceinline__ float unit_coord(uint64_t u) {
    return __fsub_rn(__fmul_rn(__uint2float_rn((uint32_t)(u >> 40)), 0x1p-24f), 0.5f);
}
__device__ __forceinline__ double unit_double(uint64_t u) {
    return __dmul_rn(__ull2double_rn(u >> 11), 0x1p-53);
}

__global__ void k_gen_uniform(uint64_t seed, uint64_t n, float *x, float *y, float *z) {
    const uint64_t sm = mix64(seed);
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        x[i] = unit_coord(draw(sm, 3 * i + 0));
        y[i] = unit_coord(draw(sm, 3 * i + 1));
        z[i] = unit_coord(draw(sm, 3 * i + 2));
    }
}

struct PlummerTable {
    float centre[64 * 3];
    double scale[64];
};

__global__ void k_gen_plummer(uint64_t seed, uint64_t n, PlummerTable tab, float *x, float *y,
                              float *z) {
    const uint64_t sm = mix64(seed);
    const float hi = 0x1.fffffep-2f;  // nextafter(0.5f, -1)
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t c = i * 64;
        const uint64_t sel = draw(sm, c) >> 40;
        float p[3];
        if (sel * 10 < 9ull * (1ull << 24)) {
            const int k = (int)(draw(sm, c + 1) % 64);
            double w = unit_double(draw(sm, c + 2));
            w = fmax(w, unit_double(draw(sm, c + 3)));
            w = fmax(w, unit_double(draw(sm, c + 4)));
            const double r = __ddiv_rn(__dmul_rn(tab.scale[k], w),
                                       __dsqrt_rn(__dsub_rn(1.0, __dmul_rn(w, w))));
            double v0 = 1.0, v1 = 0.0, v2 = 0.0, q = 1.0;
            for (int t = 0; t < 19; ++t) {
                const double u0 = __dsub_rn(__dmul_rn(2.0, unit_double(draw(sm, c + 5 + 3 * t + 0))), 1.0);
                const double u1 = __dsub_rn(__dmul_rn(2.0, unit_double(draw(sm, c + 5 + 3 * t + 1))), 1.0);
                const double u2 = __dsub_rn(__dmul_rn(2.0, unit_double(draw(sm, c + 5 + 3 * t + 2))), 1.0);
                const double qq = __dadd_rn(__dadd_rn(__dmul_rn(u0, u0), __dmul_rn(u1, u1)), __dmul_rn(u2, u2));
                if (qq > 0.0 && qq <= 1.0) {
                    v0 = u0;
                    v1 = u1;
                    v2 = u2;
                    q = qq;
                    break;
                }
            }
            const double s = __ddiv_rn(r, __dsqrt_rn(q));
            const double vv[3] = {v0, v1, v2};
            for (int a = 0; a < 3; ++a) {
                const float f = __double2float_rn(__dadd_rn((double)tab.centre[3 * k + a], __dmul_rn(vv[a], s)));
                p[a] = fminf(fmaxf(f, -0.5f), hi);
            }
        } else {
            for (int a = 0; a < 3; ++a) p[a] = unit_coord(draw(sm, c + 2 + a));
        }
        x[i] = p[0];
        y[i] = p[1];
        z[i] = p[2];
    }
}

inline int grid_for(uint64_t n, int threads, int cap) {
    uint64_t g = (n + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > (uint64_t)cap) g = cap;
    return (int)g;
}

}  // namespace

// ------------------------------------------------------------------------------------
// Launchers
// ------------------------------------------------------------------------------------
void launch_init(const Level &v, uint64_t n, const float lower[3], const float upper[3],
                 uint32_t d, int heap_cells, cudaStream_t st) {
    uint64_t work = n > (uint64_t)heap_cells * 13 ? n : (uint64_t)heap_cells * 13;
    k_init<<<grid_for(work, 256, 152 * 16), 256, 0, st>>>(v, (uint32_t)n, lower[0], lower[1],
                                                        lower[2], upper[0], upper[1], upper[2], d,
                                                        heap_cells);
}

void launch_level_kernel(Kernel k, const Level &v, int grid, int arg, cudaStream_t st) {
    switch (k) {
        case kKPlan: k_plan<<<1, 1024, 0, st>>>(v); break;
        case kKHist: k_hist<<<grid, kThreads, 0, st>>>(v); break;
        case kKResolve:
            k_resolve<<<grid_for((uint64_t)v.C * 32, kThreads, 1 << 30), kThreads, 0, st>>>(v);
            break;
        case kKPartCount: k_part_count<<<grid, kThreads, 0, st>>>(v); break;
        case kKPartScan: k_part_scan<<<grid_for(v.C, 1, grid), kThreads, 0, st>>>(v); break;
        case kKPartTables: k_part_tables<<<grid, kThreads, 0, st>>>(v); break;
        case kKPartSwap: k_part_swap<<<grid, kThreads, 0, st>>>(v); break;
        case kKPartFinish:
            k_part_finish<<<grid_for(v.C, kThreads, 1 << 30), kThreads, 0, st>>>(v, arg);
            break;
        case kKCountLeft: k_count_left<<<grid, kThreads, 0, st>>>(v); break;
        default: break;
    }
}

void launch_gen_uniform(uint64_t seed, uint64_t n, float *x, float *y, float *z,
                        cudaStream_t st) {
    k_gen_uniform<<<grid_for(n, 256, 152 * 32), 256, 0, st>>>(seed, n, x, y, z);
}

void launch_gen_plummer(uint64_t seed, uint64_t n, const float *centres, const double *scales,
                        float *x, float *y, float *z, cudaStream_t st) {
    PlummerTable tab;
    for (int i = 0; i < 64 * 3; ++i) tab.centre[i] = centres[i];
    for (int i = 0; i < 64; ++i) tab.scale[i] = scales[i];
    k_gen_plummer<<<grid_for(n, 256, 152 * 32), 256, 0, st>>>(seed, n, tab, x, y, z);
}

}  // namespace orb
