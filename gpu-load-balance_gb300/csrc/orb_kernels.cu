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
// Beside them: the bisection of cells of at most one tile in one launch (a warp per cell),
// the subtree kernel (one CTA finishes a cell's last levels with its particles in L2), the
// optional sampled first pass, the service count-left, seeded generators and the batched
// and served forms' helpers.
#include <cuda_runtime.h>
#include <stdint.h>

#include "orb_internal.cuh"

namespace orb {

const char *const kKernelNames[kNumKernels] = {
    "init", "plan", "count_left_hist", "bisect_resolve", "part_classify", "part_scan",
    "part_cells", "part_swap", "part_finish", "count_left", "generate", "bisect_cta",
    "tile_map", "bisect_tile", "warm_start", "subtree_check", "subtree",
    "count_left_sample", "count_left_sample_pick", "weighted_start", "count_left_weighted",
    "bisect_resolve_weighted", "stage_gather"};

namespace {

__device__ __forceinline__ void add_bytes(const Level &v, Kernel k, unsigned long long b) {
    atomicAdd(&v.counters->bytes[k], b);
}

// Programmatic dependent launch (level kernels are launched with it): wait until the
// previous kernel of the stream has finished and its writes are visible, then let the next
// kernel's CTAs be scheduled as this kernel's CTAs retire (its launch and ramp-up overlap
// this kernel's tail). Every level kernel calls this before it reads anything a previous
// kernel wrote; without a programmatic dependency both instructions do nothing.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" :::);
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
__device__ __forceinline__ uint32_t warp_excl_scan(uint32_t v, uint32_t *total) {
    const int lane = threadIdx.x & 31;
    uint32_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    *total = __shfl_sync(0xffffffffu, inc, 31);
    return inc - v;
}

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
    r.c = v.htile_cell ? (int)v.htile_cell[t] : find_cell(v.tile_off, v.C, t);
    r.slot = level_slot(v, r.c);
    r.local = t - v.tile_off[r.c];
    const uint2 rg = v.ranges[r.slot];
    r.e0 = rg.x + r.local * (uint32_t)kTile;
    r.e1 = min(rg.y, r.e0 + (uint32_t)kTile);
    return r;
}

// Capacity of a cell's compaction list: cells the histogram passes bisect (more than one
// tile) get n/8 keys, at least 2048 (16x the sparse threshold's bracket): room for the
// sampled bracket of a first pass (at most kPredCompactShare of the keys) and for the
// bracket of a sparse pass.
__host__ __device__ __forceinline__ uint32_t list_capacity(uint32_t n) {
    return n > (uint32_t)kTile ? (n / 8 > 2048u ? n / 8 : 2048u) : 0u;
}

// Cells of more than kTile keys (the count passes' cells) get the deepest tree, so the cold
// passes reach the iteration cap.
static_assert(kTile >= (2 << kMaxBinsLog2), "cells of more than kTile keys get trees of depth 11");
static_assert(kColdHistPasses * kMaxBinsLog2 >= kMaxIterations, "3 cold passes reach the cap");
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

// Batched init: every instance's root cell and root range (heap and ranges are zeroed by
// the host before) and idx = position relative to the instance. blockIdx.y walks the
// instances, blockIdx.x their particles.
__global__ void k_init_batch(Level v, const BatchRoot *roots, int k) {
    for (int i = blockIdx.y; i < k; i += gridDim.y) {
        const BatchRoot r = roots[i];
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            orb_cell_t c;
            c.id = 0;
            c.nLeafCells = (int32_t)r.d;
            c.prevCutAxis = -1;
            c.cutAxis = 0;  // orbit.cpp:75
            c.foundCut = 0;
            c.pad_[0] = c.pad_[1] = c.pad_[2] = 0;
            for (int a = 0; a < 3; ++a) {
                c.lower[a] = r.lower[a];
                c.upper[a] = r.upper[a];
            }
            c.cutMarginLeft = r.lower[0];  // setCutMargin, orbit.cpp:76
            c.cutMarginRight = r.upper[0];
            v.heap[r.heap_base] = c;
            v.ranges[r.heap_base] = make_uint2(r.offset, r.offset + r.n);
        }
        if (v.idx)
            for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < r.n; p += gridDim.x * blockDim.x)
                v.idx[r.offset + p] = p;
    }
}

// Warm builds: whether a hinted bracket [L, R) can hold the cut the bisection looks for,
// given the counts of keys below L and below R. Outside it every tested cut would keep
// moving the same margin: count(< L) already too high, or count(< R) still too low.
__device__ __forceinline__ bool warm_bracket_holds(uint32_t below_L, uint32_t below_R, uint32_t n,
                                                   float ratio) {
    return convergence(below_L, n, ratio) <= 0 && convergence(below_R, n, ratio) >= 0;
}

// Restart of a cell whose hinted bracket missed: the reference's own start, the cell's extent
// along its cut axis (setCutMargin, src/cell.h:123-126).
__device__ __forceinline__ void warm_reset(orb_cell_t &cell, float &L, float &R, BuildCounters *ctr) {
    const int a = eff_axis(cell.cutAxis);
    L = cell.lower[a];
    R = cell.upper[a];
    cell.cutMarginLeft = L;
    cell.cutMarginRight = R;
    atomicAdd(&ctr->warm_resets, 1u);
}

// ------------------------------------------------------------------------------------
// Plan: per-cell tile and histogram offsets (single CTA, any C).
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_plan(Level v) {
    pdl_enter();
    if (v.skip && *(volatile const uint32_t *)v.skip) return;  // subtrees took this level
    __shared__ uint32_t sh[96];
    const int C = v.C, tid = threadIdx.x, nt = blockDim.x;
    const int per = (C + nt - 1) / nt;
    const int c0 = min(C, tid * per), c1 = min(C, c0 + per);
    uint32_t ta = 0, tb = 0, tp = 0, tc = 0;
    for (int c = c0; c < c1; ++c) {
        const uint2 rg = v.ranges[level_slot(v, c)];
        const uint32_t n = rg.y - rg.x;
        ta += (n + kTile - 1) / kTile;
        tb += 1u << tree_depth(n);
        tp += (n + kPTile - 1) / kPTile;
        tc += list_capacity(n);
    }
    uint32_t tot_a, tot_b, tot_p, tot_c;
    uint2 p = block_excl_scan2(ta, tb, sh, &tot_a, &tot_b);
    const uint2 pc = block_excl_scan2(tp, tc, sh, &tot_p, &tot_c);
    uint32_t pp = pc.x, cc = pc.y;
    for (int c = c0; c < c1; ++c) {
        const uint2 rg = v.ranges[level_slot(v, c)];
        const uint32_t n = rg.y - rg.x;
        v.tile_off[c] = p.x;
        v.hist_off[c] = p.y;
        v.ptile_off[c] = pp;
        v.cmp_off[c] = cc;
        pp += (n + kPTile - 1) / kPTile;
        cc += list_capacity(n);
        p.x += (n + kTile - 1) / kTile;
        p.y += 1u << tree_depth(n);
    }
    if (tid == 0) {
        v.tile_off[C] = tot_a;
        v.hist_off[C] = tot_b;
        v.ptile_off[C] = tot_p;
        v.cmp_off[C] = tot_c;
    }
}

// Warm builds, after the plan: a cell whose previous tree cut on the same axis starts from
// the hinted bracket (clipped to its extent) when that narrows it. Its first count pass is
// then sparse: most keys lie outside. One thread per cell.
__global__ void k_warm_start(Level v) {
    pdl_enter();
    if (v.skip && *(volatile const uint32_t *)v.skip) return;  // subtrees took this level
    const int c = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    uint32_t nwarm = 0;
    if (c < v.C) {
        const int slot = level_slot(v, c);
        orb_cell_t &cell = v.heap[slot];
        const uint2 rg = v.ranges[slot];
        const uint32_t n = rg.y - rg.x;
        const float2 h = v.hint[slot];
        uint8_t w = 0;
        if (n > 1 && !isnan(h.x) && v.hint_axis[slot] == cell.cutAxis && cell.cutAxis >= 0) {
            // half-width w x extent / sqrt(n): about w sqrt(n) keys each side if evenly spread,
            // the scale by which a median drifts when the particles move a little
            const float L = cell.cutMarginLeft, R = cell.cutMarginRight;
            const float half = __fdiv_rn(h.y, sqrtf((float)n));
            const float Lw = fmaxf(L, __fsub_rn(h.x, half)), Rw = fminf(R, __fadd_rn(h.x, half));
            if (Lw < Rw && (Lw > L || Rw < R)) {
                cell.cutMarginLeft = Lw;
                cell.cutMarginRight = Rw;
                w = 1;
                // keys in the bracket if spread evenly, capped so the first pass is sparse
                const float share = __fdiv_rn(__fsub_rn(Rw, Lw), __fsub_rn(R, L));
                const uint32_t tiles = (n + kTile - 1) / kTile;
                v.inb[c] = min((uint32_t)fminf((float)n, ceilf(share * (float)n)), v.sparse_per_tile * tiles);
                nwarm = 1;
            }
        }
        v.warm[c] = w;
    }
    nwarm = warp_sum(nwarm);
    if ((threadIdx.x & 31) == 0 && nwarm) atomicAdd(&v.counters->warm_cells, nwarm);
}

// ------------------------------------------------------------------------------------
// Count-left histogram pass
// ------------------------------------------------------------------------------------
// The midpoint tree over [L, R] with nb = 2^K leaves: edge e(0) = L, e(nb) = R, and the
// inner node j is the midpoint of its two nearest ancestors, i.e. exactly the cut the
// reference's bisection computes at that node (src/cell.h:74-76).
// Inner edges of the subtree of S leaves over [lo, hi] = [e(base), e(base + S)], written to
// e[base .. base + S): each the midpoint of its two nearest ancestors, as in the full tree.
template <int S>
__device__ __forceinline__ void fill_sub(float *e, uint32_t base, float lo, float hi) {
    float loc[S + 1];
    loc[0] = lo;
    loc[S] = hi;
#pragma unroll
    for (int st = S / 2; st >= 1; st /= 2) {
#pragma unroll
        for (int j = st; j < S; j += 2 * st) loc[j] = mid_cut(loc[j - st], loc[j + st]);
    }
#pragma unroll
    for (int j = 0; j < S; ++j) e[base + j] = loc[j];
}

// Edge table e[0 .. 2^K] of the midpoint tree over [L, R], filled by nt threads (ti = this
// thread's index, 2^K <= 16 nt): each descends once to the subtree of 2^K / nt leaves it
// owns, then fills that subtree. The caller synchronises.
__device__ void fill_edges(float *e, float L, float R, int K, uint32_t ti, uint32_t nt) {
    const uint32_t nb = 1u << K;
    int ks = 0;
    while ((nt << ks) < nb) ++ks;
    const uint32_t S = 1u << ks, base = ti * S;
    if (base < nb) {
        float lo = L, hi = R;
        for (int d = K - 1; d >= ks; --d) {
            const float mm = mid_cut(lo, hi);
            if (base & (1u << d))
                lo = mm;
            else
                hi = mm;
        }
        switch (ks) {
            case 0: e[base] = lo; break;
            case 1: fill_sub<2>(e, base, lo, hi); break;
            case 2: fill_sub<4>(e, base, lo, hi); break;
            case 3: fill_sub<8>(e, base, lo, hi); break;
            default: fill_sub<16>(e, base, lo, hi); break;
        }
    }
    if (ti == 0) e[nb] = R;
}

// Leaf of key k (L <= k < R) in that tree: the reference's descent itself (k below the
// midpoint: left half, else right half), K midpoints.
__device__ __forceinline__ int tree_bin(float k, float L, float R, int K) {
    float lo = L, hi = R;
    int b = 0;
    for (int d = K - 1; d >= 0; --d) {
        const float mm = mid_cut(lo, hi);
        if (k < mm) {
            hi = mm;
        } else {
            lo = mm;
            b += 1 << d;
        }
    }
    return b;
}

// Edge e(j) of that tree (e(0) = L, e(2^K) = R): the lower end of leaf j, reached by the same
// midpoints as tree_bin. The edges are non-decreasing (a midpoint of [lo, hi] rounds into
// [lo, hi]), so tree_bin(k) >= j exactly when k >= e(j), for L <= k < R.
__device__ __forceinline__ float tree_edge(float L, float R, int K, uint32_t j) {
    if (j >= (1u << K)) return R;
    float lo = L, hi = R;
    for (int d = K - 1; d >= 0; --d) {
        const float mm = mid_cut(lo, hi);
        if (j & (1u << d))
            lo = mm;
        else
            hi = mm;
    }
    return lo;
}

// Bin of key k (L <= k < R) in the edge table e[0..nb]: the largest b with e[b] <= k, i.e.
// the leaf the bisection's descent reaches. The spacing of the edges is uniform to a few
// ulps, so the scaled guess is off by at most one except in brackets only a few ulps
// wide, which fall back to a binary search over the table.
template <class EdgeAt>
__device__ __forceinline__ int edge_bin(float k, float L, float scale, int top, EdgeAt e) {
    int g = __float2int_rz((k - L) * scale);
    g = min(max(g, 0), top);
    if (k < e(g)) {
        --g;
        if (g >= 0 && !(k < e(g))) return g;
    } else if (!(k < e(g + 1))) {
        ++g;
        if (g <= top && k < e(g + 1)) return g;
    } else {
        return g;
    }
    int lo = 0, hi = top;  // largest b in [0, top] with e(b) <= k (e(0) = L <= k)
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (e(mid) <= k)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// Margin of the scaled guess, in bins. The tree's edges deviate from the linear edges
// L + j (R-L)/2^K by at most K u/2 <= 5.5u (every midpoint rounds once, to within u/2 of the
// mean of its two endpoints; u = spacing of floats at max(|L|, |R|)). The guess
// t = fl(fl(k-L) * scale), scale = fl(2^K / fl(R-L)), is within 1.01 u S + 2^K 2^-22 of the
// exact (k-L) S, S = 2^K/(R-L). A fractional part of t farther than
// m = 8 u scale + 2^K 2^-21 from 0 and 1 therefore puts k strictly between the edges of
// bin floor(t). Returns 1 (guess never trusted) for non-finite or tiny brackets.
__device__ __forceinline__ float bin_margin(float L, float R, float scale, uint32_t nb) {
    const float M = fmaxf(fabsf(L), fabsf(R));
    const int e = (__float_as_int(M) >> 23) & 0xff;
    if (e < 24 || e == 0xff) return 1.0f;
    const float u = __int_as_float((e - 23) << 23);
    return __fadd_ru(__fmul_ru(__fmul_ru(8.0f, u), scale), __fmul_ru((float)nb, 0x1p-21f));
}

// edge_bin() over a table in shared memory, out of line: it runs for a few keys only, and
// the streaming loops that call it stay small enough for the instruction cache.
__device__ __noinline__ int edge_bin_slow(float k, float L, float scale, int top, const float *e) {
    return edge_bin(k, L, scale, top, [&](int j) { return e[j]; });
}

// The scaled guess with no float<->int conversion. For a key whose guess t = (k-L) scale lies
// in [0, 2^11), y = fl(fl(k-L) scale + 2^11) is 2^11 + t rounded to 12 fraction bits, so the
// encoding of y minus that of 2^11 holds the bin above bit 12 and the fraction below it. Its
// error is that of fl(fl(k-L) scale) except the last rounding, 2^-13 bins instead of
// t 2^-24, which the margin taken at 2^11 bins or more (2^-10) covers. The guess is exact
// when its fraction f = i/4096 lies in (m, 1 - m), i.e. i in [mi+1, 4095-mi] with
// mi = floor(4096 m) (4096 m is exact). `base` is the encoding of 2^11 plus mi+1, so the test
// is a subtraction and two unsigned comparisons; a key below L (y under 2^11 or negative),
// at or past R (a bin past the table) or NaN fails it.
static_assert(kMaxBinsLog2 <= 11, "guess_bin holds bins below 2^11");
struct Guess {
    float L, scale;
    uint32_t base, lim, span;
};

__device__ __forceinline__ Guess make_guess(float L, float R, float scale, uint32_t nb) {
    Guess g;
    g.L = L;
    g.scale = scale;
    const float M = __fmul_rn(bin_margin(L, R, scale, max(nb, 2048u)), 4096.0f);
    const uint32_t mi = M < 2048.0f ? (uint32_t)M : 0u;  // M >= 2048 or NaN: accept nothing
    g.base = __float_as_uint(2048.0f) + mi + 1u;
    g.lim = nb << 12;
    g.span = M < 2048.0f ? 4095u - 2u * mi : 0u;
    return g;
}

// The guessed bin of k in *b; true when it is the exact bin (edge_bin's answer).
__device__ __forceinline__ bool guess_bin(const Guess &g, float k, uint32_t *b) {
    const uint32_t e = __float_as_uint(__fmaf_rn(__fsub_rn(k, g.L), g.scale, 2048.0f)) - g.base;
    *b = e >> 12;
    return e < g.lim && (e & 0xfffu) < g.span;
}

// Exact bin of L <= k < R by the edge table e[0..top+1] (in shared memory) for a key the
// scaled guess did not settle: floor(t) of the same guess, then its neighbours (the guess is
// off by at most one bin when the margin lets it be trusted at all: bins are then more than
// 16 ulps wide); a search over the table otherwise (out of line: brackets a few ulps wide).
__device__ __forceinline__ uint32_t near_bin(float k, const Guess &gs, const float *e, uint32_t top) {
    const uint32_t t = __float_as_uint(__fmaf_rn(__fsub_rn(k, gs.L), gs.scale, 2048.0f)) - 0x45000000u;
    const uint32_t g = min(t >> 12, top);  // 0x45000000: the encoding of 2048.0f (t >= 0 for k >= L)
    if (k < e[g]) {
        if (g > 0 && !(k < e[g - 1])) return g - 1;
    } else if (!(k < e[g + 1])) {
        if (g < top && k < e[g + 2]) return g + 1;
    } else {
        return g;
    }
    return (uint32_t)edge_bin_slow(k, gs.L, gs.scale, (int)top, e);
}

// edge_bin() with the guess accepted outright when guess_bin() proves it; L <= k < R.
__device__ __forceinline__ int fast_bin(float k, const Guess &g, int top, const float *e) {
    uint32_t b;
    if (guess_bin(g, k, &b)) return (int)b;
    return edge_bin_slow(k, g.L, g.scale, top, e);
}



// A sparse pass sends its bracket keys to the cell's global bins, or to shared bins first
// when its bracket holds more than kSparseGlobalKeys keys a tile.
constexpr uint32_t kSparseGlobalKeys = 8;
constexpr int kCmpTile = 2048;  // bracket keys a CTA compacts for one cell's run of tiles, or
                                // for one tile of a sampled pass (more: the cell keeps no list)

// The cell a count pass's CTA is working on, in shared memory (thread 0 fills it when the
// CTA's tiles move to a new cell): the rare paths read it there, so the streaming loop keeps
// only what it needs in registers.
constexpr uint32_t kHDense = 1, kHLocal = 2, kHCompact = 4, kHListed = 8, kHPred = 16;
struct HistCell {
    const float *keys;  // the cut axis
    uint32_t *gh;       // the cell's global bins
    float L, R, scale;
    int K;
    uint32_t mode;      // kHDense, kHPred (sampled bracket; kHCompact: its keys to the
                        // list), else sparse (kHLocal: bracket keys to shared bins first;
                        // kHCompact: and to the list), or kHListed
    uint32_t base, end; // the cell's key range [base, end)
    uint32_t t0;        // its first tile
    uint32_t below;     // dense: keys below L met by the exact path
    float pa, pb;       // kHPred: the sampled bracket [e(lo), e(hi)) of the tree over [L, R)
    Guess gs;           // dense and kHPred: the scaled guess
};

// Count pass over a cell whose bracket keys an earlier pass compacted: tile j of the cell's
// t tiles takes the j-th of t equal runs of the list and bins its keys inside [L, R) (the
// keys below L are already counted: resolve carried them). Returns the keys read.
__device__ __noinline__ uint32_t listed_tile(const Level &v, int c, uint32_t local, const HistCell *hc) {
    const float L = hc->L, R = hc->R;
    const int K = hc->K;
    uint32_t *gh = hc->gh;
    const uint32_t cnt = v.cmp_cnt[c];
    // the list split evenly over the cell's tiles, so the CTAs of all of them share it
    const uint32_t tiles = v.tile_off[c + 1] - v.tile_off[c];
    const uint32_t chunk = (cnt + tiles - 1) / tiles;
    const uint32_t lo = local * chunk, hi = min(cnt, lo + chunk);
    const float *list = v.cmp_keys + v.cmp_off[c];
    for (uint32_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const float k = list[i];
        if (k >= L && k < R) atomicAdd(&gh[tree_bin(k, L, R, K)], 1u);
    }
    return hi > lo ? hi - lo : 0u;
}

// Appends the bracket keys a CTA compacted for cell c (*s_ncmp of them in s_cmp) to the cell's
// list and clears the count: one reservation per run of the cell's tiles; an overflow (of the
// buffer or the list) marks the cell as having no list. Returns the keys written. Every
// thread of the CTA calls it once its scans are done.
__device__ __noinline__ uint32_t append_list(const Level &v, int c, const float *s_cmp, uint32_t *s_ncmp,
                                             uint32_t *s_base) {
    __syncthreads();  // every key of the tile kept
    const uint32_t nk = *s_ncmp;
    if (threadIdx.x == 0) {
        const uint32_t cap = v.cmp_off[c + 1] - v.cmp_off[c];
        *s_base = 0xffffffffu;
        if (nk > (uint32_t)kCmpTile) {
            v.cmp_bad[c] = 1;
        } else if (nk) {
            const uint32_t b = atomicAdd(&v.cmp_cnt[c], nk);
            if (b + nk > cap)
                v.cmp_bad[c] = 1;
            else
                *s_base = b;
        }
    }
    __syncthreads();
    const uint32_t b = *s_base;
    if (threadIdx.x == 0) *s_ncmp = 0;
    uint32_t wrote = 0;
    if (b != 0xffffffffu) {
        float *list = v.cmp_keys + v.cmp_off[c] + b;
        for (uint32_t i = threadIdx.x; i < nk; i += blockDim.x) list[i] = s_cmp[i];
        wrote = nk;
    }
    __syncthreads();  // s_cmp and the count are reused by the next tile
    return wrote;
}

// A sparse pass's bracket key (L <= k < R): into the cell's bins (shared when kHLocal) and,
// with kHCompact, into the tile's list buffer.
__device__ __forceinline__ void sparse_key(float k, const HistCell *hc, uint32_t *s_hist, float *s_cmp,
                                        uint32_t *s_ncmp) {
    const uint32_t mode = hc->mode;
    const uint32_t b = (uint32_t)tree_bin(k, hc->L, hc->R, hc->K);
    atomicAdd(mode & kHLocal ? &s_hist[b] : &hc->gh[b], 1u);
    if (mode & kHCompact) {
        const uint32_t i = atomicAdd(s_ncmp, 1u);
        if (i < (uint32_t)kCmpTile) s_cmp[i] = k;
    }
}

// A dense pass's key the scaled guess did not settle: below L counted, inside [L, R) binned
// by the edge table (near_bin), at or past R (or NaN) ignored.
__device__ __forceinline__ void dense_exact(float k, HistCell *hc, uint32_t *s_hist, const float *s_edge) {
    const float L = hc->L, R = hc->R;
    if (k < L)
        atomicAdd(&hc->below, 1u);
    else if (k < R)
        atomicAdd(&s_hist[near_bin(k, hc->gs, s_edge, (1u << hc->K) - 1u)], 1u);
}

// A sampled pass's bracket key (e(lo) <= k < e(hi), inside [L, R)): its bin by the scaled
// guess (the edge table when the guess is not proven) into the shared bins and,
// when the pass compacts, into the tile's list buffer (one shared reservation for the
// threads that arrive together).
__device__ __noinline__ void pred_key(float k, const HistCell *hc, uint32_t *s_hist, float *s_cmp,
                                      uint32_t *s_ncmp, const float *s_edge) {
    uint32_t g;
    if (!guess_bin(hc->gs, k, &g)) g = near_bin(k, hc->gs, s_edge, (1u << hc->K) - 1u);
    atomicAdd(&s_hist[g], 1u);
    if (hc->mode & kHCompact) {
        const uint32_t m = __activemask();
        const uint32_t lane = threadIdx.x & 31u;
        const uint32_t leader = (uint32_t)__ffs(m) - 1u;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(s_ncmp, (uint32_t)__popc(m));
        base = __shfl_sync(m, base, (int)leader);
        const uint32_t i = base + (uint32_t)__popc(m & ((1u << lane) - 1u));
        if (i < (uint32_t)kCmpTile) s_cmp[i] = k;
    }
}

// A compile-time flag passed to a generic lambda.
template <bool B>
struct Flag {
    static constexpr bool value = B;
};

// Keys per thread per round of the histogram pass (float4 loads issued together).
constexpr int kHistVec = 4;

constexpr int kGroup = 4 * kHistVec;  // keys a thread holds per round

// The keys [e0, e1) of one tile (at most kTile keys), visited by the CTA's threads, for a
// pass that leaves a few percent of its keys (the sampled pass). The 16-byte aligned body is
// read in rounds of kHistVec float4 loads a thread (all issued before any key is used); each
// key goes through settle(k), branch-free code for the common case that returns false for a
// key it leaves; a round's left keys are visited right after it through rest(k) (reloaded
// while its lines are still in L1). The unaligned head and tail go through visit(k). `pad`
// fills the missing lanes of the last round: settle(pad) must count nothing (a pad it leaves
// is skipped).
template <uint32_t NT, class Settle, class Rest, class Visit>
__device__ __forceinline__ void scan_tile(const float *keys, uint32_t e0, uint32_t e1, float pad,
                                          Settle settle, Rest rest, Visit visit) {
    const uint32_t ti = threadIdx.x;  // NT = blockDim.x
    const uintptr_t addr = reinterpret_cast<uintptr_t>(keys + e0);
    const uint32_t a0 = min(e1, e0 + (uint32_t)(((16u - (addr & 15u)) & 15u) >> 2));
    for (uint32_t i = e0 + ti; i < a0; i += NT) visit(__ldg(keys + i));
    const uint32_t n4 = (e1 - a0) >> 2;
    const float4 *k4 = reinterpret_cast<const float4 *>(keys + a0);
    const float *kb = keys + a0;
    uint32_t j0 = 0;
    auto round = [&](auto full) {
        float4 q[kHistVec];
#pragma unroll
        for (int u = 0; u < kHistVec; ++u) {
            const uint32_t j = j0 + u * NT + ti;
            if (decltype(full)::value)
                q[u] = __ldg(k4 + j);
            else
                q[u] = j < n4 ? __ldg(k4 + j) : make_float4(pad, pad, pad, pad);
        }
        uint32_t miss = 0;  // bit 4u + c: component c of load u left
#pragma unroll
        for (int u = 0; u < kHistVec; ++u) {
            const float kk[4] = {q[u].x, q[u].y, q[u].z, q[u].w};
#pragma unroll
            for (int c = 0; c < 4; ++c) miss |= (uint32_t)!settle(kk[c]) << (4 * u + c);
        }
        while (miss) {
            const uint32_t b = (uint32_t)__ffs(miss) - 1u;
            miss &= miss - 1u;
            const uint32_t j = j0 + (b >> 2) * NT + ti;
            if (j < n4) rest(__ldg(kb + 4 * j + (b & 3u)));  // else a pad lane
        }
    };
    for (; j0 + kHistVec * NT <= n4; j0 += kHistVec * NT) round(Flag<true>());
    if (j0 < n4) round(Flag<false>());
    for (uint32_t i = a0 + (n4 << 2) + ti; i < e1; i += NT) visit(__ldg(keys + i));
}

// Group visitor that applies a per-key visitor to each key in order.
template <class Visit>
__device__ __forceinline__ auto each(Visit &visit) {
    return [&visit](const float (&k)[kGroup]) {
#pragma unroll
        for (int i = 0; i < kGroup; ++i) visit(k[i]);
    };
}

// Keys [e0, e1) of one axis, visited by `nt` threads (ti = this thread's index): scalar
// head to 16-byte alignment and scalar tail through visit(k), float4 body (kHistVec loads
// in flight a thread) through group(k[kGroup]). `pad` fills the body's missing lanes and
// must be a value the visitors ignore.
// NC: read-only loads (keys not written during the kernel); false: coherent loads, for a
// kernel that moves the keys it reads (k_subtree).
template <bool NC = true, class Visit, class Group>
__device__ __forceinline__ void visit_keys(const float *keys, uint32_t e0, uint32_t e1, float pad,
                                           uint32_t ti, uint32_t nt, Visit visit, Group group) {
    auto ld = [](const float *p) { return NC ? __ldg(p) : *p; };
    auto ld4 = [](const float4 *p) { return NC ? __ldg(p) : *p; };
    const uintptr_t addr = reinterpret_cast<uintptr_t>(keys + e0);
    const uint32_t a0 = min(e1, e0 + (uint32_t)(((16u - (addr & 15u)) & 15u) >> 2));
    for (uint32_t i = e0 + ti; i < a0; i += nt) visit(ld(keys + i));
    const uint32_t n4 = (e1 - a0) >> 2;
    const float4 *k4 = reinterpret_cast<const float4 *>(keys + a0);
    for (uint32_t j0 = 0; j0 < n4; j0 += kHistVec * nt) {
        float4 q[kHistVec];
#pragma unroll
        for (int u = 0; u < kHistVec; ++u) {
            const uint32_t j = j0 + u * nt + ti;
            q[u] = j < n4 ? ld4(k4 + j) : make_float4(pad, pad, pad, pad);
        }
        float k[kGroup];
#pragma unroll
        for (int u = 0; u < kHistVec; ++u) {
            k[4 * u] = q[u].x;
            k[4 * u + 1] = q[u].y;
            k[4 * u + 2] = q[u].z;
            k[4 * u + 3] = q[u].w;
        }
        group(k);
    }
    for (uint32_t i = a0 + (n4 << 2) + ti; i < e1; i += nt) visit(ld(keys + i));
}

// The dense pass's tile [e0, e1) in the first pass of a cold level: every key binned by the
// scaled guess into the CTA's shared bins (a key the guess does not settle counted in the
// lane's spare bin and binned exactly right after its round). Rounds of kHistVec float4
// loads a thread; the unaligned head and tail and a last partial round key by key.
__device__ __forceinline__ void dense_tile(const float *keys, uint32_t e0, uint32_t e1, const Guess gs,
                                           uint32_t *s_hist, HistCell *hc, const float *s_edge) {
    const uint32_t ti = threadIdx.x;
    const uint32_t spare = (gs.lim >> 12) + (ti & 31u);
    auto one = [&](float k) {
        uint32_t g;
        if (guess_bin(gs, k, &g))
            atomicAdd(&s_hist[g], 1u);
        else
            dense_exact(k, hc, s_hist, s_edge);
    };
    const uintptr_t addr = reinterpret_cast<uintptr_t>(keys + e0);
    const uint32_t a0 = min(e1, e0 + (uint32_t)(((16u - (addr & 15u)) & 15u) >> 2));
    for (uint32_t i = e0 + ti; i < a0; i += kThreads) one(__ldg(keys + i));
    const uint32_t n4 = (e1 - a0) >> 2;
    const float4 *k4 = reinterpret_cast<const float4 *>(keys + a0);
    const float *kb = keys + a0;
    uint32_t j0 = 0;
#pragma unroll 1
    for (; j0 + kHistVec * kThreads <= n4; j0 += kHistVec * kThreads) {
        float4 q[kHistVec];
#pragma unroll
        for (int u = 0; u < kHistVec; ++u) q[u] = __ldg(k4 + j0 + u * kThreads + ti);
        uint32_t miss = 0;
#pragma unroll
        for (int u = 0; u < kHistVec; ++u) {
            const float kk[4] = {q[u].x, q[u].y, q[u].z, q[u].w};
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                uint32_t g;
                const bool ok = guess_bin(gs, kk[c], &g);
                atomicAdd(&s_hist[ok ? g : spare], 1u);
                if (!ok) miss |= 1u << (4 * u + c);
            }
        }
        while (miss) {
            const uint32_t b = (uint32_t)__ffs(miss) - 1u;
            miss &= miss - 1u;
            dense_exact(__ldg(kb + 4 * (j0 + (b >> 2) * kThreads + ti) + (b & 3u)), hc, s_hist, s_edge);
        }
    }
    for (uint32_t j = j0 + ti; j < n4; j += kThreads) {
        const float4 q = __ldg(k4 + j);
        one(q.x);
        one(q.y);
        one(q.z);
        one(q.w);
    }
    for (uint32_t i = a0 + (n4 << 2) + ti; i < e1; i += kThreads) one(__ldg(keys + i));
}

// A sparse pass's tile [e0, e1): keys below L counted in `below`, keys inside [L, R) (a few a
// tile) handed to key(k) right after their round, keys at or above R and NaN ignored. Same
// rounds as dense_tile.
template <class Key>
__device__ __forceinline__ void sparse_tile(const float *keys, uint32_t e0, uint32_t e1, float L, float R,
                                            uint32_t &below, Key key) {
    const uint32_t ti = threadIdx.x;
    auto one = [&](float k) {
        if (k < L)
            ++below;
        else if (k < R)
            key(k);
    };
    const uintptr_t addr = reinterpret_cast<uintptr_t>(keys + e0);
    const uint32_t a0 = min(e1, e0 + (uint32_t)(((16u - (addr & 15u)) & 15u) >> 2));
    for (uint32_t i = e0 + ti; i < a0; i += kThreads) one(__ldg(keys + i));
    const uint32_t n4 = (e1 - a0) >> 2;
    const float4 *k4 = reinterpret_cast<const float4 *>(keys + a0);
    const float *kb = keys + a0;
    uint32_t j0 = 0;
#pragma unroll 1
    for (; j0 + kHistVec * kThreads <= n4; j0 += kHistVec * kThreads) {
        float4 q[kHistVec];
#pragma unroll
        for (int u = 0; u < kHistVec; ++u) q[u] = __ldg(k4 + j0 + u * kThreads + ti);
        uint32_t miss = 0;
#pragma unroll
        for (int u = 0; u < kHistVec; ++u) {
            const float kk[4] = {q[u].x, q[u].y, q[u].z, q[u].w};
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                if (kk[c] < L) ++below;
                if (kk[c] >= L && kk[c] < R) miss |= 1u << (4 * u + c);
            }
        }
        while (miss) {
            const uint32_t b = (uint32_t)__ffs(miss) - 1u;
            miss &= miss - 1u;
            key(__ldg(kb + 4 * (j0 + (b >> 2) * kThreads + ti) + (b & 3u)));
        }
    }
    for (uint32_t j = j0 + ti; j < n4; j += kThreads) {
        const float4 q = __ldg(k4 + j);
        one(q.x);
        one(q.y);
        one(q.z);
        one(q.w);
    }
    for (uint32_t i = a0 + (n4 << 2) + ti; i < e1; i += kThreads) one(__ldg(keys + i));
}

// Whether pass v.pass over cell c (`tiles` tiles) is sparse: only the bracket's keys are
// binned, the keys below it counted. The first pass of a cold level is dense for every cell;
// later passes are sparse once the bracket holds at most sparse_per_tile keys a tile.
__device__ __forceinline__ bool sparse_pass(const Level &v, int c, uint32_t tiles) {
    return !(v.pass == 0 && v.warm == nullptr) && v.inb[c] <= v.sparse_per_tile * tiles;
}

// ------------------------------------------------------------------------------------
// Sampled first pass. The first count pass of a cold level bins every key of a cell into
// the 2^K leaves of its midpoint tree. k_sample_bin and k_sample_pick predict from a strided
// sample of the cell
// (one key per 2^kSampleShift) a run of leaves [lo, hi) holding the cut: the sample's
// median +- pred_sigmas standard errors (sqrt(s)/2 sample keys), widened to leaf edges
// a = e(lo), b = e(hi). That pass then counts the keys below a and bins only the keys of
// [a, b). Its replay in k_resolve is the reference loop unchanged once the exact counts
// show count(< a) with difference <= -3 and count(< b) with difference >= 3: every tested
// cut below a then has a count <= count(< a) and moves L, every cut above b has one
// >= count(< b) and moves R (the float test is monotone in the count), and cuts inside
// [a, b] get their exact counts from the bins. Otherwise the pass is discarded and the
// next one bins every key. Same cuts, same integer counts, same iterations either way.
// (k_resolve checks the counts; sample sizes and widths only change the speed.)
// ------------------------------------------------------------------------------------
constexpr uint32_t kPredValid = 1u << 25, kPredCompact = 1u << 24;
__device__ __forceinline__ uint32_t pred_lo(uint32_t p) { return p & 0xfffu; }
__device__ __forceinline__ uint32_t pred_hi(uint32_t p) { return (p >> 12) & 0xfffu; }
constexpr int kSampleThreads = 256;
constexpr int kSampleShift = 8;              // one sample key per 256 keys of the cell
constexpr uint32_t kSampleMax = 16384;       // sample keys per cell at most
constexpr uint32_t kSampleMin = 1024;        // fewer: no prediction (a dense first pass)
constexpr uint32_t kSamplePerCta = 4 * kSampleThreads;
constexpr float kPredCompactShare = 0.09f;   // compact the bracket keys when the sample puts
                                             // at most this share of the cell inside it
static_assert(kPredCompactShare * kTile * 1.25f < kCmpTile, "a tile's bracket keys fit the buffer");

__device__ __forceinline__ uint32_t sample_count(uint32_t n) {
    const uint32_t ns = min(n >> kSampleShift, kSampleMax);
    return ns >= kSampleMin ? ns : 0u;
}

// Sample binning: CTA (x, y) takes samples [x kSamplePerCta, (x+1) kSamplePerCta) of the
// cells y, y + gridDim.y, ...; sample j of a cell of n keys is the key at position
// ((2j+1) n / (2 ns)) (fixed point), binned into the cell's histogram bins (all zero
// between passes) by the scaled guess or the descent; samples below L are counted in
// pred[c], which k_sample_pick then replaces by the prediction.
__global__ void __launch_bounds__(kSampleThreads) k_sample_bin(Level v) {
    pdl_enter();
    if (v.skip && *(volatile const uint32_t *)v.skip) return;  // subtrees took this level
    const uint32_t ti = threadIdx.x;
    for (int c = blockIdx.y; c < v.C; c += gridDim.y) {
        if (v.state[c] != kActive) continue;
        const int slot = level_slot(v, c);
        const uint2 rg = v.ranges[slot];
        const uint32_t n = rg.y - rg.x;
        const uint32_t ns = sample_count(n);
        const uint32_t j0 = blockIdx.x * kSamplePerCta;
        if (j0 >= ns) continue;
        const orb_cell_t &cell = v.heap[slot];
        const float L = cell.cutMarginLeft, R = cell.cutMarginRight;
        const int K = v.hist_k[c];
        const uint32_t nb = 1u << K;
        const float *keys = axis_keys(v, eff_axis(cell.cutAxis)) + rg.x;
        uint32_t *gh = v.hist + v.hist_off[c];
        // (2j+1) step >> 17 < n for j < ns: step = floor(n 2^16 / ns) < 2^37, products < 2^52
        const uint64_t step = ((uint64_t)n << 16) / ns;
        float k[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint32_t j = j0 + u * kSampleThreads + ti;
            k[u] = j < ns ? __ldg(keys + (uint32_t)(((2ull * j + 1ull) * step) >> 17)) : R;
        }
        const float scale = __fdiv_rn((float)nb, __fsub_rn(R, L));
        const Guess gs = make_guess(L, R, scale, nb);
        uint32_t below = 0;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (k[u] < L) {
                ++below;
            } else if (k[u] < R) {
                uint32_t g;
                if (!guess_bin(gs, k[u], &g)) g = (uint32_t)tree_bin(k[u], L, R, K);
                atomicAdd(&gh[g], 1u);
            }
        }
        below = warp_sum(below);
        if ((ti & 31u) == 0 && below) atomicAdd(&v.pred[c], below);
        if (ti == 0) add_bytes(v, kKSample, 4ull * min(kSamplePerCta, ns - j0));
    }
}

// One CTA per sampled cell (cells y, y + gridDim.x, ...): the leaves [lo, hi) around the
// sample median (+- pred_sigmas standard errors), packed into pred[c]; the bins are cleared
// again. Each thread holds 8 consecutive bins in registers.
constexpr int kPickThreads = 256;
static_assert((1 << kMaxBinsLog2) == 8 * kPickThreads, "8 bins a thread");
__global__ void __launch_bounds__(kPickThreads) k_sample_pick(Level v) {
    pdl_enter();
    if (v.skip && *(volatile const uint32_t *)v.skip) return;  // subtrees took this level
    __shared__ uint32_t s_red[72];
    const uint32_t ti = threadIdx.x;
    for (int c = blockIdx.x; c < v.C; c += gridDim.x) {
        if (v.state[c] != kActive) continue;
        const uint2 rg = v.ranges[level_slot(v, c)];
        const uint32_t ns = sample_count(rg.y - rg.x);
        if (!ns) continue;
        const uint32_t nb = 1u << v.hist_k[c];
        uint4 *gh4 = reinterpret_cast<uint4 *>(v.hist + v.hist_off[c]);
        const uint32_t below = v.pred[c];  // samples below L
        // thread t owns leaves [8t, 8t + 8) (none past nb)
        uint32_t h[8];
        if (8 * ti < nb) {
            const uint4 a = gh4[2 * ti], b = gh4[2 * ti + 1];
            h[0] = a.x; h[1] = a.y; h[2] = a.z; h[3] = a.w;
            h[4] = b.x; h[5] = b.y; h[6] = b.z; h[7] = b.w;
            gh4[2 * ti] = make_uint4(0u, 0u, 0u, 0u);
            gh4[2 * ti + 1] = make_uint4(0u, 0u, 0u, 0u);
        } else {
#pragma unroll
            for (int i = 0; i < 8; ++i) h[i] = 0u;
        }
        uint32_t run = 0;
#pragma unroll
        for (int i = 0; i < 8; ++i) run += h[i];
        uint32_t total, unused;
        const uint32_t pre = block_excl_scan2(run, 0u, s_red, &total, &unused).x;
        const float half = 0.5f * (float)ns, w = v.pred_sigmas * 0.5f * sqrtf((float)ns);
        const float r_lo = half - w, r_hi = half + w;
        // cum(j) = samples below edge e(j) = below + bins [0, j); count the edges j in [0, nb]
        // with cum(j) <= r_lo and with cum(j) < r_hi
        uint32_t n_le = 0, n_lt = 0, cum = below + pre;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const bool own = 8 * ti + i < nb;
            n_le += own && (float)cum <= r_lo;
            n_lt += own && (float)cum < r_hi;
            cum += h[i];
        }
        if (ti == 0) {
            n_le += (float)(below + total) <= r_lo;
            n_lt += (float)(below + total) < r_hi;
        }
        n_le = block_sum(n_le, s_red);
        n_lt = block_sum(n_lt, s_red);
        // lo: the last edge with at most r_lo samples below it; hi: the first with at least r_hi
        const uint32_t lo = n_le ? n_le - 1u : 0u, hi = min(n_lt, nb);
        uint32_t ca = 0, cb = 0;
        cum = below + pre;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            if (8 * ti + i == lo) ca = cum;
            if (8 * ti + i == hi) cb = cum;
            cum += h[i];
        }
        ca = block_sum(ca, s_red);
        cb = hi == nb ? below + total : block_sum(cb, s_red);
        if (ti == 0) {
            uint32_t p = 0u;
            if (n_le > 0 && lo < hi && (lo > 0 || hi < nb)) {
                const float share = (float)(cb - ca) / (float)ns;
                p = lo | (hi << 12) | kPredValid | (share <= kPredCompactShare ? kPredCompact : 0u);
                atomicAdd(&v.counters->pred_cells, 1u);
            }
            v.pred[c] = p;
        }
        __syncthreads();  // s_red reused by the next cell
    }
}

// One count-left pass over the tiles of the level's active cells (cells of more than one
// tile), a tile loop over all CTAs. Dense cells are binned into a shared-memory histogram
// added to the cell's global bins; sparse cells (few keys in the bracket, known from the
// previous pass) count the keys below the bracket and send the bracket's keys to the global
// bins (to shared bins first when there are more than a few a tile). Each CTA takes a run of
// consecutive tiles (runs of equal length to one tile); a cell's shared bins, count below
// and compacted keys stay with the CTA while its tiles follow one another and are added to
// the global ones once per run.
// Allowed: the modes this instance handles (the other paths are compiled out, which keeps
// each instance's streaming loop within its registers): kHFirstDense, the first pass of a
// cold level without sampled brackets (every cell dense); kHFirstSampled, the first pass of
// a sampled level (sampled or dense cells); kHRest, every other pass.
constexpr uint32_t kHSparse = 32;  // (allowed only) the sparse modes
constexpr uint32_t kHFirstDense = kHDense;
constexpr uint32_t kHFirstSampled = kHDense | kHPred | kHCompact;
constexpr uint32_t kHRest = kHDense | kHLocal | kHCompact | kHListed | kHSparse;
template <uint32_t Allowed>
__global__ void __launch_bounds__(kThreads, kHistBlocksPerSm) k_hist(Level v) {
    pdl_enter();
    if (v.skip && *(volatile const uint32_t *)v.skip) return;  // subtrees took this level
    constexpr bool kAny = Allowed != kHDense;
    __shared__ uint32_t s_hist[(1 << kMaxBinsLog2) + 32];  // + the dense loop's spare bins
    __shared__ float s_edge[(1 << kMaxBinsLog2) + 1];      // dense and sampled: the tree's edges
    __shared__ uint32_t s_red[32];
    __shared__ float s_cmp[(Allowed & kHCompact) ? kCmpTile : 1];  // bracket keys on their way to the list
    __shared__ uint32_t s_ncmp, s_base;
    __shared__ HistCell s_hc;
    __shared__ uint32_t s_run[2];           // the CTA's tiles [first, end)
    __shared__ unsigned long long s_bytes;  // thread 0's count of bytes read
    if (blockIdx.x == 0 && threadIdx.x == 0) v.counters->any_active[v.pass & 1] = 0u;
    // every cell of the level finished in an earlier pass: nothing to bin
    if (v.pass > 0 && *(volatile uint32_t *)&v.counters->any_active[(v.pass - 1) & 1] == 0u) return;
    if (threadIdx.x == 0) {
        const uint64_t total = v.tile_off[v.C];
        s_run[0] = (uint32_t)(total * blockIdx.x / gridDim.x);
        s_run[1] = (uint32_t)(total * (blockIdx.x + 1) / gridDim.x);
        s_bytes = 0;
        s_ncmp = 0;
    }
    __syncthreads();
    int cur = -1;        // the cell s_hc describes (every thread follows it)
    uint32_t below = 0;  // sparse: this thread's keys below L in the cell's tiles so far
    // the current cell's count below L and its shared bins to the global ones
    auto end_cell = [&]() {
        below = block_sum(below, s_red);
        const uint32_t mode = s_hc.mode;
        if (threadIdx.x == 0) {
            const uint32_t tot = below + s_hc.below;
            if (tot) atomicAdd(&v.below[cur], tot);
        }
        if (mode & (kHDense | kHLocal | kHPred)) {
            const uint32_t nb = 1u << s_hc.K;
            uint32_t *gh = s_hc.gh;
            for (uint32_t b = threadIdx.x; b < nb; b += kThreads) {
                const uint32_t h = s_hist[b];
                if (h) atomicAdd(&gh[b], h);
            }
        }
        if ((Allowed & kHCompact) && (mode & kHCompact)) {
            const uint32_t wrote = append_list(v, cur, s_cmp, &s_ncmp, &s_base);
            if (threadIdx.x == 0) s_bytes += 4ull * wrote;
        }
        __syncthreads();  // s_hc and s_hist free for the next cell
        below = 0;
    };
    const uint32_t t_end = s_run[1];
    auto tile_cell = [&](uint32_t t) {
        return t < t_end ? (v.htile_cell ? (int)v.htile_cell[t] : find_cell(v.tile_off, v.C, t)) : -1;
    };
    int c_next = tile_cell(s_run[0]);
    int skip_c = -1;  // an inactive cell whose tiles are being passed over
    for (uint32_t t = s_run[0]; t < t_end; ++t) {
        const int c = c_next;
        c_next = tile_cell(t + 1);  // the next tile's cell, loaded while this tile is read
        if (c == skip_c) continue;
        if (c != cur) {
            if (v.state[c] != kActive) {  // the run's tiles of a cell are consecutive
                skip_c = c;
                continue;
            }
            if (cur >= 0) end_cell();
            cur = c;
            if (threadIdx.x == 0) {
                const int slot = level_slot(v, c);
                const orb_cell_t &cell = v.heap[slot];
                const uint2 rg = v.ranges[slot];
                const uint32_t t0 = v.tile_off[c], tiles = v.tile_off[c + 1] - t0;
                const float L = cell.cutMarginLeft, R = cell.cutMarginRight;
                const int K = v.hist_k[c];
                const uint32_t nb = 1u << K;
                const float scale = __fdiv_rn((float)nb, __fsub_rn(R, L));
                uint32_t mode;
                const uint32_t pr = (Allowed & kHPred) && v.pass == 0 && v.pred ? v.pred[c] : 0u;
                if (!kAny)
                    mode = kHDense;  // a cold first pass without sampled brackets
                else if ((Allowed & kHListed) && v.listed[c])
                    mode = kHListed;
                else if (pr & kPredValid)
                    mode = kHPred | (pr & kPredCompact ? kHCompact : 0u);
                else if (!sparse_pass(v, c, tiles))
                    mode = kHDense;
                else
                    // more than a few bracket keys a tile: shared bins first; more than a few a
                    // bin after this pass (a further pass follows): compacted into the list
                    mode = (v.inb[c] > kSparseGlobalKeys * tiles ? kHLocal : 0u) |
                           (v.inb[c] > (8u << K) ? kHCompact : 0u);
                s_hc.keys = axis_keys(v, eff_axis(cell.cutAxis));
                s_hc.gh = v.hist + v.hist_off[c];
                s_hc.L = L;
                s_hc.R = R;
                s_hc.scale = scale;
                s_hc.K = K;
                s_hc.mode = mode;
                s_hc.base = rg.x;
                s_hc.end = rg.y;
                s_hc.t0 = t0;
                s_hc.below = 0;
                s_hc.pa = pr & kPredValid ? tree_edge(L, R, K, pred_lo(pr)) : L;
                s_hc.pb = pr & kPredValid ? tree_edge(L, R, K, pred_hi(pr)) : R;
                s_hc.gs = make_guess(L, R, scale, nb);
            }
            __syncthreads();
            if (s_hc.mode & (kHDense | kHLocal | kHPred)) {
                for (uint32_t j = threadIdx.x; j < (1u << s_hc.K); j += kThreads) s_hist[j] = 0u;
                if (s_hc.mode & (kHDense | kHPred))
                    fill_edges(s_edge, s_hc.L, s_hc.R, s_hc.K, threadIdx.x, kThreads);
                __syncthreads();
            }
        }
        const uint32_t local = t - s_hc.t0;
        const uint32_t mode = s_hc.mode;
        if ((Allowed & kHListed) && (mode & kHListed)) {
            const uint32_t nread = listed_tile(v, c, local, &s_hc);
            if (threadIdx.x == 0) s_bytes += 4ull * nread;
            continue;
        }
        const uint32_t e0 = s_hc.base + local * (uint32_t)kTile;
        const uint32_t e1 = min(s_hc.end, e0 + (uint32_t)kTile);
        const float *keys = s_hc.keys;
        if ((Allowed & kHPred) && (mode & kHPred)) {
            // sampled bracket [pa, pb): keys below it counted, keys inside it (a few percent)
            // binned afterwards (and compacted, the list flushed after every tile so the
            // buffer holds one tile's keys), keys above it and NaN ignored
            const float pa = s_hc.pa, pb = s_hc.pb;
            auto key = [&](float k) { pred_key(k, &s_hc, s_hist, s_cmp, &s_ncmp, s_edge); };
            scan_tile<kThreads>(
                keys, e0, e1, s_hc.R,
                [&](float k) {
                    below += k < pa;
                    return !(k >= pa && k < pb);
                },
                key,
                [&](float k) {
                    if (k < pa)
                        ++below;
                    else if (k < pb)
                        key(k);
                });
            if (mode & kHCompact) {
                const uint32_t wrote = append_list(v, c, s_cmp, &s_ncmp, &s_base);
                if (threadIdx.x == 0) s_bytes += 4ull * wrote;
            }
        } else if (!kAny || (mode & kHDense)) {
            // every key by the scaled guess (no range test: guess_bin fails keys outside
            // [L, R) and NaN, which dense_exact then counts or ignores)
            dense_tile(keys, e0, e1, s_hc.gs, s_hist, &s_hc, s_edge);
        } else if (Allowed & kHSparse) {
            // keys below L counted, keys in [L, R) (few) binned after their round
            sparse_tile(keys, e0, e1, s_hc.L, s_hc.R, below,
                        [&](float k) { sparse_key(k, &s_hc, s_hist, s_cmp, &s_ncmp); });
        }
        if (threadIdx.x == 0) s_bytes += 4ull * (e1 - e0);
    }
    if (cur >= 0) end_cell();
    if (threadIdx.x == 0 && s_bytes) add_bytes(v, kKHist, s_bytes);
}

// ------------------------------------------------------------------------------------
// Bisection of one-tile cells (kWarpKeys < n <= kTile keys): one warp per cell, the whole
// reference loop (src/orbit.cpp:146-232) in one launch. Histogram rounds over the midpoint
// tree of the current bracket (about 16 keys a bin, warp-private shared-memory bins) each
// replay up to K iterations on the prefix counts; once the bracket holds at most
// kListKeys keys they are gathered into registers and every remaining iteration is a
// register count plus a warp sum. Every round streams the cell's keys (L2-resident after
// the first).
// ------------------------------------------------------------------------------------
constexpr int kWarpKeysPerLane = kWarpKeys / 32;

// Bisection of a small cell (at most kWarpKeys keys) by one warp: the keys held in registers,
// every iteration of the reference loop (src/orbit.cpp:146-232) a register count plus a
// warp reduction.
__device__ __forceinline__ void bisect_small(const Level &v, int c, uint32_t lane) {
    const int slot = level_slot(v, c);
    orb_cell_t &cell = v.heap[slot];
    const uint2 rg = v.ranges[slot];
    const uint32_t n = rg.y - rg.x;
    const float ratio = leaf_ratio(cell.nLeafCells);  // src/orbit.cpp:204
    const float *keys = axis_keys(v, eff_axis(cell.cutAxis));
    float k[kWarpKeysPerLane];
#pragma unroll
    for (int j = 0; j < kWarpKeysPerLane; ++j) {
        const uint32_t i = (uint32_t)(j * 32 + lane);
        k[j] = i < n ? __ldg(keys + rg.x + i) : __int_as_float(0x7fc00000);  // NaN: never below
    }
    float L = cell.cutMarginLeft, R = cell.cutMarginRight;
    if (v.warm && v.warm[c]) {
        // hinted bracket: keep it only if it holds the target
        uint32_t bl = 0, br = 0;
#pragma unroll
        for (int j = 0; j < kWarpKeysPerLane; ++j) {
            bl += k[j] < L;
            br += k[j] < R;
        }
        if (!warm_bracket_holds(warp_sum(bl), warp_sum(br), n, ratio)) {
            const int a = eff_axis(cell.cutAxis);
            L = cell.lower[a];
            R = cell.upper[a];
            if (lane == 0) atomicAdd(&v.counters->warm_resets, 1u);
        }
        if (lane == 0) v.warm[c] = 0;
    }
    uint32_t it = 0;
    uint8_t st = kActive;
    while (st == kActive) {
        if (it >= (uint32_t)kMaxIterations) {
            st = kCapped;
            break;
        }
        const float cut = mid_cut(L, R);
        uint32_t cnt = 0;
#pragma unroll
        for (int j = 0; j < kWarpKeysPerLane; ++j) cnt += k[j] < cut;
        cnt = warp_sum(cnt);
        ++it;
        const int dir = convergence(cnt, n, ratio);
        if (dir == 0)
            st = kFound;
        else if (dir > 0)
            R = cut;
        else
            L = cut;
    }
    if (lane == 0) {
        cell.cutMarginLeft = L;
        cell.cutMarginRight = R;
        cell.foundCut = st == kFound ? 1 : 0;
        v.iters[c] = (uint8_t)it;
        v.state[c] = st;
        atomicMax(&v.counters->max_iters, it);
        if (st == kCapped) atomicAdd(&v.counters->unfound, 1u);
        add_bytes(v, kKBisectTile, 4ull * n);  // the launch that bisects it
    }
}

constexpr int kTileBinsLog2 = 9;
constexpr int kTileBins = 1 << kTileBinsLog2;
constexpr int kListPerLane = 8;     // bracket keys a lane can hold
constexpr uint32_t kListKeys = 64;  // bracket size that switches to the register list

__global__ void __launch_bounds__(kThreads, kTileBlocksPerSm) k_bisect_tile(Level v) {
    pdl_enter();
    if (v.skip && *(volatile const uint32_t *)v.skip) return;  // subtrees took this level
    __shared__ uint32_t s_bins[kThreads / 32][kTileBins];
    __shared__ float s_edges[kThreads / 32][kTileBins + 1];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t *bins = s_bins[warp];
    float *edges = s_edges[warp];
    const int nwarps = (int)(gridDim.x * (blockDim.x >> 5));
    unsigned long long bytes = 0;
    for (int c = (int)(blockIdx.x * (blockDim.x >> 5) + warp); c < v.C; c += nwarps) {
        const uint8_t state = v.state[c];
        if (state == kSmall) {
            bisect_small(v, c, lane);
            continue;
        }
        if (state != kOneTile) continue;
        const int slot = level_slot(v, c);
        orb_cell_t &cell = v.heap[slot];
        const uint2 rg = v.ranges[slot];
        const uint32_t n = rg.y - rg.x;
        const float ratio = leaf_ratio(cell.nLeafCells);  // src/orbit.cpp:204
        const float *keys = axis_keys(v, eff_axis(cell.cutAxis));
        float L = cell.cutMarginLeft, R = cell.cutMarginRight;
        uint32_t it = 0, cand = n;
        int st = kActive;
        bool warm = v.warm && v.warm[c];  // hinted bracket, checked by the first round
        while (st == kActive) {
            bytes += 4ull * n;
            if (cand <= kListKeys) {
                // the bracket's keys into registers (each lane keeps its own), keys below L
                float kl[kListPerLane];
                uint32_t nk = 0, below = 0;
                bool over = false;
                auto gather = [&](float k) {
                    if (k < L) {
                        ++below;
                    } else if (k < R) {
                        if (nk < (uint32_t)kListPerLane) {
#pragma unroll
                            for (int q = 0; q < kListPerLane; ++q)
                                if (q == (int)nk) kl[q] = k;
                        } else {
                            over = true;
                        }
                        ++nk;
                    }
                };
                visit_keys(keys, rg.x, rg.y, R, lane, 32, gather, each(gather));
                if (!__any_sync(0xffffffffu, over)) {
                    below = warp_sum(below);
                    while (st == kActive) {
                        if (it >= (uint32_t)kMaxIterations) {
                            st = kCapped;
                            break;
                        }
                        const float cut = mid_cut(L, R);
                        uint32_t cnt = 0;
#pragma unroll
                        for (int q = 0; q < kListPerLane; ++q) cnt += (q < (int)nk) && kl[q] < cut;
                        const uint32_t cl = below + warp_sum(cnt);
                        ++it;
                        const int dir = convergence(cl, n, ratio);
                        if (dir == 0)
                            st = kFound;
                        else if (dir > 0)
                            R = cut;
                        else
                            L = cut;
                    }
                    break;
                }
                // a lane met more than it can hold: one more histogram round instead
            }
            const int K = max(1, min(kTileBinsLog2, 28 - __clz(max(cand, 1u))));
            const uint32_t nb = 1u << K;
            for (uint32_t j = lane; j < nb; j += 32) bins[j] = 0u;
            fill_edges(edges, L, R, K, lane, 32);
            __syncwarp();
            const float scale = __fdiv_rn((float)nb, __fsub_rn(R, L));
            const Guess gs = make_guess(L, R, scale, nb);
            const int top = (int)nb - 1;
            uint32_t below = 0;
            auto one = [&](float k) {
                if (k < L)
                    ++below;
                else if (k < R)
                    atomicAdd(&bins[fast_bin(k, gs, top, edges)], 1u);
            };
            visit_keys(keys, rg.x, rg.y, R, lane, 32, one, each(one));
            __syncwarp();
            below = warp_sum(below);
            // exclusive prefix of the bins in place (each lane its own run of bins)
            const uint32_t per = max(1u, nb >> 5), j0 = lane * per, j1 = min(nb, j0 + per);
            uint32_t loc = 0;
            for (uint32_t j = j0; j < j1; ++j) loc += bins[j];
            uint32_t tot;
            uint32_t run = warp_excl_scan(loc, &tot);
            for (uint32_t j = j0; j < j1; ++j) {
                const uint32_t h = bins[j];
                bins[j] = run;
                run += h;
            }
            __syncwarp();
            if (warm) {
                warm = false;
                if (!warm_bracket_holds(below, below + tot, n, ratio)) {  // restart on the extent
                    const int a = eff_axis(cell.cutAxis);
                    L = cell.lower[a];
                    R = cell.upper[a];
                    cand = n;
                    if (lane == 0) atomicAdd(&v.counters->warm_resets, 1u);
                    __syncwarp();
                    continue;
                }
            }
            // replay up to K iterations (identically in every lane)
            uint32_t pos = 0, width = nb;
            for (int step = 0; step < K; ++step) {
                if (it >= (uint32_t)kMaxIterations) {
                    st = kCapped;
                    break;
                }
                const uint32_t half = width >> 1;
                const uint32_t cl = below + bins[pos + half];
                ++it;
                const int dir = convergence(cl, n, ratio);
                if (dir == 0) {
                    st = kFound;
                    break;
                }
                const float cut = mid_cut(L, R);
                if (dir > 0) {
                    R = cut;
                } else {
                    L = cut;
                    pos += half;
                }
                width = half;
            }
            if (st == kActive && it >= (uint32_t)kMaxIterations) st = kCapped;
            if (st == kActive) cand = (pos + 1 < nb ? bins[pos + 1] : tot) - bins[pos];
            __syncwarp();  // the bins are rewritten by the next round
        }
        if (lane == 0) {
            cell.cutMarginLeft = L;
            cell.cutMarginRight = R;
            cell.foundCut = st == kFound ? 1 : 0;
            v.iters[c] = (uint8_t)it;
            v.state[c] = (uint8_t)st;
            if (v.warm) v.warm[c] = 0;
            atomicMax(&v.counters->max_iters, it);
            if (st == kCapped) atomicAdd(&v.counters->unfound, 1u);
        }
    }
    if (lane == 0 && bytes) add_bytes(v, kKBisectTile, bytes);
}

// ------------------------------------------------------------------------------------
// Resolve: replay up to K bisection iterations per cell on its histogram (warp per cell).
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_resolve(Level v) {
    pdl_enter();
    if (v.skip && *(volatile const uint32_t *)v.skip) return;  // subtrees took this level
    const int c = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (c >= v.C) return;
    if (v.state[c] != kActive) return;
    const int slot = level_slot(v, c);
    orb_cell_t &cell = v.heap[slot];
    const uint2 rg = v.ranges[slot];
    const uint32_t n = rg.y - rg.x;
    const float ratio = leaf_ratio(cell.nLeafCells);  // src/orbit.cpp:204
    const int K = v.hist_k[c];
    uint32_t *g = v.hist + v.hist_off[c];
    float L = cell.cutMarginLeft, R = cell.cutMarginRight;
    uint32_t it = v.iters[c];
    uint32_t prefix = v.below[c];
    uint32_t pos = 0, width = 1u << K;
    uint8_t st = kActive;
    // The replay reads the bins through two loads: lane l first sums its run of 2^K/32 bins
    // (the steps whose halves span whole runs add up lanes), then, once a half lies inside
    // one run, the lanes hold that run's bins two each. No other step waits on memory.
    const uint32_t RUN = max((1u << K) >> 5, 1u);  // bins a lane's run covers (K = 4: lanes
                                                    // 16.. hold none)
    uint32_t run_sum = 0;
    if (RUN >= 4) {
        const uint4 *g4 = reinterpret_cast<const uint4 *>(g + lane * RUN);
#pragma unroll 4
        for (uint32_t j = 0; j < RUN / 4; ++j) {
            const uint4 w = g4[j];
            run_sum += w.x + w.y + w.z + w.w;
        }
    } else {
        for (uint32_t j = 0; j < RUN; ++j)
            if (lane * RUN + j < (1u << K)) run_sum += g[lane * RUN + j];
    }
    uint32_t q = 0xffffffffu;  // the run whose bins the lanes hold
    uint2 pair = make_uint2(0u, 0u);
    // bins [a, a + w) summed over the warp (a multiple of w, w a power of two)
    auto sum_bins = [&](uint32_t a, uint32_t w) -> uint32_t {
        if (w >= RUN) {
            const uint32_t l0 = a / RUN, l1 = (a + w) / RUN;
            return warp_sum(lane >= l0 && lane < l1 ? run_sum : 0u);
        }
        const uint32_t r = a / RUN;
        if (r != q) {
            q = r;
            const uint32_t b0 = r * RUN + 2 * lane;
            pair.x = 2 * lane < RUN ? g[b0] : 0u;
            pair.y = 2 * lane + 1 < RUN ? g[b0 + 1] : 0u;
        }
        const uint32_t b0 = q * RUN + 2 * lane;
        return warp_sum((b0 >= a && b0 < a + w ? pair.x : 0u) + (b0 + 1 >= a && b0 + 1 < a + w ? pair.y : 0u));
    };
    uint32_t first_half = 0xffffffffu;  // bins below the first cut, when already summed
    const uint32_t pr = v.pass == 0 && v.pred ? v.pred[c] : 0u;
    if (pr & kPredValid) {
        // sampled pass: prefix = keys below e(lo), the bins hold the keys of [e(lo), e(hi));
        // the replay below is exact when the cut lies between them (see k_sample_bin)
        const uint32_t tot = sum_bins(0, 1u << K);
        const bool holds = convergence(prefix, n, ratio) < 0 && convergence(prefix + tot, n, ratio) > 0;
        __syncwarp();
        if (!holds) {
            for (uint32_t b = lane; b < (1u << K); b += 32) g[b] = 0u;
            if (lane == 0) {
                v.inb[c] = n;  // the next pass bins every key (dense)
                v.below[c] = 0;
                v.listed[c] = 0;
                v.cmp_cnt[c] = 0;
                v.cmp_bad[c] = 0;
                v.counters->any_active[v.pass & 1] = 1u;
                atomicAdd(&v.counters->pred_misses, 1u);
                add_bytes(v, kKResolve, 8ull << K);
            }
            return;
        }
    }
    if (v.warm && v.warm[c]) {
        // first pass of a hinted bracket: check it holds the target before replaying (the
        // total and the first step's count)
        const uint32_t h0 = 1u << (K - 1);
        const uint32_t lo = sum_bins(0, h0), hi = sum_bins(h0, h0);
        first_half = lo;
        const bool holds = warm_bracket_holds(prefix, prefix + lo + hi, n, ratio);
        __syncwarp();
        if (!holds) {
            for (uint32_t b = lane; b < (1u << K); b += 32) g[b] = 0u;
            if (lane == 0) {
                warm_reset(cell, L, R, v.counters);
                v.warm[c] = 0;
                v.inb[c] = n;
                v.below[c] = 0;
                v.listed[c] = 0;
                v.cmp_cnt[c] = 0;
                v.cmp_bad[c] = 0;
                v.counters->any_active[v.pass & 1] = 1u;
            }
            return;  // the next pass bins the whole extent
        }
        if (lane == 0) v.warm[c] = 0;
    }
    for (int step = 0; step < K; ++step) {
        if (it >= (uint32_t)kMaxIterations) {
            st = kCapped;
            break;
        }
        const uint32_t half = width >> 1;
        const uint32_t sum = step == 0 && first_half != 0xffffffffu ? first_half : sum_bins(pos, half);
        const uint32_t cl = prefix + sum;
        ++it;
        const int dir = convergence(cl, n, ratio);
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
    const uint32_t next_inb = sum_bins(pos, 1);  // keys in the bracket the next pass would bin
    // the next pass reads the cell's list when this pass read one or wrote a complete one
    // (a sparse pass compacts its bracket keys); then the keys below the new L are known
    const uint32_t tiles = v.tile_off[c + 1] - v.tile_off[c];
    const bool compacted = pr & kPredValid ? (pr & kPredCompact) != 0
                                           : sparse_pass(v, c, tiles) && v.inb[c] > (8u << K);
    const bool list_next = v.listed[c] || (compacted && !v.cmp_bad[c]);
    __syncwarp();
    for (uint32_t b = lane; b < (1u << K); b += 32) g[b] = 0u;
    if (st == kActive && lane == 0) {
        v.inb[c] = next_inb;
        v.listed[c] = list_next ? 1 : 0;
    }
    if (lane == 0) {
        add_bytes(v, kKResolve, 8ull << K);  // bins read and cleared
        cell.cutMarginLeft = L;
        cell.cutMarginRight = R;
        cell.foundCut = st == kFound ? 1 : 0;
        v.iters[c] = (uint8_t)it;
        v.state[c] = st;
        v.below[c] = st == kActive && list_next ? prefix : 0u;
        atomicMax(&v.counters->max_iters, it);
        if (st == kCapped) atomicAdd(&v.counters->unfound, 1u);
        if (st == kActive) {
            v.counters->any_active[v.pass & 1] = 1u;
            // the last pass leaves no cell active (tree depth 11): flag it if one does
            if (v.pass == v.last_pass) atomicExch(&v.counters->error, 1u);
        }
    }
}



// ------------------------------------------------------------------------------------
// Bisection with one CTA per cell, for levels with many cells (no multi-CTA passes, no
// global histograms, no host round trip). Every round bins the candidate keys of the cell
// into a shared-memory midpoint tree and replays up to K iterations of the reference loop
// (src/orbit.cpp:146-232) on it; then the keys of the remaining bracket become the
// candidates of the next round. Candidates start as the cell's keys in global memory, or
// in the shared list when they fit; as soon as the bracket fits the list it is compacted
// into it. `base` counts the keys already known to lie below L. Same cuts, same integer
// counts, same float test as the reference.
// ------------------------------------------------------------------------------------
constexpr int kCtaThreads = 512;
constexpr uint32_t kListCap = 8192;                     // shared list of candidate keys
constexpr uint32_t kListPerThread = kListCap / kCtaThreads;
constexpr size_t kCtaSmemBytes = kListCap * sizeof(float) +
                                 (1u << kMaxBinsLog2) * sizeof(uint32_t) +
                                 ((1u << kMaxBinsLog2) + 1) * sizeof(float);

__global__ void __launch_bounds__(kCtaThreads) k_bisect_cta(Level v) {
    pdl_enter();
    if (v.skip && *(volatile const uint32_t *)v.skip) return;  // subtrees took this level
    extern __shared__ __align__(16) unsigned char cta_smem[];
    float *list = reinterpret_cast<float *>(cta_smem);
    uint32_t *s_hist = reinterpret_cast<uint32_t *>(list + kListCap);
    float *s_edge = reinterpret_cast<float *>(s_hist + (1u << kMaxBinsLog2));
    __shared__ uint32_t sh[96];
    __shared__ uint32_t s_fill;
    const uint32_t tid = threadIdx.x;
    constexpr uint32_t kBins = 1u << kMaxBinsLog2;
    for (int c = blockIdx.x; c < v.C; c += gridDim.x) {
        const int slot = level_slot(v, c);
        orb_cell_t &cell = v.heap[slot];
        const uint2 rg = v.ranges[slot];
        const uint32_t n = rg.y - rg.x;
        const float ratio = leaf_ratio(cell.nLeafCells);  // src/orbit.cpp:204
        const float *keys = axis_keys(v, eff_axis(cell.cutAxis));
        float L = cell.cutMarginLeft, R = cell.cutMarginRight;
        uint32_t it = 0, base = 0, m = n, inb = n;
        int st = kActive;
        bool in_list = n <= kListCap;
        unsigned long long bytes = 0;
        if (in_list) {
            for (uint32_t i = tid; i < n; i += blockDim.x) list[i] = __ldg(keys + rg.x + i);
            bytes += 4ull * n;
        }
        for (;;) {
            // ---- histogram round over the candidates, tree depth from their count
            const uint32_t cand = in_list ? m : inb;
            const int K = max(1, min(kMaxBinsLog2, 32 - __clz(max(cand, 1u))));
            const uint32_t nb = 1u << K;
            for (uint32_t j = tid; j < kBins; j += blockDim.x) s_hist[j] = 0u;
            fill_edges(s_edge, L, R, K, tid, blockDim.x);
            __syncthreads();
            const float scale = __fdividef((float)nb, R - L);
            uint32_t below = 0;
            auto visit = [&](float k) {
                if (k < L) {
                    ++below;
                } else if (k < R) {
                    const int g = edge_bin(k, L, scale, (int)nb - 1, [&](int j) { return s_edge[j]; });
                    atomicAdd(&s_hist[g], 1u);
                }
            };
            if (in_list) {
                for (uint32_t i = tid; i < m; i += blockDim.x) visit(list[i]);
            } else {
                for_keys(keys, rg.x, rg.y, visit);
                bytes += 4ull * n;
            }
            below = base + block_sum(below, sh);
            // exclusive prefix of the bins in place (4 bins per thread)
            uint32_t h4[4], loc = 0;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                h4[q] = s_hist[tid * 4 + q];
                loc += h4[q];
            }
            uint32_t tot_a, tot_b;
            const uint2 ex = block_excl_scan2(loc, 0u, sh, &tot_a, &tot_b);
            uint32_t run = ex.x;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                s_hist[tid * 4 + q] = run;
                run += h4[q];
            }
            __syncthreads();
            // ---- replay up to K iterations (identically in every thread)
            uint32_t pos = 0, width = nb;
            for (int step = 0; step < K; ++step) {
                if (it >= (uint32_t)kMaxIterations) {
                    st = kCapped;
                    break;
                }
                const uint32_t half = width >> 1;
                const uint32_t cl = below + s_hist[pos + half];
                ++it;
                const int dir = convergence(cl, n, ratio);
                if (dir == 0) {
                    st = kFound;
                    break;
                }
                const float cut = mid_cut(L, R);
                if (dir > 0) {
                    R = cut;
                } else {
                    L = cut;
                    pos += half;
                }
                width = half;
            }
            if (st == kActive && it >= (uint32_t)kMaxIterations) st = kCapped;
            if (st != kActive) break;
            // keys in the new bracket [L, R) (entry nb of the prefix is the round's total)
            inb = (pos + 1 < nb ? s_hist[pos + 1] : tot_a) - s_hist[pos];
            __syncthreads();
            // ---- the new bracket's keys become the candidates
            if (in_list) {
                // every thread reads its keys, then (after the barrier in block_sum) the
                // keys of the new bracket are appended, one warp-aggregated slot per round
                float kq[kListPerThread];
                uint32_t blw = 0;
#pragma unroll
                for (uint32_t q = 0; q < kListPerThread; ++q) {
                    const uint32_t i = tid + q * kCtaThreads;
                    kq[q] = i < m ? list[i] : R;  // R: neither below L nor kept
                    blw += kq[q] < L;
                }
                if (tid == 0) s_fill = 0;
                base += block_sum(blw, sh);
                const uint32_t lane = tid & 31;
#pragma unroll
                for (uint32_t q = 0; q < kListPerThread; ++q) {
                    const bool keep = !(kq[q] < L) && kq[q] < R;
                    const uint32_t bal = __ballot_sync(0xffffffffu, keep);
                    uint32_t wb = 0;
                    if (lane == 0 && bal) wb = atomicAdd(&s_fill, (uint32_t)__popc(bal));
                    wb = __shfl_sync(0xffffffffu, wb, 0);
                    if (keep) list[wb + __popc(bal & ((1u << lane) - 1u))] = kq[q];
                }
                __syncthreads();
                m = s_fill;
            } else if (inb <= kListCap) {
                if (tid == 0) s_fill = 0;
                __syncthreads();
                uint32_t blw = 0;
                for_keys(keys, rg.x, rg.y, [&](float k) {
                    if (k < L)
                        ++blw;
                    else if (k < R)
                        list[atomicAdd(&s_fill, 1u)] = k;
                });
                bytes += 4ull * n;
                base = block_sum(blw, sh);
                m = s_fill;
                in_list = true;
            }
            __syncthreads();
        }
        if (tid == 0) {
            cell.cutMarginLeft = L;
            cell.cutMarginRight = R;
            cell.foundCut = st == kFound ? 1 : 0;
            v.iters[c] = (uint8_t)it;
            v.state[c] = (uint8_t)st;
            atomicMax(&v.counters->max_iters, it);
            if (st == kCapped) atomicAdd(&v.counters->unfound, 1u);
            add_bytes(v, kKBisectCta, bytes);
        }
        __syncthreads();
    }
}

// Tile -> cell maps of the level (one binary search per tile, once per level).
// ... and the per-cell state of the level, in parallel (the plan only computes the offsets).
__global__ void k_tile_map(Level v) {
    pdl_enter();
    if (v.skip && *(volatile const uint32_t *)v.skip) return;  // subtrees took this level
    const uint32_t ht = v.tile_off[v.C], pt = v.ptile_off[v.C], C = (uint32_t)v.C;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < max(max(ht, pt), C);
         t += gridDim.x * blockDim.x) {
        if (t < ht) v.htile_cell[t] = find_cell(v.tile_off, v.C, t);
        if (t < pt) v.ptile_cell[t] = find_cell(v.ptile_off, v.C, t);
        if (t < C) {
            const uint2 rg = v.ranges[level_slot(v, (int)t)];
            const uint32_t n = rg.y - rg.x;
            v.hist_k[t] = (uint8_t)tree_depth(n);
            v.state[t] = n <= (uint32_t)kWarpKeys ? kSmall : (n <= (uint32_t)kTile ? kOneTile : kActive);
            v.iters[t] = 0;
            v.below[t] = 0;
            v.inb[t] = n;
            v.cmp_cnt[t] = 0;
            v.listed[t] = 0;
            v.cmp_bad[t] = 0;
            if (v.pred) v.pred[t] = 0u;  // no sampled bracket unless k_sample_pick sets one
        }
    }
}

// ------------------------------------------------------------------------------------
// Partition
//
// Partition tiles are kPTile consecutive positions of one cell. Per tile, the classify
// pass stores two bitmasks (key >= cut, key <= cut) and their counts; one scan over all
// tiles of the level gives every tile its exclusive prefix (in-cell prefix = difference
// with the cell's first tile). A warp per cell then finds s and the split index i, and a
// CTA per tile performs the swaps of the pairs whose left element lies in that tile.
// ------------------------------------------------------------------------------------
__device__ __forceinline__ float cell_cut(const orb_cell_t &c) {
    return mid_cut(c.cutMarginLeft, c.cutMarginRight);
}


// Status word of one scan block in the look-back: flag (bits 62-63), count of keys
// >= cut (bits 31-61) and keys <= cut (bits 0-30). Level totals stay below 2^31.
constexpr unsigned long long kStAggregate = 1ull << 62;
constexpr unsigned long long kStInclusive = 2ull << 62;
constexpr unsigned long long kStFlags = 3ull << 62;

__device__ __forceinline__ unsigned long long pack_status(unsigned long long flag, uint32_t g,
                                                          uint32_t l) {
    return flag | ((unsigned long long)g << 31) | (unsigned long long)l;
}

// P1: bitmasks of keys >= cut and keys <= cut per partition tile, and their counts.
// One warp per tile: the metadata chains (tile -> cell -> range, cut) of the CTA's warps
// overlap, and each lane keeps kClassifyLoads loads in flight. The mask words are staged in
// shared memory and stored coalesced.
constexpr int kClassifyLoads = 16;

__global__ void __launch_bounds__(kThreads) k_part_classify(Level v) {
    pdl_enter();
    if (v.skip && *(volatile const uint32_t *)v.skip) return;  // subtrees took this level
    __shared__ uint32_t s_words[kThreads / 32][2][kPWords];
    const uint32_t total = v.ptile_off[v.C];
    const int lane = threadIdx.x & 31;
    uint32_t(*sw)[kPWords] = s_words[threadIdx.x >> 5];
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    unsigned long long bytes = 0;
    for (uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < total; t += nwarps) {
        const int c = v.ptile_cell ? (int)v.ptile_cell[t] : find_cell(v.ptile_off, v.C, t);
        const uint32_t t0 = v.ptile_off[c];
        const int slot = level_slot(v, c);
        const orb_cell_t &cell = v.heap[slot];
        const float cut = cell_cut(cell);
        const float *keys = axis_keys(v, eff_axis(cell.cutAxis));
        const uint2 rg = v.ranges[slot];
        const uint32_t p0 = rg.x + (t - t0) * (uint32_t)kPTile;
        const uint32_t m = min((uint32_t)kPTile, rg.y - p0);
        uint32_t cg = 0, cl = 0;
#pragma unroll 1
        for (int r = 0; r < kPWords; r += kClassifyLoads) {
            float k[kClassifyLoads];
#pragma unroll
            for (int u = 0; u < kClassifyLoads; ++u) {
                const uint32_t i = (uint32_t)(r + u) * 32u + lane;
                k[u] = i < m ? __ldg(keys + p0 + i) : 0.0f;
            }
#pragma unroll
            for (int u = 0; u < kClassifyLoads; ++u) {
                const int w = r + u;
                const bool valid = (uint32_t)w * 32u + lane < m;
                const uint32_t gb = __ballot_sync(0xffffffffu, valid && !(k[u] < cut));
                const uint32_t lb = __ballot_sync(0xffffffffu, valid && !(k[u] > cut));
                if (lane == u) {
                    sw[0][w] = gb;
                    sw[1][w] = lb;
                }
                cg += __popc(gb);
                cl += __popc(lb);
            }
        }
        uint32_t *gw = v.ge_bits + (size_t)t * kPWords;
        uint32_t *lw = v.le_bits + (size_t)t * kPWords;
        __syncwarp();
#pragma unroll
        for (int q = 0; q < kPWords / 32; ++q) {
            gw[q * 32 + lane] = sw[0][q * 32 + lane];
            lw[q * 32 + lane] = sw[1][q * 32 + lane];
        }
        __syncwarp();
        if (lane == 0) {
            v.pt_ge[t] = cg;
            v.pt_le[t] = cl;
            bytes += 4ull * m + 8ull * kPWords + 8ull;
        }
    }
    if (lane == 0 && bytes) add_bytes(v, kKPartClassify, bytes);
}

// P2: global exclusive prefix of the per-tile counts over every tile of the level:
// pt_*_pre[t] = sum over tiles before t, entry [total] = grand total. Blocks of 1024 tiles
// take logical indices by ticket and chain their prefixes with a decoupled look-back (a
// block only waits on blocks that started before it; the wait is bounded all the same).
// In-cell prefixes are differences with the cell's first tile.
constexpr int kScanBlock = 1024;

__global__ void __launch_bounds__(kScanBlock) k_tile_scan(Level v) {
    pdl_enter();
    if (v.skip && *(volatile const uint32_t *)v.skip) return;  // subtrees took this level
    __shared__ uint32_t sh[96];
    __shared__ uint32_t s_b;
    __shared__ uint32_t s_pre[2];
    const uint32_t total = v.ptile_off[v.C];
    const uint32_t nblk = total / kScanBlock + 1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    volatile unsigned long long *status = v.pt_status;
    if (threadIdx.x == 0) s_b = atomicAdd(v.ticket, 1u);
    __syncthreads();
    const uint32_t b = s_b;
    if (b >= nblk) return;
    const uint32_t t = b * kScanBlock + threadIdx.x;
    const uint32_t g = t < total ? v.pt_ge[t] : 0u;
    const uint32_t l = t < total ? v.pt_le[t] : 0u;
    uint32_t ag, al;
    const uint2 ex = block_excl_scan2(g, l, sh, &ag, &al);
    if (warp == 0) {
        uint32_t pg = 0, pl = 0;
        if (b == 0) {
            if (lane == 0) status[0] = pack_status(kStInclusive, ag, al);
        } else {
            if (lane == 0) status[b] = pack_status(kStAggregate, ag, al);
            long long j = (long long)b - 1;
            for (;;) {  // 32 predecessors at a time; blocks before 0 count as inclusive zero
                const long long jj = j - lane;
                unsigned long long st = kStInclusive;
                if (jj >= 0) {
                    uint32_t spins = 0;
                    while (((st = status[jj]) & kStFlags) == 0ull) {
                        if (++spins > v.spin_limit) {
                            atomicExch(&v.counters->error, 1u);
                            st = kStInclusive;
                            break;
                        }
                        __nanosleep(64);
                    }
                }
                const uint32_t incl = __ballot_sync(0xffffffffu, (st & kStFlags) == kStInclusive);
                const int first = incl ? __ffs(incl) - 1 : 32;
                const bool take = lane <= first;
                pg += warp_sum(take ? (uint32_t)((st >> 31) & 0x7fffffffull) : 0u);
                pl += warp_sum(take ? (uint32_t)(st & 0x7fffffffull) : 0u);
                if (incl) break;
                j -= 32;
            }
            if (lane == 0) status[b] = pack_status(kStInclusive, pg + ag, pl + al);
        }
        if (lane == 0) {
            s_pre[0] = pg;
            s_pre[1] = pl;
        }
    }
    __syncthreads();
    if (t <= total) {
        v.pt_ge_pre[t] = s_pre[0] + ex.x;
        v.pt_le_pre[t] = s_pre[1] + ex.y;
    }
    if (threadIdx.x == 0) add_bytes(v, kKPartScan, 16ull * min((uint32_t)kScanBlock, total + 1 - b * kScanBlock));
}

// Position (cell-relative) of the set bit with in-cell rank `rank` among the bitmasks of
// tiles [t0, t1), `pre` the level's global exclusive tile prefix (warp-cooperative; every
// lane returns the answer).
__device__ uint32_t warp_select(const uint32_t *bits, const uint32_t *pre, uint32_t t0, uint32_t t1,
                                uint32_t rank) {
    const int lane = threadIdx.x & 31;
    const uint32_t base0 = pre[t0];
    uint32_t lo = t0, hi = t1 - 1;  // largest t with pre[t] - base0 <= rank
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (pre[mid] - base0 <= rank)
            lo = mid;
        else
            hi = mid - 1;
    }
    const uint32_t r = rank - (pre[lo] - base0);
    const uint32_t *w = bits + (size_t)lo * kPWords + lane * (kPWords / 32);
    uint32_t words[kPWords / 32];
    uint32_t cnt = 0;
#pragma unroll
    for (int j = 0; j < kPWords / 32; ++j) {
        words[j] = w[j];
        cnt += __popc(words[j]);
    }
    uint32_t tot;
    const uint32_t ex = warp_excl_scan(cnt, &tot);
    const bool mine = r >= ex && r < ex + cnt;
    uint32_t pos = 0;
    if (mine) {
        uint32_t rr = r - ex;
#pragma unroll
        for (int j = 0; j < kPWords / 32; ++j) {
            const uint32_t pc = __popc(words[j]);
            if (rr < pc) {
                uint32_t word = words[j];
                for (uint32_t q = 0; q < rr; ++q) word &= word - 1;  // drop rr lowest set bits
                pos = (lo - t0) * (uint32_t)kPTile + (uint32_t)(lane * (kPWords / 32) + j) * 32u +
                      (uint32_t)(__ffs(word) - 1);
                rr = 0xffffffffu;
                break;
            }
            rr -= pc;
        }
    }
    const uint32_t who = __ballot_sync(0xffffffffu, mine);
    return __shfl_sync(0xffffffffu, pos, __ffs(who) - 1);
}

// A look-back wait of the tile scan (or a bisection) gave up and flagged the build: the tile
// prefixes may be incomplete, so the kernels that read them do nothing and the build
// returns ORB_ERR_TIMEOUT.
__device__ __forceinline__ bool scan_failed(const Level &v) {
    return *(volatile const uint32_t *)&v.counters->error != 0u;
}

// P3: per cell (one warp): totals, the swap count s and the split index i.
//   s = max_x min(f(x), g(x)), f(x) = #{>= cut in [0,x)}, g(x) = #{<= cut in [x,n)}
//   i = min(L_{s+1}, R_s); i == n marks the clamped case (every key below the cut).
__global__ void __launch_bounds__(kThreads) k_part_cells(Level v) {
    pdl_enter();
    if (v.skip && *(volatile const uint32_t *)v.skip) return;  // subtrees took this level
    if (scan_failed(v)) return;  // a look-back wait gave up: the prefixes are not valid
    const int c = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (c >= v.C) return;
    const int slot = level_slot(v, c);
    const uint2 rg = v.ranges[slot];
    const uint32_t n = rg.y - rg.x;
    const uint32_t t0 = v.ptile_off[c], t1 = v.ptile_off[c + 1];
    const uint32_t G0 = v.pt_ge_pre[t0], L0 = v.pt_le_pre[t0];
    const uint32_t ge_tot = v.pt_ge_pre[t1] - G0, le_tot = v.pt_le_pre[t1] - L0;
    uint32_t s = 0, i = n;
    if (t1 > t0) {
        // crossing tile: first tile whose end has f >= g (the last tile always does)
        uint32_t lo = t0, hi = t1 - 1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            const uint32_t f_end = v.pt_ge_pre[mid + 1] - G0;
            const uint32_t g_end = le_tot - (v.pt_le_pre[mid + 1] - L0);
            if (f_end >= g_end)
                hi = mid;
            else
                lo = mid + 1;
        }
        const uint32_t *gw = v.ge_bits + (size_t)lo * kPWords + lane * (kPWords / 32);
        const uint32_t *lw = v.le_bits + (size_t)lo * kPWords + lane * (kPWords / 32);
        uint32_t gwd[kPWords / 32], lwd[kPWords / 32];
        uint32_t cg = 0, cl = 0;
#pragma unroll
        for (int j = 0; j < kPWords / 32; ++j) {
            gwd[j] = gw[j];
            lwd[j] = lw[j];
            cg += __popc(gwd[j]);
            cl += __popc(lwd[j]);
        }
        uint32_t tg, tl;
        const uint32_t eg = warp_excl_scan(cg, &tg);
        const uint32_t el = warp_excl_scan(cl, &tl);
        uint32_t f = (v.pt_ge_pre[lo] - G0) + eg;
        uint32_t g = le_tot - (v.pt_le_pre[lo] - L0) - el;
        uint32_t best = min(f, g);
#pragma unroll
        for (int j = 0; j < kPWords / 32; ++j) {
            uint32_t a = gwd[j], b = lwd[j];
            for (int q = 0; q < 32; ++q) {
                f += a & 1u;
                g -= b & 1u;
                a >>= 1;
                b >>= 1;
                best = max(best, min(f, g));
            }
        }
        s = warp_max(best);
        if (ge_tot > s) i = min(i, warp_select(v.ge_bits, v.pt_ge_pre, t0, t1, s));
        if (s >= 1) i = min(i, warp_select(v.le_bits, v.pt_le_pre, t0, t1, le_tot - s));
    }
    if (lane == 0) {
        v.part_s[c] = s;
        v.part_i[c] = i;
        v.part_le[c] = le_tot;
        add_bytes(v, kKPartCells, 16ull * 3 + (t1 > t0 ? 3ull * 2 * 4 * kPWords : 0ull));
    }
}

// Writes the cell-relative positions of the set bits of one tile's mask whose in-cell rank
// lies in [lo, hi) to out[f(rank)], f(rank) = rank - lo (forward) or (top - rank) (reverse).
// Block-cooperative; `sh` holds >= 96 words.
__device__ __forceinline__ void emit_positions(const uint32_t *words, uint32_t rank_base,
                                               uint32_t lo, uint32_t hi, uint32_t rel_base,
                                               bool reverse, uint32_t top, uint32_t *out,
                                               uint32_t *sh) {
    const uint32_t tid = threadIdx.x;
    const uint32_t w = tid < (uint32_t)kPWords ? words[tid] : 0u;
    uint32_t ta, tb;
    const uint2 ex = block_excl_scan2(__popc(w), 0u, sh, &ta, &tb);
    uint32_t r = rank_base + ex.x;
    uint32_t word = w;
    while (word) {
        const uint32_t b = (uint32_t)(__ffs(word) - 1);
        word &= word - 1;
        if (r >= lo && r < hi) out[reverse ? top - r : r - lo] = rel_base + tid * 32u + b;
        ++r;
    }
}

// (y or z null: that array is not moved at this level; builds from host memory reorder it
// later through the permutation, see orb_build)
__device__ __forceinline__ void swap_particles(const Level &v, uint32_t a, uint32_t b) {
    const float xa = v.x[a], xb = v.x[b];
    v.x[a] = xb;
    v.x[b] = xa;
    if (v.y) {
        const float ya = v.y[a], yb = v.y[b];
        v.y[a] = yb;
        v.y[b] = ya;
    }
    if (v.z) {
        const float za = v.z[a], zb = v.z[b];
        v.z[a] = zb;
        v.z[b] = za;
    }
    if (v.idx) {
        const uint32_t ia = v.idx[a], ib = v.idx[b];
        v.idx[a] = ib;
        v.idx[b] = ia;
    }
    if (v.wt) {
        const uint32_t wa = v.wt[a], wb = v.wt[b];
        v.wt[a] = wb;
        v.wt[b] = wa;
    }
}

// Largest u in [lo, hi] with pre[u] - base <= r, for a nondecreasing pre with
// pre[lo] - base <= r: a 32-way search (every lane probes one point per round, the passing
// probes are a prefix of the lanes), three rounds for 2^15 candidates. Warp-uniform result.
__device__ __forceinline__ uint32_t warp_last_at_most(const uint32_t *pre, uint32_t base,
                                                      uint32_t lo, uint32_t hi, uint32_t r) {
    const uint32_t lane = threadIdx.x & 31;
    while (lo < hi) {
        const uint32_t step = (hi - lo + 31) / 32;
        const uint32_t u = lo + (lane + 1) * step;
        const bool ok = u <= hi && pre[u] - base <= r;
        const uint32_t cnt = (uint32_t)__popc(__ballot_sync(0xffffffffu, ok));
        lo += cnt * step;
        hi = min(hi, lo + step - 1);
    }
    return lo;
}

// P4: the Hoare swaps. The CTA of tile t takes the pairs (L_k, R_k) whose left element
// L_k lies in t (k < s); their right partners are the keys <= cut of left-to-right rank
// le_tot-1-k, found in the right tiles' masks. Positions of each side are disjoint
// (L_k < i <= R_k), so the CTAs never touch the same particle.
// Tuning (compile time): pairs per thread per round, and the CTAs per SM the register
// budget is sized for (4 x 256 threads: 64 registers a thread).
#ifndef ORB_SWAP_BATCH
#define ORB_SWAP_BATCH 4
#endif
#ifndef ORB_SWAP_MIN_BLOCKS
#define ORB_SWAP_MIN_BLOCKS 4
#endif
#ifndef ORB_SWAP_THREADS
#define ORB_SWAP_THREADS 256  // threads of a swap CTA (at least kPWords: one mask word each)
#endif
constexpr int kSwapThreads = ORB_SWAP_THREADS;
static_assert(kSwapThreads >= kPWords && kSwapThreads % 32 == 0, "a swap CTA scans a tile's mask words");
// kWt: weighted builds, whose weights move with their particles. kYZ: bit 0 y moves, bit 1 z
// moves (3 normally; the first levels of a build from host memory move x before y and z have
// arrived, see orb_build).
template <bool kWt, int kYZ>
__global__ void __launch_bounds__(kSwapThreads, ORB_SWAP_MIN_BLOCKS) k_part_swap(Level v) {
    pdl_enter();
    if (v.skip && *(volatile const uint32_t *)v.skip) return;  // subtrees took this level
    if (scan_failed(v)) return;  // a look-back wait gave up: the prefixes are not valid
    __shared__ uint32_t posL[kPTile];
    __shared__ uint32_t posR[kPTile];
    __shared__ uint32_t sh[96];
    const uint32_t total = v.ptile_off[v.C];
    unsigned long long bytes = 0;  // pairs swapped by this CTA
    for (uint32_t t = blockIdx.x; t < total; t += gridDim.x) {
        const int c = v.ptile_cell ? (int)v.ptile_cell[t] : find_cell(v.ptile_off, v.C, t);
        const uint32_t t0 = v.ptile_off[c], t1 = v.ptile_off[c + 1];
        const uint32_t s = v.part_s[c];
        const uint32_t G0 = v.pt_ge_pre[t0], L0 = v.pt_le_pre[t0];
        const uint32_t ka = v.pt_ge_pre[t] - G0;
        const uint32_t kb = min(s, v.pt_ge_pre[t + 1] - G0);
        if (ka >= kb) continue;
        const uint32_t cnt = kb - ka;
        const uint32_t le_tot = v.part_le[c];
        const uint32_t b = v.ranges[level_slot(v, c)].x;
        // left elements: ranks [ka, kb) of this tile's >= mask, in order
        emit_positions(v.ge_bits + (size_t)t * kPWords, ka, ka, kb, (t - t0) * (uint32_t)kPTile,
                       false, 0u, posL, sh);
        // right partners: left-to-right <= ranks [le_tot-kb, le_tot-ka); rank r pairs with
        // k = le_tot-1-r, stored at posR[k - ka] = posR[(le_tot-1-ka) - r]
        const uint32_t ra = le_tot - kb, rb = le_tot - ka;
        const uint32_t u0 = warp_last_at_most(v.pt_le_pre, L0, t0, t1 - 1, ra);
        for (uint32_t u = u0; u < t1 && v.pt_le_pre[u] - L0 < rb; ++u)
            emit_positions(v.le_bits + (size_t)u * kPWords, v.pt_le_pre[u] - L0, ra, rb,
                           (u - t0) * (uint32_t)kPTile, true, le_tot - 1 - ka, posR, sh);
        __syncthreads();
        // kB pairs per thread per round: every load is issued before any store
        constexpr int kB = ORB_SWAP_BATCH;
        for (uint32_t j0 = 0; j0 < cnt; j0 += kB * blockDim.x) {
            uint32_t pa[kB], pb[kB];
            float xa[kB], xb[kB], ya[kB], yb[kB], za[kB], zb[kB];
            uint32_t ia[kB], ib[kB], wa[kB], wb[kB];
#pragma unroll
            for (int q = 0; q < kB; ++q) {
                const uint32_t j = j0 + q * blockDim.x + threadIdx.x;
                const bool ok = j < cnt;
                pa[q] = ok ? b + posL[j] : 0xffffffffu;
                pb[q] = ok ? b + posR[j] : 0xffffffffu;
                if (ok) {
                    xa[q] = v.x[pa[q]];
                    xb[q] = v.x[pb[q]];
                    if constexpr ((kYZ & 1) != 0) {
                        ya[q] = v.y[pa[q]];
                        yb[q] = v.y[pb[q]];
                    }
                    if constexpr ((kYZ & 2) != 0) {
                        za[q] = v.z[pa[q]];
                        zb[q] = v.z[pb[q]];
                    }
                    if (v.idx) {
                        ia[q] = v.idx[pa[q]];
                        ib[q] = v.idx[pb[q]];
                    }
                    if constexpr (kWt) {
                        wa[q] = v.wt[pa[q]];
                        wb[q] = v.wt[pb[q]];
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < kB; ++q) {
                if (pa[q] == 0xffffffffu) continue;
                v.x[pa[q]] = xb[q];
                v.x[pb[q]] = xa[q];
                if constexpr ((kYZ & 1) != 0) {
                    v.y[pa[q]] = yb[q];
                    v.y[pb[q]] = ya[q];
                }
                if constexpr ((kYZ & 2) != 0) {
                    v.z[pa[q]] = zb[q];
                    v.z[pb[q]] = za[q];
                }
                if (v.idx) {
                    v.idx[pa[q]] = ib[q];
                    v.idx[pb[q]] = ia[q];
                }
                if constexpr (kWt) {
                    v.wt[pa[q]] = wb[q];
                    v.wt[pb[q]] = wa[q];
                }
            }
        }
        bytes += cnt;
        __syncthreads();
    }
    // per pair: both elements of x, y, z (and idx, weights) read and written
    if (threadIdx.x == 0 && bytes)
        add_bytes(v, kKPartSwap, (16ull * (1 + (kYZ & 1) + ((kYZ >> 1) & 1)) + (v.idx ? 16ull : 0ull) +
                                  (kWt ? 16ull : 0ull)) * bytes);
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

// Final swap(i, n-1) of a partitioned cell (src/services/partition.cpp:52), its children's
// ranges and (optionally) its children's cells.
__device__ void finish_cell(const Level &v, int slot, uint32_t i, bool do_split) {
    const orb_cell_t cell = v.heap[slot];
    const uint2 rg = v.ranges[slot];
    const uint32_t n = rg.y - rg.x;
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

// P5: finish_cell for every cell of the level.
__global__ void __launch_bounds__(kThreads) k_part_finish(Level v, int do_split) {
    pdl_enter();
    if (v.skip && *(volatile const uint32_t *)v.skip) return;  // subtrees took this level
    if (scan_failed(v)) return;  // a look-back wait gave up: the prefixes are not valid
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= v.C) return;
    finish_cell(v, level_slot(v, c), v.part_i[c], do_split != 0);
}

// ------------------------------------------------------------------------------------
// Subtrees: once every cell of a level holds at most kSubMax particles, one CTA takes a
// cell and finishes all the levels below it (bisection, Hoare partition and split of each
// descendant, breadth first), the same steps as the level kernels at CTA scale. A cell's
// particles (at most 408 KB) stay in L2 across its levels instead of crossing DRAM once per
// level, and the level kernels of those levels do not run.
// ------------------------------------------------------------------------------------
constexpr uint32_t kSubMax = kSubMaxParticles;  // particles of a cell a CTA can take (masks)
constexpr int kSubWords = (int)(kSubMax / 32);
constexpr int kSubThreads = 256;
constexpr int kSubBinsLog2 = 9;
constexpr int kSubQueue = 64;                 // descendants of one level held at once

constexpr int kSubList = 256;                 // bracket keys gathered for the last iterations
constexpr int kSubRankBlocks = (int)(kSubMax / 64) + 2;

struct SubSmem {
    uint32_t ge[kSubWords], le[kSubWords];           // key >= cut, key <= cut
    uint32_t pge[kSubWords + 1], ple[kSubWords + 1];  // exclusive prefix popcounts
    uint16_t tge[kSubRankBlocks], tle[kSubRankBlocks];  // word holding rank 64 b
    uint32_t bins[1 << kSubBinsLog2];
    float edges[(1 << kSubBinsLog2) + 1];
    float list[kSubList];
    uint32_t red[96];
    int queue[2][kSubQueue];
    uint32_t word, count;                            // broadcast values
    int root;                                        // the CTA's current root cell
};

// Position of the bit of rank r (0-based) in w (r < popc(w)).
__device__ __forceinline__ uint32_t select_in_word(uint32_t w, uint32_t r) {
    uint32_t pos = 0;
#pragma unroll
    for (int step = 16; step >= 1; step >>= 1) {
        const uint32_t c = (uint32_t)__popc(w & ((1u << step) - 1u));
        if (r >= c) {
            r -= c;
            w >>= step;
            pos += (uint32_t)step;
        }
    }
    return pos;
}

// sub_select() through the rank table t (t[b] = the word holding rank 64 b): a few steps
// from the table's word instead of a search.
__device__ __forceinline__ uint32_t sub_select_t(const uint32_t *bits, const uint32_t *pre,
                                                 const uint16_t *t, uint32_t r) {
    uint32_t w = t[r >> 6];
    while (pre[w + 1] <= r) ++w;
    return w * 32u + select_in_word(bits[w], r - pre[w]);
}

// Position (cell-relative) of the set bit of rank r (0-based) of the mask `bits`, given
// its exclusive word prefix `pre` over W words.
__device__ __forceinline__ uint32_t sub_select(const uint32_t *bits, const uint32_t *pre, int W,
                                               uint32_t r) {
    int lo = 0, hi = W - 1;  // last word with pre <= r
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pre[mid] <= r)
            lo = mid;
        else
            hi = mid - 1;
    }
    return (uint32_t)lo * 32u + select_in_word(bits[lo], r - pre[lo]);
}

// The reference's bisection (src/orbit.cpp:146-232) of one cell by the CTA: a warp with the
// keys in registers for at most kWarpKeys keys, else rounds of a shared-memory histogram over
// the midpoint tree of the bracket (tree depth from the keys left in it) each replaying up to
// K iterations, as k_bisect_tile does per warp.
__device__ void sub_bisect(const Level &v, int slot, SubSmem &sm, unsigned long long &bytes) {
    orb_cell_t &cell = v.heap[slot];
    const uint2 rg = v.ranges[slot];
    const uint32_t n = rg.y - rg.x;
    // subtrees run for d a power of two only: every cell below has an even leaf count
    const float ratio = 0.5f;  // leaf_ratio(cell.nLeafCells), src/orbit.cpp:204
    const float *keys = axis_keys(v, eff_axis(cell.cutAxis));
    const uint32_t tid = threadIdx.x, lane = tid & 31;
    float L = cell.cutMarginLeft, R = cell.cutMarginRight;
    uint32_t it = 0;
    int st = kActive;
    if (n <= (uint32_t)kWarpKeys) {
        if (tid < 32) {
            float k[kWarpKeysPerLane];
#pragma unroll
            for (int j = 0; j < kWarpKeysPerLane; ++j) {
                const uint32_t i = (uint32_t)(j * 32) + lane;
                k[j] = i < n ? keys[rg.x + i] : __int_as_float(0x7fc00000);  // coherent: moved here
            }
            while (st == kActive) {
                if (it >= (uint32_t)kMaxIterations) {
                    st = kCapped;
                    break;
                }
                const float cut = mid_cut(L, R);
                uint32_t cnt = 0;
#pragma unroll
                for (int j = 0; j < kWarpKeysPerLane; ++j) cnt += k[j] < cut;
                cnt = warp_sum(cnt);
                ++it;
                const int dir = convergence(cnt, n, ratio);
                if (dir == 0)
                    st = kFound;
                else if (dir > 0)
                    R = cut;
                else
                    L = cut;
            }
        }
        if (tid == 0) bytes += 4ull * n;
    } else {
        uint32_t cand = n;
        while (st == kActive) {
            // about one key a bin once the bracket is small: two rounds for most cells
            const int K = max(1, min(kSubBinsLog2, 32 - __clz(max(cand, 1u))));
            const uint32_t nb = 1u << K;
            for (uint32_t j = tid; j < nb; j += blockDim.x) sm.bins[j] = 0u;
            fill_edges(sm.edges, L, R, K, tid, blockDim.x);
            __syncthreads();
            const float scale = __fdiv_rn((float)nb, __fsub_rn(R, L));
            const Guess gs = make_guess(L, R, scale, nb);
            const int top = (int)nb - 1;
            uint32_t below = 0;
            auto one = [&](float k) {
                if (k < L)
                    ++below;
                else if (k < R)
                    atomicAdd(&sm.bins[fast_bin(k, gs, top, sm.edges)], 1u);
            };
            visit_keys<false>(keys, rg.x, rg.y, R, tid, blockDim.x, one, each(one));
            if (tid == 0) bytes += 4ull * n;
            below = block_sum(below, sm.red);
            // exclusive prefix of the bins in place (each thread its own run)
            const uint32_t per = max(1u, nb / blockDim.x), j0 = tid * per, j1 = min(nb, j0 + per);
            uint32_t loc = 0;
            for (uint32_t j = j0; j < j1; ++j) loc += sm.bins[j];
            uint32_t tot, unused;
            uint32_t run = block_excl_scan2(loc, 0u, sm.red, &tot, &unused).x;
            for (uint32_t j = j0; j < j1; ++j) {
                const uint32_t h = sm.bins[j];
                sm.bins[j] = run;
                run += h;
            }
            __syncthreads();
            uint32_t pos = 0, width = nb;
            for (int step = 0; step < K; ++step) {
                if (it >= (uint32_t)kMaxIterations) {
                    st = kCapped;
                    break;
                }
                const uint32_t half = width >> 1;
                const uint32_t cl = below + sm.bins[pos + half];
                ++it;
                const int dir = convergence(cl, n, ratio);
                if (dir == 0) {
                    st = kFound;
                    break;
                }
                const float cut = mid_cut(L, R);
                if (dir > 0) {
                    R = cut;
                } else {
                    L = cut;
                    pos += half;
                }
                width = half;
            }
            if (st == kActive && it >= (uint32_t)kMaxIterations) st = kCapped;
            if (st == kActive) cand = (pos + 1 < nb ? sm.bins[pos + 1] : tot) - sm.bins[pos];
            const uint32_t below_L = below + sm.bins[pos];  // keys below the new L
            __syncthreads();  // the bins are rewritten by the next round
            if (st == kActive && cand <= (uint32_t)kSubList) {
                // the bracket's keys into a shared list; warp 0 finishes the bisection on it
                if (tid == 0) sm.count = 0;
                __syncthreads();
                auto gather = [&](float k) {
                    if (!(k < L) && k < R) sm.list[atomicAdd(&sm.count, 1u)] = k;
                };
                visit_keys<false>(keys, rg.x, rg.y, R, tid, blockDim.x, gather, each(gather));
                if (tid == 0) bytes += 4ull * n;
                __syncthreads();
                if (tid < 32) {
                    const uint32_t m = sm.count;
                    constexpr int kPer = kSubList / 32;
                    float kl[kPer];
#pragma unroll
                    for (int q = 0; q < kPer; ++q) {
                        const uint32_t i = (uint32_t)q * 32u + lane;
                        kl[q] = i < m ? sm.list[i] : R;  // R: never below a cut in [L, R]
                    }
                    while (st == kActive) {
                        if (it >= (uint32_t)kMaxIterations) {
                            st = kCapped;
                            break;
                        }
                        const float cut = mid_cut(L, R);
                        uint32_t c = 0;
#pragma unroll
                        for (int q = 0; q < kPer; ++q) c += kl[q] < cut;
                        const uint32_t cl = below_L + warp_sum(c);
                        ++it;
                        const int dir = convergence(cl, n, ratio);
                        if (dir == 0)
                            st = kFound;
                        else if (dir > 0)
                            R = cut;
                        else
                            L = cut;
                    }
                }
                break;  // warp 0 holds the result (thread 0 writes it)
            }
        }
    }
    if (tid == 0) {
        cell.cutMarginLeft = L;
        cell.cutMarginRight = R;
        cell.foundCut = st == kFound ? 1 : 0;
        atomicMax(&v.counters->max_iters, it);
        if (st == kCapped) atomicAdd(&v.counters->unfound, 1u);
    }
    __syncthreads();
}

// Hoare partition of one cell by the CTA (same characterisation as the level kernels: the
// pairs (L_k, R_k), k < s, swapped, then i = min(L_{s+1}, R_s) and swap(i, n-1)), then the
// split into its children.
__device__ void sub_partition(const Level &v, int slot, SubSmem &sm, unsigned long long &bytes) {
    const orb_cell_t &cell = v.heap[slot];
    const uint2 rg = v.ranges[slot];
    const uint32_t n = rg.y - rg.x, b = rg.x;
    const float *keys = axis_keys(v, eff_axis(cell.cutAxis));
    const float cut = cell_cut(cell);
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    const int W = (int)((n + 31) / 32);
    // masks: a warp per word, kSubLoads words of a warp in flight at once
    constexpr int kSubLoads = 8;
    for (int w0 = (int)warp; w0 < W; w0 += (int)nwarps * kSubLoads) {
        float k[kSubLoads];
#pragma unroll
        for (int u = 0; u < kSubLoads; ++u) {
            const int w = w0 + u * (int)nwarps;
            const uint32_t i = (uint32_t)w * 32u + lane;
            k[u] = (w < W && i < n) ? keys[b + i] : 0.0f;  // coherent: the CTA moved these keys
        }
#pragma unroll
        for (int u = 0; u < kSubLoads; ++u) {
            const int w = w0 + u * (int)nwarps;
            if (w >= W) break;
            const bool valid = (uint32_t)w * 32u + lane < n;
            const uint32_t gb = __ballot_sync(0xffffffffu, valid && !(k[u] < cut));
            const uint32_t lb = __ballot_sync(0xffffffffu, valid && !(k[u] > cut));
            if (lane == 0) {
                sm.ge[w] = gb;
                sm.le[w] = lb;
            }
        }
    }
    __syncthreads();
    // exclusive prefix popcounts of both masks
    const int per = (W + (int)blockDim.x - 1) / (int)blockDim.x;
    const int w0 = (int)tid * per, w1 = min(W, w0 + per);
    uint32_t cg = 0, cl = 0;
    for (int w = w0; w < w1; ++w) {
        cg += __popc(sm.ge[w]);
        cl += __popc(sm.le[w]);
    }
    uint32_t ge_tot, le_tot;
    const uint2 ex = block_excl_scan2(cg, cl, sm.red, &ge_tot, &le_tot);
    uint32_t rg_ = ex.x, rl = ex.y;
    for (int w = w0; w < w1; ++w) {
        sm.pge[w] = rg_;
        sm.ple[w] = rl;
        rg_ += __popc(sm.ge[w]);
        rl += __popc(sm.le[w]);
    }
    if (tid == 0) {
        sm.pge[W] = ge_tot;
        sm.ple[W] = le_tot;
    }
    __syncthreads();  // prefixes complete
    // rank tables: the word holding rank 64 b of each mask
    for (int w = (int)tid; w < W; w += (int)blockDim.x) {
        for (uint32_t r = (sm.pge[w] + 63u) & ~63u; r < sm.pge[w + 1]; r += 64u) sm.tge[r >> 6] = (uint16_t)w;
        for (uint32_t r = (sm.ple[w] + 63u) & ~63u; r < sm.ple[w + 1]; r += 64u) sm.tle[r >> 6] = (uint16_t)w;
    }
    // s = max over x of min(#>= in [0,x), #<= in [x,n)): min(f, g) rises while f < g and
    // falls after, so the maximum lies in the first word at whose end f >= g (one thread)
    if (tid == 0) {
        uint32_t s_max = 0;
        if (W > 0) {
            int lo = 0, hi = W - 1;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (sm.pge[mid + 1] >= le_tot - sm.ple[mid + 1])
                    hi = mid;
                else
                    lo = mid + 1;
            }
            uint32_t f = sm.pge[lo], g = le_tot - sm.ple[lo];
            uint32_t a = sm.ge[lo], c = sm.le[lo];
            s_max = min(f, g);
            for (int q = 0; q < 32; ++q) {
                f += a & 1u;
                g -= c & 1u;
                a >>= 1;
                c >>= 1;
                s_max = max(s_max, min(f, g));
            }
        }
        sm.count = s_max;
    }
    __syncthreads();
    const uint32_t s_pairs = sm.count;
    // split index i = min(L_{s+1}, R_s); n when every key is below the cut
    if (tid == 0) {
        uint32_t i = n;
        if (ge_tot > s_pairs) i = min(i, sub_select(sm.ge, sm.pge, W, s_pairs));
        if (s_pairs >= 1) i = min(i, sub_select(sm.le, sm.ple, W, le_tot - s_pairs));
        sm.word = i;
    }
    // the swaps: pair k = (rank k of >=, rank le_tot-1-k of <=); sides disjoint; a thread
    // loads kSubPairs pairs before it stores any
    constexpr int kSubPairs = 2;
    for (uint32_t k0 = tid; k0 < s_pairs; k0 += blockDim.x * kSubPairs) {
        uint32_t pa[kSubPairs], pb[kSubPairs];
        float xa[kSubPairs], xb[kSubPairs], ya[kSubPairs], yb[kSubPairs], za[kSubPairs], zb[kSubPairs];
        uint32_t ia[kSubPairs], ib[kSubPairs];
#pragma unroll
        for (int q = 0; q < kSubPairs; ++q) {
            const uint32_t k = k0 + q * blockDim.x;
            pa[q] = pb[q] = 0xffffffffu;
            if (k < s_pairs) {
                pa[q] = b + sub_select_t(sm.ge, sm.pge, sm.tge, k);
                pb[q] = b + sub_select_t(sm.le, sm.ple, sm.tle, le_tot - 1 - k);
                xa[q] = v.x[pa[q]];
                xb[q] = v.x[pb[q]];
                ya[q] = v.y[pa[q]];
                yb[q] = v.y[pb[q]];
                za[q] = v.z[pa[q]];
                zb[q] = v.z[pb[q]];
                if (v.idx) {
                    ia[q] = v.idx[pa[q]];
                    ib[q] = v.idx[pb[q]];
                }
            }
        }
#pragma unroll
        for (int q = 0; q < kSubPairs; ++q) {
            if (pa[q] == 0xffffffffu) continue;
            v.x[pa[q]] = xb[q];
            v.x[pb[q]] = xa[q];
            v.y[pa[q]] = yb[q];
            v.y[pb[q]] = ya[q];
            v.z[pa[q]] = zb[q];
            v.z[pb[q]] = za[q];
            if (v.idx) {
                v.idx[pa[q]] = ib[q];
                v.idx[pb[q]] = ia[q];
            }
        }
    }
    if (tid == 0) bytes += (v.idx ? 64ull : 48ull) * s_pairs + 4ull * n;
    __syncthreads();  // swaps done, sm.word visible
    if (tid == 0) finish_cell(v, slot, sm.word, true);
    __syncthreads();
}

// ---- small cells (at most kWarpKeys particles) by one warp each, inside the subtree kernel:
// the same bisection and Hoare characterisation as sub_bisect / sub_partition, with the
// cell's keys in the warp's registers (lane l holds positions 32 j + l) and its masks one
// word a lane, so the CTA's warps finish eight small cells at once.

// Position of the set bit of rank r in the warp's mask (lane w holds word w, pre = its
// exclusive prefix popcount, W <= 32 words); r may differ from lane to lane: each lane
// searches the lanes' prefixes for the last word with pre <= r (5 shuffle steps, every lane
// taking part in every shuffle).
__device__ __forceinline__ uint32_t warp_mask_select(uint32_t word, uint32_t pre, uint32_t W,
                                                     uint32_t r) {
    int lo = 0, hi = (int)W - 1;
#pragma unroll
    for (int step = 0; step < 5; ++step) {
        const int mid = (lo + hi + 1) >> 1;
        const uint32_t pm = __shfl_sync(0xffffffffu, pre, mid);
        if (lo < hi) {
            if (pm <= r)
                lo = mid;
            else
                hi = mid - 1;
        }
    }
    const uint32_t ww = __shfl_sync(0xffffffffu, word, lo);
    const uint32_t pw = __shfl_sync(0xffffffffu, pre, lo);
    return (uint32_t)lo * 32u + select_in_word(ww, r - pw);
}

// The bisection of one small cell by the calling warp (src/orbit.cpp:146-232).
__device__ __noinline__ void warp_bisect_cell(const Level &v, int slot, uint32_t lane, unsigned long long &bytes) {
    orb_cell_t &cell = v.heap[slot];
    const uint2 rg = v.ranges[slot];
    const uint32_t n = rg.y - rg.x;
    const float ratio = 0.5f;  // subtrees: powers of two only (leaf_ratio of an even count)
    const float *keys = axis_keys(v, eff_axis(cell.cutAxis));
    float k[kWarpKeysPerLane];
#pragma unroll
    for (int j = 0; j < kWarpKeysPerLane; ++j) {
        const uint32_t i = (uint32_t)(j * 32) + lane;
        k[j] = i < n ? keys[rg.x + i] : __int_as_float(0x7fc00000);  // coherent: moved here
    }
    float L = cell.cutMarginLeft, R = cell.cutMarginRight;
    uint32_t it = 0;
    int st = kActive;
    while (st == kActive) {
        if (it >= (uint32_t)kMaxIterations) {
            st = kCapped;
            break;
        }
        const float cut = mid_cut(L, R);
        uint32_t cnt = 0;
#pragma unroll
        for (int j = 0; j < kWarpKeysPerLane; ++j) cnt += k[j] < cut;
        cnt = warp_sum(cnt);
        ++it;
        const int dir = convergence(cnt, n, ratio);
        if (dir == 0)
            st = kFound;
        else if (dir > 0)
            R = cut;
        else
            L = cut;
    }
    if (lane == 0) {
        cell.cutMarginLeft = L;
        cell.cutMarginRight = R;
        cell.foundCut = st == kFound ? 1 : 0;
        atomicMax(&v.counters->max_iters, it);
        if (st == kCapped) atomicAdd(&v.counters->unfound, 1u);
        bytes += 4ull * n;
    }
    __syncwarp();
}

// The Hoare partition (src/services/partition.cpp:30-52) of one small cell by the calling
// warp: masks of keys >= cut and <= cut (word w: positions 32 w .. 32 w + 31), the swap count
// s from the word where the two counts cross, the pairs (L_k, R_k) k < s swapped lane by
// lane, then i = min(L_{s+1}, R_s) and the final swap and split by lane 0 (finish_cell).
__device__ __noinline__ void warp_partition_cell(const Level &v, int slot, uint32_t lane, unsigned long long &bytes) {
    const orb_cell_t &cell = v.heap[slot];
    const uint2 rg = v.ranges[slot];
    const uint32_t n = rg.y - rg.x, b = rg.x;
    const float *keys = axis_keys(v, eff_axis(cell.cutAxis));
    const float cut = cell_cut(cell);
    const uint32_t W = (n + 31) / 32;
    uint32_t gw = 0, lw = 0;  // this lane's words (w = lane)
    for (uint32_t w = 0; w < W; ++w) {
        const uint32_t i = w * 32u + lane;
        const float k = i < n ? keys[b + i] : 0.0f;  // coherent: moved here
        const uint32_t gb = __ballot_sync(0xffffffffu, i < n && !(k < cut));
        const uint32_t lb = __ballot_sync(0xffffffffu, i < n && !(k > cut));
        if (lane == w) {
            gw = gb;
            lw = lb;
        }
    }
    uint32_t ge_tot, le_tot;
    const uint32_t pge = warp_excl_scan((uint32_t)__popc(gw), &ge_tot);
    const uint32_t ple = warp_excl_scan((uint32_t)__popc(lw), &le_tot);
    // s = max over x of min(#>= in [0,x), #<= in [x,n)): it lies in the first word at whose end
    // f >= g (f rises, g falls)
    uint32_t s = 0;
    if (W > 0) {
        const bool cross = lane < W && pge + (uint32_t)__popc(gw) >= le_tot - ple - (uint32_t)__popc(lw);
        const uint32_t cb = __ballot_sync(0xffffffffu, cross);
        const int w = cb ? __ffs(cb) - 1 : (int)W - 1;
        uint32_t f = __shfl_sync(0xffffffffu, pge, w), g = le_tot - __shfl_sync(0xffffffffu, ple, w);
        uint32_t a = __shfl_sync(0xffffffffu, gw, w), c = __shfl_sync(0xffffffffu, lw, w);
        s = min(f, g);
        for (int q = 0; q < 32; ++q) {
            f += a & 1u;
            g -= c & 1u;
            a >>= 1;
            c >>= 1;
            s = max(s, min(f, g));
        }
    }
    uint32_t i = n;  // split index, n when every key is below the cut
    if (ge_tot > s) i = min(i, warp_mask_select(gw, pge, W, s));
    if (s >= 1) i = min(i, warp_mask_select(lw, ple, W, le_tot - s));
    for (uint32_t k0 = 0; k0 < s; k0 += 32) {
        const uint32_t k = k0 + lane;
        const uint32_t kk = k < s ? k : s - 1;  // every lane runs the selects (shuffles)
        const uint32_t pa = b + warp_mask_select(gw, pge, W, kk);
        const uint32_t pb = b + warp_mask_select(lw, ple, W, le_tot - 1 - kk);
        if (k < s) {
            const float xa = v.x[pa], xb = v.x[pb], ya = v.y[pa], yb = v.y[pb];
            const float za = v.z[pa], zb = v.z[pb];
            v.x[pa] = xb;
            v.x[pb] = xa;
            v.y[pa] = yb;
            v.y[pb] = ya;
            v.z[pa] = zb;
            v.z[pb] = za;
            if (v.idx) {
                const uint32_t ia = v.idx[pa], ib = v.idx[pb];
                v.idx[pa] = ib;
                v.idx[pb] = ia;
            }
        }
    }
    __syncwarp();  // the swaps are visible to lane 0's final swap
    if (lane == 0) {
        bytes += (v.idx ? 64ull : 48ull) * s + 4ull * n;
        finish_cell(v, slot, i, true);
    }
    __syncwarp();
}

// Levels below a cell in a full build: log2 of its leaf count (d is a power of two).
__device__ __forceinline__ int levels_below(const orb_cell_t &c) {
    return c.nLeafCells > 1 ? 31 - __clz((uint32_t)c.nLeafCells) : 0;
}

// Flag for k_subtree: every cell of the level fits a CTA and has at most `max_levels`
// (<= kSubLevels, the descendant queue) levels below it. One CTA.
constexpr int kSubLevels = kSubMaxLevels;
static_assert((2 << (kSubLevels - 1)) <= kSubQueue, "the last level's children fit the queue");
__global__ void __launch_bounds__(1024) k_subtree_check(Level v, int max_levels) {
    pdl_enter();
    __shared__ uint32_t sh[96];
    uint32_t mx = 0, ml = 0;
    for (int c = threadIdx.x; c < v.C; c += blockDim.x) {
        const int slot = level_slot(v, c);
        const uint2 rg = v.ranges[slot];
        mx = max(mx, rg.y - rg.x);
        ml = max(ml, (uint32_t)levels_below(v.heap[slot]));
    }
    mx = block_max(mx, sh);
    ml = block_max(ml, sh);
    if (v.win_cnt)
        for (int w = threadIdx.x; w < kMaxWindows; w += blockDim.x) v.win_cnt[w] = 0u;
    if (threadIdx.x == 0) {
        const uint32_t take = mx <= kSubMax && (int)ml <= min(max_levels, kSubLevels) ? 1u : 0u;
        *v.skip = take;
        v.counters->sub_next = 0u;  // the subtree kernel's work queue starts at the level's first cell
        if (v.hwin) {
            __threadfence_system();
            *(volatile uint32_t *)&v.hwin->decision = take ? 1u : 2u;
        }
    }
}

// One CTA per cell of the level: every level below it (its leaf count's log2), breadth
// first; with window reports (v.hwin), the last cell of each window reports it to the host.
// kWarpSmall: cells of at most kWarpKeys particles go to one warp each (the CTA's warps side
// by side); without it every cell is the whole CTA's (the instance for trees whose cells
// never get that small keeps its registers for the CTA path). Same results either way.
template <bool kWarpSmall>
__global__ void __launch_bounds__(kSubThreads, 4) k_subtree(Level v) {
    pdl_enter();
    __shared__ SubSmem sm;
    if (*(volatile const uint32_t *)v.skip == 0u) return;  // the level kernels run instead
    unsigned long long bytes = 0;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (int k = 0;; ++k) {
        // root cells: from a queue where cells can be small or uneven (CTAs that finish small
        // cells take more), else one in gridDim.x
        int c;
        if constexpr (kWarpSmall) {
            if (threadIdx.x == 0) sm.root = (int)atomicAdd(&v.counters->sub_next, 1u);
            __syncthreads();
            c = sm.root;
        } else {
            c = (int)blockIdx.x + k * (int)gridDim.x;
        }
        if (c >= v.C) break;
        int cur = 0, nq = 1;
        const int root = level_slot(v, c);
        const int levels = levels_below(v.heap[root]);
        if (threadIdx.x == 0) sm.queue[0][0] = root;
        __syncthreads();
        for (int l = 0; l < levels; ++l) {
            // children of queue entry q at 2q, 2q+1 of the next level's queue (the warp path:
            // here, before the cells are processed in any order; else after each cell below)
            if (kWarpSmall && (int)threadIdx.x < nq && 2 * (int)threadIdx.x + 2 <= kSubQueue) {
                const int slot = sm.queue[cur][threadIdx.x];
                const int id = v.heap[slot].id;
                sm.queue[cur ^ 1][2 * threadIdx.x] = slot + id + 1;
                sm.queue[cur ^ 1][2 * threadIdx.x + 1] = slot + id + 2;
            }
            // cells of more than kWarpKeys particles by the whole CTA, one after the other
            for (int q = 0; q < nq; ++q) {
                const int slot = sm.queue[cur][q];
                const uint2 rg = v.ranges[slot];
                if (kWarpSmall && rg.y - rg.x <= (uint32_t)kWarpKeys) continue;  // CTA-uniform
                sub_bisect(v, slot, sm, bytes);
                sub_partition(v, slot, sm, bytes);
                if (!kWarpSmall && threadIdx.x == 0 && 2 * q + 2 <= kSubQueue) {
                    const int id = v.heap[slot].id;
                    sm.queue[cur ^ 1][2 * q] = slot + id + 1;
                    sm.queue[cur ^ 1][2 * q + 1] = slot + id + 2;
                }
            }
            // the small ones by one warp each, the CTA's warps side by side
            for (int q = (int)warp; kWarpSmall && q < nq; q += (int)nwarps) {
                const int slot = sm.queue[cur][q];
                const uint2 rg = v.ranges[slot];
                if (rg.y - rg.x > (uint32_t)kWarpKeys) continue;  // warp-uniform
                warp_bisect_cell(v, slot, lane, bytes);
                warp_partition_cell(v, slot, lane, bytes);
            }
            __syncthreads();
            cur ^= 1;
            nq = 2 * nq;
        }
        if (v.hwin) {
            // the cell is final: every thread's writes made visible beyond the GPU, then the
            // last cell of its window reports the window's particle range to the host
            __threadfence_system();
            __syncthreads();
            if (threadIdx.x == 0) {
                const uint32_t w = (uint32_t)c / v.win_cells;
                const uint32_t first = w * v.win_cells, last = min(first + v.win_cells, (uint32_t)v.C) - 1u;
                if (atomicAdd(&v.win_cnt[w], 1u) == last - first) {
                    __threadfence_system();
                    const uint2 r = make_uint2(v.ranges[level_slot(v, (int)first)].x,
                                               v.ranges[level_slot(v, (int)last)].y);
                    volatile uint32_t *hr = &v.hwin->range[w].x;
                    hr[0] = r.x;
                    hr[1] = r.y;
                    __threadfence_system();
                    *(volatile uint32_t *)&v.hwin->done[w] = 1u;
                }
            }
        }
    }
    // lane 0 of every warp counted the small cells its warp finished (thread 0 the rest too)
    if (lane == 0 && bytes) add_bytes(v, kKSubtree, bytes);
}

// ------------------------------------------------------------------------------------
// Weighted builds: the reference's bisection loop on integer weight sums instead of counts
// (the thesis's weighted ORB, documentation/notes.tex:259-271; never implemented by the
// reference). Per level: every cell starts active; kWPasses passes each bin the weights of
// every active cell's bracket into its midpoint tree of depth kWBinsLog2 (the exact
// descent: the reference's own cuts) and sum the weights below the bracket; a resolve per
// cell replays up to kWBinsLog2 iterations of the loop on the prefix sums with the weighted
// test. Integer sums: the same results in any order.
// ------------------------------------------------------------------------------------
__global__ void k_wstart(Level v) {
    pdl_enter();
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < (uint32_t)v.C;
         c += gridDim.x * blockDim.x) {
        v.state[c] = kActive;
        v.iters[c] = 0;
        v.wbelow[c] = 0ull;
        v.wtot[c] = 0ull;
    }
    const uint64_t nb = (uint64_t)v.C * kWBins;
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nb;
         j += (uint64_t)gridDim.x * blockDim.x)
        v.whist[j] = 0ull;
}

__device__ __forceinline__ unsigned long long block_sum_u64(unsigned long long x,
                                                            unsigned long long *sh) {
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0) sh[warp] = x;
    __syncthreads();
    unsigned long long t = 0;
    for (int w = 0; w < nw; ++w) t += sh[w];
    return t;
}

__global__ void __launch_bounds__(kThreads) k_whist(Level v) {
    pdl_enter();
    __shared__ unsigned long long s_bins[kWBins];
    __shared__ unsigned long long s_red[kThreads / 32];
    const uint32_t total = v.tile_off[v.C];
    unsigned long long bytes = 0, wkeys = 0;  // this thread's bracket weight reads; the CTA's keys
    for (uint32_t t = blockIdx.x; t < total; t += gridDim.x) {
        const TileRef tr = tile_ref(v, t);
        if (v.state[tr.c] != kActive) continue;  // block-uniform
        const orb_cell_t &cell = v.heap[tr.slot];
        const float L = cell.cutMarginLeft, R = cell.cutMarginRight;
        const float *keys = axis_keys(v, eff_axis(cell.cutAxis));
        for (uint32_t j = threadIdx.x; j < (uint32_t)kWBins; j += blockDim.x) s_bins[j] = 0ull;
        __syncthreads();
        unsigned long long below = 0, tot = 0;
        // kWLoads keys of a thread in flight per round. The first pass reads every weight
        // (the cell's total and the weight below its bracket); later passes read the weights
        // of the keys inside the bracket only (the weight below it is carried by k_wresolve).
        constexpr int kWLoads = 4;
        const uint32_t nt = blockDim.x;
        const bool first = v.pass == 0;
        for (uint32_t p0 = tr.e0 + threadIdx.x; p0 < tr.e1; p0 += nt * kWLoads) {
            float k[kWLoads];
            uint32_t w[kWLoads];
#pragma unroll
            for (int u = 0; u < kWLoads; ++u) {
                const uint32_t p = p0 + (uint32_t)u * nt;
                k[u] = p < tr.e1 ? __ldg(keys + p) : L;
                w[u] = first && p < tr.e1 ? __ldg(v.wt + p) : 0u;
            }
#pragma unroll
            for (int u = 0; u < kWLoads; ++u) {
                const uint32_t p = p0 + (uint32_t)u * nt;
                if (p >= tr.e1) continue;
                if (first) {
                    tot += w[u];
                    if (k[u] < L) below += w[u];
                }
                if (k[u] >= L && k[u] < R) {
                    const uint32_t wk = first ? w[u] : __ldg(v.wt + p);
                    if (wk) atomicAdd(&s_bins[tree_bin(k[u], L, R, kWBinsLog2)], (unsigned long long)wk);
                    if (!first) ++bytes;  // a weight read (counted in 4-byte units below)
                }
            }
        }
        if (first) {
            below = block_sum_u64(below, s_red);
            tot = block_sum_u64(tot, s_red);
        }
        __syncthreads();
        unsigned long long *g = v.whist + (size_t)tr.c * kWBins;
        for (uint32_t j = threadIdx.x; j < (uint32_t)kWBins; j += blockDim.x)
            if (s_bins[j]) atomicAdd(&g[j], s_bins[j]);
        if (threadIdx.x == 0 && first) {
            if (below) atomicAdd(&v.wbelow[tr.c], below);
            if (tot) atomicAdd(&v.wtot[tr.c], tot);
        }
        if (threadIdx.x == 0) wkeys += tr.e1 - tr.e0;
        __syncthreads();  // s_bins reused by the next tile
    }
    // 4 B per key read (every pass), 4 B per weight read (every key in the first pass, the
    // bracket's keys after it): per thread in-bracket weight reads summed over the block
    const unsigned long long wr = v.pass == 0 ? 0ull : block_sum_u64(bytes, s_red);
    if (threadIdx.x == 0) {
        const unsigned long long b = 4ull * wkeys * (v.pass == 0 ? 2ull : 1ull) + 4ull * wr;
        if (b) add_bytes(v, kKWHist, b);
    }
}

// A warp per cell: the replay of up to kWBinsLog2 iterations of src/orbit.cpp:146-232 on the
// pass's weight bins, with the weighted test; the bins and the weight below are cleared for
// the next pass.
__global__ void __launch_bounds__(kThreads) k_wresolve(Level v) {
    pdl_enter();
    __shared__ unsigned long long s_pre[kThreads / 32][kWBins];
    const int c = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (c >= v.C) return;
    if (v.state[c] != kActive) return;  // warp-uniform
    unsigned long long *pre = s_pre[threadIdx.x >> 5];
    unsigned long long *g = v.whist + (size_t)c * kWBins;
    constexpr int kPer = kWBins / 32;
    unsigned long long loc[kPer], run = 0;
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
        loc[j] = g[lane * kPer + j];
        g[lane * kPer + j] = 0ull;
        run += loc[j];
    }
    // exclusive prefix of the lanes' runs
    unsigned long long inc = run;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    unsigned long long acc = inc - run;
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
        pre[lane * kPer + j] = acc;
        acc += loc[j];
    }
    __syncwarp();
    const int slot = level_slot(v, c);
    orb_cell_t &cell = v.heap[slot];
    const uint2 rg = v.ranges[slot];
    const uint32_t n = rg.y - rg.x;
    const unsigned long long W = v.wtot[c], below = v.wbelow[c];
    float L = cell.cutMarginLeft, R = cell.cutMarginRight;
    uint32_t it = v.iters[c], pos = 0, width = kWBins;
    uint8_t st = kActive;
    for (int step = 0; step < kWBinsLog2; ++step) {
        if (it >= (uint32_t)kMaxIterations) {
            st = kCapped;
            break;
        }
        const uint32_t half = width >> 1;
        const unsigned long long wl = below + pre[pos + half];
        ++it;
        const int dir = convergence_weighted(wl, W, n, cell.nLeafCells);
        if (dir == 0) {
            st = kFound;
            break;
        }
        const float cut = mid_cut(L, R);
        if (dir > 0) {
            R = cut;
        } else {
            L = cut;
            pos += half;
        }
        width = half;
    }
    if (st == kActive && it >= (uint32_t)kMaxIterations) st = kCapped;
    __syncwarp();
    if (lane == 0) {
        cell.cutMarginLeft = L;
        cell.cutMarginRight = R;
        cell.foundCut = st == kFound ? 1 : 0;
        v.iters[c] = (uint8_t)it;
        v.state[c] = st;
        // the weight below the new bracket [L, R): below the old one plus the bins left of it
        v.wbelow[c] = below + pre[pos];
        if (st != kActive) atomicMax(&v.counters->max_iters, it);
        if (st == kCapped) atomicAdd(&v.counters->unfound, 1u);
    }
}

// ------------------------------------------------------------------------------------
// Service count-left: one plain pass at getCut() per cell, found cells skipped.
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_count_left(Level v) {
    pdl_enter();
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

// The reference's xorshf96 stream (src/services/init.cu:11-25): thread g continues the
// stream from starts[g] (its state after g * chunk draws, computed on the host by a GF(2)
// jump) for `chunk` draws; draw j is coordinate j % 3 of particle j / 3. Value:
// (float)z / 2^64 - 0.5 (exact scaling, then the subtraction rounded once: the reference's
// double subtraction rounded to float gives the same float).
__global__ void k_gen_xorshf96(const unsigned long long *starts, uint64_t draws, uint32_t chunk,
                               float *x, float *y, float *z) {
    const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t j0 = g * chunk;
    if (j0 >= draws) return;
    unsigned long long sx = starts[3 * g], sy = starts[3 * g + 1], sz = starts[3 * g + 2];
    const uint64_t j1 = min(draws, j0 + chunk);
    float *dst[3] = {x, y, z};
    for (uint64_t j = j0; j < j1; ++j) {
        sx ^= sx << 16;
        sx ^= sx >> 5;
        sx ^= sx << 1;
        const unsigned long long t = sx;
        sx = sy;
        sy = sz;
        sz = t ^ sx ^ sy;
        const float q = __fmul_rn(__ull2float_rn(sz), 0x1p-64f);
        dst[j % 3][j / 3] = __fsub_rn(q, 0.5f);
    }
}

__global__ void k_copy_instances(const uint32_t *src, uint32_t *dst, const BatchRoot *roots, int k) {
    for (int i = blockIdx.y; i < k; i += gridDim.y) {
        const BatchRoot r = roots[i];
        for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < r.n; p += gridDim.x * blockDim.x)
            dst[r.offset + p] = src[r.offset + p];
    }
}

// Box-Muller pairs from the counter-based stream: coordinate a of particle i uses draws
// (seed, 2*(3i+a)) and (seed, 2*(3i+a)+1).
__global__ void k_displace(float *x, float *y, float *z, uint64_t offset, uint64_t n,
                           uint64_t seed, float sigma, float lo0, float lo1, float lo2,
                           float hi0, float hi1, float hi2) {
    const uint64_t sm = mix64(seed);
    float *c[3] = {x, y, z};
    const float lo[3] = {lo0, lo1, lo2};
    const float hi[3] = {nextafterf(hi0, lo0), nextafterf(hi1, lo1), nextafterf(hi2, lo2)};
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        for (int a = 0; a < 3; ++a) {
            const uint64_t q = 2 * (3 * i + a);
            const float u1 = ((float)(uint32_t)(draw(sm, q) >> 40) + 1.0f) * 0x1p-24f;  // (0, 1]
            const float u2 = (float)(uint32_t)(draw(sm, q + 1) >> 40) * 0x1p-24f;       // [0, 1)
            const float g = sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
            const float p = c[a][offset + i] + sigma * g;
            c[a][offset + i] = fminf(fmaxf(p, lo[a]), hi[a]);
        }
    }
}

__global__ void k_iota_u32(uint32_t *dst, uint64_t n) {
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n;
         p += (uint64_t)gridDim.x * blockDim.x)
        dst[p] = (uint32_t)p;
}

__global__ void k_gather_u32(uint32_t *dst, const uint32_t *src, const uint32_t *perm, uint64_t off,
                             uint64_t n) {
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n;
         p += (uint64_t)gridDim.x * blockDim.x)
        dst[off + p] = src[off + perm[off + p]];
}

#ifndef ORB_GATHER_QUADS
#define ORB_GATHER_QUADS 4  // quads of a thread in flight in the stage gather
#endif
// Staged builds from host memory: a coordinate that arrived after the first levels moved the
// other coordinates takes their order through the permutation, dst[p] = src[idx[p]].
__global__ void __launch_bounds__(256) k_stage_gather(float *__restrict__ dst, const float *__restrict__ src,
                                                      const uint32_t *__restrict__ idx, uint64_t n,
                                                      BuildCounters *ctr) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t n4 = n / 4;  // dst and idx are 16-byte aligned allocations
    const uint4 *idx4 = reinterpret_cast<const uint4 *>(idx);
    float4 *dst4 = reinterpret_cast<float4 *>(dst);
    // kQ quads per thread and step: all index loads, then all 4 kQ gathers, in flight
    constexpr int kQ = ORB_GATHER_QUADS;
    uint64_t q = g;
    for (; q + (kQ - 1) * stride < n4; q += kQ * stride) {
        uint4 i[kQ];
#pragma unroll
        for (int u = 0; u < kQ; ++u) i[u] = idx4[q + u * stride];
        float4 a[kQ];
#pragma unroll
        for (int u = 0; u < kQ; ++u) a[u] = make_float4(src[i[u].x], src[i[u].y], src[i[u].z], src[i[u].w]);
#pragma unroll
        for (int u = 0; u < kQ; ++u) dst4[q + u * stride] = a[u];
    }
    for (; q < n4; q += stride) {
        const uint4 i = idx4[q];
        dst4[q] = make_float4(src[i.x], src[i.y], src[i.z], src[i.w]);
    }
    for (uint64_t p = n4 * 4 + g; p < n; p += stride) dst[p] = src[idx[p]];
    // per particle: its index and the gathered value read, the value written
    if (g == 0) atomicAdd(&ctr->bytes[kKStageGather], 12ull * n);
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
void launch_init_batch(const Level &v, const BatchRoot *roots, int k, uint64_t n_total,
                       cudaStream_t st) {
    (void)n_total;
    if (k > 0) k_init_batch<<<dim3(64, (unsigned)(k < 65535 ? k : 65535)), 256, 0, st>>>(v, roots, k);
}

void launch_init(const Level &v, uint64_t n, const float lower[3], const float upper[3],
                 uint32_t d, int heap_cells, cudaStream_t st) {
    uint64_t work = n > (uint64_t)heap_cells * 13 ? n : (uint64_t)heap_cells * 13;
    k_init<<<grid_for(work, 256, 152 * 16), 256, 0, st>>>(v, (uint32_t)n, lower[0], lower[1],
                                                        lower[2], upper[0], upper[1], upper[2], d,
                                                        heap_cells);
}

// A level kernel on the stream, with the programmatic-dependent-launch attribute when the
// context uses it (the kernels wait for their predecessor in pdl_enter()).
template <class... P, class... A>
void launch_kernel(bool pdl, void (*kern)(P...), dim3 grid, dim3 block, size_t smem,
                   cudaStream_t st, A... args) {
    if (!pdl) {
        kern<<<grid, block, smem, st>>>(args...);
        return;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kern, args...);
}

void launch_level_kernel(Kernel k, const Level &v, int grid, int arg, cudaStream_t st) {
    const bool p = v.pdl != 0;
    const dim3 T(kThreads);
    const unsigned per_cell_warps = (unsigned)grid_for((uint64_t)v.C * 32, kThreads, 1 << 30);
    switch (k) {
        case kKPlan: launch_kernel(p, k_plan, dim3(1), dim3(1024), 0, st, v); break;
        case kKHist:  // arg: 1 first pass, all cells dense; 2 first pass of a sampled level
            if (arg == 1)
                launch_kernel(p, k_hist<kHFirstDense>, dim3(grid), T, 0, st, v);
            else if (arg == 2)
                launch_kernel(p, k_hist<kHFirstSampled>, dim3(grid), T, 0, st, v);
            else
                launch_kernel(p, k_hist<kHRest>, dim3(grid), T, 0, st, v);
            break;
        case kKBisectTile: launch_kernel(p, k_bisect_tile, dim3(grid), T, 0, st, v); break;
        case kKWarmStart:
            launch_kernel(p, k_warm_start, dim3(grid_for((uint64_t)v.C, kThreads, 1 << 30)), T, 0, st, v);
            break;
        case kKSubtreeCheck: launch_kernel(p, k_subtree_check, dim3(1), dim3(1024), 0, st, v, arg); break;
        case kKSubtree:  // arg: 1 when cells of at most kWarpKeys particles can occur
            if (arg)
                launch_kernel(p, k_subtree<true>, dim3(grid), dim3(kSubThreads), 0, st, v);
            else
                launch_kernel(p, k_subtree<false>, dim3(grid), dim3(kSubThreads), 0, st, v);
            break;
        case kKBisectCta:
            launch_kernel(p, k_bisect_cta, dim3(grid), dim3(kCtaThreads), kCtaSmemBytes, st, v);
            break;
        case kKTileMap: launch_kernel(p, k_tile_map, dim3(grid), T, 0, st, v); break;
        case kKResolve: launch_kernel(p, k_resolve, dim3(per_cell_warps), T, 0, st, v); break;
        case kKPartClassify: launch_kernel(p, k_part_classify, dim3(grid), T, 0, st, v); break;
        case kKPartScan: launch_kernel(p, k_tile_scan, dim3(arg), dim3(kScanBlock), 0, st, v); break;
        case kKPartCells: launch_kernel(p, k_part_cells, dim3(per_cell_warps), T, 0, st, v); break;
        case kKPartSwap:
            if (v.wt)
                launch_kernel(p, k_part_swap<true, 3>, dim3(grid), dim3(kSwapThreads), 0, st, v);
            else if (!v.y)
                launch_kernel(p, k_part_swap<false, 0>, dim3(grid), dim3(kSwapThreads), 0, st, v);
            else if (!v.z)
                launch_kernel(p, k_part_swap<false, 1>, dim3(grid), dim3(kSwapThreads), 0, st, v);
            else
                launch_kernel(p, k_part_swap<false, 3>, dim3(grid), dim3(kSwapThreads), 0, st, v);
            break;
        case kKWStart: launch_kernel(p, k_wstart, dim3(grid), T, 0, st, v); break;
        case kKWHist: launch_kernel(p, k_whist, dim3(grid), T, 0, st, v); break;
        case kKWResolve: launch_kernel(p, k_wresolve, dim3(per_cell_warps), T, 0, st, v); break;
        case kKPartFinish:
            launch_kernel(p, k_part_finish, dim3(grid_for(v.C, kThreads, 1 << 30)), T, 0, st, v, arg);
            break;
        case kKCountLeft: launch_kernel(p, k_count_left, dim3(grid), T, 0, st, v); break;
        case kKSample:
            launch_kernel(p, k_sample_bin, dim3(kSampleMax / kSamplePerCta, (unsigned)min(v.C, 65535)),
                          dim3(kSampleThreads), 0, st, v);
            break;
        case kKSamplePick:
            launch_kernel(p, k_sample_pick, dim3((unsigned)min(v.C, 65535)), dim3(kPickThreads), 0, st, v);
            break;
        default: break;
    }
}

cudaError_t configure_kernels() {
    return cudaFuncSetAttribute(k_bisect_cta, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)kCtaSmemBytes);
}

int swap_blocks_per_sm() {
    // the swap's CTAs walk the tiles grid-stride: one resident wave, none waiting behind it
    static const int blocks = [] {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_part_swap<false, 3>, kSwapThreads, 0) != cudaSuccess ||
            b < 1) {
            cudaGetLastError();
            b = ORB_SWAP_MIN_BLOCKS;
        }
        return b;
    }();
    return blocks;
}

void launch_copy_instances(const uint32_t *src, uint32_t *dst, const BatchRoot *roots, int k,
                           cudaStream_t st) {
    if (k > 0)
        k_copy_instances<<<dim3(64, (unsigned)(k < 65535 ? k : 65535)), 256, 0, st>>>(src, dst, roots, k);
}

void launch_displace(float *x, float *y, float *z, uint64_t offset, uint64_t n, uint64_t seed,
                     float sigma, const float lower[3], const float upper[3], cudaStream_t st) {
    if (n == 0) return;
    k_displace<<<grid_for(n, 256, 152 * 16), 256, 0, st>>>(x, y, z, offset, n, seed, sigma, lower[0],
                                                          lower[1], lower[2], upper[0], upper[1],
                                                          upper[2]);
}

void launch_iota_u32(uint32_t *dst, uint64_t n, cudaStream_t st) {
    if (n) k_iota_u32<<<grid_for(n, 256, 152 * 16), 256, 0, st>>>(dst, n);
}

void launch_stage_gather(float *dst, const float *src, const uint32_t *idx, uint64_t n,
                         BuildCounters *ctr, int num_sms, cudaStream_t st) {
    if (n) k_stage_gather<<<grid_for((n + 3) / 4, 256, num_sms * 8), 256, 0, st>>>(dst, src, idx, n, ctr);
}

void launch_gather_u32(uint32_t *dst, const uint32_t *src, const uint32_t *perm, uint64_t off,
                       uint64_t n, cudaStream_t st) {
    if (n) k_gather_u32<<<grid_for(n, 256, 152 * 16), 256, 0, st>>>(dst, src, perm, off, n);
}

void launch_gen_xorshf96(const unsigned long long *starts, uint64_t draws, uint32_t chunk,
                         float *x, float *y, float *z, cudaStream_t st) {
    const uint64_t threads = (draws + chunk - 1) / chunk;
    k_gen_xorshf96<<<(unsigned)((threads + 127) / 128), 128, 0, st>>>(starts, draws, chunk, x, y, z);
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
