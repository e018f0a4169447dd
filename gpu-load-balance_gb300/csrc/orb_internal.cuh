// Internal declarations of the ORB engine: device helpers shared by the kernels and the
// launch interface the host driver uses. Nothing here is part of the C ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "orb/orb.h"
#include "orb_leaf_ratio.h"

namespace orb {

static_assert(sizeof(orb_cell_t) == 52, "orb_cell_t must keep the reference's 52-byte Cell layout");

constexpr int kMaxIterations = 32;   // bisection cap, src/orbit.cpp:149
constexpr int kTile = 16384;         // keys per tile of the count-left passes
constexpr int kPTile = 4096;         // positions per tile of the partition passes
constexpr int kPWords = kPTile / 32; // bitmask words per partition tile
constexpr int kMaxBinsLog2 = 11;     // deepest midpoint tree one histogram pass resolves
// Histogram passes per level. The count passes bisect cells of more than kTile keys, whose
// trees have depth 11 (tree_depth), so 3 passes (33 iterations) reach the 32-iteration cap
// of every cell. A first pass that is discarded (a warm or sampled bracket that missed the
// cut) costs one more, hence 4 for levels that may have one.
constexpr int kHistPasses = 4;
constexpr int kColdHistPasses = 3;
constexpr int kThreads = 256;
// resident CTAs of the count-left pass (its launch bound: 65536 / (256 x 6) = 40 registers)
#ifndef ORB_HIST_BLOCKS_PER_SM
#define ORB_HIST_BLOCKS_PER_SM 6
#endif
constexpr int kHistBlocksPerSm = ORB_HIST_BLOCKS_PER_SM;
constexpr int kTileBlocksPerSm = 4;  // resident CTAs of the one-tile cell bisection
constexpr int kSubtreeBlocksPerSm = 4;  // CTAs of the subtree kernel per SM (its grid)
#ifndef ORB_SUB_MAX
#define ORB_SUB_MAX 34816  // 2^15 + 2048: a 2^27-particle tree takes its last 4 levels
#endif
constexpr uint32_t kSubMaxParticles = ORB_SUB_MAX;  // largest cell one subtree CTA takes
constexpr int kSubMaxLevels = 6;              // deepest tree one subtree CTA finishes

// Weighted builds: every active cell's bracket is binned into a midpoint tree of this depth
// per pass (its weights summed per bin), so kWPasses passes reach the 32-iteration cap.
constexpr int kWBinsLog2 = 8;
constexpr int kWBins = 1 << kWBinsLog2;
constexpr int kWPasses = 4;
static_assert(kWPasses * kWBinsLog2 >= 32, "the weighted passes reach the iteration cap");

// kSmall: at most kWarpKeys keys (one warp bisects it); kOneTile: at most kTile keys (one CTA)
enum CellState : uint8_t { kActive = 0, kFound = 1, kCapped = 2, kSmall = 3, kOneTile = 4 };
constexpr int kWarpKeys = 1024;      // cells up to this size bisect in one warp's registers
// Polls of a decoupled look-back wait (64 ns apart) before it gives up: about 0.3 s, far
// beyond any real wait; the kernel then flags the error and finishes its work.
constexpr uint32_t kLookbackSpinLimit = 1u << 22;

// Kernel kinds, for launch counting, event timing and algorithmic-byte accounting.
enum Kernel : int {
    kKInit = 0,
    kKPlan,
    kKHist,
    kKResolve,
    kKPartClassify,
    kKPartScan,
    kKPartCells,
    kKPartSwap,
    kKPartFinish,
    kKCountLeft,
    kKGenerate,
    kKBisectCta,
    kKTileMap,
    kKBisectTile,
    kKWarmStart,
    kKSubtreeCheck,
    kKSubtree,
    kKSample,
    kKSamplePick,
    kKWStart,
    kKWHist,
    kKWResolve,
    kKStageGather,
    kNumKernels
};
static_assert(kNumKernels <= 32, "BuildCounters::bytes holds 32 kernel kinds");
extern const char *const kKernelNames[kNumKernels];

// Device-side counters of one build (read back at the end).
struct BuildCounters {
    uint32_t degenerate;
    uint32_t zero_volume;
    uint32_t unfound;
    uint32_t max_iters;
    uint32_t any_active[2];  // pass p: cleared by hist p, set by resolve p if a cell goes on
    uint32_t error;       // set when a bounded device wait gave up
    uint32_t ticket;      // block ticket of the tile scan (reset before each launch)
    uint32_t warm_cells;  // warm builds: cells that started from a hinted bracket
    uint32_t warm_resets; // ... whose hinted bracket missed the target (restarted cold)
    uint32_t pred_cells;  // cells whose first count pass used a sampled bracket
    uint32_t pred_misses; // ... whose sampled bracket did not hold the cut (binned again)
    uint32_t sub_next;    // next root cell of the subtree kernel's work queue
    unsigned long long bytes[32];  // algorithmic bytes per Kernel kind
};

// Builds from host memory: the subtree kernel reports, per window of consecutive root cells,
// when every cell of the window is final, into pinned host memory that the host polls while
// the kernel runs; the host then copies the window's particles back while later windows are
// still being built.
constexpr int kMaxWindows = 64;
struct HostWindows {
    uint32_t decision;           // 0 not yet, 1 the subtree kernel finishes the tree, 2 refused
    uint32_t done[kMaxWindows];  // 1: window w final, its particles in range[w]
    uint2 range[kMaxWindows];
};

// Everything a level's kernels need. Cells of the level are heap slots [base, base + C)
// unless `slots` is non-null (service calls over an arbitrary cell list).
struct Level {
    float *x, *y, *z;
    uint32_t *idx;          // original particle index (perm), may be null
    orb_cell_t *heap;
    uint2 *ranges;          // {begin, end} per heap slot, absolute positions
    const int *slots;       // optional explicit slot list [C]
    int base;
    int C;
    int pass;               // histogram pass index within the level
    int last_pass;          // index of the level's last histogram pass
    // plan
    uint32_t *tile_off;     // [C+1] first tile of each cell
    uint32_t *htile_cell;   // [tiles] cell of each count-left tile (null: binary search)
    uint32_t *ptile_cell;   // [ptiles] cell of each partition tile (null: binary search)
    uint32_t *hist_off;     // [C+1] first bin of each cell in the histogram pool
    uint8_t *hist_k;        // [C]   tree depth of each cell's histogram
    uint8_t *state;         // [C]   CellState
    uint8_t *iters;         // [C]   bisection iterations done
    uint32_t *hist;         // histogram pool (kept all-zero between passes)
    uint32_t *below;        // [C]   keys below the left margin in the current pass
    uint32_t *inb;          // [C]   keys inside the current bracket (n before the first pass)
    // in-bracket compaction: a sparse pass also writes its bracket keys to the cell's list;
    // every later pass of the cell reads the list only (count below L carried by resolve)
    uint32_t *cmp_off;      // [C+1] first list slot of each cell (capacity = difference)
    uint32_t *cmp_cnt;      // [C]   keys written to the list
    float *cmp_keys;        // the lists
    uint8_t *listed;        // [C]   1: this pass reads the cell's list instead of its keys
    uint8_t *cmp_bad;       // [C]   1: a tile's bracket keys overflowed (no list)
    // sampled first pass: leaves [lo, hi) of the first pass's midpoint tree predicted to hold
    // the cut (k_sample_bin, k_sample_pick); that pass counts the keys below leaf lo and bins
    // only the keys of [lo, hi). Packed (lo | hi << 12 | flags); 0: no prediction (dense)
    uint32_t *pred;         // [C]
    float pred_sigmas;      // half-width of the sampled bracket in standard errors (0: off)
    // partition
    uint32_t *ptile_off;    // [C+1] first partition tile of each cell
    uint32_t *ge_bits;      // [ptiles * kPWords] bit p: key >= cut
    uint32_t *le_bits;      // [ptiles * kPWords] bit p: key <= cut
    uint32_t *pt_ge;        // [ptiles] set bits per tile
    uint32_t *pt_le;
    uint32_t *pt_ge_pre;    // [ptiles+1] exclusive prefix over all tiles of the level
    uint32_t *pt_le_pre;
    unsigned long long *pt_status;  // look-back status word per scan block (zeroed per level)
    uint32_t *ticket;       // block ticket counter of the tile scan
    uint32_t *part_s;       // [C] number of Hoare swaps
    uint32_t *part_i;       // [C] split index (cell-relative); n when clamped
    uint32_t *part_le;      // [C] keys <= cut in the cell
    uint32_t *out_counts;   // service calls: per-cell result
    uint32_t sparse_per_tile;  // count pass: sparse once the bracket holds <= this x tiles keys
    uint32_t spin_limit;    // polls of one look-back wait before it gives up (error flag)
    int pdl;                // level kernels launched with programmatic dependent launch
    // warm builds (null otherwise): per heap slot the previous tree's cut and w x its extent
    // (x NaN: no hint) and that tree's cut axis
    const float2 *hint;     // (cut, w x extent) from the previous tree
    const int *hint_axis;
    uint8_t *warm;          // [C] 1 while a hinted bracket is not yet checked
    // subtrees: 1 when one CTA per cell finishes the tree from this level down (then the
    // level kernels of the levels below return at once); null when not attempted
    uint32_t *skip;
    // window reports (null otherwise): the host-mapped reports, a finished-cell counter per
    // window, root cells per window
    HostWindows *hwin;
    uint32_t *win_cnt;
    uint32_t win_cells;
    // weighted builds (null otherwise): an integer weight per particle, moved with it, and
    // per cell of the level its weight bins (kWBins), the weight below its bracket and its
    // total weight
    uint32_t *wt;
    unsigned long long *whist;
    unsigned long long *wbelow;
    unsigned long long *wtot;
    BuildCounters *counters;
};

__device__ __forceinline__ int level_slot(const Level &v, int c) {
    return v.slots ? v.slots[c] : v.base + c;
}

__device__ __forceinline__ int eff_axis(int a) { return a < 0 ? 0 : a; }

// getCut(), src/cell.h:74-76: float sum, halved (exact, no FMA, no FTZ).
__device__ __forceinline__ float mid_cut(float lo, float hi) {
    return __fmul_rn(__fadd_rn(hi, lo), 0.5f);
}

// src/orbit.cpp:204-208: difference = int(float(cl) - float(c) * ratio), found when
// |difference| < 3, else the right margin moves for a positive difference and the left one
// otherwise. ratio = leaf_ratio(nLeafCells) (0.5f when the leaf count is even). The
// uint->float roundings above 2^24 are kept. Returns 0 found, +1 right margin, -1 left.
__device__ __forceinline__ int convergence(uint32_t count_left, uint32_t count, float ratio) {
    float prod = __fmul_rn(__uint2float_rn(count), ratio);
    float diff = __fsub_rn(__uint2float_rn(count_left), prod);
    int difference = __float2int_rz(diff);
    if (difference > -3 && difference < 3) return 0;
    return difference > 0 ? 1 : -1;
}

// The weighted test (no counterpart in the reference, whose thesis specifies weighted ORB,
// documentation/notes.tex:259-271, and whose code never implements it): the reference's
// |W_left - ratio W| < 3 (src/orbit.cpp:204-208) with the tolerance scaled by the cell's
// mean weight W/n, exact in 128-bit integers: D = k W_left - ceil(k/2) W for k leaves;
// found when D == 0 or n |D| < 3 k W; else +1 (D > 0, the right margin moves) or -1. With
// unit weights: |cl - ratio c| < 3 exactly, the reference's float32 test wherever that test
// is exact (fewer than 2^24 particles, an even k).
__device__ __forceinline__ int convergence_weighted(unsigned long long w_left,
                                                    unsigned long long w_cell, uint32_t n,
                                                    int32_t n_leaf) {
    const __int128 k = n_leaf, half = (n_leaf + 1) / 2;
    const __int128 D = k * (__int128)w_left - half * (__int128)w_cell;
    const unsigned __int128 ad = (unsigned __int128)(D < 0 ? -D : D);
    if (D == 0 || (unsigned __int128)n * ad < (unsigned __int128)3 * (unsigned __int128)k * w_cell)
        return 0;
    return D > 0 ? 1 : -1;
}

__device__ __forceinline__ const float *axis_keys(const Level &v, int axis) {
    return axis == 0 ? v.x : (axis == 1 ? v.y : v.z);
}

// Level slices of the reference's driver for a root of d leaves (src/orbit.cpp:104-107,
// src/cell.h:65-72): level l (from 1) takes the heap cells [2^(l-1)-1, b_l] with
// b_l = min(getNCellsOnLastLevel(), 2^l) - 2, getNCellsOnLastLevel() = 2d - 2^ceil(log2 d).
// For a power of two that is every cell of the level. For other d the reference's loop
// stops at getNLevels() - 1 = ceil(log2 d) - 1, and a slice may come out partial or empty
// (b_l < 2^(l-1)-1; the reference then calls its services with a non-positive cell count,
// which is undefined; here such a level has no cells).
struct Slices {
    uint32_t depth;  // getNLevels()
    uint32_t last;   // getNCellsOnLastLevel()
    bool pow2;
    explicit Slices(uint32_t d) {
        depth = 0;
        while ((1ull << depth) < d) ++depth;
        last = (uint32_t)(2ull * d - (1ull << depth));
        pow2 = (d & (d - 1)) == 0;
    }
    // most split levels: log2(d) for a power of two, else the reference's bound
    uint32_t max_levels() const { return pow2 ? depth : (depth ? depth - 1 : 0); }
    int first(uint32_t l) const { return (1 << (l - 1)) - 1; }
    int count(uint32_t l) const {
        const int b = (int)std::min<uint64_t>(last, 1ull << l) - 2;
        return std::max(0, b - first(l) + 1);
    }
    // heap cells a build of `levels` levels fills: ids [0, 2 b + 3) for the last level with
    // cells (children 2b+1, 2b+2 of its last cell b), the root alone without levels
    uint64_t filled(uint32_t levels) const {
        uint64_t f = 1;
        for (uint32_t l = 1; l <= levels; ++l)
            if (count(l) > 0) f = 2ull * (uint64_t)(first(l) + count(l) - 1) + 3;
        return f;
    }
};

// Root of one instance of a batched build.
struct BatchRoot {
    uint32_t offset;     // first particle
    uint32_t n;          // particles
    uint32_t d;          // leaf cells
    uint32_t heap_base;  // heap slot of the root
    float lower[3], upper[3];
};

// Host-side launchers (orb_kernels.cu). `grid` is the CTA count of the tile loops.
void launch_init(const Level &v, uint64_t n, const float lower[3], const float upper[3],
                 uint32_t d, int heap_cells, cudaStream_t st);
void launch_level_kernel(Kernel k, const Level &v, int grid, int arg, cudaStream_t st);
void launch_init_batch(const Level &v, const BatchRoot *roots, int k, uint64_t n_total,
                       cudaStream_t st);
// dst[p] = src[p] for the positions of every instance (2-D grid: instance x particles)
void launch_copy_instances(const uint32_t *src, uint32_t *dst, const BatchRoot *roots, int k,
                           cudaStream_t st);
// Gaussian displacement of the particles [offset, offset+n): x += sigma * N(0,1) per
// coordinate, clamped to [lower, nextafter(upper, lower)] (seeded, counter-based)
void launch_displace(float *x, float *y, float *z, uint64_t offset, uint64_t n, uint64_t seed,
                     float sigma, const float lower[3], const float upper[3], cudaStream_t st);
cudaError_t configure_kernels();  // once per device (dynamic shared memory limits)
int swap_blocks_per_sm();         // resident CTAs of the swap kernel per SM (its grid)
void launch_gen_uniform(uint64_t seed, uint64_t n, float *x, float *y, float *z,
                        cudaStream_t st);
// `draws` draws of the reference's xorshf96 stream, thread g from starts[3g..3g+2] for `chunk`
void launch_gen_xorshf96(const unsigned long long *starts, uint64_t draws, uint32_t chunk,
                         float *x, float *y, float *z, cudaStream_t st);
void launch_gen_plummer(uint64_t seed, uint64_t n, const float *centres, const double *scales,
                        float *x, float *y, float *z, cudaStream_t st);

// Context internals used by the request server (orb_server.cu).
cudaStream_t ctx_stream(orb_ctx *ctx);
void ctx_disable_graphs(orb_ctx *ctx);
void launch_iota_u32(uint32_t *dst, uint64_t n, cudaStream_t st);  // dst[p] = p
// gather: dst[off+p] = src[off + perm[off+p]] for p < n (instance-relative permutation)
void launch_stage_gather(float *dst, const float *src, const uint32_t *idx, uint64_t n,
                         BuildCounters *ctr, int num_sms, cudaStream_t st);
void launch_gather_u32(uint32_t *dst, const uint32_t *src, const uint32_t *perm, uint64_t off,
                       uint64_t n, cudaStream_t st);

}  // namespace orb
