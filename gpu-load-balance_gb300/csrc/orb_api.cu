// Host driver and C ABI of the ORB engine (include/orb/orb.h).
//
// orb_build runs the reference's master() level loop (src/orbit.cpp:102-275) with every
// step on the device: per level a plan, histogram/resolve passes that replay the
// bisection, the parallel Hoare partition and the split, and the last levels one CTA per
// cell. The work is captured in CUDA graphs and replayed; the host reads one flag per build
// (whether the device took the subtree path for the last levels).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <list>
#include <mutex>
#include <new>
#include <thread>
#include <atomic>
#include <string>
#include <utility>
#include <vector>

#include "orb_internal.cuh"

using namespace orb;

namespace {

template <class T>
struct DevBuf {
    T *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t n, bool zero = false) {
        if (n <= cap && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        size_t want = n < 16 ? 16 : n;
        cudaError_t e = cudaMalloc(reinterpret_cast<void **>(&p), want * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            return e;
        }
        cap = want;
        if (zero) e = cudaMemset(p, 0, want * sizeof(T));
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};



}  // namespace

struct orb_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    // builds from host memory: y and z are copied on copy_stream while the root level (cut
    // along x) bisects; the first partition waits for yz_ready (yz_pending: not yet waited)
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t yz_ready = nullptr;
    bool yz_pending = false;
    // staged builds from host memory (stage_coords): y arrives in yraw while level 1 (cut
    // along x) runs, z in zraw while level 2 runs; y_ready marks y's copy, yz_ready z's
    cudaEvent_t y_ready = nullptr;
    bool use_stage = true;  // ORB_NO_STAGE=1 turns staged builds off
    DevBuf<float> yraw, zraw;
    std::string err;

    DevBuf<float> x, y, z;
    DevBuf<uint32_t> idx;
    DevBuf<orb_cell_t> heap;
    DevBuf<uint2> ranges;
    DevBuf<uint32_t> tile_off, hist_off, below, inb, part_s, part_i, part_le, out_counts;
    DevBuf<uint32_t> htile_cell, ptile_cell;
    // test hooks (orb_test_set_scan_wait): polls of a look-back wait, and the value the
    // tile scan's block ticket starts from (0 normally; 1 leaves the first block's status
    // unpublished, so its successor's wait runs out)
    uint32_t spin_limit = kLookbackSpinLimit;
    uint32_t scan_ticket_start = 0;
    // launch tuning (orb_set_tuning / orb_autotune_batch); cta_min_cells = 0 means never
    orb_tuning tune = {(uint32_t)kHistBlocksPerSm, 8u, (uint32_t)kTileBlocksPerSm, 64u, 0u, 4u, 0u};
    DevBuf<uint8_t> hist_k, state, iters, listed, cmp_bad;
    DevBuf<uint32_t> cmp_off, cmp_cnt, pred;
    DevBuf<float> cmp_keys;
    DevBuf<uint32_t> hist;
    DevBuf<uint32_t> ptile_off, ge_bits, le_bits, pt_ge, pt_le, pt_ge_pre, pt_le_pre;
    DevBuf<unsigned long long> pt_status;
    DevBuf<int> slots;
    DevBuf<BuildCounters> counters;
    DevBuf<orb_cell_t> staging;
    DevBuf<BatchRoot> batch_roots;
    DevBuf<int> batch_slots;
    DevBuf<float> tune_src[3], tune_work[3];  // autotuner: input copy, build arrays
    DevBuf<float2> hint;      // warm builds: starting bracket per heap slot
    DevBuf<int> hint_axis;
    DevBuf<uint8_t> warm;
    DevBuf<uint32_t> sub_flag;  // subtree path taken (one word)
    DevBuf<uint32_t> w;         // weighted builds from host memory: the weights
    DevBuf<unsigned long long> gen_starts;  // xorshf96 generator: chunk start states
    DevBuf<unsigned long long> whist, wbelow, wtot;  // weighted builds: per-cell weight sums
    BuildCounters *h_counters = nullptr;  // pinned
    uint32_t *h_sub_flag = nullptr;       // pinned: the subtree path was taken

    // service layer state
    bool loaded = false;
    uint64_t loaded_n = 0;
    uint32_t loaded_cells = 0;

    // profiling: launch counts always; CUDA-event durations when `prof_timing` is set
    uint32_t prof_mask = 0;  // kernel kinds whose launches are event-timed
    bool capturing = false;  // inside a graph capture
    uint64_t launches[kNumKernels] = {};
    double prof_ms[kNumKernels] = {};
    double prof_bytes[kNumKernels] = {};
    struct Rec {
        int kind;
        cudaEvent_t a, b;
    };
    std::vector<Rec> recs;
    std::vector<cudaEvent_t> ev_pool;

    // CUDA graphs of recent builds' device work (most recent first), replayed when the
    // configuration matches
    bool use_graphs = true;
    // level kernels launched with programmatic dependent launch (ORB_NO_PDL=1: plain launches)
    bool use_pdl = true;
    struct Graph {
        std::vector<uint64_t> key;
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        std::vector<Rec> recs;  // event pairs recorded inside the graph (profiling)
        uint64_t launches[kNumKernels] = {};
        uint32_t passes = 0;
    };
    std::list<Graph> graphs;
    std::vector<Graph *> ran;  // graphs replayed since their profiles were last read
    static constexpr size_t kMaxGraphs = 256;
    // window reports of the subtree kernel (builds from host memory): pinned and mapped
    uint32_t e2e_windows = 16;  // ORB_E2E_WINDOWS (0: the particles are copied back after the build)
    HostWindows *h_win = nullptr, *d_win = nullptr;
    DevBuf<uint32_t> win_cnt;
};

namespace {

orb_status fail(orb_ctx *ctx, orb_status s, const std::string &msg) {
    if (ctx) ctx->err = msg;
    return s;
}

orb_status cuda_fail(orb_ctx *ctx, cudaError_t e, const char *what) {
    std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return fail(ctx, e == cudaErrorMemoryAllocation ? ORB_ERR_OUT_OF_MEMORY : ORB_ERR_CUDA, m);
}

#define ORB_CUDA(call)                                                   \
    do {                                                                 \
        cudaError_t e_ = (call);                                         \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call);         \
    } while (0)

bool is_device_ptr(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

orb_status ensure_ptile_buffers(orb_ctx *ctx, uint64_t ptiles) {
    ORB_CUDA(ctx->ptile_cell.ensure(ptiles));
    ORB_CUDA(ctx->ge_bits.ensure(ptiles * kPWords));
    ORB_CUDA(ctx->le_bits.ensure(ptiles * kPWords));
    ORB_CUDA(ctx->pt_ge.ensure(ptiles));
    ORB_CUDA(ctx->pt_le.ensure(ptiles));
    ORB_CUDA(ctx->pt_ge_pre.ensure(ptiles + 1));
    ORB_CUDA(ctx->pt_le_pre.ensure(ptiles + 1));
    ORB_CUDA(ctx->pt_status.ensure(ptiles + 1));
    return ORB_OK;
}

// Level buffers for up to `max_cells` cells per level over n particles.
orb_status ensure_level_buffers(orb_ctx *ctx, uint64_t n, uint32_t max_cells, uint32_t heap_cells) {
    const uint64_t max_ptiles = n / kPTile + max_cells + 2;
    const uint64_t max_bins = n / 2 + 16ull * max_cells + 16;
    ORB_CUDA(ctx->heap.ensure(heap_cells));
    ORB_CUDA(ctx->ranges.ensure(heap_cells));
    ORB_CUDA(ctx->tile_off.ensure(max_cells + 1));
    ORB_CUDA(ctx->htile_cell.ensure(n / kTile + max_cells + 2));
    ORB_CUDA(ctx->hist_off.ensure(max_cells + 1));
    ORB_CUDA(ctx->below.ensure(max_cells));
    ORB_CUDA(ctx->inb.ensure(max_cells));
    ORB_CUDA(ctx->part_s.ensure(max_cells));
    ORB_CUDA(ctx->part_i.ensure(max_cells));
    ORB_CUDA(ctx->part_le.ensure(max_cells));
    ORB_CUDA(ctx->out_counts.ensure(max_cells));
    ORB_CUDA(ctx->hist_k.ensure(max_cells));
    ORB_CUDA(ctx->state.ensure(max_cells));
    ORB_CUDA(ctx->iters.ensure(max_cells));
    ORB_CUDA(ctx->listed.ensure(max_cells));
    ORB_CUDA(ctx->cmp_bad.ensure(max_cells));
    ORB_CUDA(ctx->cmp_off.ensure(max_cells + 1));
    ORB_CUDA(ctx->cmp_cnt.ensure(max_cells));
    ORB_CUDA(ctx->pred.ensure(max_cells));
    // compaction lists: n/8 per cell of more than one tile, at least 2048 (list_capacity)
    ORB_CUDA(ctx->cmp_keys.ensure(n / 8 + 2048ull * (n / kTile + 1) + 16));
    ORB_CUDA(ctx->slots.ensure(max_cells));
    ORB_CUDA(ctx->hist.ensure(max_bins, true));
    ORB_CUDA(ctx->ptile_off.ensure(max_cells + 1));
    ORB_CUDA(ctx->counters.ensure(1, true));
    return ensure_ptile_buffers(ctx, max_ptiles);
}

Level make_level(orb_ctx *ctx, float *x, float *y, float *z) {
    Level v;
    std::memset(&v, 0, sizeof v);
    v.x = x;
    v.y = y;
    v.z = z;
    v.idx = ctx->idx.p;
    v.heap = ctx->heap.p;
    v.ranges = ctx->ranges.p;
    v.slots = nullptr;
    v.tile_off = ctx->tile_off.p;
    v.htile_cell = ctx->htile_cell.p;
    v.ptile_cell = ctx->ptile_cell.p;
    v.hist_off = ctx->hist_off.p;
    v.hist_k = ctx->hist_k.p;
    v.state = ctx->state.p;
    v.iters = ctx->iters.p;
    v.listed = ctx->listed.p;
    v.cmp_bad = ctx->cmp_bad.p;
    v.cmp_off = ctx->cmp_off.p;
    v.cmp_cnt = ctx->cmp_cnt.p;
    v.cmp_keys = ctx->cmp_keys.p;
    v.pred = ctx->pred.p;
    v.pred_sigmas = (float)ctx->tune.predict_sigmas;
    v.hist = ctx->hist.p;
    v.below = ctx->below.p;
    v.inb = ctx->inb.p;
    v.ptile_off = ctx->ptile_off.p;
    v.ge_bits = ctx->ge_bits.p;
    v.le_bits = ctx->le_bits.p;
    v.pt_ge = ctx->pt_ge.p;
    v.pt_le = ctx->pt_le.p;
    v.pt_ge_pre = ctx->pt_ge_pre.p;
    v.pt_le_pre = ctx->pt_le_pre.p;
    v.pt_status = ctx->pt_status.p;
    v.ticket = &ctx->counters.p->ticket;
    v.part_s = ctx->part_s.p;
    v.part_i = ctx->part_i.p;
    v.part_le = ctx->part_le.p;
    v.out_counts = ctx->out_counts.p;
    v.sparse_per_tile = ctx->tune.sparse_keys_per_tile;
    v.spin_limit = ctx->spin_limit;
    v.pdl = ctx->use_pdl ? 1 : 0;
    v.counters = ctx->counters.p;
    return v;
}

int pass_grid(orb_ctx *ctx) { return ctx->num_sms * (int)ctx->tune.part_blocks_per_sm; }

cudaEvent_t take_event(orb_ctx *ctx) {
    if (!ctx->ev_pool.empty()) {
        cudaEvent_t e = ctx->ev_pool.back();
        ctx->ev_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    return e;
}

// Launches one level kernel on the context stream; counted, and event-timed if enabled.
void run_kernel(orb_ctx *ctx, Kernel k, const Level &v, int grid, int arg = 0) {
    ctx->launches[k] += 1;
    cudaEvent_t a = nullptr, b = nullptr;
    if (ctx->prof_mask & (1u << k)) {
        a = take_event(ctx);
        b = take_event(ctx);
    }
    // Inside a stream capture the records are external, so they become event nodes of the
    // graph and every replay times the kernel again.
    const unsigned rf = ctx->capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
    if (a && b) cudaEventRecordWithFlags(a, ctx->stream, rf);
    launch_level_kernel(k, v, grid, arg, ctx->stream);
    if (a && b) {
        cudaEventRecordWithFlags(b, ctx->stream, rf);
        ctx->recs.push_back({(int)k, a, b});
    }
}

// dst[p] = src[idx[p]] on the build stream (staged builds), timed like a level kernel.
void run_stage_gather(orb_ctx *ctx, float *dst, const float *src, uint64_t n) {
    ctx->launches[kKStageGather] += 1;
    cudaEvent_t a = nullptr, b = nullptr;
    if (ctx->prof_mask & (1u << kKStageGather)) {
        a = take_event(ctx);
        b = take_event(ctx);
    }
    const unsigned rf = ctx->capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
    if (a && b) cudaEventRecordWithFlags(a, ctx->stream, rf);
    launch_stage_gather(dst, src, ctx->idx.p, n, ctx->counters.p, ctx->num_sms, ctx->stream);
    if (a && b) {
        cudaEventRecordWithFlags(b, ctx->stream, rf);
        ctx->recs.push_back({(int)kKStageGather, a, b});
    }
}

// Folds finished event pairs into the per-kernel totals (stream must be idle).
void collect_profile(orb_ctx *ctx) {
    for (auto &r : ctx->recs) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) ctx->prof_ms[r.kind] += ms;
        ctx->ev_pool.push_back(r.a);
        ctx->ev_pool.push_back(r.b);
    }
    ctx->recs.clear();
    cudaGetLastError();
}

void drop_graph(orb_ctx *ctx, orb_ctx::Graph &g) {
    ctx->ran.erase(std::remove(ctx->ran.begin(), ctx->ran.end(), &g), ctx->ran.end());
    if (g.exec) cudaGraphExecDestroy(g.exec);
    if (g.graph) cudaGraphDestroy(g.graph);
    for (auto &r : g.recs) {
        ctx->ev_pool.push_back(r.a);
        ctx->ev_pool.push_back(r.b);
    }
    g = orb_ctx::Graph();
}

void drop_all_graphs(orb_ctx *ctx) {
    for (auto &g : ctx->graphs) drop_graph(ctx, g);
    ctx->graphs.clear();
    ctx->ran.clear();
}

// Adds the event durations of the graphs replayed since the last call to the per-kernel
// totals (their replays must have finished).
void collect_graph_profile(orb_ctx *ctx) {
    for (orb_ctx::Graph *g : ctx->ran)
        for (auto &r : g->recs) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) ctx->prof_ms[r.kind] += ms;
        }
    ctx->ran.clear();
    cudaGetLastError();
}

// Runs `body` (device work only, no host synchronisation) on the context stream, through a
// CUDA graph keyed by `key`: captured on first use, replayed while the key stays the same.
template <class Body>
orb_status run_graphed(orb_ctx *ctx, const std::vector<uint64_t> &key, uint32_t *passes, Body &&body) {
    cudaStream_t s = ctx->stream;
    if (!ctx->use_graphs) return body(passes);
    auto hit = ctx->graphs.begin();
    for (; hit != ctx->graphs.end(); ++hit)
        if (hit->key == key) break;
    if (hit != ctx->graphs.end()) {
        ctx->graphs.splice(ctx->graphs.begin(), ctx->graphs, hit);  // most recent first
    } else {
        if (ctx->graphs.size() >= orb_ctx::kMaxGraphs) {
            drop_graph(ctx, ctx->graphs.back());
            ctx->graphs.pop_back();
        }
        ctx->graphs.emplace_front();
        orb_ctx::Graph &g = ctx->graphs.front();
        uint64_t before[kNumKernels];
        std::memcpy(before, ctx->launches, sizeof before);
        collect_profile(ctx);  // keep pending records out of the graph's list
        ORB_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        ctx->capturing = true;
        uint32_t p = 0;
        orb_status st = body(&p);
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamEndCapture(s, &graph);
        ctx->capturing = false;
        if (st != ORB_OK || e != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            for (auto &r : ctx->recs) {
                ctx->ev_pool.push_back(r.a);
                ctx->ev_pool.push_back(r.b);
            }
            ctx->recs.clear();
            ctx->graphs.pop_front();
            cudaGetLastError();
            return st != ORB_OK ? st : cuda_fail(ctx, e, "cudaStreamEndCapture");
        }
        g.graph = graph;
        cudaError_t ie = cudaGraphInstantiate(&g.exec, graph, 0);
        if (ie != cudaSuccess) {
            drop_graph(ctx, g);
            ctx->graphs.pop_front();
            return cuda_fail(ctx, ie, "cudaGraphInstantiate");
        }
        g.recs.swap(ctx->recs);
        for (int k = 0; k < kNumKernels; ++k) {
            g.launches[k] = ctx->launches[k] - before[k];
            ctx->launches[k] = before[k];
        }
        g.passes = p;
        g.key = key;
    }
    orb_ctx::Graph &g = ctx->graphs.front();
    ORB_CUDA(cudaGraphLaunch(g.exec, s));
    for (int k = 0; k < kNumKernels; ++k) ctx->launches[k] += g.launches[k];
    *passes += g.passes;
    if (std::find(ctx->ran.begin(), ctx->ran.end(), &g) == ctx->ran.end()) ctx->ran.push_back(&g);
    return ORB_OK;
}

// Key of the device work of a build: sizes, box, every buffer address the kernels use.
void key_add(std::vector<uint64_t> &key, const void *p) { key.push_back((uint64_t)(uintptr_t)p); }
void key_add_f(std::vector<uint64_t> &key, float f) {
    uint32_t u;
    std::memcpy(&u, &f, sizeof u);
    key.push_back(u);
}
std::vector<uint64_t> level_key(orb_ctx *ctx, const Level &v) {
    std::vector<uint64_t> key;
    for (const void *p : {(const void *)v.x, (const void *)v.y, (const void *)v.z, (const void *)v.idx,
                          (const void *)v.heap, (const void *)v.ranges, (const void *)v.tile_off,
                          (const void *)v.hist_off, (const void *)v.hist_k, (const void *)v.state,
                          (const void *)v.iters, (const void *)v.hist, (const void *)v.below,
                          (const void *)v.listed, (const void *)v.cmp_keys, (const void *)v.cmp_off,
                          (const void *)v.inb, (const void *)v.htile_cell,
                          (const void *)v.ptile_cell, (const void *)v.ptile_off, (const void *)v.ge_bits,
                          (const void *)v.le_bits, (const void *)v.pt_ge, (const void *)v.pt_le,
                          (const void *)v.pt_ge_pre, (const void *)v.pt_le_pre, (const void *)v.pt_status,
                          (const void *)v.part_s, (const void *)v.part_i, (const void *)v.part_le,
                          (const void *)v.pred, (const void *)v.counters, (const void *)v.wt,
                          (const void *)v.whist, (const void *)v.wbelow, (const void *)v.wtot})
        key_add(key, p);
    key.push_back((uint64_t)ctx->pt_status.cap);
    key_add(key, ctx->sub_flag.p);
    key.push_back(ctx->prof_mask);
    key.push_back(((uint64_t)ctx->spin_limit << 8) | ctx->scan_ticket_start);
    key.push_back(ctx->use_pdl ? 1u : 0u);
    for (uint32_t t : {ctx->tune.hist_blocks_per_sm, ctx->tune.part_blocks_per_sm, ctx->tune.tile_blocks_per_sm,
                       ctx->tune.sparse_keys_per_tile, ctx->tune.cta_min_cells, ctx->tune.subtree_levels,
                       ctx->tune.predict_sigmas})
        key.push_back(t);
    return key;
}

void partition_level(orb_ctx *ctx, const Level &v, bool do_split) {
    const int g = pass_grid(ctx);
    // look-back state of the tile scan: status words cleared, ticket at zero
    cudaMemsetAsync(ctx->pt_status.p, 0, ctx->pt_status.cap * sizeof(unsigned long long), ctx->stream);
    cudaMemsetAsync(&ctx->counters.p->ticket, 0, sizeof(uint32_t), ctx->stream);
    if (ctx->scan_ticket_start)  // test hook: the low byte (little-endian) of the ticket
        cudaMemsetAsync(&ctx->counters.p->ticket, (int)ctx->scan_ticket_start, 1, ctx->stream);
    run_kernel(ctx, kKPartClassify, v, g);
    run_kernel(ctx, kKPartScan, v, g, (int)(ctx->pt_ge_pre.cap / 1024 + 1));
    run_kernel(ctx, kKPartCells, v, g);
    if (ctx->yz_pending) {  // the first kernel that reads y and z
        cudaStreamWaitEvent(ctx->stream, ctx->yz_ready, ctx->capturing ? cudaEventWaitExternal : 0);
        ctx->yz_pending = false;
    }
    run_kernel(ctx, kKPartSwap, v, ctx->num_sms * swap_blocks_per_sm());
    run_kernel(ctx, kKPartFinish, v, g, do_split ? 1 : 0);
}

// Bisection of every cell of the level to completion (found or capped): a fixed number of
// histogram/resolve passes, with no host round trip (a pass after the level is done exits
// at once on the device).
// first: the count pass the first pass uses: 1 every cell dense (a cold level without
// sampled brackets), 2 a sampled level, 0 the general one (warm builds).
orb_status run_bisection(orb_ctx *ctx, Level v, uint32_t *passes, int first) {
    // a cold first pass over every key is never discarded: 3 passes reach the cap
    const int npasses = first == 1 ? kColdHistPasses : kHistPasses;
    v.last_pass = npasses - 1;
    for (int pass = 0; pass < npasses; ++pass) {
        v.pass = pass;
        run_kernel(ctx, kKHist, v, ctx->num_sms * (int)ctx->tune.hist_blocks_per_sm,
                   pass == 0 ? first : 0);
        run_kernel(ctx, kKResolve, v, pass_grid(ctx));
        ++*passes;
    }
    ORB_CUDA(cudaGetLastError());
    return ORB_OK;
}

// One level of the tree: heap slots [base, base + C) or the explicit slot list `slots`.
struct LevelDesc {
    int base;
    const int *slots;
    int C;
};

// The reference's level loop (src/orbit.cpp:102-275) over every cell of every level: plan,
// bisection (one warp for small cells, one CTA per cell or the multi-CTA histogram passes
// for the rest), partition and split.
// The level from which subtree CTAs finish the tree (-1: none): the first level whose cells
// (at most max_n >> l particles plus a few per split: each split leaves a cell within 3 of
// half) all fit one CTA, that has enough cells to fill the GPU, and that is at most
// tune.subtree_levels levels above the leaves. full: every tree is built to its leaves.
int subtree_from(const orb_ctx *ctx, const std::vector<LevelDesc> &lv, uint64_t max_n, bool full) {
    const uint32_t want = std::min<uint32_t>(ctx->tune.subtree_levels, (uint32_t)kSubMaxLevels);
    if (!full || want == 0) return -1;
    for (size_t li = 0; li < lv.size(); ++li) {
        const uint64_t expect = (max_n >> li) + 1 + 8ull * li;
        if (expect <= kSubMaxParticles && (uint64_t)lv[li].C >= 2ull * (uint64_t)ctx->num_sms &&
            lv.size() - li <= want)
            return (int)li;
    }
    return -1;
}

// sub_from >= 0: from level lv[sub_from] down, one CTA per cell finishes the tree when every
// cell of that level fits one (k_subtree_check decides on the device); the level kernels of
// those levels then return at once.
// max_n: the largest instance's particles (cells of level l hold about max_n >> l); levels
// whose cells can be large enough get a sampled first count pass (k_sample_bin, k_sample_pick).
// rest = false: the levels above sub_from, then (sub_from >= 0) the subtree check and the
// subtree kernel for the levels from sub_from down; rest = true: the levels from sub_from
// down one by one, for builds whose subtree path the device refused.
// [from, to): only those levels (staged builds run the levels in pieces).
orb_status run_levels(orb_ctx *ctx, Level v, const std::vector<LevelDesc> &lv, uint32_t *passes,
                      int sub_from, uint64_t max_n, bool rest = false, size_t from = 0,
                      size_t to = SIZE_MAX) {
    to = std::min(to, lv.size());
    for (size_t li = rest ? (size_t)sub_from : from; li < to; ++li) {
        const LevelDesc &d = lv[li];
        v.base = d.base;
        v.slots = d.slots;
        v.C = d.C;
        if (!rest && (int)li == sub_from) {
            if (v.C == 0) break;
            v.skip = ctx->sub_flag.p;
            run_kernel(ctx, kKSubtreeCheck, v, 1, (int)(lv.size() - li));
            // the warp path for small cells when the deepest split cells can be that small
            // (about max_n >> (levels - 1) particles, twice kWarpKeys allowing for uneven cells)
            const bool small = (max_n >> (lv.size() - 1)) <= 2ull * kWarpKeys;
            run_kernel(ctx, kKSubtree, v, std::min(v.C, ctx->num_sms * kSubtreeBlocksPerSm), small ? 1 : 0);
            break;
        }
        if (v.C == 0) continue;
        run_kernel(ctx, kKPlan, v, 1);
        run_kernel(ctx, kKTileMap, v, pass_grid(ctx));
        if (v.hint) run_kernel(ctx, kKWarmStart, v, 1);  // warm build: hinted brackets
        if (v.wt) {
            // weighted build: every cell through the weighted passes (kWPasses reach the cap)
            run_kernel(ctx, kKWStart, v, pass_grid(ctx));
            for (int pass = 0; pass < kWPasses; ++pass) {
                v.pass = pass;
                run_kernel(ctx, kKWHist, v, pass_grid(ctx));
                run_kernel(ctx, kKWResolve, v, 0);
                ++*passes;
            }
        } else if (ctx->tune.cta_min_cells && !v.hint && (uint32_t)v.C >= ctx->tune.cta_min_cells) {
            // many cells: one CTA bisects one cell, no host round trip
            run_kernel(ctx, kKBisectCta, v, std::min(v.C, ctx->num_sms * 4));
        } else {
            // cold levels with cells of at least 2^18 particles: sampled brackets for the
            // first count pass (decided per cell on the device; result-invariant)
            const bool sampled =
                !v.hint && ctx->tune.predict_sigmas && (max_n >> li) + 8ull * li >= (1ull << 18);
            if (sampled) {
                run_kernel(ctx, kKSample, v, 0);
                run_kernel(ctx, kKSamplePick, v, 0);
            }
            run_kernel(ctx, kKBisectTile, v, std::min(v.C, ctx->num_sms * (int)ctx->tune.tile_blocks_per_sm));
            orb_status st = run_bisection(ctx, v, passes, v.hint ? 0 : (sampled ? 2 : 1));
            if (st != ORB_OK) return st;
        }
        partition_level(ctx, v, true);
        ORB_CUDA(cudaGetLastError());
    }
    return ORB_OK;
}

// After the main graph of a build that planned subtrees (sub_from >= 0): waits for it and
// reads whether the device took the subtree path (*taken). When it refused (a cell too large
// for one CTA), a second graph runs the level kernels of the levels from sub_from down. The
// build's end event is recorded again after it.
orb_status finish_subtree_levels(orb_ctx *ctx, Level v, const std::vector<LevelDesc> &lv,
                                 std::vector<uint64_t> key, uint32_t *passes, int sub_from,
                                 uint64_t max_n, bool *taken) {
    *taken = false;
    if (sub_from < 0) return ORB_OK;
    ORB_CUDA(cudaMemcpyAsync(ctx->h_sub_flag, ctx->sub_flag.p, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                             ctx->stream));
    ORB_CUDA(cudaStreamSynchronize(ctx->stream));
    *taken = *ctx->h_sub_flag != 0;
    if (*taken) return ORB_OK;
    if (ctx->use_graphs) collect_graph_profile(ctx);  // the main graph's kernel events
    key.push_back(0x5E57u);  // the levels from sub_from down
    v.skip = nullptr;
    orb_status st = run_graphed(ctx, key, passes, [&](uint32_t *pp) -> orb_status {
        return run_levels(ctx, v, lv, pp, sub_from, max_n, true);
    });
    if (st != ORB_OK) return st;
    ORB_CUDA(cudaEventRecord(ctx->ev[1], ctx->stream));
    return ORB_OK;
}

}  // namespace

namespace orb {
cudaStream_t ctx_stream(orb_ctx *ctx) { return ctx->stream; }
void ctx_disable_graphs(orb_ctx *ctx) {
    ctx->use_graphs = false;
    drop_all_graphs(ctx);
}
}  // namespace orb

extern "C" {

int orb_abi_version(void) { return ORB_ABI_VERSION; }

const char *orb_status_string(orb_status s) {
    switch (s) {
        case ORB_OK: return "ok";
        case ORB_ERR_INVALID_ARGUMENT: return "invalid argument";
        case ORB_ERR_CUDA: return "CUDA error";
        case ORB_ERR_OUT_OF_MEMORY: return "out of memory";
        case ORB_ERR_CAPACITY: return "capacity exceeded";
        case ORB_ERR_NOT_LOADED: return "no particles loaded";
        case ORB_ERR_TIMEOUT: return "timeout";
    }
    return "unknown status";
}

const char *orb_last_error(const orb_ctx *ctx) { return ctx ? ctx->err.c_str() : ""; }

orb_status orb_ctx_create(int device, const orb_opts *opts, orb_ctx **out) {
    if (!out) return ORB_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (opts && opts->flags != 0) return ORB_ERR_INVALID_ARGUMENT;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess) return ORB_ERR_CUDA;
    if (device < 0 || device >= count) return ORB_ERR_INVALID_ARGUMENT;
    orb_ctx *ctx = new (std::nothrow) orb_ctx();
    if (!ctx) return ORB_ERR_OUT_OF_MEMORY;
    ctx->device = device;
    orb_status st = ORB_OK;
    do {
        if ((e = cudaSetDevice(device)) != cudaSuccess) { st = cuda_fail(ctx, e, "cudaSetDevice"); break; }
        if ((e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess) {
            st = cuda_fail(ctx, e, "cudaDeviceGetAttribute");
            break;
        }
        if ((e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess) {
            st = cuda_fail(ctx, e, "cudaStreamCreate");
            break;
        }
        for (auto &ev : ctx->ev)
            if ((e = cudaEventCreate(&ev)) != cudaSuccess) { st = cuda_fail(ctx, e, "cudaEventCreate"); break; }
        if (st != ORB_OK) break;
        if ((e = configure_kernels()) != cudaSuccess) {
            st = cuda_fail(ctx, e, "cudaFuncSetAttribute");
            break;
        }
        {
            const char *env = std::getenv("ORB_CTA_MIN_CELLS");
            // Measured on GB300 (2^27 particles, 2^16 leaves): the multi-CTA histogram passes
            // beat one-CTA-per-cell at every level, so the CTA path is opt-in.
            ctx->tune.cta_min_cells = env ? (uint32_t)std::max(0, std::atoi(env)) : 0u;
            const char *ng = std::getenv("ORB_NO_GRAPHS");
            ctx->use_graphs = !(ng && ng[0] && ng[0] != '0');
            const char *np = std::getenv("ORB_NO_PDL");
            ctx->use_pdl = !(np && np[0] && np[0] != '0');
            const char *ns = std::getenv("ORB_NO_STAGE");
            ctx->use_stage = !(ns && ns[0] && ns[0] != '0');
            const char *ew = std::getenv("ORB_E2E_WINDOWS");
            if (ew && ew[0]) ctx->e2e_windows = (uint32_t)std::min<long>(std::max<long>(0, std::atol(ew)), kMaxWindows);
        }
        if ((e = cudaMallocHost(reinterpret_cast<void **>(&ctx->h_counters), sizeof(BuildCounters))) != cudaSuccess ||
            (e = cudaMallocHost(reinterpret_cast<void **>(&ctx->h_sub_flag), sizeof(uint32_t))) != cudaSuccess ||
            (e = cudaHostAlloc(reinterpret_cast<void **>(&ctx->h_win), sizeof(HostWindows), cudaHostAllocMapped)) !=
                cudaSuccess ||
            (e = cudaHostGetDevicePointer(reinterpret_cast<void **>(&ctx->d_win), ctx->h_win, 0)) != cudaSuccess) {
            st = cuda_fail(ctx, e, "cudaMallocHost");
            break;
        }
        if (opts && (opts->reserve_particles || opts->reserve_leaves)) {
            uint64_t n = opts->reserve_particles;
            uint32_t d = opts->reserve_leaves ? opts->reserve_leaves : 1;
            if (ctx->x.ensure(n) || ctx->y.ensure(n) || ctx->z.ensure(n) || ctx->idx.ensure(n)) {
                st = fail(ctx, ORB_ERR_OUT_OF_MEMORY, "reserve failed");
                break;
            }
            st = ensure_level_buffers(ctx, n, d, 2 * d - 1);
        }
    } while (0);
    if (st != ORB_OK) {
        orb_ctx_destroy(ctx);
        return st;
    }
    *out = ctx;
    return ORB_OK;
}

orb_status orb_ctx_destroy(orb_ctx *ctx) {
    if (!ctx) return ORB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    ctx->x.release(); ctx->y.release(); ctx->z.release();
    ctx->yraw.release(); ctx->zraw.release();
    ctx->idx.release();
    ctx->heap.release(); ctx->ranges.release();
    ctx->tile_off.release(); ctx->hist_off.release(); ctx->below.release(); ctx->inb.release();
    ctx->part_s.release(); ctx->part_i.release(); ctx->part_le.release(); ctx->out_counts.release();
    ctx->hist_k.release(); ctx->state.release(); ctx->iters.release(); ctx->hist.release();
    ctx->ptile_off.release(); ctx->ge_bits.release(); ctx->le_bits.release(); ctx->pt_ge.release();
    ctx->pt_le.release(); ctx->pt_ge_pre.release(); ctx->pt_le_pre.release(); ctx->pt_status.release();
    ctx->slots.release(); ctx->counters.release(); ctx->staging.release();
    ctx->htile_cell.release(); ctx->ptile_cell.release();
    ctx->batch_roots.release(); ctx->batch_slots.release();
    for (int a = 0; a < 3; ++a) {
        ctx->tune_src[a].release();
        ctx->tune_work[a].release();
    }
    ctx->hint.release(); ctx->hint_axis.release(); ctx->warm.release(); ctx->sub_flag.release();
    ctx->w.release(); ctx->whist.release(); ctx->wbelow.release(); ctx->wtot.release();
    ctx->gen_starts.release();
    ctx->listed.release(); ctx->cmp_bad.release(); ctx->cmp_off.release(); ctx->cmp_cnt.release();
    ctx->cmp_keys.release();
    if (ctx->h_counters) cudaFreeHost(ctx->h_counters);
    if (ctx->h_sub_flag) cudaFreeHost(ctx->h_sub_flag);
    if (ctx->h_win) cudaFreeHost(ctx->h_win);
    ctx->win_cnt.release();
    collect_profile(ctx);
    drop_all_graphs(ctx);
    for (auto e : ctx->ev_pool) cudaEventDestroy(e);
    for (auto &ev : ctx->ev)
        if (ev) cudaEventDestroy(ev);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    if (ctx->yz_ready) cudaEventDestroy(ctx->yz_ready);
    if (ctx->y_ready) cudaEventDestroy(ctx->y_ready);
    delete ctx;
    return ORB_OK;
}

// After a failed build from host memory: the copies the build queued may still be reading
// or writing the caller's arrays, so wait for them before the caller gets control back.
static void drain_host_copies(orb_ctx *ctx) {
    if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    ctx->yz_pending = false;
    cudaGetLastError();
}

static orb_status build_single(orb_ctx *ctx, float *x, float *y, float *z, uint32_t *w,
                               bool weighted, uint64_t n, uint32_t d, uint32_t levels,
                               const float lower[3], const float upper[3], orb_cell_t *heap,
                               uint32_t *ranges, uint32_t *perm, uint32_t flags,
                               orb_build_info *info);

orb_status orb_build(orb_ctx *ctx, float *x, float *y, float *z, uint64_t n, uint32_t d,
                     uint32_t levels, const float lower[3], const float upper[3],
                     orb_cell_t *heap, uint32_t *ranges, uint32_t *perm, uint32_t flags,
                     orb_build_info *info) {
    const orb_status st = build_single(ctx, x, y, z, nullptr, false, n, d, levels, lower, upper,
                                       heap, ranges, perm, flags, info);
    if (st != ORB_OK && ctx && !(flags & ORB_DEVICE_POINTERS)) drain_host_copies(ctx);
    return st;
}

orb_status orb_build_weighted(orb_ctx *ctx, float *x, float *y, float *z, uint32_t *w, uint64_t n,
                              uint32_t d, uint32_t levels, const float lower[3],
                              const float upper[3], orb_cell_t *heap, uint32_t *ranges,
                              uint32_t *perm, uint32_t flags, orb_build_info *info) {
    if (!ctx) return ORB_ERR_INVALID_ARGUMENT;
    if (n > 0 && !w) return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "null weights");
    const orb_status st = build_single(ctx, x, y, z, w, true, n, d, levels, lower, upper, heap,
                                       ranges, perm, flags, info);
    if (st != ORB_OK && !(flags & ORB_DEVICE_POINTERS)) drain_host_copies(ctx);
    return st;
}

static orb_status build_single(orb_ctx *ctx, float *x, float *y, float *z, uint32_t *w,
                               bool weighted, uint64_t n, uint32_t d, uint32_t levels,
                               const float lower[3], const float upper[3], orb_cell_t *heap,
                               uint32_t *ranges, uint32_t *perm, uint32_t flags,
                               orb_build_info *info) {
    if (!ctx) return ORB_ERR_INVALID_ARGUMENT;
    ctx->err.clear();
    if (flags & ~ORB_DEVICE_POINTERS) return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "unknown flags");
    if ((n > 0 && (!x || !y || !z)) || !heap || !ranges || !lower || !upper)
        return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "null pointer");
    if (d == 0) return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "d must be at least 1");
    if (n >= (1ull << 31)) return fail(ctx, ORB_ERR_CAPACITY, "n must be below 2^31");
    if (d > (1u << 30)) return fail(ctx, ORB_ERR_CAPACITY, "d too large");
    const Slices sl(d);
    if (levels == 0) levels = sl.max_levels();
    if (levels > sl.max_levels())
        return fail(ctx, ORB_ERR_INVALID_ARGUMENT,
                    "levels exceeds log2(d) (d a power of two) or the reference's bound "
                    "ceil(log2 d) - 1 (other d)");
    const bool dev = (flags & ORB_DEVICE_POINTERS) != 0;
    if (dev && n > 0 && (!is_device_ptr(x) || !is_device_ptr(y) || !is_device_ptr(z) ||
                         (perm && !is_device_ptr(perm)) || (w && !is_device_ptr(w))))
        return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "ORB_DEVICE_POINTERS set but a pointer is not device memory");

    ORB_CUDA(cudaSetDevice(ctx->device));
    const uint32_t heap_cells = 2 * d - 1;
    uint32_t max_cells = 1;
    for (uint32_t l = 1; l <= levels; ++l) max_cells = std::max(max_cells, (uint32_t)sl.count(l));
    orb_status st = ensure_level_buffers(ctx, n, max_cells, heap_cells);
    if (st != ORB_OK) return st;
    ORB_CUDA(ctx->idx.ensure(n + 1));
    if (weighted) {
        ORB_CUDA(ctx->whist.ensure((size_t)max_cells * kWBins));
        ORB_CUDA(ctx->wbelow.ensure(max_cells));
        ORB_CUDA(ctx->wtot.ensure(max_cells));
        if (!dev) ORB_CUDA(ctx->w.ensure(n + 1));
    }
    float *dx = x, *dy = y, *dz = z;
    uint32_t *dw = weighted ? (dev ? w : ctx->w.p) : nullptr;
    cudaStream_t s = ctx->stream;
    float h2d_ms = 0.f, d2h_ms = 0.f;
    ctx->yz_pending = false;
    std::vector<LevelDesc> lv;
    for (uint32_t l = 1; l <= levels; ++l)
        lv.push_back({sl.first(l), nullptr, sl.count(l)});  // src/orbit.cpp:104-107
    // subtrees finish complete unweighted trees only: d a power of two, built to its leaves
    const int sub_from = subtree_from(ctx, lv, n, !weighted && sl.pow2 && levels == sl.depth);
    if (sub_from >= 0) ORB_CUDA(ctx->sub_flag.ensure(1));
    // Staged build from host memory: the copies of x, y and z follow one another, and the
    // levels start as soon as the coordinates they read are on the device. Level 1 cuts along
    // x (src/orbit.cpp:75), so it runs on x alone while y arrives; its swaps move x and the
    // permutation, and y then takes the new order through the permutation. Level 2 cuts each
    // cell along its longest side, whose y and z extents are the root box's and whose x
    // extent is at most the root's: with y at least as long as z (and longer than zero), the
    // first-longest rule of setCutAxis (src/cell.h:102-121) picks x or y there, so level 2
    // runs on x and y while z arrives. Same cuts, same swaps: the result is the unstaged one.
    const float y_ext = upper[1] - lower[1], z_ext = upper[2] - lower[2];
    const bool staged = !dev && n && !weighted && ctx->use_stage && levels >= 2 &&
                        (sub_from < 0 || sub_from >= 2) && y_ext > 0.f && y_ext >= z_ext;
    if (!dev) {
        ORB_CUDA(ctx->x.ensure(n + 1));
        ORB_CUDA(ctx->y.ensure(n + 1));
        ORB_CUDA(ctx->z.ensure(n + 1));
        dx = ctx->x.p;
        dy = ctx->y.p;
        dz = ctx->z.p;
        if (staged) {
            ORB_CUDA(ctx->yraw.ensure(n + 1));
            ORB_CUDA(ctx->zraw.ensure(n + 1));
        }
        ORB_CUDA(cudaEventRecord(ctx->ev[2], s));
        if (n) {
            // x first on the build stream, y and z on the copy stream: a staged build copies
            // them one after another; otherwise they cross together while the root level (cut
            // along x, src/orbit.cpp:75) bisects, and its partition waits for them
            if (!ctx->copy_stream) ORB_CUDA(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
            if (!ctx->yz_ready) ORB_CUDA(cudaEventCreateWithFlags(&ctx->yz_ready, cudaEventDisableTiming));
            if (!ctx->y_ready) ORB_CUDA(cudaEventCreateWithFlags(&ctx->y_ready, cudaEventDisableTiming));
            ORB_CUDA(cudaMemcpyAsync(dx, x, n * sizeof(float), cudaMemcpyHostToDevice, s));
            if (weighted)  // the root level's bisection reads x and the weights
                ORB_CUDA(cudaMemcpyAsync(dw, w, n * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
            if (staged) {  // one copy at a time, in the order the levels need them
                // y_ready marks the end of x's copy (the copy stream waits for it), then y's
                ORB_CUDA(cudaEventRecord(ctx->y_ready, s));
                ORB_CUDA(cudaStreamWaitEvent(ctx->copy_stream, ctx->y_ready, 0));
                ORB_CUDA(cudaMemcpyAsync(ctx->yraw.p, y, n * sizeof(float), cudaMemcpyHostToDevice,
                                         ctx->copy_stream));
                ORB_CUDA(cudaEventRecord(ctx->y_ready, ctx->copy_stream));
                ORB_CUDA(cudaMemcpyAsync(ctx->zraw.p, z, n * sizeof(float), cudaMemcpyHostToDevice,
                                         ctx->copy_stream));
            } else {
                ORB_CUDA(cudaStreamWaitEvent(ctx->copy_stream, ctx->ev[2], 0));
                ORB_CUDA(cudaMemcpyAsync(dy, y, n * sizeof(float), cudaMemcpyHostToDevice, ctx->copy_stream));
                ORB_CUDA(cudaMemcpyAsync(dz, z, n * sizeof(float), cudaMemcpyHostToDevice, ctx->copy_stream));
                ctx->yz_pending = true;
            }
            ORB_CUDA(cudaEventRecord(ctx->yz_ready, ctx->copy_stream));
            ORB_CUDA(cudaEventRecord(ctx->ev[3], ctx->copy_stream));
        } else {
            ORB_CUDA(cudaEventRecord(ctx->ev[3], s));
        }
    }
    ORB_CUDA(cudaEventRecord(ctx->ev[0], s));
    Level v = make_level(ctx, dx, dy, dz);
    if (!perm) v.idx = nullptr;  // no permutation asked for: only x, y, z move
    if (weighted) {
        v.wt = dw;
        v.whist = ctx->whist.p;
        v.wbelow = ctx->wbelow.p;
        v.wtot = ctx->wtot.p;
    }
    std::vector<uint64_t> key = level_key(ctx, v);
    key.push_back(0xB111D);  // single build
    key.push_back(n);
    key.push_back(d);
    key.push_back(levels);
    for (int a = 0; a < 3; ++a) {
        key_add_f(key, lower[a]);
        key_add_f(key, upper[a]);
    }
    key.push_back((uint64_t)(int64_t)sub_from);
    // window reports (builds from host memory that plan subtrees): the subtree kernel reports
    // each window of consecutive root cells once all of them are final, and the host copies
    // that window back while the kernel builds the next ones
    const bool windows = !dev && n && !weighted && sub_from >= 0 && ctx->e2e_windows > 0;
    uint32_t nwin = 0;
    if (windows) {
        ORB_CUDA(ctx->win_cnt.ensure(kMaxWindows));
        const uint32_t cs = (uint32_t)lv[sub_from].C;
        const uint32_t m = std::min<uint32_t>(ctx->e2e_windows, cs);
        v.hwin = ctx->d_win;
        v.win_cnt = ctx->win_cnt.p;
        v.win_cells = (cs + m - 1) / m;
        nwin = (cs + v.win_cells - 1) / v.win_cells;
        std::memset(ctx->h_win, 0, sizeof(HostWindows));  // the device writes it during the build
    }
    key_add(key, v.hwin);
    key_add(key, v.win_cnt);
    key.push_back(v.win_cells);
    key.push_back(ctx->yz_pending ? 1u : 0u);  // the graph waits for y and z before the first swap
    key.push_back(staged ? 1u : 0u);
    key_add(key, ctx->yraw.p);
    key_add(key, ctx->zraw.p);
    key_add(key, ctx->idx.p);
    uint32_t passes = 0;
    st = run_graphed(ctx, key, &passes, [&](uint32_t *pp) -> orb_status {
        ctx->launches[kKInit] += 1;
        if (!staged) {
            launch_init(v, n, lower, upper, d, (int)heap_cells, s);
            ORB_CUDA(cudaGetLastError());
            return run_levels(ctx, v, lv, pp, sub_from, n);
        }
        const unsigned wf = ctx->capturing ? cudaEventWaitExternal : 0;
        Level v1 = v;  // level 1: x and the permutation
        v1.y = v1.z = nullptr;
        v1.idx = ctx->idx.p;
        launch_init(v1, n, lower, upper, d, (int)heap_cells, s);
        ORB_CUDA(cudaGetLastError());
        orb_status ls = run_levels(ctx, v1, lv, pp, sub_from, n, false, 0, 1);
        if (ls != ORB_OK) return ls;
        ORB_CUDA(cudaStreamWaitEvent(s, ctx->y_ready, wf));
        run_stage_gather(ctx, dy, ctx->yraw.p, n);
        Level v2 = v1;  // level 2: x, y and the permutation
        v2.y = dy;
        if ((ls = run_levels(ctx, v2, lv, pp, sub_from, n, false, 1, 2)) != ORB_OK) return ls;
        ORB_CUDA(cudaStreamWaitEvent(s, ctx->yz_ready, wf));
        run_stage_gather(ctx, dz, ctx->zraw.p, n);
        ORB_CUDA(cudaGetLastError());
        return run_levels(ctx, v, lv, pp, sub_from, n, false, 2);  // the rest
    });
    if (st != ORB_OK) return st;
    if (ctx->yz_pending || (!dev && n)) {
        // a replayed graph holds the wait; a build without a partition (no levels) waits here
        ctx->yz_pending = false;
        ORB_CUDA(cudaStreamWaitEvent(s, ctx->yz_ready, 0));
    }
    // the windows: the host waits for each report (or for the build's end) and queues the
    // window's copies back on the copy stream; *all: every window was reported
    bool win_started = false;
    auto stream_windows = [&](bool *all) -> orb_status {
        *all = false;
        HostWindows *hw = ctx->h_win;
        auto wait_for = [&](volatile uint32_t *flag) -> bool {  // false: the build ended first
            for (uint32_t it = 0;; ++it) {
                if (*flag) return true;
                if ((it & 31u) == 31u) {
                    const cudaError_t q = cudaStreamQuery(s);
                    if (q != cudaErrorNotReady) {
                        cudaGetLastError();
                        return *flag != 0;
                    }
                }
                std::this_thread::yield();
            }
        };
        if (!wait_for(&hw->decision) || hw->decision != 1u) return ORB_OK;
        for (uint32_t w = 0; w < nwin; ++w) {
            if (!wait_for(&hw->done[w])) return ORB_OK;
            std::atomic_thread_fence(std::memory_order_acquire);
            const volatile uint32_t *hr = &hw->range[w].x;
            const uint2 r = make_uint2(hr[0], hr[1]);
            cudaStream_t cs = ctx->copy_stream;
            if (!win_started) {
                // the copies in ended before the first window (the build waited for them)
                ORB_CUDA(cudaEventSynchronize(ctx->ev[3]));
                ORB_CUDA(cudaEventElapsedTime(&h2d_ms, ctx->ev[2], ctx->ev[3]));
                ORB_CUDA(cudaEventRecord(ctx->ev[2], cs));
                win_started = true;
            }
            if (r.y < r.x || r.y > n) return ORB_OK;  // not a range of this build: copy all after it
            const size_t b = r.x, m = r.y - r.x;
            if (!m) continue;
            ORB_CUDA(cudaMemcpyAsync(x + b, dx + b, m * sizeof(float), cudaMemcpyDeviceToHost, cs));
            ORB_CUDA(cudaMemcpyAsync(y + b, dy + b, m * sizeof(float), cudaMemcpyDeviceToHost, cs));
            ORB_CUDA(cudaMemcpyAsync(z + b, dz + b, m * sizeof(float), cudaMemcpyDeviceToHost, cs));
            if (perm)
                ORB_CUDA(cudaMemcpyAsync(perm + b, ctx->idx.p + b, m * sizeof(uint32_t), cudaMemcpyDeviceToHost, cs));
        }
        *all = true;
        return ORB_OK;
    };
    ORB_CUDA(cudaEventRecord(ctx->ev[1], s));
    bool streamed = false;
    if (windows && (st = stream_windows(&streamed)) != ORB_OK) return st;
    bool taken = false;  // the subtree kernel finished the tree
    st = finish_subtree_levels(ctx, v, lv, key, &passes, sub_from, n, &taken);
    if (st != ORB_OK) return st;
    bool written = false;  // the particles are in the host arrays (or on their way there)
    if (!dev) {
        ORB_CUDA(cudaStreamSynchronize(s));
        if (!win_started) ORB_CUDA(cudaEventElapsedTime(&h2d_ms, ctx->ev[2], ctx->ev[3]));
        written = streamed && taken;
        if (!win_started) ORB_CUDA(cudaEventRecord(ctx->ev[2], s));
        if (n && !written) {
            ORB_CUDA(cudaMemcpyAsync(x, dx, n * sizeof(float), cudaMemcpyDeviceToHost, s));
            ORB_CUDA(cudaMemcpyAsync(y, dy, n * sizeof(float), cudaMemcpyDeviceToHost, s));
            ORB_CUDA(cudaMemcpyAsync(z, dz, n * sizeof(float), cudaMemcpyDeviceToHost, s));
        }
        if (n && weighted)  // the weights, reordered with their particles
            ORB_CUDA(cudaMemcpyAsync(w, dw, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    }
    if (perm && n && !written)
        ORB_CUDA(cudaMemcpyAsync(perm, ctx->idx.p, n * sizeof(uint32_t),
                                 dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
    ORB_CUDA(cudaMemcpyAsync(heap, ctx->heap.p, heap_cells * sizeof(orb_cell_t), cudaMemcpyDeviceToHost, s));
    ORB_CUDA(cudaMemcpyAsync(ranges, ctx->ranges.p, heap_cells * sizeof(uint2), cudaMemcpyDeviceToHost, s));
    ORB_CUDA(cudaMemcpyAsync(ctx->h_counters, ctx->counters.p, sizeof(BuildCounters), cudaMemcpyDeviceToHost, s));
    const bool on_cs = win_started;  // copies back on the copy stream
    if (on_cs && !written) {  // and some on the context stream after them: both timed
        ORB_CUDA(cudaEventRecord(ctx->ev[3], s));
        ORB_CUDA(cudaStreamWaitEvent(ctx->copy_stream, ctx->ev[3], 0));
    }
    if (!dev) ORB_CUDA(cudaEventRecord(ctx->ev[3], on_cs ? ctx->copy_stream : s));
    ORB_CUDA(cudaStreamSynchronize(s));
    if (on_cs) ORB_CUDA(cudaStreamSynchronize(ctx->copy_stream));
    if (ctx->h_counters->error)
        return fail(ctx, ORB_ERR_TIMEOUT, "a bounded device wait gave up or a bisection did not finish");
    float dev_ms = 0.f;
    ORB_CUDA(cudaEventElapsedTime(&dev_ms, ctx->ev[0], ctx->ev[1]));
    collect_profile(ctx);
    if (ctx->use_graphs) collect_graph_profile(ctx);
    for (int k = 0; k < kNumKernels; ++k) ctx->prof_bytes[k] += (double)ctx->h_counters->bytes[k];
    if (!dev) ORB_CUDA(cudaEventElapsedTime(&d2h_ms, ctx->ev[2], ctx->ev[3]));
    if (info) {
        std::memset(info, 0, sizeof *info);
        info->levels_built = levels;
        info->degenerate_cells = ctx->h_counters->degenerate;
        info->zero_volume_cells = ctx->h_counters->zero_volume;
        info->unfound_cells = ctx->h_counters->unfound;
        info->max_iterations = ctx->h_counters->max_iters;
        info->count_passes = passes;
        info->device_ms = dev_ms;
        info->h2d_ms = h2d_ms;
        info->d2h_ms = d2h_ms;
        info->warm_cells = ctx->h_counters->warm_cells;
        info->warm_resets = ctx->h_counters->warm_resets;
        info->sampled_cells = ctx->h_counters->pred_cells;
        info->sampled_misses = ctx->h_counters->pred_misses;
    }
    return ORB_OK;
}

// The reference's xorshf96 (src/services/init.cu:11-25) is a linear map of its 192-bit state
// over GF(2): s -> M s. Its stream is cut into chunks of kXsChunk draws; the start of chunk g
// is M^(offset + g kXsChunk) s0, by a matrix power (squaring) and one product per chunk.
namespace xs96 {
struct State {
    unsigned long long w[3];
};
inline void step(State &s) {
    unsigned long long x = s.w[0];
    x ^= x << 16;
    x ^= x >> 5;
    x ^= x << 1;
    const unsigned long long t = x;
    s.w[0] = s.w[1];
    s.w[1] = s.w[2];
    s.w[2] = t ^ s.w[0] ^ s.w[1];
}
struct Mat {
    State col[192];  // column j: the image of state bit j
};
inline State apply(const Mat &m, const State &v) {
    State r = {{0, 0, 0}};
    for (int j = 0; j < 192; ++j)
        if ((v.w[j >> 6] >> (j & 63)) & 1ull)
            for (int k = 0; k < 3; ++k) r.w[k] ^= m.col[j].w[k];
    return r;
}
inline Mat mul(const Mat &a, const Mat &b) {  // a b
    Mat c;
    for (int j = 0; j < 192; ++j) c.col[j] = apply(a, b.col[j]);
    return c;
}
inline Mat power(uint64_t k) {  // M^k
    Mat base, acc;
    for (int j = 0; j < 192; ++j) {
        State e = {{0, 0, 0}};
        e.w[j >> 6] = 1ull << (j & 63);
        acc.col[j] = e;
        step(e);
        base.col[j] = e;
    }
    for (; k; k >>= 1) {
        if (k & 1) acc = mul(acc, base);
        base = mul(base, base);
    }
    return acc;
}
constexpr uint32_t kXsChunk = 4096;
}  // namespace xs96

orb_status orb_generate(orb_ctx *ctx, int kind, uint64_t seed, uint64_t n, float *x, float *y,
                        float *z, uint32_t flags) {
    if (!ctx) return ORB_ERR_INVALID_ARGUMENT;
    ctx->err.clear();
    if (kind != ORB_GEN_UNIFORM && kind != ORB_GEN_PLUMMER && kind != ORB_GEN_XORSHF96)
        return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "unknown generator kind");
    if (n == 0) return ORB_OK;
    if (!x || !y || !z) return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "null pointer");
    ORB_CUDA(cudaSetDevice(ctx->device));
    const bool dev = (flags & ORB_DEVICE_POINTERS) != 0;
    float *dx = x, *dy = y, *dz = z;
    if (!dev) {
        ORB_CUDA(ctx->x.ensure(n));
        ORB_CUDA(ctx->y.ensure(n));
        ORB_CUDA(ctx->z.ensure(n));
        dx = ctx->x.p;
        dy = ctx->y.p;
        dz = ctx->z.p;
    }
    ctx->launches[kKGenerate] += 1;
    if (kind == ORB_GEN_XORSHF96) {
        // chunk starts: M^seed s0 (seed = draws to skip), then one jump of kXsChunk per chunk
        static std::mutex mu;
        static bool have = false;
        static xs96::Mat jump;
        {
            std::lock_guard<std::mutex> g(mu);
            if (!have) {
                jump = xs96::power(xs96::kXsChunk);
                have = true;
            }
        }
        const uint64_t draws = 3 * n, chunks = (draws + xs96::kXsChunk - 1) / xs96::kXsChunk;
        std::vector<unsigned long long> starts(3 * chunks);
        xs96::State s0 = {{123456789ull, 362436069ull, 521288629ull}};  // init.cu:11
        if (seed) s0 = xs96::apply(xs96::power(seed), s0);
        for (uint64_t g = 0; g < chunks; ++g) {
            for (int k = 0; k < 3; ++k) starts[3 * g + k] = s0.w[k];
            s0 = xs96::apply(jump, s0);
        }
        ORB_CUDA(ctx->gen_starts.ensure(starts.size()));
        ORB_CUDA(cudaMemcpyAsync(ctx->gen_starts.p, starts.data(), starts.size() * sizeof(unsigned long long),
                                 cudaMemcpyHostToDevice, ctx->stream));
        launch_gen_xorshf96(ctx->gen_starts.p, draws, xs96::kXsChunk, dx, dy, dz, ctx->stream);
        ORB_CUDA(cudaStreamSynchronize(ctx->stream));  // `starts` goes out of scope
    } else if (kind == ORB_GEN_UNIFORM) {
        launch_gen_uniform(seed, n, dx, dy, dz, ctx->stream);
    } else {
        // Cluster table, computed on the host exactly as the CPU oracle computes it.
        float centres[64 * 3];
        double scales[64];
        auto mix64 = [](uint64_t zz) {
            zz += 0x9E3779B97F4A7C15ull;
            zz = (zz ^ (zz >> 30)) * 0xBF58476D1CE4E5B9ull;
            zz = (zz ^ (zz >> 27)) * 0x94D049BB133111EBull;
            return zz ^ (zz >> 31);
        };
        auto draw = [&](uint64_t sd, uint64_t c) { return mix64(mix64(sd) + c * 0xD1B54A32D192ED03ull); };
        const uint64_t dom = seed ^ 0xC1A57E5C1A57E5C1ull;
        for (int k = 0; k < 64; ++k) {
            for (int a = 0; a < 3; ++a) {
                volatile float f = (float)(uint32_t)(draw(dom, 4 * k + a) >> 40);
                volatile float g = f * 0x1p-24f;
                centres[3 * k + a] = g - 0.5f;
            }
            double u = (double)(draw(dom, 4 * k + 3) >> 11) * 0x1p-53;
            scales[k] = 0.005 * std::pow(10.0, u);
        }
        launch_gen_plummer(seed, n, centres, scales, dx, dy, dz, ctx->stream);
    }
    ORB_CUDA(cudaGetLastError());
    if (!dev) {
        ORB_CUDA(cudaMemcpyAsync(x, dx, n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
        ORB_CUDA(cudaMemcpyAsync(y, dy, n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
        ORB_CUDA(cudaMemcpyAsync(z, dz, n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    }
    ORB_CUDA(cudaStreamSynchronize(ctx->stream));
    return ORB_OK;
}

// ---------------------------------------------------------------------------------------
// Service layer
// ---------------------------------------------------------------------------------------
orb_status orb_load_particles(orb_ctx *ctx, const float *x, const float *y, const float *z,
                              uint64_t n, uint32_t max_cells, uint32_t flags) {
    if (!ctx) return ORB_ERR_INVALID_ARGUMENT;
    ctx->err.clear();
    if ((n > 0 && (!x || !y || !z)) || max_cells == 0)
        return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "null pointer or max_cells == 0");
    if (n >= (1ull << 31)) return fail(ctx, ORB_ERR_CAPACITY, "n must be below 2^31");
    ORB_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    orb_status st = ensure_level_buffers(ctx, n, max_cells, max_cells);
    if (st != ORB_OK) return st;
    ORB_CUDA(ctx->x.ensure(n + 1));
    ORB_CUDA(ctx->y.ensure(n + 1));
    ORB_CUDA(ctx->z.ensure(n + 1));
    ORB_CUDA(ctx->idx.ensure(n + 1));
    ORB_CUDA(ctx->staging.ensure(max_cells));
    const cudaMemcpyKind k = (flags & ORB_DEVICE_POINTERS) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (n) {
        ORB_CUDA(cudaMemcpyAsync(ctx->x.p, x, n * sizeof(float), k, s));
        ORB_CUDA(cudaMemcpyAsync(ctx->y.p, y, n * sizeof(float), k, s));
        ORB_CUDA(cudaMemcpyAsync(ctx->z.p, z, n * sizeof(float), k, s));
    }
    // identity permutation and range map {root = [0, n)} (src/services/init.cu:63-66)
    std::vector<uint32_t> iota(n);
    for (uint64_t i = 0; i < n; ++i) iota[i] = (uint32_t)i;
    if (n) ORB_CUDA(cudaMemcpyAsync(ctx->idx.p, iota.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    ORB_CUDA(cudaMemsetAsync(ctx->ranges.p, 0, max_cells * sizeof(uint2), s));
    uint2 root = make_uint2(0u, (uint32_t)n);
    ORB_CUDA(cudaMemcpyAsync(ctx->ranges.p, &root, sizeof root, cudaMemcpyHostToDevice, s));
    ORB_CUDA(cudaMemsetAsync(ctx->counters.p, 0, sizeof(BuildCounters), s));
    ORB_CUDA(cudaStreamSynchronize(s));
    ctx->loaded = true;
    ctx->loaded_n = n;
    ctx->loaded_cells = max_cells;
    return ORB_OK;
}

orb_status orb_store_particles(orb_ctx *ctx, float *x, float *y, float *z, uint32_t *perm,
                               uint32_t flags) {
    if (!ctx) return ORB_ERR_INVALID_ARGUMENT;
    ctx->err.clear();
    if (!ctx->loaded) return fail(ctx, ORB_ERR_NOT_LOADED, "no particles loaded");
    const uint64_t n = ctx->loaded_n;
    if (n && (!x || !y || !z)) return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "null pointer");
    ORB_CUDA(cudaSetDevice(ctx->device));
    const cudaMemcpyKind k = (flags & ORB_DEVICE_POINTERS) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    cudaStream_t s = ctx->stream;
    if (n) {
        ORB_CUDA(cudaMemcpyAsync(x, ctx->x.p, n * sizeof(float), k, s));
        ORB_CUDA(cudaMemcpyAsync(y, ctx->y.p, n * sizeof(float), k, s));
        ORB_CUDA(cudaMemcpyAsync(z, ctx->z.p, n * sizeof(float), k, s));
        if (perm) ORB_CUDA(cudaMemcpyAsync(perm, ctx->idx.p, n * sizeof(uint32_t), k, s));
    }
    ORB_CUDA(cudaStreamSynchronize(s));
    return ORB_OK;
}

static orb_status service_prepare(orb_ctx *ctx, const orb_cell_t *cells, uint32_t n_cells,
                                  bool need_children, Level *out) {
    if (!ctx->loaded) return fail(ctx, ORB_ERR_NOT_LOADED, "no particles loaded");
    if (n_cells && !cells) return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "null cells");
    std::vector<uint8_t> seen(ctx->loaded_cells, 0);
    std::vector<int> ids(n_cells);
    for (uint32_t i = 0; i < n_cells; ++i) {
        const int64_t id = cells[i].id;
        const int64_t hi = need_children ? 2 * id + 2 : id;
        if (id < 0 || hi >= (int64_t)ctx->loaded_cells)
            return fail(ctx, ORB_ERR_CAPACITY, "cell id outside the range map");
        if (seen[id]) return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "duplicate cell id");
        seen[id] = 1;
        ids[i] = (int)id;
    }
    cudaStream_t s = ctx->stream;
    // Size the per-tile buffers from the cells' actual ranges; reject overlapping cells
    // (each tile and each rank table entry must belong to exactly one cell).
    std::vector<uint2> rg(ctx->loaded_cells);
    ORB_CUDA(cudaMemcpyAsync(rg.data(), ctx->ranges.p, rg.size() * sizeof(uint2), cudaMemcpyDeviceToHost, s));
    ORB_CUDA(cudaStreamSynchronize(s));
    std::vector<std::pair<uint32_t, uint32_t>> spans;
    uint64_t tiles = 0;
    for (uint32_t i = 0; i < n_cells; ++i) {
        const uint2 r = rg[ids[i]];
        if (r.y < r.x || r.y > ctx->loaded_n) return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "corrupt range map");
        tiles += (r.y - r.x + kPTile - 1) / kPTile;
        if (r.y > r.x) spans.emplace_back(r.x, r.y);
    }
    std::sort(spans.begin(), spans.end());
    for (size_t i = 1; i < spans.size(); ++i)
        if (spans[i].first < spans[i - 1].second)
            return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "cells with overlapping particle ranges");
    {
        orb_status pst = ensure_ptile_buffers(ctx, tiles + 2);
        if (pst != ORB_OK) return pst;
    }
    // Each cell is placed at heap slot == id, so child slots are 2id+1 and 2id+2.
    if (n_cells) {
        ORB_CUDA(cudaMemcpyAsync(ctx->slots.p, ids.data(), n_cells * sizeof(int), cudaMemcpyHostToDevice, s));
        for (uint32_t i = 0; i < n_cells; ++i)
            ORB_CUDA(cudaMemcpyAsync(ctx->heap.p + ids[i], cells + i, sizeof(orb_cell_t), cudaMemcpyHostToDevice, s));
    }
    Level v = make_level(ctx, ctx->x.p, ctx->y.p, ctx->z.p);
    v.slots = ctx->slots.p;
    v.base = 0;
    v.C = (int)n_cells;
    *out = v;
    return ORB_OK;
}

orb_status orb_count(orb_ctx *ctx, const orb_cell_t *cells, uint32_t n_cells, uint32_t *out) {
    if (!ctx) return ORB_ERR_INVALID_ARGUMENT;
    ctx->err.clear();
    if (!ctx->loaded) return fail(ctx, ORB_ERR_NOT_LOADED, "no particles loaded");
    if (n_cells && (!cells || !out)) return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "null pointer");
    ORB_CUDA(cudaSetDevice(ctx->device));
    std::vector<uint2> rg(ctx->loaded_cells);
    ORB_CUDA(cudaMemcpyAsync(rg.data(), ctx->ranges.p, rg.size() * sizeof(uint2), cudaMemcpyDeviceToHost, ctx->stream));
    ORB_CUDA(cudaStreamSynchronize(ctx->stream));
    for (uint32_t i = 0; i < n_cells; ++i) {
        const int64_t id = cells[i].id;
        if (id < 0 || id >= (int64_t)ctx->loaded_cells)
            return fail(ctx, ORB_ERR_CAPACITY, "cell id outside the range map");
        out[i] = rg[id].y - rg[id].x;  // src/services/count.cpp:14-17
    }
    return ORB_OK;
}

orb_status orb_count_left(orb_ctx *ctx, const orb_cell_t *cells, uint32_t n_cells, uint32_t *out) {
    if (!ctx) return ORB_ERR_INVALID_ARGUMENT;
    ctx->err.clear();
    if (n_cells && !out) return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "null out");
    ORB_CUDA(cudaSetDevice(ctx->device));
    Level v;
    orb_status st = service_prepare(ctx, cells, n_cells, false, &v);
    if (st != ORB_OK || n_cells == 0) return st;
    cudaStream_t s = ctx->stream;
    ORB_CUDA(cudaMemsetAsync(ctx->out_counts.p, 0, n_cells * sizeof(uint32_t), s));
    run_kernel(ctx, kKPlan, v, 1);
    run_kernel(ctx, kKTileMap, v, pass_grid(ctx));
    run_kernel(ctx, kKCountLeft, v, pass_grid(ctx));
    ORB_CUDA(cudaGetLastError());
    std::vector<uint32_t> res(n_cells);
    collect_profile(ctx);
    ORB_CUDA(cudaMemcpyAsync(res.data(), ctx->out_counts.p, n_cells * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    ORB_CUDA(cudaStreamSynchronize(s));
    for (uint32_t i = 0; i < n_cells; ++i)
        if (!cells[i].foundCut) out[i] = res[i];  // src/services/countLeft.cpp:19-21
    return ORB_OK;
}

orb_status orb_partition(orb_ctx *ctx, const orb_cell_t *cells, uint32_t n_cells) {
    if (!ctx) return ORB_ERR_INVALID_ARGUMENT;
    ctx->err.clear();
    ORB_CUDA(cudaSetDevice(ctx->device));
    Level v;
    orb_status st = service_prepare(ctx, cells, n_cells, true, &v);
    if (st != ORB_OK || n_cells == 0) return st;
    cudaStream_t s = ctx->stream;
    ORB_CUDA(cudaMemsetAsync(&ctx->counters.p->error, 0, sizeof(uint32_t), s));
    run_kernel(ctx, kKPlan, v, 1);
    run_kernel(ctx, kKTileMap, v, pass_grid(ctx));
    partition_level(ctx, v, false);
    ORB_CUDA(cudaGetLastError());
    ORB_CUDA(cudaMemcpyAsync(&ctx->h_counters->error, &ctx->counters.p->error, sizeof(uint32_t),
                             cudaMemcpyDeviceToHost, s));
    ORB_CUDA(cudaStreamSynchronize(s));
    collect_profile(ctx);
    if (ctx->h_counters->error)
        return fail(ctx, ORB_ERR_TIMEOUT, "a bounded device wait gave up or a bisection did not finish");
    return ORB_OK;
}

orb_status orb_get_ranges(orb_ctx *ctx, uint32_t *ranges, uint32_t n_cells) {
    if (!ctx) return ORB_ERR_INVALID_ARGUMENT;
    ctx->err.clear();
    if (!ctx->loaded) return fail(ctx, ORB_ERR_NOT_LOADED, "no particles loaded");
    if (!ranges || n_cells > ctx->loaded_cells) return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "bad range request");
    ORB_CUDA(cudaSetDevice(ctx->device));
    ORB_CUDA(cudaMemcpyAsync(ranges, ctx->ranges.p, n_cells * sizeof(uint2), cudaMemcpyDeviceToHost, ctx->stream));
    ORB_CUDA(cudaStreamSynchronize(ctx->stream));
    return ORB_OK;
}

orb_status orb_set_ranges(orb_ctx *ctx, const uint32_t *ranges, uint32_t n_cells) {
    if (!ctx) return ORB_ERR_INVALID_ARGUMENT;
    ctx->err.clear();
    if (!ctx->loaded) return fail(ctx, ORB_ERR_NOT_LOADED, "no particles loaded");
    if (!ranges || n_cells > ctx->loaded_cells) return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "bad range request");
    for (uint32_t i = 0; i < n_cells; ++i)
        if (ranges[2 * i] > ranges[2 * i + 1] || ranges[2 * i + 1] > ctx->loaded_n)
            return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "range outside the loaded particles");
    ORB_CUDA(cudaSetDevice(ctx->device));
    ORB_CUDA(cudaMemcpyAsync(ctx->ranges.p, ranges, n_cells * sizeof(uint2), cudaMemcpyHostToDevice, ctx->stream));
    ORB_CUDA(cudaStreamSynchronize(ctx->stream));
    return ORB_OK;
}

// ---------------------------------------------------------------------------------------
// Batched builds
// ---------------------------------------------------------------------------------------
// Batched build; with prev_heaps, a warm build (widths[i] > 0: instance i's cells start from
// the previous tree's cuts, see orb_build_batch_warm).
static orb_status build_batch_impl(orb_ctx *ctx, float *x, float *y, float *z, uint64_t n_total,
                                   const orb_batch_instance *inst, uint32_t k,
                                   const orb_cell_t *prev_heaps, const float *widths,
                                   orb_cell_t *heaps, uint32_t *ranges, uint32_t *perm,
                                   uint32_t flags, orb_build_info *info) {
    if (!ctx) return ORB_ERR_INVALID_ARGUMENT;
    ctx->err.clear();
    ctx->yz_pending = false;  // batched builds copy their inputs before the build
    if (flags & ~ORB_DEVICE_POINTERS) return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "unknown flags");
    if ((n_total > 0 && (!x || !y || !z)) || (k > 0 && (!inst || !heaps || !ranges)))
        return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "null pointer");
    if (n_total >= (1ull << 31)) return fail(ctx, ORB_ERR_CAPACITY, "n_total must be below 2^31");
    const bool dev = (flags & ORB_DEVICE_POINTERS) != 0;
    if (dev && n_total > 0 && (!is_device_ptr(x) || !is_device_ptr(y) || !is_device_ptr(z) ||
                               (perm && !is_device_ptr(perm))))
        return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "ORB_DEVICE_POINTERS set but a pointer is not device memory");
    // validate instances, heap bases, per-level slot lists
    std::vector<BatchRoot> roots(k);
    std::vector<uint32_t> lev(k);
    uint64_t heap_cells = 0;
    uint32_t max_levels = 0;
    std::vector<std::pair<uint64_t, uint64_t>> spans;
    for (uint32_t i = 0; i < k; ++i) {
        const orb_batch_instance &b = inst[i];
        if (b.d == 0 || b.d > (1u << 30))
            return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "instance d must be in [1, 2^30]");
        if (b.offset + b.n > n_total) return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "instance outside the arrays");
        const Slices sl(b.d);
        const uint32_t L = b.levels ? b.levels : sl.max_levels();
        if (L > sl.max_levels())
            return fail(ctx, ORB_ERR_INVALID_ARGUMENT,
                        "instance levels exceeds log2(d) (d a power of two) or ceil(log2 d) - 1");
        lev[i] = L;
        max_levels = std::max(max_levels, L);
        BatchRoot &r = roots[i];
        r.offset = (uint32_t)b.offset;
        r.n = (uint32_t)b.n;
        r.d = b.d;
        r.heap_base = (uint32_t)heap_cells;
        for (int a = 0; a < 3; ++a) {
            r.lower[a] = b.lower[a];
            r.upper[a] = b.upper[a];
        }
        heap_cells += 2ull * b.d - 1;
        if (b.n) spans.emplace_back(b.offset, b.offset + b.n);
    }
    if (heap_cells >= (1ull << 31)) return fail(ctx, ORB_ERR_CAPACITY, "too many cells");
    std::sort(spans.begin(), spans.end());
    for (size_t i = 1; i < spans.size(); ++i)
        if (spans[i].first < spans[i - 1].second)
            return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "instances overlap");
    std::vector<int> slots;
    std::vector<LevelDesc> lv;
    std::vector<size_t> lv_off;
    uint32_t max_cells = 1;
    for (uint32_t l = 1; l <= max_levels; ++l) {
        lv_off.push_back(slots.size());
        for (uint32_t i = 0; i < k; ++i) {
            if (lev[i] < l) continue;
            const Slices sl(inst[i].d);
            const int first = (int)roots[i].heap_base + sl.first(l);
            for (int j = 0; j < sl.count(l); ++j) slots.push_back(first + j);
        }
        max_cells = std::max<uint32_t>(max_cells, (uint32_t)(slots.size() - lv_off.back()));
    }
    ORB_CUDA(cudaSetDevice(ctx->device));
    orb_status st = ensure_level_buffers(ctx, n_total, max_cells, (uint32_t)heap_cells);
    if (st != ORB_OK) return st;
    ORB_CUDA(ctx->idx.ensure(n_total + 1));
    ORB_CUDA(ctx->batch_roots.ensure(k + 1));
    ORB_CUDA(ctx->batch_slots.ensure(slots.size() + 1));
    cudaStream_t s = ctx->stream;
    float *dx = x, *dy = y, *dz = z;
    float h2d_ms = 0.f, d2h_ms = 0.f;
    if (!dev) {
        ORB_CUDA(ctx->x.ensure(n_total + 1));
        ORB_CUDA(ctx->y.ensure(n_total + 1));
        ORB_CUDA(ctx->z.ensure(n_total + 1));
        dx = ctx->x.p;
        dy = ctx->y.p;
        dz = ctx->z.p;
        ORB_CUDA(cudaEventRecord(ctx->ev[2], s));
        if (n_total) {
            ORB_CUDA(cudaMemcpyAsync(dx, x, n_total * sizeof(float), cudaMemcpyHostToDevice, s));
            ORB_CUDA(cudaMemcpyAsync(dy, y, n_total * sizeof(float), cudaMemcpyHostToDevice, s));
            ORB_CUDA(cudaMemcpyAsync(dz, z, n_total * sizeof(float), cudaMemcpyHostToDevice, s));
        }
        ORB_CUDA(cudaEventRecord(ctx->ev[3], s));
    }
    bool warm = false;
    if (prev_heaps) {
        // starting brackets from the previous trees on the cut axis: cut +- w x extent / sqrt(n)
        std::vector<float2> hint(heap_cells);
        std::vector<int> hint_axis(heap_cells, -2);
        const float nan = std::numeric_limits<float>::quiet_NaN();
        for (uint32_t i = 0; i < k; ++i) {
            const uint64_t hb = roots[i].heap_base, hc = 2ull * inst[i].d - 1;
            for (uint64_t j = 0; j < hc; ++j) {
                hint[hb + j] = make_float2(nan, nan);
                const orb_cell_t &p = prev_heaps[hb + j];
                if (!(widths[i] > 0.f) || p.nLeafCells < 2 || p.cutAxis < 0 || p.cutAxis > 2) continue;
                const int a = p.cutAxis;
                const float cut = (p.cutMarginRight + p.cutMarginLeft) * 0.5f;
                // (cut, w x extent); the device divides the extent part by sqrt(n) of the cell
                const float wext = widths[i] * (p.upper[a] - p.lower[a]);
                if (!std::isfinite(cut) || !std::isfinite(wext)) continue;
                hint[hb + j] = make_float2(cut, wext);
                hint_axis[hb + j] = a;
                warm = true;
            }
        }
        if (warm) {
            ORB_CUDA(ctx->hint.ensure(heap_cells + 1));
            ORB_CUDA(ctx->hint_axis.ensure(heap_cells + 1));
            ORB_CUDA(ctx->warm.ensure(max_cells + 1));
            ORB_CUDA(cudaMemcpyAsync(ctx->hint.p, hint.data(), heap_cells * sizeof(float2), cudaMemcpyHostToDevice, s));
            ORB_CUDA(cudaMemcpyAsync(ctx->hint_axis.p, hint_axis.data(), heap_cells * sizeof(int), cudaMemcpyHostToDevice, s));
            ORB_CUDA(cudaStreamSynchronize(s));  // the host vectors go out of scope
        }
    }
    if (k) ORB_CUDA(cudaMemcpyAsync(ctx->batch_roots.p, roots.data(), k * sizeof(BatchRoot), cudaMemcpyHostToDevice, s));
    if (!slots.empty())
        ORB_CUDA(cudaMemcpyAsync(ctx->batch_slots.p, slots.data(), slots.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    ORB_CUDA(cudaEventRecord(ctx->ev[0], s));
    Level v = make_level(ctx, dx, dy, dz);
    if (!perm) v.idx = nullptr;  // no permutation asked for: only x, y, z move
    if (warm) {
        v.hint = ctx->hint.p;
        v.hint_axis = ctx->hint_axis.p;
        v.warm = ctx->warm.p;
    }
    for (uint32_t l = 1; l <= max_levels; ++l) {
        const size_t a = lv_off[l - 1], b = l < max_levels ? lv_off[l] : slots.size();
        lv.push_back({0, ctx->batch_slots.p + a, (int)(b - a)});
    }
    std::vector<uint64_t> key = level_key(ctx, v);
    key.push_back(warm ? 0xBA7C4A : 0xBA7C4);  // batched build (warm)
    key_add(key, v.hint);
    key_add(key, v.warm);
    key.push_back(n_total);
    key_add(key, ctx->batch_roots.p);
    key_add(key, ctx->batch_slots.p);
    for (uint32_t i = 0; i < k; ++i) {
        key.push_back(inst[i].offset);
        key.push_back(inst[i].n);
        key.push_back(((uint64_t)inst[i].d << 32) | lev[i]);
        for (int a = 0; a < 3; ++a) {
            key_add_f(key, inst[i].lower[a]);
            key_add_f(key, inst[i].upper[a]);
        }
    }
    // subtrees when every instance is built to its leaves; in warm builds the subtree levels
    // bisect from each cell's extent (hints apply to the levels above them)
    bool full = true;
    uint64_t max_n = 0;
    for (uint32_t i = 0; i < k; ++i) {
        const Slices sl(inst[i].d);
        full = full && sl.pow2 && lev[i] == sl.depth;
        max_n = std::max<uint64_t>(max_n, inst[i].n);
    }
    const int sub_from = subtree_from(ctx, lv, max_n, full);
    if (sub_from >= 0) ORB_CUDA(ctx->sub_flag.ensure(1));
    key.push_back((uint64_t)(int64_t)sub_from);
    uint32_t passes = 0;
    st = run_graphed(ctx, key, &passes, [&](uint32_t *pp) -> orb_status {
        ORB_CUDA(cudaMemsetAsync(ctx->heap.p, 0, heap_cells * sizeof(orb_cell_t), s));
        ORB_CUDA(cudaMemsetAsync(ctx->ranges.p, 0, heap_cells * sizeof(uint2), s));
        ORB_CUDA(cudaMemsetAsync(ctx->counters.p, 0, sizeof(BuildCounters), s));
        ctx->launches[kKInit] += 1;
        launch_init_batch(v, ctx->batch_roots.p, (int)k, n_total, s);
        ORB_CUDA(cudaGetLastError());
        return run_levels(ctx, v, lv, pp, sub_from, max_n);
    });
    if (st != ORB_OK) return st;
    ORB_CUDA(cudaEventRecord(ctx->ev[1], s));
    bool taken = false;
    st = finish_subtree_levels(ctx, v, lv, key, &passes, sub_from, max_n, &taken);
    if (st != ORB_OK) return st;
    if (!dev) {
        ORB_CUDA(cudaStreamSynchronize(s));
        ORB_CUDA(cudaEventElapsedTime(&h2d_ms, ctx->ev[2], ctx->ev[3]));
        ORB_CUDA(cudaEventRecord(ctx->ev[2], s));
        if (n_total) {
            ORB_CUDA(cudaMemcpyAsync(x, dx, n_total * sizeof(float), cudaMemcpyDeviceToHost, s));
            ORB_CUDA(cudaMemcpyAsync(y, dy, n_total * sizeof(float), cudaMemcpyDeviceToHost, s));
            ORB_CUDA(cudaMemcpyAsync(z, dz, n_total * sizeof(float), cudaMemcpyDeviceToHost, s));
        }
    }
    if (perm && n_total) {
        if (dev) {  // only the instances' positions: the rest of `perm` is the caller's
            launch_copy_instances(ctx->idx.p, perm, ctx->batch_roots.p, (int)k, s);
            ORB_CUDA(cudaGetLastError());
        } else {
            ORB_CUDA(cudaMemcpyAsync(perm, ctx->idx.p, n_total * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        }
    }
    if (heap_cells) {
        ORB_CUDA(cudaMemcpyAsync(heaps, ctx->heap.p, heap_cells * sizeof(orb_cell_t), cudaMemcpyDeviceToHost, s));
        ORB_CUDA(cudaMemcpyAsync(ranges, ctx->ranges.p, heap_cells * sizeof(uint2), cudaMemcpyDeviceToHost, s));
    }
    ORB_CUDA(cudaMemcpyAsync(ctx->h_counters, ctx->counters.p, sizeof(BuildCounters), cudaMemcpyDeviceToHost, s));
    if (!dev) ORB_CUDA(cudaEventRecord(ctx->ev[3], s));
    ORB_CUDA(cudaStreamSynchronize(s));
    if (ctx->h_counters->error)
        return fail(ctx, ORB_ERR_TIMEOUT, "a bounded device wait gave up or a bisection did not finish");
    // ranges relative to each instance (cells the build filled)
    for (uint32_t i = 0; i < k; ++i) {
        const uint64_t filled = Slices(inst[i].d).filled(lev[i]);
        uint32_t *r = ranges + 2ull * roots[i].heap_base;
        for (uint64_t j = 0; j < 2 * filled; ++j) r[j] -= roots[i].offset;
    }
    float dev_ms = 0.f;
    ORB_CUDA(cudaEventElapsedTime(&dev_ms, ctx->ev[0], ctx->ev[1]));
    collect_profile(ctx);
    if (ctx->use_graphs) collect_graph_profile(ctx);
    for (int kk = 0; kk < kNumKernels; ++kk) ctx->prof_bytes[kk] += (double)ctx->h_counters->bytes[kk];
    if (!dev) ORB_CUDA(cudaEventElapsedTime(&d2h_ms, ctx->ev[2], ctx->ev[3]));
    if (info) {
        std::memset(info, 0, sizeof *info);
        info->levels_built = max_levels;
        info->degenerate_cells = ctx->h_counters->degenerate;
        info->zero_volume_cells = ctx->h_counters->zero_volume;
        info->unfound_cells = ctx->h_counters->unfound;
        info->max_iterations = ctx->h_counters->max_iters;
        info->count_passes = passes;
        info->device_ms = dev_ms;
        info->h2d_ms = h2d_ms;
        info->d2h_ms = d2h_ms;
        info->warm_cells = ctx->h_counters->warm_cells;
        info->warm_resets = ctx->h_counters->warm_resets;
        info->sampled_cells = ctx->h_counters->pred_cells;
        info->sampled_misses = ctx->h_counters->pred_misses;
    }
    return ORB_OK;
}

orb_status orb_build_batch(orb_ctx *ctx, float *x, float *y, float *z, uint64_t n_total,
                           const orb_batch_instance *inst, uint32_t k, orb_cell_t *heaps,
                           uint32_t *ranges, uint32_t *perm, uint32_t flags,
                           orb_build_info *info) {
    const orb_status st = build_batch_impl(ctx, x, y, z, n_total, inst, k, nullptr, nullptr, heaps,
                                           ranges, perm, flags, info);
    if (st != ORB_OK && ctx && !(flags & ORB_DEVICE_POINTERS)) drain_host_copies(ctx);
    return st;
}

orb_status orb_build_batch_warm(orb_ctx *ctx, float *x, float *y, float *z, uint64_t n_total,
                                const orb_batch_instance *inst, uint32_t k,
                                const orb_cell_t *prev_heaps, const float *widths,
                                orb_cell_t *heaps, uint32_t *ranges, uint32_t *perm,
                                uint32_t flags, orb_build_info *info) {
    if (!ctx) return ORB_ERR_INVALID_ARGUMENT;
    ctx->err.clear();
    if (k > 0 && (!prev_heaps || !widths)) return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "null prev_heaps or widths");
    for (uint32_t i = 0; i < k; ++i)
        if (!(widths[i] >= 0.f) || !std::isfinite(widths[i]))
            return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "widths must be finite and >= 0");
    const orb_status st = build_batch_impl(ctx, x, y, z, n_total, inst, k, prev_heaps, widths,
                                           heaps, ranges, perm, flags, info);
    if (st != ORB_OK && !(flags & ORB_DEVICE_POINTERS)) drain_host_copies(ctx);
    return st;
}

orb_status orb_build_warm(orb_ctx *ctx, float *x, float *y, float *z, uint64_t n, uint32_t d,
                          uint32_t levels, const float lower[3], const float upper[3],
                          const orb_cell_t *prev_heap, float width, orb_cell_t *heap_out,
                          uint32_t *ranges_out, uint32_t *perm, uint32_t flags,
                          orb_build_info *info) {
    if (!ctx) return ORB_ERR_INVALID_ARGUMENT;
    ctx->err.clear();
    if (!lower || !upper) return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "null box");
    orb_batch_instance b;
    b.offset = 0;
    b.n = n;
    b.d = d;
    b.levels = levels;
    for (int a = 0; a < 3; ++a) {
        b.lower[a] = lower[a];
        b.upper[a] = upper[a];
    }
    return orb_build_batch_warm(ctx, x, y, z, n, &b, 1, prev_heap, &width, heap_out, ranges_out, perm,
                                flags, info);
}

orb_status orb_test_set_scan_wait(orb_ctx *ctx, uint32_t spin_limit, uint32_t ticket_start) {
    if (!ctx) return ORB_ERR_INVALID_ARGUMENT;
    ctx->err.clear();
    if (ticket_start > 255) return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "ticket_start above 255");
    ctx->spin_limit = spin_limit ? spin_limit : kLookbackSpinLimit;
    ctx->scan_ticket_start = ticket_start;
    return ORB_OK;
}

orb_status orb_get_tuning(orb_ctx *ctx, orb_tuning *out) {
    if (!ctx || !out) return ORB_ERR_INVALID_ARGUMENT;
    *out = ctx->tune;
    return ORB_OK;
}

static bool tuning_valid(const orb_tuning &t) {
    return t.hist_blocks_per_sm >= 1 && t.hist_blocks_per_sm <= 8 &&
           t.part_blocks_per_sm >= 1 && t.part_blocks_per_sm <= 16 && t.tile_blocks_per_sm >= 1 &&
           t.tile_blocks_per_sm <= 8 && t.sparse_keys_per_tile >= 1 &&
           t.sparse_keys_per_tile <= (uint32_t)kTile && t.subtree_levels <= (uint32_t)kSubMaxLevels &&
           t.predict_sigmas <= 16;
}

orb_status orb_set_tuning(orb_ctx *ctx, const orb_tuning *t) {
    if (!ctx) return ORB_ERR_INVALID_ARGUMENT;
    ctx->err.clear();
    if (!t || !tuning_valid(*t)) return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "tuning parameter out of range");
    ctx->tune = *t;
    return ORB_OK;
}

orb_status orb_autotune_batch(orb_ctx *ctx, const float *x, const float *y, const float *z,
                              uint64_t n_total, const orb_batch_instance *inst, uint32_t k,
                              uint32_t flags, uint32_t reps, orb_tuning *best, float *best_ms) {
    if (!ctx) return ORB_ERR_INVALID_ARGUMENT;
    ctx->err.clear();
    if (flags & ~ORB_DEVICE_POINTERS) return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "unknown flags");
    if (!best || !best_ms || reps < 1 || reps > 100 || k == 0 || !inst ||
        (n_total > 0 && (!x || !y || !z)))
        return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "null pointer, no instances or reps outside 1..100");
    if (n_total >= (1ull << 31)) return fail(ctx, ORB_ERR_CAPACITY, "n_total must be below 2^31");
    const bool dev = (flags & ORB_DEVICE_POINTERS) != 0;
    if (dev && n_total > 0 && (!is_device_ptr(x) || !is_device_ptr(y) || !is_device_ptr(z)))
        return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "ORB_DEVICE_POINTERS set but a pointer is not device memory");
    uint64_t heap_cells = 0;
    for (uint32_t i = 0; i < k; ++i) {
        if (inst[i].d == 0 || inst[i].d > (1u << 30)) return fail(ctx, ORB_ERR_INVALID_ARGUMENT, "instance d");
        heap_cells += 2ull * inst[i].d - 1;
    }
    ORB_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const float *in[3] = {x, y, z};
    for (int a = 0; a < 3; ++a) {
        ORB_CUDA(ctx->tune_src[a].ensure(n_total + 1));
        ORB_CUDA(ctx->tune_work[a].ensure(n_total + 1));
        if (n_total)
            ORB_CUDA(cudaMemcpyAsync(ctx->tune_src[a].p, in[a], n_total * sizeof(float),
                                     dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
    }
    std::vector<orb_cell_t> heaps(heap_cells), ref_heaps;
    std::vector<uint32_t> ranges(2 * heap_cells), ref_ranges;
    // median device time of `reps` builds (after one untimed build: graph capture)
    auto trial = [&](const orb_tuning &t, float *ms) -> orb_status {
        ctx->tune = t;
        std::vector<float> times;
        for (uint32_t r = 0; r <= reps; ++r) {
            for (int a = 0; a < 3; ++a)
                if (n_total)
                    ORB_CUDA(cudaMemcpyAsync(ctx->tune_work[a].p, ctx->tune_src[a].p,
                                             n_total * sizeof(float), cudaMemcpyDeviceToDevice, s));
            orb_build_info info;
            orb_status st = orb_build_batch(ctx, ctx->tune_work[0].p, ctx->tune_work[1].p,
                                            ctx->tune_work[2].p, n_total, inst, k, heaps.data(),
                                            ranges.data(), nullptr, ORB_DEVICE_POINTERS, &info);
            if (st != ORB_OK) return st;
            if (r == 0) {
                if (ref_heaps.empty()) {
                    ref_heaps = heaps;
                    ref_ranges = ranges;
                } else if (std::memcmp(ref_heaps.data(), heaps.data(), heaps.size() * sizeof(orb_cell_t)) ||
                           ref_ranges != ranges) {
                    return fail(ctx, ORB_ERR_CUDA, "autotune: a candidate setting built a different tree");
                }
            } else {
                times.push_back(info.device_ms);
            }
        }
        std::sort(times.begin(), times.end());
        *ms = times[times.size() / 2];
        return ORB_OK;
    };
    const orb_tuning start = ctx->tune;
    orb_tuning cur = start;
    float cur_ms = 0.f;
    orb_status st = trial(cur, &cur_ms);
    if (st != ORB_OK) {
        ctx->tune = start;
        return st;
    }
    // coordinate descent over result-invariant parameters
    static const uint32_t hist_c[] = {4, 6, 8}, part_c[] = {4, 8, 16}, tile_c[] = {2, 4},
                          sparse_c[] = {16, 64, 256}, cta_c[] = {0, 512, 4096},
                          sub_c[] = {0, 2, 3, 4, 6}, pred_c[] = {0, 4, 5, 7};
    struct Axis {
        uint32_t orb_tuning::*field;
        const uint32_t *vals;
        int n;
    };
    const Axis axes[] = {{&orb_tuning::hist_blocks_per_sm, hist_c, 3},
                         {&orb_tuning::part_blocks_per_sm, part_c, 3},
                         {&orb_tuning::tile_blocks_per_sm, tile_c, 2},
                         {&orb_tuning::sparse_keys_per_tile, sparse_c, 3},
                         {&orb_tuning::cta_min_cells, cta_c, 3},
                         {&orb_tuning::subtree_levels, sub_c, 5},
                         {&orb_tuning::predict_sigmas, pred_c, 4}};
    for (const Axis &ax : axes) {
        const orb_tuning base = cur;
        for (int i = 0; i < ax.n; ++i) {
            if (ax.vals[i] == base.*ax.field) continue;
            orb_tuning t = base;
            t.*ax.field = ax.vals[i];
            float ms = 0.f;
            st = trial(t, &ms);
            if (st != ORB_OK) {
                ctx->tune = start;
                return st;
            }
            if (ms < 0.98f * cur_ms) {  // keep a candidate only for a clear gain
                cur = t;
                cur_ms = ms;
            }
        }
    }
    ctx->tune = cur;
    *best = cur;
    *best_ms = cur_ms;
    return ORB_OK;
}

// ---------------------------------------------------------------------------------------
// Profiling
// ---------------------------------------------------------------------------------------
orb_status orb_profile_reset(orb_ctx *ctx, uint32_t timing_mask) {
    if (!ctx) return ORB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    collect_profile(ctx);
    for (int k = 0; k < kNumKernels; ++k) {
        ctx->launches[k] = 0;
        ctx->prof_ms[k] = 0.0;
        ctx->prof_bytes[k] = 0.0;
    }
    ctx->prof_mask = timing_mask;
    return ORB_OK;
}

int orb_profile_kernel_index(const char *name) {
    if (!name) return -1;
    for (int k = 0; k < kNumKernels; ++k)
        if (std::strcmp(name, kKernelNames[k]) == 0) return k;
    return -1;
}

int orb_profile_read(orb_ctx *ctx, orb_kernel_stat *out, int max_entries) {
    if (!ctx) return -1;
    int n = 0;
    for (int k = 0; k < kNumKernels; ++k) {
        if (!ctx->launches[k]) continue;
        if (out && n < max_entries) {
            orb_kernel_stat &o = out[n];
            std::memset(&o, 0, sizeof o);
            std::strncpy(o.name, kKernelNames[k], sizeof(o.name) - 1);
            o.launches = ctx->launches[k];
            o.total_ms = ctx->prof_ms[k];
            o.bytes = ctx->prof_bytes[k];
        }
        ++n;
    }
    return n;
}

}  // extern "C"
