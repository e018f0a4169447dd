// ORB request server (continuous batching), include/orb/orb.h orb_server_*.
//
// The reference builds one tree per program run (src/orbit.cpp:22-289). The server keeps
// many instances resident on the GPU and answers a stream of requests: builds of new
// instances and rebalances (Gaussian displacement + rebuild) of resident ones.
//
//  * Resident state: every instance owns a contiguous slot of a device particle arena
//    (x, y, z, the permutation of the last build, the original index of every particle),
//    sized from the HBM budget; its latest cell heap and range map are kept on the host.
//  * Admission: a build is admitted when its slot can be allocated in the arena (first
//    fit); a rebalance when its instance is not already in flight. Requests that do not fit
//    wait in FIFO order until memory frees up (orb_server_release).
//  * Continuous batching: each lane (its own engine context and stream) takes every
//    admissible pending request, up to max_batch, into one batched build; with several
//    lanes, batches overlap on the device while new requests queue for the next free lane.
//  * Results are bit-identical to the same operations run one at a time: a batched build is
//    bit-identical per instance to a plain build, and each instance's operations are applied
//    in submission order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "orb_internal.cuh"

namespace {

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// First-fit allocator of particle ranges in the arena.
class RangeAlloc {
   public:
    explicit RangeAlloc(uint64_t cap) { if (cap) free_[0] = cap; }
    bool alloc(uint64_t n, uint64_t *off) {
        if (n == 0) {
            *off = 0;
            return true;
        }
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= n) {
                *off = it->first;
                const uint64_t rest = it->second - n, at = it->first + n;
                free_.erase(it);
                if (rest) free_[at] = rest;
                used_ += n;
                return true;
            }
        }
        return false;
    }
    void release(uint64_t off, uint64_t n) {
        if (n == 0) return;
        used_ -= n;
        auto it = free_.emplace(off, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    uint64_t used() const { return used_; }

   private:
    std::map<uint64_t, uint64_t> free_;
    uint64_t used_ = 0;
};

enum ReqKind { kBuild = 0, kGenerate = 1, kRebalance = 2 };

struct Req {
    uint64_t id = 0;
    uint64_t inst = 0;
    int kind = kBuild;
    std::vector<float> hx, hy, hz;  // kBuild: the particles, copied at submission
    int gen_kind = 0;               // kGenerate
    uint64_t seed = 0;              // kGenerate: generator seed; kRebalance: displacement seed
    float sigma = 0.f;
    float warm = 0.f;               // kRebalance: > 0 = warm rebuild, bracket half-width
    double t_submit = 0, t_start = 0, t_done = 0;
    orb_status status = ORB_OK;
    bool done = false;
    uint32_t batch = 0;  // requests in the batch that served it
};

struct Inst {
    uint64_t id = 0;
    uint64_t off = 0, n = 0;
    uint32_t d = 0, levels = 0;
    float lower[3], upper[3];
    bool allocated = false, built = false, released = false;
    int inflight = 0;  // requests admitted and not finished
    std::vector<orb_cell_t> heap;
    std::vector<uint32_t> ranges;
};

}  // namespace

struct orb_server {
    int device = 0;
    orb_server_opts opts{};
    uint64_t arena_cap = 0;
    float *ax = nullptr, *ay = nullptr, *az = nullptr;
    uint32_t *aperm = nullptr, *aident = nullptr, *atmp = nullptr;
    std::unique_ptr<RangeAlloc> arena;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Req *> pending;
    std::unordered_map<uint64_t, std::unique_ptr<Req>> reqs;
    std::unordered_map<uint64_t, Inst> insts;
    std::deque<uint64_t> finished;  // completed request ids not yet polled
    struct Lane {
        orb_ctx *ctx = nullptr;
        std::thread th;
    };
    std::vector<Lane> lanes;
    bool stop = false;
    uint64_t next_id = 1;
    orb_server_stats stats{};
};

namespace {

// Requests admissible right now, FIFO, up to max_batch. Caller holds the lock.
std::vector<Req *> admit(orb_server *sv) {
    std::vector<Req *> batch;
    const uint32_t cap = sv->opts.max_batch ? sv->opts.max_batch : 0xffffffffu;
    std::vector<uint64_t> taken;  // instances with a request in this batch
    for (auto it = sv->pending.begin(); it != sv->pending.end() && batch.size() < cap;) {
        Req *r = *it;
        Inst &in = sv->insts[r->inst];
        bool ok = false;
        // one request per instance per batch, in submission order per instance
        const bool earlier_pending = std::find(taken.begin(), taken.end(), r->inst) != taken.end();
        if (!earlier_pending && in.inflight == 0) {
            if (r->kind == kRebalance) {
                ok = in.built && !in.released;
            } else if (in.allocated) {
                ok = true;
            } else {
                uint64_t off;
                if (sv->arena->alloc(in.n, &off)) {
                    in.off = off;
                    in.allocated = true;
                    ok = true;
                }
            }
        }
        if (r->kind == kRebalance && !earlier_pending && in.inflight == 0 && (!in.built || in.released)) {
            // target gone: finish with an error
            r->status = ORB_ERR_INVALID_ARGUMENT;
            r->done = true;
            r->t_start = r->t_done = now_s();
            sv->finished.push_back(r->id);
            it = sv->pending.erase(it);
            sv->cv_done.notify_all();
            continue;
        }
        if (ok) {
            in.inflight += 1;
            taken.push_back(r->inst);
            batch.push_back(r);
            it = sv->pending.erase(it);
        } else {
            if (std::find(taken.begin(), taken.end(), r->inst) == taken.end()) taken.push_back(r->inst);
            ++it;
        }
    }
    return batch;
}

void lane_loop(orb_server *sv, int lane) {
    cudaSetDevice(sv->device);
    orb_ctx *ctx = sv->lanes[lane].ctx;
    cudaStream_t st = orb::ctx_stream(ctx);
    std::vector<orb_cell_t> heaps, prev;
    std::vector<uint32_t> rgs;
    std::vector<float> widths;
    for (;;) {
        std::vector<Req *> batch;
        std::vector<Inst *> ins;  // element pointers of an unordered_map stay valid
        {
            std::unique_lock<std::mutex> lk(sv->mu);
            for (;;) {
                if (sv->stop) return;
                batch = admit(sv);
                if (!batch.empty()) break;
                sv->cv_work.wait(lk);
            }
            const double t = now_s();
            for (Req *r : batch) {
                r->t_start = t;
                r->batch = (uint32_t)batch.size();
                ins.push_back(&sv->insts.at(r->inst));
            }
        }
        // device work of the batch on this lane's stream
        std::vector<orb_batch_instance> desc(batch.size());
        orb_status status = ORB_OK;
        size_t heap_cells = 0;
        for (size_t i = 0; i < batch.size(); ++i) {
            Req *r = batch[i];
            Inst &in = *ins[i];  // only this lane touches an admitted instance
            orb_batch_instance &b = desc[i];
            b.offset = in.off;
            b.n = in.n;
            b.d = in.d;
            b.levels = in.levels;
            std::memcpy(b.lower, in.lower, sizeof b.lower);
            std::memcpy(b.upper, in.upper, sizeof b.upper);
            heap_cells += 2ull * in.d - 1;
            if (status != ORB_OK) continue;
            if (r->kind == kBuild && in.n) {
                cudaMemcpyAsync(sv->ax + in.off, r->hx.data(), in.n * sizeof(float), cudaMemcpyHostToDevice, st);
                cudaMemcpyAsync(sv->ay + in.off, r->hy.data(), in.n * sizeof(float), cudaMemcpyHostToDevice, st);
                cudaMemcpyAsync(sv->az + in.off, r->hz.data(), in.n * sizeof(float), cudaMemcpyHostToDevice, st);
            } else if (r->kind == kGenerate && in.n) {
                status = orb_generate(ctx, r->gen_kind, r->seed, in.n, sv->ax + in.off, sv->ay + in.off,
                                      sv->az + in.off, ORB_DEVICE_POINTERS);
            } else if (r->kind == kRebalance) {
                orb::launch_displace(sv->ax, sv->ay, sv->az, in.off, in.n, r->seed, r->sigma, in.lower,
                                     in.upper, st);
            }
            if (r->kind != kRebalance)  // identity of a new instance's particles
                orb::launch_iota_u32(sv->aident + in.off, in.n, st);
        }
        if (cudaGetLastError() != cudaSuccess && status == ORB_OK) status = ORB_ERR_CUDA;
        heaps.resize(std::max<size_t>(heap_cells, 1));
        rgs.resize(2 * std::max<size_t>(heap_cells, 1));
        orb_build_info info;
        // warm rebalances start from their instance's current tree (a labelled mode: not
        // bit-identical with a cold rebuild); every other request of the batch builds cold
        bool any_warm = false;
        for (size_t i = 0; i < batch.size(); ++i)
            any_warm |= batch[i]->kind == kRebalance && batch[i]->warm > 0.f && ins[i]->heap.size() == 2ull * ins[i]->d - 1;
        if (status == ORB_OK && any_warm) {
            prev.assign(std::max<size_t>(heap_cells, 1), orb_cell_t{});
            widths.assign(batch.size(), 0.f);
            size_t hb = 0;
            for (size_t i = 0; i < batch.size(); ++i) {
                const size_t hc = 2ull * ins[i]->d - 1;
                if (batch[i]->kind == kRebalance && batch[i]->warm > 0.f && ins[i]->heap.size() == hc) {
                    std::copy(ins[i]->heap.begin(), ins[i]->heap.end(), prev.begin() + hb);
                    widths[i] = batch[i]->warm;
                }
                hb += hc;
            }
            status = orb_build_batch_warm(ctx, sv->ax, sv->ay, sv->az, sv->arena_cap, desc.data(),
                                          (uint32_t)desc.size(), prev.data(), widths.data(), heaps.data(),
                                          rgs.data(), sv->aperm, ORB_DEVICE_POINTERS, &info);
        } else if (status == ORB_OK) {
            status = orb_build_batch(ctx, sv->ax, sv->ay, sv->az, sv->arena_cap, desc.data(), (uint32_t)desc.size(),
                                     heaps.data(), rgs.data(), sv->aperm, ORB_DEVICE_POINTERS, &info);
        }
        if (status == ORB_OK) {
            // original index of every particle: ident <- ident[perm] per instance
            for (const orb_batch_instance &b : desc) {
                orb::launch_gather_u32(sv->atmp, sv->aident, sv->aperm, b.offset, b.n, st);
                if (b.n)
                    cudaMemcpyAsync(sv->aident + b.offset, sv->atmp + b.offset, b.n * sizeof(uint32_t),
                                    cudaMemcpyDeviceToDevice, st);
            }
            if (cudaStreamSynchronize(st) != cudaSuccess) status = ORB_ERR_CUDA;
        }
        {
            std::lock_guard<std::mutex> lk(sv->mu);
            const double t = now_s();
            size_t hb = 0;
            for (size_t i = 0; i < batch.size(); ++i) {
                Req *r = batch[i];
                Inst &in = *ins[i];
                const size_t hc = 2ull * in.d - 1;
                if (status == ORB_OK) {
                    in.heap.assign(heaps.begin() + hb, heaps.begin() + hb + hc);
                    in.ranges.assign(rgs.begin() + 2 * hb, rgs.begin() + 2 * (hb + hc));
                    in.built = true;
                }
                hb += hc;
                in.inflight -= 1;
                r->status = status;
                r->done = true;
                r->t_done = t;
                r->hx.clear();
                r->hx.shrink_to_fit();
                r->hy.clear();
                r->hy.shrink_to_fit();
                r->hz.clear();
                r->hz.shrink_to_fit();
                sv->finished.push_back(r->id);
                sv->stats.requests_done += 1;
                if (r->kind == kRebalance)
                    sv->stats.rebalances += 1;
                else
                    sv->stats.builds += 1;
                sv->stats.particles_built += in.n;
            }
            sv->stats.batches += 1;
            sv->stats.max_batch_seen = std::max<uint32_t>(sv->stats.max_batch_seen, (uint32_t)batch.size());
        }
        sv->cv_done.notify_all();
        sv->cv_work.notify_all();
    }
}

orb_status submit(orb_server *sv, std::unique_ptr<Req> r, uint64_t *request_id) {
    std::lock_guard<std::mutex> lk(sv->mu);
    r->id = sv->next_id++;
    r->t_submit = now_s();
    if (request_id) *request_id = r->id;
    sv->pending.push_back(r.get());
    sv->reqs[r->id] = std::move(r);
    sv->stats.requests_submitted += 1;
    sv->cv_work.notify_all();
    return ORB_OK;
}

orb_status new_instance(orb_server *sv, uint64_t n, uint32_t d, uint32_t levels, const float lower[3],
                        const float upper[3], std::unique_ptr<Req> &r, uint64_t *request_id) {
    if (d == 0 || d > (1u << 30)) return ORB_ERR_INVALID_ARGUMENT;
    const uint32_t ylev = orb::Slices(d).max_levels();
    if (levels > ylev) return ORB_ERR_INVALID_ARGUMENT;
    if (n > sv->arena_cap) return ORB_ERR_CAPACITY;  // can never be admitted
    std::lock_guard<std::mutex> lk(sv->mu);
    const uint64_t id = sv->next_id;  // the build request's id names the instance
    Inst in;
    in.id = id;
    in.n = n;
    in.d = d;
    in.levels = levels ? levels : ylev;
    for (int a = 0; a < 3; ++a) {
        in.lower[a] = lower ? lower[a] : -0.5f;
        in.upper[a] = upper ? upper[a] : 0.5f;
    }
    sv->insts[id] = std::move(in);
    r->inst = id;
    r->id = sv->next_id++;
    r->t_submit = now_s();
    if (request_id) *request_id = r->id;
    sv->pending.push_back(r.get());
    sv->reqs[r->id] = std::move(r);
    sv->stats.requests_submitted += 1;
    sv->cv_work.notify_all();
    return ORB_OK;
}

void fill_result(const Req &r, orb_request_result *out) {
    out->request_id = r.id;
    out->instance_id = r.inst;
    out->status = r.status;
    out->kind = r.kind == kRebalance ? 1 : 0;
    out->batch_size = r.batch;
    out->submit_s = r.t_submit;
    out->start_s = r.t_start;
    out->done_s = r.t_done;
}

}  // namespace

extern "C" {

orb_status orb_server_create(int device, const orb_server_opts *opts, orb_server **out) {
    if (!out || !opts || opts->hbm_budget_bytes == 0) return ORB_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    const uint32_t lanes = opts->lanes ? opts->lanes : 2;
    if (lanes > 16) return ORB_ERR_INVALID_ARGUMENT;
    if (cudaSetDevice(device) != cudaSuccess) return ORB_ERR_CUDA;
    orb_server *sv = new (std::nothrow) orb_server();
    if (!sv) return ORB_ERR_OUT_OF_MEMORY;
    sv->device = device;
    sv->opts = *opts;
    sv->opts.lanes = lanes;
    // Per arena particle: x,y,z + perm + identity + gather scratch (24 B) and each lane's
    // build scratch (about 9 B: permutation, histogram pool, edge tables, bitmasks, tiles).
    sv->arena_cap = opts->hbm_budget_bytes / (24ull + 9ull * lanes);
    if (sv->arena_cap >= (1ull << 31)) sv->arena_cap = (1ull << 31) - 1;
    sv->arena.reset(new RangeAlloc(sv->arena_cap));
    orb_status st = ORB_OK;
    const size_t nb = (size_t)sv->arena_cap + 1;
    if (cudaMalloc(&sv->ax, nb * 4) || cudaMalloc(&sv->ay, nb * 4) || cudaMalloc(&sv->az, nb * 4) ||
        cudaMalloc(&sv->aperm, nb * 4) || cudaMalloc(&sv->aident, nb * 4) || cudaMalloc(&sv->atmp, nb * 4)) {
        cudaGetLastError();
        st = ORB_ERR_OUT_OF_MEMORY;
    }
    sv->lanes.resize(lanes);
    for (uint32_t i = 0; st == ORB_OK && i < lanes; ++i) {
        orb_opts o{};
        st = orb_ctx_create(device, &o, &sv->lanes[i].ctx);
        if (st == ORB_OK) orb::ctx_disable_graphs(sv->lanes[i].ctx);  // every batch differs
    }
    if (st != ORB_OK) {
        sv->lanes.clear();
        orb_server_destroy(sv);
        return st;
    }
    for (uint32_t i = 0; i < lanes; ++i) sv->lanes[i].th = std::thread(lane_loop, sv, (int)i);
    *out = sv;
    return ORB_OK;
}

orb_status orb_server_destroy(orb_server *sv) {
    if (!sv) return ORB_ERR_INVALID_ARGUMENT;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stop = true;
    }
    sv->cv_work.notify_all();
    for (auto &l : sv->lanes)
        if (l.th.joinable()) l.th.join();
    for (auto &l : sv->lanes)
        if (l.ctx) orb_ctx_destroy(l.ctx);
    cudaSetDevice(sv->device);
    for (void *p : {(void *)sv->ax, (void *)sv->ay, (void *)sv->az, (void *)sv->aperm, (void *)sv->aident,
                    (void *)sv->atmp})
        if (p) cudaFree(p);
    delete sv;
    return ORB_OK;
}

orb_status orb_server_submit_build(orb_server *sv, const float *x, const float *y, const float *z,
                                   uint64_t n, uint32_t d, uint32_t levels, const float lower[3],
                                   const float upper[3], uint64_t *request_id) {
    if (!sv || (n && (!x || !y || !z))) return ORB_ERR_INVALID_ARGUMENT;
    std::unique_ptr<Req> r(new Req());
    r->kind = kBuild;
    r->hx.assign(x, x + n);
    r->hy.assign(y, y + n);
    r->hz.assign(z, z + n);
    return new_instance(sv, n, d, levels, lower, upper, r, request_id);
}

orb_status orb_server_submit_generate(orb_server *sv, int kind, uint64_t seed, uint64_t n, uint32_t d,
                                      uint32_t levels, uint64_t *request_id) {
    if (!sv || (kind != ORB_GEN_UNIFORM && kind != ORB_GEN_PLUMMER)) return ORB_ERR_INVALID_ARGUMENT;
    std::unique_ptr<Req> r(new Req());
    r->kind = kGenerate;
    r->gen_kind = kind;
    r->seed = seed;
    return new_instance(sv, n, d, levels, nullptr, nullptr, r, request_id);
}

static orb_status submit_rebalance(orb_server *sv, uint64_t instance_id, uint64_t seed, float sigma,
                                   float warm, uint64_t *request_id) {
    if (!sv || !(sigma >= 0.f) || !(warm >= 0.f) || !std::isfinite(warm)) return ORB_ERR_INVALID_ARGUMENT;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        auto it = sv->insts.find(instance_id);
        if (it == sv->insts.end() || it->second.released) return ORB_ERR_INVALID_ARGUMENT;
    }
    std::unique_ptr<Req> r(new Req());
    r->kind = kRebalance;
    r->inst = instance_id;
    r->seed = seed;
    r->sigma = sigma;
    r->warm = warm;
    return submit(sv, std::move(r), request_id);
}

orb_status orb_server_submit_rebalance(orb_server *sv, uint64_t instance_id, uint64_t seed, float sigma,
                                       uint64_t *request_id) {
    return submit_rebalance(sv, instance_id, seed, sigma, 0.f, request_id);
}

orb_status orb_server_submit_rebalance_warm(orb_server *sv, uint64_t instance_id, uint64_t seed,
                                            float sigma, float width, uint64_t *request_id) {
    if (!(width > 0.f)) return ORB_ERR_INVALID_ARGUMENT;
    return submit_rebalance(sv, instance_id, seed, sigma, width, request_id);
}

orb_status orb_server_wait(orb_server *sv, uint64_t request_id, orb_request_result *out) {
    if (!sv) return ORB_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(sv->mu);
    auto it = sv->reqs.find(request_id);
    if (it == sv->reqs.end()) return ORB_ERR_INVALID_ARGUMENT;
    Req *r = it->second.get();
    sv->cv_done.wait(lk, [&] { return r->done; });
    if (out) fill_result(*r, out);
    return r->status;
}

orb_status orb_server_poll(orb_server *sv, orb_request_result *out, uint32_t max, uint32_t *n_out) {
    if (!sv || !n_out) return ORB_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(sv->mu);
    uint32_t n = 0;
    while (n < max && !sv->finished.empty()) {
        const uint64_t id = sv->finished.front();
        sv->finished.pop_front();
        if (out) fill_result(*sv->reqs.at(id), &out[n]);
        ++n;
    }
    *n_out = n;
    return ORB_OK;
}

orb_status orb_server_fetch(orb_server *sv, uint64_t instance_id, orb_cell_t *heap, uint32_t *ranges,
                            float *x, float *y, float *z, uint32_t *ident) {
    if (!sv) return ORB_ERR_INVALID_ARGUMENT;
    uint64_t off, n;
    {
        std::unique_lock<std::mutex> lk(sv->mu);
        auto it = sv->insts.find(instance_id);
        if (it == sv->insts.end() || it->second.released) return ORB_ERR_INVALID_ARGUMENT;
        Inst &in = it->second;
        sv->cv_done.wait(lk, [&] { return in.inflight == 0; });
        if (!in.built) return ORB_ERR_NOT_LOADED;
        if (heap) std::memcpy(heap, in.heap.data(), in.heap.size() * sizeof(orb_cell_t));
        if (ranges) std::memcpy(ranges, in.ranges.data(), in.ranges.size() * sizeof(uint32_t));
        off = in.off;
        n = in.n;
        in.inflight += 1;  // hold the slot while copying
    }
    cudaSetDevice(sv->device);
    cudaError_t e = cudaSuccess;
    if (n) {
        if (x && !e) e = cudaMemcpy(x, sv->ax + off, n * 4, cudaMemcpyDeviceToHost);
        if (y && !e) e = cudaMemcpy(y, sv->ay + off, n * 4, cudaMemcpyDeviceToHost);
        if (z && !e) e = cudaMemcpy(z, sv->az + off, n * 4, cudaMemcpyDeviceToHost);
        if (ident && !e) e = cudaMemcpy(ident, sv->aident + off, n * 4, cudaMemcpyDeviceToHost);
    }
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->insts.at(instance_id).inflight -= 1;
    }
    sv->cv_work.notify_all();
    return e == cudaSuccess ? ORB_OK : ORB_ERR_CUDA;
}

orb_status orb_server_release(orb_server *sv, uint64_t instance_id) {
    if (!sv) return ORB_ERR_INVALID_ARGUMENT;
    {
        std::unique_lock<std::mutex> lk(sv->mu);
        auto it = sv->insts.find(instance_id);
        if (it == sv->insts.end() || it->second.released) return ORB_ERR_INVALID_ARGUMENT;
        Inst &in = it->second;
        // wait for every pending and in-flight request of the instance
        sv->cv_done.wait(lk, [&] {
            if (in.inflight) return false;
            for (Req *r : sv->pending)
                if (r->inst == instance_id) return false;
            return true;
        });
        if (in.allocated) sv->arena->release(in.off, in.n);
        in.allocated = false;
        in.released = true;
        in.heap.clear();
        in.ranges.clear();
    }
    sv->cv_work.notify_all();  // memory freed: waiting builds may now be admitted
    return ORB_OK;
}

orb_status orb_server_get_stats(orb_server *sv, orb_server_stats *out) {
    if (!sv || !out) return ORB_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(sv->mu);
    *out = sv->stats;
    out->arena_particles = sv->arena_cap;
    out->arena_used = sv->arena->used();
    out->pending = (uint32_t)sv->pending.size();
    return ORB_OK;
}

}  // extern "C"
