// ORB oracle: CPU restatement of the reference's o=0 path. TEST INFRASTRUCTURE ONLY.
// The product library never links or calls this file. Build with -ffp-contract=off so the
// float32 control arithmetic is evaluated as separately rounded operations, as the
// reference's x86-64 build does.
#include "orb_oracle.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------------------------------
// Seeded counter-based generator (splitmix64 finaliser). Identical in the engine's
// device generator; tests compare the two bit for bit.
// ---------------------------------------------------------------------------------------
inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

inline uint64_t draw(uint64_t seed, uint64_t counter) {
    return mix64(mix64(seed) + counter * 0xD1B54A32D192ED03ull);
}

// 24 random bits on the 2^-24 grid of [-0.5, 0.5): exact in float32.
inline float unit_coord(uint64_t u) {
    return (float)(uint32_t)(u >> 40) * 0x1p-24f - 0.5f;
}

inline double unit_double(uint64_t u) { return (double)(u >> 11) * 0x1p-53; }

constexpr uint64_t kClusterDomain = 0xC1A57E5C1A57E5C1ull;
constexpr int kClusters = 64;
constexpr uint64_t kPlummerStride = 64;  // counters reserved per particle

template <class F>
void parallel_chunks(uint64_t n, int nthreads, F &&f) {
    if (nthreads <= 1 || n < (1u << 16)) {
        f(0, n);
        return;
    }
    std::vector<std::thread> th;
    uint64_t chunk = (n + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; ++t) {
        uint64_t b = t * chunk, e = std::min<uint64_t>(n, b + chunk);
        if (b >= e) break;
        th.emplace_back([&f, b, e] { f(b, e); });
    }
    for (auto &t : th) t.join();
}

// ---------------------------------------------------------------------------------------
// Reference Cell semantics (src/cell.h).
// ---------------------------------------------------------------------------------------
using Cell = oracle_cell_t;
static_assert(sizeof(Cell) == 52, "Cell must keep the reference's 52-byte layout");

Cell make_cell(int id, int n_leaf, const float *lower, const float *upper) {  // cell.h:19-45
    Cell c;
    std::memset(&c, 0, sizeof c);
    c.id = id;
    c.nLeafCells = n_leaf;
    c.foundCut = 0;
    c.prevCutAxis = -1;
    c.cutAxis = -1;
    c.cutMarginLeft = 0.0f;
    c.cutMarginRight = 0.0f;
    for (int k = 0; k < 3; ++k) {
        c.lower[k] = lower[k];
        c.upper[k] = upper[k];
    }
    return c;
}

inline float get_cut(const Cell &c) {  // cell.h:74-76
    return (float)((double)(c.cutMarginRight + c.cutMarginLeft) / 2.0);
}

inline int eff_axis(const Cell &c) { return c.cutAxis < 0 ? 0 : c.cutAxis; }

void set_cut_axis(Cell &c, uint32_t *zero_volume) {  // cell.h:102-121
    int max_d = -1;
    float max_size = 0.0f;
    for (int k = 0; k < 3; ++k) {
        float size = c.upper[k] - c.lower[k];
        if (size > max_size) {
            max_size = size;
            max_d = k;
        }
    }
    c.cutAxis = max_d;
    if (max_d < 0 && zero_volume) ++*zero_volume;
}

void set_cut_margin(Cell &c) {  // cell.h:123-126 (axis -1 -> axis 0, see header)
    int a = eff_axis(c);
    c.cutMarginLeft = c.lower[a];
    c.cutMarginRight = c.upper[a];
}

void split(const Cell &p, Cell &left, Cell &right, uint32_t *zero_volume) {  // cell.h:78-100
    int n_left = (int)std::ceil(p.nLeafCells / 2.0);
    int n_right = p.nLeafCells - n_left;
    float cut = get_cut(p);
    int a = eff_axis(p);
    left = make_cell(2 * p.id + 1, n_left, p.lower, p.upper);
    left.upper[a] = cut;
    left.prevCutAxis = p.cutAxis;
    right = make_cell(2 * p.id + 2, n_right, p.lower, p.upper);
    right.lower[a] = cut;
    right.prevCutAxis = p.cutAxis;
    // orbit.cpp:240-243
    set_cut_axis(right, zero_volume);
    set_cut_margin(right);
    set_cut_axis(left, zero_volume);
    set_cut_margin(left);
}

// orbit.cpp:204-208: ratio = ceil(n/2.0)/n as float; difference = int(float(cl) - float(c)*ratio)
int convergence(uint32_t count_left, uint32_t count, int32_t n_leaf, int32_t *diff_out) {
    float ratio = (float)(std::ceil(n_leaf / 2.0) / n_leaf);
    float prod = (float)count * ratio;
    float diff_f = (float)count_left - prod;
    int32_t difference = (int32_t)diff_f;
    if (diff_out) *diff_out = difference;
    if (std::abs(difference) < 3) return 0;
    return difference > 0 ? 1 : -1;
}

// Weighted ORB (documentation/notes.tex:259-271, 326-336: the left cell gets the share
// ceil(k/2)/k of the cell's weight; never implemented by the reference). Weights are
// integers, so the sums are exact in any order. The test is the reference's
// |W_left - ratio W| < 3 (src/orbit.cpp:204-208) with the tolerance scaled by the cell's
// mean weight W/n and evaluated exactly in 128-bit integers:
//   D = k W_left - ceil(k/2) W;  found when D == 0 or n |D| < 3 k W;  else the right margin
//   moves for D > 0 and the left one for D < 0.
// With every weight 1 this is |cl - ratio c| < 3 exactly: the reference's float32 test
// whenever that test is exact (counts below 2^24, an even k).
int convergence_weighted(uint64_t w_left, uint64_t w_cell, uint64_t n, int32_t n_leaf) {
    const __int128 k = n_leaf, half = (n_leaf + 1) / 2;
    const __int128 D = k * (__int128)w_left - half * (__int128)w_cell;
    const unsigned __int128 ad = (unsigned __int128)(D < 0 ? -D : D);
    if (D == 0 || (unsigned __int128)n * ad < (unsigned __int128)3 * (unsigned __int128)k * w_cell) return 0;
    return D > 0 ? 1 : -1;
}

uint64_t weight_left(const float *keys, const uint32_t *w, uint64_t begin, uint64_t end, float cut) {
    uint64_t s = 0;
    for (uint64_t p = begin; p < end; ++p) s += keys[p] < cut ? w[p] : 0u;
    return s;
}

uint32_t count_left(const float *keys, uint64_t begin, uint64_t end, float cut) {  // countLeft.cpp:31-36
    uint32_t n_left = 0;
    for (const float *p = keys + begin, *e = keys + end; p < e; ++p) n_left += *p < cut;
    return n_left;
}

inline void swap3(float *x, float *y, float *z, uint32_t *perm, int64_t a, int64_t b,
                  uint32_t *wt = nullptr) {
    std::swap(x[a], x[b]);
    std::swap(y[a], y[b]);
    std::swap(z[a], z[b]);
    if (perm) std::swap(perm[a], perm[b]);
    if (wt) std::swap(wt[a], wt[b]);
}

// partition.cpp:30-52 with the scan clamped at the cell end (weights, if any, move with
// their particles).
int64_t hoare(float *x, float *y, float *z, uint32_t *perm, int64_t begin, int64_t end,
              int axis, float cut, bool final_swap, int *degenerate, uint32_t *wt = nullptr) {
    float *key = axis == 0 ? x : (axis == 1 ? y : z);
    int64_t i = begin - 1, j = end;
    for (;;) {
        do {
            ++i;
        } while (i < end && key[i] < cut);
        do {
            --j;
        } while (j >= begin && key[j] > cut);
        if (i >= j) break;
        swap3(x, y, z, perm, i, j, wt);
    }
    if (i < end) {
        if (final_swap) swap3(x, y, z, perm, i, end - 1, wt);
        if (degenerate) *degenerate = 0;
    } else {
        i = end;
        if (degenerate) *degenerate = 1;
    }
    return i;
}

// Persistent worker pool: one thread per rank, fork/join per phase (MDL RunService).
class RankPool {
   public:
    explicit RankPool(int n) : n_(n) {
        for (int r = 1; r < n; ++r) workers_.emplace_back([this, r] { loop(r); });
    }
    ~RankPool() {
        {
            std::lock_guard<std::mutex> g(m_);
            stop_ = true;
            ++gen_;
        }
        cv_.notify_all();
        for (auto &t : workers_) t.join();
    }
    void run(const std::function<void(int)> &f) {
        if (n_ == 1) {
            f(0);
            return;
        }
        {
            std::lock_guard<std::mutex> g(m_);
            fn_ = f;
            pending_ = n_ - 1;
            ++gen_;
        }
        cv_.notify_all();
        f(0);
        std::unique_lock<std::mutex> lk(m_);
        done_.wait(lk, [&] { return pending_ == 0; });
    }

   private:
    void loop(int r) {
        uint64_t seen = 0;
        for (;;) {
            std::function<void(int)> f;
            {
                std::unique_lock<std::mutex> lk(m_);
                cv_.wait(lk, [&] { return gen_ != seen; });
                seen = gen_;
                if (stop_) return;
                f = fn_;
            }
            f(r);
            {
                std::lock_guard<std::mutex> g(m_);
                if (--pending_ == 0) done_.notify_one();
            }
        }
    }
    int n_;
    std::vector<std::thread> workers_;
    std::mutex m_;
    std::condition_variable cv_, done_;
    std::function<void(int)> fn_;
    int pending_ = 0;
    uint64_t gen_ = 0;
    bool stop_ = false;
};

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

}  // namespace

extern "C" {

uint64_t oracle_draw(uint64_t seed, uint64_t counter) { return draw(seed, counter); }

void oracle_gen_uniform(uint64_t seed, uint64_t n, float *x, float *y, float *z, int nthreads) {
    parallel_chunks(n, nthreads, [=](uint64_t b, uint64_t e) {
        for (uint64_t i = b; i < e; ++i) {
            x[i] = unit_coord(draw(seed, 3 * i + 0));
            y[i] = unit_coord(draw(seed, 3 * i + 1));
            z[i] = unit_coord(draw(seed, 3 * i + 2));
        }
    });
}

void oracle_plummer_clusters(uint64_t seed, float *centres, double *scales) {
    const uint64_t dom = seed ^ kClusterDomain;
    for (int k = 0; k < kClusters; ++k) {
        for (int a = 0; a < 3; ++a) centres[3 * k + a] = unit_coord(draw(dom, 4 * k + a));
        double u = unit_double(draw(dom, 4 * k + 3));
        scales[k] = 0.005 * std::pow(10.0, u);  // log-uniform in [0.005, 0.05)
    }
}

void oracle_gen_plummer(uint64_t seed, uint64_t n, float *x, float *y, float *z, int nthreads) {
    float centres[3 * kClusters];
    double scales[kClusters];
    oracle_plummer_clusters(seed, centres, scales);
    const float hi = std::nextafter(0.5f, -1.0f);
    parallel_chunks(n, nthreads, [&](uint64_t b, uint64_t e) {
        for (uint64_t i = b; i < e; ++i) {
            const uint64_t c = i * kPlummerStride;
            uint64_t sel = draw(seed, c) >> 40;
            float p[3];
            if (sel * 10 < 9ull * (1ull << 24)) {  // 90%: Plummer sphere member
                int k = (int)(draw(seed, c + 1) % kClusters);
                double w = unit_double(draw(seed, c + 2));
                w = std::fmax(w, unit_double(draw(seed, c + 3)));
                w = std::fmax(w, unit_double(draw(seed, c + 4)));
                // Plummer enclosed mass m(r) = r^3/(r^2+a^2)^1.5; w = m^(1/3) has density 3w^2,
                // so w = max of three uniforms and r = a w / sqrt(1 - w^2).
                double r = scales[k] * w / std::sqrt(1.0 - w * w);
                double v[3] = {1.0, 0.0, 0.0}, q = 1.0;
                for (int t = 0; t < 19; ++t) {
                    double u[3];
                    for (int a = 0; a < 3; ++a)
                        u[a] = 2.0 * unit_double(draw(seed, c + 5 + 3 * t + a)) - 1.0;
                    double qq = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
                    if (qq > 0.0 && qq <= 1.0) {
                        v[0] = u[0];
                        v[1] = u[1];
                        v[2] = u[2];
                        q = qq;
                        break;
                    }
                }
                double s = r / std::sqrt(q);
                for (int a = 0; a < 3; ++a) {
                    float f = (float)((double)centres[3 * k + a] + v[a] * s);
                    p[a] = std::fmin(std::fmax(f, -0.5f), hi);
                }
            } else {  // 10%: uniform background
                for (int a = 0; a < 3; ++a) p[a] = unit_coord(draw(seed, c + 2 + a));
            }
            x[i] = p[0];
            y[i] = p[1];
            z[i] = p[2];
        }
    });
}

// The reference's generator, src/services/init.cu:11-25: three 64-bit words (unsigned long on
// its LP64 targets) from the seeds 123456789, 362436069, 521288629 at process start, one
// xorshift step per draw, the value (float)z / ULONG_MAX - 0.5 (the division in float by
// the float nearest ULONG_MAX, 2^64; the subtraction in double, then rounded to float), and
// particles(i, d) filled for i = 0.., d = 0, 1, 2 (init.cu:48-52): the single-rank input of
// `orbit N d 0`.
void oracle_gen_xorshf96(uint64_t n, float *x, float *y, float *z) {
    uint64_t sx = 123456789, sy = 362436069, sz = 521288629;
    auto draw = [&]() -> float {
        uint64_t t;
        sx ^= sx << 16;
        sx ^= sx >> 5;
        sx ^= sx << 1;
        t = sx;
        sx = sy;
        sy = sz;
        sz = t ^ sx ^ sy;
        return (float)sz / (float)UINT64_MAX - 0.5;
    };
    for (uint64_t i = 0; i < n; ++i) {
        x[i] = draw();
        y[i] = draw();
        z[i] = draw();
    }
}

float oracle_get_cut(float margin_left, float margin_right) {
    Cell c;
    c.cutMarginLeft = margin_left;
    c.cutMarginRight = margin_right;
    return get_cut(c);
}

int oracle_convergence(uint32_t count_left_v, uint32_t count, int32_t n_leaf_cells,
                       int32_t *difference_out) {
    return convergence(count_left_v, count, n_leaf_cells, difference_out);
}

uint32_t oracle_count_left(const float *keys, uint64_t begin, uint64_t end, float cut) {
    return count_left(keys, begin, end, cut);
}

int64_t oracle_hoare(float *x, float *y, float *z, uint32_t *perm, uint64_t begin, uint64_t end,
                     int axis, float cut, int final_swap, int *degenerate) {
    return hoare(x, y, z, perm, (int64_t)begin, (int64_t)end, axis, cut, final_swap != 0,
                 degenerate);
}

// Cell::getNLevels() and getNCellsOnLastLevel() (src/cell.h:65-72) for nLeafCells = d:
// depth = ceil(log2 d), last = 2d - 2^depth.
void oracle_level_shape(uint32_t d, uint32_t *depth, uint32_t *last) {
    uint32_t k = 0;
    while ((1ull << k) < d) ++k;
    *depth = k;
    *last = (uint32_t)(2ull * d - (1ull << k));
}

// Split levels a build of d leaves may run: log2(d) for a power of two (every cell split
// down to one leaf); otherwise the reference driver's own bound, getNLevels() - 1
// (src/orbit.cpp:102), since its level slices name no complete level below it.
uint32_t oracle_max_levels(uint32_t d) {
    uint32_t depth, last;
    oracle_level_shape(d, &depth, &last);
    if ((d & (d - 1)) == 0) return depth;
    return depth ? depth - 1 : 0;
}

int oracle_build(float *x, float *y, float *z, uint64_t n, uint32_t d, uint32_t levels,
                 const float lower[3], const float upper[3], oracle_cell_t *heap,
                 uint32_t *ranges, uint32_t *perm, uint8_t *iters, int nranks, int make_axis,
                 int threads, oracle_stats_t *stats) {
    if (!x || !y || !z || !heap || !ranges || d == 0 || d > (1u << 30)) return -1;
    if (n >= (1ull << 31)) return -2;
    if (levels > oracle_max_levels(d) || levels >= ORACLE_MAX_LEVELS) return -3;
    if (nranks < 1) nranks = 1;
    if ((uint64_t)nranks > std::max<uint64_t>(n, 1)) nranks = (int)std::max<uint64_t>(n, 1);
    if (threads < 1 || nranks > 1) threads = 1;  // cell-parallel only in single-rank mode
    uint32_t depth, last_cells;
    oracle_level_shape(d, &depth, &last_cells);

    oracle_stats_t st;
    std::memset(&st, 0, sizeof st);
    st.nranks = (uint32_t)nranks;
    const double t0 = now_s();

    const uint64_t heap_size = 2ull * d - 1;
    std::memset(heap, 0, heap_size * sizeof(Cell));
    std::memset(ranges, 0, (size_t)nranks * heap_size * 2 * sizeof(uint32_t));
    if (iters) std::memset(iters, 0, heap_size);
    if (perm)
        for (uint64_t i = 0; i < n; ++i) perm[i] = (uint32_t)i;

    // orbit.cpp:74-81
    Cell root = make_cell(0, (int)d, lower, upper);
    root.cutAxis = 0;
    set_cut_margin(root);
    heap[0] = root;

    // Rank slabs (orbit.cpp:83: N/Threads() particles per rank; the remainder goes to the
    // last rank here so every particle is owned).
    struct Rank {
        uint64_t off, n;
        uint32_t *rng;
        std::vector<float> axis_t;
        std::vector<uint32_t> out;
    };
    std::vector<Rank> rk(nranks);
    for (int r = 0; r < nranks; ++r) {
        rk[r].off = (n / nranks) * r;
        rk[r].n = (r == nranks - 1) ? n - rk[r].off : n / nranks;
        rk[r].rng = ranges + (size_t)r * heap_size * 2;
        rk[r].rng[0] = 0;
        rk[r].rng[1] = (uint32_t)rk[r].n;
        if (make_axis) rk[r].axis_t.resize(rk[r].n + 1);
    }
    RankPool pool(std::max(nranks, threads));

    std::vector<uint32_t> counts, counts_left;
    std::vector<std::atomic<uint32_t>> degen(1);
    degen[0] = 0;

    for (uint32_t l = 1; l <= levels; ++l) {
        // orbit.cpp:104-111: cells [2^(l-1)-1, min(getNCellsOnLastLevel(), 2^l) - 2]. For
        // some d that is not a power of two the slice is empty (b < a); the reference then
        // runs its services on a non-positive cell count, which is undefined: here the
        // level does nothing.
        const int a = (1 << (l - 1)) - 1;
        const int b = std::min<int>((int)last_cells, 1 << l) - 2;
        const int n_cells = b - a + 1;
        if (n_cells <= 0) {
            st.levels_built = l;
            continue;
        }
        Cell *cells = heap + a;
        counts.assign(n_cells, 0);
        counts_left.assign(n_cells, 0);

        if (make_axis) {  // makeAxis.cpp:16-30
            double ts = now_s();
            pool.run([&](int r) {
                if (r >= nranks) return;
                Rank &R = rk[r];
                for (int c = 0; c < n_cells; ++c) {
                    const Cell &cell = cells[c];
                    uint32_t bg = R.rng[2 * cell.id], en = R.rng[2 * cell.id + 1];
                    const float *src = (eff_axis(cell) == 0 ? x : eff_axis(cell) == 1 ? y : z) + R.off;
                    if (en > bg) std::memcpy(R.axis_t.data() + bg, src + bg, (en - bg) * sizeof(float));
                }
            });
            st.t_make_axis_s += now_s() - ts;
        }

        // count.cpp:14-17 + Combine (sum over ranks)
        for (int r = 0; r < nranks; ++r)
            for (int c = 0; c < n_cells; ++c)
                counts[c] += rk[r].rng[2 * cells[c].id + 1] - rk[r].rng[2 * cells[c].id];

        // orbit.cpp:146-232
        double ts = now_s();
        if (threads > 1) {
            // Single rank, cells in parallel. The loop of orbit.cpp:146-232 treats the cells of
            // a level independently: a cell's margins, counts and its test depend on that cell
            // alone, and the loop ends for it once it is found or at the 32nd sweep, whatever
            // the other cells do. So every cell runs its own loop here, with the same counts,
            // the same test and the same cap: identical cells, iterations and statistics.
            // A level of fewer cells than threads splits each count over the threads instead
            // (an integer sum, so the split does not change it).
            const float *axes[3] = {x, y, z};
            std::vector<uint32_t> jdone(n_cells, 0);
            std::vector<uint64_t> counted(n_cells, 0);
            auto bisect = [&](int c, auto &&count_fn) {
                Cell &cell = cells[c];
                int j = 0;
                while (!cell.foundCut && j < 32) {
                    ++j;
                    const uint32_t bg = rk[0].rng[2 * cell.id], en = rk[0].rng[2 * cell.id + 1];
                    const uint32_t cl = count_fn(axes[eff_axis(cell)], bg, en, get_cut(cell));
                    counted[c] += counts[c];
                    if (iters) iters[cell.id] = (uint8_t)j;
                    const int dir = convergence(cl, counts[c], cell.nLeafCells, nullptr);
                    if (dir == 0)
                        cell.foundCut = 1;
                    else if (dir > 0)
                        cell.cutMarginRight = get_cut(cell);
                    else
                        cell.cutMarginLeft = get_cut(cell);
                }
                jdone[c] = (uint32_t)j;
            };
            if (n_cells >= threads) {
                std::atomic<int> next(0);
                pool.run([&](int) {
                    for (int c; (c = next.fetch_add(1)) < n_cells;)
                        bisect(c, [](const float *k, uint32_t bg, uint32_t en, float cut) {
                            return count_left(k, bg, en, cut);
                        });
                });
            } else {
                std::vector<uint32_t> part(threads);
                for (int c = 0; c < n_cells; ++c)
                    bisect(c, [&](const float *k, uint32_t bg, uint32_t en, float cut) {
                        const uint64_t len = en - bg, chunk = (len + threads - 1) / threads;
                        pool.run([&](int t) {
                            const uint64_t b0 = std::min<uint64_t>(len, t * chunk);
                            const uint64_t e0 = std::min<uint64_t>(len, b0 + chunk);
                            part[t] = count_left(k, bg + b0, bg + e0, cut);
                        });
                        uint32_t s = 0;
                        for (uint32_t v : part) s += v;
                        return s;
                    });
            }
            uint32_t jmax = 0;
            for (int c = 0; c < n_cells; ++c) {
                jmax = std::max(jmax, jdone[c]);
                st.cell_counts += jdone[c];
                st.elements_counted += counted[c];
                st.elements_per_level[l - 1] += counted[c];
            }
            // the level loop of orbit.cpp:148 runs until every cell is found or 32 sweeps
            st.iterations[l - 1] = jmax;
        } else {
            bool found_all = false;
            int j = 0;
            while (!found_all && j < 32) {
                ++j;
                found_all = true;
                pool.run([&](int r) {  // countLeft.cpp:16-39 on every rank
                    if (r >= nranks) return;
                    Rank &R = rk[r];
                    R.out.assign(n_cells, 0);
                    for (int c = 0; c < n_cells; ++c) {
                        const Cell &cell = cells[c];
                        if (cell.foundCut) continue;
                        uint32_t bg = R.rng[2 * cell.id], en = R.rng[2 * cell.id + 1];
                        const float *keys;
                        if (make_axis) {
                            keys = R.axis_t.data();
                        } else {
                            int ax = eff_axis(cell);
                            keys = (ax == 0 ? x : ax == 1 ? y : z) + R.off;
                        }
                        R.out[c] = count_left(keys, bg, en, get_cut(cell));
                    }
                });
                for (int c = 0; c < n_cells; ++c) {  // Combine: elementwise sum
                    uint32_t s = 0;
                    for (int r = 0; r < nranks; ++r) s += rk[r].out[c];
                    counts_left[c] = s;
                }
                for (int c = 0; c < n_cells; ++c) {
                    Cell &cell = cells[c];
                    if (cell.foundCut) continue;
                    ++st.cell_counts;
                    st.elements_counted += counts[c];
                    st.elements_per_level[l - 1] += counts[c];
                    if (iters) iters[cell.id] = (uint8_t)j;
                    int dir = convergence(counts_left[c], counts[c], cell.nLeafCells, nullptr);
                    if (dir == 0) {
                        cell.foundCut = 1;
                    } else if (dir > 0) {
                        cell.cutMarginRight = get_cut(cell);
                        found_all = false;
                    } else {
                        cell.cutMarginLeft = get_cut(cell);
                        found_all = false;
                    }
                }
            }
            st.iterations[l - 1] = (uint32_t)j;
        }
        st.t_count_s += now_s() - ts;
        for (int c = 0; c < n_cells; ++c)
            if (!cells[c].foundCut) ++st.unfound_cells;

        // orbit.cpp:235-250
        for (int c = 0; c < n_cells; ++c) {
            Cell lc, rc;
            split(cells[c], lc, rc, &st.zero_volume_cells);
            heap[lc.id] = lc;
            heap[rc.id] = rc;
        }

        // partition.cpp:18-62 on every rank (single rank with threads: cells in parallel,
        // their ranges are disjoint)
        ts = now_s();
        auto part_cell = [&](Rank &R, const Cell &cell) -> uint32_t {
            uint32_t bg = R.rng[2 * cell.id], en = R.rng[2 * cell.id + 1];
            int dg = 0;
            int64_t i = hoare(x + R.off, y + R.off, z + R.off, perm ? perm + R.off : nullptr, bg, en,
                              eff_axis(cell), get_cut(cell), true, &dg);
            const int lcid = 2 * cell.id + 1, rcid = 2 * cell.id + 2;
            R.rng[2 * lcid] = bg;
            R.rng[2 * lcid + 1] = (uint32_t)i;
            R.rng[2 * rcid] = (uint32_t)i;
            R.rng[2 * rcid + 1] = en;
            return (uint32_t)dg;
        };
        if (threads > 1) {
            std::atomic<int> next(0);
            pool.run([&](int) {
                uint32_t local_degen = 0;
                for (int c; (c = next.fetch_add(1)) < n_cells;) local_degen += part_cell(rk[0], cells[c]);
                degen[0] += local_degen;
            });
        } else {
            pool.run([&](int r) {
                if (r >= nranks) return;
                uint32_t local_degen = 0;
                for (int c = 0; c < n_cells; ++c) local_degen += part_cell(rk[r], cells[c]);
                degen[0] += local_degen;
            });
        }
        st.t_partition_s += now_s() - ts;
        st.levels_built = l;
    }
    st.degenerate_cells = degen[0];
    st.t_total_s = now_s() - t0;
    if (stats) *stats = st;
    return 0;
}

int oracle_convergence_weighted(uint64_t w_left, uint64_t w_cell, uint64_t n, int32_t n_leaf) {
    return convergence_weighted(w_left, w_cell, n, n_leaf);
}

int oracle_build_weighted(float *x, float *y, float *z, uint32_t *w, uint64_t n, uint32_t d,
                          uint32_t levels, const float lower[3], const float upper[3],
                          oracle_cell_t *heap, uint32_t *ranges, uint32_t *perm, uint8_t *iters,
                          int threads, oracle_stats_t *stats) {
    if (!x || !y || !z || !w || !heap || !ranges || d == 0 || d > (1u << 30)) return -1;
    if (n >= (1ull << 31)) return -2;
    if (levels > oracle_max_levels(d) || levels >= ORACLE_MAX_LEVELS) return -3;
    if (threads < 1) threads = 1;
    uint32_t depth, last_cells;
    oracle_level_shape(d, &depth, &last_cells);
    oracle_stats_t st;
    std::memset(&st, 0, sizeof st);
    st.nranks = 1;
    const double t0 = now_s();
    const uint64_t heap_size = 2ull * d - 1;
    std::memset(heap, 0, heap_size * sizeof(Cell));
    std::memset(ranges, 0, heap_size * 2 * sizeof(uint32_t));
    if (iters) std::memset(iters, 0, heap_size);
    if (perm)
        for (uint64_t i = 0; i < n; ++i) perm[i] = (uint32_t)i;
    Cell root = make_cell(0, (int)d, lower, upper);  // orbit.cpp:74-81
    root.cutAxis = 0;
    set_cut_margin(root);
    heap[0] = root;
    ranges[0] = 0;
    ranges[1] = (uint32_t)n;
    RankPool pool(threads);
    std::atomic<uint32_t> degen(0), unfound(0);
    const float *axes[3] = {x, y, z};
    for (uint32_t l = 1; l <= levels; ++l) {
        const int a = (1 << (l - 1)) - 1;
        const int b = std::min<int>((int)last_cells, 1 << l) - 2;
        const int n_cells = b - a + 1;
        if (n_cells <= 0) {
            st.levels_built = l;
            continue;
        }
        Cell *cells = heap + a;
        std::vector<uint32_t> jdone(n_cells, 0);
        std::atomic<int> next(0);
        // the loop of orbit.cpp:146-232 per cell (independent of the other cells), with the
        // weight sums in place of the counts
        pool.run([&](int) {
            for (int c; (c = next.fetch_add(1)) < n_cells;) {
                Cell &cell = cells[c];
                const uint32_t bg = ranges[2 * cell.id], en = ranges[2 * cell.id + 1];
                uint64_t w_cell = 0;
                for (uint32_t p = bg; p < en; ++p) w_cell += w[p];
                int j = 0;
                while (!cell.foundCut && j < 32) {
                    ++j;
                    const uint64_t wl = weight_left(axes[eff_axis(cell)], w, bg, en, get_cut(cell));
                    const int dir = convergence_weighted(wl, w_cell, en - bg, cell.nLeafCells);
                    if (dir == 0)
                        cell.foundCut = 1;
                    else if (dir > 0)
                        cell.cutMarginRight = get_cut(cell);
                    else
                        cell.cutMarginLeft = get_cut(cell);
                }
                if (iters) iters[cell.id] = (uint8_t)j;
                jdone[c] = (uint32_t)j;
                if (!cell.foundCut) ++unfound;
            }
        });
        uint32_t jmax = 0;
        for (int c = 0; c < n_cells; ++c) {
            jmax = std::max(jmax, jdone[c]);
            st.cell_counts += jdone[c];
        }
        st.iterations[l - 1] = jmax;
        for (int c = 0; c < n_cells; ++c) {  // orbit.cpp:235-250
            Cell lc, rc;
            split(cells[c], lc, rc, &st.zero_volume_cells);
            heap[lc.id] = lc;
            heap[rc.id] = rc;
        }
        next = 0;
        pool.run([&](int) {  // partition.cpp:18-62, weights moving with their particles
            for (int c; (c = next.fetch_add(1)) < n_cells;) {
                const Cell &cell = cells[c];
                const uint32_t bg = ranges[2 * cell.id], en = ranges[2 * cell.id + 1];
                int dg = 0;
                const int64_t i = hoare(x, y, z, perm, bg, en, eff_axis(cell), get_cut(cell), true,
                                        &dg, w);
                degen += (uint32_t)dg;
                const int lcid = 2 * cell.id + 1, rcid = 2 * cell.id + 2;
                ranges[2 * lcid] = bg;
                ranges[2 * lcid + 1] = (uint32_t)i;
                ranges[2 * rcid] = (uint32_t)i;
                ranges[2 * rcid + 1] = en;
            }
        });
        st.levels_built = l;
    }
    st.degenerate_cells = degen;
    st.unfound_cells = unfound;
    st.t_total_s = now_s() - t0;
    if (stats) *stats = st;
    return 0;
}

}  // extern "C"
