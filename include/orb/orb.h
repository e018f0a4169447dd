/*
 * orb.h: C ABI of the GB300 ORB (orthogonal recursive bisection) engine.
 *
 * The engine builds the reference's ORB cell tree on one GPU (sm_103a): float32 particles
 * go in; the particles come back reordered so that every cell's particles are contiguous,
 * together with the cell heap (the reference's 52-byte struct Cell) and the cell-to-range
 * map. Results are bit-exact with the reference's CPU path (orbit mode o=0).
 *
 * Every call returns an orb_status and never exits the process. A context owns one CUDA
 * stream and its device buffers; calls on one context must not run concurrently from
 * several host threads (use one context per thread).
 *
 * Reference interfaces replaced (paths within andrinr/gpu-load-balance):
 *   orb_build          the master() driver of src/orbit.cpp:22-289 (particles in, heap out)
 *   orb_load_particles ServiceInit + ServiceCopyParticles (src/services/init.cu:27-144,
 *                      src/services/copyParticles.cu:10-60)
 *   orb_count          ServiceCount::Service (src/services/count.cpp:8-19)
 *   orb_count_left     ServiceCountLeft::Service (src/services/countLeft.cpp:9-42), the CPU
 *                      rule `key < cut` and the skip of cells whose cut is found; it replaces
 *                      ServiceCountLeftGPUAxis (src/services/countLeftGPUAxis.cu:188-259)
 *   orb_partition      ServicePartition::Service (src/services/partition.cpp:18-65)
 *   orb_get_ranges / orb_set_ranges   LocalData::cellToRangeMap (src/services/pst.h:6-41)
 *   orb_store_particles  the particle array the services leave partitioned in LocalData
 */
#ifndef ORB_ORB_H
#define ORB_ORB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORB_ABI_VERSION 3

typedef enum orb_status {
    ORB_OK = 0,
    ORB_ERR_INVALID_ARGUMENT = 1, /* null pointer, d = 0, levels beyond the most for d ... */
    ORB_ERR_CUDA = 2,             /* a CUDA runtime call failed; see orb_last_error */
    ORB_ERR_OUT_OF_MEMORY = 3,    /* a device or pinned allocation failed */
    ORB_ERR_CAPACITY = 4,         /* the request exceeds a limit of the engine */
    ORB_ERR_NOT_LOADED = 5,       /* a service call before orb_load_particles */
    ORB_ERR_TIMEOUT = 6           /* a bounded device wait gave up */
} orb_status;

/*
 * Byte-for-byte the reference's struct Cell (src/cell.h:9-17), 52 bytes:
 * id@0 nLeafCells@4 prevCutAxis@8 cutAxis@12 foundCut@16 cutMarginLeft@20
 * cutMarginRight@24 lower@28 upper@40. The cut of a cell is
 * (float)((double)(cutMarginRight + cutMarginLeft) / 2.0) (src/cell.h:74-76).
 */
typedef struct orb_cell {
    int32_t id;
    int32_t nLeafCells;
    int32_t prevCutAxis;
    int32_t cutAxis;
    uint8_t foundCut;
    uint8_t pad_[3];
    float cutMarginLeft;
    float cutMarginRight;
    float lower[3];
    float upper[3];
} orb_cell_t;

typedef struct orb_ctx orb_ctx;

typedef struct orb_opts {
    uint64_t reserve_particles; /* pre-size device buffers for this many particles (0 = lazy) */
    uint32_t reserve_leaves;    /* pre-size cell buffers for this many leaves (0 = lazy) */
    uint32_t flags;             /* reserved, must be 0 */
} orb_opts;

/* orb_build / orb_load_particles / orb_store_particles flags */
#define ORB_DEVICE_POINTERS 0x1u /* x,y,z (and perm) are device pointers; x,y,z are
                                    partitioned in place on the device */

typedef struct orb_build_info {
    uint32_t levels_built;
    uint32_t degenerate_cells;  /* Hoare scan clamped at the cell end: every key below the
                                   cut, including empty cells (the reference reads and
                                   swaps outside the cell there, partition.cpp:38,52) */
    uint32_t zero_volume_cells; /* setCutAxis found no positive extent (cutAxis = -1) */
    uint32_t unfound_cells;     /* bisection stopped by the 32-sweep cap (orbit.cpp:149) */
    uint32_t max_iterations;    /* most bisection iterations any cell used */
    uint32_t count_passes;      /* device passes over cell keys used by the bisection */
    float device_ms;            /* device time of the build (CUDA events on the ctx stream) */
    float h2d_ms;               /* host->device copy time (host-pointer calls) */
    float d2h_ms;               /* device->host copy time (host-pointer calls) */
    uint32_t warm_cells;        /* warm builds: cells that started from a hinted bracket */
    uint32_t warm_resets;       /* ... whose hinted bracket missed the target and restarted */
    uint32_t sampled_cells;     /* cells whose first count pass used a bracket predicted from a
                                   sample of their keys (result-invariant, see orb_tuning) */
    uint32_t sampled_misses;    /* ... whose predicted bracket did not hold the cut (that pass
                                   was repeated over every key) */
} orb_build_info;

/* Context lifetime. device = CUDA ordinal. opts may be NULL. */
orb_status orb_ctx_create(int device, const orb_opts *opts, orb_ctx **out);
orb_status orb_ctx_destroy(orb_ctx *ctx);
const char *orb_status_string(orb_status s);
/* Text of the last error on this context (empty string if none). */
const char *orb_last_error(const orb_ctx *ctx);
int orb_abi_version(void);

/*
 * Build the ORB tree of n particles into d leaf cells (1 <= d <= 2^30).
 *   x, y, z   n coordinates each, partitioned in place (reference order after the build)
 *   levels    split levels. Level l splits the heap cells [2^(l-1)-1, min(2d - 2^D, 2^l) - 2],
 *             D = ceil(log2 d) (the reference's slices, src/orbit.cpp:104-107 with
 *             src/cell.h:65-72); a cell of k leaves gives ceil(k/2) to its left child
 *             (src/cell.h:79) and its bisection tests against ratio ceil(k/2)/k
 *             (src/orbit.cpp:204).
 *             d a power of two: 0 selects log2(d) (d leaves); log2(d)-1 is the reference
 *             driver's own loop bound (src/orbit.cpp:102) and gives d/2 leaves.
 *             Other d: at most the reference's bound D-1, which 0 selects (its slices name
 *             no complete level below it; a slice that comes out empty is a level without
 *             cells, where the reference's services are called with a non-positive count).
 *   lower, upper  root box (the reference uses [-0.5,0.5]^3, src/orbit.cpp:45-46)
 *   heap      out: 2d-1 cells; cells deeper than `levels` are zeroed
 *   ranges    out: 2*(2d-1) uint32, {begin,end} per heap cell (cellToRangeMap)
 *   perm      out, optional (NULL): original index of the particle now at each position
 *   flags     ORB_DEVICE_POINTERS: x,y,z,perm are device pointers (heap/ranges stay host)
 *   info      out, optional
 * n must be below 2^31 (the reference's int indices).
 * From host arrays the copies overlap the build: x, y and z are copied in one after another
 * and each level starts once the coordinates it reads have arrived (when the box's y side is
 * at least as long as its z side), and the particles are copied back in windows while the
 * last levels are still being built. Page-locked (pinned) arrays make both copies faster. A
 * call that fails waits for its copies before it returns.
 */
orb_status orb_build(orb_ctx *ctx, float *x, float *y, float *z, uint64_t n, uint32_t d,
                     uint32_t levels, const float lower[3], const float upper[3],
                     orb_cell_t *heap, uint32_t *ranges, uint32_t *perm, uint32_t flags,
                     orb_build_info *info);

/*
 * Weighted build (no counterpart in the reference's code; its thesis specifies weighted ORB,
 * documentation/notes.tex:259-271, 326-336, and the reference never implements it). Every
 * particle carries an integer weight w[i] (work units, e.g. timesteps); the weights are
 * reordered with their particles. A cell of k leaves looks for the cut that gives its left
 * child the share ceil(k/2)/k of its weight W, with the reference's loop (midpoint cuts of
 * the bracket, at most 32 sweeps, src/orbit.cpp:146-232) and its test made exact and weighted:
 *   D = k W_left - ceil(k/2) W   (W_left: the weights of the keys below the cut)
 *   found when D == 0 or n |D| < 3 k W (n particles: |W_left - ratio W| below 3 mean weights);
 *   otherwise the right margin moves when D > 0, the left one when D < 0.
 * The sums are 64-bit integers, so the result does not depend on the order of summation. With
 * every weight 1 the test is |cl - ratio c| < 3 exactly, which is the reference's float32 test
 * wherever that test is exact (cells below 2^24 particles, an even leaf count): the tree is
 * then orb_build's. Arguments as orb_build, plus w: n weights (host, or device with
 * ORB_DEVICE_POINTERS), permuted in place. Uses the level-by-level path for every level.
 */
orb_status orb_build_weighted(orb_ctx *ctx, float *x, float *y, float *z, uint32_t *w, uint64_t n,
                              uint32_t d, uint32_t levels, const float lower[3],
                              const float upper[3], orb_cell_t *heap, uint32_t *ranges,
                              uint32_t *perm, uint32_t flags, orb_build_info *info);

/*
 * Batched build (no counterpart in the reference, which builds one tree per run): k
 * independent ORB instances of uneven sizes, packed in one set of particle arrays, built
 * together level by level (every level's kernels cover the cells of all instances).
 * Each instance's result is bit-identical to orb_build on that instance alone.
 *   x, y, z    n_total packed coordinates; instance i owns [offset_i, offset_i + n_i)
 *              (instances may not overlap); partitioned in place
 *   inst       k instance descriptors
 *   heaps      out: the instances' heaps back to back, instance i at sum_{j<i}(2 d_j - 1)
 *   ranges     out: 2 uint32 per heap cell, relative to the instance's offset
 *   perm       out, optional: per position, the original index within its instance
 *   flags      ORB_DEVICE_POINTERS for device x,y,z,perm (heaps/ranges stay host)
 */
typedef struct orb_batch_instance {
    uint64_t offset;
    uint64_t n;
    uint32_t d;      /* leaf cells, 1 .. 2^30 */
    uint32_t levels; /* 0 = the most for d (as orb_build) */
    float lower[3];
    float upper[3];
} orb_batch_instance;

orb_status orb_build_batch(orb_ctx *ctx, float *x, float *y, float *z, uint64_t n_total,
                           const orb_batch_instance *inst, uint32_t k, orb_cell_t *heaps,
                           uint32_t *ranges, uint32_t *perm, uint32_t flags,
                           orb_build_info *info);

/*
 * Warm-started builds (no counterpart in the reference; the thesis's improved root finding,
 * notes.tex:2565, and the unused FAST_MEDIAN branch, src/orbit.cpp:214-227, point at it).
 * For rebuilding a tree after small particle moves: each cell's bisection starts from the
 * previous tree's cut of the same cell +- width x that cell's extent / sqrt(n) (n = the new
 * cell's particles: about width x sqrt(n) keys on each side when evenly spread, the scale by
 * which a median drifts under small independent moves), clipped to the new cell, when the
 * cut axis is unchanged, instead of the cell's whole extent. The bracket is
 * checked on the first count; one that does not hold the target restarts from the extent.
 * Every cut still passes the reference's convergence test (or the 32-sweep cap), but the
 * midpoint sequence differs from a cold build, so the tree is NOT bit-identical with
 * orb_build on the same particles: a separate, labelled mode.
 *   prev_heaps: the previous trees, laid out like heaps (instance i at sum_{j<i}(2 d_j - 1));
 *   widths[i]:  instance i's bracket factor (above; 8 is a good start), 0 = cold build.
 */
orb_status orb_build_batch_warm(orb_ctx *ctx, float *x, float *y, float *z, uint64_t n_total,
                                const orb_batch_instance *inst, uint32_t k,
                                const orb_cell_t *prev_heaps, const float *widths,
                                orb_cell_t *heaps, uint32_t *ranges, uint32_t *perm,
                                uint32_t flags, orb_build_info *info);
orb_status orb_build_warm(orb_ctx *ctx, float *x, float *y, float *z, uint64_t n, uint32_t d,
                          uint32_t levels, const float lower[3], const float upper[3],
                          const orb_cell_t *prev_heap, float width, orb_cell_t *heap_out,
                          uint32_t *ranges_out, uint32_t *perm, uint32_t flags,
                          orb_build_info *info);

/*
 * Launch tuning of a context (no counterpart in the reference). Every parameter changes
 * only how the work is spread over the GPU, never a result: trees, ranges and particle
 * order are the same under any valid setting.
 */
typedef struct orb_tuning {
    uint32_t hist_blocks_per_sm;   /* count-left pass: CTAs per SM, 1..8 (default 8) */
    uint32_t part_blocks_per_sm;   /* partition passes: CTAs per SM, 1..16 (default 8) */
    uint32_t tile_blocks_per_sm;   /* one-tile cell bisection: CTAs per SM, 1..8 (default 4) */
    uint32_t sparse_keys_per_tile; /* compaction threshold: a count pass sends a cell's bracket
                                      keys straight to its global bins (instead of binning all
                                      keys in shared memory) once the bracket holds at most
                                      this many keys per tile, 1..16384 (default 64) */
    uint32_t cta_min_cells;        /* levels with at least this many cells bisect one cell per
                                      CTA; 0 = never (default) */
    uint32_t subtree_levels;       /* the last levels (at most this many, 0..6, default 4) are
                                      finished by one CTA per cell once every cell of a level
                                      fits one (at most 34816 particles); 0 = never */
    uint32_t predict_sigmas;       /* first count pass of cells of at least 2^18 particles: the
                                      keys are binned only inside a bracket predicted from a
                                      strided sample (its median +- this many standard errors),
                                      checked exactly, repeated over every key when it misses;
                                      0..16, 0 = never (default 0: slower on the measured
                                      workloads; the autotuner tries it) */
} orb_tuning;

orb_status orb_get_tuning(orb_ctx *ctx, orb_tuning *out);
orb_status orb_set_tuning(orb_ctx *ctx, const orb_tuning *t); /* ORB_ERR_INVALID_ARGUMENT
                                                                 outside the ranges above */

/*
 * Autotuner: times batched builds of the given instances (x,y,z host or, with
 * ORB_DEVICE_POINTERS, device arrays; they are copied, never modified) under candidate
 * settings, one parameter at a time (coordinate descent from the current setting), `reps`
 * builds per candidate (median device time), and checks that every candidate builds the
 * same trees. The fastest setting becomes the context's; it is returned in *best with its
 * median build time in *best_ms.
 */
orb_status orb_autotune_batch(orb_ctx *ctx, const float *x, const float *y, const float *z,
                              uint64_t n_total, const orb_batch_instance *inst, uint32_t k,
                              uint32_t flags, uint32_t reps, orb_tuning *best, float *best_ms);

/*
 * Request server with continuous batching (no counterpart in the reference, which builds
 * one tree per run). Instances stay resident on the GPU: their particles live in a device
 * arena sized from hbm_budget_bytes; builds are admitted when their particles fit in the
 * arena (otherwise they wait until orb_server_release frees memory), rebalances when their
 * instance is idle. Each of `lanes` worker threads (own stream) takes every admissible
 * pending request, up to max_batch (0 = no limit), into one batched build, so requests that
 * arrive while others run are picked up by the next free lane and batches overlap on the
 * device. Each instance's requests are applied in submission order; results are
 * bit-identical to running the same requests one at a time.
 */
typedef struct orb_server orb_server;

typedef struct orb_server_opts {
    uint64_t hbm_budget_bytes; /* device memory for the arena and the lanes' scratch */
    uint32_t max_batch;        /* most requests per batched build (0 = no limit) */
    uint32_t lanes;            /* concurrent batches (0 = 2) */
} orb_server_opts;

typedef struct orb_request_result {
    uint64_t request_id;
    uint64_t instance_id; /* the id of the build request that created the instance */
    int32_t status;       /* orb_status of the request */
    int32_t kind;         /* 0 build, 1 rebalance */
    uint32_t batch_size;  /* requests in the batched build that served it */
    uint32_t pad_;
    double submit_s, start_s, done_s; /* steady-clock seconds */
} orb_request_result;

typedef struct orb_server_stats {
    uint64_t requests_submitted, requests_done, builds, rebalances, batches;
    uint64_t particles_built, arena_particles, arena_used;
    uint32_t max_batch_seen, pending;
} orb_server_stats;

orb_status orb_server_create(int device, const orb_server_opts *opts, orb_server **out);
/* Stops the lanes (pending requests are dropped) and frees the device memory. */
orb_status orb_server_destroy(orb_server *sv);
/* New instance from host particles (copied at submission); instance id = *request_id. */
orb_status orb_server_submit_build(orb_server *sv, const float *x, const float *y, const float *z,
                                   uint64_t n, uint32_t d, uint32_t levels, const float lower[3],
                                   const float upper[3], uint64_t *request_id);
/* New instance from the seeded generator (orb_generate kinds), box [-0.5,0.5)^3. */
orb_status orb_server_submit_generate(orb_server *sv, int kind, uint64_t seed, uint64_t n,
                                      uint32_t d, uint32_t levels, uint64_t *request_id);
/* Rebalance a resident instance: every coordinate += sigma * N(0,1) (seeded), clamped to the
   instance's box, then the tree is rebuilt with the reference's rule. */
orb_status orb_server_submit_rebalance(orb_server *sv, uint64_t instance_id, uint64_t seed,
                                       float sigma, uint64_t *request_id);
/* Warm rebalance: as above, but the rebuild starts every cell from the instance's previous
 * cut (orb_build_batch_warm with this width factor); not bit-identical with a cold rebuild.
 * width > 0. */
orb_status orb_server_submit_rebalance_warm(orb_server *sv, uint64_t instance_id, uint64_t seed,
                                            float sigma, float width, uint64_t *request_id);
/* Blocks until the request finishes; returns its status. */
orb_status orb_server_wait(orb_server *sv, uint64_t request_id, orb_request_result *out);
/* Finished requests not yet polled (up to max). */
orb_status orb_server_poll(orb_server *sv, orb_request_result *out, uint32_t max, uint32_t *n_out);
/* Latest tree and particles of an instance (host buffers, each may be NULL): heap 2d-1 cells,
   ranges 2(2d-1), x,y,z and the original index of the particle at each position (n). */
orb_status orb_server_fetch(orb_server *sv, uint64_t instance_id, orb_cell_t *heap, uint32_t *ranges,
                            float *x, float *y, float *z, uint32_t *ident);
/* Frees the instance's arena slot after its pending requests finish. */
orb_status orb_server_release(orb_server *sv, uint64_t instance_id);
orb_status orb_server_get_stats(orb_server *sv, orb_server_stats *out);

/*
 * Service layer: the reference's per-rank services over particles resident in the context.
 * orb_load_particles copies n particles in (host or device per flags), sets the range map
 * to root = [0, n) and sizes it for cell ids below max_cells.
 */
orb_status orb_load_particles(orb_ctx *ctx, const float *x, const float *y, const float *z,
                              uint64_t n, uint32_t max_cells, uint32_t flags);
/* Copies the resident (partitioned) particles out; perm optional. */
orb_status orb_store_particles(orb_ctx *ctx, float *x, float *y, float *z, uint32_t *perm,
                               uint32_t flags);
/* out[i] = end - begin of cells[i] (host arrays). */
orb_status orb_count(orb_ctx *ctx, const orb_cell_t *cells, uint32_t n_cells, uint32_t *out);
/* out[i] = #{p in cell i : key[p] < getCut(cell i)} on cutAxis; found cells are skipped
   (out[i] left untouched), as src/services/countLeft.cpp:19-21. */
orb_status orb_count_left(orb_ctx *ctx, const orb_cell_t *cells, uint32_t n_cells,
                          uint32_t *out);
/* Hoare-partition every cell at getCut() on cutAxis and set the children's ranges
   (ids 2*id+1, 2*id+2), as src/services/partition.cpp:18-65. */
orb_status orb_partition(orb_ctx *ctx, const orb_cell_t *cells, uint32_t n_cells);
/* Range map access: 2*n_cells uint32 for cell ids [0, n_cells). */
orb_status orb_get_ranges(orb_ctx *ctx, uint32_t *ranges, uint32_t n_cells);
orb_status orb_set_ranges(orb_ctx *ctx, const uint32_t *ranges, uint32_t n_cells);

/*
 * Seeded synthetic particles: the engine's counter-based generators (every size and seed
 * reproducible) and the reference's own input stream.
 *   kind ORB_GEN_UNIFORM: i.i.d. on the 2^-24 grid of [-0.5,0.5)^3
 *   kind ORB_GEN_PLUMMER: 90% from 64 Plummer spheres (scale radii log-uniform in
 *                         [0.005,0.05)), 10% uniform background, clipped to the box
 *   kind ORB_GEN_XORSHF96: the reference's xorshf96 (ServiceInit, src/services/init.cu:11-25,
 *                         48-52): from its process-start seeds, x_0, y_0, z_0, x_1, ... each
 *                         (float)z / ULONG_MAX - 0.5 in [-0.5, 0.5]; `seed` = draws of the
 *                         stream to skip first (0: the input of a single-rank `orbit N d 0`).
 *                         Generated on the device by jumps of the generator's linear map.
 * Writes n floats to each of x,y,z (device pointers if ORB_DEVICE_POINTERS, else host).
 */
#define ORB_GEN_UNIFORM 0
#define ORB_GEN_PLUMMER 1
#define ORB_GEN_XORSHF96 2
orb_status orb_generate(orb_ctx *ctx, int kind, uint64_t seed, uint64_t n, float *x, float *y,
                        float *z, uint32_t flags);

/*
 * Per-kernel profile of a context (no reference counterpart; the reference prints phase
 * wall-clock timers, src/orbit.cpp:284-286). Launch counts are always kept. Launches of the
 * kernel kinds selected by timing_mask (bit orb_profile_kernel_index(name); 0xffffffff =
 * all) are bracketed by CUDA events on the context stream and their durations summed.
 * `bytes` is the algorithmic traffic those launches moved (keys read, masks written,
 * particles swapped), counted on the device.
 */
typedef struct orb_kernel_stat {
    char name[32];
    uint64_t launches;
    double total_ms;
    double bytes;
} orb_kernel_stat;
orb_status orb_profile_reset(orb_ctx *ctx, uint32_t timing_mask);
/* Index of a kernel kind by the name orb_profile_read reports, or -1. */
int orb_profile_kernel_index(const char *name);
/* Writes up to max_entries stats (kernels launched at least once); returns how many exist. */
int orb_profile_read(orb_ctx *ctx, orb_kernel_stat *out, int max_entries);

/*
 * Count-left that allocates nothing. It has no counterpart in the reference; it is the
 * service count-left (same `key < getCut()` rule on cutAxis, found cells left untouched)
 * for callers that must not allocate device memory while they run. Examples are a
 * simulation code that has reserved the whole device in its own memory pool, where
 * cudaMalloc would fail or fragment that pool, or one that cannot take the device-wide
 * synchronisation cudaMalloc/cudaFree imply while its other streams are busy.
 *   x, y, z   n device coordinates;  cells: n_cells device orb_cell_t
 *   ranges    device range map, 2 uint32 {begin,end} per cell id, n_ranges ids; a cell
 *             whose id or range lies outside the map or [0,n] counts as empty
 *   out       device uint32[n_cells]
 *   stream    cudaStream_t to run on (NULL = default stream); the call only enqueues work
 * Scratch is one static device array of ORB_STATIC_MAX_CELLS cells (512 KiB per GPU,
 * held until the process exits); n_cells above that returns ORB_ERR_CAPACITY. The call
 * uses the calling thread's current device. Its first call on a device resolves the
 * array's address (cudaGetSymbolAddress); make that first call before any stream capture.
 * That address is kept until the process exits: do not call it on a device after a
 * cudaDeviceReset of that device.
 * Every call shares the one array (the kernels clear it first), so calls that overlap on
 * the GPU, on different streams or threads, race and must be serialised by the caller.
 */
#define ORB_STATIC_MAX_CELLS 65536
orb_status orb_count_left_static(const float *x, const float *y, const float *z, uint64_t n,
                                 const orb_cell_t *cells, uint32_t n_cells,
                                 const uint32_t *ranges, uint32_t n_ranges, uint32_t *out,
                                 void *stream);

/*
 * Test hook of the bounded device waits (no counterpart in the reference, whose errors end
 * the process, src/constants.h:19-23). The partition's tile scan chains its blocks with a
 * decoupled look-back; each wait polls a predecessor's status at most spin_limit times
 * (0 = the default, about 2^22 polls), then flags the build and gives up: the kernels that
 * would read the scan's prefixes do nothing and the build returns ORB_ERR_TIMEOUT. The
 * context stays usable. ticket_start (0..255, normally 0) is the value the scan's block
 * ticket starts from: 1 means no block takes the first status slot, so its successor's
 * wait runs out, a wait that can never end made into one that ends in a bounded time.
 * Settings stay until changed; (0, 0) restores the defaults.
 */
orb_status orb_test_set_scan_wait(orb_ctx *ctx, uint32_t spin_limit, uint32_t ticket_start);

#ifdef __cplusplus
}
#endif

#endif /* ORB_ORB_H */
