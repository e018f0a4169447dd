/*
 * ORB oracle: a CPU restatement of the reference's CPU-only path (orbit mode o=0).
 *
 * TEST INFRASTRUCTURE ONLY. Nothing in the product library links, loads or calls this
 * code; the tests, the smoke check and the benchmark's CPU-baseline leg use it as the
 * checker and as the timed CPU baseline.
 *
 * Reference files followed (paths within andrinr/gpu-load-balance):
 *   src/cell.h:9-126                 Cell layout, getCut, cut(), setCutAxis, setCutMargin
 *   src/orbit.cpp:74-81              root cell (cutAxis forced to 0) and cell heap
 *   src/orbit.cpp:102-111            level slices of the heap
 *   src/orbit.cpp:146-232            bisection loop, float32 convergence test, 32-iteration cap
 *   src/orbit.cpp:235-250            split of every cell of the level
 *   src/services/count.cpp:14-17     cell sizes from the range map
 *   src/services/makeAxis.cpp:16-30  gather of the cut-axis coordinate (timed baseline only)
 *   src/services/countLeft.cpp:16-39 count of keys strictly below the cut, found cells skipped
 *   src/services/partition.cpp:24-62 Hoare partition with the final swap(i, end-1)
 *   src/services/countLeft.cpp:44-53 rank combine = elementwise sum (multi-rank mode)
 *
 * Where the reference reads or writes outside a cell (Hoare scan running off the cell end
 * when every key is below the cut, including empty cells; src/services/partition.cpp:38,52)
 * the oracle clamps the scan at the cell end, skips the final swap and counts the cell in
 * `degenerate_cells`. Where setCutAxis finds no positive extent (cutAxis = -1,
 * src/cell.h:102-121) the oracle stores -1 in the heap, uses axis 0 for that cell's
 * count and partition with margins (lower[0], upper[0]), and counts it in
 * `zero_volume_cells`. The GPU engine implements the same rules.
 */
#ifndef ORB_ORACLE_H
#define ORB_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Byte-for-byte the reference's struct Cell (src/cell.h:9-17): 52 bytes. */
typedef struct oracle_cell {
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
} oracle_cell_t;

#define ORACLE_MAX_LEVELS 40

typedef struct oracle_stats {
    uint32_t levels_built;
    uint32_t iterations[ORACLE_MAX_LEVELS]; /* bisection sweeps (j) per level */
    uint64_t cell_counts;                   /* count-left evaluations (cell x iteration) */
    uint64_t elements_counted;              /* keys read by count-left over the build */
    uint32_t degenerate_cells;              /* Hoare scan clamped at the cell end */
    uint32_t zero_volume_cells;             /* setCutAxis found no positive extent */
    uint32_t unfound_cells;                 /* bisection stopped by the 32-sweep cap */
    uint32_t nranks;
    double t_make_axis_s;
    double t_count_s;
    double t_partition_s;
    double t_total_s;
    uint64_t elements_per_level[ORACLE_MAX_LEVELS]; /* elements_counted by level */
} oracle_stats_t;

/* Seeded generators shared bit-for-bit with the engine's device generator. */
uint64_t oracle_draw(uint64_t seed, uint64_t counter);
void oracle_gen_uniform(uint64_t seed, uint64_t n, float *x, float *y, float *z, int nthreads);
void oracle_plummer_clusters(uint64_t seed, float *centres /*64*3*/, double *scales /*64*/);
void oracle_gen_plummer(uint64_t seed, uint64_t n, float *x, float *y, float *z, int nthreads);

/* The reference's own generator (src/services/init.cu:11-25), the stream a single-rank
 * `orbit N d 0` builds from: x_0, y_0, z_0, x_1, ... from the process-start seeds. */
void oracle_gen_xorshf96(uint64_t n, float *x, float *y, float *z);

/* Reference arithmetic primitives. */
float oracle_get_cut(float margin_left, float margin_right);
/* Returns 0 = found, +1 = move the right margin to the cut, -1 = move the left margin. */
int oracle_convergence(uint32_t count_left, uint32_t count, int32_t n_leaf_cells,
                       int32_t *difference_out);
uint32_t oracle_count_left(const float *keys, uint64_t begin, uint64_t end, float cut);
/* Hoare partition of [begin,end) of x,y,z (and perm if non-null) on `axis` at `cut`.
 * Returns the split index i; *degenerate set to 1 when the scan was clamped. */
int64_t oracle_hoare(float *x, float *y, float *z, uint32_t *perm, uint64_t begin,
                     uint64_t end, int axis, float cut, int final_swap, int *degenerate);

/*
 * Full ORB build, in place on x,y,z (the particle order after the build is the
 * reference's partitioned order).
 *   d        leaf cells (1 .. 2^30); heap holds 2d-1 cells, ranges 2*(2d-1) uint32
 *   levels   split levels to run, at most oracle_max_levels(d). Level l takes the heap cells
 *            [2^(l-1)-1, min(getNCellsOnLastLevel(), 2^l) - 2] (src/orbit.cpp:104-107); for
 *            a power of two that is every cell of the level, log2(d) levels give d leaves
 *            and log2(d)-1 is the reference's own loop bound (src/orbit.cpp:102). For any
 *            other d the reference's bound getNLevels()-1 is the most; a slice that comes out
 *            empty (b < a) is a level without cells.
 *   perm     optional: original index of the particle at each position
 *   iters    optional: bisection iterations spent on each heap cell
 *   nranks   1 = canonical single-rank oracle. >1 = the reference's MDL semantics: the
 *            particles are split into nranks contiguous slabs, per-cell counts are summed
 *            over ranks and each rank partitions its own slab (run on nranks threads).
 *            `ranges` then holds nranks consecutive range maps.
 *   make_axis  1 = also perform the per-level cut-axis gather the reference performs
 *            (src/services/makeAxis.cpp); results are identical, only timing changes.
 *   threads  single-rank mode only: the cells of a level are bisected and partitioned on
 *            this many threads (each cell runs its own loop of src/orbit.cpp:146-232, which
 *            depends on that cell alone), and a level of fewer cells splits each count over
 *            the threads. Results and statistics are those of threads = 1.
 * Returns 0 on success, a negative value on invalid arguments.
 */
int oracle_build(float *x, float *y, float *z, uint64_t n, uint32_t d, uint32_t levels,
                 const float lower[3], const float upper[3], oracle_cell_t *heap,
                 uint32_t *ranges, uint32_t *perm, uint8_t *iters, int nranks,
                 int make_axis, int threads, oracle_stats_t *stats);

/*
 * Weighted ORB (documentation/notes.tex:259-271, 326-336; the reference never implemented
 * it): each particle carries an integer weight w[i] (work units), permuted with it. A cell's
 * bisection looks for the cut that gives its left child the share ceil(k/2)/k of the cell's
 * weight W (k leaves), with the reference's loop (src/orbit.cpp:146-232: midpoint cuts, at
 * most 32 sweeps) and its test made exact and weighted (oracle_convergence_weighted):
 *   D = k W_left - ceil(k/2) W; found when D == 0 or n |D| < 3 k W (n particles); the right
 *   margin moves for D > 0, the left one for D < 0.
 * W_left is the integer sum of the weights of the keys below the cut. With unit weights the
 * test is |cl - c ratio| < 3 exactly, the reference's float32 test wherever that is exact
 * (cells below 2^24 particles, even k): the tree is then the unweighted one.
 * Single rank; threads as in oracle_build. Same outputs as oracle_build, w permuted too.
 */
int oracle_convergence_weighted(uint64_t w_left, uint64_t w_cell, uint64_t n, int32_t n_leaf);
int oracle_build_weighted(float *x, float *y, float *z, uint32_t *w, uint64_t n, uint32_t d,
                          uint32_t levels, const float lower[3], const float upper[3],
                          oracle_cell_t *heap, uint32_t *ranges, uint32_t *perm, uint8_t *iters,
                          int threads, oracle_stats_t *stats);

/* Cell::getNLevels() (depth = ceil(log2 d)) and getNCellsOnLastLevel() (2d - 2^depth) of
 * src/cell.h:65-72. */
void oracle_level_shape(uint32_t d, uint32_t *depth, uint32_t *last);
/* Most split levels of a build of d leaves: log2(d) for a power of two, else the
 * reference's bound getNLevels() - 1. */
uint32_t oracle_max_levels(uint32_t d);

#ifdef __cplusplus
}
#endif

#endif
