// Test infrastructure: the reference's own Cell arithmetic (src/cell.h of
// andrinr/gpu-load-balance, compiled unchanged from the reference's source tree by
// `make ref`), behind a C ABI for the oracle's tests. It computes a bracket's cut and a
// cell's split exactly as the reference's driver does (src/orbit.cpp:74-76 for the root,
// src/orbit.cpp:235-243 for the split), so the oracle's restatement of those steps can be
// compared with the reference's code itself. Nothing outside the tests loads it.
#include <cstring>
#include <tuple>

#include "cell.h"

static_assert(sizeof(Cell) == 52, "the reference's Cell is the 52-byte heap record");

extern "C" {

int ref_cell_size(void) { return (int)sizeof(Cell); }

// Cell::getCut() (src/cell.h:74-76) of the bracket [left, right].
float ref_get_cut(float left, float right) {
    float z[3] = {0.f, 0.f, 0.f};
    Cell c(0, 2, z, z);
    c.cutMarginLeft = left;
    c.cutMarginRight = right;
    return c.getCut();
}

// The root as the reference's driver sets it up: Cell(0, d, lower, upper), cutAxis = 0,
// setCutMargin() (src/orbit.cpp:74-76).
void ref_root(int d, const float *lower, const float *upper, void *out52) {
    float lo[3] = {lower[0], lower[1], lower[2]}, hi[3] = {upper[0], upper[1], upper[2]};
    Cell root(0, d, lo, hi);
    root.cutAxis = 0;
    root.setCutMargin();
    std::memcpy(out52, &root, sizeof root);
}

// The split of the parent cell (its final margins and cut axis) as src/orbit.cpp:235-243
// does it: cut(), then the right child's and the left child's setCutAxis() and
// setCutMargin(). A child whose box has no positive extent gets cutAxis -1, for which the
// reference's setCutMargin() reads outside the box: it is not called then (returns 1).
int ref_split(const void *parent52, void *left52, void *right52) {
    Cell p;
    std::memcpy(&p, parent52, sizeof p);
    Cell l, r;
    std::tie(l, r) = p.cut();
    int undefined = 0;
    r.setCutAxis();
    if (r.cutAxis >= 0) r.setCutMargin(); else undefined = 1;
    l.setCutAxis();
    if (l.cutAxis >= 0) l.setCutMargin(); else undefined = 1;
    std::memcpy(left52, &l, sizeof l);
    std::memcpy(right52, &r, sizeof r);
    return undefined;
}

// Cell::getNLevels() and getNCellsOnLastLevel() (src/cell.h:65-72) for nLeafCells = d.
void ref_levels(int d, int *n_levels, int *n_cells_last) {
    float z[3] = {0.f, 0.f, 0.f};
    Cell c(0, d, z, z);
    *n_levels = c.getNLevels();
    *n_cells_last = c.getNCellsOnLastLevel();
}

}  // extern "C"
