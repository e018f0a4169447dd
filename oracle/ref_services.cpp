// Test infrastructure: whole ORB builds computed by the reference's own CPU services.
//
// src/services/count.cpp, countLeft.cpp, makeAxis.cpp and partition.cpp of
// andrinr/gpu-load-balance and its src/cell.h are compiled unchanged from the reference's
// source tree (`make -C oracle ref`), against three shim headers of this repository
// (oracle/refshim: the Blitz++ Array subset, the MDL declarations and the CUDA type names
// the headers mention). This driver sequences them the way the reference's master()
// sequences its MDL services for orbit mode o=0 (src/orbit.cpp:74-250): per level the cut
// axis gather (makeAxis), the cell sizes (count + Combine), the bisection loop (countLeft +
// Combine on every rank, the float32 test of src/orbit.cpp:204-230 on the summed counts,
// at most 32 sweeps), the split with the reference's Cell::cut(), setCutAxis() and
// setCutMargin(), and the Hoare partition on every rank. With nranks > 1 each rank owns a
// slab of the particles and its own LocalData, as under MDL, and the counts are summed by
// the services' own Combine().
//
// The reference's Hoare scan reads and swaps outside a cell whose keys all lie below the
// cut (src/services/partition.cpp:38,52); each rank's particle columns carry guard elements
// so those reads stay inside this driver's memory, but such builds are not comparable and
// the tests use inputs without such cells. Nothing outside the tests loads this library.
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>
#include <tuple>
#include <vector>

#include "cell.h"
#include "count.h"
#include "countLeft.h"
#include "makeAxis.h"
#include "partition.h"

static_assert(sizeof(Cell) == 52, "the reference's Cell is the 52-byte heap record");

// MDL's traversal (src/services/TraversePST.cpp) walks the PST tree and calls Service() on
// each leaf; here refsvc_build below calls every rank's Service() and Combine() itself, so the
// traversal entry points only forward to the leaf.
int TraversePST::operator()(int nIn, void *pIn, void *pOut) {
    return Traverse(node_pst, pIn, nIn, pOut, getMaxBytesOut());
}
int TraversePST::Traverse(PST pst, void *vin, int nIn, void *vout, int nOut) {
    return Service(pst, vin, nIn, vout, nOut);
}
int TraversePST::Traverse(unsigned, PST, void *, int, void *, int) { return 0; }
int TraversePST::Recurse(PST pst, void *vin, int nIn, void *vout, int nOut) {
    return Service(pst, vin, nIn, vout, nOut);
}
int TraverseCombinePST::Recurse(PST pst, void *vin, int nIn, void *vout, int nOut) {
    return Service(pst, vin, nIn, vout, nOut);
}

namespace {

// The services keep Service()/Combine() protected; these derived callers expose them.
template <class S>
struct Call : S {
    explicit Call(PST p) : S(p) {}
    int service(PST p, void *in, int nIn, void *out, int nOut) { return this->Service(p, in, nIn, out, nOut); }
    int combine(void *a, void *b, int nIn, int n1, int n2) { return this->Combine(a, b, nIn, n1, n2); }
};

struct Rank {
    uint64_t off = 0, n = 0;
    std::vector<float> cols;   // 3 columns of n + 2 floats: a guard, the slab, a guard
    std::vector<float> axis;   // particlesT with a guard on each side
    std::vector<unsigned int> rng;  // cellToRangeMap, heap_cells x 2
    LocalData lcl;
    std::unique_ptr<pstNode> node;
};

}  // namespace

extern "C" {

int refsvc_cell_size(void) { return (int)sizeof(Cell); }

// Whole build of d leaves over `levels` levels (the oracle's level slices, src/orbit.cpp:
// 104-107) on nranks slabs (the oracle's slab split: n/nranks each, the remainder on the
// last rank). x, y, z are partitioned in place slab by slab; heap gets 2d-1 cells (pad bytes
// zeroed), ranges nranks consecutive maps of 2(2d-1) uint32. Returns 0, or -1 on arguments
// the reference's driver does not take.
int refsvc_build(float *x, float *y, float *z, uint64_t n, uint32_t d, uint32_t levels,
                 const float lower[3], const float upper[3], void *heap_out, uint32_t *ranges_out,
                 int nranks) {
    if (!x || !y || !z || !heap_out || !ranges_out || d == 0 || nranks < 1) return -1;
    if ((uint64_t)nranks > (n ? n : 1)) nranks = (int)(n ? n : 1);
    const int heap_cells = (int)(2 * d - 1);
    std::vector<Cell> heap(heap_cells);
    std::memset(heap.data(), 0, heap.size() * sizeof(Cell));

    float lo[3] = {lower[0], lower[1], lower[2]}, hi[3] = {upper[0], upper[1], upper[2]};
    Cell root(0, (int)d, lo, hi);  // src/orbit.cpp:74-76
    root.cutAxis = 0;
    root.setCutMargin();
    heap[0] = root;

    const float guard = std::numeric_limits<float>::quiet_NaN();
    std::vector<Rank> rk(nranks);
    for (int r = 0; r < nranks; ++r) {
        Rank &R = rk[r];
        R.off = (n / nranks) * r;
        R.n = (r == nranks - 1) ? n - R.off : n / nranks;
        const uint64_t ld = R.n + 2;
        R.cols.assign(3 * ld + 2, guard);
        const float *src[3] = {x, y, z};
        for (int a = 0; a < 3; ++a)
            std::memcpy(R.cols.data() + a * ld + 1, src[a] + R.off, R.n * sizeof(float));
        R.axis.assign(R.n + 4, guard);
        R.rng.assign(2 * (size_t)heap_cells, 0u);
        R.rng[1] = (unsigned int)R.n;
        // column-major (position, axis) over the slab, as init.cu sets lcl->particles up
        R.lcl.particles = blitz::Array<float, 2>(R.cols.data() + 1, (int)R.n, 3, 1, (std::ptrdiff_t)ld);
        R.lcl.particlesT = blitz::Array<float, 1>(R.axis.data() + 1, (int)R.n + 2);
        R.lcl.cellToRangeMap = blitz::Array<unsigned int, 2>(R.rng.data(), heap_cells, 2, 2, 1);
        R.node.reset(new pstNode(nullptr));
        R.node->lcl = &R.lcl;
    }
    Call<ServiceMakeAxis> make_axis(nullptr);
    Call<ServiceCount> count(nullptr);
    Call<ServiceCountLeft> count_left(nullptr);
    Call<ServicePartition> partition(nullptr);

    const int depth = root.getNLevels(), last = root.getNCellsOnLastLevel();
    for (uint32_t l = 1; l <= levels; ++l) {
        const int a = (int)std::pow(2, (l - 1)) - 1;  // src/orbit.cpp:104-107
        const int b = std::min(last, (int)std::pow(2, l)) - 2;
        const int n_cells = b - a + 1;
        if (n_cells <= 0 || b >= heap_cells) continue;
        (void)depth;
        Cell *cells = heap.data() + a;
        const int n_in = n_cells * (int)sizeof(Cell);
        std::vector<unsigned int> o_counts(n_cells), o_left(n_cells), tmp(n_cells);
        int dummy = 0;
        for (int r = 0; r < nranks; ++r)  // PST_MAKEAXIS
            make_axis.service(rk[r].node.get(), cells, n_in, &dummy, sizeof dummy);
        for (int r = 0; r < nranks; ++r) {  // PST_COUNT on every rank, then Combine
            unsigned int *dst = r == 0 ? o_counts.data() : tmp.data();
            count.service(rk[r].node.get(), cells, n_in, dst, n_cells * (int)sizeof(unsigned int));
            if (r) count.combine(o_counts.data(), tmp.data(), n_in, n_cells * 4, n_cells * 4);
        }
        bool found_all = false;  // src/orbit.cpp:146-232
        int j = 0;
        while (!found_all && j < 32) {
            j++;
            found_all = true;
            for (int r = 0; r < nranks; ++r) {  // PST_COUNTLEFT on every rank, then Combine
                unsigned int *dst = r == 0 ? o_left.data() : tmp.data();
                if (r) std::memset(tmp.data(), 0, tmp.size() * sizeof(unsigned int));
                count_left.service(rk[r].node.get(), cells, n_in, dst, n_cells * (int)sizeof(unsigned int));
                if (r) count_left.combine(o_left.data(), tmp.data(), n_in, n_cells * 4, n_cells * 4);
            }
            for (int i = 0; i < n_cells; ++i) {
                if (cells[i].foundCut) continue;
                float ratio = ceil(cells[i].nLeafCells / 2.0) / cells[i].nLeafCells;
                int difference = o_left[i] - o_counts[i] * ratio;
                if (abs(difference) < 3) {
                    cells[i].foundCut = true;
                } else if (difference > 0) {
                    cells[i].cutMarginRight = cells[i].getCut();
                    found_all = false;
                } else {
                    cells[i].cutMarginLeft = cells[i].getCut();
                    found_all = false;
                }
            }
        }
        for (int i = 0; i < n_cells; ++i) {  // src/orbit.cpp:235-250
            Cell cellLeft, cellRight;
            std::tie(cellLeft, cellRight) = cells[i].cut();
            cellRight.setCutAxis();
            cellRight.setCutMargin();
            cellLeft.setCutAxis();
            cellLeft.setCutMargin();
            heap[cells[i].getLeftChildId()] = cellLeft;
            heap[cells[i].getRightChildId()] = cellRight;
        }
        for (int r = 0; r < nranks; ++r)  // PST_PARTITION on every rank
            partition.service(rk[r].node.get(), cells, n_in, &dummy, sizeof dummy);
    }

    // outputs: the heap (pad bytes zeroed: the reference's Cell leaves them unset), every
    // rank's range map and its partitioned slab
    unsigned char *hout = static_cast<unsigned char *>(heap_out);
    for (int c = 0; c < heap_cells; ++c) {
        std::memcpy(hout + 52 * (size_t)c, &heap[c], 52);
        std::memset(hout + 52 * (size_t)c + 17, 0, 3);
    }
    for (int r = 0; r < nranks; ++r) {
        Rank &R = rk[r];
        const uint64_t ld = R.n + 2;
        float *dst[3] = {x, y, z};
        for (int a = 0; a < 3; ++a)
            std::memcpy(dst[a] + R.off, R.cols.data() + a * ld + 1, R.n * sizeof(float));
        std::memcpy(ranges_out + (size_t)r * 2 * heap_cells, R.rng.data(), R.rng.size() * sizeof(unsigned int));
    }
    return 0;
}

}  // extern "C"
