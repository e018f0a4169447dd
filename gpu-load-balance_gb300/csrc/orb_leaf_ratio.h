// leaf_ratio(): the split ratio of the reference's convergence test for a cell of n leaves.
// Host and device code (plain integer arithmetic), also compiled by the CPU tests against
// the reference's own double expression.
#pragma once

#include <stdint.h>

#ifndef __CUDACC__
#ifndef __host__
#define __host__
#endif
#ifndef __device__
#define __device__
#endif
#ifndef __forceinline__
#define __forceinline__ inline
#endif
#endif

namespace orb {

// The ratio of src/orbit.cpp:204, float(ceil(n/2.0) / n) for a cell of n leaves: the
// quotient rounded to double, then to float. 0.5f for an even n. For an odd n the two
// roundings are done here in integer arithmetic: the 53-bit quotient (two 64-bit divisions)
// rounds to nearest even, then its top 24 bits round to nearest even again, which is what
// the reference's double division and float conversion give.
__host__ __device__ __forceinline__ float leaf_ratio(int32_t n_leaf) {
    if (n_leaf <= 1) return 1.0f;  // ceil(1/2.0)/1 (and never a bisected cell below that)
    const uint64_t b = (uint64_t)n_leaf;
    if ((b & 1u) == 0) return 0.5f;
    const uint64_t a = (b + 1) >> 1;  // ceil(b/2); 1/2 < a/b < 1
    // m0 = floor(a 2^53 / b), r = a 2^53 mod b, in two steps (a 2^22 < 2^53, r1 2^31 < 2^62)
    const uint64_t t = a << 22;
    const uint64_t q1 = t / b, r1 = t % b;
    const uint64_t u = r1 << 31;
    const uint64_t q2 = u / b, r2 = u % b;
    uint64_t m = (q1 << 31) + q2;  // in [2^52, 2^53): a/b = m 2^-53 + r2 / (b 2^53)
    if (2 * r2 > b) ++m;           // b is odd: never a tie
    // the double m 2^-53 to float: keep 24 of its 53 bits, nearest even
    uint64_t f = m >> 29;
    const uint64_t rem = m & ((1ull << 29) - 1);
    if (rem > (1ull << 28) || (rem == (1ull << 28) && (f & 1u))) ++f;
    return (float)(uint32_t)f * 0x1p-24f;  // f <= 2^24: exact
}

}  // namespace orb
