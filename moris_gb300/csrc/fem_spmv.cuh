// fem_spmv.cuh -- CSR row products with a few lanes per row.
//
// The element operators give about 81 nonzeros per row (27 nodes x 3
// components for linear B-splines).  On GB300 the FP64 pipe, not HBM, bounds
// a CSR product, so the kernel should issue little besides the FMAs: with a
// whole warp per row the 5-step shuffle reduction and the idle lanes of the
// last pass cost about twice the useful FMAs; with kLanesPerRow = 4 lanes per
// row (8 rows per warp) a row takes 21 FMA passes and a 2-step reduction, and
// every load still fills whole 32-byte sectors.
#pragma once

#include <cstdint>

namespace fem {

constexpr int kLanesPerRow = 4;

// sum_k v[k] x[ci[k]] over CSR row `row` (row < n), reduced over the
// kLanesPerRow lanes of a group; every lane of the warp must call it
// (rows >= n contribute zero).  sub = lane index within the group.
__device__ __forceinline__ double csr_row_dot(int64_t n, const int32_t* __restrict__ rp,
                                              const int32_t* __restrict__ ci, const double* __restrict__ v,
                                              const double* __restrict__ x, int64_t row, int sub) {
    double s = 0.0;
    if (row < n) {
        const int k1 = __ldg(rp + row + 1);
        for (int k = __ldg(rp + row) + sub; k < k1; k += kLanesPerRow) s = fma(__ldg(v + k), __ldg(x + __ldg(ci + k)), s);
    }
#pragma unroll
    for (int o = kLanesPerRow / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
}

}  // namespace fem
