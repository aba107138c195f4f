// fem_bits.cuh -- bit tests on FP64 values in the integer pipe.
//
// The element kernels are bound by the FP64 pipe (16 cycles per warp
// instruction on GB300, whatever the number of active lanes).  A zero or
// finiteness test written on the value, or on its bit pattern through a plain
// bitcast, is folded by the compiler into an FP64 compare (DSETP) that takes
// the same pipe time as an FMA.  The 64-bit pattern is therefore split into
// its two 32-bit words by an opaque move, and the tests run on the words.
#pragma once
#include <cstdint>

__device__ __forceinline__ void fem_words(double x, uint32_t& lo, uint32_t& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "d"(x));
}
// x is neither +0 nor -0 (NaN counts as nonzero, as x != 0.0 does)
__device__ __forceinline__ bool fem_nonzero(double x) {
    uint32_t lo, hi;
    fem_words(x, lo, hi);
    return ((hi << 1) | lo) != 0u;
}
// x is neither infinite nor NaN (exponent field not all ones)
__device__ __forceinline__ bool fem_finite(double x) {
    uint32_t lo, hi;
    fem_words(x, lo, hi);
    return (hi & 0x7ff00000u) != 0x7ff00000u;
}
