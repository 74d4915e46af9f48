// fp64_exact.cuh -- FP64 operations that give IEEE's bits with less work on
// the FP64 pipe (GB300's FP64 rate is a small fraction of its FP32 rate, and
// the bit-exact FP64 kernels are bound by it).  Included by the kernels built
// with --fmad=false (f64_kernels.cu, sample_kernels.cu).
#pragma once

#include <cuda_runtime.h>

namespace lsgb {
namespace {

constexpr double RCP6 = 1.0 / 6.0;  // RN(1/6)

// a / b rounded to nearest, from y = RN(1/b): Markstein's theorem (P.
// Markstein, "Computation of elementary functions on the IBM RISC System/6000
// processor", IBM J. Res. Dev. 34(1), 1990; Muller et al., Handbook of
// Floating-Point Arithmetic, the section on division with an FMA): when q
// is within one ulp of a / b and y within half an ulp of 1 / b, the
// remainder r = a - b q is exact with one FMA and RN(q + r y) = RN(a / b).
// q = RN(a y) is within one ulp of a / b.  The theorem needs a, b, the
// quotient and the remainder clear of underflow and overflow, so a outside
// [2^-500, 2^501) (zeros too, whose sign the FMAs would not keep), or b
// outside it, takes IEEE division.  Every result is
// the IEEE quotient bit for bit, at one multiply and two FMAs where a
// division costs a reciprocal approximation and several FMAs.
__device__ __noinline__ double div_ieee(double a, double b) { return a / b; }

// Biased exponent of x in [523, 1523], i.e. 2^-500 <= |x| < 2^501, tested on
// the integer pipe (the FP64 pipe is the kernels' bottleneck).
__device__ __forceinline__ bool mid_range(double x) {
    const unsigned e = ((unsigned)__double2hiint(x) >> 20) & 0x7ffu;
    return e - 523u <= 1000u;
}

__device__ __forceinline__ double div_rn(double a, double b, double y) {
    if (!(mid_range(a) && mid_range(b))) return div_ieee(a, b);
    const double q = __dmul_rn(a, y);
    const double r = __fma_rn(-q, b, a);
    return __fma_rn(r, y, q);
}

// x * 2^K, exact: for a normal x whose product stays normal, the exponent
// field moves by K on the integer pipe; zeros, subnormals and the edges of
// the range take the FP64 multiply (whose result is the same product).
__device__ __noinline__ double mul_ieee(double x, double c) { return x * c; }

template <int K>
__device__ __forceinline__ double mul_pow2(double x) {
    const int hi = __double2hiint(x);
    const unsigned e = ((unsigned)hi >> 20) & 0x7ffu;
    // exponent field range of a normal x with a normal product
    constexpr unsigned lo = (unsigned)(K < 0 ? 1 - K : 1), hi_e = (unsigned)(K > 0 ? 0x7fe - K : 0x7fe);
    if (e - lo > hi_e - lo) return mul_ieee(x, K > 0 ? (double)(1 << K) : 1.0 / (double)(1 << -K));
    return __hiloint2double(hi + K * (1 << 20), __double2loint(x));
}

}  // namespace
}  // namespace lsgb
