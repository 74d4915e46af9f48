// weno_f32x2.cuh -- packed-f32x2 building blocks of the FP32 stage kernels
// (stage3d_f32.cu, stage2d_f32.cu): the per-face WENO-5 reconstructions of
// weno5_left / weno5_right (Local_code/level-set_MPI_3D/include/weno5.h:28-81)
// evaluated on pairs of values at once.  The pair is whatever the kernel
// packs: two z-planes in 3D, two rows in 2D.  Also the asynchronous-copy
// primitives both kernels stage with.
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"

namespace lsgb {
namespace wf {

__device__ __forceinline__ float2 c2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(c2(-1.0f), b, a); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float2 div2(float2 n, float2 d) {
    return mul2(n, make_float2(rcp_approx(d.x), rcp_approx(d.y)));
}

// 144 (1e-6 + beta)^2 of the triple (a, b, c), beta as computeSmoothnessIndicators
// (weno5.h:28-37): 13/12 (a - 2b + c)^2 + 1/4 (c - a)^2.  The WENO weights are
// ratios of products of two indicators each, so the common factor 144 cancels.
__device__ __forceinline__ float2 qbeta(float2 a, float2 b, float2 c) {
    const float2 t = add2(fma2(c2(-2.0f), b, a), c);
    const float2 r = sub2(c, a);
    const float2 s = fma2(mul2(c2(13.0f), t), t, fma2(mul2(c2(3.0f), r), r, c2(12.0e-6f)));
    return mul2(s, s);
}

// Both reconstructions at the face between cells f-1 and f, times 6: the 1/6
// of the candidate polynomials is folded into the derivative's 1/(6h).  The
// weights are the reference's linear weights over the products of the other
// two indicators, scaled by 10 (ratios are unchanged):
//   L: (0.1 q(f-1) q(f), 0.6 q(f-2) q(f), 0.3 q(f-2) q(f-1)) x 10
//   R: (0.3 q(f-1) q(f), 0.6 q(f+1) q(f-1), 0.1 q(f+1) q(f)) x 10
__device__ __forceinline__ void face(float2 g0, float2 g1, float2 g2, float2 g3, float2 g4, float2 g5,
                                     float2 qm2, float2 qm1, float2 q0, float2 qp1, float2& L, float2& R) {
    const float2 Pa = fma2(c2(2.0f), g0, fma2(c2(-7.0f), g1, mul2(c2(11.0f), g2)));
    const float2 Pb = fma2(c2(5.0f), g2, fma2(c2(2.0f), g3, make_float2(-g1.x, -g1.y)));
    const float2 Pc = fma2(c2(2.0f), g2, fma2(c2(5.0f), g3, make_float2(-g4.x, -g4.y)));
    const float2 Pr = fma2(c2(11.0f), g3, fma2(c2(-7.0f), g4, mul2(c2(2.0f), g5)));
    const float2 q12 = mul2(qm1, q0);
    const float2 lw1 = mul2(c2(6.0f), mul2(qm2, q0));
    const float2 lw2 = mul2(c2(3.0f), mul2(qm2, qm1));
    const float2 rw0 = mul2(c2(3.0f), q12);
    const float2 rw1 = mul2(c2(6.0f), mul2(qp1, qm1));
    const float2 rw2 = mul2(qp1, q0);
    L = div2(fma2(q12, Pa, fma2(lw1, Pb, mul2(lw2, Pc))), add2(add2(q12, lw1), lw2));
    R = div2(fma2(rw0, Pr, fma2(rw1, Pc, mul2(rw2, Pb))), add2(add2(rw0, rw1), rw2));
}

// Shared-memory address of a generic pointer into shared memory.
__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Ampere-style asynchronous 4-byte copies global -> shared; completion per
// thread by groups (the copies depend on nothing but the memory system).
__device__ __forceinline__ void cp_async4(float* dst, const float* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(saddr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Coordinate map for tile loads: any offset (ragged tiles reach past n).
__device__ __forceinline__ int wrapg(int x, int n, int bc) {
    if (bc == LSGB_BC_PERIODIC) {
        x %= n;
        return x < 0 ? x + n : x;
    }
    return x < 0 ? 0 : (x >= n ? n - 1 : x);
}


// Both reconstructions at a face from its six samples s[0], s[st], .. s[5 st],
// with the four indicators computed on the spot.
__device__ __forceinline__ void face6(const float2* s, int st, float2& L, float2& R) {
    const float2 g0 = s[0], g1 = s[st], g2 = s[2 * st], g3 = s[3 * st], g4 = s[4 * st], g5 = s[5 * st];
    face(g0, g1, g2, g3, g4, g5, qbeta(g0, g1, g2), qbeta(g1, g2, g3), qbeta(g2, g3, g4), qbeta(g3, g4, g5), L, R);
}

// x face of column tx (lane tx) with the indicators shared across the warp:
// each lane computes q at its own column and one edge indicator (q(-2),
// q(-1) in lanes 0, 1; q(32) in lane 31), the rest come by shuffles.
__device__ __forceinline__ float2 shfl_up2(float2 v, int d) {
    return make_float2(__shfl_up_sync(0xffffffffu, v.x, d), __shfl_up_sync(0xffffffffu, v.y, d));
}
__device__ __forceinline__ float2 shfl_dn2(float2 v, int d) {
    return make_float2(__shfl_down_sync(0xffffffffu, v.x, d), __shfl_down_sync(0xffffffffu, v.y, d));
}
__device__ __forceinline__ void xface_shfl(const float2* s, int lane, float2& L, float2& R) {
    const float2 g0 = s[0], g1 = s[1], g2 = s[2], g3 = s[3], g4 = s[4], g5 = s[5];
    const bool lo = lane < 2;
    const float2 qc = qbeta(g2, g3, g4);
    const float2 qe = qbeta(lo ? g0 : g3, lo ? g1 : g4, lo ? g2 : g5);
    const float2 u2 = shfl_up2(qc, 2), u1 = shfl_up2(qc, 1), d1 = shfl_dn2(qc, 1), e1 = shfl_dn2(qe, 1);
    const float2 qm2 = lane >= 2 ? u2 : qe;
    const float2 qm1 = lane >= 1 ? u1 : e1;
    const float2 qp1 = lane <= 30 ? d1 : qe;
    face(g0, g1, g2, g3, g4, g5, qm2, qm1, qc, qp1, L, R);
}

}  // namespace wf
}  // namespace lsgb
