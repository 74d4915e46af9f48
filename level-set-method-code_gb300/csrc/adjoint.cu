// adjoint.cu -- discrete adjoint (vector-Jacobian products) of the fused RK3
// stage and of the HCR-2 pseudo-step, on compact periodic fields.
//
// The forward maps being differentiated are the stage kernels of
// f64_kernels.cu / stage3d_f32.cu (computeRHS3D + rk3Stage{1,2,3}_3D,
// Local_code/level-set_MPI_3D/include/rk3.h:31-121, with the WENO-5 of
// weno5.h:28-196) and the pseudo-step reinitStep3D
// (reinitialization.h:95-193).  Piecewise choices are frozen at the forward
// state: the upwind branch u_eff >= 0 (weno5.h:99), the Godunov selection of
// weno5_gradient_magnitude_3d (weno5.h:202-248), the crossing flags and the
// stability mask of the interface constraint, and the s_l > epsilon gate.
// Everything else (WENO weights, |grad G|, u_eff, sign(phi0), r~) is
// differentiated exactly.
//
// Each transpose is two passes and needs no atomics, so results do not
// depend on scheduling:
//   coef pass    one thread per cell c forms lambda_c * dF_c/dG_{c+o} for every
//                stencil offset o and stores it in plane o (structure of
//                arrays), plus the point-wise parameter sensitivities;
//   gather pass  one thread per cell m sums plane o at m - o over all o in a
//                fixed order.
// Boundaries: periodic axes wrap, zero-gradient axes clamp (map_axis, as in
// the forward kernels).  The wrapped map is a bijection, so on periodic axes
// the gather reads one source per offset.  The clamped map is not: cell m
// receives plane o from c = m - o only when c lies inside the grid, and the
// first / last cell of a clamped axis also receives plane o of every cell
// whose stencil point c + o was clamped onto it (c + o < 0 or >= n).  The
// gather kernels add those terms in their ZG form.
#include "common.cuh"

#include <type_traits>

namespace lsgb {
namespace {

constexpr double ADJ_WENO_EPS = 1.0e-6;  // weno5.h:22

struct Idx {
    int nx, ny, nz;
    __device__ __forceinline__ long long at(int i, int j, int k) const {
        return (long long)i + (long long)nx * ((long long)j + (long long)ny * k);
    }
};

__device__ __forceinline__ int wrap(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }
// any integer onto [0, n)
__device__ __forceinline__ int wrapn(int i, int n) {
    i %= n;
    return i < 0 ? i + n : i;
}
// z plane of an unwrapped slab index: wrapped (periodic) or clamped
__device__ __forceinline__ int zmap(int k, int n, int bc) {
    return bc == LSGB_BC_PERIODIC ? wrapn(k, n) : (k < 0 ? 0 : (k >= n ? n - 1 : k));
}
// cells of a clamped axis whose stencil point c + o lands on the edge cell e
// (0 or n-1) only by clamping: c in [lo, hi]
__device__ __forceinline__ void clamped_sources(int e, int o, int n, int& lo, int& hi) {
    if (e == 0 && o < 0) { lo = 0; hi = min(-o - 1, n - 1); }
    else if (e == n - 1 && o > 0) { lo = max(n - o, 0); hi = n - 1; }
    else { lo = 1; hi = 0; }
}

// Reciprocal: IEEE in the FP64 adjoint; the approximate MUFU reciprocal in
// the FP32 adjoint (its relative error, ~1e-7, is below FP32 rounding of the
// sums it feeds).
__device__ __forceinline__ double rcpx(double x) { return 1.0 / x; }
__device__ __forceinline__ float rcpx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// WENO reconstruction f = sum_k w_k p_k over the candidate stencils of
// (a0..a4) with linear weights (d0, d1, d2), and df/da.  With
// alpha_k = d_k / (eps + beta_k)^2 and w_k = alpha_k / sum alpha:
//   df/da_j = sum_k w_k dp_k/da_j - 2 sum_k (p_k - f) w_k / (eps + beta_k) dbeta_k/da_j.
// beta_k = 13/12 (a_k - 2 a_{k+1} + a_{k+2})^2 + 1/4 (a_{k+2} - a_k)^2 is the
// reference's indicator (weno5.h:28-37).  weno5_left (:39-58) is
// (a) = (v0..v4), d = (0.1, 0.6, 0.3); weno5_right (:60-81) is the same
// formula on the reversed stencil with d = (0.3, 0.6, 0.1).
template <typename R>
__device__ __forceinline__ void weno_grad(R a0, R a1, R a2, R a3, R a4, R d0, R d1, R d2, R& f, R* df) {
    const R eps = (R)ADJ_WENO_EPS;
    const R c1312 = (R)(13.0 / 12.0), c136 = (R)(13.0 / 6.0), c133 = (R)(13.0 / 3.0);
    const R e0 = a0 - (R)2 * a1 + a2, e1 = a1 - (R)2 * a2 + a3, e2 = a2 - (R)2 * a3 + a4;
    const R h0 = a2 - a0, h1 = a3 - a1, h2 = a4 - a2;
    const R q0 = eps + c1312 * e0 * e0 + (R)0.25 * h0 * h0;
    const R q1 = eps + c1312 * e1 * e1 + (R)0.25 * h1 * h1;
    const R q2 = eps + c1312 * e2 * e2 + (R)0.25 * h2 * h2;
    const R r0 = rcpx(q0), r1 = rcpx(q1), r2 = rcpx(q2);
    const R al0 = d0 * r0 * r0, al1 = d1 * r1 * r1, al2 = d2 * r2 * r2;
    const R inv = rcpx(al0 + al1 + al2);
    const R w0 = al0 * inv, w1 = al1 * inv, w2 = al2 * inv;
    const R sixth = (R)(1.0 / 6.0);
    const R p0 = ((R)2 * a0 - (R)7 * a1 + (R)11 * a2) * sixth;
    const R p1 = (-a1 + (R)5 * a2 + (R)2 * a3) * sixth;
    const R p2 = ((R)2 * a2 + (R)5 * a3 - a4) * sixth;
    f = w0 * p0 + w1 * p1 + w2 * p2;
    const R c0 = (R)-2 * (p0 - f) * w0 * r0;
    const R cc1 = (R)-2 * (p1 - f) * w1 * r1;
    const R c2 = (R)-2 * (p2 - f) * w2 * r2;
    // dbeta_k / d(a_k, a_{k+1}, a_{k+2})
    const R b0l = c136 * e0 - (R)0.5 * h0, b0m = -c133 * e0, b0r = c136 * e0 + (R)0.5 * h0;
    const R b1l = c136 * e1 - (R)0.5 * h1, b1m = -c133 * e1, b1r = c136 * e1 + (R)0.5 * h1;
    const R b2l = c136 * e2 - (R)0.5 * h2, b2m = -c133 * e2, b2r = c136 * e2 + (R)0.5 * h2;
    df[0] = w0 * ((R)2 * sixth) + c0 * b0l;
    df[1] = w0 * ((R)-7 * sixth) + w1 * (-sixth) + c0 * b0m + cc1 * b1l;
    df[2] = w0 * ((R)11 * sixth) + w1 * ((R)5 * sixth) + w2 * ((R)2 * sixth) + c0 * b0r + cc1 * b1m + c2 * b2l;
    df[3] = w1 * ((R)2 * sixth) + w2 * ((R)5 * sixth) + cc1 * b1r + c2 * b2m;
    df[4] = w2 * (-sixth) + c2 * b2r;
}

// Upwind WENO derivative D = (f_{i+1/2} - f_{i-1/2}) / h of the 7-point line
// s[0..6] = G[i-3..i+3] (weno5_dx_3d, weno5.h:90-124) and dD/ds, without a
// branch on the upwind direction: with w[m] = s[m] (vel >= 0) or s[6-m]
// (vel < 0) both cases are X = f(w0..w4), Y = f(w1..w5) with linear weights
// (0.1, 0.6, 0.3) or (0.3, 0.6, 0.1), and D = +-(Y - X) / h (weno5_left at
// i -+ 1/2 in the first case, weno5_right on the mirrored stencils in the
// second).  Lanes of a warp with different upwind directions follow one path.
template <typename R>
__device__ __forceinline__ void axis_grad(const R* s, R vel, R inv_h, R& D, R* dD) {
    const bool p = vel >= (R)0;
    R w[7];
#pragma unroll
    for (int m = 0; m < 7; ++m) w[m] = p ? s[m] : s[6 - m];
    const R d0 = p ? (R)0.1 : (R)0.3, d2 = p ? (R)0.3 : (R)0.1;
    R X, Y, tX[5], tY[5];
    weno_grad(w[0], w[1], w[2], w[3], w[4], d0, (R)0.6, d2, X, tX);
    weno_grad(w[1], w[2], w[3], w[4], w[5], d0, (R)0.6, d2, Y, tY);
    const R sg = p ? inv_h : -inv_h;
    R dW[7];
    dW[0] = -tX[0] * sg;
#pragma unroll
    for (int m = 1; m <= 4; ++m) dW[m] = (tY[m - 1] - tX[m]) * sg;
    dW[5] = tY[4] * sg;
    dW[6] = (R)0;
#pragma unroll
    for (int m = 0; m < 7; ++m) dD[m] = p ? dW[m] : dW[6 - m];
    D = (Y - X) * sg;
}

// ---------------------------------------------------------------------------
// RK3 stage
// ---------------------------------------------------------------------------

// Planes of the stage transpose: 0 = centre, then per axis the offsets
// -3, -2, -1, +1, +2, +3 (axis a uses planes 1 + 6a .. 6 + 6a).
__device__ __forceinline__ int stage_off(int q) { return q < 3 ? q - 3 : q - 2; }

// ZG: some axis is zero-gradient (neighbours through map_axis); otherwise
// every axis wraps.
template <typename T, int DIM, bool ZG>
__global__ void __launch_bounds__(256) stage_adj_coef_kernel(AdjStageArgs a) {
    const Geo g = a.g;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int kl = DIM == 3 ? blockIdx.z * blockDim.z + threadIdx.z : 0;  // slab-local plane
    if (i >= g.nx || j >= g.ny || kl >= (DIM == 3 ? a.zn + 6 : 1)) return;
    const int ku = DIM == 3 ? a.z0 - 3 + kl : 0;  // unwrapped plane
    const long long sy = g.nx, sz = (long long)g.nx * g.ny;
    const long long P = DIM == 3 ? (long long)(a.zn + 6) * sz : g.cells();
    T* cp = (T*)a.coef + (i + sy * j + sz * kl);  // plane 0 of this cell; plane o at cp + o P
    if (ZG && DIM == 3 && g.bcz != LSGB_BC_PERIODIC && (ku < 0 || ku >= g.nz)) {
        // a plane outside a clamped z axis: no cell, no coefficients
#pragma unroll
        for (int o = 0; o < ADJ_PLANES; ++o) cp[o * P] = (T)0;
        return;
    }
    const int k = DIM == 3 ? (ZG ? zmap(ku, g.nz, g.bcz) : wrapn(ku, g.nz)) : 0;
    const bool own = DIM == 2 || (ku >= a.z0 && ku < a.z0 + a.zn);  // parameter gradients
    typedef T R;
    const T* __restrict__ G = (const T*)a.Gin;
    const long long c = i + sy * j + sz * k;
    const T* Gc = G + c;
    R s[3][7];
#pragma unroll
    for (int d = -3; d <= 3; ++d) {
        const int xi = ZG ? map_axis(i + d, g.nx, g.bcx) : wrap(i + d, g.nx);
        const int yj = ZG ? map_axis(j + d, g.ny, g.bcy) : wrap(j + d, g.ny);
        s[0][d + 3] = Gc[xi - i];
        s[1][d + 3] = Gc[(long long)(yj - j) * sy];
        if (DIM == 3) {
            const int zk = ZG ? map_axis(k + d, g.nz, g.bcz) : wrap(k + d, g.nz);
            s[2][d + 3] = Gc[(long long)(zk - k) * sz];
        }
    }
    const R S = a.sl ? ((const T*)a.sl)[c] : (R)a.s_l;
    const R ih[3] = {(R)(1.0 / a.dx), (R)(1.0 / a.dy), (R)(1.0 / a.dz)};
    R gr[3] = {(R)0, (R)0, (R)0};
    R gm = (R)1;
    const bool active = (double)S > a.eps;
    if (active) {
        R q = (R)0;
#pragma unroll
        for (int ax = 0; ax < DIM; ++ax) {
            gr[ax] = (s[ax][4] - s[ax][2]) * ((R)0.5 * ih[ax]);
            q += gr[ax] * gr[ax];
        }
        gm = sqrt(q + (R)a.eps);
    }
    const R igm = rcpx(gm);
    const T* vel[3] = {(const T*)a.u, (const T*)a.v, (const T*)a.w};
    R ue[3], D[3], dD[3][7];
#pragma unroll
    for (int ax = 0; ax < DIM; ++ax) {
        ue[ax] = vel[ax][c] - S * gr[ax] * igm;
        axis_grad(s[ax], ue[ax], ih[ax], D[ax], dD[ax]);
    }
    // R = -(sum_a ue_a D_a);  dR/dg_b = S (D_b / gm - (D . g) g_b / gm^3);  dR/dS = (D . g) / gm
    R dg = (R)0;
#pragma unroll
    for (int ax = 0; ax < DIM; ++ax) dg += D[ax] * gr[ax];
    const R wc = (R)(a.cdt) * ((const T*)a.lam)[c];
    R centre = (R)0;
#pragma unroll
    for (int ax = 0; ax < DIM; ++ax) {
        R dRg = (R)0;
        if (active) dRg = S * igm * (D[ax] - dg * gr[ax] * igm * igm);
        const R half = dRg * ((R)0.5 * ih[ax]);
        centre += -ue[ax] * dD[ax][3];
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const int sidx = stage_off(q) + 3;
            R v = -ue[ax] * dD[ax][sidx];
            if (sidx == 4) v += half;
            if (sidx == 2) v -= half;
            cp[(1 + 6 * ax + q) * P] = (T)(wc * v);
        }
    }
    cp[0] = (T)(wc * centre);
    if (a.gS && own) a.gS[c] += (double)(wc * (active ? dg * igm : (R)0));
    if (a.gu && own) {
        a.gu[c] += (double)(-wc * D[0]);
        a.gv[c] += (double)(-wc * D[1]);
        if (DIM == 3) a.gw[c] += (double)(-wc * D[2]);
    }
}

// ---- FP32 3D coefficient pass on plane pairs ---------------------------------
// The same transpose as stage_adj_coef_kernel<float, 3>, for the cells
// (i, j, k) and (i, j, k+1) of one thread at once: every per-cell quantity is
// a float2 over the plane pair and the arithmetic runs as packed f32x2
// operations (the mirrored stencil makes both cells follow one code path).
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 operator+(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 operator-(float2 a, float2 b) { return __ffma2_rn(f2(-1.0f), b, a); }
__device__ __forceinline__ float2 operator*(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 operator-(float2 a) { return __fmul2_rn(f2(-1.0f), a); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 rcp2(float2 a) { return make_float2(rcpx(a.x), rcpx(a.y)); }
__device__ __forceinline__ float2 sel2(bool px, bool py, float2 a, float2 b) {
    return make_float2(px ? a.x : b.x, py ? a.y : b.y);
}

__device__ __forceinline__ void weno_grad2(float2 a0, float2 a1, float2 a2, float2 a3, float2 a4, float2 d0, float2 d2,
                                           float2& f, float2* df) {
    const float2 e0 = fma2(f2(-2.0f), a1, a0) + a2, e1 = fma2(f2(-2.0f), a2, a1) + a3, e2 = fma2(f2(-2.0f), a3, a2) + a4;
    const float2 h0 = a2 - a0, h1 = a3 - a1, h2 = a4 - a2;
    const float2 c1312 = f2(13.0f / 12.0f), q4 = f2(0.25f), eps = f2((float)ADJ_WENO_EPS);
    const float2 q0 = fma2(c1312 * e0, e0, fma2(q4 * h0, h0, eps));
    const float2 q1 = fma2(c1312 * e1, e1, fma2(q4 * h1, h1, eps));
    const float2 q2 = fma2(c1312 * e2, e2, fma2(q4 * h2, h2, eps));
    const float2 r0 = rcp2(q0), r1 = rcp2(q1), r2 = rcp2(q2);
    const float2 al0 = d0 * r0 * r0, al1 = f2(0.6f) * r1 * r1, al2 = d2 * r2 * r2;
    const float2 inv = rcp2(al0 + al1 + al2);
    const float2 w0 = al0 * inv, w1 = al1 * inv, w2 = al2 * inv;
    const float sixth = 1.0f / 6.0f;
    const float2 p0 = fma2(f2(2.0f * sixth), a0, fma2(f2(-7.0f * sixth), a1, f2(11.0f * sixth) * a2));
    const float2 p1 = fma2(f2(-sixth), a1, fma2(f2(5.0f * sixth), a2, f2(2.0f * sixth) * a3));
    const float2 p2 = fma2(f2(2.0f * sixth), a2, fma2(f2(5.0f * sixth), a3, f2(-sixth) * a4));
    f = fma2(w0, p0, fma2(w1, p1, w2 * p2));
    const float2 c0 = f2(-2.0f) * (p0 - f) * w0 * r0;
    const float2 cc1 = f2(-2.0f) * (p1 - f) * w1 * r1;
    const float2 c2 = f2(-2.0f) * (p2 - f) * w2 * r2;
    const float2 k136 = f2(13.0f / 6.0f), k133 = f2(-13.0f / 3.0f), hf = f2(0.5f);
    const float2 b0l = fma2(k136, e0, -(hf * h0)), b0m = k133 * e0, b0r = fma2(k136, e0, hf * h0);
    const float2 b1l = fma2(k136, e1, -(hf * h1)), b1m = k133 * e1, b1r = fma2(k136, e1, hf * h1);
    const float2 b2l = fma2(k136, e2, -(hf * h2)), b2m = k133 * e2, b2r = fma2(k136, e2, hf * h2);
    df[0] = fma2(w0, f2(2.0f * sixth), c0 * b0l);
    df[1] = fma2(w0, f2(-7.0f * sixth), fma2(w1, f2(-sixth), fma2(c0, b0m, cc1 * b1l)));
    df[2] = fma2(w0, f2(11.0f * sixth), fma2(w1, f2(5.0f * sixth), fma2(w2, f2(2.0f * sixth),
                 fma2(c0, b0r, fma2(cc1, b1m, c2 * b2l)))));
    df[3] = fma2(w1, f2(2.0f * sixth), fma2(w2, f2(5.0f * sixth), fma2(cc1, b1r, c2 * b2m)));
    df[4] = fma2(w2, f2(-sixth), c2 * b2r);
}

__device__ __forceinline__ void axis_grad2(const float2* s, float2 vel, float inv_h, float2& D, float2* dD) {
    const bool px = vel.x >= 0.0f, py = vel.y >= 0.0f;
    float2 w[7];
#pragma unroll
    for (int m = 0; m < 7; ++m) w[m] = sel2(px, py, s[m], s[6 - m]);
    const float2 d0 = make_float2(px ? 0.1f : 0.3f, py ? 0.1f : 0.3f);
    const float2 d2 = make_float2(px ? 0.3f : 0.1f, py ? 0.3f : 0.1f);
    float2 X, Y, tX[5], tY[5];
    weno_grad2(w[0], w[1], w[2], w[3], w[4], d0, d2, X, tX);
    weno_grad2(w[1], w[2], w[3], w[4], w[5], d0, d2, Y, tY);
    const float2 sg = make_float2(px ? inv_h : -inv_h, py ? inv_h : -inv_h);
    float2 dW[7];
    dW[0] = -(tX[0] * sg);
#pragma unroll
    for (int m = 1; m <= 4; ++m) dW[m] = (tY[m - 1] - tX[m]) * sg;
    dW[5] = tY[4] * sg;
    dW[6] = f2(0.0f);
#pragma unroll
    for (int m = 0; m < 7; ++m) dD[m] = sel2(px, py, dW[m], dW[6 - m]);
    D = (Y - X) * sg;
}

template <bool ZG>
__global__ void __launch_bounds__(256, 3) stage_adj_coef_pair_kernel(AdjStageArgs a) {
    const Geo g = a.g;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int kl = 2 * (blockIdx.z * blockDim.z + threadIdx.z);  // slab-local plane of the pair
    const int nl = a.zn + 6;
    if (i >= g.nx || j >= g.ny || kl >= nl) return;
    const bool two = kl + 1 < nl;  // an odd slab leaves the last thread one plane
    const int ku = a.z0 - 3 + kl;
    const int k = ZG ? zmap(ku, g.nz, g.bcz) : wrapn(ku, g.nz), k1 = ZG ? zmap(ku + 1, g.nz, g.bcz) : wrapn(ku + 1, g.nz);
    // planes outside a clamped z axis hold no cell: their coefficients are 0
    const bool zper = !ZG || g.bcz == LSGB_BC_PERIODIC;
    const bool in0 = zper || (ku >= 0 && ku < g.nz), in1 = zper || (ku + 1 >= 0 && ku + 1 < g.nz);
    const bool own0 = ku >= a.z0 && ku < a.z0 + a.zn;
    const bool own1 = two && ku + 1 >= a.z0 && ku + 1 < a.z0 + a.zn;
    const float* __restrict__ G = (const float*)a.Gin;
    const long long sy = g.nx, sz = (long long)g.nx * g.ny;
    const long long c = i + sy * j + sz * k;
    const long long c1 = i + sy * j + sz * k1;
    const float* Gc = G + c;
    // The central differences first (two samples per axis); then one axis
    // at a time: its 7-point line, the WENO derivative and the four
    // coefficients that do not involve the other axes, stored at once.  The
    // +-1 offsets wait for dg (every axis's D), so only their partial values
    // stay live.
    float zq[8];
#pragma unroll
    for (int d = 0; d < 8; ++d) zq[d] = G[i + sy * j + sz * (ZG ? zmap(ku - 3 + d, g.nz, g.bcz) : wrapn(ku - 3 + d, g.nz))];
    auto sample = [&](int ax, int d) -> float2 {  // G at offset d (-3 .. 3) along axis ax, planes k and k+1
        if (ax == 2) return make_float2(zq[d + 3], zq[d + 4]);
        const long long o = ax == 0 ? (long long)((ZG ? map_axis(i + d, g.nx, g.bcx) : wrap(i + d, g.nx)) - i)
                                    : (long long)((ZG ? map_axis(j + d, g.ny, g.bcy) : wrap(j + d, g.ny)) - j) * sy;
        return make_float2(Gc[o], G[c1 + o]);
    };
    const float* sl = (const float*)a.sl;
    const float2 S = sl ? make_float2(sl[c], sl[c1]) : f2((float)a.s_l);
    const float ih[3] = {(float)(1.0 / a.dx), (float)(1.0 / a.dy), (float)(1.0 / a.dz)};
    const float epsf = (float)a.eps;
    const bool actx = (double)S.x > a.eps, acty = (double)S.y > a.eps;
    float2 gr[3], q = f2(0.0f);
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        gr[ax] = (sample(ax, 1) - sample(ax, -1)) * f2(0.5f * ih[ax]);
        gr[ax] = make_float2(actx ? gr[ax].x : 0.0f, acty ? gr[ax].y : 0.0f);
        q = fma2(gr[ax], gr[ax], q);
    }
    const float2 gm = make_float2(actx ? sqrtf(q.x + epsf) : 1.0f, acty ? sqrtf(q.y + epsf) : 1.0f);
    const float2 igm = rcp2(gm);
    const float* vel[3] = {(const float*)a.u, (const float*)a.v, (const float*)a.w};
    const float* lam = (const float*)a.lam;
    const float2 wc = ZG ? f2((float)a.cdt) * make_float2(in0 ? lam[c] : 0.0f, in1 ? lam[c1] : 0.0f)
                         : f2((float)a.cdt) * make_float2(lam[c], lam[c1]);
    const long long P = (long long)nl * sz;  // plane stride of the slab buffer
    float* cp0 = (float*)a.coef + (i + sy * j + sz * kl);
    float* cp1 = cp0 + sz;
    float2 D[3], vm1[3], vp1[3], centre = f2(0.0f);
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        float2 line[7], dD[7];
#pragma unroll
        for (int d = -3; d <= 3; ++d) line[d + 3] = sample(ax, d);
        const float2 ue = make_float2(vel[ax][c], vel[ax][c1]) - S * gr[ax] * igm;
        axis_grad2(line, ue, ih[ax], D[ax], dD);
        centre = centre - ue * dD[3];
#pragma unroll
        for (int q6 = 0; q6 < 6; ++q6) {
            const int sidx = stage_off(q6) + 3;
            const float2 v = -(ue * dD[sidx]);
            if (sidx == 2) { vm1[ax] = v; continue; }
            if (sidx == 4) { vp1[ax] = v; continue; }
            const float2 o = wc * v;
            const long long po = (long long)(1 + 6 * ax + q6) * P;
            cp0[po] = o.x;
            if (two) cp1[po] = o.y;
        }
    }
    float2 dg = f2(0.0f);
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) dg = fma2(D[ax], gr[ax], dg);
    const float2 igm2 = igm * igm;
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        float2 dRg = S * igm * (D[ax] - dg * gr[ax] * igm2);
        dRg = make_float2(actx ? dRg.x : 0.0f, acty ? dRg.y : 0.0f);
        const float2 half = dRg * f2(0.5f * ih[ax]);
        const float2 om = wc * (vm1[ax] - half), op = wc * (vp1[ax] + half);
        const long long pm = (long long)(1 + 6 * ax + 2) * P, pp = (long long)(1 + 6 * ax + 3) * P;
        cp0[pm] = om.x;
        cp0[pp] = op.x;
        if (two) {
            cp1[pm] = om.y;
            cp1[pp] = op.y;
        }
    }
    const float2 oc = wc * centre;
    cp0[0] = oc.x;
    if (two) cp1[0] = oc.y;
    if (a.gS) {
        const float2 gs = wc * dg * igm;
        if (own0) a.gS[c] += (double)(actx ? gs.x : 0.0f);
        if (own1) a.gS[c1] += (double)(acty ? gs.y : 0.0f);
    }
    if (a.gu) {
        double* gp[3] = {a.gu, a.gv, a.gw};
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const float2 gv = -(wc * D[ax]);
            if (own0) gp[ax][c] += (double)gv.x;
            if (own1) gp[ax][c1] += (double)gv.y;
        }
    }
}

// out[m] = c_self lam[m] + addend[m] + sum_o plane_o[m - o];
// acc[m] = (acc_init ? 0 : acc[m]) + c_n lam[m] when acc is given.
// ZG: some axis is zero-gradient (sources outside the grid skipped, clamped
// sources added on the edge cells).
template <typename T, int DIM, bool ZG>
__global__ void __launch_bounds__(256) stage_adj_gather_kernel(AdjGatherArgs a) {
    const Geo g = a.g;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int kk = DIM == 3 ? blockIdx.z * blockDim.z + threadIdx.z : 0;
    if (i >= g.nx || j >= g.ny || kk >= (DIM == 3 ? a.zn : 1)) return;
    const int k = DIM == 3 ? a.z0 + kk : 0;
    const long long sy = g.nx, sz = (long long)g.nx * g.ny;
    const long long m = i + sy * j + sz * k;
    const long long P = DIM == 3 ? (long long)(a.zn + 6) * sz : g.cells();
    const int kl = DIM == 3 ? kk + 3 : 0;  // slab-local plane of m
    const T* __restrict__ cm = (const T*)a.coef + (i + sy * j + sz * kl);  // plane 0 at cell m
    const T lam = ((const T*)a.lam)[m];
    T sum = cm[0];
    if (!ZG) {
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const int o = stage_off(q);
            sum += cm[(1 + q) * P + (wrap(i - o, g.nx) - i)];
        }
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const int o = stage_off(q);
            sum += cm[(7 + q) * P + (long long)(wrap(j - o, g.ny) - j) * sy];
        }
        if (DIM == 3) {
#pragma unroll
            for (int q = 0; q < 6; ++q) {
                const int o = stage_off(q);
                sum += cm[(13 + q) * P - (long long)o * sz];  // source plane kl - o of the slab
            }
        }
    } else {
        const int at[3] = {i, j, k};
        const int n[3] = {g.nx, g.ny, g.nz};
        const int bc[3] = {g.bcx, g.bcy, g.bcz};
        const long long str[3] = {1, sy, sz};
#pragma unroll
        for (int ax = 0; ax < DIM; ++ax) {
            const bool per = bc[ax] == LSGB_BC_PERIODIC;
#pragma unroll
            for (int q = 0; q < 6; ++q) {
                const int o = stage_off(q);
                const long long pl = (long long)(1 + 6 * ax + q) * P;
                // z: the slab buffer is indexed by unwrapped plane, and its planes
                // outside a clamped axis hold zeros
                int src = at[ax] - o;
                if (per && ax < 2) src = wrap(src, n[ax]);
                if (per || ax == 2 || (src >= 0 && src < n[ax])) sum += cm[pl + (long long)(src - at[ax]) * str[ax]];
            }
            if (!per && (at[ax] == 0 || at[ax] == n[ax] - 1)) {
#pragma unroll
                for (int q = 0; q < 6; ++q) {
                    const int o = stage_off(q);
                    const long long pl = (long long)(1 + 6 * ax + q) * P;
                    int lo, hi;
                    clamped_sources(at[ax], o, n[ax], lo, hi);
                    for (int cc = lo; cc <= hi; ++cc) sum += cm[pl + (long long)(cc - at[ax]) * str[ax]];
                }
            }
        }
    }
    T out = (T)a.c_self * lam + sum;
    if (a.addend) out += ((const T*)a.addend)[m];
    ((T*)a.out)[m] = out;
    if (a.acc) {
        T* acc = (T*)a.acc;
        acc[m] = (a.acc_init ? (T)0 : acc[m]) + (T)a.c_n * lam;
    }
}

// ---------------------------------------------------------------------------
// HCR-2 pseudo-step
// ---------------------------------------------------------------------------

// Planes: 0..6 for phi^m (centre, -x, +x, -y, +y, -z, +z), 7..13 for phi0.
__device__ __forceinline__ void nb_off(int q, int& ox, int& oy, int& oz) {
    ox = oy = oz = 0;
    const int sgn = (q & 1) ? 1 : -1;
    if (q < 2) ox = sgn;
    else if (q < 4) oy = sgn;
    else oz = sgn;
}

template <typename T, int DIM, bool ZG>
__global__ void __launch_bounds__(256) reinit_adj_coef_kernel(AdjReinitArgs a) {
    const Geo g = a.g;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = DIM == 3 ? blockIdx.z * blockDim.z + threadIdx.z : 0;
    if (i >= g.nx || j >= g.ny || k >= g.nz) return;
    typedef T R;
    const Idx ix{g.nx, g.ny, g.nz};
    const long long c = ix.at(i, j, k);
    const T* __restrict__ phin = (const T*)a.phin;
    const T* __restrict__ phi0 = (const T*)a.phi0;
    long long nb[6];
#pragma unroll
    for (int q = 0; q < 2 * DIM; ++q) {
        int ox, oy, oz;
        nb_off(q, ox, oy, oz);
        if (ZG)
            nb[q] = ix.at(map_axis(i + ox, g.nx, g.bcx), map_axis(j + oy, g.ny, g.bcy),
                          DIM == 3 ? map_axis(k + oz, g.nz, g.bcz) : 0);
        else
            nb[q] = ix.at(wrap(i + ox, g.nx), wrap(j + oy, g.ny), wrap(k + oz, g.nz));
    }
    const R phi = phin[c], ph0 = phi0[c];
    R pn[6], p0[6];
#pragma unroll
    for (int q = 0; q < 2 * DIM; ++q) { pn[q] = phin[nb[q]]; p0[q] = phi0[nb[q]]; }
    const R dx = (R)a.dx;
    const R h[3] = {(R)a.dx, (R)a.dy, (R)a.dz};
    const R rad = sqrt(ph0 * ph0 + dx * dx);
    const R S = ph0 / rad;  // smoothSign (reinitialization.h:24)
    const R dS = dx * dx / (rad * rad * rad);
    const bool pos = S > (R)0;
    // Godunov |grad phi|^2 with the selected one-sided difference per axis
    R gsq = (R)0, dgc = (R)0, dgn[6];
#pragma unroll
    for (int ax = 0; ax < DIM; ++ax) {
        const R inv = (R)1 / h[ax];
        const R dm = (phi - pn[2 * ax]) * inv;
        const R dp = (pn[2 * ax + 1] - phi) * inv;
        const R A = pos ? (dm > (R)0 ? dm : (R)0) : (dm < (R)0 ? dm : (R)0);
        const R B = pos ? (dp < (R)0 ? dp : (R)0) : (dp > (R)0 ? dp : (R)0);
        dgn[2 * ax] = dgn[2 * ax + 1] = (R)0;
        if (A * A >= B * B) {
            gsq += A * A;  // d(A^2) = 2 A dA, dA = (dphi - dpn_minus) / h where A = dm
            dgc += (R)2 * A * inv;
            dgn[2 * ax] = (R)-2 * A * inv;
        } else {
            gsq += B * B;
            dgc += (R)-2 * B * inv;
            dgn[2 * ax + 1] = (R)2 * B * inv;
        }
    }
    const R sq = sqrt(gsq);
    const R dterm = sq > (R)0 ? -S / ((R)2 * sq) : (R)0;  // d term / d gsq
    R cphi = dterm * dgc;          // d(term + forcing) / d phi_c
    R c0 = -(sq - (R)1) * dS;      // d(term + forcing) / d phi0_c
    R cn[6], c0n[6];
#pragma unroll
    for (int q = 0; q < 2 * DIM; ++q) { cn[q] = dterm * dgn[q]; c0n[q] = (R)0; }
    // interface constraint (computeInterfaceCrossings3D :46-89, stability
    // check :95-130, forcing :160-178), evaluated in FP64 as in the forward
    int flag = 0;
#pragma unroll
    for (int q = 0; q < 2 * DIM; ++q)
        if ((double)ph0 * (double)p0[q] < 0.0) flag |= 1 << q;
    if (flag) {
        bool stable = (phi > (R)0) == (ph0 > (R)0);
#pragma unroll
        for (int q = 0; q < 2 * DIM; ++q)
            if ((flag >> q) & 1) stable = stable && ((pn[q] > (R)0) == (p0[q] > (R)0));
        if (stable) {
            double sum0 = 0.0, sumn = 0.0;
#pragma unroll
            for (int q = 0; q < 2 * DIM; ++q)
                if ((flag >> q) & 1) { sum0 += (double)p0[q]; sumn += (double)pn[q]; }
            const double bdx = a.beta / a.dx;
            const bool has_rt = fabs(sum0) > 1e-15;
            const double rt = has_rt ? (double)ph0 / sum0 : 0.0;
            cphi += (R)(-bdx);
            if (has_rt) {
                const double drt_c = 1.0 / sum0, drt_n = -(double)ph0 / (sum0 * sum0);
                c0 += (R)(bdx * sumn * drt_c);
#pragma unroll
                for (int q = 0; q < 2 * DIM; ++q)
                    if ((flag >> q) & 1) {
                        cn[q] += (R)(bdx * rt);
                        c0n[q] = (R)(bdx * sumn * drt_n);
                    }
            }
        }
    }
    const R mu = ((const T*)a.mu)[c];
    const R md = mu * (R)a.dtau;
    T* coef = (T*)a.coef;
    const long long P = g.cells();
    coef[c] = (T)(mu + md * cphi);
    coef[7 * P + c] = (T)(md * c0);
#pragma unroll
    for (int q = 0; q < 2 * DIM; ++q) {
        coef[(long long)(1 + q) * P + c] = (T)(md * cn[q]);
        coef[(long long)(8 + q) * P + c] = (T)(md * c0n[q]);
    }
}

// mu_out[m] = sum_o plane_o[m - o]  (o over centre and the 2 DIM neighbours)
// lam0[m]   = (first ? 0 : lam0[m]) + sum_o plane_{7+o}[m - o]
// last:      mu_out[m] += lam0[m]   (phi^0 = phi0)
// ZG: on a clamped axis a source outside the grid is skipped, and the edge
// cell also takes its own plane of the offset that points out of the grid.
template <typename T, int DIM, bool ZG>
__global__ void __launch_bounds__(256) reinit_adj_gather_kernel(AdjReinitGatherArgs a) {
    const Geo g = a.g;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = DIM == 3 ? blockIdx.z * blockDim.z + threadIdx.z : 0;
    if (i >= g.nx || j >= g.ny || k >= g.nz) return;
    const Idx ix{g.nx, g.ny, g.nz};
    const long long m = ix.at(i, j, k);
    const long long P = g.cells();
    const T* __restrict__ coef = (const T*)a.coef;
    T s = coef[m], s0 = coef[7 * P + m];
#pragma unroll
    for (int q = 0; q < 2 * DIM; ++q) {
        int ox, oy, oz;
        nb_off(q, ox, oy, oz);
        // plane q of cell c holds d F_c / d phi_{c + o}: cell m receives it from c = m - o
        if (!ZG) {
            const long long c = ix.at(wrap(i - ox, g.nx), wrap(j - oy, g.ny), wrap(k - oz, g.nz));
            s += coef[(long long)(1 + q) * P + c];
            s0 += coef[(long long)(8 + q) * P + c];
        } else {
            const int ax = q >> 1, o = (q & 1) ? 1 : -1;
            const int at = ax == 0 ? i : (ax == 1 ? j : k);
            const int n = ax == 0 ? g.nx : (ax == 1 ? g.ny : g.nz);
            const bool per = (ax == 0 ? g.bcx : (ax == 1 ? g.bcy : g.bcz)) == LSGB_BC_PERIODIC;
            const int src = per ? wrap(at - o, n) : at - o;
            if (per || (src >= 0 && src < n)) {
                const long long c = ix.at(ax == 0 ? src : i, ax == 1 ? src : j, ax == 2 ? src : k);
                s += coef[(long long)(1 + q) * P + c];
                s0 += coef[(long long)(8 + q) * P + c];
            }
            if (!per && ((o < 0 && at == 0) || (o > 0 && at == n - 1))) {
                s += coef[(long long)(1 + q) * P + m];
                s0 += coef[(long long)(8 + q) * P + m];
            }
        }
    }
    T* lam0 = (T*)a.lam0;
    const T l0 = (a.first ? (T)0 : lam0[m]) + s0;
    if (a.last) ((T*)a.mu_out)[m] = s + l0;
    else {
        ((T*)a.mu_out)[m] = s;
        lam0[m] = l0;
    }
}

// ---------------------------------------------------------------------------
// smoothed-Heaviside mismatch  L = 1/2 sum (H(G) - H(Gt))^2 dV,
// H(g) = (1 - tanh(g / eps)) / 2; lam = dL/dG = (H(G) - H(Gt)) H'(G) dV
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) heaviside_kernel(long long n, const T* __restrict__ G,
                                                                const double* __restrict__ Gt, double eps,
                                                                double dv, T* __restrict__ lam,
                                                                double* __restrict__ partials) {
    __shared__ double red[RED_THREADS];
    double acc = 0.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const double th = tanh((double)G[e] / eps);
        const double d = 0.5 * (1.0 - th) - 0.5 * (1.0 - tanh(Gt[e] / eps));
        acc += 0.5 * d * d * dv;
        if (lam) lam[e] = (T)(d * (-0.5 * (1.0 - th * th) / eps) * dv);
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = RED_THREADS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) partials[blockIdx.x] = red[0];
}

__global__ void __launch_bounds__(RED_THREADS) sum_partials_kernel(const double* __restrict__ partials, int n,
                                                                   double* __restrict__ out) {
    __shared__ double red[RED_THREADS];
    double acc = 0.0;
    for (int e = threadIdx.x; e < n; e += blockDim.x) acc += partials[e];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = RED_THREADS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = red[0];
}

bool zero_gradient(const Geo& g) {
    return g.bcx != LSGB_BC_PERIODIC || g.bcy != LSGB_BC_PERIODIC || (g.dim == 3 && g.bcz != LSGB_BC_PERIODIC);
}

dim3 cell_block(const Geo& g) { return g.dim == 3 ? dim3(32, 4, 2) : dim3(32, 8, 1); }
dim3 cell_grid(const Geo& g, dim3 b) {
    return dim3((g.nx + b.x - 1) / b.x, (g.ny + b.y - 1) / b.y, g.dim == 3 ? (g.nz + b.z - 1) / b.z : 1);
}

}  // namespace

template <typename T>
cudaError_t launch_stage_adj(const AdjStageArgs& c, const AdjGatherArgs& gth, cudaStream_t st) {
    const dim3 b = cell_block(c.g), gr = cell_grid(c.g, b);
    if (c.g.dim == 3) {
        const int nl = c.zn + 6;
        if (std::is_same<T, float>::value) {
            // plane pairs: half the threads along z
            const dim3 gp(gr.x, gr.y, (unsigned)((nl + 2 * b.z - 1) / (2 * b.z)));
            if (zero_gradient(c.g)) stage_adj_coef_pair_kernel<true><<<gp, b, 0, st>>>(c);
            else stage_adj_coef_pair_kernel<false><<<gp, b, 0, st>>>(c);
        } else {
            const dim3 gc(gr.x, gr.y, (unsigned)((nl + b.z - 1) / b.z));
            if (zero_gradient(c.g)) stage_adj_coef_kernel<T, 3, true><<<gc, b, 0, st>>>(c);
            else stage_adj_coef_kernel<T, 3, false><<<gc, b, 0, st>>>(c);
        }
        const dim3 gg(gr.x, gr.y, (unsigned)((gth.zn + b.z - 1) / b.z));
        if (zero_gradient(c.g)) stage_adj_gather_kernel<T, 3, true><<<gg, b, 0, st>>>(gth);
        else stage_adj_gather_kernel<T, 3, false><<<gg, b, 0, st>>>(gth);
    } else {
        if (zero_gradient(c.g)) stage_adj_coef_kernel<T, 2, true><<<gr, b, 0, st>>>(c);
        else stage_adj_coef_kernel<T, 2, false><<<gr, b, 0, st>>>(c);
        if (zero_gradient(c.g)) stage_adj_gather_kernel<T, 2, true><<<gr, b, 0, st>>>(gth);
        else stage_adj_gather_kernel<T, 2, false><<<gr, b, 0, st>>>(gth);
    }
    count_launches(2);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_reinit_adj(const AdjReinitArgs& c, const AdjReinitGatherArgs& gth, cudaStream_t st) {
    const dim3 b = cell_block(c.g), gr = cell_grid(c.g, b);
    if (c.g.dim == 3) {
        if (zero_gradient(c.g)) reinit_adj_coef_kernel<T, 3, true><<<gr, b, 0, st>>>(c);
        else reinit_adj_coef_kernel<T, 3, false><<<gr, b, 0, st>>>(c);
        if (zero_gradient(c.g)) reinit_adj_gather_kernel<T, 3, true><<<gr, b, 0, st>>>(gth);
        else reinit_adj_gather_kernel<T, 3, false><<<gr, b, 0, st>>>(gth);
    } else {
        if (zero_gradient(c.g)) reinit_adj_coef_kernel<T, 2, true><<<gr, b, 0, st>>>(c);
        else reinit_adj_coef_kernel<T, 2, false><<<gr, b, 0, st>>>(c);
        if (zero_gradient(c.g)) reinit_adj_gather_kernel<T, 2, true><<<gr, b, 0, st>>>(gth);
        else reinit_adj_gather_kernel<T, 2, false><<<gr, b, 0, st>>>(gth);
    }
    count_launches(2);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_heaviside(const Geo& g, const T* G, const double* Gt, double eps, double dv, T* lam,
                             double* partials, double* out, cudaStream_t st) {
    heaviside_kernel<T><<<RED_BLOCKS, RED_THREADS, 0, st>>>(g.cells(), G, Gt, eps, dv, lam, partials);
    sum_partials_kernel<<<1, RED_THREADS, 0, st>>>(partials, RED_BLOCKS, out);
    count_launches(2);
    return cudaGetLastError();
}

template cudaError_t launch_stage_adj<float>(const AdjStageArgs&, const AdjGatherArgs&, cudaStream_t);
template cudaError_t launch_stage_adj<double>(const AdjStageArgs&, const AdjGatherArgs&, cudaStream_t);
template cudaError_t launch_reinit_adj<float>(const AdjReinitArgs&, const AdjReinitGatherArgs&, cudaStream_t);
template cudaError_t launch_reinit_adj<double>(const AdjReinitArgs&, const AdjReinitGatherArgs&, cudaStream_t);
template cudaError_t launch_heaviside<float>(const Geo&, const float*, const double*, double, double, float*,
                                             double*, double*, cudaStream_t);
template cudaError_t launch_heaviside<double>(const Geo&, const double*, const double*, double, double, double*,
                                              double*, double*, cudaStream_t);

}  // namespace lsgb
