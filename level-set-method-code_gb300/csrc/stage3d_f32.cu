// stage3d_f32.cu -- the FP32-bulk 3D RK3 stage kernel (the throughput path).
//
// One launch = one TVD-RK3 stage over the whole grid, fused: the u_eff WENO-5
// right-hand side of computeRHS3D (Local_code/level-set_MPI_3D/include/
// rk3.h:31-81, weno5.h:28-196) and the stage combination of rk3Stage{1,2,3}_3D
// (rk3.h:87-121).  Compact arrays, periodic / zero-gradient neighbours by
// index mapping (no ghost cells, no boundary pass).
//
// Shape (2.5D blocking, two planes per step):
//   - a CTA owns a 32 x 8 column tile and marches a chunk of 64 z-planes two
//     at a time; thread (x, y) owns the cells (x, y, k) and (x, y, k+1);
//   - every per-cell quantity is held as a float2 over the plane pair, so the
//     arithmetic runs as Blackwell's packed f32x2 FMA / MUL / ADD and every
//     shared-memory read of a stencil point is one 8-byte load that serves
//     both planes;
//   - the plane pair plus a 3-cell x/y halo is staged in shared memory
//     (double buffered, halo prefetched one pair ahead);
//   - the squared regularised smoothness indicators q = (1e-6 + beta)^2 are
//     computed once per cell and axis (shared memory for x and y, registers
//     for z) and read by the faces;
//   - WENO is evaluated per FACE: each face value is computed once and read by
//     the two cells that share it, for both upwind directions -- the
//     left-biased reconstruction of weno5_left (weno5.h:39-58) and the
//     right-biased one of weno5_right (weno5.h:60-81), whose candidate
//     polynomials share two of three terms -- so no cell branches on its
//     upwind direction before the final selection.
//
// Face between cells f-1 and f, samples g_m = G[f-3+m], m = 0..5:
//   L(f-1) = (w0 Pa + w1 Pb + w2 Pc) / (w0 + w1 + w2),
//            w = (0.1 q(f-1) q(f), 0.6 q(f-2) q(f), 0.3 q(f-2) q(f-1))
//   R(f)   = (v0 Pa' + v1 Pc + v2 Pb) / (v0 + v1 + v2),
//            v = (0.3 q(f-1) q(f), 0.6 q(f+1) q(f-1), 0.1 q(f+1) q(f))
//   Pa = (2g0-7g1+11g2)/6, Pb = (-g1+5g2+2g3)/6, Pc = (2g2+5g3-g4)/6,
//   Pa' = (11g3-7g4+2g5)/6.
// (d_k / q_k weights multiplied through by q0 q1 q2; one approximate
// reciprocal per value.)  Cell i takes (L(i) - L(i-1)) / h if u_eff >= 0 and
// (R(i+1) - R(i)) / h otherwise.  In the code the indicators carry a factor
// 144 and the weights a factor 10 (both cancel in the ratios), and the face
// values a factor 6 that the derivative's 1/(6h) removes.
#include "common.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstring>
#include <mutex>

namespace lsgb {
namespace {

constexpr int TX = 32;
constexpr int TY = 8;
constexpr int NT = TX * TY;
constexpr int MAXZC = 64;       // longest z chunk a CTA marches (planes, even)
constexpr int PW = TX + 6;      // staged plane tile
constexpr int PH = TY + 6;
constexpr int QXW = TX + 4;     // x-indicators for tile x in [-2, TX+1]
constexpr int QYH = TY + 4;     // y-indicators for tile y in [-2, TY+1]
constexpr int NQX = QXW * TY;
constexpr int NQY = TX * QYH;
constexpr int NFX = (TX + 1) * TY;
constexpr int NFY = TX * (TY + 1);
constexpr int RING = PW * PH - TX * TY;
constexpr int RPT = (RING + NT - 1) / NT;
constexpr int NQ = NQX + NQY;
constexpr int NF = NFX + NFY;
constexpr int MINB = 3;         // resident CTAs per SM the register budget targets
constexpr int NSTAGE = 3;                // TMA pipeline depth (plane pairs in flight)
constexpr int NFIELD = 5;                // u, v, w, G^n, S_L
constexpr int FTILE = 2 * TY * TX;       // floats of one field tile (2 planes)
constexpr long long WAIT_CYCLES = 2000000000LL;  // bounded mbarrier wait (~1 s of SM clock)

struct TmaMaps {
    CUtensorMap m[NFIELD];
};

struct Coef {
    float inv_dx, inv_dy, inv_dz, inv_2dx, inv_2dy, inv_2dz, s_l, eps, dt;
    int zc;  // z-chunk length (even, <= MAXZC): tile shape chosen per grid by the autotuner
};

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

// Coordinate map for tile loads: any offset (ragged tiles reach past n).
__device__ __forceinline__ int wrapg(int x, int n, int bc) {
    if (bc == LSGB_BC_PERIODIC) {
        x %= n;
        return x < 0 ? x + n : x;
    }
    return x < 0 ? 0 : (x >= n ? n - 1 : x);
}


// ---- TMA / mbarrier primitives (PTX) ----------------------------------------
__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* b, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(saddr(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Poll with a limit: returns false if the phase did not complete within
// WAIT_CYCLES SM clocks (about a second).
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity) {
    if (mbar_test(b, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_test(b, parity))
        if (clock64() - t0 > WAIT_CYCLES) return false;
    return true;
}
__device__ __forceinline__ void tma_load_3d(float* dst, const CUtensorMap* tm, int x, int y, int z, uint64_t* b) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(saddr(dst)), "l"(tm), "r"(x), "r"(y), "r"(z), "r"(saddr(b))
        : "memory");
}

// IDX: element offsets (int when the field has < 2^31 cells).  TMA: stream
// u, v, w, G^n and S_L through a NSTAGE-deep pipeline of bulk tensor copies
// (one thread issues, mbarriers signal arrival); otherwise plain loads.
template <int STAGE, bool TMA, typename IDX>
__global__ void __launch_bounds__(NT, MINB)
stage3d_f32_pair(Geo g, const float* __restrict__ Gin, const float* __restrict__ Gn,
                 float* __restrict__ Gout, const float* __restrict__ u, const float* __restrict__ v,
                 const float* __restrict__ w, const float* __restrict__ sl, Coef c,
                 const __grid_constant__ TmaMaps tm, int* __restrict__ err) {
    __shared__ float2 P2[2][PH][PW];
    __shared__ float2 QA[NQ];          // x-indicators [TY][QXW], then y-indicators [QYH][TX]
    __shared__ float2 FL[NF], FR[NF];  // x-faces [TY][TX+1], then y-faces [TY+1][TX]
    __shared__ IDX zoff[MAXZC + 10];
    __shared__ __align__(8) uint64_t mbar[NSTAGE];
    extern __shared__ __align__(128) float stg[];  // NSTAGE x NFIELD x FTILE (TMA only)

    const int tx = threadIdx.x, ty = threadIdx.y;
    const int t = ty * TX + tx;
    const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
    const int z0 = blockIdx.z * c.zc;
    const int z1 = min(z0 + c.zc, g.nz);
    const int niter = (z1 - z0 + 1) / 2;
    const IDX sz = (IDX)g.nx * g.ny;
    const bool valid = (i0 + tx) < g.nx && (j0 + ty) < g.ny;
    const IDX col = (IDX)wrapg(j0 + ty, g.ny, g.bcy) * g.nx + wrapg(i0 + tx, g.nx, g.bcx);
    const bool has_sl = sl != nullptr;

    // ---- fixed per-thread task tables (offsets into one staged plane) ----
    // halo ring of the staged plane pair: 3 full rows above and below, 3 cells
    // left and right of each tile row
    int ring_s[RPT];
    IDX ring_g[RPT];
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
        const int q = t + r * NT;
        int ly, lx;
        if (q < 3 * PW) {
            ly = q / PW; lx = q % PW;
        } else if (q < 6 * PW) {
            ly = PH - 3 + (q - 3 * PW) / PW; lx = (q - 3 * PW) % PW;
        } else {
            const int s = (q - 6 * PW) % 6;
            ly = 3 + (q - 6 * PW) / 6;
            lx = s < 3 ? s : TX + s;
        }
        ring_s[r] = q < RING ? ly * PW + lx : -1;
        ring_g[r] = q < RING ? (IDX)wrapg(j0 + ly - 3, g.ny, g.bcy) * g.nx + wrapg(i0 + lx - 3, g.nx, g.bcx) : 0;
    }
    // Indicator and face tasks, x and y in separate lists with compile-time
    // strides.  Every thread has one task of each kind (slot A, index t);
    // the remainder goes to whole warps (slot B): x-indicators 256..287 to
    // threads 224..255, y-indicators 256..383 to threads 0..127, x-faces
    // 256..263 to threads 248..255, y-faces 256..287 to threads 128..159, so
    // no warp carries more than 3 + 3 tasks.  Offsets in float2 elements of
    // one staged plane (P) and of the indicator array (QA).
    //   x-indicator q: row q / QXW, column q % QXW -> P[row+3][cx..cx+2]
    //   y-indicator q: cy = q / TX, cl = q % TX     -> P[cy..cy+2][cl+3]
    //   x-face f: row f / (TX+1), fc = f % (TX+1)  -> P[row+3][fc..fc+5], QA[row][fc..fc+3]
    //   y-face f: rr = f / TX, cl = f % TX          -> P[rr..rr+5][cl+3], QY[rr..rr+3][cl]
    const int xi_a = (t / QXW + 3) * PW + t % QXW;
    const bool has_xi_b = t >= NT - (NQX - NT);
    const int xi_b = ((t + NQX - NT) / QXW + 3) * PW + (t + NQX - NT) % QXW;
    const int yi_a = ty * PW + tx + 3;
    const bool has_yi_b = t < NQY - NT;
    const int yi_b = (ty + NT / TX) * PW + tx + 3;
    const int fx_a_src = (t / (TX + 1) + 3) * PW + t % (TX + 1);
    const int fx_a_q = (t / (TX + 1)) * QXW + t % (TX + 1);
    const bool has_fx_b = t >= NT - (NFX - NT);
    const int fxb = t + NFX - NT;  // face index of slot B
    const int fx_b_src = (fxb / (TX + 1) + 3) * PW + fxb % (TX + 1);
    const int fx_b_q = (fxb / (TX + 1)) * QXW + fxb % (TX + 1);
    const bool has_fy_b = t >= NT / 2 && t < NT / 2 + (NFY - NT);
    // y-face slot A = face (ty, tx): P[ty..ty+5][tx+3], QY[ty..ty+3][tx]
    // y-face slot B = face (TY, tx)
    // plane offsets of z-indices z0-3 .. z1+6 (periodic wrap or clamp), one
    // table per CTA so the loop does no index arithmetic on z
    for (int d = t; d < c.zc + 10; d += NT) {
        int kk = z0 - 3 + d;
        if (g.bcz == LSGB_BC_PERIODIC) {
            while (kk < 0) kk += g.nz;
            while (kk >= g.nz) kk -= g.nz;
        } else {
            kk = kk < 0 ? 0 : (kk >= g.nz ? g.nz - 1 : kk);
        }
        zoff[d] = (IDX)kk * sz;
    }

    // ---- TMA pipeline prologue ----
    auto issue = [&](int it, int s) {
        const int kz = z0 + 2 * it;
        float* base = stg + s * NFIELD * FTILE;
        const uint32_t nf = 3 + (STAGE > 1 ? 1 : 0) + (has_sl ? 1 : 0);
        mbar_expect_tx(&mbar[s], nf * FTILE * 4);
        tma_load_3d(base + 0 * FTILE, &tm.m[0], i0, j0, kz, &mbar[s]);
        tma_load_3d(base + 1 * FTILE, &tm.m[1], i0, j0, kz, &mbar[s]);
        tma_load_3d(base + 2 * FTILE, &tm.m[2], i0, j0, kz, &mbar[s]);
        if (STAGE > 1) tma_load_3d(base + 3 * FTILE, &tm.m[3], i0, j0, kz, &mbar[s]);
        if (has_sl) tma_load_3d(base + 4 * FTILE, &tm.m[4], i0, j0, kz, &mbar[s]);
    };
    if (TMA && t == 0) {
        for (int s = 0; s < NSTAGE; ++s) mbar_init(&mbar[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();  // zoff table and barriers ready
    if (TMA && t == 0)
        for (int it = 0; it < NSTAGE - 1 && it < niter; ++it) issue(it, it);

    // ---- z queues: G(k-3 .. k+4) and q_z(k-1 .. k+1) of the own column ----
    float zq[8];
#pragma unroll
    for (int d = 0; d < 8; ++d) zq[d] = __ldg(Gin + zoff[d] + col);
    float2 qz_a = qbeta(make_float2(zq[1], zq[2]), make_float2(zq[2], zq[3]), make_float2(zq[3], zq[4]));  // (q(k-1), q(k))
    float qz_k1 = qbeta(make_float2(zq[3], zq[3]), make_float2(zq[4], zq[4]), make_float2(zq[5], zq[5])).x;  // q(k+1)
    const float qz_m2 = qbeta(make_float2(zq[0], zq[0]), make_float2(zq[1], zq[1]), make_float2(zq[2], zq[2])).x;  // q(k-2)
    // face k-1/2 (between k-1 and k): samples G(k-3..k+2), q(k-2), q(k-1), q(k), q(k+1)
    float zprevL, zprevR;
    {
        float2 L, R;
        face(c2(zq[0]), c2(zq[1]), c2(zq[2]), c2(zq[3]), c2(zq[4]), c2(zq[5]), c2(qz_m2), c2(qz_a.x),
             c2(qz_a.y), c2(qz_k1), L, R);
        zprevL = L.x;
        zprevR = R.x;
    }
    float2 ring_v[RPT];
#pragma unroll
    for (int r = 0; r < RPT; ++r)
        ring_v[r] = ring_s[r] >= 0 ? make_float2(__ldg(Gin + zoff[3] + ring_g[r]), __ldg(Gin + zoff[4] + ring_g[r]))
                                   : make_float2(0.0f, 0.0f);

    int buf = 0;
    int cs = 0;         // TMA stage of this iteration (it % NSTAGE)
    uint32_t cph = 0;   // its mbarrier phase parity ((it / NSTAGE) & 1)
    for (int it = 0; it < niter; ++it) {
        const int k = z0 + 2 * it;
        const IDX* zo = zoff + 2 * it + 3;  // zo[d] = offset of plane k + d
        float2* P = &P2[buf][0][0];
        P[(ty + 3) * PW + tx + 3] = make_float2(zq[3], zq[4]);
#pragma unroll
        for (int r = 0; r < RPT; ++r)
            if (ring_s[r] >= 0) P[ring_s[r]] = ring_v[r];

        // loads for this pair's update (plain path) and the next pair's staging
        const IDX oa = zo[0] + col;
        const IDX ob = zo[1] + col;
        float2 uu, vv, ww, gn = c2(0.0f), s_l = c2(c.s_l);
        if (!TMA) {
            uu = make_float2(__ldg(u + oa), __ldg(u + ob));
            vv = make_float2(__ldg(v + oa), __ldg(v + ob));
            ww = make_float2(__ldg(w + oa), __ldg(w + ob));
            if (STAGE > 1) gn = make_float2(__ldg(Gn + oa), __ldg(Gn + ob));
            if (has_sl) s_l = make_float2(__ldg(sl + oa), __ldg(sl + ob));
        }
        const float zn0 = __ldg(Gin + zo[5] + col);
        const float zn1 = __ldg(Gin + zo[6] + col);
        if (it + 1 < niter) {
            const IDX na = zo[2], nb = zo[3];
#pragma unroll
            for (int r = 0; r < RPT; ++r)
                if (ring_s[r] >= 0) ring_v[r] = make_float2(__ldg(Gin + na + ring_g[r]), __ldg(Gin + nb + ring_g[r]));
        }
        __syncthreads();
        if (TMA && t == 0 && it + NSTAGE - 1 < niter) {
            // the stage being refilled was last read in iteration it-1, which
            // every thread finished before the barrier above
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(it + NSTAGE - 1, cs == 0 ? NSTAGE - 1 : cs - 1);
        }

        // ---- per-cell indicators (x, y in shared memory; z in registers) ----
        QA[t] = qbeta(P[xi_a], P[xi_a + 1], P[xi_a + 2]);
        if (has_xi_b) QA[t + NQX - NT] = qbeta(P[xi_b], P[xi_b + 1], P[xi_b + 2]);
        QA[NQX + t] = qbeta(P[yi_a], P[yi_a + PW], P[yi_a + 2 * PW]);
        if (has_yi_b) QA[NQX + NT + t] = qbeta(P[yi_b], P[yi_b + PW], P[yi_b + 2 * PW]);
        // q_z(k+2), q_z(k+3): triples centred at k+2 and k+3
        const float2 qz_b = qbeta(make_float2(zq[4], zq[5]), make_float2(zq[5], zq[6]), make_float2(zq[6], zq[7]));
        if (TMA) {
            const bool ok = mbar_wait(&mbar[cs], cph);
            if (__syncthreads_or(!ok)) {
                // a bulk copy did not arrive in time: flag it, give the copies
                // still in flight a bounded chance to land, and leave
                if (t == 0) {
                    atomicExch(err, 1);
                    for (int j = it; j < niter && j < it + NSTAGE; ++j)
                        mbar_wait(&mbar[j % NSTAGE], (uint32_t)((j / NSTAGE) & 1));
                }
                return;
            }
        } else {
            __syncthreads();
        }

        // ---- faces ----
        {
            float2 L, R;
            const float2* sx = P + fx_a_src;
            const float2* qx = QA + fx_a_q;
            face(sx[0], sx[1], sx[2], sx[3], sx[4], sx[5], qx[0], qx[1], qx[2], qx[3], L, R);
            FL[t] = L;
            FR[t] = R;
            if (has_fx_b) {
                sx = P + fx_b_src;
                qx = QA + fx_b_q;
                face(sx[0], sx[1], sx[2], sx[3], sx[4], sx[5], qx[0], qx[1], qx[2], qx[3], L, R);
                FL[fxb] = L;
                FR[fxb] = R;
            }
            const float2* sy = P + yi_a;  // P[ty][tx+3]
            const float2* qy = QA + NQX + t;
            face(sy[0], sy[PW], sy[2 * PW], sy[3 * PW], sy[4 * PW], sy[5 * PW], qy[0], qy[TX], qy[2 * TX],
                 qy[3 * TX], L, R);
            FL[NFX + t] = L;
            FR[NFX + t] = R;
            if (has_fy_b) {
                // face row TY: P[TY..TY+5][tx+3], QY[TY..TY+3][tx]
                sy = P + TY * PW + tx + 3;
                qy = QA + NQX + TY * TX + tx;
                face(sy[0], sy[PW], sy[2 * PW], sy[3 * PW], sy[4 * PW], sy[5 * PW], qy[0], qy[TX], qy[2 * TX],
                     qy[3 * TX], L, R);
                FL[NFX + TY * TX + tx] = L;
                FR[NFX + TY * TX + tx] = R;
            }
        }
        // z faces k+1/2 and k+3/2 as one pair: samples G(k-2+m), G(k-1+m)
        float2 zL, zR;
        face(make_float2(zq[1], zq[2]), make_float2(zq[2], zq[3]), make_float2(zq[3], zq[4]),
             make_float2(zq[4], zq[5]), make_float2(zq[5], zq[6]), make_float2(zq[6], zq[7]),
             make_float2(qz_a.x, qz_a.y), make_float2(qz_a.y, qz_k1), make_float2(qz_k1, qz_b.x),
             qz_b, zL, zR);
        __syncthreads();

        // ---- cell update for planes k, k+1 ----
        if (TMA) {
            const float* sb = stg + cs * NFIELD * FTILE + ty * TX + tx;
            uu = make_float2(sb[0 * FTILE], sb[0 * FTILE + TX * TY]);
            vv = make_float2(sb[1 * FTILE], sb[1 * FTILE + TX * TY]);
            ww = make_float2(sb[2 * FTILE], sb[2 * FTILE + TX * TY]);
            if (STAGE > 1) gn = make_float2(sb[3 * FTILE], sb[3 * FTILE + TX * TY]);
            if (has_sl) s_l = make_float2(sb[4 * FTILE], sb[4 * FTILE + TX * TY]);
        }
        const float2* ctr = P + (ty + 3) * PW + tx + 3;
        const float2 gc = ctr[0];
        float2 ue = uu, ve = vv, we = ww;
        {
            const float2 gx = mul2(sub2(ctr[1], ctr[-1]), c2(c.inv_2dx));
            const float2 gy = mul2(sub2(ctr[PW], ctr[-PW]), c2(c.inv_2dy));
            const float2 gz = mul2(make_float2(zq[4] - zq[2], zq[5] - zq[3]), c2(c.inv_2dz));
            const float2 sq = fma2(gx, gx, fma2(gy, gy, fma2(gz, gz, c2(c.eps))));
            const float2 f = make_float2(s_l.x > c.eps ? -s_l.x * rsqrtf(sq.x) : 0.0f,
                                         s_l.y > c.eps ? -s_l.y * rsqrtf(sq.y) : 0.0f);
            ue = fma2(f, gx, ue);
            ve = fma2(f, gy, ve);
            we = fma2(f, gz, we);
        }
        const int xf = ty * (TX + 1) + tx, yfc = NFX + ty * TX + tx;
        const float2 dxL = sub2(FL[xf + 1], FL[xf]);
        const float2 dxR = sub2(FR[xf + 1], FR[xf]);
        const float2 dyL = sub2(FL[yfc + TX], FL[yfc]);
        const float2 dyR = sub2(FR[yfc + TX], FR[yfc]);
        // z: plane k uses faces (k-1/2, k+1/2) = (prev, zL.x); plane k+1 (zL.x, zL.y)
        const float2 dzL = sub2(zL, make_float2(zprevL, zL.x));
        const float2 dzR = sub2(zR, make_float2(zprevR, zR.x));
        const float2 dgx = mul2(make_float2(ue.x >= 0.0f ? dxL.x : dxR.x, ue.y >= 0.0f ? dxL.y : dxR.y), c2(c.inv_dx));
        const float2 dgy = mul2(make_float2(ve.x >= 0.0f ? dyL.x : dyR.x, ve.y >= 0.0f ? dyL.y : dyR.y), c2(c.inv_dy));
        const float2 dgz = mul2(make_float2(we.x >= 0.0f ? dzL.x : dzR.x, we.y >= 0.0f ? dzL.y : dzR.y), c2(c.inv_dz));
        const float2 nrhs = fma2(ue, dgx, fma2(ve, dgy, mul2(we, dgz)));  // = -rhs
        float2 out;
        if (STAGE == 1) out = fma2(c2(-c.dt), nrhs, gc);
        else if (STAGE == 2) out = fma2(c2(-0.25f * c.dt), nrhs, fma2(c2(0.75f), gn, mul2(c2(0.25f), gc)));
        else out = fma2(c2(-(2.0f / 3.0f) * c.dt), nrhs, fma2(c2(1.0f / 3.0f), gn, mul2(c2(2.0f / 3.0f), gc)));
        if (valid) {
            Gout[oa] = out.x;
            if (k + 1 < z1) Gout[oa + sz] = out.y;
        }

        // ---- advance the z queues by two planes ----
#pragma unroll
        for (int d = 0; d < 6; ++d) zq[d] = zq[d + 2];
        zq[6] = zn0;
        zq[7] = zn1;
        qz_a = make_float2(qz_k1, qz_b.x);   // (q(k+1), q(k+2)) -> new (q(k'-1), q(k'))
        qz_k1 = qz_b.y;                      // q(k+3) -> new q(k'+1)
        zprevL = zL.y;
        zprevR = zR.y;
        buf ^= 1;
        if (++cs == NSTAGE) {
            cs = 0;
            cph ^= 1u;
        }
    }
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no -lcuda).
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    });
    return fn;
}

// 3D map over a compact FP32 field with a (32, 8, 2) box; zero fill outside.
bool encode_field(CUtensorMap* m, const float* ptr, const Geo& g) {
    PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
    if (!fn || !ptr) return false;
    cuuint64_t dims[3] = {(cuuint64_t)g.nx, (cuuint64_t)g.ny, (cuuint64_t)g.nz};
    cuuint64_t strides[2] = {(cuuint64_t)g.nx * 4, (cuuint64_t)g.nx * g.ny * 4};
    cuuint32_t box[3] = {TX, TY, 2};
    cuuint32_t estr[3] = {1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void*)ptr, dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int STAGE, bool TMA, typename IDX>
cudaError_t launch_one(const StageArgs& a, const Coef& c, const TmaMaps& tm, int* err, cudaStream_t st) {
    const dim3 block(TX, TY, 1);
    const dim3 grid((a.g.nx + TX - 1) / TX, (a.g.ny + TY - 1) / TY, (a.g.nz + c.zc - 1) / c.zc);
    const size_t dyn = TMA ? (size_t)NSTAGE * NFIELD * FTILE * sizeof(float) : 0;
    auto kern = stage3d_f32_pair<STAGE, TMA, IDX>;
    if (TMA) {
        static bool attr_set = false;  // per instantiation
        if (!attr_set) {
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
            if (e != cudaSuccess) return e;
            attr_set = true;
        }
    }
    kern<<<grid, block, dyn, st>>>(a.g, (const float*)a.Gin, (const float*)a.Gn, (float*)a.Gout,
                                    (const float*)a.u, (const float*)a.v, (const float*)a.w,
                                    (const float*)a.sl, c, tm, err);
    return cudaGetLastError();
}

template <bool TMA, typename IDX>
cudaError_t launch_stage(const StageArgs& a, const Coef& c, const TmaMaps& tm, int* err, cudaStream_t st) {
    if (a.stage == 1) return launch_one<1, TMA, IDX>(a, c, tm, err, st);
    if (a.stage == 2) return launch_one<2, TMA, IDX>(a, c, tm, err, st);
    return launch_one<3, TMA, IDX>(a, c, tm, err, st);
}

}  // namespace

cudaError_t launch_stage3d_f32_tiled(const StageArgs& a, int* err, cudaStream_t st) {
    Coef c;
    // face values carry a factor 6 (see face())
    c.inv_dx = (float)(1.0 / (6.0 * a.dx));
    c.inv_dy = (float)(1.0 / (6.0 * a.dy));
    c.inv_dz = (float)(1.0 / (6.0 * a.dz));
    c.inv_2dx = (float)(1.0 / (2.0 * a.dx));
    c.inv_2dy = (float)(1.0 / (2.0 * a.dy));
    c.inv_2dz = (float)(1.0 / (2.0 * a.dz));
    c.s_l = (float)a.s_l;
    c.eps = (float)a.eps;
    c.dt = (float)a.dt;
    c.zc = (a.tile == 16 || a.tile == 32) ? a.tile : MAXZC;
    TmaMaps tm;
    std::memset(&tm, 0, sizeof(tm));
    // bulk tensor copies need 16-byte row pitch and an error flag to report into
    bool tma = err != nullptr && (a.g.nx % 4) == 0;
    const void* fields[NFIELD] = {a.u, a.v, a.w, a.stage > 1 ? a.Gn : nullptr, a.sl};
    for (int f = 0; f < NFIELD && tma; ++f)
        if (fields[f] && !encode_field(&tm.m[f], (const float*)fields[f], a.g)) tma = false;
    const bool small = a.g.cells() < (1LL << 31) - 1;
    cudaError_t e;
    if (tma) e = small ? launch_stage<true, int>(a, c, tm, err, st) : launch_stage<true, long long>(a, c, tm, err, st);
    else e = small ? launch_stage<false, int>(a, c, tm, err, st) : launch_stage<false, long long>(a, c, tm, err, st);
    count_launches(1);
    return e;
}

}  // namespace lsgb
