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
// (R(i+1) - R(i)) / h otherwise.
#include "common.cuh"

namespace lsgb {
namespace {

constexpr int TX = 32;
constexpr int TY = 8;
constexpr int NT = TX * TY;
constexpr int ZC = 64;          // planes per CTA (even)
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
constexpr int QXPT = (NQX + NT - 1) / NT;
constexpr int QYPT = (NQY + NT - 1) / NT;
constexpr int FXPT = (NFX + NT - 1) / NT;
constexpr int FYPT = (NFY + NT - 1) / NT;

struct Coef {
    float inv_dx, inv_dy, inv_dz, inv_2dx, inv_2dy, inv_2dz, s_l, eps, dt;
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

// (1e-6 + beta)^2 of the triple (a, b, c); beta as computeSmoothnessIndicators
// (weno5.h:28-37): 13/12 (a - 2b + c)^2 + 1/4 (c - a)^2.
__device__ __forceinline__ float2 qbeta(float2 a, float2 b, float2 c) {
    const float2 t = add2(fma2(c2(-2.0f), b, a), c);
    const float2 r = sub2(c, a);
    const float2 B = fma2(mul2(c2(13.0f / 12.0f), t), t, mul2(mul2(c2(0.25f), r), r));
    const float2 s = add2(B, c2(1.0e-6f));
    return mul2(s, s);
}

// Both reconstructions at the face between cells f-1 and f.
__device__ __forceinline__ void face(float2 g0, float2 g1, float2 g2, float2 g3, float2 g4, float2 g5,
                                     float2 qm2, float2 qm1, float2 q0, float2 qp1, float2& L, float2& R) {
    const float2 Pa = fma2(c2(1.0f / 3.0f), g0, fma2(c2(-7.0f / 6.0f), g1, mul2(c2(11.0f / 6.0f), g2)));
    const float2 Pb = fma2(c2(-1.0f / 6.0f), g1, fma2(c2(5.0f / 6.0f), g2, mul2(c2(1.0f / 3.0f), g3)));
    const float2 Pc = fma2(c2(1.0f / 3.0f), g2, fma2(c2(5.0f / 6.0f), g3, mul2(c2(-1.0f / 6.0f), g4)));
    const float2 Pr = fma2(c2(11.0f / 6.0f), g3, fma2(c2(-7.0f / 6.0f), g4, mul2(c2(1.0f / 3.0f), g5)));
    const float2 q12 = mul2(qm1, q0);
    const float2 lw0 = mul2(c2(0.1f), q12);
    const float2 lw1 = mul2(c2(0.6f), mul2(qm2, q0));
    const float2 lw2 = mul2(c2(0.3f), mul2(qm2, qm1));
    const float2 rw0 = mul2(c2(0.3f), q12);
    const float2 rw1 = mul2(c2(0.6f), mul2(qp1, qm1));
    const float2 rw2 = mul2(c2(0.1f), mul2(qp1, q0));
    L = div2(fma2(lw0, Pa, fma2(lw1, Pb, mul2(lw2, Pc))), add2(add2(lw0, lw1), lw2));
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

template <int STAGE>
__global__ void __launch_bounds__(NT, 2)
stage3d_f32_pair(Geo g, const float* __restrict__ Gin, const float* __restrict__ Gn,
                 float* __restrict__ Gout, const float* __restrict__ u, const float* __restrict__ v,
                 const float* __restrict__ w, const float* __restrict__ sl, Coef c) {
    __shared__ float2 P2[2][PH][PW];
    __shared__ float2 QX[TY][QXW];
    __shared__ float2 QY[QYH][TX];
    __shared__ float2 FXL[TY][TX + 1], FXR[TY][TX + 1];
    __shared__ float2 FYL[TY + 1][TX], FYR[TY + 1][TX];

    const int tx = threadIdx.x, ty = threadIdx.y;
    const int t = ty * TX + tx;
    const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
    const int z0 = blockIdx.z * ZC;
    const int z1 = min(z0 + ZC, g.nz);
    const long long sz = (long long)g.nx * g.ny;
    const bool valid = (i0 + tx) < g.nx && (j0 + ty) < g.ny;
    const int col = wrapg(j0 + ty, g.ny, g.bcy) * g.nx + wrapg(i0 + tx, g.nx, g.bcx);

    // ---- fixed per-thread task tables (offsets into one staged plane) ----
    int ring_s[RPT], ring_g[RPT];
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
        ring_g[r] = q < RING ? wrapg(j0 + ly - 3, g.ny, g.bcy) * g.nx + wrapg(i0 + lx - 3, g.nx, g.bcx) : 0;
    }
    int qx_src[QXPT], qy_src[QYPT], fx_src[FXPT], fy_src[FYPT];
#pragma unroll
    for (int r = 0; r < QXPT; ++r) {  // x-indicator of tile cell (cx-2, row): samples P2[row+3][cx..cx+2]
        const int q = t + r * NT, row = q / QXW, cx = q % QXW;
        qx_src[r] = q < NQX ? (row + 3) * PW + cx : -1;
    }
#pragma unroll
    for (int r = 0; r < QYPT; ++r) {  // y-indicator of tile cell (col, cy-2): samples P2[cy..cy+2][col+3]
        const int q = t + r * NT, cy = q / TX, cl = q % TX;
        qy_src[r] = q < NQY ? cy * PW + cl + 3 : -1;
    }
#pragma unroll
    for (int r = 0; r < FXPT; ++r) {  // x-face f in row: samples P2[row+3][f..f+5], QX[row][f..f+3]
        const int q = t + r * NT, row = q / (TX + 1), f = q % (TX + 1);
        fx_src[r] = q < NFX ? row * 65536 + f : -1;
    }
#pragma unroll
    for (int r = 0; r < FYPT; ++r) {  // y-face between rows rr-1, rr: P2[rr..rr+5][cl+3], QY[rr..rr+3][cl]
        const int q = t + r * NT, rr = q / TX, cl = q % TX;
        fy_src[r] = q < NFY ? rr * 65536 + cl : -1;
    }

    // plane offset of z-index k, k in [z0 - 3, z1 + 6): the wrap needs no
    // integer division (one conditional add / subtract per chunk edge)
    auto plane = [&](int k) -> long long {
        int kk = k;
        if (g.bcz == LSGB_BC_PERIODIC) {
            while (kk < 0) kk += g.nz;
            while (kk >= g.nz) kk -= g.nz;
        } else {
            kk = kk < 0 ? 0 : (kk >= g.nz ? g.nz - 1 : kk);
        }
        return (long long)kk * sz;
    };

    // ---- z queues: G(k-3 .. k+4) and q_z(k-1 .. k+1) of the own column ----
    float zq[8];
#pragma unroll
    for (int d = 0; d < 8; ++d) zq[d] = __ldg(Gin + plane(z0 - 3 + d) + col);
    // indicators at k-1, k, k+1 (triples centred there)
    float2 qz_a = qbeta(make_float2(zq[1], zq[2]), make_float2(zq[2], zq[3]), make_float2(zq[3], zq[4]));  // (q(k-1), q(k))
    float qz_k1 = qbeta(make_float2(zq[3], zq[3]), make_float2(zq[4], zq[4]), make_float2(zq[5], zq[5])).x;  // q(k+1)
    float qz_m2 = qbeta(make_float2(zq[0], zq[0]), make_float2(zq[1], zq[1]), make_float2(zq[2], zq[2])).x;  // q(k-2)
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
    {
        const long long pa = plane(z0), pb = plane(z0 + 1);
#pragma unroll
        for (int r = 0; r < RPT; ++r)
            ring_v[r] = ring_s[r] >= 0 ? make_float2(__ldg(Gin + pa + ring_g[r]), __ldg(Gin + pb + ring_g[r]))
                                       : make_float2(0.0f, 0.0f);
    }

    int buf = 0;
    for (int k = z0; k < z1; k += 2) {
        float2* P = &P2[buf][0][0];
        P[(ty + 3) * PW + tx + 3] = make_float2(zq[3], zq[4]);
#pragma unroll
        for (int r = 0; r < RPT; ++r)
            if (ring_s[r] >= 0) P[ring_s[r]] = ring_v[r];

        // loads for this pair's update and the next pair's staging
        const long long oa = (long long)k * sz + col;
        const long long ob = plane(k + 1) + col;
        const float2 uu = make_float2(__ldg(u + oa), __ldg(u + ob));
        const float2 vv = make_float2(__ldg(v + oa), __ldg(v + ob));
        const float2 ww = make_float2(__ldg(w + oa), __ldg(w + ob));
        float2 gn = c2(0.0f);
        if (STAGE > 1) gn = make_float2(__ldg(Gn + oa), __ldg(Gn + ob));
        float2 s_l = c2(c.s_l);
        if (sl) s_l = make_float2(__ldg(sl + oa), __ldg(sl + ob));
        const float zn0 = __ldg(Gin + plane(k + 5) + col);
        const float zn1 = __ldg(Gin + plane(k + 6) + col);
        if (k + 2 < z1) {
            const long long na = plane(k + 2), nb = plane(k + 3);
#pragma unroll
            for (int r = 0; r < RPT; ++r)
                if (ring_s[r] >= 0) ring_v[r] = make_float2(__ldg(Gin + na + ring_g[r]), __ldg(Gin + nb + ring_g[r]));
        }
        __syncthreads();

        // ---- per-cell indicators (x, y in shared memory; z in registers) ----
#pragma unroll
        for (int r = 0; r < QXPT; ++r)
            if (qx_src[r] >= 0) {
                const float2* s = P + qx_src[r];
                (&QX[0][0])[t + r * NT] = qbeta(s[0], s[1], s[2]);
            }
#pragma unroll
        for (int r = 0; r < QYPT; ++r)
            if (qy_src[r] >= 0) {
                const float2* s = P + qy_src[r];
                (&QY[0][0])[t + r * NT] = qbeta(s[0], s[PW], s[2 * PW]);
            }
        // q_z(k+2), q_z(k+3): triples centred at k+2 and k+3
        const float2 qz_b = qbeta(make_float2(zq[4], zq[5]), make_float2(zq[5], zq[6]), make_float2(zq[6], zq[7]));
        __syncthreads();

        // ---- faces ----
#pragma unroll
        for (int r = 0; r < FXPT; ++r)
            if (fx_src[r] >= 0) {
                const int row = fx_src[r] >> 16, f = fx_src[r] & 0xffff;
                const float2* s = P + (row + 3) * PW + f;
                const float2* q = &QX[row][f];
                float2 L, R;
                face(s[0], s[1], s[2], s[3], s[4], s[5], q[0], q[1], q[2], q[3], L, R);
                FXL[row][f] = L;
                FXR[row][f] = R;
            }
#pragma unroll
        for (int r = 0; r < FYPT; ++r)
            if (fy_src[r] >= 0) {
                const int rr = fy_src[r] >> 16, cl = fy_src[r] & 0xffff;
                const float2* s = P + rr * PW + cl + 3;
                const float2* q = &QY[rr][cl];
                float2 L, R;
                face(s[0], s[PW], s[2 * PW], s[3 * PW], s[4 * PW], s[5 * PW], q[0], q[TX], q[2 * TX],
                     q[3 * TX], L, R);
                FYL[rr][cl] = L;
                FYR[rr][cl] = R;
            }
        // z faces k+1/2 and k+3/2 as one pair: samples G(k-2+m), G(k-1+m)
        float2 zL, zR;
        face(make_float2(zq[1], zq[2]), make_float2(zq[2], zq[3]), make_float2(zq[3], zq[4]),
             make_float2(zq[4], zq[5]), make_float2(zq[5], zq[6]), make_float2(zq[6], zq[7]),
             make_float2(qz_a.x, qz_a.y), make_float2(qz_a.y, qz_k1), make_float2(qz_k1, qz_b.x),
             qz_b, zL, zR);
        __syncthreads();

        // ---- cell update for planes k, k+1 ----
        const float2* ctr = P + (ty + 3) * PW + tx + 3;
        const float2 gc = ctr[0];
        float2 ue = uu, ve = vv, we = ww;
        {
            const float2 gx = mul2(sub2(ctr[1], ctr[-1]), c2(c.inv_2dx));
            const float2 gy = mul2(sub2(ctr[PW], ctr[-PW]), c2(c.inv_2dy));
            const float2 gz = mul2(make_float2(zq[4] - zq[2], zq[5] - zq[3]), c2(c.inv_2dz));
            const float2 sq = fma2(gx, gx, fma2(gy, gy, fma2(gz, gz, c2(c.eps))));
            const float2 f = make_float2(s_l.x > c.eps ? s_l.x * rsqrtf(sq.x) : 0.0f,
                                         s_l.y > c.eps ? s_l.y * rsqrtf(sq.y) : 0.0f);
            const float2 nf = mul2(f, c2(-1.0f));
            ue = fma2(nf, gx, ue);
            ve = fma2(nf, gy, ve);
            we = fma2(nf, gz, we);
        }
        const float2 dxL = sub2(FXL[ty][tx + 1], FXL[ty][tx]);
        const float2 dxR = sub2(FXR[ty][tx + 1], FXR[ty][tx]);
        const float2 dyL = sub2(FYL[ty + 1][tx], FYL[ty][tx]);
        const float2 dyR = sub2(FYR[ty + 1][tx], FYR[ty][tx]);
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
        qz_m2 = qz_a.y;                      // unused past the prologue; kept for clarity
        qz_a = make_float2(qz_k1, qz_b.x);   // (q(k+1), q(k+2)) -> new (q(k'-1), q(k'))
        qz_k1 = qz_b.y;                      // q(k+3) -> new q(k'+1)
        zprevL = zL.y;
        zprevR = zR.y;
        buf ^= 1;
    }
}

}  // namespace

cudaError_t launch_stage3d_f32_tiled(const StageArgs& a, cudaStream_t st) {
    Coef c;
    c.inv_dx = (float)(1.0 / a.dx);
    c.inv_dy = (float)(1.0 / a.dy);
    c.inv_dz = (float)(1.0 / a.dz);
    c.inv_2dx = (float)(1.0 / (2.0 * a.dx));
    c.inv_2dy = (float)(1.0 / (2.0 * a.dy));
    c.inv_2dz = (float)(1.0 / (2.0 * a.dz));
    c.s_l = (float)a.s_l;
    c.eps = (float)a.eps;
    c.dt = (float)a.dt;
    const dim3 block(TX, TY, 1);
    const dim3 grid((a.g.nx + TX - 1) / TX, (a.g.ny + TY - 1) / TY, (a.g.nz + ZC - 1) / ZC);
    const float* Gin = (const float*)a.Gin;
    const float* Gn = (const float*)a.Gn;
    float* Gout = (float*)a.Gout;
    const float* u = (const float*)a.u;
    const float* v = (const float*)a.v;
    const float* w = (const float*)a.w;
    const float* sl = (const float*)a.sl;
    if (a.stage == 1) stage3d_f32_pair<1><<<grid, block, 0, st>>>(a.g, Gin, Gn, Gout, u, v, w, sl, c);
    else if (a.stage == 2) stage3d_f32_pair<2><<<grid, block, 0, st>>>(a.g, Gin, Gn, Gout, u, v, w, sl, c);
    else stage3d_f32_pair<3><<<grid, block, 0, st>>>(a.g, Gin, Gn, Gout, u, v, w, sl, c);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace lsgb
