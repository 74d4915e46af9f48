// stage3d_f32.cu -- the FP32-bulk 3D RK3 stage kernel (the throughput path).
//
// One launch = one TVD-RK3 stage over the whole grid, fused: the u_eff WENO-5
// right-hand side of computeRHS3D (Local_code/level-set_MPI_3D/include/
// rk3.h:31-81, weno5.h:28-196) and the stage combination of rk3Stage{1,2,3}_3D
// (rk3.h:87-121).  Compact arrays, periodic / zero-gradient neighbours by
// index mapping (no ghost cells, no boundary pass).
//
// Shape (2.5D blocking, register-blocked in y and z):
//   - a CTA of 32 x 8 threads owns a 32 x 16 column tile and marches a chunk
//     of up to 64 z-planes two at a time; thread (x, ty) owns the cells of
//     rows 2 ty and 2 ty + 1 in planes k and k + 1 (four cells);
//   - every per-cell quantity is a float2 over the plane pair, so the
//     arithmetic runs as Blackwell's packed f32x2 FMA / MUL / ADD;
//   - z: each thread keeps the G values of its two columns in register queues
//     (G(k-3 .. k+4)), with the z indicators and the last z face carried;
//   - y: each thread reads an 8-row window of the staged plane pair into
//     registers and evaluates its rows' y faces there;
//   - x: the only direction that goes through shared memory -- the plane
//     pair plus a 3-cell halo is staged (double buffered, halo prefetched one
//     pair ahead), every x face is computed once by one lane and stored, and
//     its indicators are shared across the warp by shuffles;
//   - u, v, w, G^n and S_L stream through a 3-deep pipeline of TMA bulk
//     tensor copies (one thread issues, mbarriers with bounded waits signal
//     arrival), or per-thread cp.async copies where a field's row pitch is
//     not 16-byte aligned.
// Two barriers per plane pair.  The kernel is bound by the FP32 pipe (packed
// f32x2 instructions occupy it for two cycles), not by HBM or shared memory.
//
// WENO is evaluated per FACE: each face value is computed once and read by
// the two cells that share it, for both upwind directions -- the
// left-biased reconstruction of weno5_left (weno5.h:39-58) and the
// right-biased one of weno5_right (weno5.h:60-81), whose candidate
// polynomials share two of three terms -- so no cell branches on its upwind
// direction before the final selection.
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
#include "weno_f32x2.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstring>
#include <mutex>

namespace lsgb {
namespace {

using namespace wf;

constexpr int TX = 32;                        // tile columns (one warp's lanes)
constexpr int TY = 8;                         // thread rows of a CTA
constexpr int NT = TX * TY;
constexpr int RY = 2;                         // cell rows per thread
constexpr int BY = TY * RY;                   // tile rows
constexpr int MAXZC = 64;                     // longest z chunk a CTA marches (planes, even)
constexpr int PW = TX + 6;                    // staged plane tile: columns
constexpr int BPH = BY + 6;                   //                    rows
constexpr int BRING = PW * BPH - TX * BY;     // halo ring of one staged plane
constexpr int BRPT = (BRING + NT - 1) / NT;   // ring cells per thread
constexpr int BNFX = (TX + 1) * BY;           // x faces of the tile
constexpr int NSTAGE = 3;                     // TMA pipeline depth (plane pairs in flight)
constexpr int NFIELD = 5;                     // u, v, w, G^n, S_L
constexpr int BFTILE = 2 * BY * TX;           // floats of one staged field tile (2 planes)
// bounded mbarrier wait: about 1 s at the full SM clock.  The limit counts SM
// clock cycles, not wall time, so on a GPU time-sliced between processes a
// slow but healthy copy can run into it.
constexpr long long WAIT_CYCLES = 2000000000LL;

struct TmaMaps {
    CUtensorMap m[NFIELD];
};

struct Coef {
    float inv_dx, inv_dy, inv_dz, inv_2dx, inv_2dy, inv_2dz, s_l, eps, dt;
    int zc;  // z-chunk length (even, <= MAXZC): tile shape chosen per grid by the autotuner
    int drop;  // test hook: issue no bulk copies, so every wait runs into its limit
    float tf;  // deformation vortex time factor cos(pi t / T) (DEFO kernels)
};

// One instance of a grouped launch (stage3d_f32_group): its fields, stage
// coefficients, tile grid (gx x gy column tiles, z-chunks of c.zc planes)
// and its first block in the launch.
struct Group3 {
    CUtensorMap m[NFIELD];  // u, v, w, G^n (= G), S_L; bulk-tensor staging where tma != 0
    Geo g;
    float *G, *A, *B;
    const float *u, *v, *w, *sl;
    int* err;
    Coef c;
    int gx, gy, blk0, tma;
};

// ---- TMA / mbarrier primitives (PTX) ----------------------------------------

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

// Update of one plane pair from its centre values, the neighbour
// differences G(+1) - G(-1) along x, y, z, the staged point-wise fields and
// the face differences.
template <int STAGE>
__device__ __forceinline__ float2 cell_pair(const Coef& c, float2 gc, float2 gxd, float2 gyd, float2 gzd, float2 uu,
                                            float2 vv, float2 ww, float2 gn, float2 s_l, float2 dxL, float2 dxR,
                                            float2 dyL, float2 dyR, float2 dzL, float2 dzR) {
    float2 ue = uu, ve = vv, we = ww;
    const float2 gx = mul2(gxd, c2(c.inv_2dx));
    const float2 gy = mul2(gyd, c2(c.inv_2dy));
    const float2 gz = mul2(gzd, c2(c.inv_2dz));
    const float2 sq = fma2(gx, gx, fma2(gy, gy, fma2(gz, gz, c2(c.eps))));
    const float2 f = make_float2(s_l.x > c.eps ? -s_l.x * rsqrtf(sq.x) : 0.0f,
                                 s_l.y > c.eps ? -s_l.y * rsqrtf(sq.y) : 0.0f);
    ue = fma2(f, gx, ue);
    ve = fma2(f, gy, ve);
    we = fma2(f, gz, we);
    const float2 dgx = mul2(make_float2(ue.x >= 0.0f ? dxL.x : dxR.x, ue.y >= 0.0f ? dxL.y : dxR.y), c2(c.inv_dx));
    const float2 dgy = mul2(make_float2(ve.x >= 0.0f ? dyL.x : dyR.x, ve.y >= 0.0f ? dyL.y : dyR.y), c2(c.inv_dy));
    const float2 dgz = mul2(make_float2(we.x >= 0.0f ? dzL.x : dzR.x, we.y >= 0.0f ? dzL.y : dzR.y), c2(c.inv_dz));
    const float2 nrhs = fma2(ue, dgx, fma2(ve, dgy, mul2(we, dgz)));  // = -rhs
    if (STAGE == 1) return fma2(c2(-c.dt), nrhs, gc);
    if (STAGE == 2) return fma2(c2(-0.25f * c.dt), nrhs, fma2(c2(0.75f), gn, mul2(c2(0.25f), gc)));
    return fma2(c2(-(2.0f / 3.0f) * c.dt), nrhs, fma2(c2(1.0f / 3.0f), gn, mul2(c2(2.0f / 3.0f), gc)));
}

// Per-column z state: G(k-3 .. k+4), q(k-1), q(k), q(k+1), face k-1/2.
struct ZCol {
    float zq[8];
    float2 qa;
    float qk1, pL, pR;
};

template <typename IDX>
__device__ __forceinline__ void zcol_init(ZCol& z, const float* __restrict__ Gin, const IDX* zoff, IDX col) {
#pragma unroll
    for (int d = 0; d < 8; ++d) z.zq[d] = __ldg(Gin + zoff[d] + col);
    z.qa = qbeta(make_float2(z.zq[1], z.zq[2]), make_float2(z.zq[2], z.zq[3]), make_float2(z.zq[3], z.zq[4]));
    z.qk1 = qbeta(c2(z.zq[3]), c2(z.zq[4]), c2(z.zq[5])).x;
    const float qm2 = qbeta(c2(z.zq[0]), c2(z.zq[1]), c2(z.zq[2])).x;
    float2 L, R;
    face(c2(z.zq[0]), c2(z.zq[1]), c2(z.zq[2]), c2(z.zq[3]), c2(z.zq[4]), c2(z.zq[5]), c2(qm2), c2(z.qa.x),
         c2(z.qa.y), c2(z.qk1), L, R);
    z.pL = L.x;
    z.pR = R.x;
}

// z faces k+1/2, k+3/2 of a column -> face differences of planes k, k+1;
// advances the queue by two planes (zn0, zn1 = G(k+5), G(k+6)).
__device__ __forceinline__ void zcol_step(ZCol& z, float zn0, float zn1, float2& dzL, float2& dzR, float2& gzd) {
    const float2 qb = qbeta(make_float2(z.zq[4], z.zq[5]), make_float2(z.zq[5], z.zq[6]),
                            make_float2(z.zq[6], z.zq[7]));
    float2 L, R;
    face(make_float2(z.zq[1], z.zq[2]), make_float2(z.zq[2], z.zq[3]), make_float2(z.zq[3], z.zq[4]),
         make_float2(z.zq[4], z.zq[5]), make_float2(z.zq[5], z.zq[6]), make_float2(z.zq[6], z.zq[7]),
         make_float2(z.qa.x, z.qa.y), make_float2(z.qa.y, z.qk1), make_float2(z.qk1, qb.x), qb, L, R);
    dzL = sub2(L, make_float2(z.pL, L.x));
    dzR = sub2(R, make_float2(z.pR, R.x));
    gzd = make_float2(z.zq[4] - z.zq[2], z.zq[5] - z.zq[3]);
#pragma unroll
    for (int d = 0; d < 6; ++d) z.zq[d] = z.zq[d + 2];
    z.zq[6] = zn0;
    z.zq[7] = zn1;
    z.qa = make_float2(z.qk1, qb.x);
    z.qk1 = qb.y;
    z.pL = L.y;
    z.pR = R.y;
}

// IDX: element offsets (int when the field has < 2^31 cells).  u, v, w, G^n
// and S_L stream through an NSTAGE-deep pipeline of shared-memory stages:
// TMA = bulk tensor copies of the CTA's tile (one thread issues, mbarriers
// signal arrival); otherwise every thread copies its own four cells with
// cp.async and waits for its own copies.
// DEFO: the velocity is the deformation vortex (computeDeformationVelocity,
// Local_code/level-set_MPI_3D/include/initial_conditions.h:232-247) formed
// from the factor tables defo at time factor c.tf -- a per-row factor of the
// thread's two rows times a per-plane factor -- instead of read from u, v, w
// (the same FP32 products as launch_deformation_f32 writes).
// Static shared memory of one CTA (the staging ring of the point-wise fields
// is the dynamic part).  The grouped kernel, which runs either staging form,
// holds it once in this struct; the single-instance kernel declares the same
// arrays separately (passing the struct's members there cost 3 % at 512^3,
// measured A/B).
template <typename IDX>
struct StageSmem {
    float2 P2[2][BPH][PW];
    float2 FL[BNFX], FR[BNFX];  // x faces [BY][TX+1]
    IDX zoff[MAXZC + 10];
    uint64_t mbar[NSTAGE];
};

// The CTA's work: the column tile (bx, by) of z-chunk bz.  tmaps: the five
// fields' tensor maps (TMA form only).
template <int STAGE, bool TMA, typename IDX, bool DEFO>
__device__ __forceinline__ void
stage3d_body(const Geo& g, const float* __restrict__ Gin, const float* __restrict__ Gn, float* __restrict__ Gout,
             const float* __restrict__ u, const float* __restrict__ v, const float* __restrict__ w,
             const float* __restrict__ sl, const Coef& c, const CUtensorMap* tmaps, int* __restrict__ err,
             int hsl /* sl != nullptr */, const float* __restrict__ defo, int bx, int by, int bz,
             float2 (*P2)[BPH][PW], float2* FL, float2* FR, IDX* zoff, uint64_t* mbar, bool global_maps = false) {
    extern __shared__ __align__(128) float stg[];  // NSTAGE x NFIELD x BFTILE

    const int tx = threadIdx.x, ty = threadIdx.y;
    const int t = ty * TX + tx;
    const int i0 = bx * TX, j0 = by * BY;
    const int z0 = bz * c.zc;
    const int z1 = min(z0 + c.zc, g.nz);
    const int niter = (z1 - z0 + 1) / 2;
    const IDX sz = (IDX)g.nx * g.ny;
    const bool has_sl = hsl != 0;
    const int ra = RY * ty;  // tile row of cell row A; row B = ra + 1
    const bool xin = (i0 + tx) < g.nx;
    const bool va = xin && (j0 + ra) < g.ny;
    const bool vb = xin && (j0 + ra + 1) < g.ny;
    const int gxc = wrapg(i0 + tx, g.nx, g.bcx);
    const IDX colA = (IDX)wrapg(j0 + ra, g.ny, g.bcy) * g.nx + gxc;
    const IDX colB = (IDX)wrapg(j0 + ra + 1, g.ny, g.bcy) * g.nx + gxc;

    // halo ring of the staged plane pair: 3 full rows above and below, 3
    // cells left and right of each tile row
    int ring_s[BRPT];
    IDX ring_g[BRPT];
#pragma unroll
    for (int r = 0; r < BRPT; ++r) {
        const int q = t + r * NT;
        int ly, lx;
        if (q < 3 * PW) {
            ly = q / PW; lx = q % PW;
        } else if (q < 6 * PW) {
            ly = BPH - 3 + (q - 3 * PW) / PW; lx = (q - 3 * PW) % PW;
        } else {
            const int s = (q - 6 * PW) % 6;
            ly = 3 + (q - 6 * PW) / 6;
            lx = s < 3 ? s : TX + s;
        }
        ring_s[r] = q < BRING ? ly * PW + lx : -1;
        ring_g[r] = q < BRING ? (IDX)wrapg(j0 + ly - 3, g.ny, g.bcy) * g.nx + wrapg(i0 + lx - 3, g.nx, g.bcx) : 0;
    }
    // x-face tasks: face column tx of rows ra and ra + 1 (samples
    // P[row + 3][tx .. tx + 5]); the right-edge faces (column TX) of all BY
    // rows go to the first BY lanes of the last warp
    const bool has_fx_c = ty == TY - 1 && tx < BY;
    // plane offsets of z-indices z0-3 .. z0+zc+6 (periodic wrap or clamp), one
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
    auto issue = [&](int it, int s) {
        const int kz = z0 + 2 * it;
        float* base = stg + s * NFIELD * BFTILE;
        const uint32_t nf = (DEFO ? 0 : 3) + (STAGE > 1 ? 1 : 0) + (has_sl ? 1 : 0);
        mbar_expect_tx(&mbar[s], nf * BFTILE * 4);
        if (!DEFO) {
            tma_load_3d(base + 0 * BFTILE, tmaps + 0, i0, j0, kz, &mbar[s]);
            tma_load_3d(base + 1 * BFTILE, tmaps + 1, i0, j0, kz, &mbar[s]);
            tma_load_3d(base + 2 * BFTILE, tmaps + 2, i0, j0, kz, &mbar[s]);
        }
        if (STAGE > 1) tma_load_3d(base + 3 * BFTILE, tmaps + 3, i0, j0, kz, &mbar[s]);
        if (has_sl) tma_load_3d(base + 4 * BFTILE, tmaps + 4, i0, j0, kz, &mbar[s]);
    };
    // plain form: this thread's cells of rows ra, ra + 1, planes k, k + 1
    auto fetch = [&](int it, int s) {
        const IDX* zf = zoff + 2 * it + 3;
        float* base = stg + s * NFIELD * BFTILE + ra * TX + tx;
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
            for (int p = 0; p < 2; ++p) {
                const IDX o = zf[p] + (h ? colB : colA);
                float* d = base + h * TX + p * BY * TX;
                if (!DEFO) {
                    cp_async4(d, u + o);
                    cp_async4(d + BFTILE, v + o);
                    cp_async4(d + 2 * BFTILE, w + o);
                }
                if (STAGE > 1) cp_async4(d + 3 * BFTILE, Gn + o);
                if (has_sl) cp_async4(d + 4 * BFTILE, sl + o);
            }
    };
    if (TMA && t == 0) {
        for (int s = 0; s < NSTAGE; ++s) mbar_init(&mbar[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        // tensor maps that a copy wrote into global memory: make them visible
        // to the bulk-copy unit before the first copy reads them
        if (global_maps)
            for (int f = 0; f < NFIELD; ++f)
                asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(tmaps + f) : "memory");
    }
    __syncthreads();  // zoff table and barriers ready
    if (TMA && t == 0 && !c.drop)
        for (int it = 0; it < NSTAGE - 1 && it < niter; ++it) issue(it, it);
    if (!TMA)
        for (int it = 0; it < NSTAGE - 1; ++it) {
            if (it < niter) fetch(it, it);
            cp_async_commit();  // one group per iteration, empty ones included
        }

    // deformation vortex: per-row factors of rows A and B (constant over the march)
    float dfu[2] = {0.0f, 0.0f}, dfv[2] = {0.0f, 0.0f}, dfw[2] = {0.0f, 0.0f};
    if (DEFO) {
        const DeformTables d = deform_tables(g, defo);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int jr = wrapg(j0 + ra + h, g.ny, g.bcy);
            dfu[h] = 2.0f * __ldg(d.sqx + gxc) * __ldg(d.s2y + jr) * c.tf;
            dfv[h] = -__ldg(d.s2x + gxc) * __ldg(d.sqy + jr) * c.tf;
            dfw[h] = -__ldg(d.s2x + gxc) * __ldg(d.s2y + jr) * c.tf;
        }
    }

    ZCol za, zb;
    zcol_init(za, Gin, zoff, colA);
    zcol_init(zb, Gin, zoff, colB);
    float2 ring_v[BRPT];
#pragma unroll
    for (int r = 0; r < BRPT; ++r)
        ring_v[r] = ring_s[r] >= 0 ? make_float2(__ldg(Gin + zoff[3] + ring_g[r]), __ldg(Gin + zoff[4] + ring_g[r]))
                                   : make_float2(0.0f, 0.0f);

    int buf = 0;
    int cs = 0;        // TMA stage of this iteration (it % NSTAGE)
    uint32_t cph = 0;  // its mbarrier phase parity ((it / NSTAGE) & 1)
    for (int it = 0; it < niter; ++it) {
        const int k = z0 + 2 * it;
        const IDX* zo = zoff + 2 * it + 3;  // zo[d] = offset of plane k + d
        float2* P = &P2[buf][0][0];
        P[(ra + 3) * PW + tx + 3] = make_float2(za.zq[3], za.zq[4]);
        P[(ra + 4) * PW + tx + 3] = make_float2(zb.zq[3], zb.zq[4]);
#pragma unroll
        for (int r = 0; r < BRPT; ++r)
            if (ring_s[r] >= 0) P[ring_s[r]] = ring_v[r];
        // next planes of the own columns and the next pair's halo
        const float na0 = __ldg(Gin + zo[5] + colA), na1 = __ldg(Gin + zo[6] + colA);
        const float nb0 = __ldg(Gin + zo[5] + colB), nb1 = __ldg(Gin + zo[6] + colB);
        if (it + 1 < niter) {
#pragma unroll
            for (int r = 0; r < BRPT; ++r)
                if (ring_s[r] >= 0)
                    ring_v[r] = make_float2(__ldg(Gin + zo[2] + ring_g[r]), __ldg(Gin + zo[3] + ring_g[r]));
        }
        __syncthreads();
        // refill the stage last read in iteration it-1, which every thread
        // finished before the barrier above
        if (TMA && t == 0 && !c.drop && it + NSTAGE - 1 < niter) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(it + NSTAGE - 1, cs == 0 ? NSTAGE - 1 : cs - 1);
        }
        if (!TMA) {
            if (it + NSTAGE - 1 < niter) fetch(it + NSTAGE - 1, cs == 0 ? NSTAGE - 1 : cs - 1);
            cp_async_commit();
        }
        // ---- x faces ----
        {
            float2 L, R;
            xface_shfl(P + (ra + 3) * PW + tx, tx, L, R);
            FL[ra * (TX + 1) + tx] = L;
            FR[ra * (TX + 1) + tx] = R;
            xface_shfl(P + (ra + 4) * PW + tx, tx, L, R);
            FL[(ra + 1) * (TX + 1) + tx] = L;
            FR[(ra + 1) * (TX + 1) + tx] = R;
            if (has_fx_c) {
                face6(P + (tx + 3) * PW + TX, 1, L, R);
                FL[tx * (TX + 1) + TX] = L;
                FR[tx * (TX + 1) + TX] = R;
            }
        }
        // ---- y: window of tile rows ra - 3 .. ra + 4, faces ra, ra + 1, ra + 2 ----
        float2 dyLA, dyRA, dyLB, dyRB, gyA, gyB, gxA, gxB;
        {
            const float2* col = P + ra * PW + tx + 3;
            float2 y[8];
#pragma unroll
            for (int m = 0; m < 8; ++m) y[m] = col[m * PW];
            float2 q[7];
#pragma unroll
            for (int m = 1; m < 7; ++m) q[m] = qbeta(y[m - 1], y[m], y[m + 1]);
            float2 L0, R0, L1, R1, L2, R2;
            face(y[0], y[1], y[2], y[3], y[4], y[5], q[1], q[2], q[3], q[4], L0, R0);
            face(y[1], y[2], y[3], y[4], y[5], y[6], q[2], q[3], q[4], q[5], L1, R1);
            face(y[2], y[3], y[4], y[5], y[6], y[7], q[3], q[4], q[5], q[6], L2, R2);
            dyLA = sub2(L1, L0);
            dyRA = sub2(R1, R0);
            dyLB = sub2(L2, L1);
            dyRB = sub2(R2, R1);
            gyA = sub2(y[4], y[2]);
            gyB = sub2(y[5], y[3]);
            gxA = sub2(col[3 * PW + 1], col[3 * PW - 1]);
            gxB = sub2(col[4 * PW + 1], col[4 * PW - 1]);
        }
        // ---- z faces of both columns ----
        float2 dzLA, dzRA, dzLB, dzRB, gzA, gzB;
        zcol_step(za, na0, na1, dzLA, dzRA, gzA);
        zcol_step(zb, nb0, nb1, dzLB, dzRB, gzB);
        if (TMA) {
            const bool ok = mbar_wait(&mbar[cs], cph);
            if (__syncthreads_or(!ok)) {
                // a bulk copy did not arrive in time: flag it, give the copies
                // still in flight (issued by thread 0) a bounded chance to
                // land, and leave.  Flag 2 when copies had been issued: one
                // that missed its limit may still land in shared memory that
                // a later block owns, so the handle is not used again.  Flag
                // 1 only when none were (the drop-copies test hook).  (The
                // drain's own results are not read: using them here slowed
                // the whole loop by 4 %.)
                if (t == 0) {
                    const int issued = c.drop ? 0 : min(niter, it + NSTAGE);  // iterations whose copies went out
                    atomicMax(err, issued > it ? 2 : 1);
                    for (int j = it; j < issued; ++j) mbar_wait(&mbar[j % NSTAGE], (uint32_t)((j / NSTAGE) & 1));
                }
                return;
            }
        } else {
            cp_async_wait<NSTAGE - 1>();  // this iteration's group (own cells only)
            __syncthreads();              // x faces complete
        }

        // ---- cell update, rows A and B ----
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const IDX o = zo[0] + (h ? colB : colA);
            const float* f = stg + cs * NFIELD * BFTILE + (ra + h) * TX + tx;
            constexpr int pl = BY * TX;
            float2 uu, vv, ww;
            if (DEFO) {
                const DeformTables d = deform_tables(g, defo);
                const float2 zs2 = make_float2(__ldg(d.s2z + k), __ldg(d.s2z + k + 1));  // entry nz is 0
                const float2 zsq = make_float2(__ldg(d.sqz + k), __ldg(d.sqz + k + 1));
                uu = mul2(c2(dfu[h]), zs2);
                vv = mul2(c2(dfv[h]), zs2);
                ww = mul2(c2(dfw[h]), zsq);
            } else {
                uu = make_float2(f[0], f[pl]);
                vv = make_float2(f[BFTILE], f[BFTILE + pl]);
                ww = make_float2(f[2 * BFTILE], f[2 * BFTILE + pl]);
            }
            const float2 gn = STAGE > 1 ? make_float2(f[3 * BFTILE], f[3 * BFTILE + pl]) : c2(0.0f);
            const float2 s_l = has_sl ? make_float2(f[4 * BFTILE], f[4 * BFTILE + pl]) : c2(c.s_l);
            const int xf = (ra + h) * (TX + 1) + tx;
            // centre values G(k), G(k+1): the queues already advanced by two planes
            const float2 gc = h ? make_float2(zb.zq[1], zb.zq[2]) : make_float2(za.zq[1], za.zq[2]);
            const float2 out = cell_pair<STAGE>(
                c, gc, h ? gxB : gxA, h ? gyB : gyA, h ? gzB : gzA, uu, vv, ww, gn, s_l,
                sub2(FL[xf + 1], FL[xf]), sub2(FR[xf + 1], FR[xf]), h ? dyLB : dyLA, h ? dyRB : dyRA,
                h ? dzLB : dzLA, h ? dzRB : dzRA);
            if (h ? vb : va) {
                Gout[o] = out.x;
                if (k + 1 < z1) Gout[o + sz] = out.y;
            }
        }
        buf ^= 1;
        if (++cs == NSTAGE) {
            cs = 0;
            cph ^= 1u;
        }
    }
}

template <int STAGE, bool TMA, typename IDX, bool DEFO>
__global__ void __launch_bounds__(NT, 2)
stage3d_f32_col2(Geo g, const float* __restrict__ Gin, const float* __restrict__ Gn, float* __restrict__ Gout,
                 const float* __restrict__ u, const float* __restrict__ v, const float* __restrict__ w,
                 const float* __restrict__ sl, Coef c, const __grid_constant__ TmaMaps tm, int* __restrict__ err,
                 int hsl /* sl != nullptr */, const float* __restrict__ defo) {
    __shared__ float2 P2[2][BPH][PW];
    __shared__ float2 FL[BNFX], FR[BNFX];
    __shared__ IDX zoff[MAXZC + 10];
    __shared__ __align__(8) uint64_t mbar[NSTAGE];
    stage3d_body<STAGE, TMA, IDX, DEFO>(g, Gin, Gn, Gout, u, v, w, sl, c, tm.m, err, hsl, defo, blockIdx.x,
                                        blockIdx.y, blockIdx.z, P2, FL, FR, zoff, mbar);
}

// Grouped form: one launch advances one RK3 stage of every 3D instance of a
// batch.  Block b belongs to instance owner[b], whose blocks start at its
// blk0; within it, blocks run over (x tile, y tile, z chunk) as the
// single-instance grid does.  Fixed buffer roles: stage 1 reads G and
// writes A, stage 2 A -> B, stage 3 B -> G (G^n = G throughout).  Staging per
// instance: bulk tensor copies from the descriptor's tensor maps where the
// row pitch allows (nx % 4 == 0), per-thread cp.async copies otherwise;
// 32-bit offsets.
template <int STAGE>
__global__ void __launch_bounds__(NT, 2) stage3d_f32_group(const Group3* __restrict__ ins,
                                                            const int* __restrict__ owner) {
    const Group3* d = ins + owner[blockIdx.x];
    int l = (int)blockIdx.x - d->blk0;
    const int bx = l % d->gx;
    l /= d->gx;
    const int by = l % d->gy;
    const int bz = l / d->gy;
    const float* Gin = STAGE == 1 ? d->G : (STAGE == 2 ? d->A : d->B);
    float* Gout = STAGE == 1 ? d->A : (STAGE == 2 ? d->B : d->G);
    const Coef c = d->c;
    __shared__ StageSmem<int> sm;
    if (d->tma)
        stage3d_body<STAGE, true, int, false>(d->g, Gin, d->G, Gout, d->u, d->v, d->w, d->sl, c, d->m, d->err,
                                              d->sl != nullptr, nullptr, bx, by, bz, sm.P2, sm.FL, sm.FR, sm.zoff, sm.mbar, true);
    else
        stage3d_body<STAGE, false, int, false>(d->g, Gin, d->G, Gout, d->u, d->v, d->w, d->sl, c, nullptr, d->err,
                                               d->sl != nullptr, nullptr, bx, by, bz, sm.P2, sm.FL, sm.FR, sm.zoff, sm.mbar);
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

// 3D map over a compact FP32 field with a (32, rows, depth) box; zero fill outside.
bool encode_field(CUtensorMap* m, const float* ptr, const Geo& g, int rows, int depth) {
    PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
    if (!fn || !ptr) return false;
    cuuint64_t dims[3] = {(cuuint64_t)g.nx, (cuuint64_t)g.ny, (cuuint64_t)g.nz};
    cuuint64_t strides[2] = {(cuuint64_t)g.nx * 4, (cuuint64_t)g.nx * g.ny * 4};
    cuuint32_t box[3] = {TX, (cuuint32_t)rows, (cuuint32_t)depth};
    cuuint32_t estr[3] = {1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void*)ptr, dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int STAGE, bool TMA, typename IDX, bool DEFO>
cudaError_t launch_one(const StageArgs& a, const Coef& c, const TmaMaps& tm, int* err, cudaStream_t st) {
    const dim3 block(TX, TY, 1);
    const dim3 grid((a.g.nx + TX - 1) / TX, (a.g.ny + BY - 1) / BY, (a.g.nz + c.zc - 1) / c.zc);
    const size_t dyn = (size_t)NSTAGE * NFIELD * BFTILE * sizeof(float);
    auto kern = stage3d_f32_col2<STAGE, TMA, IDX, DEFO>;
    // once per instantiation (thread-safe initialisation of a local static)
    static const cudaError_t attr = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
    if (attr != cudaSuccess) return attr;
    kern<<<grid, block, dyn, st>>>(a.g, (const float*)a.Gin, (const float*)a.Gn, (float*)a.Gout,
                                    (const float*)a.u, (const float*)a.v, (const float*)a.w,
                                    (const float*)a.sl, c, tm, err, a.sl != nullptr, a.defo);
    return cudaGetLastError();
}

template <bool TMA, typename IDX, bool DEFO = false>
cudaError_t launch_stage(const StageArgs& a, const Coef& c, const TmaMaps& tm, int* err, cudaStream_t st) {
    if (a.stage == 1) return launch_one<1, TMA, IDX, DEFO>(a, c, tm, err, st);
    if (a.stage == 2) return launch_one<2, TMA, IDX, DEFO>(a, c, tm, err, st);
    return launch_one<3, TMA, IDX, DEFO>(a, c, tm, err, st);
}

// z-chunk of the default tile shape: the longest chunk that still gives every
// SM at least six CTAs (two resident at a time, so the last wave's tail and a
// chunk's queue prologue stay small), else the shortest.  Calibrated on
// 160^3 .. 512^3 against the timed alternatives (lsgb_solver_autotune picks
// per grid by measurement).
int default_zc(const Geo& g) {
    static const int sms = [] {
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        return n > 0 ? n : 1;
    }();
    const long long cols = (long long)((g.nx + TX - 1) / TX) * ((g.ny + BY - 1) / BY);
    for (int zc : {MAXZC, 32})
        if (cols * ((g.nz + zc - 1) / zc) >= 6LL * sms) return zc;
    return 16;
}

}  // namespace

bool stage3d_f32_fuses_deformation(const Geo& g) {
    return g.dim == 3 && (g.nx % 4) == 0 && g.cells() < (1LL << 31) - 1;
}

namespace {

Coef make_coef(const StageArgs& a) {
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
    c.zc = (a.tile == 16 || a.tile == 32 || a.tile == MAXZC) ? a.tile : default_zc(a.g);
    c.drop = a.drop_copies;
    c.tf = a.tf;
    return c;
}

}  // namespace

size_t group3_desc_bytes() { return sizeof(Group3); }

void group3_fill(const GroupInst* in, int n, void* out, std::vector<int>& owner) {
    Group3* d = (Group3*)out;
    long long blk = 0;
    for (int q = 0; q < n; ++q) {
        Group3 e;
        std::memset(&e, 0, sizeof(e));
        const StageArgs& a = in[q].a;
        e.g = a.g;
        e.G = in[q].G;
        e.A = in[q].A;
        e.B = in[q].B;
        e.u = (const float*)a.u;
        e.v = (const float*)a.v;
        e.w = (const float*)a.w;
        e.sl = (const float*)a.sl;
        e.err = a.err;
        e.c = make_coef(a);
        e.c.drop = 0;
        // bulk-tensor staging needs a 16-byte row pitch and an error flag for
        // its bounded waits
        bool tma = a.err != nullptr && (a.g.nx % 4) == 0;
        const float* fields[NFIELD] = {e.u, e.v, e.w, e.G, e.sl};
        for (int f = 0; f < NFIELD && tma; ++f)
            if (fields[f] && !encode_field(&e.m[f], fields[f], a.g, BY, 2)) tma = false;
        e.tma = tma ? 1 : 0;
        e.gx = (a.g.nx + TX - 1) / TX;
        e.gy = (a.g.ny + BY - 1) / BY;
        e.blk0 = (int)blk;
        const long long nb = (long long)e.gx * e.gy * ((a.g.nz + e.c.zc - 1) / e.c.zc);
        blk += nb;
        owner.insert(owner.end(), (size_t)nb, q);
        d[q] = e;
    }
}

// Planes a CTA of this instance marches (its z-chunk, or the whole grid when
// shorter): the block-length key the batch orders its 3D instances by.
int stage3d_chunk_planes(const StageArgs& a) {
    const int zc = (a.tile == 16 || a.tile == 32 || a.tile == MAXZC) ? a.tile : default_zc(a.g);
    return a.g.nz < zc ? a.g.nz : zc;
}

cudaError_t launch_stage3d_f32_group(const void* desc, const int* owner, int n, long long blocks, int stage,
                                     cudaStream_t st) {
    if (n <= 0 || blocks <= 0) return cudaSuccess;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
    const size_t dyn = (size_t)NSTAGE * NFIELD * BFTILE * sizeof(float);
    auto set = [dyn](const void* k) { return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn); };
    static const cudaError_t attr = [&] {
        cudaError_t e = set((const void*)stage3d_f32_group<1>);
        if (e == cudaSuccess) e = set((const void*)stage3d_f32_group<2>);
        if (e == cudaSuccess) e = set((const void*)stage3d_f32_group<3>);
        return e;
    }();
    if (attr != cudaSuccess) return attr;
    const dim3 block(TX, TY, 1), grid((unsigned)blocks, 1, 1);
    const Group3* d = (const Group3*)desc;
    if (stage == 1) stage3d_f32_group<1><<<grid, block, dyn, st>>>(d, owner);
    else if (stage == 2) stage3d_f32_group<2><<<grid, block, dyn, st>>>(d, owner);
    else stage3d_f32_group<3><<<grid, block, dyn, st>>>(d, owner);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_stage3d_f32_tiled(const StageArgs& a, int* err, cudaStream_t st) {
    Coef c = make_coef(a);
    TmaMaps tm;
    std::memset(&tm, 0, sizeof(tm));
    // bulk tensor copies need 16-byte row pitch and an error flag to report into
    bool tma = err != nullptr && (a.g.nx % 4) == 0;
    const bool defo = a.defo != nullptr;
    const void* fields[NFIELD] = {defo ? nullptr : a.u, defo ? nullptr : a.v, defo ? nullptr : a.w,
                                  a.stage > 1 ? a.Gn : nullptr, a.sl};
    for (int f = 0; f < NFIELD && tma; ++f)
        if (fields[f] && !encode_field(&tm.m[f], (const float*)fields[f], a.g, BY, 2)) tma = false;
    const bool small = a.g.cells() < (1LL << 31) - 1;
    cudaError_t e;
    if (defo) {
        // the fused velocity exists in the bulk-tensor form with 32-bit offsets
        // (stage3d_f32_fuses_deformation); the caller fills u, v, w otherwise
        if (!tma || !small) return cudaErrorNotSupported;
        e = launch_stage<true, int, true>(a, c, tm, err, st);
    } else if (tma) e = small ? launch_stage<true, int>(a, c, tm, err, st) : launch_stage<true, long long>(a, c, tm, err, st);
    else e = small ? launch_stage<false, int>(a, c, tm, err, st) : launch_stage<false, long long>(a, c, tm, err, st);
    count_launches(1);
    return e;
}

}  // namespace lsgb
