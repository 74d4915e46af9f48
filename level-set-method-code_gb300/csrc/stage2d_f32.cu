// stage2d_f32.cu -- the FP32-bulk 2D RK3 stage kernel.
//
// One launch = one TVD-RK3 stage over the whole 2D grid, fused: the u_eff
// WENO-5 right-hand side of computeRHS (Local_code/level-set_MPI_2D/include/
// rk3.h:54-98, weno5.h:135-230) and the stage combination of rk3Stage1..3
// (rk3.h:104-150).  Compact arrays, periodic / zero-gradient neighbours by
// index mapping.
//
// Shape: a CTA of 32 x TY threads works on 32 x 4 TY tiles (TY = 8: 32 x 32,
// the default; TY = 4: 32 x 16, more tiles for small grids -- the two tile
// shapes the autotuner picks from); thread (x, ty) owns rows 4 ty .. 4 ty + 3
// of column x as two row pairs, and every per-cell quantity is a float2 over
// a row pair (packed f32x2 arithmetic).  The grid is persistent (as many CTAs
// as fit on the GPU, at most one per tile); a CTA takes tiles blockIdx.x,
// blockIdx.x + gridDim.x, ...  In the grouped form (one launch for every 2D
// instance of a batch) the tile list runs over all instances.
//   - The tile plus a halo (3 columns left and right, 4 rows above and below)
//     is staged in shared memory as row pairs by asynchronous copies, double
//     buffered: the next tile's copies are in flight while this one computes.
//   - x: every x face of the tile is computed once, by the lane of its
//     column, with its indicators shared across the warp by shuffles, and
//     stored; the two cells that share it read it after the barrier.
//   - y: each thread reads its column's 12-row window and evaluates the
//     faces of its rows (as face pairs) in registers.
// The face values are the per-face WENO reconstructions of weno_f32x2.cuh
// (both upwind biases per face, indicators times 144, weights times 10,
// values times 6), the same arithmetic as the 3D kernel.
#include "common.cuh"
#include "weno_f32x2.cuh"

#include <cstring>

namespace lsgb {
namespace {

using namespace wf;

constexpr int TX = 32;                 // tile columns (one warp's lanes)
constexpr int RPT = 4;                 // cell rows per thread (two row pairs)
constexpr int PW = TX + 6;             // staged columns: tile x -3 .. TX+2

// Tile shape for TY thread rows per CTA.
template <int TYV>
struct Shape {
    static constexpr int TY = TYV;                  // thread rows of a CTA
    static constexpr int NT = TX * TY;
    static constexpr int BY = TY * RPT;             // tile rows
    static constexpr int PP = (BY + 8) / 2;         // staged row pairs: tile rows -4 .. BY+3
    static constexpr int NST = PP * PW;             // staged float2 entries
    static constexpr int NFX = (TX + 1) * (BY / 2); // x faces of the tile, per row pair
};

struct Coef2 {
    float inv_dx, inv_dy, inv_2dx, inv_2dy, s_l, eps, dt;
};

// One tile's work: the instance's fields and coefficients, the tile origin.
struct Tile2 {
    Geo g;
    const float *Gin, *Gn, *u, *v, *sl;
    float* Gout;
    Coef2 c;
    int i0, j0;
};

// One instance of a grouped launch: fixed buffers (stage 1 G -> A, 2 A -> B,
// 3 B -> G), coefficients, tile columns and its first tile in the list.
struct Group2 {
    Geo g;
    float *G, *A, *B;
    const float *u, *v, *sl;
    Coef2 c;
    int ntx, tile0;
};

// Stage update of one row pair from its centre values, the neighbour
// differences G(+1) - G(-1) along x and y, the point-wise fields and the
// face differences; the 2D form of the 3D kernel's cell update.
template <int STAGE>
__device__ __forceinline__ float2 cell2(const Coef2& c, float2 gc, float2 gxd, float2 gyd, float2 uu, float2 vv,
                                        float2 gn, float2 s_l, float2 dxL, float2 dxR, float2 dyL, float2 dyR) {
    const float2 gx = mul2(gxd, c2(c.inv_2dx));
    const float2 gy = mul2(gyd, c2(c.inv_2dy));
    const float2 sq = fma2(gx, gx, fma2(gy, gy, c2(c.eps)));
    const float2 f = make_float2(s_l.x > c.eps ? -s_l.x * rsqrtf(sq.x) : 0.0f,
                                 s_l.y > c.eps ? -s_l.y * rsqrtf(sq.y) : 0.0f);
    const float2 ue = fma2(f, gx, uu);
    const float2 ve = fma2(f, gy, vv);
    const float2 dgx = mul2(make_float2(ue.x >= 0.0f ? dxL.x : dxR.x, ue.y >= 0.0f ? dxL.y : dxR.y), c2(c.inv_dx));
    const float2 dgy = mul2(make_float2(ve.x >= 0.0f ? dyL.x : dyR.x, ve.y >= 0.0f ? dyL.y : dyR.y), c2(c.inv_dy));
    const float2 nrhs = fma2(ue, dgx, mul2(ve, dgy));  // = -rhs
    if (STAGE == 1) return fma2(c2(-c.dt), nrhs, gc);
    if (STAGE == 2) return fma2(c2(-0.25f * c.dt), nrhs, fma2(c2(0.75f), gn, mul2(c2(0.25f), gc)));
    return fma2(c2(-(2.0f / 3.0f) * c.dt), nrhs, fma2(c2(1.0f / 3.0f), gn, mul2(c2(2.0f / 3.0f), gc)));
}

// Issue the asynchronous copies that stage tile (i0, j0) plus its halo into
// P (every entry: two rows of one column).  Tiles whose halo lies inside the
// grid copy with plain offsets, the others through the index map.
template <typename IDX, typename S>
__device__ __forceinline__ void stage_tile(float2* P, const float* __restrict__ Gin, const Geo& g, int i0, int j0,
                                           int t) {
    constexpr int NST = S::NST, NT = S::NT, PP = S::PP;
    const IDX nx = g.nx;
    const bool inner = i0 >= 3 && i0 + PW - 3 <= g.nx && j0 >= 4 && j0 + 2 * PP - 4 <= g.ny;
    if (inner) {
        const float* base = Gin + (IDX)(j0 - 4) * nx + (i0 - 3);
        for (int e = t; e < NST; e += NT) {
            const int pp = e / PW, lx = e - pp * PW;
            const float* q = base + (IDX)(2 * pp) * nx + lx;
            cp_async4((float*)(P + e), q);
            cp_async4((float*)(P + e) + 1, q + nx);
        }
    } else {
        for (int e = t; e < NST; e += NT) {
            const int pp = e / PW, lx = e - pp * PW;
            const IDX x = wrapg(i0 + lx - 3, g.nx, g.bcx);
            const int r0 = j0 + 2 * pp - 4;
            cp_async4((float*)(P + e), Gin + (IDX)wrapg(r0, g.ny, g.bcy) * nx + x);
            cp_async4((float*)(P + e) + 1, Gin + (IDX)wrapg(r0 + 1, g.ny, g.bcy) * nx + x);
        }
    }
}

// Tile sources: tile index -> Tile2.  One instance (tiles in row-major
// order of ntx tile columns) ...
struct OneSrc {
    static constexpr bool kShared = false;  // cheap to evaluate: every thread does
    Geo g;
    const float *Gin, *Gn, *u, *v, *sl;
    float* Gout;
    Coef2 c;
    int ntx, by;
    __device__ __forceinline__ Tile2 operator()(int tile) const {
        return Tile2{g, Gin, Gn, u, v, sl, Gout, c, (tile % ntx) * TX, (tile / ntx) * by};
    }
};

// ... or every instance of a batch: tile t belongs to instance owner[t],
// whose tiles start at its tile0; for RK3 stage STAGE.
// Evaluating it costs a chain of global loads, so one thread evaluates each
// tile's entry ahead of time and the CTA reads it from shared memory.
template <int STAGE>
struct GroupSrc {
    static constexpr bool kShared = true;
    const Group2* ins;
    const int* owner;
    int by;
    __device__ __forceinline__ Tile2 operator()(int tile) const {
        const Group2* d = ins + __ldg(owner + tile);
        const int l = tile - d->tile0;
        return Tile2{d->g, STAGE == 1 ? d->G : (STAGE == 2 ? d->A : d->B), d->G, d->u, d->v, d->sl,
                     STAGE == 1 ? d->A : (STAGE == 2 ? d->B : d->G), d->c, (l % d->ntx) * TX, (l / d->ntx) * by};
    }
};

template <int STAGE, typename IDX, int TYV, typename SRC>
__device__ __forceinline__ void stage2d_body(const SRC& src, int ntiles) {
    using S = Shape<TYV>;
    constexpr int TY = S::TY, BY = S::BY, NST = S::NST, NFX = S::NFX;
    __shared__ float2 Pbuf[2][NST];        // [PP][PW]: (row 2p-4, row 2p-3) of tile column x-3
    __shared__ float2 FL[NFX], FR[NFX];    // x faces [BY/2][TX+1]
    __shared__ Tile2 tinfo[2];             // entries of this and the next tile (kShared sources)
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int t = ty * TX + tx;
    int tile = blockIdx.x;
    if (tile < ntiles) {
        const Tile2 f = src(tile);
        if (SRC::kShared && t == 0) tinfo[0] = f;
        stage_tile<IDX, S>(Pbuf[0], f.Gin, f.g, f.i0, f.j0, t);
    }
    cp_async_commit();
    if (SRC::kShared) __syncthreads();  // tinfo[0] visible
    for (int buf = 0; tile < ntiles; tile += gridDim.x, buf ^= 1) {
        // the next tile's entry, read after this iteration's first barrier;
        // its slot was last read before the previous iteration's barriers
        if (SRC::kShared && t == 0 && tile + (int)gridDim.x < ntiles) tinfo[buf ^ 1] = src(tile + gridDim.x);
        const Tile2 T = SRC::kShared ? tinfo[buf] : src(tile);
        const Geo& g = T.g;
        const Coef2& c = T.c;
        const float* __restrict__ u = T.u;
        const float* __restrict__ v = T.v;
        const float* __restrict__ Gn = T.Gn;
        const float* __restrict__ sl = T.sl;
        float* __restrict__ Gout = T.Gout;
        const IDX nx = g.nx;
        const int i0 = T.i0, j0 = T.j0;
        const float2* P = Pbuf[buf];
        // point-wise fields of the own cells (rows clamped into range; rows past
        // the grid are computed but not stored)
        const int gxc = wrapg(i0 + tx, g.nx, g.bcx);
        float2 uu[2], vv[2], gn[2], s_l[2];
        IDX orow[4];
#pragma unroll
        for (int r = 0; r < RPT; ++r) orow[r] = (IDX)min(j0 + RPT * ty + r, g.ny - 1) * nx + gxc;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const IDX a = orow[2 * h], b = orow[2 * h + 1];
            uu[h] = make_float2(__ldg(u + a), __ldg(u + b));
            vv[h] = make_float2(__ldg(v + a), __ldg(v + b));
            gn[h] = STAGE > 1 ? make_float2(__ldg(Gn + a), __ldg(Gn + b)) : c2(0.0f);
            s_l[h] = sl ? make_float2(__ldg(sl + a), __ldg(sl + b)) : c2(c.s_l);
        }
        // this tile's copies done and visible; every thread is past the previous
        // tile, so the other buffer and the face arrays are free
        cp_async_wait<0>();
        __syncthreads();
        {
            const int tn = tile + gridDim.x;
            if (tn < ntiles) {
                const Tile2 f = SRC::kShared ? tinfo[buf ^ 1] : src(tn);
                stage_tile<IDX, S>(Pbuf[buf ^ 1], f.Gin, f.g, f.i0, f.j0, t);
            }
            cp_async_commit();
        }

        // ---- x faces of the own row pairs; the tile's right-edge faces (column
        // TX) of all BY/2 row pairs go to the first lanes of the last warp ----
        const int pa = 2 * ty + 2;  // staged pair of rows 4ty, 4ty+1 (pair pa+1: rows 4ty+2, 4ty+3)
        {
            float2 L, R;
            xface_shfl(P + pa * PW + tx, tx, L, R);
            FL[(pa - 2) * (TX + 1) + tx] = L;
            FR[(pa - 2) * (TX + 1) + tx] = R;
            xface_shfl(P + (pa + 1) * PW + tx, tx, L, R);
            FL[(pa - 1) * (TX + 1) + tx] = L;
            FR[(pa - 1) * (TX + 1) + tx] = R;
            if (ty == TY - 1 && tx < BY / 2) {
                face6(P + (tx + 2) * PW + TX, 1, L, R);
                FL[tx * (TX + 1) + TX] = L;
                FR[tx * (TX + 1) + TX] = R;
            }
        }
        // ---- y: window of tile rows 4ty-4 .. 4ty+7 of column tx; y[m] = row 4ty-4+m ----
        float y[12];
#pragma unroll
        for (int m = 0; m < 6; ++m) {
            const float2 w = P[(2 * ty + m) * PW + tx + 3];
            y[2 * m] = w.x;
            y[2 * m + 1] = w.y;
        }
        // indicators q(r) of rows 4ty-2 .. 4ty+6, qy[m] = q(row 4ty-4+m), m = 2 .. 10
        float qy[11];
#pragma unroll
        for (int m = 2; m < 10; m += 2) {
            const float2 q = qbeta(make_float2(y[m - 1], y[m]), make_float2(y[m], y[m + 1]),
                                   make_float2(y[m + 1], y[m + 2]));
            qy[m] = q.x;
            qy[m + 1] = q.y;
        }
        qy[10] = qbeta(c2(y[9]), c2(y[10]), c2(y[11])).x;
        // face pairs (f, f+1), f = 4ty + 2h: samples rows f-3 .. f+3, indicators q(f-2) .. q(f+2)
        float2 FyL[3], FyR[3];
#pragma unroll
        for (int h = 0; h < 3; ++h) {
            const int m = 2 * h + 1;  // window index of row f-3
            face(make_float2(y[m], y[m + 1]), make_float2(y[m + 1], y[m + 2]), make_float2(y[m + 2], y[m + 3]),
                 make_float2(y[m + 3], y[m + 4]), make_float2(y[m + 4], y[m + 5]), make_float2(y[m + 5], y[m + 6]),
                 make_float2(qy[m + 1], qy[m + 2]), make_float2(qy[m + 2], qy[m + 3]),
                 make_float2(qy[m + 3], qy[m + 4]), make_float2(qy[m + 4], qy[m + 5]), FyL[h], FyR[h]);
        }
        __syncthreads();  // x faces complete

        // ---- cell update, row pairs A (4ty, 4ty+1) and B (4ty+2, 4ty+3) ----
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const float2* ctr = P + (pa + h) * PW + tx + 3;
            const int xf = (pa - 2 + h) * (TX + 1) + tx;
            const int m = 4 + 2 * h;  // window index of the pair's first row
            const float2 nextL = make_float2(FyL[h].y, FyL[h + 1].x), nextR = make_float2(FyR[h].y, FyR[h + 1].x);
            const float2 out = cell2<STAGE>(
                c, ctr[0], sub2(ctr[1], ctr[-1]), sub2(make_float2(y[m + 1], y[m + 2]), make_float2(y[m - 1], y[m])),
                uu[h], vv[h], gn[h], s_l[h], sub2(FL[xf + 1], FL[xf]), sub2(FR[xf + 1], FR[xf]), sub2(nextL, FyL[h]),
                sub2(nextR, FyR[h]));
            const int r = j0 + RPT * ty + 2 * h;
            if (i0 + tx < g.nx) {
                if (r < g.ny) Gout[orow[2 * h]] = out.x;
                if (r + 1 < g.ny) Gout[orow[2 * h + 1]] = out.y;
            }
        }
    }
}

template <int STAGE, typename IDX, int TYV>
__global__ void __launch_bounds__(Shape<TYV>::NT, 24 / TYV) stage2d_f32_rows(OneSrc src, int ntiles) {
    stage2d_body<STAGE, IDX, TYV>(src, ntiles);
}

template <int STAGE, int TYV>
__global__ void __launch_bounds__(Shape<TYV>::NT, 24 / TYV) stage2d_f32_group(const Group2* __restrict__ ins,
                                                                              const int* __restrict__ owner,
                                                                              int ntiles) {
    stage2d_body<STAGE, int, TYV>(GroupSrc<STAGE>{ins, owner, Shape<TYV>::BY}, ntiles);
}

// Resident CTAs of a kernel on the whole GPU.
int resident_ctas(const void* kern, int threads) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, 0);
    return (sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
}

template <int STAGE, typename IDX, int TYV>
cudaError_t launch2(const StageArgs& a, const Coef2& c, cudaStream_t st) {
    using S = Shape<TYV>;
    static const int resident = resident_ctas((const void*)stage2d_f32_rows<STAGE, IDX, TYV>, S::NT);
    const int ntx = (a.g.nx + TX - 1) / TX;
    const int ntiles = ntx * ((a.g.ny + S::BY - 1) / S::BY);
    const dim3 block(TX, S::TY, 1);
    const dim3 grid(ntiles < resident ? ntiles : resident, 1, 1);
    OneSrc src{a.g, (const float*)a.Gin, (const float*)a.Gn, (const float*)a.u, (const float*)a.v,
               (const float*)a.sl, (float*)a.Gout, c, ntx, S::BY};
    stage2d_f32_rows<STAGE, IDX, TYV><<<grid, block, 0, st>>>(src, ntiles);
    return cudaGetLastError();
}

template <int STAGE, int TYV>
cudaError_t launch2_group(const Group2* d, const int* owner, int ntiles, cudaStream_t st) {
    using S = Shape<TYV>;
    static const int resident = resident_ctas((const void*)stage2d_f32_group<STAGE, TYV>, S::NT);
    const dim3 block(TX, S::TY, 1);
    const dim3 grid(ntiles < resident ? ntiles : resident, 1, 1);
    stage2d_f32_group<STAGE, TYV><<<grid, block, 0, st>>>(d, owner, ntiles);
    return cudaGetLastError();
}

Coef2 make_coef2(const StageArgs& a) {
    Coef2 c;
    // face values carry a factor 6 (see face())
    c.inv_dx = (float)(1.0 / (6.0 * a.dx));
    c.inv_dy = (float)(1.0 / (6.0 * a.dy));
    c.inv_2dx = (float)(1.0 / (2.0 * a.dx));
    c.inv_2dy = (float)(1.0 / (2.0 * a.dy));
    c.s_l = (float)a.s_l;
    c.eps = (float)a.eps;
    c.dt = (float)a.dt;
    return c;
}

}  // namespace

// Tile shape of a tile choice: 16 -> 32 x 16 tiles, anything else 32 x 32.
cudaError_t launch_stage2d_f32_tiled(const StageArgs& a, cudaStream_t st) {
    const Coef2 c = make_coef2(a);
    const bool small = a.g.cells() < (1LL << 31) - 1;
    const bool t16 = a.tile == 16;
    cudaError_t e;
#define LSGB_L2(ST) (small ? (t16 ? launch2<ST, int, 4>(a, c, st) : launch2<ST, int, 8>(a, c, st)) \
                           : (t16 ? launch2<ST, long long, 4>(a, c, st) : launch2<ST, long long, 8>(a, c, st)))
    if (a.stage == 1) e = LSGB_L2(1);
    else if (a.stage == 2) e = LSGB_L2(2);
    else e = LSGB_L2(3);
#undef LSGB_L2
    count_launches(1);
    return e;
}

size_t group2_desc_bytes() { return sizeof(Group2); }

void group2_fill(const GroupInst* in, int n, int shape, void* out, std::vector<int>& owner) {
    Group2* d = (Group2*)out;
    const int by = shape == 16 ? Shape<4>::BY : Shape<8>::BY;
    long long tiles = 0;
    for (int q = 0; q < n; ++q) {
        Group2 e;
        memset(&e, 0, sizeof(e));
        const StageArgs& a = in[q].a;
        e.g = a.g;
        e.G = in[q].G;
        e.A = in[q].A;
        e.B = in[q].B;
        e.u = (const float*)a.u;
        e.v = (const float*)a.v;
        e.sl = (const float*)a.sl;
        e.c = make_coef2(a);
        e.ntx = (a.g.nx + TX - 1) / TX;
        e.tile0 = (int)tiles;
        const long long nt = (long long)e.ntx * ((a.g.ny + by - 1) / by);
        tiles += nt;
        owner.insert(owner.end(), (size_t)nt, q);
        d[q] = e;
    }
}

cudaError_t launch_stage2d_f32_group(const void* table, const int* owner, int n, long long tiles, int stage,
                                     int shape, cudaStream_t st) {
    if (n <= 0 || tiles <= 0) return cudaSuccess;
    if (tiles > 0x7fffffffLL) return cudaErrorInvalidValue;
    const Group2* d = (const Group2*)table;
    const int nt = (int)tiles;
    cudaError_t e;
    if (shape == 16) {
        e = stage == 1 ? launch2_group<1, 4>(d, owner, nt, st)
                       : (stage == 2 ? launch2_group<2, 4>(d, owner, nt, st) : launch2_group<3, 4>(d, owner, nt, st));
    } else {
        e = stage == 1 ? launch2_group<1, 8>(d, owner, nt, st)
                       : (stage == 2 ? launch2_group<2, 8>(d, owner, nt, st) : launch2_group<3, 8>(d, owner, nt, st));
    }
    count_launches(1);
    return e;
}

}  // namespace lsgb
