// sample_kernels.cu -- the sample surface (sample/field.cpp,
// sample/weno5_rk3.cpp of the reference): 2D Field2D arrays [ny+6][nx+6],
// the local Lax-Friedrichs G-equation Hamiltonian with both one-sided WENO-5
// derivatives, TVD-RK3 with the anchored + periodic boundary pair after every
// stage, and the first-order reinitialisation.  FP64 in the reference's
// operation order, compiled with --fmad=false: bit-identical to the
// reference's compiled sources.
//
// Every kernel takes n_inst instances stored back to back (stride = one
// ghosted array); blockIdx.z is the instance.  The frequency-sweep workload
// of the reference (one process per forcing frequency) runs as one launch
// per stage over all frequencies.  Quotients by a known or shared divisor
// and products by powers of two use fp64_exact.cuh (the same bits).
#include "common.cuh"
#include "fp64_exact.cuh"

namespace lsgb {
namespace {

constexpr double SEPS = 1e-6;  // EPSILON, sample/weno5_rk3.cpp:8

struct S2 {
    int nx, ny;
    long long nxT, stride;  // row length, elements per instance
    __device__ __forceinline__ long long at(int j, int i) const { return (long long)j * nxT + i; }
};

// beta, sample/weno5_rk3.cpp:11-14; std::pow(x, 2) is the rounded product x*x
__device__ __forceinline__ double s_beta(double f0, double f1, double f2) {
    const double a = f0 - mul_pow2<1>(f1) + f2;
    const double b = f0 - mul_pow2<2>(f1) + 3.0 * f2;
    return (13.0 / 12.0) * (a * a) + mul_pow2<-2>(b * b);
}

// weno5_left, sample/weno5_rk3.cpp:17-32.  weno5_right (:35-50) called with
// the descending arguments of weno5_deriv_x/y evaluates the same operations
// on the ascending stencil, so the right-biased derivative at i is the
// left-biased one at i+1: every cell needs the three face values
// F(i-1/2), F(i+1/2), F(i+3/2).
__device__ __forceinline__ double s_face(double v0, double v1, double v2, double v3, double v4) {
    const double b0 = s_beta(v0, v1, v2);
    const double b1 = s_beta(v1, v2, v3);
    const double b2 = s_beta(v2, v3, v4);
    const double a0 = 0.1 / ((SEPS + b0) * (SEPS + b0));
    const double a1 = 0.6 / ((SEPS + b1) * (SEPS + b1));
    const double a2 = 0.3 / ((SEPS + b2) * (SEPS + b2));
    const double sum = a0 + a1 + a2;
    const double rsum = 1.0 / sum;
    const double w0 = div_rn(a0, sum, rsum), w1 = div_rn(a1, sum, rsum), w2 = div_rn(a2, sum, rsum);
    return div_rn(w0 * (mul_pow2<1>(v0) - 7.0 * v1 + 11.0 * v2), 6.0, RCP6)
         + div_rn(w1 * (-v1 + 5.0 * v2 + mul_pow2<1>(v3)), 6.0, RCP6)
         + div_rn(w2 * (mul_pow2<1>(v2) + 5.0 * v3 - v4), 6.0, RCP6);
}

__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }  // std::max
__device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }  // std::min

// -H of compute_geqn_rhs (sample/weno5_rk3.cpp:111-143) from the one-sided
// derivatives of the cell.
__device__ __forceinline__ double llf_rhs(double Gdxm, double Gdxp, double Gdym, double Gdyp, double uu, double vv,
                                          double S_L) {
    const double Gdx_mean = mul_pow2<-1>(Gdxm + Gdxp);
    const double Gdy_mean = mul_pow2<-1>(Gdym + Gdyp);
    const double transport = uu * Gdx_mean + vv * Gdy_mean;
    const double propagation = S_L * sqrt(Gdx_mean * Gdx_mean + Gdy_mean * Gdy_mean);
    const double nm = sqrt(Gdxm * Gdxm + Gdym * Gdym + 1e-14);
    const double np = sqrt(Gdxp * Gdxp + Gdyp * Gdyp + 1e-14);
    const double s_xm = uu - S_L * Gdxm / nm;
    const double s_xp = uu - S_L * Gdxp / np;
    const double alpha_x = smax(fabs(s_xm), fabs(s_xp));
    const double s_ym = vv - S_L * Gdym / nm;
    const double s_yp = vv - S_L * Gdyp / np;
    const double alpha_y = smax(fabs(s_ym), fabs(s_yp));
    const double alpha = smax(alpha_x, alpha_y);
    const double diss_x = mul_pow2<-1>(alpha * (Gdxp - Gdxm));
    const double diss_y = mul_pow2<-1>(alpha * (Gdyp - Gdym));
    const double H = transport - propagation - (diss_x + diss_y);
    return -H;
}

// Stage tile: 32 x 16 interior cells (one per thread).  The G tile with its
// 3-cell halo is staged in shared memory; every face value F(i+1/2) the tile
// needs is computed once (34 x 16 x-faces, 32 x 18 y-faces: 2.19 per cell)
// and read by the two cells that share it.
constexpr int STX = 32, STY = 16;
constexpr int SW = STX + 6, SH = STY + 6;
constexpr int NFXS = (STX + 2) * STY, NFYS = STX * (STY + 2);

// Velocity at a cell: the fields (u, v) when given, else the instance's
// uniform pair vel[2 * (step * n_inst + inst) + {0, 1}] with step = *ctr.
struct Vel {
    const double* u;
    const double* v;
    const double* vel;
    const int* ctr;
    int n_inst;
};

__device__ __forceinline__ void vel_at(const Vel& V, const S2& s, int q, long long c, double& uu, double& vv) {
    if (V.u) {
        uu = V.u[q * s.stride + c];
        vv = V.v[q * s.stride + c];
    } else {
        const long long k = 2LL * ((long long)(*V.ctr) * V.n_inst + q);
        uu = V.vel[k];
        vv = V.vel[k + 1];
    }
}

// One RK3 stage of RK3_step (sample/weno5_rk3.cpp:166-185) on the interior:
//   STAGE 1: out = Gn + dt L(Gin)                 (Gin == Gn)
//   STAGE 2: out = 0.75 Gn + 0.25 (Gin + dt L(Gin))
//   STAGE 3: out = 1/3 Gn + 2/3 (Gin + dt L(Gin))  (out == Gn allowed)
// STAGE 0: out = L(Gin), the drop-in compute_geqn_rhs.
template <int STAGE>
__global__ void __launch_bounds__(STX * STY) sample_stage_kernel(S2 s, const double* __restrict__ Gin_,
                                                           const double* Gn, double* out, Vel V, double dx,
                                                           double dy, double dt, double S_L) {
    __shared__ double tile[SH][SW];
    __shared__ double fx[STY][STX + 2];   // fx[y][k] = F(i0 - 1 + k + 1/2) on row j0 + y
    __shared__ double fy[STY + 2][STX];   // fy[k][x] = F(j0 - 1 + k + 1/2) on column i0 + x
    const int q = blockIdx.z;
    const double* __restrict__ Gin = Gin_ + q * s.stride;
    const int i0 = blockIdx.x * STX + 3, j0 = blockIdx.y * STY + 3;
    const int tid = threadIdx.y * STX + threadIdx.x;
    const int nxT = (int)s.nxT, nyT = s.ny + 6;
    for (int e = tid; e < SW * SH; e += STX * STY) {
        const int ty = e / SW, tx = e - ty * SW;
        const int gj = j0 - 3 + ty, gi = i0 - 3 + tx;
        tile[ty][tx] = (gj < nyT && gi < nxT) ? Gin[s.at(gj, gi)] : 0.0;
    }
    __syncthreads();
    // faces needed by interior cells: x-face i in [2, nx+3], y-face j in [2, ny+3]
    for (int e = tid; e < NFXS + NFYS; e += STX * STY) {
        if (e < NFXS) {
            const int y = e / (STX + 2), k = e - y * (STX + 2);
            const int fi = i0 - 1 + k;
            if (fi <= s.nx + 3 && j0 + y <= s.ny + 2) {
                const double* r = &tile[y + 3][k];  // G[fi - 2 .. fi + 2] start at tile col (fi - 2) - (i0 - 3) = k
                fx[y][k] = s_face(r[0], r[1], r[2], r[3], r[4]);
            }
        } else {
            const int f = e - NFXS;
            const int k = f / STX, x = f - k * STX;
            const int fj = j0 - 1 + k;
            if (fj <= s.ny + 3 && i0 + x <= s.nx + 2)
                fy[k][x] = s_face(tile[k][x + 3], tile[k + 1][x + 3], tile[k + 2][x + 3], tile[k + 3][x + 3],
                                  tile[k + 4][x + 3]);
        }
    }
    __syncthreads();
    const int x = threadIdx.x, y = threadIdx.y;
    const int i = i0 + x, j = j0 + y;
    if (i > s.nx + 2 || j > s.ny + 2) return;
    const double rdx = 1.0 / dx, rdy = 1.0 / dy;
    const double Gdxm = div_rn(fx[y][x + 1] - fx[y][x], dx, rdx), Gdxp = div_rn(fx[y][x + 2] - fx[y][x + 1], dx, rdx);
    const double Gdym = div_rn(fy[y + 1][x] - fy[y][x], dy, rdy), Gdyp = div_rn(fy[y + 2][x] - fy[y + 1][x], dy, rdy);
    const long long c = s.at(j, i);
    double uu, vv;
    vel_at(V, s, q, c, uu, vv);
    const double r = llf_rhs(Gdxm, Gdxp, Gdym, Gdyp, uu, vv, S_L);
    const long long e = q * s.stride + c;
    double o;
    if (STAGE == 0) o = r;
    else if (STAGE == 1) o = Gn[e] + dt * r;
    else if (STAGE == 2) o = 0.75 * Gn[e] + mul_pow2<-2>(tile[y + 3][x + 3] + dt * r);
    else o = (1.0 / 3.0) * Gn[e] + (2.0 / 3.0) * (tile[y + 3][x + 3] + dt * r);
    out[e] = o;
}

// apply_anchored_bc followed by apply_periodic (sample/field.cpp:37-63,
// :16-34) as one pass, after the interior has been written: row 3 takes the
// initial field's row 3, row ny+2 becomes 2 G[ny+1] - G[ny] (row ny read
// after the anchoring), and every ghost cell takes the value of its
// periodic image.  Each write is computed from cells no thread writes.
// bump != 0: thread 0 of instance 0 advances the velocity step counter.
__device__ __forceinline__ double anchored_interior(const double* G, const double* init, const S2& s, int j, int i) {
    if (j == 3) return init[s.at(3, i)];
    if (j == s.ny + 2) {
        const double below = (s.ny == 3) ? init[s.at(3, i)] : G[s.at(s.ny, i)];
        return 2.0 * G[s.at(s.ny + 1, i)] - below;
    }
    return G[s.at(j, i)];
}

__global__ void __launch_bounds__(256) sample_stage_bc_kernel(S2 s, double* G_, const double* init_,
                                                              long long init_stride, int* ctr, int bump) {
    const int nyT = s.ny + 6;
    const long long total = s.nxT * nyT;
    const int q = blockIdx.y;
    double* G = G_ + q * s.stride;
    const double* init = init_ + q * init_stride;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % s.nxT);
        const int j = (int)(e / s.nxT);
        const bool gx = i < 3 || i > s.nx + 2, gy = j < 3 || j > s.ny + 2;
        if (!gx && !gy && j != 3 && j != s.ny + 2) continue;
        const int ii = i < 3 ? i + s.nx : (i > s.nx + 2 ? i - s.nx : i);
        const int jj = j < 3 ? j + s.ny : (j > s.ny + 2 ? j - s.ny : j);
        G[e] = anchored_interior(G, init, s, jj, ii);
    }
    if (bump && q == 0 && blockIdx.x == 0 && threadIdx.x == 0) *ctr += 1;
}

// apply_anchored_bc alone (sample/field.cpp:37-63), sequential per column
// for the bottom/top rows, then per row for the left/right columns.
__global__ void sample_anchor_cols_kernel(S2 s, double* G_, const double* init_, long long init_stride) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    if (i >= s.nxT) return;
    double* d = G_ + q * s.stride;
    const double* init = init_ + q * init_stride;
    const int ny = s.ny;
    d[s.at(3, i)] = init[s.at(3, i)];
    d[s.at(2, i)] = 2.0 * d[s.at(3, i)] - d[s.at(4, i)];
    d[s.at(1, i)] = 2.0 * d[s.at(2, i)] - d[s.at(3, i)];
    d[s.at(0, i)] = 2.0 * d[s.at(1, i)] - d[s.at(2, i)];
    d[s.at(ny + 2, i)] = 2.0 * d[s.at(ny + 1, i)] - d[s.at(ny, i)];
    d[s.at(ny + 3, i)] = 2.0 * d[s.at(ny + 2, i)] - d[s.at(ny + 1, i)];
    d[s.at(ny + 4, i)] = 2.0 * d[s.at(ny + 3, i)] - d[s.at(ny + 2, i)];
    d[s.at(ny + 5, i)] = 2.0 * d[s.at(ny + 4, i)] - d[s.at(ny + 3, i)];
}

__global__ void sample_anchor_rows_kernel(S2 s, double* G_) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    if (j >= s.ny + 6) return;
    double* d = G_ + q * s.stride;
    const int nx = s.nx;
    d[s.at(j, 2)] = 2.0 * d[s.at(j, 3)] - d[s.at(j, 4)];
    d[s.at(j, 1)] = 2.0 * d[s.at(j, 2)] - d[s.at(j, 3)];
    d[s.at(j, 0)] = 2.0 * d[s.at(j, 1)] - d[s.at(j, 2)];
    d[s.at(j, nx + 3)] = 2.0 * d[s.at(j, nx + 2)] - d[s.at(j, nx + 1)];
    d[s.at(j, nx + 4)] = 2.0 * d[s.at(j, nx + 3)] - d[s.at(j, nx + 2)];
    d[s.at(j, nx + 5)] = 2.0 * d[s.at(j, nx + 4)] - d[s.at(j, nx + 3)];
}

// apply_periodic alone (sample/field.cpp:16-34): ghost cells take their
// periodic images (the x pass then the y pass give the same values).
__global__ void __launch_bounds__(256) sample_periodic_kernel(S2 s, double* G_) {
    const long long total = s.nxT * (s.ny + 6);
    double* G = G_ + blockIdx.y * s.stride;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % s.nxT);
        const int j = (int)(e / s.nxT);
        const bool gx = i < 3 || i > s.nx + 2, gy = j < 3 || j > s.ny + 2;
        if (!gx && !gy) continue;
        const int ii = i < 3 ? i + s.nx : (i > s.nx + 2 ? i - s.nx : i);
        const int jj = j < 3 ? j + s.ny : (j > s.ny + 2 ? j - s.ny : j);
        G[e] = G[s.at(jj, ii)];
    }
}

// One pseudo-step of Field2D::reinitialize (sample/field.cpp:72-105) on the
// interior: phinew = phi + dtau * (-s (|grad phi| - 1)), s from the initial
// field.  The boundary pass follows as the two anchor kernels.
__global__ void __launch_bounds__(256) sample_reinit_kernel(S2 s, const double* __restrict__ phi_,
                                                            double* __restrict__ out_, const double* __restrict__ init_,
                                                            long long init_stride, double dx, double dy, double dtau) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 3;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 3;
    const int q = blockIdx.z;
    if (i > s.nx + 2 || j > s.ny + 2) return;
    const double* phi = phi_ + q * s.stride;
    const double* init = init_ + q * init_stride;
    const double g0 = init[s.at(j, i)];
    const double sg = g0 / sqrt(g0 * g0 + dx * dx);
    const double c = phi[s.at(j, i)];
    const double rdx = 1.0 / dx, rdy = 1.0 / dy;
    const double dGdx_pos = div_rn(c - phi[s.at(j, i - 1)], dx, rdx);
    const double dGdx_neg = div_rn(phi[s.at(j, i + 1)] - c, dx, rdx);
    const double dGdy_pos = div_rn(c - phi[s.at(j - 1, i)], dy, rdy);
    const double dGdy_neg = div_rn(phi[s.at(j + 1, i)] - c, dy, rdy);
    double grad;
    if (sg > 0.0) {
        const double px = smax(smax(dGdx_pos, 0.0), -smin(dGdx_neg, 0.0));
        const double py = smax(smax(dGdy_pos, 0.0), -smin(dGdy_neg, 0.0));
        grad = sqrt(px * px + py * py);
    } else {
        const double px = smax(smax(-dGdx_pos, 0.0), smin(dGdx_neg, 0.0));
        const double py = smax(smax(-dGdy_pos, 0.0), smin(dGdy_neg, 0.0));
        grad = sqrt(px * px + py * py);
    }
    const double rhs = -sg * (grad - 1.0);
    out_[q * s.stride + s.at(j, i)] = c + dtau * rhs;
}

// compute_first_order_upwind (sample/first_order_upwind.cpp:6-69): the
// first-order upwind step from G into out over j = 3 .. ny+3, i = 3 .. nx+3
// (the reference's inclusive bounds on the ghosted sizes, one ghost row and
// column past the interior on the high side); the copy kernel below writes
// the same range back into G (the reference's G_new -> G loop).
__global__ void __launch_bounds__(256) sample_fou_kernel(S2 s, const double* __restrict__ G,
                                                         const double* __restrict__ u,
                                                         const double* __restrict__ v, double* __restrict__ out,
                                                         double dx, double dy, double dt, double S_L) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 3;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 3;
    if (i > s.nx + 3 || j > s.ny + 3) return;
    const double EPS = 1e-10;
    const double c = G[s.at(j, i)];
    const double Gx_mns = (c - G[s.at(j, i - 1)]) / dx;
    const double Gx_pls = (G[s.at(j, i + 1)] - c) / dx;
    const double Gy_mns = (c - G[s.at(j - 1, i)]) / dy;
    const double Gy_pls = (G[s.at(j + 1, i)] - c) / dy;
    const double dG_dx = 0.5 * (Gx_mns + Gx_pls);
    const double dG_dy = 0.5 * (Gy_mns + Gy_pls);
    const double mag_sq = dG_dx * dG_dx + dG_dy * dG_dy;
    double u_first = u[s.at(j, i)], v_first = v[s.at(j, i)];
    if (mag_sq > EPS * EPS) {
        const double mag = sqrt(mag_sq);
        u_first = u_first - S_L * dG_dx / mag;
        v_first = v_first - S_L * dG_dy / mag;
    }
    const double a_pls = smax(u_first, 0.0), a_mns = smin(u_first, 0.0);
    const double b_pls = smax(v_first, 0.0), b_mns = smin(v_first, 0.0);
    out[s.at(j, i)] = c - dt * (a_pls * Gx_mns + a_mns * Gx_pls + b_pls * Gy_mns + b_mns * Gy_pls);
}

__global__ void __launch_bounds__(256) sample_fou_copy_kernel(S2 s, const double* __restrict__ src,
                                                              double* __restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 3;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 3;
    if (i > s.nx + 3 || j > s.ny + 3) return;
    dst[s.at(j, i)] = src[s.at(j, i)];
}

__global__ void zero_ghosts_kernel(S2 s, double* G_) {
    const long long total = s.nxT * (s.ny + 6);
    double* G = G_ + blockIdx.y * s.stride;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % s.nxT);
        const int j = (int)(e / s.nxT);
        if (i < 3 || i > s.nx + 2 || j < 3 || j > s.ny + 2) G[e] = 0.0;
    }
}

S2 make_s2(int nx, int ny) {
    S2 s;
    s.nx = nx;
    s.ny = ny;
    s.nxT = nx + 6;
    s.stride = (long long)(nx + 6) * (ny + 6);
    return s;
}

dim3 interior_grid(const S2& s, int n_inst, dim3 b) {
    return dim3((s.nx + b.x - 1) / b.x, (s.ny + b.y - 1) / b.y, n_inst);
}

unsigned ghost_blocks(const S2& s) {
    const long long total = s.stride;
    long long b = (total + 255) / 256;
    return (unsigned)(b < 1024 ? b : 1024);
}

}  // namespace

cudaError_t sample_launch_stage(const SampleArgs& a, int stage, const double* Gin, const double* Gn, double* out,
                                cudaStream_t st) {
    const S2 s = make_s2(a.nx, a.ny);
    const dim3 b(STX, STY, 1), gr = interior_grid(s, a.n_inst, b);
    Vel V{a.u, a.v, a.vel, a.ctr, a.n_inst};
    switch (stage) {
        case 0: sample_stage_kernel<0><<<gr, b, 0, st>>>(s, Gin, Gn, out, V, a.dx, a.dy, a.dt, a.S_L); break;
        case 1: sample_stage_kernel<1><<<gr, b, 0, st>>>(s, Gin, Gn, out, V, a.dx, a.dy, a.dt, a.S_L); break;
        case 2: sample_stage_kernel<2><<<gr, b, 0, st>>>(s, Gin, Gn, out, V, a.dx, a.dy, a.dt, a.S_L); break;
        default: sample_stage_kernel<3><<<gr, b, 0, st>>>(s, Gin, Gn, out, V, a.dx, a.dy, a.dt, a.S_L); break;
    }
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t sample_launch_stage_bc(const SampleArgs& a, double* G, bool bump, cudaStream_t st) {
    const S2 s = make_s2(a.nx, a.ny);
    sample_stage_bc_kernel<<<dim3(ghost_blocks(s), a.n_inst), 256, 0, st>>>(s, G, a.init, a.init_stride,
                                                                              a.ctr, bump ? 1 : 0);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t sample_launch_anchored(const SampleArgs& a, double* G, cudaStream_t st) {
    const S2 s = make_s2(a.nx, a.ny);
    sample_anchor_cols_kernel<<<dim3((unsigned)((s.nxT + 127) / 128), a.n_inst), 128, 0, st>>>(s, G, a.init,
                                                                                              a.init_stride);
    sample_anchor_rows_kernel<<<dim3((unsigned)((s.ny + 6 + 127) / 128), a.n_inst), 128, 0, st>>>(s, G);
    count_launches(2);
    return cudaGetLastError();
}

cudaError_t sample_launch_periodic(const SampleArgs& a, double* G, cudaStream_t st) {
    const S2 s = make_s2(a.nx, a.ny);
    sample_periodic_kernel<<<dim3(ghost_blocks(s), a.n_inst), 256, 0, st>>>(s, G);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t sample_launch_reinit_step(const SampleArgs& a, const double* phi, double* out, double dtau,
                                      cudaStream_t st) {
    const S2 s = make_s2(a.nx, a.ny);
    const dim3 b(32, 8, 1), gr = interior_grid(s, a.n_inst, b);
    sample_reinit_kernel<<<gr, b, 0, st>>>(s, phi, out, a.init, a.init_stride, a.dx, a.dy, dtau);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t sample_launch_first_order_upwind(const SampleArgs& a, double* G, double* tmp, cudaStream_t st) {
    const S2 s = make_s2(a.nx, a.ny);
    const dim3 b(32, 8, 1), gr((s.nx + 1 + b.x - 1) / b.x, (s.ny + 1 + b.y - 1) / b.y, 1);
    sample_fou_kernel<<<gr, b, 0, st>>>(s, G, a.u, a.v, tmp, a.dx, a.dy, a.dt, a.S_L);
    sample_fou_copy_kernel<<<gr, b, 0, st>>>(s, tmp, G);
    count_launches(2);
    return cudaGetLastError();
}

cudaError_t sample_launch_zero_ghosts(const SampleArgs& a, double* G, cudaStream_t st) {
    const S2 s = make_s2(a.nx, a.ny);
    zero_ghosts_kernel<<<dim3(ghost_blocks(s), a.n_inst), 256, 0, st>>>(s, G);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace lsgb
