// f32_kernels.cu -- FP32-bulk form of the hot path.
//
// Same scheme as the reference (Local_code/level-set_MPI_3D/include/weno5.h,
// rk3.h, reinitialization.h): u_eff WENO-5 upwinding, TVD RK3, HCR-2.  The
// WENO/RK3/reinit arithmetic runs in FP32 with fused multiply-adds and one
// approximate reciprocal per reconstruction; the HCR-2 interface constraint
// (r~ = phi0 / sum phi0_nb and the forcing beta (r~ sum phi - phi) / dx, the
// sub-cell position of G = 0) is evaluated in FP64 on the flagged cells.
// Accuracy against the FP64 path is measured, not assumed (tests/test_gpu_f32.py,
// lsgb/precision.py, and the precision_vs_fp64 entry of bench.py's line).
//
// WENO-5 in mirrored form: with sgn = (u_eff >= 0), the 7 samples G[i-3..i+3]
// are read as w[m] = G[i-3+m] (sgn) or G[i+3-m] (!sgn).  Both the left-biased
// pair of weno5_left (weno5.h:39-58) and the right-biased pair of weno5_right
// (weno5.h:60-81) are then X = R(w0..w4) and Y = R(w1..w5) of one formula,
// with the optimal weights (0.1, 0.6, 0.3) for sgn and the reference's
// (0.3, 0.6, 0.1) otherwise; the derivative is +-(Y - X)/h.  The smoothness
// indicators of the four triples centred at w1..w4 are shared by X and Y.
#include "common.cuh"

namespace lsgb {
namespace {

constexpr float F_WENO_EPS = 1.0e-6f;

// WENO reconstruction from the 5-point window (a..e) with the squared
// regularised indicators q0..q2 of its three sub-stencils.  Division-free
// weights: omega_k ~ d_k / q_k, so with Q_k = prod_{j != k} q_j the value is
// sum d_k Q_k P_k / sum d_k Q_k.  P_k carry a factor 6 that the denominator
// removes.
__device__ __forceinline__ float recon(float a, float b, float c, float d, float e,
                                       float q0, float q1, float q2, float q01, float q02,
                                       float q12, float d0, float d2) {
    const float P0 = fmaf(2.0f, a, fmaf(-7.0f, b, 11.0f * c));
    const float P1 = fmaf(-1.0f, b, fmaf(5.0f, c, 2.0f * d));
    const float P2 = fmaf(2.0f, c, fmaf(5.0f, d, -e));
    const float w0 = d0 * q12, w1 = 0.6f * q02, w2 = d2 * q01;
    const float num = fmaf(w0, P0, fmaf(w1, P1, w2 * P2));
    const float den = 6.0f * (w0 + w1 + w2);
    return __fdividef(num, den);
}

__device__ __forceinline__ float qbeta(float a, float b, float c) {
    const float t = fmaf(-2.0f, b, a) + c;
    const float r = c - a;
    const float B = fmaf(13.0f / 12.0f * t, t, 0.25f * r * r);
    const float s = F_WENO_EPS + B;
    return s * s;
}

// Upwind WENO-5 derivative from s[0..6] = G[i-3..i+3], times 1/h.
__device__ __forceinline__ float weno_deriv_f32(const float* s, float vel, float inv_h) {
    const bool p = vel >= 0.0f;
    float w[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) w[m] = p ? s[m] : s[6 - m];
    const float Q1 = qbeta(w[0], w[1], w[2]);
    const float Q2 = qbeta(w[1], w[2], w[3]);
    const float Q3 = qbeta(w[2], w[3], w[4]);
    const float Q4 = qbeta(w[3], w[4], w[5]);
    const float Q23 = Q2 * Q3;
    const float d0 = p ? 0.1f : 0.3f;
    const float d2 = p ? 0.3f : 0.1f;
    const float X = recon(w[0], w[1], w[2], w[3], w[4], Q1, Q2, Q3, Q1 * Q2, Q1 * Q3, Q23, d0, d2);
    const float Y = recon(w[1], w[2], w[3], w[4], w[5], Q2, Q3, Q4, Q23, Q2 * Q4, Q3 * Q4, d0, d2);
    const float diff = Y - X;
    return (p ? diff : -diff) * inv_h;
}

struct F32Coef {
    float inv_dx, inv_dy, inv_dz, inv_2dx, inv_2dy, inv_2dz, s_l, eps, dt;
};

// Fused RK3 stage on compact FP32 arrays, one thread per cell, periodic or
// zero-gradient index mapping at the domain edges.
template <int DIM, int STAGE, typename IDX>
__global__ void __launch_bounds__(256) stage_f32_kernel(Geo g, const float* __restrict__ Gin,
                                                        const float* __restrict__ Gn,
                                                        float* __restrict__ Gout,
                                                        const float* __restrict__ u,
                                                        const float* __restrict__ v,
                                                        const float* __restrict__ w,
                                                        const float* __restrict__ sl, F32Coef c) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    int k = DIM == 3 ? blockIdx.z * blockDim.z + threadIdx.z : 0;
    if (i >= g.nx || j >= g.ny || k >= g.nz) return;
    const IDX sy = g.nx;
    const IDX sz = (IDX)g.nx * g.ny;
    const IDX plane = (IDX)k * sz;
    const IDX row = (IDX)j * sy + plane;
    const IDX id = row + i;

    float sx[7], syv[7], szv[7];
#pragma unroll
    for (int d = -3; d <= 3; ++d) {
        sx[d + 3] = __ldg(Gin + (row + map_axis(i + d, g.nx, g.bcx)));
        syv[d + 3] = __ldg(Gin + ((IDX)map_axis(j + d, g.ny, g.bcy) * sy + plane + i));
        if (DIM == 3) szv[d + 3] = __ldg(Gin + ((IDX)map_axis(k + d, g.nz, g.bcz) * sz + (IDX)j * sy + i));
    }
    const float s_l = sl ? __ldg(sl + id) : c.s_l;
    float ue = __ldg(u + id), ve = __ldg(v + id), we = 0.0f;
    if (DIM == 3) we = __ldg(w + id);
    if (s_l > c.eps) {
        const float gx = (sx[4] - sx[2]) * c.inv_2dx;
        const float gy = (syv[4] - syv[2]) * c.inv_2dy;
        float sq = fmaf(gx, gx, fmaf(gy, gy, c.eps));
        float gz = 0.0f;
        if (DIM == 3) { gz = (szv[4] - szv[2]) * c.inv_2dz; sq = fmaf(gz, gz, sq); }
        const float f = s_l * rsqrtf(sq);
        ue = fmaf(-f, gx, ue);
        ve = fmaf(-f, gy, ve);
        if (DIM == 3) we = fmaf(-f, gz, we);
    }
    float rhs = ue * weno_deriv_f32(sx, ue, c.inv_dx);
    rhs = fmaf(ve, weno_deriv_f32(syv, ve, c.inv_dy), rhs);
    if (DIM == 3) rhs = fmaf(we, weno_deriv_f32(szv, we, c.inv_dz), rhs);
    rhs = -rhs;

    float out;
    if (STAGE == 1) {
        out = fmaf(c.dt, rhs, sx[3]);
    } else if (STAGE == 2) {
        const float gn = __ldg(Gn + id);
        out = fmaf(0.25f * c.dt, rhs, fmaf(0.75f, gn, 0.25f * sx[3]));
    } else {
        const float gn = __ldg(Gn + id);
        out = fmaf((2.0f / 3.0f) * c.dt, rhs, fmaf(1.0f / 3.0f, gn, (2.0f / 3.0f) * sx[3]));
    }
    Gout[id] = out;
}

// One HCR-2 pseudo-step (reinitStep3D, reinitialization.h:136-193) in FP32
// with the interface constraint in FP64: the crossing flags and
// r~ = phi0_c / sum(phi0 of crossing neighbours) (computeInterfaceCrossings3D,
// :46-89) are recomputed from phi0 in FP64, and on flagged cells the forcing
// and the update are formed in FP64 before the final rounding.
// The pseudo-step at one cell from its value phi, phi0 and the neighbour
// values pn / p0 in the order -x, +x, -y, +y (, -z, +z), in two parts: the
// FP32 Godunov term and the constraint's crossing flags / stability test
// (reinit_cell_f32), and the FP64 constrained update of a forced cell
// (reinit_forced_f64).
template <int DIM>
__device__ __forceinline__ float reinit_cell_f32(float phi, float ph0, const float* pn, const float* p0,
                                                 float inv_dx, float inv_dy, float inv_dz, float dx2,
                                                 int& flag, bool& forced) {
    const float S = ph0 * rsqrtf(fmaf(ph0, ph0, dx2));
    // Godunov term of an axis: max(a^2, b^2) with a = max(D-, 0), b = min(D+, 0)
    // for S > 0 and the mirrored choice otherwise.  Only the squares enter, so
    // with sg = +-1/h (exact sign flip) it is max(sg (phi - phi_-),
    // sg (phi - phi_+), 0)^2 -- the same rounded values, fewer operations.
    const float sg = S > 0.0f ? 1.0f : -1.0f;
    float gsq = 0.0f;
    const float inv[3] = {inv_dx, inv_dy, inv_dz};
#pragma unroll
    for (int ax = 0; ax < DIM; ++ax) {
        const float si = sg * inv[ax];
        const float m = fmaxf(fmaxf((phi - pn[2 * ax]) * si, (phi - pn[2 * ax + 1]) * si), 0.0f);
        gsq = __fadd_rn(gsq, __fmul_rn(m, m));
    }
    const float term = -S * (sqrtf(gsq) - 1.0f);

    // interface constraint.  The crossing test phi0_c * phi0_nb < 0 of
    // computeInterfaceCrossings3D is a sign test: the exact product of two
    // floats is never rounded to zero in FP64, so comparing signs in FP32
    // decides it identically; only flagged cells go on to FP64 arithmetic.
    flag = 0;
    // no crossing where phi0 and all its neighbours lie strictly on one side
    // (most cells): the per-neighbour tests below would all fail there
    float lo = p0[0], hi = p0[0];
#pragma unroll
    for (int q = 1; q < 2 * DIM; ++q) {
        lo = fminf(lo, p0[q]);
        hi = fmaxf(hi, p0[q]);
    }
    if (!((ph0 > 0.0f && lo > 0.0f) || (ph0 < 0.0f && hi < 0.0f))) {
#pragma unroll
        for (int q = 0; q < 2 * DIM; ++q)
            if ((ph0 < 0.0f && p0[q] > 0.0f) || (ph0 > 0.0f && p0[q] < 0.0f)) flag |= 1 << q;
    }
    bool stable = flag != 0 && (phi > 0.0f) == (ph0 > 0.0f);
#pragma unroll
    for (int q = 0; q < 2 * DIM; ++q)
        if ((flag >> q) & 1) stable = stable && ((pn[q] > 0.0f) == (p0[q] > 0.0f));
    forced = stable;
    return term;
}

// FP64 update of a forced cell: r~ from the crossing neighbours' phi0, the
// forcing beta (r~ sum(phi of crossing neighbours) - phi) / dx, and
// phi + dtau (term + forcing), rounded once to FP32.
template <int DIM>
__device__ __forceinline__ float reinit_forced_f64(float phi, float ph0, float term, int flag, const float* pn,
                                                   const float* p0, double dx, double dtau, double beta) {
    double sum0 = 0.0;
    int cnt = 0;
#pragma unroll
    for (int q = 0; q < 2 * DIM; ++q)
        if ((flag >> q) & 1) { sum0 += (double)p0[q]; cnt++; }
    const double rt = (cnt > 0 && fabs(sum0) > 1e-15) ? (double)ph0 / sum0 : 0.0;
    double sum = 0.0;
#pragma unroll
    for (int q = 0; q < 2 * DIM; ++q)
        if ((flag >> q) & 1) sum += (double)pn[q];
    const double forcing = beta * (rt * sum - (double)phi) / dx;
    return (float)((double)phi + dtau * ((double)term + forcing));
}

// Neighbour offset along one axis: +-stride inside, the periodic image or
// the clamped cell (offset 0) at the ends.
template <typename IDX>
__device__ __forceinline__ IDX nb_off(int c, int n, int bc, IDX stride, bool up) {
    if (up) return c < n - 1 ? stride : (bc == LSGB_BC_PERIODIC ? -(IDX)(n - 1) * stride : (IDX)0);
    return c > 0 ? -stride : (bc == LSGB_BC_PERIODIC ? (IDX)(n - 1) * stride : (IDX)0);
}

constexpr int RT = 256;  // threads of a pseudo-step block

// One pseudo-step, one thread per cell.  Forced cells (the interface band)
// are rare and their FP64 update is long, so a block queues them in shared
// memory and finishes them with dense lanes after the FP32 pass: a warp that
// holds one forced cell no longer runs the FP64 sequence for all 32 lanes.
template <int DIM, typename IDX>
__global__ void __launch_bounds__(RT) reinit_f32_kernel(Geo g, const float* __restrict__ phin,
                                                        const float* __restrict__ phi0,
                                                        float* __restrict__ phinew, float inv_dx,
                                                        float inv_dy, float inv_dz, float dx2,
                                                        float dtau_f, double dx, double dtau,
                                                        double beta) {
    __shared__ int nq;
    __shared__ IDX q_id[RT];
    __shared__ int q_flag[RT];
    __shared__ float q_phi[RT], q_ph0[RT], q_term[RT];
    __shared__ float q_pn[2 * DIM][RT], q_p0[2 * DIM][RT];
    const int t = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    if (t == 0) nq = 0;
    __syncthreads();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    int k = DIM == 3 ? blockIdx.z * blockDim.z + threadIdx.z : 0;
    if (i < g.nx && j < g.ny && k < g.nz) {
        const IDX sy = g.nx;
        const IDX sz = (IDX)g.nx * g.ny;
        const IDX id = (IDX)j * sy + (IDX)k * sz + i;
        IDX nb[6];
        nb[0] = id + nb_off<IDX>(i, g.nx, g.bcx, (IDX)1, false);
        nb[1] = id + nb_off<IDX>(i, g.nx, g.bcx, (IDX)1, true);
        nb[2] = id + nb_off<IDX>(j, g.ny, g.bcy, sy, false);
        nb[3] = id + nb_off<IDX>(j, g.ny, g.bcy, sy, true);
        if (DIM == 3) {
            nb[4] = id + nb_off<IDX>(k, g.nz, g.bcz, sz, false);
            nb[5] = id + nb_off<IDX>(k, g.nz, g.bcz, sz, true);
        }
        const float phi = __ldg(phin + id);
        const float ph0 = __ldg(phi0 + id);
        float pn[6], p0[6];
#pragma unroll
        for (int q = 0; q < 2 * DIM; ++q) {
            pn[q] = __ldg(phin + nb[q]);
            p0[q] = __ldg(phi0 + nb[q]);
        }
        int flag;
        bool forced;
        const float term = reinit_cell_f32<DIM>(phi, ph0, pn, p0, inv_dx, inv_dy, inv_dz, dx2, flag, forced);
        if (forced) {
            const int e = atomicAdd(&nq, 1);
            q_id[e] = id;
            q_flag[e] = flag;
            q_phi[e] = phi;
            q_ph0[e] = ph0;
            q_term[e] = term;
#pragma unroll
            for (int q = 0; q < 2 * DIM; ++q) {
                q_pn[q][e] = pn[q];
                q_p0[q][e] = p0[q];
            }
        } else {
            phinew[id] = fmaf(dtau_f, term, phi);
        }
    }
    __syncthreads();
    for (int e = t; e < nq; e += RT) {
        float pn[6], p0[6];
#pragma unroll
        for (int q = 0; q < 2 * DIM; ++q) {
            pn[q] = q_pn[q][e];
            p0[q] = q_p0[q][e];
        }
        phinew[q_id[e]] = reinit_forced_f64<DIM>(q_phi[e], q_ph0[e], q_term[e], q_flag[e], pn, p0, dx, dtau, beta);
    }
}

inline dim3 cell_block(const Geo& g) { return g.dim == 3 ? dim3(32, 4, 2) : dim3(32, 8, 1); }
inline dim3 cell_grid(const Geo& g, dim3 b) {
    return dim3((g.nx + b.x - 1) / b.x, (g.ny + b.y - 1) / b.y, (g.nz + b.z - 1) / b.z);
}

}  // namespace

cudaError_t launch_stage_f32(const StageArgs& a, cudaStream_t st) {
    if (a.lay.ghosted) return cudaErrorInvalidValue;  // FP32 fields are compact only
    F32Coef c;
    c.inv_dx = (float)(1.0 / a.dx);
    c.inv_dy = (float)(1.0 / a.dy);
    c.inv_dz = (float)(1.0 / a.dz);
    c.inv_2dx = (float)(1.0 / (2.0 * a.dx));
    c.inv_2dy = (float)(1.0 / (2.0 * a.dy));
    c.inv_2dz = (float)(1.0 / (2.0 * a.dz));
    c.s_l = (float)a.s_l;
    c.eps = (float)a.eps;
    c.dt = (float)a.dt;
    dim3 b = cell_block(a.g);
    if (a.g.dim == 2 && (a.tile == 2 || a.tile == 4)) b.y = a.tile;  // tuned 2D block height (32 x {2,4,8})
    dim3 gr = cell_grid(a.g, b);
    const float* Gin = (const float*)a.Gin;
    const float* Gn = (const float*)a.Gn;
    float* Gout = (float*)a.Gout;
    const float* u = (const float*)a.u;
    const float* v = (const float*)a.v;
    const float* w = (const float*)a.w;
    const float* sl = (const float*)a.sl;
#define LSGB_S32(D, S, I) stage_f32_kernel<D, S, I><<<gr, b, 0, st>>>(a.g, Gin, Gn, Gout, u, v, w, sl, c)
    if (a.g.dim == 3) return launch_stage3d_f32_tiled(a, a.err, st);
    if (a.g.cells() < (1LL << 31) - 1) {  // 32-bit element offsets
        if (a.stage == 1) LSGB_S32(2, 1, int); else if (a.stage == 2) LSGB_S32(2, 2, int); else LSGB_S32(2, 3, int);
    } else {
        if (a.stage == 1) LSGB_S32(2, 1, long long);
        else if (a.stage == 2) LSGB_S32(2, 2, long long);
        else LSGB_S32(2, 3, long long);
    }
#undef LSGB_S32
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_reinit_f32(const ReinitArgs& a, cudaStream_t st) {
    if (a.lay.ghosted) return cudaErrorInvalidValue;
    dim3 b = cell_block(a.g), gr = cell_grid(a.g, b);
    const float* pn = (const float*)a.phin;
    const float* p0 = (const float*)a.phi0;
    float* out = (float*)a.phinew;
    const float ix = (float)(1.0 / a.dx), iy = (float)(1.0 / a.dy), iz = (float)(1.0 / a.dz);
    const float dx2 = (float)(a.dx * a.dx);
    const bool small = a.g.cells() < (1LL << 31) - 1;  // 32-bit element offsets
#define LSGB_R32(D, I) reinit_f32_kernel<D, I><<<gr, b, 0, st>>>(a.g, pn, p0, out, ix, iy, iz, dx2, (float)a.dtau, \
                                                                  a.dx, a.dtau, a.beta)
    if (a.g.dim == 3) {
        if (small) LSGB_R32(3, int); else LSGB_R32(3, long long);
    } else {
        if (small) LSGB_R32(2, int); else LSGB_R32(2, long long);
    }
#undef LSGB_R32
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace lsgb
