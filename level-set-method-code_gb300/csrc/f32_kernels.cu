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
// The stage kernels themselves live in stage2d_f32.cu and stage3d_f32.cu;
// this file holds the HCR-2 pseudo-step and the stage dispatch.
#include "common.cuh"

namespace lsgb {
namespace {

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
    forced = false;
    // no crossing where phi0 and all its neighbours lie strictly on one side
    // (most cells): the per-neighbour tests below would all fail there.  The
    // tests run only in warps with a lane near the interface.
    float lo = p0[0], hi = p0[0];
#pragma unroll
    for (int q = 1; q < 2 * DIM; ++q) {
        lo = fminf(lo, p0[q]);
        hi = fmaxf(hi, p0[q]);
    }
    const bool near = !((ph0 > 0.0f && lo > 0.0f) || (ph0 < 0.0f && hi < 0.0f));
    // (the lanes of a warp that reach this point together: cells past the
    // grid's edge never do)
    if (__any_sync(__activemask(), near)) {
        if (near) {
#pragma unroll
            for (int q = 0; q < 2 * DIM; ++q)
                if ((ph0 < 0.0f && p0[q] > 0.0f) || (ph0 > 0.0f && p0[q] < 0.0f)) flag |= 1 << q;
        }
        bool stable = flag != 0 && (phi > 0.0f) == (ph0 > 0.0f);
#pragma unroll
        for (int q = 0; q < 2 * DIM; ++q)
            if ((flag >> q) & 1) stable = stable && ((pn[q] > 0.0f) == (p0[q] > 0.0f));
        forced = stable;
    }
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
// SAME: phin and phi0 are one array (the first pseudo-step of a
// reinitialisation), so each neighbour is loaded once.  phi0_copy (nullable)
// receives phi0 at every cell.  LOOP: the caller runs the body for several
// cell blocks in turn, so the forced-cell queue ends with a barrier.
template <int DIM, typename IDX, bool SAME = false, bool LOOP = false>
__device__ __forceinline__ void reinit_f32_body(const Geo& g, const float* __restrict__ phin,
                                                const float* __restrict__ phi0, float* __restrict__ phinew,
                                                float inv_dx, float inv_dy, float inv_dz, float dx2, float dtau_f,
                                                double dx, double dtau, double beta, int bx, int by, int bz,
                                                float* __restrict__ phi0_copy = nullptr) {
    __shared__ int nq;
    __shared__ IDX q_id[RT];
    __shared__ int q_flag[RT];
    __shared__ float q_phi[RT], q_ph0[RT], q_term[RT];
    __shared__ float q_pn[2 * DIM][RT], q_p0[2 * DIM][RT];
    const int t = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    // (ordered before the queue's first use by the barrier of __syncthreads_or)
    if (t == 0) nq = 0;
    bool forced = false;
    int i = bx * blockDim.x + threadIdx.x;
    int j = by * blockDim.y + threadIdx.y;
    int k = DIM == 3 ? bz * blockDim.z + threadIdx.z : 0;
    IDX c_id = 0;  // a forced cell's values until it is queued
    int c_flag = 0;
    float c_phi = 0.0f, c_ph0 = 0.0f, c_term = 0.0f, c_pn[6], c_p0[6];
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
        const float ph0 = __ldg(phi0 + id);
        const float phi = SAME ? ph0 : __ldg(phin + id);
        float pn[6], p0[6];
#pragma unroll
        for (int q = 0; q < 2 * DIM; ++q) {
            p0[q] = __ldg(phi0 + nb[q]);
            pn[q] = SAME ? p0[q] : __ldg(phin + nb[q]);
        }
        if (phi0_copy) phi0_copy[id] = ph0;
        int flag;
        const float term = reinit_cell_f32<DIM>(phi, ph0, pn, p0, inv_dx, inv_dy, inv_dz, dx2, flag, forced);
        if (forced) {
            c_id = id;
            c_flag = flag;
            c_phi = phi;
            c_ph0 = ph0;
            c_term = term;
#pragma unroll
            for (int q = 0; q < 2 * DIM; ++q) {
                c_pn[q] = pn[q];
                c_p0[q] = p0[q];
            }
        } else {
            phinew[id] = fmaf(dtau_f, term, phi);
        }
    }
    // most blocks hold no forced cell: one barrier and done
    if (!__syncthreads_or(forced)) return;
    if (forced) {
        const int e = atomicAdd(&nq, 1);
        q_id[e] = c_id;
        q_flag[e] = c_flag;
        q_phi[e] = c_phi;
        q_ph0[e] = c_ph0;
        q_term[e] = c_term;
#pragma unroll
        for (int q = 0; q < 2 * DIM; ++q) {
            q_pn[q][e] = c_pn[q];
            q_p0[q][e] = c_p0[q];
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
    if (LOOP) __syncthreads();  // the queue is free again for the next cell block
}

template <int DIM, typename IDX, bool SAME>
__global__ void __launch_bounds__(RT) reinit_f32_kernel(Geo g, const float* __restrict__ phin,
                                                        const float* __restrict__ phi0,
                                                        float* __restrict__ phinew, float inv_dx,
                                                        float inv_dy, float inv_dz, float dx2,
                                                        float dtau_f, double dx, double dtau,
                                                        double beta, float* __restrict__ phi0_copy) {
    reinit_f32_body<DIM, IDX, SAME>(g, phin, phi0, phinew, inv_dx, inv_dy, inv_dz, dx2, dtau_f, dx, dtau, beta,
                                    blockIdx.x, blockIdx.y, blockIdx.z, phi0_copy);
}

// One instance of the grouped HCR-2 and copy-back launches: buffers, the
// pseudo-step coefficients, its block grid (gx x gy x gz cell blocks) and its
// first block in the pseudo-step and copy launches.
struct GroupR {
    Geo g;
    float *G, *A, *B;
    float inv_dx, inv_dy, inv_dz, dx2, dtau_f;
    double dx, dtau, beta;
    int gx, gy, gz, blk0, cblk0;
};

// Cell blocks a grouped pseudo-step block works through, consecutive along
// the last axis (z in 3D, y in 2D): one descriptor fetch for all of them.
constexpr int RZL = 4;

constexpr int CPB = 4096;  // floats per block of the copy back

// Grouped HCR-2 pseudo-step `iter` of `iters` for every instance (same
// dimensionality); block b belongs to instance owner[b] and works through
// RZL cell blocks along the last axis.  Buffer roles: with an even count
// (copy_free) they are the handle's -- iteration 0 reads G as both fields,
// writes A and keeps phi0 in B; odd iterations A -> G and even ones G -> A,
// phi0 from B, so the result lands in G.  With an odd count phi0 stays in G,
// the iterations ping-pong A / B and copy_back_group moves the result.
template <int DIM, bool FIRST>
__global__ void __launch_bounds__(RT) reinit_f32_group(const GroupR* __restrict__ ins, const int* __restrict__ owner,
                                                       int iter, int copy_free) {
    const GroupR* d = ins + owner[blockIdx.x];
    int l = (int)blockIdx.x - d->blk0;
    const int bx = l % d->gx;
    l /= d->gx;
    const int last = DIM == 3 ? d->gz : d->gy;  // cell blocks along the last axis
    const int by0 = DIM == 3 ? l % d->gy : l * RZL;
    const int bz0 = DIM == 3 ? (l / d->gy) * RZL : 0;
    const Geo g = d->g;
    float* out;
    const float* in;
    const float* p0;
    float* p0_copy = nullptr;
    if (copy_free) {
        out = iter & 1 ? d->G : d->A;
        in = FIRST ? d->G : (iter & 1 ? d->A : d->G);
        p0 = FIRST ? d->G : d->B;
        if (FIRST) p0_copy = d->B;
    } else {
        out = iter & 1 ? d->B : d->A;
        in = FIRST ? d->G : ((iter - 1) & 1 ? d->B : d->A);
        p0 = d->G;
    }
    for (int q = 0; q < RZL; ++q) {
        const int by = DIM == 3 ? by0 : by0 + q, bz = DIM == 3 ? bz0 + q : 0;
        if ((DIM == 3 ? bz : by) >= last) break;  // the same for the whole block
        reinit_f32_body<DIM, int, FIRST, true>(g, in, p0, out, d->inv_dx, d->inv_dy, d->inv_dz, d->dx2, d->dtau_f,
                                               d->dx, d->dtau, d->beta, bx, by, bz, p0_copy);
    }
}

// G <- the buffer the last of `iters` pseudo-steps wrote, every instance.
__global__ void __launch_bounds__(256) copy_back_group(const GroupR* __restrict__ ins, const int* __restrict__ owner,
                                                       int iters) {
    const GroupR* d = ins + owner[blockIdx.x];
    const float* src = (iters - 1) & 1 ? d->B : d->A;
    const long long cells = d->g.cells();
    const long long e0 = (long long)((int)blockIdx.x - d->cblk0) * CPB;
    const long long e1 = e0 + CPB < cells ? e0 + CPB : cells;
    for (long long e = e0 + threadIdx.x; e < e1; e += 256) d->G[e] = src[e];
}

inline dim3 cell_block(const Geo& g) { return g.dim == 3 ? dim3(32, 4, 2) : dim3(32, 8, 1); }
inline dim3 cell_grid(const Geo& g, dim3 b) {
    return dim3((g.nx + b.x - 1) / b.x, (g.ny + b.y - 1) / b.y, (g.nz + b.z - 1) / b.z);
}

}  // namespace

cudaError_t launch_stage_f32(const StageArgs& a, cudaStream_t st) {
    if (a.lay.ghosted) return cudaErrorInvalidValue;  // FP32 fields are compact only
    if (a.g.dim == 3) return launch_stage3d_f32_tiled(a, a.err, st);
    return launch_stage2d_f32_tiled(a, st);
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
    const bool same = pn == p0;
    float* cp = (float*)a.phi0_copy;
#define LSGB_R32(D, I, SM) reinit_f32_kernel<D, I, SM><<<gr, b, 0, st>>>(a.g, pn, p0, out, ix, iy, iz, dx2, \
                                                                          (float)a.dtau, a.dx, a.dtau, a.beta, cp)
    if (a.g.dim == 3) {
        if (small) { if (same) LSGB_R32(3, int, true); else LSGB_R32(3, int, false); }
        else { if (same) LSGB_R32(3, long long, true); else LSGB_R32(3, long long, false); }
    } else {
        if (small) { if (same) LSGB_R32(2, int, true); else LSGB_R32(2, int, false); }
        else { if (same) LSGB_R32(2, long long, true); else LSGB_R32(2, long long, false); }
    }
#undef LSGB_R32
    count_launches(1);
    return cudaGetLastError();
}

size_t groupr_desc_bytes() { return sizeof(GroupR); }

void groupr_fill(const GroupInst* in, int n, void* host_table, std::vector<int>& owner,
                 std::vector<int>& copy_owner) {
    GroupR* d = (GroupR*)host_table;
    long long blk = 0, cblk = 0;
    for (int q = 0; q < n; ++q) {
        GroupR e;
        memset(&e, 0, sizeof(e));
        const StageArgs& a = in[q].a;
        e.g = a.g;
        e.G = in[q].G;
        e.A = in[q].A;
        e.B = in[q].B;
        const double dz = a.g.dim == 3 ? a.dz : a.dx;
        e.inv_dx = (float)(1.0 / a.dx);
        e.inv_dy = (float)(1.0 / a.dy);
        e.inv_dz = (float)(1.0 / dz);
        e.dx2 = (float)(a.dx * a.dx);
        e.dtau_f = (float)in[q].dtau;
        e.dx = a.dx;
        e.dtau = in[q].dtau;
        e.beta = in[q].beta;
        const dim3 b = cell_block(a.g), gr = cell_grid(a.g, b);
        e.gx = (int)gr.x;
        e.gy = (int)gr.y;
        e.gz = (int)gr.z;
        e.blk0 = (int)blk;
        e.cblk0 = (int)cblk;
        // blocks of RZL cell blocks along the last axis
        const long long nb = a.g.dim == 3 ? (long long)gr.x * gr.y * ((gr.z + RZL - 1) / RZL)
                                          : (long long)gr.x * ((gr.y + RZL - 1) / RZL);
        const long long nc = (a.g.cells() + CPB - 1) / CPB;
        blk += nb;
        cblk += nc;
        owner.insert(owner.end(), (size_t)nb, q);
        copy_owner.insert(copy_owner.end(), (size_t)nc, q);
        d[q] = e;
    }
}

cudaError_t launch_reinit_f32_group(const void* table, const int* owner, int n, long long blocks, int dim, int iter,
                                    int iters, cudaStream_t st) {
    if (n <= 0 || blocks <= 0) return cudaSuccess;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
    const GroupR* d = (const GroupR*)table;
    const unsigned nb = (unsigned)blocks;
    const int cf = iters % 2 == 0;
    if (dim == 3) {
        if (iter == 0) reinit_f32_group<3, true><<<nb, dim3(32, 4, 2), 0, st>>>(d, owner, iter, cf);
        else reinit_f32_group<3, false><<<nb, dim3(32, 4, 2), 0, st>>>(d, owner, iter, cf);
    } else {
        if (iter == 0) reinit_f32_group<2, true><<<nb, dim3(32, 8, 1), 0, st>>>(d, owner, iter, cf);
        else reinit_f32_group<2, false><<<nb, dim3(32, 8, 1), 0, st>>>(d, owner, iter, cf);
    }
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_copy_back_group(const void* table, const int* copy_owner, int n, long long copy_blocks, int iters,
                                   cudaStream_t st) {
    // an even count leaves the result in G (reinit_f32_group's buffer roles)
    if (n <= 0 || copy_blocks <= 0 || iters <= 0 || iters % 2 == 0) return cudaSuccess;
    if (copy_blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
    copy_back_group<<<(unsigned)copy_blocks, 256, 0, st>>>((const GroupR*)table, copy_owner, iters);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace lsgb
