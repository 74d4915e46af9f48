// f64_kernels.cu -- FP64 kernels that reproduce the reference's arithmetic.
//
// Compiled with --fmad=false: every a*b+c below stays a rounded multiply and a
// rounded add, divisions and sqrt are IEEE round-to-nearest (a quotient by a
// known or shared divisor is formed as a corrected product, div_rn, which
// gives the same bits), and expressions keep the reference's evaluation order.  With the same inputs the results
// are bit-identical to the reference CPU solver
// (Local_code/level-set_MPI_3D/include/{weno5,rk3,reinitialization}.h and the
// 2D twins), which tests/test_gpu_parity.py checks.
//
// Kernel shapes: one thread per interior cell (blocks of 32 x 4 x 2 in 3D,
// 32 x 8 in 2D).  FP64 on GB300 runs far below the HBM roof (the step is
// bound by the FP64 pipe), so these kernels
// favour exactness and simple addressing; the throughput path is the FP32 form
// in f32_kernels.cu.
#include "common.cuh"
#include "fp64_exact.cuh"

namespace lsgb {
namespace {

constexpr double WENO_EPS = 1.0e-6;  // weno5.h:22

// Smoothness indicator of the triple (a, b, c) = (v[k], v[k+1], v[k+2]),
// computeSmoothnessIndicators, weno5.h:28-37 (non-standard second term).
__device__ __forceinline__ double sm_beta(double a, double b, double c) {
    double d2 = c - mul_pow2<1>(b) + a;
    const double h = c - a;
    return (13.0 / 12.0) * d2 * d2 + mul_pow2<-2>(h) * h;
}

// weno5_left, weno5.h:39-58: value at i+1/2 from G[i-2..i+2].
__device__ __forceinline__ double weno_left(double v0, double v1, double v2, double v3, double v4) {
    double b0 = sm_beta(v0, v1, v2);
    double b1 = sm_beta(v1, v2, v3);
    double b2 = sm_beta(v2, v3, v4);
    double a0 = 0.1 / ((WENO_EPS + b0) * (WENO_EPS + b0));
    double a1 = 0.6 / ((WENO_EPS + b1) * (WENO_EPS + b1));
    double a2 = 0.3 / ((WENO_EPS + b2) * (WENO_EPS + b2));
    double s = a0 + a1 + a2;
    const double rs = 1.0 / s;
    double w0 = div_rn(a0, s, rs), w1 = div_rn(a1, s, rs), w2 = div_rn(a2, s, rs);
    double p0 = div_rn(mul_pow2<1>(v0) - 7.0 * v1 + 11.0 * v2, 6.0, RCP6);
    double p1 = div_rn(-v1 + 5.0 * v2 + mul_pow2<1>(v3), 6.0, RCP6);
    double p2 = div_rn(mul_pow2<1>(v2) + 5.0 * v3 - v4, 6.0, RCP6);
    return w0 * p0 + w1 * p1 + w2 * p2;
}

// weno5_right, weno5.h:60-81: value at i-1/2 from G[i-2..i+2]; indicators
// on the mirrored stencil.
__device__ __forceinline__ double weno_right(double v0, double v1, double v2, double v3, double v4) {
    double b0 = sm_beta(v4, v3, v2);
    double b1 = sm_beta(v3, v2, v1);
    double b2 = sm_beta(v2, v1, v0);
    double a0 = 0.3 / ((WENO_EPS + b0) * (WENO_EPS + b0));
    double a1 = 0.6 / ((WENO_EPS + b1) * (WENO_EPS + b1));
    double a2 = 0.1 / ((WENO_EPS + b2) * (WENO_EPS + b2));
    double s = a0 + a1 + a2;
    const double rs = 1.0 / s;
    double w0 = div_rn(a0, s, rs), w1 = div_rn(a1, s, rs), w2 = div_rn(a2, s, rs);
    double p0 = div_rn(11.0 * v2 - 7.0 * v3 + mul_pow2<1>(v4), 6.0, RCP6);
    double p1 = div_rn(mul_pow2<1>(v1) + 5.0 * v2 - v3, 6.0, RCP6);
    double p2 = div_rn(-v0 + 5.0 * v1 + mul_pow2<1>(v2), 6.0, RCP6);
    return w0 * p0 + w1 * p1 + w2 * p2;
}

// weno5_dx_3d / _dy_3d / _dz_3d (weno5.h:90-196): s[0..6] = G[i-3..i+3]
// along the axis; branch on vel >= 0 (weno5.h:99).  rh = RN(1 / h).
__device__ __forceinline__ double weno_deriv(const double* s, double vel, double h, double rh) {
    double gl, gr;
    if (vel >= 0.0) {
        gl = weno_left(s[0], s[1], s[2], s[3], s[4]);
        gr = weno_left(s[1], s[2], s[3], s[4], s[5]);
    } else {
        gl = weno_right(s[1], s[2], s[3], s[4], s[5]);
        gr = weno_right(s[2], s[3], s[4], s[5], s[6]);
    }
    return div_rn(gr - gl, h, rh);
}

// Stencil reader: element offset of interior coordinate (i + d) etc.  In the
// ghosted layout the neighbours are read from the ghost cells the caller's
// boundary fill left (as the reference does); in the compact layout the
// coordinates wrap / clamp.
template <bool GH>
struct Nb {
    long long sy, sz;
    int i, j, k, nx, ny, nz, bcx, bcy, bcz;
    long long row;  // j*sy + k*sz of the centre

    __device__ __forceinline__ long long c() const { return row + i; }
    __device__ __forceinline__ long long x(int d) const {
        return GH ? row + i + d : row + map_axis(i + d, nx, bcx);
    }
    __device__ __forceinline__ long long y(int d) const {
        return GH ? row + i + d * sy : (long long)map_axis(j + d, ny, bcy) * sy + (long long)k * sz + i;
    }
    __device__ __forceinline__ long long z(int d) const {
        return GH ? row + i + d * sz : (long long)map_axis(k + d, nz, bcz) * sz + (long long)j * sy + i;
    }
};

template <bool GH>
__device__ __forceinline__ Nb<GH> make_nb(const Geo& g, const Lay& lay, int i, int j, int k) {
    Nb<GH> n;
    n.sy = lay.sy; n.sz = lay.sz;
    n.i = i; n.j = j; n.k = k;
    n.nx = g.nx; n.ny = g.ny; n.nz = g.nz;
    n.bcx = g.bcx; n.bcy = g.bcy; n.bcz = g.bcz;
    n.row = (long long)j * lay.sy + (long long)k * lay.sz;
    return n;
}

// Fused RK3 stage: rhs of computeRHS3D (rk3.h:31-81) / computeRHS (2D
// rk3.h:54-98) at the cell, combined as rk3Stage{1,2,3}_3D (rk3.h:87-121).
template <int DIM, int STAGE, bool GH>
__global__ void __launch_bounds__(256) stage_f64_kernel(StageArgs a) {
    const Geo g = a.g;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    int k = DIM == 3 ? blockIdx.z * blockDim.z + threadIdx.z : 0;
    if (i >= g.nx || j >= g.ny || k >= g.nz) return;
    const double* __restrict__ G = (const double*)a.Gin + a.lay.off;
    const Nb<GH> n = make_nb<GH>(g, a.lay, i, j, k);
    const long long id = n.c();

    double sx[7], sy[7], sz[7];
#pragma unroll
    for (int d = -3; d <= 3; ++d) {
        sx[d + 3] = G[n.x(d)];
        sy[d + 3] = G[n.y(d)];
        if (DIM == 3) sz[d + 3] = G[n.z(d)];
    }

    double s_l = a.sl ? ((const double*)a.sl)[a.lay.off + id] : a.s_l;
    double gx = 0.0, gy = 0.0, gz = 0.0, gm = 1.0, rgm = 1.0;
    const double hx2 = 2.0 * a.dx, hy2 = 2.0 * a.dy, hz2 = 2.0 * a.dz;
    if (s_l > a.eps) {
        gx = div_rn(sx[4] - sx[2], hx2, 1.0 / hx2);
        gy = div_rn(sy[4] - sy[2], hy2, 1.0 / hy2);
        if (DIM == 3) {
            gz = div_rn(sz[4] - sz[2], hz2, 1.0 / hz2);
            gm = sqrt(gx * gx + gy * gy + gz * gz + a.eps);
        } else {
            gm = sqrt(gx * gx + gy * gy + a.eps);
        }
        rgm = 1.0 / gm;
    }
    const double ue = ((const double*)a.u)[a.lay.off + id] - div_rn(s_l * gx, gm, rgm);
    const double ve = ((const double*)a.v)[a.lay.off + id] - div_rn(s_l * gy, gm, rgm);
    double rhs;
    if (DIM == 3) {
        const double we = ((const double*)a.w)[a.lay.off + id] - div_rn(s_l * gz, gm, rgm);
        double dgx = weno_deriv(sx, ue, a.dx, 1.0 / a.dx);
        double dgy = weno_deriv(sy, ve, a.dy, 1.0 / a.dy);
        double dgz = weno_deriv(sz, we, a.dz, 1.0 / a.dz);
        rhs = -(ue * dgx + ve * dgy + we * dgz);
    } else {
        double dgx = weno_deriv(sx, ue, a.dx, 1.0 / a.dx);
        double dgy = weno_deriv(sy, ve, a.dy, 1.0 / a.dy);
        rhs = -(ue * dgx + ve * dgy);
    }

    const double dt = a.dt;
    double out;
    if (STAGE == 1) {
        out = sx[3] + dt * rhs;  // G_n + dt L(G_n), Gin == Gn
    } else if (STAGE == 2) {
        const double gn = ((const double*)a.Gn)[a.lay.off + id];
        out = 0.75 * gn + 0.25 * sx[3] + 0.25 * dt * rhs;
    } else {
        const double gn = ((const double*)a.Gn)[a.lay.off + id];
        const double a0 = 1.0 / 3.0, a2 = 2.0 / 3.0, b3 = 2.0 / 3.0;
        out = a0 * gn + a2 * sx[3] + b3 * dt * rhs;
    }
    ((double*)a.Gout)[a.lay.off + id] = out;
}

// ---- face-shared FP64 stage ------------------------------------------------
//
// The same stage, computing each WENO face value once.  Cell i's right face
// and cell i+1's left face are the same reconstruction of the same five
// values when both cells are upwinded the same way, so the value is shared;
// a face between cells of opposite upwind directions needs both biases.  A
// CTA owns a tile of cells (3D 32 x 8 x 3, 2D 32 x 16; block 32 x 8, three
// or two cells per thread) and works in four phases over the tile staged with its
// 3-cell halo in shared memory:
//   1. u_eff of every cell (the reference's operations), its upwind bias per
//      axis into shared memory;
//   2. the list of (face, bias) reconstructions the tile's cells use, one
//      entry per needed value, compacted by a block scan;
//   3. the list evaluated densely, one entry per thread at a time (about 3.4
//      reconstructions per cell in place of 6, each with 4 IEEE divisions
//      and 6 quotients by a known reciprocal);
//   4. per cell, (face right - face left) / h per axis, the rhs and the stage
//      combination, as stage_f64_kernel.
// Every face value is the reference's weno5_left / weno5_right of the same
// five samples (weno_either), so the fields are bit-identical to
// stage_f64_kernel's.

// weno5_left(v) (right = false) or weno5_right(v) (right = true) in one code
// path: weno5_right evaluates the indicators on the mirrored stencil m with
// the linear weights (0.3, 0.6, 0.1), and its candidate polynomials group
// their terms differently; each polynomial's two operand orders are picked
// per bias, so every rounding is the reference's.
__device__ __forceinline__ double weno_either(double v0, double v1, double v2, double v3, double v4, bool right) {
    const double m0 = right ? v4 : v0, m1 = right ? v3 : v1, m2 = v2, m3 = right ? v1 : v3, m4 = right ? v0 : v4;
    const double b0 = sm_beta(m0, m1, m2);
    const double b1 = sm_beta(m1, m2, m3);
    const double b2 = sm_beta(m2, m3, m4);
    const double d0 = right ? 0.3 : 0.1, d2 = right ? 0.1 : 0.3;
    const double a0 = d0 / ((WENO_EPS + b0) * (WENO_EPS + b0));
    const double a1 = 0.6 / ((WENO_EPS + b1) * (WENO_EPS + b1));
    const double a2 = d2 / ((WENO_EPS + b2) * (WENO_EPS + b2));
    const double s = a0 + a1 + a2;
    // the three weights share one reciprocal; every quotient is still IEEE's
    const double rs = 1.0 / s;
    const double w0 = div_rn(a0, s, rs), w1 = div_rn(a1, s, rs), w2 = div_rn(a2, s, rs);
    // left (2 v0 - 7 v1) + 11 v2; right (11 v2 - 7 v3) + 2 v4
    const double t0 = mul_pow2<1>(m0), t2 = 11.0 * m2;
    const double p0 = div_rn((right ? t2 : t0) - 7.0 * m1 + (right ? t0 : t2), 6.0, RCP6);
    // left (-v1 + 5 v2) + 2 v3; right (2 v1 + 5 v2) - v3
    const double n1 = -m1, u3 = mul_pow2<1>(m3);
    const double p1 = div_rn((right ? u3 : n1) + 5.0 * m2 + (right ? n1 : u3), 6.0, RCP6);
    // left (2 v2 + 5 v3) - v4; right (-v0 + 5 v1) + 2 v2
    const double u2 = mul_pow2<1>(m2), n4 = -m4;
    const double p2 = div_rn((right ? n4 : u2) + 5.0 * m3 + (right ? u2 : n4), 6.0, RCP6);
    return w0 * p0 + w1 * p1 + w2 * p2;
}

template <int DIM>
struct FaceTile {
    static constexpr int TX = 32, TY = DIM == 3 ? 8 : 16, TZ = DIM == 3 ? 3 : 1;
    static constexpr int NT = 256, CPT = TX * TY * TZ / NT;  // threads, cells per thread
    static constexpr int SX = TX + 6, SY = TY + 6, SZ = DIM == 3 ? TZ + 6 : 1;
    static constexpr int NFX = (TX + 1) * TY * TZ, NFY = TX * (TY + 1) * TZ;
    static constexpr int NFZ = DIM == 3 ? TX * TY * (TZ + 1) : 0;
    static constexpr int NF = NFX + NFY + NFZ;
    static constexpr int NCELL = TX * TY * TZ;
    // dynamic shared memory: staged G, face values [NF][2], task list, biases, scan
    static constexpr size_t OFF_FV = sizeof(double) * SX * SY * SZ;
    static constexpr size_t OFF_TASK = OFF_FV + sizeof(double) * 2 * NF;
    static constexpr size_t OFF_BIAS = OFF_TASK + sizeof(int) * 2 * NF;
    static constexpr size_t OFF_SCAN = OFF_BIAS + NCELL;
    static constexpr size_t BYTES = OFF_SCAN + sizeof(int) * (NT + 1);
};

// Tile-local face f: its axis and the tile coordinates of the cell on its
// low side (which may be -1 on the axis).
template <int DIM>
__device__ __forceinline__ void face_of(int f, int& ax, int& cx, int& cy, int& cz) {
    using T = FaceTile<DIM>;
    if (f < T::NFX) {
        ax = 0;
        cx = f % (T::TX + 1) - 1;
        const int r = f / (T::TX + 1);
        cy = r % T::TY;
        cz = r / T::TY;
    } else if (f < T::NFX + T::NFY) {
        const int q = f - T::NFX;
        ax = 1;
        cx = q % T::TX;
        const int r = q / T::TX;
        cy = r % (T::TY + 1) - 1;
        cz = r / (T::TY + 1);
    } else {
        const int q = f - T::NFX - T::NFY;
        ax = 2;
        cx = q % T::TX;
        const int r = q / T::TX;
        cy = r % T::TY;
        cz = r / T::TY - 1;
    }
}

// Face ids on the low and high side of cell (cx, cy, cz) along axis ax.
template <int DIM>
__device__ __forceinline__ int face_id(int ax, int cx, int cy, int cz, int hi) {
    using T = FaceTile<DIM>;
    if (ax == 0) return (cz * T::TY + cy) * (T::TX + 1) + cx + hi;
    if (ax == 1) return T::NFX + (cz * (T::TY + 1) + cy + hi) * T::TX + cx;
    return T::NFX + T::NFY + ((cz + hi) * T::TY + cy) * T::TX + cx;
}

template <int DIM, int STAGE, bool GH>
__global__ void __launch_bounds__(256) stage_f64_faces(StageArgs a) {
    using T = FaceTile<DIM>;
    extern __shared__ __align__(16) unsigned char fsm[];
    double* Gs = (double*)fsm;                    // [SZ][SY][SX], tile origin at (3, 3, 3)
    double* fv = (double*)(fsm + T::OFF_FV);      // [NF][2]: bias 0 = left-biased, 1 = right-biased
    int* task = (int*)(fsm + T::OFF_TASK);
    unsigned char* bias = fsm + T::OFF_BIAS;      // per cell: bit ax set = u_eff(ax) < 0 (right-biased)
    int* scan = (int*)(fsm + T::OFF_SCAN);
    const Geo g = a.g;
    const int t = threadIdx.y * 32 + threadIdx.x;
    const int i0 = blockIdx.x * T::TX, j0 = blockIdx.y * T::TY, k0 = DIM == 3 ? blockIdx.z * T::TZ : 0;
    const double* __restrict__ G = (const double*)a.Gin + a.lay.off;
    const long long sy = a.lay.sy, sz = a.lay.sz;

    // ---- stage the tile and its halo.  Coordinates within 3 of the grid come
    // from the ghost cells (ghosted layout) or wrap / clamp (compact); positions
    // further out belong only to cells past the grid edge and are clamped.
    auto coord = [](int x, int n, int bc) {
        if (GH) return x < -NG ? -NG : (x > n + NG - 1 ? n + NG - 1 : x);
        if (x < -NG || x > n + NG - 1) return x < 0 ? 0 : n - 1;
        return map_axis(x, n, bc);
    };
    for (int e = t; e < T::SX * T::SY * T::SZ; e += T::NT) {
        const int lx = e % T::SX, ly = (e / T::SX) % T::SY, lz = e / (T::SX * T::SY);
        const int x = coord(i0 + lx - 3, g.nx, g.bcx), y = coord(j0 + ly - 3, g.ny, g.bcy);
        const int z = DIM == 3 ? coord(k0 + lz - 3, g.nz, g.bcz) : 0;
        Gs[e] = G[(long long)z * sz + (long long)y * sy + x];
    }
    __syncthreads();

    // ---- 1. u_eff and the upwind bias of the own cells (stage_f64_kernel's
    // operations; quotients by a known reciprocal, div_rn)
    const double h2[3] = {2.0 * a.dx, 2.0 * a.dy, 2.0 * a.dz};
    const double rh2[3] = {1.0 / h2[0], 1.0 / h2[1], 1.0 / h2[2]};
    double ue[T::CPT], ve[T::CPT], we[T::CPT];
#pragma unroll
    for (int q = 0; q < T::CPT; ++q) {
        const int c = t + q * T::NT;
        const int cx = c % T::TX, cy = (c / T::TX) % T::TY, cz = c / (T::TX * T::TY);
        const int i = i0 + cx, j = j0 + cy, k = k0 + cz;
        ue[q] = ve[q] = we[q] = 0.0;
        unsigned char b = 0;
        if (i < g.nx && j < g.ny && k < g.nz) {
            const double* P = Gs + ((cz + (DIM == 3 ? 3 : 0)) * T::SY + cy + 3) * T::SX + cx + 3;
            const long long id = (long long)k * sz + (long long)j * sy + i;
            const double s_l = a.sl ? ((const double*)a.sl)[a.lay.off + id] : a.s_l;
            double gx = 0.0, gy = 0.0, gz = 0.0, gm = 1.0, rgm = 1.0;
            if (s_l > a.eps) {
                gx = div_rn(P[1] - P[-1], h2[0], rh2[0]);
                gy = div_rn(P[T::SX] - P[-T::SX], h2[1], rh2[1]);
                if (DIM == 3) {
                    gz = div_rn(P[T::SX * T::SY] - P[-T::SX * T::SY], h2[2], rh2[2]);
                    gm = sqrt(gx * gx + gy * gy + gz * gz + a.eps);
                } else {
                    gm = sqrt(gx * gx + gy * gy + a.eps);
                }
                rgm = 1.0 / gm;
            }
            ue[q] = ((const double*)a.u)[a.lay.off + id] - div_rn(s_l * gx, gm, rgm);
            ve[q] = ((const double*)a.v)[a.lay.off + id] - div_rn(s_l * gy, gm, rgm);
            if (DIM == 3) we[q] = ((const double*)a.w)[a.lay.off + id] - div_rn(s_l * gz, gm, rgm);
            b = (ue[q] >= 0.0 ? 0 : 1) | (ve[q] >= 0.0 ? 0 : 2) | (DIM == 3 && !(we[q] >= 0.0) ? 4 : 0);
        }
        bias[c] = b;
    }
    __syncthreads();

    // ---- 2. the needed (face, bias) values: a face serves the tile cells on
    // either side that lie in the grid, each with its own bias
    auto in_grid = [&](int cx, int cy, int cz) {
        return cx >= 0 && cx < T::TX && cy >= 0 && cy < T::TY && cz >= 0 && cz < T::TZ && i0 + cx < g.nx &&
               j0 + cy < g.ny && k0 + cz < g.nz;
    };
    auto needs = [&](int f) {
        int ax, cx, cy, cz;
        face_of<DIM>(f, ax, cx, cy, cz);
        const int dx = ax == 0, dy = ax == 1, dz = ax == 2;
        int m = 0;
        if (in_grid(cx, cy, cz)) m |= 1 << ((bias[(cz * T::TY + cy) * T::TX + cx] >> ax) & 1);
        if (in_grid(cx + dx, cy + dy, cz + dz))
            m |= 1 << ((bias[((cz + dz) * T::TY + cy + dy) * T::TX + cx + dx] >> ax) & 1);
        return m;  // bit 0: left-biased value, bit 1: right-biased value
    };
    int cnt = 0;
    for (int f = t; f < T::NF; f += T::NT) cnt += __popc(needs(f));
    scan[t] = cnt;
    __syncthreads();
    for (int o = 1; o < T::NT; o <<= 1) {  // inclusive scan of the counts
        const int add = t >= o ? scan[t - o] : 0;
        __syncthreads();
        scan[t] += add;
        __syncthreads();
    }
    int pos = scan[t] - cnt;
    const int ntask = scan[T::NT - 1];
    for (int f = t; f < T::NF; f += T::NT) {
        const int m = needs(f);
        if (m & 1) task[pos++] = 2 * f;
        if (m & 2) task[pos++] = 2 * f + 1;
    }
    __syncthreads();

    // ---- 3. the values: face f between tile cells c and c + e_ax; the
    // left-biased value reads G[c-2 .. c+2], the right-biased G[c-1 .. c+3]
    for (int q = t; q < ntask; q += T::NT) {
        const int f = task[q] >> 1;
        const bool right = task[q] & 1;
        int ax, cx, cy, cz;
        face_of<DIM>(f, ax, cx, cy, cz);
        const int st = ax == 0 ? 1 : (ax == 1 ? T::SX : T::SX * T::SY);
        const double* P = Gs + ((cz + (DIM == 3 ? 3 : 0)) * T::SY + cy + 3) * T::SX + cx + 3 + (right ? st : 0);
        fv[2 * f + (right ? 1 : 0)] = weno_either(P[-2 * st], P[-st], P[0], P[st], P[2 * st], right);
    }
    __syncthreads();

    // ---- 4. derivatives, rhs, stage combination
    const double dt = a.dt;
    const double rh[3] = {1.0 / a.dx, 1.0 / a.dy, 1.0 / a.dz};
#pragma unroll
    for (int q = 0; q < T::CPT; ++q) {
        const int c = t + q * T::NT;
        const int cx = c % T::TX, cy = (c / T::TX) % T::TY, cz = c / (T::TX * T::TY);
        const int i = i0 + cx, j = j0 + cy, k = k0 + cz;
        if (!(i < g.nx && j < g.ny && k < g.nz)) continue;
        const int b = bias[c];
        auto deriv = [&](int ax, double h) {
            const int r = (b >> ax) & 1;
            return div_rn(fv[2 * face_id<DIM>(ax, cx, cy, cz, 1) + r] - fv[2 * face_id<DIM>(ax, cx, cy, cz, 0) + r], h,
                          rh[ax]);
        };
        double rhs;
        if (DIM == 3) {
            const double dgx = deriv(0, a.dx), dgy = deriv(1, a.dy), dgz = deriv(2, a.dz);
            rhs = -(ue[q] * dgx + ve[q] * dgy + we[q] * dgz);
        } else {
            const double dgx = deriv(0, a.dx), dgy = deriv(1, a.dy);
            rhs = -(ue[q] * dgx + ve[q] * dgy);
        }
        const long long id = (long long)k * sz + (long long)j * sy + i;
        const double gc = Gs[((cz + (DIM == 3 ? 3 : 0)) * T::SY + cy + 3) * T::SX + cx + 3];
        double out;
        if (STAGE == 1) {
            out = gc + dt * rhs;
        } else if (STAGE == 2) {
            const double gn = ((const double*)a.Gn)[a.lay.off + id];
            out = 0.75 * gn + 0.25 * gc + 0.25 * dt * rhs;
        } else {
            const double gn = ((const double*)a.Gn)[a.lay.off + id];
            const double a0 = 1.0 / 3.0, a2 = 2.0 / 3.0, b3 = 2.0 / 3.0;
            out = a0 * gn + a2 * gc + b3 * dt * rhs;
        }
        ((double*)a.Gout)[a.lay.off + id] = out;
    }
}

// div_rn against IEEE division on n seeded pairs: divisors are the solver's
// (6, 2^-9, 1/192, 1/200, 2/512, sums of WENO weights) and random ones in
// [2^-40, 2^40]; dividends are random in [2^-80, 2^80] with either sign,
// exact multiples of the divisor, and values next to a rounding midpoint of
// the quotient.  Also mul_pow2 against the FP64 multiply on values over the
// whole exponent range (subnormals, zeros and the largest finite values
// included).  Mismatching bit patterns are counted.
__device__ __forceinline__ uint64_t mix64(uint64_t x) {
    x += 0x9e3779b97f4a7c15ULL;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
    return x ^ (x >> 31);
}

__device__ __forceinline__ double rand_in(uint64_t bits, int emin, int emax) {
    const int e = emin + (int)((bits >> 52) % (uint64_t)(emax - emin + 1));
    return ldexp(1.0 + (double)(bits & ((1ULL << 52) - 1)) * 0x1p-52, e);
}

__global__ void div_check_kernel(long long n, uint64_t seed, unsigned long long* bad) {
    unsigned long long local = 0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const uint64_t h0 = mix64(seed ^ (uint64_t)e), h1 = mix64(h0), h2 = mix64(h1), h3 = mix64(h2);
        double b;
        switch (h0 % 8) {
            case 0: b = 6.0; break;
            case 1: b = 0x1p-9; break;
            case 2: b = 1.0 / 192.0; break;
            case 3: b = 1.0 / 200.0; break;
            case 4: b = 2.0 / 512.0; break;
            case 5: b = rand_in(h1, -3, 40); break;  // WENO weight sums
            default: b = rand_in(h1, -40, 40); break;
        }
        double a;
        switch (h2 % 4) {
            case 0: a = (double)(long long)(h3 % 2000001) - 1000000.0; a = a * b; break;  // exact quotients
            case 1: {  // next to a rounding midpoint: RN(b (q + ulp(q) / 2)) moved by -8 .. 7 ulps
                const double q = rand_in(h3, -20, 20);
                a = __fma_rn(b, q, b * ldexp(0.5, ilogb(q) - 52));
                a += (double)((int)(h3 >> 60) - 8) * ldexp(1.0, ilogb(a) - 52);
                break;
            }
            default: a = rand_in(h3, -80, 80); break;
        }
        if (h2 & 16) a = -a;
        if (h2 & 32) b = -b;
        const double y = 1.0 / b;
        const double r = div_rn(a, b, y), ref = a / b;
        if (__double_as_longlong(r) != __double_as_longlong(ref)) local++;
        // any bit pattern but NaN: every exponent field, either sign
        const uint64_t h4 = mix64(h3);
        double x = __longlong_as_double((long long)(h4 & 0xfffffffffffffULL) |
                                        (long long)((h4 >> 52) % 0x7ffULL) << 52);
        if (h4 & (1ULL << 63)) x = -x;
        if ((h2 >> 8) % 64 == 0) x = (h4 & 1) ? 0.0 : -0.0;
        const double pr[4] = {mul_pow2<1>(x), mul_pow2<2>(x), mul_pow2<-1>(x), mul_pow2<-2>(x)};
        const double pe[4] = {x * 2.0, x * 4.0, x * 0.5, x * 0.25};
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (__double_as_longlong(pr[q]) != __double_as_longlong(pe[q])) local++;
    }
    if (local) atomicAdd(bad, local);
}

// Godunov first-order |grad phi|^2 term of one axis by sign(S),
// weno5_gradient_magnitude_3d (weno5.h:202-248).
__device__ __forceinline__ double godunov_axis(double dm, double dp, bool pos) {
    double a, b;
    if (pos) { a = fmax(dm, 0.0); b = fmin(dp, 0.0); }
    else { a = fmin(dm, 0.0); b = fmax(dp, 0.0); }
    return fmax(a * a, b * b);
}

// Sign pattern and r~ of computeInterfaceCrossings3D (reinitialization.h:46-89)
// from phi0 values c (centre) and nb[0..2*DIM) in the order -x,+x,-y,+y,-z,+z.
template <int DIM>
__device__ __forceinline__ void crossing_of(double c, const double* nb, int& flag, double& rt) {
    double sum = 0.0;
    int cnt = 0;
    flag = 0;
#pragma unroll
    for (int q = 0; q < 2 * DIM; ++q) {
        if (c * nb[q] < 0.0) { sum += nb[q]; cnt++; flag |= 1 << q; }
    }
    rt = (cnt > 0 && fabs(sum) > 1e-15) ? c / sum : 0.0;
}

// One HCR-2 pseudo-step, reinitStep3D (reinitialization.h:136-193) with
// checkStabilityConstraint3D (:95-130).  STORED: r~/flag read from arrays
// (drop-in); otherwise recomputed from phi0 with the same operations.
template <int DIM, bool GH, bool STORED>
__global__ void __launch_bounds__(256) reinit_f64_kernel(Geo g, Lay lay, const double* __restrict__ phin_,
                                                         const double* __restrict__ phi0_,
                                                         double* __restrict__ phinew_,
                                                         const double* __restrict__ rt_,
                                                         const int32_t* __restrict__ flag_,
                                                         double dx, double dy, double dz,
                                                         double dtau, double beta) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    int k = DIM == 3 ? blockIdx.z * blockDim.z + threadIdx.z : 0;
    if (i >= g.nx || j >= g.ny || k >= g.nz) return;
    const double* phin = phin_ + lay.off;
    const double* phi0 = phi0_ + lay.off;
    const Nb<GH> n = make_nb<GH>(g, lay, i, j, k);
    const long long id = n.c();
    long long nbi[6];
    nbi[0] = n.x(-1); nbi[1] = n.x(1); nbi[2] = n.y(-1); nbi[3] = n.y(1);
    if (DIM == 3) { nbi[4] = n.z(-1); nbi[5] = n.z(1); }

    const double phi = phin[id];
    const double ph0 = phi0[id];
    double pn[6];
#pragma unroll
    for (int q = 0; q < 2 * DIM; ++q) pn[q] = phin[nbi[q]];

    const double S = ph0 / sqrt(ph0 * ph0 + dx * dx);  // smoothSign, reinitialization.h:24
    const bool pos = S > 0.0;
    const double rdx = 1.0 / dx, rdy = 1.0 / dy, rdz = 1.0 / dz;
    double gsq = godunov_axis(div_rn(phi - pn[0], dx, rdx), div_rn(pn[1] - phi, dx, rdx), pos)
               + godunov_axis(div_rn(phi - pn[2], dy, rdy), div_rn(pn[3] - phi, dy, rdy), pos);
    if (DIM == 3) gsq = gsq + godunov_axis(div_rn(phi - pn[4], dz, rdz), div_rn(pn[5] - phi, dz, rdz), pos);
    const double term = -S * (sqrt(gsq) - 1.0);

    int flag;
    double rt;
    if (STORED) {
        flag = flag_[lay.off + id];
        rt = rt_[lay.off + id];
    } else {
        double p0nb[6];
#pragma unroll
        for (int q = 0; q < 2 * DIM; ++q) p0nb[q] = phi0[nbi[q]];
        crossing_of<DIM>(ph0, p0nb, flag, rt);
    }
    double forcing = 0.0;
    if (flag != 0) {
        bool stable = (phi > 0.0) == (ph0 > 0.0);
#pragma unroll
        for (int q = 0; q < 2 * DIM; ++q)
            if ((flag >> q) & 1) stable = stable && ((pn[q] > 0.0) == (phi0[nbi[q]] > 0.0));
        if (stable) {
            double sum = 0.0;
#pragma unroll
            for (int q = 0; q < 2 * DIM; ++q)
                if ((flag >> q) & 1) sum += pn[q];
            forcing = div_rn(beta * (rt * sum - phi), dx, rdx);
        }
    }
    phinew_[lay.off + id] = phi + dtau * (term + forcing);
}

template <int DIM, bool GH>
__global__ void __launch_bounds__(256) crossings_f64_kernel(Geo g, Lay lay, const double* __restrict__ phi0_,
                                                            double* __restrict__ rt_,
                                                            int32_t* __restrict__ flag_) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    int k = DIM == 3 ? blockIdx.z * blockDim.z + threadIdx.z : 0;
    if (i >= g.nx || j >= g.ny || k >= g.nz) return;
    const double* phi0 = phi0_ + lay.off;
    const Nb<GH> n = make_nb<GH>(g, lay, i, j, k);
    double nb[6];
    nb[0] = phi0[n.x(-1)]; nb[1] = phi0[n.x(1)]; nb[2] = phi0[n.y(-1)]; nb[3] = phi0[n.y(1)];
    if (DIM == 3) { nb[4] = phi0[n.z(-1)]; nb[5] = phi0[n.z(1)]; }
    int flag;
    double rt;
    crossing_of<DIM>(phi0[n.c()], nb, flag, rt);
    rt_[lay.off + n.c()] = rt;
    flag_[lay.off + n.c()] = flag;
}

// Ghost fill of a ghosted array: every ghost element takes the value of its
// periodic image / clamped neighbour in the interior.
__global__ void bc_fill_f64_kernel(Geo g, double* G) {
    const long long nxT = g.nx + 2 * NG, nyT = g.ny + 2 * NG;
    const long long nzT = g.dim == 3 ? g.nz + 2 * NG : 1;
    const long long total = nxT * nyT * nzT;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        int i = (int)(e % nxT);
        int j = (int)((e / nxT) % nyT);
        int k = (int)(e / (nxT * nyT));
        int ii = i - NG, jj = j - NG, kk = g.dim == 3 ? k - NG : 0;
        bool ghost = ii < 0 || ii >= g.nx || jj < 0 || jj >= g.ny ||
                     (g.dim == 3 && (kk < 0 || kk >= g.nz));
        if (!ghost) continue;
        int si = map_axis(ii, g.nx, g.bcx) + NG;
        int sj = map_axis(jj, g.ny, g.bcy) + NG;
        int sk = g.dim == 3 ? map_axis(kk, g.nz, g.bcz) + NG : 0;
        G[e] = G[(long long)sk * nxT * nyT + (long long)sj * nxT + si];
    }
}

// src (FP64, any layout) -> dst compact T
template <typename T>
__global__ void pack_kernel(Geo g, const double* __restrict__ src, Lay sl, T* __restrict__ dst) {
    const long long n = g.cells();
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        int i = (int)(e % g.nx);
        int j = (int)((e / g.nx) % g.ny);
        int k = (int)(e / ((long long)g.nx * g.ny));
        dst[e] = (T)src[sl.off + i + (long long)j * sl.sy + (long long)k * sl.sz];
    }
}

// src compact T -> dst FP64 in layout dl (ghosts filled from the images)
template <typename T>
__global__ void unpack_kernel(Geo g, const T* __restrict__ src, double* __restrict__ dst, Lay dl) {
    if (!dl.ghosted) {
        const long long n = g.cells();
        for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
             e += (long long)gridDim.x * blockDim.x)
            dst[e] = (double)src[e];
        return;
    }
    const long long nxT = g.nx + 2 * NG, nyT = g.ny + 2 * NG;
    const long long nzT = g.dim == 3 ? g.nz + 2 * NG : 1;
    const long long total = nxT * nyT * nzT;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        int i = (int)(e % nxT);
        int j = (int)((e / nxT) % nyT);
        int k = (int)(e / (nxT * nyT));
        int si = map_axis(i - NG, g.nx, g.bcx);
        int sj = map_axis(j - NG, g.ny, g.bcy);
        int sk = g.dim == 3 ? map_axis(k - NG, g.nz, g.bcz) : 0;
        dst[e] = (double)src[(long long)sk * g.nx * g.ny + (long long)sj * g.nx + si];
    }
}

inline dim3 cell_grid(const Geo& g, dim3 b) {
    return dim3((g.nx + b.x - 1) / b.x, (g.ny + b.y - 1) / b.y, (g.nz + b.z - 1) / b.z);
}
// One thread per cell, 32 x 8 (2D) or 32 x 4 x 2 (3D) blocks.  A grid too
// small to give every SM two blocks gets lower blocks instead, down to single
// rows: the FP64 work per cell is a long dependent chain (IEEE divisions), so
// on small grids the time is set by how many SMs share it.  The per-cell
// arithmetic does not depend on the block shape.
inline dim3 cell_block(const Geo& g) {
    static const int sms = [] {
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        return n > 0 ? n : 1;
    }();
    dim3 b = g.dim == 3 ? dim3(32, 4, 2) : dim3(32, 8, 1);
    while (b.y * b.z > 1) {
        const dim3 gr = cell_grid(g, b);
        if ((long long)gr.x * gr.y * gr.z >= 2LL * sms) break;
        if (b.z > 1) b.z /= 2; else b.y /= 2;
    }
    return b;
}

inline unsigned flat_blocks(long long n) {
    long long b = (n + 255) / 256;
    return (unsigned)(b > 152 * 64 ? 152 * 64 : (b < 1 ? 1 : b));
}

}  // namespace

namespace {

template <int DIM, int STAGE, bool GH>
cudaError_t launch_faces(const StageArgs& a, cudaStream_t st) {
    using T = FaceTile<DIM>;
    auto kern = stage_f64_faces<DIM, STAGE, GH>;
    static const cudaError_t attr =
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T::BYTES);
    if (attr != cudaSuccess) return attr;
    const dim3 grid((a.g.nx + T::TX - 1) / T::TX, (a.g.ny + T::TY - 1) / T::TY,
                    DIM == 3 ? (a.g.nz + T::TZ - 1) / T::TZ : 1);
    kern<<<grid, dim3(32, 8, 1), T::BYTES, st>>>(a);
    return cudaGetLastError();
}

// Face-shared tiles (tile 2), or one thread per cell (tile 1); by default the
// tiles where they give every SM at least two CTAs, the per-cell kernel on
// grids too small for that (its lower blocks spread them over every SM).
bool use_faces(const StageArgs& a) {
    if (a.tile == 1) return false;
    if (a.tile == 2) return true;
    static const int sms = [] {
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        return n > 0 ? n : 1;
    }();
    const long long tiles = a.g.dim == 3 ? (long long)((a.g.nx + 31) / 32) * ((a.g.ny + 7) / 8) * ((a.g.nz + 1) / 2)
                                         : (long long)((a.g.nx + 31) / 32) * ((a.g.ny + 15) / 16);
    return tiles >= 2LL * sms;
}

}  // namespace

cudaError_t launch_div_check(long long n, uint64_t seed, unsigned long long* bad, cudaStream_t st) {
    div_check_kernel<<<152 * 8, 256, 0, st>>>(n, seed, bad);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_stage_f64(const StageArgs& a, cudaStream_t st) {
    const bool gh = a.lay.ghosted != 0;
    if (use_faces(a)) {
        cudaError_t e;
#define LSGB_FACES(D, GHV) (a.stage == 1 ? launch_faces<D, 1, GHV>(a, st) \
                                         : (a.stage == 2 ? launch_faces<D, 2, GHV>(a, st) : launch_faces<D, 3, GHV>(a, st)))
        if (a.g.dim == 3) e = gh ? LSGB_FACES(3, true) : LSGB_FACES(3, false);
        else e = gh ? LSGB_FACES(2, true) : LSGB_FACES(2, false);
#undef LSGB_FACES
        count_launches(1);
        return e;
    }
    dim3 b = cell_block(a.g), gr = cell_grid(a.g, b);
#define LSGB_STAGE(D, S, GHV) stage_f64_kernel<D, S, GHV><<<gr, b, 0, st>>>(a)
    if (a.g.dim == 3) {
        if (gh) {
            if (a.stage == 1) LSGB_STAGE(3, 1, true); else if (a.stage == 2) LSGB_STAGE(3, 2, true); else LSGB_STAGE(3, 3, true);
        } else {
            if (a.stage == 1) LSGB_STAGE(3, 1, false); else if (a.stage == 2) LSGB_STAGE(3, 2, false); else LSGB_STAGE(3, 3, false);
        }
    } else {
        if (gh) {
            if (a.stage == 1) LSGB_STAGE(2, 1, true); else if (a.stage == 2) LSGB_STAGE(2, 2, true); else LSGB_STAGE(2, 3, true);
        } else {
            if (a.stage == 1) LSGB_STAGE(2, 1, false); else if (a.stage == 2) LSGB_STAGE(2, 2, false); else LSGB_STAGE(2, 3, false);
        }
    }
#undef LSGB_STAGE
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_reinit_f64(const ReinitArgs& a, cudaStream_t st) {
    dim3 b = cell_block(a.g), gr = cell_grid(a.g, b);
    const double* pn = (const double*)a.phin;
    const double* p0 = (const double*)a.phi0;
    double* out = (double*)a.phinew;
    if (a.g.dim == 3) {
        if (a.lay.ghosted)
            reinit_f64_kernel<3, true, false><<<gr, b, 0, st>>>(a.g, a.lay, pn, p0, out, nullptr, nullptr, a.dx, a.dy, a.dz, a.dtau, a.beta);
        else
            reinit_f64_kernel<3, false, false><<<gr, b, 0, st>>>(a.g, a.lay, pn, p0, out, nullptr, nullptr, a.dx, a.dy, a.dz, a.dtau, a.beta);
    } else {
        if (a.lay.ghosted)
            reinit_f64_kernel<2, true, false><<<gr, b, 0, st>>>(a.g, a.lay, pn, p0, out, nullptr, nullptr, a.dx, a.dy, a.dz, a.dtau, a.beta);
        else
            reinit_f64_kernel<2, false, false><<<gr, b, 0, st>>>(a.g, a.lay, pn, p0, out, nullptr, nullptr, a.dx, a.dy, a.dz, a.dtau, a.beta);
    }
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_crossings_f64(const Geo& g, const Lay& lay, const double* phi0, double* rt,
                                 int32_t* flag, cudaStream_t st) {
    dim3 b = cell_block(g), gr = cell_grid(g, b);
    if (g.dim == 3) {
        if (lay.ghosted) crossings_f64_kernel<3, true><<<gr, b, 0, st>>>(g, lay, phi0, rt, flag);
        else crossings_f64_kernel<3, false><<<gr, b, 0, st>>>(g, lay, phi0, rt, flag);
    } else {
        if (lay.ghosted) crossings_f64_kernel<2, true><<<gr, b, 0, st>>>(g, lay, phi0, rt, flag);
        else crossings_f64_kernel<2, false><<<gr, b, 0, st>>>(g, lay, phi0, rt, flag);
    }
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_reinit_step_stored_f64(const Geo& g, const Lay& lay, const double* phin,
                                          double* phinew, const double* phi0, const double* rt,
                                          const int32_t* flag, double dx, double dy, double dz,
                                          double dtau, double beta, cudaStream_t st) {
    dim3 b = cell_block(g), gr = cell_grid(g, b);
    if (g.dim == 3) {
        if (lay.ghosted)
            reinit_f64_kernel<3, true, true><<<gr, b, 0, st>>>(g, lay, phin, phi0, phinew, rt, flag, dx, dy, dz, dtau, beta);
        else
            reinit_f64_kernel<3, false, true><<<gr, b, 0, st>>>(g, lay, phin, phi0, phinew, rt, flag, dx, dy, dz, dtau, beta);
    } else {
        if (lay.ghosted)
            reinit_f64_kernel<2, true, true><<<gr, b, 0, st>>>(g, lay, phin, phi0, phinew, rt, flag, dx, dy, dz, dtau, beta);
        else
            reinit_f64_kernel<2, false, true><<<gr, b, 0, st>>>(g, lay, phin, phi0, phinew, rt, flag, dx, dy, dz, dtau, beta);
    }
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_bc_fill_f64(const Geo& g, double* G, cudaStream_t st) {
    bc_fill_f64_kernel<<<flat_blocks(layout_elems(g, 1)), 256, 0, st>>>(g, G);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_pack_f64(const Geo& g, const double* src, const Lay& sl, double* dst, cudaStream_t st) {
    pack_kernel<double><<<flat_blocks(g.cells()), 256, 0, st>>>(g, src, sl, dst);
    count_launches(1);
    return cudaGetLastError();
}
cudaError_t launch_pack_f32(const Geo& g, const double* src, const Lay& sl, float* dst, cudaStream_t st) {
    pack_kernel<float><<<flat_blocks(g.cells()), 256, 0, st>>>(g, src, sl, dst);
    count_launches(1);
    return cudaGetLastError();
}
cudaError_t launch_unpack_f64(const Geo& g, const double* src, double* dst, const Lay& dl, cudaStream_t st) {
    unpack_kernel<double><<<flat_blocks(layout_elems(g, dl.ghosted)), 256, 0, st>>>(g, src, dst, dl);
    count_launches(1);
    return cudaGetLastError();
}
cudaError_t launch_unpack_f32(const Geo& g, const float* src, double* dst, const Lay& dl, cudaStream_t st) {
    unpack_kernel<float><<<flat_blocks(layout_elems(g, dl.ghosted)), 256, 0, st>>>(g, src, dst, dl);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace lsgb
