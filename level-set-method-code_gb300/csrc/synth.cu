// synth.cu -- on-device generator of the synthetic benchmark fields.
//
// The benchmark grids (256^3, 512^3) are too large to build on the host in a
// reasonable time, so the fields are evaluated here in FP64 from a small mode
// table that the host draws from a seed (lsgb/synthetic.py holds the same
// formulas in numpy for the small grids the tests compare against):
//   G0(x) = |x - c| - (r0 + sum_m amp_m * Pbar_lm(cos theta) * trig_m(phi))
//   u(x)  = sum_m C_m cos(2 pi k_m . x + phase_m)
// with cell centres x_i = i * dx on the periodic unit box.  amp_m already
// carries the normalisation that makes max |Pbar_lm * trig_m| = 1.
#include "common.cuh"

namespace lsgb {
namespace {

__constant__ lsgb_synth c_synth;

// Associated Legendre P_l^m(x) for 0 <= m <= l <= 4 (no Condon-Shortley phase).
__device__ double assoc_legendre(int l, int m, double x) {
    const double s = sqrt(fmax(0.0, 1.0 - x * x));
    // P_m^m = (2m-1)!! s^m
    double pmm = 1.0;
    for (int q = 1; q <= m; ++q) pmm *= (2.0 * q - 1.0) * s;
    if (l == m) return pmm;
    double pm1 = x * (2.0 * m + 1.0) * pmm;
    if (l == m + 1) return pm1;
    double pl = 0.0;
    for (int ll = m + 2; ll <= l; ++ll) {
        pl = (x * (2.0 * ll - 1.0) * pm1 - (ll + m - 1.0) * pmm) / (ll - m);
        pmm = pm1;
        pm1 = pl;
    }
    return pl;
}

__global__ void synth_kernel(Geo g, double dx, double dy, double dz, double* __restrict__ G,
                             double* __restrict__ u, double* __restrict__ v,
                             double* __restrict__ w) {
    const lsgb_synth& d = c_synth;
    const long long n = g.cells();
    const long long nxy = (long long)g.nx * g.ny;
    const double two_pi = 6.283185307179586476925286766559;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(e / nxy);
        const long long r = e - (long long)k * nxy;
        const int j = (int)(r / g.nx);
        const int i = (int)(r - (long long)j * g.nx);
        const double x = i * dx, y = j * dy, z = g.dim == 3 ? k * dz : 0.0;
        const double px = x - d.center[0], py = y - d.center[1], pz = g.dim == 3 ? z - d.center[2] : 0.0;
        const double rad = sqrt(px * px + py * py + pz * pz);
        double radius = d.r0;
        if (g.dim == 3 && rad > 0.0) {
            const double ct = pz / rad;
            const double ph = atan2(py, px);
            for (int m = 0; m < d.n_shape_modes; ++m) {
                const int l = d.shape_l[m], mm = d.shape_m[m];
                const int am = mm < 0 ? -mm : mm;
                const double trig = mm >= 0 ? cos(am * ph) : sin(am * ph);
                radius += d.shape_amp[m] * assoc_legendre(l, am, ct) * trig;
            }
        }
        G[e] = rad - radius;
        double uu = 0.0, vv = 0.0, ww = 0.0;
        for (int m = 0; m < d.n_vel_modes; ++m) {
            const double th = two_pi * (d.vel_k[m][0] * x + d.vel_k[m][1] * y + d.vel_k[m][2] * z) +
                              d.vel_phase[m];
            const double cs = cos(th);
            uu += d.vel_c[m][0] * cs;
            vv += d.vel_c[m][1] * cs;
            ww += d.vel_c[m][2] * cs;
        }
        const double sc = d.vel_scale > 0.0 ? d.vel_scale : 1.0;
        u[e] = uu * sc;
        v[e] = vv * sc;
        if (g.dim == 3) w[e] = ww * sc;
    }
}

__global__ void scale3_kernel(long long n, double s, double* u, double* v, double* w) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        u[e] *= s;
        v[e] *= s;
        if (w) w[e] *= s;
    }
}

// computeDeformationVelocity (Local_code/level-set_MPI_3D/include/
// initial_conditions.h:232-247) at the cell centres x_i = i * dx, written
// straight into the compact velocity arrays of the solver.  The field is a
// product of per-axis factors, so the sines are evaluated once per axis
// index and every cell only forms products.
//
// FP64: tab = [sin(pi x_i)][sin(2 pi x_i)] [.. y ..] [.. z ..] [cos(pi t / T)]
// per call, and each cell forms the reference's products in its order:
// exactly the values of evaluating the sines at every cell.
// at.tab set: the time is at.tab[*at.base + at.q] (a batch's per-step table).
__global__ void deformation_factors_f64_kernel(Geo g, double dx, double dy, double dz, double t, double Tp,
                                               LiveAt at, double* __restrict__ tab) {
    const double pi = 3.14159265358979323846;
    const int n[3] = {g.nx, g.ny, g.nz};
    const double h[3] = {dx, dy, dz};
    int base = 0;
    for (int a = 0; a < 3; ++a) {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n[a]; i += gridDim.x * blockDim.x) {
            const double x = i * h[a];
            tab[base + i] = sin(pi * x);
            tab[base + n[a] + i] = sin(2.0 * pi * x);
        }
        base += 2 * n[a];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const double tt = at.tab ? ((const double*)at.tab)[*at.base + at.q] : t;
        tab[base] = cos(pi * tt / Tp);
    }
}

// One thread per cell of a row segment; rows (j, k) strided over gridDim.y.
__global__ void deformation_f64_kernel(Geo g, const double* __restrict__ tab, double* __restrict__ u,
                                       double* __restrict__ v, double* __restrict__ w) {
    const double* s1x = tab;
    const double* s2x = s1x + g.nx;
    const double* s1y = s2x + g.nx;
    const double* s2y = s1y + g.ny;
    const double* s1z = s2y + g.ny;
    const double* s2z = s1z + g.nz;
    const double tf = s2z[g.nz];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.nx) return;
    const double spx = s1x[i], s2px = s2x[i];
    const long long rows = (long long)g.ny * g.nz;
    for (long long row = blockIdx.y; row < rows; row += gridDim.y) {
        const int k = (int)(row / g.ny);
        const int j = (int)(row - (long long)k * g.ny);
        const double spy = s1y[j], s2py = s2y[j], spz = s1z[k], s2pz = s2z[k];
        const long long e = row * g.nx + i;
        u[e] = 2.0 * spx * spx * s2py * s2pz * tf;
        v[e] = -s2px * spy * spy * s2pz * tf;
        w[e] = -s2px * s2py * spz * spz * tf;
    }
}

// FP32: time-independent tables, per axis [sin^2(pi x_i)] and
// [sin(2 pi x_i)] (n + 1 entries each, the last 0), computed in FP64 and
// rounded once.  With tf = cos(pi t / T) rounded to FP32 the cell values are
//   u = (2 sq_x s2_y tf) s2_z,  v = (-s2_x sq_y tf) s2_z,  w = (-s2_x s2_y tf) sq_z,
// products in FP32 in this order -- the order the fused stage kernel uses
// (per-row factor times per-plane factor), so both give the same bits.
__global__ void deformation_tables_f32_kernel(Geo g, double dx, double dy, double dz, float* __restrict__ tab) {
    const double pi = 3.14159265358979323846;
    const int n[3] = {g.nx, g.ny, g.nz};
    const double h[3] = {dx, dy, dz};
    int base = 0;
    for (int a = 0; a < 3; ++a) {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= n[a]; i += gridDim.x * blockDim.x) {
            const double x = i * h[a];
            const double s1 = sin(pi * x);
            tab[base + i] = i < n[a] ? (float)(s1 * s1) : 0.0f;
            tab[base + n[a] + 1 + i] = i < n[a] ? (float)sin(2.0 * pi * x) : 0.0f;
        }
        base += 2 * (n[a] + 1);
    }
}

// at.tab set: tf = at.tab[*at.base + at.q] (a batch's per-step table).
__global__ void deformation_f32_kernel(Geo g, const float* __restrict__ tab, float tf, LiveAt at,
                                       float* __restrict__ u, float* __restrict__ v, float* __restrict__ w) {
    const DeformTables d = deform_tables(g, tab);
    if (at.tab) tf = ((const float*)at.tab)[*at.base + at.q];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.nx) return;
    const long long rows = (long long)g.ny * g.nz;
    for (long long row = blockIdx.y; row < rows; row += gridDim.y) {
        const int k = (int)(row / g.ny);
        const int j = (int)(row - (long long)k * g.ny);
        const long long e = row * g.nx + i;
        u[e] = (2.0f * d.sqx[i] * d.s2y[j] * tf) * d.s2z[k];
        v[e] = (-d.s2x[i] * d.sqy[j] * tf) * d.s2z[k];
        w[e] = (-d.s2x[i] * d.s2y[j] * tf) * d.sqz[k];
    }
}

__global__ void live_advance_kernel(int* base, int n) { *base += n; }

dim3 deformation_grid(const Geo& g) {
    const long long rows = (long long)g.ny * g.nz;
    return dim3((g.nx + 127) / 128, (unsigned)(rows < 65535 ? rows : 65535));
}

}  // namespace

cudaError_t launch_deformation_f64(const Geo& g, double dx, double dy, double dz, double t, double Tp,
                                   double* u, double* v, double* w, cudaStream_t st, LiveAt at) {
    double* tab = nullptr;
    const size_t ntab = 2 * ((size_t)g.nx + g.ny + g.nz) + 1;
    cudaError_t e = cudaMallocAsync((void**)&tab, ntab * sizeof(double), st);
    if (e != cudaSuccess) return e;
    deformation_factors_f64_kernel<<<8, 256, 0, st>>>(g, dx, dy, dz, t, Tp, at, tab);
    deformation_f64_kernel<<<deformation_grid(g), 128, 0, st>>>(g, tab, u, v, w);
    count_launches(2);
    e = cudaGetLastError();
    const cudaError_t f = cudaFreeAsync(tab, st);
    return e != cudaSuccess ? e : f;
}

cudaError_t launch_live_advance(int* base, int n, cudaStream_t st) {
    live_advance_kernel<<<1, 1, 0, st>>>(base, n);
    count_launches(1);
    return cudaGetLastError();
}

size_t deformation_table_floats(const Geo& g) { return 2 * ((size_t)g.nx + g.ny + g.nz + 3); }

cudaError_t launch_deformation_tables_f32(const Geo& g, double dx, double dy, double dz, float* tab,
                                          cudaStream_t st) {
    deformation_tables_f32_kernel<<<8, 256, 0, st>>>(g, dx, dy, dz, tab);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_deformation_f32(const Geo& g, const float* tab, float tf, float* u, float* v, float* w,
                                   cudaStream_t st, LiveAt at) {
    deformation_f32_kernel<<<deformation_grid(g), 128, 0, st>>>(g, tab, tf, at, u, v, w);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_synth(const Geo& g, const lsgb_synth& d, double dx, double dy, double dz,
                         double* G, double* u, double* v, double* w, cudaStream_t st) {
    cudaError_t e = cudaMemcpyToSymbolAsync(c_synth, &d, sizeof(d), 0, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    long long blocks = (g.cells() + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    synth_kernel<<<(unsigned)blocks, 256, 0, st>>>(g, dx, dy, dz, G, u, v, w);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_scale3(long long n, double s, double* u, double* v, double* w, cudaStream_t st) {
    long long blocks = (n + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    scale3_kernel<<<(unsigned)blocks, 256, 0, st>>>(n, s, u, v, w);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace lsgb
