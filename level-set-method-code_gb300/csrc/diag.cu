// diag.cu -- the error / conservation diagnostics of the reference's analysis
// script (Local_code/level-set_MPI_3D/scripts/analyze_error.m) as one
// deterministic device reduction over a state G (compact, FP32 or FP64) and a
// reference field Gr (compact FP64):
//   1. L2 (RMS) and L_inf of G - Gr, RMS of Gr            (analyze_error.m:33-44)
//   2. interface distance: every grid edge that G's zero set crosses gives a
//      crossing point p (linear interpolation); its distance to Gr's zero set
//      is estimated as |Gr(p)| / |grad Gr(p)| (first order, exact for a
//      signed-distance Gr), and symmetrically for Gr's crossings against G.
//      Mean and max of those distances stand in for the contour-based mean
//      interface error and Hausdorff distance of :51-84
//   3. volume by cell count and by the smoothed Heaviside
//      H(phi) = (1 + phi/eps + sin(pi phi/eps)/pi) / 2 on |phi| <= eps, eps = dx,
//      of -G (:88-107, heaviside_smooth :264-271), for G and Gr
//   4. |grad G| (central differences) over the band |G| < 3 dx: mean and
//      standard deviation (:109-133)
// Neighbours wrap (periodic axes) or clamp (zero-gradient axes).
#include "common.cuh"

namespace lsgb {
namespace {

constexpr int DQ = 14;  // reduced quantities per block
// sums: 0 sq diff, 2 sq ref, 3 neg count, 4 neg count ref, 5 H, 6 H ref,
// 7 band count, 8 band |grad|, 9 band |grad|^2, 10 iface sum, 12 iface count;
// maxes: 1 |diff|, 11 iface max, 13 unused
__device__ __forceinline__ bool is_max(int q) { return q == 1 || q == 11 || q == 13; }

__device__ __forceinline__ double heaviside_smooth(double phi, double eps) {
    if (phi > eps) return 1.0;
    if (phi < -eps) return 0.0;
    const double pi = 3.14159265358979323846;
    return 0.5 * (1.0 + phi / eps + sin(pi * phi / eps) / pi);
}

template <typename T>
struct Field {
    const T* p;
    Geo g;
    __device__ __forceinline__ double at(int i, int j, int k) const {
        return (double)p[((long long)k * g.ny + j) * g.nx + i];
    }
};

// |grad f| at cell (i, j, k) by central differences
template <typename F>
__device__ __forceinline__ double grad_mag(const F& f, const Geo& g, int i, int j, int k, double dx, double dy,
                                           double dz) {
    const double gx = (f.at(map_axis(i + 1, g.nx, g.bcx), j, k) - f.at(map_axis(i - 1, g.nx, g.bcx), j, k)) / (2 * dx);
    const double gy = (f.at(i, map_axis(j + 1, g.ny, g.bcy), k) - f.at(i, map_axis(j - 1, g.ny, g.bcy), k)) / (2 * dy);
    double s = gx * gx + gy * gy;
    if (g.dim == 3) {
        const double gz = (f.at(i, j, map_axis(k + 1, g.nz, g.bcz)) - f.at(i, j, map_axis(k - 1, g.nz, g.bcz))) / (2 * dz);
        s += gz * gz;
    }
    return sqrt(s);
}

template <typename T>
__global__ void __launch_bounds__(RED_THREADS) diag_kernel(Geo g, const T* __restrict__ G,
                                                           const double* __restrict__ Gr, double dx, double dy,
                                                           double dz, double* __restrict__ partials) {
    __shared__ double red[RED_THREADS];
    double acc[DQ];
#pragma unroll
    for (int q = 0; q < DQ; ++q) acc[q] = 0.0;
    const Field<T> f{G, g};
    const Field<double> r{Gr, g};
    const long long n = g.cells();
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % g.nx);
        const int j = (int)((e / g.nx) % g.ny);
        const int k = (int)(e / ((long long)g.nx * g.ny));
        const double a = f.at(i, j, k);
        const double b = r.at(i, j, k);
        const double d = a - b;
        acc[0] += d * d;
        acc[1] = fmax(acc[1], fabs(d));
        acc[2] += b * b;
        acc[3] += a < 0.0 ? 1.0 : 0.0;
        acc[4] += b < 0.0 ? 1.0 : 0.0;
        acc[5] += heaviside_smooth(-a, dx);
        acc[6] += heaviside_smooth(-b, dx);
        if (fabs(a) < 3.0 * dx) {
            const double gm = grad_mag(f, g, i, j, k, dx, dy, dz);
            acc[7] += 1.0;
            acc[8] += gm;
            acc[9] += gm * gm;
        }
        // edges to the +1 neighbour on each axis
        for (int ax = 0; ax < g.dim; ++ax) {
            int i2 = i, j2 = j, k2 = k;
            bool ok = true;
            if (ax == 0) { i2 = i + 1; if (i2 >= g.nx) { if (g.bcx == LSGB_BC_PERIODIC) i2 = 0; else ok = false; } }
            if (ax == 1) { j2 = j + 1; if (j2 >= g.ny) { if (g.bcy == LSGB_BC_PERIODIC) j2 = 0; else ok = false; } }
            if (ax == 2) { k2 = k + 1; if (k2 >= g.nz) { if (g.bcz == LSGB_BC_PERIODIC) k2 = 0; else ok = false; } }
            if (!ok) continue;
            const double a2 = f.at(i2, j2, k2), b2 = r.at(i2, j2, k2);
            // crossing of one field, distance to the other's zero set
            for (int side = 0; side < 2; ++side) {
                const double p0 = side ? b : a, p1 = side ? b2 : a2;
                if (!(p0 * p1 < 0.0)) continue;
                const double t = p0 / (p0 - p1);
                const double o0 = side ? a : b, o1 = side ? a2 : b2;
                const double ov = o0 + t * (o1 - o0);
                double g0, g1;
                if (side) {
                    g0 = grad_mag(f, g, i, j, k, dx, dy, dz);
                    g1 = grad_mag(f, g, i2, j2, k2, dx, dy, dz);
                } else {
                    g0 = grad_mag(r, g, i, j, k, dx, dy, dz);
                    g1 = grad_mag(r, g, i2, j2, k2, dx, dy, dz);
                }
                const double gp = g0 + t * (g1 - g0);
                const double dist = gp > 0.0 ? fabs(ov) / gp : fabs(ov);
                acc[10] += dist;
                acc[11] = fmax(acc[11], dist);
                acc[12] += 1.0;
            }
        }
    }
    for (int q = 0; q < DQ; ++q) {
        red[threadIdx.x] = acc[q];
        __syncthreads();
        for (int s = RED_THREADS / 2; s > 0; s >>= 1) {
            if (threadIdx.x < s)
                red[threadIdx.x] = is_max(q) ? fmax(red[threadIdx.x], red[threadIdx.x + s])
                                             : red[threadIdx.x] + red[threadIdx.x + s];
            __syncthreads();
        }
        if (threadIdx.x == 0) partials[(long long)q * RED_BLOCKS + blockIdx.x] = red[0];
        __syncthreads();
    }
}

__global__ void __launch_bounds__(RED_THREADS) diag_final_kernel(const double* __restrict__ partials,
                                                                 double* __restrict__ out) {
    __shared__ double red[RED_THREADS];
    for (int q = 0; q < DQ; ++q) {
        double v = 0.0;
        for (int b = threadIdx.x; b < RED_BLOCKS; b += blockDim.x) {
            const double x = partials[(long long)q * RED_BLOCKS + b];
            v = is_max(q) ? fmax(v, x) : v + x;
        }
        red[threadIdx.x] = v;
        __syncthreads();
        for (int s = RED_THREADS / 2; s > 0; s >>= 1) {
            if (threadIdx.x < s)
                red[threadIdx.x] = is_max(q) ? fmax(red[threadIdx.x], red[threadIdx.x + s])
                                             : red[threadIdx.x] + red[threadIdx.x + s];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[q] = red[0];
        __syncthreads();
    }
}

}  // namespace

size_t diag_scratch_bytes() { return sizeof(double) * ((size_t)DQ * RED_BLOCKS + DQ); }

template <typename T>
cudaError_t launch_diagnostics(const Geo& g, const T* G, const double* Gr, double dx, double dy, double dz,
                               double* scratch, cudaStream_t st) {
    diag_kernel<T><<<RED_BLOCKS, RED_THREADS, 0, st>>>(g, G, Gr, dx, dy, dz, scratch);
    diag_final_kernel<<<1, RED_THREADS, 0, st>>>(scratch, scratch + (size_t)DQ * RED_BLOCKS);
    count_launches(2);
    return cudaGetLastError();
}
template cudaError_t launch_diagnostics<float>(const Geo&, const float*, const double*, double, double, double,
                                               double*, cudaStream_t);
template cudaError_t launch_diagnostics<double>(const Geo&, const double*, const double*, double, double, double,
                                                double*, cudaStream_t);

}  // namespace lsgb
