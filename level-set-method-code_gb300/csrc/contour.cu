// contour.cu -- the interface position error of the reference's analysis
// script (Local_code/level-set_MPI_3D/scripts/analyze_error.m:51-84) on the
// device: the zero contours of two fields as point sets, each point's
// distance to the nearest point of the other set, then
//   hausdorff = max over both directions of those distances   (:76)
//   mean      = their mean over both sets together            (:77)
//
// Points.  The script extracts the zero contours with contourc, whose
// vertices are the linear-interpolation crossings of the level on the grid
// edges.  Here every grid edge between two interior cells whose values
// change sign (one < 0, the other >= 0) gives one point: for an edge along
// axis a from cell c to c + e_a, t = F(c) / (F(c) - F(c + e_a)) and the point
// is c + t e_a, in coordinates x = i dx, y = j dy, z = k dz (the script's
// linspace(0, 1, n) grid when dx = 1/(n-1)).  In 3D the same edges give the
// vertices of the zero isosurface.  As in the script, no edge wraps around a
// periodic axis and distances are plain Euclidean.  (contourc also repeats
// the first vertex of a closed curve; that duplicate is not reproduced.)
//
// Nearest points.  The target set is binned on a uniform grid of 2 x 2 x 2
// cells (counting sort); a query searches the bins in shells of growing
// Chebyshev radius r around its own bin and stops once its best squared
// distance is at most (r * smallest bin width)^2, which no point of a later
// shell can beat.  The minimum of exactly computed squared distances does not
// depend on the visiting order, so the result is the brute-force minimum bit
// for bit.  Sums and maxima are deterministic two-pass reductions.
//
// Compiled with --fmad=false: every distance is the plain IEEE expression
// ((xa - xb)^2 + (ya - yb)^2) + (za - zb)^2, then one sqrt.
#include "common.cuh"

#include <cmath>
#include <vector>

namespace lsgb {
namespace {

constexpr int CT = 256;       // threads per block
constexpr int CPT = 8;        // cells per thread in the crossing passes
constexpr int CPB = CT * CPT; // cells per block
constexpr int BINW = 2;       // bin width in cells

struct Pts {
    double* x;
    double* y;
    double* z;
    int* bin;
};

struct BinGeo {
    int nbx, nby, nbz;
    double sx, sy, sz;  // bin widths
    __host__ __device__ long long count() const { return (long long)nbx * nby * nbz; }
};

template <typename T>
__device__ __forceinline__ double val(const T* F, const Geo& g, int i, int j, int k) {
    return (double)F[((long long)k * g.ny + j) * g.nx + i];
}

// Crossings on the +x, +y (+z) edges of cell e; calls f(axis, t) for each.
template <typename T, typename Fn>
__device__ __forceinline__ void crossings(const T* F, const Geo& g, long long e, Fn f) {
    const int i = (int)(e % g.nx);
    const int j = (int)((e / g.nx) % g.ny);
    const int k = (int)(e / ((long long)g.nx * g.ny));
    const double a = val(F, g, i, j, k);
    for (int ax = 0; ax < g.dim; ++ax) {
        const int i2 = i + (ax == 0), j2 = j + (ax == 1), k2 = k + (ax == 2);
        if (i2 >= g.nx || j2 >= g.ny || k2 >= g.nz) continue;
        const double b = val(F, g, i2, j2, k2);
        if ((a < 0.0) != (b < 0.0)) f(ax, i, j, k, a / (a - b));
    }
}

// Pass 1: crossings of block b's cells [b CPB, (b+1) CPB).
template <typename T>
__global__ void __launch_bounds__(CT) xing_count(Geo g, const T* __restrict__ F, int* __restrict__ counts) {
    const long long n = g.cells();
    const long long e0 = (long long)blockIdx.x * CPB + (long long)threadIdx.x * CPT;
    int c = 0;
    for (int q = 0; q < CPT; ++q)
        if (e0 + q < n) crossings(F, g, e0 + q, [&](int, int, int, int, double) { ++c; });
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    __shared__ int ws[CT / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int s = 0;
        for (int w = 0; w < CT / 32; ++w) s += ws[w];
        counts[blockIdx.x] = s;
    }
}

// Exclusive scan of n ints by one block, in place, into 64-bit offsets
// (out[n] = total).  Chunks of CT with a running carry.
__global__ void __launch_bounds__(CT) scan_one_block(const int* __restrict__ in, long long* __restrict__ out,
                                                     long long n) {
    __shared__ long long s[CT];
    long long carry = 0;
    for (long long base = 0; base < n; base += CT) {
        const long long q = base + threadIdx.x;
        const long long v = q < n ? in[q] : 0;
        s[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < CT; o <<= 1) {  // Hillis-Steele inclusive scan
            const long long add = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
            __syncthreads();
            s[threadIdx.x] += add;
            __syncthreads();
        }
        if (q < n) out[q] = carry + s[threadIdx.x] - v;
        const long long tot = s[CT - 1];
        __syncthreads();
        carry += tot;
    }
    if (threadIdx.x == 0) out[n] = carry;
}

// Pass 2: the points of block b in cell order (thread order, then the cell's
// axes), at the block's offset.
template <typename T>
__global__ void __launch_bounds__(CT) xing_emit(Geo g, const T* __restrict__ F, const long long* __restrict__ off,
                                                double dx, double dy, double dz, BinGeo bg, Pts p) {
    const long long n = g.cells();
    const long long e0 = (long long)blockIdx.x * CPB + (long long)threadIdx.x * CPT;
    int c = 0;
    for (int q = 0; q < CPT; ++q)
        if (e0 + q < n) crossings(F, g, e0 + q, [&](int, int, int, int, double) { ++c; });
    __shared__ int s[CT];
    s[threadIdx.x] = c;
    __syncthreads();
    for (int o = 1; o < CT; o <<= 1) {
        const int add = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
        __syncthreads();
        s[threadIdx.x] += add;
        __syncthreads();
    }
    long long w = off[blockIdx.x] + s[threadIdx.x] - c;
    for (int q = 0; q < CPT; ++q)
        if (e0 + q < n)
            crossings(F, g, e0 + q, [&](int ax, int i, int j, int k, double t) {
                p.x[w] = ax == 0 ? ((double)i + t) * dx : (double)i * dx;
                p.y[w] = ax == 1 ? ((double)j + t) * dy : (double)j * dy;
                p.z[w] = ax == 2 ? ((double)k + t) * dz : (double)k * dz;
                p.bin[w] = ((k / BINW) * bg.nby + j / BINW) * bg.nbx + i / BINW;
                ++w;
            });
}

__global__ void bin_count(long long n, const int* __restrict__ bin, int* __restrict__ cnt) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
        atomicAdd(cnt + bin[q], 1);
}

// Device-wide exclusive scan of n ints (n < 2^31): per-block sums, one-block
// scan of the sums, per-block scan with the block's offset.
__global__ void __launch_bounds__(CT) block_sums(const int* __restrict__ in, long long n, int chunk,
                                                 int* __restrict__ sums) {
    const long long b0 = (long long)blockIdx.x * chunk;
    int v = 0;
    for (int q = threadIdx.x; q < chunk; q += CT)
        if (b0 + q < n) v += in[b0 + q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __shared__ int ws[CT / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        int s = 0;
        for (int w = 0; w < CT / 32; ++w) s += ws[w];
        sums[blockIdx.x] = s;
    }
}

__global__ void __launch_bounds__(CT) block_scan_apply(const int* __restrict__ in, long long n, int chunk,
                                                       const long long* __restrict__ boff, int* __restrict__ out) {
    __shared__ int s[CT];
    const long long b0 = (long long)blockIdx.x * chunk;
    long long carry = boff[blockIdx.x];
    for (int base = 0; base < chunk; base += CT) {
        const long long q = b0 + base + threadIdx.x;
        const int v = (base + (int)threadIdx.x < chunk && q < n) ? in[q] : 0;
        s[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < CT; o <<= 1) {
            const int add = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
            __syncthreads();
            s[threadIdx.x] += add;
            __syncthreads();
        }
        if (base + (int)threadIdx.x < chunk && q < n) out[q] = (int)(carry + s[threadIdx.x] - v);
        const int tot = s[CT - 1];
        __syncthreads();
        carry += tot;
    }
}

__global__ void bin_scatter(long long n, Pts p, int* __restrict__ cursor, double* __restrict__ sx,
                            double* __restrict__ sy, double* __restrict__ sz) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int slot = atomicAdd(cursor + p.bin[q], 1);
        sx[slot] = p.x[q];
        sy[slot] = p.y[q];
        sz[slot] = p.z[q];
    }
}

// Distance from each query point to the nearest target point.
__global__ void __launch_bounds__(CT) nearest(long long nq, Pts qp, BinGeo bg, const int* __restrict__ start,
                                              const int* __restrict__ cnt, const double* __restrict__ tx,
                                              const double* __restrict__ ty, const double* __restrict__ tz,
                                              double* __restrict__ dist) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= nq) return;
    const double px = qp.x[q], py = qp.y[q], pz = qp.z[q];
    const int b = qp.bin[q];
    const int bi = b % bg.nbx, bj = (b / bg.nbx) % bg.nby, bk = b / (bg.nbx * bg.nby);
    const double smin = fmin(bg.sx, fmin(bg.sy, bg.nbz > 1 ? bg.sz : bg.sx));
    const int rmax = max(bg.nbx, max(bg.nby, bg.nbz));
    double best = INFINITY;
    for (int r = 0; r <= rmax; ++r) {
        const int k0 = max(bk - r, 0), k1 = min(bk + r, bg.nbz - 1);
        const int j0 = max(bj - r, 0), j1 = min(bj + r, bg.nby - 1);
        for (int kk = k0; kk <= k1; ++kk)
            for (int jj = j0; jj <= j1; ++jj) {
                const bool edge = abs(kk - bk) == r || abs(jj - bj) == r;
                // on the shell's faces every x in range, else only x = bi -+ r
                for (int ii = edge ? bi - r : bi - r; ii <= bi + r; ii += (edge || r == 0) ? 1 : 2 * r) {
                    if (ii < 0 || ii >= bg.nbx) continue;
                    const int bb = (kk * bg.nby + jj) * bg.nbx + ii;
                    const int s0 = start[bb], s1 = s0 + cnt[bb];
                    for (int m = s0; m < s1; ++m) {
                        const double ex = tx[m] - px, ey = ty[m] - py, ez = tz[m] - pz;
                        const double d2 = (ex * ex + ey * ey) + ez * ez;
                        best = fmin(best, d2);
                    }
                }
            }
        const double lim = (double)r * smin;
        if (best <= lim * lim) break;
    }
    dist[q] = sqrt(best);
}

// Deterministic sum and max of n doubles: RED_BLOCKS fixed slices, then one block.
__global__ void __launch_bounds__(RED_THREADS) sum_max_pass1(long long n, const double* __restrict__ v,
                                                             double* __restrict__ part) {
    __shared__ double ss[RED_THREADS], sm[RED_THREADS];
    double s = 0.0, m = 0.0;
    for (long long q = blockIdx.x * (long long)RED_THREADS + threadIdx.x; q < n; q += (long long)RED_BLOCKS * RED_THREADS) {
        s += v[q];
        m = fmax(m, v[q]);
    }
    ss[threadIdx.x] = s;
    sm[threadIdx.x] = m;
    __syncthreads();
    for (int o = RED_THREADS / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            ss[threadIdx.x] += ss[threadIdx.x + o];
            sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + o]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[blockIdx.x] = ss[0];
        part[RED_BLOCKS + blockIdx.x] = sm[0];
    }
}

__global__ void __launch_bounds__(RED_THREADS) sum_max_pass2(const double* __restrict__ part, double* __restrict__ out) {
    __shared__ double ss[RED_THREADS], sm[RED_THREADS];
    double s = 0.0, m = 0.0;
    for (int q = threadIdx.x; q < RED_BLOCKS; q += RED_THREADS) {
        s += part[q];
        m = fmax(m, part[RED_BLOCKS + q]);
    }
    ss[threadIdx.x] = s;
    sm[threadIdx.x] = m;
    __syncthreads();
    for (int o = RED_THREADS / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            ss[threadIdx.x] += ss[threadIdx.x + o];
            sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + o]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = ss[0];
        out[1] = sm[0];
    }
}

// Device allocations of one call, released on every path.
struct Arena {
    cudaStream_t st;
    std::vector<void*> ptrs;
    cudaError_t err = cudaSuccess;
    template <typename T>
    T* get(long long n) {
        void* p = nullptr;
        if (err == cudaSuccess) err = cudaMallocAsync(&p, sizeof(T) * (size_t)(n > 0 ? n : 1), st);
        if (err == cudaSuccess) ptrs.push_back(p);
        return (T*)p;
    }
    ~Arena() {
        for (void* p : ptrs) cudaFreeAsync(p, st);
    }
};

int grid_of(long long n) { return (int)std::min<long long>((n + CT - 1) / CT, 4096 * 152LL); }

// The contour points of F (count on the host, then emission).
template <typename T>
cudaError_t extract(const Geo& g, const T* F, double dx, double dy, double dz, const BinGeo& bg, Arena& ar,
                    Pts* out, long long* n_out, cudaStream_t st) {
    const long long nb = (g.cells() + CPB - 1) / CPB;
    int* counts = ar.get<int>(nb);
    long long* off = ar.get<long long>(nb + 1);
    if (ar.err != cudaSuccess) return ar.err;
    xing_count<T><<<(unsigned)nb, CT, 0, st>>>(g, F, counts);
    scan_one_block<<<1, CT, 0, st>>>(counts, off, nb);
    count_launches(2);
    long long total = 0;
    cudaError_t e = cudaMemcpyAsync(&total, off + nb, sizeof(long long), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    Pts p;
    p.x = ar.get<double>(total);
    p.y = ar.get<double>(total);
    p.z = ar.get<double>(total);
    p.bin = ar.get<int>(total);
    if (ar.err != cudaSuccess) return ar.err;
    xing_emit<T><<<(unsigned)nb, CT, 0, st>>>(g, F, off, dx, dy, dz, bg, p);
    count_launches(1);
    *out = p;
    *n_out = total;
    return cudaGetLastError();
}

// Distances of the query points to the nearest target point, and their sum and max.
cudaError_t distances(const Pts& q, long long nq, const Pts& t, long long nt, const BinGeo& bg, Arena& ar,
                      double sum_max[2], cudaStream_t st) {
    const long long nbins = bg.count();
    int* cnt = ar.get<int>(nbins);
    int* start = ar.get<int>(nbins);
    int* cursor = ar.get<int>(nbins);
    double* tx = ar.get<double>(nt);
    double* ty = ar.get<double>(nt);
    double* tz = ar.get<double>(nt);
    double* dist = ar.get<double>(nq);
    double* part = ar.get<double>(2 * RED_BLOCKS + 2);
    const int chunk = 4096;
    const long long nblk = (nbins + chunk - 1) / chunk;
    int* sums = ar.get<int>(nblk);
    long long* boff = ar.get<long long>(nblk + 1);
    if (ar.err != cudaSuccess) return ar.err;
    cudaError_t e = cudaMemsetAsync(cnt, 0, sizeof(int) * (size_t)nbins, st);
    if (e != cudaSuccess) return e;
    bin_count<<<grid_of(nt), CT, 0, st>>>(nt, t.bin, cnt);
    block_sums<<<(unsigned)nblk, CT, 0, st>>>(cnt, nbins, chunk, sums);
    scan_one_block<<<1, CT, 0, st>>>(sums, boff, nblk);
    block_scan_apply<<<(unsigned)nblk, CT, 0, st>>>(cnt, nbins, chunk, boff, start);
    count_launches(4);
    e = cudaMemcpyAsync(cursor, start, sizeof(int) * (size_t)nbins, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return e;
    bin_scatter<<<grid_of(nt), CT, 0, st>>>(nt, t, cursor, tx, ty, tz);
    nearest<<<(unsigned)((nq + CT - 1) / CT), CT, 0, st>>>(nq, q, bg, start, cnt, tx, ty, tz, dist);
    sum_max_pass1<<<RED_BLOCKS, RED_THREADS, 0, st>>>(nq, dist, part);
    sum_max_pass2<<<1, RED_THREADS, 0, st>>>(part, part + 2 * RED_BLOCKS);
    count_launches(4);
    e = cudaMemcpyAsync(sum_max, part + 2 * RED_BLOCKS, 2 * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e;
}

}  // namespace

template <typename T>
cudaError_t contour_distances(const Geo& g, const T* G, const double* Gr, double dx, double dy, double dz,
                              ContourDist* out, cudaStream_t st) {
    BinGeo bg;
    bg.nbx = (g.nx + BINW - 1) / BINW;
    bg.nby = (g.ny + BINW - 1) / BINW;
    bg.nbz = g.dim == 3 ? (g.nz + BINW - 1) / BINW : 1;
    bg.sx = BINW * dx;
    bg.sy = BINW * dy;
    bg.sz = BINW * dz;
    Arena ar{st};
    Pts pg, pr;
    long long ng = 0, nr = 0;
    cudaError_t e = extract<T>(g, G, dx, dy, dz, bg, ar, &pg, &ng, st);
    if (e == cudaSuccess) e = extract<double>(g, Gr, dx, dy, dz, bg, ar, &pr, &nr, st);
    if (e != cudaSuccess) return e;
    out->points = ng;
    out->points_ref = nr;
    if (ng == 0 || nr == 0) {  // "Could not extract interface contours"
        out->hausdorff = out->mean = NAN;
        return cudaSuccess;
    }
    double a[2], b[2];
    e = distances(pg, ng, pr, nr, bg, ar, a, st);
    if (e == cudaSuccess) e = distances(pr, nr, pg, ng, bg, ar, b, st);
    if (e != cudaSuccess) return e;
    out->hausdorff = std::fmax(a[1], b[1]);
    out->mean = (a[0] + b[0]) / (double)(ng + nr);
    return cudaSuccess;
}
template cudaError_t contour_distances<float>(const Geo&, const float*, const double*, double, double, double,
                                              ContourDist*, cudaStream_t);
template cudaError_t contour_distances<double>(const Geo&, const double*, const double*, double, double, double,
                                               ContourDist*, cudaStream_t);

}  // namespace lsgb
