// reduce.cu -- deterministic on-device reductions over the interior cells.
//
// Two passes with a fixed grid: pass 1 reduces a grid-stride share per block
// (warp shuffles, then one shared-memory step across the block's warps) into
// `partials`; pass 2 reduces the partials in a single block in a fixed order.
// The result is therefore the same bits on every run for a given grid size.
// Sums accumulate in FP64 whatever the field precision.
//
// Reference counterparts: computeInterfaceVolume (Local_code/level-set_MPI_3D/
// include/io.h:263-288), computeL2Error3D (io.h:229-258), and the velocity
// maximum behind calculateTimeStep (config.h:272-293).  The reference copies
// the field to the host for these (Local_code/level-set_GPU_3D/src/main.cu:54-104).
#include "common.cuh"

#include <cfloat>

namespace lsgb {
namespace {

enum { OP_SUM = 0, OP_MAX = 1 };

template <int OP>
__device__ __forceinline__ double combine(double a, double b) {
    return OP == OP_SUM ? a + b : fmax(a, b);
}

template <int OP>
__device__ __forceinline__ double identity() {
    return OP == OP_SUM ? 0.0 : -DBL_MAX;
}

// Block-wide reduction of two values; result valid in thread 0.
template <int OP>
__device__ __forceinline__ void block_reduce2(double& a, double& b) {
    __shared__ double sa[RED_THREADS / 32], sb[RED_THREADS / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a = combine<OP>(a, __shfl_down_sync(0xffffffffu, a, o));
        b = combine<OP>(b, __shfl_down_sync(0xffffffffu, b, o));
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { sa[wid] = a; sb[wid] = b; }
    __syncthreads();
    if (wid == 0) {
        a = lane < RED_THREADS / 32 ? sa[lane] : identity<OP>();
        b = lane < RED_THREADS / 32 ? sb[lane] : identity<OP>();
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a = combine<OP>(a, __shfl_down_sync(0xffffffffu, a, o));
            b = combine<OP>(b, __shfl_down_sync(0xffffffffu, b, o));
        }
    }
}

template <int OP, typename F>
__global__ void __launch_bounds__(RED_THREADS) red_pass1(Geo g, F f, double* partials) {
    double a = identity<OP>(), b = identity<OP>();
    const long long n = g.cells();
    const long long nxy = (long long)g.nx * g.ny;
    for (long long e = blockIdx.x * (long long)RED_THREADS + threadIdx.x; e < n;
         e += (long long)gridDim.x * RED_THREADS) {
        const int k = (int)(e / nxy);
        const long long r = e - (long long)k * nxy;
        const int j = (int)(r / g.nx);
        const int i = (int)(r - (long long)j * g.nx);
        double x, y;
        f(i, j, k, x, y);
        a = combine<OP>(a, x);
        b = combine<OP>(b, y);
    }
    block_reduce2<OP>(a, b);
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = a;
        partials[2 * blockIdx.x + 1] = b;
    }
}

template <int OP>
__global__ void __launch_bounds__(RED_THREADS) red_pass2(int nblocks, const double* partials, double* out) {
    double a = identity<OP>(), b = identity<OP>();
    for (int q = threadIdx.x; q < nblocks; q += RED_THREADS) {
        a = combine<OP>(a, partials[2 * q]);
        b = combine<OP>(b, partials[2 * q + 1]);
    }
    block_reduce2<OP>(a, b);
    if (threadIdx.x == 0) { out[0] = a; out[1] = b; }
}

template <int OP, typename F>
cudaError_t run_reduce(const Geo& g, F f, double* partials, double* out, cudaStream_t st) {
    long long want = (g.cells() + RED_THREADS - 1) / RED_THREADS;
    int nb = (int)(want < RED_BLOCKS ? (want < 1 ? 1 : want) : RED_BLOCKS);
    red_pass1<OP><<<nb, RED_THREADS, 0, st>>>(g, f, partials);
    red_pass2<OP><<<1, RED_THREADS, 0, st>>>(nb, partials, out);
    count_launches(2);
    return cudaGetLastError();
}

__host__ __device__ __forceinline__ long long addr(const Lay& l, int i, int j, int k) {
    return l.off + i + (long long)j * l.sy + (long long)k * l.sz;
}

template <typename T>
struct CountNeg {
    Lay l;
    const T* G;
    __device__ void operator()(int i, int j, int k, double& x, double& y) const {
        x = G[addr(l, i, j, k)] < (T)0 ? 1.0 : 0.0;
        y = 0.0;
    }
};

template <typename T>
struct SqDiff {
    Lay l, rl;
    const T* G;
    const double* R;
    __device__ void operator()(int i, int j, int k, double& x, double& y) const {
        const double d = (double)G[addr(l, i, j, k)] - R[addr(rl, i, j, k)];
        x = d * d;
        y = 0.0;
    }
};

template <typename T>
struct Speed {
    Lay l;
    const T *u, *v, *w;
    __device__ void operator()(int i, int j, int k, double& x, double& y) const {
        const long long a = addr(l, i, j, k);
        const double uu = (double)u[a], vv = (double)v[a], ww = w ? (double)w[a] : 0.0;
        x = fabs(uu) + fabs(vv) + fabs(ww);
        y = sqrt(uu * uu + vv * vv + ww * ww);
    }
};

template <typename T>
struct NonFinite {
    Lay l;
    const T* G;
    __device__ void operator()(int i, int j, int k, double& x, double& y) const {
        x = isfinite((double)G[addr(l, i, j, k)]) ? 0.0 : 1.0;
        y = 0.0;
    }
};

}  // namespace

template <typename T>
cudaError_t launch_count_negative(const Geo& g, const Lay& lay, const T* G, double* partials,
                                  double* out, cudaStream_t st) {
    return run_reduce<OP_SUM>(g, CountNeg<T>{lay, G}, partials, out, st);
}

template <typename T>
cudaError_t launch_sq_diff(const Geo& g, const Lay& lay, const T* G, const double* Gref,
                           const Lay& ref_lay, double* partials, double* out, cudaStream_t st) {
    return run_reduce<OP_SUM>(g, SqDiff<T>{lay, ref_lay, G, Gref}, partials, out, st);
}

template <typename T>
cudaError_t launch_max_speed(const Geo& g, const Lay& lay, const T* u, const T* v, const T* w,
                             double* partials, double* out, cudaStream_t st) {
    return run_reduce<OP_MAX>(g, Speed<T>{lay, u, v, g.dim == 3 ? w : nullptr}, partials, out, st);
}

template <typename T>
cudaError_t launch_nonfinite(const Geo& g, const Lay& lay, const T* G, double* partials,
                             double* out, cudaStream_t st) {
    return run_reduce<OP_SUM>(g, NonFinite<T>{lay, G}, partials, out, st);
}

template cudaError_t launch_count_negative<float>(const Geo&, const Lay&, const float*, double*, double*, cudaStream_t);
template cudaError_t launch_count_negative<double>(const Geo&, const Lay&, const double*, double*, double*, cudaStream_t);
template cudaError_t launch_sq_diff<float>(const Geo&, const Lay&, const float*, const double*, const Lay&, double*, double*, cudaStream_t);
template cudaError_t launch_sq_diff<double>(const Geo&, const Lay&, const double*, const double*, const Lay&, double*, double*, cudaStream_t);
template cudaError_t launch_max_speed<float>(const Geo&, const Lay&, const float*, const float*, const float*, double*, double*, cudaStream_t);
template cudaError_t launch_max_speed<double>(const Geo&, const Lay&, const double*, const double*, const double*, double*, double*, cudaStream_t);
template cudaError_t launch_nonfinite<float>(const Geo&, const Lay&, const float*, double*, double*, cudaStream_t);
template cudaError_t launch_nonfinite<double>(const Geo&, const Lay&, const double*, double*, double*, cudaStream_t);

}  // namespace lsgb
