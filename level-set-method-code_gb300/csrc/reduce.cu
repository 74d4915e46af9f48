// reduce.cu -- deterministic on-device reductions over the interior cells.
//
// Two passes with a fixed grid: pass 1 reduces a fixed share of rows per
// block (warp shuffles, then one shared-memory step across the block's warps)
// into `partials`; pass 2 reduces the partials in a single block in a fixed
// order.  The result is therefore the same bits on every run for a given grid
// size.  Sums accumulate in FP64 whatever the field precision; counts in
// 64-bit integers (exact; FP64 adds run at a small fraction of the FP32 rate
// on this GPU).
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

// Pass 1: one warp per row of the interior (rows (j, k) dealt round-robin
// to the grid's warps, lanes along x), so the loads are coalesced and no
// per-cell index arithmetic is needed.  The functor F keeps a per-thread
// state (F::State), adds cells to it (F::add) and hands two doubles to the
// block reduction (F::finish); F::OP is the combining operation.
template <typename F>
__global__ void __launch_bounds__(RED_THREADS) red_pass1(Geo g, F f, double* partials) {
    typename F::State st = F::init();
    constexpr int WPB = RED_THREADS / 32;
    const int lane = threadIdx.x & 31;
    const int nrows = g.ny * g.nz;
    for (int row = blockIdx.x * WPB + (threadIdx.x >> 5); row < nrows; row += gridDim.x * WPB) {
        const int k = row / g.ny;
        const int j = row - k * g.ny;
        for (int i = lane; i < g.nx; i += 32) f.add(st, i, j, k);
    }
    double a, b;
    F::finish(st, a, b);
    block_reduce2<F::OP>(a, b);
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = a;
        partials[2 * blockIdx.x + 1] = b;
    }
}

// Pass 2 over the block partials; SQRT_B takes the square root of the second
// result (a maximum of squares: sqrt is monotone, so this is the maximum of
// the roots bit for bit).
template <int OP, bool SQRT_B>
__global__ void __launch_bounds__(RED_THREADS) red_pass2(int nblocks, const double* partials, double* out) {
    double a = identity<OP>(), b = identity<OP>();
    for (int q = threadIdx.x; q < nblocks; q += RED_THREADS) {
        a = combine<OP>(a, partials[2 * q]);
        b = combine<OP>(b, partials[2 * q + 1]);
    }
    block_reduce2<OP>(a, b);
    if (threadIdx.x == 0) {
        out[0] = a;
        out[1] = SQRT_B ? sqrt(b) : b;
    }
}

template <typename F, bool SQRT_B = false>
cudaError_t run_reduce(const Geo& g, F f, double* partials, double* out, cudaStream_t st) {
    const long long rows = (long long)g.ny * g.nz;
    const long long want = (rows + RED_THREADS / 32 - 1) / (RED_THREADS / 32);
    const int nb = (int)(want < RED_BLOCKS ? (want < 1 ? 1 : want) : RED_BLOCKS);
    red_pass1<F><<<nb, RED_THREADS, 0, st>>>(g, f, partials);
    red_pass2<F::OP, SQRT_B><<<1, RED_THREADS, 0, st>>>(nb, partials, out);
    count_launches(2);
    return cudaGetLastError();
}

__host__ __device__ __forceinline__ long long addr(const Lay& l, int i, int j, int k) {
    return l.off + i + (long long)j * l.sy + (long long)k * l.sz;
}

// Cells with G < 0, counted exactly in a 64-bit integer per thread.
template <typename T>
struct CountNeg {
    static constexpr int OP = OP_SUM;
    using State = long long;
    Lay l;
    const T* G;
    __device__ static State init() { return 0; }
    __device__ void add(State& s, int i, int j, int k) const { s += G[addr(l, i, j, k)] < (T)0 ? 1 : 0; }
    __device__ static void finish(State s, double& a, double& b) { a = (double)s; b = 0.0; }
};

// sum of (G - R)^2 in FP64.
template <typename T>
struct SqDiff {
    static constexpr int OP = OP_SUM;
    using State = double;
    Lay l, rl;
    const T* G;
    const double* R;
    __device__ static State init() { return 0.0; }
    __device__ void add(State& s, int i, int j, int k) const {
        const double d = (double)G[addr(l, i, j, k)] - R[addr(rl, i, j, k)];
        s += d * d;
    }
    __device__ static void finish(State s, double& a, double& b) { a = s; b = 0.0; }
};

// max(|u| + |v| + |w|) and max(u^2 + v^2 + w^2) in FP64 (the root is taken
// once, in pass 2).
template <typename T>
struct Speed {
    static constexpr int OP = OP_MAX;
    struct State {
        double l1, sq;
    };
    Lay l;
    const T *u, *v, *w;
    __device__ static State init() { return State{-DBL_MAX, -DBL_MAX}; }
    __device__ void add(State& s, int i, int j, int k) const {
        const long long a = addr(l, i, j, k);
        const double uu = (double)u[a], vv = (double)v[a], ww = w ? (double)w[a] : 0.0;
        s.l1 = fmax(s.l1, fabs(uu) + fabs(vv) + fabs(ww));
        s.sq = fmax(s.sq, uu * uu + vv * vv + ww * ww);
    }
    __device__ static void finish(State s, double& a, double& b) { a = s.l1; b = s.sq; }
};

// Cells whose value is not finite, counted exactly.
template <typename T>
struct NonFinite {
    static constexpr int OP = OP_SUM;
    using State = long long;
    Lay l;
    const T* G;
    __device__ static State init() { return 0; }
    __device__ void add(State& s, int i, int j, int k) const { s += isfinite((double)G[addr(l, i, j, k)]) ? 0 : 1; }
    __device__ static void finish(State s, double& a, double& b) { a = (double)s; b = 0.0; }
};

}  // namespace

template <typename T>
cudaError_t launch_count_negative(const Geo& g, const Lay& lay, const T* G, double* partials,
                                  double* out, cudaStream_t st) {
    return run_reduce(g, CountNeg<T>{lay, G}, partials, out, st);
}

template <typename T>
cudaError_t launch_sq_diff(const Geo& g, const Lay& lay, const T* G, const double* Gref,
                           const Lay& ref_lay, double* partials, double* out, cudaStream_t st) {
    return run_reduce(g, SqDiff<T>{lay, ref_lay, G, Gref}, partials, out, st);
}

template <typename T>
cudaError_t launch_max_speed(const Geo& g, const Lay& lay, const T* u, const T* v, const T* w,
                             double* partials, double* out, cudaStream_t st) {
    return run_reduce<Speed<T>, true>(g, Speed<T>{lay, u, v, g.dim == 3 ? w : nullptr}, partials, out, st);
}

template <typename T>
cudaError_t launch_nonfinite(const Geo& g, const Lay& lay, const T* G, double* partials,
                             double* out, cudaStream_t st) {
    return run_reduce(g, NonFinite<T>{lay, G}, partials, out, st);
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
