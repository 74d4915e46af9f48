// noalloc.cu -- allocation-free variant of the interface-volume reduction.
//
// lsgb_volume_f64 takes its reduction scratch from cudaMallocAsync on every
// call.  Some callers cannot let the library allocate device memory at that
// point:
//   - a host application whose own memory pool has already reserved the
//     device (a framework's caching allocator, or a coupled flow solver that
//     sizes its pool to the whole GPU), where an extra cudaMalloc fails or
//     forces the pool to give memory back;
//   - a monitoring hook that runs inside the caller's time loop and must not
//     block in the allocator.
// lsgb_volume_f64_noalloc serves them: its scratch is the file-scope device
// array below, a fixed 512 KiB that every GPU which loads the library keeps
// until the process exits.
//
// Contract (repeated in include/lsgb.h):
//   - At most LSGB_NOALLOC_MAX_CELLS interior cells per call (one partial
//     count per LSGB_NOALLOC_CHUNK cells, LSGB_NOALLOC_MAX_PARTIALS partials);
//     larger grids are rejected with LSGB_ERR_INVALID.
//   - The first call on a device looks up the array's device address
//     (cudaGetSymbolAddress, with that device current) and caches it for
//     that device's current context; make that first call before any stream
//     capture.  A call after cudaDeviceReset (a new context) looks it up
//     again.
//   - All calls share the one array, which keeps the last call's contents.
//     Calls whose work overlaps on the GPU (different streams, no ordering
//     between them) race on it and may return wrong results.
//   - No cudaMalloc, cudaFree or allocating library routine is called.
#include "common.cuh"

#include <cuda.h>

#include <mutex>

namespace lsgb {
namespace {

constexpr long long CHUNK = LSGB_NOALLOC_CHUNK;
constexpr int MAX_PARTIALS = LSGB_NOALLOC_MAX_PARTIALS;
constexpr int NA_THREADS = 256;

// partials[0 .. MAX_PARTIALS) then the result slot.
static __device__ __align__(256) double g_noalloc_scratch[MAX_PARTIALS + 2];

// Pass 1: block b counts the interior cells with G < 0 among the cells
// [b*CHUNK, (b+1)*CHUNK) of the interior (x fastest), and overwrites
// partials[b].  Every slot pass 2 reads is written here first, so nothing
// from an earlier call is ever summed and no slot needs clearing.
__global__ void __launch_bounds__(NA_THREADS) noalloc_count_pass1(Geo g, Lay l, const double* __restrict__ G,
                                                                  double* __restrict__ partials) {
    const long long n = g.cells();
    const long long nxy = (long long)g.nx * g.ny;
    const long long begin = (long long)blockIdx.x * CHUNK;
    long long end = begin + CHUNK;
    if (end > n) end = n;
    unsigned int cnt = 0;
    for (long long e = begin + threadIdx.x; e < end; e += NA_THREADS) {
        const int k = (int)(e / nxy);
        const long long r = e - (long long)k * nxy;
        const int j = (int)(r / g.nx);
        const int i = (int)(r - (long long)j * g.nx);
        cnt += G[l.off + i + (long long)j * l.sy + (long long)k * l.sz] < 0.0 ? 1u : 0u;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    __shared__ unsigned int warp_cnt[NA_THREADS / 32];
    if ((threadIdx.x & 31) == 0) warp_cnt[threadIdx.x >> 5] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int tot = 0;
        for (int q = 0; q < NA_THREADS / 32; ++q) tot += warp_cnt[q];
        partials[blockIdx.x] = (double)tot;
    }
}

// Pass 2: one block sums partials[0 .. nb) in a fixed order into the result slot.
__global__ void __launch_bounds__(NA_THREADS) noalloc_count_pass2(int nb, double* __restrict__ scratch) {
    double s = 0.0;
    for (int q = threadIdx.x; q < nb; q += NA_THREADS) s += scratch[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    __shared__ double warp_sum[NA_THREADS / 32];
    if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double tot = 0.0;
        for (int q = 0; q < NA_THREADS / 32; ++q) tot += warp_sum[q];
        scratch[MAX_PARTIALS] = tot;
    }
}

constexpr int MAX_DEVICES = 64;
std::mutex g_setup_mu;
double* g_scratch_addr[MAX_DEVICES] = {nullptr};
unsigned long long g_scratch_ctx[MAX_DEVICES] = {0};  // context the address belongs to

// Unique id of the calling thread's current context (cuCtxGetId, through the
// runtime's driver entry points, so the library needs no -lcuda), or 0 when
// it cannot be read.  Ids are never reused within a process, unlike context
// handles.
unsigned long long current_context_id() {
    typedef CUresult (*GetCurrent)(CUcontext*);
    typedef CUresult (*GetId)(CUcontext, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = (GetCurrent)p;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = (GetId)p;
    });
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS)
        return 0;
    return id;
}

// Device address of g_noalloc_scratch on the current device, looked up once
// per device and context: after cudaDeviceReset the primary context is
// created anew and the array lives at a new address, so a changed context id
// triggers a fresh lookup.  In host code the array's name is only a
// host-side stand-in, so it is never handed to a kernel directly.
cudaError_t scratch_address(double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= MAX_DEVICES) return cudaErrorInvalidDevice;
    const unsigned long long ctx = current_context_id();  // 0 before the device's first runtime call
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_addr[dev] || ctx == 0 || ctx != g_scratch_ctx[dev]) {
        double* p = nullptr;
        e = cudaGetSymbolAddress((void**)&p, g_noalloc_scratch);  // creates the context if needed
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = p;
        g_scratch_ctx[dev] = ctx ? ctx : current_context_id();
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

}  // namespace

// Called by lsgb_volume_f64_noalloc (api.cu) after the argument checks;
// `count` receives the exact number of interior cells with G < 0.
cudaError_t noalloc_count_negative_f64(const Geo& g, const Lay& lay, const double* G, double* count,
                                       cudaStream_t st) {
    double* scratch = nullptr;
    cudaError_t e = scratch_address(&scratch);
    if (e != cudaSuccess) return e;
    const long long n = g.cells();
    const int nb = (int)((n + CHUNK - 1) / CHUNK);
    if (nb < 1 || nb > MAX_PARTIALS) return cudaErrorInvalidValue;  // screened by the caller
    noalloc_count_pass1<<<nb, NA_THREADS, 0, st>>>(g, lay, G, scratch);
    noalloc_count_pass2<<<1, NA_THREADS, 0, st>>>(nb, scratch);
    count_launches(2);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = cudaMemcpyAsync(count, scratch + MAX_PARTIALS, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(st);
}

}  // namespace lsgb
