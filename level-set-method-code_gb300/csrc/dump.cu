// dump.cu -- the reference's binary G dump image on the device.
//
// saveFieldBinary3D (Local_code/level-set_MPI_3D/include/io.h:33-131) writes
// int32[4] {nx, ny, nz, nghost} and then the whole ghosted FP64 array, whose
// x and z ghosts are what the boundary fill left and whose y ghosts are
// copies of the first / last interior row (io.h:112-124); the 2D
// saveFieldBinary (Local_code/level-set_MPI_2D/include/io.h:26-109) writes
// int32[3] {nx, ny, nghost} and the same kind of array.  These kernels build
// the FP64 array part; the host writes the header.
#include "common.cuh"

namespace lsgb {
namespace {

// From a compact state field: element (k, j, i) of the ghosted image takes
// the state at (map_z(k), clamp(j), map_x(i)) -- the boundary fill's value
// in x and z, the nearest interior row in y.
template <typename T>
__global__ void dump_compact_kernel(Geo g, const T* __restrict__ G, double* __restrict__ out) {
    const long long nxT = g.nx + 2 * NG, nyT = g.ny + 2 * NG;
    const long long nzT = g.dim == 3 ? g.nz + 2 * NG : 1;
    const long long total = nxT * nyT * nzT;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % nxT);
        const int j = (int)((e / nxT) % nyT);
        const int k = (int)(e / (nxT * nyT));
        const int si = map_axis(i - NG, g.nx, g.bcx);
        int sj = j - NG;
        sj = sj < 0 ? 0 : (sj >= g.ny ? g.ny - 1 : sj);
        const int sk = g.dim == 3 ? map_axis(k - NG, g.nz, g.bcz) : 0;
        out[e] = (double)G[((long long)sk * g.ny + sj) * g.nx + si];
    }
}

// From a ghosted FP64 array as the caller holds it: the y ghost rows become
// copies of the first / last interior row, everything else is copied.
__global__ void dump_ghosted_kernel(Geo g, const double* __restrict__ G, double* __restrict__ out) {
    const long long nxT = g.nx + 2 * NG, nyT = g.ny + 2 * NG;
    const long long nzT = g.dim == 3 ? g.nz + 2 * NG : 1;
    const long long total = nxT * nyT * nzT;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long i = e % nxT;
        const int j = (int)((e / nxT) % nyT);
        const long long k = e / (nxT * nyT);
        const int sj = j < NG ? NG : (j >= g.ny + NG ? g.ny + NG - 1 : j);
        out[e] = G[(k * nyT + sj) * nxT + i];
    }
}

unsigned blocks_for(long long n) {
    long long b = (n + 255) / 256;
    return (unsigned)(b < 4096 ? (b < 1 ? 1 : b) : 4096);
}

}  // namespace

template <typename T>
cudaError_t launch_dump_compact(const Geo& g, const T* G, double* out, cudaStream_t st) {
    dump_compact_kernel<T><<<blocks_for(layout_elems(g, 1)), 256, 0, st>>>(g, G, out);
    count_launches(1);
    return cudaGetLastError();
}
template cudaError_t launch_dump_compact<float>(const Geo&, const float*, double*, cudaStream_t);
template cudaError_t launch_dump_compact<double>(const Geo&, const double*, double*, cudaStream_t);

cudaError_t launch_dump_ghosted(const Geo& g, const double* G, double* out, cudaStream_t st) {
    dump_ghosted_kernel<<<blocks_for(layout_elems(g, 1)), 256, 0, st>>>(g, G, out);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace lsgb
