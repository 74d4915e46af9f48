// common.cuh -- shared declarations of the GB300 level-set library.
//
// Geometry, array layouts and the internal launch interface between the
// translation units:
//   f64_kernels.cu  FP64 kernels in the reference's exact operation order
//                   (compiled with --fmad=false)
//   f32_kernels.cu  FP32-bulk kernels (tiled, fast math) with the FP64 HCR-2
//                   interface constraint
//   reduce.cu       deterministic two-pass reductions (volume, L2, max speed)
//   synth.cu        on-device synthetic benchmark fields
//   api.cu          the C ABI (include/lsgb.h), solver handle, CUDA graphs
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <vector>

#include "../../include/lsgb.h"

namespace lsgb {

constexpr int NG = 3;  // ghost cells per side (reference config.h:31)

// Interior grid and boundary codes.
struct Geo {
    int dim;
    int nx, ny, nz;        // nz == 1 in 2D
    int bcx, bcy, bcz;     // LSGB_BC_*
    __host__ __device__ long long cells() const { return (long long)nx * ny * nz; }
};

// Storage of one field: element (i, j, k) of the interior lives at
// off + i + j * sy + k * sz.  Ghosted arrays (the reference layout) have
// off = 3 + 3 sy + 3 sz; compact arrays off = 0.
struct Lay {
    long long off, sy, sz;
    int ghosted;
};

inline Lay ghosted_layout(const Geo& g) {
    Lay l;
    long long nxT = g.nx + 2 * NG, nyT = g.ny + 2 * NG;
    l.sy = nxT;
    l.sz = g.dim == 3 ? nxT * nyT : 0;
    l.off = NG + NG * l.sy + (g.dim == 3 ? NG * l.sz : 0);
    l.ghosted = 1;
    return l;
}

inline Lay compact_layout(const Geo& g) {
    Lay l;
    l.sy = g.nx;
    l.sz = g.dim == 3 ? (long long)g.nx * g.ny : 0;
    l.off = 0;
    l.ghosted = 0;
    return l;
}

inline long long layout_elems(const Geo& g, int ghosted) {
    if (ghosted)
        return (long long)(g.nx + 2 * NG) * (g.ny + 2 * NG) * (g.dim == 3 ? g.nz + 2 * NG : 1);
    return g.cells();
}

// Periodic wrap / zero-gradient clamp of an interior coordinate that is at
// most 3 cells outside [0, n).  Periodic needs n >= 3 (checked at set-up).
__host__ __device__ __forceinline__ int map_axis(int i, int n, int bc) {
    if (bc == LSGB_BC_PERIODIC) return i < 0 ? i + n : (i >= n ? i - n : i);
    return i < 0 ? 0 : (i >= n ? n - 1 : i);
}

// Physics / step coefficients handed to the stage kernels.
struct StageArgs {
    Geo g;
    Lay lay;                 // layout of G fields and velocity
    const void* Gin;         // field the RHS is evaluated on
    const void* Gn;          // field at the start of the RK3 step
    void* Gout;
    const void* u;
    const void* v;
    const void* w;
    const void* sl;          // nullable per-cell flame speed (same layout)
    double s_l, eps, dx, dy, dz, dt;
    int stage;               // 1, 2, 3
    int* err;                // nullable device error flag (bounded waits)
    int tile;                // tile-shape choice (0 = default; see lsgb_solver_set_tile)
    int drop_copies;         // test hook: the TMA-fed kernel issues no bulk copies (its waits time out)
    // FP32 3D only: when set, the velocity is the deformation vortex evaluated
    // in the stage kernel from these factor tables at time factor tf (u, v, w unused)
    const float* defo;
    float tf;
};

// HCR-2 pseudo-step arguments (handle path: r~ and flags recomputed from phi0).
struct ReinitArgs {
    Geo g;
    Lay lay;
    const void* phin;
    const void* phi0;
    void* phinew;
    double dx, dy, dz, dtau, beta;
    // FP32 only, nullable: the pseudo-step also stores phi0 here (a copy that
    // lets a later pseudo-step write its result into phi0's buffer)
    void* phi0_copy = nullptr;
};

// Drop-in (ghosted, FP64) reinit pieces with stored r~ and flags.
cudaError_t launch_crossings_f64(const Geo& g, const Lay& lay, const double* phi0,
                                 double* rt, int32_t* flag, cudaStream_t st);
cudaError_t launch_reinit_step_stored_f64(const Geo& g, const Lay& lay, const double* phin,
                                          double* phinew, const double* phi0, const double* rt,
                                          const int32_t* flag, double dx, double dy, double dz,
                                          double dtau, double beta, cudaStream_t st);

cudaError_t launch_stage_f64(const StageArgs& a, cudaStream_t st);
cudaError_t launch_stage_f32(const StageArgs& a, cudaStream_t st);
// err: device flag set when a bounded in-kernel wait gives up (nullable: no TMA path)
cudaError_t launch_stage3d_f32_tiled(const StageArgs& a, int* err, cudaStream_t st);
// Grids on which launch_stage3d_f32_tiled evaluates the deformation vortex in
// the stage kernel (StageArgs::defo): nx % 4 == 0 (bulk-tensor staging) and
// fewer than 2^31 cells.
bool stage3d_f32_fuses_deformation(const Geo& g);
// The 2D FP32 stage (stage2d_f32.cu): row-pair tiles of 32 x 32 cells.
cudaError_t launch_stage2d_f32_tiled(const StageArgs& a, cudaStream_t st);
cudaError_t launch_reinit_f64(const ReinitArgs& a, cudaStream_t st);
cudaError_t launch_reinit_f32(const ReinitArgs& a, cudaStream_t st);

// Grouped launches of a batch (FP32, compact, < 2^31 cells per instance):
// one launch runs a stage (or an HCR-2 pseudo-step, or the copy back) of
// every instance of one dimensionality.  The host fills one descriptor per
// instance (*_fill returns the launch's blocks or tiles), copies the table to
// the device, and launches with the device table.
struct GroupInst {
    StageArgs a;        // geometry, physics, velocity, S_L, tile choice, error flag
    float *G, *A, *B;   // the instance's fixed buffers (stage 1 G->A, 2 A->B, 3 B->G)
    double dtau, beta;  // HCR-2 pseudo-step
};
// Each *_fill writes the descriptors and appends, for every block (tile) of
// the launch, the index of its instance to `owner` (a lookup table the
// kernels read once per block / tile).
size_t group3_desc_bytes();
// Planes one CTA of this 3D instance marches (its z-chunk, or nz if shorter)
int stage3d_chunk_planes(const StageArgs& a);
void group3_fill(const GroupInst* in, int n, void* host_table, std::vector<int>& owner);
cudaError_t launch_stage3d_f32_group(const void* table, const int* owner, int n, long long blocks, int stage,
                                     cudaStream_t st);
// 2D: shape 32 (32 x 32 tiles) or 16 (32 x 16 tiles), one shape per launch
size_t group2_desc_bytes();
void group2_fill(const GroupInst* in, int n, int shape, void* host_table, std::vector<int>& owner);
cudaError_t launch_stage2d_f32_group(const void* table, const int* owner, int n, long long tiles, int stage,
                                     int shape, cudaStream_t st);
// HCR-2 pseudo-step `iter` (0-based) of `iters` for every instance.  Even
// count: the handle's copy-free roles (iter 0: G -> A keeping phi0 in B; odd
// iters A -> G, even ones G -> A, phi0 from B), the result in G and no copy
// back.  Odd count: iter 0 reads G, iter m > 0 reads the buffer pseudo-step
// m-1 wrote (A for even m-1, B for odd), iteration m writes A (m even) or B
// (m odd), and the copy back sets G to the last one's buffer.  All instances
// of one table have the same dimensionality.
size_t groupr_desc_bytes();
void groupr_fill(const GroupInst* in, int n, void* host_table, std::vector<int>& owner,
                 std::vector<int>& copy_owner);
cudaError_t launch_reinit_f32_group(const void* table, const int* owner, int n, long long blocks, int dim, int iter,
                                    int iters, cudaStream_t st);
cudaError_t launch_copy_back_group(const void* table, const int* copy_owner, int n, long long copy_blocks, int iters,
                                   cudaStream_t st);

// Ghost fill of a ghosted FP64 array from its interior (periodic images /
// zero-gradient copies), the state the reference's boundary fill leaves.
cudaError_t launch_bc_fill_f64(const Geo& g, double* G, cudaStream_t st);

// Layout / precision conversion between an FP64 array (src layout) and a
// compact T array; to_ghosted also fills the ghosts.
cudaError_t launch_pack_f64(const Geo& g, const double* src, const Lay& src_lay, double* dst,
                            cudaStream_t st);
cudaError_t launch_pack_f32(const Geo& g, const double* src, const Lay& src_lay, float* dst,
                            cudaStream_t st);
cudaError_t launch_unpack_f64(const Geo& g, const double* src, double* dst, const Lay& dst_lay,
                              cudaStream_t st);
cudaError_t launch_unpack_f32(const Geo& g, const float* src, double* dst, const Lay& dst_lay,
                              cudaStream_t st);

// Reductions.  `partials` is scratch of at least reduce_scratch_bytes();
// results land in device memory `out` (host reads them after a sync).
constexpr int RED_BLOCKS = 1024;
constexpr int RED_THREADS = 256;
inline size_t reduce_scratch_bytes() { return sizeof(double) * 2 * (RED_BLOCKS + 1); }

// out[0] = count of interior cells with G < 0 (as double, exact below 2^53)
template <typename T>
cudaError_t launch_count_negative(const Geo& g, const Lay& lay, const T* G, double* partials,
                                  double* out, cudaStream_t st);
// out[0] = sum over interior of (G - Gref)^2 in FP64 (Gref FP64, its own layout)
template <typename T>
cudaError_t launch_sq_diff(const Geo& g, const Lay& lay, const T* G, const double* Gref,
                           const Lay& ref_lay, double* partials, double* out, cudaStream_t st);
// out[0] = max over interior of |u|+|v|(+|w|); out[1] = max of sqrt(u^2+v^2+w^2)
template <typename T>
cudaError_t launch_max_speed(const Geo& g, const Lay& lay, const T* u, const T* v, const T* w,
                             double* partials, double* out, cudaStream_t st);
// out[0] = 1 if any interior G is not finite
template <typename T>
cudaError_t launch_nonfinite(const Geo& g, const Lay& lay, const T* G, double* partials,
                             double* out, cudaStream_t st);

// Self-test of the FP64 kernels' division by a known reciprocal against IEEE
// division: bad (device) counts mismatching results over n seeded pairs.
cudaError_t launch_div_check(long long n, uint64_t seed, unsigned long long* bad, cudaStream_t st);

// Synthetic fields: writes FP64 compact arrays G, u, v, w (w ignored in 2D).
cudaError_t launch_synth(const Geo& g, const lsgb_synth& d, double dx, double dy, double dz,
                         double* G, double* u, double* v, double* w, cudaStream_t st);
// Deformation vortex (synth.cu).  FP64: the reference's per-cell products at
// time t.  FP32: time-independent factor tables (deformation_table_floats
// floats, built once per grid) and the field at tf = cos(pi t / T).
// LiveAt: when tab is set, the time (FP64, double t) or time factor (FP32,
// float tf) is read on the device from tab[*base + q] instead -- a batch's
// per-step table, with base advanced on the device between graph replays.
struct LiveAt {
    const void* tab = nullptr;
    const int* base = nullptr;
    int q = 0;
};
cudaError_t launch_deformation_f64(const Geo& g, double dx, double dy, double dz, double t, double Tp,
                                   double* u, double* v, double* w, cudaStream_t st, LiveAt at = LiveAt());
size_t deformation_table_floats(const Geo& g);
cudaError_t launch_deformation_tables_f32(const Geo& g, double dx, double dy, double dz, float* tab,
                                          cudaStream_t st);
cudaError_t launch_deformation_f32(const Geo& g, const float* tab, float tf, float* u, float* v, float* w,
                                   cudaStream_t st, LiveAt at = LiveAt());
// *base += n (one thread): a batch's live-table cursor after a launch sequence
cudaError_t launch_live_advance(int* base, int n, cudaStream_t st);

// Views into the FP32 factor tables: per axis [sin^2(pi x_i)], [sin(2 pi x_i)],
// n + 1 entries each (the last 0, so a plane pair may read one past nz).
struct DeformTables {
    const float *sqx, *s2x, *sqy, *s2y, *sqz, *s2z;
};
__host__ __device__ __forceinline__ DeformTables deform_tables(const Geo& g, const float* tab) {
    DeformTables d;
    d.sqx = tab;
    d.s2x = d.sqx + g.nx + 1;
    d.sqy = d.s2x + g.nx + 1;
    d.s2y = d.sqy + g.ny + 1;
    d.sqz = d.s2y + g.ny + 1;
    d.s2z = d.sqz + g.nz + 1;
    return d;
}
cudaError_t launch_scale3(long long n, double s, double* u, double* v, double* w, cudaStream_t st);

// Allocation-free interior G < 0 count (noalloc.cu); writes the host double
// *count and synchronises st.  Grid size screened by the caller.
cudaError_t noalloc_count_negative_f64(const Geo& g, const Lay& lay, const double* G, double* count,
                                       cudaStream_t st);

// Discrete adjoint (adjoint.cu).  Compact periodic fields of type T; the
// stage transpose has ADJ_PLANES coefficient planes, computed in z slabs
// (lsgb_adjoint_set_slab; one slab by default).
constexpr int ADJ_PLANES = 19;

// coefficient pass of the stage transpose: lam = adjoint of the stage
// output, cdt = (RHS weight of the stage) * dt; gS/gu/gv/gw (nullable, FP64)
// accumulate the point-wise parameter sensitivities.
struct AdjStageArgs {
    Geo g;
    const void* Gin;
    const void* u;
    const void* v;
    const void* w;
    const void* sl;
    double s_l, eps, dx, dy, dz, cdt;
    const void* lam;
    void* coef;
    double* gS;
    double* gu;
    double* gv;
    double* gw;
    // 3D z-slab: the pass covers the (unwrapped) planes z0-3 .. z0+zn+2 and
    // stores plane k of the slab at slab-local index k - (z0 - 3); plane
    // stride of the coefficient buffer = (zn + 6) nx ny.  Parameter
    // gradients only for z0 <= k < z0 + zn.  2D: z0 = 0, zn = 1, no halo.
    int z0, zn;
};
// gather pass: out = c_self lam + addend + transpose; acc (+)= c_n lam
struct AdjGatherArgs {
    Geo g;
    const void* coef;
    const void* lam;
    const void* addend;
    void* out;
    void* acc;
    int acc_init;
    double c_self, c_n;
    int z0, zn;  // planes gathered (3D): z0 .. z0+zn-1, coefficients as in AdjStageArgs
};
struct AdjReinitArgs {
    Geo g;
    const void* phin;
    const void* phi0;
    const void* mu;
    void* coef;
    double dx, dy, dz, dtau, beta;
};
struct AdjReinitGatherArgs {
    Geo g;
    const void* coef;
    void* mu_out;
    void* lam0;
    int first, last;
};
template <typename T>
cudaError_t launch_stage_adj(const AdjStageArgs& c, const AdjGatherArgs& gth, cudaStream_t st);
template <typename T>
cudaError_t launch_reinit_adj(const AdjReinitArgs& c, const AdjReinitGatherArgs& gth, cudaStream_t st);
// loss = 1/2 sum (H(G) - H(Gt))^2 dv into out[0]; lam (nullable) = dL/dG
template <typename T>
cudaError_t launch_heaviside(const Geo& g, const T* G, const double* Gt, double eps, double dv, T* lam,
                             double* partials, double* out, cudaStream_t st);

// Sample surface (sample_kernels.cu): n_inst Field2D arrays [ny+6][nx+6]
// back to back.  Velocity: the ghosted fields u, v (same stride) or, when u
// is NULL, the uniform pairs vel[2 (step n_inst + inst) + {0,1}] at
// step = *ctr.  init: the anchoring field (init_stride 0 = shared).
struct SampleArgs {
    int nx, ny, n_inst;
    const double* u;
    const double* v;
    const double* vel;
    int* ctr;
    const double* init;
    long long init_stride;
    double dx, dy, dt, S_L;
};
// stage 0 = the right-hand side alone (out = L(Gin)); 1..3 = RK3 stages
cudaError_t sample_launch_stage(const SampleArgs& a, int stage, const double* Gin, const double* Gn, double* out,
                                cudaStream_t st);
// anchored + periodic pair after a stage; bump advances *ctr
cudaError_t sample_launch_stage_bc(const SampleArgs& a, double* G, bool bump, cudaStream_t st);
cudaError_t sample_launch_anchored(const SampleArgs& a, double* G, cudaStream_t st);
cudaError_t sample_launch_periodic(const SampleArgs& a, double* G, cudaStream_t st);
cudaError_t sample_launch_reinit_step(const SampleArgs& a, const double* phi, double* out, double dtau,
                                      cudaStream_t st);
cudaError_t sample_launch_zero_ghosts(const SampleArgs& a, double* G, cudaStream_t st);
// compute_first_order_upwind, in place on G through tmp (one array)
cudaError_t sample_launch_first_order_upwind(const SampleArgs& a, double* G, double* tmp, cudaStream_t st);

// The FP64 array part of the reference's binary dump (dump.cu): from a
// compact state (x/z ghosts as the boundary fill leaves them, y ghosts =
// nearest interior row) or from a caller's ghosted array (y ghosts replaced).
template <typename T>
cudaError_t launch_dump_compact(const Geo& g, const T* G, double* out, cudaStream_t st);
cudaError_t launch_dump_ghosted(const Geo& g, const double* G, double* out, cudaStream_t st);

// analyze_error.m diagnostics (diag.cu): 14 reduced values at
// scratch + 14 * RED_BLOCKS (see diag.cu for their meaning).
size_t diag_scratch_bytes();
template <typename T>
cudaError_t launch_diagnostics(const Geo& g, const T* G, const double* Gr, double dx, double dy, double dz,
                               double* scratch, cudaStream_t st);

// Interface position error of analyze_error.m:51-84 (contour.cu): the zero
// contours of G and Gr as grid-edge crossing points, each point's distance
// to the nearest point of the other set; Hausdorff = the largest, mean over
// both sets.  NaN when either set is empty.  Synchronises the stream.
struct ContourDist {
    double hausdorff, mean;
    long long points, points_ref;
};
template <typename T>
cudaError_t contour_distances(const Geo& g, const T* G, const double* Gr, double dx, double dy, double dz,
                              ContourDist* out, cudaStream_t st);

// Bookkeeping of kernel launches (lsgb_launch_count).
void count_launches(uint64_t n);

}  // namespace lsgb
