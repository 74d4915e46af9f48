// api.cu -- the C ABI declared in include/lsgb.h.
//
// Host logic only: parameter checks, error reporting, the drop-in FP64
// entry points over caller-owned ghosted arrays, and the solver handle that
// keeps compact device-resident fields and sequences the kernels of
// f64_kernels.cu / f32_kernels.cu / reduce.cu / synth.cu on one stream.
#include "common.cuh"
#include "host.hpp"

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

namespace lsgb {

static std::atomic<uint64_t> g_launches{0};
void count_launches(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
// launches recorded into a graph during capture run only when the graph does
void uncount_launches(uint64_t n) { g_launches.fetch_sub(n, std::memory_order_relaxed); }

// Host helpers shared with the other host-side translation units (host.hpp).

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}


Geo geo_of(const lsgb_params& p) {
    Geo g;
    g.dim = p.dim;
    g.nx = p.nx;
    g.ny = p.ny;
    g.nz = p.dim == 3 ? p.nz : 1;
    g.bcx = p.bc_x;
    g.bcy = p.bc_y;
    g.bcz = p.dim == 3 ? p.bc_z : LSGB_BC_PERIODIC;
    return g;
}

bool finite_pos(double x) { return std::isfinite(x) && x > 0.0; }

int check_params(const lsgb_params* p) {
    if (!p) return fail(LSGB_ERR_INVALID, "params is NULL");
    if (p->dim != 2 && p->dim != 3) return fail(LSGB_ERR_INVALID, "dim must be 2 or 3 (got %d)", p->dim);
    if (p->nghost != NG) return fail(LSGB_ERR_INVALID, "nghost must be 3 (got %d)", p->nghost);
    if (p->nx < 3 || p->ny < 3 || (p->dim == 3 && p->nz < 3))
        return fail(LSGB_ERR_INVALID, "every axis needs at least 3 interior cells (got %d x %d x %d)",
                    p->nx, p->ny, p->dim == 3 ? p->nz : 1);
    long long tot = (long long)(p->nx + 6) * (p->ny + 6) * (p->dim == 3 ? p->nz + 6 : 1);
    if (tot > (1LL << 34)) return fail(LSGB_ERR_INVALID, "grid too large (%lld cells with ghosts)", tot);
    if (!finite_pos(p->dx) || !finite_pos(p->dy) || (p->dim == 3 && !finite_pos(p->dz)))
        return fail(LSGB_ERR_INVALID, "grid spacing must be positive and finite");
    if (!std::isfinite(p->dt) || p->dt < 0.0) return fail(LSGB_ERR_INVALID, "dt must be finite and >= 0");
    if (!std::isfinite(p->s_l)) return fail(LSGB_ERR_INVALID, "s_l must be finite");
    if (!std::isfinite(p->epsilon) || p->epsilon < 0.0) return fail(LSGB_ERR_INVALID, "epsilon must be finite and >= 0");
    int bcs[3] = {p->bc_x, p->bc_y, p->dim == 3 ? p->bc_z : 0};
    for (int a = 0; a < 3; ++a)
        if (bcs[a] != LSGB_BC_PERIODIC && bcs[a] != LSGB_BC_ZERO_GRADIENT)
            return fail(LSGB_ERR_INVALID, "unknown boundary code %d on axis %d", bcs[a], a);
    if (p->enable_reinit) {
        if (p->reinit_interval < 1) return fail(LSGB_ERR_INVALID, "reinit_interval must be >= 1");
        if (p->reinit_iterations < 0) return fail(LSGB_ERR_INVALID, "reinit_iterations must be >= 0");
        if (!std::isfinite(p->reinit_dtau) || !std::isfinite(p->reinit_beta))
            return fail(LSGB_ERR_INVALID, "reinit_dtau / reinit_beta must be finite");
    }
    return LSGB_OK;
}

int check_dev(const void* ptr, const char* name) {
    if (!ptr) return fail(LSGB_ERR_INVALID, "%s is NULL", name);
    cudaPointerAttributes at;
    cudaError_t e = cudaPointerGetAttributes(&at, ptr);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(LSGB_ERR_INVALID, "%s: cudaPointerGetAttributes failed: %s", name, cudaGetErrorString(e));
    }
    if (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)
        return fail(LSGB_ERR_INVALID, "%s is not device memory", name);
    return LSGB_OK;
}

StageArgs stage_args(const lsgb_params& p, const Geo& g, const Lay& lay) {
    StageArgs a;
    std::memset(&a, 0, sizeof(a));
    a.g = g;
    a.lay = lay;
    a.s_l = p.s_l;
    a.eps = p.epsilon;
    a.dx = p.dx;
    a.dy = p.dy;
    a.dz = p.dim == 3 ? p.dz : p.dx;
    a.dt = p.dt;
    return a;
}

double cell_volume(const lsgb_params& p) {
    return p.dim == 3 ? p.dx * p.dy * p.dz : p.dx * p.dy;
}

// Stream-ordered scratch for one reduction call of the drop-in API
// (partials + two result slots).
struct CallScratch {
    double* d = nullptr;
    cudaStream_t st;
    explicit CallScratch(cudaStream_t s) : st(s) {}
    int alloc() {
        cudaError_t e = cudaMallocAsync((void**)&d, reduce_scratch_bytes() + 2 * sizeof(double), st);
        if (e != cudaSuccess) { d = nullptr; return fail(LSGB_ERR_ALLOC, "scratch allocation failed: %s", cudaGetErrorString(e)); }
        return LSGB_OK;
    }
    double* partials() const { return d; }
    double* out() const { return d + 2 * (RED_BLOCKS + 1); }
    ~CallScratch() { if (d) cudaFreeAsync(d, st); }
};

int read_result(const double* dev, double* host2, cudaStream_t st) {
    LSGB_CUDA(cudaMemcpyAsync(host2, dev, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
    LSGB_CUDA(cudaStreamSynchronize(st));
    return LSGB_OK;
}

}  // namespace lsgb

using namespace lsgb;

// ---------------------------------------------------------------------------
// misc
// ---------------------------------------------------------------------------
extern "C" void lsgb_params_default(lsgb_params* p, int dim, int nx, int ny, int nz) {
    std::memset(p, 0, sizeof(*p));
    p->dim = dim;
    p->nx = nx;
    p->ny = ny;
    p->nz = dim == 3 ? nz : 1;
    p->nghost = NG;
    p->dx = 1.0 / nx;
    p->dy = 1.0 / ny;
    p->dz = dim == 3 ? 1.0 / nz : p->dx;
    p->s_l = 0.0;
    p->dt = 1.0e-3;
    p->cfl = 0.2;
    p->epsilon = 1.0e-10;
    p->enable_reinit = 0;
    p->reinit_interval = 10;
    p->reinit_iterations = 2;
    double h = dim == 3 ? std::fmin(p->dx, std::fmin(p->dy, p->dz)) : std::fmin(p->dx, p->dy);
    p->reinit_dtau = 0.25 * h;
    p->reinit_beta = 0.5;
    p->bc_x = p->bc_y = p->bc_z = LSGB_BC_PERIODIC;
}

extern "C" int lsgb_params_check(const lsgb_params* p) { return check_params(p); }
extern "C" const char* lsgb_last_error(void) { return g_err.c_str(); }
extern "C" const char* lsgb_version(void) { return "lsgb 0.1 (sm_103a)"; }
extern "C" uint64_t lsgb_launch_count(void) { return g_launches.load(); }

extern "C" int lsgb_cfl_dt(const lsgb_params* p, double max_speed, double* dt) {
    LSGB_TRY(check_params(p));
    if (!dt) return fail(LSGB_ERR_INVALID, "dt is NULL");
    double speed = max_speed + p->s_l;
    if (speed < p->epsilon) speed = 2.0;
    double dmin = p->dim == 3 ? std::fmin(p->dx, std::fmin(p->dy, p->dz)) : std::fmin(p->dx, p->dy);
    *dt = p->cfl * dmin / speed;
    return LSGB_OK;
}

// ---------------------------------------------------------------------------
// drop-in FP64 entry points (ghosted, caller-owned device buffers)
// ---------------------------------------------------------------------------
extern "C" int lsgb_rk3_step_f64(const lsgb_params* p, const double* G_n, double* G_new,
                                 double* G_1, double* G_2, const double* u, const double* v,
                                 const double* w, const double* s_l_field, void* stream) {
    LSGB_TRY(check_params(p));
    LSGB_TRY(check_dev(G_n, "G_n"));
    LSGB_TRY(check_dev(G_new, "G_new"));
    LSGB_TRY(check_dev(G_1, "G_1"));
    LSGB_TRY(check_dev(G_2, "G_2"));
    LSGB_TRY(check_dev(u, "u"));
    LSGB_TRY(check_dev(v, "v"));
    if (p->dim == 3) LSGB_TRY(check_dev(w, "w"));
    if (s_l_field) LSGB_TRY(check_dev(s_l_field, "s_l_field"));
    if (G_new == G_n || G_1 == G_n || G_2 == G_n || G_1 == G_2 || G_new == G_2)
        return fail(LSGB_ERR_INVALID, "G_new, G_1, G_2 must be distinct from G_n and each other");
    cudaStream_t st = (cudaStream_t)stream;
    Geo g = geo_of(*p);
    Lay lay = ghosted_layout(g);
    StageArgs a = stage_args(*p, g, lay);
    a.u = u; a.v = v; a.w = w; a.sl = s_l_field;
    a.Gn = G_n;
    a.Gin = G_n; a.Gout = G_1; a.stage = 1;
    LSGB_CUDA(launch_stage_f64(a, st));
    LSGB_CUDA(launch_bc_fill_f64(g, G_1, st));
    a.Gin = G_1; a.Gout = G_2; a.stage = 2;
    LSGB_CUDA(launch_stage_f64(a, st));
    LSGB_CUDA(launch_bc_fill_f64(g, G_2, st));
    a.Gin = G_2; a.Gout = G_new; a.stage = 3;
    LSGB_CUDA(launch_stage_f64(a, st));
    LSGB_CUDA(launch_bc_fill_f64(g, G_new, st));
    return LSGB_OK;
}

extern "C" int lsgb_apply_bc_f64(const lsgb_params* p, double* G, void* stream) {
    LSGB_TRY(check_params(p));
    LSGB_TRY(check_dev(G, "G"));
    LSGB_CUDA(launch_bc_fill_f64(geo_of(*p), G, (cudaStream_t)stream));
    return LSGB_OK;
}

extern "C" int lsgb_reinit_f64(const lsgb_params* p, double** phi, double** phi_tmp,
                               double* phi0, double* r_tilde, int32_t* flag, void* stream) {
    LSGB_TRY(check_params(p));
    if (!phi || !phi_tmp) return fail(LSGB_ERR_INVALID, "phi / phi_tmp handles are NULL");
    LSGB_TRY(check_dev(*phi, "*phi"));
    LSGB_TRY(check_dev(*phi_tmp, "*phi_tmp"));
    LSGB_TRY(check_dev(phi0, "phi0"));
    LSGB_TRY(check_dev(r_tilde, "r_tilde"));
    LSGB_TRY(check_dev(flag, "flag"));
    cudaStream_t st = (cudaStream_t)stream;
    Geo g = geo_of(*p);
    Lay lay = ghosted_layout(g);
    size_t bytes = sizeof(double) * (size_t)layout_elems(g, 1);
    LSGB_CUDA(cudaMemcpyAsync(phi0, *phi, bytes, cudaMemcpyDeviceToDevice, st));
    LSGB_CUDA(launch_bc_fill_f64(g, phi0, st));
    LSGB_CUDA(launch_crossings_f64(g, lay, phi0, r_tilde, flag, st));
    double* a = *phi;
    double* b = *phi_tmp;
    for (int it = 0; it < p->reinit_iterations; ++it) {
        LSGB_CUDA(launch_reinit_step_stored_f64(g, lay, a, b, phi0, r_tilde, flag, p->dx, p->dy,
                                                p->dim == 3 ? p->dz : p->dx, p->reinit_dtau,
                                                p->reinit_beta, st));
        std::swap(a, b);
        LSGB_CUDA(launch_bc_fill_f64(g, a, st));
    }
    *phi = a;
    *phi_tmp = b;
    return LSGB_OK;
}

extern "C" int lsgb_volume_f64(const lsgb_params* p, const double* G, double* volume,
                               int64_t* count, void* stream) {
    LSGB_TRY(check_params(p));
    LSGB_TRY(check_dev(G, "G"));
    cudaStream_t st = (cudaStream_t)stream;
    Geo g = geo_of(*p);
    CallScratch s(st);
    LSGB_TRY(s.alloc());
    LSGB_CUDA(launch_count_negative<double>(g, ghosted_layout(g), G, s.partials(), s.out(), st));
    double r[2];
    LSGB_TRY(read_result(s.out(), r, st));
    if (count) *count = (int64_t)r[0];
    if (volume) *volume = r[0] * cell_volume(*p);
    return LSGB_OK;
}

extern "C" int lsgb_volume_f64_noalloc(const lsgb_params* p, const double* G, double* volume,
                                       int64_t* count, void* stream) {
    LSGB_TRY(check_params(p));
    Geo g = geo_of(*p);
    if (g.cells() > LSGB_NOALLOC_MAX_CELLS)
        return fail(LSGB_ERR_INVALID,
                    "grid has %lld interior cells; lsgb_volume_f64_noalloc accepts at most %lld "
                    "(use lsgb_volume_f64)", g.cells(), (long long)LSGB_NOALLOC_MAX_CELLS);
    LSGB_TRY(check_dev(G, "G"));
    double cnt = 0.0;
    LSGB_CUDA(noalloc_count_negative_f64(g, ghosted_layout(g), G, &cnt, (cudaStream_t)stream));
    if (count) *count = (int64_t)cnt;
    if (volume) *volume = cnt * cell_volume(*p);
    return LSGB_OK;
}

extern "C" int lsgb_l2_error_f64(const lsgb_params* p, const double* G, const double* G_ref,
                                 double* l2, void* stream) {
    LSGB_TRY(check_params(p));
    LSGB_TRY(check_dev(G, "G"));
    LSGB_TRY(check_dev(G_ref, "G_ref"));
    if (!l2) return fail(LSGB_ERR_INVALID, "l2 is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    Geo g = geo_of(*p);
    Lay lay = ghosted_layout(g);
    CallScratch s(st);
    LSGB_TRY(s.alloc());
    LSGB_CUDA(launch_sq_diff<double>(g, lay, G, G_ref, lay, s.partials(), s.out(), st));
    double r[2];
    LSGB_TRY(read_result(s.out(), r, st));
    *l2 = std::sqrt(r[0] / (double)g.cells());
    return LSGB_OK;
}

extern "C" int lsgb_max_speed_f64(const lsgb_params* p, const double* u, const double* v,
                                  const double* w, double* max_speed, void* stream) {
    LSGB_TRY(check_params(p));
    LSGB_TRY(check_dev(u, "u"));
    LSGB_TRY(check_dev(v, "v"));
    if (p->dim == 3) LSGB_TRY(check_dev(w, "w"));
    if (!max_speed) return fail(LSGB_ERR_INVALID, "max_speed is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    Geo g = geo_of(*p);
    CallScratch s(st);
    LSGB_TRY(s.alloc());
    LSGB_CUDA(launch_max_speed<double>(g, ghosted_layout(g), u, v, w, s.partials(), s.out(), st));
    double r[2];
    LSGB_TRY(read_result(s.out(), r, st));
    *max_speed = r[0];
    return LSGB_OK;
}

// ---------------------------------------------------------------------------
// solver handle
// ---------------------------------------------------------------------------
struct lsgb_solver {
    lsgb_params p;
    Geo g;
    Lay lay;            // compact
    int prec;
    size_t esz;         // bytes per element of the state fields
    cudaStream_t st = nullptr;
    bool own_stream = false;
    void* G = nullptr;  // current field
    void* A = nullptr;  // the two other state buffers
    void* B = nullptr;
    void* u = nullptr;
    void* v = nullptr;
    void* w = nullptr;
    void* sl = nullptr;
    double* stage64 = nullptr;   // FP64 ghosted staging for host/layout conversion
    double* scratch = nullptr;   // reduction partials + results
    double* h_res = nullptr;     // pinned result slots
    int step = 0;
    // live deformation velocity (lsgb_solver_set_velocity_deformation_live):
    // every step uses the vortex at time vel_t, which then advances by dt
    bool vel_live = false;
    double vel_t = 0.0, vel_T = 1.0;
    float* defo_f32 = nullptr;  // FP32 factor tables of the vortex (built once)
    // set while a batch advances a live instance: the vortex time (FP64) or
    // time factor (FP32) of each step comes from the batch's device table
    LiveAt batch_live;
    int tile = 0;  // tile-shape choice handed to the stage kernels (0 = default)
    int drop_copies = 0;  // test hook (lsgb_solver_debug_drop_copies)
    // set when a kernel gave up with bulk copies still in flight into its
    // shared memory: every later call fails until the handle is destroyed
    bool unusable = false;
    bool have_G = false, have_vel = false;
    // kernel timing (lsgb_solver_enable_timing)
    bool timing = false;
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_used = 0;
    std::vector<std::pair<size_t, int>> ev_marks;  // (first event index, kind 0 stage / 1 reinit)
    struct Snapshots* snap = nullptr;  // asynchronous dump writer (lsgb_solver_snapshot)
};

// Asynchronous dump files: the image is packed on the solver's stream into
// one of two device slots, copied to a pinned host slot on a copy stream, and
// written to its file by a writer thread, so the time loop keeps running.
struct Snapshots {
    int device = 0;
    size_t hdr = 0, data = 0;          // header / array bytes of one image
    double* dev[2] = {nullptr, nullptr};
    char* host[2] = {nullptr, nullptr};
    cudaEvent_t packed[2] = {nullptr, nullptr}, copied[2] = {nullptr, nullptr};
    cudaStream_t cs = nullptr;
    bool busy[2] = {false, false};
    int next = 0;
    std::mutex m;
    std::condition_variable cv;
    std::deque<std::pair<int, std::string>> jobs;
    bool stop = false;
    std::string err;                   // first failure, reported by lsgb_solver_snapshot_wait
    std::thread th;
};

namespace {

size_t nbytes(const lsgb_solver* s) { return s->esz * (size_t)s->g.cells(); }

// Device flag (one int after the reduction slots) that kernels with bounded
// waits set when a wait gives up; cleared when reported.
int* err_flag(lsgb_solver* s) { return (int*)(s->scratch + 2 * (RED_BLOCKS + 1) + 2); }

// Flag values: 2 = a wait gave up while the block's bulk copies were in
// flight; the kernel drains them with bounded waits, but a copy that missed
// its limit may still write into shared memory that a later block owns, so
// the handle is marked unusable.  1 = a wait gave up with no copy in flight
// (the drop-copies test hook): the handle recovers once the flag is reported
// and cleared.
int flag_result(lsgb_solver* s, int flag) {
    if (!flag) return LSGB_OK;
    cudaMemsetAsync(err_flag(s), 0, sizeof(int), s->st);
    if (flag >= 2) {
        s->unusable = true;
        return fail(LSGB_ERR_CUDA, "a bounded in-kernel wait gave up with bulk copies still in flight; the handle "
                                   "is unusable: synchronise its stream and destroy it");
    }
    return fail(LSGB_ERR_CUDA, "a bounded in-kernel wait gave up (bulk copy did not arrive); results of the "
                               "last steps are not valid");
}

int ensure_stage(lsgb_solver* s) {
    if (s->stage64) return LSGB_OK;
    size_t b = sizeof(double) * (size_t)layout_elems(s->g, 1);
    cudaError_t e = cudaMalloc((void**)&s->stage64, b);
    if (e != cudaSuccess) { s->stage64 = nullptr; return fail(LSGB_ERR_ALLOC, "staging allocation (%zu B): %s", b, cudaGetErrorString(e)); }
    return LSGB_OK;
}

// Bring an FP64 array (layout, memory) into the compact state field dst.
int load_field(lsgb_solver* s, void* dst, const double* src, int layout, int memory) {
    Lay sl = layout == LSGB_LAYOUT_GHOSTED ? ghosted_layout(s->g) : compact_layout(s->g);
    size_t sbytes = sizeof(double) * (size_t)layout_elems(s->g, sl.ghosted);
    const double* dsrc = src;
    if (memory == LSGB_MEM_HOST) {
        if (s->prec == LSGB_PREC_F64 && !sl.ghosted) {
            LSGB_CUDA(cudaMemcpyAsync(dst, src, sbytes, cudaMemcpyHostToDevice, s->st));
            return LSGB_OK;
        }
        LSGB_TRY(ensure_stage(s));
        LSGB_CUDA(cudaMemcpyAsync(s->stage64, src, sbytes, cudaMemcpyHostToDevice, s->st));
        dsrc = s->stage64;
    } else {
        LSGB_TRY(check_dev(src, "field"));
        if (s->prec == LSGB_PREC_F64 && !sl.ghosted) {
            LSGB_CUDA(cudaMemcpyAsync(dst, src, sbytes, cudaMemcpyDeviceToDevice, s->st));
            return LSGB_OK;
        }
    }
    if (s->prec == LSGB_PREC_F64) LSGB_CUDA(launch_pack_f64(s->g, dsrc, sl, (double*)dst, s->st));
    else LSGB_CUDA(launch_pack_f32(s->g, dsrc, sl, (float*)dst, s->st));
    return LSGB_OK;
}

int alloc_field(lsgb_solver* s, void** f) {
    cudaError_t e = cudaMalloc(f, nbytes(s));
    if (e != cudaSuccess) { *f = nullptr; return fail(LSGB_ERR_ALLOC, "field allocation (%zu B): %s", nbytes(s), cudaGetErrorString(e)); }
    return LSGB_OK;
}

// Event pair around one timed launch (no-op unless timing is enabled).
int timed_begin(lsgb_solver* s, int kind, size_t* idx) {
    if (!s->timing) return LSGB_OK;
    while (s->ev_pool.size() < s->ev_used + 2) {
        cudaEvent_t e;
        LSGB_CUDA(cudaEventCreate(&e));
        s->ev_pool.push_back(e);
    }
    *idx = s->ev_used;
    s->ev_used += 2;
    s->ev_marks.push_back({*idx, kind});
    LSGB_CUDA(cudaEventRecord(s->ev_pool[*idx], s->st));
    return LSGB_OK;
}

int timed_end(lsgb_solver* s, size_t idx) {
    if (!s->timing) return LSGB_OK;
    LSGB_CUDA(cudaEventRecord(s->ev_pool[idx + 1], s->st));
    return LSGB_OK;
}

int launch_stage(lsgb_solver* s, const StageArgs& a) {
    size_t ev = 0;
    LSGB_TRY(timed_begin(s, 0, &ev));
    if (s->prec == LSGB_PREC_F64) LSGB_CUDA(launch_stage_f64(a, s->st));
    else LSGB_CUDA(launch_stage_f32(a, s->st));
    LSGB_TRY(timed_end(s, ev));
    return LSGB_OK;
}

// ---- deformation vortex (computeDeformationVelocity, Local_code/level-set_MPI_3D/
// include/initial_conditions.h:232-247; recomputed every step as in src/main.cpp:297-299)

int ensure_defo_tables(lsgb_solver* s) {
    if (s->defo_f32) return LSGB_OK;
    const size_t b = sizeof(float) * deformation_table_floats(s->g);
    cudaError_t e = cudaMalloc((void**)&s->defo_f32, b);
    if (e != cudaSuccess) { s->defo_f32 = nullptr; return fail(LSGB_ERR_ALLOC, "deformation tables: %s", cudaGetErrorString(e)); }
    LSGB_CUDA(launch_deformation_tables_f32(s->g, s->p.dx, s->p.dy, s->p.dz, s->defo_f32, s->st));
    return LSGB_OK;
}

float defo_time_factor(double t, double T) { return (float)std::cos(3.14159265358979323846 * t / T); }

// Write the vortex at time t (or at the time the device table of at names)
// into (u, v, w) on stream st.
int fill_deformation_into(lsgb_solver* s, double t, double T, void* u, void* v, void* w, cudaStream_t st,
                          LiveAt at = LiveAt()) {
    if (s->prec == LSGB_PREC_F64) {
        LSGB_CUDA(launch_deformation_f64(s->g, s->p.dx, s->p.dy, s->p.dz, t, T, (double*)u, (double*)v, (double*)w,
                                         st, at));
    } else {
        LSGB_TRY(ensure_defo_tables(s));
        LSGB_CUDA(launch_deformation_f32(s->g, s->defo_f32, defo_time_factor(t, T), (float*)u, (float*)v, (float*)w,
                                         st, at));
    }
    return LSGB_OK;
}

// Write the vortex at time t into the stored velocity arrays.
int fill_deformation(lsgb_solver* s, double t, double T) {
    return fill_deformation_into(s, t, T, s->u, s->v, s->w, s->st, s->batch_live);
}

// Live vortex evaluated inside the FP32 3D stage kernel (no u, v, w traffic).
// (Not inside a batch: its launches refill the arrays from the device table.)
bool live_fused(const lsgb_solver* s) {
    return s->vel_live && !s->batch_live.tab && s->prec == LSGB_PREC_F32 && stage3d_f32_fuses_deformation(s->g);
}

// Velocity operands of a stage launch: the stored arrays, or the fused vortex.
void velocity_args(const lsgb_solver* s, StageArgs& a) {
    a.u = s->u; a.v = s->v; a.w = s->w;
    if (live_fused(s)) {
        a.defo = s->defo_f32;
        a.tf = defo_time_factor(s->vel_t, s->vel_T);
    }
}

// Bring the stored arrays up to date before a call that reads them.
int materialize_velocity(lsgb_solver* s) {
    return s->vel_live ? fill_deformation(s, s->vel_t, s->vel_T) : LSGB_OK;
}

// One TVD-RK3 step: G -> A (stage 1), A -> B (stage 2), (G, B) -> G (stage 3).
// Stage 3 writes in place: G^n enters only point-wise, read by the thread that
// writes the same cell, so every cell's G^n is read before it is replaced.
// The buffers keep their roles, which makes captured step sequences
// replayable.
int rk3_step(lsgb_solver* s) {
    if (s->vel_live && !live_fused(s)) LSGB_TRY(fill_deformation(s, s->vel_t, s->vel_T));
    StageArgs a = stage_args(s->p, s->g, s->lay);
    velocity_args(s, a);
    a.sl = s->sl;
    a.err = err_flag(s);
    a.tile = s->tile;
    a.drop_copies = s->drop_copies;
    a.Gn = s->G;
    a.Gin = s->G; a.Gout = s->A; a.stage = 1;
    LSGB_TRY(launch_stage(s, a));
    a.Gin = s->A; a.Gout = s->B; a.stage = 2;
    LSGB_TRY(launch_stage(s, a));
    a.Gin = s->B; a.Gout = s->G; a.stage = 3;
    LSGB_TRY(launch_stage(s, a));
    return LSGB_OK;
}

// HCR-2 with phi0 = the current G buffer (left untouched until the end),
// pseudo-steps ping-ponging through A and B; r~ and flags are recomputed from phi0 inside
// each pseudo-step (same operations as the stored form).
int reinit(lsgb_solver* s) {
    if (s->p.reinit_iterations <= 0) return LSGB_OK;
    ReinitArgs r;
    r.g = s->g;
    r.lay = s->lay;
    r.phi0 = s->G;
    r.dx = s->p.dx;
    r.dy = s->p.dy;
    r.dz = s->p.dim == 3 ? s->p.dz : s->p.dx;
    r.dtau = s->p.reinit_dtau;
    r.beta = s->p.reinit_beta;
    const int M = s->p.reinit_iterations;
    if (s->prec == LSGB_PREC_F32 && M % 2 == 0) {
        // Even pseudo-step counts end in G without a copy: the first step
        // (phi = phi0 = G) writes A and keeps phi0 in B, so G is free; the
        // others alternate A -> G, G -> A and read phi0 from B.  The values
        // are those of the copy form below.
        for (int it = 0; it < M; ++it) {
            r.phin = it == 0 ? s->G : (it % 2 ? s->A : s->G);
            r.phi0 = it == 0 ? s->G : s->B;
            r.phinew = it % 2 ? s->G : s->A;
            r.phi0_copy = it == 0 ? s->B : nullptr;
            size_t ev = 0;
            LSGB_TRY(timed_begin(s, 1, &ev));
            LSGB_CUDA(launch_reinit_f32(r, s->st));
            LSGB_TRY(timed_end(s, ev));
        }
        return LSGB_OK;
    }
    void* cur = s->G;
    void* bufs[2] = {s->A, s->B};
    for (int it = 0; it < s->p.reinit_iterations; ++it) {
        r.phin = cur;
        r.phinew = bufs[it & 1];
        size_t ev = 0;
        LSGB_TRY(timed_begin(s, 1, &ev));
        if (s->prec == LSGB_PREC_F64) LSGB_CUDA(launch_reinit_f64(r, s->st));
        else LSGB_CUDA(launch_reinit_f32(r, s->st));
        LSGB_TRY(timed_end(s, ev));
        cur = bufs[it & 1];
    }
    // the result goes back into G (one copy per reinitialisation, so the
    // buffers keep their roles)
    LSGB_CUDA(cudaMemcpyAsync(s->G, cur, nbytes(s), cudaMemcpyDeviceToDevice, s->st));
    return LSGB_OK;
}

// Reads the two result slots and the in-kernel error flag (synchronises).
int reduce_read(lsgb_solver* s, double* r2) {
    LSGB_CUDA(cudaMemcpyAsync(s->h_res, s->scratch + 2 * (RED_BLOCKS + 1), 3 * sizeof(double),
                              cudaMemcpyDeviceToHost, s->st));
    LSGB_CUDA(cudaStreamSynchronize(s->st));
    r2[0] = s->h_res[0];
    r2[1] = s->h_res[1];
    return flag_result(s, ((const int*)(s->h_res + 2))[0]);
}

// The flag alone (after a synchronising call that did not read it).
int check_flag(lsgb_solver* s) {
    LSGB_CUDA(cudaMemcpyAsync(s->h_res + 2, err_flag(s), sizeof(int), cudaMemcpyDeviceToHost, s->st));
    LSGB_CUDA(cudaStreamSynchronize(s->st));
    return flag_result(s, ((const int*)(s->h_res + 2))[0]);
}

double* red_out(lsgb_solver* s) { return s->scratch + 2 * (RED_BLOCKS + 1); }

int solver_ok(const lsgb_solver* s) {
    if (!s) return fail(LSGB_ERR_INVALID, "solver is NULL");
    if (s->unusable)
        return fail(LSGB_ERR_CUDA, "handle unusable after an in-kernel wait gave up with copies in flight; "
                                   "destroy it");
    return LSGB_OK;
}

}  // namespace

extern "C" int lsgb_solver_create(const lsgb_params* p, int precision, lsgb_solver** out) {
    LSGB_TRY(check_params(p));
    if (!out) return fail(LSGB_ERR_INVALID, "out is NULL");
    if (precision != LSGB_PREC_F64 && precision != LSGB_PREC_F32)
        return fail(LSGB_ERR_INVALID, "unknown precision %d", precision);
    lsgb_solver* s = new lsgb_solver();
    s->p = *p;
    if (s->p.dim == 2) { s->p.nz = 1; s->p.dz = s->p.dx; s->p.bc_z = LSGB_BC_PERIODIC; }
    s->g = geo_of(s->p);
    s->lay = compact_layout(s->g);
    s->prec = precision;
    s->esz = precision == LSGB_PREC_F64 ? sizeof(double) : sizeof(float);
    int rc = LSGB_OK;
    cudaError_t e = cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete s; return fail(LSGB_ERR_CUDA, "stream creation: %s", cudaGetErrorString(e)); }
    s->own_stream = true;
    void** fields[6] = {&s->G, &s->A, &s->B, &s->u, &s->v, &s->w};
    for (int q = 0; q < (s->p.dim == 3 ? 6 : 5) && rc == LSGB_OK; ++q) rc = alloc_field(s, fields[q]);
    if (rc == LSGB_OK) {
        e = cudaMalloc((void**)&s->scratch, reduce_scratch_bytes() + 4 * sizeof(double));
        if (e != cudaSuccess) rc = fail(LSGB_ERR_ALLOC, "scratch: %s", cudaGetErrorString(e));
        else if ((e = cudaMemset(s->scratch, 0, reduce_scratch_bytes() + 4 * sizeof(double))) != cudaSuccess)
            rc = fail(LSGB_ERR_CUDA, "scratch: %s", cudaGetErrorString(e));
    }
    if (rc == LSGB_OK) {
        e = cudaMallocHost((void**)&s->h_res, 4 * sizeof(double));
        if (e != cudaSuccess) rc = fail(LSGB_ERR_ALLOC, "pinned result slots: %s", cudaGetErrorString(e));
    }
    if (rc != LSGB_OK) {
        std::string keep = g_err;
        lsgb_solver_destroy(s);
        g_err = keep;
        return rc;
    }
    *out = s;
    return LSGB_OK;
}

void snapshots_close(lsgb_solver* s);

extern "C" int lsgb_solver_destroy(lsgb_solver* s) {
    if (!s) return LSGB_OK;
    if (s->st) cudaStreamSynchronize(s->st);
    snapshots_close(s);
    void* ptrs[10] = {s->G, s->A, s->B, s->u, s->v, s->w, s->sl, s->stage64, s->scratch, s->defo_f32};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    if (s->h_res) cudaFreeHost(s->h_res);
    for (cudaEvent_t e : s->ev_pool) cudaEventDestroy(e);
    if (s->own_stream && s->st) cudaStreamDestroy(s->st);
    delete s;
    return LSGB_OK;
}

extern "C" int lsgb_solver_set_stream(lsgb_solver* s, void* stream) {
    LSGB_TRY(solver_ok(s));
    LSGB_CUDA(cudaStreamSynchronize(s->st));
    if (s->own_stream) cudaStreamDestroy(s->st);
    if (stream) {
        s->st = (cudaStream_t)stream;
        s->own_stream = false;
    } else {
        LSGB_CUDA(cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking));
        s->own_stream = true;
    }
    return LSGB_OK;
}

extern "C" int lsgb_solver_get_params(const lsgb_solver* s, lsgb_params* p) {
    LSGB_TRY(solver_ok(s));
    if (!p) return fail(LSGB_ERR_INVALID, "p is NULL");
    *p = s->p;
    return LSGB_OK;
}

extern "C" int lsgb_solver_set_dt(lsgb_solver* s, double dt) {
    LSGB_TRY(solver_ok(s));
    if (!std::isfinite(dt) || dt < 0.0) return fail(LSGB_ERR_INVALID, "dt must be finite and >= 0");
    s->p.dt = dt;
    return LSGB_OK;
}

extern "C" int lsgb_solver_set_fields(lsgb_solver* s, const double* G, const double* u,
                                      const double* v, const double* w, int layout, int memory) {
    LSGB_TRY(solver_ok(s));
    if (layout != LSGB_LAYOUT_GHOSTED && layout != LSGB_LAYOUT_COMPACT)
        return fail(LSGB_ERR_INVALID, "unknown layout %d", layout);
    if (memory != LSGB_MEM_HOST && memory != LSGB_MEM_DEVICE)
        return fail(LSGB_ERR_INVALID, "unknown memory kind %d", memory);
    if (G) { LSGB_TRY(load_field(s, s->G, G, layout, memory)); s->have_G = true; }
    if (u) LSGB_TRY(load_field(s, s->u, u, layout, memory));
    if (v) LSGB_TRY(load_field(s, s->v, v, layout, memory));
    if (w && s->p.dim == 3) LSGB_TRY(load_field(s, s->w, w, layout, memory));
    if (u && v && (w || s->p.dim == 2)) s->have_vel = true;
    if (u || v || w) s->vel_live = false;
    return LSGB_OK;
}

extern "C" int lsgb_solver_set_sl_field(lsgb_solver* s, const double* sl, int layout, int memory) {
    LSGB_TRY(solver_ok(s));
    if (!sl) {
        if (s->sl) { LSGB_CUDA(cudaStreamSynchronize(s->st)); cudaFree(s->sl); s->sl = nullptr; }
        return LSGB_OK;
    }
    if (!s->sl) LSGB_TRY(alloc_field(s, &s->sl));
    return load_field(s, s->sl, sl, layout, memory);
}

extern "C" int lsgb_solver_get_G(lsgb_solver* s, double* G, int layout, int memory) {
    LSGB_TRY(solver_ok(s));
    if (!G) return fail(LSGB_ERR_INVALID, "G is NULL");
    if (!s->have_G) return fail(LSGB_ERR_STATE, "G has not been set");
    Lay dl = layout == LSGB_LAYOUT_GHOSTED ? ghosted_layout(s->g) : compact_layout(s->g);
    size_t dbytes = sizeof(double) * (size_t)layout_elems(s->g, dl.ghosted);
    double* ddst = G;
    if (memory == LSGB_MEM_HOST) {
        if (s->prec == LSGB_PREC_F64 && !dl.ghosted) {
            LSGB_CUDA(cudaMemcpyAsync(G, s->G, dbytes, cudaMemcpyDeviceToHost, s->st));
            LSGB_CUDA(cudaStreamSynchronize(s->st));
            return LSGB_OK;
        }
        LSGB_TRY(ensure_stage(s));
        ddst = s->stage64;
    } else {
        LSGB_TRY(check_dev(G, "G"));
    }
    if (s->prec == LSGB_PREC_F64) LSGB_CUDA(launch_unpack_f64(s->g, (const double*)s->G, ddst, dl, s->st));
    else LSGB_CUDA(launch_unpack_f32(s->g, (const float*)s->G, ddst, dl, s->st));
    if (memory == LSGB_MEM_HOST) {
        LSGB_CUDA(cudaMemcpyAsync(G, ddst, dbytes, cudaMemcpyDeviceToHost, s->st));
        LSGB_CUDA(cudaStreamSynchronize(s->st));
    }
    LSGB_TRY(check_flag(s));
    return LSGB_OK;
}

extern "C" int lsgb_solver_advance(lsgb_solver* s, int n_steps) {
    LSGB_TRY(solver_ok(s));
    if (n_steps < 0) return fail(LSGB_ERR_INVALID, "n_steps < 0");
    if (!s->have_G || !s->have_vel) return fail(LSGB_ERR_STATE, "fields not set");
    for (int q = 0; q < n_steps; ++q) {
        LSGB_TRY(rk3_step(s));
        if (s->p.enable_reinit && s->step > 0 && s->step % s->p.reinit_interval == 0)
            LSGB_TRY(reinit(s));
        s->step++;
        if (s->vel_live) s->vel_t += s->p.dt;  // current_time += params.dt (src/main.cpp:315)
    }
    return LSGB_OK;
}

extern "C" int lsgb_solver_get_time(const lsgb_solver* s, double* t) {
    LSGB_TRY(solver_ok(s));
    if (!t) return fail(LSGB_ERR_INVALID, "t is NULL");
    *t = s->vel_t;
    return LSGB_OK;
}

extern "C" int lsgb_solver_reinit(lsgb_solver* s) {
    LSGB_TRY(solver_ok(s));
    if (!s->have_G) return fail(LSGB_ERR_STATE, "G has not been set");
    return reinit(s);
}

extern "C" int lsgb_solver_get_step(const lsgb_solver* s, int* step) {
    LSGB_TRY(solver_ok(s));
    if (!step) return fail(LSGB_ERR_INVALID, "step is NULL");
    *step = s->step;
    return LSGB_OK;
}

extern "C" int lsgb_solver_set_step(lsgb_solver* s, int step) {
    LSGB_TRY(solver_ok(s));
    if (step < 0) return fail(LSGB_ERR_INVALID, "step < 0");
    s->step = step;
    return LSGB_OK;
}

extern "C" int lsgb_solver_volume(lsgb_solver* s, double* volume, int64_t* count) {
    LSGB_TRY(solver_ok(s));
    if (!s->have_G) return fail(LSGB_ERR_STATE, "G has not been set");
    if (s->prec == LSGB_PREC_F64)
        LSGB_CUDA(launch_count_negative<double>(s->g, s->lay, (const double*)s->G, s->scratch, red_out(s), s->st));
    else
        LSGB_CUDA(launch_count_negative<float>(s->g, s->lay, (const float*)s->G, s->scratch, red_out(s), s->st));
    double r[2];
    LSGB_TRY(reduce_read(s, r));
    if (count) *count = (int64_t)r[0];
    if (volume) *volume = r[0] * cell_volume(s->p);
    return LSGB_OK;
}

extern "C" int lsgb_solver_max_speed(lsgb_solver* s, double* max_speed) {
    LSGB_TRY(solver_ok(s));
    if (!s->have_vel) return fail(LSGB_ERR_STATE, "velocity has not been set");
    if (!max_speed) return fail(LSGB_ERR_INVALID, "max_speed is NULL");
    LSGB_TRY(materialize_velocity(s));
    if (s->prec == LSGB_PREC_F64)
        LSGB_CUDA(launch_max_speed<double>(s->g, s->lay, (const double*)s->u, (const double*)s->v,
                                           (const double*)s->w, s->scratch, red_out(s), s->st));
    else
        LSGB_CUDA(launch_max_speed<float>(s->g, s->lay, (const float*)s->u, (const float*)s->v,
                                          (const float*)s->w, s->scratch, red_out(s), s->st));
    double r[2];
    LSGB_TRY(reduce_read(s, r));
    *max_speed = r[0];
    return LSGB_OK;
}

extern "C" int lsgb_solver_compute_dt(lsgb_solver* s, double cfl, double* dt) {
    double ms;
    LSGB_TRY(lsgb_solver_max_speed(s, &ms));
    lsgb_params p = s->p;
    p.cfl = cfl;
    double d;
    LSGB_TRY(lsgb_cfl_dt(&p, ms, &d));
    s->p.cfl = cfl;
    s->p.dt = d;
    if (dt) *dt = d;
    return LSGB_OK;
}

extern "C" int lsgb_solver_l2_error(lsgb_solver* s, const double* G_ref, int layout, int memory,
                                    double* l2) {
    LSGB_TRY(solver_ok(s));
    if (!G_ref || !l2) return fail(LSGB_ERR_INVALID, "G_ref / l2 is NULL");
    if (!s->have_G) return fail(LSGB_ERR_STATE, "G has not been set");
    Lay rl = layout == LSGB_LAYOUT_GHOSTED ? ghosted_layout(s->g) : compact_layout(s->g);
    const double* ref = G_ref;
    if (memory == LSGB_MEM_HOST) {
        LSGB_TRY(ensure_stage(s));
        LSGB_CUDA(cudaMemcpyAsync(s->stage64, G_ref, sizeof(double) * (size_t)layout_elems(s->g, rl.ghosted),
                                  cudaMemcpyHostToDevice, s->st));
        ref = s->stage64;
    } else {
        LSGB_TRY(check_dev(G_ref, "G_ref"));
    }
    if (s->prec == LSGB_PREC_F64)
        LSGB_CUDA(launch_sq_diff<double>(s->g, s->lay, (const double*)s->G, ref, rl, s->scratch, red_out(s), s->st));
    else
        LSGB_CUDA(launch_sq_diff<float>(s->g, s->lay, (const float*)s->G, ref, rl, s->scratch, red_out(s), s->st));
    double r[2];
    LSGB_TRY(reduce_read(s, r));
    *l2 = std::sqrt(r[0] / (double)s->g.cells());
    return LSGB_OK;
}

extern "C" int lsgb_solver_run_host(lsgb_solver* s, const double* G, const double* u,
                                    const double* v, const double* w, int n_steps, double* G_out,
                                    int layout) {
    LSGB_TRY(solver_ok(s));
    if (!G || !G_out) return fail(LSGB_ERR_INVALID, "G / G_out is NULL");
    LSGB_TRY(lsgb_solver_set_fields(s, G, u, v, w, layout, LSGB_MEM_HOST));
    LSGB_TRY(lsgb_solver_advance(s, n_steps));
    LSGB_TRY(lsgb_solver_get_G(s, G_out, layout, LSGB_MEM_HOST));
    return LSGB_OK;
}

extern "C" int lsgb_solver_synth(lsgb_solver* s, const lsgb_synth* d) {
    LSGB_TRY(solver_ok(s));
    if (!d) return fail(LSGB_ERR_INVALID, "descriptor is NULL");
    if (d->n_shape_modes < 0 || d->n_shape_modes > LSGB_MAX_MODES || d->n_vel_modes < 0 ||
        d->n_vel_modes > LSGB_MAX_MODES)
        return fail(LSGB_ERR_INVALID, "mode counts must lie in [0, %d]", LSGB_MAX_MODES);
    for (int m = 0; m < d->n_shape_modes; ++m)
        if (d->shape_l[m] < 0 || d->shape_l[m] > 4 || d->shape_m[m] > d->shape_l[m] || -d->shape_m[m] > d->shape_l[m])
            return fail(LSGB_ERR_INVALID, "shape mode %d: need 0 <= |m| <= l <= 4", m);
    const long long n = s->g.cells();
    double* tmp[4] = {nullptr, nullptr, nullptr, nullptr};
    const bool direct = s->prec == LSGB_PREC_F64;
    if (direct) {
        tmp[0] = (double*)s->G; tmp[1] = (double*)s->u; tmp[2] = (double*)s->v;
        tmp[3] = s->p.dim == 3 ? (double*)s->w : nullptr;
    } else {
        for (int q = 0; q < (s->p.dim == 3 ? 4 : 3); ++q) {
            cudaError_t e = cudaMallocAsync((void**)&tmp[q], sizeof(double) * (size_t)n, s->st);
            if (e != cudaSuccess) {
                for (int r = 0; r < q; ++r) cudaFreeAsync(tmp[r], s->st);
                return fail(LSGB_ERR_ALLOC, "synth temporaries: %s", cudaGetErrorString(e));
            }
        }
    }
    int rc = LSGB_OK;
    Lay cl = compact_layout(s->g);
    double dz = s->p.dim == 3 ? s->p.dz : s->p.dx;
    cudaError_t e = launch_synth(s->g, *d, s->p.dx, s->p.dy, dz, tmp[0], tmp[1], tmp[2], tmp[3], s->st);
    if (e != cudaSuccess) rc = fail(LSGB_ERR_CUDA, "synth kernel: %s", cudaGetErrorString(e));
    if (rc == LSGB_OK && d->vel_scale <= 0.0) {
        // normalise to max |u|_2 = 1
        e = launch_max_speed<double>(s->g, cl, tmp[1], tmp[2], tmp[3], s->scratch, red_out(s), s->st);
        double r[2] = {0, 0};
        if (e == cudaSuccess) rc = reduce_read(s, r);
        else rc = fail(LSGB_ERR_CUDA, "synth normalisation: %s", cudaGetErrorString(e));
        if (rc == LSGB_OK && r[1] > 0.0) {
            e = launch_scale3(n, 1.0 / r[1], tmp[1], tmp[2], tmp[3], s->st);
            if (e != cudaSuccess) rc = fail(LSGB_ERR_CUDA, "synth scale: %s", cudaGetErrorString(e));
        }
    }
    if (!direct) {
        void* dst[4] = {s->G, s->u, s->v, s->w};
        for (int q = 0; q < (s->p.dim == 3 ? 4 : 3) && rc == LSGB_OK; ++q) {
            e = launch_pack_f32(s->g, tmp[q], cl, (float*)dst[q], s->st);
            if (e != cudaSuccess) rc = fail(LSGB_ERR_CUDA, "synth convert: %s", cudaGetErrorString(e));
        }
        for (int q = 0; q < 4; ++q)
            if (tmp[q]) cudaFreeAsync(tmp[q], s->st);
    }
    if (rc == LSGB_OK) { s->have_G = true; s->have_vel = true; s->vel_live = false; }
    return rc;
}

extern "C" int lsgb_solver_set_velocity_deformation(lsgb_solver* s, double t, double T) {
    LSGB_TRY(solver_ok(s));
    if (s->p.dim != 3) return fail(LSGB_ERR_INVALID, "the deformation vortex is a 3D field");
    if (!std::isfinite(t) || !std::isfinite(T) || T == 0.0) return fail(LSGB_ERR_INVALID, "bad t / T");
    LSGB_TRY(fill_deformation(s, t, T));
    s->vel_live = false;
    s->have_vel = true;
    return LSGB_OK;
}

extern "C" int lsgb_solver_set_velocity_deformation_live(lsgb_solver* s, double t, double T) {
    LSGB_TRY(solver_ok(s));
    if (s->p.dim != 3) return fail(LSGB_ERR_INVALID, "the deformation vortex is a 3D field");
    if (!std::isfinite(t) || !std::isfinite(T) || T == 0.0) return fail(LSGB_ERR_INVALID, "bad t / T");
    if (s->prec == LSGB_PREC_F32) LSGB_TRY(ensure_defo_tables(s));
    s->vel_live = true;
    s->vel_t = t;
    s->vel_T = T;
    s->have_vel = true;
    return LSGB_OK;
}

extern "C" int lsgb_solver_get_field(lsgb_solver* s, int which, double* out, int layout, int memory) {
    LSGB_TRY(solver_ok(s));
    if (which == LSGB_FIELD_G) return lsgb_solver_get_G(s, out, layout, memory);
    void* f = which == LSGB_FIELD_U ? s->u : which == LSGB_FIELD_V ? s->v
            : which == LSGB_FIELD_W ? (s->p.dim == 3 ? s->w : nullptr)
            : which == LSGB_FIELD_SL ? s->sl : nullptr;
    if (!f) return fail(LSGB_ERR_INVALID, "field %d is not resident", which);
    if (!out) return fail(LSGB_ERR_INVALID, "out is NULL");
    if (which == LSGB_FIELD_U || which == LSGB_FIELD_V || which == LSGB_FIELD_W) LSGB_TRY(materialize_velocity(s));
    void* keep = s->G;
    bool had = s->have_G;
    s->G = f;
    s->have_G = true;
    int rc = lsgb_solver_get_G(s, out, layout, memory);
    s->G = keep;
    s->have_G = had;
    return rc;
}

extern "C" int lsgb_solver_enable_timing(lsgb_solver* s, int enable) {
    LSGB_TRY(solver_ok(s));
    LSGB_CUDA(cudaStreamSynchronize(s->st));
    s->timing = enable != 0;
    s->ev_used = 0;
    s->ev_marks.clear();
    return LSGB_OK;
}

extern "C" int lsgb_solver_kernel_times(lsgb_solver* s, double* stage_ms, int64_t* stage_launches,
                                        double* reinit_ms, int64_t* reinit_launches) {
    LSGB_TRY(solver_ok(s));
    LSGB_CUDA(cudaStreamSynchronize(s->st));
    double t[2] = {0.0, 0.0};
    int64_t c[2] = {0, 0};
    for (const auto& m : s->ev_marks) {
        float ms = 0.0f;
        LSGB_CUDA(cudaEventElapsedTime(&ms, s->ev_pool[m.first], s->ev_pool[m.first + 1]));
        t[m.second] += ms;
        c[m.second] += 1;
    }
    if (stage_ms) *stage_ms = t[0];
    if (stage_launches) *stage_launches = c[0];
    if (reinit_ms) *reinit_ms = t[1];
    if (reinit_launches) *reinit_launches = c[1];
    return LSGB_OK;
}

// ---------------------------------------------------------------------------
// tile shapes and the autotuner
// ---------------------------------------------------------------------------
namespace {

// Tile shapes the FP32 kernels accept: the z-chunk length of the 3D tiles.
// The 2D FP32 kernel (32 x 32 tiles) and the FP64 kernels have one shape.
// Tile choices of the stage kernels: FP32 3D z-chunk (16, 32, 64 planes),
// FP32 2D tile height (32: 32 x 32 tiles, 16: 32 x 16), FP64 kernel form
// (1: one thread per cell, 2: face-shared tiles).
int tile_candidates(const lsgb_solver* s, int* c) {
    if (s->prec != LSGB_PREC_F32) { c[0] = 1; c[1] = 2; return 2; }
    if (s->p.dim == 2) { c[0] = 32; c[1] = 16; return 2; }
    c[0] = 16; c[1] = 32; c[2] = 64; return 3;
}

}  // namespace

extern "C" int lsgb_solver_set_tile(lsgb_solver* s, int tile) {
    LSGB_TRY(solver_ok(s));
    int c[4], n = tile_candidates(s, c);
    bool ok = tile == 0;
    for (int i = 0; i < n; ++i) ok = ok || tile == c[i];
    if (!ok) return fail(LSGB_ERR_INVALID, "tile %d is not a shape of this solver", tile);
    s->tile = tile;
    return LSGB_OK;
}

extern "C" int lsgb_solver_get_tile(const lsgb_solver* s, int* tile) {
    LSGB_TRY(solver_ok(s));
    if (!tile) return fail(LSGB_ERR_INVALID, "tile is NULL");
    *tile = s->tile;
    return LSGB_OK;
}

extern "C" int lsgb_debug_f64_div_check(long long n, unsigned long long seed, long long* mismatches) {
    if (n < 0 || !mismatches) return fail(LSGB_ERR_INVALID, "n < 0 or mismatches is NULL");
    unsigned long long* d = nullptr;
    LSGB_CUDA(cudaMalloc((void**)&d, sizeof(unsigned long long)));
    cudaError_t e = cudaMemset(d, 0, sizeof(unsigned long long));
    if (e == cudaSuccess) e = launch_div_check(n, seed, d, nullptr);
    unsigned long long h = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return fail(LSGB_ERR_CUDA, "division check: %s", cudaGetErrorString(e));
    *mismatches = (long long)h;
    return LSGB_OK;
}

extern "C" int lsgb_solver_debug_drop_copies(lsgb_solver* s, int on) {
    LSGB_TRY(solver_ok(s));
    s->drop_copies = on ? 1 : 0;
    return LSGB_OK;
}

// Times one RK3 stage-1 launch (G -> A, the state is not touched) for every
// candidate shape with CUDA events on the handle's stream and keeps the
// fastest.  Needs G and the velocity set.
extern "C" int lsgb_solver_autotune(lsgb_solver* s, int reps, int* best_tile, float* best_ms) {
    LSGB_TRY(solver_ok(s));
    if (!s->have_G || !s->have_vel) return fail(LSGB_ERR_STATE, "fields not set");
    int c[4], n = tile_candidates(s, c);
    if (n == 0) {
        if (best_tile) *best_tile = 0;
        if (best_ms) *best_ms = 0.0f;
        return LSGB_OK;
    }
    if (reps < 1) reps = 3;
    cudaEvent_t e0, e1;
    LSGB_CUDA(cudaEventCreate(&e0));
    LSGB_CUDA(cudaEventCreate(&e1));
    int best = c[0];
    float tbest = 1e30f;
    int rc = LSGB_OK;
    for (int i = 0; i < n && rc == LSGB_OK; ++i) {
        StageArgs a = stage_args(s->p, s->g, s->lay);
        velocity_args(s, a);
        a.sl = s->sl;
        a.err = err_flag(s);
        a.tile = c[i];
        a.Gn = s->G; a.Gin = s->G; a.Gout = s->A; a.stage = 1;
        rc = launch_stage(s, a);  // warm-up
        if (rc != LSGB_OK) break;
        cudaEventRecord(e0, s->st);
        for (int r = 0; r < reps && rc == LSGB_OK; ++r) rc = launch_stage(s, a);
        cudaEventRecord(e1, s->st);
        if (cudaEventSynchronize(e1) != cudaSuccess) { rc = fail(LSGB_ERR_CUDA, "autotune timing failed"); break; }
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        ms /= reps;
        if (ms < tbest) { tbest = ms; best = c[i]; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    LSGB_TRY(rc);
    LSGB_TRY(check_flag(s));
    s->tile = best;
    if (best_tile) *best_tile = best;
    if (best_ms) *best_ms = tbest;
    return LSGB_OK;
}

// ---------------------------------------------------------------------------
// batches: many independent instances advanced together in CUDA graphs
// ---------------------------------------------------------------------------
struct lsgb_batch {
    int prec;
    std::vector<lsgb_solver*> inst;
    cudaStream_t main = nullptr;
    std::vector<cudaStream_t> lanes;
    std::vector<cudaEvent_t> lane_done;
    cudaEvent_t fork = nullptr, done = nullptr;
    cudaGraphExec_t block = nullptr;  // one reinit period of steps for every instance
    int block_len = 0;
    int64_t graph_launches = 0, graph_kernels = 0;
    // grouped form (FP32): one launch per stage / pseudo-step / copy for all
    // instances of one dimensionality, driven by descriptor tables
    int mode = LSGB_BATCH_GROUPED;
    bool grouped = false;             // the captured graph uses the grouped launches
    int shape2 = 32;                  // 2D tile height of the grouped launches
    std::vector<int> i3, i2;          // instance indices by dimensionality
    std::vector<char> h_tab;
    void* d_tab = nullptr;
    size_t d_tab_bytes = 0;
    // table layout: descriptors (3D stage, 2D stage, 3D / 2D HCR-2), then the
    // owner tables (block / tile -> instance) of each launch kind
    size_t off3 = 0, off2 = 0, offr3 = 0, offr2 = 0;
    size_t oo3 = 0, oo2 = 0, oor3 = 0, oor2 = 0, ooc3 = 0, ooc2 = 0;
    long long blk3 = 0, tiles2 = 0, rblk3 = 0, rblk2 = 0, cblk3 = 0, cblk2 = 0;
    int iters = 0;                    // HCR-2 pseudo-steps (uniform over the batch)
    std::vector<long long> sig;       // launch shapes the captured graph was made with
    // live deformation velocity: per live instance a slot of live_cap entries
    // (FP64 time or FP32 time factor of each step of one advance call), and
    // the device cursor the launches index it from
    std::vector<int> live;            // instance indices with live velocity
    std::vector<long long> live_sig;  // live set + table the captured graph was made with
    char* live_tab = nullptr;
    int* live_base = nullptr;
    size_t live_cap = 0;
    char* live_h = nullptr;           // pinned staging of the table
    size_t live_h_bytes = 0;
    cudaEvent_t live_copied = nullptr;  // the last upload from live_h
};

namespace {

int batch_ok(const lsgb_batch* b) {
    if (!b) return fail(LSGB_ERR_INVALID, "batch is NULL");
    return LSGB_OK;
}

void batch_drop_graph(lsgb_batch* b) {
    if (b->block) cudaGraphExecDestroy(b->block);
    b->block = nullptr;
    b->block_len = 0;
}

// Instances share one step counter and one reinit cadence, which lets the
// batch replay a captured period.
int batch_uniform(const lsgb_batch* b, int* step, int* interval, int* reinit) {
    const lsgb_solver* f = b->inst[0];
    for (const lsgb_solver* s : b->inst)
        if (s->step != f->step || s->p.enable_reinit != f->p.enable_reinit ||
            (f->p.enable_reinit && s->p.reinit_interval != f->p.reinit_interval))
            return fail(LSGB_ERR_STATE, "batched instances need the same step counter and reinit cadence");
    *step = f->step;
    *interval = f->p.enable_reinit ? f->p.reinit_interval : 1;
    *reinit = f->p.enable_reinit;
    return LSGB_OK;
}

// Launches n steps for every instance on the lanes (each instance keeps its
// lane), with the reinit cadence of the reference main loop.
int batch_launch_steps(lsgb_batch* b, int n_steps) {
    LSGB_CUDA(cudaEventRecord(b->fork, b->main));
    for (cudaStream_t l : b->lanes) LSGB_CUDA(cudaStreamWaitEvent(l, b->fork, 0));
    for (int q = 0; q < n_steps; ++q) {
        for (size_t i = 0; i < b->inst.size(); ++i) {
            lsgb_solver* s = b->inst[i];
            cudaStream_t own = s->st;
            s->st = b->lanes[i % b->lanes.size()];
            s->batch_live.q = q;
            int rc = rk3_step(s);
            if (rc == LSGB_OK && s->p.enable_reinit && s->step > 0 && s->step % s->p.reinit_interval == 0)
                rc = reinit(s);
            s->st = own;
            LSGB_TRY(rc);
            s->step++;
        }
    }
    for (size_t l = 0; l < b->lanes.size(); ++l) {
        LSGB_CUDA(cudaEventRecord(b->lane_done[l], b->lanes[l]));
        LSGB_CUDA(cudaStreamWaitEvent(b->main, b->lane_done[l], 0));
    }
    if (!b->live.empty()) LSGB_CUDA(launch_live_advance(b->live_base, n_steps, b->main));
    return LSGB_OK;
}

// The grouped form applies when every instance is FP32 with fewer than 2^31
// cells and all share the HCR-2 pseudo-step count.
bool batch_grouped_ok(const lsgb_batch* b) {
    if (b->mode != LSGB_BATCH_GROUPED || b->prec != LSGB_PREC_F32 || b->inst.empty()) return false;
    for (const lsgb_solver* s : b->inst) {
        if (s->g.cells() >= (1LL << 31) - 1) return false;
        if (s->p.enable_reinit && s->p.reinit_iterations != b->inst[0]->p.reinit_iterations) return false;
    }
    return true;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Fill and upload the descriptor tables from the instances' current
// parameters (dt, S_L, tiles).  Ordered on the batch stream before the
// launches that read it.  3D instances go longest blocks first (the block
// scheduler starts blocks roughly in index order, so the short blocks of
// small instances fill the tail of the launch).
int batch_tables(lsgb_batch* b) {
    b->i3.clear();
    b->i2.clear();
    for (size_t i = 0; i < b->inst.size(); ++i) (b->inst[i]->p.dim == 3 ? b->i3 : b->i2).push_back((int)i);
    auto gi = [&](int i) {
        lsgb_solver* s = b->inst[i];
        GroupInst e;
        e.a = stage_args(s->p, s->g, s->lay);
        velocity_args(s, e.a);
        e.a.sl = s->sl;
        e.a.err = err_flag(s);
        e.a.tile = s->tile;
        e.G = (float*)s->G;
        e.A = (float*)s->A;
        e.B = (float*)s->B;
        e.dtau = s->p.reinit_dtau;
        e.beta = s->p.reinit_beta;
        return e;
    };
    std::vector<GroupInst> g3, g2;
    for (int i : b->i3) g3.push_back(gi(i));
    for (int i : b->i2) g2.push_back(gi(i));
    {
        std::vector<size_t> ord(g3.size());
        for (size_t q = 0; q < ord.size(); ++q) ord[q] = q;
        std::stable_sort(ord.begin(), ord.end(), [&](size_t x, size_t y) {
            const int px = stage3d_chunk_planes(g3[x].a), py = stage3d_chunk_planes(g3[y].a);
            return px != py ? px > py : g3[x].a.g.cells() > g3[y].a.g.cells();
        });
        std::vector<GroupInst> g(g3.size());
        std::vector<int> ix(g3.size());
        for (size_t q = 0; q < ord.size(); ++q) { g[q] = g3[ord[q]]; ix[q] = b->i3[ord[q]]; }
        g3.swap(g);
        b->i3.swap(ix);
    }
    const int n3 = (int)g3.size(), n2 = (int)g2.size();
    std::vector<char> d3(group3_desc_bytes() * n3 + 64), d2(group2_desc_bytes() * n2 + 64);
    std::vector<char> r3(groupr_desc_bytes() * n3 + 64), r2(groupr_desc_bytes() * n2 + 64);
    auto al64 = [](std::vector<char>& v) { return v.data() + ((64 - ((uintptr_t)v.data() & 63)) & 63); };
    std::vector<int> o3, o2, or3, or2, oc3, oc2;
    if (n3) group3_fill(g3.data(), n3, al64(d3), o3);
    if (n2) group2_fill(g2.data(), n2, b->shape2, al64(d2), o2);
    if (n3) groupr_fill(g3.data(), n3, al64(r3), or3, oc3);
    if (n2) groupr_fill(g2.data(), n2, al64(r2), or2, oc2);
    b->blk3 = (long long)o3.size();
    b->tiles2 = (long long)o2.size();
    b->rblk3 = (long long)or3.size();
    b->rblk2 = (long long)or2.size();
    b->cblk3 = (long long)oc3.size();
    b->cblk2 = (long long)oc2.size();
    for (long long x : {b->blk3, b->tiles2, b->rblk3, b->rblk2, b->cblk3, b->cblk2})
        if (x > 0x7fffffffLL) return fail(LSGB_ERR_UNSUPPORTED, "batch too large for one grouped launch");
    b->iters = b->inst[0]->p.enable_reinit ? b->inst[0]->p.reinit_iterations : 0;
    size_t off = 0;
    auto place = [&](size_t bytes) { const size_t o = off; off = align256(off + bytes); return o; };
    b->off3 = place(group3_desc_bytes() * n3);
    b->off2 = place(group2_desc_bytes() * n2);
    b->offr3 = place(groupr_desc_bytes() * n3);
    b->offr2 = place(groupr_desc_bytes() * n2);
    b->oo3 = place(sizeof(int) * o3.size());
    b->oo2 = place(sizeof(int) * o2.size());
    b->oor3 = place(sizeof(int) * or3.size());
    b->oor2 = place(sizeof(int) * or2.size());
    b->ooc3 = place(sizeof(int) * oc3.size());
    b->ooc2 = place(sizeof(int) * oc2.size());
    const size_t total = off;
    b->h_tab.assign(total + 64, 0);  // the descriptors hold 64-byte aligned tensor maps
    char* h = al64(b->h_tab);
    std::memcpy(h + b->off3, al64(d3), group3_desc_bytes() * n3);
    std::memcpy(h + b->off2, al64(d2), group2_desc_bytes() * n2);
    std::memcpy(h + b->offr3, al64(r3), groupr_desc_bytes() * n3);
    std::memcpy(h + b->offr2, al64(r2), groupr_desc_bytes() * n2);
    std::memcpy(h + b->oo3, o3.data(), sizeof(int) * o3.size());
    std::memcpy(h + b->oo2, o2.data(), sizeof(int) * o2.size());
    std::memcpy(h + b->oor3, or3.data(), sizeof(int) * or3.size());
    std::memcpy(h + b->oor2, or2.data(), sizeof(int) * or2.size());
    std::memcpy(h + b->ooc3, oc3.data(), sizeof(int) * oc3.size());
    std::memcpy(h + b->ooc2, oc2.data(), sizeof(int) * oc2.size());
    if (total > b->d_tab_bytes) {
        if (b->d_tab) cudaFree(b->d_tab);
        b->d_tab = nullptr;
        b->d_tab_bytes = 0;
        cudaError_t e = cudaMalloc(&b->d_tab, total);
        if (e != cudaSuccess) return fail(LSGB_ERR_ALLOC, "batch tables: %s", cudaGetErrorString(e));
        b->d_tab_bytes = total;
    }
    LSGB_CUDA(cudaMemcpyAsync(b->d_tab, h, total, cudaMemcpyHostToDevice, b->main));
    return LSGB_OK;
}

// Steps of the grouped form, with the reference main loop's reinit cadence
// (the instances share the step counter).  The 3D and the 2D instances form
// two independent chains of launches; they run on two of the batch's streams
// (forked from and joined back into the batch stream), so the 2D launches
// fill the GPU beside the 3D ones.
int batch_launch_steps_grouped(lsgb_batch* b, int n_steps) {
    const char* d = (const char*)b->d_tab;
    const int n3 = (int)b->i3.size(), n2 = (int)b->i2.size();
    cudaStream_t s3 = b->lanes[0], s2 = b->lanes.size() > 1 ? b->lanes[1] : b->lanes[0];
    LSGB_CUDA(cudaEventRecord(b->fork, b->main));
    LSGB_CUDA(cudaStreamWaitEvent(s3, b->fork, 0));
    if (s2 != s3) LSGB_CUDA(cudaStreamWaitEvent(s2, b->fork, 0));
    const int* o3 = (const int*)(d + b->oo3);
    const int* o2 = (const int*)(d + b->oo2);
    for (int q = 0; q < n_steps; ++q) {
        for (int i : b->live) {  // live instances (3D): the vortex of this step into u, v, w
            lsgb_solver* s = b->inst[i];
            s->batch_live.q = q;
            LSGB_TRY(fill_deformation_into(s, s->vel_t, s->vel_T, s->u, s->v, s->w, s3, s->batch_live));
        }
        for (int stage = 1; stage <= 3; ++stage) {
            LSGB_CUDA(launch_stage3d_f32_group(d + b->off3, o3, n3, b->blk3, stage, s3));
            LSGB_CUDA(launch_stage2d_f32_group(d + b->off2, o2, n2, b->tiles2, stage, b->shape2, s2));
        }
        const lsgb_solver* f = b->inst[0];
        if (f->p.enable_reinit && f->step > 0 && f->step % f->p.reinit_interval == 0 && b->iters > 0) {
            for (int it = 0; it < b->iters; ++it) {
                LSGB_CUDA(launch_reinit_f32_group(d + b->offr3, (const int*)(d + b->oor3), n3, b->rblk3, 3, it,
                                                  b->iters, s3));
                LSGB_CUDA(launch_reinit_f32_group(d + b->offr2, (const int*)(d + b->oor2), n2, b->rblk2, 2, it,
                                                  b->iters, s2));
            }
            LSGB_CUDA(launch_copy_back_group(d + b->offr3, (const int*)(d + b->ooc3), n3, b->cblk3, b->iters, s3));
            LSGB_CUDA(launch_copy_back_group(d + b->offr2, (const int*)(d + b->ooc2), n2, b->cblk2, b->iters, s2));
        }
        for (lsgb_solver* s : b->inst) s->step++;
    }
    LSGB_CUDA(cudaEventRecord(b->lane_done[0], s3));
    LSGB_CUDA(cudaStreamWaitEvent(b->main, b->lane_done[0], 0));
    if (s2 != s3) {
        LSGB_CUDA(cudaEventRecord(b->lane_done[1], s2));
        LSGB_CUDA(cudaStreamWaitEvent(b->main, b->lane_done[1], 0));
    }
    if (!b->live.empty()) LSGB_CUDA(launch_live_advance(b->live_base, n_steps, b->main));
    return LSGB_OK;
}

// Live instances of an advance call of n_steps: their per-step vortex times
// (FP64) or time factors (FP32), accumulated as lsgb_solver_advance does
// (t += dt after every step) and evaluated with the same host function, go
// into the device table; the launches read entry *live_base + q.  A grown
// table drops the captured graph (its launches hold the table's address).
int batch_live_begin(lsgb_batch* b, int n_steps) {
    b->live.clear();
    for (size_t i = 0; i < b->inst.size(); ++i)
        if (b->inst[i]->vel_live) b->live.push_back((int)i);
    if (b->live.empty()) {
        if (!b->live_sig.empty()) batch_drop_graph(b);
        b->live_sig.clear();
        return LSGB_OK;
    }
    const size_t esz = b->prec == LSGB_PREC_F64 ? sizeof(double) : sizeof(float);
    size_t cap = std::max<size_t>(b->live_cap, 64);
    while (cap < (size_t)n_steps) cap *= 2;
    const size_t bytes = cap * esz * b->live.size();
    if (!b->live_base) {
        cudaError_t e = cudaMalloc((void**)&b->live_base, 256);
        if (e != cudaSuccess) { b->live_base = nullptr; return fail(LSGB_ERR_ALLOC, "batch live cursor: %s", cudaGetErrorString(e)); }
    }
    if (!b->live_copied) LSGB_CUDA(cudaEventCreateWithFlags(&b->live_copied, cudaEventDisableTiming));
    LSGB_CUDA(cudaEventSynchronize(b->live_copied));  // live_h is free again
    if (cap != b->live_cap || bytes > b->live_h_bytes) {
        LSGB_CUDA(cudaStreamSynchronize(b->main));
        if (b->live_tab) cudaFree(b->live_tab);
        if (b->live_h) cudaFreeHost(b->live_h);
        b->live_tab = nullptr;
        b->live_h = nullptr;
        b->live_cap = b->live_h_bytes = 0;
        cudaError_t e = cudaMalloc((void**)&b->live_tab, bytes);
        if (e != cudaSuccess) { b->live_tab = nullptr; return fail(LSGB_ERR_ALLOC, "batch live table: %s", cudaGetErrorString(e)); }
        e = cudaMallocHost((void**)&b->live_h, bytes);
        if (e != cudaSuccess) { b->live_h = nullptr; return fail(LSGB_ERR_ALLOC, "batch live staging: %s", cudaGetErrorString(e)); }
        b->live_cap = cap;
        b->live_h_bytes = bytes;
    }
    std::vector<long long> sig = {(long long)(uintptr_t)b->live_tab, (long long)cap};
    for (int i : b->live) sig.push_back(i);
    if (sig != b->live_sig) batch_drop_graph(b);
    b->live_sig = sig;
    for (size_t r = 0; r < b->live.size(); ++r) {
        lsgb_solver* s = b->inst[b->live[r]];
        char* slot = b->live_h + r * cap * esz;
        double t = s->vel_t;
        for (int n = 0; n < n_steps; ++n) {
            if (esz == sizeof(double)) ((double*)slot)[n] = t;
            else ((float*)slot)[n] = defo_time_factor(t, s->vel_T);
            t += s->p.dt;
        }
        s->batch_live.tab = b->live_tab + r * cap * esz;
        s->batch_live.base = b->live_base;
        s->batch_live.q = 0;
    }
    LSGB_CUDA(cudaMemcpyAsync(b->live_tab, b->live_h, cap * esz * b->live.size(), cudaMemcpyHostToDevice, b->main));
    LSGB_CUDA(cudaEventRecord(b->live_copied, b->main));
    LSGB_CUDA(cudaMemsetAsync(b->live_base, 0, sizeof(int), b->main));
    return LSGB_OK;
}

// After an advance call: the live instances' clocks move on by n_steps
// steps and they leave the batch's table.
void batch_live_end(lsgb_batch* b, int n_steps, bool advanced) {
    for (int i : b->live) {
        lsgb_solver* s = b->inst[i];
        if (advanced)
            for (int n = 0; n < n_steps; ++n) s->vel_t += s->p.dt;
        s->batch_live = LiveAt();
    }
}

}  // namespace

extern "C" int lsgb_batch_create(int precision, int n_lanes, lsgb_batch** out) {
    if (!out) return fail(LSGB_ERR_INVALID, "out is NULL");
    if (precision != LSGB_PREC_F64 && precision != LSGB_PREC_F32)
        return fail(LSGB_ERR_INVALID, "unknown precision %d", precision);
    if (n_lanes < 1 || n_lanes > 64) return fail(LSGB_ERR_INVALID, "n_lanes must lie in [1, 64]");
    lsgb_batch* b = new lsgb_batch();
    b->prec = precision;
    cudaError_t e = cudaStreamCreateWithFlags(&b->main, cudaStreamNonBlocking);
    for (int l = 0; l < n_lanes && e == cudaSuccess; ++l) {
        cudaStream_t st;
        cudaEvent_t ev;
        e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        if (e == cudaSuccess) b->lanes.push_back(st);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e == cudaSuccess) b->lane_done.push_back(ev);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        lsgb_batch_destroy(b);
        return fail(LSGB_ERR_CUDA, "batch streams: %s", cudaGetErrorString(e));
    }
    *out = b;
    return LSGB_OK;
}

extern "C" int lsgb_batch_destroy(lsgb_batch* b) {
    if (!b) return LSGB_OK;
    if (b->main) cudaStreamSynchronize(b->main);
    batch_drop_graph(b);
    if (b->d_tab) cudaFree(b->d_tab);
    if (b->live_tab) cudaFree(b->live_tab);
    if (b->live_base) cudaFree(b->live_base);
    if (b->live_h) cudaFreeHost(b->live_h);
    if (b->live_copied) cudaEventDestroy(b->live_copied);
    for (lsgb_solver* s : b->inst) lsgb_solver_destroy(s);
    for (cudaStream_t l : b->lanes) cudaStreamDestroy(l);
    for (cudaEvent_t ev : b->lane_done) cudaEventDestroy(ev);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->done) cudaEventDestroy(b->done);
    if (b->main) cudaStreamDestroy(b->main);
    delete b;
    return LSGB_OK;
}

extern "C" int lsgb_batch_add(lsgb_batch* b, const lsgb_params* p, lsgb_solver** solver, int* index) {
    LSGB_TRY(batch_ok(b));
    lsgb_solver* s = nullptr;
    LSGB_TRY(lsgb_solver_create(p, b->prec, &s));
    b->inst.push_back(s);
    batch_drop_graph(b);
    if (solver) *solver = s;
    if (index) *index = (int)b->inst.size() - 1;
    return LSGB_OK;
}

extern "C" int lsgb_batch_size(const lsgb_batch* b, int* n) {
    LSGB_TRY(batch_ok(b));
    if (!n) return fail(LSGB_ERR_INVALID, "n is NULL");
    *n = (int)b->inst.size();
    return LSGB_OK;
}

extern "C" int lsgb_batch_solver(lsgb_batch* b, int index, lsgb_solver** out) {
    LSGB_TRY(batch_ok(b));
    if (!out || index < 0 || index >= (int)b->inst.size()) return fail(LSGB_ERR_INVALID, "bad instance index");
    *out = b->inst[index];
    return LSGB_OK;
}

namespace {

// One RK3 stage-1 launch (G -> A, the state is not touched) of every
// instance, spread over the lanes as a step spreads them, `reps` times;
// CUDA-event time per repetition on the batch stream.
int batch_time_stage1(lsgb_batch* b, int reps, float* ms) {
    cudaEvent_t e0, e1;
    LSGB_CUDA(cudaEventCreate(&e0));
    LSGB_CUDA(cudaEventCreate(&e1));
    int rc = LSGB_OK;
    cudaEventRecord(e0, b->main);
    cudaEventRecord(b->fork, b->main);
    for (cudaStream_t l : b->lanes) cudaStreamWaitEvent(l, b->fork, 0);
    for (int r = 0; r < reps && rc == LSGB_OK; ++r)
        for (size_t i = 0; i < b->inst.size() && rc == LSGB_OK; ++i) {
            lsgb_solver* s = b->inst[i];
            cudaStream_t own = s->st;
            s->st = b->lanes[i % b->lanes.size()];
            StageArgs a = stage_args(s->p, s->g, s->lay);
            a.u = s->u; a.v = s->v; a.w = s->w; a.sl = s->sl;
            a.err = err_flag(s);
            a.tile = s->tile;
            a.Gn = s->G; a.Gin = s->G; a.Gout = s->A; a.stage = 1;
            rc = launch_stage(s, a);
            s->st = own;
        }
    for (size_t l = 0; l < b->lanes.size(); ++l) {
        cudaEventRecord(b->lane_done[l], b->lanes[l]);
        cudaStreamWaitEvent(b->main, b->lane_done[l], 0);
    }
    cudaEventRecord(e1, b->main);
    if (cudaEventSynchronize(e1) != cudaSuccess && rc == LSGB_OK) rc = fail(LSGB_ERR_CUDA, "batch timing failed");
    float t = 0.0f;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = t / (reps > 0 ? reps : 1);
    return rc;
}

}  // namespace

namespace {

// One grouped RK3 stage-1 launch (G -> A, the state is not touched) of the
// batch's 3D (dim 3) or 2D instances, `reps` times; CUDA-event time per
// repetition on the batch stream.
int batch_time_group(lsgb_batch* b, int dim, int reps, float* ms) {
    LSGB_TRY(batch_tables(b));
    cudaEvent_t e0, e1;
    LSGB_CUDA(cudaEventCreate(&e0));
    LSGB_CUDA(cudaEventCreate(&e1));
    const char* d = (const char*)b->d_tab;
    cudaError_t e = cudaEventRecord(e0, b->main);
    for (int r = 0; r < reps && e == cudaSuccess; ++r)
        e = dim == 3 ? launch_stage3d_f32_group(d + b->off3, (const int*)(d + b->oo3), (int)b->i3.size(), b->blk3, 1,
                                                b->main)
                     : launch_stage2d_f32_group(d + b->off2, (const int*)(d + b->oo2), (int)b->i2.size(), b->tiles2, 1,
                                                b->shape2, b->main);
    if (e == cudaSuccess) e = cudaEventRecord(e1, b->main);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float t = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return fail(LSGB_ERR_CUDA, "batch timing: %s", cudaGetErrorString(e));
    *ms = t / (reps > 0 ? reps : 1);
    return LSGB_OK;
}

// Grouped form: the per-instance 3D z-chunks from the single-instance tuning
// against each uniform chunk, timed as one grouped 3D launch; then the 2D
// tile height, timed as one grouped 2D launch.  The fastest choices stay.
int batch_autotune_grouped(lsgb_batch* b, int reps) {
    std::vector<int> tuned(b->inst.size());
    for (size_t i = 0; i < b->inst.size(); ++i) tuned[i] = b->inst[i]->tile;
    bool any3 = false, any2 = false;
    for (const lsgb_solver* s : b->inst) (s->p.dim == 3 ? any3 : any2) = true;
    float t = 0.0f, best = 0.0f;
    if (any3) {
        std::vector<int> pick = tuned;
        LSGB_TRY(batch_time_group(b, 3, 1, &t));  // warm-up
        LSGB_TRY(batch_time_group(b, 3, reps, &best));
        for (int zc : {16, 32, 64}) {
            for (lsgb_solver* s : b->inst)
                if (s->p.dim == 3) s->tile = zc;
            LSGB_TRY(batch_time_group(b, 3, reps, &t));
            if (t < best) {
                best = t;
                for (size_t i = 0; i < b->inst.size(); ++i) pick[i] = b->inst[i]->tile;
            }
        }
        for (size_t i = 0; i < b->inst.size(); ++i)
            if (b->inst[i]->p.dim == 3) b->inst[i]->tile = pick[i];
    }
    if (any2) {
        int pick = 32;
        for (int shape : {32, 16}) {
            b->shape2 = shape;
            if (shape == 32) LSGB_TRY(batch_time_group(b, 2, 1, &t));  // warm-up
            LSGB_TRY(batch_time_group(b, 2, reps, &t));
            if (shape == 32 || t < best) {
                best = t;
                pick = shape;
            }
        }
        b->shape2 = pick;
        for (lsgb_solver* s : b->inst)
            if (s->p.dim == 2) s->tile = pick;
    }
    LSGB_TRY(batch_tables(b));
    for (lsgb_solver* s : b->inst) LSGB_TRY(check_flag(s));
    return LSGB_OK;
}

}  // namespace

// Tiles for throughput of the whole batch: every instance's fastest shape
// alone (lsgb_solver_autotune), then the choices that apply to the batch as
// a whole, timed together.  Grouped form: batch_autotune_grouped.  Lanes
// form: each uniform z-chunk for the 3D instances over the lanes.  (Alone,
// short chunks win by filling the SMs; run together, the instances fill them
// and long chunks win by their smaller halo overhead.)
extern "C" int lsgb_batch_autotune(lsgb_batch* b, int reps) {
    LSGB_TRY(batch_ok(b));
    // live instances are timed on the vortex at their current time
    for (lsgb_solver* s : b->inst)
        if (s->vel_live) LSGB_TRY(materialize_velocity(s));
    for (lsgb_solver* s : b->inst) LSGB_TRY(lsgb_solver_autotune(s, reps, nullptr, nullptr));
    batch_drop_graph(b);
    if (b->prec != LSGB_PREC_F32 || b->inst.empty()) return LSGB_OK;
    for (lsgb_solver* s : b->inst)
        if (!s->have_G || !s->have_vel) return LSGB_OK;
    if (reps < 1) reps = 3;
    if (batch_grouped_ok(b)) return batch_autotune_grouped(b, reps);
    std::vector<int> best(b->inst.size());
    for (size_t i = 0; i < b->inst.size(); ++i) best[i] = b->inst[i]->tile;
    float t_best = 0.0f;
    LSGB_TRY(batch_time_stage1(b, 1, &t_best));  // warm-up
    LSGB_TRY(batch_time_stage1(b, reps, &t_best));
    const std::vector<int> tuned = best;
    for (int zc : {16, 32, 64}) {
        bool any = false;
        for (size_t i = 0; i < b->inst.size(); ++i) {
            lsgb_solver* s = b->inst[i];
            s->tile = s->p.dim == 3 ? zc : tuned[i];
            any = any || s->p.dim == 3;
        }
        if (!any) break;
        float t = 0.0f;
        LSGB_TRY(batch_time_stage1(b, reps, &t));
        if (t < t_best) {
            t_best = t;
            for (size_t i = 0; i < b->inst.size(); ++i) best[i] = b->inst[i]->tile;
        }
    }
    for (size_t i = 0; i < b->inst.size(); ++i) b->inst[i]->tile = best[i];
    for (lsgb_solver* s : b->inst) LSGB_TRY(check_flag(s));
    return LSGB_OK;
}

extern "C" int lsgb_batch_advance(lsgb_batch* b, int n_steps) {
    LSGB_TRY(batch_ok(b));
    if (n_steps < 0) return fail(LSGB_ERR_INVALID, "n_steps < 0");
    if (b->inst.empty() || n_steps == 0) return LSGB_OK;
    for (lsgb_solver* s : b->inst)
        if (!s->have_G || !s->have_vel) return fail(LSGB_ERR_STATE, "an instance has no fields");
    int step = 0, interval = 1, reinit_on = 0;
    LSGB_TRY(batch_uniform(b, &step, &interval, &reinit_on));
    // live instances read each step's vortex time from a device table
    struct LiveScope {
        lsgb_batch* b;
        int n;
        bool ok = false;
        ~LiveScope() { batch_live_end(b, n, ok); }
    } live_scope{b, n_steps};
    // order the batch after any work queued on the instances' own streams
    for (lsgb_solver* s : b->inst) {
        LSGB_CUDA(cudaEventRecord(b->done, s->st));
        LSGB_CUDA(cudaStreamWaitEvent(b->main, b->done, 0));
    }
    LSGB_TRY(batch_live_begin(b, n_steps));
    // Steps before the first period boundary run as direct launches.  A
    // period starts at a step s with s % interval == 1 (the reinit then runs
    // after its last step), so its launch sequence is the same every time and
    // one captured graph replays it.
    // grouped form: refresh the descriptor tables (dt, S_L, tiles may have
    // changed); a captured graph stays valid while the launch shapes do
    const bool grouped = batch_grouped_ok(b);
    if (grouped) {
        LSGB_TRY(batch_tables(b));
        const std::vector<long long> sig = {b->blk3, b->tiles2, b->rblk3, b->rblk2, b->cblk3, b->cblk2,
                                            (long long)b->shape2, (long long)b->iters,
                                            (long long)b->i3.size(), (long long)b->i2.size()};
        if (b->block && (!b->grouped || sig != b->sig)) batch_drop_graph(b);
        b->sig = sig;
    } else if (b->block && b->grouped) {
        batch_drop_graph(b);
    }
    auto launch = [&](int n) -> int {
        return grouped ? batch_launch_steps_grouped(b, n) : batch_launch_steps(b, n);
    };
    int remaining = n_steps;
    auto direct = [&](int n) -> int {
        LSGB_TRY(launch(n));
        remaining -= n;
        return LSGB_OK;
    };
    const int L = interval;
    int head = 0;
    while (head < remaining && (L == 1 ? false : ((step + head) % L) != 1)) head++;
    if (head > 0) LSGB_TRY(direct(head));
    if (remaining >= L) {
        if (!b->block || b->block_len != L) {
            batch_drop_graph(b);
            // capture one period; batch_launch_steps advances the host-side
            // step counters, which are restored after the capture
            std::vector<int> steps0;
            for (lsgb_solver* s : b->inst) steps0.push_back(s->step);
            uint64_t k0 = lsgb_launch_count();
            LSGB_CUDA(cudaStreamBeginCapture(b->main, cudaStreamCaptureModeThreadLocal));
            int rc = launch(L);
            cudaGraph_t graph = nullptr;
            cudaError_t e = cudaStreamEndCapture(b->main, &graph);
            for (size_t i = 0; i < b->inst.size(); ++i) b->inst[i]->step = steps0[i];
            if (rc != LSGB_OK) { if (graph) cudaGraphDestroy(graph); return rc; }
            if (e != cudaSuccess) return fail(LSGB_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
            e = cudaGraphInstantiate(&b->block, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) { b->block = nullptr; return fail(LSGB_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e)); }
            b->block_len = L;
            b->grouped = grouped;
            b->graph_kernels = (int64_t)(lsgb_launch_count() - k0);
            uncount_launches((uint64_t)b->graph_kernels);
        }
        while (remaining >= L) {
            LSGB_CUDA(cudaGraphLaunch(b->block, b->main));
            count_launches((uint64_t)b->graph_kernels);
            b->graph_launches++;
            for (lsgb_solver* s : b->inst) s->step += L;
            remaining -= L;
        }
    }
    if (remaining > 0) LSGB_TRY(direct(remaining));
    live_scope.ok = true;
    // later calls on an instance's own stream see the batch's results
    LSGB_CUDA(cudaEventRecord(b->done, b->main));
    for (lsgb_solver* s : b->inst) LSGB_CUDA(cudaStreamWaitEvent(s->st, b->done, 0));
    return LSGB_OK;
}

extern "C" int lsgb_batch_set_mode(lsgb_batch* b, int mode) {
    LSGB_TRY(batch_ok(b));
    if (mode != LSGB_BATCH_GROUPED && mode != LSGB_BATCH_LANES) return fail(LSGB_ERR_INVALID, "unknown batch mode %d", mode);
    if (mode != b->mode) batch_drop_graph(b);
    b->mode = mode;
    return LSGB_OK;
}

extern "C" int lsgb_batch_get_mode(const lsgb_batch* b, int* mode) {
    LSGB_TRY(batch_ok(b));
    if (!mode) return fail(LSGB_ERR_INVALID, "mode is NULL");
    *mode = batch_grouped_ok(b) ? LSGB_BATCH_GROUPED : LSGB_BATCH_LANES;
    return LSGB_OK;
}

extern "C" int lsgb_batch_sync(lsgb_batch* b) {
    LSGB_TRY(batch_ok(b));
    LSGB_CUDA(cudaStreamSynchronize(b->main));
    for (lsgb_solver* s : b->inst) LSGB_TRY(check_flag(s));
    return LSGB_OK;
}

extern "C" int lsgb_batch_stats(const lsgb_batch* b, int64_t* graph_launches, int64_t* kernels_per_graph) {
    LSGB_TRY(batch_ok(b));
    if (graph_launches) *graph_launches = b->graph_launches;
    if (kernels_per_graph) *kernels_per_graph = b->graph_kernels;
    return LSGB_OK;
}

extern "C" int lsgb_batch_stream(lsgb_batch* b, void** stream) {
    LSGB_TRY(batch_ok(b));
    if (!stream) return fail(LSGB_ERR_INVALID, "stream is NULL");
    *stream = (void*)b->main;
    return LSGB_OK;
}

// ---------------------------------------------------------------------------
// discrete adjoint (adjoint.cu kernels)
// ---------------------------------------------------------------------------

struct lsgb_adjoint {
    lsgb_solver* s = nullptr;
    int ckpt = 20;             // checkpoint interval (steps)
    int n_steps = 0;           // steps of the last forward
    int step0 = 0;             // solver step when that forward started
    bool have_fwd = false, have_seed = false, have_target = false, have_grad = false;
    double eps = 0.0;          // Heaviside width
    int grads = LSGB_GRAD_SL | LSGB_GRAD_VELOCITY;  // parameter gradients accumulated
    size_t slot = 0;           // bytes per field slot (multiple of 256)
    int tape_slots = 0, ckpt_slots = 0;
    char* tape = nullptr;      // the recompute tape the next launches use (one of tape_buf)
    char* tape_buf[2] = {nullptr, nullptr};  // two tapes: segment n-1 is recorded while n is reversed
    cudaStream_t rs = nullptr;               // recording stream (second tape only)
    cudaEvent_t ev_rec[2] = {nullptr, nullptr}, ev_rev[2] = {nullptr, nullptr};
    char* ckpts = nullptr;     // G at every segment start
    void* coef = nullptr;      // coefficient planes (stage slab or HCR-2 full domain)
    int slab = 1;              // z planes per coefficient slab of the stage transpose (3D)
    int slab_auto = 1;         // the slab chosen at creation
    size_t coef_bytes = 0;
    void* lam[4] = {nullptr, nullptr, nullptr, nullptr};  // lambda buffers (solver precision)
    double* grad[4] = {nullptr, nullptr, nullptr, nullptr};  // dL/dS_L, dL/du, dL/dv, dL/dw
    double* target = nullptr;  // FP64 compact target
    // live deformation velocity during the recorded forward: the vortex time
    // at every checkpoint, and the fields the recompute (vel[0..2], recording
    // stream) and the reverse sweep (vel[3..5], solver stream) refill per step
    bool live = false;
    double live_T = 1.0;
    std::vector<double> ckpt_t;
    char* vel = nullptr;
};

namespace {

// Slots of one recorded step on the tape: stage inputs, HCR-2 inputs
// phi^0 .. phi^{M-1} (phi^0 = phi0), and the slot holding the step's result.
struct TapeStep {
    int gn, g1, g2;
    int r0;      // first HCR-2 slot, -1 when no reinitialisation follows the step
    int out;
    double t;    // vortex time of the step (live velocity)
};

bool reinit_after(const lsgb_params& p, int step) {
    return p.enable_reinit && p.reinit_iterations > 0 && step > 0 && step % p.reinit_interval == 0;
}

// Tape layout of the steps [t0, t1) starting in slot 0.
std::vector<TapeStep> tape_plan(const lsgb_params& p, int t0, int t1, int* slots) {
    std::vector<TapeStep> v;
    int cur = 0;
    for (int t = t0; t < t1; ++t) {
        TapeStep r;
        r.gn = cur; r.g1 = cur + 1; r.g2 = cur + 2;
        int next = cur + 3;
        r.r0 = -1;
        if (reinit_after(p, t)) { r.r0 = next; next += p.reinit_iterations; }
        r.out = next;
        cur = next;
        v.push_back(r);
    }
    *slots = cur + 1;
    return v;
}

// The tape plan of checkpoint segment seg, with the vortex time of every
// step accumulated as the forward did (t += dt after each step).
std::vector<TapeStep> segment_plan(const lsgb_adjoint* a, int seg, int* slots) {
    const lsgb_solver* s = a->s;
    const int t0 = a->step0 + seg * a->ckpt, t1 = std::min(t0 + a->ckpt, a->step0 + a->n_steps);
    std::vector<TapeStep> plan = tape_plan(s->p, t0, t1, slots);
    double t = a->live ? a->ckpt_t[seg] : 0.0;
    for (TapeStep& r : plan) {
        r.t = t;
        t += s->p.dt;
    }
    return plan;
}

// velocity field q (0..2) of set b (0 = recompute, 1 = reverse sweep)
void* live_vel(lsgb_adjoint* a, int b, int q) { return a->vel + (size_t)(3 * b + q) * a->slot; }

int adj_ok(const lsgb_adjoint* a) {
    if (!a || !a->s) return fail(LSGB_ERR_INVALID, "adjoint handle is NULL");
    return LSGB_OK;
}

int adj_alloc(void** p, size_t bytes, const char* what) {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) { *p = nullptr; return fail(LSGB_ERR_ALLOC, "%s (%zu B): %s", what, bytes, cudaGetErrorString(e)); }
    return LSGB_OK;
}

void* tslot(lsgb_adjoint* a, int q) { return a->tape + (size_t)q * a->slot; }

// Recompute the steps [t0, t1) from tape slot 0 with the solver's kernels,
// keeping every stage and pseudo-step input.
int adj_record(lsgb_adjoint* a, const std::vector<TapeStep>& plan) {
    lsgb_solver* s = a->s;
    StageArgs st = stage_args(s->p, s->g, s->lay);
    st.u = s->u; st.v = s->v; st.w = s->w; st.sl = s->sl;
    st.err = err_flag(s);
    st.tile = s->tile;
    ReinitArgs r;
    r.g = s->g;
    r.lay = s->lay;
    r.dx = s->p.dx;
    r.dy = s->p.dy;
    r.dz = s->p.dim == 3 ? s->p.dz : s->p.dx;
    r.dtau = s->p.reinit_dtau;
    r.beta = s->p.reinit_beta;
    for (const TapeStep& t : plan) {
        if (a->live) {
            LSGB_TRY(fill_deformation_into(s, t.t, a->live_T, live_vel(a, 0, 0), live_vel(a, 0, 1), live_vel(a, 0, 2),
                                           s->st));
            st.u = live_vel(a, 0, 0); st.v = live_vel(a, 0, 1); st.w = live_vel(a, 0, 2);
        }
        st.Gn = tslot(a, t.gn);
        st.Gin = tslot(a, t.gn); st.Gout = tslot(a, t.g1); st.stage = 1;
        LSGB_TRY(launch_stage(s, st));
        st.Gin = tslot(a, t.g1); st.Gout = tslot(a, t.g2); st.stage = 2;
        LSGB_TRY(launch_stage(s, st));
        st.Gin = tslot(a, t.g2); st.stage = 3;
        st.Gout = tslot(a, t.r0 >= 0 ? t.r0 : t.out);
        LSGB_TRY(launch_stage(s, st));
        if (t.r0 >= 0) {
            r.phi0 = tslot(a, t.r0);
            for (int m = 0; m < s->p.reinit_iterations; ++m) {
                r.phin = tslot(a, t.r0 + m);
                r.phinew = tslot(a, m + 1 < s->p.reinit_iterations ? t.r0 + m + 1 : t.out);
                if (s->prec == LSGB_PREC_F64) LSGB_CUDA(launch_reinit_f64(r, s->st));
                else LSGB_CUDA(launch_reinit_f32(r, s->st));
            }
        }
    }
    return LSGB_OK;
}

template <typename T>
int adj_reverse_step(lsgb_adjoint* a, const TapeStep& t, void** L) {
    lsgb_solver* s = a->s;
    const Geo g = s->g;
    void* others[3];
    int q = 0;
    for (int b = 0; b < 4; ++b)
        if (a->lam[b] != *L) others[q++] = a->lam[b];
    void* X = others[0];
    void* Y = others[1];
    void* ACC = others[2];
    if (t.r0 >= 0) {
        // phi^{m+1} = F(phi^m, phi0), m = M-1 .. 0
        const int M = s->p.reinit_iterations;
        AdjReinitArgs rc;
        rc.g = g;
        rc.phi0 = tslot(a, t.r0);
        rc.coef = a->coef;
        rc.dx = s->p.dx;
        rc.dy = s->p.dy;
        rc.dz = s->p.dim == 3 ? s->p.dz : s->p.dx;
        rc.dtau = s->p.reinit_dtau;
        rc.beta = s->p.reinit_beta;
        AdjReinitGatherArgs rg;
        rg.g = g;
        rg.coef = a->coef;
        rg.lam0 = ACC;
        void* mu = *L;
        void* spare = X;
        for (int m = M - 1; m >= 0; --m) {
            rc.phin = tslot(a, t.r0 + m);
            rc.mu = mu;
            rg.mu_out = spare;
            rg.first = m == M - 1;
            rg.last = m == 0;
            LSGB_CUDA(launch_reinit_adj<T>(rc, rg, s->st));
            std::swap(mu, spare);
        }
        *L = mu;
        X = spare;
    }
    AdjStageArgs c;
    std::memset(&c, 0, sizeof(c));
    c.g = g;
    c.u = s->u; c.v = s->v; c.w = s->w; c.sl = s->sl;
    if (a->live) {
        LSGB_TRY(fill_deformation_into(s, t.t, a->live_T, live_vel(a, 1, 0), live_vel(a, 1, 1), live_vel(a, 1, 2),
                                       s->st));
        c.u = live_vel(a, 1, 0); c.v = live_vel(a, 1, 1); c.w = live_vel(a, 1, 2);
    }
    c.s_l = s->p.s_l;
    c.eps = s->p.epsilon;
    c.dx = s->p.dx;
    c.dy = s->p.dy;
    c.dz = s->p.dim == 3 ? s->p.dz : s->p.dx;
    c.coef = a->coef;
    c.gS = (a->grads & LSGB_GRAD_SL) ? a->grad[0] : nullptr;
    const bool vel = (a->grads & LSGB_GRAD_VELOCITY) != 0;
    c.gu = vel ? a->grad[1] : nullptr;
    c.gv = vel ? a->grad[2] : nullptr;
    c.gw = vel && s->p.dim == 3 ? a->grad[3] : nullptr;
    AdjGatherArgs gt;
    std::memset(&gt, 0, sizeof(gt));
    gt.g = g;
    gt.coef = a->coef;
    const double dt = s->p.dt;
    // stage 3: G^{n+1} = 1/3 G^n + 2/3 G2 + 2/3 dt L(G2)
    // one stage transpose, slab by slab along z
    auto stage = [&]() -> int {
        const int nz = g.dim == 3 ? g.nz : 1;
        const int step = g.dim == 3 ? a->slab : 1;
        for (int z0 = 0; z0 < nz; z0 += step) {
            c.z0 = gt.z0 = z0;
            c.zn = gt.zn = std::min(step, nz - z0);
            LSGB_CUDA(launch_stage_adj<T>(c, gt, s->st));
        }
        return LSGB_OK;
    };
    c.Gin = tslot(a, t.g2); c.cdt = 2.0 / 3.0 * dt; c.lam = *L;
    gt.lam = *L; gt.out = X; gt.acc = ACC; gt.acc_init = 1; gt.c_self = 2.0 / 3.0; gt.c_n = 1.0 / 3.0;
    gt.addend = nullptr;
    LSGB_TRY(stage());
    // stage 2: G2 = 3/4 G^n + 1/4 G1 + 1/4 dt L(G1)
    c.Gin = tslot(a, t.g1); c.cdt = 0.25 * dt; c.lam = X;
    gt.lam = X; gt.out = Y; gt.acc = ACC; gt.acc_init = 0; gt.c_self = 0.25; gt.c_n = 0.75;
    LSGB_TRY(stage());
    // stage 1: G1 = G^n + dt L(G^n)
    c.Gin = tslot(a, t.gn); c.cdt = dt; c.lam = Y;
    gt.lam = Y; gt.out = *L; gt.acc = nullptr; gt.addend = ACC; gt.c_self = 1.0; gt.c_n = 0.0;
    LSGB_TRY(stage());
    return LSGB_OK;
}

// FP64 array (layout, memory) -> FP64 compact device array dst.
int load_f64_compact(lsgb_solver* s, double* dst, const double* src, int layout, int memory) {
    Lay sl = layout == LSGB_LAYOUT_GHOSTED ? ghosted_layout(s->g) : compact_layout(s->g);
    size_t sbytes = sizeof(double) * (size_t)layout_elems(s->g, sl.ghosted);
    const double* dsrc = src;
    if (memory == LSGB_MEM_HOST) {
        if (!sl.ghosted) {
            LSGB_CUDA(cudaMemcpyAsync(dst, src, sbytes, cudaMemcpyHostToDevice, s->st));
            return LSGB_OK;
        }
        LSGB_TRY(ensure_stage(s));
        LSGB_CUDA(cudaMemcpyAsync(s->stage64, src, sbytes, cudaMemcpyHostToDevice, s->st));
        dsrc = s->stage64;
    } else {
        LSGB_TRY(check_dev(src, "field"));
    }
    LSGB_CUDA(launch_pack_f64(s->g, dsrc, sl, dst, s->st));
    return LSGB_OK;
}

// compact device array (FP64 or FP32) -> FP64 out (layout, memory); synchronises.
int store_compact(lsgb_solver* s, const void* src, bool f64, double* out, int layout, int memory) {
    Lay dl = layout == LSGB_LAYOUT_GHOSTED ? ghosted_layout(s->g) : compact_layout(s->g);
    size_t dbytes = sizeof(double) * (size_t)layout_elems(s->g, dl.ghosted);
    double* ddst = out;
    if (memory == LSGB_MEM_HOST) {
        LSGB_TRY(ensure_stage(s));
        ddst = s->stage64;
    } else {
        LSGB_TRY(check_dev(out, "out"));
    }
    if (f64) LSGB_CUDA(launch_unpack_f64(s->g, (const double*)src, ddst, dl, s->st));
    else LSGB_CUDA(launch_unpack_f32(s->g, (const float*)src, ddst, dl, s->st));
    if (memory == LSGB_MEM_HOST) LSGB_CUDA(cudaMemcpyAsync(out, ddst, dbytes, cudaMemcpyDeviceToHost, s->st));
    LSGB_CUDA(cudaStreamSynchronize(s->st));
    return LSGB_OK;
}

}  // namespace

extern "C" int lsgb_adjoint_create(lsgb_solver* s, int checkpoint_interval, lsgb_adjoint** out) {
    LSGB_TRY(solver_ok(s));
    if (!out) return fail(LSGB_ERR_INVALID, "out is NULL");
    if (checkpoint_interval < 1) return fail(LSGB_ERR_INVALID, "checkpoint_interval must be >= 1");
    lsgb_adjoint* a = new lsgb_adjoint();
    a->s = s;
    a->ckpt = checkpoint_interval;
    a->slot = (nbytes(s) + 255) / 256 * 256;
    // Stage transpose in z slabs: by default one slab spans the whole domain
    // (measured fastest at 192^3: slabs small enough for their 19 coefficient
    // planes to stay in L2 between the two passes lost more to the 3-plane
    // halo recompute and the extra launches than they saved in HBM
    // traffic).  The buffer also holds the HCR-2 transpose's 14 planes.
    const size_t slice = (size_t)s->g.nx * s->g.ny * s->esz;  // one z plane of one coefficient
    size_t planes_needed;
    if (s->g.dim == 3) {
        a->slab = s->g.nz;
        planes_needed = std::max((size_t)ADJ_PLANES * (s->g.nz + 6), (size_t)14 * s->g.nz);
    } else {
        a->slab = 1;
        planes_needed = (size_t)ADJ_PLANES;
    }
    a->slab_auto = a->slab;
    a->coef_bytes = planes_needed * slice;
    int rc = adj_alloc(&a->coef, a->coef_bytes, "adjoint coefficient planes");
    for (int b = 0; b < 4 && rc == LSGB_OK; ++b) rc = adj_alloc(&a->lam[b], a->slot, "adjoint field");
    for (int b = 0; b < 4 && rc == LSGB_OK; ++b)
        rc = adj_alloc((void**)&a->grad[b], sizeof(double) * (size_t)s->g.cells(), "gradient field");
    if (rc != LSGB_OK) {
        std::string keep = g_err;
        lsgb_adjoint_destroy(a);
        g_err = keep;
        return rc;
    }
    *out = a;
    return LSGB_OK;
}

extern "C" int lsgb_adjoint_destroy(lsgb_adjoint* a) {
    if (!a) return LSGB_OK;
    if (a->s && a->s->st) cudaStreamSynchronize(a->s->st);
    if (a->rs) cudaStreamSynchronize(a->rs);
    void* ptrs[] = {a->tape_buf[0], a->tape_buf[1], a->ckpts, a->coef, a->lam[0], a->lam[1], a->lam[2],
                    a->lam[3], a->grad[0], a->grad[1], a->grad[2], a->grad[3], a->target, a->vel};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    for (int b = 0; b < 2; ++b) {
        if (a->ev_rec[b]) cudaEventDestroy(a->ev_rec[b]);
        if (a->ev_rev[b]) cudaEventDestroy(a->ev_rev[b]);
    }
    if (a->rs) cudaStreamDestroy(a->rs);
    delete a;
    return LSGB_OK;
}

extern "C" int lsgb_adjoint_set_grads(lsgb_adjoint* a, int mask) {
    LSGB_TRY(adj_ok(a));
    if (mask & ~(LSGB_GRAD_SL | LSGB_GRAD_VELOCITY)) return fail(LSGB_ERR_INVALID, "unknown gradient bits 0x%x", mask);
    a->grads = mask;
    a->have_grad = false;
    return LSGB_OK;
}

extern "C" int lsgb_adjoint_set_slab(lsgb_adjoint* a, int planes) {
    LSGB_TRY(adj_ok(a));
    const lsgb_solver* s = a->s;
    if (s->g.dim != 3) return fail(LSGB_ERR_INVALID, "z slabs apply to 3D grids");
    if (planes < 0) return fail(LSGB_ERR_INVALID, "planes < 0");
    const int want = planes == 0 ? a->slab_auto : std::min(planes, s->g.nz);
    const size_t slice = (size_t)s->g.nx * s->g.ny * s->esz;
    if ((size_t)ADJ_PLANES * (want + 6) * slice > a->coef_bytes)
        return fail(LSGB_ERR_INVALID, "a %d-plane slab does not fit the coefficient buffer", want);
    a->slab = want;
    return LSGB_OK;
}

extern "C" int lsgb_adjoint_forward(lsgb_adjoint* a, int n_steps) {
    LSGB_TRY(adj_ok(a));
    lsgb_solver* s = a->s;
    if (n_steps < 1) return fail(LSGB_ERR_INVALID, "n_steps must be >= 1");
    if (!s->have_G || !s->have_vel) return fail(LSGB_ERR_STATE, "fields not set");
    const int nseg = (n_steps + a->ckpt - 1) / a->ckpt;
    if (s->vel_live && !a->vel) {
        LSGB_CUDA(cudaStreamSynchronize(s->st));
        LSGB_TRY(adj_alloc((void**)&a->vel, 6 * a->slot, "live velocity fields"));
    }
    if (nseg > a->ckpt_slots) {
        LSGB_CUDA(cudaStreamSynchronize(s->st));
        if (a->ckpts) cudaFree(a->ckpts);
        a->ckpts = nullptr;
        a->ckpt_slots = 0;
        LSGB_TRY(adj_alloc((void**)&a->ckpts, (size_t)nseg * a->slot, "checkpoints"));
        a->ckpt_slots = nseg;
    }
    a->step0 = s->step;
    a->have_fwd = a->have_seed = a->have_grad = false;
    a->live = s->vel_live;
    a->live_T = s->vel_T;
    a->ckpt_t.assign(nseg, 0.0);
    for (int seg = 0; seg < nseg; ++seg) {
        a->ckpt_t[seg] = s->vel_t;
        LSGB_CUDA(cudaMemcpyAsync(a->ckpts + (size_t)seg * a->slot, s->G, nbytes(s), cudaMemcpyDeviceToDevice, s->st));
        const int n = std::min(a->ckpt, n_steps - seg * a->ckpt);
        LSGB_TRY(lsgb_solver_advance(s, n));
    }
    a->n_steps = n_steps;
    a->have_fwd = true;
    return LSGB_OK;
}

extern "C" int lsgb_adjoint_set_target(lsgb_adjoint* a, const double* G_target, int layout, int memory,
                                       double eps) {
    LSGB_TRY(adj_ok(a));
    if (!G_target) return fail(LSGB_ERR_INVALID, "G_target is NULL");
    if (!std::isfinite(eps) || eps <= 0.0) return fail(LSGB_ERR_INVALID, "eps must be positive");
    if (layout != LSGB_LAYOUT_GHOSTED && layout != LSGB_LAYOUT_COMPACT)
        return fail(LSGB_ERR_INVALID, "unknown layout %d", layout);
    if (memory != LSGB_MEM_HOST && memory != LSGB_MEM_DEVICE)
        return fail(LSGB_ERR_INVALID, "unknown memory kind %d", memory);
    if (!a->target)
        LSGB_TRY(adj_alloc((void**)&a->target, sizeof(double) * (size_t)a->s->g.cells(), "target field"));
    LSGB_TRY(load_f64_compact(a->s, a->target, G_target, layout, memory));
    a->eps = eps;
    a->have_target = true;
    return LSGB_OK;
}

extern "C" int lsgb_adjoint_loss(lsgb_adjoint* a, int seed, double* loss) {
    LSGB_TRY(adj_ok(a));
    lsgb_solver* s = a->s;
    if (!a->have_target) return fail(LSGB_ERR_STATE, "no target set");
    if (!s->have_G) return fail(LSGB_ERR_STATE, "G has not been set");
    const double dv = cell_volume(s->p);
    if (s->prec == LSGB_PREC_F64)
        LSGB_CUDA(launch_heaviside<double>(s->g, (const double*)s->G, a->target, a->eps, dv,
                                           seed ? (double*)a->lam[0] : nullptr, s->scratch, red_out(s), s->st));
    else
        LSGB_CUDA(launch_heaviside<float>(s->g, (const float*)s->G, a->target, a->eps, dv,
                                          seed ? (float*)a->lam[0] : nullptr, s->scratch, red_out(s), s->st));
    double r[2];
    LSGB_TRY(reduce_read(s, r));
    if (loss) *loss = r[0];
    if (seed) a->have_seed = true;
    return LSGB_OK;
}

extern "C" int lsgb_adjoint_backward(lsgb_adjoint* a, const double* dL_dGT, int layout, int memory) {
    LSGB_TRY(adj_ok(a));
    lsgb_solver* s = a->s;
    if (!a->have_fwd) return fail(LSGB_ERR_STATE, "no forward recorded");
    if (dL_dGT) {
        if (layout != LSGB_LAYOUT_GHOSTED && layout != LSGB_LAYOUT_COMPACT)
            return fail(LSGB_ERR_INVALID, "unknown layout %d", layout);
        if (memory != LSGB_MEM_HOST && memory != LSGB_MEM_DEVICE)
            return fail(LSGB_ERR_INVALID, "unknown memory kind %d", memory);
        LSGB_TRY(load_field(s, a->lam[0], dL_dGT, layout, memory));
    } else if (!a->have_seed) {
        return fail(LSGB_ERR_STATE, "no seed: pass dL_dGT or call lsgb_adjoint_loss with seed");
    }
    a->have_seed = false;
    // tape size: the longest segment plan
    const int nseg = (a->n_steps + a->ckpt - 1) / a->ckpt;
    int need = 0;
    for (int seg = 0; seg < nseg; ++seg) {
        const int t0 = a->step0 + seg * a->ckpt, t1 = std::min(t0 + a->ckpt, a->step0 + a->n_steps);
        int slots = 0;
        tape_plan(s->p, t0, t1, &slots);
        need = std::max(need, slots);
    }
    if (need > a->tape_slots) {
        LSGB_CUDA(cudaStreamSynchronize(s->st));
        if (a->rs) LSGB_CUDA(cudaStreamSynchronize(a->rs));
        for (int b = 0; b < 2; ++b) {
            if (a->tape_buf[b]) cudaFree(a->tape_buf[b]);
            a->tape_buf[b] = nullptr;
        }
        a->tape_slots = 0;
        LSGB_TRY(adj_alloc((void**)&a->tape_buf[0], (size_t)need * a->slot, "adjoint tape"));
        // the second tape is optional: without it the segments are recorded in turn
        if (nseg > 1 && cudaMalloc((void**)&a->tape_buf[1], (size_t)need * a->slot) != cudaSuccess) {
            cudaGetLastError();
            a->tape_buf[1] = nullptr;
        }
        a->tape_slots = need;
    }
    const bool two = a->tape_buf[1] != nullptr;
    if (two && !a->rs) {
        LSGB_CUDA(cudaStreamCreateWithFlags(&a->rs, cudaStreamNonBlocking));
        for (int b = 0; b < 2; ++b) {
            LSGB_CUDA(cudaEventCreateWithFlags(&a->ev_rec[b], cudaEventDisableTiming));
            LSGB_CUDA(cudaEventCreateWithFlags(&a->ev_rev[b], cudaEventDisableTiming));
        }
    }
    for (int b = 0; b < 4; ++b)
        if ((b == 0 && (a->grads & LSGB_GRAD_SL)) || (b > 0 && (a->grads & LSGB_GRAD_VELOCITY)))
            LSGB_CUDA(cudaMemsetAsync(a->grad[b], 0, sizeof(double) * (size_t)s->g.cells(), s->st));
    // Segment seg's tape: its checkpoint re-advanced with the forward kernels
    // on stream st into tape buffer b.
    auto record = [&](int seg, int b, cudaStream_t st) -> int {
        int slots = 0;
        const std::vector<TapeStep> plan = segment_plan(a, seg, &slots);
        a->tape = a->tape_buf[b];
        cudaStream_t own = s->st;
        s->st = st;
        int rc = LSGB_OK;
        if (cudaMemcpyAsync(tslot(a, 0), a->ckpts + (size_t)seg * a->slot, nbytes(s), cudaMemcpyDeviceToDevice,
                            st) != cudaSuccess)
            rc = fail(LSGB_ERR_CUDA, "checkpoint restore: %s", cudaGetErrorString(cudaGetLastError()));
        if (rc == LSGB_OK) rc = adj_record(a, plan);
        s->st = own;
        return rc;
    };
    // With two tapes, segment seg-1 is recorded on the recording stream while
    // segment seg is reversed on the solver's stream (the recording of a
    // buffer waits for the reversal that last read it).  Same kernels and
    // inputs either way, so the gradients are the same bits.
    if (two) {
        LSGB_CUDA(cudaEventRecord(a->ev_rec[0], s->st));
        LSGB_CUDA(cudaStreamWaitEvent(a->rs, a->ev_rec[0], 0));
        LSGB_TRY(record(nseg - 1, 0, a->rs));
        LSGB_CUDA(cudaEventRecord(a->ev_rec[0], a->rs));
    }
    // the current adjoint field lives in one of the four buffers
    void* L = a->lam[0];
    int cur = 0;
    for (int seg = nseg - 1; seg >= 0; --seg) {
        if (two) {
            LSGB_CUDA(cudaStreamWaitEvent(s->st, a->ev_rec[cur], 0));
            if (seg > 0) {
                if (seg + 1 < nseg) LSGB_CUDA(cudaStreamWaitEvent(a->rs, a->ev_rev[cur ^ 1], 0));
                LSGB_TRY(record(seg - 1, cur ^ 1, a->rs));
                LSGB_CUDA(cudaEventRecord(a->ev_rec[cur ^ 1], a->rs));
            }
        } else {
            LSGB_TRY(record(seg, 0, s->st));
        }
        int slots = 0;
        const std::vector<TapeStep> plan = segment_plan(a, seg, &slots);
        a->tape = a->tape_buf[cur];
        for (int q = (int)plan.size() - 1; q >= 0; --q) {
            if (s->prec == LSGB_PREC_F64) LSGB_TRY(adj_reverse_step<double>(a, plan[q], &L));
            else LSGB_TRY(adj_reverse_step<float>(a, plan[q], &L));
        }
        if (two) {
            LSGB_CUDA(cudaEventRecord(a->ev_rev[cur], s->st));
            cur ^= 1;
        }
    }
    // keep dL/dG_0 in lam[0]
    if (L != a->lam[0]) {
        for (int b = 1; b < 4; ++b)
            if (a->lam[b] == L) std::swap(a->lam[0], a->lam[b]);
    }
    LSGB_TRY(check_flag(s));
    a->have_grad = true;
    return LSGB_OK;
}

extern "C" int lsgb_adjoint_get_grad(lsgb_adjoint* a, int which, double* out, int layout, int memory) {
    LSGB_TRY(adj_ok(a));
    lsgb_solver* s = a->s;
    if (!a->have_grad) return fail(LSGB_ERR_STATE, "no backward has run");
    if (!out) return fail(LSGB_ERR_INVALID, "out is NULL");
    if (layout != LSGB_LAYOUT_GHOSTED && layout != LSGB_LAYOUT_COMPACT)
        return fail(LSGB_ERR_INVALID, "unknown layout %d", layout);
    if (memory != LSGB_MEM_HOST && memory != LSGB_MEM_DEVICE)
        return fail(LSGB_ERR_INVALID, "unknown memory kind %d", memory);
    switch (which) {
        case LSGB_FIELD_G: return store_compact(s, a->lam[0], s->prec == LSGB_PREC_F64, out, layout, memory);
        case LSGB_FIELD_SL:
            if (!(a->grads & LSGB_GRAD_SL)) return fail(LSGB_ERR_STATE, "dL/dS_L was not requested");
            return store_compact(s, a->grad[0], true, out, layout, memory);
        case LSGB_FIELD_U:
        case LSGB_FIELD_V:
        case LSGB_FIELD_W:
            if (!(a->grads & LSGB_GRAD_VELOCITY)) return fail(LSGB_ERR_STATE, "velocity gradients were not requested");
            if (which == LSGB_FIELD_W && s->p.dim != 3) return fail(LSGB_ERR_INVALID, "no w in 2D");
            return store_compact(s, a->grad[which == LSGB_FIELD_U ? 1 : which == LSGB_FIELD_V ? 2 : 3], true, out,
                                 layout, memory);
        default: return fail(LSGB_ERR_INVALID, "unknown field %d", which);
    }
}

// ---------------------------------------------------------------------------
// binary dumps (dump.cu kernels)
// ---------------------------------------------------------------------------

namespace {

// int32 header of saveFieldBinary3D (io.h:86-88) / 2D saveFieldBinary (2D io.h:86-88)
size_t dump_header(const lsgb_params& p, int32_t* h) {
    if (p.dim == 3) {
        h[0] = p.nx; h[1] = p.ny; h[2] = p.nz; h[3] = p.nghost;
        return 4 * sizeof(int32_t);
    }
    h[0] = p.nx; h[1] = p.ny; h[2] = p.nghost;
    return 3 * sizeof(int32_t);
}

size_t dump_data_bytes(const Geo& g) { return sizeof(double) * (size_t)layout_elems(g, 1); }

// the image's array part from the solver state into dst (device, aligned)
int dump_pack_state(lsgb_solver* s, double* dst, cudaStream_t st) {
    if (s->prec == LSGB_PREC_F64) LSGB_CUDA(launch_dump_compact<double>(s->g, (const double*)s->G, dst, st));
    else LSGB_CUDA(launch_dump_compact<float>(s->g, (const float*)s->G, dst, st));
    return LSGB_OK;
}

void snapshot_writer(Snapshots* sn) {
    cudaSetDevice(sn->device);
    for (;;) {
        std::pair<int, std::string> job;
        {
            std::unique_lock<std::mutex> lk(sn->m);
            sn->cv.wait(lk, [&] { return sn->stop || !sn->jobs.empty(); });
            if (sn->jobs.empty()) return;
            job = sn->jobs.front();
            sn->jobs.pop_front();
        }
        std::string msg;
        cudaError_t e = cudaEventSynchronize(sn->copied[job.first]);
        if (e != cudaSuccess) {
            msg = std::string("snapshot copy: ") + cudaGetErrorString(e);
        } else {
            FILE* f = std::fopen(job.second.c_str(), "wb");
            const size_t n = sn->hdr + sn->data;
            if (!f) msg = "cannot open " + job.second;
            else {
                if (std::fwrite(sn->host[job.first], 1, n, f) != n) msg = "short write to " + job.second;
                if (std::fclose(f) != 0 && msg.empty()) msg = "close failed for " + job.second;
            }
        }
        std::lock_guard<std::mutex> lk(sn->m);
        if (!msg.empty() && sn->err.empty()) sn->err = msg;
        sn->busy[job.first] = false;
        sn->cv.notify_all();
    }
}

int snapshots_open(lsgb_solver* s) {
    if (s->snap) return LSGB_OK;
    Snapshots* sn = new Snapshots();
    int32_t h[4];
    sn->hdr = dump_header(s->p, h);
    sn->data = dump_data_bytes(s->g);
    cudaGetDevice(&sn->device);
    cudaError_t e = cudaStreamCreateWithFlags(&sn->cs, cudaStreamNonBlocking);
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
        e = cudaMalloc((void**)&sn->dev[k], sn->data);
        if (e == cudaSuccess) e = cudaMallocHost((void**)&sn->host[k], sn->hdr + sn->data);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sn->packed[k], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sn->copied[k], cudaEventDisableTiming);
    }
    s->snap = sn;
    if (e != cudaSuccess) {
        std::string why = cudaGetErrorString(e);
        snapshots_close(s);
        return fail(LSGB_ERR_ALLOC, "snapshot buffers: %s", why.c_str());
    }
    sn->th = std::thread(snapshot_writer, sn);
    return LSGB_OK;
}

}  // namespace

void snapshots_close(lsgb_solver* s) {
    Snapshots* sn = s->snap;
    if (!sn) return;
    if (sn->th.joinable()) {
        {
            std::lock_guard<std::mutex> lk(sn->m);
            sn->stop = true;
        }
        sn->cv.notify_all();
        sn->th.join();  // the writer drains the queue before it stops
    }
    for (int k = 0; k < 2; ++k) {
        if (sn->dev[k]) cudaFree(sn->dev[k]);
        if (sn->host[k]) cudaFreeHost(sn->host[k]);
        if (sn->packed[k]) cudaEventDestroy(sn->packed[k]);
        if (sn->copied[k]) cudaEventDestroy(sn->copied[k]);
    }
    if (sn->cs) cudaStreamDestroy(sn->cs);
    delete sn;
    s->snap = nullptr;
}

extern "C" int lsgb_dump_bytes(const lsgb_params* p, size_t* bytes) {
    LSGB_TRY(check_params(p));
    if (!bytes) return fail(LSGB_ERR_INVALID, "bytes is NULL");
    int32_t h[4];
    *bytes = dump_header(*p, h) + dump_data_bytes(geo_of(*p));
    return LSGB_OK;
}

extern "C" int lsgb_dump_f64(const lsgb_params* p, const double* G, void* out, int memory, void* stream) {
    LSGB_TRY(check_params(p));
    LSGB_TRY(check_dev(G, "G"));
    if (!out) return fail(LSGB_ERR_INVALID, "out is NULL");
    if (memory != LSGB_MEM_HOST && memory != LSGB_MEM_DEVICE)
        return fail(LSGB_ERR_INVALID, "unknown memory kind %d", memory);
    if (memory == LSGB_MEM_DEVICE) LSGB_TRY(check_dev(out, "out"));
    cudaStream_t st = (cudaStream_t)stream;
    const Geo g = geo_of(*p);
    int32_t h[4];
    const size_t hb = dump_header(*p, h), db = dump_data_bytes(g);
    double* tmp = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&tmp, db, st);
    if (e != cudaSuccess) return fail(LSGB_ERR_ALLOC, "dump staging (%zu B): %s", db, cudaGetErrorString(e));
    int rc = LSGB_OK;
    e = launch_dump_ghosted(g, G, tmp, st);
    if (e == cudaSuccess) {
        char* o = (char*)out;
        if (memory == LSGB_MEM_HOST) {
            std::memcpy(o, h, hb);
            e = cudaMemcpyAsync(o + hb, tmp, db, cudaMemcpyDeviceToHost, st);
        } else {
            e = cudaMemcpyAsync(o, h, hb, cudaMemcpyHostToDevice, st);
            if (e == cudaSuccess) e = cudaMemcpyAsync(o + hb, tmp, db, cudaMemcpyDeviceToDevice, st);
        }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = fail(LSGB_ERR_CUDA, "dump: %s", cudaGetErrorString(e));
    cudaFreeAsync(tmp, st);
    return rc;
}

extern "C" int lsgb_solver_dump(lsgb_solver* s, void* out, int memory) {
    LSGB_TRY(solver_ok(s));
    if (!out) return fail(LSGB_ERR_INVALID, "out is NULL");
    if (!s->have_G) return fail(LSGB_ERR_STATE, "G has not been set");
    if (memory != LSGB_MEM_HOST && memory != LSGB_MEM_DEVICE)
        return fail(LSGB_ERR_INVALID, "unknown memory kind %d", memory);
    if (memory == LSGB_MEM_DEVICE) LSGB_TRY(check_dev(out, "out"));
    LSGB_TRY(ensure_stage(s));
    int32_t h[4];
    const size_t hb = dump_header(s->p, h), db = dump_data_bytes(s->g);
    LSGB_TRY(dump_pack_state(s, s->stage64, s->st));
    char* o = (char*)out;
    if (memory == LSGB_MEM_HOST) {
        std::memcpy(o, h, hb);
        LSGB_CUDA(cudaMemcpyAsync(o + hb, s->stage64, db, cudaMemcpyDeviceToHost, s->st));
    } else {
        LSGB_CUDA(cudaMemcpyAsync(o, h, hb, cudaMemcpyHostToDevice, s->st));
        LSGB_CUDA(cudaMemcpyAsync(o + hb, s->stage64, db, cudaMemcpyDeviceToDevice, s->st));
    }
    LSGB_CUDA(cudaStreamSynchronize(s->st));
    return check_flag(s);
}

extern "C" int lsgb_solver_snapshot(lsgb_solver* s, const char* path) {
    LSGB_TRY(solver_ok(s));
    if (!path || !*path) return fail(LSGB_ERR_INVALID, "path is empty");
    if (!s->have_G) return fail(LSGB_ERR_STATE, "G has not been set");
    LSGB_TRY(snapshots_open(s));
    Snapshots* sn = s->snap;
    const int k = sn->next;
    {
        std::unique_lock<std::mutex> lk(sn->m);
        sn->cv.wait(lk, [&] { return !sn->busy[k]; });  // the slot's previous file is written
    }
    LSGB_TRY(dump_pack_state(s, sn->dev[k], s->st));
    LSGB_CUDA(cudaEventRecord(sn->packed[k], s->st));
    LSGB_CUDA(cudaStreamWaitEvent(sn->cs, sn->packed[k], 0));
    int32_t h[4];
    dump_header(s->p, h);
    std::memcpy(sn->host[k], h, sn->hdr);
    LSGB_CUDA(cudaMemcpyAsync(sn->host[k] + sn->hdr, sn->dev[k], sn->data, cudaMemcpyDeviceToHost, sn->cs));
    LSGB_CUDA(cudaEventRecord(sn->copied[k], sn->cs));
    {
        std::lock_guard<std::mutex> lk(sn->m);
        sn->busy[k] = true;
        sn->jobs.emplace_back(k, std::string(path));
    }
    sn->cv.notify_all();
    sn->next = k ^ 1;
    return LSGB_OK;
}

extern "C" int lsgb_solver_snapshot_wait(lsgb_solver* s) {
    LSGB_TRY(solver_ok(s));
    Snapshots* sn = s->snap;
    if (!sn) return LSGB_OK;
    std::unique_lock<std::mutex> lk(sn->m);
    sn->cv.wait(lk, [&] { return sn->jobs.empty() && !sn->busy[0] && !sn->busy[1]; });
    if (!sn->err.empty()) {
        std::string e = sn->err;
        sn->err.clear();
        return fail(LSGB_ERR_INVALID, "snapshot: %s", e.c_str());
    }
    return LSGB_OK;
}

// ---------------------------------------------------------------------------
// analyze_error.m diagnostics (diag.cu)
// ---------------------------------------------------------------------------
extern "C" int lsgb_solver_diagnostics(lsgb_solver* s, const double* G_ref, int layout, int memory,
                                       lsgb_diagnostics* out) {
    LSGB_TRY(solver_ok(s));
    if (!G_ref || !out) return fail(LSGB_ERR_INVALID, "G_ref and out must be given");
    if (!s->have_G) return fail(LSGB_ERR_STATE, "G has not been set");
    if (layout != LSGB_LAYOUT_GHOSTED && layout != LSGB_LAYOUT_COMPACT)
        return fail(LSGB_ERR_INVALID, "unknown layout %d", layout);
    if (memory != LSGB_MEM_HOST && memory != LSGB_MEM_DEVICE)
        return fail(LSGB_ERR_INVALID, "unknown memory kind %d", memory);
    double* ref = nullptr;
    double* scr = nullptr;
    const size_t rb = sizeof(double) * (size_t)s->g.cells();
    cudaError_t e = cudaMallocAsync((void**)&ref, rb, s->st);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&scr, diag_scratch_bytes(), s->st);
    if (e != cudaSuccess) {
        if (ref) cudaFreeAsync(ref, s->st);
        return fail(LSGB_ERR_ALLOC, "diagnostics scratch: %s", cudaGetErrorString(e));
    }
    int rc = load_f64_compact(s, ref, G_ref, layout, memory);
    double r[14];
    ContourDist cd{};
    if (rc == LSGB_OK) {
        const double dz = s->p.dim == 3 ? s->p.dz : s->p.dx;
        e = s->prec == LSGB_PREC_F64
                ? launch_diagnostics<double>(s->g, (const double*)s->G, ref, s->p.dx, s->p.dy, dz, scr, s->st)
                : launch_diagnostics<float>(s->g, (const float*)s->G, ref, s->p.dx, s->p.dy, dz, scr, s->st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(r, scr + (diag_scratch_bytes() / sizeof(double) - 14), sizeof(r),
                                cudaMemcpyDeviceToHost, s->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
        // contour-point distances of the script's interface position error
        if (e == cudaSuccess)
            e = s->prec == LSGB_PREC_F64
                    ? contour_distances<double>(s->g, (const double*)s->G, ref, s->p.dx, s->p.dy, dz, &cd, s->st)
                    : contour_distances<float>(s->g, (const float*)s->G, ref, s->p.dx, s->p.dy, dz, &cd, s->st);
        if (e != cudaSuccess) rc = fail(LSGB_ERR_CUDA, "diagnostics: %s", cudaGetErrorString(e));
    }
    cudaFreeAsync(ref, s->st);
    cudaFreeAsync(scr, s->st);
    if (rc != LSGB_OK) return rc;
    const double N = (double)s->g.cells(), dv = cell_volume(s->p);
    out->l2 = std::sqrt(r[0] / N);
    out->linf = r[1];
    const double ref_rms = std::sqrt(r[2] / N);
    out->l2_rel = ref_rms > 0.0 ? out->l2 / ref_rms : 0.0;
    out->volume = r[3] * dv;
    out->volume_ref = r[4] * dv;
    out->volume_smooth = r[5] * dv;
    out->volume_smooth_ref = r[6] * dv;
    out->band_cells = (int64_t)r[7];
    out->grad_mean = r[7] > 0.0 ? r[8] / r[7] : 0.0;
    out->grad_std = r[7] > 1.0 ? std::sqrt(std::max(0.0, (r[9] - r[7] * out->grad_mean * out->grad_mean) / (r[7] - 1.0))) : 0.0;
    out->iface_points = (int64_t)r[12];
    out->iface_mean = r[12] > 0.0 ? r[10] / r[12] : 0.0;
    out->iface_max = r[11];
    out->contour_hausdorff = cd.hausdorff;
    out->contour_mean = cd.mean;
    out->contour_points = (int64_t)cd.points;
    out->contour_points_ref = (int64_t)cd.points_ref;
    return check_flag(s);
}
