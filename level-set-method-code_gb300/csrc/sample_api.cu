// sample_api.cu -- C ABI of the sample surface (include/lsgb.h, lsgb_sample_*):
// argument checks and the launch sequences of RK3_step, the boundary passes,
// the reinitialisation and the forced time loop of sample/main.cpp over the
// kernels of sample_kernels.cu.
#include "common.cuh"
#include "host.hpp"

#include <cmath>
#include <vector>

using namespace lsgb;

namespace {

int check_grid(int nx, int ny) {
    if (nx < 3 || ny < 3) return fail(LSGB_ERR_INVALID, "the sample surface needs nx, ny >= 3 (got %d x %d)", nx, ny);
    if ((long long)(nx + 6) * (ny + 6) > (1LL << 31)) return fail(LSGB_ERR_INVALID, "grid too large");
    return LSGB_OK;
}

int check_spacing(double dx, double dy) {
    if (!(std::isfinite(dx) && dx > 0.0 && std::isfinite(dy) && dy > 0.0))
        return fail(LSGB_ERR_INVALID, "dx, dy must be positive and finite");
    return LSGB_OK;
}

size_t field_bytes(int nx, int ny) { return sizeof(double) * (size_t)(nx + 6) * (ny + 6); }

// Stream-ordered work arrays when the caller passes none.
struct Work {
    double* p = nullptr;
    bool own = false;
    cudaStream_t st;
    explicit Work(cudaStream_t s) : st(s) {}
    int get(double* given, size_t bytes) {
        if (given) {
            p = given;
            return check_dev(given, "work");
        }
        cudaError_t e = cudaMallocAsync((void**)&p, bytes, st);
        if (e != cudaSuccess) { p = nullptr; return fail(LSGB_ERR_ALLOC, "work arrays (%zu B): %s", bytes, cudaGetErrorString(e)); }
        own = true;
        return LSGB_OK;
    }
    ~Work() { if (own && p) cudaFreeAsync(p, st); }
};

SampleArgs sample_args(int nx, int ny, int n_inst, double dx, double dy, double dt, double S_L) {
    SampleArgs a;
    a.nx = nx; a.ny = ny; a.n_inst = n_inst;
    a.u = a.v = a.vel = nullptr;
    a.ctr = nullptr;
    a.init = nullptr;
    a.init_stride = 0;
    a.dx = dx; a.dy = dy; a.dt = dt; a.S_L = S_L;
    return a;
}

// The three stages of RK3_step with the boundary pair after each
// (sample/weno5_rk3.cpp:166-187): G -> G1, (G, G1) -> G2, (G, G2) -> G.
int rk3_sequence(const SampleArgs& a, double* G, double* G1, double* G2, bool bump, cudaStream_t st) {
    LSGB_CUDA(sample_launch_stage(a, 1, G, G, G1, st));
    LSGB_CUDA(sample_launch_stage_bc(a, G1, false, st));
    LSGB_CUDA(sample_launch_stage(a, 2, G1, G, G2, st));
    LSGB_CUDA(sample_launch_stage_bc(a, G2, false, st));
    LSGB_CUDA(sample_launch_stage(a, 3, G2, G, G, st));
    LSGB_CUDA(sample_launch_stage_bc(a, G, bump, st));
    return LSGB_OK;
}

}  // namespace

extern "C" int lsgb_sample_rhs(int nx, int ny, const double* G, const double* u, const double* v, double* rhs,
                               double dx, double dy, double S_L, void* stream) {
    LSGB_TRY(check_grid(nx, ny));
    LSGB_TRY(check_spacing(dx, dy));
    if (!std::isfinite(S_L)) return fail(LSGB_ERR_INVALID, "S_L must be finite");
    LSGB_TRY(check_dev(G, "G"));
    LSGB_TRY(check_dev(u, "u"));
    LSGB_TRY(check_dev(v, "v"));
    LSGB_TRY(check_dev(rhs, "rhs"));
    if (rhs == G) return fail(LSGB_ERR_INVALID, "rhs must not alias G");
    cudaStream_t st = (cudaStream_t)stream;
    SampleArgs a = sample_args(nx, ny, 1, dx, dy, 0.0, S_L);
    a.u = u;
    a.v = v;
    LSGB_CUDA(sample_launch_zero_ghosts(a, rhs, st));
    LSGB_CUDA(sample_launch_stage(a, 0, G, G, rhs, st));
    return LSGB_OK;
}

extern "C" int lsgb_sample_rk3_step(int nx, int ny, double* G, const double* u, const double* v, double dx,
                                    double dy, double dt, double S_L, const double* G_initial, double* work,
                                    void* stream) {
    LSGB_TRY(check_grid(nx, ny));
    LSGB_TRY(check_spacing(dx, dy));
    if (!std::isfinite(dt) || !std::isfinite(S_L)) return fail(LSGB_ERR_INVALID, "dt and S_L must be finite");
    LSGB_TRY(check_dev(G, "G"));
    LSGB_TRY(check_dev(u, "u"));
    LSGB_TRY(check_dev(v, "v"));
    LSGB_TRY(check_dev(G_initial, "G_initial"));
    cudaStream_t st = (cudaStream_t)stream;
    Work w(st);
    LSGB_TRY(w.get(work, 2 * field_bytes(nx, ny)));
    SampleArgs a = sample_args(nx, ny, 1, dx, dy, dt, S_L);
    a.u = u;
    a.v = v;
    a.init = G_initial;
    const size_t n = (size_t)(nx + 6) * (ny + 6);
    return rk3_sequence(a, G, w.p, w.p + n, false, st);
}

extern "C" int lsgb_sample_first_order_upwind(int nx, int ny, double* G, const double* u, const double* v,
                                              double dx, double dy, double dt, double S_L, double* work,
                                              void* stream) {
    LSGB_TRY(check_grid(nx, ny));
    LSGB_TRY(check_spacing(dx, dy));
    if (!std::isfinite(dt) || !std::isfinite(S_L)) return fail(LSGB_ERR_INVALID, "dt and S_L must be finite");
    LSGB_TRY(check_dev(G, "G"));
    LSGB_TRY(check_dev(u, "u"));
    LSGB_TRY(check_dev(v, "v"));
    cudaStream_t st = (cudaStream_t)stream;
    Work w(st);
    LSGB_TRY(w.get(work, field_bytes(nx, ny)));
    SampleArgs a = sample_args(nx, ny, 1, dx, dy, dt, S_L);
    a.u = u;
    a.v = v;
    LSGB_CUDA(sample_launch_first_order_upwind(a, G, w.p, st));
    return LSGB_OK;
}

extern "C" int lsgb_sample_apply_periodic(int nx, int ny, double* G, void* stream) {
    LSGB_TRY(check_grid(nx, ny));
    LSGB_TRY(check_dev(G, "G"));
    SampleArgs a = sample_args(nx, ny, 1, 1.0, 1.0, 0.0, 0.0);
    LSGB_CUDA(sample_launch_periodic(a, G, (cudaStream_t)stream));
    return LSGB_OK;
}

extern "C" int lsgb_sample_apply_anchored_bc(int nx, int ny, double* G, const double* G_initial, void* stream) {
    LSGB_TRY(check_grid(nx, ny));
    LSGB_TRY(check_dev(G, "G"));
    LSGB_TRY(check_dev(G_initial, "G_initial"));
    SampleArgs a = sample_args(nx, ny, 1, 1.0, 1.0, 0.0, 0.0);
    a.init = G_initial;
    LSGB_CUDA(sample_launch_anchored(a, G, (cudaStream_t)stream));
    return LSGB_OK;
}

extern "C" int lsgb_sample_reinitialize(int nx, int ny, double* G, const double* G_initial, double dx, double dy,
                                        int num_iters, double* work, void* stream) {
    LSGB_TRY(check_grid(nx, ny));
    LSGB_TRY(check_spacing(dx, dy));
    if (num_iters < 0) return fail(LSGB_ERR_INVALID, "num_iters < 0");
    LSGB_TRY(check_dev(G, "G"));
    LSGB_TRY(check_dev(G_initial, "G_initial"));
    if (num_iters == 0) return LSGB_OK;
    cudaStream_t st = (cudaStream_t)stream;
    Work w(st);
    LSGB_TRY(w.get(work, field_bytes(nx, ny)));
    SampleArgs a = sample_args(nx, ny, 1, dx, dy, 0.0, 0.0);
    a.init = G_initial;
    const double dtau = 0.2 * (dy < dx ? dy : dx);  // std::min(dx, dy), sample/field.cpp:68
    double* cur = G;
    double* nxt = w.p;
    for (int it = 0; it < num_iters; ++it) {
        LSGB_CUDA(sample_launch_reinit_step(a, cur, nxt, dtau, st));
        LSGB_CUDA(sample_launch_anchored(a, nxt, st));
        double* t = cur; cur = nxt; nxt = t;
    }
    if (cur != G) LSGB_CUDA(cudaMemcpyAsync(G, cur, field_bytes(nx, ny), cudaMemcpyDeviceToDevice, st));
    return LSGB_OK;
}

extern "C" int lsgb_sample_run(int n_inst, int nx, int ny, int n_steps, double* G, const double* G_initial,
                               int shared_initial, double dx, double dy, double dt, double S_L,
                               const lsgb_sample_forcing* forcing, const int* freq, double* t, double* work,
                               void* stream) {
    LSGB_TRY(check_grid(nx, ny));
    LSGB_TRY(check_spacing(dx, dy));
    if (n_inst < 1 || n_inst > 65535) return fail(LSGB_ERR_INVALID, "n_inst must be in [1, 65535]");
    if (n_steps < 0) return fail(LSGB_ERR_INVALID, "n_steps < 0");
    if (!forcing || !freq || !t) return fail(LSGB_ERR_INVALID, "forcing, freq and t must be given");
    if (!std::isfinite(dt) || !std::isfinite(S_L)) return fail(LSGB_ERR_INVALID, "dt and S_L must be finite");
    LSGB_TRY(check_dev(G, "G"));
    LSGB_TRY(check_dev(G_initial, "G_initial"));
    if ((double)n_steps * n_inst * 2 > 1e9) return fail(LSGB_ERR_INVALID, "n_steps x n_inst too large for one call");
    if (n_steps == 0) return LSGB_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t n = (size_t)(nx + 6) * (ny + 6);
    // the forced velocity of every step and instance, with the reference's
    // own time accumulation (sample/main.cpp:131-136, :147)
    std::vector<double> vel((size_t)n_steps * n_inst * 2);
    for (int q = 0; q < n_inst; ++q) {
        double tt = t[q];
        for (int s = 0; s < n_steps; ++s) {
            const double c = cos(freq[q] * 2 * M_PI * (tt));
            vel[2 * ((size_t)s * n_inst + q)] = forcing->u0 + forcing->eps_u * forcing->v0 * c;
            vel[2 * ((size_t)s * n_inst + q) + 1] = forcing->v0 + forcing->eps_v * forcing->v0 * c;
            tt += dt;
        }
        t[q] = tt;
    }
    Work w(st), wv(st);
    LSGB_TRY(w.get(work, 2 * n_inst * n * sizeof(double)));
    const size_t vel_bytes = vel.size() * sizeof(double);
    const size_t vel_slot = (vel_bytes + 255) / 256 * 256;
    LSGB_TRY(wv.get(nullptr, vel_slot + 256));
    double* G1 = w.p;
    double* G2 = w.p + n_inst * n;
    double* dvel = wv.p;
    int* ctr = (int*)((char*)wv.p + vel_slot);
    LSGB_CUDA(cudaMemcpyAsync(dvel, vel.data(), vel_bytes, cudaMemcpyHostToDevice, st));
    LSGB_CUDA(cudaMemsetAsync(ctr, 0, sizeof(int), st));
    SampleArgs a = sample_args(nx, ny, n_inst, dx, dy, dt, S_L);
    a.vel = dvel;
    a.ctr = ctr;
    a.init = G_initial;
    a.init_stride = shared_initial ? 0 : (long long)n;
    // first step's boundary pair (sample/main.cpp:127-128); later steps start
    // from the state the stage-3 boundary pass leaves, which equals what the
    // loop's post-step and pre-step passes produce
    LSGB_CUDA(sample_launch_anchored(a, G, st));
    LSGB_CUDA(sample_launch_periodic(a, G, st));
    for (int s = 0; s < n_steps; ++s) LSGB_TRY(rk3_sequence(a, G, G1, G2, true, st));
    // the loop's post-step pair (sample/main.cpp:140-141)
    LSGB_CUDA(sample_launch_periodic(a, G, st));
    LSGB_CUDA(sample_launch_anchored(a, G, st));
    // the velocity table is host memory: finish before it goes away
    LSGB_CUDA(cudaStreamSynchronize(st));
    return LSGB_OK;
}
