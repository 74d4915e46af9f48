// extern "C" driver around the reference's sample surface (sample/field.cpp,
// sample/weno5_rk3.cpp, sample/first_order_upwind.cpp), compiled from those files in place by build_ref.sh
// into oracle/_ref/libref_sample.so.  Test infrastructure only.
//
// Arrays cross the boundary as flat row-major [ny+6][nx+6] doubles, the
// element order of Field2D::data (sample/field.hpp:8); they are copied into
// and out of Field2D objects around each reference call.
#include <cmath>
#include <cstring>
#include <vector>

#include "field.hpp"
#include "first_order_upwind.hpp"
#include "weno5_rk3.hpp"

namespace {

void to_field(Field2D& f, const double* src) {
    for (int j = 0; j < f.ny + 6; ++j)
        std::memcpy(f.data[j].data(), src + (size_t)j * (f.nx + 6), sizeof(double) * (f.nx + 6));
}

void from_field(const Field2D& f, double* dst) {
    for (int j = 0; j < f.ny + 6; ++j)
        std::memcpy(dst + (size_t)j * (f.nx + 6), f.data[j].data(), sizeof(double) * (f.nx + 6));
}

}  // namespace

extern "C" {

// compute_geqn_rhs (sample/weno5_rk3.cpp:91-145)
void refs_rhs(int nx, int ny, const double* G, const double* u, const double* v, double* rhs, double dx,
              double dy, double S_L) {
    Field2D g(nx, ny), uf(nx, ny), vf(nx, ny), r(nx, ny);
    to_field(g, G);
    to_field(uf, u);
    to_field(vf, v);
    compute_geqn_rhs(g.data, uf.data, vf.data, r.data, dx, dy, S_L);
    from_field(r, rhs);
}

// RK3_step (sample/weno5_rk3.cpp:148-188), in place on G
void refs_rk3_step(int nx, int ny, double* G, const double* u, const double* v, double dx, double dy, double dt,
                   double S_L, const double* G_initial) {
    Field2D g(nx, ny), uf(nx, ny), vf(nx, ny), g0(nx, ny);
    to_field(g, G);
    to_field(uf, u);
    to_field(vf, v);
    to_field(g0, G_initial);
    RK3_step(g, uf, vf, dx, dy, dt, S_L, g0);
    from_field(g, G);
}

// compute_first_order_upwind (sample/first_order_upwind.cpp:6-69), in place on G
void refs_first_order_upwind(int nx, int ny, double* G, const double* u, const double* v, double dx, double dy,
                             double dt, double S_L) {
    Field2D g(nx, ny), uf(nx, ny), vf(nx, ny);
    to_field(g, G);
    to_field(uf, u);
    to_field(vf, v);
    compute_first_order_upwind(g.data, uf.data, vf.data, dx, dy, dt, S_L);
    from_field(g, G);
}

void refs_apply_periodic(int nx, int ny, double* G) {
    Field2D g(nx, ny);
    to_field(g, G);
    g.apply_periodic();
    from_field(g, G);
}

void refs_apply_anchored_bc(int nx, int ny, double* G, const double* G_initial) {
    Field2D g(nx, ny), g0(nx, ny);
    to_field(g, G);
    to_field(g0, G_initial);
    g.apply_anchored_bc(g0);
    from_field(g, G);
}

void refs_reinitialize(int nx, int ny, double* G, const double* G_initial, double dx, double dy, int iters) {
    Field2D g(nx, ny), g0(nx, ny);
    to_field(g, G);
    to_field(g0, G_initial);
    g.reinitialize(g0, dx, dy, iters);
    from_field(g, G);
}

// The time loop of sample/main.cpp:126-148 for n_steps steps from time *t:
// BCs, the spatially uniform forced velocity u0 + eps_u v0 cos(2 pi f t),
// v0 + eps_v v0 cos(2 pi f t), RK3_step, BCs, t += dt.
void refs_run(int nx, int ny, int n_steps, double* G, const double* G_initial, double dx, double dy, double dt,
              double S_L, double u0, double v0, double eps_u, double eps_v, int freq, double* t) {
    Field2D g(nx, ny), g0(nx, ny), u(nx, ny), v(nx, ny);
    to_field(g, G);
    to_field(g0, G_initial);
    double tt = *t;
    for (int s = 0; s < n_steps; ++s) {
        g.apply_anchored_bc(g0);
        g.apply_periodic();
        for (int j = 0; j < ny + 6; ++j)
            for (int i = 0; i < nx + 6; ++i) {
                u.data[j][i] = u0 + eps_u * v0 * cos(freq * 2 * M_PI * (tt));
                v.data[j][i] = v0 + eps_v * v0 * cos(freq * 2 * M_PI * (tt));
            }
        RK3_step(g, u, v, dx, dy, dt, S_L, g0);
        g.apply_periodic();
        g.apply_anchored_bc(g0);
        tt += dt;
    }
    *t = tt;
    from_field(g, G);
}

}  // extern "C"
