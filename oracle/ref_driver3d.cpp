/*
 * Oracle driver over the reference's 3D CPU solver (test infrastructure).
 *
 * Compiled by oracle/build_ref.sh with -I<reference>/Local_code/level-set_MPI_3D/include
 * and -Ioracle/mpi_stub; the reference headers are used unmodified.  Every
 * entry point below sets the reference's SimParams at run time (grid size and
 * spacing included: the solver functions read only params.*, never the
 * compile-time NX/DX) and calls the reference function it names.
 */
#include "config.h"
#include "weno5.h"
#include "boundary.h"
#include "rk3.h"
#include "reinitialization.h"
#include "io.h"
#include "initial_conditions.h"

#include "../oracle_params.h"

#include <vector>
#include <cstring>

static SimParams to_sim(const orc_params* p) {
    SimParams s = initDefaultParams();
    s.nx = p->nx; s.ny = p->ny; s.nz = p->nz;
    s.nghost = 3;
    s.nx_total = p->nx + 6; s.ny_total = p->ny + 6; s.nz_total = p->nz + 6;
    s.dx = p->dx; s.dy = p->dy; s.dz = p->dz;
    /* one rank, periodic Y through self exchange (config.h:242-265) */
    s.local_ny = p->ny;
    s.local_ny_total = p->ny + 6;
    setupMPIDomainDecomposition(s, 0, 1);
    s.s_l = p->s_l;
    s.dt = p->dt;
    s.epsilon = p->epsilon;
    s.enable_reinit = p->enable_reinit != 0;
    s.reinit_interval = p->reinit_interval;
    s.reinit_iterations = p->reinit_iterations;
    s.reinit_dtau = p->reinit_dtau;
    s.reinit_beta = p->reinit_beta;
    return s;
}

static long long total3(const orc_params* p) {
    return (long long)(p->nx + 6) * (p->ny + 6) * (p->nz + 6);
}

extern "C" {

/* rk3TimeStep3D (Local_code/level-set_MPI_3D/include/rk3.h:131) */
void ref3d_rk3_step(const orc_params* p, double* G_n, double* G_new, double* G_1, double* G_2,
                    double* G_rhs, const double* u, const double* v, const double* w) {
    SimParams s = to_sim(p);
    rk3TimeStep3D(G_n, G_new, G_1, G_2, G_rhs, u, v, w, s);
}

/* computeRHS3D (rk3.h:31): interior RHS only */
void ref3d_rhs(const orc_params* p, const double* G, double* G_rhs, const double* u,
               const double* v, const double* w) {
    SimParams s = to_sim(p);
    computeRHS3D(G, G_rhs, u, v, w, s);
}

/* applyBoundaryConditions3D (boundary.h:250) */
void ref3d_apply_bc(const orc_params* p, double* G) {
    SimParams s = to_sim(p);
    applyBoundaryConditions3D(G, s);
}

/* reinitializeWithSwap3D (reinitialization.h:199).  The reference swaps the
 * caller's pointers; this wrapper copies the final field back into phi so
 * the caller's buffer identity does not change. */
void ref3d_reinit(const orc_params* p, double* phi, double* phi_tmp, double* phi0,
                  double* r_tilde, int* flag) {
    SimParams s = to_sim(p);
    s.enable_reinit = true;
    double* a = phi;
    double* b = phi_tmp;
    reinitializeWithSwap3D(&a, &b, phi0, r_tilde, flag, s);
    if (a != phi) std::memcpy(phi, a, sizeof(double) * (size_t)total3(p));
}

/* computeInterfaceCrossings3D (reinitialization.h:46) */
void ref3d_crossings(const orc_params* p, const double* phi0, double* r_tilde, int* flag) {
    SimParams s = to_sim(p);
    computeInterfaceCrossings3D(phi0, r_tilde, flag, s);
}

/* computeInterfaceVolume / computeL2Error3D (io.h:263 / io.h:229) */
double ref3d_volume(const orc_params* p, const double* G) {
    SimParams s = to_sim(p);
    return computeInterfaceVolume(G, s);
}
double ref3d_l2(const orc_params* p, const double* G, const double* G_ref) {
    SimParams s = to_sim(p);
    return computeL2Error3D(G, G_ref, s);
}

/* The reference main loop for a fixed velocity field and a fixed step count
 * (Local_code/level-set_MPI_3D/src/main.cpp:291-316 with the velocity update
 * and the final-step dt clip left out): RK3 step, swap, reinit when
 * enable_reinit && step > 0 && step % interval == 0.  G (ghosted) is updated
 * in place; the velocity gets the reference's BC first (main.cpp:260). */
void ref3d_run(const orc_params* p, int n_steps, double* G, const double* u_in,
               const double* v_in, const double* w_in) {
    SimParams s = to_sim(p);
    size_t n = (size_t)total3(p);
    std::vector<double> Gc(G, G + n), Gnew(n, 0.0), G1(n, 0.0), G2(n, 0.0), Grhs(n, 0.0);
    std::vector<double> u(u_in, u_in + n), v(v_in, v_in + n), w(w_in, w_in + n);
    std::vector<double> tmp(n, 0.0), phi0(n, 0.0), rt(n, 0.0);
    std::vector<int> flag(n, 0);
    applyBoundaryConditions3D(Gc.data(), s);
    applyVelocityBoundaryConditions3D(u.data(), v.data(), w.data(), s);
    double* pG = Gc.data();
    double* pGn = Gnew.data();
    double* pT = tmp.data();
    for (int step = 0; step < n_steps; ++step) {
        rk3TimeStep3D(pG, pGn, G1.data(), G2.data(), Grhs.data(), u.data(), v.data(), w.data(), s);
        double* t = pG; pG = pGn; pGn = t;
        if (s.enable_reinit && step > 0 && step % s.reinit_interval == 0) {
            /* reinitializeWithSwap3D swaps pG with the temp buffer; track both */
            reinitializeWithSwap3D(&pG, &pT, phi0.data(), rt.data(), flag.data(), s);
        }
    }
    std::memcpy(G, pG, sizeof(double) * n);
}

/* The reference's default 3D case end to end: sphere-deformation test with
 * the default compile-time parameters (64^3, DX = 1/63, DT = 1e-3, T = 1.5,
 * S_L = 0, no reinit), time-dependent velocity recomputed each step and the
 * final-step dt clip (src/main.cpp:180-334).  Returns the logged scalars. */
void ref3d_deformation_test(double* l2_out, double* v0_out, double* v1_out, int* steps_out,
                            double* G_final /* ghosted 70^3, may be NULL */) {
    SimParams params = initDefaultParams();
    setupMPIDomainDecomposition(params, 0, 1);
    params.dt = calculateTimeStep(params);
    size_t n = (size_t)params.nx_total * params.local_ny_total * params.nz_total;
    std::vector<double> G(n, 0.0), G_new(n, 0.0), G_1(n, 0.0), G_2(n, 0.0), G_rhs(n, 0.0),
        G_init(n, 0.0), u(n, 0.0), v(n, 0.0), w(n, 0.0);
    initSphereTestCase(G.data(), u.data(), v.data(), w.data(), params);
    applyBoundaryConditions3D(G.data(), params);
    applyVelocityBoundaryConditions3D(u.data(), v.data(), w.data(), params);
    copyInitialField(G.data(), G_init.data(), (int)n);
    *v0_out = computeInterfaceVolume(G.data(), params);
    double* pG = G.data();
    double* pGn = G_new.data();
    double current_time = 0.0;
    int step = 0;
    int max_steps = (int)(params.t_final / params.dt) + 100;
    while (current_time < params.t_final && step < max_steps) {
        if (current_time + params.dt > params.t_final) params.dt = params.t_final - current_time;
        params.current_time = current_time;
        updateDeformationVelocity(u.data(), v.data(), w.data(), params);
        applyVelocityBoundaryConditions3D(u.data(), v.data(), w.data(), params);
        rk3TimeStep3D(pG, pGn, G_1.data(), G_2.data(), G_rhs.data(), u.data(), v.data(), w.data(),
                      params);
        double* t = pG; pG = pGn; pGn = t;
        current_time += params.dt;
        step++;
    }
    *l2_out = computeL2Error3D(pG, G_init.data(), params);
    *v1_out = computeInterfaceVolume(pG, params);
    *steps_out = step;
    if (G_final) std::memcpy(G_final, pG, sizeof(double) * n);
}

/* computeDeformationVelocity (initial_conditions.h:232) on the ghosted grid
 * used by the deformation test, for one time value. */
void ref3d_deformation_velocity(double t, double* u, double* v, double* w) {
    SimParams params = initDefaultParams();
    setupMPIDomainDecomposition(params, 0, 1);
    params.current_time = t;
    initDeformationVelocity3D(u, v, w, params);
}


/* the reference's binary dump writer on a ghosted array (io.h) */
int ref3d_save_binary(const orc_params* p, const double* G, const char* path) {
    SimParams s = to_sim(p);
    return saveFieldBinary3D(path, G, s, 0.0) ? 0 : 1;
}

}  // extern "C"
