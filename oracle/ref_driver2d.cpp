/*
 * Oracle driver over the reference's 2D CPU solver (test infrastructure).
 *
 * Compiled by oracle/build_ref.sh with -I<reference>/Local_code/level-set_MPI_2D/include
 * and -Ioracle/mpi_stub; the reference headers are used unmodified.  With one
 * rank, periodic Y is the reference's own Y exchange with the rank as its own
 * neighbour (neighbor_below = neighbor_above = 0, the pattern of
 * Local_code/level-set_MPI_3D/include/config.h:263-264); zero-gradient Y is the
 * reference default at the global ends (boundary.h:224-228, MPI_PROC_NULL).
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
    s.nx = p->nx; s.ny = p->ny;
    s.nghost = 3;
    s.nx_total = p->nx + 6; s.ny_total = p->ny + 6;
    s.dx = p->dx; s.dy = p->dy;
    s.rank = 0; s.num_procs = 1;
    s.local_ny = p->ny;
    s.local_ny_total = p->ny + 6;
    s.y_start = 0;
    s.neighbor_below = p->periodic_y ? 0 : MPI_PROC_NULL;
    s.neighbor_above = p->periodic_y ? 0 : MPI_PROC_NULL;
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

static size_t total2(const orc_params* p) { return (size_t)(p->nx + 6) * (p->ny + 6); }

extern "C" {

/* rk3TimeStep (Local_code/level-set_MPI_2D/include/rk3.h:168) */
void ref2d_rk3_step(const orc_params* p, double* G_n, double* G_new, double* G_1, double* G_2,
                    double* G_rhs, const double* u, const double* v) {
    SimParams s = to_sim(p);
    rk3TimeStep(G_n, G_new, G_1, G_2, G_rhs, u, v, s);
}

/* computeRHS (rk3.h:54) */
void ref2d_rhs(const orc_params* p, const double* G, double* G_rhs, const double* u,
               const double* v) {
    SimParams s = to_sim(p);
    computeRHS(G, G_rhs, u, v, s);
}

/* applyBoundaryConditions (boundary.h:217) */
void ref2d_apply_bc(const orc_params* p, double* G) {
    SimParams s = to_sim(p);
    applyBoundaryConditions(G, s);
}

/* reinitializeWithSwap (reinitialization.h:321); result copied back into phi */
void ref2d_reinit(const orc_params* p, double* phi, double* phi_tmp, double* phi0,
                  double* r_tilde, int* flag) {
    SimParams s = to_sim(p);
    s.enable_reinit = true;
    double* a = phi;
    double* b = phi_tmp;
    reinitializeWithSwap(&a, &b, phi0, r_tilde, flag, s);
    if (a != phi) std::memcpy(phi, a, sizeof(double) * total2(p));
}

/* computeInterfaceCrossings (reinitialization.h:75) */
void ref2d_crossings(const orc_params* p, const double* phi0, double* r_tilde, int* flag) {
    SimParams s = to_sim(p);
    computeInterfaceCrossings(phi0, r_tilde, flag, s);
}

/* computeInterfaceArea / computeL2Error (io.h:225 / io.h:194) */
double ref2d_area(const orc_params* p, const double* G) {
    SimParams s = to_sim(p);
    return computeInterfaceArea(G, s);
}
double ref2d_l2(const orc_params* p, const double* G, const double* G_ref) {
    SimParams s = to_sim(p);
    return computeL2Error(G, G_ref, s);
}

/* Main loop for a fixed velocity and a fixed step count
 * (Local_code/level-set_MPI_2D/src/main.cpp:314-334 without the final-step dt
 * clip); velocity BC first (main.cpp:281). */
void ref2d_run(const orc_params* p, int n_steps, double* G, const double* u_in,
               const double* v_in) {
    SimParams s = to_sim(p);
    size_t n = total2(p);
    std::vector<double> Gc(G, G + n), Gnew(n, 0.0), G1(n, 0.0), G2(n, 0.0), Grhs(n, 0.0);
    std::vector<double> u(u_in, u_in + n), v(v_in, v_in + n);
    std::vector<double> tmp(n, 0.0), phi0(n, 0.0), rt(n, 0.0);
    std::vector<int> flag(n, 0);
    applyBoundaryConditions(Gc.data(), s);
    applyVelocityBoundaryConditions(u.data(), v.data(), s);
    double* pG = Gc.data();
    double* pGn = Gnew.data();
    double* pT = tmp.data();
    for (int step = 0; step < n_steps; ++step) {
        rk3TimeStep(pG, pGn, G1.data(), G2.data(), Grhs.data(), u.data(), v.data(), s);
        double* t = pG; pG = pGn; pGn = t;
        if (s.enable_reinit && step > 0 && step % s.reinit_interval == 0) {
            reinitializeWithSwap(&pG, &pT, phi0.data(), rt.data(), flag.data(), s);
        }
    }
    std::memcpy(G, pG, sizeof(double) * n);
}


/* The reference's 2D known-answer case (src/main.cpp:198-371 run with
 * -t zalesak; logs in Local_code/level-set_MPI_2D/log/<n>x<n>.log): Zalesak's
 * slotted disk rotated once about (0.5, 0.5) on an n x n grid of [0,1]^2
 * (dx = 1/(n-1)), periodic X, zero-gradient Y, S_L = 0, no reinit, dt from
 * calculateTimeStep with u_const = 1 and the final-step clip.  Outputs: the
 * ghosted initial G (after the boundary fill), u, v, the final G, and
 * out = {L2 error, initial area, final area, steps}. */
void ref2d_zalesak(int n, double* G0_out, double* u_out, double* v_out, double* G_final, double* out) {
    SimParams s = initDefaultParams();
    s.nx = n; s.ny = n;
    s.nghost = 3;
    s.nx_total = n + 6; s.ny_total = n + 6;
    s.dx = (DOMAIN_X_MAX - DOMAIN_X_MIN) / (n - 1);
    s.dy = (DOMAIN_Y_MAX - DOMAIN_Y_MIN) / (n - 1);
    setupMPIDomainDecomposition(s, 0, 1);
    s.s_l = S_L;
    s.u_const = U_CONST;
    s.v_const = V_CONST;
    s.t_final = T_FINAL;
    s.cfl = CFL;
    s.enable_reinit = false;
    s.dt = calculateTimeStep(s);
    const size_t tot = (size_t)s.nx_total * s.local_ny_total;
    std::vector<double> G(tot, 0.0), Gnew(tot, 0.0), G1(tot, 0.0), G2(tot, 0.0), Grhs(tot, 0.0), Gi(tot, 0.0),
        u(tot, 0.0), v(tot, 0.0);
    initZalesakTestCase(G.data(), u.data(), v.data(), s);
    applyBoundaryConditions(G.data(), s);
    applyVelocityBoundaryConditions(u.data(), v.data(), s);
    copyInitialField(G.data(), Gi.data(), (int)tot);
    const double area0 = computeInterfaceArea(G.data(), s);
    if (G0_out) std::memcpy(G0_out, G.data(), sizeof(double) * tot);
    if (u_out) std::memcpy(u_out, u.data(), sizeof(double) * tot);
    if (v_out) std::memcpy(v_out, v.data(), sizeof(double) * tot);
    double* pG = G.data();
    double* pGn = Gnew.data();
    double current_time = 0.0;
    int step = 0;
    const int max_steps = (int)(s.t_final / s.dt) + 100;
    while (current_time < s.t_final && step < max_steps) {
        if (current_time + s.dt > s.t_final) s.dt = s.t_final - current_time;
        rk3TimeStep(pG, pGn, G1.data(), G2.data(), Grhs.data(), u.data(), v.data(), s);
        double* t = pG; pG = pGn; pGn = t;
        current_time += s.dt;
        step++;
    }
    out[0] = computeL2Error(pG, Gi.data(), s);
    out[1] = area0;
    out[2] = computeInterfaceArea(pG, s);
    out[3] = (double)step;
    if (G_final) std::memcpy(G_final, pG, sizeof(double) * tot);
}

/* the reference's binary dump writer on a ghosted array (io.h) */
int ref2d_save_binary(const orc_params* p, const double* G, const char* path) {
    SimParams s = to_sim(p);
    return saveFieldBinary(path, G, s) ? 0 : 1;
}

}  // extern "C"
