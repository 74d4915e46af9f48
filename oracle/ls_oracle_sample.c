/*
 * ls_oracle_sample.c -- CPU restatement of the reference's sample surface
 * (juhoon196/Level-set-method-code, sample/field.cpp and
 * sample/weno5_rk3.cpp): the 2D Field2D solver with the local Lax-Friedrichs
 * G-equation Hamiltonian, anchored + periodic boundaries and the first-order
 * reinitialisation.  Test infrastructure ONLY: tests/, __graft_entry__.smoke()
 * and bench.py's CPU legs use it as the checker of the CUDA kernels; the
 * product library never links or calls it.
 *
 * Arrays are flat row-major [ny+6][nx+6] doubles, the element order of
 * Field2D::data (sample/field.hpp:8).  Every floating-point expression keeps
 * the reference's operation order; with -ffp-contract=off the results equal
 * the reference's compiled sources bit for bit (tests/test_oracle_sample.py,
 * against oracle/_ref/libref_sample.so and tests/golden/).  std::pow(x, 2)
 * appears here as x * x: gcc folds the reference's pow(x, 2.0) to that
 * single rounded product.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

#define SEPS 1e-6  /* EPSILON, sample/weno5_rk3.cpp:8 */

#define AT(a, j, i) (a)[(size_t)(j) * (size_t)nxT + (size_t)(i)]

/* beta, sample/weno5_rk3.cpp:11-14 (second term (f0 - 4 f1 + 3 f2)^2) */
static inline double s_beta(double f0, double f1, double f2) {
    double a = f0 - 2.0 * f1 + f2;
    double b = f0 - 4.0 * f1 + 3.0 * f2;
    return (13.0 / 12.0) * (a * a) + (1.0 / 4.0) * (b * b);
}

/* weno5_left, sample/weno5_rk3.cpp:17-32 */
static inline double s_left(double v0, double v1, double v2, double v3, double v4) {
    double b0 = s_beta(v0, v1, v2);
    double b1 = s_beta(v1, v2, v3);
    double b2 = s_beta(v2, v3, v4);
    double a0 = 0.1 / ((SEPS + b0) * (SEPS + b0));
    double a1 = 0.6 / ((SEPS + b1) * (SEPS + b1));
    double a2 = 0.3 / ((SEPS + b2) * (SEPS + b2));
    double sum = a0 + a1 + a2;
    double w0 = a0 / sum, w1 = a1 / sum, w2 = a2 / sum;
    return w0 * (2.0 * v0 - 7.0 * v1 + 11.0 * v2) / 6.0
         + w1 * (-v1 + 5.0 * v2 + 2.0 * v3) / 6.0
         + w2 * (2.0 * v2 + 5.0 * v3 - v4) / 6.0;
}

/* weno5_right, sample/weno5_rk3.cpp:35-50, called with its arguments in
 * the order weno5_deriv_x/y pass them (descending index). */
static inline double s_right(double v0, double v1, double v2, double v3, double v4) {
    double b0 = s_beta(v4, v3, v2);
    double b1 = s_beta(v3, v2, v1);
    double b2 = s_beta(v2, v1, v0);
    double a0 = 0.1 / ((SEPS + b0) * (SEPS + b0));
    double a1 = 0.6 / ((SEPS + b1) * (SEPS + b1));
    double a2 = 0.3 / ((SEPS + b2) * (SEPS + b2));
    double sum = a0 + a1 + a2;
    double w0 = a0 / sum, w1 = a1 / sum, w2 = a2 / sum;
    return w0 * (2.0 * v4 - 7.0 * v3 + 11.0 * v2) / 6.0
         + w1 * (-v3 + 5.0 * v2 + 2.0 * v1) / 6.0
         + w2 * (2.0 * v2 + 5.0 * v1 - v0) / 6.0;
}

static inline double smax(double a, double b) { return (a < b) ? b : a; }  /* std::max */
static inline double smin(double a, double b) { return (b < a) ? b : a; }  /* std::min */

/* compute_geqn_rhs, sample/weno5_rk3.cpp:91-145 (derivatives of
 * weno5_deriv_x/y :53-87).  u, v may be NULL: then the scalars uc, vc are
 * the (uniform) velocity. */
static void rhs_any(int nx, int ny, const double* G, const double* u, const double* v, double uc, double vc,
                    double* rhs, double dx, double dy, double S_L) {
    const int nxT = nx + 6, nyT = ny + 6;
    memset(rhs, 0, sizeof(double) * (size_t)nxT * nyT);
#pragma omp parallel for
    for (int j = 3; j <= ny + 2; ++j) {
        for (int i = 3; i <= nx + 2; ++i) {
            double Gdxm = (s_left(AT(G, j, i - 2), AT(G, j, i - 1), AT(G, j, i), AT(G, j, i + 1), AT(G, j, i + 2))
                         - s_left(AT(G, j, i - 3), AT(G, j, i - 2), AT(G, j, i - 1), AT(G, j, i), AT(G, j, i + 1))) / dx;
            double Gdxp = (s_right(AT(G, j, i + 3), AT(G, j, i + 2), AT(G, j, i + 1), AT(G, j, i), AT(G, j, i - 1))
                         - s_right(AT(G, j, i + 2), AT(G, j, i + 1), AT(G, j, i), AT(G, j, i - 1), AT(G, j, i - 2))) / dx;
            double Gdym = (s_left(AT(G, j - 2, i), AT(G, j - 1, i), AT(G, j, i), AT(G, j + 1, i), AT(G, j + 2, i))
                         - s_left(AT(G, j - 3, i), AT(G, j - 2, i), AT(G, j - 1, i), AT(G, j, i), AT(G, j + 1, i))) / dy;
            double Gdyp = (s_right(AT(G, j + 3, i), AT(G, j + 2, i), AT(G, j + 1, i), AT(G, j, i), AT(G, j - 1, i))
                         - s_right(AT(G, j + 2, i), AT(G, j + 1, i), AT(G, j, i), AT(G, j - 1, i), AT(G, j - 2, i))) / dy;
            double uu = u ? AT(u, j, i) : uc;
            double vv = v ? AT(v, j, i) : vc;
            double Gdx_mean = 0.5 * (Gdxm + Gdxp);
            double Gdy_mean = 0.5 * (Gdym + Gdyp);
            double transport = uu * Gdx_mean + vv * Gdy_mean;
            double propagation = S_L * sqrt(Gdx_mean * Gdx_mean + Gdy_mean * Gdy_mean);
            double s_xm = uu - S_L * Gdxm / sqrt(Gdxm * Gdxm + Gdym * Gdym + 1e-14);
            double s_xp = uu - S_L * Gdxp / sqrt(Gdxp * Gdxp + Gdyp * Gdyp + 1e-14);
            double alpha_x = smax(fabs(s_xm), fabs(s_xp));
            double s_ym = vv - S_L * Gdym / sqrt(Gdxm * Gdxm + Gdym * Gdym + 1e-14);
            double s_yp = vv - S_L * Gdyp / sqrt(Gdxp * Gdxp + Gdyp * Gdyp + 1e-14);
            double alpha_y = smax(fabs(s_ym), fabs(s_yp));
            double alpha = smax(alpha_x, alpha_y);
            double diss_x = alpha * (Gdxp - Gdxm) * 0.5;
            double diss_y = alpha * (Gdyp - Gdym) * 0.5;
            double H = transport - propagation - (diss_x + diss_y);
            AT(rhs, j, i) = -H;
        }
    }
}

void orcs_rhs(int nx, int ny, const double* G, const double* u, const double* v, double* rhs, double dx, double dy,
              double S_L) {
    rhs_any(nx, ny, G, u, v, 0.0, 0.0, rhs, dx, dy, S_L);
}

/* Field2D::apply_periodic, sample/field.cpp:16-34 */
void orcs_apply_periodic(int nx, int ny, double* d) {
    const int nxT = nx + 6, nyT = ny + 6;
    for (int j = 0; j < nyT; ++j)
        for (int k = 0; k < 3; ++k) {
            AT(d, j, k) = AT(d, j, nx + k);
            AT(d, j, nx + 3 + k) = AT(d, j, 3 + k);
        }
    for (int i = 0; i < nxT; ++i)
        for (int k = 0; k < 3; ++k) {
            AT(d, k, i) = AT(d, ny + k, i);
            AT(d, ny + 3 + k, i) = AT(d, 3 + k, i);
        }
}

/* Field2D::apply_anchored_bc, sample/field.cpp:37-63 (also the boundary
 * pass of Field2D::reinitialize, :107-126) */
void orcs_apply_anchored_bc(int nx, int ny, double* d, const double* init) {
    const int nxT = nx + 6, nyT = ny + 6;
    for (int i = 0; i < nxT; ++i) {
        AT(d, 3, i) = AT(init, 3, i);
        AT(d, 2, i) = 2.0 * AT(d, 3, i) - AT(d, 4, i);
        AT(d, 1, i) = 2.0 * AT(d, 2, i) - AT(d, 3, i);
        AT(d, 0, i) = 2.0 * AT(d, 1, i) - AT(d, 2, i);
    }
    for (int i = 0; i < nxT; ++i) {
        AT(d, ny + 2, i) = 2.0 * AT(d, ny + 1, i) - AT(d, ny, i);
        AT(d, ny + 3, i) = 2.0 * AT(d, ny + 2, i) - AT(d, ny + 1, i);
        AT(d, ny + 4, i) = 2.0 * AT(d, ny + 3, i) - AT(d, ny + 2, i);
        AT(d, ny + 5, i) = 2.0 * AT(d, ny + 4, i) - AT(d, ny + 3, i);
    }
    for (int j = 0; j < nyT; ++j) {
        AT(d, j, 2) = 2.0 * AT(d, j, 3) - AT(d, j, 4);
        AT(d, j, 1) = 2.0 * AT(d, j, 2) - AT(d, j, 3);
        AT(d, j, 0) = 2.0 * AT(d, j, 1) - AT(d, j, 2);
        AT(d, j, nx + 3) = 2.0 * AT(d, j, nx + 2) - AT(d, j, nx + 1);
        AT(d, j, nx + 4) = 2.0 * AT(d, j, nx + 3) - AT(d, j, nx + 2);
        AT(d, j, nx + 5) = 2.0 * AT(d, j, nx + 4) - AT(d, j, nx + 3);
    }
}

/* RK3_step, sample/weno5_rk3.cpp:148-188 (G1, G2 start as zero fields) */
static void rk3_any(int nx, int ny, double* G, const double* u, const double* v, double uc, double vc, double dx,
                    double dy, double dt, double S_L, const double* init) {
    const int nxT = nx + 6, nyT = ny + 6;
    const size_t n = (size_t)nxT * nyT;
    double* G1 = calloc(n, sizeof(double));
    double* G2 = calloc(n, sizeof(double));
    double* rhs = calloc(n, sizeof(double));
    rhs_any(nx, ny, G, u, v, uc, vc, rhs, dx, dy, S_L);
    for (int j = 3; j <= ny + 2; ++j)
        for (int i = 3; i <= nx + 2; ++i) AT(G1, j, i) = AT(G, j, i) + dt * AT(rhs, j, i);
    orcs_apply_anchored_bc(nx, ny, G1, init);
    orcs_apply_periodic(nx, ny, G1);
    rhs_any(nx, ny, G1, u, v, uc, vc, rhs, dx, dy, S_L);
    for (int j = 3; j <= ny + 2; ++j)
        for (int i = 3; i <= nx + 2; ++i)
            AT(G2, j, i) = 0.75 * AT(G, j, i) + 0.25 * (AT(G1, j, i) + dt * AT(rhs, j, i));
    orcs_apply_anchored_bc(nx, ny, G2, init);
    orcs_apply_periodic(nx, ny, G2);
    rhs_any(nx, ny, G2, u, v, uc, vc, rhs, dx, dy, S_L);
    for (int j = 3; j <= ny + 2; ++j)
        for (int i = 3; i <= nx + 2; ++i)
            AT(G, j, i) = (1.0 / 3.0) * AT(G, j, i) + (2.0 / 3.0) * (AT(G2, j, i) + dt * AT(rhs, j, i));
    orcs_apply_anchored_bc(nx, ny, G, init);
    orcs_apply_periodic(nx, ny, G);
    free(G1);
    free(G2);
    free(rhs);
}

void orcs_rk3_step(int nx, int ny, double* G, const double* u, const double* v, double dx, double dy, double dt,
                   double S_L, const double* init) {
    rk3_any(nx, ny, G, u, v, 0.0, 0.0, dx, dy, dt, S_L, init);
}

/* compute_first_order_upwind, sample/first_order_upwind.cpp:6-69: the
 * first-order upwind G-equation step (Jacobi, in place on G).  The loops run
 * over j = 3 .. ny+3 and i = 3 .. nx+3 inclusive (the reference's bounds
 * `<= ny-3` / `<= nx-3` on the ghosted sizes), which includes the first
 * ghost row and column on the high side. */
void orcs_first_order_upwind(int nx, int ny, double* G, const double* u, const double* v, double dx, double dy,
                             double dt, double S_L) {
    const int nxT = nx + 6, nyT = ny + 6;
    const size_t n = (size_t)nxT * nyT;
    const double EPS = 1e-10;
    double* Gn = malloc(n * sizeof(double));
    memcpy(Gn, G, n * sizeof(double));
    for (int j = 3; j <= nyT - 3; ++j)
        for (int i = 3; i <= nxT - 3; ++i) {
            const double Gx_mns = (AT(G, j, i) - AT(G, j, i - 1)) / dx;
            const double Gx_pls = (AT(G, j, i + 1) - AT(G, j, i)) / dx;
            const double Gy_mns = (AT(G, j, i) - AT(G, j - 1, i)) / dy;
            const double Gy_pls = (AT(G, j + 1, i) - AT(G, j, i)) / dy;
            const double dG_dx = 0.5 * (Gx_mns + Gx_pls);
            const double dG_dy = 0.5 * (Gy_mns + Gy_pls);
            const double mag_sq = dG_dx * dG_dx + dG_dy * dG_dy;
            double u_first, v_first;
            if (mag_sq > EPS * EPS) {
                const double mag = sqrt(mag_sq);
                u_first = AT(u, j, i) - S_L * dG_dx / mag;
                v_first = AT(v, j, i) - S_L * dG_dy / mag;
            } else {
                u_first = AT(u, j, i);
                v_first = AT(v, j, i);
            }
            const double a_pls = smax(u_first, 0.0), a_mns = smin(u_first, 0.0);
            const double b_pls = smax(v_first, 0.0), b_mns = smin(v_first, 0.0);
            AT(Gn, j, i) = AT(G, j, i) - dt * (a_pls * Gx_mns + a_mns * Gx_pls + b_pls * Gy_mns + b_mns * Gy_pls);
        }
    for (int j = 3; j <= nyT - 3; ++j)
        for (int i = 3; i <= nxT - 3; ++i) AT(G, j, i) = AT(Gn, j, i);
    free(Gn);
}

/* Field2D::reinitialize, sample/field.cpp:66-129 */
void orcs_reinitialize(int nx, int ny, double* G, const double* init, double dx, double dy, int iters) {
    const int nxT = nx + 6, nyT = ny + 6;
    const size_t n = (size_t)nxT * nyT;
    const double dtau = 0.2 * smin(dx, dy);
    double* phi = malloc(n * sizeof(double));
    double* rhs = malloc(n * sizeof(double));
    memcpy(phi, G, n * sizeof(double));
    for (int it = 0; it < iters; ++it) {
        memset(rhs, 0, n * sizeof(double));
#pragma omp parallel for
        for (int j = 3; j <= ny + 2; ++j) {
            for (int i = 3; i <= nx + 2; ++i) {
                double g0 = AT(init, j, i);
                double s = g0 / sqrt(g0 * g0 + dx * dx);
                double dGdx_pos = (AT(phi, j, i) - AT(phi, j, i - 1)) / dx;
                double dGdx_neg = (AT(phi, j, i + 1) - AT(phi, j, i)) / dx;
                double dGdy_pos = (AT(phi, j, i) - AT(phi, j - 1, i)) / dy;
                double dGdy_neg = (AT(phi, j + 1, i) - AT(phi, j, i)) / dy;
                double grad;
                if (s > 0.0) {
                    double px = smax(smax(dGdx_pos, 0.0), -smin(dGdx_neg, 0.0));
                    double py = smax(smax(dGdy_pos, 0.0), -smin(dGdy_neg, 0.0));
                    grad = sqrt(px * px + py * py);
                } else {
                    double qx = smax(smax(-dGdx_pos, 0.0), smin(dGdx_neg, 0.0));
                    double qy = smax(smax(-dGdy_pos, 0.0), smin(dGdy_neg, 0.0));
                    grad = sqrt(qx * qx + qy * qy);
                }
                AT(rhs, j, i) = -s * (grad - 1.0);
            }
        }
        for (int j = 3; j <= ny + 2; ++j)
            for (int i = 3; i <= nx + 2; ++i) AT(phi, j, i) += dtau * AT(rhs, j, i);
        orcs_apply_anchored_bc(nx, ny, phi, init);
    }
    memcpy(G, phi, n * sizeof(double));
    free(phi);
    free(rhs);
}

/* The time loop of sample/main.cpp:126-148 for n_steps steps from time *t,
 * with the spatially uniform forced velocity of :131-136. */
void orcs_run(int nx, int ny, int n_steps, double* G, const double* init, double dx, double dy, double dt,
              double S_L, double u0, double v0, double eps_u, double eps_v, int freq, double* t) {
    double tt = *t;
    for (int s = 0; s < n_steps; ++s) {
        orcs_apply_anchored_bc(nx, ny, G, init);
        orcs_apply_periodic(nx, ny, G);
        double uc = u0 + eps_u * v0 * cos(freq * 2 * M_PI * (tt));
        double vc = v0 + eps_v * v0 * cos(freq * 2 * M_PI * (tt));
        rk3_any(nx, ny, G, NULL, NULL, uc, vc, dx, dy, dt, S_L, init);
        orcs_apply_periodic(nx, ny, G);
        orcs_apply_anchored_bc(nx, ny, G, init);
        tt += dt;
    }
    *t = tt;
}
