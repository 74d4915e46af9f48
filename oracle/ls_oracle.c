/*
 * ls_oracle.c -- CPU restatement of the reference's G-equation level-set hot
 * path, used ONLY as the checker of the CUDA implementation (tests/,
 * __graft_entry__.smoke(), and the cpu_baseline / reference legs of bench.py).
 * It is never linked into, or called by, the product library.
 *
 * What it restates (reference = juhoon196/Level-set-method-code):
 *   3D: Local_code/level-set_MPI_3D/include/{weno5,rk3,boundary,reinitialization,io}.h
 *   2D: Local_code/level-set_MPI_2D/include/{weno5,rk3,boundary,reinitialization,io}.h
 * Each function cites the lines it follows.  The floating-point operations
 * are written in the reference's order and the file is compiled with
 * -ffp-contract=off, so results are bit-identical to the reference built the
 * same way (pinned by tests/test_oracle.py against oracle/_ref and the
 * committed golden fixtures).
 *
 * Additions the reference does not have (restated from the formulas the
 * reference uses, and marked as such):
 *   - an optional per-cell flame-speed field S_L(x): the reference's
 *     params.s_l read at the cell index instead (rk3.h:54-77 with
 *     s_l -> sl[index], including the s_l > epsilon gate per cell);
 *   - a field-max CFL time step (config.h:272-293 with the velocity maximum
 *     taken over the grid instead of the constant velocities).
 *
 * Layout: ghosted row-major, index = k*nxT*nyT + j*nxT + i with 3 ghost
 * cells per side (config.h:301-306).  Cell loops run in parallel with OpenMP
 * over the outermost index; every cell is independent, so the thread count
 * does not change any bit.  Reductions run sequentially in the reference's
 * loop order.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "oracle_params.h"

#define NG 3
#define WENO_EPS 1.0e-6

typedef struct {
    int nx, ny, nz;      /* interior */
    int nxT, nyT, nzT;   /* ghosted */
    long sy, sz;         /* strides */
} grid_t;

static grid_t grid3(const orc_params* p) {
    grid_t g;
    g.nx = p->nx; g.ny = p->ny; g.nz = p->nz;
    g.nxT = p->nx + 2 * NG; g.nyT = p->ny + 2 * NG; g.nzT = p->nz + 2 * NG;
    g.sy = g.nxT; g.sz = (long)g.nxT * g.nyT;
    return g;
}

static grid_t grid2(const orc_params* p) {
    grid_t g;
    g.nx = p->nx; g.ny = p->ny; g.nz = 1;
    g.nxT = p->nx + 2 * NG; g.nyT = p->ny + 2 * NG; g.nzT = 1;
    g.sy = g.nxT; g.sz = 0;
    return g;
}

/* ---------------------------------------------------------------------------
 * Decision tape (3D; an addition for checking the discrete adjoint, not in
 * the reference).  The forward map has switching decisions: the upwind
 * branch u_eff >= 0 per axis (weno5.h:99), the Godunov one-sided choice per
 * axis of the pseudo-step (weno5.h:202-248), the crossing flags of
 * computeInterfaceCrossings3D (reinitialization.h:46-89) and the stability
 * test (:95-130).  Mode 1 records them per interior cell while computing as
 * usual (same bits); mode 2 replays recorded ones in place of the tests, so a
 * perturbed run follows the base run's branches and is a smooth function of
 * its inputs: the map whose derivative the discrete adjoint computes.
 *   stage  [calls of rhs3][cells]: bit a = axis a right-biased (u_eff < 0)
 *   pseudo [pseudo-steps][cells]:  bits 2a..2a+1 = axis a choice (0 none, 1
 *          the backward difference, 2 the forward one), bit 6 = stable
 *   flags  [reinitialisations][cells]: the crossing flags
 * ------------------------------------------------------------------------- */
static struct {
    int mode;                 /* 0 off, 1 record, 2 replay */
    unsigned char *stage, *pseudo, *flags;
    long n_stage, n_pseudo, n_flags;  /* capacities in calls */
    long c_stage, c_pseudo, c_flags;  /* calls so far */
    int overflow;
} tape;

void orc_tape_set(int mode, unsigned char* stage, long n_stage, unsigned char* pseudo, long n_pseudo,
                  unsigned char* flags, long n_flags) {
    tape.mode = mode;
    tape.stage = stage; tape.pseudo = pseudo; tape.flags = flags;
    tape.n_stage = n_stage; tape.n_pseudo = n_pseudo; tape.n_flags = n_flags;
    tape.c_stage = tape.c_pseudo = tape.c_flags = 0;
    tape.overflow = 0;
}

/* calls used so far (stage, pseudo-step, reinitialisation) and the overflow flag */
void orc_tape_counts(long* out) {
    out[0] = tape.c_stage; out[1] = tape.c_pseudo; out[2] = tape.c_flags; out[3] = tape.overflow;
}

/* The tape row of the next call of a kind (NULL when off or full). */
static unsigned char* tape_row(unsigned char* base, long* used, long cap, long cells) {
    if (tape.mode == 0) return NULL;
    if (*used >= cap) { tape.overflow = 1; return NULL; }
    return base + (*used)++ * cells;
}

/* ---------------------------------------------------------------------------
 * WENO-5 reconstruction, weno5.h:28-81 (3D) == weno5.h:39-122 (2D).
 * beta uses the reference's non-standard second term 1/4 (v[k+2]-v[k])^2 for
 * all three sub-stencils, and weights d_k / (eps + beta_k)^2.
 * ------------------------------------------------------------------------- */
static inline double smooth_beta(double a, double b, double c) {
    /* triple (v[k], v[k+1], v[k+2]) = (a, b, c):  weno5.h:29-30 */
    double d2 = c - 2.0 * b + a;
    return (13.0 / 12.0) * d2 * d2 + 0.25 * (c - a) * (c - a);
}

/* weno5_left (weno5.h:39-58): value at i+1/2 from v = G[i-2..i+2] */
static inline double weno_left(const double v[5]) {
    double b0 = smooth_beta(v[0], v[1], v[2]);
    double b1 = smooth_beta(v[1], v[2], v[3]);
    double b2 = smooth_beta(v[2], v[3], v[4]);
    double a0 = 0.1 / ((WENO_EPS + b0) * (WENO_EPS + b0));
    double a1 = 0.6 / ((WENO_EPS + b1) * (WENO_EPS + b1));
    double a2 = 0.3 / ((WENO_EPS + b2) * (WENO_EPS + b2));
    double s = a0 + a1 + a2;
    double w0 = a0 / s, w1 = a1 / s, w2 = a2 / s;
    double p0 = (2.0 * v[0] - 7.0 * v[1] + 11.0 * v[2]) / 6.0;
    double p1 = (-v[1] + 5.0 * v[2] + 2.0 * v[3]) / 6.0;
    double p2 = (2.0 * v[2] + 5.0 * v[3] - v[4]) / 6.0;
    return w0 * p0 + w1 * p1 + w2 * p2;
}

/* weno5_right (weno5.h:60-81): value at i-1/2 from v = G[i-2..i+2]; the
 * smoothness indicators are taken on the mirrored stencil. */
static inline double weno_right(const double v[5]) {
    double b0 = smooth_beta(v[4], v[3], v[2]);
    double b1 = smooth_beta(v[3], v[2], v[1]);
    double b2 = smooth_beta(v[2], v[1], v[0]);
    double a0 = 0.3 / ((WENO_EPS + b0) * (WENO_EPS + b0));
    double a1 = 0.6 / ((WENO_EPS + b1) * (WENO_EPS + b1));
    double a2 = 0.1 / ((WENO_EPS + b2) * (WENO_EPS + b2));
    double s = a0 + a1 + a2;
    double w0 = a0 / s, w1 = a1 / s, w2 = a2 / s;
    double p0 = (11.0 * v[2] - 7.0 * v[3] + 2.0 * v[4]) / 6.0;
    double p1 = (2.0 * v[1] + 5.0 * v[2] - v[3]) / 6.0;
    double p2 = (-v[0] + 5.0 * v[1] + 2.0 * v[2]) / 6.0;
    return w0 * p0 + w1 * p1 + w2 * p2;
}

/* Upwind WENO-5 derivative along one axis, weno5.h:90-122 (x), :127 (y),
 * :164 (z): c points at the cell, s is the stride along the axis.
 * Branch on vel >= 0 (not > 0), weno5.h:99. */
static inline double weno_deriv_b(const double* c, long s, int left, double h) {
    double v[5] = {c[-2 * s], c[-s], c[0], c[s], c[2 * s]};
    if (left) {
        double vl[5] = {c[-3 * s], c[-2 * s], c[-s], c[0], c[s]};
        double gl = weno_left(vl);
        double gr = weno_left(v);
        return (gr - gl) / h;
    } else {
        double vr[5] = {c[-s], c[0], c[s], c[2 * s], c[3 * s]};
        double gl = weno_right(v);
        double gr = weno_right(vr);
        return (gr - gl) / h;
    }
}

static inline double weno_deriv(const double* c, long s, double vel, double h) {
    return weno_deriv_b(c, s, vel >= 0.0, h);
}

/* ---------------------------------------------------------------------------
 * Spatial operator: computeRHS3D (rk3.h:31-81), computeRHS (2D rk3.h:54-98).
 * rhs = -(u_eff * Dx + v_eff * Dy [+ w_eff * Dz]) on interior cells, with
 * u_eff = u - s_l * gx / |grad G|, gx central, |grad G| = sqrt(sum g^2 + eps),
 * only when s_l > epsilon.  sl (nullable) is the per-cell flame speed.
 * ------------------------------------------------------------------------- */
static void rhs3(const orc_params* p, const grid_t* g, const double* G, double* R,
                 const double* u, const double* v, const double* w, const double* sl) {
    int k;
    unsigned char* trow = tape_row(tape.stage, &tape.c_stage, tape.n_stage, (long)g->nx * g->ny * g->nz);
    const int tmode = trow ? tape.mode : 0;
#pragma omp parallel for schedule(static)
    for (k = NG; k < g->nz + NG; k++) {
        for (int j = NG; j < g->ny + NG; j++) {
            for (int i = NG; i < g->nx + NG; i++) {
                long id = k * g->sz + j * g->sy + i;
                const double* c = G + id;
                double s_l = sl ? sl[id] : p->s_l;
                double gx = 0.0, gy = 0.0, gz = 0.0, gm = 1.0;
                if (s_l > p->epsilon) {
                    gx = (c[1] - c[-1]) / (2.0 * p->dx);
                    gy = (c[g->sy] - c[-g->sy]) / (2.0 * p->dy);
                    gz = (c[g->sz] - c[-g->sz]) / (2.0 * p->dz);
                    gm = sqrt(gx * gx + gy * gy + gz * gz + p->epsilon);
                }
                double ue = u[id] - s_l * gx / gm;
                double ve = v[id] - s_l * gy / gm;
                double we = w[id] - s_l * gz / gm;
                int lx = ue >= 0.0, ly = ve >= 0.0, lz = we >= 0.0;
                if (tmode) {
                    unsigned char* t = trow + ((long)(k - NG) * g->ny + (j - NG)) * g->nx + (i - NG);
                    if (tmode == 1) *t = (unsigned char)(!lx | (!ly << 1) | (!lz << 2));
                    else { lx = !(*t & 1); ly = !(*t & 2); lz = !(*t & 4); }
                }
                double dgx = weno_deriv_b(c, 1, lx, p->dx);
                double dgy = weno_deriv_b(c, g->sy, ly, p->dy);
                double dgz = weno_deriv_b(c, g->sz, lz, p->dz);
                R[id] = -(ue * dgx + ve * dgy + we * dgz);
            }
        }
    }
}

static void rhs2(const orc_params* p, const grid_t* g, const double* G, double* R,
                 const double* u, const double* v, const double* sl) {
    int j;
#pragma omp parallel for schedule(static)
    for (j = NG; j < g->ny + NG; j++) {
        for (int i = NG; i < g->nx + NG; i++) {
            long id = j * g->sy + i;
            const double* c = G + id;
            double s_l = sl ? sl[id] : p->s_l;
            double gx = 0.0, gy = 0.0, gm = 1.0;
            if (s_l > p->epsilon) {
                gx = (c[1] - c[-1]) / (2.0 * p->dx);
                gy = (c[g->sy] - c[-g->sy]) / (2.0 * p->dy);
                gm = sqrt(gx * gx + gy * gy + p->epsilon);
            }
            double ue = u[id] - s_l * gx / gm;
            double ve = v[id] - s_l * gy / gm;
            double dgx = weno_deriv(c, 1, ue, p->dx);
            double dgy = weno_deriv(c, g->sy, ve, p->dy);
            R[id] = -(ue * dgx + ve * dgy);
        }
    }
}

/* ---------------------------------------------------------------------------
 * Boundary fill.
 * 3D, applyBoundaryConditions3D (boundary.h:250-261): periodic Y through the
 * one-rank self exchange (boundary.h:37-138: bottom ghosts <- last 3 interior
 * rows, top ghosts <- first 3, over all i and k), then periodic X over all
 * (j, k) (:144-163), then periodic Z over all (i, j) (:169-188).
 * 2D, applyBoundaryConditions (2D boundary.h:217-229): Y exchange when Y is
 * periodic, periodic X over all j (:98-114), zero-gradient Y at the ends when
 * it is not (:126-147).
 * ------------------------------------------------------------------------- */
static void bc3(const grid_t* g, double* G) {
    int k;
#pragma omp parallel for schedule(static)
    for (k = 0; k < g->nzT; k++) {
        for (int gg = 0; gg < NG; gg++) {
            memcpy(G + k * g->sz + gg * g->sy, G + k * g->sz + (g->ny + gg) * g->sy,
                   sizeof(double) * g->nxT);
            memcpy(G + k * g->sz + (g->ny + NG + gg) * g->sy, G + k * g->sz + (NG + gg) * g->sy,
                   sizeof(double) * g->nxT);
        }
    }
#pragma omp parallel for schedule(static)
    for (k = 0; k < g->nzT; k++) {
        for (int j = 0; j < g->nyT; j++) {
            double* row = G + k * g->sz + j * g->sy;
            for (int gg = 0; gg < NG; gg++) {
                row[gg] = row[g->nx + gg];
                row[g->nx + NG + gg] = row[NG + gg];
            }
        }
    }
    int j;
#pragma omp parallel for schedule(static)
    for (j = 0; j < g->nyT; j++) {
        for (int gg = 0; gg < NG; gg++) {
            memcpy(G + gg * g->sz + j * g->sy, G + (g->nz + gg) * g->sz + j * g->sy,
                   sizeof(double) * g->nxT);
            memcpy(G + (g->nz + NG + gg) * g->sz + j * g->sy, G + (NG + gg) * g->sz + j * g->sy,
                   sizeof(double) * g->nxT);
        }
    }
}

static void bc2(const orc_params* p, const grid_t* g, double* G) {
    if (p->periodic_y) {
        for (int gg = 0; gg < NG; gg++) {
            memcpy(G + gg * g->sy, G + (g->ny + gg) * g->sy, sizeof(double) * g->nxT);
            memcpy(G + (g->ny + NG + gg) * g->sy, G + (NG + gg) * g->sy, sizeof(double) * g->nxT);
        }
    }
    for (int j = 0; j < g->nyT; j++) {
        double* row = G + j * g->sy;
        for (int gg = 0; gg < NG; gg++) {
            row[gg] = row[g->nx + gg];
            row[g->nx + NG + gg] = row[NG + gg];
        }
    }
    if (!p->periodic_y) {
        for (int i = 0; i < g->nxT; i++) {
            double bot = G[NG * g->sy + i];
            double top = G[(g->ny + NG - 1) * g->sy + i];
            for (int gg = 0; gg < NG; gg++) {
                G[gg * g->sy + i] = bot;
                G[(g->ny + NG + gg) * g->sy + i] = top;
            }
        }
    }
}

/* ---------------------------------------------------------------------------
 * TVD RK3 (Shu-Osher), rk3Stage{1,2,3}_3D (rk3.h:87-121) and the 2D stages
 * (2D rk3.h:103-150): combinations over the WHOLE ghosted array (ghost rhs
 * entries stay 0), then the boundary fill after each stage (rk3.h:131-150).
 * ------------------------------------------------------------------------- */
static void stage_combine(int stage, long n, const double* Gn, const double* Gs, const double* R,
                          double* out, double dt) {
    long id;
    if (stage == 1) {
#pragma omp parallel for schedule(static)
        for (id = 0; id < n; id++) out[id] = Gn[id] + dt * R[id];
    } else if (stage == 2) {
#pragma omp parallel for schedule(static)
        for (id = 0; id < n; id++) out[id] = 0.75 * Gn[id] + 0.25 * Gs[id] + 0.25 * dt * R[id];
    } else {
        double a0 = 1.0 / 3.0, a2 = 2.0 / 3.0, b3 = 2.0 / 3.0;
#pragma omp parallel for schedule(static)
        for (id = 0; id < n; id++) out[id] = a0 * Gn[id] + a2 * Gs[id] + b3 * dt * R[id];
    }
}

static long total_of(const grid_t* g) { return (long)g->nxT * g->nyT * g->nzT; }

void orc3d_rk3_step(const orc_params* p, double* Gn, double* Gnew, double* G1, double* G2,
                    double* R, const double* u, const double* v, const double* w,
                    const double* sl) {
    grid_t g = grid3(p);
    long n = total_of(&g);
    rhs3(p, &g, Gn, R, u, v, w, sl);
    stage_combine(1, n, Gn, Gn, R, G1, p->dt);
    bc3(&g, G1);
    rhs3(p, &g, G1, R, u, v, w, sl);
    stage_combine(2, n, Gn, G1, R, G2, p->dt);
    bc3(&g, G2);
    rhs3(p, &g, G2, R, u, v, w, sl);
    stage_combine(3, n, Gn, G2, R, Gnew, p->dt);
    bc3(&g, Gnew);
}

void orc2d_rk3_step(const orc_params* p, double* Gn, double* Gnew, double* G1, double* G2,
                    double* R, const double* u, const double* v, const double* sl) {
    grid_t g = grid2(p);
    long n = total_of(&g);
    rhs2(p, &g, Gn, R, u, v, sl);
    stage_combine(1, n, Gn, Gn, R, G1, p->dt);
    bc2(p, &g, G1);
    rhs2(p, &g, G1, R, u, v, sl);
    stage_combine(2, n, Gn, G1, R, G2, p->dt);
    bc2(p, &g, G2);
    rhs2(p, &g, G2, R, u, v, sl);
    stage_combine(3, n, Gn, G2, R, Gnew, p->dt);
    bc2(p, &g, Gnew);
}

void orc3d_rhs(const orc_params* p, const double* G, double* R, const double* u, const double* v,
               const double* w, const double* sl) {
    grid_t g = grid3(p);
    rhs3(p, &g, G, R, u, v, w, sl);
}

void orc2d_rhs(const orc_params* p, const double* G, double* R, const double* u, const double* v,
               const double* sl) {
    grid_t g = grid2(p);
    rhs2(p, &g, G, R, u, v, sl);
}

void orc3d_apply_bc(const orc_params* p, double* G) {
    grid_t g = grid3(p);
    bc3(&g, G);
}

void orc2d_apply_bc(const orc_params* p, double* G) {
    grid_t g = grid2(p);
    bc2(p, &g, G);
}

/* ---------------------------------------------------------------------------
 * HCR-2 constrained reinitialisation.
 * 3D: reinitialization.h:24-228; 2D: 2D reinitialization.h:37-360.
 * ------------------------------------------------------------------------- */

/* computeInterfaceCrossings3D (reinitialization.h:46-89): flag bit per
 * neighbour with phi0_c * phi0_nb < 0 (1:-x 2:+x 4:-y 8:+y 16:-z 32:+z), and
 * r~ = phi0_c / sum(phi0 of flagged neighbours) if any and |sum| > 1e-15. */
static void crossings(const grid_t* g, int dim, const double* phi0, double* rt, int* flag) {
    int k;
    int nz = dim == 3 ? g->nz : 1;
    int k0 = dim == 3 ? NG : 0;
    long st[6] = {-1, 1, -g->sy, g->sy, -g->sz, g->sz};
    int nnb = 2 * dim;
    unsigned char* trow = dim == 3 ? tape_row(tape.flags, &tape.c_flags, tape.n_flags,
                                              (long)g->nx * g->ny * g->nz) : NULL;
    const int tmode = trow ? tape.mode : 0;
#pragma omp parallel for schedule(static)
    for (k = k0; k < k0 + nz; k++) {
        for (int j = NG; j < g->ny + NG; j++) {
            for (int i = NG; i < g->nx + NG; i++) {
                long id = k * g->sz + j * g->sy + i;
                double pc = phi0[id];
                double sum = 0.0;
                int cnt = 0, f = 0;
                rt[id] = 0.0;
                unsigned char* t = tmode ? trow + ((long)(k - NG) * g->ny + (j - NG)) * g->nx + (i - NG) : NULL;
                for (int n = 0; n < nnb; n++) {
                    double pn = phi0[id + st[n]];
                    int cross = tmode == 2 ? (*t >> n) & 1 : pc * pn < 0.0;
                    if (cross) { sum += pn; cnt++; f |= 1 << n; }
                }
                if (tmode == 1) *t = (unsigned char)f;
                flag[id] = f;
                if (cnt > 0 && fabs(sum) > 1e-15) rt[id] = pc / sum;
            }
        }
    }
}

/* Godunov first-order |grad phi| by sign(S): weno5_gradient_magnitude_3d
 * (weno5.h:202-248) / weno5_gradient_magnitude (2D weno5.h:234-267). */
static inline double godunov_axis(double dm, double dp, int pos) {
    double a, b;
    if (pos) { a = fmax(dm, 0.0); b = fmin(dp, 0.0); }
    else { a = fmin(dm, 0.0); b = fmax(dp, 0.0); }
    return fmax(a * a, b * b);
}

/* reinitStep3D (reinitialization.h:136-193) with checkStabilityConstraint3D
 * (:95-130): phi_new = phi + dtau * (-S (|grad phi| - 1) + F), where
 * F = beta (r~ sum(phi_n of flagged neighbours) - phi) / dx on flagged cells
 * whose sign and flagged neighbours' signs match phi0. */
static void reinit_step(const orc_params* p, const grid_t* g, int dim, const double* phin,
                        double* phinew, const double* phi0, const double* rt, const int* flag) {
    int k;
    int nz = dim == 3 ? g->nz : 1;
    int k0 = dim == 3 ? NG : 0;
    long st[6] = {-1, 1, -g->sy, g->sy, -g->sz, g->sz};
    int nnb = 2 * dim;
    double dtau = p->reinit_dtau;
    unsigned char* trow = dim == 3 ? tape_row(tape.pseudo, &tape.c_pseudo, tape.n_pseudo,
                                              (long)g->nx * g->ny * g->nz) : NULL;
    const int tmode = trow ? tape.mode : 0;
#pragma omp parallel for schedule(static)
    for (k = k0; k < k0 + nz; k++) {
        for (int j = NG; j < g->ny + NG; j++) {
            for (int i = NG; i < g->nx + NG; i++) {
                long id = k * g->sz + j * g->sy + i;
                double phi = phin[id];
                double ph0 = phi0[id];
                double S = ph0 / sqrt(ph0 * ph0 + p->dx * p->dx);
                const double* c = phin + id;
                int pos = S > 0.0;
                double gsq;
                unsigned char* t = tmode ? trow + ((long)(k - NG) * g->ny + (j - NG)) * g->nx + (i - NG) : NULL;
                if (tmode == 0) {
                    gsq = godunov_axis((c[0] - c[-1]) / p->dx, (c[1] - c[0]) / p->dx, pos)
                        + godunov_axis((c[0] - c[-g->sy]) / p->dy, (c[g->sy] - c[0]) / p->dy, pos);
                    if (dim == 3)
                        gsq = gsq + godunov_axis((c[0] - c[-g->sz]) / p->dz, (c[g->sz] - c[0]) / p->dz, pos);
                } else {
                    /* per axis: record which one-sided difference the Godunov
                     * maximum took (none when the selected term is zero), or
                     * use the recorded one; the sum is formed as above */
                    const double hh[3] = {p->dx, p->dy, p->dz};
                    const long ss[3] = {1, g->sy, g->sz};
                    double term3[3];
                    unsigned char code = tmode == 2 ? *t : 0;
                    for (int ax = 0; ax < 3; ax++) {
                        double dm = (c[0] - c[-ss[ax]]) / hh[ax], dp = (c[ss[ax]] - c[0]) / hh[ax];
                        int sel;
                        if (tmode == 1) {
                            double a, b;
                            if (pos) { a = fmax(dm, 0.0); b = fmin(dp, 0.0); }
                            else { a = fmin(dm, 0.0); b = fmax(dp, 0.0); }
                            sel = a * a >= b * b ? (a != 0.0 ? 1 : 0) : 2;
                            code |= (unsigned char)(sel << (2 * ax));
                        } else {
                            sel = (code >> (2 * ax)) & 3;
                        }
                        term3[ax] = sel == 1 ? dm * dm : (sel == 2 ? dp * dp : 0.0);
                    }
                    gsq = term3[0] + term3[1] + term3[2];
                    if (tmode == 1) *t = code;
                }
                double gm = sqrt(gsq);
                double term = -S * (gm - 1.0);
                double forcing = 0.0;
                int f = flag[id];
                if (f != 0) {
                    int stable = (phin[id] > 0.0) == (phi0[id] > 0.0);
                    for (int n = 0; n < nnb && stable; n++)
                        if (f & (1 << n))
                            if ((phin[id + st[n]] > 0.0) != (phi0[id + st[n]] > 0.0)) stable = 0;
                    if (tmode == 1) *t |= (unsigned char)(stable << 6);
                    if (tmode == 2) stable = (*t >> 6) & 1;
                    if (stable) {
                        double sum = 0.0;
                        for (int n = 0; n < nnb; n++)
                            if (f & (1 << n)) sum += phin[id + st[n]];
                        forcing = p->reinit_beta * (rt[id] * sum - phi) / p->dx;
                    }
                }
                phinew[id] = phi + dtau * (term + forcing);
            }
        }
    }
}

/* reinitializeWithSwap3D (reinitialization.h:199-228) / reinitializeWithSwap
 * (2D reinitialization.h:321-360): phi0 <- phi (whole array) + BC, crossings,
 * then iterations of {step, swap, BC}.  The final field is left in phi (the
 * caller's buffer); phi_tmp is scratch. */
static void reinit_any(const orc_params* p, int dim, double* phi, double* tmp, double* phi0,
                       double* rt, int* flag) {
    grid_t g = dim == 3 ? grid3(p) : grid2(p);
    long n = total_of(&g);
    memcpy(phi0, phi, sizeof(double) * n);
    if (dim == 3) bc3(&g, phi0); else bc2(p, &g, phi0);
    crossings(&g, dim, phi0, rt, flag);
    double* a = phi;
    double* b = tmp;
    for (int it = 0; it < p->reinit_iterations; it++) {
        reinit_step(p, &g, dim, a, b, phi0, rt, flag);
        double* t = a; a = b; b = t;
        if (dim == 3) bc3(&g, a); else bc2(p, &g, a);
    }
    if (a != phi) memcpy(phi, a, sizeof(double) * n);
}

void orc3d_reinit(const orc_params* p, double* phi, double* tmp, double* phi0, double* rt, int* flag) {
    reinit_any(p, 3, phi, tmp, phi0, rt, flag);
}
void orc2d_reinit(const orc_params* p, double* phi, double* tmp, double* phi0, double* rt, int* flag) {
    reinit_any(p, 2, phi, tmp, phi0, rt, flag);
}
void orc3d_crossings(const orc_params* p, const double* phi0, double* rt, int* flag) {
    grid_t g = grid3(p);
    crossings(&g, 3, phi0, rt, flag);
}
void orc2d_crossings(const orc_params* p, const double* phi0, double* rt, int* flag) {
    grid_t g = grid2(p);
    crossings(&g, 2, phi0, rt, flag);
}

/* ---------------------------------------------------------------------------
 * Reductions.  computeInterfaceVolume (io.h:263-288) adds dx*dy*dz once per
 * cell with G < 0, in loop order; computeL2Error3D (io.h:229-258) is
 * sqrt(sum (G - G_ref)^2 / count) over interior cells.  2D: io.h:194-249.
 * ------------------------------------------------------------------------- */
double orc3d_volume(const orc_params* p, const double* G, long* count_out) {
    grid_t g = grid3(p);
    double vol = 0.0;
    long cnt = 0;
    for (int k = NG; k < g.nz + NG; k++)
        for (int j = NG; j < g.ny + NG; j++)
            for (int i = NG; i < g.nx + NG; i++)
                if (G[k * g.sz + j * g.sy + i] < 0.0) { vol += p->dx * p->dy * p->dz; cnt++; }
    if (count_out) *count_out = cnt;
    return vol;
}

double orc2d_area(const orc_params* p, const double* G, long* count_out) {
    grid_t g = grid2(p);
    double a = 0.0;
    long cnt = 0;
    for (int j = NG; j < g.ny + NG; j++)
        for (int i = NG; i < g.nx + NG; i++)
            if (G[j * g.sy + i] < 0.0) { a += p->dx * p->dy; cnt++; }
    if (count_out) *count_out = cnt;
    return a;
}

double orc_l2(const orc_params* p, int dim, const double* G, const double* Gref) {
    grid_t g = dim == 3 ? grid3(p) : grid2(p);
    int k0 = dim == 3 ? NG : 0, nz = dim == 3 ? g.nz : 1;
    double sum = 0.0;
    long cnt = 0;
    for (int k = k0; k < k0 + nz; k++)
        for (int j = NG; j < g.ny + NG; j++)
            for (int i = NG; i < g.nx + NG; i++) {
                long id = k * g.sz + j * g.sy + i;
                double d = G[id] - Gref[id];
                sum += d * d;
                cnt++;
            }
    return sqrt(sum / cnt);
}

/* Field-max speed max(|u|+|v|+|w|) over interior cells and the CFL step
 * cfl * min(dx,dy,dz) / (max_speed + s_l), with the reference's fallback
 * speed 2.0 below epsilon (config.h:272-293; the maximum over cells replaces
 * the constant velocities -- an addition). */
double orc_max_speed(const orc_params* p, int dim, const double* u, const double* v,
                     const double* w) {
    grid_t g = dim == 3 ? grid3(p) : grid2(p);
    int k0 = dim == 3 ? NG : 0, nz = dim == 3 ? g.nz : 1;
    double m = 0.0;
    for (int k = k0; k < k0 + nz; k++)
        for (int j = NG; j < g.ny + NG; j++)
            for (int i = NG; i < g.nx + NG; i++) {
                long id = k * g.sz + j * g.sy + i;
                double s = fabs(u[id]) + fabs(v[id]);
                if (dim == 3) s = s + fabs(w[id]);
                if (s > m) m = s;
            }
    return m;
}

double orc_cfl_dt(const orc_params* p, int dim, double cfl, double max_speed) {
    double speed = max_speed + p->s_l;
    if (speed < p->epsilon) speed = 2.0;
    double dmin = dim == 3 ? fmin(p->dx, fmin(p->dy, p->dz)) : fmin(p->dx, p->dy);
    return cfl * dmin / speed;
}

/* ---------------------------------------------------------------------------
 * Time loop for a fixed velocity and step count, the reference main loop
 * (Local_code/level-set_MPI_3D/src/main.cpp:291-316, 2D src/main.cpp:314-334)
 * without the final-step clip: BC on G and velocity first, then per step
 * {RK3, swap, reinit if enable && step > 0 && step % interval == 0}.
 * step0 offsets the step counter (a run split in segments keeps the cadence).
 * G is updated in place; velocity arrays are copied.
 * ------------------------------------------------------------------------- */
/* The loop itself on G in place, with velocities whose ghosts are already
 * filled (read in place).  Scratch: 5 fields + the flag array.  Stage 2 of
 * each step writes G2 over G1 (the combination is point-wise, so every cell
 * reads its own G1 value before overwriting it: the same bits as separate
 * buffers), and the reinitialisation's ping-pong partner is the rhs buffer,
 * which holds nothing between steps.  Returns 0, or -1 if the scratch
 * allocation fails. */
static int run_core(const orc_params* p, int dim, int n_steps, int step0, double* G,
                    const double* u, const double* v, const double* w, const double* sl) {
    grid_t g = dim == 3 ? grid3(p) : grid2(p);
    long n = total_of(&g);
    size_t bytes = sizeof(double) * (size_t)n;
    double* buf = (double*)calloc((size_t)n * 5, sizeof(double));
    int* flag = (int*)calloc((size_t)n, sizeof(int));
    if (!buf || !flag) {
        free(buf);
        free(flag);
        return -1;
    }
    double *Gnew = buf, *G1 = buf + n, *R = buf + 2 * n, *phi0 = buf + 3 * n, *rt = buf + 4 * n;
    if (dim == 3) bc3(&g, G); else bc2(p, &g, G);
    double* a = G;
    double* b = Gnew;
    for (int s = 0; s < n_steps; s++) {
        int step = step0 + s;
        if (dim == 3) orc3d_rk3_step(p, a, b, G1, G1, R, u, v, w, sl);
        else orc2d_rk3_step(p, a, b, G1, G1, R, u, v, sl);
        double* t = a; a = b; b = t;
        if (p->enable_reinit && step > 0 && step % p->reinit_interval == 0)
            reinit_any(p, dim, a, R, phi0, rt, flag);
    }
    if (a != G) memcpy(G, a, bytes);
    free(buf);
    free(flag);
    return 0;
}

static int run_any(const orc_params* p, int dim, int n_steps, int step0, double* G,
                   const double* u_in, const double* v_in, const double* w_in, const double* sl) {
    grid_t g = dim == 3 ? grid3(p) : grid2(p);
    long n = total_of(&g);
    size_t bytes = sizeof(double) * (size_t)n;
    double* vel = (double*)calloc((size_t)n * 3, sizeof(double));
    if (!vel) return -1;
    double *u = vel, *v = vel + n, *w = vel + 2 * n;
    memcpy(u, u_in, bytes);
    memcpy(v, v_in, bytes);
    if (dim == 3) memcpy(w, w_in, bytes);
    if (dim == 3) { bc3(&g, u); bc3(&g, v); bc3(&g, w); }
    else { bc2(p, &g, u); bc2(p, &g, v); }
    int rc = run_core(p, dim, n_steps, step0, G, u, v, dim == 3 ? w : NULL, sl);
    free(vel);
    return rc;
}

int orc3d_run(const orc_params* p, int n_steps, int step0, double* G, const double* u,
              const double* v, const double* w, const double* sl) {
    return run_any(p, 3, n_steps, step0, G, u, v, w, sl);
}

int orc2d_run(const orc_params* p, int n_steps, int step0, double* G, const double* u,
              const double* v, const double* sl) {
    return run_any(p, 2, n_steps, step0, G, u, v, NULL, sl);
}

/* The same loop for grids too large to copy the velocity: u, v, w must
 * already hold their boundary images (as bc3 / bc2 leaves them); they are
 * only read. */
int orc3d_run_filled(const orc_params* p, int n_steps, int step0, double* G, const double* u,
                     const double* v, const double* w, const double* sl) {
    return run_core(p, 3, n_steps, step0, G, u, v, w, sl);
}

int orc2d_run_filled(const orc_params* p, int n_steps, int step0, double* G, const double* u,
                     const double* v, const double* sl) {
    return run_core(p, 2, n_steps, step0, G, u, v, NULL, sl);
}

/* ---------------------------------------------------------------------------
 * The reference's default 3D test case (for the golden-log pin).
 * initSphere (Local_code/level-set_MPI_3D/include/initial_conditions.h:119-139)
 * with signedDistanceSphere (:52-58), computeDeformationVelocity (:232-247)
 * over the whole ghosted grid (initDeformationVelocity3D, :252-273), and the
 * main loop of src/main.cpp:180-334 with its final-step dt clip.  Coordinates
 * x = (i - 3) * dx (config.h:321-328).
 * ------------------------------------------------------------------------- */
#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

void orc3d_sphere(const orc_params* p, double cx, double cy, double cz, double r, double* G) {
    grid_t g = grid3(p);
    for (int k = 0; k < g.nzT; k++)
        for (int j = 0; j < g.nyT; j++)
            for (int i = 0; i < g.nxT; i++) {
                double x = 0.0 + (i - NG) * p->dx, y = 0.0 + (j - NG) * p->dy, z = 0.0 + (k - NG) * p->dz;
                double ddx = x - cx, ddy = y - cy, ddz = z - cz;
                G[k * g.sz + j * g.sy + i] = sqrt(ddx * ddx + ddy * ddy + ddz * ddz) - r;
            }
}

void orc3d_deformation_velocity(const orc_params* p, double t, double T, double* u, double* v,
                                double* w) {
    grid_t g = grid3(p);
    int k;
#pragma omp parallel for schedule(static)
    for (k = 0; k < g.nzT; k++)
        for (int j = 0; j < g.nyT; j++)
            for (int i = 0; i < g.nxT; i++) {
                double x = 0.0 + (i - NG) * p->dx, y = 0.0 + (j - NG) * p->dy, z = 0.0 + (k - NG) * p->dz;
                double tf = cos(M_PI * t / T);
                double spx = sin(M_PI * x), s2px = sin(2.0 * M_PI * x);
                double spy = sin(M_PI * y), s2py = sin(2.0 * M_PI * y);
                double spz = sin(M_PI * z), s2pz = sin(2.0 * M_PI * z);
                long id = k * g.sz + j * g.sy + i;
                u[id] = 2.0 * spx * spx * s2py * s2pz * tf;
                v[id] = -s2px * spy * spy * s2pz * tf;
                w[id] = -s2px * s2py * spz * spz * tf;
            }
}

/* Runs the default case (nx = ny = nz = n, dx = 1/(n-1), dt = 1e-3,
 * T = 1.5, S_L = 0, no reinit); returns final L2 vs the initial field, the
 * initial and final G < 0 volumes and the step count. */
void orc3d_deformation_test(int n, double* l2_out, double* v0_out, double* v1_out, int* steps_out) {
    orc_params p;
    memset(&p, 0, sizeof(p));
    p.nx = p.ny = p.nz = n;
    p.dx = p.dy = p.dz = (1.0 - 0.0) / (n - 1);
    p.dt = 0.001;
    p.s_l = 0.0;
    p.epsilon = 1.0e-10;
    double T = 1.5;
    grid_t g = grid3(&p);
    long N = total_of(&g);
    double* buf = (double*)calloc((size_t)N * 9, sizeof(double));
    double *G = buf, *Gn = buf + N, *G1 = buf + 2 * N, *G2 = buf + 3 * N, *R = buf + 4 * N;
    double *G0 = buf + 5 * N, *u = buf + 6 * N, *v = buf + 7 * N, *w = buf + 8 * N;
    orc3d_sphere(&p, 0.35, 0.35, 0.35, 0.15, G);
    orc3d_deformation_velocity(&p, 0.0, T, u, v, w);
    bc3(&g, G);
    bc3(&g, u); bc3(&g, v); bc3(&g, w);
    memcpy(G0, G, sizeof(double) * N);
    *v0_out = orc3d_volume(&p, G, NULL);
    double t = 0.0;
    int step = 0;
    int max_steps = (int)(T / p.dt) + 100;
    double* a = G;
    double* b = Gn;
    while (t < T && step < max_steps) {
        if (t + p.dt > T) p.dt = T - t;
        orc3d_deformation_velocity(&p, t, T, u, v, w);
        bc3(&g, u); bc3(&g, v); bc3(&g, w);
        orc3d_rk3_step(&p, a, b, G1, G2, R, u, v, w, NULL);
        double* tmp = a; a = b; b = tmp;
        t += p.dt;
        step++;
    }
    *l2_out = orc_l2(&p, 3, a, G0);
    *v1_out = orc3d_volume(&p, a, NULL);
    *steps_out = step;
    free(buf);
}
