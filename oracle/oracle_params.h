/*
 * Parameter block shared by the two CPU oracles (test infrastructure only):
 *   - oracle/_ref/libref{2d,3d}.so : the reference's own solver headers,
 *     compiled unmodified by oracle/build_ref.sh against oracle/mpi_stub;
 *   - oracle/_build/liboracle.so   : the plain-C restatement (ls_oracle.c).
 *
 * Fields follow the reference's SimParams
 * (Local_code/level-set_MPI_3D/include/config.h:134-175) restricted to what
 * the hot path reads.  Arrays are in the reference's ghosted row-major
 * layout: index = k*nxT*nyT + j*nxT + i with nxT = nx + 6, nyT = ny + 6,
 * nzT = nz + 6 (config.h:301-306); 2D arrays drop the k term.
 */
#ifndef LSGB_ORACLE_PARAMS_H
#define LSGB_ORACLE_PARAMS_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_params {
    int nx, ny, nz;          /* interior cells; nz is ignored in 2D */
    double dx, dy, dz;
    double dt;
    double s_l;
    double epsilon;          /* 1e-10 in the reference (config.h:104) */
    int enable_reinit;
    int reinit_interval;
    int reinit_iterations;
    double reinit_dtau;
    double reinit_beta;
    int periodic_y;          /* 2D: 1 = periodic Y (self exchange), 0 = zero-gradient Y ends */
} orc_params;

#ifdef __cplusplus
}
#endif

#endif
