/*
 * lsgb.h -- C ABI of the GB300 level-set (G-equation) solver.
 *
 * Advances dG/dt + u_eff . grad G = 0, u_eff = u - S_L grad G / |grad G|, with
 * WENO-5 upwind derivatives and TVD (Shu-Osher) RK3, and the HCR-2
 * constrained reinitialisation, on one NVIDIA GB300 (sm_103a).
 *
 * Reference solver being replaced (juhoon196/Level-set-method-code):
 * Local_code/level-set_MPI_3D (3D) and Local_code/level-set_MPI_2D (2D),
 * whose hot-path functions are header-inline C++ called from src/main.cpp.
 * Each entry point below names the reference function it stands in for.
 *
 * Conventions
 *   - Every function returns LSGB_OK (0) or an LSGB_ERR_* code; the message of
 *     the last failure on the calling thread is lsgb_last_error().  Nothing
 *     calls exit() or abort().
 *   - "Device" pointers are CUDA device (or managed) memory of the current
 *     device; stream arguments are cudaStream_t values passed as void*
 *     (NULL = the legacy default stream).  Work is stream-ordered; functions
 *     that return a host scalar synchronise that stream.
 *   - Field layout LSGB_LAYOUT_GHOSTED is the reference's: 3 ghost cells per
 *     side, row-major, index k*(nx+6)*(ny+6) + j*(nx+6) + i
 *     (Local_code/level-set_MPI_3D/include/config.h:301-306); 2D arrays have no
 *     k term.  LSGB_LAYOUT_COMPACT is interior cells only, index
 *     k*nx*ny + j*nx + i.
 *   - The FP64 functions reproduce the reference's IEEE double arithmetic
 *     operation for operation (no fused multiply-adds).
 */
#ifndef LSGB_H
#define LSGB_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define LSGB_API __attribute__((visibility("default")))
#else
#define LSGB_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define LSGB_OK 0
#define LSGB_ERR_INVALID 1   /* bad argument or parameter block */
#define LSGB_ERR_CUDA 2      /* a CUDA runtime call or kernel launch failed */
#define LSGB_ERR_ALLOC 3     /* device or pinned-host allocation failed */
#define LSGB_ERR_NUMERIC 4   /* non-finite value detected in a reduction */
#define LSGB_ERR_STATE 5     /* call out of order (fields not set, ...) */
#define LSGB_ERR_UNSUPPORTED 6

/* boundary treatment per axis */
#define LSGB_BC_PERIODIC 0       /* boundary.h:144-188 (3D), 2D boundary.h:98-114 */
#define LSGB_BC_ZERO_GRADIENT 1  /* 2D boundary.h:126-147 */

/* arithmetic of a solver handle */
#define LSGB_PREC_F64 0  /* plain FP64, the reference's arithmetic */
#define LSGB_PREC_F32 1  /* FP32 bulk; FP64 HCR-2 interface constraint and reductions */

/* array layouts */
#define LSGB_LAYOUT_GHOSTED 0
#define LSGB_LAYOUT_COMPACT 1

/* where a pointer lives */
#define LSGB_MEM_HOST 0
#define LSGB_MEM_DEVICE 1

/*
 * Parameter block: the fields of the reference's SimParams that the hot path
 * reads (Local_code/level-set_MPI_3D/include/config.h:134-175), with the MPI
 * decomposition fields replaced by one boundary code per axis.  Defaults as in
 * config.h:88-107 come from lsgb_params_default().
 */
typedef struct lsgb_params {
    int dim;                /* 2 or 3 */
    int nx, ny, nz;         /* interior cells; nz is ignored when dim == 2 */
    int nghost;             /* must be 3 (config.h:31) */
    double dx, dy, dz;      /* spacing; dz ignored when dim == 2 */
    double s_l;             /* laminar flame speed (uniform) */
    double dt;              /* time step */
    double cfl;             /* CFL number used by lsgb_cfl_dt */
    double epsilon;         /* 1e-10: S_L gate and |grad G| regulariser (rk3.h:54-65) */
    int enable_reinit;      /* HCR-2 on/off */
    int reinit_interval;    /* reinit when step > 0 && step % interval == 0 (src/main.cpp:310) */
    int reinit_iterations;  /* pseudo-time steps per reinit */
    double reinit_dtau;     /* pseudo-time step, 0.25 * min spacing by default */
    double reinit_beta;     /* HCR-2 forcing weight, 0.5 */
    int bc_x, bc_y, bc_z;   /* LSGB_BC_* per axis */
} lsgb_params;

/* Fills *p with the reference's defaults for an nx x ny x nz grid on the unit
 * cube/square with spacing 1/n (periodic on every axis). */
LSGB_API void lsgb_params_default(lsgb_params* p, int dim, int nx, int ny, int nz);

/* Checks a parameter block; LSGB_OK or LSGB_ERR_INVALID with a message. */
LSGB_API int lsgb_params_check(const lsgb_params* p);

/* Message of the last failed call on this thread ("" if none). */
LSGB_API const char* lsgb_last_error(void);

/* Library version string. */
LSGB_API const char* lsgb_version(void);

/* Number of CUDA kernels this library has launched in this process (graph
 * replays count every kernel node). */
LSGB_API uint64_t lsgb_launch_count(void);

/* ------------------------------------------------------------------------
 * Drop-in entry points: device pointers in the reference's GHOSTED layout,
 * FP64, the reference's calling convention (the caller owns every buffer).
 * ------------------------------------------------------------------------ */

/* One TVD-RK3 step G_n -> G_new, boundary fill after each stage.
 * Replaces rk3TimeStep3D (Local_code/level-set_MPI_3D/include/rk3.h:131-150)
 * and rk3TimeStep (Local_code/level-set_MPI_2D/include/rk3.h:168-187).
 * The reference's G_rhs scratch array is not needed: the RHS is fused into
 * each stage.  G_1 and G_2 receive the stage fields as in the reference.
 * w is ignored in 2D.  s_l_field (nullable, ghosted) is a per-cell flame
 * speed that replaces p->s_l cell by cell (an addition; NULL = uniform). */
LSGB_API int lsgb_rk3_step_f64(const lsgb_params* p, const double* G_n, double* G_new, double* G_1,
                      double* G_2, const double* u, const double* v, const double* w,
                      const double* s_l_field, void* stream);

/* Ghost fill: applyBoundaryConditions3D (boundary.h:250-261) / 2D
 * applyBoundaryConditions (2D boundary.h:217-229). */
LSGB_API int lsgb_apply_bc_f64(const lsgb_params* p, double* G, void* stream);

/* HCR-2 reinitialisation with the reference's pointer swap: on return *phi
 * holds the result and *phi_tmp the other buffer; phi0, r_tilde and flag
 * receive what the reference leaves in them.
 * Replaces reinitializeWithSwap3D (Local_code/level-set_MPI_3D/include/reinitialization.h:199-228)
 * and reinitializeWithSwap (Local_code/level-set_MPI_2D/include/reinitialization.h:321-360).
 * Runs regardless of p->enable_reinit (the caller decides the cadence). */
LSGB_API int lsgb_reinit_f64(const lsgb_params* p, double** phi, double** phi_tmp, double* phi0,
                    double* r_tilde, int32_t* flag, void* stream);

/* sum of dx*dy*dz over interior cells with G < 0 and that cell count.
 * Replaces computeInterfaceVolume (io.h:263-288) / computeInterfaceArea
 * (2D io.h:225-249).  Synchronises the stream. */
LSGB_API int lsgb_volume_f64(const lsgb_params* p, const double* G, double* volume, int64_t* count,
                    void* stream);

/* Allocation-free form of lsgb_volume_f64, for callers that must not have the
 * library allocate device memory during the call: a host whose own pool
 * already holds the device, or a monitoring hook inside the caller's time
 * loop that may not block in the allocator.  No counterpart in the reference.
 * Same results as lsgb_volume_f64 (exact count, volume = count * cell volume).
 * Its scratch is one fixed device array inside the library (512 KiB, kept by
 * every GPU that loads the library until the process exits):
 *   - at most LSGB_NOALLOC_MAX_CELLS interior cells (2^30, e.g. 1024^3) per
 *     call; larger grids return LSGB_ERR_INVALID;
 *   - the first call on a device (and again the first after a
 *     cudaDeviceReset, which gives the device a new context) looks the
 *     array's address up; make that first call before any stream capture;
 *   - all calls share the array: calls that overlap on the GPU race.
 * Synchronises the stream.  Calls no cudaMalloc / cudaFree. */
#define LSGB_NOALLOC_CHUNK 16384
#define LSGB_NOALLOC_MAX_PARTIALS 65536
#define LSGB_NOALLOC_MAX_CELLS ((long long)LSGB_NOALLOC_CHUNK * LSGB_NOALLOC_MAX_PARTIALS)
LSGB_API int lsgb_volume_f64_noalloc(const lsgb_params* p, const double* G, double* volume,
                                     int64_t* count, void* stream);

/* sqrt(mean over interior of (G - G_ref)^2).  Replaces computeL2Error3D
 * (io.h:229-258) / computeL2Error (2D io.h:194-220).  Synchronises. */
LSGB_API int lsgb_l2_error_f64(const lsgb_params* p, const double* G, const double* G_ref, double* l2,
                      void* stream);

/* max over interior cells of |u|+|v|(+|w|).  Synchronises. */
LSGB_API int lsgb_max_speed_f64(const lsgb_params* p, const double* u, const double* v, const double* w,
                       double* max_speed, void* stream);

/* CFL step cfl * min spacing / (max_speed + s_l), 2.0 as the speed below
 * epsilon: calculateTimeStep (config.h:272-293) with the field maximum in
 * place of the constant velocities.  Host only. */
LSGB_API int lsgb_cfl_dt(const lsgb_params* p, double max_speed, double* dt);

/* ------------------------------------------------------------------------
 * Solver handle: device-resident fields in the compact layout, FP64 or the
 * FP32-bulk form, steps captured in CUDA graphs.  This is the fast path.
 * ------------------------------------------------------------------------ */
typedef struct lsgb_solver lsgb_solver;

LSGB_API int lsgb_solver_create(const lsgb_params* p, int precision, lsgb_solver** out);
LSGB_API int lsgb_solver_destroy(lsgb_solver* s);

/* Stream the handle issues its work on (void* cudaStream_t; NULL = own stream). */
LSGB_API int lsgb_solver_set_stream(lsgb_solver* s, void* stream);

/* Current parameters (dt may have been set by lsgb_solver_compute_dt). */
LSGB_API int lsgb_solver_get_params(const lsgb_solver* s, lsgb_params* p);

/* Replace dt (e.g. the reference's final-step clip). */
LSGB_API int lsgb_solver_set_dt(lsgb_solver* s, double dt);

/* Load G and the velocity (w ignored in 2D) from FP64 arrays of the given
 * layout in host or device memory; FP32 handles convert on the device.  Any
 * pointer may be NULL to keep the current field. */
LSGB_API int lsgb_solver_set_fields(lsgb_solver* s, const double* G, const double* u, const double* v,
                           const double* w, int layout, int memory);

/* Per-cell flame speed (FP64, given layout/memory); NULL restores uniform p->s_l. */
LSGB_API int lsgb_solver_set_sl_field(lsgb_solver* s, const double* sl, int layout, int memory);

/* Store G as FP64 in the given layout (ghost cells filled as the reference's
 * boundary fill leaves them) to host or device memory. */
LSGB_API int lsgb_solver_get_G(lsgb_solver* s, double* G, int layout, int memory);

/* Advance n_steps TVD-RK3 steps; HCR-2 runs after the step whose counter
 * satisfies enable_reinit && step > 0 && step % reinit_interval == 0, the
 * counter then increments (Local_code/level-set_MPI_3D/src/main.cpp:291-316).
 * Asynchronous on the handle's stream. */
LSGB_API int lsgb_solver_advance(lsgb_solver* s, int n_steps);

/* Run one HCR-2 reinitialisation now (reinitializeWithSwap3D). */
LSGB_API int lsgb_solver_reinit(lsgb_solver* s);

/* Step counter used for the reinit cadence. */
LSGB_API int lsgb_solver_get_step(const lsgb_solver* s, int* step);
LSGB_API int lsgb_solver_set_step(lsgb_solver* s, int step);

/* Reductions over the current G / velocity (FP64 accumulation; synchronise). */
LSGB_API int lsgb_solver_volume(lsgb_solver* s, double* volume, int64_t* count);
LSGB_API int lsgb_solver_max_speed(lsgb_solver* s, double* max_speed);
/* Sets dt from the CFL formula with the field-max speed; returns it. */
LSGB_API int lsgb_solver_compute_dt(lsgb_solver* s, double cfl, double* dt);
/* L2 difference of G against an FP64 field (given layout/memory). */
LSGB_API int lsgb_solver_l2_error(lsgb_solver* s, const double* G_ref, int layout, int memory, double* l2);

/* End to end on host buffers, the call a host-side caller makes: upload G, u,
 * v, w (FP64, given layout, host memory), advance n_steps, download G into
 * G_out (same layout).  Synchronises.  Any velocity pointer may be NULL to
 * keep the resident field. */
LSGB_API int lsgb_solver_run_host(lsgb_solver* s, const double* G, const double* u, const double* v,
                         const double* w, int n_steps, double* G_out, int layout);

/* Store one resident field as FP64 (given layout / memory): which = 0 G,
 * 1 u, 2 v, 3 w, 4 the per-cell S_L field.  Ghosts are filled as the
 * reference's boundary fill leaves them. */
#define LSGB_FIELD_G 0
#define LSGB_FIELD_U 1
#define LSGB_FIELD_V 2
#define LSGB_FIELD_W 3
#define LSGB_FIELD_SL 4
LSGB_API int lsgb_solver_get_field(lsgb_solver* s, int which, double* out, int layout, int memory);

/* Kernel timing with CUDA events on the handle's stream, for roofline
 * accounting.  While enabled, every RK3 stage launch and every HCR-2
 * pseudo-step launch is bracketed by events; lsgb_solver_kernel_times
 * synchronises and returns the summed durations (ms) and launch counts since
 * the last enable. */
LSGB_API int lsgb_solver_enable_timing(lsgb_solver* s, int enable);
LSGB_API int lsgb_solver_kernel_times(lsgb_solver* s, double* stage_ms, int64_t* stage_launches,
                                      double* reinit_ms, int64_t* reinit_launches);

/* Tile shape of the stage kernels; 0 = default.  FP32 3D: the z-chunk
 * length (16, 32, 64; default: the chunk length that fills the GPU's SMs
 * best for the grid).  FP32 2D: the tile height (32: 32 x 32 tiles, the
 * default; 16: 32 x 16).  FP64: 1 = one thread per cell, 2 = face-shared
 * tiles (each WENO face value computed once for the cells on both sides;
 * default where the grid gives every SM two tiles).  Every shape gives
 * bit-identical results; only the speed differs. */
LSGB_API int lsgb_solver_set_tile(lsgb_solver* s, int tile);
LSGB_API int lsgb_solver_get_tile(const lsgb_solver* s, int* tile);

/* Test hook for the time-out path: while on, the TMA-fed FP32 3D stage kernel
 * issues no bulk copies, so each of its CTAs gives up its bounded wait after
 * about a second, sets the handle's device error flag and returns; the next
 * synchronising call (lsgb_solver_get_G, ...) reports LSGB_ERR_CUDA and clears
 * the flag.  The context stays usable.  Off by default; no other effect. */
LSGB_API int lsgb_solver_debug_drop_copies(lsgb_solver* s, int on);
/* Test hook: the FP64 kernels divide by a known divisor b as a one-multiply,
 * two-FMA correction of a * RN(1/b) (Markstein's theorem), and multiply by
 * 2, 4, 1/2, 1/4 as exponent shifts.  Compares those with IEEE division and
 * multiplication on n seeded cases (the solver's divisors and random ones;
 * random, exact-multiple and near-midpoint dividends; multiplicands over the
 * whole exponent range) and writes the number of results that differ in any
 * bit.  Synchronises. */
LSGB_API int lsgb_debug_f64_div_check(long long n, unsigned long long seed, long long* mismatches);

/* Autotuner: times one stage launch per candidate tile shape (reps launches
 * each, CUDA events on the handle's stream; the state G is not modified) and
 * keeps the fastest.  Needs G and the velocity.  Handles with one shape
 * report tile 0 and time 0. */
LSGB_API int lsgb_solver_autotune(lsgb_solver* s, int reps, int* best_tile, float* best_ms);

/* ------------------------------------------------------------------------
 * Batches: many independent instances (any mix of 2D and 3D sizes, one
 * precision) advanced together.  Instances keep their own lsgb_solver handle
 * for fields, reductions and output; lsgb_batch_advance runs all of them with
 * one captured CUDA graph per reinit period.  Instances must share the step
 * counter and the reinit cadence.  Each instance's result equals its
 * single-instance run bit for bit.  Not in the reference (its variants run
 * one instance per process, e.g. the sweep of sample/submit_all.sh:9-11).
 * Two forms of the graph:
 *   LSGB_BATCH_GROUPED (default; FP32, every instance < 2^31 cells, one HCR-2
 *     pseudo-step count): one kernel launch per RK3 stage and per
 *     pseudo-step (and, for an odd pseudo-step count, for the copy back)
 *     for all 3D instances, and one for all 2D ones;
 *     the kernels walk a block / tile list that spans the instances, with
 *     each instance's fields and coefficients in a descriptor table;
 *   LSGB_BATCH_LANES (FP64 batches, or on request): each instance's own
 *     launches, spread over n_lanes concurrent streams.
 * ------------------------------------------------------------------------ */
#define LSGB_BATCH_GROUPED 0
#define LSGB_BATCH_LANES 1
typedef struct lsgb_batch lsgb_batch;
LSGB_API int lsgb_batch_create(int precision, int n_lanes, lsgb_batch** out);
LSGB_API int lsgb_batch_destroy(lsgb_batch* b);
/* New instance owned by the batch; *solver (nullable) is its handle. */
LSGB_API int lsgb_batch_add(lsgb_batch* b, const lsgb_params* p, lsgb_solver** solver, int* index);
LSGB_API int lsgb_batch_size(const lsgb_batch* b, int* n);
LSGB_API int lsgb_batch_solver(lsgb_batch* b, int index, lsgb_solver** out);
/* lsgb_solver_autotune on every instance, then (FP32) each uniform z-chunk
 * (16, 32, 64) for the 3D instances against that, timed as one stage of the
 * whole batch, and in the grouped form the 2D tile height (32 x 32 or
 * 32 x 16 tiles), timed as one grouped 2D stage; the fastest choices stay. */
LSGB_API int lsgb_batch_autotune(lsgb_batch* b, int reps);
/* Request a form (LSGB_BATCH_GROUPED / LSGB_BATCH_LANES); get_mode reports
 * the form the next advance uses (grouped only where it applies). */
LSGB_API int lsgb_batch_set_mode(lsgb_batch* b, int mode);
LSGB_API int lsgb_batch_get_mode(const lsgb_batch* b, int* mode);
/* Advance every instance n_steps steps (asynchronous on the batch stream;
 * later calls on an instance's own handle are ordered after it). */
LSGB_API int lsgb_batch_advance(lsgb_batch* b, int n_steps);
/* Wait for the batch and report any in-kernel wait that gave up. */
LSGB_API int lsgb_batch_sync(lsgb_batch* b);
/* Graph replays so far and kernels per replayed graph. */
LSGB_API int lsgb_batch_stats(const lsgb_batch* b, int64_t* graph_launches, int64_t* kernels_per_graph);
/* The batch's stream (void* cudaStream_t), for events around lsgb_batch_advance. */
LSGB_API int lsgb_batch_stream(lsgb_batch* b, void** stream);

/* ------------------------------------------------------------------------
 * Discrete adjoint of lsgb_solver_advance (not in the reference, which has no
 * gradients).  The forward records checkpoints of G every checkpoint_interval
 * steps; the backward recomputes one checkpoint segment at a time on a tape
 * (every RK3 stage input and every HCR-2 pseudo-step input) and runs the
 * vector-Jacobian products of the stage kernels and the pseudo-steps in
 * reverse.  Upwind branches, Godunov selections, crossing flags and the
 * stability mask are taken from the forward state.  Periodic and
 * zero-gradient axes in any mix (on a zero-gradient axis the transpose of the
 * clamped neighbour map adds the clamped stencil points back onto the edge
 * cells).
 * Gradients are deterministic (no atomics) and independent of the checkpoint
 * interval.
 * ------------------------------------------------------------------------ */
typedef struct lsgb_adjoint lsgb_adjoint;
LSGB_API int lsgb_adjoint_create(lsgb_solver* s, int checkpoint_interval, lsgb_adjoint** out);
LSGB_API int lsgb_adjoint_destroy(lsgb_adjoint* a);
/* Parameter gradients the backward accumulates (default: both).  dL/dG_0 is
 * always formed. */
#define LSGB_GRAD_SL 1
#define LSGB_GRAD_VELOCITY 2
LSGB_API int lsgb_adjoint_set_grads(lsgb_adjoint* a, int mask);
/* z planes per slab of the 3D stage transpose (0 = the default, one slab for
 * the whole domain).  Smaller slabs keep each slab's 19 coefficient planes
 * L2-resident between the two passes at the cost of a 3-plane halo recompute
 * and more launches.  Any slab gives bit-identical gradients. */
LSGB_API int lsgb_adjoint_set_slab(lsgb_adjoint* a, int planes);
/* Advance the solver n_steps steps (same results as lsgb_solver_advance),
 * recording checkpoints; the solver ends at G_T.  With live deformation
 * velocity (lsgb_solver_set_velocity_deformation_live) the checkpoints also
 * keep the vortex time, and the backward evaluates the vortex at every step's
 * time; dL/du, dL/dv, dL/dw are then the gradients with respect to a steady
 * field added to the vortex at every step (the per-step sensitivities summed). */
LSGB_API int lsgb_adjoint_forward(lsgb_adjoint* a, int n_steps);
/* Target field for the smoothed-Heaviside mismatch
 *   L = 1/2 sum_cells (H(G_T) - H(G_target))^2 dV,  H(g) = (1 - tanh(g / eps)) / 2. */
LSGB_API int lsgb_adjoint_set_target(lsgb_adjoint* a, const double* G_target, int layout, int memory,
                                     double eps);
/* L of the solver's current G against the target; seed != 0 also stores
 * dL/dG_T as the seed of the next backward. */
LSGB_API int lsgb_adjoint_loss(lsgb_adjoint* a, int seed, double* loss);
/* Reverse sweep over the last forward.  dL_dGT (FP64, layout / memory) is the
 * seed; NULL uses the seed stored by lsgb_adjoint_loss. */
LSGB_API int lsgb_adjoint_backward(lsgb_adjoint* a, const double* dL_dGT, int layout, int memory);
/* Gradient of the last backward as FP64: which = LSGB_FIELD_G (dL/dG_0),
 * LSGB_FIELD_U / _V / _W (velocity), LSGB_FIELD_SL (per-cell S_L; with a
 * scalar S_L the sum of this field is dL/dS_L). */
LSGB_API int lsgb_adjoint_get_grad(lsgb_adjoint* a, int which, double* out, int layout, int memory);

/* Deformation-vortex velocity of the reference's default 3D test case at time
 * t with period T, evaluated on the device at the cell centres x_i = i * dx
 * into the stored u, v, w: computeDeformationVelocity /
 * updateDeformationVelocity
 * (Local_code/level-set_MPI_3D/include/initial_conditions.h:232-282).  FP64
 * handles get the reference's products of FP64 sines; FP32 handles form the
 * products in FP32 from factor tables.  Ends live mode (below). */
LSGB_API int lsgb_solver_set_velocity_deformation(lsgb_solver* s, double t, double T);
/* Live mode: from now on every step uses the vortex at the handle's time,
 * which starts at t and advances by dt after each step -- the reference's
 * loop (src/main.cpp:291-316: velocity at current_time, RK3 step, reinit,
 * current_time += dt) inside one lsgb_solver_advance.  FP32 3D handles with
 * nx % 4 == 0 and fewer than 2^31 cells evaluate the vortex inside the stage
 * kernel (no u, v, w traffic); other handles refill u, v, w before each step.
 * Either way the fields equal a per-step lsgb_solver_set_velocity_deformation
 * loop bit for bit.  Calls that read u, v, w (lsgb_solver_max_speed,
 * lsgb_solver_get_field) see the vortex at the current time.  Setting
 * velocity arrays ends live mode.  Batches advance live handles too: the
 * host evaluates every step's time (FP64) or time factor (FP32) of an
 * lsgb_batch_advance call as above into a device table, and the batch's
 * launches (captured graphs included) refill u, v, w from it, indexed by a
 * device-side step cursor -- the same bits as the handle advanced alone.
 * The adjoint follows live handles (lsgb_adjoint_forward). */
LSGB_API int lsgb_solver_set_velocity_deformation_live(lsgb_solver* s, double t, double T);
/* The live-mode time (the t of the next step). */
LSGB_API int lsgb_solver_get_time(const lsgb_solver* s, double* t);

/* Error and conservation diagnostics of the reference's analysis script
 * (Local_code/level-set_MPI_3D/scripts/analyze_error.m) between the solver's
 * G and a reference field G_ref (FP64, given layout / memory), as one device
 * reduction.  Synchronises. */
typedef struct lsgb_diagnostics {
    double l2, linf, l2_rel;        /* RMS and max of G - G_ref; l2 / RMS(G_ref)   (:33-44) */
    double volume, volume_ref;      /* cells with G < 0 times the cell volume      (:88-98) */
    double volume_smooth, volume_smooth_ref;  /* smoothed Heaviside of -G, eps = dx (:100-107, :264-271) */
    double grad_mean, grad_std;     /* |grad G| (central differences) where |G| < 3 dx (:109-133) */
    double iface_mean, iface_max;   /* first-order interface distance: each zero set's grid-edge
                                       crossing points p against the other field, |G(p)| / |grad G(p)|;
                                       mean and max (a cheap estimate beside the contour metric below) */
    int64_t band_cells, iface_points;
    double contour_hausdorff;       /* the script's interface position error (:51-84): zero contours
                                       of G and G_ref as grid-edge crossing points (contourc's
                                       vertices; in 3D the isosurface's), every point's distance to
                                       the nearest point of the other set; the largest of them */
    double contour_mean;            /* their mean over both sets (the "mean interface error") */
    int64_t contour_points, contour_points_ref;  /* points of G's / G_ref's zero set; when either is
                                                    0 the two distances above are NaN */
} lsgb_diagnostics;
LSGB_API int lsgb_solver_diagnostics(lsgb_solver* s, const double* G_ref, int layout, int memory,
                                     lsgb_diagnostics* out);

/* ------------------------------------------------------------------------
 * Binary G dumps in the reference's .bin format: int32 {nx, ny, nz, nghost}
 * (3D) or {nx, ny, nghost} (2D), then the whole ghosted FP64 array, whose x
 * (and z) ghosts are what the boundary fill leaves and whose y ghosts copy the
 * first / last interior row.  Replaces saveFieldBinary3D
 * (Local_code/level-set_MPI_3D/include/io.h:33-131) and saveFieldBinary
 * (Local_code/level-set_MPI_2D/include/io.h:26-109); the reference's doc
 * comment promises a double[4] {time, dx, dy, dz} header block that its code
 * never writes, and neither does this.
 * ------------------------------------------------------------------------ */
/* Bytes of one dump image (header + array). */
LSGB_API int lsgb_dump_bytes(const lsgb_params* p, size_t* bytes);
/* Image of a ghosted FP64 device array G into out (lsgb_dump_bytes bytes,
 * host or device memory).  Synchronises the stream. */
LSGB_API int lsgb_dump_f64(const lsgb_params* p, const double* G, void* out, int memory, void* stream);
/* Image of a solver's current G (either precision; FP32 values widened). */
LSGB_API int lsgb_solver_dump(lsgb_solver* s, void* out, int memory);
/* Write the current G's image to the file `path` without stopping the time
 * loop: the image is packed on the solver's stream, copied to pinned host
 * memory on a second stream and written by a background thread (two images
 * in flight; a third call waits for the older one).  Later steps may run
 * while the file is written.  lsgb_solver_snapshot_wait waits for every
 * pending file and reports the first failure. */
LSGB_API int lsgb_solver_snapshot(lsgb_solver* s, const char* path);
LSGB_API int lsgb_solver_snapshot_wait(lsgb_solver* s);

/* ------------------------------------------------------------------------
 * Sample surface: the reference's 2D Field2D solver (sample/field.hpp,
 * sample/weno5_rk3.hpp).  Arrays are FP64 device buffers in Field2D's element
 * order, row-major [ny+6][nx+6] with 3 ghost cells per side (the same map as
 * LSGB_LAYOUT_GHOSTED in 2D), owned by the caller.  Results equal the
 * reference's compiled sources bit for bit.  Calls are stream-ordered on
 * `stream` (NULL = legacy default stream); `work` arguments are optional
 * device scratch (NULL = stream-ordered allocation inside the call).
 * ------------------------------------------------------------------------ */
/* compute_geqn_rhs (sample/weno5_rk3.hpp:10-16, weno5_rk3.cpp:91-145): the
 * local Lax-Friedrichs rhs = -H on the interior; ghost cells of rhs = 0. */
LSGB_API int lsgb_sample_rhs(int nx, int ny, const double* G, const double* u, const double* v, double* rhs,
                             double dx, double dy, double S_L, void* stream);
/* RK3_step (sample/weno5_rk3.hpp:20-25, weno5_rk3.cpp:148-188): in place on
 * G; work = 2 arrays. */
LSGB_API int lsgb_sample_rk3_step(int nx, int ny, double* G, const double* u, const double* v, double dx,
                                  double dy, double dt, double S_L, const double* G_initial, double* work,
                                  void* stream);
/* compute_first_order_upwind (sample/first_order_upwind.hpp:4-12,
 * first_order_upwind.cpp:6-69): the first-order upwind step, in place on G,
 * over the reference's range j = 3 .. ny+3, i = 3 .. nx+3 (one ghost row and
 * column past the interior on the high side); work = 1 array. */
LSGB_API int lsgb_sample_first_order_upwind(int nx, int ny, double* G, const double* u, const double* v, double dx,
                                            double dy, double dt, double S_L, double* work, void* stream);
/* Field2D::apply_periodic / apply_anchored_bc (sample/field.hpp:15-18,
 * field.cpp:16-63). */
LSGB_API int lsgb_sample_apply_periodic(int nx, int ny, double* G, void* stream);
LSGB_API int lsgb_sample_apply_anchored_bc(int nx, int ny, double* G, const double* G_initial, void* stream);
/* Field2D::reinitialize (sample/field.hpp:20, field.cpp:66-129); work = 1 array. */
LSGB_API int lsgb_sample_reinitialize(int nx, int ny, double* G, const double* G_initial, double dx, double dy,
                                      int num_iters, double* work, void* stream);

/* The forced time loop of sample/main.cpp:126-148 for n_steps steps, over
 * n_inst instances at once (the reference runs one process per forcing
 * frequency, sample/submit_all.sh): instance q is the array G + q (nx+6)(ny+6)
 * with the spatially uniform velocity
 *   u = u0 + eps_u v0 cos(2 pi freq[q] t),  v = v0 + eps_v v0 cos(2 pi freq[q] t)
 * evaluated at its own time t[q], which advances by dt per step (host arrays
 * freq and t; t is updated).  G_initial is one array shared by all instances
 * (shared_initial != 0) or n_inst arrays.  work = 2 n_inst arrays.
 * Synchronises the stream before returning. */
typedef struct lsgb_sample_forcing {
    double u0, v0, eps_u, eps_v;
} lsgb_sample_forcing;
LSGB_API int lsgb_sample_run(int n_inst, int nx, int ny, int n_steps, double* G, const double* G_initial,
                             int shared_initial, double dx, double dy, double dt, double S_L,
                             const lsgb_sample_forcing* forcing, const int* freq, double* t, double* work,
                             void* stream);

/* ------------------------------------------------------------------------
 * Synthetic benchmark fields, generated on the device (FP64 arithmetic).
 *   G0 = |x - c| - (r0 + sum_m a_m Y_lm(theta, phi))      (sphere; 3D)
 *   G0 = |x - c| - r0                                    (circle; 2D)
 *   u  = sum_m c_m cos(2 pi k_m . x + phi_m), c_m = 2 pi k_m x a_m (curl of
 *        A = sum a_m sin(2 pi k_m . x + phi_m)), scaled by vel_scale.
 * Mode tables are drawn on the host from the seed (see lsgb/synthetic.py).
 * ------------------------------------------------------------------------ */
#define LSGB_MAX_MODES 32
typedef struct lsgb_synth {
    double center[3];
    double r0;
    int n_shape_modes;                 /* spherical-harmonic perturbations */
    int shape_l[LSGB_MAX_MODES];
    int shape_m[LSGB_MAX_MODES];
    double shape_amp[LSGB_MAX_MODES];
    int n_vel_modes;                   /* Fourier modes of the vector potential */
    double vel_k[LSGB_MAX_MODES][3];
    double vel_c[LSGB_MAX_MODES][3];   /* 2 pi k x a (before vel_scale) */
    double vel_phase[LSGB_MAX_MODES];
    double vel_scale;
} lsgb_synth;

/* Fill G, u, v, w of the handle from the description (device side). */
LSGB_API int lsgb_solver_synth(lsgb_solver* s, const lsgb_synth* d);

#ifdef __cplusplus
}
#endif

#endif /* LSGB_H */
