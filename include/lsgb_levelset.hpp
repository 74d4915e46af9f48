// lsgb_levelset.hpp -- C++ mirror of the reference's hot-path functions over
// the lsgb C ABI (include/lsgb.h).
//
// The reference (juhoon196/Level-set-method-code) exposes its solver as
// header-inline C++ functions taking raw arrays and a SimParams struct.  This
// header keeps those names, argument orders and meanings, so a caller of
// Local_code/level-set_MPI_3D (or _2D, or the single-GPU variants) can switch
// by changing includes:
//
//   reference                                          here (device arrays)
//   rk3TimeStep3D        rk3.h:131                     lsgb::rk3TimeStep3D
//   reinitializeWithSwap3D reinitialization.h:199      lsgb::reinitializeWithSwap3D
//   applyBoundaryConditions3D boundary.h:250           lsgb::applyBoundaryConditions3D
//   computeInterfaceVolume io.h:263                    lsgb::computeInterfaceVolume
//   computeL2Error3D     io.h:229                      lsgb::computeL2Error3D
//   calculateTimeStep    config.h:272                  lsgb::calculateTimeStep (field max)
//   saveFieldBinary3D    io.h:33                       lsgb::saveFieldBinary3D (device array)
//   2D: rk3TimeStep (2D rk3.h:168), reinitializeWithSwap (2D reinitialization.h:321),
//       applyBoundaryConditions (2D boundary.h:217), computeInterfaceArea (2D io.h:225),
//       computeL2Error (2D io.h:194), saveFieldBinary (2D io.h:26)
//
// The caller's own SimParams type is read field by field (any struct with the
// reference's member names works).  Arrays are CUDA device arrays in the
// reference's ghosted layout, as in Local_code/level-set_GPU_3D.  Where the
// reference aborts the process on a CUDA error (config.cuh CUDA_CHECK), these
// wrappers throw lsgb::Error with the library's message.
#pragma once

#include <cstdio>
#include <stdexcept>
#include <string>

#include "lsgb.h"

namespace lsgb {

#ifndef LSGB_ERROR_DEFINED
#define LSGB_ERROR_DEFINED
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc) {
    if (rc != LSGB_OK) throw Error(rc, std::string("lsgb: ") + lsgb_last_error());
}
#endif

// Reference SimParams (3D, Local_code/level-set_MPI_3D/include/config.h:134-175)
// -> lsgb_params.  Periodic on every axis, as applyBoundaryConditions3D.
template <class SimParams>
inline lsgb_params params3d(const SimParams& sp) {
    lsgb_params p;
    lsgb_params_default(&p, 3, sp.nx, sp.ny, sp.nz);
    p.dx = sp.dx; p.dy = sp.dy; p.dz = sp.dz;
    p.s_l = sp.s_l;
    p.dt = sp.dt;
    p.cfl = sp.cfl;
    p.epsilon = sp.epsilon;
    p.enable_reinit = sp.enable_reinit ? 1 : 0;
    p.reinit_interval = sp.reinit_interval;
    p.reinit_iterations = sp.reinit_iterations;
    p.reinit_dtau = sp.reinit_dtau;
    p.reinit_beta = sp.reinit_beta;
    return p;
}

// Reference SimParams (2D, Local_code/level-set_MPI_2D/include/config.h:123-160).
// Periodic X; Y periodic when the rank is its own Y neighbour, zero-gradient
// at the ends otherwise (boundary.h:217-229 with one rank).
template <class SimParams>
inline lsgb_params params2d(const SimParams& sp, bool periodic_y) {
    lsgb_params p;
    lsgb_params_default(&p, 2, sp.nx, sp.ny, 1);
    p.dx = sp.dx; p.dy = sp.dy;
    p.s_l = sp.s_l;
    p.dt = sp.dt;
    p.cfl = sp.cfl;
    p.epsilon = sp.epsilon;
    p.enable_reinit = sp.enable_reinit ? 1 : 0;
    p.reinit_interval = sp.reinit_interval;
    p.reinit_iterations = sp.reinit_iterations;
    p.reinit_dtau = sp.reinit_dtau;
    p.reinit_beta = sp.reinit_beta;
    p.bc_y = periodic_y ? LSGB_BC_PERIODIC : LSGB_BC_ZERO_GRADIENT;
    return p;
}

// ---- 3D ---------------------------------------------------------------------
// G_rhs is accepted for signature compatibility and not touched (the RHS is
// fused into each stage kernel).
template <class SimParams>
inline void rk3TimeStep3D(double* G_n, double* G_new, double* G_1, double* G_2, double* /*G_rhs*/,
                          const double* u, const double* v, const double* w, SimParams& params,
                          void* stream = nullptr) {
    lsgb_params p = params3d(params);
    check(lsgb_rk3_step_f64(&p, G_n, G_new, G_1, G_2, u, v, w, nullptr, stream));
}

template <class SimParams>
inline void reinitializeWithSwap3D(double** phi, double** phi_tmp, double* phi0, double* r_tilde,
                                   int* interface_flag, SimParams& params, void* stream = nullptr) {
    if (!params.enable_reinit) return;  // reinitialization.h:202
    lsgb_params p = params3d(params);
    check(lsgb_reinit_f64(&p, phi, phi_tmp, phi0, r_tilde, reinterpret_cast<int32_t*>(interface_flag), stream));
}

template <class SimParams>
inline void applyBoundaryConditions3D(double* G, SimParams& params, void* stream = nullptr) {
    lsgb_params p = params3d(params);
    check(lsgb_apply_bc_f64(&p, G, stream));
}

template <class SimParams>
inline double computeInterfaceVolume(const double* G, SimParams& params, void* stream = nullptr) {
    lsgb_params p = params3d(params);
    double v = 0.0;
    check(lsgb_volume_f64(&p, G, &v, nullptr, stream));
    return v;
}

template <class SimParams>
inline double computeL2Error3D(const double* G, const double* G_ref, SimParams& params,
                               void* stream = nullptr) {
    lsgb_params p = params3d(params);
    double l2 = 0.0;
    check(lsgb_l2_error_f64(&p, G, G_ref, &l2, stream));
    return l2;
}

// calculateTimeStep with the velocity maximum taken over the field.
template <class SimParams>
inline double calculateTimeStep(const SimParams& params, const double* u, const double* v,
                                const double* w, void* stream = nullptr) {
    if (params.dt > 0.0) return params.dt;  // config.h:275-277
    lsgb_params p = params3d(params);
    double ms = 0.0, dt = 0.0;
    check(lsgb_max_speed_f64(&p, u, v, w, &ms, stream));
    check(lsgb_cfl_dt(&p, ms, &dt));
    return dt;
}

// ---- 2D ---------------------------------------------------------------------
template <class SimParams>
inline void rk3TimeStep(double* G_n, double* G_new, double* G_1, double* G_2, double* /*G_rhs*/,
                        const double* u, const double* v, SimParams& params, bool periodic_y = true,
                        void* stream = nullptr) {
    lsgb_params p = params2d(params, periodic_y);
    check(lsgb_rk3_step_f64(&p, G_n, G_new, G_1, G_2, u, v, nullptr, nullptr, stream));
}

template <class SimParams>
inline void reinitializeWithSwap(double** phi, double** phi_tmp, double* phi0, double* r_tilde,
                                 int* interface_flag, SimParams& params, bool periodic_y = true,
                                 void* stream = nullptr) {
    if (!params.enable_reinit) return;  // 2D reinitialization.h:325
    lsgb_params p = params2d(params, periodic_y);
    check(lsgb_reinit_f64(&p, phi, phi_tmp, phi0, r_tilde, reinterpret_cast<int32_t*>(interface_flag), stream));
}

template <class SimParams>
inline void applyBoundaryConditions(double* G, SimParams& params, bool periodic_y = true,
                                    void* stream = nullptr) {
    lsgb_params p = params2d(params, periodic_y);
    check(lsgb_apply_bc_f64(&p, G, stream));
}

template <class SimParams>
inline double computeInterfaceArea(const double* G, SimParams& params, bool periodic_y = true,
                                   void* stream = nullptr) {
    lsgb_params p = params2d(params, periodic_y);
    double a = 0.0;
    check(lsgb_volume_f64(&p, G, &a, nullptr, stream));
    return a;
}

template <class SimParams>
inline double computeL2Error(const double* G, const double* G_ref, SimParams& params,
                             bool periodic_y = true, void* stream = nullptr) {
    lsgb_params p = params2d(params, periodic_y);
    double l2 = 0.0;
    check(lsgb_l2_error_f64(&p, G, G_ref, &l2, stream));
    return l2;
}

// ---- RAII handle over the device-resident fast path ---------------------------
// The reference's binary dump of a ghosted device array: int32 header, then
// the array with its y ghosts copied from the nearest interior row
// (saveFieldBinary3D, io.h:33-131; the 2D saveFieldBinary, 2D io.h:26-109).
// current_time is accepted for the signature; the reference does not write it.
inline bool write_dump_file(const char* filename, const lsgb_params& p, const double* G) {
    size_t n = 0;
    check(lsgb_dump_bytes(&p, &n));
    std::string buf(n, '\0');
    check(lsgb_dump_f64(&p, G, &buf[0], LSGB_MEM_HOST, nullptr));
    FILE* fp = std::fopen(filename, "wb");
    if (!fp) return false;
    const bool ok = std::fwrite(buf.data(), 1, n, fp) == n;
    return std::fclose(fp) == 0 && ok;
}

template <class SimParams>
inline bool saveFieldBinary3D(const char* filename, const double* G, SimParams& params, double current_time = 0.0) {
    (void)current_time;
    return write_dump_file(filename, params3d(params), G);
}

template <class SimParams>
inline bool saveFieldBinary(const char* filename, const double* G, SimParams& params, bool periodic_y = true) {
    return write_dump_file(filename, params2d(params, periodic_y), G);
}

class Solver {
  public:
    Solver(const lsgb_params& p, int precision = LSGB_PREC_F64) { check(lsgb_solver_create(&p, precision, &h_)); }
    ~Solver() { lsgb_solver_destroy(h_); }
    Solver(const Solver&) = delete;
    Solver& operator=(const Solver&) = delete;

    void setFields(const double* G, const double* u, const double* v, const double* w,
                   int layout = LSGB_LAYOUT_GHOSTED, int memory = LSGB_MEM_HOST) {
        check(lsgb_solver_set_fields(h_, G, u, v, w, layout, memory));
    }
    void advance(int n_steps) { check(lsgb_solver_advance(h_, n_steps)); }
    void getG(double* G, int layout = LSGB_LAYOUT_GHOSTED, int memory = LSGB_MEM_HOST) {
        check(lsgb_solver_get_G(h_, G, layout, memory));
    }
    double volume() {
        double v = 0.0;
        check(lsgb_solver_volume(h_, &v, nullptr));
        return v;
    }
    double computeDt(double cfl) {
        double dt = 0.0;
        check(lsgb_solver_compute_dt(h_, cfl, &dt));
        return dt;
    }
    // The deformation test's per-step velocity (updateDeformationVelocity before
    // every rk3TimeStep3D, src/main.cpp:297-299) kept inside advance(): the
    // vortex at the handle's time, which starts at t and advances by dt a step.
    void deformationVelocityLive(double t, double t_final) {
        check(lsgb_solver_set_velocity_deformation_live(h_, t, t_final));
    }
    double time() const {
        double t = 0.0;
        check(lsgb_solver_get_time(h_, &t));
        return t;
    }
    lsgb_solver* handle() { return h_; }

  private:
    lsgb_solver* h_ = nullptr;
};

}  // namespace lsgb
