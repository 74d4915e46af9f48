// lsgb_sample.hpp -- C++ mirror of the reference's sample surface
// (sample/field.hpp, sample/weno5_rk3.hpp, the dump helpers of
// sample/main.cpp) over the lsgb C ABI (include/lsgb.h, lsgb_sample_*).
//
//   reference                                   here
//   Field2D(int nx, int ny)   field.hpp:10      lsgb::sample::Field2D (device storage)
//   Field2D::fill             field.hpp:12      Field2D::fill
//   Field2D::apply_periodic   field.hpp:15      Field2D::apply_periodic
//   Field2D::apply_anchored_bc field.hpp:18     Field2D::apply_anchored_bc
//   Field2D::reinitialize     field.hpp:21      Field2D::reinitialize
//   compute_geqn_rhs          weno5_rk3.hpp:10  lsgb::sample::compute_geqn_rhs (Field2D arguments)
//   RK3_step                  weno5_rk3.hpp:20  lsgb::sample::RK3_step (same signature)
//   compute_first_order_upwind first_order_upwind.hpp:4
//                                               lsgb::sample::compute_first_order_upwind (Field2D arguments)
//   save_G_to_bin             main.cpp:34       lsgb::sample::save_G_to_bin
//   load_field_from_bin       main.cpp:16       lsgb::sample::load_field_from_bin
//
// The reference's Field2D keeps data[ny+6][nx+6] in host vectors; this one
// keeps the same elements, row-major, in one device array (`dev`), and
// moves them with upload / download.  Arithmetic results are those of the
// reference bit for bit.  Errors throw lsgb::Error (the reference exits).
#pragma once

#include <cuda_runtime.h>

#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

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

namespace sample {

inline void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw Error(LSGB_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

class Field2D {
  public:
    int nx, ny;           // interior size (field.hpp:7)
    double* dev = nullptr;  // [ny+6][nx+6], row-major, device memory

    Field2D(int nx_, int ny_) : nx(nx_), ny(ny_) {
        cuda_check(cudaMalloc((void**)&dev, bytes()), "Field2D allocation");
        cuda_check(cudaMemset(dev, 0, bytes()), "Field2D zero fill");  // the reference zero-fills
    }
    ~Field2D() { if (dev) cudaFree(dev); }
    Field2D(const Field2D& o) : nx(o.nx), ny(o.ny) {
        cuda_check(cudaMalloc((void**)&dev, bytes()), "Field2D allocation");
        cuda_check(cudaMemcpy(dev, o.dev, bytes(), cudaMemcpyDeviceToDevice), "Field2D copy");
    }
    Field2D& operator=(const Field2D& o) {
        if (this != &o) {
            if (o.nx != nx || o.ny != ny) throw Error(LSGB_ERR_INVALID, "Field2D assignment between sizes");
            cuda_check(cudaMemcpy(dev, o.dev, bytes(), cudaMemcpyDeviceToDevice), "Field2D copy");
        }
        return *this;
    }

    size_t count() const { return (size_t)(nx + 6) * (ny + 6); }
    size_t bytes() const { return count() * sizeof(double); }

    void fill(double value = 0.0) {
        std::vector<double> h(count(), value);
        upload(h.data());
    }
    void upload(const double* host) { cuda_check(cudaMemcpy(dev, host, bytes(), cudaMemcpyHostToDevice), "upload"); }
    void download(double* host) const { cuda_check(cudaMemcpy(host, dev, bytes(), cudaMemcpyDeviceToHost), "download"); }

    void apply_periodic() { check(lsgb_sample_apply_periodic(nx, ny, dev, nullptr)); }
    void apply_anchored_bc(const Field2D& initial) {
        check(lsgb_sample_apply_anchored_bc(nx, ny, dev, initial.dev, nullptr));
    }
    void reinitialize(const Field2D& initial, double dx, double dy, int num_iters) {
        check(lsgb_sample_reinitialize(nx, ny, dev, initial.dev, dx, dy, num_iters, nullptr, nullptr));
    }
};

inline void compute_geqn_rhs(const Field2D& G, const Field2D& u, const Field2D& v, Field2D& rhs, double dx,
                             double dy, double S_L) {
    check(lsgb_sample_rhs(G.nx, G.ny, G.dev, u.dev, v.dev, rhs.dev, dx, dy, S_L, nullptr));
}

inline void RK3_step(Field2D& G_field, const Field2D& u_field, const Field2D& v_field, double dx, double dy,
                     double dt, double S_L, const Field2D& G_initial) {
    check(lsgb_sample_rk3_step(G_field.nx, G_field.ny, G_field.dev, u_field.dev, v_field.dev, dx, dy, dt, S_L,
                               G_initial.dev, nullptr, nullptr));
}

inline void compute_first_order_upwind(Field2D& G, const Field2D& u, const Field2D& v, double dx, double dy,
                                       double dt, double S_L) {
    check(lsgb_sample_first_order_upwind(G.nx, G.ny, G.dev, u.dev, v.dev, dx, dy, dt, S_L, nullptr, nullptr));
}

// Interior rows only, each nx doubles, no header (main.cpp:34-51): the
// files sample/read_G.m reads.
inline void save_G_to_bin(const Field2D& G, const std::string& filename) {
    std::vector<double> h(G.count());
    G.download(h.data());
    FILE* f = std::fopen(filename.c_str(), "wb");
    if (!f) throw Error(LSGB_ERR_INVALID, "cannot open " + filename);
    const size_t nxT = (size_t)G.nx + 6;
    for (int j = 3; j <= G.ny + 2; ++j) std::fwrite(h.data() + j * nxT + 3, sizeof(double), (size_t)G.nx, f);
    std::fclose(f);
}

// The reference's loader (main.cpp:16-32) reads ny rows of nx doubles into
// rows 2 .. ny+1 starting at column 2, one cell up and left of where
// save_G_to_bin took them; this keeps that placement.
inline void load_field_from_bin(Field2D& field, const std::string& filename, int nx, int ny) {
    std::vector<double> h(field.count());
    field.download(h.data());
    FILE* f = std::fopen(filename.c_str(), "rb");
    if (!f) throw Error(LSGB_ERR_INVALID, "file not found: " + filename);
    const size_t nxT = (size_t)field.nx + 6;
    for (int j = 2; j <= ny + 1; ++j)
        if (std::fread(h.data() + j * nxT + 2, sizeof(double), (size_t)nx, f) != (size_t)nx) {
            std::fclose(f);
            throw Error(LSGB_ERR_INVALID, "short read: " + filename);
        }
    std::fclose(f);
    field.upload(h.data());
}

}  // namespace sample
}  // namespace lsgb
