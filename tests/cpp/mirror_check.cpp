// Drives the C++ mirror (include/lsgb_levelset.hpp) the way the reference's
// driver drives its own functions (Local_code/level-set_MPI_3D/src/main.cpp:
// rk3TimeStep3D, swap, reinitializeWithSwap3D, computeInterfaceVolume), on
// device arrays.  Reads G,u,v,w (ghosted FP64, raw) from argv[1]..argv[4],
// runs n steps with reinit every `interval`, writes G to argv[5] and prints
// the volume.  Built and run by tests/test_cpp_mirror.py.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "lsgb_levelset.hpp"

// The caller's own parameter struct: the reference's member names.
struct SimParams {
    int nx, ny, nz;
    double dx, dy, dz;
    double s_l, dt, cfl, epsilon;
    bool enable_reinit;
    int reinit_interval, reinit_iterations;
    double reinit_dtau, reinit_beta;
};

static std::vector<double> read_all(const char* path, size_t n) {
    std::vector<double> v(n);
    FILE* f = std::fopen(path, "rb");
    if (!f || std::fread(v.data(), sizeof(double), n, f) != n) { std::fprintf(stderr, "read %s\n", path); std::exit(2); }
    std::fclose(f);
    return v;
}

int main(int argc, char** argv) {
    if (argc < 12) { std::fprintf(stderr, "usage\n"); return 2; }
    SimParams sp{};
    sp.nx = std::atoi(argv[6]); sp.ny = std::atoi(argv[7]); sp.nz = std::atoi(argv[8]);
    sp.dx = 1.0 / sp.nx; sp.dy = 1.0 / sp.ny; sp.dz = 1.0 / sp.nz;
    sp.s_l = std::atof(argv[9]);
    sp.dt = std::atof(argv[10]);
    sp.cfl = 0.5;
    sp.epsilon = 1e-10;
    sp.enable_reinit = true;
    sp.reinit_interval = 3;
    sp.reinit_iterations = 3;
    sp.reinit_dtau = 0.25 * (sp.dx < sp.dy ? (sp.dx < sp.dz ? sp.dx : sp.dz) : (sp.dy < sp.dz ? sp.dy : sp.dz));
    sp.reinit_beta = 0.5;
    int nsteps = std::atoi(argv[11]);
    size_t n = (size_t)(sp.nx + 6) * (sp.ny + 6) * (sp.nz + 6);
    size_t b = n * sizeof(double);
    double *G, *Gn, *G1, *G2, *u, *v, *w, *tmp, *phi0, *rt;
    int* flag;
    double** bufs[] = {&G, &Gn, &G1, &G2, &u, &v, &w, &tmp, &phi0, &rt};
    for (double** q : bufs) cudaMalloc((void**)q, b);
    cudaMalloc((void**)&flag, n * sizeof(int));
    const char* names[4] = {argv[1], argv[2], argv[3], argv[4]};
    double* dst[4] = {G, u, v, w};
    for (int q = 0; q < 4; ++q) {
        auto h = read_all(names[q], n);
        cudaMemcpy(dst[q], h.data(), b, cudaMemcpyHostToDevice);
    }
    try {
        // initial boundary fill of G and the velocity (src/main.cpp:259-260)
        lsgb::applyBoundaryConditions3D(G, sp);
        lsgb::applyBoundaryConditions3D(u, sp);
        lsgb::applyBoundaryConditions3D(v, sp);
        lsgb::applyBoundaryConditions3D(w, sp);
        for (int step = 0; step < nsteps; ++step) {
            lsgb::rk3TimeStep3D(G, Gn, G1, G2, nullptr, u, v, w, sp);
            double* t = G; G = Gn; Gn = t;
            if (sp.enable_reinit && step > 0 && step % sp.reinit_interval == 0)
                lsgb::reinitializeWithSwap3D(&G, &tmp, phi0, rt, flag, sp);
        }
        double vol = lsgb::computeInterfaceVolume(G, sp);
        std::vector<double> out(n);
        cudaMemcpy(out.data(), G, b, cudaMemcpyDeviceToHost);
        FILE* f = std::fopen(argv[5], "wb");
        std::fwrite(out.data(), sizeof(double), n, f);
        std::fclose(f);
        std::printf("volume %.17g\n", vol);
        // the reference's end-of-run dump (src/main.cpp:378)
        if (argc > 12 && !lsgb::saveFieldBinary3D(argv[12], G, sp, 0.0)) return 3;
    } catch (const lsgb::Error& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
