// Drives the sample-surface mirror (include/lsgb_sample.hpp) the way the
// reference's sample/main.cpp drives Field2D and RK3_step: anchored and
// periodic boundaries, the forced uniform velocity, RK3_step, boundaries,
// t += dt; then save_G_to_bin.  Reads the initial G (raw [ny+6][nx+6]
// doubles) from argv[1], writes the interior dump to argv[2].
//   sample_check G0.bin out.bin nx ny dt steps freq
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "lsgb_levelset.hpp"
#include "lsgb_sample.hpp"

using lsgb::sample::Field2D;

int main(int argc, char** argv) {
    if (argc < 8) { std::fprintf(stderr, "usage\n"); return 2; }
    const int nx = std::atoi(argv[3]), ny = std::atoi(argv[4]);
    const double dt = std::atof(argv[5]);
    const int steps = std::atoi(argv[6]), freq = std::atoi(argv[7]);
    const double LX = 0.02, LY = 0.02, DX = LX / (nx - 1), DY = LY / (ny - 1), SL = 0.4;
    const double u0 = 0.0, v0 = 0.8, epsilon_u = 0.05, epsilon_v = 0.05;
    std::vector<double> h((size_t)(nx + 6) * (ny + 6));
    FILE* f = std::fopen(argv[1], "rb");
    if (!f || std::fread(h.data(), sizeof(double), h.size(), f) != h.size()) { std::fprintf(stderr, "read\n"); return 2; }
    std::fclose(f);
    try {
        Field2D G(nx, ny), u(nx, ny), v(nx, ny), G_initial(nx, ny);
        G.upload(h.data());
        G_initial.upload(h.data());
        double t = 0.0;
        for (int step = 0; step < steps; ++step) {
            G.apply_anchored_bc(G_initial);
            G.apply_periodic();
            u.fill(u0 + epsilon_u * v0 * cos(freq * 2 * M_PI * (t)));
            v.fill(v0 + epsilon_v * v0 * cos(freq * 2 * M_PI * (t)));
            lsgb::sample::RK3_step(G, u, v, DX, DY, dt, SL, G_initial);
            G.apply_periodic();
            G.apply_anchored_bc(G_initial);
            t += dt;
        }
        lsgb::sample::save_G_to_bin(G, argv[2]);
        std::printf("t %.17g\n", t);
    } catch (const lsgb::Error& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
