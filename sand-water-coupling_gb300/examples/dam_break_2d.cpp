// dam_break_2d.cpp -- C++ caller of the GB300 DualParticleSphLiquid (the
// reference-shaped class in include/swc/DualParticleSphLiquid.hpp): the 2D dam
// break (40 x 80 particles at 0.01 in [0,1]^2, two wall layers, gravity,
// dt 1e-3), advanced `steps` times; prints one line per step.
//   dam_break_2d <steps> frames <F>: instead, F frames at 100 frames/s through
//   swc::Simulator (CFL 0.5 substeps, frame files under dam_break_2d_frames/);
//   prints one line per substep and one per frame.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>

#include "swc/DualParticleSphLiquid.hpp"
#include "swc/Simulator.hpp"

int main(int argc, char ** argv) {
    const int steps = argc > 1 ? std::atoi(argv[1]) : 10;
    const double sp = 0.01, r = sp / 2, m = 1000 * sp * sp;
    auto grid = swc::NodeGrid<2>::staggered(3, sp, {100, 100}, {0.5, 0.5});
    swc_solver_opts o;
    swc_default_solver_opts(&o);
    swc::DualParticleSphLiquid<2> liquid(grid, r, m, &o);
    liquid.enableGravity(true);
    liquid.setKappa(m / 1000);
    std::mt19937_64 rng(0);
    std::uniform_real_distribution<double> jit(-1e-4, 1e-4);
    std::vector<double> pos, vel, bpos, bnrm;
    for (int j = 0; j < 80; j++)
        for (int i = 0; i < 40; i++) {
            pos.push_back((i + 0.5) * sp + jit(rng));
            pos.push_back((j + 0.5) * sp + jit(rng));
            vel.push_back(0);
            vel.push_back(0);
        }
    for (int j = -2; j < 102; j++)
        for (int i = -2; i < 102; i++) {
            if (i >= 0 && i < 100 && j >= 0 && j < 100) continue;
            const double x = (i + 0.5) * sp, y = (j + 0.5) * sp;
            double nx = x < 0 ? 1 : (x > 1 ? -1 : 0), ny = y < 0 ? 1 : (y > 1 ? -1 : 0);
            const double l = std::sqrt(nx * nx + ny * ny);
            bpos.push_back(x);
            bpos.push_back(y);
            bnrm.push_back(nx / l);
            bnrm.push_back(ny / l);
        }
    liquid.addParticles(pos, vel);
    liquid.setBoundary(bpos, bnrm);
    try {
        if (argc > 3 && std::string(argv[2]) == "frames") {
            swc::Simulator<swc::DualParticleSphLiquid<2>> sim("dam_break_2d_frames", 0, unsigned(std::atoi(argv[3])) + 1,
                                                              100, 0.5, &liquid);
            sim.onSubstep = [&](double dt) {
                std::printf("substep dt %.17g  cg %d\n", dt, liquid.lastStats().cg_iterations);
            };
            sim.onFrame = [](unsigned f) { std::printf("frame %u\n", f); };
            sim.Simulate();
            return 0;
        }
        liquid.initialize();
        for (int s = 0; s < steps; s++) {
            liquid.advance(1e-3);
            const auto & st = liquid.lastStats();
            std::printf("step %d  N_v %lld  cg %d  |r|/|b| %.2e  %.3f ms\n", s, (long long) st.n_virtual,
                        st.cg_iterations, st.rel_residual, st.device_ms);
        }
        liquid.saveFrame("dam_break_2d_out/last");
    } catch (const swc::Error & e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
