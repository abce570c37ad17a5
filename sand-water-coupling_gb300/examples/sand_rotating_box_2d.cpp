// sand_rotating_box_2d.cpp -- C++ caller of the GB300 DEMParticleSand (the
// reference-shaped class in include/swc/DEMParticleSand.hpp): the 2D scene of
// DEMParticleSandBuilder case 0 at scale 30 (a hexagonally packed box of half-length
// 1/8 rotating at 2 rad/s, boundary particles of the box [-1/2, 1/2]^2 sampled over
// half-length 1.2), stepped as the Simulator does at frame rate 10000 and CFL 0.4;
// prints one line per frame.
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "swc/DEMParticleSand.hpp"
#include "swc/Simulator.hpp"

namespace {

// Shapes::generateBox / BoundaryParticles::addSurface packing in 2D: rows of a
// hexagonal lattice at spacing 2r (Cores/Utilities/Shapes.h:34-46).
template<class Keep>
void packed_box_2d(double r, double half, std::vector<double> & out, Keep keep) {
    const double sp = 2 * r, s3 = std::sqrt(3.0);
    const int xs = int(std::round(half * 2 / sp));
    const int ys = int(std::round((half * 2 / sp - 1) * 2 / s3 + 1));
    const double ox = -(xs - 1) * sp / 2, oy = -(ys - 1) * s3 / 2 * sp / 2;
    for (int j = 0; j < ys; j++)
        for (int i = 0; i < xs - (j & 1); i++) {
            const double x = ox + ((j & 1) ? 0.5 : 0.0) * sp + i * sp, y = oy + j * s3 / 2 * sp;
            if (keep(x, y)) {
                out.push_back(x);
                out.push_back(y);
            }
        }
}

}  // namespace

int main(int argc, char ** argv) {
    const int frames = argc > 1 ? std::atoi(argv[1]) : 10;
    const int scale = 30;
    const double r = 1.0 / 2 / scale / 2, omega = 2.0;
    swc::DEMParticleSand<2> sand(r);
    std::vector<double> pos, vel, bpos, bnrm;
    packed_box_2d(r, 1.0 / 8, pos, [](double, double) { return true; });
    for (size_t i = 0; i < pos.size(); i += 2) {  // Shapes::generateRotate (Shapes.h:95-101)
        vel.push_back(omega * pos[i + 1]);
        vel.push_back(-omega * pos[i]);
    }
    sand.addShape(pos, vel);
    sand.setMass(1000.0 / double(pos.size() / 2));
    // ComplementarySurface(ImplicitBox(-1/2, 1)): points outside or on the box, normals into it
    packed_box_2d(r, 1.2, bpos, [](double x, double y) { return std::fmax(std::fabs(x), std::fabs(y)) >= 0.5; });
    for (size_t i = 0; i < bpos.size(); i += 2) {
        const double px = std::fabs(bpos[i]) - 0.5, py = std::fabs(bpos[i + 1]) - 0.5;
        double nx = std::fmax(px, 0.0) * (bpos[i] < 0 ? -1 : 1), ny = std::fmax(py, 0.0) * (bpos[i + 1] < 0 ? -1 : 1);
        if (px <= 0 && py <= 0) {  // on the box: the axis of the largest coordinate
            nx = px >= py ? (bpos[i] < 0 ? -1 : 1) : 0;
            ny = px >= py ? 0 : (bpos[i + 1] < 0 ? -1 : 1);
        }
        const double l = std::sqrt(nx * nx + ny * ny);
        bnrm.push_back(-nx / l);
        bnrm.push_back(-ny / l);
    }
    sand.setBoundary(bpos, bnrm);
    try {
        sand.initialize();
        const unsigned rate = 10000;
        const double cfl = 0.4, frame = 1.0 / rate;
        // frames of 1 / rate substepped as Simulator::advanceTimeBySteps does
        // (Cores/Physics/Simulator.cpp:103-128)
        swc::Simulator<swc::DEMParticleSand<2>> driver("sand_rotating_box_2d_out", 1, 1, rate, cfl, &sand);
        for (int f = 0; f < frames; f++) {
            const int steps = int(driver.advanceTimeBySteps(frame).size());
            const auto & v = sand.velocities();
            double vmax = 0;
            for (size_t i = 0; i < v.size(); i += 2) vmax = std::fmax(vmax, std::hypot(v[i], v[i + 1]));
            std::printf("frame %d  steps %d  N %zu  boundary %zu  max|v| %.6f\n", f, steps, sand.size(),
                        bpos.size() / 2, vmax);
        }
        sand.saveFrame("sand_rotating_box_2d_out/last");
        sand.writeFrame("sand_rotating_box_2d_out/last");
    } catch (const swc::SandError & e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
