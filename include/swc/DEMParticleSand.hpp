// DEMParticleSand.hpp -- C++20 drop-in for PhysX::DEMParticleSand<Dim>
// (Cores/Physics/DEMParticleSand.{h,cpp} of skytang0205/sand-water-coupling)
// running on one GB300 through the C ABI in swc_sand.h.
//
// Same method names and meaning as the reference's Simulation interface
// (Cores/Physics/Simulation.h:25-34): initialize(), advance(dt),
// getTimeStep(frameRate, stepRate), dimension(), writeFrame(frameDir, staticDraw),
// saveFrame(frameDir), loadFrame(frameDir); plus addShape (DEMParticleSand.cpp:167-175)
// and the DEMParticle setters setYoung / setPoisson / setfricangle
// (Cores/Structures/DEMParticle.cpp:44-60), which apply from the next initialize().
// Positions and velocities are FP64 arrays of Dim components per particle.
// Errors throw swc::SandError carrying the swc_status code.
#pragma once

#include <cmath>
#include <cstdint>
#include <filesystem>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../swc_sand.h"

namespace swc {

class SandError : public std::runtime_error {
public:
    SandError(int status, const std::string & where, const std::string & detail)
        : std::runtime_error(where + ": " + swc_status_str(status) + (detail.empty() ? "" : " (" + detail + ")")),
          status_(status) {}
    int status() const { return status_; }

private:
    int status_;
};

template<int Dim> class DEMParticleSand {
    static_assert(Dim == 2 || Dim == 3, "Dimension must be 2 or 3.");

public:
    // DEMParticleSand(particleRadius) (DEMParticleSand.h:30-31).
    explicit DEMParticleSand(double particleRadius) {
        swc_sand_default_params(&params_);
        params_.dim    = Dim;
        params_.radius = particleRadius;
    }
    DEMParticleSand(const DEMParticleSand &)             = delete;
    DEMParticleSand & operator=(const DEMParticleSand &) = delete;
    ~DEMParticleSand() {
        if (ctx_) swc_sand_destroy(ctx_);
    }

    void setYoung(double k) { params_.young = k; }
    void setPoisson(double k) { params_.poisson = k; }
    void setfricangle(double k) { params_.fric_angle = k; }
    void setMass(double m) { params_.mass = m; }
    void enableGravity(bool on) { params_.enable_gravity = on ? 1 : 0; }

    void addShape(const std::vector<double> & pos, const std::vector<double> & vel) {
        pull();
        pos_.insert(pos_.end(), pos.begin(), pos.end());
        vel_.insert(vel_.end(), vel.begin(), vel.end());
        dirty_ = true;
    }
    // BoundaryParticles::addSurface result: positions and normals (DEMParticleSandBuilder.h:46-50).
    void setBoundary(const std::vector<double> & pos, const std::vector<double> & normals) {
        bpos_ = pos;
        bnrm_ = normals;
    }

    int dimension() const { return Dim; }
    size_t size() const { return pos_.size() / Dim; }

    void initialize() {
        if (ctx_) swc_sand_destroy(ctx_);
        ctx_ = nullptr;
        check(swc_sand_create(&params_, &ctx_), "swc_sand_create");
        check(swc_sand_set_particles(ctx_, pos_.data(), vel_.data(), int64_t(size())), "swc_sand_set_particles");
        check(swc_sand_set_boundary(ctx_, bpos_.data(), bnrm_.data(), int64_t(bpos_.size() / Dim)),
              "swc_sand_set_boundary");
        check(swc_sand_initialize(ctx_), "swc_sand_initialize");
        dirty_ = false;
    }

    void advance(double dt) {
        push();
        check(swc_sand_advance(ctx_, dt), "swc_sand_advance");
        stale_ = true;
    }

    double getTimeStep(unsigned frameRate, double stepRate) {
        (void) frameRate;
        push();
        double dt = 0;
        check(swc_sand_get_time_step(ctx_, stepRate, &dt), "swc_sand_get_time_step");
        return dt;
    }

    const std::vector<double> & positions() { return pull(), pos_; }
    const std::vector<double> & velocities() { return pull(), vel_; }

    // saveFrame / loadFrame: particles.sav, velocities.sav as raw FP64 (DEMParticleSand.cpp:55-76).
    void saveFrame(const std::string & frameDir) {
        std::filesystem::create_directories(frameDir);
        pull();
        writeRaw(frameDir + "/particles.sav", pos_);
        writeRaw(frameDir + "/velocities.sav", vel_);
    }
    void loadFrame(const std::string & frameDir) {
        pos_   = readRaw(frameDir + "/particles.sav");
        vel_   = readRaw(frameDir + "/velocities.sav");
        dirty_ = true;
        stale_ = false;
    }
    // particles.mesh: count, positions, unit-z normals in 3D, |v| (DEMParticleSand.cpp:31-41).
    void writeFrame(const std::string & frameDir, bool staticDraw = false) {
        (void) staticDraw;
        std::filesystem::create_directories(frameDir);
        pull();
        std::ofstream f(frameDir + "/particles.mesh", std::ios::binary);
        const uint32_t cnt = uint32_t(size());
        f.write(reinterpret_cast<const char *>(&cnt), 4);
        for (double p : pos_) {
            const float v = float(p);
            f.write(reinterpret_cast<const char *>(&v), 4);
        }
        if constexpr (Dim == 3) {
            const float z[3] = {0, 0, 1};
            for (size_t i = 0; i < size(); i++) f.write(reinterpret_cast<const char *>(z), 12);
        }
        for (size_t i = 0; i < size(); i++) {
            double s = 0;
            for (int a = 0; a < Dim; a++) s += vel_[i * Dim + a] * vel_[i * Dim + a];
            const float v = float(std::sqrt(s));
            f.write(reinterpret_cast<const char *>(&v), 4);
        }
    }

private:
    void check(int rc, const char * where) const {
        if (rc != SWC_OK) throw SandError(rc, where, ctx_ ? swc_sand_last_error(ctx_) : "");
    }
    void push() {
        if (!ctx_) initialize();
        if (dirty_) {
            check(swc_sand_set_particles(ctx_, pos_.data(), vel_.data(), int64_t(size())), "swc_sand_set_particles");
            dirty_ = false;
        }
    }
    void pull() {
        if (stale_ && ctx_) {
            check(swc_sand_get_particles(ctx_, pos_.data(), vel_.data(), int64_t(size())), "swc_sand_get_particles");
            stale_ = false;
        }
    }
    static void writeRaw(const std::string & path, const std::vector<double> & a) {
        std::ofstream f(path, std::ios::binary);
        f.write(reinterpret_cast<const char *>(a.data()), std::streamsize(a.size() * sizeof(double)));
    }
    static std::vector<double> readRaw(const std::string & path) {
        std::ifstream f(path, std::ios::binary | std::ios::ate);
        if (!f) throw SandError(SWC_BAD_ARG, "loadFrame", "cannot open " + path);
        const auto bytes = size_t(f.tellg());
        std::vector<double> a(bytes / sizeof(double));
        f.seekg(0);
        f.read(reinterpret_cast<char *>(a.data()), std::streamsize(bytes));
        return a;
    }

    swc_sand_params params_{};
    swc_sand * ctx_ = nullptr;
    std::vector<double> pos_, vel_, bpos_, bnrm_;
    bool dirty_ = false, stale_ = false;
};

}  // namespace swc
