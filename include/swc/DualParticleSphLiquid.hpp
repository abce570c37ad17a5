// DualParticleSphLiquid.hpp -- C++20 drop-in for PhysX::DualParticleSphLiquid<Dim>
// (Cores/Physics/DualParticleSphLiquid.{h,cpp} of skytang0205/sand-water-coupling)
// running on one GB300 through the C ABI in swc.h.
//
// Same method names and meaning as the reference's Simulation interface
// (Cores/Physics/Simulation.h:25-34):
//   initialize(), advance(dt), getTimeStep(frameRate, stepRate), dimension(),
//   writeDescription(path), writeFrame(frameDir, staticDraw), saveFrame(frameDir),
//   loadFrame(frameDir); swc::Simulator (Simulator.hpp) drives it frame by frame.
// Positions and velocities are exchanged as FP64 arrays of Dim components per
// particle (the reference's VectorDr storage order).  Errors throw
// swc::Error carrying the swc_status code instead of calling std::exit.
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../swc.h"

namespace swc {

class Error : public std::runtime_error {
public:
    Error(int status, const std::string & where, const std::string & detail)
        : std::runtime_error(where + ": " + swc_status_str(status) + (detail.empty() ? "" : " (" + detail + ")")),
          status_(status) {}
    int status() const { return status_; }

private:
    int status_;
};

// Node lattice of StaggeredGrid(boundaryWidth, spacing, resolution, center)
// (Cores/Structures/StaggeredGrid.cpp:20-34): origin and node counts.
template<int Dim> struct NodeGrid {
    std::array<double, 3> origin{};
    std::array<int32_t, 3> size{1, 1, 1};
    double spacing = 0;

    static NodeGrid staggered(int boundaryWidth, double spacing, const std::array<int, Dim> & resolution,
                              const std::array<double, Dim> & center) {
        NodeGrid g;
        g.spacing = spacing;
        for (int a = 0; a < Dim; a++) {
            const int res = resolution[a] + 2 * boundaryWidth;
            g.origin[a]   = center[a] - double(res) * spacing / 2;
            g.size[a]     = res + 1;
        }
        return g;
    }
};

template<int Dim> class DualParticleSphLiquid {
    static_assert(Dim == 2 || Dim == 3, "Dimension must be 2 or 3.");

public:
    // Reference constructor: DualParticleSphLiquid(const StaggeredGrid<Dim>& grid, real particleRadius)
    // with the virtual particles on the grid's nodes (DualParticleSphLiquid.h:27-29).
    DualParticleSphLiquid(const NodeGrid<Dim> & grid, double particleRadius, double mass,
                          const swc_solver_opts * opts = nullptr) {
        std::memset(&scene_, 0, sizeof(scene_));
        scene_.dim             = Dim;
        scene_.enable_gravity  = 0;  // SmthParticleHydrodLiquid::_enableGravity defaults to false
        scene_.particle_radius = particleRadius;
        scene_.mass            = mass;
        scene_.boundary_mass   = mass;
        scene_.grid_spacing    = grid.spacing;
        for (int a = 0; a < 3; a++) {
            scene_.grid_origin[a] = grid.origin[a];
            scene_.grid_size[a]   = grid.size[a];
        }
        scene_.gravity[1]     = -9.8;  // kGravity on component 1 (SmthParticleHydrodLiquid.cpp:86)
        scene_.viscosity      = 0.01;  // _viscosityCoeff (SmthParticleHydrodLiquid.h:28)
        scene_.target_density = -1;    // max rho_i at initialize (DualParticleSphLiquid.cpp:91)
        scene_.kappa          = -1;    // 1 / packed kernel sum (DualParticleSphLiquid.cpp:98)
        if (opts) opts_ = *opts;
        else swc_default_solver_opts(&opts_);
    }
    DualParticleSphLiquid(const DualParticleSphLiquid &)             = delete;
    DualParticleSphLiquid & operator=(const DualParticleSphLiquid &) = delete;
    ~DualParticleSphLiquid() {
        if (ctx_) swc_destroy(ctx_);
    }

    // Optional scene switches before initialize().
    void enableGravity(bool on, const std::array<double, 3> & g = {0, -9.8, 0}) {
        scene_.enable_gravity = on ? 1 : 0;
        for (int a = 0; a < 3; a++) scene_.gravity[a] = g[a];
    }
    void setViscosity(double coeff) { scene_.viscosity = coeff; }
    void setTargetDensity(double rho0) { scene_.target_density = rho0; }
    void setKappa(double kappa) { scene_.kappa = kappa; }

    // SmthParticleHydrodLiquid::addShape (SmthParticleHydrodLiquid.cpp:124-131).
    void addParticles(const std::vector<double> & pos, const std::vector<double> & vel) {
        pos_.insert(pos_.end(), pos.begin(), pos.end());
        vel_.insert(vel_.end(), vel.begin(), vel.end());
        dirty_ = true;
    }
    // BoundaryParticles with inward normals and velocities.
    void setBoundary(const std::vector<double> & pos, const std::vector<double> & normals,
                     const std::vector<double> & vel = {}) {
        bpos_ = pos;
        bnrm_ = normals;
        bvel_ = vel.empty() ? std::vector<double>(pos.size(), 0.0) : vel;
    }

    int dimension() const { return Dim; }

    void initialize() {
        ensure();
        check(swc_initialize(ctx_), "swc_initialize");
    }

    void advance(double dt) {
        ensure();
        const int rc = swc_advance(ctx_, dt, &stats_);
        if (rc != SWC_OK && !(rc == SWC_CG_NOT_CONVERGED && !throwOnNonConvergence)) check(rc, "swc_advance");
        dirty_host_ = true;
    }

    double getTimeStep(unsigned frameRate, double stepRate) const {
        (void) frameRate;
        double dt = 0;
        check(swc_get_time_step(ctx_, stepRate, &dt), "swc_get_time_step");
        return dt;
    }

    const std::vector<double> & positions() { return pull().first; }
    const std::vector<double> & velocities() { return pull().second; }
    const swc_stats & lastStats() const { return stats_; }
    swc_ctx * handle() { return ctx_; }

    // SmthParticleHydrodLiquid::saveFrame / loadFrame: raw FP64 arrays
    // (SmthParticleHydrodLiquid.cpp:34-55, Cores/Utilities/IO.h:19-26), plus dual_state.sav
    // (n, N_v, rho0, alpha0, kappa, V_i[n], p[N_v]) so that a resumed run keeps the
    // initial volumes and scalars: the reference's resume skips initialize
    // (Simulator.cpp:43-45) and loses them.
    void saveFrame(const std::string & frameDir) {
        std::filesystem::create_directories(frameDir);
        pull();
        writeRaw(frameDir + "/particles.sav", pos_);
        writeRaw(frameDir + "/velocities.sav", vel_);
        const int64_t n = int64_t(pos_.size() / Dim), nv = ctx_ ? swc_num_virtual(ctx_) : 0;
        std::vector<double> vol(static_cast<size_t>(n)), p(static_cast<size_t>(std::max<int64_t>(nv, 0)));
        double rho0 = 0, alpha0 = 0, kappa = 0;
        if (ctx_) {
            check(swc_get_real_info(ctx_, nullptr, vol.data(), n), "swc_get_real_info");
            if (nv > 0)
                check(swc_get_virtual(ctx_, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, p.data(), nv),
                      "swc_get_virtual");
            check(swc_get_scalars(ctx_, &rho0, &alpha0, &kappa), "swc_get_scalars");
        }
        std::ofstream f(frameDir + "/dual_state.sav", std::ios::binary);
        const int64_t hdr[2] = {n, int64_t(p.size())};
        const double  sc[3]  = {rho0, alpha0, kappa};
        f.write(reinterpret_cast<const char *>(hdr), sizeof(hdr));
        f.write(reinterpret_cast<const char *>(sc), sizeof(sc));
        f.write(reinterpret_cast<const char *>(vol.data()), std::streamsize(vol.size() * sizeof(double)));
        f.write(reinterpret_cast<const char *>(p.data()), std::streamsize(p.size() * sizeof(double)));
    }
    void loadFrame(const std::string & frameDir) {
        pos_ = readRaw(frameDir + "/particles.sav");
        vel_ = readRaw(frameDir + "/velocities.sav");
        dirty_ = true;
        ensure();
        check(swc_initialize(ctx_), "swc_initialize");  // boundary information
        std::ifstream f(frameDir + "/dual_state.sav", std::ios::binary);
        if (!f) return;
        int64_t hdr[2];
        double  sc[3];
        f.read(reinterpret_cast<char *>(hdr), sizeof(hdr));
        f.read(reinterpret_cast<char *>(sc), sizeof(sc));
        std::vector<double> vol(static_cast<size_t>(hdr[0])), p(static_cast<size_t>(hdr[1]));
        f.read(reinterpret_cast<char *>(vol.data()), std::streamsize(vol.size() * sizeof(double)));
        f.read(reinterpret_cast<char *>(p.data()), std::streamsize(p.size() * sizeof(double)));
        if (!f) throw Error(SWC_BAD_ARG, "loadFrame", "truncated " + frameDir + "/dual_state.sav");
        check(swc_set_volumes(ctx_, vol.data(), hdr[0]), "swc_set_volumes");
        check(swc_set_scalars(ctx_, sc[0], sc[1], sc[2]), "swc_set_scalars");
        check(swc_set_pressure(ctx_, p.data(), hdr[1]), "swc_set_pressure");
    }
    // description.yaml objects of DualParticleSphLiquid::writeDescription
    // (DualParticleSphLiquid.cpp:8-40) as YAML text, with the dimension line the
    // Simulator adds (Simulator.cpp:33-39).
    void writeDescription(const std::string & path) const {
        std::ofstream f(path);
        f << "dimension: " << Dim << "\nobjects:\n";
        const char * names[3] = {"particles", "virtual_particles", "boundary_particles"};
        for (int k = 0; k < 3; k++)
            f << "  - name: " << names[k] << "\n    data_mode: dynamic\n    primitive_type: point_list\n"
              << "    material:\n      diffuse_albedo: [0.203921569, 0.423529412, 0.611764706, 1]\n"
              << "    indexed: false\n    color_map:\n      enabled: " << (k < 2 ? "true" : "false") << "\n";
    }
    // particles.mesh of writeFrame (DualParticleSphLiquid.cpp:42-52).
    void writeFrame(const std::string & frameDir, bool staticDraw = false) {
        (void) staticDraw;
        std::filesystem::create_directories(frameDir);
        pull();
        const size_t n = pos_.size() / Dim;
        std::ofstream f(frameDir + "/particles.mesh", std::ios::binary);
        const uint32_t cnt = uint32_t(n);
        f.write(reinterpret_cast<const char *>(&cnt), 4);
        for (size_t i = 0; i < n * Dim; i++) {
            const float v = float(pos_[i]);
            f.write(reinterpret_cast<const char *>(&v), 4);
        }
        if constexpr (Dim == 3) {
            const float z[3] = {0, 0, 1};
            for (size_t i = 0; i < n; i++) f.write(reinterpret_cast<const char *>(z), 12);
        }
        for (size_t i = 0; i < n; i++) {
            double s = 0;
            for (int a = 0; a < Dim; a++) s += vel_[i * Dim + a] * vel_[i * Dim + a];
            const float v = float(std::sqrt(s));
            f.write(reinterpret_cast<const char *>(&v), 4);
        }
    }

    bool throwOnNonConvergence = false;

private:
    void check(int rc, const char * where) const {
        if (rc != SWC_OK) throw Error(rc, where, ctx_ ? swc_last_error(ctx_) : "");
    }
    void ensure() {
        if (!ctx_) check(swc_create(&scene_, &opts_, &ctx_), "swc_create");
        if (dirty_) {
            const int64_t n = int64_t(pos_.size() / Dim);
            check(swc_set_particles(ctx_, pos_.data(), vel_.empty() ? nullptr : vel_.data(), n), "swc_set_particles");
            if (!boundary_set_) {
                const int64_t nb = int64_t(bpos_.size() / Dim);
                check(swc_set_boundary(ctx_, bpos_.data(), bnrm_.data(), bvel_.data(), nb), "swc_set_boundary");
                boundary_set_ = true;
            }
            dirty_ = false;
        }
    }
    std::pair<std::vector<double> &, std::vector<double> &> pull() {
        if (dirty_host_ && ctx_) {
            const int64_t n = int64_t(pos_.size() / Dim);
            check(swc_get_particles(ctx_, pos_.data(), vel_.data(), n), "swc_get_particles");
            dirty_host_ = false;
        }
        return {pos_, vel_};
    }
    static void writeRaw(const std::string & p, const std::vector<double> & a) {
        std::ofstream f(p, std::ios::binary);
        f.write(reinterpret_cast<const char *>(a.data()), std::streamsize(a.size() * sizeof(double)));
    }
    static std::vector<double> readRaw(const std::string & p) {
        std::ifstream f(p, std::ios::binary | std::ios::ate);
        const auto bytes = size_t(f.tellg());
        std::vector<double> a(bytes / sizeof(double));
        f.seekg(0);
        f.read(reinterpret_cast<char *>(a.data()), std::streamsize(bytes));
        return a;
    }

    swc_scene           scene_{};
    swc_solver_opts     opts_{};
    swc_ctx *           ctx_ = nullptr;
    swc_stats           stats_{};
    std::vector<double> pos_, vel_, bpos_, bnrm_, bvel_;
    bool                dirty_ = true, dirty_host_ = false, boundary_set_ = false;
};

}  // namespace swc
