// dem_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU FP64 restatement of the DEM sand step of skytang0205/sand-water-coupling
// (DEMParticleSand<Dim>::advance, Cores/Physics/DEMParticleSand.cpp:90-152, with
// the contact model of DEMParticle, Cores/Structures/DEMParticle.cpp:15-134).
// Only the tests, the smoke check and the CPU-baseline leg of the benchmark load
// it; the product never links or calls it.
//
// Parity status: the reference cannot be compiled here (Eigen and yaml-cpp are
// absent) and ships no DEM tests or fixtures, so this restatement is pinned by
// analytic known answers (two-particle contacts, the Coulomb cap, the boundary
// friction cases, the unreachable capillary branch) -- "parity unpinned"
// against an executable of the reference.
//
// Reference behaviour kept on purpose:
//   * neighbours of a sand particle are the particles with |x_j - x_i|^2 < (2r)^2
//     (kernel_rate 2, DEMParticle.cpp:17; strict test of the hash searcher),
//     boundary neighbours those within 4r (BoundaryParticles' default kernel_rate 4,
//     Cores/Structures/SmoothedParticles.h:124-126);
//   * the pair term carries no mass: v_i += dt * sum_j F_ij, and the boundary
//     friction term is added without dt (DEMParticleSand.cpp:130-150);
//   * the penetration depth uses the distance before its clamp to 1e-4 r, the
//     normal uses the clamped one (DEMParticle.cpp:77-80);
//   * phi of the capillary term takes a single-precision sqrtf
//     (DEMParticle.cpp:103).  The capillary branch needs H = |d| - 2r > 1e-6,
//     which no visited pair has (|d| < 2r), so it never contributes; it is
//     restated for completeness and checked on its own.
// One deliberate choice: the reference updates velocities[i] inside a parallel
// loop that reads velocities[j] of other particles, so its result depends on
// thread timing.  Here every particle reads the velocities from the start of
// the pass (the order-independent reading); the GPU does the same.
#include "orc_core.h"

namespace orc {

struct DemParams {
    int32_t dim;
    int32_t enable_gravity;
    double  radius;       // particle radius r (DEMParticleSand(particleRadius))
    double  mass;         // particle and boundary mass (DEMParticleSand.cpp:79)
    double  young;        // DEMParticle::setYoung (default 1e9, DEMParticle.cpp:18)
    double  poisson;      // DEMParticle::setPoisson (default 0.3)
    double  fric_angle;   // DEMParticle::setfricangle, radians (default 0.5)
};

// DEMParticle's constants (DEMParticle.cpp:15-33) and its Bezier coefficient
// QuadraticBezierCoeff::calculate (Cores/Structures/DEMParticle.h:14-55).
struct DemModel {
    double r = 0, K_norm = 0, K_tang = 0, tan_fric = 0;
    double contact_angle = 0, v_bridge = 0, d_rupture = 0, coeff_c = 0;

    static double bezier(double py0, double py1, double px1, double py2, double sr) {
        const double a = (px1 + 1.) / 4., b = -2. * a, c = b * b, d = -4. * (1. + b - px1), e = 2. * (1. + b - px1);
        if (sr < 0.) return py0;
        if (sr >= 1.) return py2;
        if (sr <= px1) {
            const double t = sr / px1, omt = 1. - t;
            return omt * omt * py0 + 2 * t * omt * py1 + t * t * py1;
        }
        const double t = (b + std::sqrt(c + d * (px1 - sr))) / e, omt = 1. - t;
        return omt * omt * py1 + 2 * t * omt * py1 + t * t * py2;
    }
    void set(const DemParams & p) {
        r             = p.radius;
        K_norm        = p.young * r;
        K_tang        = K_norm * p.poisson;
        tan_fric      = std::tan(p.fric_angle);
        contact_angle = 30. / 180. * std::numbers::pi;
        v_bridge      = 4. / 3. * std::numbers::pi * std::pow(r, 3.) * 0.01 * 0.01;
        d_rupture = (1.f + 0.5f * contact_angle) * (std::pow(v_bridge, 1. / 3.) + 0.1 * std::pow(v_bridge, 2. / 3.));
        coeff_c   = bezier(0.8, 1., 0.1, 0.1, 0.1);  // G.calculate(sr), c0 = 0.8, cmc = 1, cmcp = sr = 0.1, csat = 0.1
    }
};

// DEMParticle::ComputeDemForces (DEMParticle.cpp:69-96): d = x_j - x_i, w = v_j - v_i.
template<int D> Vec<D> demContact(const DemModel & M, const Vec<D> & d, const Vec<D> & w) {
    Vec<D> f{};
    double dist      = norm<D>(d);
    const double pen = 2 * M.r - dist;
    if (pen > 0.) {
        if (dist <= 0.0001 * M.r) dist = 0.0001 * M.r;
        Vec<D> n;
        for (int a = 0; a < D; a++) n[a] = d[a] * (1 / dist);
        const double dn = dot<D>(w, n);
        Vec<D> normal, shear;
        for (int a = 0; a < D; a++) {
            normal[a] = M.K_norm * pen * n[a];
            shear[a]  = -M.K_tang * (w[a] - dn * n[a]);
        }
        const double max_fs = norm<D>(normal) * M.tan_fric, sn = norm<D>(shear);
        if (sn > max_fs)
            for (int a = 0; a < D; a++) shear[a] = shear[a] * max_fs / sn;
        for (int a = 0; a < D; a++) f[a] = -normal[a] - shear[a];
    }
    return f;
}

// DEMParticle::ComputeDemCapillaryForces (DEMParticle.cpp:98-124).
template<int D> Vec<D> demCapillary(const DemModel & M, const Vec<D> & d) {
    Vec<D> f{};
    const double dist = norm<D>(d);
    const double H    = dist - 2 * M.r;
    if (H < M.d_rupture && H > 0.000001) {
        const double dd  = -H + std::sqrt(H * H + M.v_bridge / (std::numbers::pi * M.r));
        const double phi = std::sqrt(2. * H / M.r *
                                     (-1.f + sqrtf(float(1.f + M.v_bridge / (std::numbers::pi * M.r * H * H)))));
        const double neck = -2. * std::numbers::pi * M.coeff_c * M.r * std::cos(M.contact_angle) / (1. + H / (2. * dd));
        const double surf = -2. * std::numbers::pi * M.coeff_c * M.r * phi * std::sin(M.contact_angle);
        for (int a = 0; a < D; a++) f[a] = -(d[a] * (1 / dist)) * (neck + surf);
    }
    return f;
}

// Boundary friction of one boundary particle (DEMParticleSand.cpp:138-149):
// dv = v_i - v_b, n_b its normal, V_b its volume, w = W_4r(x_i - x_b).
template<int D> Vec<D> demBoundary(const DemModel & M, const Vec<D> & dv, const Vec<D> & nb, double Vb, double w) {
    const double dvn = dot<D>(nb, dv);
    Vec<D> Fn, Ft, out;
    for (int a = 0; a < D; a++) {
        Fn[a] = -Vb * std::min(dvn, 0.) * nb[a] * w;
        Ft[a] = -M.K_tang * (dv[a] - dvn * nb[a]);
    }
    const double nt = norm<D>(Ft), nn = norm<D>(Fn);
    if (nt <= 0.000001) {
        for (int a = 0; a < D; a++) out[a] = Fn[a] + Ft[a];
    } else {
        const bool keep = nn * M.tan_fric > nt;
        for (int a = 0; a < D; a++) out[a] = Fn[a] + (keep ? Ft[a] : (nn * M.tan_fric / nt) * Ft[a]);
    }
    return out;
}

template<int D> struct DemOracle {
    DemParams P{};
    DemModel M;
    Kernel Kb;  // boundary kernel, radius 4r
    std::vector<Vec<D>> x, v;
    std::vector<Vec<D>> xb, nb, vb;
    std::vector<double> rhob, volb;
    HashGrid<D> grid, bgrid;

    explicit DemOracle(const DemParams & p) : P(p) {
        M.set(p);
        Kb = Kernel(p.radius, D, 4);
        grid.setRadius(2 * p.radius);
        bgrid.setRadius(4 * p.radius);
    }

    // DEMParticleSand::initialize (DEMParticleSand.cpp:78-88): boundary densities and
    // volumes from the boundary particles alone (SmoothedParticles::computeInfo,
    // Cores/Structures/SmoothedParticles.cpp:25-41).
    void initialize() {
        bgrid.reset(xb);
        rhob.assign(xb.size(), 0);
        volb.assign(xb.size(), 0);
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < (long long) xb.size(); i++) {
            double s = 0;
            bgrid.forEach(xb, xb[i], [&](int, const Vec<D> & p) { s += Kb.W(norm<D>(sub<D>(xb[i], p))); });
            rhob[i] = P.mass * s;
            volb[i] = P.mass / rhob[i];
        }
        grid.reset(x);
    }

    // DEMParticleSand::advance (DEMParticleSand.cpp:90-94).
    void advance(double dt) {
        const long long n = (long long) x.size();
        // moveParticles (DEMParticleSand.cpp:98-109)
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < n; i++)
            for (int a = 0; a < D; a++) x[i][a] += v[i][a] * dt;
        grid.reset(x);
        // applyPressureForce (DEMParticleSand.cpp:118-152), velocities read at the pass start
        std::vector<Vec<D>> vnew(v.size());
#pragma omp parallel for schedule(dynamic, 256)
        for (long long i = 0; i < n; i++) {
            Vec<D> fs{};
            grid.forEach(x, x[i], [&](int j, const Vec<D> & pj) {
                const Vec<D> d = sub<D>(pj, x[i]), w = sub<D>(v[j], v[i]);
                const Vec<D> f0 = demContact<D>(M, d, w), f1 = demCapillary<D>(M, d);
                for (int a = 0; a < D; a++) fs[a] += f0[a] + f1[a];
            });
            Vec<D> force;
            for (int a = 0; a < D; a++) force[a] = fs[a] * dt;
            if (!xb.empty())
                bgrid.forEach(xb, x[i], [&](int j, const Vec<D> & pb) {
                    Vec<D> dv;
                    for (int a = 0; a < D; a++) dv[a] = v[i][a] - (vb.empty() ? 0. : vb[j][a]);
                    const Vec<D> f = demBoundary<D>(M, dv, nb[j], volb[j], Kb.W(norm<D>(sub<D>(x[i], pb))));
                    for (int a = 0; a < D; a++) force[a] += f[a];
                });
            for (int a = 0; a < D; a++) vnew[i][a] = v[i][a] + force[a];
        }
        v.swap(vnew);
        // applyExternalForces (DEMParticleSand.cpp:111-115)
        if (P.enable_gravity)
            for (long long i = 0; i < n; i++) v[i][1] -= kGravity * dt;
    }

    static constexpr double kGravity = 9.8;  // Cores/Utilities/Constants.h:7

    // DEMParticleSand::getTimeStep (DEMParticleSand.h:38-40).
    double timeStep(double step_rate) const {
        double vmax = 0;
        for (const auto & w : v) vmax = std::max(vmax, norm<D>(w));
        return step_rate * P.radius * 2 / vmax;
    }
};

struct DemHandle {
    int dim;
    DemOracle<2> * o2 = nullptr;
    DemOracle<3> * o3 = nullptr;
    ~DemHandle() {
        delete o2;
        delete o3;
    }
};

template<int D> void loadVec(std::vector<Vec<D>> & dst, const double * src, long long n) {
    dst.resize(size_t(n));
    for (long long i = 0; i < n; i++)
        for (int a = 0; a < D; a++) dst[i][a] = src[i * D + a];
}
template<int D> void storeVec(const std::vector<Vec<D>> & src, double * dst) {
    for (size_t i = 0; i < src.size(); i++)
        for (int a = 0; a < D; a++) dst[i * D + a] = src[i][a];
}

}  // namespace orc

using orc::DemHandle;

#define DEM_DISPATCH(h, body)          \
    do {                               \
        if ((h)->dim == 2) {           \
            auto & o = *(h)->o2;       \
            constexpr int D = 2;       \
            body;                      \
        } else {                       \
            auto & o = *(h)->o3;       \
            constexpr int D = 3;       \
            body;                      \
        }                              \
    } while (0)

extern "C" {

DemHandle * dem_create(const orc::DemParams * p) {
    if (!p || (p->dim != 2 && p->dim != 3) || !(p->radius > 0)) return nullptr;
    auto * h = new DemHandle();
    h->dim   = p->dim;
    if (p->dim == 2) h->o2 = new orc::DemOracle<2>(*p);
    else h->o3 = new orc::DemOracle<3>(*p);
    return h;
}
void dem_destroy(DemHandle * h) { delete h; }

void dem_set_particles(DemHandle * h, long long n, const double * x, const double * v) {
    DEM_DISPATCH(h, {
        orc::loadVec<D>(o.x, x, n);
        orc::loadVec<D>(o.v, v, n);
        (void) D;
    });
}
void dem_get_particles(DemHandle * h, double * x, double * v) {
    DEM_DISPATCH(h, {
        if (x) orc::storeVec<D>(o.x, x);
        if (v) orc::storeVec<D>(o.v, v);
    });
}
// vb may be null (the reference's boundary velocity field stays zero).
void dem_set_boundary(DemHandle * h, long long nb, const double * xb, const double * nrm, const double * vb) {
    DEM_DISPATCH(h, {
        orc::loadVec<D>(o.xb, xb, nb);
        orc::loadVec<D>(o.nb, nrm, nb);
        if (vb) orc::loadVec<D>(o.vb, vb, nb);
        else o.vb.clear();
    });
}
void dem_initialize(DemHandle * h) { DEM_DISPATCH(h, o.initialize(); (void) D); }
void dem_advance(DemHandle * h, double dt) { DEM_DISPATCH(h, o.advance(dt); (void) D); }
void dem_get_boundary_info(DemHandle * h, double * rho, double * vol) {
    DEM_DISPATCH(h, {
        (void) D;
        for (size_t i = 0; i < o.rhob.size(); i++) {
            if (rho) rho[i] = o.rhob[i];
            if (vol) vol[i] = o.volb[i];
        }
    });
}
double dem_time_step(DemHandle * h, double step_rate) {
    double dt = 0;
    DEM_DISPATCH(h, dt = o.timeStep(step_rate); (void) D);
    return dt;
}
// The model constants after DemModel::set: K_norm, K_tang, tan_fric, d_rupture, coeff_c, v_bridge.
void dem_model(const orc::DemParams * p, double * out) {
    orc::DemModel M;
    M.set(*p);
    out[0] = M.K_norm;
    out[1] = M.K_tang;
    out[2] = M.tan_fric;
    out[3] = M.d_rupture;
    out[4] = M.coeff_c;
    out[5] = M.v_bridge;
}
// One pair / boundary term for known-answer tests (3 components; dim selects 2 or 3).
void dem_pair_force(const orc::DemParams * p, const double * d, const double * w, double * contact, double * capillary) {
    orc::DemModel M;
    M.set(*p);
    if (p->dim == 2) {
        const orc::Vec<2> dd{d[0], d[1]}, ww{w[0], w[1]};
        const auto f0 = orc::demContact<2>(M, dd, ww), f1 = orc::demCapillary<2>(M, dd);
        for (int a = 0; a < 2; a++) contact[a] = f0[a], capillary[a] = f1[a];
        contact[2] = capillary[2] = 0;
    } else {
        const orc::Vec<3> dd{d[0], d[1], d[2]}, ww{w[0], w[1], w[2]};
        const auto f0 = orc::demContact<3>(M, dd, ww), f1 = orc::demCapillary<3>(M, dd);
        for (int a = 0; a < 3; a++) contact[a] = f0[a], capillary[a] = f1[a];
    }
}
void dem_boundary_term(const orc::DemParams * p, const double * dv, const double * nb, double Vb, double w,
                       double * out) {
    orc::DemModel M;
    M.set(*p);
    const orc::Vec<3> a{dv[0], dv[1], p->dim == 3 ? dv[2] : 0.}, b{nb[0], nb[1], p->dim == 3 ? nb[2] : 0.};
    const auto f = orc::demBoundary<3>(M, a, b, Vb, w);
    for (int k = 0; k < 3; k++) out[k] = f[k];
}

}  // extern "C"
