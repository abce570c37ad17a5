// swc_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU FP64 restatement of the dual-particle ("virtual particle") SPH pressure
// projection of skytang0205/sand-water-coupling.  It exists to check the GPU
// product: only the tests, the smoke check and the CPU-baseline leg of the
// benchmark load it.  The product never links or calls it.
//
// Parity status: the reference cannot be compiled here (Eigen and yaml-cpp are
// absent) and ships no tests, fixtures or golden vectors, so this oracle is
// pinned only by analytic known answers (kernel normalisation, packed-lattice
// kernel sums, lattice neighbour counts, operator identities) -- "parity
// unpinned" against an executable of the reference.  CG iteration counts
// depend on Eigen's reduction order (Eigen version unpinned by the reference).
//
// Every function cites the reference file:line it restates (paths relative to
// the reference project root).  Reference quirks are kept on purpose:
//   * V_i = m / rho_i is computed once in initialize and then travels with the
//     particle id (Cores/Physics/DualParticleSphLiquid.cpp:88-89).
//   * rho_I uses the virtual kernel W_H but the real searcher (radius h), so W_H
//     is truncated at h (Cores/Structures/VirtualParticle.cpp:18-27).
//   * gradientKernel(d) = -W'(|d|) d/|d|  (Cores/Structures/SmoothedParticles.h:96-98).
//   * eta = 1e-6 absolute in alpha_IJ (VirtualParticle.cpp:157).
//   * the CG warm start keeps the stale prefix of the previous pressure vector
//     (Cores/Structures/ParticlesBasedData.h:25-29 via VirtualParticle.cpp:95).
//   * virtual nodes are activated when the real-particle weight exceeds 1e-6
//     (VirtualParticle.cpp:56).
#include "orc_core.h"

namespace orc {

struct Params {
    int32_t dim;
    int32_t enable_gravity;
    double  particle_radius;
    double  mass;
    double  boundary_mass;
    double  grid_origin[3];
    double  grid_spacing;
    int32_t grid_size[3];
    int32_t max_iterations;
    double  gravity[3];
    double  viscosity;
    double  target_density;  // <= 0: max rho_i at initialize (reference behaviour)
    double  kappa;           // < 0: 1 / packed kernel sum (reference behaviour)
    double  tolerance;
};

// Deterministic FP64 sum: fixed 4096-element blocks, independent of thread count.
inline double blockedSum(const std::vector<double> & t) {
    const size_t B = 4096, nb = (t.size() + B - 1) / B;
    std::vector<double> part(nb, 0.0);
#pragma omp parallel for schedule(static)
    for (long long b = 0; b < (long long) nb; b++) {
        double s = 0;
        const size_t e = std::min(t.size(), size_t(b + 1) * B);
        for (size_t i = size_t(b) * B; i < e; i++) s += t[i];
        part[b] = s;
    }
    double s = 0;
    for (double v : part) s += v;
    return s;
}

template<int D> struct Oracle {
    Params P{};
    Kernel Kh, KH;  // real/boundary kernel (radius h) and virtual kernel (radius H)

    std::vector<Vec<D>> x, v;  // real particles
    std::vector<double> rho, vol;
    std::vector<Vec<D>> xb, nb, vb;  // boundary particles
    std::vector<double> rhob, volb;
    std::vector<Vec<D>> xv;  // virtual particles (active nodes in x-fastest order)
    std::vector<int64_t> node;
    std::vector<double> rhov, volv, div, alphaHat, pres;
    std::vector<Vec<D>> vbar;
    std::vector<int64_t> rowStart;
    std::vector<int32_t> col;
    std::vector<double>  val;

    Searcher<D> sReal, sBnd, sVirt;
    double rho0 = 0, alpha0 = -1e6, kappa = 0;
    int cgIters = 0, cgEigenIters = 0, status = 0;
    double cgRelRes = 0, rhsNorm = 0;

    void setup(const Params & p) {
        P = p;
        Kh = Kernel(P.particle_radius, D);
        KH = Kernel(P.grid_spacing, D);
        sReal.setRadius(Kh.h);
        sBnd.setRadius(Kh.h);
        sVirt.setRadius(KH.h);
    }

    Vec<D> nodePos(const std::array<int64_t, D> & k) const {
        Vec<D> p;
        for (int a = 0; a < D; a++) p[a] = P.grid_origin[a] + double(k[a]) * P.grid_spacing;
        return p;
    }

    // SmoothedParticles::computeDensities (SmoothedParticles.cpp:25-31, getNeighborWeight :48-54).
    void computeRealDensities() {
        rho.assign(x.size(), 0);
#pragma omp parallel for schedule(dynamic, 256)
        for (long long i = 0; i < (long long) x.size(); i++) {
            double s = 0;
            sReal.forEach(x, x[i], [&](int, const Vec<D> & pj) { s += Kh.W(norm<D>(sub<D>(x[i], pj))); });
            rho[i] = P.mass * s;
        }
    }

    // SmthParticleHydrodLiquid::moveParticles (Cores/Physics/SmthParticleHydrodLiquid.cpp:72-82),
    // no colliders are registered for the dual-particle liquid.
    void moveParticles(double dt) {
#pragma omp parallel for
        for (long long i = 0; i < (long long) x.size(); i++)
            for (int a = 0; a < D; a++) x[i][a] += v[i][a] * dt;
        sReal.reset(x);
        computeRealDensities();
    }

    // applyExternalForces (SmthParticleHydrodLiquid.cpp:84-88); gravity vector is a
    // parameter (the reference subtracts 9.8 dt from component 1).
    void applyExternalForces(double dt) {
        if (!P.enable_gravity) return;
#pragma omp parallel for
        for (long long i = 0; i < (long long) x.size(); i++)
            for (int a = 0; a < D; a++) v[i][a] += P.gravity[a] * dt;
    }

    // applyViscosityForce (SmthParticleHydrodLiquid.cpp:90-98) with
    // ParticlesBasedVectorField::divFreeLaplacianAtDataPoint (ParticlesBasedVectorField.cpp:56-69).
    void applyViscosityForce(double dt) {
        if (P.viscosity == 0) return;
        std::vector<Vec<D>> nv = v;
#pragma omp parallel for schedule(dynamic, 256)
        for (long long i = 0; i < (long long) x.size(); i++) {
            Vec<D> lapl{};
            sReal.forEach(x, x[i], [&](int j, const Vec<D> & pj) {
                const auto dp = sub<D>(pj, x[i]);
                bool any      = false;
                for (int a = 0; a < D; a++) any |= dp[a] != 0;
                if (!any) return;
                const double s = dot<D>(sub<D>(v[j], v[i]), dp) / dot<D>(dp, dp);
                const auto   g = gradKernel<D>(Kh, dp);
                for (int a = 0; a < D; a++) lapl[a] += s * g[a] / rho[j];
            });
            for (int a = 0; a < D; a++) nv[i][a] += P.viscosity * (lapl[a] * 2 * (D + 2.0) * P.mass) * dt;
        }
        v.swap(nv);
    }

    // VirtualParticle::generateParticles (Cores/Structures/VirtualParticle.cpp:45-62):
    // weight over every node of the node grid, x-fastest compaction (Grid.cpp:231-244),
    // then computeInfo (:18-38).
    void generateParticles() {
        const int64_t nx = P.grid_size[0], ny = P.grid_size[1], nz = D == 3 ? P.grid_size[2] : 1;
        const int64_t total = nx * ny * nz;
        std::vector<double> w(total, 0);
#pragma omp parallel for schedule(dynamic, 64)
        for (long long id = 0; id < (long long) total; id++) {
            std::array<int64_t, D> k;
            k[0] = id % nx;
            k[1] = (id / nx) % ny;
            if constexpr (D == 3) k[2] = id / (nx * ny);
            const auto pI = nodePos(k);
            double s = 0;
            sReal.forEach(x, pI, [&](int, const Vec<D> & pj) { s += Kh.W(norm<D>(sub<D>(pI, pj))); });
            w[id] = s;
        }
        xv.clear();
        node.clear();
        for (int64_t id = 0; id < total; id++)
            if (w[id] > 1e-6) {
                std::array<int64_t, D> k;
                k[0] = id % nx;
                k[1] = (id / nx) % ny;
                if constexpr (D == 3) k[2] = id / (nx * ny);
                xv.push_back(nodePos(k));
                node.push_back(id);
            }
        sVirt.reset(xv);
        const size_t n = xv.size();
        rhov.assign(n, 0);
        volv.assign(n, 0);
#pragma omp parallel for schedule(dynamic, 64)
        for (long long I = 0; I < (long long) n; I++) {
            double r = 0, V = 0;
            sReal.forEach(x, xv[I], [&](int j, const Vec<D> & pj) {
                const double d = norm<D>(sub<D>(xv[I], pj));
                r += KH.W(d);  // virtual kernel over the real searcher (truncated at h)
                V += vol[j] * vol[j] * Kh.W(d);
            });
            rhov[I] = r * P.mass;
            volv[I] = V;
        }
    }

    // VirtualParticle::calculateCoef (VirtualParticle.cpp:149-169), stored row-wise with
    // duplicates merged and columns ascending (the column order Eigen's setFromTriplets
    // gives).  The only duplicate is the diagonal: the search visits J = I (distance 0,
    // alpha_II = 0 since W'(0) = 0) and the clamped diagonal is added to it.  Two passes
    // (count, then fill) build the CSR arrays in place.
    void calculateCoef(double a0) {
        const size_t n = xv.size();
        alphaHat.assign(n, 0);
        rowStart.assign(n + 1, 0);
#pragma omp parallel for schedule(dynamic, 64)
        for (long long I = 0; I < (long long) n; I++) {
            int64_t c = 0;
            sVirt.forEach(xv, xv[I], [&](int, const Vec<D> &) { c++; });
            rowStart[I + 1] = c;
        }
        for (size_t I = 0; I < n; I++) rowStart[I + 1] += rowStart[I];
        col.resize(rowStart[n]);
        val.resize(rowStart[n]);
        std::vector<int> bad;
#pragma omp parallel for schedule(dynamic, 64)
        for (long long I = 0; I < (long long) n; I++) {
            double sum = 0;
            int64_t o = rowStart[I], self = -1;
            sVirt.forEach(xv, xv[I], [&](int J, const Vec<D> & pJ) {
                const double r = norm<D>(sub<D>(xv[I], pJ));
                const double a = 2. * volv[J] * KH.dW(r) / (r + 1e-6);
                sum -= a;
                if (J == int(I)) self = o;
                col[o] = J, val[o] = a, o++;
            });
            const double dg = std::max(sum, a0);
            alphaHat[I] = dg;
            if (self < 0) {
#pragma omp critical
                bad.push_back(int(I));
                continue;
            }
            val[self] += dg;
            // sort the row by column (the search order is not the column order)
            const int64_t b = rowStart[I], e = rowStart[I + 1];
            std::vector<std::pair<int, double>> row(size_t(e - b));
            for (int64_t t = b; t < e; t++) row[size_t(t - b)] = {col[t], val[t]};
            std::sort(row.begin(), row.end(), [](auto & l, auto & r) { return l.first < r.first; });
            for (int64_t t = b; t < e; t++) col[t] = row[size_t(t - b)].first, val[t] = row[size_t(t - b)].second;
        }
        if (!bad.empty()) {
            std::fprintf(stderr, "oracle: virtual node %d does not find itself within H\n", bad[0]);
            std::abort();
        }
    }

    void spmv(const std::vector<double> & in, std::vector<double> & out) const {
        const size_t n = xv.size();
        out.resize(n);
#pragma omp parallel for schedule(static)
        for (long long I = 0; I < (long long) n; I++) {
            double s = 0;
            for (int64_t e = rowStart[I]; e < rowStart[I + 1]; e++) s += val[e] * in[col[e]];
            out[I] = s;
        }
    }

    double vdot(const std::vector<double> & a, const std::vector<double> & b) const {
        std::vector<double> t(a.size());
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < (long long) a.size(); i++) t[i] = a[i] * b[i];
        return blockedSum(t);
    }

    // IterativeSolver::solve (Cores/Solvers/IterativeSolver.h:21-40): textbook
    // Hestenes-Stiefel CG, identity preconditioner, warm start from `pres`,
    // tolerance max(tol, eps/|b|), relative test |r|^2 < tol^2 |b|^2, at most
    // 2n iterations by default.  Failure returns status 1 instead of exit(-1).
    void solve() {
        const size_t n = xv.size();
        auto & xx = pres;
        const auto & b = div;
        const double bb = vdot(b, b);
        rhsNorm = std::sqrt(bb);
        cgIters = cgEigenIters = 0;
        status = 0;
        if (n == 0) { cgRelRes = 0; return; }
        if (bb == 0) {
            std::fill(xx.begin(), xx.end(), 0.0);
            cgRelRes = 0;
            return;
        }
        const double tol = std::max(P.tolerance, std::numeric_limits<double>::epsilon() / rhsNorm);
        const int64_t maxIt = P.max_iterations >= 0 ? P.max_iterations : 2 * int64_t(n);
        const double threshold = std::max(tol * tol * bb, std::numeric_limits<double>::min());
        std::vector<double> r(n), q(n), p(n);
        spmv(xx, q);
        for (size_t i = 0; i < n; i++) r[i] = b[i] - q[i];
        double rr = vdot(r, r);
        if (rr < threshold) { cgRelRes = std::sqrt(rr / bb); return; }
        p = r;
        double absNew = rr;
        int64_t it = 0;
        int spmvs = 0;
        while (it < maxIt) {
            spmv(p, q);
            spmvs++;
            const double alpha = absNew / vdot(p, q);
#pragma omp parallel for schedule(static)
            for (long long i = 0; i < (long long) n; i++) {
                xx[i] += alpha * p[i];
                r[i] -= alpha * q[i];
            }
            rr = vdot(r, r);
            if (rr < threshold) break;
            const double absOld = absNew;
            absNew = rr;
            const double beta = absNew / absOld;
#pragma omp parallel for schedule(static)
            for (long long i = 0; i < (long long) n; i++) p[i] = r[i] + beta * p[i];
            it++;
        }
        cgEigenIters = int(it);
        cgIters = spmvs;
        cgRelRes = std::sqrt(rr / bb);
        status = cgRelRes <= tol ? 0 : 1;
    }

    // VirtualParticle::calculateVelocity (VirtualParticle.cpp:137-147) and calculateDiv
    // (:172-201) with ParticlesBasedVectorField::operator()/divergence
    // (ParticlesBasedVectorField.cpp:5-21) and getBiasWeight/getBiasGradient
    // (SmoothedParticles.cpp:56-72).
    void buildRhs() {
        const size_t n = xv.size();
        vbar.assign(n, Vec<D>{});
        div.assign(n, 0);
        const double mb = P.boundary_mass;
#pragma omp parallel for schedule(dynamic, 64)
        for (long long I = 0; I < (long long) n; I++) {
            const auto & pI = xv[I];
            Vec<D> velR{}, velB{}, gR{}, gB{};
            double bwR = 0, bwB = 0, divR = 0, divB = 0;
            sReal.forEach(x, pI, [&](int j, const Vec<D> & pj) {
                const auto d = sub<D>(pI, pj);
                const double w = Kh.W(norm<D>(d));
                for (int a = 0; a < D; a++) velR[a] += v[j][a] * w / rho[j];
                bwR += vol[j] * w;
                const auto g = gradKernel<D>(Kh, d);
                divR += dot<D>(v[j], g) * vol[j];
                for (int a = 0; a < D; a++) gR[a] += vol[j] * g[a];
            });
            sBnd.forEach(xb, pI, [&](int j, const Vec<D> & pj) {
                const auto d = sub<D>(pI, pj);
                const double w = Kh.W(norm<D>(d));
                for (int a = 0; a < D; a++) velB[a] += vb[j][a] * w / rhob[j];
                bwB += volb[j] * w;
                const auto g = gradKernel<D>(Kh, d);
                divB += dot<D>(vb[j], g) * volb[j];
                for (int a = 0; a < D; a++) gB[a] += volb[j] * g[a];
            });
            const double den = bwR + bwB + 1e-6;
            Vec<D> vb_;
            for (int a = 0; a < D; a++) vb_[a] = (velR[a] * P.mass + velB[a] * mb) / den;
            vbar[I] = vb_;
            div[I] = divR - dot<D>(vb_, gR) + divB - dot<D>(vb_, gB)
                - kappa * std::max(rhov[I] - rho0, 0.) / rho0;
        }
    }

    // VirtualParticle::applyPressureGradient (VirtualParticle.cpp:111-134).
    void applyPressureGradient() {
#pragma omp parallel for schedule(dynamic, 64)
        for (long long i = 0; i < (long long) x.size(); i++) {
            const auto & pi = x[i];
            Vec<D> f{};
            sVirt.forEach(xv, pi, [&](int J, const Vec<D> & pJ) {
                const auto g = gradKernel<D>(KH, sub<D>(pi, pJ));
                for (int a = 0; a < D; a++) f[a] += volv[J] * pres[J] * g[a];
            });
            sBnd.forEach(xb, pi, [&](int j, const Vec<D> & pj) {
                const double vn = std::min(dot<D>(nb[j], sub<D>(v[i], vb[j])), 0.);
                const double w  = Kh.W(norm<D>(sub<D>(pi, pj)));
                for (int a = 0; a < D; a++) f[a] -= volb[j] * vn * nb[j][a] * w;
            });
            for (int a = 0; a < D; a++) v[i][a] += f[a];
        }
    }

    // VirtualParticle::project / buildLinearSystem (VirtualParticle.cpp:76-103).
    void project() {
        pres.resize(xv.size(), 0.0);  // stale-prefix warm start
        buildRhs();
        calculateCoef(alpha0);
        solve();
        applyPressureGradient();
    }

    // DualParticleSphLiquid::initialize (Cores/Physics/DualParticleSphLiquid.cpp:78-110);
    // the boundary set is supplied by the scene instead of the hard-coded box shell.
    void initialize() {
        sReal.reset(x);
        computeRealDensities();
        vol.resize(x.size());
        for (size_t i = 0; i < x.size(); i++) vol[i] = P.mass / rho[i];
        rho0 = 0;
        for (double r : rho) rho0 = std::max(rho0, r);
        if (P.target_density > 0) rho0 = P.target_density;
        sBnd.reset(xb);
        rhob.assign(xb.size(), 0);
        volb.assign(xb.size(), 0);
#pragma omp parallel for schedule(dynamic, 256)
        for (long long j = 0; j < (long long) xb.size(); j++) {
            double s = 0;
            sBnd.forEach(xb, xb[j], [&](int, const Vec<D> & pk) { s += Kh.W(norm<D>(sub<D>(xb[j], pk))); });
            rhob[j] = P.boundary_mass * s;
            volb[j] = P.boundary_mass / rhob[j];
        }
        // VirtualParticle::setAlpha (VirtualParticle.cpp:64-73): clamp off, alpha0 = max diagonal.
        generateParticles();
        calculateCoef(-1e6);
        alpha0 = -1e6;
        for (double a : alphaHat) alpha0 = std::max(alpha0, a);
        kappa = P.kappa >= 0 ? P.kappa : 1. / Kh.packedSum(D);
        pres.clear();
    }

    // Moving solids (the paddle-tank extension; the reference's boundary is static
    // after initialize): flagged boundary particles turn rigidly by -omega dt about
    // the vertical (y) axis through c, their normals with them, v_b = omega x
    // (x_b - c) in the scene's convention (v_x = omega r_z, v_z = -omega r_x);
    // the boundary grid is rebuilt and V_b keeps its initial value.
    std::vector<unsigned char> moving;
    double motionC[3] = {0, 0, 0}, omega = 0;
    bool hasMotion = false;
    void moveBoundary(double dt) {
        if constexpr (D == 3) {
            const double ca = std::cos(omega * dt), sa = std::sin(omega * dt);
            for (size_t i = 0; i < xb.size(); i++) {
                if (!moving[i]) continue;
                const double rx = xb[i][0] - motionC[0], rz = xb[i][2] - motionC[2];
                const double nx = rx * ca + rz * sa, nz = -rx * sa + rz * ca;
                xb[i][0]        = motionC[0] + nx;
                xb[i][2]        = motionC[2] + nz;
                const double mx = nb[i][0] * ca + nb[i][2] * sa, mz = -nb[i][0] * sa + nb[i][2] * ca;
                nb[i][0]        = mx;
                nb[i][2]        = mz;
                vb[i][0]        = omega * nz;
                vb[i][2]        = -omega * nx;
            }
            sBnd.reset(xb);
        }
    }

    // DualParticleSphLiquid::advance (DualParticleSphLiquid.cpp:112-126).
    void advance(double dt) {
        if (hasMotion) moveBoundary(dt);
        moveParticles(dt);
        applyExternalForces(dt);
        applyViscosityForce(dt);
        generateParticles();
        project();
    }
};

struct Handle {
    int dim;
    Oracle<2> o2;
    Oracle<3> o3;
};

template<int D> void loadVecs(std::vector<Vec<D>> & dst, const double * src, int64_t n) {
    dst.resize(n);
    for (int64_t i = 0; i < n; i++)
        for (int a = 0; a < D; a++) dst[i][a] = src ? src[i * D + a] : 0.0;
}
template<int D> int64_t hashCandidates(const Oracle<D> & O, int which, int64_t nq, const double * q) {
    HashGrid<D> g;
    g.setRadius(which == 2 ? O.KH.h : O.Kh.h);
    g.reset(which == 0 ? O.x : which == 1 ? O.xb : O.xv);
    int64_t total = 0;
#pragma omp parallel for reduction(+ : total) schedule(dynamic, 64)
    for (long long t = 0; t < (long long) nq; t++) {
        Vec<D> p;
        for (int a = 0; a < D; a++) p[a] = q[t * D + a];
        total += g.candidates(p);
    }
    return total;
}
template<int D> void storeVecs(const std::vector<Vec<D>> & src, double * dst) {
    for (size_t i = 0; i < src.size(); i++)
        for (int a = 0; a < D; a++) dst[i * D + a] = src[i][a];
}

}  // namespace orc

using orc::Handle;

#define DISPATCH(h, ...)                                                                                              \
    do {                                                                                                               \
        if ((h)->dim == 2) {                                                                                           \
            auto & O = (h)->o2;                                                                                        \
            constexpr int D = 2;                                                                                       \
            (void) D;                                                                                                  \
            __VA_ARGS__;                                                                                               \
        } else {                                                                                                       \
            auto & O = (h)->o3;                                                                                        \
            constexpr int D = 3;                                                                                       \
            (void) D;                                                                                                  \
            __VA_ARGS__;                                                                                               \
        }                                                                                                              \
    } while (0)

extern "C" {

Handle * orc_create(const orc::Params * p) {
    if (!p || (p->dim != 2 && p->dim != 3)) return nullptr;
    auto h = new Handle();
    h->dim = p->dim;
    DISPATCH(h, O.setup(*p));
    return h;
}
void orc_destroy(Handle * h) { delete h; }
int orc_num_threads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void) n;
#endif
}

void orc_set_particles(Handle * h, int64_t n, const double * x, const double * v) {
    DISPATCH(h, { orc::loadVecs<D>(O.x, x, n); orc::loadVecs<D>(O.v, v, n); });
}
void orc_get_particles(Handle * h, double * x, double * v) {
    DISPATCH(h, { if (x) orc::storeVecs<D>(O.x, x); if (v) orc::storeVecs<D>(O.v, v); });
}
void orc_set_boundary(Handle * h, int64_t n, const double * x, const double * nrm, const double * v) {
    DISPATCH(h, {
        orc::loadVecs<D>(O.xb, x, n);
        orc::loadVecs<D>(O.nb, nrm, n);
        orc::loadVecs<D>(O.vb, v, n);
        O.sBnd.reset(O.xb);  // a replayed step needs no initialize
    });
}
// Searcher of every neighbour query: 0 = the reference's hash grid (its enumeration
// order; default), 1 = the cell grid over the same cells (same sets, other order).
void orc_set_searcher(Handle * h, int cells) {
    DISPATCH(h, {
        for (auto * s : {&O.sReal, &O.sBnd, &O.sVirt}) s->useCells = cells != 0;
        O.sReal.reset(O.x);
        O.sBnd.reset(O.xb);
        O.sVirt.reset(O.xv);
    });
}
// Candidates the reference's hash grid visits (bucket entries before the distance
// test) summed over nq query points, for the real (which 0), boundary (1) or
// virtual (2) set as it stands: the reference searcher's cost.
int64_t orc_hash_candidates(Handle * h, int which, int64_t nq, const double * q) {
    return h->dim == 2 ? orc::hashCandidates<2>(h->o2, which, nq, q) : orc::hashCandidates<3>(h->o3, which, nq, q);
}
void orc_set_boundary_motion(Handle * h, const unsigned char * moving, const double * center, double omega) {
    DISPATCH(h, {
        O.moving.assign(moving, moving + O.xb.size());
        for (int a = 0; a < 3; a++) O.motionC[a] = center[a];
        O.omega     = omega;
        O.hasMotion = true;
    });
}
void orc_initialize(Handle * h) { DISPATCH(h, O.initialize()); }
void orc_advance(Handle * h, double dt) { DISPATCH(h, O.advance(dt)); }
void orc_move_and_forces(Handle * h, double dt) {
    DISPATCH(h, { O.moveParticles(dt); O.applyExternalForces(dt); O.applyViscosityForce(dt); });
}
// Projection of the current state: rho_i from current positions, virtual generation,
// then project (the second half of advance).
void orc_project(Handle * h) {
    DISPATCH(h, {
        O.sReal.reset(O.x);
        O.computeRealDensities();
        O.generateParticles();
        O.project();
    });
}
void orc_compute_densities(Handle * h) { DISPATCH(h, { O.sReal.reset(O.x); O.computeRealDensities(); }); }

// Scalars: rho0, alpha0, kappa.
void orc_get_scalars(Handle * h, double * out3) { DISPATCH(h, { out3[0] = O.rho0; out3[1] = O.alpha0; out3[2] = O.kappa; }); }
void orc_set_scalars(Handle * h, const double * in3) { DISPATCH(h, { O.rho0 = in3[0]; O.alpha0 = in3[1]; O.kappa = in3[2]; }); }
void orc_get_real_info(Handle * h, double * rho, double * vol) {
    DISPATCH(h, {
        if (rho) std::copy(O.rho.begin(), O.rho.end(), rho);
        if (vol) std::copy(O.vol.begin(), O.vol.end(), vol);
    });
}
void orc_set_volumes(Handle * h, const double * vol) { DISPATCH(h, O.vol.assign(vol, vol + O.x.size())); }
void orc_get_boundary_info(Handle * h, double * rho, double * vol) {
    DISPATCH(h, {
        if (rho) std::copy(O.rhob.begin(), O.rhob.end(), rho);
        if (vol) std::copy(O.volb.begin(), O.volb.end(), vol);
    });
}
void orc_set_boundary_info(Handle * h, const double * rho, const double * vol) {
    DISPATCH(h, { O.rhob.assign(rho, rho + O.xb.size()); O.volb.assign(vol, vol + O.xb.size()); });
}
int64_t orc_num_virtual(Handle * h) {
    int64_t n = 0;
    DISPATCH(h, n = int64_t(O.xv.size()));
    return n;
}
// Per active node (x-fastest order): node id, rho_I, V_I, vbar (n*dim), D_I, alpha_hat, p.
void orc_get_virtual(Handle * h, int64_t * node, double * rho, double * vol, double * vbar, double * dv,
                     double * ahat, double * p) {
    DISPATCH(h, {
        const size_t n = O.xv.size();
        if (node) std::copy(O.node.begin(), O.node.end(), node);
        if (rho) std::copy(O.rhov.begin(), O.rhov.end(), rho);
        if (vol) std::copy(O.volv.begin(), O.volv.end(), vol);
        if (vbar && O.vbar.size() == n) orc::storeVecs<D>(O.vbar, vbar);
        if (dv && O.div.size() == n) std::copy(O.div.begin(), O.div.end(), dv);
        if (ahat && O.alphaHat.size() == n) std::copy(O.alphaHat.begin(), O.alphaHat.end(), ahat);
        if (p && O.pres.size() == n) std::copy(O.pres.begin(), O.pres.end(), p);
    });
}
// Pressure vector used as the next warm start (reference: the stale prefix survives resize).
void orc_set_pressure(Handle * h, int64_t n, const double * p) { DISPATCH(h, O.pres.assign(p, p + n)); }
// y = A x with the operator assembled by the last project / initialize.
void orc_apply_operator(Handle * h, const double * in, double * out) {
    DISPATCH(h, {
        std::vector<double> a(in, in + O.xv.size()), b;
        O.spmv(a, b);
        std::copy(b.begin(), b.end(), out);
    });
}
// Solver statistics: iterations (SpMV count), iterations as Eigen reports them,
// relative residual, |b|, status.
void orc_get_stats(Handle * h, int32_t * iters, int32_t * eigenIters, double * relres, double * bnorm, int32_t * status) {
    DISPATCH(h, {
        *iters = O.cgIters;
        *eigenIters = O.cgEigenIters;
        *relres = O.cgRelRes;
        *bnorm = O.rhsNorm;
        *status = O.status;
    });
}
// Neighbour query with the reference searcher semantics: for each query point, the
// sorted ids of real particles (which=0), boundary particles (1) or virtual
// particles (2) with |x_j - q|^2 < radius^2.  Returns counts; fills `ids` (CSR by
// query) when non-null.
void orc_neighbors(Handle * h, int which, int64_t nq, const double * q, int64_t * counts, int64_t * offsets, int64_t * ids) {
    DISPATCH(h, {
        const auto & S = which == 0 ? O.sReal : which == 1 ? O.sBnd : O.sVirt;
        const auto & X = which == 0 ? O.x : which == 1 ? O.xb : O.xv;
        for (int64_t t = 0; t < nq; t++) {
            orc::Vec<D> p;
            for (int a = 0; a < D; a++) p[a] = q[t * D + a];
            std::vector<int64_t> got;
            S.forEach(X, p, [&](int j, const orc::Vec<D> &) { got.push_back(j); });
            std::sort(got.begin(), got.end());
            counts[t] = int64_t(got.size());
            if (ids) std::copy(got.begin(), got.end(), ids + offsets[t]);
        }
    });
}
// Kernel evaluations for known-answer tests: which 0 = W, 1 = W'; radius = particle radius.
double orc_kernel(int dim, double radius, int which, double dist) {
    orc::Kernel k(radius, dim);
    return which == 0 ? k.W(dist) : k.dW(dist);
}
double orc_packed_kernel_sum(int dim, double radius) { return orc::Kernel(radius, dim).packedSum(dim); }

}  // extern "C"
