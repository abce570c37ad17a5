// orc_core.h -- TEST INFRASTRUCTURE ONLY.
//
// Pieces of the CPU FP64 oracle shared by the liquid projection
// (swc_oracle.cpp) and the DEM sand step (dem_oracle.cpp): the cubic-spline
// kernel, small fixed-size vectors and the reference's spatial hash searcher.
#pragma once

#include <algorithm>
#include <array>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <numbers>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif


namespace orc {

using ullong = unsigned long long;

// Cubic-spline kernel of SmoothedParticles (Cores/Structures/SmoothedParticles.h:60-72,
// coefficients Cores/Structures/SmoothedParticles.cpp:17-22).
struct Kernel {
    double radius, h, h2, inv_h, inv_h2, c0, c1;
    Kernel() = default;
    Kernel(double r, int dim, double rate = 4) {
        radius = r;
        h      = r * rate;
        h2     = h * h;
        inv_h  = 1 / h;
        inv_h2 = 1 / h2;
        c0     = std::numbers::inv_pi * inv_h2 * (dim == 2 ? 40.0 / 7 : 8 * inv_h);
        c1     = 6 * inv_h * c0;
    }
    double W(double dist) const {
        const double x = dist * inv_h;
        if (x < .5) return c0 * (6 * x * x * (x - 1) + 1);
        if (x < 1) return c0 * 2 * (1 - x) * (1 - x) * (1 - x);
        return 0;
    }
    double dW(double dist) const {
        const double x = dist * inv_h;
        if (x < .5) return c1 * x * (3 * x - 2);
        if (x < 1) return c1 * (1 - x) * (x - 1);
        return 0;
    }
    // SmoothedParticles::getPackedKernelSum (Cores/Structures/SmoothedParticles.cpp:74-80).
    double packedSum(int dim) const {
        if (dim == 2) return W(0) + W(radius * 2) * 6 + W(radius * 2 * std::numbers::sqrt3) * 6;
        return W(0) + W(radius * 2) * 12 + W(radius * 2 * std::numbers::sqrt2) * 6
            + W(radius * 2 * std::numbers::sqrt3) * 24;
    }
};

template<int D> using Vec = std::array<double, D>;

template<int D> inline double dot(const Vec<D> & a, const Vec<D> & b) {
    double s = 0;
    for (int k = 0; k < D; k++) s += a[k] * b[k];
    return s;
}
template<int D> inline Vec<D> sub(const Vec<D> & a, const Vec<D> & b) {
    Vec<D> c;
    for (int k = 0; k < D; k++) c[k] = a[k] - b[k];
    return c;
}
template<int D> inline double norm(const Vec<D> & a) { return std::sqrt(dot<D>(a, a)); }

// -grad W as SmoothedParticles::gradientKernel (SmoothedParticles.h:96-98); a zero
// offset normalises to zero (and W'(0) = 0 anyway).
template<int D> inline Vec<D> gradKernel(const Kernel & k, const Vec<D> & d) {
    const double r = norm<D>(d);
    Vec<D> g{};
    if (r > 0) {
        const double s = -k.dW(r);
        for (int a = 0; a < D; a++) g[a] = s * (d[a] / r);
    }
    return g;
}

// Spatial hash with 2N buckets and a 3^D cell query
// (Cores/Structures/ParticlesNearbySearcher.h:37-74, ParticlesNearbySearcher.cpp:10-35,
// Grid::getQuadraticLower Cores/Structures/Grid.h:70, quadraticNearbyDataPoints Grid.cpp:26-45).
// The visited set is every j with |x_j - x|^2 < h^2 (strict).
template<int D> struct HashGrid {
    static constexpr ullong kP0 = 73856093, kP1 = 19349663, kP2 = 83492791;
    double h = 1, inv_h = 1, h2 = 1;
    std::vector<std::vector<int>> buckets;

    void setRadius(double kr) { h = kr, inv_h = 1 / kr, h2 = kr * kr; }
    std::array<int, D> lower(const Vec<D> & p) const {
        std::array<int, D> c;
        for (int a = 0; a < D; a++) c[a] = int(std::floor(p[a] * inv_h - 0.5));
        return c;
    }
    int key(const std::array<int, D> & c) const {
        ullong v = kP0 * ullong(c[0]) | kP1 * ullong(c[1]);
        if constexpr (D == 3) v |= kP2 * ullong(c[2]);
        return int(v % ullong(buckets.size()));
    }
    void reset(const std::vector<Vec<D>> & pos) {
        buckets.assign(pos.size() * 2, {});
        for (int i = 0; i < int(pos.size()); i++) {
            auto c = lower(pos[i]);
            for (int a = 0; a < D; a++) c[a] += 1;
            buckets[key(c)].push_back(i);
        }
    }
    template<class F> void forEach(const std::vector<Vec<D>> & pos, const Vec<D> & q, F && f) const {
        if (buckets.empty()) return;
        constexpr int K = D == 2 ? 9 : 27;
        std::array<int, K> keys;
        const auto lo = lower(q);
        int n = 0;
        if constexpr (D == 2) {
            for (int j = 0; j < 3; j++)
                for (int i = 0; i < 3; i++) keys[n++] = key({lo[0] + i, lo[1] + j});
        } else {
            for (int k = 0; k < 3; k++)
                for (int j = 0; j < 3; j++)
                    for (int i = 0; i < 3; i++) keys[n++] = key({lo[0] + i, lo[1] + j, lo[2] + k});
        }
        std::sort(keys.begin(), keys.end());
        for (int t = 0; t < K; t++) {
            if (t && keys[t] == keys[t - 1]) continue;
            for (const int j : buckets[keys[t]]) {
                const auto d = sub<D>(pos[j], q);
                if (dot<D>(d, d) < h2) f(j, pos[j]);
            }
        }
    }
};

}  // namespace orc
