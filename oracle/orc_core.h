// orc_core.h -- TEST INFRASTRUCTURE ONLY.
//
// Pieces of the CPU FP64 oracle shared by the liquid projection
// (swc_oracle.cpp) and the DEM sand step (dem_oracle.cpp): the cubic-spline
// kernel, small fixed-size vectors, the reference's spatial hash searcher and a
// cell-grid searcher that visits the same neighbour sets.
#pragma once

#include <algorithm>
#include <array>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
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
    // Number of bucket entries a query at q visits before the distance test (the
    // reference's per-query cost).
    int64_t candidates(const Vec<D> & q) const {
        if (buckets.empty()) return 0;
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
        int64_t c = 0;
        for (int t = 0; t < K; t++)
            if (!t || keys[t] != keys[t - 1]) c += int64_t(buckets[keys[t]].size());
        return c;
    }
};

// Uniform grid over the hash grid's own cells (side h; a particle at x lives in
// cell floor(x / h - 1/2) + 1 and a query at q visits cells floor(q / h - 1/2) + {0, 1, 2}
// per axis), stored as a counting sort: it visits exactly the reference
// searcher's set (every j with |x_j - q|^2 < h^2), in cell order instead of
// bucket order, so FP64 sums differ from the hash grid's only in rounding.  The
// reference's hash degenerates when its bucket count 2N is a power of two: the
// low bits of an OR of three products are mostly ones, so few buckets fill (at
// N = 128^3 a query visits ~3e5 candidates instead of ~2e2).  Large scenes use
// this grid; the hash grid stays the default for the reference's enumeration order.
template<int D> struct CellGrid {
    using Cell = std::array<int64_t, D>;
    double h = 1, inv_h = 1, h2 = 1;
    Cell lo{}, ext{};
    bool dense = true;
    std::vector<int64_t> start;  // dense: offsets per cell of the box (+1); sparse: per distinct cell (+1)
    std::vector<Cell> ucells;    // sparse: distinct cells, ordered by (z, y, x)
    std::vector<int> ids;        // particle ids by cell, ascending within a cell
    int64_t n = 0;

    static bool before(const Cell & a, const Cell & b) {
        for (int t = D - 1; t >= 0; t--)
            if (a[t] != b[t]) return a[t] < b[t];
        return false;
    }
    void setRadius(double kr) { h = kr, inv_h = 1 / kr, h2 = kr * kr; }
    Cell lower(const Vec<D> & p) const {
        Cell c;
        for (int a = 0; a < D; a++) c[a] = int64_t(std::floor(p[a] * inv_h - 0.5));
        return c;
    }
    int64_t lin(const Cell & c) const {
        int64_t k = 0;
        for (int a = D - 1; a >= 0; a--) k = k * ext[a] + (c[a] - lo[a]);
        return k;
    }
    void reset(const std::vector<Vec<D>> & pos) {
        n = int64_t(pos.size());
        ids.assign(pos.size(), 0);
        start.clear();
        ucells.clear();
        if (!n) return;
        std::vector<Cell> c(pos.size());
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < (long long) n; i++) {
            c[i] = lower(pos[i]);
            for (int a = 0; a < D; a++) c[i][a] += 1;
        }
        Cell hi;
        lo = hi = c[0];
        for (int64_t i = 1; i < n; i++)
            for (int a = 0; a < D; a++) lo[a] = std::min(lo[a], c[i][a]), hi[a] = std::max(hi[a], c[i][a]);
        double total = 1;
        for (int a = 0; a < D; a++) ext[a] = hi[a] - lo[a] + 1, total *= double(ext[a]);
        dense = total <= double(8 * n + (int64_t(1) << 20));
        if (dense) {
            const int64_t nc = int64_t(total);
            std::vector<int64_t> key(pos.size());
#pragma omp parallel for schedule(static)
            for (long long i = 0; i < (long long) n; i++) key[i] = lin(c[i]);
            start.assign(nc + 1, 0);
            for (int64_t i = 0; i < n; i++) start[key[i] + 1]++;
            for (int64_t k = 0; k < nc; k++) start[k + 1] += start[k];
            std::vector<int64_t> fill(start.begin(), start.end() - 1);
            for (int64_t i = 0; i < n; i++) ids[fill[key[i]]++] = int(i);
        } else {
            // far outliers: distinct cells sorted, located by binary search
            for (int64_t i = 0; i < n; i++) ids[i] = int(i);
            std::stable_sort(ids.begin(), ids.end(), [&](int a, int b) { return before(c[a], c[b]); });
            for (int64_t t = 0; t < n; t++) {
                const Cell & k = c[ids[t]];
                if (ucells.empty() || ucells.back() != k) ucells.push_back(k), start.push_back(t);
            }
            start.push_back(n);
        }
    }
    template<class F> void forEach(const std::vector<Vec<D>> & pos, const Vec<D> & q, F && f) const {
        if (!n) return;
        const Cell ql = lower(q);
        Cell c;
        auto visit = [&]() {
            int64_t b, e;
            if (dense) {
                for (int a = 0; a < D; a++)
                    if (c[a] < lo[a] || c[a] >= lo[a] + ext[a]) return;
                const int64_t k = lin(c);
                b = start[k], e = start[k + 1];
            } else {
                const auto it = std::lower_bound(ucells.begin(), ucells.end(), c, before);
                if (it == ucells.end() || *it != c) return;
                const size_t u = size_t(it - ucells.begin());
                b = start[u], e = start[u + 1];
            }
            for (int64_t t = b; t < e; t++) {
                const int j = ids[t];
                const auto d = sub<D>(pos[j], q);
                if (dot<D>(d, d) < h2) f(j, pos[j]);
            }
        };
        if constexpr (D == 2) {
            for (int j = 0; j < 3; j++)
                for (int i = 0; i < 3; i++) c = {ql[0] + i, ql[1] + j}, visit();
        } else {
            for (int k = 0; k < 3; k++)
                for (int j = 0; j < 3; j++)
                    for (int i = 0; i < 3; i++) c = {ql[0] + i, ql[1] + j, ql[2] + k}, visit();
        }
    }
};

// The oracle's searcher: the reference's hash grid (default) or the cell grid.
template<int D> struct Searcher {
    HashGrid<D> hash;
    CellGrid<D> cells;
    bool useCells = false;
    void setRadius(double kr) { hash.setRadius(kr), cells.setRadius(kr); }
    void reset(const std::vector<Vec<D>> & pos) {
        if (useCells) cells.reset(pos), hash.buckets.clear();
        else hash.reset(pos), cells.reset({});
    }
    template<class F> void forEach(const std::vector<Vec<D>> & pos, const Vec<D> & q, F && f) const {
        if (useCells) cells.forEach(pos, q, f);
        else hash.forEach(pos, q, f);
    }
};

}  // namespace orc
