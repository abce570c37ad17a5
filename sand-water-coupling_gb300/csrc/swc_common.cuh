// swc_common.cuh -- shared device-side definitions of the GB300 dual-particle
// SPH projection: lattice and brick addressing, the cubic-spline kernel, the
// float-float (double-float) accumulator used by the CG reductions, and the
// launcher declarations shared between translation units.
//
// Layout in HBM
//   * Real and boundary particles are kept sorted by cell (cells are the node
//     cells of the virtual-node lattice, x fastest), as SoA float4 arrays:
//       pos = (x, y, z, V_i)    vel = (vx, vy, vz, m / rho_i)
//     plus an int32 id (original index).  cellStart[ncells + 1] indexes them.
//   * Node-lattice data (virtual particles) lives in 8x8x8 bricks (16x16 in 2D),
//     addressed directly by brick id: value(node) = a[brick * BN + local].  Only
//     bricks flagged active are touched; inactive bricks read as zero.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace swc {

// --------------------------------------------------------------------------
// Brick geometry
// --------------------------------------------------------------------------
template<int DIM> struct BrickGeom;
template<> struct BrickGeom<3> {
    static constexpr int BX = 8, BY = 8, BZ = 8, BN = 512;
    static constexpr int HALO = 4;                                    // virtual stencil reach (|k|^2 < 16)
    static constexpr int TX = BX + 2 * HALO, TY = BY + 2 * HALO, TZ = BZ + 2 * HALO;
    static constexpr int PX = 20;  // row pitch: 16-byte aligned rows, conflict-free LDS.128 for 8 rows
    static constexpr int PXY = PX * TY;
    static constexpr int TILE = PXY * TZ;
};
template<> struct BrickGeom<2> {
    static constexpr int BX = 16, BY = 16, BZ = 1, BN = 256;
    static constexpr int HALO = 4;
    static constexpr int TX = BX + 2 * HALO, TY = BY + 2 * HALO, TZ = 1;
    static constexpr int PX = 24;
    static constexpr int PXY = PX * TY;
    static constexpr int TILE = PXY;
};

// Lattice of nodes (= cells) of the virtual-particle grid.
struct Lattice {
    float  ox, oy, oz;      // node-grid origin (FP32)
    float  dx, inv_dx;      // node spacing
    double ox_d, oy_d, oz_d, dx_d;  // FP64 copies for exact re-tests
    int    nx, ny, nz;      // node counts (nz = 1 in 2D)
    int    bnx, bny, bnz;   // brick counts
    int    nbricks;
    long long ncells;
};

// Kernel / physical constants, passed by value to the particle and node
// kernels.  Keep it at 128 bytes or less (it is 120): 136 bytes, with nothing of
// the kernels' code changed, made the virtual gather 1.8x and the density and
// viscosity passes 4% slower on GB300 (measured with 8 bytes of padding, fast,
// against 16, slow).
struct Phys {
    float h, h2, inv_h, c0h, c1h;   // real / boundary kernel, support h = 4 r
    float H, H2, inv_H, c0H, c1H;   // virtual kernel, support H = 4 * grid spacing
    double h_d, inv_h_d, c0h_d;     // FP64 copies for the activation re-test
    float tie2;                     // band around h^2 of an FP64 re-test of membership within h
    float mass, bmass, inv_mass;
    float rho0, kappa, alpha0;
    int   cell_lo, cell_hi;         // node-centred cell window for a radius-h query
    float gx, gy, gz;               // gravity
    float viscosity;
    int   gravity_on;
};

// ---------------------------------------------------------------------------
// Float-float ("double-single") arithmetic: a value is the unevaluated sum
// hi + lo of two floats with |lo| <= ulp(hi) / 2 (about 48 significant bits)
// on the FP32 pipe, where GB300's FP64 rate is a small fraction of it.  The
// error-free steps are Knuth's two-sum and the FMA form of the exact product
// (Ogita, Rump and Oishi, "Accurate sum and dot product", 2005); the explicit
// _rn intrinsics keep the compiler from contracting or reassociating them.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void two_sum(float a, float b, float & s, float & e) {
    s              = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e              = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// s + e = a + b exactly when |a| >= |b| (or a == 0)
__device__ __forceinline__ void fast_two_sum(float a, float b, float & s, float & e) {
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}
// (hi, lo) += v * (dt + dt_lo)
__device__ __forceinline__ void ff_add_product(float & hi, float & lo, float v, float dt, float dt_lo) {
    const float p  = __fmul_rn(v, dt);
    const float pe = __fmaf_rn(v, dt_lo, __fmaf_rn(v, dt, -p));
    float s, e;
    two_sum(hi, p, s, e);
    e = __fadd_rn(e, __fadd_rn(lo, pe));
    fast_two_sum(s, e, hi, lo);
}
// (h, l) = (ah + al) - (bh + bl)
__device__ __forceinline__ void ff_diff(float ah, float al, float bh, float bl, float & h, float & l) {
    float s, e;
    two_sum(ah, -bh, s, e);
    e = __fadd_rn(e, __fsub_rn(al, bl));
    fast_two_sum(s, e, h, l);
}
// (sh, sl) += (h + l)^2
__device__ __forceinline__ void ff_sqr_add(float h, float l, float & sh, float & sl) {
    const float p  = __fmul_rn(h, h);
    const float c  = __fmaf_rn(__fmul_rn(2.f, h), l, __fmaf_rn(h, h, -p));
    float s, e;
    two_sum(sh, p, s, e);
    e = __fadd_rn(e, __fadd_rn(sl, c));
    fast_two_sum(s, e, sh, sl);
}

// Programmatic dependent launch: a kernel launched with programmatic stream
// serialization waits here until the preceding kernel's memory is visible
// (a no-op for an ordinary launch), then lets the next kernel's blocks be
// dispatched while it runs, which hides the launch gap between short kernels.
__device__ __forceinline__ void pdl_wait_and_release() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Launch with programmatic stream serialization: the kernel's blocks may be
// dispatched while the previous kernel on the stream drains; every kernel
// launched this way calls pdl_wait_and_release() before it touches memory.
template<class Kern, class... Args>
inline void launch_pdl(Kern kernel, dim3 grid, dim3 block, size_t smem, cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim          = grid;
    cfg.blockDim         = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream           = st;
    cudaLaunchAttribute at[1];
    at[0].id                                         = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs    = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, args...);
}

// 1/sqrt(x) for normal x (every caller clamps x >= 1e-30): the hardware
// approximation without the rescaling of denormal inputs that rsqrtf adds.
__device__ __forceinline__ float rsqrt_n(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// --------------------------------------------------------------------------
// Cubic spline (reference: Cores/Structures/SmoothedParticles.h:60-72).
// --------------------------------------------------------------------------
__device__ __forceinline__ float kW(float r, float inv_h, float c0) {
    const float x = r * inv_h;
    if (x < 0.5f) return c0 * (6.f * x * x * (x - 1.f) + 1.f);
    if (x < 1.f) {
        const float t = 1.f - x;
        return c0 * 2.f * t * t * t;
    }
    return 0.f;
}
__device__ __forceinline__ float kdW(float r, float inv_h, float c1) {
    const float x = r * inv_h;
    if (x < 0.5f) return c1 * x * (3.f * x - 2.f);
    if (x < 1.f) return -c1 * (1.f - x) * (1.f - x);
    return 0.f;
}
// W_h(r) and -W'_h(r)/r from r^2 without a division: with q = r/h,
// -W'/r = -c1 (3q - 2)/h for q < 1/2 and c1 (1 - q)^2 / r otherwise; at r = 0 the
// factor stays finite and multiplies a zero offset (gradientKernel(0) = 0).
__device__ __forceinline__ void kernel_and_grad(float r2, float inv_h, float c0, float c1, float & w, float & gsc) {
    const float rinv = rsqrt_n(fmaxf(r2, 1e-30f));
    const float q    = r2 * rinv * inv_h;
    const float t    = 1.f - q;
    const bool inner = q < 0.5f;
    w   = inner ? c0 * (6.f * q * q * (q - 1.f) + 1.f) : (q < 1.f ? c0 * 2.f * t * t * t : 0.f);
    gsc = inner ? -c1 * inv_h * (3.f * q - 2.f) : (q < 1.f ? c1 * t * t * rinv : 0.f);
}
// Packed FP32x2 helpers (two particles or two nodes per thread).
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 max02(float2 a) { return make_float2(fmaxf(a.x, 0.f), fmaxf(a.y, 0.f)); }

// Cubic spline of two squared distances in the clamped form used by the packed
// kernels: with q = r / h, a = max(1 - q, 0) (0 where the mask is off) and
// b = max(a - 1/2, 0),
//   W_h = 2 c0h w,          w = a^3 - 4 b^3,
//   -W'_h(r) / r = c1h g,   g = (a^2 - 4 b^2) / r,
// which equals the piecewise form (q < 1/2: 1 - 6q^2 + 6q^3 and (2 - 3q)/h;
// 1/2 <= q < 1: 2 (1 - q)^3 and (1 - q)^2 / r; 0 beyond).  ri = 1/r (r2 >= 1e-30).
struct Spline2 {
    float2 w, g, ri;
};
__device__ __forceinline__ Spline2 spline2(float2 r2, bool m0, bool m1, float inv_h) {
    Spline2 o;
    o.ri            = make_float2(rsqrt_n(fmaxf(r2.x, 1e-30f)), rsqrt_n(fmaxf(r2.y, 1e-30f)));
    const float2 q  = mul2(mul2(r2, o.ri), f2(inv_h));
    float2 a        = max02(fma2(q, f2(-1.f), f2(1.f)));
    a               = make_float2(m0 ? a.x : 0.f, m1 ? a.y : 0.f);
    const float2 b  = max02(add2(a, f2(-0.5f)));
    const float2 a2 = mul2(a, a), b2 = mul2(b, b);
    o.w             = fma2(mul2(b2, b), f2(-4.f), mul2(a2, a));
    o.g             = mul2(fma2(b2, f2(-4.f), a2), o.ri);
    return o;
}

__device__ __forceinline__ double kW_d(double r, double inv_h, double c0) {
    const double x = r * inv_h;
    if (x < .5) return c0 * (6 * x * x * (x - 1) + 1);
    if (x < 1) return c0 * 2 * (1 - x) * (1 - x) * (1 - x);
    return 0;
}

// --------------------------------------------------------------------------
// Float-float accumulation (error-free transforms, Knuth TwoSum / FMA TwoProd).
// Products are exact; sums keep ~44 significant bits.  Used below the warp
// level; warp partials are converted to FP64 and summed in FP64.
// --------------------------------------------------------------------------
struct FF {
    float hi, lo;
};
__device__ __forceinline__ void ff_add(FF & a, float b) {
    const float s  = __fadd_rn(a.hi, b);
    const float bb = __fsub_rn(s, a.hi);
    const float e  = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    a.hi = s;
    a.lo = __fadd_rn(a.lo, e);
}
__device__ __forceinline__ void ff_add_prod(FF & a, float x, float y) {
    const float p  = __fmul_rn(x, y);
    const float pe = __fmaf_rn(x, y, -p);
    ff_add(a, p);
    a.lo = __fadd_rn(a.lo, pe);
}
__device__ __forceinline__ double ff_to_double(const FF & a) { return double(a.hi) + double(a.lo); }

// Block-wide FP64 sum of one double per thread; result valid in thread 0.
template<int NT> __device__ __forceinline__ double block_sum_double(double v, double * sm) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sm[w] = v;
    __syncthreads();
    double s = 0;
    if (threadIdx.x == 0) {
        for (int i = 0; i < NT / 32; i++) s += sm[i];
    }
    __syncthreads();
    return s;
}

// Warp-level reduction of a float-float value to FP64 (lane 0), then block FP64 sum.
template<int NT> __device__ __forceinline__ double block_sum_ff(FF a, double * sm) {
    double v = ff_to_double(a);
    return block_sum_double<NT>(v, sm);
}

// Block-wide FP64 sum returned to every thread of the block.
template<int NT> __device__ __forceinline__ double block_sum_double_all(double v, double * sm) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sm[w] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int i = 0; i < NT / 32; i++) s += sm[i];
        sm[NT / 32] = s;
    }
    __syncthreads();
    return sm[NT / 32];
}

// Grid-wide deterministic reduction of NV values.  Thread 0 of every block
// publishes its block's values part[k] at partials[k * gridDim.x + blockIdx.x];
// the block that arrives last sums each value over all blocks with all of its
// threads in a fixed order and returns true with the totals in out[k] (every
// thread of that block).  `sm` needs NT/32 + 1 doubles, `flag` is a shared int.
template<int NT, int NV>
__device__ __forceinline__ bool grid_reduce(const double (&part)[NV], double * partials, unsigned int * ticket,
                                            double (&out)[NV], double * sm, int * flag) {
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) partials[k * gridDim.x + blockIdx.x] = part[k];
        __threadfence();
        *flag = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!*flag) return false;
    __threadfence();
#pragma unroll
    for (int k = 0; k < NV; k++) {
        double s = 0;
        for (unsigned int i = threadIdx.x; i < gridDim.x; i += NT) s += __ldcg(partials + k * gridDim.x + i);
        out[k] = block_sum_double_all<NT>(s, sm);
    }
    if (threadIdx.x == 0) *ticket = 0u;
    return true;
}

// --------------------------------------------------------------------------
// Node / brick addressing.
// --------------------------------------------------------------------------
template<int DIM> __device__ __forceinline__ long long node_slot(const Lattice & L, int x, int y, int z) {
    using G = BrickGeom<DIM>;
    const int bx = x / G::BX, by = y / G::BY, bz = DIM == 3 ? z / G::BZ : 0;
    const int lx = x - bx * G::BX, ly = y - by * G::BY, lz = DIM == 3 ? z - bz * G::BZ : 0;
    const long long b = (long long) bx + (long long) L.bnx * (by + (long long) L.bny * bz);
    return b * G::BN + lx + G::BX * (ly + G::BY * lz);
}
__device__ __forceinline__ int brick_of(const Lattice & L, int x, int y, int z, int bxs, int bys, int bzs) {
    return x / bxs + L.bnx * (y / bys + L.bny * (z / bzs));
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Cell index of a position (cells = node cells, clamped to the lattice).
template<int DIM> __device__ __forceinline__ int3 cell_of(const Lattice & L, float x, float y, float z) {
    int3 c;
    c.x = clampi(__float2int_rd((x - L.ox) * L.inv_dx), 0, L.nx - 1);
    c.y = clampi(__float2int_rd((y - L.oy) * L.inv_dx), 0, L.ny - 1);
    c.z = DIM == 3 ? clampi(__float2int_rd((z - L.oz) * L.inv_dx), 0, L.nz - 1) : 0;
    return c;
}
__device__ __forceinline__ long long cell_linear(const Lattice & L, int3 c) {
    return (long long) c.x + (long long) L.nx * (c.y + (long long) L.ny * c.z);
}

// Lower / upper edge of cell row `c` along an axis: border cells extend to infinity
// (they also hold particles clamped in from outside the lattice).
__device__ __forceinline__ float slab_dist(float q, int c, int n, float o, float dx) {
    const float lo = (c == 0) ? -3.0e38f : o + c * dx;
    const float hi = (c == n - 1) ? 3.0e38f : o + (c + 1) * dx;
    return q < lo ? lo - q : (q > hi ? q - hi : 0.f);
}

// Neighbour iteration over cells for a query point and radius R (particle
// queries): rows pruned by their slab distance, x-range per row from the
// remaining radius; f(j) for every particle j of the visited cells.
template<int DIM, class F>
__device__ __forceinline__ void for_each_in_radius(const Lattice & L, const int * __restrict__ cellStart,
                                                   float qx, float qy, float qz, float R, float R2, F && f) {
    const int cy0 = clampi(__float2int_rd((qy - R - L.oy) * L.inv_dx), 0, L.ny - 1);
    const int cy1 = clampi(__float2int_rd((qy + R - L.oy) * L.inv_dx), 0, L.ny - 1);
    int cz0 = 0, cz1 = 0;
    if (DIM == 3) {
        cz0 = clampi(__float2int_rd((qz - R - L.oz) * L.inv_dx), 0, L.nz - 1);
        cz1 = clampi(__float2int_rd((qz + R - L.oz) * L.inv_dx), 0, L.nz - 1);
    }
    for (int cz = cz0; cz <= cz1; cz++) {
        const float dz  = DIM == 3 ? slab_dist(qz, cz, L.nz, L.oz, L.dx) : 0.f;
        const float rz2 = R2 - dz * dz;
        if (rz2 <= 0.f) continue;
        for (int cy = cy0; cy <= cy1; cy++) {
            const float dy  = slab_dist(qy, cy, L.ny, L.oy, L.dx);
            const float rem = rz2 - dy * dy;
            if (rem <= 0.f) continue;
            const float rx = sqrtf(rem) * 1.000001f + 1e-7f * L.dx;
            const int cx0  = clampi(__float2int_rd((qx - rx - L.ox) * L.inv_dx), 0, L.nx - 1);
            const int cx1  = clampi(__float2int_rd((qx + rx - L.ox) * L.inv_dx), 0, L.nx - 1);
            const long long row = (long long) L.nx * (cy + (long long) L.ny * cz);
            const int b = cellStart[row + cx0], e = cellStart[row + cx1 + 1];
            for (int j = b; j < e; j++) f(j);
        }
    }
}

// The same visit for two query points a and b at once (neighbours in the
// sorted order, normally in one cell row): rows within R of either point and,
// per row, the union of the two x-ranges, so f(j) sees every particle that
// either single-point visit would (and a few more, which the caller's exact
// distance tests reject).  The x reach comes from the hardware rsqrt with a
// relative margin of 1e-5 (its error is below 3e-7).
template<int DIM, class F>
__device__ __forceinline__ void for_each_in_radius2(const Lattice & L, const int * __restrict__ cellStart, float3 a,
                                                    float3 b, float R, float R2, F && f) {
    const int cy0 = clampi(__float2int_rd((fminf(a.y, b.y) - R - L.oy) * L.inv_dx), 0, L.ny - 1);
    const int cy1 = clampi(__float2int_rd((fmaxf(a.y, b.y) + R - L.oy) * L.inv_dx), 0, L.ny - 1);
    int cz0 = 0, cz1 = 0;
    if (DIM == 3) {
        cz0 = clampi(__float2int_rd((fminf(a.z, b.z) - R - L.oz) * L.inv_dx), 0, L.nz - 1);
        cz1 = clampi(__float2int_rd((fmaxf(a.z, b.z) + R - L.oz) * L.inv_dx), 0, L.nz - 1);
    }
    for (int cz = cz0; cz <= cz1; cz++) {
        float rza = R2, rzb = R2;
        if (DIM == 3) {
            const float da = slab_dist(a.z, cz, L.nz, L.oz, L.dx), db = slab_dist(b.z, cz, L.nz, L.oz, L.dx);
            rza -= da * da;
            rzb -= db * db;
        }
        if (rza <= 0.f && rzb <= 0.f) continue;
        for (int cy = cy0; cy <= cy1; cy++) {
            const float ya = slab_dist(a.y, cy, L.ny, L.oy, L.dx), yb = slab_dist(b.y, cy, L.ny, L.oy, L.dx);
            const float ra = rza - ya * ya, rb = rzb - yb * yb;
            if (ra <= 0.f && rb <= 0.f) continue;
            float lo = 3.0e38f, hi = -3.0e38f;
            if (ra > 0.f) {
                const float rx = ra * rsqrt_n(fmaxf(ra, 1e-30f)) * 1.00001f + 1e-6f * L.dx;
                lo = a.x - rx;
                hi = a.x + rx;
            }
            if (rb > 0.f) {
                const float rx = rb * rsqrt_n(fmaxf(rb, 1e-30f)) * 1.00001f + 1e-6f * L.dx;
                lo = fminf(lo, b.x - rx);
                hi = fmaxf(hi, b.x + rx);
            }
            const int cx0 = clampi(__float2int_rd((lo - L.ox) * L.inv_dx), 0, L.nx - 1);
            const int cx1 = clampi(__float2int_rd((hi - L.ox) * L.inv_dx), 0, L.nx - 1);
            const long long row = (long long) L.nx * (cy + (long long) L.ny * cz);
            const int jb = cellStart[row + cx0], je = cellStart[row + cx1 + 1];
            for (int j = jb; j < je; j++) f(j);
        }
    }
}

// Row-parallel form of for_each_in_radius for one query point: the caller's
// lane `lane` of `nl` visits the rows lane, lane + nl, ... of the (z, y) row
// window (same pruning and x-ranges), so a warp walks one point's neighbours
// about 25 times faster than a single thread (used for the few particles left
// over by the paired kernels).
template<int DIM, class F>
__device__ __forceinline__ void for_rows_in_radius(const Lattice & L, const int * __restrict__ cellStart, float qx,
                                                   float qy, float qz, float R, float R2, int lane, int nl, F && f) {
    const int cy0 = clampi(__float2int_rd((qy - R - L.oy) * L.inv_dx), 0, L.ny - 1);
    const int cy1 = clampi(__float2int_rd((qy + R - L.oy) * L.inv_dx), 0, L.ny - 1);
    int cz0 = 0, cz1 = 0;
    if (DIM == 3) {
        cz0 = clampi(__float2int_rd((qz - R - L.oz) * L.inv_dx), 0, L.nz - 1);
        cz1 = clampi(__float2int_rd((qz + R - L.oz) * L.inv_dx), 0, L.nz - 1);
    }
    const int nyr = cy1 - cy0 + 1, nrows = nyr * (cz1 - cz0 + 1);
    for (int r = lane; r < nrows; r += nl) {
        const int cy = cy0 + r % nyr, cz = cz0 + r / nyr;
        const float dz = DIM == 3 ? slab_dist(qz, cz, L.nz, L.oz, L.dx) : 0.f;
        const float dy = slab_dist(qy, cy, L.ny, L.oy, L.dx);
        const float rem = R2 - dz * dz - dy * dy;
        if (rem <= 0.f) continue;
        const float rx = rem * rsqrt_n(fmaxf(rem, 1e-30f)) * 1.00001f + 1e-6f * L.dx;
        const int cx0  = clampi(__float2int_rd((qx - rx - L.ox) * L.inv_dx), 0, L.nx - 1);
        const int cx1  = clampi(__float2int_rd((qx + rx - L.ox) * L.inv_dx), 0, L.nx - 1);
        const long long row = (long long) L.nx * (cy + (long long) L.ny * cz);
        const int jb = cellStart[row + cx0], je = cellStart[row + cx1 + 1];
        for (int j = jb; j < je; j++) f(j);
    }
}

// Deterministic warp sum (xor butterfly; every lane gets the total).
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// End of a kernel that consumed the counter q[0]: the last block to get here
// zeroes q[0] and the finish counter q[1], so the pair is zeroed once, at
// allocation.  Every thread of every block calls it after its last read of q[0].
__device__ __forceinline__ void grid_done_reset(int * q) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(q + 1, 1) == int(gridDim.x) - 1) {
            atomicExch(q, 0);
            atomicExch(q + 1, 0);
        }
    }
}

// Two consecutive sorted particles share one neighbour visit when they lie in
// the same cell row at most one cell apart.
template<int DIM> __device__ __forceinline__ bool near_pair(const Lattice & L, float4 a, float4 b) {
    const int3 ca = cell_of<DIM>(L, a.x, a.y, a.z), cb = cell_of<DIM>(L, b.x, b.y, b.z);
    return ca.y == cb.y && ca.z == cb.z && abs(ca.x - cb.x) <= 1;
}

// Friction-free wall term of the pressure-gradient update for particle
// (q, vi): - sum_b V_b min(n_b.(v_i - v_b), 0) n_b W_h(x_i - x_b)
// (VirtualParticle::applyPressureGradient, Cores/Structures/VirtualParticle.cpp:122-128).
template<int DIM>
__device__ __forceinline__ float3 wall_term(const Lattice & L, const Phys & P, const int * __restrict__ bcellStart,
                                            const float4 * __restrict__ bpos, const float4 * __restrict__ bvel,
                                            const float4 * __restrict__ bnrm, float4 q, float4 vi) {
    float3 f = make_float3(0.f, 0.f, 0.f);
    for_each_in_radius<DIM>(L, bcellStart, q.x, q.y, q.z, P.h, P.h2, [&](int j) {
        const float4 p = bpos[j];
        const float dx = q.x - p.x, dy = q.y - p.y, dz = q.z - p.z;
        const float r2 = dx * dx + dy * dy + dz * dz;
        if (r2 < P.h2) {
            const float4 nb = bnrm[j];
            const float4 vb = bvel[j];
            const float vn  = fminf(nb.x * (vi.x - vb.x) + nb.y * (vi.y - vb.y) + nb.z * (vi.z - vb.z), 0.f);
            const float c   = p.w * vn * kW(sqrtf(r2), P.inv_h, P.c0h);
            f.x -= c * nb.x;
            f.y -= c * nb.y;
            f.z -= c * nb.z;
        }
    });
    return f;
}

// --------------------------------------------------------------------------
// CG device state (one per context).
// --------------------------------------------------------------------------
struct CgState {
    double bb;         // |b|^2
    double rr;         // |r_i|^2
    double rr_prev;    // |r_{i-1}|^2
    double pq;         // d_i . A d_i
    double threshold;  // max(tol^2 |b|^2, DBL_MIN)
    double rr0;        // initial |r_0|^2
    int    iter;       // completed iterations (SpMV count in the loop)
    int    done;       // 0 running, 1 converged, 2 max iterations, 3 breakdown / NaN
    int    max_iter;
    int    start;      // start kept by k_cg_start: 0 prediction, 1 base
    double sums[4];    // residual sums of the CG start: |r|^2, |b|^2 (prediction / only start), |r|^2, |b|^2 (base)
    unsigned int ticket[4];
    int    is_last[4];
};

}  // namespace swc
