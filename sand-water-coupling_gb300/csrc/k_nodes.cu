// k_nodes.cu -- virtual-node (lattice) kernels of the dual-particle SPH
// projection: active-brick list, the fused virtual gather (weight, rho_I, V_I,
// vbar_I, D_I in one pass), reference-order compaction, the clamped diagonal
// alpha_hat, warm starts and the matrix-free CG (stencil SpMV fused with the
// search-direction update, and the x/r update), all with deterministic
// FP64 reductions.
#include "swc_kernels.h"
#include "swc_tiles.cuh"

namespace swc {


// ---------------------------------------------------------------------------
// Active-brick list (single CTA, ascending brick id).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_brick_list(const unsigned char * __restrict__ bflag, int nbricks,
                                                     int * __restrict__ list, int * __restrict__ count) {
    pdl_wait_and_release();
    __shared__ int sm[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nbricks; base += 1024) {
        const int i = base + threadIdx.x;
        const int v = (i < nbricks && bflag[i]) ? 1 : 0;
        int x       = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if ((threadIdx.x & 31) >= o) x += y;
        }
        if ((threadIdx.x & 31) == 31) sm[threadIdx.x >> 5] = x;
        __syncthreads();
        if (threadIdx.x < 32) {
            int w = sm[threadIdx.x];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, w, o);
                if (threadIdx.x >= o) w += y;
            }
            sm[threadIdx.x] = w;
        }
        __syncthreads();
        const int incl = x + ((threadIdx.x >> 5) ? sm[(threadIdx.x >> 5) - 1] : 0) + carry;
        if (v) list[incl - 1] = i;
        __syncthreads();
        if (threadIdx.x == 1023) carry = incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) *count = carry;
}

// Sums of two x-adjacent nodes, packed as FP32x2 (.x: node n, .y: node n + 1).
// The kernel scale factors are applied once at the end:
//   W_h = 2 c0h w,  -W'_h / r = c1h g,  W_H = c0H wH  (see pair_add).
struct NodeSums2 {
    float2 wsum, rhoI, VI, cnt, ux, uy, uz, bw, dvg, gx, gy, gz;
};

// Contributions of one particle (position / volume p, velocity / m-over-rho u)
// to two nodes at x offsets dxx = x_I - x_j (dy, dz shared), squared distances
// r2 and masks m0 / m1 = (r2 < h^2).
// With q = r / h, a = max(1 - q, 0) and b = max(a - 1/2, 0) the cubic spline is
//   W_h = c0h (2 a^3 - 8 b^3) = 2 c0h w,   w = a^3 - 4 b^3,
//   -W'_h(r) / r = (6 c0h / h) (a^2 - 4 b^2) / r = c1h g,
// (q < 1/2: 2 - 3q over h; 1/2 <= q < 1: (1 - q)^2 / r; 0 beyond), and a node
// only takes particles with r^2 < h^2 (a is zeroed otherwise).  rho_I uses W_H
// truncated at h: for H >= 2h (FAST_H) only its inner branch
// wH = 1 + 6 x^2 (x - 1), x = r / H, is reached; otherwise wH = 2 aH^3 - 8 bH^3.
// FEAT adds the real-neighbour count (a feature of the learned warm start).
template<bool REAL, bool FAST_H, bool FEAT>
__device__ __forceinline__ void pair_add(NodeSums2 & s, const Phys & P, float2 dxx, float dy, float dz, float2 r2,
                                         bool m0, bool m1, float4 p, float4 u) {
    const float2 ri = make_float2(rsqrt_n(fmaxf(r2.x, 1e-30f)), rsqrt_n(fmaxf(r2.y, 1e-30f)));
    const float2 q  = mul2(mul2(r2, ri), f2(P.inv_h));
    float2 a        = max02(fma2(q, f2(-1.f), f2(1.f)));
    a               = make_float2(m0 ? a.x : 0.f, m1 ? a.y : 0.f);
    const float2 b  = max02(add2(a, f2(-0.5f)));
    const float2 a2 = mul2(a, a), b2 = mul2(b, b);
    const float2 w  = fma2(mul2(b2, b), f2(-4.f), mul2(a2, a));
    const float2 g  = mul2(fma2(b2, f2(-4.f), a2), ri);
    if (REAL) {
        float2 wH;
        const float2 x = mul2(q, f2(P.h * P.inv_H));
        if (FAST_H) {
            wH = fma2(mul2(mul2(x, x), add2(x, f2(-1.f))), f2(6.f), f2(1.f));
            wH = make_float2(m0 ? wH.x : 0.f, m1 ? wH.y : 0.f);
        } else {
            float2 aH = max02(fma2(x, f2(-1.f), f2(1.f)));
            aH        = make_float2(m0 ? aH.x : 0.f, m1 ? aH.y : 0.f);
            const float2 bH = max02(add2(aH, f2(-0.5f)));
            wH = fma2(mul2(mul2(bH, bH), bH), f2(-8.f), mul2(mul2(mul2(aH, aH), aH), f2(2.f)));
        }
        s.wsum = add2(s.wsum, w);
        s.rhoI = add2(s.rhoI, wH);
        s.VI   = fma2(f2(p.w * p.w), w, s.VI);
        if (FEAT) s.cnt = add2(s.cnt, make_float2(m0 ? 1.f : 0.f, m1 ? 1.f : 0.f));
    }
    const float2 mw = mul2(f2(u.w), w);
    s.ux  = fma2(f2(u.x), mw, s.ux);
    s.uy  = fma2(f2(u.y), mw, s.uy);
    s.uz  = fma2(f2(u.z), mw, s.uz);
    s.bw  = fma2(f2(p.w), w, s.bw);
    const float2 c  = mul2(f2(p.w), g);
    const float2 ud = fma2(f2(u.x), dxx, f2(fmaf(u.y, dy, u.z * dz)));
    s.dvg = fma2(c, ud, s.dvg);
    s.gx  = fma2(c, dxx, s.gx);
    s.gy  = fma2(c, f2(dy), s.gy);
    s.gz  = fma2(c, f2(dz), s.gz);
}

// ---------------------------------------------------------------------------
// Fused virtual gather.  For every node of an active brick, one pass over the
// real and boundary particles within h gives (reference VirtualParticle.cpp):
//   weight  = sum_j W_h                                  (:50-56, activation > 1e-6)
//   rho_I   = m sum_j W_H  (real searcher -> W_H truncated at h)   (:18-27)
//   V_I     = sum_j V_j^2 W_h                            (:29-38)
//   vbar_I  = [sum (m/rho)_j v_j W_h] / [sum V_j W_h + 1e-6]        (:137-147)
//   D_I     = sum V_j v_j.g_j - vbar_I . sum V_j g_j - kappa max(rho_I - rho0, 0)/rho0   (:172-201)
// with g_j = -W'_h(r) (x_I - x_j)/r  and sums over real + boundary particles
// (boundary: m_b, rho_b, V_b) except weight, rho_I and V_I (real only).
// Each thread handles NX consecutive nodes along x: the candidate particles of a
// cell row are loaded once for all of them and tested by exact distance, so
// every node still sums exactly its neighbours within h, in cell-row order.
// Five 128-thread blocks per SM (96 registers, no spills): 10% faster than the
// unconstrained 109-register build at four blocks.
// ---------------------------------------------------------------------------
template<int DIM, bool FAST_H, bool FEAT>
__global__ void __launch_bounds__(128, 5) k_node_gather(Lattice L, Phys P, const int * __restrict__ blist,
                                                    const int * __restrict__ bcount, NodeArrays N,
                                                    const float4 * __restrict__ pos, const float4 * __restrict__ vel,
                                                    const int * __restrict__ cellStart,
                                                    const float4 * __restrict__ bpos,
                                                    const float4 * __restrict__ bvel,
                                                    const int * __restrict__ bcellStart,
                                                    const unsigned char * __restrict__ bnear,
                                                    const unsigned char * __restrict__ bcell, int * queue) {
    pdl_wait_and_release();
    using G          = BrickGeom<DIM>;
    constexpr int NX = 2;
    constexpr int XS = G::BX / NX;  // thread columns per brick row
    constexpr int TPB = G::BN / NX;
    __shared__ int slot;
    const int nb = *bcount;
    for (int bi = queue_take(queue, &slot); bi < nb; bi = queue_take(queue, &slot)) {
        const int b     = blist[bi];
        const int3 bc   = brick_coords(L, b);
        const bool walls = bnear[b] != 0;  // boundary particles only near walls
        for (int l4 = threadIdx.x; l4 < TPB; l4 += blockDim.x) {
            const int lx0 = (l4 % XS) * NX, ly = (l4 / XS) % G::BY, lz = l4 / (XS * G::BY);
            const int x0 = bc.x * G::BX + lx0, y = bc.y * G::BY + ly, z = bc.z * G::BZ + lz;
            const long long s0 = (long long) b * G::BN + lx0 + G::BX * (ly + G::BY * lz);
            const bool row_in = y < L.ny && (DIM == 2 || z < L.nz);
            // and, per node pair, only when a node's cell is within reach of the boundary
            int npass = 1;
            if (walls && row_in && x0 < L.nx) {
                const long long c0 = (long long) x0 + (long long) L.nx * (y + (long long) L.ny * z);
                if (bcell[c0] || (x0 + 1 < L.nx && bcell[c0 + 1])) npass = 2;
            }
            NodeSums2 a;
            a.wsum = a.rhoI = a.VI = a.cnt = a.ux = a.uy = a.uz = a.bw = a.dvg = a.gx = a.gy = a.gz = f2(0.f);
            // node positions of the FP64 lattice (the oracle's nodes) as float-float
            // pairs: x_I - x_j = (hi - x_j) + lo is then exact to a few ulp of the
            // offset, where an FP32 node position would carry ~1e-7 of rounding
            float2 xn, xl, yzn, yzl;
            {
                const double xd0 = L.ox_d + x0 * L.dx_d, xd1 = L.ox_d + (x0 + 1) * L.dx_d, yd = L.oy_d + y * L.dx_d,
                             zd = DIM == 3 ? L.oz_d + z * L.dx_d : 0.0;
                xn  = make_float2(float(xd0), float(xd1));
                xl  = make_float2(float(xd0 - double(xn.x)), float(xd1 - double(xn.y)));
                yzn = make_float2(float(yd), float(zd));
                yzl = make_float2(float(yd - double(yzn.x)), float(zd - double(yzn.y)));
            }
            const int cxa = max(x0 + P.cell_lo, 0), cxb = min(x0 + NX - 1 + P.cell_hi, L.nx - 1);
            const int cy0 = max(y + P.cell_lo, 0), cy1 = min(y + P.cell_hi, L.ny - 1);
            const int cz0 = DIM == 3 ? max(z + P.cell_lo, 0) : 0, cz1 = DIM == 3 ? min(z + P.cell_hi, L.nz - 1) : 0;
            if (row_in) {
#pragma unroll 1
                for (int pass = 0; pass < npass; pass++) {
                    const int * cs   = pass == 0 ? cellStart : bcellStart;
                    const float4 * X = pass == 0 ? pos : bpos;
                    const float4 * U = pass == 0 ? vel : bvel;
                    // cell rows (cy, cz) in order; the next row's range and the next
                    // candidate's position / velocity are loaded one step ahead
                    int cy = cy0, cz = cz0;
                    long long row = (long long) L.nx * (cy + (long long) L.ny * cz);
                    int jb = cs[row + cxa], je = cs[row + cxb + 1];
                    for (;;) {
                        int ny = cy + 1, nz = cz;
                        if (ny > cy1) ny = cy0, nz++;
                        const bool more = nz <= cz1;
                        int nb_ = 0, ne_ = 0;
                        if (more) {
                            const long long nrow = (long long) L.nx * (ny + (long long) L.ny * nz);
                            nb_ = cs[nrow + cxa];
                            ne_ = cs[nrow + cxb + 1];
                        }
                        float4 pn = make_float4(0.f, 0.f, 0.f, 0.f), un = pn;
                        if (jb < je) pn = X[jb], un = U[jb];
                        for (int j = jb; j < je; j++) {
                            const float4 p = pn, u = un;
                            if (j + 1 < je) pn = X[j + 1], un = U[j + 1];
                            const float2 dyz = add2(add2(yzn, make_float2(-p.y, -p.z)), yzl);
                            const float dy = dyz.x, dz = DIM == 3 ? dyz.y : 0.f;
                            const float ryz = fmaf(dz, dz, dy * dy);
                            if (ryz >= P.h2 + P.tie2) continue;
                            const float2 dxx = add2(add2(xn, f2(-p.x)), xl);
                            const float2 r2  = fma2(dxx, dxx, f2(ryz));
                            const float2 e2  = add2(r2, f2(-P.h2));
                            bool m0 = e2.x < 0.f, m1 = e2.y < 0.f;
                            if (pass == 0 && fminf(fabsf(e2.x), fabsf(e2.y)) < P.tie2) {
                                // rho_I sums W_H cut at h, which jumps there: membership
                                // within rounding of r = h is decided in FP64 from the
                                // exact positions, as the oracle's strict |d|^2 < h^2
                                // (summed x, y, z in the oracle's order)
                                const double xd0 = L.ox_d + x0 * L.dx_d, xd1 = L.ox_d + (x0 + 1) * L.dx_d;
                                const double yd = L.oy_d + y * L.dx_d, zd = DIM == 3 ? L.oz_d + z * L.dx_d : 0.0;
                                const double hh = P.h_d * P.h_d, ey = double(p.y) - yd, ez = double(p.z) - zd;
                                const double e0 = double(p.x) - xd0, e1 = double(p.x) - xd1;
                                const double s0 = fma(ey, ey, e0 * e0), s1 = fma(ey, ey, e1 * e1);
                                m0 = (DIM == 3 ? fma(ez, ez, s0) : s0) < hh;
                                m1 = (DIM == 3 ? fma(ez, ez, s1) : s1) < hh;
                            }
                            if (!(m0 || m1)) continue;
                            if (pass == 0) pair_add<true, FAST_H, FEAT>(a, P, dxx, dy, dz, r2, m0, m1, p, u);
                            else pair_add<false, FAST_H, FEAT>(a, P, dxx, dy, dz, r2, m0, m1, p, u);
                        }
                        if (!more) break;
                        cy = ny, cz = nz, jb = nb_, je = ne_;
                    }
                }
            }
#pragma unroll
            for (int n = 0; n < NX; n++) {
                const int x       = x0 + n;
                const long long s = s0 + n;
                if (!row_in || x >= L.nx) {
                    N.flag[s] = 0;
                    N.V[s]    = 0.f;
                    N.D[s]    = 0.f;
                    N.rho[s]  = 0.f;
                    if (N.nreal) N.nreal[s] = 0;
                    if (N.vbar) N.vbar[s] = make_float4(0.f, 0.f, 0.f, 0.f);
                    continue;
                }
                auto pick = [n](float2 v) { return n == 0 ? v.x : v.y; };
                const float w2 = 2.f * P.c0h;
                const float wsum = w2 * pick(a.wsum);
                const float gx = P.c1h * pick(a.gx), gy = P.c1h * pick(a.gy), gz = P.c1h * pick(a.gz);
                bool active = wsum > 1e-6f;
                if (fabsf(wsum - 1e-6f) <= 1e-9f) {
                    // borderline: redo the weight in FP64 from the same float positions
                    const double xd = L.ox_d + x * L.dx_d, yd = L.oy_d + y * L.dx_d,
                                 zd = DIM == 3 ? L.oz_d + z * L.dx_d : 0.0;
                    const int cx0 = max(x + P.cell_lo, 0), cx1 = min(x + P.cell_hi, L.nx - 1);
                    double ws = 0;
                    for (int cz = cz0; cz <= cz1; cz++)
                        for (int cy = cy0; cy <= cy1; cy++) {
                            const long long row = (long long) L.nx * (cy + (long long) L.ny * cz);
                            for (int j = cellStart[row + cx0]; j < cellStart[row + cx1 + 1]; j++) {
                                const float4 p  = pos[j];
                                const double ex = xd - p.x, ey = yd - p.y, ez = DIM == 3 ? zd - p.z : 0.0;
                                const double r2 = ex * ex + ey * ey + ez * ez;
                                if (r2 < P.h_d * P.h_d) ws += kW_d(sqrt(r2), P.inv_h_d, P.c0h_d);
                            }
                        }
                    active = ws > 1e-6;
                }
                const float den = w2 * pick(a.bw) + 1e-6f;
                const float vbx = w2 * pick(a.ux) / den, vby = w2 * pick(a.uy) / den, vbz = w2 * pick(a.uz) / den;
                const float rho = pick(a.rhoI) * (P.mass * P.c0H);
                const float Dv  = P.c1h * pick(a.dvg) - (vbx * gx + vby * gy + vbz * gz) -
                                 P.kappa * fmaxf(rho - P.rho0, 0.f) / P.rho0;
                N.flag[s] = active ? 1 : 0;
                N.V[s]    = active ? w2 * pick(a.VI) : 0.f;
                N.D[s]    = active ? Dv : 0.f;
                N.rho[s]  = active ? rho : 0.f;
                if (FEAT) N.nreal[s] = (unsigned short) min(int(pick(a.cnt)), 65535);
                if (N.vbar) N.vbar[s] = make_float4(vbx, vby, vbz, 0.f);
            }
        }
    }
    queue_finish(queue);
}

// ---------------------------------------------------------------------------
// Reference-order (x-fastest over the whole node grid, Grid.cpp:231-244)
// compaction: per (row, brick column) segment counts, scanned.
// ---------------------------------------------------------------------------
template<int DIM>
__global__ void __launch_bounds__(kNT) k_segment_count(Lattice L, const int * __restrict__ blist,
                                                       const int * __restrict__ bcount,
                                                       const unsigned char * __restrict__ flag, int * __restrict__ seg) {
    pdl_wait_and_release();
    using G      = BrickGeom<DIM>;
    const int nb = *bcount;
    constexpr int ROWS = G::BY * G::BZ;
    for (int bi = blockIdx.x; bi < nb; bi += gridDim.x) {
        const int b   = blist[bi];
        const int3 bc = brick_coords(L, b);
        for (int rrow = threadIdx.x; rrow < ROWS; rrow += kNT) {
            const int ly = rrow % G::BY, lz = rrow / G::BY;
            const int y = bc.y * G::BY + ly, z = bc.z * G::BZ + lz;
            if (y >= L.ny || (DIM == 3 && z >= L.nz)) continue;
            const unsigned char * f = flag + (long long) b * G::BN + G::BX * rrow;
            int c = 0;
#pragma unroll
            for (int k = 0; k < G::BX; k++) c += f[k];
            seg[((long long) z * L.ny + y) * L.bnx + bc.x] = c;
        }
    }
}

// alpha0 calibration (VirtualParticle::setAlpha, VirtualParticle.cpp:64-73):
// max over active nodes of -sum_J alpha_IJ, accumulated in FP64.
template<int DIM>
__global__ void __launch_bounds__(kNT) k_diag_max_f64(Lattice L, const int * __restrict__ blist,
                                                      const int * __restrict__ bcount,
                                                      const unsigned char * __restrict__ bflag, NodeArrays N,
                                                      StencilD S, unsigned long long * __restrict__ out_bits) {
    using G = BrickGeom<DIM>;
    __shared__ float tile[G::TILE];
    const int nb = *bcount;
    double m     = -1e300;
    for (int bi = blockIdx.x; bi < nb; bi += gridDim.x) {
        const int b   = blist[bi];
        const int3 bc = brick_coords(L, b);
        __syncthreads();
        load_tile<DIM>(L, bflag, bc, tile, [&](long long s) { return N.V[s]; });
        __syncthreads();
        for (int l = threadIdx.x; l < G::BN; l += kNT) {
            const long long s = (long long) b * G::BN + l;
            if (N.flag[s]) m = fmax(m, -stencil_apply_d<DIM>(tile, tile_center<DIM>(l), S));
        }
    }
    // positive doubles order like their bit patterns; the diagonal is >= 0
    if (m >= 0) atomicMax(out_bits, (unsigned long long) __double_as_longlong(m));
}

// ---------------------------------------------------------------------------
// Warm start of the CG solution vector x (in place; x keeps the previous
// step's pressure in the same lattice slots).
//   prefix: reference behaviour, p0[I] = p_prev[I] for I < min(Nv_prev, Nv)
//           (ParticlesBasedData::resize keeps the stale prefix,
//           Cores/Structures/ParticlesBasedData.h:25-29, VirtualParticle.cpp:95)
//   node:   previous pressure of the same node, 0 if it was inactive
//   zero:   0
//   given:  caller-supplied values in brick layout
//   extrap: extrapolation in time of the same node's pressure.  With p1, p2,
//           p3 the node's pressure one, two, three steps back (x, xm1, xm2 on
//           entry; a value counts where the node was active at that step and
//           `history` covers it), p0 = 3 p1 - 3 p2 + p3 (quadratic) with three
//           steps, 2 p1 - p2 with two, p1 with one, else 0.  The history shifts
//           (xm1 = p1, xm2 = p2, both 0 where inactive) and, when d2p is
//           allocated, d2p = p1 - 2 p2 + p3 (0 without three steps).  Every slot of an active brick is
//           written; a slot's history is read only when the node was active
//           at every step it spans, which also means its brick was visited
//           (and its history shifted) at each of those steps.
// ---------------------------------------------------------------------------
template<int DIM>
__global__ void __launch_bounds__(kNT) k_warm_start(Lattice L, const int * __restrict__ blist,
                                                    const int * __restrict__ bcount, const int * __restrict__ seg_off,
                                                    BrickArrays B, NodeArrays N, int mode, int history,
                                                    const float * __restrict__ pcomp,
                                                    const int * __restrict__ nv_prev, const float * __restrict__ given) {
    using G      = BrickGeom<DIM>;
    const int nb = *bcount;
    const int np = nv_prev ? *nv_prev : 0;
    for (int bi = blockIdx.x; bi < nb; bi += gridDim.x) {
        const int b   = blist[bi];
        const int3 bc = brick_coords(L, b);
        for (int l = threadIdx.x; l < G::BN; l += kNT) {
            const long long s = (long long) b * G::BN + l;
            float v           = 0.f;
            if (N.flag[s]) {
                if (mode == kWarmPrefix) {
                    const int lx = l % G::BX, ly = (l / G::BX) % G::BY, lz = l / (G::BX * G::BY);
                    const long long I = compact_index<DIM>(L, seg_off, N.flag, b, bc.x, bc.x * G::BX + lx,
                                                           bc.y * G::BY + ly, bc.z * G::BZ + lz, l);
                    v = I < np ? pcomp[I] : 0.f;
                } else if (mode == kWarmNode) {
                    v = (B.flag_prev[b] && N.flag_prev[s]) ? N.x[s] : 0.f;
                } else if (mode == kWarmGiven) {
                    v = given[s];
                }
            }
            N.x[s] = v;
        }
    }
}

// History mode (extrap above) as a 16-byte streaming pass over the slots of the
// active bricks.
template<int DIM>
__global__ void __launch_bounds__(kNT) k_warm_history(const int * __restrict__ blist, const int * __restrict__ bcount,
                                                      BrickArrays B, NodeArrays N, int history) {
    pdl_wait_and_release();
    using G = BrickGeom<DIM>;
    constexpr int Q = G::BN / 4;
    const long long total = (long long) (*bcount) * Q;
    for (long long e = blockIdx.x * (long long) kNT + threadIdx.x; e < total; e += (long long) gridDim.x * kNT) {
        const int b       = blist[e / Q];
        const long long s = (long long) b * G::BN + 4 * (e % Q);
        const bool b1 = B.flag_prev[b] != 0, b2 = history >= 1 && B.flag_m2[b], b3 = history >= 2 && B.flag_m3[b];
        const uchar4 f = *reinterpret_cast<const uchar4 *>(N.flag + s);
        const uchar4 f1 = *reinterpret_cast<const uchar4 *>(N.flag_prev + s);
        const uchar4 f2 = *reinterpret_cast<const uchar4 *>(N.flag_m2 + s);
        const uchar4 f3 = *reinterpret_cast<const uchar4 *>(N.flag_m3 + s);
        const float4 x = *reinterpret_cast<const float4 *>(N.x + s), x1 = *reinterpret_cast<const float4 *>(N.xm1 + s),
                     x2 = *reinterpret_cast<const float4 *>(N.xm2 + s);
        float v[4], p1[4], p2[4], d2[4];
        const unsigned char fa[4] = {f.x, f.y, f.z, f.w}, fb[4] = {f1.x, f1.y, f1.z, f1.w},
                            fc[4] = {f2.x, f2.y, f2.z, f2.w}, fd[4] = {f3.x, f3.y, f3.z, f3.w};
        const float xa[4] = {x.x, x.y, x.z, x.w}, xb[4] = {x1.x, x1.y, x1.z, x1.w}, xc[4] = {x2.x, x2.y, x2.z, x2.w};
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const bool a1 = b1 && fb[k], a2 = a1 && b2 && fc[k], a3 = a2 && b3 && fd[k];
            p1[k] = a1 ? xa[k] : 0.f;
            p2[k] = a2 ? xb[k] : 0.f;
            const float p3 = a3 ? xc[k] : 0.f;
            const float d1 = a2 ? p1[k] - p2[k] : 0.f;
            d2[k] = a3 ? (p1[k] - 2.f * p2[k]) + p3 : 0.f;
            v[k]  = fa[k] ? (p1[k] + d1) + d2[k] : 0.f;
        }
        *reinterpret_cast<float4 *>(N.x + s)   = make_float4(v[0], v[1], v[2], v[3]);
        *reinterpret_cast<float4 *>(N.xm1 + s) = make_float4(p1[0], p1[1], p1[2], p1[3]);
        *reinterpret_cast<float4 *>(N.xm2 + s) = make_float4(p2[0], p2[1], p2[2], p2[3]);
        if (N.d2p) *reinterpret_cast<float4 *>(N.d2p + s) = make_float4(d2[0], d2[1], d2[2], d2[3]);
    }
}

// Export in reference order (x-fastest active nodes): node id, rho_I, V_I,
// vbar_I, D_I, alpha_hat_I, p_I; pcomp receives p in compact order (the next
// step's prefix warm start).
template<int DIM>
__global__ void __launch_bounds__(kNT) k_compact_export(Lattice L, const int * __restrict__ blist,
                                                        const int * __restrict__ bcount, const int * __restrict__ seg_off,
                                                        NodeArrays N, float * __restrict__ pcomp,
                                                        long long * __restrict__ node_id, double * __restrict__ rho,
                                                        double * __restrict__ vol, double * __restrict__ vbar,
                                                        double * __restrict__ div, double * __restrict__ ahat,
                                                        double * __restrict__ p, unsigned short * __restrict__ nreal_out) {
    using G      = BrickGeom<DIM>;
    const int nb = *bcount;
    for (int bi = blockIdx.x; bi < nb; bi += gridDim.x) {
        const int b   = blist[bi];
        const int3 bc = brick_coords(L, b);
        for (int l = threadIdx.x; l < G::BN; l += kNT) {
            const long long s = (long long) b * G::BN + l;
            if (!N.flag[s]) continue;
            const int lx = l % G::BX, ly = (l / G::BX) % G::BY, lz = l / (G::BX * G::BY);
            const int x = bc.x * G::BX + lx, y = bc.y * G::BY + ly, z = bc.z * G::BZ + lz;
            const long long I = compact_index<DIM>(L, seg_off, N.flag, b, bc.x, x, y, z, l);
            if (pcomp) pcomp[I] = N.x[s];
            if (node_id) node_id[I] = (long long) x + (long long) L.nx * (y + (long long) L.ny * z);
            if (rho) rho[I] = N.rho[s];
            if (vol) vol[I] = N.V[s];
            if (div) div[I] = N.D[s];
            if (ahat) ahat[I] = N.ahat[s];
            if (p) p[I] = N.x[s];
            if (nreal_out && N.nreal) nreal_out[I] = N.nreal[s];
            if (vbar && N.vbar) {
                const float4 v = N.vbar[s];
                vbar[I * DIM]     = v.x;
                vbar[I * DIM + 1] = v.y;
                if (DIM == 3) vbar[I * DIM + 2] = v.z;
            }
        }
    }
}

// Compact-order FP64 vector -> brick layout float (0 on inactive nodes).
template<int DIM>
__global__ void __launch_bounds__(kNT) k_compact_import(Lattice L, const int * __restrict__ blist,
                                                        const int * __restrict__ bcount, const int * __restrict__ seg_off,
                                                        NodeArrays N, const double * __restrict__ in,
                                                        float * __restrict__ out) {
    using G      = BrickGeom<DIM>;
    const int nb = *bcount;
    for (int bi = blockIdx.x; bi < nb; bi += gridDim.x) {
        const int b   = blist[bi];
        const int3 bc = brick_coords(L, b);
        for (int l = threadIdx.x; l < G::BN; l += kNT) {
            const long long s = (long long) b * G::BN + l;
            float v           = 0.f;
            if (N.flag[s]) {
                const int lx = l % G::BX, ly = (l / G::BX) % G::BY, lz = l / (G::BX * G::BY);
                const long long I = compact_index<DIM>(L, seg_off, N.flag, b, bc.x, bc.x * G::BX + lx,
                                                       bc.y * G::BY + ly, bc.z * G::BZ + lz, l);
                v = float(in[I]);
            }
            out[s] = v;
        }
    }
}

template<int DIM>
__global__ void __launch_bounds__(kNT) k_zero_active(const int * __restrict__ blist, const int * __restrict__ bcount,
                                                     float * __restrict__ a) {
    using G      = BrickGeom<DIM>;
    const int nb = *bcount;
    for (int bi = blockIdx.x; bi < nb; bi += gridDim.x) {
        const long long base = (long long) blist[bi] * G::BN;
        for (int l = threadIdx.x; l < G::BN; l += kNT) a[base + l] = 0.f;
    }
}

// ---------------------------------------------------------------------------
// Pressure-gradient update (VirtualParticle::applyPressureGradient,
// Cores/Structures/VirtualParticle.cpp:111-134):
//   v_i += sum_{J in N_H(i)} V_J p_J gradW_H(x_i - x_J)
//          - sum_{b in N_h(i)} V_b min(n_b.(v_i - v_b), 0) n_b W_h(x_i - x_b)
// One CTA per brick holding particles: u = V p over the brick + 4-node halo is
// staged in shared memory, distances are taken in lattice units (H = 4).
// ---------------------------------------------------------------------------

// sum_J u_J gradW_H(d) for lattice offsets d (in node units) with |d| < 4:
// gradientKernel = -W'_H(r) d / r (SmoothedParticles.h:96-98).
// Zero for r2 >= 16 (outside the support); finite at r2 = 0 where it multiplies
// a zero offset.
__device__ __forceinline__ float grad_scale(float r2, float c1H) {
    // -W'(r) / r_u with W' = c1 q (3q - 2) (q < 1/2) or -c1 (1 - q)^2 (q < 1), q = r_u / 4:
    //   r_u < 2:       c1 (1/2 - 3 r_u / 16)
    //   2 <= r_u < 4:  c1 (1 / r_u - 1/2 + r_u / 16)
    const float rinv = rsqrt_n(fmaxf(r2, 1e-20f));
    const float r    = r2 * rinv;
    const float gin  = fmaf(-0.1875f, r, 0.5f);
    const float gout = rinv + fmaf(0.0625f, r, -0.5f);
    return c1H * (r2 < 4.f ? gin : (r2 < 16.f ? gout : 0.f));
}

// Two nodes of a row at x offsets dx (packed FP32x2 arithmetic): returns
// w = u (a^2 - 4 b^2) / r with a = 1 - r/4, b = max(a - 1/2, 0) and r clamped
// to 4, i.e. the grad_scale factor above without c1H (r < 2: 1/2 - 3r/16;
// 2 <= r < 4: 1/r - 1/2 + r/16; 0 beyond), and adds w dx to sx.
// e = dyz2 + 1e-30 keeps r2 > 0 (a node at the particle adds 0).
__device__ __forceinline__ float2 grad_w2(float2 dx, float e, float2 u, float2 & sx) {
    float2 r2       = __ffma2_rn(dx, dx, make_float2(e, e));
    r2              = make_float2(fminf(r2.x, 16.f), fminf(r2.y, 16.f));
    const float2 ri = make_float2(rsqrt_n(r2.x), rsqrt_n(r2.y));
    const float2 r  = __fmul2_rn(r2, ri);
    const float2 a  = __ffma2_rn(r, make_float2(-0.25f, -0.25f), make_float2(1.f, 1.f));
    float2 b        = __fadd2_rn(a, make_float2(-0.5f, -0.5f));
    b               = make_float2(fmaxf(b.x, 0.f), fmaxf(b.y, 0.f));
    float2 g        = __fmul2_rn(a, a);
    g               = __ffma2_rn(__fmul2_rn(b, b), make_float2(-4.f, -4.f), g);
    const float2 w  = __fmul2_rn(__fmul2_rn(g, ri), u);
    sx              = __ffma2_rn(w, dx, sx);
    return w;
}

// One row of the 8-node x-window (node k at dx = fx - k, fx in [3, 4); dxp
// holds the pairs (2,3) (4,5) (1,6) (0,7)): sx += sum w dx, returns the pair
// sums of w.  Nodes 0 and 7 have |dx| >= 3 and lie outside H when dyz2 >= 7;
// nodes 1 and 6 have |dx| >= 2 and lie outside when dyz2 >= 12.
__device__ __forceinline__ float2 gradient_row(const float * trow, const float2 (&dxp)[4], float dyz2, float2 & sx) {
    const float e = dyz2 + 1e-30f;
    float2 sg     = grad_w2(dxp[0], e, make_float2(trow[2], trow[3]), sx);
    sg            = __fadd2_rn(sg, grad_w2(dxp[1], e, make_float2(trow[4], trow[5]), sx));
    if (dyz2 < 12.f) {
        sg = __fadd2_rn(sg, grad_w2(dxp[2], e, make_float2(trow[1], trow[6]), sx));
        if (dyz2 < 7.f) sg = __fadd2_rn(sg, grad_w2(dxp[3], e, make_float2(trow[0], trow[7]), sx));
    }
    return sg;
}

// Global-memory path for particles outside the staged tile (clamped in from
// outside the node lattice).
template<int DIM>
__device__ float3 gradient_virtual_global(const Lattice & L, const Phys & P, const unsigned char * __restrict__ bflag,
                                          const NodeArrays & N, float4 q) {
    using G  = BrickGeom<DIM>;
    float3 f = make_float3(0.f, 0.f, 0.f);
    const float ux = (q.x - L.ox) * L.inv_dx, uy = (q.y - L.oy) * L.inv_dx, uz = DIM == 3 ? (q.z - L.oz) * L.inv_dx : 0.f;
    const int y0 = max(__float2int_ru(uy - 4.f), 0), y1 = min(__float2int_rd(uy + 4.f), L.ny - 1);
    int z0 = 0, z1 = 0;
    if (DIM == 3) z0 = max(__float2int_ru(uz - 4.f), 0), z1 = min(__float2int_rd(uz + 4.f), L.nz - 1);
    for (int kz = z0; kz <= z1; kz++) {
        const float dz = DIM == 3 ? uz - kz : 0.f;
        for (int ky = y0; ky <= y1; ky++) {
            const float dy  = uy - ky;
            const float rem = 16.f - dy * dy - dz * dz;
            if (rem <= 0.f) continue;
            const float rn = sqrtf(rem);
            const int x0 = max(__float2int_ru(ux - rn), 0), x1 = min(__float2int_rd(ux + rn), L.nx - 1);
            for (int kx = x0; kx <= x1; kx++) {
                const int brick = kx / G::BX + L.bnx * (ky / G::BY + L.bny * (DIM == 3 ? kz / G::BZ : 0));
                if (!bflag[brick]) continue;
                const long long s = node_slot<DIM>(L, kx, ky, kz);
                const float u     = N.V[s] * N.x[s];
                const float dx    = ux - kx;
                const float r2    = dx * dx + dy * dy + dz * dz;
                if (u == 0.f || r2 >= 16.f || r2 <= 0.f) continue;
                const float g = grad_scale(r2, P.c1H) * u;
                f.x += g * dx;
                f.y += g * dy;
                f.z += g * dz;
            }
        }
    }
    return f;
}

constexpr int kGradNT = 256;  // threads per block of the pressure gradient (one particle brick per block)

template<int DIM>
__global__ void __launch_bounds__(kGradNT) k_pressure_gradient(Lattice L, Phys P, const unsigned char * __restrict__ bflag,
                                                           NodeArrays N, const int * __restrict__ plist,
                                                           const int * __restrict__ pcount,
                                                           const unsigned char * __restrict__ bnear,
                                                           const float4 * __restrict__ pos, float4 * __restrict__ vel,
                                                           const int * __restrict__ cellStart,
                                                           const float4 * __restrict__ bpos,
                                                           const float4 * __restrict__ bvel,
                                                           const float4 * __restrict__ bnrm,
                                                           const int * __restrict__ bcellStart,
                                                           const unsigned char * __restrict__ bcell, int * queue) {
    pdl_wait_and_release();
    using G = BrickGeom<DIM>;
    // Row pitch 24 in 3D: a warp's particles span about four consecutive cell
    // rows of one z-plane, whose 8-node windows then fall in disjoint banks
    // (24 dy mod 32 = 0, 24, 16, 8).
    constexpr int PX = DIM == 3 ? 24 : G::PX;
    __shared__ __align__(16) float tile[PX * G::TY * G::TZ];
    constexpr int ROWS = G::BY * G::BZ;  // cell rows of a brick
    __shared__ int rinc[ROWS], rbeg[ROWS];
    __shared__ int slot;
    const int nb = *pcount;
    const int t  = threadIdx.x;
    for (int bi = queue_take(queue, &slot); bi < nb; bi = queue_take(queue, &slot)) {
        const int b   = plist[bi];
        const int3 bc = brick_coords(L, b);
        const int x0 = bc.x * G::BX, x1 = min(x0 + G::BX, L.nx);
        load_tile4<DIM, kGradNT, PX>(L, bflag, bc, tile, [&](long long s) {
            const float4 v = *reinterpret_cast<const float4 *>(N.V + s), x = *reinterpret_cast<const float4 *>(N.x + s);
            return make_float4(v.x * x.x, v.y * x.y, v.z * x.z, v.w * x.w);
        });
        // particles of the brick: the cell rows' sorted ranges, enumerated
        // row after row (inclusive scan of the row counts in rinc)
        if (t < 32 * ((ROWS + 31) / 32)) {
            int cnt = 0, jb = 0;
            if (t < ROWS) {
                const int y = bc.y * G::BY + t % G::BY, z = DIM == 3 ? bc.z * G::BZ + t / G::BY : 0;
                if (y < L.ny && (DIM == 2 || z < L.nz)) {
                    const long long rbase = (long long) L.nx * (y + (long long) L.ny * z);
                    jb  = cellStart[rbase + x0];
                    cnt = cellStart[rbase + x1] - jb;
                }
            }
            int inc = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, inc, o);
                if ((t & 31) >= o) inc += v;
            }
            if (t < ROWS) {
                rinc[t] = inc;
                rbeg[t] = jb - (inc - cnt);
            }
        }
        __syncthreads();
        if (ROWS > 32 && t >= 32 && t < ROWS) {
            const int w0 = rinc[31];
            rinc[t] += w0;
            rbeg[t] -= w0;
        }
        __syncthreads();
        const int total  = rinc[ROWS - 1];
        const bool walls = bnear[b] != 0;
        // tile origin (node of tile index 0) of the FP64 lattice as float-float
        // pairs: a particle's offset from it, (q - hi) - lo, is exact to a few ulp
        // (the tile spans 16 nodes), where (q - origin) / dx - index would carry
        // the FP32 rounding of q - origin (~1e-7 at |q| ~ 2)
        const double tod_x = L.ox_d + (x0 - G::HALO) * L.dx_d, tod_y = L.oy_d + (bc.y * G::BY - G::HALO) * L.dx_d;
        const double tod_z = DIM == 3 ? L.oz_d + (bc.z * G::BZ - G::HALO) * L.dx_d : 0.0;
        const float tox = float(tod_x), toy = float(tod_y), toz = float(tod_z);
        const float tlx = float(tod_x - double(tox)), tly = float(tod_y - double(toy)), tlz = float(tod_z - double(toz));
        for (int p = t; p < total; p += kGradNT) {
            int lo = 0, hi = ROWS - 1;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (rinc[mid] > p) hi = mid;
                else lo = mid + 1;
            }
            const int j     = rbeg[lo] + p;
            const float4 q  = pos[j];
            const float4 vi = vel[j];
            const float ux = ((q.x - tox) - tlx) * L.inv_dx, uy = ((q.y - toy) - tly) * L.inv_dx;
            const float uz = DIM == 3 ? ((q.z - toz) - tlz) * L.inv_dx : 0.f;
            float3 f = make_float3(0.f, 0.f, 0.f);
            const bool inside = ux >= 3.f && ux < float(G::TX) - 4.f && uy >= 3.f && uy < float(G::TY) - 4.f &&
                                (DIM == 2 || (uz >= 3.f && uz < float(G::TZ) - 4.f));
            if (inside) {
                // nodes within H of the particle lie in the 8^DIM window
                // floor(u) - 3 .. floor(u) + 4 (offset -4 is excluded: r2 < 16)
                const int cx = int(ux), cy = int(uy), cz = DIM == 3 ? int(uz) : 0;
                const float fx = ux - float(cx - 3);
                const float2 dxp[4] = {make_float2(fx - 2.f, fx - 3.f), make_float2(fx - 4.f, fx - 5.f),
                                       make_float2(fx - 1.f, fx - 6.f), make_float2(fx, fx - 7.f)};
                float2 sx = make_float2(0.f, 0.f);
                float fy = 0.f, fz = 0.f;
                for (int oz = 0; oz < (DIM == 3 ? 8 : 1); oz++) {
                    const int kz    = DIM == 3 ? cz - 3 + oz : 0;
                    const float dz  = DIM == 3 ? uz - float(kz) : 0.f;
                    const float dz2 = dz * dz;
#pragma unroll 2
                    for (int oy = 0; oy < 8; oy++) {
                        const int ky     = cy - 3 + oy;
                        const float dy   = uy - float(ky);
                        const float dyz2 = fmaf(dy, dy, dz2);
                        if (dyz2 >= 16.f) continue;
                        const float * trow = tile + PX * (ky + G::TY * kz) + (cx - 3);
                        const float2 sg = gradient_row(trow, dxp, dyz2, sx);
                        const float s   = sg.x + sg.y;
                        fy = fmaf(dy, s, fy);
                        fz = fmaf(dz, s, fz);
                    }
                }
                f = make_float3(P.c1H * (sx.x + sx.y), P.c1H * fy, P.c1H * fz);
            } else {
                f = gradient_virtual_global<DIM>(L, P, bflag, N, q);
            }
            // the wall sum only for particles whose cell is within reach of the boundary
            if (walls && bcell[cell_linear(L, cell_of<DIM>(L, q.x, q.y, q.z))]) {
                const float3 w = wall_term<DIM>(L, P, bcellStart, bpos, bvel, bnrm, q, vi);
                f.x += w.x;
                f.y += w.y;
                f.z += w.z;
            }
            float4 o = vi;
            o.x += f.x;
            o.y += f.y;
            if (DIM == 3) o.z += f.z;
            vel[j] = o;
        }
    }
    queue_finish(queue);
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
template<int DIM>
void launch_pressure_gradient(const Lattice & L, const Phys & P, const BrickArrays & B, const NodeArrays & N,
                              const int * plist, const int * pcount, const unsigned char * bnear, const float4 * pos,
                              float4 * vel, const int * cellStart, const float4 * bpos, const float4 * bvel,
                              const float4 * bnrm, const int * bcellStart, const unsigned char * bcell, int grid,
                              int * queue, cudaStream_t st) {
    launch_pdl(k_pressure_gradient<DIM>, grid, kGradNT, 0, st, L, P, B.flag, N, plist, pcount, bnear, pos, vel, cellStart, bpos,
                                                   bvel, bnrm, bcellStart, bcell, queue);
}
template<int DIM> int pressure_gradient_blocks_per_sm() {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_pressure_gradient<DIM>, kGradNT, 0) != cudaSuccess) n = 1;
    return n > 0 ? n : 1;
}
template<int DIM> int node_gather_blocks_per_sm() {
    auto blocks = [](auto kernel) {
        int k = 0;
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k, kernel, 128, 0) == cudaSuccess ? k : 1;
    };
    const int n = std::min(std::min(blocks(k_node_gather<DIM, true, true>), blocks(k_node_gather<DIM, true, false>)),
                           std::min(blocks(k_node_gather<DIM, false, true>), blocks(k_node_gather<DIM, false, false>)));
    return n > 0 ? n : 1;
}
void launch_brick_list(const unsigned char * bflag, int nbricks, int * list, int * count, cudaStream_t st) {
    launch_pdl(k_brick_list, 1, 1024, 0, st, bflag, nbricks, list, count);
}

template<int DIM>
void launch_node_gather(const Lattice & L, const Phys & P, const BrickArrays & B, const NodeArrays & N,
                        const float4 * pos, const float4 * vel, const int * cellStart, const float4 * bpos,
                        const float4 * bvel, const int * bcellStart, const unsigned char * bnear,
                        const unsigned char * bcell, int grid, int * queue, cudaStream_t st) {
    // H >= 2h: particles within h only reach the inner branch of W_H; the
    // real-neighbour counts only where N.nreal is given
    const bool fast = double(P.H) >= 2.0 * double(P.h) * (1.0 - 1e-6), feat = N.nreal != nullptr;
    auto go = [&](auto kernel) {
        launch_pdl(kernel, grid, 128, 0, st, L, P, B.list, B.count, N, pos, vel, cellStart, bpos, bvel, bcellStart, bnear,
                   bcell, queue);
    };
    if (fast) feat ? go(k_node_gather<DIM, true, true>) : go(k_node_gather<DIM, true, false>);
    else feat ? go(k_node_gather<DIM, false, true>) : go(k_node_gather<DIM, false, false>);
}

template<int DIM>
void launch_segments(const Lattice & L, const BrickArrays & B, const NodeArrays & N, int * tiles, int grid,
                     cudaStream_t st) {
    cudaMemsetAsync(B.seg, 0, sizeof(int) * B.nseg, st);
    launch_pdl(k_segment_count<DIM>, grid, kNT, 0, st, L, B.list, B.count, N.flag, B.seg);
    launch_scan(B.seg, B.nseg, B.seg_off, tiles, st);
}


template<int DIM>
void launch_diag_max_f64(const Lattice & L, const BrickArrays & B, const NodeArrays & N, const StencilD & S,
                         unsigned long long * out_bits, int grid, cudaStream_t st) {
    cudaMemsetAsync(out_bits, 0, sizeof(unsigned long long), st);
    k_diag_max_f64<DIM><<<grid, kNT, 0, st>>>(L, B.list, B.count, B.flag, N, S, out_bits);
}

template<int DIM>
void launch_warm_start(const Lattice & L, const BrickArrays & B, const NodeArrays & N, int mode, const float * pcomp,
                       const int * nv_prev, const float * given, int grid, cudaStream_t st, int history) {
    if (mode == kWarmExtrap) {
        // streaming grid: the slots of the active bricks, 4 per thread
        const long long q = (long long) L.nbricks * (BrickGeom<DIM>::BN / 4);
        launch_pdl(k_warm_history<DIM>, int(std::min<long long>((q + kNT - 1) / kNT, 152LL * 8)), kNT, 0, st, B.list, B.count, B,
                                                                                                    N, history);
        return;
    }
    k_warm_start<DIM><<<grid, kNT, 0, st>>>(L, B.list, B.count, B.seg_off, B, N, mode, history, pcomp, nv_prev,
                                            given);
}

template<int DIM>
void launch_compact_export(const Lattice & L, const BrickArrays & B, const NodeArrays & N, float * pcomp,
                           long long * node_id, double * rho, double * vol, double * vbar, double * div,
                           double * ahat, double * p, unsigned short * nreal_out, int grid, cudaStream_t st) {
    k_compact_export<DIM><<<grid, kNT, 0, st>>>(L, B.list, B.count, B.seg_off, N, pcomp, node_id, rho, vol, vbar, div,
                                                ahat, p, nreal_out);
}

template<int DIM>
void launch_compact_import(const Lattice & L, const BrickArrays & B, const NodeArrays & N, const double * in,
                           float * out, int grid, cudaStream_t st) {
    k_compact_import<DIM><<<grid, kNT, 0, st>>>(L, B.list, B.count, B.seg_off, N, in, out);
}

template<int DIM>
void launch_zero_active(const Lattice & L, const BrickArrays & B, float * a, int grid, cudaStream_t st) {
    (void) L;
    k_zero_active<DIM><<<grid, kNT, 0, st>>>(B.list, B.count, a);
}






#define SWC_INST(D)                                                                                                    \
    template void launch_node_gather<D>(const Lattice &, const Phys &, const BrickArrays &, const NodeArrays &,        \
                                        const float4 *, const float4 *, const int *, const float4 *, const float4 *,   \
                                        const int *, const unsigned char *, const unsigned char *, int, int *,         \
                                        cudaStream_t);                                                                 \
    template void launch_pressure_gradient<D>(const Lattice &, const Phys &, const BrickArrays &, const NodeArrays &,  \
                                              const int *, const int *, const unsigned char *, const float4 *,         \
                                              float4 *, const int *, const float4 *, const float4 *, const float4 *,   \
                                              const int *, const unsigned char *, int, int *, cudaStream_t);           \
    template int pressure_gradient_blocks_per_sm<D>();                                                                 \
    template int node_gather_blocks_per_sm<D>();                                                                       \
    template void launch_segments<D>(const Lattice &, const BrickArrays &, const NodeArrays &, int *, int,             \
                                     cudaStream_t);                                                                    \
    template void launch_diag_max_f64<D>(const Lattice &, const BrickArrays &, const NodeArrays &, const StencilD &,   \
                                         unsigned long long *, int, cudaStream_t);                                     \
    template void launch_warm_start<D>(const Lattice &, const BrickArrays &, const NodeArrays &, int, const float *,   \
                                       const int *, const float *, int, cudaStream_t, int);                            \
    template void launch_compact_export<D>(const Lattice &, const BrickArrays &, const NodeArrays &, float *,          \
                                           long long *, double *, double *, double *, double *, double *, double *,    \
                                           unsigned short *, int, cudaStream_t);                                       \
    template void launch_compact_import<D>(const Lattice &, const BrickArrays &, const NodeArrays &, const double *,   \
                                           float *, int, cudaStream_t);                                                \
    template void launch_zero_active<D>(const Lattice &, const BrickArrays &, float *, int, cudaStream_t);
SWC_INST(2)
SWC_INST(3)
#undef SWC_INST

}  // namespace swc
