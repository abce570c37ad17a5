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

// Contributions of one particle / boundary particle at squared distance r2 and
// offset (dx, dy, dz) = x_I - x_j to the 11 sums of a node.
struct NodeSums {
    float wsum, rhoI, VI, ux, uy, uz, bw, dvg, gx, gy, gz;
    int   cnt;
};

template<bool REAL>
__device__ __forceinline__ void add_pair(NodeSums & a, const Phys & P, float r2, float dx, float dy, float dz, float4 p,
                                         float4 u) {
    const float rinv = rsqrtf(fmaxf(r2, 1e-30f));
    const float r    = r2 * rinv;
    const float q    = r * P.inv_h;
    const float t    = 1.f - q;
    const bool inner = q < 0.5f;
    const float w    = inner ? P.c0h * (6.f * q * q * (q - 1.f) + 1.f) : P.c0h * 2.f * t * t * t;
    // -W'_h(r)/r: -c1 (3q - 2)/h inside, c1 (1 - q)^2 / r outside (zero offset at r = 0)
    const float gsc = inner ? -P.c1h * P.inv_h * (3.f * q - 2.f) : P.c1h * t * t * rinv;
    if (REAL) {
        a.wsum += w;
        a.rhoI += kW(r, P.inv_H, P.c0H);
        a.VI += p.w * p.w * w;
        a.cnt++;
    }
    const float mw = u.w * w;
    a.ux += mw * u.x;
    a.uy += mw * u.y;
    a.uz += mw * u.z;
    a.bw += p.w * w;
    const float c  = gsc * p.w;
    const float cx = c * dx, cy = c * dy, cz = c * dz;
    a.dvg += u.x * cx + u.y * cy + u.z * cz;
    a.gx += cx;
    a.gy += cy;
    a.gz += cz;
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
// ---------------------------------------------------------------------------
template<int DIM>
__global__ void __launch_bounds__(128, 4) k_node_gather(Lattice L, Phys P, const int * __restrict__ blist,
                                                       const int * __restrict__ bcount, NodeArrays N,
                                                       const float4 * __restrict__ pos, const float4 * __restrict__ vel,
                                                       const int * __restrict__ cellStart,
                                                       const float4 * __restrict__ bpos,
                                                       const float4 * __restrict__ bvel,
                                                       const int * __restrict__ bcellStart,
                                                       const unsigned char * __restrict__ bnear) {
    using G          = BrickGeom<DIM>;
    constexpr int NX = 4;
    constexpr int XS = G::BX / NX;  // thread columns per brick row
    constexpr int TPB = G::BN / NX;
    const int nb = *bcount;
    for (int bi = blockIdx.x; bi < nb; bi += gridDim.x) {
        const int b     = blist[bi];
        const int3 bc   = brick_coords(L, b);
        const int npass = bnear[b] ? 2 : 1;  // boundary particles only near walls
        for (int l4 = threadIdx.x; l4 < TPB; l4 += blockDim.x) {
            const int lx0 = (l4 % XS) * NX, ly = (l4 / XS) % G::BY, lz = l4 / (XS * G::BY);
            const int x0 = bc.x * G::BX + lx0, y = bc.y * G::BY + ly, z = bc.z * G::BZ + lz;
            const long long s0 = (long long) b * G::BN + lx0 + G::BX * (ly + G::BY * lz);
            const bool row_in = y < L.ny && (DIM == 2 || z < L.nz);
            NodeSums a[NX];
#pragma unroll
            for (int n = 0; n < NX; n++) a[n] = NodeSums{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0};
            const float xn0 = L.ox + x0 * L.dx, yn = L.oy + y * L.dx, zn = DIM == 3 ? L.oz + z * L.dx : 0.f;
            const int cxa = max(x0 + P.cell_lo, 0), cxb = min(x0 + NX - 1 + P.cell_hi, L.nx - 1);
            const int cy0 = max(y + P.cell_lo, 0), cy1 = min(y + P.cell_hi, L.ny - 1);
            const int cz0 = DIM == 3 ? max(z + P.cell_lo, 0) : 0, cz1 = DIM == 3 ? min(z + P.cell_hi, L.nz - 1) : 0;
            if (row_in) {
#pragma unroll 1
                for (int pass = 0; pass < npass; pass++) {
                    const int * cs   = pass == 0 ? cellStart : bcellStart;
                    const float4 * X = pass == 0 ? pos : bpos;
                    const float4 * U = pass == 0 ? vel : bvel;
                    for (int cz = cz0; cz <= cz1; cz++)
                        for (int cy = cy0; cy <= cy1; cy++) {
                            const long long row = (long long) L.nx * (cy + (long long) L.ny * cz);
                            const int jb = cs[row + cxa], je = cs[row + cxb + 1];
                            for (int j = jb; j < je; j++) {
                                const float4 p  = X[j];
                                const float dy  = yn - p.y, dz = zn - p.z;
                                const float ryz = dy * dy + dz * dz;
                                if (ryz >= P.h2) continue;
                                float4 u;
                                bool have_u = false;
#pragma unroll
                                for (int n = 0; n < NX; n++) {
                                    const float dx = xn0 + n * L.dx - p.x;
                                    const float r2 = dx * dx + ryz;
                                    if (r2 >= P.h2) continue;
                                    if (!have_u) {
                                        u      = U[j];
                                        have_u = true;
                                    }
                                    if (pass == 0) add_pair<true>(a[n], P, r2, dx, dy, dz, p, u);
                                    else add_pair<false>(a[n], P, r2, dx, dy, dz, p, u);
                                }
                            }
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
                const NodeSums & A = a[n];
                bool active        = A.wsum > 1e-6f;
                if (fabsf(A.wsum - 1e-6f) <= 1e-9f) {
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
                const float den = A.bw + 1e-6f;
                const float vbx = A.ux / den, vby = A.uy / den, vbz = A.uz / den;
                const float rho = A.rhoI * P.mass;
                const float Dv  = A.dvg - (vbx * A.gx + vby * A.gy + vbz * A.gz) -
                                 P.kappa * fmaxf(rho - P.rho0, 0.f) / P.rho0;
                N.flag[s] = active ? 1 : 0;
                N.V[s]    = active ? A.VI : 0.f;
                N.D[s]    = active ? Dv : 0.f;
                N.rho[s]  = active ? rho : 0.f;
                if (N.nreal) N.nreal[s] = (unsigned short) min(A.cnt, 65535);
                if (N.vbar) N.vbar[s] = make_float4(vbx, vby, vbz, 0.f);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Reference-order (x-fastest over the whole node grid, Grid.cpp:231-244)
// compaction: per (row, brick column) segment counts, scanned.
// ---------------------------------------------------------------------------
template<int DIM>
__global__ void __launch_bounds__(kNT) k_segment_count(Lattice L, const int * __restrict__ blist,
                                                       const int * __restrict__ bcount,
                                                       const unsigned char * __restrict__ flag, int * __restrict__ seg) {
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
// ---------------------------------------------------------------------------
template<int DIM>
__global__ void __launch_bounds__(kNT) k_warm_start(Lattice L, const int * __restrict__ blist,
                                                    const int * __restrict__ bcount, const int * __restrict__ seg_off,
                                                    const unsigned char * __restrict__ bflag_prev, NodeArrays N,
                                                    int mode, const float * __restrict__ pcomp,
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
                    v = (bflag_prev[b] && N.flag_prev[s]) ? N.x[s] : 0.f;
                } else if (mode == kWarmGiven) {
                    v = given[s];
                }
            }
            N.x[s] = v;
        }
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
    const float rinv = rsqrtf(fmaxf(r2, 1e-20f));
    const float r    = r2 * rinv;
    const float gin  = fmaf(-0.1875f, r, 0.5f);
    const float gout = rinv + fmaf(0.0625f, r, -0.5f);
    return c1H * (r2 < 4.f ? gin : (r2 < 16.f ? gout : 0.f));
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

template<int DIM>
__global__ void __launch_bounds__(kNT) k_pressure_gradient(Lattice L, Phys P, const unsigned char * __restrict__ bflag,
                                                           NodeArrays N, const int * __restrict__ plist,
                                                           const int * __restrict__ pcount,
                                                           const unsigned char * __restrict__ bnear,
                                                           const float4 * __restrict__ pos, float4 * __restrict__ vel,
                                                           const int * __restrict__ cellStart,
                                                           const float4 * __restrict__ bpos,
                                                           const float4 * __restrict__ bvel,
                                                           const float4 * __restrict__ bnrm,
                                                           const int * __restrict__ bcellStart) {
    using G = BrickGeom<DIM>;
    __shared__ float tile[G::TILE];
    constexpr int ROWS = G::BY * G::BZ;        // cell rows of a brick
    constexpr int PER_ROW = kNT / ROWS;       // threads per row
    const int nb = *pcount;
    for (int bi = blockIdx.x; bi < nb; bi += gridDim.x) {
        const int b   = plist[bi];
        const int3 bc = brick_coords(L, b);
        __syncthreads();
        load_tile<DIM>(L, bflag, bc, tile, [&](long long s) { return N.V[s] * N.x[s]; });
        __syncthreads();
        const bool walls = bnear[b] != 0;
        const int row    = threadIdx.x % ROWS, sub = threadIdx.x / ROWS;
        const int ly = row % G::BY, lz = row / G::BY;
        const int y = bc.y * G::BY + ly, z = bc.z * G::BZ + lz;
        if (y >= L.ny || (DIM == 3 && z >= L.nz)) continue;
        const int x0 = bc.x * G::BX, x1 = min(x0 + G::BX, L.nx);
        const long long rbase = (long long) L.nx * (y + (long long) L.ny * z);
        const int jb = cellStart[rbase + x0], je = cellStart[rbase + x1];
        // tile origin (node coordinates of tile index 0)
        const float tox = float(x0 - G::HALO), toy = float(bc.y * G::BY - G::HALO);
        const float toz = DIM == 3 ? float(bc.z * G::BZ - G::HALO) : 0.f;
        for (int j = jb + sub; j < je; j += PER_ROW) {
            const float4 q  = pos[j];
            const float4 vi = vel[j];
            const float ux = (q.x - L.ox) * L.inv_dx - tox, uy = (q.y - L.oy) * L.inv_dx - toy;
            const float uz = DIM == 3 ? (q.z - L.oz) * L.inv_dx - toz : 0.f;
            float3 f = make_float3(0.f, 0.f, 0.f);
            const bool inside = ux > 3.f && ux < float(G::TX) - 4.f && uy > 3.f && uy < float(G::TY) - 4.f &&
                                (DIM == 2 || (uz > 3.f && uz < float(G::TZ) - 4.f));
            if (inside) {
                // nodes within H lie in the 8-node x-window floor(ux) - 3 .. floor(ux) + 4 of each row
                const int kz0 = DIM == 3 ? __float2int_ru(uz - 4.f) : 0, kz1 = DIM == 3 ? __float2int_rd(uz + 4.f) : 0;
                const int ky0 = __float2int_ru(uy - 4.f), ky1 = __float2int_rd(uy + 4.f);
                const int kxb  = __float2int_rd(ux) - 3;
                const float dx0 = ux - float(kxb);
                for (int kz = kz0; kz <= kz1; kz++) {
                    const float dz = DIM == 3 ? uz - kz : 0.f;
                    for (int ky = ky0; ky <= ky1; ky++) {
                        const float dy   = uy - ky;
                        const float dyz2 = fmaf(dy, dy, dz * dz);
                        if (dyz2 >= 16.f) continue;
                        const float * trow = tile + G::PX * (ky + G::TY * kz) + kxb;
                        float sx = 0.f, sg = 0.f;  // sum g dx and sum g over the row
#pragma unroll
                        for (int i = 0; i < 8; i++) {
                            const float dx = dx0 - float(i);
                            const float g  = grad_scale(fmaf(dx, dx, dyz2), P.c1H) * trow[i];
                            sx = fmaf(g, dx, sx);
                            sg += g;
                        }
                        f.x += sx;
                        f.y = fmaf(dy, sg, f.y);
                        f.z = fmaf(dz, sg, f.z);
                    }
                }
            } else {
                f = gradient_virtual_global<DIM>(L, P, bflag, N, q);
            }
            if (walls) {
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
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
template<int DIM>
void launch_pressure_gradient(const Lattice & L, const Phys & P, const BrickArrays & B, const NodeArrays & N,
                              const int * plist, const int * pcount, const unsigned char * bnear, const float4 * pos,
                              float4 * vel, const int * cellStart, const float4 * bpos, const float4 * bvel,
                              const float4 * bnrm, const int * bcellStart, int grid, cudaStream_t st) {
    k_pressure_gradient<DIM><<<grid, kNT, 0, st>>>(L, P, B.flag, N, plist, pcount, bnear, pos, vel, cellStart, bpos,
                                                   bvel, bnrm, bcellStart);
}
void launch_brick_list(const unsigned char * bflag, int nbricks, int * list, int * count, cudaStream_t st) {
    k_brick_list<<<1, 1024, 0, st>>>(bflag, nbricks, list, count);
}

template<int DIM>
void launch_node_gather(const Lattice & L, const Phys & P, const BrickArrays & B, const NodeArrays & N,
                        const float4 * pos, const float4 * vel, const int * cellStart, const float4 * bpos,
                        const float4 * bvel, const int * bcellStart, const unsigned char * bnear, int grid,
                        cudaStream_t st) {
    k_node_gather<DIM><<<grid * 2, 128, 0, st>>>(L, P, B.list, B.count, N, pos, vel, cellStart, bpos, bvel, bcellStart,
                                             bnear);
}

template<int DIM>
void launch_segments(const Lattice & L, const BrickArrays & B, const NodeArrays & N, int * tiles, int grid,
                     cudaStream_t st) {
    cudaMemsetAsync(B.seg, 0, sizeof(int) * B.nseg, st);
    k_segment_count<DIM><<<grid, kNT, 0, st>>>(L, B.list, B.count, N.flag, B.seg);
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
                       const int * nv_prev, const float * given, int grid, cudaStream_t st) {
    k_warm_start<DIM><<<grid, kNT, 0, st>>>(L, B.list, B.count, B.seg_off, B.flag_prev, N, mode, pcomp, nv_prev,
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
                                        const int *, const unsigned char *, int, cudaStream_t);                        \
    template void launch_pressure_gradient<D>(const Lattice &, const Phys &, const BrickArrays &, const NodeArrays &,  \
                                              const int *, const int *, const unsigned char *, const float4 *,         \
                                              float4 *, const int *, const float4 *, const float4 *, const float4 *,   \
                                              const int *, int, cudaStream_t);                                         \
    template void launch_segments<D>(const Lattice &, const BrickArrays &, const NodeArrays &, int *, int,             \
                                     cudaStream_t);                                                                    \
    template void launch_diag_max_f64<D>(const Lattice &, const BrickArrays &, const NodeArrays &, const StencilD &,   \
                                         unsigned long long *, int, cudaStream_t);                                     \
    template void launch_warm_start<D>(const Lattice &, const BrickArrays &, const NodeArrays &, int, const float *,   \
                                       const int *, const float *, int, cudaStream_t);                                 \
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
