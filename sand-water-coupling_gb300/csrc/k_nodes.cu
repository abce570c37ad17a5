// k_nodes.cu -- virtual-node (lattice) kernels of the dual-particle SPH
// projection: active-brick list, the fused virtual gather (weight, rho_I, V_I,
// vbar_I, D_I in one pass), reference-order compaction, the clamped diagonal
// alpha_hat, warm starts and the matrix-free CG (stencil SpMV fused with the
// search-direction update, and the x/r update), all with deterministic
// FP64 reductions.
#include "swc_kernels.h"

namespace swc {

constexpr int kNT = 256;  // threads per block of the brick kernels

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

// Brick coordinates of brick id b.
__device__ __forceinline__ int3 brick_coords(const Lattice & L, int b) {
    return make_int3(b % L.bnx, (b / L.bnx) % L.bny, b / (L.bnx * L.bny));
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
// ---------------------------------------------------------------------------
template<int DIM>
__global__ void __launch_bounds__(kNT) k_node_gather(Lattice L, Phys P, const int * __restrict__ blist,
                                                     const int * __restrict__ bcount, NodeArrays N,
                                                     const float4 * __restrict__ pos, const float4 * __restrict__ vel,
                                                     const int * __restrict__ cellStart,
                                                     const float4 * __restrict__ bpos,
                                                     const float4 * __restrict__ bvel,
                                                     const int * __restrict__ bcellStart) {
    using G      = BrickGeom<DIM>;
    const int nb = *bcount;
    for (int bi = blockIdx.x; bi < nb; bi += gridDim.x) {
        const int b    = blist[bi];
        const int3 bc  = brick_coords(L, b);
        for (int l = threadIdx.x; l < G::BN; l += kNT) {
            const int lx = l % G::BX, ly = (l / G::BX) % G::BY, lz = l / (G::BX * G::BY);
            const int x = bc.x * G::BX + lx, y = bc.y * G::BY + ly, z = bc.z * G::BZ + lz;
            const long long s = (long long) b * G::BN + l;
            if (x >= L.nx || y >= L.ny || (DIM == 3 && z >= L.nz)) {
                N.flag[s] = 0;
                N.V[s] = 0.f;
                N.D[s] = 0.f;
                N.rho[s] = 0.f;
                if (N.nreal) N.nreal[s] = 0;
                if (N.vbar) N.vbar[s] = make_float4(0.f, 0.f, 0.f, 0.f);
                continue;
            }
            const float xn = L.ox + x * L.dx, yn = L.oy + y * L.dx, zn = DIM == 3 ? L.oz + z * L.dx : 0.f;
            float wsum = 0.f, rhoI = 0.f, VI = 0.f, ux = 0.f, uy = 0.f, uz = 0.f, bw = 0.f, dvg = 0.f, gx = 0.f,
                  gy = 0.f, gz = 0.f;
            int cnt = 0;
            const int cx0 = max(x + P.cell_lo, 0), cx1 = min(x + P.cell_hi, L.nx - 1);
            const int cy0 = max(y + P.cell_lo, 0), cy1 = min(y + P.cell_hi, L.ny - 1);
            const int cz0 = DIM == 3 ? max(z + P.cell_lo, 0) : 0, cz1 = DIM == 3 ? min(z + P.cell_hi, L.nz - 1) : 0;
#pragma unroll 1
            for (int pass = 0; pass < 2; pass++) {
                const int * cs   = pass == 0 ? cellStart : bcellStart;
                const float4 * X = pass == 0 ? pos : bpos;
                const float4 * U = pass == 0 ? vel : bvel;
                for (int cz = cz0; cz <= cz1; cz++)
                    for (int cy = cy0; cy <= cy1; cy++) {
                        const long long row = (long long) L.nx * (cy + (long long) L.ny * cz);
                        const int jb = cs[row + cx0], je = cs[row + cx1 + 1];
                        for (int j = jb; j < je; j++) {
                            const float4 p = X[j];
                            const float dx = xn - p.x, dy = yn - p.y, dz = zn - p.z;
                            const float r2 = dx * dx + dy * dy + dz * dz;
                            if (r2 >= P.h2) continue;
                            const float4 u = U[j];
                            const float r  = sqrtf(r2);
                            const float w  = kW(r, P.inv_h, P.c0h);
                            if (pass == 0) {
                                wsum += w;
                                rhoI += kW(r, P.inv_H, P.c0H);
                                VI += p.w * p.w * w;
                                cnt++;
                            }
                            const float mw = u.w * w;
                            ux += mw * u.x;
                            uy += mw * u.y;
                            uz += mw * u.z;
                            bw += p.w * w;
                            if (r > 0.f) {
                                const float c  = -kdW(r, P.inv_h, P.c1h) / r * p.w;
                                const float cx = c * dx, cy_ = c * dy, cz_ = c * dz;
                                dvg += u.x * cx + u.y * cy_ + u.z * cz_;
                                gx += cx;
                                gy += cy_;
                                gz += cz_;
                            }
                        }
                    }
            }
            bool active = wsum > 1e-6f;
            if (fabsf(wsum - 1e-6f) <= 1e-9f) {
                // borderline: redo the weight in FP64 from the same float positions
                const double xd = L.ox_d + x * L.dx_d, yd = L.oy_d + y * L.dx_d, zd = DIM == 3 ? L.oz_d + z * L.dx_d : 0.0;
                double ws = 0;
                for (int cz = cz0; cz <= cz1; cz++)
                    for (int cy = cy0; cy <= cy1; cy++) {
                        const long long row = (long long) L.nx * (cy + (long long) L.ny * cz);
                        for (int j = cellStart[row + cx0]; j < cellStart[row + cx1 + 1]; j++) {
                            const float4 p = pos[j];
                            const double dx = xd - p.x, dy = yd - p.y, dz = DIM == 3 ? zd - p.z : 0.0;
                            const double r2 = dx * dx + dy * dy + dz * dz;
                            if (r2 < P.h_d * P.h_d) ws += kW_d(sqrt(r2), P.inv_h_d, P.c0h_d);
                        }
                    }
                active = ws > 1e-6;
            }
            const float den = bw + 1e-6f;
            const float vbx = ux / den, vby = uy / den, vbz = uz / den;
            const float rho = rhoI * P.mass;
            const float Dv  = dvg - (vbx * gx + vby * gy + vbz * gz) - P.kappa * fmaxf(rho - P.rho0, 0.f) / P.rho0;
            N.flag[s] = active ? 1 : 0;
            N.V[s]    = active ? VI : 0.f;
            N.D[s]    = active ? Dv : 0.f;
            N.rho[s]  = active ? rho : 0.f;
            if (N.nreal) N.nreal[s] = (unsigned short) min(cnt, 65535);
            if (N.vbar) N.vbar[s] = make_float4(vbx, vby, vbz, 0.f);
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

template<int DIM>
__device__ __forceinline__ long long compact_index(const Lattice & L, const int * __restrict__ seg_off,
                                                   const unsigned char * __restrict__ flag, int b, int bx, int x,
                                                   int y, int z, int l) {
    using G       = BrickGeom<DIM>;
    const int lx  = l % G::BX;
    long long I   = seg_off[((long long) z * L.ny + y) * L.bnx + bx];
    const unsigned char * f = flag + (long long) b * G::BN + (l - lx);
    for (int k = 0; k < lx; k++) I += f[k];
    return I;
}

// ---------------------------------------------------------------------------
// Halo tile loading and the radial stencil.
// ---------------------------------------------------------------------------
template<int DIM, class Get>
__device__ __forceinline__ void load_tile(const Lattice & L, const unsigned char * __restrict__ bflag, int3 bc,
                                          float * tile, Get get) {
    using G       = BrickGeom<DIM>;
    constexpr int NT = G::TX * G::TY * G::TZ;
    for (int t = threadIdx.x; t < NT; t += kNT) {
        const int tx = t % G::TX, ty = (t / G::TX) % G::TY, tz = t / (G::TX * G::TY);
        const int x = bc.x * G::BX + tx - G::HALO, y = bc.y * G::BY + ty - G::HALO;
        const int z = DIM == 3 ? bc.z * G::BZ + tz - G::HALO : 0;
        float v = 0.f;
        if (x >= 0 && x < L.nx && y >= 0 && y < L.ny && (DIM == 2 || (z >= 0 && z < L.nz))) {
            const int nbx = x / G::BX, nby = y / G::BY, nbz = DIM == 3 ? z / G::BZ : 0;
            const int nbk = nbx + L.bnx * (nby + L.bny * nbz);
            if (bflag[nbk])
                v = get((long long) nbk * G::BN + (x - nbx * G::BX) + G::BX * ((y - nby * G::BY) + G::BY * (z - nbz * G::BZ)));
        }
        tile[tx + G::PX * (ty + G::TY * tz)] = v;
    }
}

template<int DIM> __device__ __forceinline__ int tile_center(int l) {
    using G      = BrickGeom<DIM>;
    const int lx = l % G::BX, ly = (l / G::BX) % G::BY, lz = l / (G::BX * G::BY);
    return (lx + G::HALO) + G::PX * ((ly + G::HALO) + G::TY * (DIM == 3 ? lz + G::HALO : 0));
}

// sum over offsets 0 < |k|^2 < 16 of c(|k|^2) * tile[center + k]
template<int DIM> __device__ __forceinline__ float stencil_apply(const float * tile, int c, const Stencil & S) {
    using G   = BrickGeom<DIM>;
    float acc = 0.f;
    constexpr int ZR = DIM == 3 ? 3 : 0;
#pragma unroll
    for (int dz = -ZR; dz <= ZR; dz++)
#pragma unroll
        for (int dy = -3; dy <= 3; dy++)
#pragma unroll
            for (int dx = -3; dx <= 3; dx++) {
                const int r2 = dx * dx + dy * dy + dz * dz;
                if (r2 > 0 && r2 < 16) acc = fmaf(S.c[r2], tile[c + dx + G::PX * (dy + G::TY * dz)], acc);
            }
    return acc;
}
template<int DIM> __device__ __forceinline__ double stencil_apply_d(const float * tile, int c, const StencilD & S) {
    using G    = BrickGeom<DIM>;
    double acc = 0.0;
    constexpr int ZR = DIM == 3 ? 3 : 0;
#pragma unroll
    for (int dz = -ZR; dz <= ZR; dz++)
#pragma unroll
        for (int dy = -3; dy <= 3; dy++)
#pragma unroll
            for (int dx = -3; dx <= 3; dx++) {
                const int r2 = dx * dx + dy * dy + dz * dz;
                if (r2 > 0 && r2 < 16) acc += S.c[r2] * double(tile[c + dx + G::PX * (dy + G::TY * dz)]);
            }
    return acc;
}

// alpha_hat_I = max(-sum_J alpha_IJ, alpha0) with alpha_IJ = c(|k|^2) V_J
// (VirtualParticle::calculateCoef, VirtualParticle.cpp:149-169); inactive rows
// become identity rows (alpha_hat = 1, rhs 0, x 0) so the brick-dense CG equals
// CG on the active set.
template<int DIM>
__global__ void __launch_bounds__(kNT) k_ahat(Lattice L, Phys P, const int * __restrict__ blist,
                                              const int * __restrict__ bcount, const unsigned char * __restrict__ bflag,
                                              NodeArrays N, Stencil S) {
    using G = BrickGeom<DIM>;
    __shared__ float tile[G::TILE];
    const int nb = *bcount;
    for (int bi = blockIdx.x; bi < nb; bi += gridDim.x) {
        const int b   = blist[bi];
        const int3 bc = brick_coords(L, b);
        __syncthreads();
        load_tile<DIM>(L, bflag, bc, tile, [&](long long s) { return N.V[s]; });
        __syncthreads();
        for (int l = threadIdx.x; l < G::BN; l += kNT) {
            const long long s = (long long) b * G::BN + l;
            const float sum   = -stencil_apply<DIM>(tile, tile_center<DIM>(l), S);
            N.ahat[s]         = N.flag[s] ? fmaxf(sum, P.alpha0) : 1.f;
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
// Matrix-free operator: (A v)_I = alpha_hat_I v_I + sum_{J != I} c(|k|^2) V_J v_J
// on active rows, identity on inactive rows.
// ---------------------------------------------------------------------------
template<int DIM>
__global__ void __launch_bounds__(kNT) k_apply_operator(Lattice L, const int * __restrict__ blist,
                                                        const int * __restrict__ bcount,
                                                        const unsigned char * __restrict__ bflag, NodeArrays N,
                                                        Stencil S, const float * __restrict__ in,
                                                        float * __restrict__ out) {
    using G = BrickGeom<DIM>;
    __shared__ float tile[G::TILE];
    const int nb = *bcount;
    for (int bi = blockIdx.x; bi < nb; bi += gridDim.x) {
        const int b   = blist[bi];
        const int3 bc = brick_coords(L, b);
        __syncthreads();
        load_tile<DIM>(L, bflag, bc, tile, [&](long long s) { return N.V[s] * in[s]; });
        __syncthreads();
        for (int l = threadIdx.x; l < G::BN; l += kNT) {
            const long long s = (long long) b * G::BN + l;
            const float v     = in[s];
            out[s] = N.flag[s] ? fmaf(N.ahat[s], v, stencil_apply<DIM>(tile, tile_center<DIM>(l), S)) : v;
        }
    }
}

// ---------------------------------------------------------------------------
// CG (textbook Hestenes-Stiefel, identity preconditioner; reference
// Cores/Solvers/IterativeSolver.h:21-40 -> Eigen ConjugateGradient).
// Scalars live in CgState on the device; every kernel returns immediately once
// `done` is set, so a captured batch of iterations can overshoot harmlessly.
// ---------------------------------------------------------------------------
template<int DIM>
__global__ void __launch_bounds__(kNT) k_cg_init(Lattice L, const int * __restrict__ blist,
                                                 const int * __restrict__ bcount,
                                                 const unsigned char * __restrict__ bflag, NodeArrays N, Stencil S,
                                                 CgState * cg, double * __restrict__ partials, double tol,
                                                 int max_iterations, const int * __restrict__ nv) {
    using G = BrickGeom<DIM>;
    __shared__ float tile[G::TILE];
    __shared__ double red[kNT / 32];
    __shared__ int last;
    const int nb = *bcount;
    FF rr{0.f, 0.f}, bb{0.f, 0.f};
    for (int bi = blockIdx.x; bi < nb; bi += gridDim.x) {
        const int b   = blist[bi];
        const int3 bc = brick_coords(L, b);
        __syncthreads();
        load_tile<DIM>(L, bflag, bc, tile, [&](long long s) { return N.V[s] * N.x[s]; });
        __syncthreads();
        for (int l = threadIdx.x; l < G::BN; l += kNT) {
            const long long s = (long long) b * G::BN + l;
            const float xv    = N.x[s];
            const float q = N.flag[s] ? fmaf(N.ahat[s], xv, stencil_apply<DIM>(tile, tile_center<DIM>(l), S)) : xv;
            const float bv = N.D[s];
            const float r  = bv - q;
            N.r[s]  = r;
            N.d0[s] = r;
            ff_add_prod(rr, r, r);
            ff_add_prod(bb, bv, bv);
        }
    }
    // two reductions: reuse the machinery twice with separate partial slots
    const double prr = block_sum_ff<kNT>(rr, red);
    const double pbb = block_sum_ff<kNT>(bb, red);
    if (threadIdx.x == 0) {
        partials[blockIdx.x]             = prr;
        partials[gridDim.x + blockIdx.x] = pbb;
        __threadfence();
        last = atomicAdd(&cg->ticket[0], 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        volatile double * vp = partials;
        double srr = 0, sbb = 0;
        for (unsigned int k = 0; k < gridDim.x; k++) srr += vp[k];
        for (unsigned int k = 0; k < gridDim.x; k++) sbb += vp[gridDim.x + k];
        cg->ticket[0] = 0u;
        cg->bb        = sbb;
        cg->rr        = srr;
        cg->rr0       = srr;
        cg->rr_prev   = 0;
        cg->pq        = 0;
        cg->iter      = 0;
        const int n   = *nv;
        cg->max_iter  = max_iterations >= 0 ? max_iterations : 2 * n;
        const double eps = 2.220446049250313e-16, dmin = 2.2250738585072014e-308;
        if (n == 0 || sbb == 0.0) {
            cg->threshold = 0;
            cg->done      = sbb == 0.0 ? 4 : 1;  // 4: zero right-hand side -> x = 0
        } else {
            const double t   = fmax(tol, eps / sqrt(sbb));
            cg->threshold    = fmax(t * t * sbb, dmin);
            cg->done         = srr < cg->threshold ? 1 : (srr != srr ? 3 : 0);
            if (cg->done == 0 && cg->max_iter <= 0) cg->done = 2;
        }
    }
}

// Iteration part 1: d_i = r_i + beta d_{i-1} (i > 0; computed on the fly for the
// halo), q = A d_i, pq = d_i . q.
template<int DIM>
__global__ void __launch_bounds__(kNT) k_cg_spmv(Lattice L, const int * __restrict__ blist,
                                                 const int * __restrict__ bcount,
                                                 const unsigned char * __restrict__ bflag, NodeArrays N, Stencil S,
                                                 CgState * cg, double * __restrict__ partials) {
    using G = BrickGeom<DIM>;
    __shared__ float tile[G::TILE];
    __shared__ double red[kNT / 32];
    __shared__ int last;
    if (cg->done) return;
    const int it      = cg->iter;
    const float beta  = it == 0 ? 0.f : float(cg->rr / cg->rr_prev);
    const float * dpv = (it & 1) ? N.d0 : N.d1;  // d_{i-1}
    float * dcur      = (it & 1) ? N.d1 : N.d0;  // d_i
    const int nb      = *bcount;
    FF pq{0.f, 0.f};
    for (int bi = blockIdx.x; bi < nb; bi += gridDim.x) {
        const int b   = blist[bi];
        const int3 bc = brick_coords(L, b);
        __syncthreads();
        if (it == 0)
            load_tile<DIM>(L, bflag, bc, tile, [&](long long s) { return N.V[s] * dcur[s]; });
        else
            load_tile<DIM>(L, bflag, bc, tile, [&](long long s) { return N.V[s] * fmaf(beta, dpv[s], N.r[s]); });
        __syncthreads();
        for (int l = threadIdx.x; l < G::BN; l += kNT) {
            const long long s = (long long) b * G::BN + l;
            float dv;
            if (it == 0) dv = dcur[s];
            else {
                dv      = fmaf(beta, dpv[s], N.r[s]);
                dcur[s] = dv;
            }
            const float q = N.flag[s] ? fmaf(N.ahat[s], dv, stencil_apply<DIM>(tile, tile_center<DIM>(l), S)) : dv;
            N.q[s]        = q;
            ff_add_prod(pq, dv, q);
        }
    }
    const double part = block_sum_ff<kNT>(pq, red);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = part;
        __threadfence();
        last = atomicAdd(&cg->ticket[1], 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        volatile double * vp = partials;
        double s = 0;
        for (unsigned int k = 0; k < gridDim.x; k++) s += vp[k];
        cg->ticket[1] = 0u;
        cg->pq        = s;
        if (!(s != 0.0) || s != s) cg->done = 3;
    }
}

// Iteration part 2: alpha = rr / pq; x += alpha d_i; r -= alpha q; rr = r.r;
// convergence test |r|^2 < threshold.
template<int DIM>
__global__ void __launch_bounds__(kNT) k_cg_update(const int * __restrict__ blist, const int * __restrict__ bcount,
                                                   NodeArrays N, CgState * cg, double * __restrict__ partials) {
    using G = BrickGeom<DIM>;
    __shared__ double red[kNT / 32];
    __shared__ int last;
    if (cg->done) return;
    const int it      = cg->iter;
    const float alpha = float(cg->rr / cg->pq);
    const float * dc  = (it & 1) ? N.d1 : N.d0;
    const int nb      = *bcount;
    FF rr{0.f, 0.f};
    for (int bi = blockIdx.x; bi < nb; bi += gridDim.x) {
        const long long base = (long long) blist[bi] * G::BN;
        for (int l = threadIdx.x; l < G::BN; l += kNT) {
            const long long s = base + l;
            N.x[s]            = fmaf(alpha, dc[s], N.x[s]);
            const float r     = fmaf(-alpha, N.q[s], N.r[s]);
            N.r[s]            = r;
            ff_add_prod(rr, r, r);
        }
    }
    const double part = block_sum_ff<kNT>(rr, red);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = part;
        __threadfence();
        last = atomicAdd(&cg->ticket[2], 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        volatile double * vp = partials;
        double s = 0;
        for (unsigned int k = 0; k < gridDim.x; k++) s += vp[k];
        cg->ticket[2] = 0u;
        cg->rr_prev   = cg->rr;
        cg->rr        = s;
        cg->iter      = it + 1;
        if (s != s) cg->done = 3;
        else if (s < cg->threshold) cg->done = 1;
        else if (it + 1 >= cg->max_iter) cg->done = 2;
    }
}

// True residual |b - A x|^2 and |b|^2 (FP64 out2[0], out2[1]).
template<int DIM>
__global__ void __launch_bounds__(kNT) k_true_residual(Lattice L, const int * __restrict__ blist,
                                                       const int * __restrict__ bcount,
                                                       const unsigned char * __restrict__ bflag, NodeArrays N,
                                                       Stencil S, double * __restrict__ partials,
                                                       unsigned int * __restrict__ ticket, double * __restrict__ out2) {
    using G = BrickGeom<DIM>;
    __shared__ float tile[G::TILE];
    __shared__ double red[kNT / 32];
    __shared__ int last;
    const int nb = *bcount;
    double rr = 0, bb = 0;
    for (int bi = blockIdx.x; bi < nb; bi += gridDim.x) {
        const int b   = blist[bi];
        const int3 bc = brick_coords(L, b);
        __syncthreads();
        load_tile<DIM>(L, bflag, bc, tile, [&](long long s) { return N.V[s] * N.x[s]; });
        __syncthreads();
        for (int l = threadIdx.x; l < G::BN; l += kNT) {
            const long long s = (long long) b * G::BN + l;
            if (!N.flag[s]) continue;
            const double q = double(N.ahat[s]) * N.x[s] + double(stencil_apply<DIM>(tile, tile_center<DIM>(l), S));
            const double r = double(N.D[s]) - q;
            rr += r * r;
            bb += double(N.D[s]) * N.D[s];
        }
    }
    const double prr = block_sum_double<kNT>(rr, red);
    const double pbb = block_sum_double<kNT>(bb, red);
    if (threadIdx.x == 0) {
        partials[blockIdx.x]             = prr;
        partials[gridDim.x + blockIdx.x] = pbb;
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        volatile double * vp = partials;
        double a = 0, c = 0;
        for (unsigned int k = 0; k < gridDim.x; k++) a += vp[k];
        for (unsigned int k = 0; k < gridDim.x; k++) c += vp[gridDim.x + k];
        out2[0] = a;
        out2[1] = c;
        *ticket = 0u;
    }
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
void launch_brick_list(const unsigned char * bflag, int nbricks, int * list, int * count, cudaStream_t st) {
    k_brick_list<<<1, 1024, 0, st>>>(bflag, nbricks, list, count);
}

template<int DIM>
void launch_node_gather(const Lattice & L, const Phys & P, const BrickArrays & B, const NodeArrays & N,
                        const float4 * pos, const float4 * vel, const int * cellStart, const float4 * bpos,
                        const float4 * bvel, const int * bcellStart, int grid, cudaStream_t st) {
    k_node_gather<DIM><<<grid, kNT, 0, st>>>(L, P, B.list, B.count, N, pos, vel, cellStart, bpos, bvel, bcellStart);
}

template<int DIM>
void launch_segments(const Lattice & L, const BrickArrays & B, const NodeArrays & N, int * tiles, int grid,
                     cudaStream_t st) {
    cudaMemsetAsync(B.seg, 0, sizeof(int) * B.nseg, st);
    k_segment_count<DIM><<<grid, kNT, 0, st>>>(L, B.list, B.count, N.flag, B.seg);
    launch_scan(B.seg, B.nseg, B.seg_off, tiles, st);
}

template<int DIM>
void launch_ahat(const Lattice & L, const Phys & P, const BrickArrays & B, const NodeArrays & N, const Stencil & S,
                 int grid, cudaStream_t st) {
    k_ahat<DIM><<<grid, kNT, 0, st>>>(L, P, B.list, B.count, B.flag, N, S);
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

template<int DIM>
void launch_apply_operator(const Lattice & L, const BrickArrays & B, const NodeArrays & N, const Stencil & S,
                           const float * in, float * out, int grid, cudaStream_t st) {
    k_apply_operator<DIM><<<grid, kNT, 0, st>>>(L, B.list, B.count, B.flag, N, S, in, out);
}

template<int DIM>
void launch_cg_init(const Lattice & L, const BrickArrays & B, const NodeArrays & N, const Stencil & S, CgState * cg,
                    double * partials, double tol, int max_iterations, const int * nv, int grid, cudaStream_t st) {
    k_cg_init<DIM><<<grid, kNT, 0, st>>>(L, B.list, B.count, B.flag, N, S, cg, partials, tol, max_iterations, nv);
}

template<int DIM>
void launch_cg_iteration(const Lattice & L, const BrickArrays & B, const NodeArrays & N, const Stencil & S,
                         CgState * cg, double * partials, int grid, cudaStream_t st) {
    k_cg_spmv<DIM><<<grid, kNT, 0, st>>>(L, B.list, B.count, B.flag, N, S, cg, partials);
    k_cg_update<DIM><<<grid, kNT, 0, st>>>(B.list, B.count, N, cg, partials);
}

template<int DIM>
void launch_cg_spmv(const Lattice & L, const BrickArrays & B, const NodeArrays & N, const Stencil & S, CgState * cg,
                    double * partials, int grid, cudaStream_t st) {
    k_cg_spmv<DIM><<<grid, kNT, 0, st>>>(L, B.list, B.count, B.flag, N, S, cg, partials);
}
template<int DIM>
void launch_cg_update(const BrickArrays & B, const NodeArrays & N, CgState * cg, double * partials, int grid,
                      cudaStream_t st) {
    k_cg_update<DIM><<<grid, kNT, 0, st>>>(B.list, B.count, N, cg, partials);
}

template<int DIM>
void launch_true_residual(const Lattice & L, const BrickArrays & B, const NodeArrays & N, const Stencil & S,
                          double * partials, double * out2, int grid, cudaStream_t st) {
    // ticket lives just past the two partial arrays
    unsigned int * ticket = reinterpret_cast<unsigned int *>(partials + 2 * grid);
    k_true_residual<DIM><<<grid, kNT, 0, st>>>(L, B.list, B.count, B.flag, N, S, partials, ticket, out2);
}

#define SWC_INST(D)                                                                                                    \
    template void launch_node_gather<D>(const Lattice &, const Phys &, const BrickArrays &, const NodeArrays &,        \
                                        const float4 *, const float4 *, const int *, const float4 *, const float4 *,   \
                                        const int *, int, cudaStream_t);                                               \
    template void launch_segments<D>(const Lattice &, const BrickArrays &, const NodeArrays &, int *, int,             \
                                     cudaStream_t);                                                                    \
    template void launch_ahat<D>(const Lattice &, const Phys &, const BrickArrays &, const NodeArrays &,               \
                                 const Stencil &, int, cudaStream_t);                                                  \
    template void launch_diag_max_f64<D>(const Lattice &, const BrickArrays &, const NodeArrays &, const StencilD &,   \
                                         unsigned long long *, int, cudaStream_t);                                     \
    template void launch_warm_start<D>(const Lattice &, const BrickArrays &, const NodeArrays &, int, const float *,   \
                                       const int *, const float *, int, cudaStream_t);                                 \
    template void launch_compact_export<D>(const Lattice &, const BrickArrays &, const NodeArrays &, float *,          \
                                           long long *, double *, double *, double *, double *, double *, double *,    \
                                           unsigned short *, int, cudaStream_t);                                       \
    template void launch_compact_import<D>(const Lattice &, const BrickArrays &, const NodeArrays &, const double *,   \
                                           float *, int, cudaStream_t);                                                \
    template void launch_zero_active<D>(const Lattice &, const BrickArrays &, float *, int, cudaStream_t);             \
    template void launch_apply_operator<D>(const Lattice &, const BrickArrays &, const NodeArrays &, const Stencil &,   \
                                           const float *, float *, int, cudaStream_t);                                 \
    template void launch_cg_init<D>(const Lattice &, const BrickArrays &, const NodeArrays &, const Stencil &,         \
                                    CgState *, double *, double, int, const int *, int, cudaStream_t);                 \
    template void launch_cg_iteration<D>(const Lattice &, const BrickArrays &, const NodeArrays &, const Stencil &,    \
                                         CgState *, double *, int, cudaStream_t);                                      \
    template void launch_cg_spmv<D>(const Lattice &, const BrickArrays &, const NodeArrays &, const Stencil &,         \
                                    CgState *, double *, int, cudaStream_t);                                           \
    template void launch_cg_update<D>(const BrickArrays &, const NodeArrays &, CgState *, double *, int, cudaStream_t); \
    template void launch_true_residual<D>(const Lattice &, const BrickArrays &, const NodeArrays &, const Stencil &,   \
                                          double *, double *, int, cudaStream_t);
SWC_INST(2)
SWC_INST(3)
#undef SWC_INST

}  // namespace swc
