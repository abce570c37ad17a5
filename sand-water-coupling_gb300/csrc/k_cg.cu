// k_cg.cu -- matrix-free virtual Laplacian and CG of the dual-particle SPH
// projection (reference: VirtualParticle::calculateCoef / solveLinearSystem,
// Cores/Structures/VirtualParticle.cpp:149-169,105-108, and the Eigen CG behind
// Cores/Solvers/IterativeSolver.h:21-40).
//
// Because virtual particles sit on lattice nodes, alpha_IJ = c(|k|^2) V_J with a
// radial coefficient table c, so
//     (A v)_I = alpha_hat_I v_I + sum_{0 < |k|^2 < 16} c(|k|^2) (V v)_{I+k}
// on active rows; inactive rows are identity rows with zero right-hand side and
// zero start, so CG over whole bricks is CG over the active set.
//
// Kernels: one CTA per brick (row-stencil kernels: one thread per brick x-row,
// 8 outputs along x in 3D), the V-weighted halo tile staged in shared memory
// with 16-byte copies.  A CG iteration is three kernels: the direction update
// d = r + beta d with u = V d (streaming), the SpMV q = A d reading u tiles by
// double-buffered cp.async, and the x/r update; dot products use exact FP32
// products summed in float-float below the warp and FP64 above, reduced
// deterministically.  A is not symmetric (alpha_IJ carries V_J) and the
// reference runs Hestenes-Stiefel CG on the full matrix, so single-reduction
// rearrangements that rely on symmetry (Chronopoulos-Gear, pipelined CG) are
// not equivalent here: on a 2D dam break the Chronopoulos-Gear form stalls
// after ~10 iterations where this form converges.
#include "swc_kernels.h"
#include "swc_tiles.cuh"

namespace swc {

template<int DIM> struct KG {
    static constexpr int NT = RowGeom<DIM>::NT;         // rows per brick
    static constexpr int BT = NT < 32 ? 32 : NT;        // threads per block
};
constexpr int kUT = 256;  // threads per block of the streaming update

__device__ __forceinline__ float4 ld4(const float * a, long long s) { return *reinterpret_cast<const float4 *>(a + s); }
__device__ __forceinline__ void st4(float * a, long long s, float4 v) { *reinterpret_cast<float4 *>(a + s) = v; }
__device__ __forceinline__ float4 mul4(float4 a, float4 b) { return make_float4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
__device__ __forceinline__ float4 fma4(float s, float4 a, float4 b) {
    return make_float4(fmaf(s, a.x, b.x), fmaf(s, a.y, b.y), fmaf(s, a.z, b.z), fmaf(s, a.w, b.w));
}
__device__ __forceinline__ float comp(const float4 & v, int j) { return j == 0 ? v.x : j == 1 ? v.y : j == 2 ? v.z : v.w; }
__device__ __forceinline__ unsigned char compb(const uchar4 & v, int j) {
    return j == 0 ? v.x : j == 1 ? v.y : j == 2 ? v.z : v.w;
}

// Slot of the first node of brick row (ly, lz).
template<int DIM> __device__ __forceinline__ long long row_base(int b, int ly, int lz) {
    using G = BrickGeom<DIM>;
    return (long long) b * G::BN + G::BX * (ly + G::BY * lz);
}

// y = A v (test hook).
template<int DIM>
__global__ void __launch_bounds__(KG<DIM>::BT) k_apply_operator(Lattice L, const int * __restrict__ blist,
                                                                const int * __restrict__ bcount,
                                                                const unsigned char * __restrict__ bflag, NodeArrays N,
                                                                Stencil S, const float * __restrict__ in,
                                                                float * __restrict__ out) {
    using G = BrickGeom<DIM>;
    __shared__ __align__(16) float tile[G::TILE];
    const int nb = *bcount;
    const int t = threadIdx.x, ly = t % G::BY, lz = t / G::BY;
    for (int bi = blockIdx.x; bi < nb; bi += gridDim.x) {
        const int b   = blist[bi];
        const int3 bc = brick_coords(L, b);
        __syncthreads();
        load_tile4<DIM>(L, bflag, bc, tile, [&](long long s) { return mul4(ld4(N.V, s), ld4(in, s)); });
        __syncthreads();
        if (t < KG<DIM>::NT) {
            float acc[G::BX];
            stencil_row<DIM>(tile, ly, lz, S, acc);
            const long long base = row_base<DIM>(b, ly, lz);
#pragma unroll
            for (int k = 0; k < G::BX / 4; k++) {
                const float4 v = ld4(in, base + 4 * k), a = ld4(N.ahat, base + 4 * k);
                const uchar4 f = *reinterpret_cast<const uchar4 *>(N.flag + base + 4 * k);
                float4 o;
                o.x = f.x ? fmaf(a.x, v.x, acc[4 * k]) : v.x;
                o.y = f.y ? fmaf(a.y, v.y, acc[4 * k + 1]) : v.y;
                o.z = f.z ? fmaf(a.z, v.z, acc[4 * k + 2]) : v.z;
                o.w = f.w ? fmaf(a.w, v.w, acc[4 * k + 3]) : v.w;
                st4(out, base + 4 * k, o);
            }
        }
    }
}

// The base start won the residual test: x = xb, r = d = rb (all slots of the
// active bricks, 16-byte streaming).
template<int DIM>
__global__ void __launch_bounds__(kUT) k_cg_pick_base(const int * __restrict__ blist, const int * __restrict__ bcount,
                                                      NodeArrays N, const float * __restrict__ xb,
                                                      const float * __restrict__ rb, const CgState * __restrict__ cg) {
    pdl_wait_and_release();
    using G = BrickGeom<DIM>;
    constexpr int Q = G::BN / 4;
    if (cg->start != 1) return;
    const int nb = *bcount;
    for (long long e = blockIdx.x * (long long) kUT + threadIdx.x; e < (long long) nb * Q; e += (long long) gridDim.x * kUT) {
        const long long s = (long long) blist[e / Q] * G::BN + 4 * (e % Q);
        const float4 r = ld4(rb, s);
        st4(N.x, s, ld4(xb, s));
        st4(N.r, s, r);
        st4(N.d, s, r);
    }
}

// Iteration part 0: d_i = r_i + beta d_{i-1} (i > 0) and u = V d_i (16-byte streaming).
template<int DIM>
__global__ void __launch_bounds__(kUT) k_cg_direction(const int * __restrict__ blist, const int * __restrict__ bcount,
                                                      NodeArrays N, const CgState * __restrict__ cg) {
    using G = BrickGeom<DIM>;
    constexpr int Q = G::BN / 4;
    pdl_wait_and_release();
    if (cg->done) return;
    const int it     = cg->iter;
    const float beta = it == 0 ? 0.f : float(cg->rr / cg->rr_prev);
    const long long total = (long long) (*bcount) * Q;
    for (long long i = blockIdx.x * (long long) kUT + threadIdx.x; i < total; i += (long long) gridDim.x * kUT) {
        const long long s = (long long) blist[i / Q] * G::BN + 4 * (i % Q);
        float4 d          = ld4(N.d, s);
        if (it > 0) {
            d = fma4(beta, d, ld4(N.r, s));
            st4(N.d, s, d);
        }
        st4(N.u, s, mul4(ld4(N.V, s), d));
    }
}

// Asynchronous copy of the u halo tile of a brick (16-byte segments, zero-filled
// outside the active set).
template<int DIM>
__device__ __forceinline__ void prefetch_u_tile(const int * tab, const float * __restrict__ u, float * tile) {
    using G            = BrickGeom<DIM>;
    using T            = SpmvTile<DIM>;
    constexpr int SEGX = T::TX / 4;
    constexpr int NSEG = SEGX * T::TY * T::TZ;
    constexpr int NT   = RowGeom<DIM>::NT;
#pragma unroll 4
    for (int t = threadIdx.x; t < NSEG; t += NT) {
        const int sx = t % SEGX, ty = (t / SEGX) % T::TY, tz = t / (SEGX * T::TY);
        const int tx = 4 * sx;
        // neighbour offset (-1, 0, 1) and local coordinate along each axis
        const int oi = (tx - T::HX + G::BX) / G::BX - 1, oj = (ty - T::HY + G::BY) / G::BY - 1;
        const int ok = DIM == 3 ? (tz - T::HZ + G::BZ) / G::BZ - 1 : 0;
        const int lx = tx - T::HX - G::BX * oi, ly = ty - T::HY - G::BY * oj;
        const int lz = DIM == 3 ? tz - T::HZ - G::BZ * ok : 0;
        const int nb = tab[(ok + 1) * 9 + (oj + 1) * 3 + (oi + 1)];
        const long long s = (long long) (nb < 0 ? 0 : nb) * G::BN + lx + G::BX * (ly + G::BY * lz);
        cp_async16(tile + tx + T::PX * (ty + T::TY * tz), u + s, nb >= 0);
    }
}

// Iteration part 1: q = A d_i and pq = d_i . q.  The u = V d tile of the next
// brick is copied asynchronously while the current one is computed.  The grid
// is the resident capacity and bricks are strided statically over it (a
// dynamic brick queue with per-brick partials measured slower: its atomics and
// per-brick block reductions cost more than the tail it removes).
template<int DIM>
__global__ void __launch_bounds__(KG<DIM>::BT) k_cg_spmv(Lattice L, const int * __restrict__ blist,
                                                         const int * __restrict__ bcount,
                                                         const unsigned char * __restrict__ bflag, NodeArrays N,
                                                         Stencil S, CgState * cg, double * __restrict__ partials) {
    using G = BrickGeom<DIM>;
    using T = SpmvTile<DIM>;
    constexpr int BT = KG<DIM>::BT;
    __shared__ __align__(16) float tile[2][T::TILE];
    __shared__ int tab[2][27];
    __shared__ double red[BT / 32 + 1];
    __shared__ int last;
    pdl_wait_and_release();
    if (cg->done) return;
    const int nb = *bcount;
    const int t = threadIdx.x, ly = t % G::BY, lz = t / G::BY;
    FF pq{0.f, 0.f};
    if (blockIdx.x < nb) neighbour_table<DIM>(L, bflag, blist[blockIdx.x], tab[0]);
    __syncthreads();
    if (blockIdx.x < nb) prefetch_u_tile<DIM>(tab[0], N.u, tile[0]);
    cp_async_commit();
    int k = 0;
    for (int bi = blockIdx.x; bi < nb; bi += gridDim.x, k ^= 1) {
        const int nxt = bi + gridDim.x;
        if (nxt < nb) neighbour_table<DIM>(L, bflag, blist[nxt], tab[k ^ 1]);
        __syncthreads();
        if (nxt < nb) prefetch_u_tile<DIM>(tab[k ^ 1], N.u, tile[k ^ 1]);
        cp_async_commit();
        cp_async_wait1();  // the current tile has landed
        __syncthreads();
        const int b = blist[bi];
        if (t < KG<DIM>::NT) {
            float acc[G::BX];
            stencil_row_t<DIM, T::PX, T::TY, T::HY, T::HZ>(tile[k], ly, lz, S, acc);
            const long long base = row_base<DIM>(b, ly, lz);
#pragma unroll
            for (int kk = 0; kk < G::BX / 4; kk++) {
                const float4 dv = ld4(N.d, base + 4 * kk);
                const float4 a  = ld4(N.ahat, base + 4 * kk);
                const uchar4 f  = *reinterpret_cast<const uchar4 *>(N.flag + base + 4 * kk);
                float q[4];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    q[j] = compb(f, j) ? fmaf(comp(a, j), comp(dv, j), acc[4 * kk + j]) : comp(dv, j);
                    ff_add_prod(pq, comp(dv, j), q[j]);
                }
                st4(N.q, base + 4 * kk, make_float4(q[0], q[1], q[2], q[3]));
            }
        }
        __syncthreads();  // tile[k] and tab[k] are refilled two iterations later
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    double part[1] = {block_sum_ff<BT>(pq, red)};
    double tot[1];
    if (grid_reduce<BT, 1>(part, partials, &cg->ticket[1], tot, red, &last) && threadIdx.x == 0) {
        cg->pq = tot[0];
        if (!(tot[0] != 0.0) || tot[0] != tot[0]) cg->done = 3;
    }
}

// Row-stencil passes on the SpMV's tile pipeline (neighbour table, halo tile
// of `src` copied with cp.async one brick ahead, static brick striding over a
// resident grid); the stencil arithmetic is stencil_row's, so the results equal
// the single-buffered versions bit for bit.
//   kRowsAhat:  alpha_hat = max(-sum_J alpha_IJ, alpha0) from src = V
//               (calculateCoef, VirtualParticle.cpp:149-169).
//   kRowsResid: r = b - A x from src = V x: r (and d when non-null) written,
//               |r|^2 and |b|^2 summed (deterministic) into sums[0..1].
enum { kRowsAhat = 0, kRowsResid = 1 };
template<int DIM, int OP>
__global__ void __launch_bounds__(KG<DIM>::BT) k_rows_tiled(Lattice L, Phys P, const int * __restrict__ blist,
                                                            const int * __restrict__ bcount,
                                                            const unsigned char * __restrict__ bflag, NodeArrays N,
                                                            Stencil S, const float * __restrict__ src,
                                                            const float * __restrict__ xin, float * __restrict__ r_out,
                                                            float * __restrict__ d_out, double * __restrict__ sums,
                                                            double * __restrict__ partials,
                                                            unsigned int * __restrict__ ticket) {
    pdl_wait_and_release();
    using G = BrickGeom<DIM>;
    using T = SpmvTile<DIM>;
    constexpr int BT = KG<DIM>::BT;
    __shared__ __align__(16) float tile[2][T::TILE];
    __shared__ int tab[2][27];
    __shared__ double red[BT / 32 + 1];
    __shared__ int last;
    const int nb = *bcount;
    const int t = threadIdx.x, ly = t % G::BY, lz = t / G::BY;
    FF rr{0.f, 0.f}, bb{0.f, 0.f};
    if (blockIdx.x < nb) neighbour_table<DIM>(L, bflag, blist[blockIdx.x], tab[0]);
    __syncthreads();
    if (blockIdx.x < nb) prefetch_u_tile<DIM>(tab[0], src, tile[0]);
    cp_async_commit();
    int k = 0;
    for (int bi = blockIdx.x; bi < nb; bi += gridDim.x, k ^= 1) {
        const int nxt = bi + gridDim.x;
        if (nxt < nb) neighbour_table<DIM>(L, bflag, blist[nxt], tab[k ^ 1]);
        __syncthreads();
        if (nxt < nb) prefetch_u_tile<DIM>(tab[k ^ 1], src, tile[k ^ 1]);
        cp_async_commit();
        cp_async_wait1();  // the current tile has landed
        __syncthreads();
        const int b = blist[bi];
        if (t < KG<DIM>::NT) {
            float acc[G::BX];
            stencil_row_t<DIM, T::PX, T::TY, T::HY, T::HZ>(tile[k], ly, lz, S, acc);
            const long long base = row_base<DIM>(b, ly, lz);
#pragma unroll
            for (int kk = 0; kk < G::BX / 4; kk++) {
                const uchar4 f = *reinterpret_cast<const uchar4 *>(N.flag + base + 4 * kk);
                if (OP == kRowsAhat) {
                    float4 a;
                    a.x = f.x ? fmaxf(-acc[4 * kk], P.alpha0) : 1.f;
                    a.y = f.y ? fmaxf(-acc[4 * kk + 1], P.alpha0) : 1.f;
                    a.z = f.z ? fmaxf(-acc[4 * kk + 2], P.alpha0) : 1.f;
                    a.w = f.w ? fmaxf(-acc[4 * kk + 3], P.alpha0) : 1.f;
                    st4(N.ahat, base + 4 * kk, a);
                } else {
                    const float4 xv = ld4(xin, base + 4 * kk), a = ld4(N.ahat, base + 4 * kk),
                                 bv = ld4(N.D, base + 4 * kk);
                    float r[4];
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        const float q = compb(f, j) ? fmaf(comp(a, j), comp(xv, j), acc[4 * kk + j]) : comp(xv, j);
                        r[j]          = comp(bv, j) - q;
                        ff_add_prod(rr, r[j], r[j]);
                        ff_add_prod(bb, comp(bv, j), comp(bv, j));
                    }
                    const float4 r4 = make_float4(r[0], r[1], r[2], r[3]);
                    st4(r_out, base + 4 * kk, r4);
                    if (d_out) st4(d_out, base + 4 * kk, r4);
                }
            }
        }
        __syncthreads();  // tile[k] and tab[k] are refilled two iterations later
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    if (OP == kRowsResid) {
        double part[2] = {block_sum_ff<BT>(rr, red), 0.0};
        part[1]        = block_sum_ff<BT>(bb, red);
        double tot[2];
        if (grid_reduce<BT, 2>(part, partials, ticket, tot, red, &last) && threadIdx.x == 0) {
            sums[0] = tot[0];
            sums[1] = tot[1];
        }
    }
}

// u = V x over the slots of the active bricks (16-byte streaming).
template<int DIM>
__global__ void __launch_bounds__(kUT) k_vmul(const int * __restrict__ blist, const int * __restrict__ bcount,
                                              const float * __restrict__ V, const float * __restrict__ x,
                                              float * __restrict__ u) {
    pdl_wait_and_release();
    using G = BrickGeom<DIM>;
    constexpr int Q = G::BN / 4;
    const long long total = (long long) (*bcount) * Q;
    for (long long e = blockIdx.x * (long long) kUT + threadIdx.x; e < total; e += (long long) gridDim.x * kUT) {
        const long long s = (long long) blist[e / Q] * G::BN + 4 * (e % Q);
        st4(u, s, mul4(ld4(V, s), ld4(x, s)));
    }
}

// CG start state from the residual sums (Eigen's stopping rule:
// |r|^2 < max(tol, eps/|b|)^2 |b|^2, cap 2 N_v).  With a second candidate
// (sums_b, the base start of the learned warm start) the prediction is kept
// when the network reported no error, its residual is finite and, unless
// keep_prediction, not larger than the base's; cg->start records the choice
// (0 prediction, 1 base) for k_cg_pick_base and the host.
__global__ void k_cg_start(CgState * cg, const double * __restrict__ sums_l, const double * __restrict__ sums_b,
                           const int * __restrict__ mlp_err, int keep_prediction, double tol, int max_iterations,
                           const int * __restrict__ nv) {
    pdl_wait_and_release();
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const double srr_l = sums_l[0], sbb = sums_l[1];
    bool keep = true;
    if (sums_b) {
        const double srr_b = sums_b[0];
        keep = (!mlp_err || *mlp_err == 0) && srr_l == srr_l && (keep_prediction || srr_l <= srr_b);
    }
    const double srr = keep ? srr_l : sums_b[0];
    cg->start   = keep ? 0 : 1;
    cg->bb      = sbb;
    cg->rr      = srr;
    cg->rr0     = srr;
    cg->rr_prev = 0;
    cg->pq      = 0;
    cg->iter    = 0;
    const int n  = *nv;
    cg->max_iter = max_iterations >= 0 ? max_iterations : 2 * n;
    const double eps = 2.220446049250313e-16, dmin = 2.2250738585072014e-308;
    if (n == 0 || sbb == 0.0) {
        cg->threshold = 0;
        cg->done      = sbb == 0.0 ? 4 : 1;  // 4: zero right-hand side -> x = 0
    } else {
        const double tt = fmax(tol, eps / sqrt(sbb));
        cg->threshold   = fmax(tt * tt * sbb, dmin);
        cg->done        = srr < cg->threshold ? 1 : (srr != srr ? 3 : 0);
        if (cg->done == 0 && cg->max_iter <= 0) cg->done = 2;
    }
}

// Iteration part 2: alpha = rr / pq; x += alpha d_i; r -= alpha q; rr = r.r;
// convergence test |r|^2 < threshold (16-byte streaming).
template<int DIM>
__global__ void __launch_bounds__(kUT) k_cg_update(const int * __restrict__ blist, const int * __restrict__ bcount,
                                                   NodeArrays N, CgState * cg, double * __restrict__ partials) {
    using G = BrickGeom<DIM>;
    constexpr int Q = G::BN / 4;
    __shared__ double red[kUT / 32 + 1];
    __shared__ int last;
    pdl_wait_and_release();
    if (cg->done) return;
    const int it      = cg->iter;
    const float alpha = float(cg->rr / cg->pq);
    const long long total = (long long) (*bcount) * Q;
    FF rr{0.f, 0.f};
    for (long long i = blockIdx.x * (long long) kUT + threadIdx.x; i < total; i += (long long) gridDim.x * kUT) {
        const long long s = (long long) blist[i / Q] * G::BN + 4 * (i % Q);
        const float4 d = ld4(N.d, s), q = ld4(N.q, s);
        float4 x = ld4(N.x, s), r = ld4(N.r, s);
        x = fma4(alpha, d, x);
        r = fma4(-alpha, q, r);
        st4(N.x, s, x);
        st4(N.r, s, r);
        ff_add_prod(rr, r.x, r.x);
        ff_add_prod(rr, r.y, r.y);
        ff_add_prod(rr, r.z, r.z);
        ff_add_prod(rr, r.w, r.w);
    }
    double part[1] = {block_sum_ff<kUT>(rr, red)};
    double tot[1];
    if (grid_reduce<kUT, 1>(part, partials, &cg->ticket[2], tot, red, &last) && threadIdx.x == 0) {
        const double s = tot[0];
        cg->rr_prev    = cg->rr;
        cg->rr         = s;
        cg->iter       = it + 1;
        if (s != s) cg->done = 3;
        else if (s < cg->threshold) cg->done = 1;
        else if (it + 1 >= cg->max_iter) cg->done = 2;
    }
}

// True residual |b - A x|^2 and |b|^2 (FP64, out2[0], out2[1]).
// |b|^2 = sum_I D_I^2 into cg->bb (the learned start's scale sD before the
// solve, when no fallback residual of the node-mapped start is needed).
template<int DIM>
__global__ void __launch_bounds__(kUT) k_rhs_norm(const int * __restrict__ blist, const int * __restrict__ bcount,
                                                  NodeArrays N, CgState * cg, double * __restrict__ partials) {
    pdl_wait_and_release();
    using G = BrickGeom<DIM>;
    constexpr int Q = G::BN / 4;
    __shared__ double red[kUT / 32 + 1];
    __shared__ int last;
    const long long total = (long long) (*bcount) * Q;
    FF bb{0.f, 0.f};
    for (long long i = blockIdx.x * (long long) kUT + threadIdx.x; i < total; i += (long long) gridDim.x * kUT) {
        const float4 d = ld4(N.D, (long long) blist[i / Q] * G::BN + 4 * (i % Q));
        ff_add_prod(bb, d.x, d.x);
        ff_add_prod(bb, d.y, d.y);
        ff_add_prod(bb, d.z, d.z);
        ff_add_prod(bb, d.w, d.w);
    }
    double part[1] = {block_sum_ff<kUT>(bb, red)};
    double tot[1];
    if (grid_reduce<kUT, 1>(part, partials, &cg->ticket[3], tot, red, &last) && threadIdx.x == 0) cg->bb = tot[0];
}

template<int DIM>
__global__ void __launch_bounds__(KG<DIM>::BT) k_true_residual(Lattice L, const int * __restrict__ blist,
                                                               const int * __restrict__ bcount,
                                                               const unsigned char * __restrict__ bflag, NodeArrays N,
                                                               Stencil S, CgState * cg, double * __restrict__ partials,
                                                               double * __restrict__ out2) {
    using G = BrickGeom<DIM>;
    constexpr int BT = KG<DIM>::BT;
    __shared__ __align__(16) float tile[G::TILE];
    __shared__ double red[BT / 32 + 1];
    __shared__ int last;
    const int nb = *bcount;
    const int t = threadIdx.x, ly = t % G::BY, lz = t / G::BY;
    double rr = 0, bb = 0;
    for (int bi = blockIdx.x; bi < nb; bi += gridDim.x) {
        const int b   = blist[bi];
        const int3 bc = brick_coords(L, b);
        __syncthreads();
        load_tile4<DIM>(L, bflag, bc, tile, [&](long long s) { return mul4(ld4(N.V, s), ld4(N.x, s)); });
        __syncthreads();
        if (t < KG<DIM>::NT) {
            float acc[G::BX];
            stencil_row<DIM>(tile, ly, lz, S, acc);
            const long long base = row_base<DIM>(b, ly, lz);
#pragma unroll
            for (int i = 0; i < G::BX; i++) {
                if (!N.flag[base + i]) continue;
                const double q = double(N.ahat[base + i]) * N.x[base + i] + double(acc[i]);
                const double r = double(N.D[base + i]) - q;
                rr += r * r;
                bb += double(N.D[base + i]) * N.D[base + i];
            }
        }
    }
    double part[2] = {block_sum_double<BT>(rr, red), 0.0};
    part[1]        = block_sum_double<BT>(bb, red);
    double tot[2];
    if (grid_reduce<BT, 2>(part, partials, &cg->ticket[3], tot, red, &last) && threadIdx.x == 0) {
        out2[0] = tot[0];
        out2[1] = tot[1];
    }
}

// ---------------------------------------------------------------------------
// Launchers (sgrid: blocks of the row-stencil kernels; ugrid: of the update)
// ---------------------------------------------------------------------------
template<int DIM>
void launch_ahat(const Lattice & L, const Phys & P, const BrickArrays & B, const NodeArrays & N, const Stencil & S,
                 int sgrid, cudaStream_t st) {
    launch_pdl(k_rows_tiled<DIM, kRowsAhat>, sgrid, KG<DIM>::BT, 0, st, L, P, B.list, B.count, B.flag, N, S, N.V, nullptr, nullptr,
                                                                nullptr, nullptr, nullptr, nullptr);
}
template<int DIM>
void launch_apply_operator(const Lattice & L, const BrickArrays & B, const NodeArrays & N, const Stencil & S,
                           const float * in, float * out, int sgrid, cudaStream_t st) {
    k_apply_operator<DIM><<<sgrid, KG<DIM>::BT, 0, st>>>(L, B.list, B.count, B.flag, N, S, in, out);
}
// r = b - A x: u = V x staged in N.u (free until the first CG direction pass),
// the tiled residual pass, the start state.
template<int DIM>
void launch_cg_init(const Lattice & L, const BrickArrays & B, const NodeArrays & N, const Stencil & S, CgState * cg,
                    double * partials, double tol, int max_iterations, const int * nv, int sgrid, int ugrid,
                    cudaStream_t st) {
    launch_pdl(k_vmul<DIM>, ugrid, kUT, 0, st, B.list, B.count, N.V, N.x, N.u);
    launch_pdl(k_rows_tiled<DIM, kRowsResid>, sgrid, KG<DIM>::BT, 0, st, L, Phys{}, B.list, B.count, B.flag, N, S, N.u, N.x,
                                                                 N.r, N.d, cg->sums, partials, &cg->ticket[0]);
    launch_pdl(k_cg_start, 1, 32, 0, st, cg, cg->sums, nullptr, nullptr, 0, tol, max_iterations, nv);
}
// Residual of one candidate start x: r = b - A x into r (and d when non-null),
// |r|^2 and |b|^2 into sums[0..1] (u = V x staged in N.u).
template<int DIM>
void launch_cg_residual(const Lattice & L, const BrickArrays & B, const NodeArrays & N, const Stencil & S,
                        const float * x, float * r, float * d, double * sums, CgState * cg, double * partials,
                        int sgrid, int ugrid, cudaStream_t st) {
    launch_pdl(k_vmul<DIM>, ugrid, kUT, 0, st, B.list, B.count, N.V, x, N.u);
    launch_pdl(k_rows_tiled<DIM, kRowsResid>, sgrid, KG<DIM>::BT, 0, st, L, Phys{}, B.list, B.count, B.flag, N, S, N.u, x, r, d,
                                                                 sums, partials, &cg->ticket[0]);
}
// Start state keeping the better of the prediction (residual in cg->sums[0..1],
// already in N.x / N.r / N.d) and the base start xb (cg->sums[2..3], residual rb),
// and the base copied in when it wins.
template<int DIM>
void launch_cg_pick(const BrickArrays & B, const NodeArrays & N, const float * xb, const float * rb,
                    const int * mlp_err, bool keep_prediction, CgState * cg, double tol, int max_iterations,
                    const int * nv, int ugrid, cudaStream_t st) {
    launch_pdl(k_cg_start, 1, 32, 0, st, cg, cg->sums, cg->sums + 2, mlp_err, keep_prediction ? 1 : 0, tol, max_iterations, nv);
    launch_pdl(k_cg_pick_base<DIM>, ugrid, kUT, 0, st, B.list, B.count, N, xb, rb, cg);
}
template<int DIM>
void launch_cg_spmv(const Lattice & L, const BrickArrays & B, const NodeArrays & N, const Stencil & S, CgState * cg,
                    double * partials, int sgrid, cudaStream_t st) {
    launch_pdl(k_cg_spmv<DIM>, sgrid, KG<DIM>::BT, 0, st, L, (const int *) B.list, (const int *) B.count,
               (const unsigned char *) B.flag, N, S, cg, partials);
}
template<int DIM> int cg_spmv_blocks_per_sm() {
    // all of the unified L1 / shared memory as shared memory: the SpMV keeps no
    // data in L1 worth more than a seventh resident block
    cudaFuncSetAttribute(k_cg_spmv<DIM>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_cg_spmv<DIM>, KG<DIM>::BT, 0) != cudaSuccess) n = 1;
    return n > 0 ? n : 1;
}
template<int DIM>
void launch_cg_update(const BrickArrays & B, const NodeArrays & N, CgState * cg, double * partials, int ugrid,
                      cudaStream_t st) {
    launch_pdl(k_cg_update<DIM>, ugrid, kUT, 0, st, (const int *) B.list, (const int *) B.count, N, cg, partials);
}
template<int DIM>
void launch_cg_direction(const BrickArrays & B, const NodeArrays & N, const CgState * cg, int ugrid, cudaStream_t st) {
    launch_pdl(k_cg_direction<DIM>, ugrid, kUT, 0, st, (const int *) B.list, (const int *) B.count, N, cg);
}
template<int DIM>
void launch_cg_iteration(const Lattice & L, const BrickArrays & B, const NodeArrays & N, const Stencil & S,
                         CgState * cg, double * partials, int sgrid, int ugrid, cudaStream_t st) {
    launch_cg_direction<DIM>(B, N, cg, ugrid, st);
    launch_cg_spmv<DIM>(L, B, N, S, cg, partials, sgrid, st);
    launch_cg_update<DIM>(B, N, cg, partials, ugrid, st);
}
template<int DIM>
void launch_true_residual(const Lattice & L, const BrickArrays & B, const NodeArrays & N, const Stencil & S,
                          CgState * cg, double * partials, double * out2, int sgrid, cudaStream_t st) {
    k_true_residual<DIM><<<sgrid, KG<DIM>::BT, 0, st>>>(L, B.list, B.count, B.flag, N, S, cg, partials, out2);
}
template<int DIM>
void launch_rhs_norm(const BrickArrays & B, const NodeArrays & N, CgState * cg, double * partials, int ugrid,
                     cudaStream_t st) {
    launch_pdl(k_rhs_norm<DIM>, ugrid, kUT, 0, st, B.list, B.count, N, cg, partials);
}

#define SWC_INST(D)                                                                                                    \
    template void launch_ahat<D>(const Lattice &, const Phys &, const BrickArrays &, const NodeArrays &,               \
                                 const Stencil &, int, cudaStream_t);                                                  \
    template void launch_apply_operator<D>(const Lattice &, const BrickArrays &, const NodeArrays &, const Stencil &,   \
                                           const float *, float *, int, cudaStream_t);                                 \
    template void launch_cg_init<D>(const Lattice &, const BrickArrays &, const NodeArrays &, const Stencil &,         \
                                    CgState *, double *, double, int, const int *, int, int, cudaStream_t);            \
    template void launch_cg_residual<D>(const Lattice &, const BrickArrays &, const NodeArrays &, const Stencil &,     \
                                        const float *, float *, float *, double *, CgState *, double *, int, int,      \
                                        cudaStream_t);                                                                 \
    template void launch_cg_pick<D>(const BrickArrays &, const NodeArrays &, const float *, const float *, const int *, \
                                    bool, CgState *, double, int, const int *, int, cudaStream_t);                     \
    template void launch_cg_spmv<D>(const Lattice &, const BrickArrays &, const NodeArrays &, const Stencil &,         \
                                    CgState *, double *, int, cudaStream_t);                                           \
    template void launch_cg_update<D>(const BrickArrays &, const NodeArrays &, CgState *, double *, int, cudaStream_t); \
    template void launch_cg_direction<D>(const BrickArrays &, const NodeArrays &, const CgState *, int, cudaStream_t); \
    template void launch_cg_iteration<D>(const Lattice &, const BrickArrays &, const NodeArrays &, const Stencil &,    \
                                         CgState *, double *, int, int, cudaStream_t);                                 \
    template void launch_true_residual<D>(const Lattice &, const BrickArrays &, const NodeArrays &, const Stencil &,   \
                                          CgState *, double *, double *, int, cudaStream_t);                           \
    template int cg_spmv_blocks_per_sm<D>();                                                                           \
    template void launch_rhs_norm<D>(const BrickArrays &, const NodeArrays &, CgState *, double *, int, cudaStream_t);
SWC_INST(2)
SWC_INST(3)
#undef SWC_INST

}  // namespace swc
