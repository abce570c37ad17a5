// k_mlp.cu -- learned CG warm start: a per-virtual-particle MLP 8 -> 64 -> 64 -> 1
// (SiLU) predicting a correction of a node's time-extrapolated pressure from
// local features and the node's pressure history.  No counterpart in the
// reference; CG still iterates to the same tolerance and the extrapolated base
// start is kept whenever the prediction starts from a larger residual.
//
// Forward pass on the 5th-generation tensor cores: M = 128 rows (nodes) per tile,
// BF16 operands staged in shared memory in the K-major no-swizzle canonical
// layout (8-row x 16-byte core matrices), tcgen05.mma kind::f16 issued by one
// thread with FP32 accumulators in TMEM (64 columns, reused by both layers), completion tracked by
// an mbarrier, accumulators read back with tcgen05.ld for the FP32 epilogues
// (bias, SiLU, final 64-wide dot).  Every wait is bounded: on timeout the kernel
// records an error, frees its TMEM and returns.
//
// Training: the fused tensor-core gradient pass of k_mlp_train.cu and Adam (FP32
// master weights), all deterministic.
#include <algorithm>
#include <cstdio>
#include <mutex>

#include "../../include/swc.h"
#include "swc_kernels.h"
#include "swc_tc.cuh"

namespace swc {

// Per-node features (the definitions of include/swc.h) from the raw node
// values D, alpha_hat, n_real, p_base (x after the history warm start), p1
// (xm1), p1 - 2 p2 + p3 (d2p) and rho, held in g[0..6].  Returns the node's
// history scale s (the unit of the target).
struct FeatScale {
    float inv_sD, inv_alpha0, inv_rho0, inv_nreal;
};
constexpr float kMlpScaleEps = SWC_MLP_SCALE_EPS;
static_assert(kMlpIn == 8, "feature layout");
__device__ __forceinline__ void node_raw(const NodeArrays & N, long long s, float (&g)[kMlpIn]) {
    g[0] = N.D[s];
    g[1] = N.ahat[s];
    g[2] = N.nreal ? float(N.nreal[s]) : 0.f;
    g[3] = N.x[s];
    g[4] = N.xm1[s];
    g[5] = N.d2p ? N.d2p[s] : 0.f;
    g[6] = N.rho[s];
    g[7] = 0.f;
}
__device__ __forceinline__ float node_features(const float (&g)[kMlpIn], const FeatScale & F, float (&f)[kMlpIn]) {
    const float w  = g[1] * F.inv_sD;
    const float d1 = ((g[3] - g[4]) - g[5]) * w, d2 = g[5] * w, q = g[4] * w;  // p_base = p1 + d1 + d2
    const float sc = sqrtf(fmaf(d1, d1, d2 * d2)) + kMlpScaleEps;
    const float is = 1.f / sc;
    f[0] = g[0] * F.inv_sD;
    f[1] = g[1] * F.inv_alpha0;
    f[2] = g[2] * F.inv_nreal;
    f[3] = d1 * is;
    f[4] = d2 * is;
    f[5] = __logf(sc);
    f[6] = q / (fabsf(q) + sc);
    f[7] = g[6] * F.inv_rho0;
    return sc;
}

// Modes of the forward kernel.
enum { kMlpFromArray = 0, kMlpFromNodes = 1 };

// TMEM columns per CTA: the layer-1 and layer-2 accumulators (N = 64 each) share
// the same 64 columns (layer 2 is issued after every thread has read layer 1
// back), so up to 512 / 64 = 8 CTAs fit the SM's TMEM.
constexpr uint32_t kMlpTmemCols = 64;
constexpr int kMlpMaxCtasPerSm  = 512 / int(kMlpTmemCols);

// params: FP32 vector (layout above); norm: f_mean[kMlpIn], f_std[kMlpIn], t_mean, t_std.
// kMlpFromArray: rows of feat[n][kMlpIn] -> out[n] (prediction t).
// kMlpFromNodes: rows = the slots of the active bricks in brick order (slot
//   blist[r / BN] * BN + r % BN, contiguous within a brick); writes the warm
//   start x[s] = p_base + t s sD / alpha_hat into N.x at active nodes.
//
// Arithmetic: W1, b1, W2, b2 are scaled by 1/2 when staged (exact in bf16 and
// FP32), so the accumulators hold h = z/2 and silu(z) = h + h tanh(h) is one
// tanh and one FMA; bias, SiLU and the final dot run as packed FP32x2 pairs.
// The X tile aliases the first 4 KB of the H1 tile: X is dead once layer 1
// completes, H1 once layer 2 completes.
template<int MODE>
__global__ void __launch_bounds__(kMlpNT, kMlpMaxCtasPerSm)
    k_mlp_forward(long long n, const float * __restrict__ params, const float * __restrict__ norm,
                  const float * __restrict__ feat, float * __restrict__ out, NodeArrays N, const int * __restrict__ blist,
                  const int * __restrict__ bcount, int bn_log2, const int * __restrict__ nv,
                  const double * __restrict__ bb, FeatScale F0, int * __restrict__ err) {
    pdl_wait_and_release();
    __shared__ __align__(1024) uint8_t sw1[kMlpH * 16 * 2];   // W1/2 [64 x 16] bf16 (K padded to 16)
    __shared__ __align__(1024) uint8_t sw2[kMlpH * kMlpH * 2];  // W2/2 [64 x 64]
    __shared__ __align__(1024) uint8_t sh[kMlpNT * kMlpH * 2];  // H1 [128 x 64]; X [128 x 16] in its first 4 KB
    __shared__ float2 sb1[kMlpH / 2], sb2[kMlpH / 2], sw3[kMlpH / 2];  // b1/2, b2/2, w3 as pairs
    __shared__ float snorm[SWC_MLP_NORM];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    __shared__ int s_fail;
    uint8_t * const sx = sh;
    const int tid = threadIdx.x, warp = tid >> 5;

    if (warp == 0) {
        tmem_alloc(&tmem_base, kMlpTmemCols);
        tmem_relinquish();
    }
    if (tid == 0) {
        mbar_init(&mbar, 1);
        s_fail = 0;
    }
    // weights -> bf16 canonical layouts, one 16-byte core-matrix row (8 k) per item
    {
        const int r = tid >> 1, k0 = (tid & 1) * 8;  // W1: 64 rows x 2 chunks = 128 items
        uint32_t pk[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int ka = k0 + 2 * j, kb = ka + 1;
            pk[j] = pack_bf16(ka < kMlpIn ? 0.5f * params[kOffW1 + r * kMlpIn + ka] : 0.f,
                              kb < kMlpIn ? 0.5f * params[kOffW1 + r * kMlpIn + kb] : 0.f);
        }
        *reinterpret_cast<uint4 *>(sw1 + canon_off(r, k0, 16)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
    }
    for (int e = tid; e < kMlpH * (kMlpH / 8); e += kMlpNT) {  // W2: 64 rows x 8 chunks
        const int r = e >> 3, k0 = (e & 7) * 8;
        const float * w = params + kOffW2 + r * kMlpH + k0;
        *reinterpret_cast<uint4 *>(sw2 + canon_off(r, k0, kMlpH)) =
            make_uint4(pack_bf16(0.5f * w[0], 0.5f * w[1]), pack_bf16(0.5f * w[2], 0.5f * w[3]),
                       pack_bf16(0.5f * w[4], 0.5f * w[5]), pack_bf16(0.5f * w[6], 0.5f * w[7]));
    }
    if (tid < kMlpH / 2) {
        sb1[tid] = make_float2(0.5f * params[kOffB1 + 2 * tid], 0.5f * params[kOffB1 + 2 * tid + 1]);
        sb2[tid] = make_float2(0.5f * params[kOffB2 + 2 * tid], 0.5f * params[kOffB2 + 2 * tid + 1]);
        sw3[tid] = make_float2(params[kOffW3 + 2 * tid], params[kOffW3 + 2 * tid + 1]);
    }
    if (tid < SWC_MLP_NORM) snorm[tid] = norm[tid];
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const float b3 = params[kOffB3];
    const uint32_t tacc = tmem_base + (uint32_t(warp * 32) << 16);  // this warp's 32 lanes
    const uint64_t dW1 = smem_desc(smem_u32(sw1), 128, 256), dW2 = smem_desc(smem_u32(sw2), 128, 1024);
    const uint64_t dX = smem_desc(smem_u32(sx), 128, 256), dH = smem_desc(smem_u32(sh), 128, 1024);
    float mean[kMlpIn], inv_std[kMlpIn];
#pragma unroll
    for (int k = 0; k < kMlpIn; k++) {
        mean[k]    = snorm[k];
        inv_std[k] = 1.f / snorm[kMlpIn + k];
    }

    long long rows = n;
    FeatScale F = F0;
    if (MODE == kMlpFromNodes) {
        rows = (long long) *bcount << bn_log2;
        // sD = RMS of the right-hand side over active nodes
        const int na    = *nv;
        const double sD = na > 0 ? sqrt(*bb / double(na)) : 1.0;
        F.inv_sD        = sD > 0 ? float(1.0 / sD) : 0.f;
    }
    uint32_t phase = 0;
    const long long ntiles = (rows + kMlpNT - 1) / kMlpNT;
    // Inputs of a tile row, gathered one tile ahead: the features in array
    // mode; the raw node values of node_raw at the row's slot in node mode
    // (`ga`: the node is active).
    auto gather = [&](long long r, float (&g)[kMlpIn], long long & gs, bool & ga) {
#pragma unroll
        for (int k = 0; k < kMlpIn; k++) g[k] = 0.f;
        gs = 0;
        ga = false;
        if (r >= rows) return;
        if (MODE == kMlpFromArray) {
#pragma unroll
            for (int k = 0; k < kMlpIn; k++) g[k] = feat[r * kMlpIn + k];
            ga = true;
        } else {
            gs = ((long long) blist[r >> bn_log2] << bn_log2) | (r & ((1 << bn_log2) - 1));
            ga = N.flag[gs] != 0;
            node_raw(N, gs, g);
        }
    };
    float gn[kMlpIn];
    long long sn = 0;
    bool an      = false;
    gather(blockIdx.x * (long long) kMlpNT + tid, gn, sn, an);
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const long long row = tile * kMlpNT + tid;
        const bool valid    = an;
        const long long s   = sn;
        const float ah = gn[1], base = gn[3];
        float f[kMlpIn];
        float sc = 1.f;
        if (MODE == kMlpFromNodes) {
            sc = node_features(gn, F, f);
        } else {
#pragma unroll
            for (int k = 0; k < kMlpIn; k++) f[k] = gn[k];
        }
        // X row: normalised features in bf16, K padded to 16
        float xn[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int k = 0; k < kMlpIn; k++) xn[k] = valid ? (f[k] - mean[k]) * inv_std[k] : 0.f;
        *reinterpret_cast<uint4 *>(sx + canon_off(tid, 0, 16)) =
            make_uint4(pack_bf16(xn[0], xn[1]), pack_bf16(xn[2], xn[3]), pack_bf16(xn[4], xn[5]), pack_bf16(xn[6], xn[7]));
        *reinterpret_cast<uint4 *>(sx + canon_off(tid, 8, 16)) = make_uint4(0u, 0u, 0u, 0u);
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
            mma_bf16(tmem_base, dX, dW1, kIdescM128N64, 0u);
            mma_commit(&mbar);
        }
        // the next tile's gathers are in flight while this tile's MMAs run
        gather((tile + gridDim.x) * kMlpNT + tid, gn, sn, an);
        if (!mbar_wait(&mbar, phase)) s_fail = 1;
        phase ^= 1u;
        tc_fence_after();
        // layer-1 epilogue: h = z/2 + b1/2, silu = h + h tanh(h) -> H1 (bf16)
#pragma unroll
        for (int cblk = 0; cblk < 4; cblk++) {
            float z[16];
            tmem_ld16(tacc + uint32_t(cblk * 16), z);
            tmem_ld_wait();
            uint32_t pk[8];
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const int c    = cblk * 8 + i;  // column pair
                const float2 h = add2(make_float2(z[2 * i], z[2 * i + 1]), sb1[c]);
                const float2 a = fma2(h, make_float2(tanh_fast(h.x), tanh_fast(h.y)), h);
                pk[i]          = pack_bf16(a.x, a.y);
            }
            *reinterpret_cast<uint4 *>(sh + canon_off(tid, cblk * 16, kMlpH)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
            *reinterpret_cast<uint4 *>(sh + canon_off(tid, cblk * 16 + 8, kMlpH)) =
                make_uint4(pk[4], pk[5], pk[6], pk[7]);
        }
        // every thread's tcgen05.ld of layer 1 is complete before layer 2 reuses the columns
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
#pragma unroll
            for (int j = 0; j < 4; j++)  // K = 64 in four K = 16 steps (2 core matrices = 256 B each)
                mma_bf16(tmem_base, dH + uint64_t((j * 256) >> 4), dW2 + uint64_t((j * 256) >> 4), kIdescM128N64,
                         j > 0 ? 1u : 0u);
            mma_commit(&mbar);
        }
        if (!mbar_wait(&mbar, phase)) s_fail = 1;
        phase ^= 1u;
        tc_fence_after();
        // layer-2 epilogue: h = z/2 + b2/2, silu, final dot as two packed partial sums
        float2 y2 = make_float2(0.f, 0.f);
#pragma unroll
        for (int cblk = 0; cblk < 4; cblk++) {
            float z[16];
            tmem_ld16(tacc + uint32_t(cblk * 16), z);
            tmem_ld_wait();
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const int c    = cblk * 8 + i;
                const float2 h = add2(make_float2(z[2 * i], z[2 * i + 1]), sb2[c]);
                const float2 a = fma2(h, make_float2(tanh_fast(h.x), tanh_fast(h.y)), h);
                y2             = fma2(sw3[c], a, y2);
            }
        }
        const float t = snorm[2 * kMlpIn] + snorm[2 * kMlpIn + 1] * (b3 + (y2.x + y2.y));
        if (valid) {
            if (MODE == kMlpFromArray) out[row] = t;
            else N.x[s] = base + sc * t / (F.inv_sD * ah);
        }
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (s_fail) break;
    }
    __syncthreads();
    if (s_fail && tid == 0) atomicExch(err, 1);
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem_base, kMlpTmemCols);
    }
}

// ---------------------------------------------------------------------------
// Training (the gradient pass is in k_mlp_train.cu).
// ---------------------------------------------------------------------------
// Adam (Kingma & Ba) with bias correction, FP32 master weights.
__global__ void k_adam(float * __restrict__ p, const float * __restrict__ g, float * __restrict__ m,
                       float * __restrict__ v, int count, float lr, float b1, float b2, float eps, float bc1,
                       float bc2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i]           = mi;
        v[i]           = vi;
        p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    }
}

// Compact index -> slot of every active node (rows of the node-mode forward).
template<int DIM>
__global__ void __launch_bounds__(256) k_slot_of(Lattice L, const int * __restrict__ blist,
                                                 const int * __restrict__ bcount, const int * __restrict__ seg_off,
                                                 const unsigned char * __restrict__ flag, int * __restrict__ slot_of) {
    using G      = BrickGeom<DIM>;
    const int nb = *bcount;
    for (int bi = blockIdx.x; bi < nb; bi += gridDim.x) {
        const int b   = blist[bi];
        const int bx  = b % L.bnx, by = (b / L.bnx) % L.bny, bz = b / (L.bnx * L.bny);
        for (int l = threadIdx.x; l < G::BN; l += 256) {
            const long long s = (long long) b * G::BN + l;
            if (!flag[s]) continue;
            const int lx = l % G::BX, ly = (l / G::BX) % G::BY, lz = l / (G::BX * G::BY);
            const int y = by * G::BY + ly, z = bz * G::BZ + lz;
            long long I = seg_off[((long long) z * L.ny + y) * L.bnx + bx];
            for (int k = 0; k < lx; k++) I += flag[s - lx + k];
            slot_of[I] = int(s);
        }
    }
}

// Target of the learned warm start for logging: (p - p_base) alpha_hat / (sD s),
// with p_base the base start kept in `prev` and s the node's history scale.
__global__ void k_mlp_targets(const int * __restrict__ nv, const int * __restrict__ slot_of,
                              const float * __restrict__ x, const float * __restrict__ prev,
                              const float * __restrict__ xm1, const float * __restrict__ d2p,
                              const float * __restrict__ ahat, const CgState * __restrict__ cg,
                              float * __restrict__ target) {
    const long long rows = *nv;
    const double sD = rows > 0 ? sqrt(cg->bb / double(rows)) : 1.0;
    const float inv = sD > 0 ? float(1.0 / sD) : 0.f;
    for (long long r = blockIdx.x * (long long) blockDim.x + threadIdx.x; r < rows; r += (long long) gridDim.x * blockDim.x) {
        const long long s = slot_of[r];
        const float w     = ahat[s] * inv;
        const float dd = d2p ? d2p[s] : 0.f;
        const float d1 = ((prev[s] - xm1[s]) - dd) * w, d2 = dd * w;
        const float sc    = sqrtf(fmaf(d1, d1, d2 * d2)) + kMlpScaleEps;
        target[r]         = (x[s] - prev[s]) * w / sc;
    }
}

// Features of every active node (training-data logging), x holding p_base.
__global__ void k_node_features(NodeArrays N, const int * __restrict__ slot_of, const int * __restrict__ nv,
                                const CgState * __restrict__ cg, FeatScale F, float * __restrict__ feat_out) {
    const long long rows = *nv;
    const double sD      = rows > 0 ? sqrt(cg->bb / double(rows)) : 1.0;
    F.inv_sD             = sD > 0 ? float(1.0 / sD) : 0.f;
    for (long long r = blockIdx.x * (long long) blockDim.x + threadIdx.x; r < rows; r += (long long) gridDim.x * blockDim.x) {
        float g[kMlpIn], f[kMlpIn];
        node_raw(N, slot_of[r], g);
        node_features(g, F, f);
#pragma unroll
        for (int k = 0; k < kMlpIn; k++) feat_out[r * kMlpIn + k] = f[k];
    }
}

// Batch gather for training: dst[i] = src[idx[i]] (kMlpIn features), dst_t[i] = src_t[idx[i]].
// Pseudo-random permutation of [0, n) for the training epochs: a four-round
// Feistel network on 2 x half bits (Luby-Rackoff; round function a 32-bit integer
// mixer, the "lowbias32" constants of C. Wellons' hash-prospector), walking the
// cycle until the value falls inside [0, n) (at most 4 n / n on average).
__device__ __forceinline__ uint32_t mix32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
__device__ __forceinline__ uint32_t feistel(uint32_t x, int half, uint4 key) {
    const uint32_t mask = (1u << half) - 1u;
    uint32_t l = x >> half, r = x & mask;
    const uint32_t k[4] = {key.x, key.y, key.z, key.w};
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const uint32_t t = l ^ (mix32(r ^ k[i]) & mask);
        l = r;
        r = t;
    }
    return (l << half) | r;
}
__device__ __forceinline__ long long shuffled(long long i, long long n, int half, uint4 key) {
    uint32_t x = uint32_t(i);
    do {
        x = feistel(x, half, key);
    } while (x >= uint32_t(n));
    return x;
}

// Rows b0 .. b0 + nb - 1 of the epoch's permutation of the n dataset rows into
// the batch buffers.
__global__ void k_gather_shuffled(const float * __restrict__ src, const float * __restrict__ src_t, long long n,
                                  long long b0, long long nb, int half, uint4 key, float * __restrict__ dst,
                                  float * __restrict__ dst_t) {
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < nb; i += (long long) gridDim.x * blockDim.x) {
        const long long j = shuffled(b0 + i, n, half, key);
#pragma unroll
        for (int k = 0; k < kMlpIn; k++) dst[i * kMlpIn + k] = src[j * kMlpIn + k];
        dst_t[i] = src_t[j];
    }
}

// Per-block sums of ((pred - target) / t_std)^2 in FP64 (the epoch loss; the host
// adds the block sums in order).
__global__ void __launch_bounds__(256) k_sq_err(const float * __restrict__ pred, const float * __restrict__ tgt,
                                                long long n, float inv_tstd, double * __restrict__ part) {
    __shared__ double sm[256];
    double s = 0;
    for (long long i = blockIdx.x * 256LL + threadIdx.x; i < n; i += gridDim.x * 256LL) {
        const double d = (double(pred[i]) - double(tgt[i])) * double(inv_tstd);
        s += d * d;
    }
    sm[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sm[0];
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
void launch_node_features(const NodeArrays & N, const int * slot_of, const int * nv, long long rows_max,
                          const CgState * cg, float inv_alpha0, float inv_rho0, float inv_nreal, float * feat_out,
                          cudaStream_t st) {
    if (rows_max <= 0) return;
    FeatScale F{0.f, inv_alpha0, inv_rho0, inv_nreal};
    k_node_features<<<int(std::min<long long>((rows_max + 255) / 256, 152 * 8)), 256, 0, st>>>(N, slot_of, nv, cg, F,
                                                                                             feat_out);
}
void launch_gather_shuffled(const float * src, const float * src_t, long long n, long long b0, long long nb, int half,
                            const unsigned * key, float * dst, float * dst_t, cudaStream_t st) {
    if (nb <= 0) return;
    k_gather_shuffled<<<int(std::min<long long>((nb + 255) / 256, 152 * 8)), 256, 0, st>>>(
        src, src_t, n, b0, nb, half, make_uint4(key[0], key[1], key[2], key[3]), dst, dst_t);
}
void launch_sq_err(const float * pred, const float * tgt, long long n, float inv_tstd, double * part, int blocks,
                   cudaStream_t st) {
    k_sq_err<<<blocks, 256, 0, st>>>(pred, tgt, n, inv_tstd, part);
}
// Resident CTAs per SM of a forward instantiation, capped by TMEM (a CTA that
// found its columns taken would wait in tcgen05.alloc).  When shared memory and
// registers alone would allow more, the launch asks for padding dynamic shared
// memory (`dyn`) until the occupancy is within the TMEM cap.
struct MlpLaunch {
    int per_sm = 0;
    size_t dyn = 0;
    int sms    = 152;
};
// Residency is computed from the kernel's registers and shared memory and the
// SM's limits.  The CUDA occupancy calculator is not used: for kernels that
// contain tcgen05.alloc it returns 1 CTA per SM for every block size and
// dynamic shared memory size (measured on GB300 with driver 580; it answers
// normally for the kernels without tensor-memory allocation), while the hardware
// runs the CTAs the registers and shared memory allow (ncu: ~40% of the 64 warps
// active at 4 warps per CTA, i.e. ~6 resident CTAs per SM).  The shape is cached
// per device; host threads share the cache under a lock.
template<int MODE>
static MlpLaunch mlp_launch_shape() {
    static std::mutex mu;
    static MlpLaunch cache[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return MlpLaunch{1, 0};
    std::lock_guard<std::mutex> lock(mu);
    if (cache[dev].per_sm) return cache[dev];
    auto kern = k_mlp_forward<MODE>;
    MlpLaunch s;
    s.per_sm = 1;
    int regs_sm = 65536, smem_sm = 233472, reserved = 1024, threads_sm = 2048, sms = 152;
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, kern) == cudaSuccess) {
        cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
        cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
        cudaDeviceGetAttribute(&threads_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev);
        cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        const int regs_cta = ((fa.numRegs + 7) / 8) * 8 * kMlpNT;
        auto fit           = [&](size_t dyn) {
            const size_t smem_cta = fa.sharedSizeBytes + dyn + size_t(reserved);
            return std::min({regs_sm / std::max(regs_cta, 1), int(size_t(smem_sm) / smem_cta), threads_sm / kMlpNT});
        };
        while (fit(s.dyn) > kMlpMaxCtasPerSm) s.dyn += 1024;  // pad until TMEM cannot be oversubscribed
        s.per_sm = std::max(1, fit(s.dyn));
        if (s.dyn) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(s.dyn));
    }
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) sms = 152;
    s.sms = sms;
    cudaGetLastError();
    cache[dev] = s;
    return s;
}
// Persistent grid: every resident CTA slot once, never more CTAs than tiles.
template<int MODE>
static void launch_forward(long long rows_max, const float * params, const float * norm, const float * feat,
                           float * out, const NodeArrays & N, const int * blist, const int * bcount, int bn_log2,
                           const int * nv, const double * bb, const FeatScale & F, int * err, cudaStream_t st) {
    const MlpLaunch s     = mlp_launch_shape<MODE>();
    const long long tiles = std::max<long long>(1, (rows_max + kMlpNT - 1) / kMlpNT);
    const int grid        = int(std::min<long long>(tiles, (long long) s.per_sm * s.sms));
    launch_pdl(k_mlp_forward<MODE>, grid, kMlpNT, s.dyn, st, rows_max, params, norm, feat, out, N, blist, bcount,
               bn_log2, nv, bb, F, err);
}
void launch_mlp_forward_array(long long n, const float * params, const float * norm, const float * feat, float * out,
                              int * err, cudaStream_t st) {
    if (n <= 0) return;
    launch_forward<kMlpFromArray>(n, params, norm, feat, out, NodeArrays{}, nullptr, nullptr, 0, nullptr, nullptr,
                                  FeatScale{}, err, st);
}
void launch_mlp_forward_nodes(const float * params, const float * norm, const NodeArrays & N, const BrickArrays & B,
                              int bn_log2, long long slots_max, const double * bb, float inv_alpha0, float inv_rho0,
                              float inv_nreal, int * err, cudaStream_t st) {
    FeatScale F{0.f, inv_alpha0, inv_rho0, inv_nreal};
    launch_forward<kMlpFromNodes>(slots_max, params, norm, nullptr, nullptr, N, B.list, B.count, bn_log2,
                                  B.seg_off + B.nseg, bb, F, err, st);
}
void launch_adam(float * p, const float * g, float * m, float * v, int count, float lr, float b1, float b2, float eps,
                 float bc1, float bc2, cudaStream_t st) {
    k_adam<<<(count + 255) / 256, 256, 0, st>>>(p, g, m, v, count, lr, b1, b2, eps, bc1, bc2);
}
template<int DIM>
void launch_slot_of(const Lattice & L, const BrickArrays & B, const NodeArrays & N, int * slot_of, int grid,
                    cudaStream_t st) {
    k_slot_of<DIM><<<grid, 256, 0, st>>>(L, B.list, B.count, B.seg_off, N.flag, slot_of);
}
void launch_mlp_targets(long long rows_max, const int * nv, const int * slot_of, const float * x, const float * prev,
                        const float * xm1, const float * d2p, const float * ahat, const CgState * cg, float * target,
                        cudaStream_t st) {
    if (rows_max <= 0) return;
    k_mlp_targets<<<int(std::min<long long>((rows_max + 255) / 256, 152 * 8)), 256, 0, st>>>(nv, slot_of, x, prev, xm1,
                                                                                           d2p, ahat, cg, target);
}
template void launch_slot_of<2>(const Lattice &, const BrickArrays &, const NodeArrays &, int *, int, cudaStream_t);
template void launch_slot_of<3>(const Lattice &, const BrickArrays &, const NodeArrays &, int *, int, cudaStream_t);

}  // namespace swc
