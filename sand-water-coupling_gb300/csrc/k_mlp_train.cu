// k_mlp_train.cu -- loss gradient of the learned warm-start network on the
// 5th-generation tensor cores (no counterpart in the reference).
//
// One fused pass per 128-row tile, one row per thread, every product a
// tcgen05.mma kind::f16 (BF16 operands in shared memory, FP32 accumulators in
// TMEM) issued by one thread:
//   Z1 = X W1^T                   (M 128, N 64, K 16)    TMEM columns [0, 64)
//   Z2 = H1 W2^T                  (M 128, N 64, K 64)    TMEM columns [64, 128)
//   dZ1' = dZ2 W2                 (M 128, N 64, K 64)    TMEM columns [64, 128)
//   D += [dZ2^T; dZ1^T] [H1 | X | 1]^T   (M 128, N 80, K = the tile's 128 rows)
//                                                        TMEM columns [128, 208)
// with the per-row epilogues on the CUDA cores in FP32:
//   h1 = silu(z1), y = w3 . silu(z2) + b3, e = y - (t - t_mean) / t_std,
//   dy = 2 e / n, dz2 = dy w3 silu'(z2), dz1 = dz1' silu'(z1).
// D accumulates over every tile a CTA takes, so after the last tile it holds the
// CTA's share of dW2 = dZ2^T H1 (rows 0-63, columns 0-63), dW1 = dZ1^T X (rows
// 64-127, columns 64-71) and the bias gradients db2, db1 (column 72, the ones
// column).  dw3 = sum_r dy h2 and db3 = sum_r dy are summed in FP32 on the CUDA
// cores (a transposing warp reduction).  The per-CTA shares are added in a
// fixed order by a second kernel, so the gradient is deterministic.
//
// Operands for the weight-gradient product have the batch rows as their K
// dimension: each thread writes its row's dz2, dz1, h1 and x into the K-major
// layouts of [dZ2^T; dZ1^T] and [H1 | X | 1]^T (2-byte stores).
//
// BF16 rounding points (an emulating oracle reproduces them): x, W1 and W2
// (W1 and W2 staged at 1/2, exact), h1, dz2 (for both dZ1' and dW2), dz1.
// Every wait on the tensor core is bounded; on timeout the kernel records an
// error, stops, frees its TMEM and the reduction writes NaN.
#include <algorithm>
#include <cstdio>
#include <mutex>

#include "swc_tc.cuh"

namespace swc {

constexpr int kTrNT             = 128;  // threads = rows per tile
constexpr int kTrN              = 80;   // N of the weight-gradient product: h1 (64), x (8), ones (1), zeros (7)
constexpr int kTrOnes           = 72;   // the ones column
constexpr uint32_t kTrTmemCols  = 256;  // Z1 [0, 64) | Z2, dZ1' [64, 128) | D [128, 208)
constexpr uint32_t kColZ1 = 0, kColZ2 = 64, kColD = 128;
constexpr int kTrCtasPerSm      = 512 / int(kTrTmemCols);
// per-CTA share: D (128 x 80), dw3 (64), db3, loss sum
constexpr int kTrShare = 128 * kTrN + kMlpH + 2;
static_assert(kTrShare == kMlpTrainShare, "share layout");

struct TrainSmem {
    uint8_t w1[kMlpH * 16 * 2];     // W1 / 2 [64 x 16] (K padded to 16)
    uint8_t w2[kMlpH * kMlpH * 2];  // W2 / 2 [64 x 64]
    uint8_t w2t[kMlpH * kMlpH * 2]; // W2^T [64 x 64]
    uint8_t x[kTrNT * 16 * 2];      // X [128 x 16]
    uint8_t h[kTrNT * kMlpH * 2];   // H1 [128 x 64], then dZ2 [128 x 64]
    uint8_t a[128 * kTrNT * 2];     // [dZ2^T; dZ1^T] [128 x 128 rows]
    uint8_t b[kTrN * kTrNT * 2];    // [H1 | X | 1 | 0]^T [80 x 128 rows]
};
constexpr size_t kTrSmem = sizeof(TrainSmem);

__device__ __forceinline__ void st_bf16(uint8_t * base, uint32_t off, float v) {
    *reinterpret_cast<__nv_bfloat16 *>(base + off) = __float2bfloat16_rn(v);
}

// Sum over the warp's 32 lanes of v[0..15] (each lane's own 16 values): after
// the call lane L holds the sum of index L >> 1 (lanes 2k and 2k + 1 agree).
__device__ __forceinline__ float warp_transpose_sum16(float (&v)[16]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int half = 8; half >= 1; half >>= 1) {
        const int off = half * 2;  // partner lane distance: 16, 8, 4, 2
        const bool up = (lane & off) != 0;
#pragma unroll
        for (int i = 0; i < half; i++) {
            const float keep = up ? v[i + half] : v[i];
            const float send = up ? v[i] : v[i + half];
            v[i]             = keep + __shfl_xor_sync(0xffffffffu, send, off);
        }
    }
    return v[0] + __shfl_xor_sync(0xffffffffu, v[0], 1);
}

__global__ void __launch_bounds__(kTrNT, kTrCtasPerSm)
    k_mlp_train_grad(long long n, const float * __restrict__ params, const float * __restrict__ norm,
                     const float * __restrict__ feat, const float * __restrict__ target, float * __restrict__ share,
                     int * __restrict__ err) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    TrainSmem & S = *reinterpret_cast<TrainSmem *>(smem_raw);
    __shared__ float2 sb1[kMlpH / 2], sb2[kMlpH / 2], sw3[kMlpH / 2];  // b1 / 2, b2 / 2, w3
    __shared__ float snorm[SWC_MLP_NORM];
    __shared__ float sred[kTrNT / 32][kMlpH];
    __shared__ float sred2[kTrNT / 32][2];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    __shared__ int s_fail;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (warp == 0) {
        tmem_alloc(&tmem_base, kTrTmemCols);
        tmem_relinquish();
    }
    if (tid == 0) {
        mbar_init(&mbar, 1);
        s_fail = 0;
    }
    // weights in the K-major canonical layouts (one 16-byte core-matrix row per item)
    {
        const int r = tid >> 1, k0 = (tid & 1) * 8;  // W1: 64 rows x 2 chunks
        uint32_t pk[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int ka = k0 + 2 * j, kb = ka + 1;
            pk[j] = pack_bf16(ka < kMlpIn ? 0.5f * params[kOffW1 + r * kMlpIn + ka] : 0.f,
                              kb < kMlpIn ? 0.5f * params[kOffW1 + r * kMlpIn + kb] : 0.f);
        }
        *reinterpret_cast<uint4 *>(S.w1 + canon_off(r, k0, 16)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
    }
    for (int e = tid; e < kMlpH * (kMlpH / 8); e += kTrNT) {
        const int r = e >> 3, k0 = (e & 7) * 8;
        const float * w = params + kOffW2 + r * kMlpH + k0;  // W2 row r (output unit), inputs k0..k0+7
        *reinterpret_cast<uint4 *>(S.w2 + canon_off(r, k0, kMlpH)) =
            make_uint4(pack_bf16(0.5f * w[0], 0.5f * w[1]), pack_bf16(0.5f * w[2], 0.5f * w[3]),
                       pack_bf16(0.5f * w[4], 0.5f * w[5]), pack_bf16(0.5f * w[6], 0.5f * w[7]));
        // W2^T row r = input unit r, K = output units k0..k0+7
        const float * c = params + kOffW2 + k0 * kMlpH + r;
        *reinterpret_cast<uint4 *>(S.w2t + canon_off(r, k0, kMlpH)) =
            make_uint4(pack_bf16(c[0], c[kMlpH]), pack_bf16(c[2 * kMlpH], c[3 * kMlpH]),
                       pack_bf16(c[4 * kMlpH], c[5 * kMlpH]), pack_bf16(c[6 * kMlpH], c[7 * kMlpH]));
    }
    // the constant rows of [H1 | X | 1 | 0]^T: ones (row 72) and zeros (rows 73-79)
    for (int e = tid; e < (kTrN - kTrOnes) * (kTrNT / 8); e += kTrNT) {
        const int r = kTrOnes + e / (kTrNT / 8), k0 = (e % (kTrNT / 8)) * 8;
        const uint32_t one = r == kTrOnes ? pack_bf16(1.f, 1.f) : 0u;
        *reinterpret_cast<uint4 *>(S.b + canon_off(r, k0, kTrNT)) = make_uint4(one, one, one, one);
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
    const uint32_t tlane = tmem_base + (uint32_t(warp * 32) << 16);  // this warp's 32 lanes
    const uint64_t dW1 = smem_desc(smem_u32(S.w1), 128, 256), dW2 = smem_desc(smem_u32(S.w2), 128, 1024);
    const uint64_t dW2t = smem_desc(smem_u32(S.w2t), 128, 1024);
    const uint64_t dX = smem_desc(smem_u32(S.x), 128, 256), dH = smem_desc(smem_u32(S.h), 128, 1024);
    const uint64_t dA = smem_desc(smem_u32(S.a), 128, 2048), dB = smem_desc(smem_u32(S.b), 128, 2048);
    const uint32_t idN64 = idesc_m128(64), idN80 = idesc_m128(kTrN);
    float mean[kMlpIn], inv_std[kMlpIn];
#pragma unroll
    for (int k = 0; k < kMlpIn; k++) {
        mean[k]    = snorm[k];
        inv_std[k] = 1.f / snorm[kMlpIn + k];
    }
    const float tm = snorm[2 * kMlpIn], its = 1.f / snorm[2 * kMlpIn + 1];
    const float inv_n = 1.f / float(n);

    float dw3[4] = {0.f, 0.f, 0.f, 0.f};  // lane's share: dw3[c * 16 + lane / 2]
    float db3 = 0.f, sq = 0.f;
    uint32_t phase = 0;
    bool pending = false;  // a weight-gradient product is in flight
    int ntile = 0;
    auto wait = [&]() {
        if (!mbar_wait(&mbar, phase)) s_fail = 1;
        phase ^= 1u;
        tc_fence_after();
    };
    auto sync_for_mma = [&]() {
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
    };
    const long long ntiles = (n + kTrNT - 1) / kTrNT;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ntile++) {
        const long long row = tile * kTrNT + tid;
        const bool valid    = row < n;
        float f[kMlpIn];
#pragma unroll
        for (int k = 0; k < kMlpIn; k++) f[k] = valid ? feat[row * kMlpIn + k] : 0.f;
        const float ty = valid ? (target[row] - tm) * its : 0.f;
        if (pending) wait();  // the previous tile's weight-gradient product has read a / b / h
        // X row (normalised, bf16, K padded to 16) and the X rows of [H1 | X | 1]^T
        float xn[8];
#pragma unroll
        for (int k = 0; k < 8; k++) xn[k] = (k < kMlpIn && valid) ? (f[k] - mean[k]) * inv_std[k] : 0.f;
        *reinterpret_cast<uint4 *>(S.x + canon_off(tid, 0, 16)) =
            make_uint4(pack_bf16(xn[0], xn[1]), pack_bf16(xn[2], xn[3]), pack_bf16(xn[4], xn[5]), pack_bf16(xn[6], xn[7]));
        *reinterpret_cast<uint4 *>(S.x + canon_off(tid, 8, 16)) = make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
        for (int k = 0; k < kMlpIn; k++) st_bf16(S.b, canon_off(kMlpH + k, tid, kTrNT), xn[k]);
        st_bf16(S.b, canon_off(kTrOnes, tid, kTrNT), valid ? 1.f : 0.f);  // rows past n add nothing to the biases
        sync_for_mma();
        if (s_fail) break;
        if (tid == 0) {
            mma_bf16(tmem_base + kColZ1, dX, dW1, idN64, 0u);
            mma_commit(&mbar);
        }
        wait();
        // layer 1: h = z1 / 2 + b1 / 2, h1 = silu(z1) = h + h tanh(h) -> H1 and the H1 rows of [H1 | X | 1]^T
#pragma unroll
        for (int cblk = 0; cblk < 4; cblk++) {
            float z[16];
            tmem_ld16(tlane + kColZ1 + uint32_t(cblk * 16), z);
            tmem_ld_wait();
            uint32_t pk[8];
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const int c    = cblk * 8 + i;
                const float2 h = add2(make_float2(z[2 * i], z[2 * i + 1]), sb1[c]);
                const float2 a = fma2(h, make_float2(tanh_fast(h.x), tanh_fast(h.y)), h);
                pk[i]          = valid ? pack_bf16(a.x, a.y) : 0u;
                *reinterpret_cast<__nv_bfloat16 *>(S.b + canon_off(2 * c, tid, kTrNT)) =
                    reinterpret_cast<const __nv_bfloat162 *>(&pk[i])->x;
                *reinterpret_cast<__nv_bfloat16 *>(S.b + canon_off(2 * c + 1, tid, kTrNT)) =
                    reinterpret_cast<const __nv_bfloat162 *>(&pk[i])->y;
            }
            *reinterpret_cast<uint4 *>(S.h + canon_off(tid, cblk * 16, kMlpH)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
            *reinterpret_cast<uint4 *>(S.h + canon_off(tid, cblk * 16 + 8, kMlpH)) =
                make_uint4(pk[4], pk[5], pk[6], pk[7]);
        }
        sync_for_mma();
        if (tid == 0) {
#pragma unroll
            for (int j = 0; j < 4; j++)
                mma_bf16(tmem_base + kColZ2, dH + uint64_t((j * 256) >> 4), dW2 + uint64_t((j * 256) >> 4), idN64,
                         j > 0 ? 1u : 0u);
            mma_commit(&mbar);
        }
        wait();
        // layer 2 and the loss: y = w3 . silu(z2) + b3, dy = 2 (y - ty) / n
        float2 y2 = make_float2(0.f, 0.f);
#pragma unroll
        for (int cblk = 0; cblk < 4; cblk++) {
            float z[16];
            tmem_ld16(tlane + kColZ2 + uint32_t(cblk * 16), z);
            tmem_ld_wait();
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const int c    = cblk * 8 + i;
                const float2 h = add2(make_float2(z[2 * i], z[2 * i + 1]), sb2[c]);
                const float2 a = fma2(h, make_float2(tanh_fast(h.x), tanh_fast(h.y)), h);
                y2             = fma2(sw3[c], a, y2);
            }
        }
        const float e  = valid ? (b3 + (y2.x + y2.y)) - ty : 0.f;
        const float dy = 2.f * e * inv_n;
        sq             = fmaf(e, e, sq);
        db3 += dy;
        // dz2 = dy w3 silu'(z2) -> dZ2 (over H1, whose product is done) and the dZ2^T rows of
        // the weight-gradient operand; dw3 += dy silu(z2) through the warp reduction
#pragma unroll
        for (int cblk = 0; cblk < 4; cblk++) {
            float z[16];
            tmem_ld16(tlane + kColZ2 + uint32_t(cblk * 16), z);
            tmem_ld_wait();
            float hv[16];
            uint32_t pk[8];
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const int c    = cblk * 8 + i;
                const float2 h = add2(make_float2(z[2 * i], z[2 * i + 1]), sb2[c]);
                // sigma(z) = (1 + tanh(z / 2)) / 2, silu = 2 h sigma, silu' = sigma (1 + 2 h (1 - sigma))
                const float2 s  = fma2(make_float2(tanh_fast(h.x), tanh_fast(h.y)), f2(0.5f), f2(0.5f));
                const float2 sl = mul2(add2(h, h), s);
                const float2 ds = mul2(s, fma2(add2(h, h), add2(f2(1.f), make_float2(-s.x, -s.y)), f2(1.f)));
                const float2 g  = mul2(mul2(f2(dy), sw3[c]), ds);
                hv[2 * i]       = dy * sl.x;
                hv[2 * i + 1]   = dy * sl.y;
                pk[i]           = pack_bf16(g.x, g.y);
                const __nv_bfloat162 gb = *reinterpret_cast<const __nv_bfloat162 *>(&pk[i]);
                *reinterpret_cast<__nv_bfloat16 *>(S.a + canon_off(2 * c, tid, kTrNT))     = gb.x;
                *reinterpret_cast<__nv_bfloat16 *>(S.a + canon_off(2 * c + 1, tid, kTrNT)) = gb.y;
            }
            *reinterpret_cast<uint4 *>(S.h + canon_off(tid, cblk * 16, kMlpH)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
            *reinterpret_cast<uint4 *>(S.h + canon_off(tid, cblk * 16 + 8, kMlpH)) =
                make_uint4(pk[4], pk[5], pk[6], pk[7]);
            dw3[cblk] += warp_transpose_sum16(hv);
        }
        sync_for_mma();
        if (tid == 0) {
#pragma unroll
            for (int j = 0; j < 4; j++)
                mma_bf16(tmem_base + kColZ2, dH + uint64_t((j * 256) >> 4), dW2t + uint64_t((j * 256) >> 4), idN64,
                         j > 0 ? 1u : 0u);
            mma_commit(&mbar);
        }
        wait();
        // dz1 = dz1' silu'(z1) -> the dZ1^T rows of the weight-gradient operand
#pragma unroll
        for (int cblk = 0; cblk < 4; cblk++) {
            float d[16], z[16];
            tmem_ld16(tlane + kColZ2 + uint32_t(cblk * 16), d);
            tmem_ld16(tlane + kColZ1 + uint32_t(cblk * 16), z);
            tmem_ld_wait();
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const int c     = cblk * 8 + i;
                const float2 h  = add2(make_float2(z[2 * i], z[2 * i + 1]), sb1[c]);
                const float2 s  = fma2(make_float2(tanh_fast(h.x), tanh_fast(h.y)), f2(0.5f), f2(0.5f));
                const float2 ds = mul2(s, fma2(add2(h, h), add2(f2(1.f), make_float2(-s.x, -s.y)), f2(1.f)));
                const float2 g  = mul2(make_float2(d[2 * i], d[2 * i + 1]), ds);
                st_bf16(S.a, canon_off(kMlpH + 2 * c, tid, kTrNT), g.x);
                st_bf16(S.a, canon_off(kMlpH + 2 * c + 1, tid, kTrNT), g.y);
            }
        }
        sync_for_mma();
        if (tid == 0) {
#pragma unroll
            for (int kk = 0; kk < kTrNT / 16; kk++)
                mma_bf16(tmem_base + kColD, dA + uint64_t((kk * 256) >> 4), dB + uint64_t((kk * 256) >> 4), idN80,
                         (ntile > 0 || kk > 0) ? 1u : 0u);
            mma_commit(&mbar);
        }
        pending = true;
    }
    if (pending) wait();
    __syncthreads();
    // the CTA's share: D rows (lane m = tid) and the FP32 sums
    float * out = share + (long long) blockIdx.x * kTrShare;
    const bool any = ntile > 0 && !s_fail;
#pragma unroll
    for (int cblk = 0; cblk < kTrN / 16; cblk++) {
        float dv[16];
        tmem_ld16(tlane + kColD + uint32_t(cblk * 16), dv);
        tmem_ld_wait();
#pragma unroll
        for (int i = 0; i < 16; i++) out[tid * kTrN + cblk * 16 + i] = any ? dv[i] : 0.f;
    }
    if ((lane & 1) == 0) {
#pragma unroll
        for (int c = 0; c < 4; c++) sred[warp][c * 16 + (lane >> 1)] = dw3[c];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        db3 += __shfl_xor_sync(0xffffffffu, db3, o);
        sq += __shfl_xor_sync(0xffffffffu, sq, o);
    }
    if (lane == 0) sred2[warp][0] = db3, sred2[warp][1] = sq;
    __syncthreads();
    if (tid < kMlpH) {
        float s = 0.f;
#pragma unroll
        for (int w = 0; w < kTrNT / 32; w++) s += sred[w][tid];
        out[128 * kTrN + tid] = s;
    }
    if (tid == 0) {
        float a = 0.f, b = 0.f;
        for (int w = 0; w < kTrNT / 32; w++) a += sred2[w][0], b += sred2[w][1];
        out[128 * kTrN + kMlpH]     = a;
        out[128 * kTrN + kMlpH + 1] = b;
        if (s_fail) atomicExch(err, 1);
    }
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem_base, kTrTmemCols);
    }
}

// Sum of the CTA shares in CTA order, scattered into the parameter layout; the
// loss (mean squared error) into *loss.  NaN everywhere when a CTA failed.
__global__ void __launch_bounds__(256) k_mlp_train_reduce(int nshare, long long n, const float * __restrict__ share,
                                                          const int * __restrict__ err, float * __restrict__ grad,
                                                          float * __restrict__ loss) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= kTrShare) return;
    float s = 0.f;
    for (int k = 0; k < nshare; k++) s += share[(long long) k * kTrShare + e];
    if (*err) s = __int_as_float(0x7fc00000);
    if (e < 128 * kTrN) {
        const int m = e / kTrN, c = e % kTrN;
        if (m < kMlpH && c < kMlpH) grad[kOffW2 + m * kMlpH + c] = s;                          // dW2[j][i]
        else if (m >= kMlpH && c >= kMlpH && c < kMlpH + kMlpIn) grad[kOffW1 + (m - kMlpH) * kMlpIn + (c - kMlpH)] = s;
        else if (c == kTrOnes) grad[(m < kMlpH ? kOffB2 + m : kOffB1 + m - kMlpH)] = s;        // db2 / db1
    } else if (e < 128 * kTrN + kMlpH) {
        grad[kOffW3 + (e - 128 * kTrN)] = s;
    } else if (e == 128 * kTrN + kMlpH) {
        grad[kOffB3] = s;
    } else {
        *loss = s / float(n);
    }
}

int mlp_train_ctas(long long n) {
    static const int sms = [] {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        return cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0 ? v : 152;
    }();
    const long long tiles = std::max<long long>(1, (n + kTrNT - 1) / kTrNT);
    return int(std::min<long long>(tiles, (long long) sms * kTrCtasPerSm));
}
size_t mlp_train_share_floats(int ctas) { return size_t(ctas) * kTrShare; }

int launch_mlp_train_grad(long long n, const float * params, const float * norm, const float * feat,
                          const float * target, float * share, int ctas, int * err, float * grad, float * loss,
                          cudaStream_t st) {
    if (n <= 0 || ctas <= 0) return -1;
    // the 90 KB of dynamic shared memory need the opt-in (a function attribute, set
    // per device on its first use; the cache is shared by host threads)
    static std::mutex mu;
    static bool attr_set[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -1;
    {
        std::lock_guard<std::mutex> lock(mu);
        if (!attr_set[dev]) {
            if (cudaFuncSetAttribute(k_mlp_train_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTrSmem)) !=
                cudaSuccess)
                return -1;
            attr_set[dev] = true;
        }
    }
    k_mlp_train_grad<<<ctas, kTrNT, kTrSmem, st>>>(n, params, norm, feat, target, share, err);
    k_mlp_train_reduce<<<(kTrShare + 255) / 256, 256, 0, st>>>(ctas, n, share, err, grad, loss);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace swc
