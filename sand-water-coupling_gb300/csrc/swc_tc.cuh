// swc_tc.cuh -- 5th-generation tensor-core helpers of the learned warm-start
// network (forward in k_mlp.cu, training gradient in k_mlp_train.cu): inline PTX
// for TMEM allocation, tcgen05.mma kind::f16 (BF16 operands, FP32 accumulators)
// issued by one thread, mbarrier completion with bounded waits, tcgen05.ld of
// the accumulators, shared-memory matrix descriptors of the K-major no-swizzle
// canonical layout, the SiLU helpers and the parameter layout of the network.
#pragma once

#include <cuda_bf16.h>

#include "../../include/swc.h"
#include "swc_kernels.h"

namespace swc {

// ---------------------------------------------------------------------------
// PTX helpers (tcgen05 / TMEM / mbarrier).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void * p) { return uint32_t(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void tmem_alloc(uint32_t * dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// D (TMEM) = A * B (+ D when accumulate), A/B described in shared memory.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t * mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
                 : "memory");
}
__device__ __forceinline__ void mbar_init(uint64_t * mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t * mbar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(mbar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t * mbar, uint32_t parity) {
    for (int i = 0; i < (1 << 22); i++)
        if (mbar_try_wait(mbar, parity)) return true;
    return false;
}

// 16 consecutive FP32 columns of this thread's TMEM lane (warp w reads lanes 32w..32w+31).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major, no swizzle; LBO = byte step between
// core matrices along K, SBO = byte step between 8-row groups.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return uint64_t((saddr & 0x3FFFFu) >> 4) | (uint64_t(lbo >> 4) << 16) | (uint64_t(sbo >> 4) << 32) |
           (uint64_t(1) << 46);
}
// Instruction descriptor, kind::f16: BF16 A and B (K-major), FP32 accumulate, M = 128, N = 64.
constexpr uint32_t kIdescM128N64 = (1u << 4) | (1u << 7) | (1u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

// Byte offset of element (r, k) of a K-major bf16 matrix with `kdim` columns.
__device__ __forceinline__ uint32_t canon_off(int r, int k, int kdim) {
    return uint32_t((r >> 3) * (kdim / 8) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// sigma(z) = (1 + tanh(z/2)) / 2 with the hardware tanh approximation (relative
// error about 2^-11, below the bf16 rounding the activations go through);
// silu(z) = z sigma(z), silu'(z) = sigma(z) (1 + z (1 - sigma(z))).
__device__ __forceinline__ float sigmoid_fast(float z) {
    float t;
    asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(0.5f * z));
    return fmaf(0.5f, t, 0.5f);
}
__device__ __forceinline__ float silu(float z) { return z * sigmoid_fast(z); }
__device__ __forceinline__ float dsilu(float z) {
    const float s = sigmoid_fast(z);
    return s * (1.f + z * (1.f - s));
}
__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&v);
}

// Instruction descriptor, kind::f16: BF16 A and B (K-major), FP32 accumulate, M = 128, N (multiple of 16).
constexpr uint32_t idesc_m128(uint32_t n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((128u >> 4) << 24);
}

constexpr int kMlpIn = SWC_MLP_IN, kMlpH = 64;
constexpr int kMlpParams = kMlpH * kMlpIn + kMlpH + kMlpH * kMlpH + kMlpH + kMlpH + 1;
static_assert(kMlpParams == SWC_MLP_PARAMS && 2 * kMlpIn + 2 == SWC_MLP_NORM, "MLP layout");
static_assert(kMlpIn <= 8, "the X row holds the features in its first 16-byte core-matrix row");
constexpr int kOffW1 = 0, kOffB1 = kOffW1 + kMlpH * kMlpIn, kOffW2 = kOffB1 + kMlpH, kOffB2 = kOffW2 + kMlpH * kMlpH,
              kOffW3 = kOffB2 + kMlpH, kOffB3 = kOffW3 + kMlpH;
constexpr int kMlpNT = 128;  // threads = rows per tile

// tanh with the hardware approximation (relative error about 2^-11).
__device__ __forceinline__ float tanh_fast(float h) {
    float t;
    asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(h));
    return t;
}

}  // namespace swc
