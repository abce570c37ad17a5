// swc_noalloc.cu -- loss gradient of the learned warm-start network for callers
// that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc at the point where they need a gradient:
// a training loop whose device memory is planned up front by its host framework
// (fixed arenas, no allocator calls between steps), code running under a memory
// budget that a late allocation could exceed, or a plugin that must not change
// the process's allocation pattern.  swc_mlp_gradient allocates its scratch on
// every call; swc_mlp_gradient_noalloc keeps the same scratch (the per-CTA
// gradient shares of the tensor-core pass and an error flag) in file-scope
// device arrays sized for SWC_MLP_NOALLOC_MAX_ROWS rows, and only launches
// kernels.
//
// The arrays exist once per device that loads this library and live until the
// process exits (about 0.7 MB).  Every call reuses them and they keep the last
// call's contents; the shares are overwritten in full by each call and only the
// error flag needs to start at zero, which each call clears.  Calls that overlap
// on the GPU (different streams, or the same arrays used by two host threads at
// once) race on the scratch.  The device addresses of the arrays are looked up
// once per device; they do not survive a cudaDeviceReset of that device.
#include <algorithm>
#include <mutex>

#include "../../include/swc.h"
#include "swc_kernels.h"

namespace swc {

namespace {

constexpr int kRows  = SWC_MLP_NOALLOC_MAX_ROWS;
constexpr int kShare = ((kRows + 127) / 128) * kMlpTrainShare;  // one share per 128-row tile at most

// Scratch of one gradient evaluation (device memory, never allocated at run time).
static __device__ __align__(256) float g_share[kShare];
static __device__ __align__(256) int g_err;

struct ScratchPtrs {
    float * share;
    int *   err;
};

constexpr int kMaxDevices = 64;
ScratchPtrs g_ptrs[kMaxDevices];
bool        g_ready[kMaxDevices];
std::mutex  g_mutex;

// Device addresses of the scratch arrays on the current device (resolved once
// per device; host code sees only host-side stand-ins for the symbols).
int scratch_for_current_device(ScratchPtrs & out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return SWC_CUDA_ERROR;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_ready[dev]) {
        ScratchPtrs p{};
        if (cudaGetSymbolAddress(reinterpret_cast<void **>(&p.share), g_share) != cudaSuccess ||
            cudaGetSymbolAddress(reinterpret_cast<void **>(&p.err), g_err) != cudaSuccess)
            return SWC_CUDA_ERROR;
        g_ptrs[dev]  = p;
        g_ready[dev] = true;
    }
    out = g_ptrs[dev];
    return SWC_OK;
}

}  // namespace
}  // namespace swc

using namespace swc;

extern "C" int swc_mlp_gradient_noalloc(const float * d_params, const float * d_norm, const float * d_features,
                                        const float * d_targets, int64_t n, float * d_grad, float * d_loss,
                                        void * stream) {
    if (!d_params || !d_norm || !d_features || !d_targets || !d_grad || !d_loss) return SWC_BAD_ARG;
    if (n <= 0 || n > SWC_MLP_NOALLOC_MAX_ROWS) return SWC_BAD_ARG;  // batch above the fixed scratch size
    ScratchPtrs s{};
    int rc = scratch_for_current_device(s);
    if (rc) return rc;
    const int ctas = mlp_train_ctas(n);
    if (mlp_train_share_floats(ctas) > size_t(kShare)) return SWC_BAD_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(s.err, 0, sizeof(int), st) != cudaSuccess) return SWC_CUDA_ERROR;
    return launch_mlp_train_grad(n, d_params, d_norm, d_features, d_targets, s.share, ctas, s.err, d_grad, d_loss, st)
               ? SWC_CUDA_ERROR
               : SWC_OK;
}
