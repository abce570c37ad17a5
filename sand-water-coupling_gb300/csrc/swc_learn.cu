// swc_learn.cu -- device-side training of the learned CG warm start and the
// stateless forward / gradient helpers of the C ABI (include/swc.h).  The
// dataset stays in device memory; every batch runs the fused tensor-core
// gradient pass (k_mlp_train.cu: forward, backward and weight gradients as
// tcgen05 BF16 products with FP32 accumulation) and an Adam step.
#include <algorithm>
#include <cstring>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/swc.h"
#include "swc_kernels.h"

using namespace swc;

namespace {
constexpr int kP = SWC_MLP_PARAMS, kN = SWC_MLP_NORM, kIn = SWC_MLP_IN;
constexpr int kLossBlocks = 512;  // block sums of the epoch loss
}

struct swc_trainer {
    long long    cap = 0, n = 0;
    int          batch = 4096;
    cudaStream_t st = nullptr;
    float *feat = nullptr, *tgt = nullptr;                       // dataset
    float *params = nullptr, *norm = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr;
    float *bfeat = nullptr, *btgt = nullptr, *pred = nullptr;    // batch
    float * fpred = nullptr;                                     // predictions of the whole dataset (epoch loss)
    double * part = nullptr;                                     // block sums of the epoch loss
    float *share = nullptr, *loss = nullptr;                     // per-CTA gradient shares, batch loss
    int    ctas  = 1;
    int *  err = nullptr;
    long long adam_t = 0;
};

namespace {

template<class T> bool talloc(T ** p, size_t count) {
    return cudaMalloc(reinterpret_cast<void **>(p), sizeof(T) * std::max<size_t>(count, 1)) == cudaSuccess;
}
template<class T> void tfree(T *& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

int forward_batch(swc_trainer * t, const float * feat, long long n, float * out) {
    launch_mlp_forward_array(n, t->params, t->norm, feat, out, t->err, t->st);
    return cudaGetLastError() == cudaSuccess ? SWC_OK : SWC_CUDA_ERROR;
}
// loss gradient of one batch (features / targets on the device) into t->grad, t->loss
int gradient_batch(swc_trainer * t, const float * feat, const float * tgt, long long n) {
    return launch_mlp_train_grad(n, t->params, t->norm, feat, tgt, t->share, t->ctas, t->err, t->grad, t->loss, t->st)
               ? SWC_CUDA_ERROR
               : SWC_OK;
}

int check_err(swc_trainer * t) {
    int e = 0;
    if (cudaMemcpyAsync(&e, t->err, sizeof(int), cudaMemcpyDeviceToHost, t->st) != cudaSuccess) return SWC_CUDA_ERROR;
    if (cudaStreamSynchronize(t->st) != cudaSuccess) return SWC_CUDA_ERROR;
    return e ? SWC_CUDA_ERROR : SWC_OK;
}

}  // namespace

extern "C" {

int swc_trainer_create(int64_t capacity, int32_t batch, swc_trainer ** out) {
    if (!out || capacity <= 0 || batch <= 0) return SWC_BAD_ARG;
    *out   = nullptr;
    auto t = new swc_trainer();
    t->cap   = capacity;
    t->batch = batch;
    const size_t B = size_t(batch);
    t->ctas = mlp_train_ctas(batch);
    bool ok = cudaStreamCreateWithFlags(&t->st, cudaStreamNonBlocking) == cudaSuccess;
    ok = ok && talloc(&t->feat, size_t(capacity) * kIn) && talloc(&t->tgt, size_t(capacity)) && talloc(&t->params, kP) &&
         talloc(&t->norm, kN) && talloc(&t->m, kP) && talloc(&t->v, kP) && talloc(&t->grad, kP) &&
         talloc(&t->bfeat, B * kIn) && talloc(&t->btgt, B) && talloc(&t->pred, B) &&
         talloc(&t->share, mlp_train_share_floats(t->ctas)) && talloc(&t->loss, 1) &&
         talloc(&t->part, kLossBlocks) && talloc(&t->err, 1);
    if (!ok) {
        swc_trainer_destroy(t);
        return SWC_OUT_OF_MEMORY;
    }
    cudaMemsetAsync(t->m, 0, sizeof(float) * kP, t->st);
    cudaMemsetAsync(t->v, 0, sizeof(float) * kP, t->st);
    cudaMemsetAsync(t->err, 0, sizeof(int), t->st);
    cudaStreamSynchronize(t->st);
    *out = t;
    return SWC_OK;
}

void swc_trainer_destroy(swc_trainer * t) {
    if (!t) return;
    if (t->st) cudaStreamSynchronize(t->st);
    for (float ** p : {&t->feat, &t->tgt, &t->params, &t->norm, &t->m, &t->v, &t->grad, &t->bfeat, &t->btgt, &t->pred,
                       &t->fpred, &t->share, &t->loss})
        tfree(*p);
    tfree(t->part);
    tfree(t->err);
    if (t->st) cudaStreamDestroy(t->st);
    delete t;
}

int swc_trainer_add(swc_trainer * t, const float * f, const float * y, int64_t n) {
    if (!t || n < 0 || (n > 0 && (!f || !y))) return SWC_BAD_ARG;
    if (t->n + n > t->cap) return SWC_BAD_ARG;
    if (cudaMemcpyAsync(t->feat + t->n * kIn, f, sizeof(float) * kIn * n, cudaMemcpyHostToDevice, t->st) != cudaSuccess ||
        cudaMemcpyAsync(t->tgt + t->n, y, sizeof(float) * n, cudaMemcpyHostToDevice, t->st) != cudaSuccess)
        return SWC_CUDA_ERROR;
    cudaStreamSynchronize(t->st);
    t->n += n;
    return SWC_OK;
}

int swc_trainer_set_params(swc_trainer * t, const float * params, const float * norm) {
    if (!t || !params || !norm) return SWC_BAD_ARG;
    if (cudaMemcpy(t->params, params, sizeof(float) * kP, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(t->norm, norm, sizeof(float) * kN, cudaMemcpyHostToDevice) != cudaSuccess)
        return SWC_CUDA_ERROR;
    cudaMemset(t->m, 0, sizeof(float) * kP);
    cudaMemset(t->v, 0, sizeof(float) * kP);
    t->adam_t = 0;
    return SWC_OK;
}

int swc_trainer_get_params(swc_trainer * t, float * params, float * norm) {
    if (!t) return SWC_BAD_ARG;
    if (params && cudaMemcpy(params, t->params, sizeof(float) * kP, cudaMemcpyDeviceToHost) != cudaSuccess)
        return SWC_CUDA_ERROR;
    if (norm && cudaMemcpy(norm, t->norm, sizeof(float) * kN, cudaMemcpyDeviceToHost) != cudaSuccess)
        return SWC_CUDA_ERROR;
    return SWC_OK;
}

int swc_trainer_fit(swc_trainer * t, int32_t epochs, float lr, uint64_t seed, float * epoch_loss) {
    if (!t || epochs < 0 || t->n <= 0) return SWC_BAD_ARG;
    if (t->n >= (1LL << 31)) return SWC_BAD_ARG;
    // each epoch visits the rows in a pseudo-random order computed on the device (a
    // keyed Feistel permutation, keys from the seed and the epoch by splitmix64)
    int half = 0;
    while ((1LL << (2 * half)) < t->n) half++;
    uint64_t state = seed;
    auto splitmix = [&state]() {
        uint64_t z = (state += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    float norm_h[kN];
    if (epoch_loss) {
        if (cudaMemcpy(norm_h, t->norm, sizeof(float) * kN, cudaMemcpyDeviceToHost) != cudaSuccess) return SWC_CUDA_ERROR;
        if (!t->fpred && !talloc(&t->fpred, size_t(t->cap))) return SWC_OUT_OF_MEMORY;
    }
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int e = 0; e < epochs; e++) {
        const uint64_t k0 = splitmix(), k1 = splitmix();
        const unsigned key[4] = {unsigned(k0), unsigned(k0 >> 32), unsigned(k1), unsigned(k1 >> 32)};
        for (long long b0 = 0; b0 < t->n; b0 += t->batch) {
            const long long nb = std::min<long long>(t->batch, t->n - b0);
            launch_gather_shuffled(t->feat, t->tgt, t->n, b0, nb, half, key, t->bfeat, t->btgt, t->st);
            if (int rc = gradient_batch(t, t->bfeat, t->btgt, nb)) return rc;
            t->adam_t++;
            const float bc1 = 1.f - std::pow(b1, float(t->adam_t)), bc2 = 1.f - std::pow(b2, float(t->adam_t));
            launch_adam(t->params, t->grad, t->m, t->v, kP, lr, b1, b2, eps, bc1, bc2, t->st);
        }
        if (epoch_loss) {
            // loss of the epoch's parameters over the whole dataset, on the device
            if (int rc = forward_batch(t, t->feat, t->n, t->fpred)) return rc;
            launch_sq_err(t->fpred, t->tgt, t->n, 1.f / norm_h[2 * kIn + 1], t->part, kLossBlocks, t->st);
            double part[kLossBlocks];
            if (cudaMemcpyAsync(part, t->part, sizeof(part), cudaMemcpyDeviceToHost, t->st) != cudaSuccess)
                return SWC_CUDA_ERROR;
            if (int rc = check_err(t)) return rc;
            double s = 0;
            for (int b = 0; b < kLossBlocks; b++) s += part[b];
            epoch_loss[e] = float(s / double(t->n));
        } else if (int rc = check_err(t)) {
            return rc;
        }
    }
    return cudaGetLastError() == cudaSuccess ? SWC_OK : SWC_CUDA_ERROR;
}

int swc_mlp_forward(const float * params, const float * norm, const float * f, int64_t n, float * out) {
    if (!params || !norm || n < 0 || (n > 0 && (!f || !out))) return SWC_BAD_ARG;
    if (n == 0) return SWC_OK;
    swc_trainer * t = nullptr;
    int rc = swc_trainer_create(n, int32_t(std::min<int64_t>(n, 1 << 20)), &t);
    if (rc) return rc;
    if ((rc = swc_trainer_set_params(t, params, norm)) || (rc = swc_trainer_add(t, f, f, 0))) {
        swc_trainer_destroy(t);
        return rc;
    }
    cudaMemcpy(t->feat, f, sizeof(float) * kIn * n, cudaMemcpyHostToDevice);
    std::vector<float> tmp;
    for (long long b0 = 0; b0 < n && !rc; b0 += t->batch) {
        const long long nb = std::min<long long>(t->batch, n - b0);
        rc = forward_batch(t, t->feat + b0 * kIn, nb, t->pred);
        cudaMemcpyAsync(out + b0, t->pred, sizeof(float) * nb, cudaMemcpyDeviceToHost, t->st);
    }
    if (!rc) rc = check_err(t);
    swc_trainer_destroy(t);
    return rc;
}

int swc_mlp_gradient(const float * params, const float * norm, const float * f, const float * y, int64_t n,
                     float * grad, float * loss) {
    if (!params || !norm || !f || !y || !grad || n <= 0 || n > (1 << 24)) return SWC_BAD_ARG;
    swc_trainer * t = nullptr;
    int rc = swc_trainer_create(n, int32_t(n), &t);
    if (rc) return rc;
    if ((rc = swc_trainer_set_params(t, params, norm))) {
        swc_trainer_destroy(t);
        return rc;
    }
    cudaMemcpy(t->bfeat, f, sizeof(float) * kIn * n, cudaMemcpyHostToDevice);
    cudaMemcpy(t->btgt, y, sizeof(float) * n, cudaMemcpyHostToDevice);
    rc = gradient_batch(t, t->bfeat, t->btgt, n);
    if (!rc) rc = check_err(t);
    if (!rc) {
        cudaMemcpy(grad, t->grad, sizeof(float) * kP, cudaMemcpyDeviceToHost);
        if (loss) cudaMemcpy(loss, t->loss, sizeof(float), cudaMemcpyDeviceToHost);
    }
    swc_trainer_destroy(t);
    return rc;
}

}  // extern "C"
