// Device side of the learned proposal's autoregressive sampling (one output
// mode per step, all chains at once) as two kernels around the MLP's GEMMs:
// feature construction for mode j, and the masked-softmax draw of mode j's
// occupation with the bookkeeping of the chain state (proposal_math.cuh;
// mlp_tc.cu fuses the whole step into one tensor-core kernel).
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <cstdio>

#include "../../include/pqperm_gb300.h"
#include "proposal_math.cuh"

namespace pqg {
void set_last_error(const char *msg);
}

namespace {

using namespace pqg::prop;

__global__ void features_kernel(int j, int B, int d, int n, const float *__restrict__ ms,
                                const int32_t *__restrict__ n_rem, const float *__restrict__ shift,
                                __nv_bfloat16 *__restrict__ X, int8_t *__restrict__ lo, int8_t *__restrict__ hi) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    float x[kF];
    int l, h;
    features(j, d, n, ms, n_rem[b], shift[static_cast<int64_t>(b) * d + j], x, l, h);
    for (int k = 0; k < kF; ++k) X[static_cast<int64_t>(b) * kF + k] = __float2bfloat16(x[k]);
    lo[b] = static_cast<int8_t>(l);
    hi[b] = static_cast<int8_t>(h);
}

__global__ void sample_kernel(int j, int B, int d, const float *__restrict__ logits, const int8_t *__restrict__ lo,
                              const int8_t *__restrict__ hi, uint64_t seed_val, const uint64_t *__restrict__ seed_dev,
                              int8_t *__restrict__ samples, int32_t *__restrict__ n_rem, float *__restrict__ shift,
                              const float *__restrict__ C, const float *__restrict__ ms, float *__restrict__ logq) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const uint64_t seed = seed_dev ? *seed_dev : seed_val;
    draw(j, b, d, logits + static_cast<int64_t>(b) * kLD, lo[b], hi[b], seed, samples, n_rem, shift, C, ms, logq);
}

int fail(cudaError_t e, const char *what) {
    char buf[200];
    snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    pqg::set_last_error(buf);
    return PQG_ERR_CUDA;
}

}  // namespace

extern "C" {

int pqg_proposal_features(int32_t j, int32_t B, int32_t d, int32_t n, const float *mode_stats, const int32_t *n_rem,
                          const float *shift, void *X_bf16, int8_t *lo, int8_t *hi, void *stream) {
    if (B <= 0 || d <= 0 || j < 0 || j >= d) {
        pqg::set_last_error("pqg_proposal_features: invalid arguments");
        return PQG_ERR_INVALID;
    }
    features_kernel<<<(B + 127) / 128, 128, 0, static_cast<cudaStream_t>(stream)>>>(
        j, B, d, n, mode_stats, n_rem, shift, static_cast<__nv_bfloat16 *>(X_bf16), lo, hi);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PQG_OK : fail(e, "pqg_proposal_features");
}

int pqg_proposal_sample(int32_t j, int32_t B, int32_t d, const float *logits, const int8_t *lo, const int8_t *hi,
                        uint64_t seed, const uint64_t *seed_dev, int8_t *samples, int32_t *n_rem, float *shift,
                        const float *C, const float *mode_stats, float *logq, void *stream) {
    if (B <= 0 || d <= 0 || j < 0 || j >= d) {
        pqg::set_last_error("pqg_proposal_sample: invalid arguments");
        return PQG_ERR_INVALID;
    }
    sample_kernel<<<(B + 127) / 128, 128, 0, static_cast<cudaStream_t>(stream)>>>(
        j, B, d, logits, lo, hi, seed, seed_dev, samples, n_rem, shift, C, mode_stats, logq);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PQG_OK : fail(e, "pqg_proposal_sample");
}

}  // extern "C"
