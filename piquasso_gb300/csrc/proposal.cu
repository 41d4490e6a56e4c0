// Device side of the learned proposal's autoregressive sampling (one output
// mode per step, all chains at once): feature construction for mode j, and the
// masked-softmax draw of the occupation of mode j with the bookkeeping of the
// chain state.  The features match piquasso_gb300/proposal.py:features().
//
// Per-mode statistics `ms` (12 floats per mode): p(0..4), the tail
// Pr(X >= 5), mu, var, the suffix sum of mu from mode j on, 3 pad.  Chain state: photons left `n_rem`, the
// running mean shift of every later mode `shift` (B x d), the pattern
// `samples` (B x d, int8) and log q (B).
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <cstdio>

#include "../../include/pqperm_gb300.h"

namespace pqg {
void set_last_error(const char *msg);
}

namespace {

constexpr int kF = 16, kLD = 8, kCap = 7, kMS = 12;

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    // SplitMix64 finaliser (Steele, Lea, Flood, "Fast splittable pseudorandom
    // number generators", OOPSLA 2014)
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

__device__ __forceinline__ float uniform01(uint64_t seed, uint64_t chain, uint64_t step) {
    const uint64_t r = mix64(seed ^ mix64(chain * 0x100000001b3ULL + step));
    return static_cast<float>(r >> 40) * (1.0f / 16777216.0f);  // 24 random bits
}

__global__ void features_kernel(int j, int B, int d, int n, const float *__restrict__ ms,
                                const int32_t *__restrict__ n_rem, const float *__restrict__ shift,
                                __nv_bfloat16 *__restrict__ X, int8_t *__restrict__ lo, int8_t *__restrict__ hi) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const float *s = ms + kMS * j;
    const int nr = n_rem[b];
    const int left = d - j;
    const float sh = shift[static_cast<int64_t>(b) * d + j];
    float x[kF];
    x[0] = 1.0f;
    x[1] = static_cast<float>(nr) / n;
    x[2] = static_cast<float>(left) / d;
    x[3] = static_cast<float>(nr) / left;
    for (int k = 0; k < 5; ++k) x[4 + k] = s[k];
    x[9] = s[6];
    x[10] = (nr - s[8]) / sqrtf(static_cast<float>(n));
    x[11] = sh;
    x[12] = s[6] + sh;
    x[13] = nr * s[6] / fmaxf(s[8], 1e-12f);
    x[14] = s[7];
    x[15] = s[5];
    for (int k = 0; k < kF; ++k) X[static_cast<int64_t>(b) * kF + k] = __float2bfloat16(x[k]);
    const int l = nr - kCap * (left - 1);
    lo[b] = static_cast<int8_t>(l > 0 ? l : 0);
    hi[b] = static_cast<int8_t>(nr < kCap ? nr : kCap);
}

__global__ void sample_kernel(int j, int B, int d, const float *__restrict__ logits, const int8_t *__restrict__ lo,
                              const int8_t *__restrict__ hi, uint64_t seed_val, const uint64_t *__restrict__ seed_dev,
                              int8_t *__restrict__ samples,
                              int32_t *__restrict__ n_rem, float *__restrict__ shift, const float *__restrict__ C,
                              const float *__restrict__ ms, float *__restrict__ logq) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const float *z = logits + static_cast<int64_t>(b) * kLD;
    const int l = lo[b], h = hi[b];
    float mx = -3.0e38f;
    for (int c = l; c <= h; ++c) mx = fmaxf(mx, z[c]);
    float tot = 0.0f;
    for (int c = l; c <= h; ++c) tot += expf(z[c] - mx);
    const uint64_t seed = seed_dev ? *seed_dev : seed_val;
    const float u = uniform01(seed, static_cast<uint64_t>(b), static_cast<uint64_t>(j)) * tot;
    int pick = h;
    float acc = 0.0f;
    for (int c = l; c <= h; ++c) {
        acc += expf(z[c] - mx);
        if (u < acc) {
            pick = c;
            break;
        }
    }
    logq[b] += (z[pick] - mx) - logf(tot);
    samples[static_cast<int64_t>(b) * d + j] = static_cast<int8_t>(pick);
    n_rem[b] -= pick;
    const float dz = (pick - ms[kMS * j + 6]) / ms[kMS * j + 7];
    float *sh = shift + static_cast<int64_t>(b) * d;
    const float *cj = C + static_cast<int64_t>(j) * d;
    for (int k = j + 1; k < d; ++k) sh[k] += cj[k] * dz;
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
