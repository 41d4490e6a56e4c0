// Per-chain arithmetic of the learned proposal's autoregressive step, shared
// by the separate feature and sampling kernels (proposal.cu) and the fused
// tensor-core step (mlp_tc.cu), so both draw identical patterns: the 16
// features of output mode j (piquasso_gb300/proposal.py:features()), the
// feasible occupation range, and the masked-softmax draw with its
// bookkeeping of the chain state.
//
// Per-mode statistics `ms` (12 floats per mode): p(0..4), the tail
// Pr(X >= 5), mu, var, the suffix sum of mu from mode j on, 3 pad.  Chain
// state: photons left n_rem, the running mean shift of every later mode
// `shift` (B x d), the pattern `samples` (B x d, int8) and log q (B).
#pragma once
#include <stdint.h>

namespace pqg {
namespace prop {

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

// Features of chain b at mode j and its occupation range [lo, hi].
__device__ __forceinline__ void features(int j, int d, int n, const float *__restrict__ ms, int nr, float sh,
                                         float (&x)[kF], int &lo, int &hi) {
    const float *s = ms + kMS * j;
    const int left = d - j;
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
    const int l = nr - kCap * (left - 1);
    lo = l > 0 ? l : 0;
    hi = nr < kCap ? nr : kCap;
}

// Draws chain b's occupation of mode j from the masked softmax of its logits
// z (occupations lo..hi) and updates the chain state.
__device__ __forceinline__ void draw(int j, int b, int d, const float *__restrict__ z, int lo, int hi, uint64_t seed,
                                     int8_t *__restrict__ samples, int32_t *__restrict__ n_rem,
                                     float *__restrict__ shift, const float *__restrict__ C,
                                     const float *__restrict__ ms, float *__restrict__ logq) {
    float mx = -3.0e38f;
    for (int c = lo; c <= hi; ++c) mx = fmaxf(mx, z[c]);
    float tot = 0.0f;
    for (int c = lo; c <= hi; ++c) tot += expf(z[c] - mx);
    const float u = uniform01(seed, static_cast<uint64_t>(b), static_cast<uint64_t>(j)) * tot;
    int pick = hi;
    float acc = 0.0f;
    for (int c = lo; c <= hi; ++c) {
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

}  // namespace prop
}  // namespace pqg
