// Elementwise and reduction kernels of the learned proposal's MLP (3 hidden
// layers of width 256, GELU, an 8-way softmax head): bias gradients, the
// masked softmax cross-entropy head and the Adam step on FP32 master weights
// with BF16 copies.  The GEMMs (forward, data and weight gradients, with
// fused bias / GELU / GELU-backward epilogues) run on the tcgen05 kernel in
// mlp_tc.cu.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <cstdio>

#include "../../include/pqperm_gb300.h"

namespace pqg {
void set_last_error(const char *msg);
}

namespace {

// Bias gradient db[n] = sum_m d[m][n], deterministic and spread over the GPU:
// blocks of 32 columns x 256 rows write partial sums (8 row lanes, fixed-order
// shared-memory sum), then a fixed-order sum over the row chunks.
constexpr int BIAS_ROWS = 256;

__global__ void bias_partial(const float *__restrict__ d, int64_t M, int64_t N, float *__restrict__ part) {
    __shared__ float s[8][33];
    const int64_t c = static_cast<int64_t>(blockIdx.x) * 32 + threadIdx.x;
    const int64_t m_lo = static_cast<int64_t>(blockIdx.y) * BIAS_ROWS;
    const int64_t m_hi = m_lo + BIAS_ROWS < M ? m_lo + BIAS_ROWS : M;
    float acc = 0.0f;
    if (c < N)
        for (int64_t m = m_lo + threadIdx.y; m < m_hi; m += 8) acc += d[m * N + c];
    s[threadIdx.y][threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.y == 0 && c < N) {
        float t = 0.0f;
        for (int k = 0; k < 8; ++k) t += s[k][threadIdx.x];
        part[static_cast<int64_t>(blockIdx.y) * N + c] = t;
    }
}

// The sum over the row chunks: 32 chunk lanes per column (lane y takes chunks
// y, y + 32, ...), then the 32 lane sums in order -- a fixed order, and
// independent loads instead of one thread's chain of `chunks` dependent adds.
constexpr int BIAS_LANES = 32;

__global__ void bias_final(const float *__restrict__ part, int64_t chunks, int64_t N, float *__restrict__ db) {
    __shared__ float s[BIAS_LANES][33];
    const int64_t c = static_cast<int64_t>(blockIdx.x) * 32 + threadIdx.x;
    float acc = 0.0f;
    if (c < N)
        for (int64_t k = threadIdx.y; k < chunks; k += BIAS_LANES) acc += part[k * N + c];
    s[threadIdx.y][threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.y == 0 && c < N) {
        float t = 0.0f;
        for (int k = 0; k < BIAS_LANES; ++k) t += s[k][threadIdx.x];
        db[c] = t;
    }
}

// Masked softmax cross-entropy over the first `classes` of `ld` logits per row.
// Class c of row m is allowed when lo[m] <= c <= hi[m].  Writes the loss of
// every row (nats), and dlogits = (softmax - onehot(target)) * scale.
__global__ void softmax_xent(const float *__restrict__ logits, int64_t M, int ld, int classes,
                             const int8_t *__restrict__ lo, const int8_t *__restrict__ hi,
                             const int8_t *__restrict__ target, float scale, float *__restrict__ loss,
                             float *__restrict__ dlogits, __nv_bfloat16 *__restrict__ dlogits_bf16) {
    const int64_t m = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (m >= M) return;
    const float *z = logits + m * ld;
    float mx = -3.0e38f;
    for (int c = lo[m]; c <= hi[m]; ++c) mx = fmaxf(mx, z[c]);
    float s = 0.0f;
    for (int c = lo[m]; c <= hi[m]; ++c) s += expf(z[c] - mx);
    const float lse = mx + logf(s);
    const int t = target ? target[m] : -1;
    if (loss) loss[m] = (t >= 0) ? lse - z[t] : 0.0f;
    if (dlogits) {
        for (int c = 0; c < ld; ++c) {
            float p = (c >= lo[m] && c <= hi[m] && c < classes) ? expf(z[c] - lse) : 0.0f;
            if (c == t) p -= 1.0f;
            dlogits[m * ld + c] = p * scale;
            if (dlogits_bf16) dlogits_bf16[m * ld + c] = __float2bfloat16(p * scale);
        }
    }
}

// Adam on FP32 master weights, refreshing the BF16 copy.
// One element of an Adam step (moments updated in place; the new weight
// returned).  Both Adam kernels call it, so that they agree bit for bit.
__device__ __forceinline__ float adam_elem(float *__restrict__ w, const float *__restrict__ g,
                                           float *__restrict__ m1, float *__restrict__ m2, int64_t e, float lr,
                                           float b1, float b2, float eps, float c1, float c2) {
    const float gi = g[e];
    const float a = b1 * m1[e] + (1.0f - b1) * gi;
    const float b = b2 * m2[e] + (1.0f - b2) * gi * gi;
    m1[e] = a;
    m2[e] = b;
    const float upd = lr * (a / c1) / (sqrtf(b / c2) + eps);
    const float nw = w[e] - upd;
    w[e] = nw;
    return nw;
}

__global__ void adam_step(float *__restrict__ w, __nv_bfloat16 *__restrict__ wb, const float *__restrict__ g,
                          float *__restrict__ m1, float *__restrict__ m2, int64_t n, float lr, float b1, float b2,
                          float eps, float c1, float c2) {
    for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < n;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float nw = adam_elem(w, g, m1, m2, e, lr, b1, b2, eps, c1, c2);
        if (wb) wb[e] = __float2bfloat16(nw);
    }
}

// Every parameter tensor of a network in one launch (blockIdx.y: the tensor),
// each with an optional BF16 copy and an optional transposed BF16 copy
// (cols x rows): the step's separate Adam launches and weight transposes,
// each a few microseconds of latency, in one.
constexpr int ADAM_MAX = 16;

struct AdamSet {
    float *w[ADAM_MAX];
    __nv_bfloat16 *wb[ADAM_MAX];
    __nv_bfloat16 *wbt[ADAM_MAX];
    const float *g[ADAM_MAX];
    float *m1[ADAM_MAX];
    float *m2[ADAM_MAX];
    int64_t rows[ADAM_MAX], cols[ADAM_MAX];
};

__global__ void adam_multi(const __grid_constant__ AdamSet s, float lr, float b1, float b2, float eps, float c1,
                           float c2) {
    const int t = blockIdx.y;
    const int64_t rows = s.rows[t], cols = s.cols[t], n = rows * cols;
    for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < n;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float nw = adam_elem(s.w[t], s.g[t], s.m1[t], s.m2[t], e, lr, b1, b2, eps, c1, c2);
        if (s.wb[t]) s.wb[t][e] = __float2bfloat16(nw);
        if (s.wbt[t]) {
            const int64_t r = e / cols, c = e - r * cols;
            s.wbt[t][c * rows + r] = __float2bfloat16(nw);
        }
    }
}

int fail_cuda(cudaError_t e, const char *what) {
    char buf[200];
    snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    pqg::set_last_error(buf);
    return PQG_ERR_CUDA;
}

}  // namespace

namespace pqg {

int mlp_column_sums_final(const float *part, int64_t chunks, int64_t N, float *out, cudaStream_t s) {
    bias_final<<<static_cast<unsigned>((N + 31) / 32), dim3(32, BIAS_LANES), 0, s>>>(part, chunks, N, out);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PQG_OK : fail_cuda(e, "pqg_mlp_gemm_tc_t (column sums)");
}

}  // namespace pqg

extern "C" {

int pqg_mlp_bias_grad(const float *d, int64_t M, int64_t N, float *db, float *scratch, void *stream) {
    if (M <= 0 || N <= 0 || !d || !db || !scratch) {
        pqg::set_last_error("pqg_mlp_bias_grad: invalid arguments");
        return PQG_ERR_INVALID;
    }
    const int64_t chunks = (M + BIAS_ROWS - 1) / BIAS_ROWS;
    if (chunks > 65535) {
        pqg::set_last_error("pqg_mlp_bias_grad: too many rows");
        return PQG_ERR_TOO_LARGE;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    bias_partial<<<dim3(static_cast<unsigned>((N + 31) / 32), static_cast<unsigned>(chunks)), dim3(32, 8), 0, s>>>(
        d, M, N, scratch);
    bias_final<<<static_cast<unsigned>((N + 31) / 32), dim3(32, BIAS_LANES), 0, s>>>(scratch, chunks, N, db);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PQG_OK : fail_cuda(e, "pqg_mlp_bias_grad");
}

int pqg_mlp_softmax_xent(const float *logits, int64_t M, int32_t ld, int32_t classes, const int8_t *lo,
                         const int8_t *hi, const int8_t *target, float scale, float *loss, float *dlogits,
                         void *dlogits_bf16, void *stream) {
    softmax_xent<<<static_cast<unsigned>((M + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        logits, M, ld, classes, lo, hi, target, scale, loss, dlogits, static_cast<__nv_bfloat16 *>(dlogits_bf16));
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PQG_OK : fail_cuda(e, "pqg_mlp_softmax_xent");
}

int pqg_mlp_adam(float *w, void *w_bf16, const float *g, float *m1, float *m2, int64_t n, float lr, float b1,
                 float b2, float eps, int64_t step, void *stream) {
    const float c1 = 1.0f - powf(b1, static_cast<float>(step));
    const float c2 = 1.0f - powf(b2, static_cast<float>(step));
    adam_step<<<512, 256, 0, static_cast<cudaStream_t>(stream)>>>(w, static_cast<__nv_bfloat16 *>(w_bf16), g, m1, m2,
                                                                  n, lr, b1, b2, eps, c1, c2);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PQG_OK : fail_cuda(e, "pqg_mlp_adam");
}

int pqg_mlp_adam_multi(int32_t count, float *const *w, void *const *w_bf16, void *const *w_bf16_t,
                       const float *const *g, float *const *m1, float *const *m2, const int64_t *rows,
                       const int64_t *cols, float lr, float b1, float b2, float eps, int64_t step, void *stream) {
    if (count < 1 || count > ADAM_MAX || !w || !g || !m1 || !m2 || !rows || !cols) {
        pqg::set_last_error("pqg_mlp_adam_multi: invalid arguments (1 <= count <= 16, non-null arrays)");
        return PQG_ERR_INVALID;
    }
    AdamSet set{};
    for (int i = 0; i < count; ++i) {
        if (!w[i] || !g[i] || !m1[i] || !m2[i] || rows[i] <= 0 || cols[i] <= 0) {
            pqg::set_last_error("pqg_mlp_adam_multi: invalid tensor");
            return PQG_ERR_INVALID;
        }
        set.w[i] = w[i];
        set.wb[i] = w_bf16 ? static_cast<__nv_bfloat16 *>(w_bf16[i]) : nullptr;
        set.wbt[i] = w_bf16_t ? static_cast<__nv_bfloat16 *>(w_bf16_t[i]) : nullptr;
        set.g[i] = g[i];
        set.m1[i] = m1[i];
        set.m2[i] = m2[i];
        set.rows[i] = rows[i];
        set.cols[i] = cols[i];
    }
    const float c1 = 1.0f - powf(b1, static_cast<float>(step));
    const float c2 = 1.0f - powf(b2, static_cast<float>(step));
    adam_multi<<<dim3(64, static_cast<unsigned>(count)), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        set, lr, b1, b2, eps, c1, c2);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PQG_OK : fail_cuda(e, "pqg_mlp_adam_multi");
}

}  // extern "C"
