// BF16 tensor-core kernels of the learned proposal's autoregressive MLP
// (3 hidden layers of width 256, GELU, a 5-way softmax head padded to 8).
//
// One GEMM kernel serves forward and backward passes:
//     C[M x N] = sum_k A(m, k) B(k, n)       (FP32 accumulation)
// with A and B read through arbitrary (row, column) strides, so transposed
// operands need no copies, staged through shared memory as BF16 and
// multiplied with warp-level BF16 MMAs (m16n8k16, FP32 accumulators).  Fused
// epilogues: bias + GELU to a BF16 activation (forward), plain FP32 output,
// and split-K partial sums for weight gradients (reduced deterministically by
// a second kernel).  Plus the GELU backward, the masked softmax cross-entropy
// head and an Adam step on FP32 master weights with BF16 copies.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <cstdio>

#include "../../include/pqperm_gb300.h"

namespace pqg {
void set_last_error(const char *msg);
}

namespace {

constexpr int BM = 64, BN = 64, BK = 32;  // block tile
constexpr int THREADS = 128;              // 4 warps, each 32 x 32 of the tile

struct Operand {
    const void *p;
    int64_t s_row, s_col;  // element strides of (m or k, k or n)
    int bf16;              // 1: __nv_bfloat16 elements, 0: float
};

__device__ __forceinline__ float ld_elem(const Operand &o, int64_t r, int64_t c) {
    const int64_t i = r * o.s_row + c * o.s_col;
    if (o.bf16) return __bfloat162float(reinterpret_cast<const __nv_bfloat16 *>(o.p)[i]);
    return reinterpret_cast<const float *>(o.p)[i];
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ void mma_bf16_16816(float (&c)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
    const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
    const float pdf = 0.39894228040143268f * expf(-0.5f * x * x);
    return cdf + x * pdf;
}

enum Epilogue : int {
    EPI_F32 = 0,        // C (float)
    EPI_BIAS_GELU = 1,  // pre = C + bias (float), act = GELU(pre) (bf16)
    EPI_SPLITK = 2,     // C partial (float) at split index blockIdx.z
    EPI_BIAS_F32 = 3,   // C + bias (float)
};

struct GemmArgs {
    Operand A, B;
    int64_t M, N, K;
    int64_t k_per_split;     // EPI_SPLITK: K range per blockIdx.z
    float *C;                // float output (or split-K partials: [splits][M][N])
    __nv_bfloat16 *act;      // EPI_BIAS_GELU: BF16 activation [M][N]
    const float *bias;       // [N]
    int epi;
};

// Shared tiles: A as [BM][BK] (row = m), B as [BN][BK] (row = n), both K-fast,
// with a 8-element pad against bank conflicts.
__global__ void __launch_bounds__(THREADS) gemm_bf16(GemmArgs g) {
    __shared__ __nv_bfloat16 As[BM][BK + 8];
    __shared__ __nv_bfloat16 Bs[BN][BK + 8];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t m0 = static_cast<int64_t>(blockIdx.y) * BM, n0 = static_cast<int64_t>(blockIdx.x) * BN;
    int64_t k_lo = 0, k_hi = g.K;
    if (g.epi == EPI_SPLITK) {
        k_lo = static_cast<int64_t>(blockIdx.z) * g.k_per_split;
        k_hi = k_lo + g.k_per_split < g.K ? k_lo + g.k_per_split : g.K;
    }
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;  // warp's 32 x 32 sub-tile
    float acc[2][4][4] = {};
    const int grp = lane >> 2, tig = lane & 3;
    for (int64_t k0 = k_lo; k0 < k_hi; k0 += BK) {
        for (int e = tid; e < BM * BK; e += THREADS) {
            const int r = e / BK, c = e % BK;
            const int64_t gm = m0 + r, gk = k0 + c;
            const float v = (gm < g.M && gk < k_hi) ? ld_elem(g.A, gm, gk) : 0.0f;
            As[r][c] = __float2bfloat16(v);
        }
        for (int e = tid; e < BN * BK; e += THREADS) {
            const int r = e / BK, c = e % BK;
            const int64_t gn = n0 + r, gk = k0 + c;
            const float v = (gn < g.N && gk < k_hi) ? ld_elem(g.B, gk, gn) : 0.0f;
            Bs[r][c] = __float2bfloat16(v);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; kk += 16) {
            uint32_t a[2][4], b[4][2];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int r = wm + i * 16 + grp;
                a[i][0] = *reinterpret_cast<const uint32_t *>(&As[r][kk + tig * 2]);
                a[i][1] = *reinterpret_cast<const uint32_t *>(&As[r + 8][kk + tig * 2]);
                a[i][2] = *reinterpret_cast<const uint32_t *>(&As[r][kk + 8 + tig * 2]);
                a[i][3] = *reinterpret_cast<const uint32_t *>(&As[r + 8][kk + 8 + tig * 2]);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int cn = wn + j * 8 + grp;
                b[j][0] = *reinterpret_cast<const uint32_t *>(&Bs[cn][kk + tig * 2]);
                b[j][1] = *reinterpret_cast<const uint32_t *>(&Bs[cn][kk + 8 + tig * 2]);
            }
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) mma_bf16_16816(acc[i][j], a[i], b[j]);
        }
        __syncthreads();
    }
    // epilogue: accumulator (i, j, q) sits at row wm + 16 i + grp (+8 for q >= 2),
    // column wn + 8 j + 2 tig + (q & 1)
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int64_t r = m0 + wm + i * 16 + grp + (q >= 2 ? 8 : 0);
                const int64_t c = n0 + wn + j * 8 + tig * 2 + (q & 1);
                if (r >= g.M || c >= g.N) continue;
                float v = acc[i][j][q];
                if (g.epi == EPI_SPLITK) {
                    g.C[(static_cast<int64_t>(blockIdx.z) * g.M + r) * g.N + c] = v;
                } else if (g.epi == EPI_BIAS_GELU) {
                    v += g.bias[c];
                    g.C[r * g.N + c] = v;
                    g.act[r * g.N + c] = __float2bfloat16(gelu(v));
                } else if (g.epi == EPI_BIAS_F32) {
                    g.C[r * g.N + c] = v + g.bias[c];
                } else {
                    g.C[r * g.N + c] = v;
                }
            }
}

// out[m][n] = sum over splits of part[s][m][n]  (fixed order: deterministic)
__global__ void splitk_reduce(const float *__restrict__ part, int splits, int64_t MN, float *__restrict__ out) {
    for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < MN;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        float s = 0.0f;
        for (int k = 0; k < splits; ++k) s += part[k * MN + e];
        out[e] = s;
    }
}

// dpre = dact * GELU'(pre)  (in place on dact, FP32)
__global__ void gelu_backward(float *__restrict__ d, const float *__restrict__ pre, int64_t n) {
    for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < n;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x)
        d[e] *= gelu_grad(pre[e]);
}

// bias gradient: db[n] = sum_m d[m][n]  (one thread per column, fixed order)
__global__ void bias_grad(const float *__restrict__ d, int64_t M, int64_t N, float *__restrict__ db) {
    const int64_t c = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= N) return;
    float s = 0.0f;
    for (int64_t m = 0; m < M; ++m) s += d[m * N + c];
    db[c] = s;
}

// Masked softmax cross-entropy over the first `classes` of `ld` logits per row.
// Class c of row m is allowed when lo[m] <= c <= hi[m].  Writes the loss of
// every row (nats), and dlogits = (softmax - onehot(target)) * scale.
__global__ void softmax_xent(const float *__restrict__ logits, int64_t M, int ld, int classes,
                             const int8_t *__restrict__ lo, const int8_t *__restrict__ hi,
                             const int8_t *__restrict__ target, float scale, float *__restrict__ loss,
                             float *__restrict__ dlogits) {
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
        }
    }
}

// Adam on FP32 master weights, refreshing the BF16 copy.
__global__ void adam_step(float *__restrict__ w, __nv_bfloat16 *__restrict__ wb, const float *__restrict__ g,
                          float *__restrict__ m1, float *__restrict__ m2, int64_t n, float lr, float b1, float b2,
                          float eps, float c1, float c2) {
    for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < n;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float gi = g[e];
        const float a = b1 * m1[e] + (1.0f - b1) * gi;
        const float b = b2 * m2[e] + (1.0f - b2) * gi * gi;
        m1[e] = a;
        m2[e] = b;
        const float upd = lr * (a / c1) / (sqrtf(b / c2) + eps);
        const float nw = w[e] - upd;
        w[e] = nw;
        if (wb) wb[e] = __float2bfloat16(nw);
    }
}

int fail_cuda(cudaError_t e, const char *what) {
    char buf[200];
    snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    pqg::set_last_error(buf);
    return PQG_ERR_CUDA;
}

}  // namespace

extern "C" {

int pqg_mlp_gemm(const void *a, int32_t a_bf16, int64_t a_s_row, int64_t a_s_col, const void *b, int32_t b_bf16,
                 int64_t b_s_row, int64_t b_s_col, int64_t M, int64_t N, int64_t K, int32_t epilogue, float *c,
                 void *act_bf16, const float *bias, float *splitk_scratch, int32_t splits, void *stream) {
    if (M <= 0 || N <= 0 || K <= 0 || !a || !b || !c) {
        pqg::set_last_error("pqg_mlp_gemm: invalid arguments");
        return PQG_ERR_INVALID;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    GemmArgs g;
    g.A = Operand{a, a_s_row, a_s_col, a_bf16};
    g.B = Operand{b, b_s_row, b_s_col, b_bf16};
    g.M = M;
    g.N = N;
    g.K = K;
    g.C = c;
    g.act = static_cast<__nv_bfloat16 *>(act_bf16);
    g.bias = bias;
    g.epi = epilogue;
    dim3 grid(static_cast<unsigned>((N + BN - 1) / BN), static_cast<unsigned>((M + BM - 1) / BM), 1);
    if (epilogue == EPI_SPLITK) {
        if (splits < 1 || !splitk_scratch) {
            pqg::set_last_error("pqg_mlp_gemm: split-K needs splits >= 1 and a scratch buffer");
            return PQG_ERR_INVALID;
        }
        int64_t kps = (K + splits - 1) / splits;
        kps = (kps + BK - 1) / BK * BK;
        g.k_per_split = kps;
        g.C = splitk_scratch;
        grid.z = static_cast<unsigned>((K + kps - 1) / kps);
        gemm_bf16<<<grid, THREADS, 0, s>>>(g);
        splitk_reduce<<<256, 256, 0, s>>>(splitk_scratch, static_cast<int>(grid.z), M * N, c);
    } else {
        g.k_per_split = K;
        gemm_bf16<<<grid, THREADS, 0, s>>>(g);
    }
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PQG_OK : fail_cuda(e, "pqg_mlp_gemm");
}

int pqg_mlp_gelu_backward(float *d, const float *pre, int64_t n, void *stream) {
    gelu_backward<<<512, 256, 0, static_cast<cudaStream_t>(stream)>>>(d, pre, n);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PQG_OK : fail_cuda(e, "pqg_mlp_gelu_backward");
}

int pqg_mlp_bias_grad(const float *d, int64_t M, int64_t N, float *db, void *stream) {
    bias_grad<<<static_cast<unsigned>((N + 127) / 128), 128, 0, static_cast<cudaStream_t>(stream)>>>(d, M, N, db);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PQG_OK : fail_cuda(e, "pqg_mlp_bias_grad");
}

int pqg_mlp_softmax_xent(const float *logits, int64_t M, int32_t ld, int32_t classes, const int8_t *lo,
                         const int8_t *hi, const int8_t *target, float scale, float *loss, float *dlogits,
                         void *stream) {
    softmax_xent<<<static_cast<unsigned>((M + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        logits, M, ld, classes, lo, hi, target, scale, loss, dlogits);
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

}  // extern "C"
