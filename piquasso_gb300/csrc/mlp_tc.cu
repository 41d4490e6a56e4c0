// Blackwell (sm_103a) tensor-core GEMM of the learned proposal's MLP:
//
//     C[M x N] = A[M x K] . B[N x K]^T        (BF16 operands, FP32 accumulation)
//
// with A and B row-major and K contiguous ("K-major"), the one layout every
// forward and backward GEMM of the network is brought into (backward
// operands by the transpose kernel below).  One CTA of 128 threads computes a
// 128 x BN tile (BN = N rounded up to 16, at most 256):
//   * TMA (cp.async.bulk.tensor.2d) stages 64-wide K chunks of A (128 x 64)
//     and B (BN x 64) into shared memory with the 128-byte swizzle, two stages
//     deep, each stage completing on an mbarrier (expect-tx bytes);
//   * one thread issues tcgen05.mma.cta_group::1.kind::f16 (M = 128, N = BN,
//     K = 16 per instruction) from shared-memory descriptors, accumulating in
//     tensor memory (TMEM, BN FP32 columns), and tcgen05.commit releases each
//     stage back to the TMA producer once its MMAs have read it;
//   * after a final commit, each warp reads its 32 accumulator rows with
//     tcgen05.ld (32x32b), turns them around in shared memory so that the
//     global stores write whole row segments, and applies the fused
//     epilogue: plain FP32, bias,
//     bias + GELU (FP32 pre-activation and BF16 activation), GELU backward
//     (dpre = acc * GELU'(pre), FP32 and BF16), or split-K partial sums.
// Rows and columns past M, N, K are zero-filled by TMA (out-of-range box
// elements) and never stored.  Every mbarrier wait is bounded: a wait that
// runs out records an error code in device memory (pqg_mlp_tc_status) and the
// CTA still waits for its issued MMAs and frees its TMEM before returning.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include <cstdio>
#include <mutex>

#include "../../include/pqperm_gb300.h"
#include "proposal_math.cuh"

namespace pqg {
void set_last_error(const char *msg);
// out[n] = sum over chunks of part[chunk][n], in chunk order (mlp.cu)
int mlp_column_sums_final(const float *part, int64_t chunks, int64_t N, float *out, cudaStream_t s);
}

namespace {

constexpr int TC_BM = 128;      // UMMA M (cta_group::1)
constexpr int TC_BK = 64;       // K chunk: one 128-byte swizzle row of BF16
constexpr int TC_STAGES = 2;
constexpr int TC_SPLITK_STAGES = 4;
constexpr int TC_THREADS = 128;
constexpr uint32_t TC_A_BYTES = TC_BM * TC_BK * 2;  // 16 KB per stage
constexpr long long TC_WAIT_LIMIT = 1ll << 22;       // try_wait rounds before giving up

enum TcEpilogue : int {
    TC_EPI_F32 = 0,        // C = acc
    TC_EPI_BIAS_GELU = 1,  // C = acc + bias (FP32), Cb = GELU(C) (BF16)
    TC_EPI_SPLITK = 2,     // C[split][m][n] = acc over the split's K range
    TC_EPI_BIAS_F32 = 3,   // C = acc + bias
    TC_EPI_DGELU = 4,      // C = acc * GELU'(pre) (FP32), Cb = BF16(C)
};

__device__ int g_tc_error;  // first failure code (0: none)

struct TcArgs {
    int64_t M, N, K;
    int64_t k_per_split;  // multiple of TC_BK
    float *C;
    __nv_bfloat16 *Cb;
    const float *bias;
    const float *pre;
    float *col_part;  // nullable: the persistent tensor-store forms' column sums of C per 32-row block
    int BN;           // tile columns (UMMA N)
    int tmem_cols;  // power of two >= max(32, BN)
    int epi;
    int pad;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// Bounded wait for the phase with the given parity; false when it ran out.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (long long i = 0; i < TC_WAIT_LIMIT; ++i) {
        uint32_t done = 0;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int32_t x, int32_t y,
                                            uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

// Tile store shared -> global through the bulk-async group of the issuing
// thread; elements outside the tensor map's extent are not written.
__device__ __forceinline__ void tma_store_2d(const CUtensorMap *map, uint32_t src, int32_t x, int32_t y) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];" ::"l"(
                     reinterpret_cast<uint64_t>(map)),
                 "r"(src), "r"(x), "r"(y)
                 : "memory");
}

// Shared-memory matrix descriptor of a K-major operand tile in the 128-byte
// swizzle layout: rows of 128 bytes, 8-row groups 1024 bytes apart (stride
// byte offset), the leading byte offset unused (one swizzle atom spans the
// chunk's K), descriptor version 1, swizzle mode 2 (128 B).
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t addr) {
    uint64_t d = 0;
    d |= static_cast<uint64_t>((addr >> 4) & 0x3FFFu);
    d |= static_cast<uint64_t>(1) << 16;
    d |= static_cast<uint64_t>(1024 >> 4) << 32;
    d |= static_cast<uint64_t>(1) << 46;
    d |= static_cast<uint64_t>(2) << 61;
    return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N = bn, M = 128.
__host__ __device__ constexpr uint32_t idesc_bf16(int bn) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(bn >> 3) << 17) |
           (static_cast<uint32_t>(TC_BM >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, int accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
        "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void record_error(int code) { atomicCAS(&g_tc_error, 0, code); }

// GELU(x) = x Phi(x), Phi(x) = (1 + erf(x / sqrt 2)) / 2, for the forward
// activations (BF16, 2^-9 relative).  erf by Abramowitz & Stegun, Handbook of
// Mathematical Functions, formula 7.1.26 (Hastings' approximation, |error| <=
// 1.5e-7): for z >= 0, 1 - erf(z) = q(t) e^{-z^2}, t = 1 / (1 + p z), q a
// fifth-degree polynomial.  The negative side takes Phi = q e^{-z^2} / 2
// directly, with no cancellation.  The reciprocal and the exponential are the
// hardware approximations (__fdividef, __expf): about 14 instructions, two of
// them on the special-function unit.  |GELU - exact| <= 4.2e-7.  The backward
// pass (gelu_grad) keeps erff.
__device__ __forceinline__ float gelu(float x) {
    const float z = fabsf(x) * 0.70710678118654752f;
    const float t = __fdividef(1.0f, __fmaf_rn(0.3275911f, z, 1.0f));
    float q = __fmaf_rn(1.061405429f, t, -1.453152027f);
    q = __fmaf_rn(q, t, 1.421413741f);
    q = __fmaf_rn(q, t, -0.284496736f);
    q = __fmaf_rn(q, t, 0.254829592f);
    q = __fmul_rn(__fmul_rn(q, t), __expf(-z * z));  // 1 - erf(z)
    const float phi = x >= 0.0f ? __fmaf_rn(-0.5f, q, 1.0f) : 0.5f * q;
    return x * phi;
}
__device__ __forceinline__ float gelu_grad(float x) {
    const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
    const float pdf = 0.39894228040143268f * expf(-0.5f * x * x);
    return cdf + x * pdf;
}

// One group of W (32 or 16; the one-tile kernel's last group may hold 16 of
// 32) accumulator columns of a warp's 32 rows (row `lane` of the group in v):
// through the padded 32 x (W + 1) `tile` so that the stores write whole row
// segments, then the fused epilogue.  rows_base: the global row of the warp's
// first row; col0: the group's first column.  Every element takes the same
// operations whatever W, so kernels with different W agree bit for bit.
template <int W>
__device__ __forceinline__ void epilogue_group_w(const TcArgs &g, float *tile, const float (&v)[W], int ncol,
                                                 int64_t rows_base, int64_t col0, float *cbase, bool vec_ok,
                                                 int lane) {
    constexpr int S = W + 1;       // tile row stride (odd: conflict-free column writes)
    constexpr int QPR = W / 4;     // column quads per row
    constexpr int RSTEP = 32 / QPR;  // rows between a lane's rows in the fast path
    for (int q = 0; q < ncol; ++q) tile[lane * S + q] = v[q];
    __syncwarp();
    if (ncol == W && vec_ok && rows_base + 32 <= g.M && col0 + W <= g.N) {
        // a whole 32 x W group: lane takes column quad q = lane % QPR of rows
        // lane / QPR, + RSTEP, ... (the same operations per element as below,
        // with the column, its bias and the row stride fixed per lane)
        const int q = lane % QPR, r0 = lane / QPR;
        const int64_t col = col0 + 4 * q;
        float4 bb = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (g.epi == TC_EPI_BIAS_GELU || g.epi == TC_EPI_BIAS_F32) bb = *reinterpret_cast<const float4 *>(g.bias + col);
        int64_t at = (rows_base + r0) * g.N + col;
        const int64_t step = RSTEP * g.N;
#pragma unroll 2
        for (int r = r0; r < 32; r += RSTEP, at += step) {
            float x[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) x[k] = tile[r * S + 4 * q + k];
            if (g.epi == TC_EPI_BIAS_GELU || g.epi == TC_EPI_BIAS_F32) {
                x[0] += bb.x, x[1] += bb.y, x[2] += bb.z, x[3] += bb.w;
            } else if (g.epi == TC_EPI_DGELU) {
                const float4 p = *reinterpret_cast<const float4 *>(g.pre + at);
                x[0] *= gelu_grad(p.x), x[1] *= gelu_grad(p.y), x[2] *= gelu_grad(p.z), x[3] *= gelu_grad(p.w);
            }
            *reinterpret_cast<float4 *>(cbase + at) = make_float4(x[0], x[1], x[2], x[3]);
            if (g.epi == TC_EPI_BIAS_GELU || g.epi == TC_EPI_DGELU) {
                const bool act = g.epi == TC_EPI_BIAS_GELU;
                __nv_bfloat162 lo2 = __floats2bfloat162_rn(act ? gelu(x[0]) : x[0], act ? gelu(x[1]) : x[1]);
                __nv_bfloat162 hi2 = __floats2bfloat162_rn(act ? gelu(x[2]) : x[2], act ? gelu(x[3]) : x[3]);
                uint2 w;
                w.x = *reinterpret_cast<uint32_t *>(&lo2);
                w.y = *reinterpret_cast<uint32_t *>(&hi2);
                *reinterpret_cast<uint2 *>(g.Cb + at) = w;
            }
        }
        return;
    }
    const int nquad = ncol / 4;
    for (int idx = lane; idx < 32 * nquad; idx += 32) {
        const int r = idx / nquad, q = idx - r * nquad;
        const int64_t row = rows_base + r;
        const int64_t col = col0 + 4 * q;
        if (row >= g.M || col >= g.N) continue;
        float x[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) x[k] = tile[r * S + 4 * q + k];
        const int64_t at = row * g.N + col;
        if (vec_ok && col + 3 < g.N) {
            if (g.epi == TC_EPI_BIAS_GELU || g.epi == TC_EPI_BIAS_F32) {
                const float4 bb = *reinterpret_cast<const float4 *>(g.bias + col);
                x[0] += bb.x, x[1] += bb.y, x[2] += bb.z, x[3] += bb.w;
            } else if (g.epi == TC_EPI_DGELU) {
                const float4 p = *reinterpret_cast<const float4 *>(g.pre + at);
                x[0] *= gelu_grad(p.x), x[1] *= gelu_grad(p.y), x[2] *= gelu_grad(p.z), x[3] *= gelu_grad(p.w);
            }
            *reinterpret_cast<float4 *>(cbase + at) = make_float4(x[0], x[1], x[2], x[3]);
            if (g.epi == TC_EPI_BIAS_GELU || g.epi == TC_EPI_DGELU) {
                const bool act = g.epi == TC_EPI_BIAS_GELU;
                __nv_bfloat162 lo2 = __floats2bfloat162_rn(act ? gelu(x[0]) : x[0], act ? gelu(x[1]) : x[1]);
                __nv_bfloat162 hi2 = __floats2bfloat162_rn(act ? gelu(x[2]) : x[2], act ? gelu(x[3]) : x[3]);
                uint2 w;
                w.x = *reinterpret_cast<uint32_t *>(&lo2);
                w.y = *reinterpret_cast<uint32_t *>(&hi2);
                *reinterpret_cast<uint2 *>(g.Cb + at) = w;
            }
        } else {
            for (int k = 0; k < 4 && col + k < g.N; ++k) {
                float y = x[k];
                if (g.epi == TC_EPI_BIAS_GELU || g.epi == TC_EPI_BIAS_F32) y += g.bias[col + k];
                if (g.epi == TC_EPI_DGELU) y *= gelu_grad(g.pre[at + k]);
                cbase[at + k] = y;
                if (g.epi == TC_EPI_BIAS_GELU) g.Cb[at + k] = __float2bfloat16(gelu(y));
                if (g.epi == TC_EPI_DGELU) g.Cb[at + k] = __float2bfloat16(y);
            }
        }
    }
}

__device__ __forceinline__ void epilogue_group(const TcArgs &g, float *tile, const float (&v)[32], int ncol,
                                               int64_t rows_base, int64_t col0, float *cbase, bool vec_ok,
                                               int lane) {
    epilogue_group_w<32>(g, tile, v, ncol, rows_base, col0, cbase, vec_ok, lane);
}

// NS: TMA stages (2; 4 for split-K, whose CTAs each walk a long K range: the
// issuing thread refills a stage only once its MMAs have completed, so the
// stages in flight are the loads that overlap).
template <int NS>
__global__ void __launch_bounds__(TC_THREADS, 1)
    gemm_tc(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b, TcArgs g) {
    extern __shared__ uint8_t tc_smem_raw[];
    // stages at a 1024-byte boundary (the swizzle atom), then the barriers
    const uint32_t raw = smem_u32(tc_smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;
    const uint32_t b_bytes = static_cast<uint32_t>(g.BN) * TC_BK * 2;
    const uint32_t stage_bytes = TC_A_BYTES + b_bytes;
    const uint32_t bar0 = base + NS * stage_bytes;  // full[s] at bar0 + 8s, empty[s] at + 8 NS + 8s, then done
    const uint32_t full0 = bar0, empty0 = bar0 + 8 * NS, done = bar0 + 16 * NS;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(tc_smem_raw + (done + 8 - raw));

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t m0 = static_cast<int64_t>(blockIdx.y) * TC_BM, n0 = static_cast<int64_t>(blockIdx.x) * g.BN;
    const int64_t k_lo = static_cast<int64_t>(blockIdx.z) * g.k_per_split;
    const int64_t k_hi = k_lo + g.k_per_split < g.K ? k_lo + g.k_per_split : g.K;
    const int nchunks = static_cast<int>((k_hi - k_lo + TC_BK - 1) / TC_BK);

    if (tid == 0) {
        for (int s = 0; s < NS; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, 1);
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(g.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (tid == 0) {
        const uint32_t idesc = idesc_bf16(g.BN);
        auto issue = [&](int c) {
            const int s = c % NS;
            const uint32_t sa = base + s * stage_bytes, sb = sa + TC_A_BYTES;
            const int32_t kx = static_cast<int32_t>(k_lo + static_cast<int64_t>(c) * TC_BK);  // multiple of 64
            mbar_expect_tx(full0 + 8 * s, stage_bytes);
            tma_load_2d(sa, &map_a, kx, static_cast<int32_t>(m0), full0 + 8 * s);
            tma_load_2d(sb, &map_b, kx, static_cast<int32_t>(n0), full0 + 8 * s);
        };
        for (int c = 0; c < NS && c < nchunks; ++c) issue(c);
        bool ok = true;
        for (int c = 0; c < nchunks && ok; ++c) {
            const int s = c % NS;
            const uint32_t parity = static_cast<uint32_t>((c / NS) & 1);
            if (!mbar_wait(full0 + 8 * s, parity)) {
                record_error(1);
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t sa = base + s * stage_bytes, sb = sa + TC_A_BYTES;
            const int64_t kc = k_hi - (k_lo + static_cast<int64_t>(c) * TC_BK);
            const int nk = kc >= TC_BK ? TC_BK / 16 : static_cast<int>((kc + 15) / 16);
            for (int kk = 0; kk < nk; ++kk)
                umma_bf16(tmem, sdesc_sw128(sa + 32u * kk), sdesc_sw128(sb + 32u * kk), idesc, (c > 0 || kk > 0) ? 1 : 0);
            umma_commit(empty0 + 8 * s);
            if (c + NS < nchunks) {
                // the stage is refilled once its MMAs have read it
                if (!mbar_wait(empty0 + 8 * s, parity)) {
                    record_error(2);
                    ok = false;
                    break;
                }
                issue(c + NS);
            }
        }
        umma_commit(done);  // arrives when every MMA issued above has completed
    }
    __syncwarp();
    // warp-uniform: the TMEM loads below are .sync.aligned
    const bool have = __all_sync(0xffffffffu, mbar_wait(done, 0));
    if (!have && lane == 0) record_error(3);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

    if (have) {
        // Each warp owns accumulator rows [32 warp, 32 warp + 32).  Per group of
        // 32 (or a last 16) columns: tcgen05.ld puts row `lane` in this thread;
        // the rows go through a padded 32 x 33 tile in the (now idle) stage
        // memory, and the epilogue then runs with 8 threads per row, so every
        // store instruction writes whole 128-byte row segments and the bias and
        // pre-activation loads are coalesced too.
        float *tile = reinterpret_cast<float *>(tc_smem_raw + (base - raw)) + warp * 32 * 33;
        const uint32_t taddr = tmem + (static_cast<uint32_t>(warp * 32) << 16);
        float *cbase = g.C + (g.epi == TC_EPI_SPLITK ? static_cast<int64_t>(blockIdx.z) * g.M * g.N : 0);
        const bool vec_ok = (g.N % 4) == 0;
        for (int j0 = 0; j0 < g.BN; j0 += 32) {
            const int ncol = g.BN - j0 >= 32 ? 32 : 16;
            float v[32];
            if (ncol == 32) {
                tmem_ld32(taddr + static_cast<uint32_t>(j0), v);
            } else {
                float h[16];
                tmem_ld16(taddr + static_cast<uint32_t>(j0), h);
#pragma unroll
                for (int q = 0; q < 16; ++q) v[q] = h[q];
            }
            epilogue_group(g, tile, v, ncol, m0 + warp * 32, n0 + j0, cbase, vec_ok, lane);
            __syncwarp();  // the tile is rewritten by the next group
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(g.tmem_cols) : "memory");
}

// Persistent form of gemm_tc for the network's hidden-layer shapes: N <= 256
// (one column tile), K <= 256, and many 128-row tiles.  One CTA per SM walks
// the row tiles blockIdx.x, blockIdx.x + gridDim.x, ...  The whole B operand
// (BN x K, at most 128 KB) is loaded once per CTA and stays in shared memory;
// A streams through 16 KB stages (kForm 0, register stores: two -- with the
// epilogue on 24 warps a second stage measured 10 % faster than one, and a
// third does not fit beside B and the staging tiles; kForm 1: three; kForm 2:
// two).  Warp roles:
//   warp 0  TMA producer: B once, then A chunk by chunk, each stage refilled
//           once the MMAs that read it have completed (empty barrier);
//   warp 1  MMA issuer and TMEM owner: two accumulators of tmem_cols columns
//           (the whole 512-column TMEM at BN = 256), so that the epilogue of
//           tile i reads one accumulator while the MMAs of tile i + 1 fill the
//           other; tcgen05.commit signals a stage's release and an
//           accumulator's completion;
//   warps 2-25  epilogue (2-17 in kForms 1 and 2 below, four a quarter,
//           every fourth group): warp w reads TMEM lanes 32 (w mod 4) .. + 31 (the
//           lane quarter its position allows), i.e. those rows of the tile;
//           the six warps of a quarter take every sixth 16-column group (at
//           most three of a 256-column tile, where sixteen warps on 32-column
//           groups took two of 32: the epilogue's latency, not its issue,
//           sets the kernel's time).  Each applies the same epilogue as
//           gemm_tc (epilogue_group_w, 16-column staging tiles) and hands the
//           accumulator back (one arrival per warp).
// The MMAs of a tile accumulate the K chunks in gemm_tc's order and the
// epilogue performs the same operations, so the results are identical bit for
// bit.  Every wait is bounded; a wait that runs out records an error code, the
// waiting role stops, and the others then run out too; before the CTA frees
// its TMEM the producer waits for the copies it issued and the issuer for its
// MMAs.
//
// kForm 1, tensor stores (every epilogue but split-K, at N a multiple of 16
// with 16-byte aligned outputs, bias and pre): each lane applies the epilogue
// to its own row of the 16-column group in registers (DGELU reads the row's 16
// values of pre, 64 contiguous bytes) and writes it to the warp's staging
// tiles -- FP32 32 x 16 in the 64-byte swizzle layout, BF16 32 x 16 in the 32-byte one, so that the row
// writes are free of bank conflicts -- and one lane hands the tiles to the TMA
// unit as tensor stores (rows past M are not written).  The next group's
// TMEM load and arithmetic run while the store reads the tiles; the tiles are
// rewritten once it has (wait_group.read).  Per element the operations are
// those of epilogue_group_w, so the two forms agree bit for bit.  Sixteen
// warps suffice for it, and their 48 KB of tiles leave room for three A
// stages beside B (at 65536 x 256 x 256: 35.5 us with the 24-warp form, 33.4
// with this one on two stages, 31.4 on three; 12 or 20 warps no faster).
//
// kForm 2 adds the transposed BF16 output (N x M, the operand layout a
// weight gradient over the rows needs; at M a multiple of 8, because a tensor
// store writes the partial 16-byte chunk at the end of a row whole): each lane also writes its row's 16
// BF16 values down a column of a 16 x 32 staging tile (two-byte stores, the
// warp's lanes on consecutive elements) and a third tensor store writes the
// tile at (rows, columns) swapped.  Its 64 KB of tiles leave room for two A
// stages.
constexpr int PT_STAGES = 2;
constexpr int PT_STORE_STAGES = 3;
constexpr int PT_EPI_WARPS = 24;
constexpr int PT_STORE_EPI_WARPS = 16;
constexpr int PT_GROUP = 16;                       // accumulator columns an epilogue step takes
constexpr int PT_TILE_FLOATS = 32 * (PT_GROUP + 1);  // a warp's staging tile, 32 x 17 floats
constexpr int PT_STORE_TILE_BYTES = 32 * PT_GROUP * 4 + 32 * PT_GROUP * 2;  // FP32 + BF16 tiles, 3 KB
constexpr int PT_TRANS_TILE_BYTES = PT_STORE_TILE_BYTES + 1024;             // + the 16 x 32 BF16 transposed tile

// kForm: 0 register stores, 1 tensor stores, 2 tensor stores and the transposed BF16 output
template <int kForm>
__host__ __device__ constexpr int pt_epi_warps() {
    return kForm ? PT_STORE_EPI_WARPS : PT_EPI_WARPS;
}

template <int kForm>
__host__ __device__ constexpr int pt_stages() {
    return kForm == 1 ? PT_STORE_STAGES : PT_STAGES;
}

template <int kForm>
__host__ __device__ constexpr uint32_t pt_warp_tile_bytes() {
    return kForm == 2 ? PT_TRANS_TILE_BYTES : PT_STORE_TILE_BYTES;
}

template <int kForm>
__host__ __device__ constexpr size_t pt_tile_bytes() {
    return kForm ? static_cast<size_t>(PT_STORE_EPI_WARPS) * pt_warp_tile_bytes<kForm>()
                 : static_cast<size_t>(PT_EPI_WARPS) * PT_TILE_FLOATS * 4;
}

template <int kForm>
__global__ void __launch_bounds__(32 * (2 + pt_epi_warps<kForm>()), 1)
    gemm_tc_persistent(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b,
                       const __grid_constant__ CUtensorMap map_c, const __grid_constant__ CUtensorMap map_cb,
                       const __grid_constant__ CUtensorMap map_ct, TcArgs g) {
    constexpr bool kStore = kForm >= 1, kTrans = kForm == 2;
    constexpr int EW = pt_epi_warps<kForm>(), NS = pt_stages<kForm>();
    extern __shared__ uint8_t tc_smem_raw[];
    const uint32_t raw = smem_u32(tc_smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;
    const int nkc = static_cast<int>((g.K + TC_BK - 1) / TC_BK);  // K chunks (<= 4)
    const uint32_t b_chunk = static_cast<uint32_t>(g.BN) * TC_BK * 2;
    const uint32_t sB = base;                                       // nkc chunks of BN x 64
    const uint32_t sA = sB + static_cast<uint32_t>(nkc) * b_chunk;  // NS x 16 KB
    const uint32_t sT = sA + NS * TC_A_BYTES;  // the epilogue warps' staging tiles (1024-byte aligned)
    const uint32_t bars = sT + static_cast<uint32_t>(pt_tile_bytes<kForm>());
    // barriers: bfull | full[S] | empty[S] | tfull[2] | tempty[2] | done
    const uint32_t bfull = bars, full0 = bars + 8, empty0 = full0 + 8 * NS, tfull0 = empty0 + 8 * NS,
                   tempty0 = tfull0 + 16, done = tempty0 + 16;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(tc_smem_raw + (done + 8 - raw));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t n_tiles = (g.M + TC_BM - 1) / TC_BM;

    if (tid == 0) {
        mbar_init(bfull, 1);
        for (int s = 0; s < NS; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, 1);
        }
        for (int a = 0; a < 2; ++a) {
            mbar_init(tfull0 + 8 * a, 1);
            mbar_init(tempty0 + 8 * a, EW);
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(2 * g.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    // Work units, walked by all three roles in the same order (unit
    // blockIdx.x, + gridDim.x, ...): whole row tiles, except that when the
    // last wave would be at most half full (a BN = 256 tile, n_tiles mod
    // gridDim.x <= gridDim.x / 2), its tiles go as two 128-column halves --
    // one MMA of N = 128 over the matching half of B each -- so that the last
    // wave costs about half a tile.  half: -1 whole tile, 0 or 1 the column half.
    const int64_t grid = gridDim.x;
    const int64_t rem = n_tiles % grid;
    const bool split_last = g.BN == 256 && n_tiles > grid && rem > 0 && 2 * rem <= grid;
    const int64_t n_whole = split_last ? n_tiles - rem : n_tiles;
    const int64_t n_units = split_last ? n_whole + 2 * rem : n_tiles;
    auto unit = [&](int64_t u, int64_t &tile, int &half) {
        if (u < n_whole) {
            tile = u;
            half = -1;
        } else {
            tile = n_whole + (u - n_whole) / 2;
            half = static_cast<int>((u - n_whole) & 1);
        }
    };

    if (warp == 0) {
        if (lane == 0) {
            mbar_expect_tx(bfull, static_cast<uint32_t>(nkc) * b_chunk);
            for (int kc = 0; kc < nkc; ++kc) tma_load_2d(sB + kc * b_chunk, &map_b, kc * TC_BK, 0, bfull);
            uint32_t it = 0;
            bool ok = true;
            for (int64_t u = blockIdx.x; u < n_units && ok; u += grid) {
                int64_t tile;
                int half;
                unit(u, tile, half);
                for (int kc = 0; kc < nkc; ++kc, ++it) {
                    const uint32_t s = it % NS, use = it / NS;
                    if (use > 0 && !mbar_wait(empty0 + 8 * s, (use - 1) & 1)) {
                        record_error(5);
                        ok = false;
                        break;
                    }
                    mbar_expect_tx(full0 + 8 * s, TC_A_BYTES);
                    tma_load_2d(sA + s * TC_A_BYTES, &map_a, kc * TC_BK, static_cast<int32_t>(tile * TC_BM),
                                full0 + 8 * s);
                }
            }
            // every copy issued has landed before the CTA can leave
            for (uint32_t k = it > NS ? it - NS : 0; k < it; ++k)
                if (!mbar_wait(full0 + 8 * (k % NS), (k / NS) & 1)) record_error(6);
            if (!mbar_wait(bfull, 0)) record_error(6);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = idesc_bf16(g.BN), idesc_half = idesc_bf16(128);
            bool ok = mbar_wait(bfull, 0);
            if (!ok) record_error(7);
            uint32_t it = 0, tl = 0;
            for (int64_t u = blockIdx.x; u < n_units && ok; u += grid, ++tl) {
                int64_t tile;
                int half;
                unit(u, tile, half);
                // a column half reads B rows 128 half .. + 127: 128 rows of 128 bytes on
                const uint32_t b_off = half > 0 ? 128u * 128u : 0u;
                const uint32_t id = half < 0 ? idesc : idesc_half;
                const uint32_t a = tl & 1, use = tl >> 1;
                if (use > 0 && !mbar_wait(tempty0 + 8 * a, (use - 1) & 1)) {
                    record_error(8);
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t acc = tmem + a * static_cast<uint32_t>(g.tmem_cols);
                for (int kc = 0; kc < nkc; ++kc, ++it) {
                    const uint32_t s = it % NS;
                    if (!mbar_wait(full0 + 8 * s, (it / NS) & 1)) {
                        record_error(9);
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t sa = sA + s * TC_A_BYTES, sb = sB + kc * b_chunk + b_off;
                    const int64_t kcols = g.K - static_cast<int64_t>(kc) * TC_BK;
                    const int nk = kcols >= TC_BK ? TC_BK / 16 : static_cast<int>((kcols + 15) / 16);
                    for (int kk = 0; kk < nk; ++kk)
                        umma_bf16(acc, sdesc_sw128(sa + 32u * kk), sdesc_sw128(sb + 32u * kk), id,
                                  (kc > 0 || kk > 0) ? 1 : 0);
                    umma_commit(empty0 + 8 * s);
                }
                if (!ok) break;
                umma_commit(tfull0 + 8 * a);
            }
            umma_commit(done);  // arrives when every MMA issued above has completed
            if (!mbar_wait(done, 0)) record_error(10);
        }
    } else {
        // epilogue warps: TMEM lane quarter q, rows 32 q .. 32 q + 31 of each
        // tile; 16-column groups h, h + EW / 4, ...
        const int q = warp & 3, h = (warp - 2) / 4;
        float *tile_f = reinterpret_cast<float *>(tc_smem_raw + (sT - raw)) + (warp - 2) * PT_TILE_FLOATS;
        const uint32_t st_c = sT + static_cast<uint32_t>(warp - 2) * pt_warp_tile_bytes<kForm>(), st_b = st_c + 2048,
                       st_t = st_c + 3072;
        const bool vec_ok = (g.N % 4) == 0;
        uint32_t tl = 0;
        for (int64_t u = blockIdx.x; u < n_units; u += grid, ++tl) {
            int64_t tile;
            int half;
            unit(u, tile, half);
            const int ncols = half < 0 ? g.BN : 128, col_base = half > 0 ? 128 : 0;
            const uint32_t a = tl & 1, use = tl >> 1;
            // warp-uniform: the TMEM loads below are .sync.aligned
            const bool have = __all_sync(0xffffffffu, mbar_wait(tfull0 + 8 * a, use & 1));
            if (!have) {
                if (lane == 0) record_error(11);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t taddr =
                tmem + a * static_cast<uint32_t>(g.tmem_cols) + (static_cast<uint32_t>(q * 32) << 16);
            // (BN is a multiple of 16, the MMA's N granularity at M = 128)
            for (int j0 = PT_GROUP * h; j0 < ncols; j0 += PT_GROUP * (EW / 4)) {
                float v[PT_GROUP];
                if constexpr (kStore) {
                    const int col0 = col_base + j0;
                    const bool bias = g.epi == TC_EPI_BIAS_F32 || g.epi == TC_EPI_BIAS_GELU,
                               act = g.epi == TC_EPI_BIAS_GELU, dgelu = g.epi == TC_EPI_DGELU;
                    // DGELU: the lane's own row of pre (64 contiguous bytes), loaded
                    // before the TMEM load so that the two latencies overlap
                    float4 pp[4];
                    if (dgelu) {
                        const int64_t row = tile * TC_BM + q * 32 + lane;
                        const float4 *src = reinterpret_cast<const float4 *>(g.pre + row * g.N + col0);
#pragma unroll
                        for (int c = 0; c < 4; ++c) pp[c] = row < g.M ? __ldg(src + c) : make_float4(0.f, 0.f, 0.f, 0.f);
                    }
                    tmem_ld16(taddr + static_cast<uint32_t>(j0), v);
                    if (bias) {
#pragma unroll
                        for (int c = 0; c < 4; ++c) {
                            const float4 bb = __ldg(reinterpret_cast<const float4 *>(g.bias + col0) + c);
                            v[4 * c] += bb.x, v[4 * c + 1] += bb.y, v[4 * c + 2] += bb.z, v[4 * c + 3] += bb.w;
                        }
                    } else if (dgelu) {
#pragma unroll
                        for (int c = 0; c < 4; ++c) {
                            v[4 * c] *= gelu_grad(pp[c].x), v[4 * c + 1] *= gelu_grad(pp[c].y);
                            v[4 * c + 2] *= gelu_grad(pp[c].z), v[4 * c + 3] *= gelu_grad(pp[c].w);
                        }
                    }
                    uint32_t pb[PT_GROUP / 2];
                    if (act || dgelu) {
#pragma unroll
                        for (int k = 0; k < PT_GROUP / 2; ++k) {
                            __nv_bfloat162 t2 = act ? __floats2bfloat162_rn(gelu(v[2 * k]), gelu(v[2 * k + 1]))
                                                    : __floats2bfloat162_rn(v[2 * k], v[2 * k + 1]);
                            pb[k] = *reinterpret_cast<uint32_t *>(&t2);
                        }
                    }
                    // the previous group's stores have read the tiles
                    if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
                    __syncwarp();
                    // row `lane`: 64 bytes of FP32, 16-byte chunk c at c ^ (lane / 2 mod 4)
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        const uint32_t at = st_c + 64u * lane + ((static_cast<uint32_t>(c) ^ ((lane >> 1) & 3)) << 4);
                        asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(at), "f"(v[4 * c]),
                                     "f"(v[4 * c + 1]), "f"(v[4 * c + 2]), "f"(v[4 * c + 3])
                                     : "memory");
                    }
                    // 32 bytes of BF16, chunk c at c ^ (lane / 4 mod 2)
                    if (act || dgelu) {
#pragma unroll
                        for (int c = 0; c < 2; ++c) {
                            const uint32_t at = st_b + 32u * lane + ((static_cast<uint32_t>(c) ^ ((lane >> 2) & 1)) << 4);
                            asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(at), "r"(pb[4 * c]),
                                         "r"(pb[4 * c + 1]), "r"(pb[4 * c + 2]), "r"(pb[4 * c + 3])
                                         : "memory");
                        }
                    }
                    // the transposed tile: column k of the group is its row k (32
                    // BF16, 64 bytes), this lane's value at element `lane`
                    if (kTrans) {
#pragma unroll
                        for (int k = 0; k < PT_GROUP / 2; ++k) {
                            const uint32_t at = st_t + 2u * lane + 128u * k;
                            asm volatile("st.shared.u16 [%0], %1;" ::"r"(at), "h"(static_cast<uint16_t>(pb[k] & 0xffffu))
                                         : "memory");
                            asm volatile("st.shared.u16 [%0], %1;" ::"r"(at + 64u), "h"(static_cast<uint16_t>(pb[k] >> 16))
                                         : "memory");
                        }
                    }
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    __syncwarp();
                    // column sums of the block's rows below M (lane c: column c, rows in
                    // order), read from the FP32 tile beside the tensor store's read
                    if (g.col_part && lane < PT_GROUP) {
                        const int64_t r0 = tile * TC_BM + q * 32;
                        const int nr = g.M - r0 >= 32 ? 32 : static_cast<int>(g.M > r0 ? g.M - r0 : 0);
                        const uint32_t cq = static_cast<uint32_t>(lane >> 2), cw = static_cast<uint32_t>(lane & 3) * 4u;
                        float sum = 0.0f;
                        for (int r = 0; r < nr; ++r) {
                            float x;
                            asm volatile("ld.shared.f32 %0, [%1];"
                                         : "=f"(x)
                                         : "r"(st_c + 64u * r + ((cq ^ ((static_cast<uint32_t>(r) >> 1) & 3u)) << 4) + cw)
                                         : "memory");
                            sum += x;
                        }
                        g.col_part[(tile * 4 + q) * g.N + col0 + lane] = sum;
                    }
                    if (lane == 0) {
                        const int32_t y = static_cast<int32_t>(tile * TC_BM + q * 32);
                        tma_store_2d(&map_c, st_c, col0, y);
                        if (act || dgelu) tma_store_2d(&map_cb, st_b, col0, y);
                        if (kTrans) tma_store_2d(&map_ct, st_t, y, col0);
                        asm volatile("cp.async.bulk.commit_group;" ::: "memory");
                    }
                } else {
                    tmem_ld16(taddr + static_cast<uint32_t>(j0), v);
                    epilogue_group_w<PT_GROUP>(g, tile_f, v, PT_GROUP, tile * TC_BM + q * 32, col_base + j0, g.C,
                                               vec_ok, lane);
                    __syncwarp();  // the tile is rewritten by the next group
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(tempty0 + 8 * a);
        }
        // the tensor stores have completed before the CTA leaves
        if (kStore && lane == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * g.tmem_cols)
                     : "memory");
}

// dst[c][r] = src[r][c] for BF16 matrices (32 x 32 tiles through shared memory).
__global__ void transpose_bf16(const __nv_bfloat16 *__restrict__ src, int64_t rows, int64_t cols, int64_t ld_src,
                               __nv_bfloat16 *__restrict__ dst, int64_t ld_dst) {
    __shared__ __nv_bfloat16 t[32][33];
    const int64_t r0 = static_cast<int64_t>(blockIdx.y) * 32, c0 = static_cast<int64_t>(blockIdx.x) * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int64_t r = r0 + i, c = c0 + threadIdx.x;
        if (r < rows && c < cols) t[i][threadIdx.x] = src[r * ld_src + c];
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int64_t c = c0 + i, r = r0 + threadIdx.x;
        if (r < rows && c < cols) dst[c * ld_dst + r] = t[threadIdx.x][i];
    }
}

// dst[c][r] = src[r][c] for BF16 matrices of whole 64 x 64 tiles with 16-byte
// aligned rows: each row of a tile is read as eight 16-byte loads into a
// padded shared tile (rows of 144 bytes), and each thread writes 32
// contiguous bytes (one sector) of an output row, gathered down a column of
// the tile (the warp's lanes on 32 consecutive columns: conflict-free).  The
// 32 x 32 kernel above, two bytes per access, takes every other shape.
constexpr int TT_EDGE = 64;
constexpr int TT_PAD = 72;

__global__ void __launch_bounds__(256) transpose_bf16_64(const uint16_t *__restrict__ src, int64_t ld_src,
                                                         uint16_t *__restrict__ dst, int64_t ld_dst) {
    __shared__ __align__(16) uint16_t t[TT_EDGE][TT_PAD];
    const int64_t r0 = static_cast<int64_t>(blockIdx.y) * TT_EDGE, c0 = static_cast<int64_t>(blockIdx.x) * TT_EDGE;
    const int tid = threadIdx.x;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int r = tid / 8 + 32 * h, ch = tid % 8;
        const uint4 v = __ldg(reinterpret_cast<const uint4 *>(src + (r0 + r) * ld_src + c0) + ch);
        *reinterpret_cast<uint4 *>(&t[r][8 * ch]) = v;
    }
    __syncthreads();
    // tile column c -> output row c0 + c, its elements 16 p .. 16 p + 15
    const int lane = tid & 31, warp = tid >> 5;
    const int c = lane + 32 * (warp & 1), p = warp >> 1;
    uint32_t w[8];
#pragma unroll
    for (int k = 0; k < 8; ++k)
        w[k] = static_cast<uint32_t>(t[16 * p + 2 * k][c]) | (static_cast<uint32_t>(t[16 * p + 2 * k + 1][c]) << 16);
    uint4 *out = reinterpret_cast<uint4 *>(dst + (c0 + c) * ld_dst + r0 + 16 * p);
    out[0] = make_uint4(w[0], w[1], w[2], w[3]);
    out[1] = make_uint4(w[4], w[5], w[6], w[7]);
}

// out[m][n] = sum over splits of part[s][m][n]  (fixed order: deterministic)
__global__ void tc_splitk_reduce(const float *__restrict__ part, int splits, int64_t MN, float *__restrict__ out) {
    for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < MN;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        float s = 0.0f;
        for (int k = 0; k < splits; ++k) s += part[k * MN + e];
        out[e] = s;
    }
}

// The same sum for MN a multiple of 4 with 16-byte aligned buffers: a block
// takes 16 output quads (float4) with 16 split lanes each (lane t sums splits
// t, t + 16, ... in order), then the 16 lane sums in order -- a fixed order,
// with every thread's loads independent of one another.
constexpr int SK_LANES = 16;

__global__ void __launch_bounds__(256) tc_splitk_reduce4(const float4 *__restrict__ part, int splits, int64_t MN4,
                                                         float4 *__restrict__ out) {
    __shared__ float4 sm[SK_LANES][16];
    const int qd = threadIdx.x & 15, kl = threadIdx.x >> 4;
    const int64_t e = static_cast<int64_t>(blockIdx.x) * 16 + qd;
    float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (e < MN4)
        for (int k = kl; k < splits; k += SK_LANES) {
            const float4 v = __ldg(part + static_cast<int64_t>(k) * MN4 + e);
            acc.x += v.x, acc.y += v.y, acc.z += v.z, acc.w += v.w;
        }
    sm[kl][qd] = acc;
    __syncthreads();
    if (kl == 0 && e < MN4) {
        float4 t = sm[0][qd];
        for (int k = 1; k < SK_LANES; ++k) t.x += sm[k][qd].x, t.y += sm[k][qd].y, t.z += sm[k][qd].z, t.w += sm[k][qd].w;
        out[e] = t;
    }
}

// ---------------------------------------------------------------------------
// The learned proposal's whole autoregressive step for output mode j, fused:
// per tile of 128 chains, the 16 features (FP32, rounded to BF16 as the
// separate feature kernel does), the four layers 16 -> 256 -> 256 -> 256 -> 8
// on tcgen05 (BF16 operands, FP32 accumulation in TMEM) with the bias + GELU
// epilogues written back to shared memory as the next layer's A operand, and
// the masked-softmax draw in the last epilogue.  The same instructions and
// roundings as the separate kernels, so the patterns are the same bit for bit;
// what goes is five launches per mode and the activations' round trips
// through HBM.
//
// Shared memory (1024-aligned): the activation tile, 4 K-chunks of 128 rows x
// 128 bytes in the 128-byte swizzle (the features use chunk 0, K = 16), two
// 32 KB weight stages, then the barriers.  The weights (W1^T 256 x 16,
// W2^T and W3^T 256 x 256, W4^T 8 x 256, K-major) stream through the stages as
// 13 TMA chunks: one of W1, four each of W2, W3 and W4 (W4's 16-row boxes
// zero-fill rows 8..15, so the last layer runs with N = 16).
// 256 threads: warps 0-3 own the rows (thread t: row t) for the features and
// the draw; in the hidden-layer epilogues warp w reads TMEM lanes
// 32 (w % 4) .. + 31 and columns 128 (w / 4) .. + 127.
constexpr int PS_THREADS = 256;
constexpr uint32_t PS_ACT_CHUNK = TC_BM * 128;  // 16 KB
constexpr uint32_t PS_STAGE = 256 * 128;        // 32 KB
constexpr int PS_CHUNKS = 13;

struct PsArgs {
    int j, B, d, n;
    const float *ms;
    const float *bias[4];
    const uint64_t *seed_dev;
    uint64_t seed;
    int8_t *samples;
    int32_t *n_rem;
    float *shift;
    const float *C;
    float *logq;
};

// byte offset of (row r, k) in a 128-row activation chunk (128-byte swizzle:
// 16-byte piece k / 8 of row r sits at piece (k / 8) ^ (r % 8))
__device__ __forceinline__ uint32_t act_off(int r, int k) {
    return static_cast<uint32_t>((r >> 3) * 1024 + (r & 7) * 128 + ((((k >> 3) ^ (r & 7)) & 7) << 4) + (k & 7) * 2);
}

__global__ void __launch_bounds__(PS_THREADS, 1)
    proposal_step_tc(const __grid_constant__ CUtensorMap w1, const __grid_constant__ CUtensorMap w2,
                     const __grid_constant__ CUtensorMap w3, const __grid_constant__ CUtensorMap w4, PsArgs a) {
    using namespace pqg::prop;
    extern __shared__ uint8_t ps_smem_raw[];
    const uint32_t raw = smem_u32(ps_smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;
    uint8_t *gbase = ps_smem_raw + (base - raw);
    const uint32_t act = base, wst = base + 4 * PS_ACT_CHUNK;
    const uint32_t bar0 = wst + 2 * PS_STAGE;  // full[2] at +0/+8, empty[2] at +16/+24, done at +32
    const uint32_t full0 = bar0, empty0 = bar0 + 16, done = bar0 + 32;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(gbase + (bar0 + 40 - base));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * TC_BM;

    if (tid == 0) {
        for (int s = 0; s < 2; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, 1);
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(256)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }

    // weight chunk g: its map, K offset and bytes
    auto issue = [&](int g) {
        const int s = g & 1;
        const CUtensorMap *m = g == 0 ? &w1 : (g < 5 ? &w2 : (g < 9 ? &w3 : &w4));
        const int c = g == 0 ? 0 : (g - 1) & 3;
        const uint32_t bytes = g < 9 ? PS_STAGE : 16 * 128;
        mbar_expect_tx(full0 + 8 * s, bytes);
        tma_load_2d(wst + s * PS_STAGE, m, 64 * c, 0, full0 + 8 * s);
    };
    int issued = 0, consumed = 0;  // thread 0's TMA bookkeeping
    if (tid == 0) {
        issue(0);
        issue(1);
        issued = 2;
    }

    // features of this thread's row, into activation chunk 0 (K = 16)
    int lo = 0, hi = 0;
    const int b = m0 + tid;
    if (tid < TC_BM) {
        float x[kF];
        if (b < a.B) {
            features(a.j, a.d, a.n, a.ms, a.n_rem[b], a.shift[static_cast<int64_t>(b) * a.d + a.j], x, lo, hi);
        } else {
#pragma unroll
            for (int k = 0; k < kF; ++k) x[k] = 0.0f;
        }
#pragma unroll
        for (int p = 0; p < 2; ++p) {
            uint4 w;
            uint32_t *wv = reinterpret_cast<uint32_t *>(&w);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                __nv_bfloat162 v = __floats2bfloat162_rn(x[8 * p + 2 * q], x[8 * p + 2 * q + 1]);
                wv[q] = *reinterpret_cast<uint32_t *>(&v);
            }
            *reinterpret_cast<uint4 *>(gbase + act_off(tid, 8 * p)) = w;
        }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    bool ok = true;   // thread 0: every wait so far succeeded
    bool have = true; // every thread: every layer's accumulators arrived
    for (int layer = 0; layer < 4; ++layer) {
        const int bn = layer < 3 ? 256 : 16;
        if (tid == 0) {
            const int g0 = layer == 0 ? 0 : 1 + 4 * (layer - 1), nch = layer == 0 ? 1 : 4;
            const uint32_t idesc = idesc_bf16(bn);
            for (int c = 0; c < nch && ok; ++c) {
                const int g = g0 + c, s = g & 1;
                const uint32_t parity = static_cast<uint32_t>((g >> 1) & 1);
                if (!mbar_wait(full0 + 8 * s, parity)) {
                    record_error(11);
                    ok = false;
                    break;
                }
                consumed = g + 1;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const int nk = layer == 0 ? 1 : 4;  // K = 16 per instruction
                for (int kk = 0; kk < nk; ++kk)
                    umma_bf16(tmem, sdesc_sw128(act + c * PS_ACT_CHUNK + 32u * kk),
                              sdesc_sw128(wst + s * PS_STAGE + 32u * kk), idesc, (c > 0 || kk > 0) ? 1 : 0);
                umma_commit(empty0 + 8 * s);
                if (g + 2 < PS_CHUNKS) {
                    // the stage is refilled once these MMAs have read it
                    if (!mbar_wait(empty0 + 8 * s, parity)) {
                        record_error(12);
                        ok = false;
                        break;
                    }
                    issue(g + 2);
                    issued = g + 3;
                }
            }
            umma_commit(done);  // arrives when every MMA issued so far has completed
        }
        __syncwarp();
        const bool arrived = __all_sync(0xffffffffu, mbar_wait(done, static_cast<uint32_t>(layer & 1)));
        if (!arrived && lane == 0) record_error(13);
        have = have && arrived;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int q = warp & 3;
        const uint32_t taddr = tmem + (static_cast<uint32_t>(q * 32) << 16);
        const int r = q * 32 + lane;
        if (layer < 3) {
            // bias + GELU, BF16, into the activation tile (row r, 128 columns)
            if (have) {
                const float *bias = a.bias[layer];
                const int c0 = (warp >> 2) * 128;
                for (int j0 = c0; j0 < c0 + 128; j0 += 32) {
                    float v[32];
                    tmem_ld32(taddr + static_cast<uint32_t>(j0), v);
#pragma unroll
                    for (int p = 0; p < 4; ++p) {
                        uint4 w;
                        uint32_t *wv = reinterpret_cast<uint32_t *>(&w);
#pragma unroll
                        for (int h = 0; h < 4; ++h) {
                            const int col = j0 + 8 * p + 2 * h;
                            const float y0 = v[8 * p + 2 * h] + bias[col];
                            const float y1 = v[8 * p + 2 * h + 1] + bias[col + 1];
                            __nv_bfloat162 t = __floats2bfloat162_rn(gelu(y0), gelu(y1));
                            wv[h] = *reinterpret_cast<uint32_t *>(&t);
                        }
                        const int k = (j0 & 63) + 8 * p;
                        *reinterpret_cast<uint4 *>(gbase + (j0 >> 6) * PS_ACT_CHUNK + act_off(r, k)) = w;
                    }
                }
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncthreads();
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        } else if (warp < 4 && have) {
            // logits (8 of the 16 columns) + bias, then the draw of row r
            float v[16];
            tmem_ld16(taddr, v);
            float z[kLD];
#pragma unroll
            for (int c = 0; c < kLD; ++c) z[c] = v[c] + a.bias[3][c];
            if (b < a.B) {
                const uint64_t seed = a.seed_dev ? *a.seed_dev : a.seed;
                draw(a.j, b, a.d, z, lo, hi, seed, a.samples, a.n_rem, a.shift, a.C, a.ms, a.logq);
            }
        }
    }
    // copies still in flight after a failed wait: wait for them (bounded)
    // before the shared memory goes away
    if (tid == 0) {
        for (int g = consumed; g < issued; ++g)
            if (!mbar_wait(full0 + 8 * (g & 1), static_cast<uint32_t>((g >> 1) & 1))) record_error(14);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(256) : "memory");
}

int fail(int code, const char *msg) {
    pqg::set_last_error(msg);
    return code;
}

int fail_cuda(cudaError_t e, const char *what) {
    char buf[200];
    snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    pqg::set_last_error(buf);
    return PQG_ERR_CUDA;
}

// The catch clause of the entry points below that take a std::call_once (and
// set the error text through a std::string): no C++ exception crosses the C ABI.
int host_failure(const char *what) noexcept {
    try {
        pqg::set_last_error(what);
    } catch (...) {
    }
    return PQG_ERR_HOST;
}

// SM count of the current device (0 if it cannot be read), looked up once.
int device_sms() {
    static std::once_flag once;
    static int sms = 0;
    std::call_once(once, [] {
        int dev = 0, n = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess)
            sms = n;
    });
    return sms;
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// Tensor map of a row-major BF16 matrix [rows x k] with row stride ld
// (elements), boxes of 64 (K) x box_rows, 128-byte swizzle, zero fill.
int make_map(CUtensorMap *map, const void *p, int64_t rows, int64_t k, int64_t ld, int box_rows) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
    if (!enc) return fail(PQG_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
    const cuuint64_t dims[2] = {static_cast<cuuint64_t>(k), static_cast<cuuint64_t>(rows)};
    const cuuint64_t strides[1] = {static_cast<cuuint64_t>(ld) * 2};
    const cuuint32_t box[2] = {static_cast<cuuint32_t>(TC_BK), static_cast<cuuint32_t>(box_rows)};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(p), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        char buf[160];
        snprintf(buf, sizeof(buf), "cuTensorMapEncodeTiled failed (%d) for a %lld x %lld operand", static_cast<int>(r),
                 static_cast<long long>(rows), static_cast<long long>(k));
        return fail(PQG_ERR_INVALID, buf);
    }
    return PQG_OK;
}

// Tensor map of the row-major output [rows x cols] (dense rows: stride cols
// elements, FP32 or BF16) for the persistent kernel's tensor stores: boxes of
// 16 columns x 32 rows, in the staging tiles' swizzle (64 bytes for FP32, 32
// for BF16: one box row).
int make_store_map(CUtensorMap *map, void *p, int64_t rows, int64_t cols, bool bf16) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
    if (!enc) return fail(PQG_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
    const cuuint64_t dims[2] = {static_cast<cuuint64_t>(cols), static_cast<cuuint64_t>(rows)};
    const cuuint64_t strides[1] = {static_cast<cuuint64_t>(cols) * (bf16 ? 2 : 4)};
    const cuuint32_t box[2] = {static_cast<cuuint32_t>(PT_GROUP), 32};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, p, dims,
                     strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     bf16 ? CU_TENSOR_MAP_SWIZZLE_32B : CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        char buf[160];
        snprintf(buf, sizeof(buf), "cuTensorMapEncodeTiled failed (%d) for a %lld x %lld output", static_cast<int>(r),
                 static_cast<long long>(rows), static_cast<long long>(cols));
        return fail(PQG_ERR_INVALID, buf);
    }
    return PQG_OK;
}

// Tensor map of the transposed BF16 output [cols x rows] (row stride ld
// elements, a multiple of 8) for the kForm 2 stores: boxes of 32 rows of the
// GEMM (the inner coordinate) x 16 columns, unswizzled 64-byte box rows.
int make_trans_map(CUtensorMap *map, void *p, int64_t rows, int64_t cols, int64_t ld) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
    if (!enc) return fail(PQG_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
    const cuuint64_t dims[2] = {static_cast<cuuint64_t>(rows), static_cast<cuuint64_t>(cols)};
    const cuuint64_t strides[1] = {static_cast<cuuint64_t>(ld) * 2};
    const cuuint32_t box[2] = {32, static_cast<cuuint32_t>(PT_GROUP)};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, p, dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        char buf[160];
        snprintf(buf, sizeof(buf), "cuTensorMapEncodeTiled failed (%d) for a %lld x %lld transposed output",
                 static_cast<int>(r), static_cast<long long>(cols), static_cast<long long>(rows));
        return fail(PQG_ERR_INVALID, buf);
    }
    return PQG_OK;
}

template <int kForm>
int launch_persistent(const CUtensorMap &ma, const CUtensorMap &mb, const CUtensorMap &mc, const CUtensorMap &mcb,
                      const CUtensorMap &mct, const TcArgs &g, int sms, cudaStream_t s) {
    const size_t psmem = 1024 + static_cast<size_t>((g.K + TC_BK - 1) / TC_BK) * g.BN * TC_BK * 2 +
                         pt_stages<kForm>() * static_cast<size_t>(TC_A_BYTES) + pt_tile_bytes<kForm>() + 128;
    static std::once_flag pattr_once;
    static cudaError_t pattr_err = cudaSuccess;
    std::call_once(pattr_once, [] {
        pattr_err = cudaFuncSetAttribute(gemm_tc_persistent<kForm>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         227 * 1024);
    });
    if (pattr_err != cudaSuccess) return fail_cuda(pattr_err, "pqg_mlp_gemm_tc (shared memory attribute)");
    gemm_tc_persistent<kForm>
        <<<static_cast<unsigned>(sms), 32 * (2 + pt_epi_warps<kForm>()), psmem, s>>>(ma, mb, mc, mcb, mct, g);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PQG_OK : fail_cuda(e, "pqg_mlp_gemm_tc");
}

// dst (cols x ld_dst) = src (rows x cols, row stride ld_src)^T, BF16: the
// 64 x 64 kernel for whole aligned tiles, else the 32 x 32 one.
int transpose_launch(const void *src, int64_t rows, int64_t cols, int64_t ld_src, void *dst, int64_t ld_dst,
                     cudaStream_t s) {
    const bool tiles64 = rows % TT_EDGE == 0 && cols % TT_EDGE == 0 && rows / TT_EDGE <= 65535 && ld_src % 8 == 0 &&
                         ld_dst % 8 == 0 && (reinterpret_cast<uintptr_t>(src) & 15u) == 0 &&
                         (reinterpret_cast<uintptr_t>(dst) & 15u) == 0;
    if (tiles64) {
        dim3 grid(static_cast<unsigned>(cols / TT_EDGE), static_cast<unsigned>(rows / TT_EDGE));
        transpose_bf16_64<<<grid, 256, 0, s>>>(static_cast<const uint16_t *>(src), ld_src,
                                                static_cast<uint16_t *>(dst), ld_dst);
    } else {
        dim3 grid(static_cast<unsigned>((cols + 31) / 32), static_cast<unsigned>((rows + 31) / 32));
        transpose_bf16<<<grid, dim3(32, 8), 0, s>>>(static_cast<const __nv_bfloat16 *>(src), rows, cols, ld_src,
                                                     static_cast<__nv_bfloat16 *>(dst), ld_dst);
    }
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PQG_OK : fail_cuda(e, "pqg_mlp_transpose_bf16");
}

// The GEMM behind both entry points; c_bf16_t (nullable): the transposed
// BF16 output, N x M with row stride ld_t.
int gemm_tc_impl(const void *a, int64_t lda, const void *b, int64_t ldb, int64_t M, int64_t N, int64_t K,
                 int32_t epilogue, float *c, void *c_bf16, const float *bias, const float *pre, float *splitk_scratch,
                 int32_t splits, void *c_bf16_t, int64_t ld_t, float *col_sums, float *col_scratch, void *stream) {
    if (M <= 0 || N <= 0 || K <= 0 || !a || !b || !c || lda < K || ldb < K || epilogue < 0 || epilogue > 4)
        return fail(PQG_ERR_INVALID, "pqg_mlp_gemm_tc: invalid arguments");
    if ((lda % 8) || (ldb % 8) || (reinterpret_cast<uintptr_t>(a) % 16) || (reinterpret_cast<uintptr_t>(b) % 16))
        return fail(PQG_ERR_INVALID, "pqg_mlp_gemm_tc: operands need 16-byte aligned rows (ld % 8 == 0)");
    if ((epilogue == TC_EPI_BIAS_GELU || epilogue == TC_EPI_BIAS_F32) && !bias)
        return fail(PQG_ERR_INVALID, "pqg_mlp_gemm_tc: epilogue needs a bias");
    if ((epilogue == TC_EPI_BIAS_GELU || epilogue == TC_EPI_DGELU) && !c_bf16)
        return fail(PQG_ERR_INVALID, "pqg_mlp_gemm_tc: epilogue needs a BF16 output");
    if (epilogue == TC_EPI_DGELU && !pre) return fail(PQG_ERR_INVALID, "pqg_mlp_gemm_tc: epilogue needs pre");
    if (M >= (1ll << 31) || N >= (1ll << 31) || K >= (1ll << 31) || (M + TC_BM - 1) / TC_BM > 65535)
        return fail(PQG_ERR_TOO_LARGE, "pqg_mlp_gemm_tc: dimension too large");
    TcArgs g{};
    g.M = M;
    g.N = N;
    g.K = K;
    g.C = c;
    g.Cb = static_cast<__nv_bfloat16 *>(c_bf16);
    g.bias = bias;
    g.pre = pre;
    g.epi = epilogue;
    g.BN = static_cast<int>(((N < 256 ? N : 256) + 15) / 16 * 16);
    g.tmem_cols = 32;
    while (g.tmem_cols < g.BN) g.tmem_cols *= 2;
    int nsplit = 1;
    g.k_per_split = (K + TC_BK - 1) / TC_BK * TC_BK;
    if (epilogue == TC_EPI_SPLITK) {
        if (splits < 1 || !splitk_scratch)
            return fail(PQG_ERR_INVALID, "pqg_mlp_gemm_tc: split-K needs splits >= 1 and a scratch buffer");
        int64_t kps = (K + splits - 1) / splits;
        kps = (kps + TC_BK - 1) / TC_BK * TC_BK;
        g.k_per_split = kps;
        nsplit = static_cast<int>((K + kps - 1) / kps);
        g.C = splitk_scratch;
    }
    CUtensorMap ma, mb;
    int st = make_map(&ma, a, M, K, lda, TC_BM);
    if (st) return st;
    st = make_map(&mb, b, N, K, ldb, g.BN);
    if (st) return st;
    // shared memory: the stages, the barriers (16 bytes a stage, 8 for done,
    // the TMEM slot: at most 76 bytes), and the slack that aligns the stages
    // to 1024 bytes; a CTA holding 256 TMEM columns asks for enough shared
    // memory that at most two share an SM (512 columns)
    const int stages = epilogue == TC_EPI_SPLITK ? TC_SPLITK_STAGES : TC_STAGES;
    size_t smem = 1024 + stages * (static_cast<size_t>(TC_A_BYTES) + static_cast<size_t>(g.BN) * TC_BK * 2) + 128;
    if (g.tmem_cols > 128 && smem < 80 * 1024) smem = 80 * 1024;
    static std::once_flag attr_once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(attr_once, [] {
        attr_err = cudaFuncSetAttribute(gemm_tc<TC_STAGES>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        if (attr_err == cudaSuccess)
            attr_err = cudaFuncSetAttribute(gemm_tc<TC_SPLITK_STAGES>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            200 * 1024);
    });
    if (attr_err != cudaSuccess) return fail_cuda(attr_err, "pqg_mlp_gemm_tc (shared memory attribute)");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // many row tiles of one column tile with the whole B in shared memory:
    // the persistent kernel, one CTA per SM
    const int64_t row_tiles = (M + TC_BM - 1) / TC_BM;
    const int sms = device_sms();
    if (epilogue != TC_EPI_SPLITK && N <= 256 && K <= 256 && sms > 0 && row_tiles >= 2 * sms) {
        // tensor stores where the outputs allow them: 16-column groups that
        // end inside the rows, 16-byte aligned bases (and bias, read as float4)
        const auto al16 = [](const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; };
        const bool bf16_out = epilogue == TC_EPI_BIAS_GELU || epilogue == TC_EPI_DGELU;
        const bool store = N % PT_GROUP == 0 && al16(c) &&
                           ((epilogue != TC_EPI_BIAS_F32 && epilogue != TC_EPI_BIAS_GELU) || al16(bias)) &&
                           (!bf16_out || al16(c_bf16)) && (epilogue != TC_EPI_DGELU || al16(pre));
        if (store) {
            CUtensorMap mc, mcb, mct;
            st = make_store_map(&mc, c, M, N, false);
            if (st) return st;
            mcb = mc;
            if (bf16_out) {
                st = make_store_map(&mcb, c_bf16, M, N, true);
                if (st) return st;
            }
            // column sums from the epilogue: per 32-row block, then the blocks in order
            if (col_sums) g.col_part = col_scratch;
            // a tensor store writes a partial 16-byte chunk at the end of a row
            // whole (measured: the seven padding columns of M = 50001 were
            // written), so the transposed rows, M long, take it at M % 8 == 0
            const bool trans = c_bf16_t && al16(c_bf16_t) && M % 8 == 0;
            if (trans) {
                st = make_trans_map(&mct, c_bf16_t, M, N, ld_t);
                if (st) return st;
                st = launch_persistent<2>(ma, mb, mc, mcb, mct, g, sms, s);
            } else {
                st = launch_persistent<1>(ma, mb, mc, mcb, mc, g, sms, s);
            }
            if (!st && col_sums) st = pqg::mlp_column_sums_final(col_scratch, row_tiles * 4, N, col_sums, s);
            if (st || trans || !c_bf16_t) return st;
            return transpose_launch(c_bf16, M, N, N, c_bf16_t, ld_t, s);
        }
        st = launch_persistent<0>(ma, mb, ma, ma, ma, g, sms, s);
        if (!st && col_sums) st = pqg_mlp_bias_grad(c, M, N, col_sums, col_scratch, stream);
        if (st || !c_bf16_t) return st;
        return transpose_launch(c_bf16, M, N, N, c_bf16_t, ld_t, s);
    }
    dim3 grid(static_cast<unsigned>((N + g.BN - 1) / g.BN), static_cast<unsigned>((M + TC_BM - 1) / TC_BM),
              static_cast<unsigned>(nsplit));
    if (stages == TC_SPLITK_STAGES)
        gemm_tc<TC_SPLITK_STAGES><<<grid, TC_THREADS, smem, s>>>(ma, mb, g);
    else
        gemm_tc<TC_STAGES><<<grid, TC_THREADS, smem, s>>>(ma, mb, g);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail_cuda(e, "pqg_mlp_gemm_tc");
    if (epilogue == TC_EPI_SPLITK) {
        const int64_t MN = M * N;
        if (MN % 4 == 0 && (reinterpret_cast<uintptr_t>(splitk_scratch) & 15u) == 0 &&
            (reinterpret_cast<uintptr_t>(c) & 15u) == 0 && (MN / 4 + 15) / 16 <= 0x7fffffff)
            tc_splitk_reduce4<<<static_cast<unsigned>((MN / 4 + 15) / 16), 256, 0, s>>>(
                reinterpret_cast<const float4 *>(splitk_scratch), nsplit, MN / 4, reinterpret_cast<float4 *>(c));
        else
            tc_splitk_reduce<<<256, 256, 0, s>>>(splitk_scratch, nsplit, MN, c);
        e = cudaGetLastError();
        if (e != cudaSuccess) return fail_cuda(e, "pqg_mlp_gemm_tc (split-K reduction)");
    }
    if (col_sums) {
        const int cs = pqg_mlp_bias_grad(c, M, N, col_sums, col_scratch, stream);
        if (cs) return cs;
    }
    if (c_bf16_t) return transpose_launch(c_bf16, M, N, N, c_bf16_t, ld_t, s);
    return PQG_OK;
}

}  // namespace

extern "C" {

int pqg_mlp_gemm_tc(const void *a, int64_t lda, const void *b, int64_t ldb, int64_t M, int64_t N, int64_t K,
                    int32_t epilogue, float *c, void *c_bf16, const float *bias, const float *pre,
                    float *splitk_scratch, int32_t splits, void *stream) try {
    return gemm_tc_impl(a, lda, b, ldb, M, N, K, epilogue, c, c_bf16, bias, pre, splitk_scratch, splits, nullptr, 0,
                        nullptr, nullptr, stream);
} catch (...) {
    return host_failure("pqg_mlp_gemm_tc: host-side failure");
}

int pqg_mlp_gemm_tc_t(const void *a, int64_t lda, const void *b, int64_t ldb, int64_t M, int64_t N, int64_t K,
                      int32_t epilogue, float *c, void *c_bf16, const float *bias, const float *pre, void *c_bf16_t,
                      int64_t ld_t, float *col_sums, float *col_scratch, void *stream) try {
    if ((epilogue != TC_EPI_BIAS_GELU && epilogue != TC_EPI_DGELU) || !c_bf16_t || ld_t < M || ld_t % 8)
        return fail(PQG_ERR_INVALID,
                    "pqg_mlp_gemm_tc_t: needs a BF16 epilogue (1 or 4) and a transposed output with ld_t >= M, "
                    "ld_t % 8 == 0");
    if (col_sums && !col_scratch)
        return fail(PQG_ERR_INVALID, "pqg_mlp_gemm_tc_t: column sums need a scratch of 4 ceil(M/128) N floats");
    return gemm_tc_impl(a, lda, b, ldb, M, N, K, epilogue, c, c_bf16, bias, pre, nullptr, 0, c_bf16_t, ld_t,
                        col_sums, col_scratch, stream);
} catch (...) {
    return host_failure("pqg_mlp_gemm_tc_t: host-side failure");
}

int pqg_mlp_transpose_bf16(const void *src, int64_t rows, int64_t cols, int64_t ld_src, void *dst, int64_t ld_dst,
                           void *stream) {
    if (rows <= 0 || cols <= 0 || !src || !dst || ld_src < cols || ld_dst < rows)
        return fail(PQG_ERR_INVALID, "pqg_mlp_transpose_bf16: invalid arguments");
    return transpose_launch(src, rows, cols, ld_src, dst, ld_dst, static_cast<cudaStream_t>(stream));
}

int pqg_proposal_step_tc(int32_t j, int32_t B, int32_t d, int32_t n, const float *mode_stats, const void *w1t,
                         const void *w2t, const void *w3t, const void *w4t, const float *b1, const float *b2,
                         const float *b3, const float *b4, uint64_t seed, const uint64_t *seed_dev, int8_t *samples,
                         int32_t *n_rem, float *shift, const float *C, float *logq, void *stream) try {
    if (B <= 0 || d <= 0 || n <= 0 || j < 0 || j >= d || !mode_stats || !w1t || !w2t || !w3t || !w4t || !b1 ||
        !b2 || !b3 || !b4 || !samples || !n_rem || !shift || !C || !logq)
        return fail(PQG_ERR_INVALID, "pqg_proposal_step_tc: invalid arguments");
    for (const void *p : {w1t, w2t, w3t, w4t})
        if (reinterpret_cast<uintptr_t>(p) % 16)
            return fail(PQG_ERR_INVALID, "pqg_proposal_step_tc: weights need 16-byte alignment");
    CUtensorMap m1, m2, m3, m4;
    int st = make_map(&m1, w1t, 256, 16, 16, 256);
    if (!st) st = make_map(&m2, w2t, 256, 256, 256, 256);
    if (!st) st = make_map(&m3, w3t, 256, 256, 256, 256);
    if (!st) st = make_map(&m4, w4t, 8, 256, 256, 16);
    if (st) return st;
    PsArgs g{};
    g.j = j;
    g.B = B;
    g.d = d;
    g.n = n;
    g.ms = mode_stats;
    g.bias[0] = b1;
    g.bias[1] = b2;
    g.bias[2] = b3;
    g.bias[3] = b4;
    g.seed_dev = seed_dev;
    g.seed = seed;
    g.samples = samples;
    g.n_rem = n_rem;
    g.shift = shift;
    g.C = C;
    g.logq = logq;
    const size_t smem = 1024 + 4 * PS_ACT_CHUNK + 2 * PS_STAGE + 64;
    static std::once_flag attr_once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(attr_once, [smem] {
        attr_err = cudaFuncSetAttribute(proposal_step_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        static_cast<int>(smem));
    });
    if (attr_err != cudaSuccess) return fail_cuda(attr_err, "pqg_proposal_step_tc (shared memory attribute)");
    proposal_step_tc<<<static_cast<unsigned>((B + TC_BM - 1) / TC_BM), PS_THREADS, smem,
                       static_cast<cudaStream_t>(stream)>>>(m1, m2, m3, m4, g);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PQG_OK : fail_cuda(e, "pqg_proposal_step_tc");
} catch (...) {
    return host_failure("pqg_proposal_step_tc: host-side failure");
}

int pqg_mlp_tc_status(int32_t *code) {
    int v = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&v, g_tc_error, sizeof(int));
    if (e != cudaSuccess) return fail_cuda(e, "pqg_mlp_tc_status");
    if (code) *code = v;
    if (v) {
        const int zero = 0;
        e = cudaMemcpyToSymbol(g_tc_error, &zero, sizeof(int));
        if (e != cudaSuccess) return fail_cuda(e, "pqg_mlp_tc_status");
    }
    return PQG_OK;
}

}  // extern "C"
