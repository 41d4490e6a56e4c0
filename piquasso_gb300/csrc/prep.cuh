// Device construction of every problem's walk data from the plan's matrix.
//
// The host uploads one matrix (FP64, interleaved complex, row-major) and, per
// problem, the matrix rows of its digits and the matrix columns it keeps
// (PqgProblem::off_idx).  This kernel builds, in the walk's precision:
//   * the DF column scales 2^-e_j with B_j = |a0_j|_1 + sum_i m_i |a_ij|_1 in
//     [2^(e_j-1), 2^e_j) (|z|_1 = |re z| + |im z| >= |z|, a bound as good as
//     the modulus to within one power of two, and cheap), so no double-float
//     column sum exceeds 1 in magnitude
//     (powers of two are exact; sum_j e_j cm_j goes to col_shift and is
//     multiplied back in the final scaling, and each e_j to col_e, which a
//     Laplace output lacking one factor of column j takes off again);
//   * the seeds, the column sums with every digit at 0: a0 + sum_i m_i a_i,
//     TwoSum-compensated in FP64;
//   * the outer digits' rows a_o, and the one-digit update rows -2 a_o / +2 a_o;
//   * the prefix table Delta(t)_j = sum_k -2 g_k(t) a_kj over the inner codes,
//     as the sum of two sub-tables over two groups of the inner digits.
// A neutral padding column (index -1) has a0 = 1 and zero rows.
//
// Work split: `slices` blocks per problem; every block of a problem computes
// the (cheap) column scales, slice 0 writes the seeds and rows, all slices
// share the prefix table's tiles of codes.  The grid loops over (problem,
// slice).  Launched with 256 threads (one per code of a tile).
#pragma once
#include "walk_df.cuh"

namespace pqg {

enum PrepFormat : int { PREP_F64 = 0, PREP_F32 = 1, PREP_DF = 2 };

// Sub-table rows (both groups) above which the prefix table is built term by
// term instead (PL + PH > 56 needs P > 700 with the best split).
#define PREP_SUB_MAX 56

struct PrepArgs {
    PqgProblem *probs;
    unsigned char *arena;
    void *delta;
    int64_t matrix_off;  // byte offset of the matrix in the arena
    int64_t mat_cols;
    int32_t n_probs;
    int32_t slices;
    int32_t dup;    // PREP_F32 only: table entries {re, re, im, im} (the packed two-seed walk)
    int32_t pairs;  // PREP_F32 only: code pairs, float4 {re_2u, re_2u+1, im_2u, im_2u+1} per column
                    // (an odd P gets a zero pad code)
};

// A scaled matrix entry of the double-float walk rounded to a multiple of
// 2^-47 (|x| < 1; x * 2^47 and back are exact).  Every seed, update row and
// prefix-table entry is then a sum of such entries below 2 in magnitude,
// itself a multiple of 2^-47: its high word on the walk's 2^-23 grid and the
// rest (at most 2^-24, 23 bits) are exact floats, and the walk's column sums
// and seed updates are exact (walk_df.cuh).  The one rounding is this one, at
// most 2^-48 per scaled entry, and it is consistent: the walk sums the
// permanent of the rounded matrix.
__device__ __forceinline__ double q47(double x) {
    return rint(x * 140737488355328.0) * 7.1054273576010019e-15;
}

__device__ __forceinline__ void split_df(double x, float &hi, float &lo) {
    hi = __double2float_rn(x);
    lo = __double2float_rn(x - static_cast<double>(hi));
}

// Reflected mixed-radix Gray code of inner code t (< P <= 2^15): the same
// code as gray_decode, in 32-bit arithmetic.
__device__ __forceinline__ void gray_decode_inner(const uint8_t *__restrict__ m, int n, uint32_t t, uint8_t *g) {
    uint8_t c[PQG_MAX_INNER];
    for (int k = 0; k < n; ++k) {
        const uint32_t L = m[k] + 1u;
        const uint32_t q = t / L;
        c[k] = static_cast<uint8_t>(t - q * L);
        t = q;
    }
    int parity = 0;
    for (int k = n - 1; k >= 0; --k) {
        const int L = m[k] + 1;
        const int code = parity ? L - 1 - c[k] : c[k];
        g[k] = static_cast<uint8_t>(code);
        parity ^= (code & 1);
    }
}

template <int FMT>
__global__ void __launch_bounds__(256) prep_problems(PrepArgs A) {
    __shared__ int rowix[1 + PQG_MAX_OUTER + PQG_MAX_INNER];
    __shared__ int colix[PQG_MAX_COLS];
    __shared__ double cscale[PQG_MAX_COLS];
    __shared__ int eshift[PQG_MAX_COLS];
    __shared__ double2 inrow[PQG_MAX_INNER][PQG_MAX_COLS];  // inner digits' rows (unscaled; unsplit tables)
    __shared__ double2 subtab[PREP_SUB_MAX][PQG_MAX_COLS];   // DL then DH (unscaled; split tables)
    __shared__ uint8_t gt[256][PQG_MAX_INNER];               // Gray digits of a tile's codes
    __shared__ int16_t gix[256][2];                          // their sub-table rows
    const double *mat = reinterpret_cast<const double *>(A.arena + A.matrix_off);
    const int64_t total = static_cast<int64_t>(A.n_probs) * A.slices;
    for (int64_t vb = blockIdx.x; vb < total; vb += gridDim.x) {
        const int ip = static_cast<int>(vb / A.slices);
        const int slice = static_cast<int>(vb - static_cast<int64_t>(ip) * A.slices);
        PqgProblem *pr = A.probs + ip;
        if (pr->kind != PQG_KIND_WALK) continue;  // uniform over the block
        const int nc = pr->nc, no = pr->n_outer, K = pr->K;
        const int nd = no + K;
        const int32_t *idx = reinterpret_cast<const int32_t *>(A.arena + pr->off_idx);
        for (int i = threadIdx.x; i < 1 + nd; i += blockDim.x) rowix[i] = idx[i];
        for (int j = threadIdx.x; j < nc; j += blockDim.x) colix[j] = idx[1 + nd + j];
        __syncthreads();
        // a0 (the prepended row) and the row of digit d (outer first, then inner)
        auto a0 = [&](int j) -> double2 {
            const int c = colix[j];
            if (c < 0) return make_double2(1.0, 0.0);
            const double *e = mat + 2 * (static_cast<int64_t>(rowix[0]) * A.mat_cols + c);
            return make_double2(e[0], e[1]);
        };
        auto ad = [&](int d, int j) -> double2 {
            const int c = colix[j];
            if (c < 0) return make_double2(0.0, 0.0);
            const double *e = mat + 2 * (static_cast<int64_t>(rowix[1 + d]) * A.mat_cols + c);
            return make_double2(e[0], e[1]);
        };
        auto mult = [&](int d) -> int { return d < no ? pr->outer_m[d] : pr->inner_m[d - no]; };
        // a scaled entry as the double-float walk takes it: rounded by q47
        // (every sum of them below is then exact in FP64: they stay below 2)
        auto qdf = [&](double x) -> double {
            if constexpr (FMT == PREP_DF) return q47(x);
            return x;
        };
        // an inner digit's row as the prefix table sums it: scaled and rounded
        // for the double-float walk (whose table is not scaled afterwards)
        auto ad_tab = [&](int d, int j) -> double2 {
            const double2 a = ad(d, j);
            if constexpr (FMT == PREP_DF) return make_double2(q47(a.x * cscale[j]), q47(a.y * cscale[j]));
            return a;
        };

        for (int j = threadIdx.x; j < nc; j += blockDim.x) {
            double s = 1.0;
            int e = 0;
            if constexpr (FMT == PREP_DF) {
                const double2 v = a0(j);
                double B = fabs(v.x) + fabs(v.y);
                for (int d = 0; d < nd; ++d) {
                    const double2 w = ad(d, j);
                    B += mult(d) * (fabs(w.x) + fabs(w.y));
                }
                if (B > 0.0) frexp(B, &e);
                s = ldexp(1.0, -e);
            }
            cscale[j] = s;
            eshift[j] = e * pr->cm[j];
            if (slice == 0) pr->col_e[j] = static_cast<int16_t>(e);
        }
        __syncthreads();

        if (slice == 0) {
            if (threadIdx.x == 0) {
                int sh = 0;
                for (int j = 0; j < nc; ++j) sh += eshift[j];
                pr->col_shift = sh;
            }
            // seeds
            for (int c = threadIdx.x; c < 2 * nc; c += blockDim.x) {
                const int j = c >> 1, part = c & 1;
                const double sc = cscale[j];
                const double2 v0 = a0(j);
                double sum = qdf((part ? v0.y : v0.x) * sc), comp = 0.0;
                for (int d = 0; d < nd; ++d) {
                    const double2 w = ad(d, j);
                    const double x = static_cast<double>(mult(d)) * qdf((part ? w.y : w.x) * sc);
                    const double t = sum + x;
                    const double bb = t - sum;
                    comp += (sum - (t - bb)) + (x - bb);
                    sum = t;
                }
                const double base = sum + comp;
                if constexpr (FMT == PREP_F64) {
                    reinterpret_cast<double *>(A.arena + pr->off_base64)[c] = base;
                } else {
                    float *b = reinterpret_cast<float *>(A.arena + pr->off_base_df);
                    split_df(base, b[2 * c], b[2 * c + 1]);
                }
            }
            // outer rows and update rows
            for (int e = threadIdx.x; e < no * 2 * nc; e += blockDim.x) {
                const int o = e / (2 * nc);
                const int c = e - o * 2 * nc;
                const int j = c >> 1, part = c & 1;
                const double2 w = ad(o, j);
                const double v = qdf((part ? w.y : w.x) * cscale[j]);
                const int64_t up = static_cast<int64_t>(2 * o) * 2 * nc + c;  // row 2o: -2 a_o
                const int64_t dn = up + 2 * nc;                                 // row 2o+1: +2 a_o
                if constexpr (FMT == PREP_F64) {
                    reinterpret_cast<double *>(A.arena + pr->off_outer64)[e] = v;
                    double *D = reinterpret_cast<double *>(A.arena + pr->off_D);
                    D[up] = -2.0 * v;
                    D[dn] = 2.0 * v;
                } else {
                    float *orow = reinterpret_cast<float *>(A.arena + pr->off_outer_df);
                    split_df(v, orow[2 * e], orow[2 * e + 1]);
                    float *D = reinterpret_cast<float *>(A.arena + pr->off_D);
                    if constexpr (FMT == PREP_DF) {  // (high words on the walk's 2^-23 grid)
                        df_split_grid(-2.0 * v, D[2 * up], D[2 * up + 1]);
                        df_split_grid(2.0 * v, D[2 * dn], D[2 * dn + 1]);
                    } else {
                        D[up] = __double2float_rn(-2.0 * v);
                        D[dn] = __double2float_rn(2.0 * v);
                    }
                }
            }
        }

        // Prefix table, in tiles of blockDim.x codes spread over the slices.
        // The inner digits split into a low group (digits 0..K1-1) and a high
        // group: Delta(t) = DL(low digits) + DH(high digits), where DL and DH
        // are the same sums over each group alone, tabulated in shared memory
        // for every value of the group's digits (PL + PH entries per column
        // instead of P, each a sum of at most K FMAs).  An entry of the table
        // then costs one FP64 add instead of K FMAs.  Every code's Gray digits
        // are decoded once, into its two sub-table indices.
        const int P = pr->P;
        int K1 = 0, PL = 1, PH = P;
        {
            int best = 1 + P, pl = 1;
            for (int k1 = 0; k1 <= K; ++k1) {
                if (k1 > 0) pl *= pr->inner_m[k1 - 1] + 1;
                const int ph = P / pl;
                if (pl + ph < best) {
                    best = pl + ph;
                    K1 = k1;
                    PL = pl;
                    PH = ph;
                }
            }
        }
        const bool split = PL + PH <= PREP_SUB_MAX;
        const int n_tiles = (P + blockDim.x - 1) / blockDim.x;
        if (slice >= n_tiles) {
            __syncthreads();  // no tile for this slice: the shared arrays are reused
            continue;
        }
        if (split) {
            for (int e = threadIdx.x; e < (PL + PH) * nc; e += blockDim.x) {
                const int u = e / nc, j = e - u * nc;
                const bool low = u < PL;
                int rest = low ? u : u - PL;
                double re = 0.0, im = 0.0;
                for (int k = low ? 0 : K1; k < (low ? K1 : K); ++k) {
                    const int L = pr->inner_m[k] + 1;
                    const int g = rest % L;
                    rest /= L;
                    if (!g) continue;
                    const double f = -2.0 * g;
                    const double2 a = ad_tab(no + k, j);
                    re = __fma_rn(f, a.x, re);
                    im = __fma_rn(f, a.y, im);
                }
                subtab[u][j] = make_double2(re, im);
            }
        } else {
            for (int k = threadIdx.x; k < K * nc; k += blockDim.x) {
                const int kk = k / nc, j = k - kk * nc;
                inrow[kk][j] = ad_tab(no + kk, j);
            }
        }
        for (int tile = slice; tile < n_tiles; tile += A.slices) {
            const int t0 = tile * blockDim.x;
            const int tc = min(static_cast<int>(blockDim.x), P - t0);
            __syncthreads();  // sub-tables / rows written, the previous tile's digits read
            if (static_cast<int>(threadIdx.x) < tc) {
                uint8_t *g = gt[threadIdx.x];
                gray_decode_inner(pr->inner_m, K, static_cast<uint32_t>(t0 + threadIdx.x), g);
                if (split) {
                    int il = 0, ih = 0, sl = 1, sh = 1;
                    for (int k = 0; k < K; ++k) {
                        const int L = pr->inner_m[k] + 1;
                        if (k < K1) {
                            il += g[k] * sl;
                            sl *= L;
                        } else {
                            ih += g[k] * sh;
                            sh *= L;
                        }
                    }
                    gix[threadIdx.x][0] = static_cast<int16_t>(il);
                    gix[threadIdx.x][1] = static_cast<int16_t>(PL + ih);
                }
            }
            __syncthreads();
            for (int e = threadIdx.x; e < tc * nc; e += blockDim.x) {
                const int tl = e / nc;
                const int j = e - tl * nc;
                double re, im;
                if (split) {
                    const double2 l = subtab[gix[tl][0]][j], h = subtab[gix[tl][1]][j];
                    re = l.x + h.x;
                    im = l.y + h.y;
                } else {
                    const uint8_t *g = gt[tl];
                    re = 0.0;
                    im = 0.0;
                    for (int k = 0; k < K; ++k) {
                        if (!g[k]) continue;
                        const double f = -2.0 * g[k];
                        const double2 a = inrow[k][j];
                        re = __fma_rn(f, a.x, re);
                        im = __fma_rn(f, a.y, im);
                    }
                }
                if constexpr (FMT != PREP_DF) {  // (the double-float rows are scaled already)
                    re *= cscale[j];
                    im *= cscale[j];
                }
                const int64_t at = pr->delta_begin + static_cast<int64_t>(t0) * nc + e;
                if constexpr (FMT == PREP_F64) {
                    reinterpret_cast<double2 *>(A.delta)[at] = make_double2(re, im);
                } else if constexpr (FMT == PREP_F32) {
                    const float fr = __double2float_rn(re), fi = __double2float_rn(im);
                    if (A.dup) {
                        reinterpret_cast<float4 *>(A.delta)[at] = make_float4(fr, fr, fi, fi);
                    } else if (A.pairs) {
                        // code t of column j: pair t/2, lane t&1 (delta_begin counts float2 slots)
                        const int t = t0 + tl;
                        float *f = reinterpret_cast<float *>(A.delta) + 2 * pr->delta_begin +
                                   (static_cast<int64_t>(t >> 1) * nc + j) * 4 + (t & 1);
                        f[0] = fr;
                        f[2] = fi;
                        if ((P & 1) && t == P - 1) {  // the zero pad code P beside the last one
                            f[1] = 0.0f;
                            f[3] = 0.0f;
                        }
                    } else {
                        reinterpret_cast<float2 *>(A.delta)[at] = make_float2(fr, fi);
                    }
                } else {  // double-float, high words on the walk's 2^-23 grid
                    float4 v;
                    df_split_grid(re, v.x, v.y);
                    df_split_grid(im, v.z, v.w);
                    reinterpret_cast<float4 *>(A.delta)[at] = v;
                }
            }
        }
        __syncthreads();  // the shared index and scale arrays are reused
    }
}

}  // namespace pqg
