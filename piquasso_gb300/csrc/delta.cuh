// Device construction of the per-problem prefix tables
//     Delta(t)_j = sum_k -2 g_k(t) a_kj
// over the inner codes t of the reflected mixed-radix Gray code, in FP64, then
// stored in the walk's precision (FP64, FP32, or double-float pairs).  One
// thread per (problem, t, column) entry, grid-stride over the whole plan; the
// tables are rebuilt whenever a plan is uploaded.
#pragma once
#include "walk_common.cuh"

namespace pqg {

enum DeltaFormat : int { DELTA_F64 = 0, DELTA_F32 = 1, DELTA_DF = 2 };

template <int FMT>
__global__ void build_delta(const PqgProblem *__restrict__ probs, int n_probs, const unsigned char *__restrict__ arena,
                            void *__restrict__ delta, int64_t total) {
    for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < total;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        // owner: the largest p with delta_begin <= e (empty tables share offsets)
        int lo = 0, hi = n_probs - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (probs[mid].delta_begin <= e)
                lo = mid;
            else
                hi = mid - 1;
        }
        const PqgProblem *pr = probs + lo;
        const int nc = pr->nc;
        const int64_t local = e - pr->delta_begin;
        const int64_t t = local / nc;
        const int j = static_cast<int>(local - t * nc);
        uint8_t g[PQG_MAX_INNER];
        gray_decode(pr->inner_m, pr->K, t, g);
        const double2 *rows = reinterpret_cast<const double2 *>(arena + pr->off_inner64);
        double re = 0.0, im = 0.0;
        for (int k = 0; k < pr->K; ++k) {
            if (!g[k]) continue;
            const double f = -2.0 * g[k];
            const double2 a = rows[static_cast<int64_t>(k) * nc + j];
            re = __fma_rn(f, a.x, re);
            im = __fma_rn(f, a.y, im);
        }
        if constexpr (FMT == DELTA_F64) {
            reinterpret_cast<double2 *>(delta)[e] = make_double2(re, im);
        } else if constexpr (FMT == DELTA_F32) {
            reinterpret_cast<float2 *>(delta)[e] = make_float2(__double2float_rn(re), __double2float_rn(im));
        } else {
            const float rh = __double2float_rn(re), ih = __double2float_rn(im);
            reinterpret_cast<float4 *>(delta)[e] =
                make_float4(rh, __double2float_rn(re - static_cast<double>(rh)), ih,
                            __double2float_rn(im - static_cast<double>(ih)));
        }
    }
}

}  // namespace pqg
