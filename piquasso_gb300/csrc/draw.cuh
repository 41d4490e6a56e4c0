// The output-mode draw of one step of the exact boson sampler, fused behind
// the batched Laplace permanents (Clifford & Clifford algorithm B, the step
// of piquasso/_simulators/passive/sampling.py:723-749 in the reference):
//
//     amp_i = sum_j cols_j L_j U[i, j],   p_i = |amp_i|^2,
//     mode  = min(#{i : cdf_i < u * cdf_last}, n_modes - 1)
//
// with L_j the Laplace permanent of column j (cols_j lowered by one) and u a
// uniform in [0, 1) from the caller.  One warp per shot: lane k holds the
// coefficient cols_k L_k of kept column k (at most 32), the lanes take 32
// output modes at a time (FP64 amplitudes), and a warp scan gives the
// cumulative sums.  Two passes over the modes: the total, then the first mode
// whose cumulative sum reaches u * total (the same sums in the same order, so
// the last cumulative sum equals the total and a mode is always found).
#pragma once
#include "walk_common.cuh"

namespace pqg {

template <typename T>
__global__ void draw_modes(const PqgProblem *__restrict__ probs, int n_probs, const unsigned char *__restrict__ arena,
                           int64_t matrix_off, int64_t n_modes, int64_t mat_cols, const T *__restrict__ lap,
                           const double *__restrict__ uniforms, int32_t *__restrict__ modes) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int ip = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (ip >= n_probs) return;  // uniform over the warp
    const PqgProblem *pr = probs + ip;
    if (pr->kind != PQG_KIND_WALK) {  // the host rejects these before the launch
        if (lane == 0) modes[pr->index] = -1;
        return;
    }
    const int32_t *col = reinterpret_cast<const int32_t *>(arena + pr->off_idx) + 1 + pr->n_outer + pr->K;
    const double *U = reinterpret_cast<const double *>(arena + matrix_off);
    const int nc = pr->nc;
    const int64_t oi = pr->out_index;
    double cr = 0.0, ci = 0.0;
    int cj = -1;  // matrix column of this lane's kept column (-1: none or padding)
    if (lane < nc) {
        cj = col[lane];
        if (cj >= 0) {
            const double m = static_cast<double>(pr->cm[lane]);
            cr = m * static_cast<double>(lap[2 * (oi + lane)]);
            ci = m * static_cast<double>(lap[2 * (oi + lane) + 1]);
        }
    }
    // p_i for mode i (0 beyond the last mode); every lane runs the shuffles
    auto prob = [&](int64_t i) -> double {
        double ar = 0.0, ai = 0.0;
        for (int k = 0; k < nc; ++k) {
            const int j = __shfl_sync(full, cj, k);
            const double xr = __shfl_sync(full, cr, k), xi = __shfl_sync(full, ci, k);
            if (j < 0 || i >= n_modes) continue;
            const double2 u = *reinterpret_cast<const double2 *>(U + 2 * (i * mat_cols + j));
            ar = fma(xr, u.x, fma(-xi, u.y, ar));
            ai = fma(xr, u.y, fma(xi, u.x, ai));
        }
        return ar * ar + ai * ai;
    };
    auto scan = [&](double p) -> double {  // inclusive warp scan
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const double t = __shfl_up_sync(full, p, off);
            if (lane >= off) p += t;
        }
        return p;
    };
    double total = 0.0;
    for (int64_t i0 = 0; i0 < n_modes; i0 += 32) total += __shfl_sync(full, scan(prob(i0 + lane)), 31);
    const double thr = uniforms[pr->index] * total;
    double carry = 0.0;
    int64_t found = n_modes - 1;
    for (int64_t i0 = 0; i0 < n_modes; i0 += 32) {
        const double s = scan(prob(i0 + lane));
        const unsigned hit = __ballot_sync(full, i0 + lane < n_modes && carry + s >= thr);
        if (hit) {
            found = i0 + __ffs(hit) - 1;
            break;
        }
        carry += __shfl_sync(full, s, 31);
    }
    if (lane == 0) modes[pr->index] = static_cast<int32_t>(found < n_modes - 1 ? found : n_modes - 1);
}

}  // namespace pqg
