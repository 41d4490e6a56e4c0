// Deterministic double-double reductions of the walk partials.
//   level 1: one warp per chunk of at most PQG_CHUNK_ITEMS items of one problem;
//   level 2: one warp per problem sums its chunks, applies 2^-(N-1) and writes
//            the output in the problem's precision (plus the low words).
// Every sum runs in a fixed order, so a problem's result does not depend on
// the batch it came in or on the launch.
#pragma once
#include "walk_common.cuh"

namespace pqg {

// Sum of n partial slots first + k*stride (k < n) in a fixed order, by one
// warp: lane 0 alone, in index order, for short runs; lanes strided over the
// slots and a shuffle tree for long ones.  The double-double adds run on the
// FP64 pipe, a thirty-second of the FP32 rate on this part, so short runs
// skip the tree (five levels of adds over mostly empty lanes).
#define PQG_REDUCE_SERIAL 8
__device__ __forceinline__ void warp_sum_slots(const double *__restrict__ src, int64_t first, int64_t stride, int64_t n,
                                               ddv &r, ddv &i) {
    const int lane = threadIdx.x & 31;
    r = ddv{0.0, 0.0};
    i = ddv{0.0, 0.0};
    if (n <= PQG_REDUCE_SERIAL) {
        if (lane == 0) {
            for (int64_t k = 0; k < n; ++k) {
                ddv a, b;
                load_partial(src, first + k * stride, a, b);
                r = dd_add(r, a);
                i = dd_add(i, b);
            }
        }
        return;
    }
    for (int64_t k = lane; k < n; k += 32) {
        ddv a, b;
        load_partial(src, first + k * stride, a, b);
        r = dd_add(r, a);
        i = dd_add(i, b);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        r = dd_add(r, dd_shfl_down(r, off));
        i = dd_add(i, dd_shfl_down(i, off));
    }
}

// Sum over n slots (first + k*stride) for each of n_out outputs (slot offset
// o): one lane per output, each summing in index order.
__device__ __forceinline__ void lane_sum_outputs(const double *__restrict__ src, int64_t first, int64_t stride,
                                                 int64_t n, int n_out, double *__restrict__ dst, int64_t dst_first) {
    for (int o = threadIdx.x & 31; o < n_out; o += 32) {
        ddv r{0.0, 0.0}, i{0.0, 0.0};
        for (int64_t k = 0; k < n; ++k) {
            ddv a, b;
            load_partial(src, first + k * stride + o, a, b);
            r = dd_add(r, a);
            i = dd_add(i, b);
        }
        store_partial(dst, dst_first + o, r, i);
    }
}

// Level 1: one warp per chunk.  chunk_out: PQG_MAX_OUT slots of 4 doubles per
// chunk.  Single-output problems (plain permanents) sum their items with
// warp_sum_slots; Laplace problems put one lane on each output.
__global__ void reduce_chunks(const PqgChunk *__restrict__ chunks, int n_chunks, const PqgProblem *__restrict__ probs,
                              const double *__restrict__ partials, double *__restrict__ chunk_out) {
    const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (w >= n_chunks) return;  // uniform over the warp
    const PqgChunk c = chunks[w];
    const PqgProblem *pr = probs + c.problem;
    const int n_out = pr->n_out;
    const int64_t first = pr->part_begin + (c.item_lo - pr->item_begin) * n_out;
    const int64_t n = c.item_hi - c.item_lo;
    const int64_t dst = static_cast<int64_t>(w) * PQG_MAX_OUT;
    if (n_out == 1) {
        ddv r, i;
        warp_sum_slots(partials, first, 1, n, r, i);
        if ((threadIdx.x & 31) == 0) store_partial(chunk_out, dst, r, i);
    } else {
        lane_sum_outputs(partials, first, n_out, n, n_out, chunk_out, dst);
    }
}

// out: 2 values per output (re, im) as T; out_lo (nullable): 2 doubles per output
template <typename T>
__global__ void finish_problems(const PqgProblem *__restrict__ probs, int n_probs, const double *__restrict__ chunk_out,
                                T *__restrict__ out, double *__restrict__ out_lo) {
    const int lane = threadIdx.x & 31;
    const int ip = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (ip >= n_probs) return;
    const PqgProblem *pr = probs + ip;
    const int64_t oi = pr->out_index;
    if (pr->kind == PQG_KIND_CONSTANT) {
        if (lane == 0) {
            out[2 * oi] = static_cast<T>(pr->cval_re);
            out[2 * oi + 1] = static_cast<T>(pr->cval_im);
            if (out_lo) {
                out_lo[2 * oi] = 0.0;
                out_lo[2 * oi + 1] = 0.0;
            }
        }
        return;
    }
    // the problem's chunk sums: one warp sum (single output) or one lane per
    // output; then 2^(col_shift - scale_exp) and the output precision
    const int n_out = pr->n_out;
    for (int o0 = 0; o0 < n_out; o0 += 32) {
        ddv r{0.0, 0.0}, i{0.0, 0.0};
        int o = o0;
        bool mine = lane == 0;
        if (n_out == 1) {
            warp_sum_slots(chunk_out, pr->chunk_begin * PQG_MAX_OUT, PQG_MAX_OUT, pr->n_chunks, r, i);
        } else {
            o = o0 + lane;
            mine = o < n_out;
            if (mine) {
                for (int64_t c = pr->chunk_begin; c < pr->chunk_begin + pr->n_chunks; ++c) {
                    ddv a, b;
                    load_partial(chunk_out, c * PQG_MAX_OUT + o, a, b);
                    r = dd_add(r, a);
                    i = dd_add(i, b);
                }
            }
        }
        if (mine) {
            // scaling by a power of two is exact in both words; ldexp avoids an
            // intermediate 2^-scale_exp that would itself overflow
            // (a Laplace output of kept column o lacks one factor of that
            // column, so one scale exponent e_o less)
            const int e = pr->col_shift - pr->scale_exp - (pr->laplace && o < pr->nc ? pr->col_e[o] : 0);
            const double rh = ldexp(r.hi, e), rl = ldexp(r.lo, e), ih = ldexp(i.hi, e), il = ldexp(i.lo, e);
            if constexpr (sizeof(T) == 8) {
                out[2 * (oi + o)] = rh;
                out[2 * (oi + o) + 1] = ih;
            } else {
                out[2 * (oi + o)] = static_cast<T>(rh + rl);
                out[2 * (oi + o) + 1] = static_cast<T>(ih + il);
            }
            if (out_lo) {
                out_lo[2 * (oi + o)] = rl;
                out_lo[2 * (oi + o) + 1] = il;
            }
        }
    }
}

}  // namespace pqg
