// Deterministic double-double reductions of the walk partials.
//   level 1: one block per chunk of at most PQG_CHUNK_ITEMS items of one problem;
//   level 2: one warp per problem sums its chunks, applies 2^-(N-1) and writes
//            the output in the problem's precision (plus the low words).
#pragma once
#include "walk_common.cuh"

namespace pqg {

__device__ __forceinline__ void block_reduce_dd(ddv &r, ddv &i, ddv *scratch /* 2 * 32 */) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        r = dd_add(r, dd_shfl_down(r, off));
        i = dd_add(i, dd_shfl_down(i, off));
    }
    __syncthreads();
    if (lane == 0) {
        scratch[2 * warp] = r;
        scratch[2 * warp + 1] = i;
    }
    __syncthreads();
    const int nw = blockDim.x >> 5;
    if (warp == 0) {
        r = lane < nw ? scratch[2 * lane] : ddv{0.0, 0.0};
        i = lane < nw ? scratch[2 * lane + 1] : ddv{0.0, 0.0};
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            r = dd_add(r, dd_shfl_down(r, off));
            i = dd_add(i, dd_shfl_down(i, off));
        }
    }
}

// chunk_out: PQG_MAX_OUT slots of 4 doubles per chunk
__global__ void reduce_chunks(const PqgChunk *__restrict__ chunks, const PqgProblem *__restrict__ probs,
                              const double *__restrict__ partials, double *__restrict__ chunk_out) {
    __shared__ ddv scratch[64];
    const PqgChunk c = chunks[blockIdx.x];
    const PqgProblem *pr = probs + c.problem;
    const int n_out = pr->n_out;
    for (int o = 0; o < n_out; ++o) {
        ddv r{0.0, 0.0}, i{0.0, 0.0};
        for (int64_t it = c.item_lo + threadIdx.x; it < c.item_hi; it += blockDim.x) {
            ddv a, b;
            load_partial(partials, pr->part_begin + (it - pr->item_begin) * n_out + o, a, b);
            r = dd_add(r, a);
            i = dd_add(i, b);
        }
        block_reduce_dd(r, i, scratch);
        if (threadIdx.x == 0) store_partial(chunk_out, static_cast<int64_t>(blockIdx.x) * PQG_MAX_OUT + o, r, i);
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
    for (int o = 0; o < pr->n_out; ++o) {
        ddv r{0.0, 0.0}, i{0.0, 0.0};
        for (int64_t c = pr->chunk_begin + lane; c < pr->chunk_begin + pr->n_chunks; c += 32) {
            ddv a, b;
            load_partial(chunk_out, c * PQG_MAX_OUT + o, a, b);
            r = dd_add(r, a);
            i = dd_add(i, b);
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            r = dd_add(r, dd_shfl_down(r, off));
            i = dd_add(i, dd_shfl_down(i, off));
        }
        if (lane == 0) {
            // scaling by a power of two is exact in both words; ldexp avoids an
            // intermediate 2^-scale_exp that would itself overflow
            const int e = pr->col_shift - pr->scale_exp;
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
