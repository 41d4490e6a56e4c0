// Deterministic double-double reductions of the walk partials.
//   level 1: one block per chunk of at most 512 items of one problem;
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
    const double4 *part = reinterpret_cast<const double4 *>(partials);
    for (int o = 0; o < n_out; ++o) {
        ddv r{0.0, 0.0}, i{0.0, 0.0};
        for (int64_t it = c.item_lo + threadIdx.x; it < c.item_hi; it += blockDim.x) {
            const double4 v = part[pr->part_begin + (it - pr->item_begin) * n_out + o];
            r = dd_add(r, ddv{v.x, v.y});
            i = dd_add(i, ddv{v.z, v.w});
        }
        block_reduce_dd(r, i, scratch);
        if (threadIdx.x == 0)
            reinterpret_cast<double4 *>(chunk_out)[static_cast<int64_t>(blockIdx.x) * PQG_MAX_OUT + o] =
                make_double4(r.hi, r.lo, i.hi, i.lo);
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
    const double4 *co = reinterpret_cast<const double4 *>(chunk_out);
    const double scale = ldexp(1.0, -pr->scale_exp);
    for (int o = 0; o < pr->n_out; ++o) {
        ddv r{0.0, 0.0}, i{0.0, 0.0};
        for (int64_t c = pr->chunk_begin + lane; c < pr->chunk_begin + pr->n_chunks; c += 32) {
            const double4 v = co[c * PQG_MAX_OUT + o];
            r = dd_add(r, ddv{v.x, v.y});
            i = dd_add(i, ddv{v.z, v.w});
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            r = dd_add(r, dd_shfl_down(r, off));
            i = dd_add(i, dd_shfl_down(i, off));
        }
        if (lane == 0) {
            // scaling by a power of two is exact in both words
            const double rh = r.hi * scale, rl = r.lo * scale, ih = i.hi * scale, il = i.lo * scale;
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
