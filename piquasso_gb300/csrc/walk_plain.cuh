// Plain permanent walk kernels (one output per problem).
//
// Persistent grid; every warp pulls work items (one problem, 32 consecutive
// outer assignments) from a device queue.  Each lane seeds its column sums in
// FP64 from scratch, then all 32 lanes walk the problem's inner Gray-code
// table in lock step: per step one column update (the changed row is the same
// for the whole warp, so its values are broadcast loads) and one product over
// the columns with their multiplicities.  The weighted terms are summed in
// short blocks and folded into a per-lane double-double; lanes are combined by
// a double-double warp reduction and the item's result is written to its
// partial slot.  Method: src/permanent.cpp:155-250 of the reference, with the
// Gray-code space split into a lock-step inner walk and per-lane outer seeds.
#pragma once
#include "walk_common.cuh"

namespace pqg {

// Complex128: FP64 column sums, updates and products.
template <int NC>
__global__ void __launch_bounds__(PQG_WALK_THREADS) walk_plain_c128(WalkArgs A) {
    const int lane = threadIdx.x & 31;
    for (;;) {
        const int64_t item = next_item(A.counter, lane);
        if (item >= A.total_items) return;
        const int ip = find_problem(A.item_begin, A.n_probs, item);
        const PqgProblem *pr = A.probs + ip;
        const int64_t local = item - pr->item_begin;
        const int64_t q = local * PQG_ITEM_LANES + lane;
        ddv sr{0.0, 0.0}, si{0.0, 0.0};
        if (q < pr->Q) {
            double cr[NC], ci[NC];
            const double wout = seed_outer<NC>(pr, A.arena, q, cr, ci);
            int cm[NC];
#pragma unroll
            for (int j = 0; j < NC; ++j) cm[j] = pr->cm[j];
            const bool ones = pr->cm_max == 1;
            const PqgStep128 *tab = reinterpret_cast<const PqgStep128 *>(A.arena + pr->off_tab);
            const double2 *D = reinterpret_cast<const double2 *>(A.arena + pr->off_D);
            const int P = pr->P;

            auto product = [&](double &xr, double &xi) {
                xr = cr[0];
                xi = ci[0];
                if (ones) {
#pragma unroll
                    for (int j = 1; j < NC; ++j) cmul(xr, xi, cr[j], ci[j]);
                } else {
                    for (int r = 1; r < cm[0]; ++r) cmul(xr, xi, cr[0], ci[0]);
#pragma unroll
                    for (int j = 1; j < NC; ++j)
                        for (int r = 0; r < cm[j]; ++r) cmul(xr, xi, cr[j], ci[j]);
                }
            };

            double ar, ai;
            product(ar, ai);  // step 0: weight 1
            for (int t = 1; t < P; ++t) {
                const double w = __ldg(&tab[t].w);
                const double2 *d = D + __ldg(&tab[t].drow);
#pragma unroll
                for (int j = 0; j < NC; ++j) {
                    const double2 v = __ldg(d + j);
                    cr[j] = __dadd_rn(cr[j], v.x);
                    ci[j] = __dadd_rn(ci[j], v.y);
                }
                double xr, xi;
                product(xr, xi);
                ar = __fma_rn(w, xr, ar);
                ai = __fma_rn(w, xi, ai);
                if ((t & 63) == 0) {
                    sr = dd_add_d(sr, ar);
                    si = dd_add_d(si, ai);
                    ar = 0.0;
                    ai = 0.0;
                }
            }
            sr = dd_mul_d(dd_add_d(sr, ar), wout);
            si = dd_mul_d(dd_add_d(si, ai), wout);
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            sr = dd_add(sr, dd_shfl_down(sr, off));
            si = dd_add(si, dd_shfl_down(si, off));
        }
        if (lane == 0) store_partial(A.partials, pr->part_begin + local, sr, si);
    }
}

// Complex64: FP32 column updates and products; FP32 TwoSum-compensated
// partial sums folded into a per-lane double-double every 128 steps.
template <int NC>
__global__ void __launch_bounds__(PQG_WALK_THREADS) walk_plain_c64(WalkArgs A) {
    const int lane = threadIdx.x & 31;
    for (;;) {
        const int64_t item = next_item(A.counter, lane);
        if (item >= A.total_items) return;
        const int ip = find_problem(A.item_begin, A.n_probs, item);
        const PqgProblem *pr = A.probs + ip;
        const int64_t local = item - pr->item_begin;
        const int64_t q = local * PQG_ITEM_LANES + lane;
        ddv sr{0.0, 0.0}, si{0.0, 0.0};
        if (q < pr->Q) {
            float cr[NC], ci[NC];
            double wout;
            {
                double dr[NC], di[NC];
                wout = seed_outer<NC>(pr, A.arena, q, dr, di);
#pragma unroll
                for (int j = 0; j < NC; ++j) {
                    cr[j] = __double2float_rn(dr[j]);
                    ci[j] = __double2float_rn(di[j]);
                }
            }
            int cm[NC];
#pragma unroll
            for (int j = 0; j < NC; ++j) cm[j] = pr->cm[j];
            const bool ones = pr->cm_max == 1;
            const PqgStep64 *tab = reinterpret_cast<const PqgStep64 *>(A.arena + pr->off_tab);
            const float2 *D = reinterpret_cast<const float2 *>(A.arena + pr->off_D);
            const int P = pr->P;

            auto product = [&](float &xr, float &xi) {
                xr = cr[0];
                xi = ci[0];
                if (ones) {
#pragma unroll
                    for (int j = 1; j < NC; ++j) cmulf(xr, xi, cr[j], ci[j]);
                } else {
                    for (int r = 1; r < cm[0]; ++r) cmulf(xr, xi, cr[0], ci[0]);
#pragma unroll
                    for (int j = 1; j < NC; ++j)
                        for (int r = 0; r < cm[j]; ++r) cmulf(xr, xi, cr[j], ci[j]);
                }
            };

            float ar, ai, er = 0.0f, ei = 0.0f;
            product(ar, ai);
            for (int t = 1; t < P; ++t) {
                const float2 e = __ldg(reinterpret_cast<const float2 *>(tab + t));
                const float w = e.x;
                const float2 *d = D + __float_as_int(e.y);
#pragma unroll
                for (int j = 0; j < NC; ++j) {
                    const float2 v = __ldg(d + j);
                    cr[j] = __fadd_rn(cr[j], v.x);
                    ci[j] = __fadd_rn(ci[j], v.y);
                }
                float xr, xi;
                product(xr, xi);
                f_two_sum_acc(ar, er, __fmul_rn(w, xr));
                f_two_sum_acc(ai, ei, __fmul_rn(w, xi));
                if ((t & 127) == 0) {
                    sr = dd_add_d(dd_add_d(sr, static_cast<double>(ar)), static_cast<double>(er));
                    si = dd_add_d(dd_add_d(si, static_cast<double>(ai)), static_cast<double>(ei));
                    ar = ai = er = ei = 0.0f;
                }
            }
            sr = dd_add_d(dd_add_d(sr, static_cast<double>(ar)), static_cast<double>(er));
            si = dd_add_d(dd_add_d(si, static_cast<double>(ai)), static_cast<double>(ei));
            sr = dd_mul_d(sr, wout);
            si = dd_mul_d(si, wout);
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            sr = dd_add(sr, dd_shfl_down(sr, off));
            si = dd_add(si, dd_shfl_down(si, off));
        }
        if (lane == 0) store_partial(A.partials, pr->part_begin + local, sr, si);
    }
}

}  // namespace pqg
