// Laplace-expansion walk kernels: for every column l, the permanent with the
// multiplicity of column l lowered by one, all from ONE Gray-code walk
// (Lemma 1 of arXiv:2005.04214, as the reference's
// src/permanent_laplace.cpp:43-240).  The reference forms each of the nc
// products separately, O(nc * N) multiplies per step; here a prefix pass and
// a suffix pass give all nc products in O(nc):
//     out_l += w * prefix_l * suffix_l * c_l^(m_l - 1),
// and the final suffix w * prod_l c_l^(m_l) is the value shared by every
// column of multiplicity zero (their exponent stays 0 in the reference).
// Work split (R consecutive outer positions per lane), seeding, one-digit
// outer steps, prefix tables and reductions are those of the plain kernels.
#pragma once
#include "walk_plain.cuh"

namespace pqg {

// Per-thread arrays that live either in registers or in a column-major slice
// of dynamic shared memory (stride = threads per block).
template <typename T, int N, bool SMEM>
struct LaneArray;

template <typename T, int N>
struct LaneArray<T, N, false> {
    T v[N];
    __device__ __forceinline__ void init(T *, int) {}
    __device__ __forceinline__ T get(int j) const { return v[j]; }
    __device__ __forceinline__ void set(int j, T x) { v[j] = x; }
};

template <typename T, int N>
struct LaneArray<T, N, true> {
    T *p;
    __device__ __forceinline__ void init(T *base, int tid) { p = base + tid; }
    __device__ __forceinline__ T get(int j) const { return p[j * PQG_WALK_THREADS]; }
    __device__ __forceinline__ void set(int j, T x) { p[j * PQG_WALK_THREADS] = x; }
};

template <int NC>
struct LaplaceC128Cfg {
    static constexpr bool PRE_SMEM = NC > 16;
    static constexpr bool ACC_SMEM = NC > 20;
    static constexpr size_t smem_bytes =
        (PRE_SMEM ? size_t(NC) * PQG_WALK_THREADS * sizeof(double2) : 0) +
        (ACC_SMEM ? size_t(NC + 1) * PQG_WALK_THREADS * sizeof(double2) : 0);
};

// Complex128 Laplace walk.  R consecutive outer positions per lane, seeded in
// FP64 and moved on by one-digit updates; the column sums of inner code t are
// seed + Delta(t).  Per-lane sums are
// plain FP64 over one inner walk (at most 512 codes), combined across lanes,
// items and chunks in double-double.
template <int NC>
__global__ void __launch_bounds__(PQG_WALK_THREADS, 1) walk_laplace_c128(WalkArgs A) {
    using Cfg = LaplaceC128Cfg<NC>;
    extern __shared__ double2 lap_smem[];
    const int lane = threadIdx.x & 31;
    LaneArray<double2, NC, Cfg::PRE_SMEM> pre;
    LaneArray<double2, NC + 1, Cfg::ACC_SMEM> acc;
    pre.init(lap_smem, threadIdx.x);
    acc.init(lap_smem + (Cfg::PRE_SMEM ? NC * PQG_WALK_THREADS : 0), threadIdx.x);

    for (;;) {
        const int64_t item = next_item(A.counter, lane);
        if (item >= A.total_items) return;
        const int ip = find_problem(A.item_begin, A.n_probs, item);
        const PqgProblem *pr = A.probs + ip;
        const int64_t local = item - pr->item_begin;
        const int64_t R = pr->R;
        const int64_t r0 = (local * PQG_ITEM_LANES + lane) * R;
        const int n_out = pr->n_out;
        const bool full = n_out > NC;
        const bool active = r0 < pr->Q;
        if (active) {
            double sr0[NC], si0[NC];  // FP64 seed of this lane's current outer position
            OuterState st;
            outer_decode(pr, r0, st);
            {
                ArF64::cs_t s[NC];
                seed_lane<ArF64, NC>(pr, A.arena, st, s);
#pragma unroll
                for (int j = 0; j < NC; ++j) {
                    sr0[j] = s[j].r;
                    si0[j] = s[j].i;
                }
            }
            double wout = outer_weight(pr, st);
            const int64_t my_R = (pr->Q - r0 < R) ? (pr->Q - r0) : R;
            const double2 *D = reinterpret_cast<const double2 *>(A.arena + pr->off_D);
            int cm[NC];
#pragma unroll
            for (int j = 0; j < NC; ++j) cm[j] = pr->cm[j];
            const bool ones = pr->cm_max == 1;
            const PqgStep *tab = reinterpret_cast<const PqgStep *>(A.arena + pr->off_tab);
            const double2 *delta = reinterpret_cast<const double2 *>(A.delta) + pr->delta_begin;
            const int P = pr->P;
#pragma unroll
            for (int l = 0; l <= NC; ++l) acc.set(l, make_double2(0.0, 0.0));

            // R consecutive outer positions: the outer weight rides on every
            // step weight (their product stays an exact integer below 2^53)
            for (int64_t seg = 0; seg < my_R; ++seg) {
            for (int t = 0; t < P; ++t) {
                const double w = __ldg(&tab[t].wd) * wout;
                // column sums of inner code t are seed + prefix-table row t,
                // formed where they are used (no per-step array of sums)
                const double2 *d = delta + static_cast<int64_t>(t) * NC;
                auto col = [&](int j, double &cr, double &ci) {
                    const double2 v = __ldg(d + j);
                    cr = __dadd_rn(sr0[j], v.x);
                    ci = __dadd_rn(si0[j], v.y);
                };
                // prefix products: pre_l = prod_{k<l} c_k^(m_k)
                double xr = 1.0, xi = 0.0;
                pre.set(0, make_double2(1.0, 0.0));
#pragma unroll
                for (int j = 0; j + 1 < NC; ++j) {
                    double cr, ci;
                    col(j, cr, ci);
                    if (j == 0 && (ones || cm[0] == 1)) {
                        xr = cr;
                        xi = ci;
                    } else {
                        const int e = ones ? 1 : cm[j];
                        for (int r = 0; r < e; ++r) cmul(xr, xi, cr, ci);
                    }
                    pre.set(j + 1, make_double2(xr, xi));
                }
                // suffix pass
                double sr = w, si = 0.0;
#pragma unroll
                for (int l = NC - 1; l >= 0; --l) {
                    double cr, ci;
                    col(l, cr, ci);
                    const double2 p = pre.get(l);
                    double tr, ti;
                    if (l == NC - 1) {
                        tr = p.x * w;
                        ti = p.y * w;
                    } else if (l == 0) {
                        tr = sr;
                        ti = si;
                    } else {
                        tr = p.x;
                        ti = p.y;
                        cmul(tr, ti, sr, si);
                    }
                    if (!ones)
                        for (int r = 1; r < cm[l]; ++r) cmul(tr, ti, cr, ci);
                    double2 a = acc.get(l);
                    a.x = __dadd_rn(a.x, tr);
                    a.y = __dadd_rn(a.y, ti);
                    acc.set(l, a);
                    if (l > 0 || full) {
                        if (l == NC - 1) {
                            sr = w * cr;
                            si = w * ci;
                            if (!ones)
                                for (int r = 1; r < cm[l]; ++r) cmul(sr, si, cr, ci);
                        } else {
                            const int e = ones ? 1 : cm[l];
                            for (int r = 0; r < e; ++r) cmul(sr, si, cr, ci);
                        }
                    }
                }
                if (full) {
                    double2 a = acc.get(NC);
                    a.x = __dadd_rn(a.x, sr);
                    a.y = __dadd_rn(a.y, si);
                    acc.set(NC, a);
                }
            }
            if (seg + 1 < my_R) {  // one-digit step to the next outer position
                bool up = false;
                const int k = outer_next(pr, st, &up);
                const double2 *d = D + (2 * k + (up ? 0 : 1)) * NC;
#pragma unroll
                for (int j = 0; j < NC; ++j) {
                    sr0[j] = __dadd_rn(sr0[j], d[j].x);
                    si0[j] = __dadd_rn(si0[j], d[j].y);
                }
                wout = outer_weight(pr, st);
            }
            }
        }
        // one output at a time: reduce over the warp, store
        // (unrolled so that a register-resident accumulator array keeps static indices)
#pragma unroll
        for (int l = 0; l <= NC; ++l) {
            if (l >= n_out) break;
            ddv r{0.0, 0.0}, i{0.0, 0.0};
            if (active) {
                const double2 a = acc.get(l);
                r = ddv{a.x, 0.0};
                i = ddv{a.y, 0.0};
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                r = dd_add(r, dd_shfl_down(r, off));
                i = dd_add(i, dd_shfl_down(i, off));
            }
            if (lane == 0) store_partial(A.partials, pr->part_begin + local * n_out + l, r, i);
        }
    }
}

template <int NC>
struct LaplaceC64Cfg {
    static constexpr bool PRE_SMEM = NC > 16;
    static constexpr size_t smem_bytes =
        (PRE_SMEM ? size_t(NC) * PQG_WALK_THREADS * sizeof(float2) : 0) +
        size_t(NC + 1) * PQG_WALK_THREADS * sizeof(float4);
};

// Complex64 Laplace walk: seed in double-float rounded to FP32, column sums
// seed + Delta(t) and products in FP32, FP32 partial sums over 32 codes folded
// into per-lane compensated FP32 sums held in shared memory (ff_fold), lanes
// combined the same way (the output is complex64; no FP64 instruction).  ONES: every column has multiplicity 1 (the sampler's
// case), so the repeated-factor code is compiled out; a fully unrolled
// 24-column step with it did not fit the instruction cache (ncu: 9.7
// no-instruction stalls per issue, 11 % issue).
template <int NC, bool ONES>
__global__ void __launch_bounds__(PQG_WALK_THREADS, walk_min_blocks_cols<NC>()) walk_laplace_c64(WalkArgs A) {
    using Cfg = LaplaceC64Cfg<NC>;
    extern __shared__ double2 lap_smem64[];
    const int lane = threadIdx.x & 31;
    // per-lane compensated FP32 sums of every output, {re, im, re_err, im_err}
    float4 *const acc_base = reinterpret_cast<float4 *>(lap_smem64);
    LaneArray<float4, NC + 1, true> acc;
    acc.init(acc_base, threadIdx.x);
    LaneArray<float2, NC, Cfg::PRE_SMEM> pre;
    pre.init(reinterpret_cast<float2 *>(lap_smem64 + (NC + 1) * PQG_WALK_THREADS), threadIdx.x);

    for (;;) {
        const int64_t item = next_item(A.counter, lane);
        if (item >= A.total_items) return;
        const int ip = find_problem(A.item_begin, A.n_probs, item);
        const PqgProblem *pr = A.probs + ip;
        const int64_t local = item - pr->item_begin;
        const int64_t R = pr->R;
        const int64_t r0 = (local * PQG_ITEM_LANES + lane) * R;
        const int n_out = pr->n_out;
        const bool full = n_out > NC;
        const bool active = r0 < pr->Q;
#pragma unroll
        for (int l = 0; l <= NC; ++l)  // (an idle lane's sums join the lane reduction too)
            acc.set(l, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
        if (active) {
            float sr0[NC], si0[NC];  // seed of the current outer position (double-float, rounded)
            OuterState st;
            outer_decode(pr, r0, st);
            {
                ArF32::cs_t s[NC];
                seed_lane<ArF32, NC>(pr, A.arena, st, s);
#pragma unroll
                for (int j = 0; j < NC; ++j) {
                    sr0[j] = s[j].r;
                    si0[j] = s[j].i;
                }
            }
            double wout = outer_weight(pr, st);
            const int64_t my_R = (pr->Q - r0 < R) ? (pr->Q - r0) : R;
            const float2 *D = reinterpret_cast<const float2 *>(A.arena + pr->off_D);
            int cm[ONES ? 1 : NC];
            if constexpr (!ONES) {
#pragma unroll
                for (int j = 0; j < NC; ++j) cm[j] = pr->cm[j];
            }
            const bool ones = ONES || pr->cm_max == 1;
            const PqgStep *tab = reinterpret_cast<const PqgStep *>(A.arena + pr->off_tab);
            const float2 *delta = reinterpret_cast<const float2 *>(A.delta) + pr->delta_begin;
            const int P = pr->P;
            float ar[NC + 1], ai[NC + 1];
#pragma unroll
            for (int l = 0; l <= NC; ++l) {
                ar[l] = 0.0f;
                ai[l] = 0.0f;
            }

            // R consecutive outer positions; the FP32 partial sums fold into
            // the compensated sums weighted by the current outer weight (ff_fold:
            // the weight as two FP32 words, the product's rounding error by an
            // FMA, TwoSum -- no FP64 instruction)
            for (int64_t seg = 0; seg < my_R; ++seg) {
            for (int t = 0; t < P; ++t) {
                const float w = __ldg(&tab[t].wf);
                const float2 *d = delta + static_cast<int64_t>(t) * NC;
                auto col = [&](int j, float &cr, float &ci) {
                    const float2 v = __ldg(d + j);
                    cr = __fadd_rn(sr0[j], v.x);
                    ci = __fadd_rn(si0[j], v.y);
                };
                float xr = 1.0f, xi = 0.0f;
                pre.set(0, make_float2(1.0f, 0.0f));
#pragma unroll
                for (int j = 0; j + 1 < NC; ++j) {
                    float cr, ci;
                    col(j, cr, ci);
                    if constexpr (ONES) {
                        if (j == 0) {
                            xr = cr;
                            xi = ci;
                        } else {
                            cmulf(xr, xi, cr, ci);
                        }
                    } else if (j == 0 && (ones || cm[0] == 1)) {
                        xr = cr;
                        xi = ci;
                    } else {
                        const int ee = ones ? 1 : cm[j];
                        for (int r = 0; r < ee; ++r) cmulf(xr, xi, cr, ci);
                    }
                    pre.set(j + 1, make_float2(xr, xi));
                }
                float sr = w, si = 0.0f;
#pragma unroll
                for (int l = NC - 1; l >= 0; --l) {
                    float cr, ci;
                    col(l, cr, ci);
                    const float2 p = pre.get(l);
                    float tr, ti;
                    if (l == NC - 1) {
                        tr = p.x * w;
                        ti = p.y * w;
                    } else if (l == 0) {
                        tr = sr;
                        ti = si;
                    } else {
                        tr = p.x;
                        ti = p.y;
                        cmulf(tr, ti, sr, si);
                    }
                    if constexpr (!ONES) {
                        if (!ones)
                            for (int r = 1; r < cm[l]; ++r) cmulf(tr, ti, cr, ci);
                    }
                    ar[l] += tr;
                    ai[l] += ti;
                    if (l > 0 || full) {
                        if (l == NC - 1) {
                            sr = w * cr;
                            si = w * ci;
                            if constexpr (!ONES) {
                                if (!ones)
                                    for (int r = 1; r < cm[l]; ++r) cmulf(sr, si, cr, ci);
                            }
                        } else if constexpr (ONES) {
                            cmulf(sr, si, cr, ci);
                        } else {
                            const int ee = ones ? 1 : cm[l];
                            for (int r = 0; r < ee; ++r) cmulf(sr, si, cr, ci);
                        }
                    }
                }
                if (full) {
                    ar[NC] += sr;
                    ai[NC] += si;
                }
                if ((t & 31) == 31 || t == P - 1) {
#pragma unroll
                    for (int l = 0; l <= NC; ++l) {
                        if (l == NC && !full) continue;
                        const float4 a = acc.get(l);
                        float2 fs = make_float2(a.x, a.y), fc = make_float2(a.z, a.w);
                        ff_fold(fs, fc, ar[l], 0.0f, ai[l], 0.0f, wout);
                        acc.set(l, make_float4(fs.x, fs.y, fc.x, fc.y));
                        ar[l] = 0.0f;
                        ai[l] = 0.0f;
                    }
                }
            }
            if (seg + 1 < my_R) {  // one-digit step to the next outer position
                bool up = false;
                const int k = outer_next(pr, st, &up);
                const float2 *d = D + (2 * k + (up ? 0 : 1)) * NC;
#pragma unroll
                for (int j = 0; j < NC; ++j) {
                    sr0[j] = __fadd_rn(sr0[j], d[j].x);
                    si0[j] = __fadd_rn(si0[j], d[j].y);
                }
                wout = outer_weight(pr, st);
            }
            }
        }
        // lane reduction: lane l sums output l (and l + 32) over the warp's 32
        // lanes with TwoSum on the FP32 pipes, reading the slices in a
        // rotated order so that each quarter-warp's float4 loads hit distinct banks
        __syncwarp();
        for (int l = lane; l < n_out; l += 32) {
            const float4 *src = acc_base + l * PQG_WALK_THREADS + (threadIdx.x & ~31);
            float2 fs = make_float2(0.0f, 0.0f), fc = fs;
#pragma unroll 8
            for (int q = 0; q < 32; ++q) {
                const float4 v = src[(q + lane) & 31];
                two_sum_acc2(fs, fc, make_float2(v.x, v.y));
                fc = __fadd2_rn(fc, make_float2(v.z, v.w));
            }
            store_partial(A.partials, pr->part_begin + local * n_out + l,
                          ddv{static_cast<double>(fs.x), static_cast<double>(fc.x)},
                          ddv{static_cast<double>(fs.y), static_cast<double>(fc.y)});
        }
        __syncwarp();  // the slices are read before the next item clears them
    }
}

// Complex64 Laplace walk for unit columns (the exact sampler's case), two
// inner codes per iteration.  Codes a = 2u and b = 2u + 1 of the same outer
// position ride in the two lanes of Blackwell's packed FP32x2 instructions
// (__fadd2_rn, __fmul2_rn, __ffma2_rn; each lane rounded as the scalar
// instruction).  The plan stores the prefix table as code pairs, one float4
// {re_a, re_b, im_a, im_b} per column (prep.cuh, `pairs`; an odd P gets a
// zero pad code of weight 0), so one load feeds both codes, and the seeds
// stay scalar: each column sum is two scalar adds into adjacent registers.
// The columns are split into two halves, each with its own prefix chain and
// suffix chain, so every pass runs two independent dependency chains of
// packed multiplies.  A block takes four consecutive items of one problem
// (one per warp) and stages that problem's code-pair table in shared memory
// (the plan caps P at PQG_PAIRS_TABLE_P codes), so the rows are broadcast
// shared-memory loads.  The step weight of each code times the lane's outer
// weight starts the suffix chains (an exact FP32 integer: the sampler's
// weights stay below 2^24), so both codes add into one FP32 partial sum per
// output (re_a + re_b, then into the sum), folded every 16 code pairs into
// per-lane TwoSum-compensated FP32 sums (value and error word), which the
// warp's lanes then combine the same way.  No FP64 instruction runs in the
// walk: on GB300 one FP64 warp instruction holds its pipe for tens of
// cycles, and an FP64 fold stalled the folding warp while its SMSP had one
// other warp to issue from.  Prefix products of both codes sit in one
// float4 per column in registers; the per-output FP32 partial sums and the
// compensated sums in column-major slices of shared memory (a partial sum
// is read and written once per output per code pair, where shared prefix
// products would cost a store and a load of a float4 per column).
template <int NC>
struct LaplaceC64PCfg {
    static constexpr int TAB_PAIRS = PQG_PAIRS_TABLE_P / 2;  // code pairs the staged table holds
    static constexpr size_t smem_bytes = size_t(NC + 1) * PQG_WALK_THREADS * sizeof(float4) +
                                         size_t(NC + 1) * PQG_WALK_THREADS * sizeof(float2) +
                                         size_t(TAB_PAIRS) * NC * sizeof(float4);
};

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
constexpr int LAP64P_G = 8;

template <int NC>
__global__ void __launch_bounds__(PQG_WALK_THREADS, 2) walk_laplace_c64p(WalkArgs A) {
    static_assert(NC >= 2, "unit-column Laplace walks have at least two columns");
    static_assert(PQG_ITEM_GROUP * 32 == PQG_WALK_THREADS, "one item per warp of a block");
    using Cfg = LaplaceC64PCfg<NC>;
    extern __shared__ double2 lap_smem64p[];
    const int lane = threadIdx.x & 31;
    // the block's problem's code-pair table (at most Cfg::TAB_PAIRS pairs: the plan caps P)
    float4 *s_tab = reinterpret_cast<float4 *>(lap_smem64p + (NC + 1) * PQG_WALK_THREADS) +
                    (NC + 1) * PQG_WALK_THREADS / 2;
    __shared__ unsigned long long s_group;
    int staged = -1;
    // per-lane compensated FP32 sums of every output, {re, im, re_err, im_err}
    float4 *const acc_base = reinterpret_cast<float4 *>(lap_smem64p);
    LaneArray<float4, NC + 1, true> acc;
    acc.init(acc_base, threadIdx.x);
    LaneArray<float2, NC + 1, true> part;  // per-lane FP32 partial sums {re, im} of every output
    part.init(reinterpret_cast<float2 *>(lap_smem64p + (NC + 1) * PQG_WALK_THREADS), threadIdx.x);
    LaneArray<float4, NC, false> pre;  // prefix products {re_a, re_b, im_a, im_b}, registers
    pre.init(nullptr, threadIdx.x);

    for (;;) {
        // a block takes PQG_ITEM_GROUP consecutive items of one problem at once
        // (one per warp; the plan makes every problem whole groups), so the
        // exit is uniform over the block
        __syncthreads();  // every warp has read the previous group and its table
        if (threadIdx.x == 0) s_group = atomicAdd(A.counter, 1ULL);
        __syncthreads();
        const int64_t item = static_cast<int64_t>(s_group) * PQG_ITEM_GROUP + (threadIdx.x >> 5);
        if (item >= A.total_items) return;
        const int ip = find_problem(A.item_begin, A.n_probs, item);
        const PqgProblem *pr = A.probs + ip;
        if (ip != staged) {
            // stage the problem's code-pair table once for the block's warps
            const float4 *src = reinterpret_cast<const float4 *>(A.delta) + pr->delta_begin / 2;
            const int np = (pr->P + 1) >> 1;
            const int n = (np < Cfg::TAB_PAIRS ? np : Cfg::TAB_PAIRS) * NC;
            for (int e = threadIdx.x; e < n; e += PQG_WALK_THREADS) s_tab[e] = src[e];
            staged = ip;
            __syncthreads();
        }
        const int64_t local = item - pr->item_begin;
        const int64_t R = pr->R;
        const int64_t r0 = (local * PQG_ITEM_LANES + lane) * R;
        const int n_out = pr->n_out;
        const bool full = n_out > NC;
        const bool active = r0 < pr->Q;
#pragma unroll
        for (int l = 0; l <= NC; ++l) {  // (an idle lane's sums join the lane reduction too)
            part.set(l, make_float2(0.0f, 0.0f));
            acc.set(l, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
        }
        if (active) {
            float sr0[NC], si0[NC];  // seed of the current outer position (double-float, rounded)
            OuterState st;
            outer_decode(pr, r0, st);
            {
                ArF32::cs_t s[NC];
                seed_lane<ArF32, NC>(pr, A.arena, st, s);
#pragma unroll
                for (int j = 0; j < NC; ++j) {
                    sr0[j] = s[j].r;
                    si0[j] = s[j].i;
                }
            }
            float wout = static_cast<float>(outer_weight(pr, st));
            const int64_t my_R = (pr->Q - r0 < R) ? (pr->Q - r0) : R;
            const float2 *D = reinterpret_cast<const float2 *>(A.arena + pr->off_D);
            const PqgStep *tab = reinterpret_cast<const PqgStep *>(A.arena + pr->off_tab);
            const int P = pr->P;
            // (the staged table holds at most Cfg::TAB_PAIRS pairs: the plan guarantees P
            // fits; the bound keeps every read inside it)
            const int pairs = ((P + 1) >> 1) < Cfg::TAB_PAIRS ? ((P + 1) >> 1) : Cfg::TAB_PAIRS;
            for (int64_t seg = 0; seg < my_R; ++seg) {
                for (int u = 0; u < pairs; ++u) {
                    const int ta = 2 * u, tb = ta + 1;
                    // step weights times the outer weight (the pad code weighs 0)
                    const float2 w2 = f2(__fmul_rn(__ldg(&tab[ta].wf), wout),
                                         tb < P ? __fmul_rn(__ldg(&tab[tb].wf), wout) : 0.0f);
                    const float4 *d = s_tab + u * NC;
                    // (plain loads, which the compiler barriers below order: the suffix
                    // pass reloads its rows rather than keeping the prefix pass's live)
                    auto col = [&](int j, float2 &cr, float2 &ci) {
                        const float4 v = d[j];
                        cr = f2(__fadd_rn(sr0[j], v.x), __fadd_rn(sr0[j], v.y));
                        ci = f2(__fadd_rn(si0[j], v.z), __fadd_rn(si0[j], v.w));
                    };
                    // Halves: low 0..H-1 and high H..NC-1.  Prefix pass: pre_l =
                    // prod_{k<l} c_k within the low half (l = 1..H-1) and
                    // prod_{H<=k<l} c_k within the high half (l = H+1..NC-1); the
                    // chains end at P_lo and P_hi, the halves' products.  Suffix pass:
                    // the high chain starts at w P_lo, the low one at w P_hi, so
                    // out_l = pre_l * (chain after the columns above l in its half)
                    // = w prod_{k != l} c_k.  (A compiler barrier every LAP64P_G steps
                    // keeps at most that many table rows in flight.)
                    constexpr int H = NC / 2;
                    float2 xlr, xli, xhr, xhi;
#pragma unroll
                    for (int i = 0; i < NC - H; ++i) {
                        if (i % LAP64P_G == 0) asm volatile("" ::: "memory");
                        if (i < H) {
                            float2 cr, ci;
                            col(i, cr, ci);
                            if (i == 0) {
                                xlr = cr;
                                xli = ci;
                            } else {
                                cmul2(xlr, xli, cr, ci);
                            }
                            if (i + 1 < H) pre.set(i + 1, make_float4(xlr.x, xlr.y, xli.x, xli.y));
                        }
                        {
                            const int j = H + i;
                            float2 cr, ci;
                            col(j, cr, ci);
                            if (i == 0) {
                                xhr = cr;
                                xhi = ci;
                            } else {
                                cmul2(xhr, xhi, cr, ci);
                            }
                            if (j + 1 < NC) pre.set(j + 1, make_float4(xhr.x, xhr.y, xhi.x, xhi.y));
                        }
                    }
                    float2 shr = __fmul2_rn(w2, xlr), shi = __fmul2_rn(w2, xli);  // w P_lo
                    float2 slr = __fmul2_rn(w2, xhr), sli = __fmul2_rn(w2, xhi);  // w P_hi
#pragma unroll
                    for (int i = 0; i < NC - H; ++i) {
                        if (i % LAP64P_G == 0) asm volatile("" ::: "memory");
                        {
                            const int l = NC - 1 - i;  // high half, from the top
                            float2 cr, ci;
                            col(l, cr, ci);
                            float2 tr = shr, ti = shi;
                            if (l > H) {
                                const float4 p = pre.get(l);
                                tr = f2(p.x, p.y);
                                ti = f2(p.z, p.w);
                                cmul2(tr, ti, shr, shi);
                            }
                            float2 q = part.get(l);
                            q.x = __fadd_rn(q.x, __fadd_rn(tr.x, tr.y));
                            q.y = __fadd_rn(q.y, __fadd_rn(ti.x, ti.y));
                            part.set(l, q);
                            if (l > H || full) cmul2(shr, shi, cr, ci);  // at l = H: w prod of every column
                        }
                        if (i < H) {
                            const int l = H - 1 - i;  // low half, from the top
                            float2 cr, ci;
                            col(l, cr, ci);
                            float2 tr = slr, ti = sli;
                            if (l > 0) {
                                const float4 p = pre.get(l);
                                tr = f2(p.x, p.y);
                                ti = f2(p.z, p.w);
                                cmul2(tr, ti, slr, sli);
                            }
                            float2 q = part.get(l);
                            q.x = __fadd_rn(q.x, __fadd_rn(tr.x, tr.y));
                            q.y = __fadd_rn(q.y, __fadd_rn(ti.x, ti.y));
                            part.set(l, q);
                            if (l > 0) cmul2(slr, sli, cr, ci);
                        }
                    }
                    if (full) {
                        float2 q = part.get(NC);
                        q.x = __fadd_rn(q.x, __fadd_rn(shr.x, shr.y));
                        q.y = __fadd_rn(q.y, __fadd_rn(shi.x, shi.y));
                        part.set(NC, q);
                    }
                    if ((u & 15) == 15 || u == pairs - 1) {
#pragma unroll
                        for (int l = 0; l <= NC; ++l) {
                            if (l == NC && !full) continue;
                            const float4 a = acc.get(l);
                            float2 s = f2(a.x, a.y), c = f2(a.z, a.w);
                            two_sum_acc2(s, c, part.get(l));
                            acc.set(l, make_float4(s.x, s.y, c.x, c.y));
                            part.set(l, make_float2(0.0f, 0.0f));
                        }
                    }
                }
                if (seg + 1 < my_R) {  // one-digit step to the next outer position
                    bool up = false;
                    const int k = outer_next(pr, st, &up);
                    const float2 *dd = D + (2 * k + (up ? 0 : 1)) * NC;
#pragma unroll
                    for (int j = 0; j < NC; ++j) {
                        sr0[j] = __fadd_rn(sr0[j], dd[j].x);
                        si0[j] = __fadd_rn(si0[j], dd[j].y);
                    }
                    wout = static_cast<float>(outer_weight(pr, st));
                }
            }
        }
        // lane reduction: lane l sums output l over the warp's 32 lanes,
        // reading the slices in a rotated order (lane l starts at lane l's
        // slot), so each quarter-warp's float4 loads hit distinct banks
        __syncwarp();
        if (lane < n_out) {
            const float4 *src = acc_base + lane * PQG_WALK_THREADS + (threadIdx.x & ~31);
            float2 s = f2(0.0f, 0.0f), c = f2(0.0f, 0.0f);
#pragma unroll 8
            for (int k = 0; k < 32; ++k) {
                const float4 v = src[(k + lane) & 31];
                two_sum_acc2(s, c, f2(v.x, v.y));
                c = __fadd2_rn(c, f2(v.z, v.w));
            }
            store_partial(A.partials, pr->part_begin + local * n_out + lane,
                          ddv{static_cast<double>(s.x), static_cast<double>(c.x)},
                          ddv{static_cast<double>(s.y), static_cast<double>(c.y)});
        }
    }
}

template <int NC>
struct LaplaceDfCfg {
    static constexpr size_t smem_bytes = size_t(2 * NC + 1) * PQG_WALK_THREADS * sizeof(float4);
};

// Complex128 Laplace walk in double-float arithmetic on the FP32 pipes (the
// default for complex128 when the plan is in the double-float domain; ONES:
// every column has multiplicity 1, the sampler's usual case): double-float
// seeds and column sums seed + Delta(t), prefix and suffix products with
// unnormalised double-float pairs (df_cmul_lazy), and the step's whole weight
// w(t) * w_outer folded into the suffix's start -- an exact FP32 integer, as
// the plan checks (max inner weight x max outer weight <= 2^24), so that one
// set of per-output double-float sums (renormalising adds) spans all of a
// lane's positions.  Those sums and the prefix products live in shared memory
// (registers hold the seeds); lanes are combined in double-double.  About
// 2^-48 per operation, against 2^-53 for the FP64 walk, on pipes 61x faster.
template <int NC, bool ONES>
__global__ void __launch_bounds__(PQG_WALK_THREADS, 2) walk_laplace_df(WalkArgs A) {
    extern __shared__ float4 lap_smem_df[];
    const int lane = threadIdx.x & 31;
    LaneArray<float4, NC + 1, true> acc;  // per-output sums {re_hi, re_lo, im_hi, im_lo}
    acc.init(lap_smem_df, threadIdx.x);
    LaneArray<float4, NC, true> pre;  // prefix products, the same layout
    pre.init(lap_smem_df + (NC + 1) * PQG_WALK_THREADS, threadIdx.x);

    for (;;) {
        const int64_t item = next_item(A.counter, lane);
        if (item >= A.total_items) return;
        const int ip = find_problem(A.item_begin, A.n_probs, item);
        const PqgProblem *pr = A.probs + ip;
        const int64_t local = item - pr->item_begin;
        const int64_t R = pr->R;
        const int64_t r0 = (local * PQG_ITEM_LANES + lane) * R;
        const int n_out = pr->n_out;
        const bool full = n_out > NC;
        const bool active = r0 < pr->Q;
#pragma unroll
        for (int l = 0; l <= NC; ++l)  // (an idle lane's sums join the lane reduction too)
            acc.set(l, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
        if (active) {
            dfl sr0[NC], si0[NC];  // double-float seed of the current outer position
            OuterState st;
            outer_decode(pr, r0, st);
            {
                ArDF::cs_t s[NC];
                seed_lane<ArDF, NC>(pr, A.arena, st, s);
#pragma unroll
                for (int j = 0; j < NC; ++j) {
                    sr0[j] = s[j].r;
                    si0[j] = s[j].i;
                }
            }
            // the outer weight as a float: the plan checks that every inner
            // weight times every outer weight is an integer below 2^24, so the
            // step's whole weight is one exact FP32 product
            float wout = static_cast<float>(outer_weight(pr, st));
            const int64_t my_R = (pr->Q - r0 < R) ? (pr->Q - r0) : R;
            const float4 *D = reinterpret_cast<const float4 *>(A.arena + pr->off_D);
            const PqgStep *tab = reinterpret_cast<const PqgStep *>(A.arena + pr->off_tab);
            const float4 *delta = reinterpret_cast<const float4 *>(A.delta) + pr->delta_begin;
            const int P = pr->P;
            // column multiplicities (repeated-column kernel): read from the
            // problem record (L1, the same for the whole warp), not registers
            const uint8_t *cm = pr->cm;
            auto add_to = [&](int l, dfl tr, dfl ti) {
                const float4 a = acc.get(l);
                const dfl r = df_add(dfl{a.x, a.y}, tr), i = df_add(dfl{a.z, a.w}, ti);
                acc.set(l, make_float4(r.hi, r.lo, i.hi, i.lo));
            };

            for (int64_t seg = 0; seg < my_R; ++seg) {
                for (int t = 0; t < P; ++t) {
                    // the whole weight, an exact FP32 integer (checked by the plan)
                    const float w = __fmul_rn(__ldg(&tab[t].wf), wout);
                    const float4 *d = delta + static_cast<int64_t>(t) * NC;
                    // column sums: high words on the 2^-23 grid (walk_df.cuh), exact
                    auto col = [&](int j, dfl &cr, dfl &ci) {
                        const float4 v = __ldg(d + j);
                        cr = df_grid_sum(sr0[j], dfl{v.x, v.y});
                        ci = df_grid_sum(si0[j], dfl{v.z, v.w});
                    };
                    // prefix products: pre_l = prod_{k<l} c_k
                    dfl xr{1.0f, 0.0f}, xi{0.0f, 0.0f};
#pragma unroll
                    for (int j = 0; j + 1 < NC; ++j) {
                        dfl cr, ci;
                        col(j, cr, ci);
                        if (j == 0) {
                            xr = cr;
                            xi = ci;
                            if constexpr (!ONES)
                                for (int r = 1; r < cm[0]; ++r) df_cmul_lazy(xr, xi, cr, ci);
                        } else if constexpr (ONES) {
                            df_cmul_lazy(xr, xi, cr, ci);
                        } else {
                            for (int r = 0; r < cm[j]; ++r) df_cmul_lazy(xr, xi, cr, ci);
                        }
                        pre.set(j + 1, make_float4(xr.hi, xr.lo, xi.hi, xi.lo));
                    }
                    // suffix pass: out_l += w * pre_l * prod_{k>l} c_k
                    dfl sr{w, 0.0f}, si{0.0f, 0.0f};
#pragma unroll
                    for (int l = NC - 1; l >= 0; --l) {
                        dfl cr, ci;
                        col(l, cr, ci);
                        dfl tr, ti;
                        if (l == NC - 1) {
                            // (pre_0 = 1 is never stored: one column reads the constant)
                            const float4 p = l == 0 ? make_float4(1.0f, 0.0f, 0.0f, 0.0f) : pre.get(l);
                            tr = df_scale(dfl{p.x, p.y}, w);
                            ti = df_scale(dfl{p.z, p.w}, w);
                        } else if (l == 0) {
                            tr = sr;
                            ti = si;
                        } else {
                            const float4 p = pre.get(l);
                            tr = dfl{p.x, p.y};
                            ti = dfl{p.z, p.w};
                            df_cmul_lazy(tr, ti, sr, si);
                        }
                        if constexpr (!ONES)  // out_l keeps cols_l - 1 factors of c_l
                            for (int r = 1; r < cm[l]; ++r) df_cmul_lazy(tr, ti, cr, ci);
                        add_to(l, tr, ti);
                        if (l > 0 || full) {
                            if (l == NC - 1) {
                                sr = df_scale(cr, w);
                                si = df_scale(ci, w);
                                if constexpr (!ONES)
                                    for (int r = 1; r < cm[l]; ++r) df_cmul_lazy(sr, si, cr, ci);
                            } else if constexpr (ONES) {
                                df_cmul_lazy(sr, si, cr, ci);
                            } else {
                                for (int r = 0; r < cm[l]; ++r) df_cmul_lazy(sr, si, cr, ci);
                            }
                        }
                    }
                    if (full) add_to(NC, sr, si);
                }
                if (seg + 1 < my_R) {  // one-digit step to the next outer position
                    bool up = false;
                    const int k = outer_next(pr, st, &up);
                    const float4 *dd = D + (2 * k + (up ? 0 : 1)) * NC;
#pragma unroll
                    for (int j = 0; j < NC; ++j) {
                        const float4 v = dd[j];
                        sr0[j] = df_grid_add(sr0[j], dfl{v.x, v.y});
                        si0[j] = df_grid_add(si0[j], dfl{v.z, v.w});
                    }
                    wout = static_cast<float>(outer_weight(pr, st));
                }
            }
        }
        // lane reduction: lane l sums output l (and l + 32) over the warp's 32
        // lanes in double-float on the FP32 pipes, reading the slices in a
        // rotated order (lane l starts at lane l's slot) so that each
        // quarter-warp's float4 loads hit distinct banks
        __syncwarp();
        for (int l = lane; l < n_out; l += 32) {
            const float4 *src = lap_smem_df + l * PQG_WALK_THREADS + (threadIdx.x & ~31);
            dfl r{0.0f, 0.0f}, i{0.0f, 0.0f};
#pragma unroll 4
            for (int k = 0; k < 32; ++k) {
                const float4 v = src[(k + lane) & 31];
                r = df_add(r, dfl{v.x, v.y});
                i = df_add(i, dfl{v.z, v.w});
            }
            store_partial(A.partials, pr->part_begin + local * n_out + l,
                          ddv{static_cast<double>(r.hi), static_cast<double>(r.lo)},
                          ddv{static_cast<double>(i.hi), static_cast<double>(i.lo)});
        }
        __syncwarp();  // the slices are read before the next item clears them
    }
}

}  // namespace pqg
