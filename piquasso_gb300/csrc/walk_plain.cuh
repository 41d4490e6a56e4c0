// Plain permanent walk kernels (one output per problem), one template for the
// three arithmetics:
//   ArF64 — complex128: FP64 column sums, updates and products;
//   ArF32 — complex64: FP32 updates and products, FP32 TwoSum-compensated sums;
//   ArDF  — complex128 accuracy on the FP32 pipes: double-float updates and
//           products (see walk_df.cuh).
// All seeds are formed at 48 bits or more (FP64 for ArF64, double-float for the
// FP32-pipe kernels, whose FP64 pipe runs at 1/61 of the FP32 rate on GB300),
// and every segment's sum is folded into a per-lane double-double.
//
// Schedule (method of the reference's src/permanent.cpp:155-250, with the
// Gray-code space split into a lock-step inner walk and per-lane outer runs):
// a persistent grid; every warp pulls work items (one problem, 32 lanes x R
// outer positions) from a device queue.  Each lane seeds its column sums at
// its first outer position, then for each of its R positions walks the
// problem's P inner codes — forward, then backward, alternately — and between
// positions applies the one-digit outer update of the reflected Gray code to
// its seed.  At inner code t the column sums are seed + Delta(t): one prefix-
// table row, the same for the whole warp (broadcast loads), one addition per
// column, no accumulated rounding; then one product over the columns.
#pragma once
#include "walk_common.cuh"
#include "walk_df.cuh"

namespace pqg {

// ------------------------------------------------------------------ policies
struct ArF64 {
    struct cs_t {
        double r, i;
    };
    using d_t = double2;  // outer update rows
    using t_t = double2;  // prefix-table entries
    struct acc_t {
        double r, i;
    };
    static constexpr bool kDfSeed = false;
    static constexpr bool kTwoChains = false;  // FP64-pipe bound: one chain
    static constexpr bool kPairSteps = false;
    static constexpr bool kTwoSeeds = false;
    __device__ __forceinline__ static cs_t from_seed64(double r, double i) { return {r, i}; }
    __device__ __forceinline__ static cs_t from_seed_df(dfl r, dfl i) { return {r.hi, i.hi}; }
    __device__ __forceinline__ static void update(cs_t &c, const d_t &d) {
        c.r = __dadd_rn(c.r, d.x);
        c.i = __dadd_rn(c.i, d.y);
    }
    __device__ __forceinline__ static cs_t sum(const cs_t &c, const d_t &d) {
        return {__dadd_rn(c.r, d.x), __dadd_rn(c.i, d.y)};
    }
    __device__ __forceinline__ static void mul(cs_t &x, const cs_t &y) { cmul(x.r, x.i, y.r, y.i); }
    __device__ __forceinline__ static acc_t zero() { return {0.0, 0.0}; }
    __device__ __forceinline__ static void accumulate(acc_t &a, const cs_t &x, const PqgStep &s) {
        a.r = __fma_rn(s.wd, x.r, a.r);
        a.i = __fma_rn(s.wd, x.i, a.i);
    }
    __device__ __forceinline__ static void fold(ddv &sr, ddv &si, const acc_t &a, double w) {
        sr = dd_add(sr, dd_mul_d(ddv{a.r, 0.0}, w));
        si = dd_add(si, dd_mul_d(ddv{a.i, 0.0}, w));
    }
};

struct ArF32 {
    struct cs_t {
        float r, i;
    };
    using d_t = float2;  // outer update rows
    using t_t = float4;  // prefix-table entries {re, re, im, im}: one load feeds both packed lanes
    struct acc_t {
        float r, cr, i, ci;  // TwoSum-compensated partial sums
    };
    static constexpr bool kDfSeed = true;
    static constexpr bool kTwoChains = true;
    // latency bound on the prefix-table loads: each lane walks two outer
    // positions against every loaded table row (half the loads per product,
    // four independent multiply chains); a lane's odd last position walks
    // alone, two codes per iteration
    static constexpr bool kPairSteps = true;
    static constexpr bool kTwoSeeds = true;
    __device__ __forceinline__ static cs_t from_seed64(double r, double i) {
        return {__double2float_rn(r), __double2float_rn(i)};
    }
    __device__ __forceinline__ static cs_t from_seed_df(dfl r, dfl i) {
        return {__fadd_rn(r.hi, r.lo), __fadd_rn(i.hi, i.lo)};
    }
    __device__ __forceinline__ static void update(cs_t &c, const d_t &d) {
        c.r = __fadd_rn(c.r, d.x);
        c.i = __fadd_rn(c.i, d.y);
    }
    __device__ __forceinline__ static cs_t sum(const cs_t &c, const t_t &d) {
        return {__fadd_rn(c.r, d.x), __fadd_rn(c.i, d.z)};
    }
    __device__ __forceinline__ static void mul(cs_t &x, const cs_t &y) { cmulf(x.r, x.i, y.r, y.i); }
    __device__ __forceinline__ static acc_t zero() { return {0.0f, 0.0f, 0.0f, 0.0f}; }
    __device__ __forceinline__ static void accumulate(acc_t &a, const cs_t &x, const PqgStep &s) {
        f_two_sum_acc(a.r, a.cr, __fmul_rn(s.wf, x.r));
        f_two_sum_acc(a.i, a.ci, __fmul_rn(s.wf, x.i));
    }
    __device__ __forceinline__ static void fold(ddv &sr, ddv &si, const acc_t &a, double w) {
        const ddv r = dd_add_d(ddv{static_cast<double>(a.r), 0.0}, static_cast<double>(a.cr));
        const ddv i = dd_add_d(ddv{static_cast<double>(a.i), 0.0}, static_cast<double>(a.ci));
        sr = dd_add(sr, dd_mul_d(r, w));
        si = dd_add(si, dd_mul_d(i, w));
    }
};

struct ArDF {
    struct cs_t {
        dfl r, i;
    };
    using d_t = float4;  // re_hi, re_lo, im_hi, im_lo
    using t_t = float4;
    struct acc_t {
        dfl r, i;
    };
    static constexpr bool kDfSeed = true;
    static constexpr bool kTwoChains = true;
    static constexpr bool kPairSteps = false;  // enough independent work per code already
    static constexpr bool kTwoSeeds = false;   // FMA-pipe bound; its seeds need the registers
    // seeds, update rows and prefix-table entries keep their high words on the
    // grid of multiples of 2^-23 (walk_df.cuh): a column sum is two exact-high adds
    __device__ __forceinline__ static cs_t from_seed64(double r, double i) {
        return {df_to_grid(df_split(r)), df_to_grid(df_split(i))};
    }
    __device__ __forceinline__ static cs_t from_seed_df(dfl r, dfl i) { return {df_to_grid(r), df_to_grid(i)}; }
    __device__ __forceinline__ static void update(cs_t &c, const d_t &d) {
        c.r = df_grid_add(c.r, dfl{d.x, d.y});
        c.i = df_grid_add(c.i, dfl{d.z, d.w});
    }
    __device__ __forceinline__ static cs_t sum(const cs_t &c, const d_t &d) {
        return {df_grid_sum(c.r, dfl{d.x, d.y}), df_grid_sum(c.i, dfl{d.z, d.w})};
    }
    // products feed products: unnormalised pairs (df_cmul_lazy); the
    // accumulation renormalises (df_scale, df_add)
    __device__ __forceinline__ static void mul(cs_t &x, const cs_t &y) { df_cmul_lazy(x.r, x.i, y.r, y.i); }
    __device__ __forceinline__ static acc_t zero() { return {{0.0f, 0.0f}, {0.0f, 0.0f}}; }
    __device__ __forceinline__ static void accumulate(acc_t &a, const cs_t &x, const PqgStep &s) {
        a.r = df_add(a.r, df_scale(x.r, s.wf));
        a.i = df_add(a.i, df_scale(x.i, s.wf));
    }
    __device__ __forceinline__ static void fold(ddv &sr, ddv &si, const acc_t &a, double w) {
        const ddv r = dd_add_d(ddv{static_cast<double>(a.r.hi), 0.0}, static_cast<double>(a.r.lo));
        const ddv i = dd_add_d(ddv{static_cast<double>(a.i.hi), 0.0}, static_cast<double>(a.i.lo));
        sr = dd_add(sr, dd_mul_d(r, w));
        si = dd_add(si, dd_mul_d(i, w));
    }
};

// --------------------------------------------------------- outer Gray state
// Per-lane position in the reflected mixed-radix Gray code over the outer
// digits (digit 0 fastest): counter digits c and code digits g.
struct OuterState {
    uint8_t c[PQG_MAX_OUTER];
    uint8_t g[PQG_MAX_OUTER];
};

// Decodes position r into the counter digits c and the reflected code g.
__device__ __forceinline__ void outer_decode(const PqgProblem *__restrict__ pr, int64_t r, OuterState &st) {
    const int n = pr->n_outer;
    for (int o = 0; o < n; ++o) {
        const int L = pr->outer_m[o] + 1;
        st.c[o] = static_cast<uint8_t>(r % L);
        r /= L;
    }
    int parity = 0;
    for (int o = n - 1; o >= 0; --o) {
        const int L = pr->outer_m[o] + 1;
        const int code = parity ? L - 1 - st.c[o] : st.c[o];
        st.g[o] = static_cast<uint8_t>(code);
        parity ^= (code & 1);
    }
}

// Advances to the next position: the incremented counter digit k is the only
// code digit that changes, by +1 when the higher code digits sum to an even
// number, else by -1.  Returns k; *up receives the direction.
__device__ __forceinline__ int outer_next(const PqgProblem *__restrict__ pr, OuterState &st, bool *up) {
    const int n = pr->n_outer;
    int k = 0;
    while (k < n - 1 && st.c[k] == pr->outer_m[k]) {
        st.c[k] = 0;
        ++k;
    }
    st.c[k] = static_cast<uint8_t>(st.c[k] + 1);
    int par = 0;
    for (int o = k + 1; o < n; ++o) par ^= (st.g[o] & 1);
    *up = (par == 0);
    st.g[k] = static_cast<uint8_t>(st.g[k] + (*up ? 1 : -1));
    return k;
}

// signed weight of the current outer code: (-1)^sum(g) prod C(m, g)
__device__ __forceinline__ double outer_weight(const PqgProblem *__restrict__ pr, const OuterState &st) {
    int64_t w = 1;
    int par = 0;
    for (int o = 0; o < pr->n_outer; ++o) {
        const int g = st.g[o];
        if (g) {
            w *= binom64(pr->outer_m[o], g);
            par += g;
        }
    }
    return (par & 1) ? -static_cast<double>(w) : static_cast<double>(w);
}

template <class Ar, int NC>
__device__ __forceinline__ void seed_lane(const PqgProblem *__restrict__ pr, const unsigned char *__restrict__ arena,
                                          const OuterState &st, typename Ar::cs_t (&cs)[NC]) {
    if constexpr (Ar::kDfSeed) {
        // double-float seed on the FP32 pipes: base - 2 sum_o g_o a_o
        const float4 *base = reinterpret_cast<const float4 *>(arena + pr->off_base_df);
        const float4 *orow = reinterpret_cast<const float4 *>(arena + pr->off_outer_df);
        dfl sr[NC], si[NC];
#pragma unroll
        for (int j = 0; j < NC; ++j) {
            const float4 v = __ldg(base + j);
            sr[j] = dfl{v.x, v.y};
            si[j] = dfl{v.z, v.w};
        }
        for (int o = 0; o < pr->n_outer; ++o) {
            const int g = st.g[o];
            if (!g) continue;
            const float f = -2.0f * static_cast<float>(g);
            const float4 *r = orow + static_cast<int64_t>(o) * NC;
#pragma unroll
            for (int j = 0; j < NC; ++j) {
                const float4 v = __ldg(r + j);
                sr[j] = df_add(sr[j], df_scale(dfl{v.x, v.y}, f));
                si[j] = df_add(si[j], df_scale(dfl{v.z, v.w}, f));
            }
        }
#pragma unroll
        for (int j = 0; j < NC; ++j) cs[j] = Ar::from_seed_df(sr[j], si[j]);
    } else {
        const double2 *base = reinterpret_cast<const double2 *>(arena + pr->off_base64);
        const double2 *orow = reinterpret_cast<const double2 *>(arena + pr->off_outer64);
        double cr[NC], ci[NC];
#pragma unroll
        for (int j = 0; j < NC; ++j) {
            const double2 v = __ldg(base + j);
            cr[j] = v.x;
            ci[j] = v.y;
        }
        for (int o = 0; o < pr->n_outer; ++o) {
            const int g = st.g[o];
            if (!g) continue;
            const double f = -2.0 * g;
            const double2 *r = orow + static_cast<int64_t>(o) * NC;
#pragma unroll
            for (int j = 0; j < NC; ++j) {
                const double2 v = __ldg(r + j);
                cr[j] = __fma_rn(f, v.x, cr[j]);
                ci[j] = __fma_rn(f, v.y, ci[j]);
            }
        }
#pragma unroll
        for (int j = 0; j < NC; ++j) cs[j] = Ar::from_seed64(cr[j], ci[j]);
    }
}

// Product of the column sums seed_j + delta_j (delta_j: the inner code's
// prefix-table row) with their multiplicities.  Each column sum is formed
// right before it enters the product, so a loaded table value is consumed at
// once.  FP32-pipe arithmetics multiply even and odd columns in two independent
// chains (twice the instruction-level parallelism of one serial chain) and
// join them at the end.
template <class Ar, int NC>
__device__ __forceinline__ typename Ar::cs_t row_product(const typename Ar::cs_t (&seed)[NC],
                                                         const typename Ar::t_t *__restrict__ d,
                                                         const uint8_t *__restrict__ cm, bool ones) {
    using cs_t = typename Ar::cs_t;
    constexpr bool two = Ar::kTwoChains && NC >= 4;
    const cs_t c0 = Ar::sum(seed[0], d[0]);
    cs_t x = c0;
    cs_t y;
    if constexpr (two) y = Ar::sum(seed[1], d[1]);
    if (ones) {
#pragma unroll
        for (int j = two ? 2 : 1; j < NC; ++j) {
            const cs_t c = Ar::sum(seed[j], d[j]);
            if (two && (j & 1))
                Ar::mul(y, c);
            else
                Ar::mul(x, c);
        }
    } else {
        for (int r = 1; r < cm[0]; ++r) Ar::mul(x, c0);
        if constexpr (two) {
            const cs_t c1 = y;
            for (int r = 1; r < cm[1]; ++r) Ar::mul(y, c1);
        }
#pragma unroll
        for (int j = two ? 2 : 1; j < NC; ++j) {
            const cs_t c = Ar::sum(seed[j], d[j]);
            for (int r = 0; r < cm[j]; ++r) {
                if (two && (j & 1))
                    Ar::mul(y, c);
                else
                    Ar::mul(x, c);
            }
        }
    }
    if constexpr (two) Ar::mul(x, y);
    return x;
}

// --------------------------------------------- packed two-seed complex64 walk
// The two outer positions a complex64 lane walks together ride side by side in
// Blackwell's packed FP32 instructions (__fadd2_rn, __fmul2_rn, __ffma2_rn:
// FADD2 / FMUL2 / FFMA2, each lane rounded as the scalar instruction): lane .x
// is position A, lane .y position B.  A column sum, a complex product and a
// compensated accumulation are then one packed instruction for both
// positions — half the FP32 instructions of two scalar walks — and every
// prefix-table value, stored duplicated {re, re, im, im}, is one 16-byte load
// that feeds both lanes.
__device__ __forceinline__ float2 f2neg(float2 a) { return make_float2(-a.x, -a.y); }

// (xr + i xi) *= (cr + i ci) per lane, with cmulf's rounding
__device__ __forceinline__ void cmul2(float2 &xr, float2 &xi, float2 cr, float2 ci) {
    const float2 r = __ffma2_rn(xr, cr, f2neg(__fmul2_rn(xi, ci)));
    const float2 i = __ffma2_rn(xr, ci, __fmul2_rn(xi, cr));
    xr = r;
    xi = i;
}

// TwoSum-compensated s += y per lane (f_two_sum_acc)
__device__ __forceinline__ void two_sum_acc2(float2 &s, float2 &c, float2 y) {
    const float2 t = __fadd2_rn(s, y);
    const float2 bb = __fadd2_rn(t, f2neg(s));
    const float2 e = __fadd2_rn(__fadd2_rn(s, f2neg(__fadd2_rn(t, f2neg(bb)))), __fadd2_rn(y, f2neg(bb)));
    s = t;
    c = __fadd2_rn(c, e);
}

// (s + c) += (a.r + a.cr, a.i + a.ci) * w, {re, im} packed, in FP32 only: the
// weight (an integer) split as w_hi + w_lo, the leading product's rounding
// error recovered exactly by an FMA, the sum by TwoSum (two_sum_acc2).  About
// 2^-44 of the lane's largest partial, far inside the complex64 walk's own
// rounding; it keeps the fold off GB300's FP64 pipe, where one warp
// instruction holds the pipe for tens of cycles.
__device__ __forceinline__ void ff_fold(float2 &s, float2 &c, float r, float cr, float i, float ci, double w) {
    const float wh = __double2float_rn(w);
    const float wl = __double2float_rn(w - static_cast<double>(wh));
    const float2 vh = make_float2(r, i), vl = make_float2(cr, ci);
    const float2 wh2 = make_float2(wh, wh), wl2 = make_float2(wl, wl);
    const float2 ph = __fmul2_rn(vh, wh2);
    const float2 pe = __ffma2_rn(vh, wh2, f2neg(ph));
    const float2 pl = __fadd2_rn(pe, __ffma2_rn(vh, wl2, __fmul2_rn(vl, wh2)));
    two_sum_acc2(s, c, ph);
    c = __fadd2_rn(c, pl);
}

// Product over the columns of (seed + table row t) for both lanes: even and
// odd columns in two packed chains (four independent chains in all).
// With REFILL, software-pipelined table loads: dq holds row t on entry; each
// entry's register is refilled with row `next`'s entry right after its column
// sum is formed, so the next code's loads are in flight a whole product
// ahead.  The rows then stay live across codes, which only the narrower
// kernels' register budgets allow (REFILL_MAX_NC; from 17 columns on the
// rows come from the block's shared-memory table instead).
constexpr int REFILL_MAX_NC = 16;
template <int NC, bool REFILL>
__device__ __forceinline__ void row_product_packed(const float2 (&sr)[NC], const float2 (&si)[NC], float4 (&dq)[NC],
                                                   const float4 *__restrict__ next, const uint8_t *__restrict__ cm,
                                                   bool ones, float2 &pr, float2 &pi) {
    constexpr bool two = NC >= 4;
    const float2 c0r = __fadd2_rn(sr[0], make_float2(dq[0].x, dq[0].y));
    const float2 c0i = __fadd2_rn(si[0], make_float2(dq[0].z, dq[0].w));
    if constexpr (REFILL) dq[0] = next[0];
    float2 xr = c0r, xi = c0i, yr, yi;
    if constexpr (two) {
        yr = __fadd2_rn(sr[1], make_float2(dq[1].x, dq[1].y));
        yi = __fadd2_rn(si[1], make_float2(dq[1].z, dq[1].w));
        if constexpr (REFILL) dq[1] = next[1];
    }
    if (ones) {
#pragma unroll
        for (int j = two ? 2 : 1; j < NC; ++j) {
            const float2 cr = __fadd2_rn(sr[j], make_float2(dq[j].x, dq[j].y));
            const float2 ci = __fadd2_rn(si[j], make_float2(dq[j].z, dq[j].w));
            if constexpr (REFILL) dq[j] = next[j];
            if (two && (j & 1))
                cmul2(yr, yi, cr, ci);
            else
                cmul2(xr, xi, cr, ci);
        }
    } else {
        for (int r = 1; r < cm[0]; ++r) cmul2(xr, xi, c0r, c0i);
        if constexpr (two) {
            const float2 c1r = yr, c1i = yi;
            for (int r = 1; r < cm[1]; ++r) cmul2(yr, yi, c1r, c1i);
        }
#pragma unroll
        for (int j = two ? 2 : 1; j < NC; ++j) {
            const float2 cr = __fadd2_rn(sr[j], make_float2(dq[j].x, dq[j].y));
            const float2 ci = __fadd2_rn(si[j], make_float2(dq[j].z, dq[j].w));
            if constexpr (REFILL) dq[j] = next[j];
            for (int r = 0; r < cm[j]; ++r) {
                if (two && (j & 1))
                    cmul2(yr, yi, cr, ci);
                else
                    cmul2(xr, xi, cr, ci);
            }
        }
    }
    if constexpr (two) cmul2(xr, xi, yr, yi);
    pr = xr;
    pi = xi;
}

// The same product reading the table row from shared memory column by
// column: a compiler barrier every G columns keeps at most G entries in
// flight, so the row never occupies 4 x NC registers (the three-block
// register budget of the shared-table kernels).
template <int NC, int G>
__device__ __forceinline__ void row_product_packed_smem(const float2 (&sr)[NC], const float2 (&si)[NC],
                                                        const float4 *row, const uint8_t *__restrict__ cm, bool ones,
                                                        float2 &pr, float2 &pi) {
    float2 xr, xi, yr, yi;
#pragma unroll
    for (int j = 0; j < NC; ++j) {
        if (j % G == 0) asm volatile("" ::: "memory");
        const float4 dj = row[j];
        const float2 cr = __fadd2_rn(sr[j], make_float2(dj.x, dj.y));
        const float2 ci = __fadd2_rn(si[j], make_float2(dj.z, dj.w));
        if (j == 0) {
            xr = cr;
            xi = ci;
            if (!ones)
                for (int r = 1; r < cm[0]; ++r) cmul2(xr, xi, cr, ci);
        } else if (j == 1) {
            yr = cr;
            yi = ci;
            if (!ones)
                for (int r = 1; r < cm[1]; ++r) cmul2(yr, yi, cr, ci);
        } else {
            const int reps = ones ? 1 : cm[j];
            for (int r = 0; r < reps; ++r) {
                if (j & 1)
                    cmul2(yr, yi, cr, ci);
                else
                    cmul2(xr, xi, cr, ci);
            }
        }
    }
    cmul2(xr, xi, yr, yi);
    pr = xr;
    pi = xi;
}

// Two codes (rows a and b of the shared-memory table) at once, columns
// interleaved: eight independent packed chains.  Each product is the same
// operation sequence as row_product_packed_smem's, so the accumulation of
// code a then code b is bit-identical to two single calls.
template <int NC, int G>
__device__ __forceinline__ void row_product_packed_smem_pair(const float2 (&sr)[NC], const float2 (&si)[NC],
                                                             const float4 *a, const float4 *b,
                                                             const uint8_t *__restrict__ cm, bool ones, float2 &pra,
                                                             float2 &pia, float2 &prb, float2 &pib) {
    float2 xra, xia, yra, yia, xrb, xib, yrb, yib;
#pragma unroll
    for (int j = 0; j < NC; ++j) {
        if (j % G == 0) asm volatile("" ::: "memory");
        const float4 da = a[j], db = b[j];
        const float2 cra = __fadd2_rn(sr[j], make_float2(da.x, da.y));
        const float2 cia = __fadd2_rn(si[j], make_float2(da.z, da.w));
        const float2 crb = __fadd2_rn(sr[j], make_float2(db.x, db.y));
        const float2 cib = __fadd2_rn(si[j], make_float2(db.z, db.w));
        const int reps = ones ? 1 : cm[j];
        if (j == 0) {
            xra = cra, xia = cia, xrb = crb, xib = cib;
            for (int r = 1; r < reps; ++r) {
                cmul2(xra, xia, cra, cia);
                cmul2(xrb, xib, crb, cib);
            }
        } else if (j == 1) {
            yra = cra, yia = cia, yrb = crb, yib = cib;
            for (int r = 1; r < reps; ++r) {
                cmul2(yra, yia, cra, cia);
                cmul2(yrb, yib, crb, cib);
            }
        } else {
            for (int r = 0; r < reps; ++r) {
                if (j & 1) {
                    cmul2(yra, yia, cra, cia);
                    cmul2(yrb, yib, crb, cib);
                } else {
                    cmul2(xra, xia, cra, cia);
                    cmul2(xrb, xib, crb, cib);
                }
            }
        }
    }
    cmul2(xra, xia, yra, yia);
    cmul2(xrb, xib, yrb, yib);
    pra = xra, pia = xia, prb = xrb, pib = xib;
}

// Blocks per SM the register allocation must allow: the column sums of the
// wider kernels need up to 255 registers per thread, and a spill inside the
// step loop costs more than the occupancy it buys.
template <int NC>
constexpr int walk_min_blocks_cols() {
    return NC <= 8 ? 4 : (NC <= 16 ? 3 : 2);
}

// The two-seed complex64 walk of 17..24 columns reads its prefix table from
// shared memory, staged once per group of items: at most smem_tab_codes<NC>()
// codes (the planner caps P there).  The table row then needs no registers.
// (Wider walks would need half-length tables to fit two blocks on an SM; at
// 28 columns that measured slower than the register-pipelined rows.)
constexpr int SMEM_TAB_NC_MIN = PQG_SMEM_TABLE_NC_MIN, SMEM_TAB_NC_MAX = PQG_SMEM_TABLE_NC_MAX,
              SMEM_TAB_G = 8;
template <int NC>
__host__ __device__ constexpr int smem_tab_codes() {
    return PQG_SMEM_TABLE_P;
}
template <class Ar, int NC>
__host__ __device__ constexpr bool plain_smem_table() {
    return Ar::kTwoSeeds && NC >= SMEM_TAB_NC_MIN && NC <= SMEM_TAB_NC_MAX;
}
template <class Ar, int NC>
struct PlainCfg {
    static constexpr size_t smem_bytes = plain_smem_table<Ar, NC>() ? smem_tab_codes<NC>() * NC * sizeof(float4) : 0;
};
template <class Ar, int NC>
constexpr int walk_min_blocks() {
    // three blocks where their tables fit an SM's 228 KB and 168 registers
    // hold the kernel without spills (measured: up to 18 columns)
    return (plain_smem_table<Ar, NC>() && NC <= 18) ? 3 : walk_min_blocks_cols<NC>();
}

// ONES: every column of every problem has multiplicity 1 (the usual case:
// unit input photons), so the repeated-factor code is compiled out — a
// smaller loop body for the instruction cache and the register allocator.
template <class Ar, int NC, bool ONES>
__global__ void __launch_bounds__(PQG_WALK_THREADS, walk_min_blocks<Ar, NC>()) walk_plain(WalkArgs A) {
    using cs_t = typename Ar::cs_t;
    using d_t = typename Ar::d_t;
    using t_t = typename Ar::t_t;
    const int lane = threadIdx.x & 31;
    // complex64: a block takes PQG_ITEM_GROUP consecutive items at once (one
    // per warp; the plan makes every problem a whole number of groups), so its
    // warps walk the same problem's prefix table together and share its lines
    // in L1; the exit is uniform over the block (total_items is a multiple of
    // the group)
    constexpr bool grouped = Ar::kTwoSeeds;
    static_assert(!grouped || PQG_ITEM_GROUP * 32 == PQG_WALK_THREADS, "one item per warp of a block");
    __shared__ unsigned long long s_group;
    // 17..24 columns: the group's prefix table in shared memory (dynamic,
    // smem_tab_codes<NC>() x NC entries, up to 96 KB: two blocks per SM), read
    // by all four warps; the table rows then need no registers
    constexpr bool smem_tab = plain_smem_table<Ar, NC>();
    extern __shared__ float4 s_tab[];
    int staged = -1;
    for (;;) {
        int64_t item;
        if constexpr (grouped) {
            __syncthreads();  // every warp has read the previous group
            if (threadIdx.x == 0) s_group = atomicAdd(A.counter, 1ULL);
            __syncthreads();
            item = static_cast<int64_t>(s_group) * PQG_ITEM_GROUP + (threadIdx.x >> 5);
        } else {
            item = next_item(A.counter, lane);
        }
        if (item >= A.total_items) return;
        const int ip = find_problem(A.item_begin, A.n_probs, item);
        const PqgProblem *pr = A.probs + ip;
        if constexpr (smem_tab) {
            // the block's four items belong to one problem: stage its prefix
            // table once (every warp finished its previous item at the loop top)
            if (ip != staged) {
                const float4 *src = reinterpret_cast<const float4 *>(A.delta) + pr->delta_begin;
                const int n = (pr->P < smem_tab_codes<NC>() ? pr->P : smem_tab_codes<NC>()) * NC;
                for (int e = threadIdx.x; e < n; e += PQG_WALK_THREADS) s_tab[e] = src[e];
                staged = ip;
                __syncthreads();
            }
        }
        const int64_t local = item - pr->item_begin;
        const int64_t R = pr->R;
        const int64_t Q = pr->Q;
        const int64_t r0 = (local * PQG_ITEM_LANES + lane) * R;
        ddv sr{0.0, 0.0}, si{0.0, 0.0};
        // two-seed (complex64) walks: compensated FP32 lane sums {re, im} and
        // their error words, folded by ff_fold (no FP64 instruction)
        float2 fs = make_float2(0.0f, 0.0f), fc = fs;
        if (r0 < Q) {
            OuterState st;
            outer_decode(pr, r0, st);
            cs_t seed[NC];
            seed_lane<Ar, NC>(pr, A.arena, st, seed);
            double wout = outer_weight(pr, st);
            // column multiplicities are read from the problem (L1) only when
            // some exceed 1; keeping them out of registers leaves room for the sums
            const uint8_t *cm = pr->cm;
            const bool ones = ONES || pr->cm_max == 1;
            const PqgStep *tab = reinterpret_cast<const PqgStep *>(A.arena + pr->off_tab);
            const d_t *D = reinterpret_cast<const d_t *>(A.arena + pr->off_D);
            const t_t *delta = reinterpret_cast<const t_t *>(A.delta) + pr->delta_begin;
            const int P = pr->P;
            // lanes of a problem's last item may own fewer positions and stop
            // early; inner walks never synchronise across lanes
            const int64_t my_R = (Q - r0 < R) ? (Q - r0) : R;
            int64_t seg = 0;
            if constexpr (Ar::kTwoSeeds) {
                // positions in pairs (seg, seg+1) in the two lanes of packed
                // FP32 instructions: lane .x the current seed, lane .y the
                // seed one outer step on; both walk the inner codes forward
                // (the column sums are seed + Delta(t), so the walk order is free).
                // The current seed lives in the pairs' .x lanes from here on, so
                // `seed` is not live across the inner walks (a remainder
                // position takes its seed back from the .x lanes)
                float2 pr2[NC], pi2[NC];
#pragma unroll
                for (int j = 0; j < NC; ++j) {
                    pr2[j].x = seed[j].r;
                    pi2[j].x = seed[j].i;
                }
                for (; seg + 1 < my_R; seg += 2) {
                    bool up = false;
                    int k = outer_next(pr, st, &up);
                    const d_t *db = D + (2 * k + (up ? 0 : 1)) * NC;
#pragma unroll
                    for (int j = 0; j < NC; ++j) {
                        const d_t dj = db[j];
                        pr2[j].y = __fadd_rn(pr2[j].x, dj.x);
                        pi2[j].y = __fadd_rn(pi2[j].x, dj.y);
                    }
                    const double wb = outer_weight(pr, st);
                    float2 accr = make_float2(0.0f, 0.0f), accrc = accr, acci = accr, accic = accr;
                    constexpr bool refill = !smem_tab && NC <= REFILL_MAX_NC;
                    float4 dq[NC];
                    if constexpr (refill) {
#pragma unroll
                        for (int j = 0; j < NC; ++j) dq[j] = delta[j];
                    }
                    // (the staged table holds at most smem_tab_codes<NC>() codes: the plan
                    // guarantees P fits; the bound keeps every read inside it)
                    const int Pw = smem_tab ? (P < smem_tab_codes<NC>() ? P : smem_tab_codes<NC>()) : P;
                    int t = 0;
                    if constexpr (smem_tab) {  // two codes at a time, then a last odd one
                        for (; t + 1 < Pw; t += 2) {
                            float2 xra, xia, xrb, xib;
                            row_product_packed_smem_pair<NC, SMEM_TAB_G>(pr2, pi2, s_tab + t * NC, s_tab + (t + 1) * NC,
                                                                         cm, ones, xra, xia, xrb, xib);
                            const float wa = tab[t].wf, wb2 = tab[t + 1].wf;
                            two_sum_acc2(accr, accrc, __fmul2_rn(make_float2(wa, wa), xra));
                            two_sum_acc2(acci, accic, __fmul2_rn(make_float2(wa, wa), xia));
                            two_sum_acc2(accr, accrc, __fmul2_rn(make_float2(wb2, wb2), xrb));
                            two_sum_acc2(acci, accic, __fmul2_rn(make_float2(wb2, wb2), xib));
                        }
                    }
                    for (; t < Pw; ++t) {
                        float2 xr, xi;
                        if constexpr (smem_tab) {
                            row_product_packed_smem<NC, SMEM_TAB_G>(pr2, pi2, s_tab + t * NC, cm, ones, xr, xi);
                        } else {
                            if constexpr (!refill) {
                                const float4 *row = delta + static_cast<int64_t>(t) * NC;
#pragma unroll
                                for (int j = 0; j < NC; ++j) dq[j] = row[j];
                            }
                            // the last code reloads its own row (in bounds, unused)
                            const int tn = t + 1 < P ? t + 1 : t;
                            row_product_packed<NC, refill>(pr2, pi2, dq, delta + static_cast<int64_t>(tn) * NC, cm,
                                                           ones, xr, xi);
                        }
                        const float wf = tab[t].wf;
                        const float2 w2 = make_float2(wf, wf);
                        two_sum_acc2(accr, accrc, __fmul2_rn(w2, xr));
                        two_sum_acc2(acci, accic, __fmul2_rn(w2, xi));
                    }
                    ff_fold(fs, fc, accr.x, accrc.x, acci.x, accic.x, wout);
                    ff_fold(fs, fc, accr.y, accrc.y, acci.y, accic.y, wb);
                    if (seg + 2 < my_R) {  // seed moves on to position seg + 2
                        k = outer_next(pr, st, &up);
                        const d_t *d = D + (2 * k + (up ? 0 : 1)) * NC;
#pragma unroll
                        for (int j = 0; j < NC; ++j) {  // Ar::update of the .y seed
                            pr2[j].x = __fadd_rn(pr2[j].y, d[j].x);
                            pi2[j].x = __fadd_rn(pi2[j].y, d[j].y);
                        }
                        wout = outer_weight(pr, st);
                    }
                }
#pragma unroll
                for (int j = 0; j < NC; ++j) seed[j] = cs_t{pr2[j].x, pi2[j].x};
            }
            for (; seg < my_R; ++seg) {
                typename Ar::acc_t acc = Ar::zero();
                // inner codes in walk order: t = s (forward) or P-1-s (backward);
                // FP32-pipe walks take two codes per iteration (independent
                // products, same accumulation order)
                const bool back = (seg & 1) != 0;
                int s = 0;
                if constexpr (Ar::kPairSteps) {
                    for (; s + 1 < P; s += 2) {
                        const int ta = back ? P - 1 - s : s;
                        const int tb = back ? ta - 1 : ta + 1;
                        const cs_t xa = row_product<Ar, NC>(seed, delta + static_cast<int64_t>(ta) * NC, cm, ones);
                        const cs_t xb = row_product<Ar, NC>(seed, delta + static_cast<int64_t>(tb) * NC, cm, ones);
                        Ar::accumulate(acc, xa, tab[ta]);
                        Ar::accumulate(acc, xb, tab[tb]);
                    }
                }
                for (; s < P; ++s) {
                    const int t = back ? P - 1 - s : s;
                    const cs_t x = row_product<Ar, NC>(seed, delta + static_cast<int64_t>(t) * NC, cm, ones);
                    Ar::accumulate(acc, x, tab[t]);
                }
                if constexpr (Ar::kTwoSeeds)
                    ff_fold(fs, fc, acc.r, acc.cr, acc.i, acc.ci, wout);
                else
                    Ar::fold(sr, si, acc, wout);
                if (seg + 1 < my_R) {
                    bool up = false;
                    const int k = outer_next(pr, st, &up);
                    const d_t *d = D + (2 * k + (up ? 0 : 1)) * NC;
#pragma unroll
                    for (int j = 0; j < NC; ++j) Ar::update(seed[j], d[j]);
                    wout = outer_weight(pr, st);
                }
            }
        }
        if constexpr (Ar::kTwoSeeds) {
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const float2 os = make_float2(__shfl_down_sync(PQG_FULL_MASK, fs.x, off),
                                              __shfl_down_sync(PQG_FULL_MASK, fs.y, off));
                const float2 oc = make_float2(__shfl_down_sync(PQG_FULL_MASK, fc.x, off),
                                              __shfl_down_sync(PQG_FULL_MASK, fc.y, off));
                two_sum_acc2(fs, fc, os);
                fc = __fadd2_rn(fc, oc);
            }
            if (lane == 0)
                store_partial(A.partials, pr->part_begin + local,
                              ddv{static_cast<double>(fs.x), static_cast<double>(fc.x)},
                              ddv{static_cast<double>(fs.y), static_cast<double>(fc.y)});
        } else {
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                sr = dd_add(sr, dd_shfl_down(sr, off));
                si = dd_add(si, dd_shfl_down(si, off));
            }
            if (lane == 0) store_partial(A.partials, pr->part_begin + local, sr, si);
        }
    }
}

// --------------------------------- double-float walk, seeds in shared memory
// The double-float walk is bound by FP32 instruction issue at two blocks per
// SM: its seeds take four registers per column (112 at 28 columns).  This
// variant keeps each lane's seeds in a column-major slice of dynamic shared
// memory (one float4 {re_hi, re_lo, im_hi, im_lo} per column, stride = the
// block's threads, so a warp's loads are conflict-free), read once per column
// and code next to the broadcast prefix-table row, so that more blocks fit an
// SM: up to 24 columns, four (125 registers, at most 48 KB each), where it
// measured 489 -> 462 us at n = 24 (FMA pipe 57 -> 65 %).  The tables use it
// for 21..24 columns: from 25 columns only three blocks fit the shared
// memory and it measured no faster, and on the 4096-pattern batch of 20
// columns the register-seeded walk tuned (12.00 ms) beat it tuned (12.63 ms).  Seeding, the one-digit
// outer updates, the products and the accumulation are the operations of
// walk_plain<ArDF> in the same order, so the results are bit-identical.
constexpr int DFS_G = 8;
template <int NC>
struct PlainDfsCfg {
    static constexpr size_t smem_bytes = size_t(NC) * PQG_WALK_THREADS * sizeof(float4);
};

template <int NC, bool ONES>
__global__ void __launch_bounds__(PQG_WALK_THREADS, 4) walk_plain_dfs(WalkArgs A) {
    using Ar = ArDF;
    using cs_t = Ar::cs_t;
    extern __shared__ float4 dfs_seed_smem[];
    float4 *seed = dfs_seed_smem + threadIdx.x;  // column j at seed[j * PQG_WALK_THREADS]
    const int lane = threadIdx.x & 31;
    auto seed_get = [&](int j) -> cs_t {
        const float4 v = seed[j * PQG_WALK_THREADS];
        return cs_t{dfl{v.x, v.y}, dfl{v.z, v.w}};
    };
    for (;;) {
        const int64_t item = next_item(A.counter, lane);
        if (item >= A.total_items) return;
        const int ip = find_problem(A.item_begin, A.n_probs, item);
        const PqgProblem *pr = A.probs + ip;
        const int64_t local = item - pr->item_begin;
        const int64_t R = pr->R;
        const int64_t Q = pr->Q;
        const int64_t r0 = (local * PQG_ITEM_LANES + lane) * R;
        ddv sr{0.0, 0.0}, si{0.0, 0.0};
        if (r0 < Q) {
            OuterState st;
            outer_decode(pr, r0, st);
            {
                // seed_lane<ArDF> column by column (the same additions per column, in order)
                const float4 *base = reinterpret_cast<const float4 *>(A.arena + pr->off_base_df);
                const float4 *orow = reinterpret_cast<const float4 *>(A.arena + pr->off_outer_df);
                for (int j = 0; j < NC; ++j) {
                    const float4 v = __ldg(base + j);
                    dfl r{v.x, v.y}, i{v.z, v.w};
                    for (int o = 0; o < pr->n_outer; ++o) {
                        const int g = st.g[o];
                        if (!g) continue;
                        const float f = -2.0f * static_cast<float>(g);
                        const float4 w = __ldg(orow + static_cast<int64_t>(o) * NC + j);
                        r = df_add(r, df_scale(dfl{w.x, w.y}, f));
                        i = df_add(i, df_scale(dfl{w.z, w.w}, f));
                    }
                    const cs_t c = Ar::from_seed_df(r, i);
                    seed[j * PQG_WALK_THREADS] = make_float4(c.r.hi, c.r.lo, c.i.hi, c.i.lo);
                }
            }
            double wout = outer_weight(pr, st);
            const uint8_t *cm = pr->cm;
            const bool ones = ONES || pr->cm_max == 1;
            const PqgStep *tab = reinterpret_cast<const PqgStep *>(A.arena + pr->off_tab);
            const float4 *D = reinterpret_cast<const float4 *>(A.arena + pr->off_D);
            const float4 *delta = reinterpret_cast<const float4 *>(A.delta) + pr->delta_begin;
            const int P = pr->P;
            const int64_t my_R = (Q - r0 < R) ? (Q - r0) : R;
            for (int64_t seg = 0; seg < my_R; ++seg) {
                Ar::acc_t acc = Ar::zero();
                const bool back = (seg & 1) != 0;
                for (int s = 0; s < P; ++s) {
                    const int t = back ? P - 1 - s : s;
                    const float4 *d = delta + static_cast<int64_t>(t) * NC;
                    // row_product<ArDF>: even and odd columns in two chains
                    constexpr bool two = NC >= 4;
                    const cs_t c0 = Ar::sum(seed_get(0), d[0]);
                    cs_t x = c0, y;
                    if constexpr (two) y = Ar::sum(seed_get(1), d[1]);
                    if (ones) {
#pragma unroll
                        for (int j = two ? 2 : 1; j < NC; ++j) {
                            // (a compiler barrier every DFS_G columns bounds the loads in flight)
                            if (j % DFS_G == 0) asm volatile("" ::: "memory");
                            const cs_t c = Ar::sum(seed_get(j), d[j]);
                            if (two && (j & 1))
                                Ar::mul(y, c);
                            else
                                Ar::mul(x, c);
                        }
                    } else {
                        for (int r = 1; r < cm[0]; ++r) Ar::mul(x, c0);
                        if constexpr (two) {
                            const cs_t c1 = y;
                            for (int r = 1; r < cm[1]; ++r) Ar::mul(y, c1);
                        }
#pragma unroll
                        for (int j = two ? 2 : 1; j < NC; ++j) {
                            const cs_t c = Ar::sum(seed_get(j), d[j]);
                            for (int r = 0; r < cm[j]; ++r) {
                                if (two && (j & 1))
                                    Ar::mul(y, c);
                                else
                                    Ar::mul(x, c);
                            }
                        }
                    }
                    if constexpr (two) Ar::mul(x, y);
                    Ar::accumulate(acc, x, tab[t]);
                }
                Ar::fold(sr, si, acc, wout);
                if (seg + 1 < my_R) {
                    bool up = false;
                    const int k = outer_next(pr, st, &up);
                    const float4 *dk = D + (2 * k + (up ? 0 : 1)) * NC;
#pragma unroll
                    for (int j = 0; j < NC; ++j) {
                        cs_t c = seed_get(j);
                        Ar::update(c, dk[j]);
                        seed[j * PQG_WALK_THREADS] = make_float4(c.r.hi, c.r.lo, c.i.hi, c.i.lo);
                    }
                    wout = outer_weight(pr, st);
                }
            }
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
