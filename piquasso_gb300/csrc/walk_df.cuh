// Complex128-accurate walk on the FP32 pipes ("double-float").
//
// GB300 executes FP64 at about 1/61 of its FP32 rate, so the plain
// complex128 walk is FP64-pipe bound.  This kernel keeps the FP64 steps the
// method's stability needs — the per-segment seeding of the column sums and
// the double-double accumulation across steps, lanes and blocks — and does the
// per-step column updates and products in double-float arithmetic: every real
// number is an unevaluated sum hi + lo of two floats, with the error-free
// transforms TwoSum (Knuth) and FMA-based TwoProduct, giving about 2^-48
// relative precision per operation (T. J. Dekker, "A floating-point technique
// for extending the available precision", Numer. Math. 18, 1971).
//
// FP32 has an 8-bit exponent, so the planner scales every column by a power of
// two such that no column sum can exceed 1 in magnitude (|c_j| <= sum_i m_i
// |a_ij| <= 1); the scale is undone exactly in the final 2^-e factor.  The
// planner only selects this arithmetic when the typical term stays far above
// the FP32 underflow threshold (see plan.cpp).  The kernel itself is the
// generic walk of walk_plain.cuh with the ArDF policy.
#pragma once
#include "walk_common.cuh"

namespace pqg {

struct dfl {
    float hi, lo;
};

// a + b, both double-float; TwoSum on the high words, then renormalise
__device__ __forceinline__ dfl df_add(dfl a, dfl b) {
    const float s = __fadd_rn(a.hi, b.hi);
    const float v = __fsub_rn(s, a.hi);
    const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, v)), __fsub_rn(b.hi, v));
    const float l = __fadd_rn(__fadd_rn(a.lo, b.lo), e);
    const float h = __fadd_rn(s, l);
    return {h, __fsub_rn(l, __fsub_rn(h, s))};
}

// Real part of a product, ah*bh - ch*dh plus the low-order cross terms, for
// double-float operands (ah + al) ... (dh + dl): FMA TwoProducts of the high
// words, a TwoSum of their difference, and the cross terms through FMAs.  The
// pair is not renormalised -- it only feeds further products: (s, low) still
// sums to the product to about 2^-48 of its terms (TwoSum kept the rounding
// error of the high words), and the next product takes the low word through
// its FMA cross terms, so only the dropped low x low term grows -- by the
// cancellation factor |p1| / |p1 - p2| that the sum already carries.  That
// keeps two dependent operations off the product chain.  The pair is
// renormalised before it is accumulated (df_scale, df_add).
__device__ __forceinline__ dfl df_mul_sub_lazy(dfl a, dfl b, dfl c, dfl d) {
    const float p1 = __fmul_rn(a.hi, b.hi);
    const float e1 = __fmaf_rn(a.hi, b.hi, -p1);
    const float p2 = __fmul_rn(c.hi, d.hi);
    const float e2 = __fmaf_rn(c.hi, d.hi, -p2);
    const float s = __fsub_rn(p1, p2);
    const float v = __fsub_rn(s, p1);
    const float t = __fadd_rn(__fsub_rn(p1, __fsub_rn(s, v)), __fsub_rn(-p2, v));
    float low = __fadd_rn(__fsub_rn(e1, e2), t);
    low = __fmaf_rn(a.hi, b.lo, low);
    low = __fmaf_rn(a.lo, b.hi, low);
    low = __fmaf_rn(-c.hi, d.lo, low);
    low = __fmaf_rn(-c.lo, d.hi, low);
    return {s, low};
}

__device__ __forceinline__ dfl df_mul_add_lazy(dfl a, dfl b, dfl c, dfl d) {
    const float p1 = __fmul_rn(a.hi, b.hi);
    const float e1 = __fmaf_rn(a.hi, b.hi, -p1);
    const float p2 = __fmul_rn(c.hi, d.hi);
    const float e2 = __fmaf_rn(c.hi, d.hi, -p2);
    const float s = __fadd_rn(p1, p2);
    const float v = __fsub_rn(s, p1);
    const float t = __fadd_rn(__fsub_rn(p1, __fsub_rn(s, v)), __fsub_rn(p2, v));
    float low = __fadd_rn(__fadd_rn(e1, e2), t);
    low = __fmaf_rn(a.hi, b.lo, low);
    low = __fmaf_rn(a.lo, b.hi, low);
    low = __fmaf_rn(c.hi, d.lo, low);
    low = __fmaf_rn(c.lo, d.hi, low);
    return {s, low};
}

__device__ __forceinline__ void df_cmul_lazy(dfl &xr, dfl &xi, dfl yr, dfl yi) {
    const dfl r = df_mul_sub_lazy(xr, yr, xi, yi);
    const dfl i = df_mul_add_lazy(xr, yi, xi, yr);
    xr = r;
    xi = i;
}

// w * x for a float w that is an exact small integer
__device__ __forceinline__ dfl df_scale(dfl x, float w) {
    const float p = __fmul_rn(w, x.hi);
    const float e = __fmaf_rn(w, x.hi, -p);
    const float l = __fmaf_rn(w, x.lo, e);
    const float h = __fadd_rn(p, l);
    return {h, __fsub_rn(l, __fsub_rn(h, p))};
}

// ------------------------------------------------ column sums on a grid
// Every value that enters a column sum of the double-float walk is below 2 in
// magnitude: the planner's power-of-two column scale makes every column sum
// (and so every seed) smaller than 1, a prefix-table entry or a one-digit
// update row is a difference of two of them.  The walk keeps the high word of
// each such value on the grid of multiples of 2^-23 (the spacing of floats in
// [1, 2)).  Two high words on that grid add exactly in FP32 -- their sum is a
// multiple of 2^-23 below 2 in magnitude, which a float represents -- so a
// column sum seed + Delta(t) is hi + hi and lo + lo, two adds instead of a
// TwoSum's eight.  The low word (at most 2^-24 in magnitude, rounded once per
// add) carries the rest to about 2^-48 absolute: the same order as the TwoSum
// sum of two double-floats of magnitude up to 1, so the grid costs the walk
// at most a few times the error of a column sum near zero.
constexpr float DF_GRID = 1.1920928955078125e-7f;  // 2^-23
constexpr float DF_GRID_INV = 8388608.0f;          // 2^23

// x on the grid: the nearest multiple of 2^-23 (x * 2^23 and back are exact)
__device__ __forceinline__ float df_grid_round(float x) {
    return __fmul_rn(rintf(__fmul_rn(x, DF_GRID_INV)), DF_GRID);
}

// A double-float of magnitude below 1 with its high word moved onto the grid:
// hi - t is exact (both are multiples of the smaller one's spacing and the
// difference is the smaller), and so is adding lo for a value on the 2^-47
// grid.  That low word can reach 1.5 * 2^-24, so its own grid part moves into
// the high word as in df_grid_add: the low word ends at most 2^-24, which
// keeps the walk's low-word sums below 2^-23 and exact.
__device__ __forceinline__ dfl df_to_grid(dfl a) {
    const float t = df_grid_round(a.hi);
    const float l = __fadd_rn(__fsub_rn(a.hi, t), a.lo);
    const float u = __fsub_rn(__fadd_rn(l, 1.5f), 1.5f);
    return {__fadd_rn(t, u), __fsub_rn(l, u)};
}

// a + b for a, b with high words on the grid and |a + b| < 1: the high words
// add exactly; the low words' grid part moves into the high word ((x + 1.5) -
// 1.5 rounds |x| < 0.5 to the grid), so the result is on the grid again with
// a low word of at most 2^-24 (the outer one-digit update of a seed).
__device__ __forceinline__ dfl df_grid_add(dfl a, dfl b) {
    const float h = __fadd_rn(a.hi, b.hi);
    const float l = __fadd_rn(a.lo, b.lo);
    const float t = __fsub_rn(__fadd_rn(l, 1.5f), 1.5f);
    return {__fadd_rn(h, t), __fsub_rn(l, t)};
}

// a + b for a, b with high words on the grid (a column sum): hi + hi and
// lo + lo are exact, and a Fast2Sum renormalises the pair -- valid since
// |hi| >= 2^-23 >= |lo| or hi = 0 -- so that the products see a low word
// below half an ulp of the high word (with a low word of up to 2^-23 beside a
// column sum of 0.1, their FMA cross terms would round at 2^-44 of the
// product).  Five operations instead of a TwoSum's eight.
__device__ __forceinline__ dfl df_grid_sum(dfl a, dfl b) {
    const float h = __fadd_rn(a.hi, b.hi);
    const float l = __fadd_rn(a.lo, b.lo);
    const float s = __fadd_rn(h, l);
    return {s, __fsub_rn(l, __fsub_rn(s, h))};
}

// x (|x| < 2) with its high word on the grid
__device__ __forceinline__ void df_split_grid(double x, float &hi, float &lo) {
    hi = static_cast<float>(rint(x * 8388608.0) * 1.1920928955078125e-7);
    lo = __double2float_rn(x - static_cast<double>(hi));
}

__device__ __forceinline__ dfl df_split(double x) {
    const float h = __double2float_rn(x);
    return {h, __double2float_rn(x - static_cast<double>(h))};
}

__device__ __forceinline__ ddv dd_add_df(ddv a, dfl x) {
    return dd_add_d(dd_add_d(a, static_cast<double>(x.hi)), static_cast<double>(x.lo));
}

}  // namespace pqg
