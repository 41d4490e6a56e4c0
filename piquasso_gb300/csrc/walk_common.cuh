// Device helpers shared by the walk and reduction kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "pqg_plan.h"

#define PQG_FULL_MASK 0xffffffffu
#define PQG_WALK_THREADS 128
#define PQG_MAX_OUT (PQG_MAX_COLS + 1)

namespace pqg {

// ------------------------------------------------------------ double-double
// Error-free transforms: Knuth's TwoSum, Dekker's Fast2Sum and an FMA-based
// TwoProduct.  The _rn intrinsics keep the compiler from contracting or
// reassociating them.
struct ddv {
    double hi, lo;
};

__device__ __forceinline__ ddv two_sum(double a, double b) {
    double s = __dadd_rn(a, b);
    double bb = __dsub_rn(s, a);
    double e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb));
    return {s, e};
}
__device__ __forceinline__ ddv fast_two_sum(double a, double b) {
    double s = __dadd_rn(a, b);
    double e = __dsub_rn(b, __dsub_rn(s, a));
    return {s, e};
}
__device__ __forceinline__ ddv dd_add(ddv a, ddv b) {
    ddv s = two_sum(a.hi, b.hi);
    ddv t = two_sum(a.lo, b.lo);
    s.lo = __dadd_rn(s.lo, t.hi);
    s = fast_two_sum(s.hi, s.lo);
    s.lo = __dadd_rn(s.lo, t.lo);
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ ddv dd_add_d(ddv a, double b) {
    ddv s = two_sum(a.hi, b);
    s.lo = __dadd_rn(s.lo, a.lo);
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ ddv dd_mul_d(ddv a, double b) {
    double p = __dmul_rn(a.hi, b);
    double e = __fma_rn(a.hi, b, -p);
    e = __fma_rn(a.lo, b, e);
    return fast_two_sum(p, e);
}
__device__ __forceinline__ ddv dd_shfl_down(ddv v, int off) {
    return {__shfl_down_sync(PQG_FULL_MASK, v.hi, off), __shfl_down_sync(PQG_FULL_MASK, v.lo, off)};
}

// FP32 TwoSum for compensated single-precision partial sums.
__device__ __forceinline__ void f_two_sum_acc(float &s, float &c, float y) {
    float t = __fadd_rn(s, y);
    float bb = __fsub_rn(t, s);
    float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bb)), __fsub_rn(y, bb));
    s = t;
    c = __fadd_rn(c, e);
}

// ------------------------------------------------------------------ complex
__device__ __forceinline__ void cmul(double &xr, double &xi, double br, double bi) {
    double r = __fma_rn(xr, br, -__dmul_rn(xi, bi));
    double i = __fma_rn(xr, bi, __dmul_rn(xi, br));
    xr = r;
    xi = i;
}
__device__ __forceinline__ void cmulf(float &xr, float &xi, float br, float bi) {
    float r = __fmaf_rn(xr, br, -__fmul_rn(xi, bi));
    float i = __fmaf_rn(xr, bi, __fmul_rn(xi, br));
    xr = r;
    xi = i;
}

// ------------------------------------------------------------------- misc
__device__ __forceinline__ int64_t binom64(int m, int g) {
    if (g < 0 || g > m) return 0;
    if (g > m - g) g = m - g;
    int64_t r = 1;
    for (int i = 1; i <= g; ++i) r = r * (m - g + i) / i;
    return r;
}

// problem owning a global work item: largest p with item_begin[p] <= item
__device__ __forceinline__ int find_problem(const int64_t *__restrict__ item_begin, int n_probs, int64_t item) {
    int lo = 0, hi = n_probs - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (__ldg(item_begin + mid) <= item)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

struct WalkArgs {
    const PqgProblem *probs;
    const int64_t *item_begin;
    const unsigned char *arena;
    const void *delta;            // prefix tables, kernel precision, indexed by delta_begin
    unsigned long long *counter;  // work-queue head, zeroed before the launch
    double *partials;             // 4 doubles per slot: re_hi, re_lo, im_hi, im_lo
    int64_t total_items;
    int32_t n_probs;
    int32_t pad;
};

// Next work item for the calling warp (one atomic per warp).
__device__ __forceinline__ int64_t next_item(unsigned long long *counter, int lane) {
    unsigned long long it = 0;
    if (lane == 0) it = atomicAdd(counter, 1ULL);
    return static_cast<int64_t>(__shfl_sync(PQG_FULL_MASK, it, 0));
}

__device__ __forceinline__ void store_partial(double *partials, int64_t slot, ddv re, ddv im) {
    double2 *p = reinterpret_cast<double2 *>(partials) + 2 * slot;
    p[0] = make_double2(re.hi, re.lo);
    p[1] = make_double2(im.hi, im.lo);
}

__device__ __forceinline__ void load_partial(const double *partials, int64_t slot, ddv &re, ddv &im) {
    const double2 *p = reinterpret_cast<const double2 *>(partials) + 2 * slot;
    const double2 a = p[0], b = p[1];
    re = ddv{a.x, a.y};
    im = ddv{b.x, b.y};
}

// Reflected mixed-radix Gray code of position r over `n` digits with
// multiplicities m (radix m + 1, digit 0 fastest): counter digits, then the
// code from the top digit down (src/n_aryGrayCodeCounter.hpp:170-194 of the
// reference, with a 64-bit position).  Writes the code digits to g.
__device__ __forceinline__ void gray_decode(const uint8_t *__restrict__ m, int n, int64_t r, uint8_t *g) {
    uint8_t c[PQG_MAX_OUTER];
    for (int o = 0; o < n; ++o) {
        const int L = m[o] + 1;
        c[o] = static_cast<uint8_t>(r % L);
        r /= L;
    }
    int parity = 0;
    for (int o = n - 1; o >= 0; --o) {
        const int L = m[o] + 1;
        const int code = parity ? L - 1 - c[o] : c[o];
        g[o] = static_cast<uint8_t>(code);
        parity ^= (code & 1);
    }
}

}  // namespace pqg
