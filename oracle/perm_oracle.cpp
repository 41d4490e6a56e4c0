// Oracle for the permanent hot path — TEST INFRASTRUCTURE ONLY.
//
// A CPU restatement, in double-double arithmetic, of piquasso's permanent with
// repeated rows and columns and of its Laplace-expansion variant.  Only tests/,
// __graft_entry__.smoke() and bench.py's cpu_baseline leg use it, and only as
// the checker: the product path (piquasso_gb300) never links or calls it.
//
// Method followed (reference paths, piquasso 8.0.1):
//   * src/permanent.cpp:49-264          permanent_cpp<T>
//   * src/permanent_laplace.cpp:43-240  permanent_laplace_cpp<T>
//   * src/n_aryGrayCodeCounter.hpp:170-254  reflected mixed-radix Gray code
//   * src/utils.hpp:43-61               binomialCoeff
// Differences, all deliberate: every scalar is a double-double (Knuth TwoSum,
// FMA-based TwoProduct), the Gray-code offset is 64-bit throughout (the
// reference truncates it to int at n_aryGrayCodeCounter.hpp:179), and the
// number of contiguous segments is a parameter instead of 4*hardware threads.
// Parity of this restatement is pinned against the reference module built by
// oracle/build_ref.sh and against the known-answer tests in tests/golden/.
//
// Build: see oracle/build.py (-O2 -ffp-contract=off, so that the error-free
// transforms below are not contracted and results agree across x86 and Arm).

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#if defined(_OPENMP)
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------- double-double
struct dd {
    double hi, lo;
};

// Knuth's TwoSum: s + e == a + b exactly.
inline dd two_sum(double a, double b) {
    double s = a + b;
    double bb = s - a;
    double e = (a - (s - bb)) + (b - bb);
    return {s, e};
}
// Dekker's Fast2Sum, valid for |a| >= |b|.
inline dd fast_two_sum(double a, double b) {
    double s = a + b;
    double e = b - (s - a);
    return {s, e};
}
// TwoProduct with a fused multiply-add: p + e == a * b exactly.
inline dd two_prod(double a, double b) {
    double p = a * b;
    double e = std::fma(a, b, -p);
    return {p, e};
}
inline dd dd_add(dd a, dd b) {
    dd s = two_sum(a.hi, b.hi);
    dd t = two_sum(a.lo, b.lo);
    s.lo += t.hi;
    s = fast_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return fast_two_sum(s.hi, s.lo);
}
inline dd dd_sub(dd a, dd b) { return dd_add(a, {-b.hi, -b.lo}); }
inline dd dd_mul(dd a, dd b) {
    dd p = two_prod(a.hi, b.hi);
    p.lo += a.hi * b.lo + a.lo * b.hi;
    return fast_two_sum(p.hi, p.lo);
}
inline dd dd_mul_d(dd a, double b) {
    dd p = two_prod(a.hi, b);
    p.lo += a.lo * b;
    return fast_two_sum(p.hi, p.lo);
}

struct ddc {
    dd re, im;
};
inline ddc ddc_add(const ddc &a, const ddc &b) { return {dd_add(a.re, b.re), dd_add(a.im, b.im)}; }
inline ddc ddc_mul(const ddc &a, const ddc &b) {
    return {dd_sub(dd_mul(a.re, b.re), dd_mul(a.im, b.im)),
            dd_add(dd_mul(a.re, b.im), dd_mul(a.im, b.re))};
}
inline ddc ddc_scale(const ddc &a, double s) { return {dd_mul_d(a.re, s), dd_mul_d(a.im, s)}; }
inline ddc ddc_from(double re, double im) { return {{re, 0.0}, {im, 0.0}}; }

// ------------------------------------------------------- binomial (utils.hpp:43-61)
int64_t binom(int64_t n, int64_t k) {
    if (k < 0 || n < 0 || k > n) return 0;
    if (k == 0 || k == n) return 1;
    if (k > n - k) k = n - k;
    int64_t r = 1;
    for (int64_t i = 1; i <= k; ++i) r = r * (n - k + i) / i;  // exact at every step
    return r;
}

// ------------------------------- reflected mixed-radix Gray code (hpp:170-254)
struct GrayCounter {
    std::vector<int> limits, chain, code;
    int64_t offset = 0, offset_max = 0;

    GrayCounter(const std::vector<int> &lim, int64_t start, int64_t last)
        : limits(lim), chain(lim.size()), code(lim.size()), offset(start), offset_max(last) {
        // counter chain = mixed-radix digits of the offset (64-bit, hpp:179 is int)
        int64_t t = start;
        for (size_t i = 0; i < limits.size(); ++i) {
            chain[i] = static_cast<int>(t % limits[i]);
            t /= limits[i];
        }
        int parity = 0;
        for (int i = static_cast<int>(limits.size()) - 1; i >= 0; --i) {
            int c = parity ? limits[i] - 1 - chain[i] : chain[i];
            code[i] = c;
            parity ^= (c & 1);
        }
    }

    // returns false once the segment is exhausted (hpp:209-254)
    bool next(int &changed, int &prev, int &val) {
        if (offset >= offset_max) return false;
        size_t k = 0;
        while (true) {
            if (chain[k] < limits[k] - 1) {
                chain[k]++;
                break;
            }
            chain[k] = 0;
            ++k;
        }
        int parity = 0;
        for (int i = static_cast<int>(limits.size()) - 1; i >= 0; --i) {
            int c = parity ? limits[i] - 1 - chain[i] : chain[i];
            parity ^= (c & 1);
            if (c != code[i]) {
                prev = code[i];
                val = c;
                code[i] = c;
                changed = i;
                break;
            }
        }
        ++offset;
        return true;
    }
};

// Input after the row reduction of permanent.cpp:54-95: row 0 is a copy of the
// first row with the smallest nonzero multiplicity, taken with multiplicity 1,
// and that row's own multiplicity is decremented.
struct Reduced {
    int nr = 0, nc = 0;            // rows/cols of the reduced matrix
    std::vector<double> a;         // interleaved re/im, row-major nr x nc
    std::vector<int> rows, cols;
    bool reduced = false;
};

Reduced reduce_rows(const double *a, int nr, int nc, const int *rows, const int *cols) {
    Reduced r;
    r.nc = nc;
    r.cols.assign(cols, cols + nc);
    int min_idx = 0, minelem = 0;
    for (int i = 0; i < nr; ++i) {
        if (minelem == 0 || (rows[i] < minelem && rows[i] != 0)) {
            minelem = rows[i];
            min_idx = i;
        }
    }
    if (nr > 0 && minelem != 0) {
        r.reduced = true;
        r.nr = nr + 1;
        r.rows.resize(nr + 1);
        r.rows[0] = 1;
        for (int i = 0; i < nr; ++i) r.rows[i + 1] = rows[i];
        r.rows[1 + min_idx] -= 1;
        r.a.resize(static_cast<size_t>(2) * r.nr * nc);
        std::memcpy(r.a.data(), a + static_cast<size_t>(2) * min_idx * nc, sizeof(double) * 2 * nc);
        std::memcpy(r.a.data() + 2 * nc, a, sizeof(double) * 2 * nr * nc);
    } else {
        r.nr = nr;
        r.rows.assign(rows, rows + nr);
        r.a.assign(a, a + static_cast<size_t>(2) * nr * nc);
    }
    return r;
}

// One contiguous Gray-code segment [first, last] of the BB/FG sum
// (permanent.cpp:157-250 and permanent_laplace.cpp:133-223 in one routine).
// `laplace` selects which products are formed: one product with every column
// at its multiplicity, or one per column l with column l's exponent lowered by one.
void walk_segment(const Reduced &R, const std::vector<int> &limits, int64_t first, int64_t last,
                  bool laplace, std::vector<ddc> &acc) {
    const int nc = R.nc;
    const int ndig = static_cast<int>(limits.size());
    GrayCounter g(limits, first, last);

    std::vector<ddc> colsum(nc);
    for (int j = 0; j < nc; ++j) colsum[j] = ddc_from(R.a[2 * j], R.a[2 * j + 1]);
    int64_t bc = 1;
    int minus_all = 0;
    for (int i = 0; i < ndig; ++i) {
        int ms = g.code[i];
        int mult = R.rows[i + 1];
        double f = static_cast<double>(mult - 2 * ms);
        const double *row = &R.a[static_cast<size_t>(2) * (i + 1) * nc];
        for (int j = 0; j < nc; ++j)
            colsum[j] = ddc_add(colsum[j], ddc_scale(ddc_from(row[2 * j], row[2 * j + 1]), f));
        minus_all += ms;
        bc *= binom(mult, ms);
    }
    int parity = (minus_all % 2 == 0) ? 1 : -1;

    const int nout = laplace ? nc : 1;
    auto add_term = [&]() {
        for (int l = 0; l < nout; ++l) {
            ddc p = ddc_from(static_cast<double>(parity), 0.0);
            for (int k = 0; k < nc; ++k) {
                int e = R.cols[k];
                if (laplace && k == l) e = e - 1;  // a negative count runs zero times
                for (int q = 0; q < e; ++q) p = ddc_mul(p, colsum[k]);
            }
            acc[l] = ddc_add(acc[l], ddc_scale(p, static_cast<double>(bc)));
        }
    };
    add_term();

    int changed = 0, prev = 0, val = 0;
    while (g.next(changed, prev, val)) {
        parity = -parity;
        const double *row = &R.a[static_cast<size_t>(2) * (changed + 1) * nc];
        double f = 2.0 * static_cast<double>(prev - val);
        for (int j = 0; j < nc; ++j)
            colsum[j] = ddc_add(colsum[j], ddc_scale(ddc_from(row[2 * j], row[2 * j + 1]), f));
        int mult = R.rows[changed + 1];
        bc = val < prev ? bc * prev / (mult - val) : bc * (mult - prev) / val;
        add_term();
    }
}

// Splits the Gray space into `segments` contiguous pieces (permanent.cpp:155-164)
// and sums the per-segment results in double-double.
void gray_sum(const Reduced &R, bool laplace, int segments, std::vector<ddc> &out) {
    std::vector<int> limits(R.nr - 1);
    int64_t idx_max = 1;
    for (int i = 0; i + 1 < R.nr; ++i) {
        limits[i] = R.rows[i + 1] + 1;
        idx_max *= limits[i];
    }
    int64_t conc = std::max<int64_t>(1, std::min<int64_t>(segments, idx_max));
    const int nout = laplace ? R.nc : 1;
    std::vector<std::vector<ddc>> part(conc, std::vector<ddc>(nout, ddc_from(0.0, 0.0)));
#if defined(_OPENMP)
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int64_t job = 0; job < conc; ++job) {
        int64_t batch = idx_max / conc;
        int64_t first = job * batch;
        int64_t last = (job == conc - 1) ? idx_max - 1 : (job + 1) * batch - 1;
        walk_segment(R, limits, first, last, laplace, part[job]);
    }
    out.assign(nout, ddc_from(0.0, 0.0));
    for (int64_t job = 0; job < conc; ++job)
        for (int l = 0; l < nout; ++l) out[l] = ddc_add(out[l], part[job][l]);
}

void store(const ddc &v, double *o) {
    o[0] = v.re.hi;
    o[1] = v.im.hi;
    o[2] = v.re.lo;
    o[3] = v.im.lo;
}

}  // namespace

extern "C" {

// Permanent of `a` (nr x nc complex128, interleaved re/im, row-major) with row
// multiplicities `rows` and column multiplicities `cols`.  Writes the
// double-double result as {re_hi, im_hi, re_lo, im_lo}.  Returns 0, or -1 when
// sum(rows) != sum(cols) (permanent.cpp:97-104 throws there).
int pqo_permanent_dd(const double *a, int nr, int nc, const int *rows, const int *cols,
                     int segments, double *out4) {
    Reduced R = reduce_rows(a, nr, nc, rows, cols);
    int64_t sr = 0, sc = 0;
    for (int v : R.rows) sr += v;
    for (int v : R.cols) sc += v;
    if (sr != sc) return -1;
    if (R.nr == 0 || R.nc == 0 || sr == 0) {  // permanent.cpp:106-108
        store(ddc_from(1.0, 0.0), out4);
        return 0;
    }
    if (R.nr == 1) {  // permanent.cpp:110-122
        ddc p = ddc_from(1.0, 0.0);
        for (int j = 0; j < R.nc; ++j)
            for (int q = 0; q < R.cols[j]; ++q) p = ddc_mul(p, ddc_from(R.a[2 * j], R.a[2 * j + 1]));
        store(p, out4);
        return 0;
    }
    std::vector<ddc> s;
    gray_sum(R, false, segments, s);
    double scale = std::ldexp(1.0, -static_cast<int>(sr - 1));  // permanent.cpp:259
    store(ddc_scale(s[0], scale), out4);
    return 0;
}

// Laplace-expansion permanents (permanent_laplace.cpp:43-240): for every column
// l, the permanent with cols[l] lowered by one.  `out` receives nc entries of
// {re_hi, im_hi, re_lo, im_lo}; returns the number of entries written (1 for the
// empty case of permanent_laplace.cpp:52-57).
int pqo_permanent_laplace_dd(const double *a, int nr, int nc, const int *rows, const int *cols,
                             int segments, double *out) {
    int64_t sr = 0, sc = 0;
    for (int i = 0; i < nr; ++i) sr += rows[i];
    for (int j = 0; j < nc; ++j) sc += cols[j];
    if (nr == 0 || nc == 0 || sr == 0 || sc == 0) {
        store(ddc_from(1.0, 0.0), out);
        return 1;
    }
    Reduced R = reduce_rows(a, nr, nc, rows, cols);
    std::vector<ddc> s;
    gray_sum(R, true, segments, s);
    double scale = std::ldexp(1.0, -static_cast<int>(sr - 1));  // permanent_laplace.cpp:227
    for (int l = 0; l < nc; ++l) store(ddc_scale(s[l], scale), out + 4 * l);
    return nc;
}

}  // extern "C"
