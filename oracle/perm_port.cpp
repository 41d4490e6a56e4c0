// CPU port of the reference permanent — TEST AND BASELINE INFRASTRUCTURE ONLY.
//
// A restatement of piquasso's own CPU implementation in its own arithmetic
// (std::complex<T>, T = double or float), its own work split
// (4 * std::thread::hardware_concurrency() contiguous Gray-code segments under
// one OpenMP parallel-for) and its own per-step operations, so that timing it on
// a host gives the reference's CPU throughput where the reference module itself
// cannot be built (it needs the reference source tree, absent on the GPU host).
// bench.py times it as the `cpu_baseline` (kind "port"); tests compare it with
// the double-double oracle.  Nothing in the product links it.
//
// Follows (reference paths, piquasso 8.0.1):
//   * src/permanent.cpp:49-264           permanent_cpp<T>
//   * src/permanent_laplace.cpp:43-240   permanent_laplace_cpp<T>
//   * src/n_aryGrayCodeCounter.hpp:170-254
// The only change is a 64-bit Gray-code offset (hpp:179 truncates to int).
//
// Build: oracle/build.py, with the reference's Release flags (-O3 -fopenmp).

#include <cmath>
#include <complex>
#include <cstdint>
#include <thread>
#include <vector>
#if defined(_OPENMP)
#include <omp.h>
#endif

namespace {

int binom_int(int n, int k) {  // utils.hpp:43-61
    if (k < 0 || n < 0 || k > n) return 0;
    if (k == 0 || k == n) return 1;
    if (k > n - k) k = n - k;
    int r = 1;
    for (int i = 1; i <= k; ++i) r = (r / i) * (n - k + i) + (r % i) * (n - k + i) / i;
    return r;
}

struct Gray {  // n_aryGrayCodeCounter.hpp:170-254, heap arrays as in the reference
    int n;
    int *lim, *chain, *code;
    int64_t offset, offset_max;
    Gray(const int *limits, int nd, int64_t start) : n(nd), offset(start) {
        lim = new int[n];
        chain = new int[n];
        code = new int[n];
        for (int i = 0; i < n; ++i) lim[i] = limits[i];
        int64_t t = start;
        for (int i = 0; i < n; ++i) {
            chain[i] = static_cast<int>(t % lim[i]);
            t /= lim[i];
        }
        int parity = 0;
        for (int i = n - 1; i >= 0; --i) {
            int c = parity ? lim[i] - 1 - chain[i] : chain[i];
            code[i] = c;
            parity ^= (c & 1);
        }
        offset_max = 0;
    }
    ~Gray() {
        delete[] lim;
        delete[] chain;
        delete[] code;
    }
    int next(int &changed, int &prev, int &val) {
        changed = 0;
        if (offset >= offset_max) return 1;
        bool upd = true;
        int k = 0;
        while (upd) {
            if (chain[k] < lim[k] - 1) {
                chain[k]++;
                upd = false;
            } else if (chain[k] == lim[k] - 1) {
                chain[k] = 0;
                upd = true;
            }
            k++;
        }
        int parity = 0;
        for (int i = n - 1; i >= 0; --i) {
            int c = parity ? lim[i] - 1 - chain[i] : chain[i];
            parity ^= (c & 1);
            if (c != code[i]) {
                prev = code[i];
                val = c;
                code[i] = c;
                changed = i;
                break;
            }
        }
        offset++;
        return 0;
    }
};

template <typename T>
struct Input {
    int nr, nc;
    std::vector<std::complex<T>> a;
    std::vector<int> rows, cols;
};

// permanent.cpp:54-95
template <typename T>
Input<T> reduce(const T *a, int nr, int nc, const int *rows, const int *cols) {
    Input<T> in;
    in.nc = nc;
    in.cols.assign(cols, cols + nc);
    int min_idx = 0, minelem = 0;
    for (int i = 0; i < nr; ++i)
        if (minelem == 0 || (rows[i] < minelem && rows[i] != 0)) {
            minelem = rows[i];
            min_idx = i;
        }
    const std::complex<T> *ac = reinterpret_cast<const std::complex<T> *>(a);
    if (nr > 0 && minelem != 0) {
        in.nr = nr + 1;
        in.rows.resize(nr + 1);
        in.rows[0] = 1;
        for (int i = 0; i < nr; ++i) in.rows[i + 1] = rows[i];
        in.rows[1 + min_idx] -= 1;
        in.a.resize(static_cast<size_t>(in.nr) * nc);
        for (int j = 0; j < nc; ++j) in.a[j] = ac[static_cast<size_t>(min_idx) * nc + j];
        for (int i = 0; i < nr; ++i)
            for (int j = 0; j < nc; ++j) in.a[static_cast<size_t>(i + 1) * nc + j] = ac[static_cast<size_t>(i) * nc + j];
    } else {
        in.nr = nr;
        in.rows.assign(rows, rows + nr);
        in.a.assign(ac, ac + static_cast<size_t>(nr) * nc);
    }
    return in;
}

template <typename T>
int permanent_port(const T *a, int nr, int nc, const int *rows, const int *cols, int nthreads, T *out) {
    using C = std::complex<T>;
    Input<T> A = reduce(a, nr, nc, rows, cols);
    int sum_rows = 0, sum_cols = 0;
    for (int v : A.rows) sum_rows += v;
    for (int v : A.cols) sum_cols += v;
    if (sum_rows != sum_cols) return -1;
    if (A.nr == 0 || A.nc == 0 || sum_rows == 0) {
        out[0] = 1;
        out[1] = 0;
        return 0;
    }
    if (A.nr == 1) {
        C r(1, 0);
        for (int i = 0; i < A.nc; ++i)
            for (int j = 0; j < A.cols[i]; ++j) r *= A.a[i];
        out[0] = r.real();
        out[1] = r.imag();
        return 0;
    }
    std::vector<C> mtx2(A.a.size());
    for (size_t i = 0; i < A.a.size(); ++i) mtx2[i] = A.a[i] * C(2.0, 0.0);
    int nd = A.nr - 1;
    std::vector<int> lim(nd);
    for (int i = 0; i < nd; ++i) lim[i] = A.rows[i + 1] + 1;
    int64_t idx_max = lim[0];
    for (int i = 1; i < nd; ++i) idx_max *= lim[i];

    unsigned hw = nthreads > 0 ? static_cast<unsigned>(nthreads) : std::thread::hardware_concurrency();
    int64_t conc = static_cast<int64_t>(hw) * 4;  // permanent.cpp:145-147
    conc = conc < idx_max ? conc : idx_max;
    std::vector<C> res(static_cast<size_t>(conc), C(0, 0));
    const int ncol = A.nc;

#if defined(_OPENMP)
#pragma omp parallel for num_threads(static_cast<unsigned int>(conc))
#endif
    for (int64_t job = 0; job < conc; ++job) {
        int64_t batch = idx_max / conc;
        int64_t first = job * batch;
        int64_t last = (job + 1) * batch - 1;
        if (job == conc - 1) last = idx_max - 1;
        Gray g(lim.data(), nd, first);
        g.offset_max = last;
        int *code = g.code;
        int bc = 1;
        std::vector<C> colsum(A.a.begin(), A.a.begin() + ncol);
        int minus_all = 0;
        for (int i = 0; i < nd; ++i) {
            int ms = code[i];
            int m = A.rows[i + 1];
            for (int j = 0; j < ncol; ++j)
                colsum[j] += A.a[static_cast<size_t>(i + 1) * ncol + j] * static_cast<T>(m - 2 * ms);
            minus_all += ms;
            bc *= binom_int(m, ms);
        }
        // the reference stores this sign in a plain `char` (src/permanent.cpp:202,
        // src/permanent_laplace.cpp:174): unsigned on aarch64, where -1 becomes
        // 255 and the reference's result is wrong; a signed type gives the same
        // values as the reference on x86-64 and the right ones everywhere
        int parity = (minus_all % 2 == 0) ? 1 : -1;
        C prod(static_cast<T>(parity), 0);
        for (int i = 0; i < ncol; ++i)
            for (int j = 0; j < A.cols[i]; ++j) prod *= colsum[i];
        C &acc = res[static_cast<size_t>(job)];
        acc += prod * static_cast<T>(bc);
        for (int64_t i = first + 1; i < last + 1; ++i) {
            int ch = 0, pv = 0, v = 0;
            if (g.next(ch, pv, v)) break;
            parity = -parity;
            int ro = ch + 1;
            prod = C(static_cast<T>(parity), 0);
            for (int j = 0; j < ncol; ++j) {
                colsum[j] += mtx2[static_cast<size_t>(ro) * ncol + j] * static_cast<T>(pv - v);
                for (int k = 0; k < A.cols[j]; ++k) prod *= colsum[j];
            }
            int m = A.rows[ch + 1];
            bc = v < pv ? bc * pv / (m - v) : bc * (m - pv) / v;
            acc += prod * static_cast<T>(bc);
        }
    }
    C perm(0, 0);
    for (const C &r : res) perm += r;
    perm /= static_cast<T>(std::ldexp(1.0, sum_rows - 1));
    out[0] = perm.real();
    out[1] = perm.imag();
    return 0;
}

template <typename T>
int laplace_port(const T *a, int nr, int nc, const int *rows, const int *cols, int nthreads, T *out) {
    using C = std::complex<T>;
    int sum_rows = 0, sum_cols = 0;
    for (int i = 0; i < nr; ++i) sum_rows += rows[i];
    for (int j = 0; j < nc; ++j) sum_cols += cols[j];
    if (nr == 0 || nc == 0 || sum_rows == 0 || sum_cols == 0) {  // permanent_laplace.cpp:52-57
        out[0] = 1;
        out[1] = 0;
        return 1;
    }
    Input<T> A = reduce(a, nr, nc, rows, cols);
    std::vector<C> mtx2(A.a.size());
    for (size_t i = 0; i < A.a.size(); ++i) mtx2[i] = A.a[i] * C(2.0, 0.0);
    int nd = A.nr - 1;
    std::vector<int> lim(nd);
    for (int i = 0; i < nd; ++i) lim[i] = A.rows[i + 1] + 1;
    int64_t idx_max = lim[0];
    for (int i = 1; i < nd; ++i) idx_max *= lim[i];
    unsigned hw = nthreads > 0 ? static_cast<unsigned>(nthreads) : std::thread::hardware_concurrency();
    int64_t conc = static_cast<int64_t>(hw) * 4;
    conc = conc < idx_max ? conc : idx_max;
    const int ncol = A.nc;
    std::vector<C> res(static_cast<size_t>(conc) * ncol);

#if defined(_OPENMP)
#pragma omp parallel for num_threads(static_cast<unsigned int>(conc))
#endif
    for (int64_t job = 0; job < conc; ++job) {
        int64_t batch = idx_max / conc;
        int64_t first = job * batch;
        int64_t last = (job + 1) * batch - 1;
        if (job == conc - 1) last = idx_max - 1;
        Gray g(lim.data(), nd, first);
        g.offset_max = last;
        int *code = g.code;
        int bc = 1;
        std::vector<C> colsum(A.a.begin(), A.a.begin() + ncol);
        int minus_all = 0;
        for (int i = 0; i < nd; ++i) {
            int ms = code[i];
            int m = A.rows[i + 1];
            for (int j = 0; j < ncol; ++j)
                colsum[j] += A.a[static_cast<size_t>(i + 1) * ncol + j] * static_cast<T>(m - 2 * ms);
            minus_all += ms;
            bc *= binom_int(m, ms);
        }
        // the reference stores this sign in a plain `char` (src/permanent.cpp:202,
        // src/permanent_laplace.cpp:174): unsigned on aarch64, where -1 becomes
        // 255 and the reference's result is wrong; a signed type gives the same
        // values as the reference on x86-64 and the right ones everywhere
        int parity = (minus_all % 2 == 0) ? 1 : -1;
        std::vector<C> prods(ncol);
        for (int l = 0; l < ncol; ++l) {
            prods[l] = static_cast<T>(parity);
            for (int i = 0; i < ncol; ++i)
                for (int j = 0; j < (i == l ? A.cols[i] - 1 : A.cols[i]); ++j) prods[l] *= colsum[i];
        }
        size_t base = static_cast<size_t>(job) * ncol;
        for (int i = 0; i < ncol; ++i) res[base + i] = prods[i] * static_cast<T>(bc);
        for (int64_t i = first + 1; i < last + 1; ++i) {
            int ch = 0, pv = 0, v = 0;
            if (g.next(ch, pv, v)) break;
            parity = -parity;
            int ro = ch + 1;
            for (int j = 0; j < ncol; ++j) colsum[j] += mtx2[static_cast<size_t>(ro) * ncol + j] * static_cast<T>(pv - v);
            for (int l = 0; l < ncol; ++l) {
                prods[l] = static_cast<T>(parity);
                for (int k = 0; k < ncol; ++k)
                    for (int j = 0; j < (k == l ? A.cols[k] - 1 : A.cols[k]); ++j) prods[l] *= colsum[k];
            }
            int m = A.rows[ch + 1];
            bc = v < pv ? bc * pv / (m - v) : bc * (m - pv) / v;
            for (int k = 0; k < ncol; ++k) res[base + k] += prods[k] * static_cast<T>(bc);
        }
    }
    T den = static_cast<T>(std::ldexp(1.0, sum_rows - 1));
    for (int l = 0; l < ncol; ++l) {
        C p(0, 0);
        for (int64_t job = 0; job < conc; ++job) p += res[static_cast<size_t>(job) * ncol + l];
        p /= den;
        out[2 * l] = p.real();
        out[2 * l + 1] = p.imag();
    }
    return ncol;
}

}  // namespace

extern "C" {

// `nthreads` <= 0 uses std::thread::hardware_concurrency(), as the reference does.
int pqo_port_permanent_c128(const double *a, int nr, int nc, const int *rows, const int *cols,
                            int nthreads, double *out2) {
    return permanent_port<double>(a, nr, nc, rows, cols, nthreads, out2);
}
int pqo_port_permanent_c64(const float *a, int nr, int nc, const int *rows, const int *cols,
                           int nthreads, float *out2) {
    return permanent_port<float>(a, nr, nc, rows, cols, nthreads, out2);
}
int pqo_port_laplace_c128(const double *a, int nr, int nc, const int *rows, const int *cols,
                          int nthreads, double *out) {
    return laplace_port<double>(a, nr, nc, rows, cols, nthreads, out);
}
int pqo_port_laplace_c64(const float *a, int nr, int nc, const int *rows, const int *cols,
                         int nthreads, float *out) {
    return laplace_port<float>(a, nr, nc, rows, cols, nthreads, out);
}

}  // extern "C"
