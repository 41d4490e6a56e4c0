// Exact binomial moments of ideal boson sampling on selected output modes:
// the dynamic program of the low-rank marginal generating function (the
// method of the reference's piquasso/_simulators/passive/marginal.py:15-92,
// 163-216), on the GPU, for many mode sets at once.
//
// For a mode set T (k modes) and every occupied input mode a with r_a
// photons, f_a(z) = sum_j v_aj z_j with v_aj = conj(U[T_j, a]), and
//
//     P(z, w) = prod_a L_{r_a}(-f_a(z) conj(f_a(w))),   L_r(-x) = sum_m c_m x^m,  c_m = C(r, m) / m!.
//
// P has nonzero coefficients only for |alpha| = |beta|: one dense complex
// block P_d (N_d x N_d, N_d = C(d + k - 1, k - 1)) per degree d.  Multiplying
// by x = f_a(z) conj(f_a(w)) maps block d to block d+1,
//
//     (T P)_{d+1} = S P_d S^H,   (S q)[alpha] = sum_j v_j q[alpha - e_j],
//
// computed for every degree and every mode set in two launches (R = P S^H,
// then S R: 2k gathered terms per element).  Each input mode applies its
// factor by Horner's rule, Q = c_r P, then Q <- c_m P + T Q for m = r-1..0,
// with double-buffered blocks (for r = 1 that is P <- P + T P).  The
// binomial moments are b_alpha = alpha! Re P_{alpha, alpha}.  Everything is
// FP64, as the reference.
//
// Host side: compositions of each degree in lexicographic order, ranked by
// the combinatorial number system; the alpha - e_j index tables (shared by
// all sets); one device allocation per call.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/pqperm_gb300.h"

namespace pqg {
void set_last_error(const char *msg);
}

namespace {

constexpr int MG_MAX_DEG = 64;

struct MgLayout {
    int64_t off[MG_MAX_DEG + 2];   // element offset of block d within a set
    int64_t roff[MG_MAX_DEG + 2];  // element offset of R_d = P_d S^H (N_d x N_{d+1}) within a set
    int64_t soff[MG_MAX_DEG + 2];  // row offset of degree d in the alpha - e_j table
    int64_t N[MG_MAX_DEG + 2];
    int64_t set_elems, set_relems;
    int32_t nblocks;               // degrees in use: 0 .. nblocks - 1
    int32_t k;
};

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// degree d with tab[d] <= e < tab[d + 1] (tab ascending, tab[0] = 0)
__device__ __forceinline__ int find_deg(const int64_t *tab, int nb, int64_t e) {
    int lo = 0, hi = nb - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tab[mid] <= e)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// R_d[a, b] = sum_l conj(v_l) P_d[a, src_{d+1}(b, l)]   for d < nblocks - 1, every set
__global__ void mg_right(MgLayout L, int n_sets, const double2 *__restrict__ P, const int32_t *__restrict__ src,
                         const double2 *__restrict__ v, double2 *__restrict__ R) {
    const int nd = L.nblocks - 1;  // R blocks 0 .. nd-1
    if (nd <= 0) return;
    const int64_t per = L.roff[nd];
    const int64_t total = per * n_sets;
    for (int64_t g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; g < total;
         g += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t s = g / per, e = g - s * per;
        const int d = find_deg(L.roff, nd, e);
        const int64_t n0 = L.N[d], n1 = L.N[d + 1];
        const int64_t loc = e - L.roff[d];
        const int64_t a = loc / n1, b = loc - a * n1;
        const double2 *Pd = P + s * L.set_elems + L.off[d] + a * n0;
        const int32_t *sb = src + (L.soff[d + 1] + b) * L.k;
        const double2 *vs = v + s * L.k;
        double2 acc = make_double2(0.0, 0.0);
        for (int l = 0; l < L.k; ++l) {
            const int32_t c = sb[l];
            if (c < 0) continue;
            const double2 t = cmul(make_double2(vs[l].x, -vs[l].y), Pd[c]);
            acc.x += t.x;
            acc.y += t.y;
        }
        R[s * L.set_relems + e] = acc;
    }
}

// Y_d = cb * B_d + (d > 0 ? S R_{d-1} : 0)   for every block in use, every set
__global__ void mg_left(MgLayout L, int n_sets, const double2 *__restrict__ R, const int32_t *__restrict__ src,
                        const double2 *__restrict__ v, const double2 *__restrict__ B, double cb,
                        double2 *__restrict__ Y) {
    const int nb = L.nblocks;
    const int64_t per = L.off[nb];
    const int64_t total = per * n_sets;
    for (int64_t g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; g < total;
         g += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t s = g / per, e = g - s * per;
        const int d = find_deg(L.off, nb, e);
        const int64_t n1 = L.N[d];
        const int64_t loc = e - L.off[d];
        const int64_t a = loc / n1, b = loc - a * n1;
        const double2 base = B[s * L.set_elems + e];
        double2 acc = make_double2(cb * base.x, cb * base.y);
        if (d > 0) {
            const double2 *Rd = R + s * L.set_relems + L.roff[d - 1];
            const int32_t *sa = src + (L.soff[d] + a) * L.k;
            const double2 *vs = v + s * L.k;
            for (int j = 0; j < L.k; ++j) {
                const int32_t c = sa[j];
                if (c < 0) continue;
                const double2 t = cmul(vs[j], Rd[c * n1 + b]);
                acc.x += t.x;
                acc.y += t.y;
            }
        }
        Y[s * L.set_elems + e] = acc;
    }
}

// Y = c X over the blocks in use
__global__ void mg_scale(MgLayout L, int n_sets, const double2 *__restrict__ X, double c, double2 *__restrict__ Y) {
    const int64_t per = L.off[L.nblocks];
    const int64_t total = per * n_sets;
    for (int64_t g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; g < total;
         g += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t s = g / per, e = g - s * per;
        const double2 x = X[s * L.set_elems + e];
        Y[s * L.set_elems + e] = make_double2(c * x.x, c * x.y);
    }
}

// diag[s][soff[d] + i] = Re P_d[i, i]
__global__ void mg_diag(MgLayout L, int n_sets, const double2 *__restrict__ P, double *__restrict__ diag) {
    const int64_t per = L.soff[L.nblocks];
    const int64_t total = per * n_sets;
    for (int64_t g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; g < total;
         g += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t s = g / per, e = g - s * per;
        const int d = find_deg(L.soff, L.nblocks, e);
        const int64_t i = e - L.soff[d];
        diag[g] = P[s * L.set_elems + L.off[d] + i * L.N[d] + i].x;
    }
}

int fail(int code, const std::string &m) {
    pqg::set_last_error(m.c_str());
    return code;
}

double binom(int64_t n, int64_t r) {
    if (r < 0 || r > n) return 0.0;
    double v = 1.0;
    for (int64_t i = 1; i <= r; ++i) v = v * static_cast<double>(n - r + i) / static_cast<double>(i);
    return std::round(v);
}

// Compositions of `deg` into k parts, lexicographic (first part ascending).
void compositions(int deg, int k, std::vector<int> &out) {
    std::vector<int> c(k, 0);
    c[k - 1] = deg;
    for (;;) {
        out.insert(out.end(), c.begin(), c.end());
        int i = k - 2, suffix = c[k - 1];
        while (i >= 0 && suffix == 0) {
            suffix += c[i];
            --i;
        }
        if (i < 0) break;
        c[i] += 1;
        for (int t = i + 1; t < k; ++t) c[t] = 0;
        c[k - 1] = suffix - 1;
    }
}

// Rank of composition c (parts summing to deg) in that order.
int64_t rank_of(const int *c, int k, int deg) {
    int64_t r = 0;
    int rem = deg;
    for (int i = 0; i + 1 < k; ++i) {
        for (int t = 0; t < c[i]; ++t) r += static_cast<int64_t>(binom(rem - t + k - i - 2, k - i - 2));
        rem -= c[i];
    }
    return r;
}

}  // namespace

extern "C" {

int pqg_binomial_moments_c128(const double *U, int64_t d, const int32_t *input, const int32_t *modes, int32_t k,
                              int32_t n_sets, double *moments, int64_t max_device_bytes) try {
    if (!U || !input || !modes || !moments || d <= 0 || k <= 0 || k > 8 || n_sets <= 0)
        return fail(PQG_ERR_INVALID, "pqg_binomial_moments_c128: invalid arguments");
    int64_t n = 0;
    for (int64_t a = 0; a < d; ++a) {
        if (input[a] < 0) return fail(PQG_ERR_INVALID, "input photon numbers must be nonnegative");
        n += input[a];
    }
    for (int64_t j = 0; j < static_cast<int64_t>(n_sets) * k; ++j)
        if (modes[j] < 0 || modes[j] >= d) return fail(PQG_ERR_INVALID, "mode index out of range");
    if (n > MG_MAX_DEG) return fail(PQG_ERR_TOO_LARGE, "more than 64 photons");
    double dense = 1.0;
    for (int j = 0; j < k; ++j) dense *= static_cast<double>(n + 1);
    if (dense * n_sets > 1.0e9) return fail(PQG_ERR_TOO_LARGE, "n_sets * (n + 1)^k moments exceed 1e9");

    MgLayout L{};
    L.k = k;
    for (int64_t deg = 0; deg <= n + 1; ++deg) L.N[deg] = static_cast<int64_t>(binom(deg + k - 1, k - 1));
    for (int64_t deg = 0; deg <= n; ++deg) {
        L.off[deg + 1] = L.off[deg] + L.N[deg] * L.N[deg];
        L.soff[deg + 1] = L.soff[deg] + L.N[deg];
        L.roff[deg + 1] = L.roff[deg] + (deg < n ? L.N[deg] * L.N[deg + 1] : 0);
    }
    L.set_elems = L.off[n + 1];
    L.set_relems = std::max<int64_t>(1, L.roff[n]);
    const double bytes = (3.0 * L.set_elems + L.set_relems) * 16.0 * n_sets + L.soff[n + 1] * 4.0 * k +
                         L.soff[n + 1] * 8.0 * n_sets + 16.0 * k * n_sets * (d + 1);
    if (max_device_bytes > 0 && bytes > static_cast<double>(max_device_bytes))
        return fail(PQG_ERR_TOO_LARGE, "binomial-moment blocks exceed the device-memory limit");

    // compositions and the alpha - e_j tables
    std::vector<std::vector<int>> comps(n + 1);
    for (int64_t deg = 0; deg <= n; ++deg) {
        comps[deg].reserve(static_cast<size_t>(L.N[deg] * k));
        compositions(static_cast<int>(deg), k, comps[deg]);
    }
    std::vector<int32_t> src(static_cast<size_t>(L.soff[n + 1] * k), -1);
    for (int64_t deg = 1; deg <= n; ++deg)
        for (int64_t i = 0; i < L.N[deg]; ++i) {
            int c[8];
            for (int j = 0; j < k; ++j) c[j] = comps[deg][i * k + j];
            for (int j = 0; j < k; ++j) {
                if (c[j] == 0) continue;
                c[j] -= 1;
                src[(L.soff[deg] + i) * k + j] = static_cast<int32_t>(rank_of(c, k, static_cast<int>(deg - 1)));
                c[j] += 1;
            }
        }
    // v per occupied input mode and set: conj(U[T_j, a])
    std::vector<int64_t> occ;
    for (int64_t a = 0; a < d; ++a)
        if (input[a] > 0) occ.push_back(a);
    std::vector<double> vtab(occ.size() * n_sets * k * 2);
    for (size_t q = 0; q < occ.size(); ++q)
        for (int s = 0; s < n_sets; ++s)
            for (int j = 0; j < k; ++j) {
                const double *u = U + 2 * (static_cast<int64_t>(modes[s * k + j]) * d + occ[q]);
                double *o = &vtab[((q * n_sets + s) * k + j) * 2];
                o[0] = u[0];
                o[1] = -u[1];
            }

    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t sz_blk = static_cast<size_t>(L.set_elems) * n_sets * sizeof(double2);
    const size_t sz_R = static_cast<size_t>(L.set_relems) * n_sets * sizeof(double2);
    const size_t sz_src = src.size() * sizeof(int32_t);
    const size_t sz_v = std::max<size_t>(16, vtab.size() * sizeof(double));
    const size_t sz_diag = static_cast<size_t>(L.soff[n + 1]) * n_sets * sizeof(double);
    const size_t o_P = 0, o_Q = o_P + al(sz_blk), o_W = o_Q + al(sz_blk), o_R = o_W + al(sz_blk),
                 o_src = o_R + al(sz_R), o_v = o_src + al(sz_src), o_diag = o_v + al(sz_v),
                 total = o_diag + al(sz_diag);
    unsigned char *dev = nullptr;
    cudaError_t err = cudaMalloc(&dev, total);
    if (err != cudaSuccess) return fail(PQG_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(err));
    double2 *P = reinterpret_cast<double2 *>(dev + o_P);
    double2 *Q = reinterpret_cast<double2 *>(dev + o_Q);
    double2 *W = reinterpret_cast<double2 *>(dev + o_W);
    double2 *R = reinterpret_cast<double2 *>(dev + o_R);
    int32_t *d_src = reinterpret_cast<int32_t *>(dev + o_src);
    double2 *d_v = reinterpret_cast<double2 *>(dev + o_v);
    double *d_diag = reinterpret_cast<double *>(dev + o_diag);
    cudaStream_t st = 0;
    int dev_id = 0, sms = 148;
    cudaGetDevice(&dev_id);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev_id);
    auto grid = [&](int64_t work) {
        return static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>((work + 255) / 256, int64_t(sms) * 32)));
    };
#define MG_CHECK(expr)                                                                        \
    do {                                                                                      \
        cudaError_t e_ = (expr);                                                              \
        if (e_ != cudaSuccess) {                                                              \
            cudaFree(dev);                                                                    \
            return fail(PQG_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_));    \
        }                                                                                     \
    } while (0)
    // Blocks above the current top degree must read as zero in every buffer:
    // each later write covers all blocks up to a nondecreasing top degree.
    MG_CHECK(cudaMemsetAsync(P, 0, sz_blk, st));
    MG_CHECK(cudaMemsetAsync(Q, 0, sz_blk, st));
    MG_CHECK(cudaMemsetAsync(W, 0, sz_blk, st));
    MG_CHECK(cudaMemcpyAsync(d_src, src.data(), sz_src, cudaMemcpyHostToDevice, st));
    if (!vtab.empty()) MG_CHECK(cudaMemcpyAsync(d_v, vtab.data(), vtab.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    {
        // P_0 = 1 in every set (host loop over sets: one element each)
        std::vector<double2> one(1, make_double2(1.0, 0.0));
        for (int s = 0; s < n_sets; ++s)
            MG_CHECK(cudaMemcpyAsync(P + static_cast<int64_t>(s) * L.set_elems, one.data(), sizeof(double2),
                                     cudaMemcpyHostToDevice, st));
        MG_CHECK(cudaStreamSynchronize(st));
    }
    int64_t maxdeg = 0;
    for (size_t q = 0; q < occ.size(); ++q) {
        const int r = input[occ[q]];
        const double2 *vq = d_v + q * n_sets * k;
        const int64_t top = std::min<int64_t>(n, maxdeg + r);
        MgLayout Lq = L;
        Lq.nblocks = static_cast<int32_t>(top + 1);
        std::vector<double> c(r + 1);
        for (int m = 0; m <= r; ++m) {
            double f = 1.0;
            for (int t = 2; t <= m; ++t) f *= t;
            c[m] = binom(r, m) / f;
        }
        // Q = c_r P; then Q <- c_m P + T Q for m = r-1 .. 0; P <- Q
        mg_scale<<<grid(L.off[top + 1] * n_sets), 256, 0, st>>>(Lq, n_sets, P, c[r], Q);
        MG_CHECK(cudaGetLastError());
        for (int m = r - 1; m >= 0; --m) {
            mg_right<<<grid(L.roff[top] * n_sets), 256, 0, st>>>(Lq, n_sets, Q, d_src, vq, R);
            MG_CHECK(cudaGetLastError());
            mg_left<<<grid(L.off[top + 1] * n_sets), 256, 0, st>>>(Lq, n_sets, R, d_src, vq, P, c[m], W);
            MG_CHECK(cudaGetLastError());
            std::swap(Q, W);
        }
        std::swap(P, Q);
        maxdeg = top;
    }
    MgLayout Lf = L;
    Lf.nblocks = static_cast<int32_t>(n + 1);
    mg_diag<<<grid(L.soff[n + 1] * n_sets), 256, 0, st>>>(Lf, n_sets, P, d_diag);
    MG_CHECK(cudaGetLastError());
    std::vector<double> diag(static_cast<size_t>(L.soff[n + 1]) * n_sets);
    MG_CHECK(cudaMemcpyAsync(diag.data(), d_diag, sz_diag, cudaMemcpyDeviceToHost, st));
    MG_CHECK(cudaStreamSynchronize(st));
#undef MG_CHECK
    cudaFree(dev);
    // dense moments over {0..n}^k per set (row-major, first mode slowest): alpha! * diag
    const int64_t D = n + 1, per = static_cast<int64_t>(dense);
    std::fill(moments, moments + per * n_sets, 0.0);
    std::vector<double> fact(n + 1, 1.0);
    for (int64_t t = 1; t <= n; ++t) fact[t] = fact[t - 1] * t;
    for (int s = 0; s < n_sets; ++s)
        for (int64_t deg = 0; deg <= n; ++deg)
            for (int64_t i = 0; i < L.N[deg]; ++i) {
                int64_t at = 0;
                double f = 1.0;
                for (int j = 0; j < k; ++j) {
                    const int cc = comps[deg][i * k + j];
                    at = at * D + cc;
                    f *= fact[cc];
                }
                moments[s * per + at] = f * diag[static_cast<size_t>(s) * L.soff[n + 1] + L.soff[deg] + i];
            }
    return PQG_OK;
} catch (const std::bad_alloc &) {
    return fail(PQG_ERR_HOST, "out of host memory");
} catch (...) {  // no C++ exception crosses the C ABI
    return fail(PQG_ERR_HOST, "host-side failure");
}

}  // extern "C"
