// Host-side planner for the permanent walk kernels.
//
// Reduction and semantics follow the reference (piquasso 8.0.1):
//   * row reduction: src/permanent.cpp:54-95 (and src/permanent_laplace.cpp:59-100):
//     a copy of the first row with the smallest nonzero multiplicity becomes
//     row 0 with multiplicity 1, and that row's multiplicity drops by one;
//   * sum check: src/permanent.cpp:97-104 (plain form only);
//   * empty input gives 1: src/permanent.cpp:106-108, permanent_laplace.cpp:52-57;
//   * normalisation 2^(N-1): src/permanent.cpp:259, permanent_laplace.cpp:227.
// Digits with multiplicity 0 and columns with multiplicity 0 contribute a
// factor of one to every term, so the planner drops them (the Laplace form
// keeps one extra output for zero-multiplicity columns, see below).  The sum
// is then the same set of terms as the reference's; only the order of
// summation differs.
#include "plan.hpp"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <functional>
#include <thread>

namespace pqg {

namespace {

// C(n, k) in FP64 (exact while below 2^53; a bound check beyond that)
double binom_d(int n, int k) {
    if (k < 0 || k > n) return 0.0;
    if (k > n - k) k = n - k;
    double r = 1.0;
    for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
    return r;
}

}  // namespace

int host_threads(int64_t n) {
    // PQG_HOST_THREADS caps the count (1: plan on the calling thread only)
    int64_t cap = 8;
    if (const char *env = std::getenv("PQG_HOST_THREADS")) cap = std::max<int64_t>(1, std::atoll(env));
    if (n < 2048 || cap == 1) return 1;  // a thread's start costs about what 100 problems do
    const unsigned hw = std::thread::hardware_concurrency();
    const int64_t by_size = n / 1024;
    return static_cast<int>(std::max<int64_t>(1, std::min<int64_t>({cap, by_size, hw ? static_cast<int64_t>(hw) : 1})));
}

void parallel_ranges(int64_t n, int nt, const std::function<void(int, int64_t, int64_t)> &fn) {
    if (nt <= 1) {
        fn(0, 0, n);
        return;
    }
    // A worker's exception (std::bad_alloc) is rethrown on the calling
    // thread after every worker has joined, as the one-thread path would.
    std::vector<std::exception_ptr> errs(static_cast<size_t>(nt));
    auto run = [&](int w, int64_t lo, int64_t hi) {
        try {
            fn(w, lo, hi);
        } catch (...) {
            errs[static_cast<size_t>(w)] = std::current_exception();
        }
    };
    std::vector<std::thread> pool;
    pool.reserve(static_cast<size_t>(nt - 1));
    const int64_t per = (n + nt - 1) / nt;
    // A worker that cannot be started (std::system_error: no thread
    // resources) leaves its range, and every later one, to the calling
    // thread; the threads already started are always joined.
    int started = 1;
    for (int w = 1; w < nt; ++w) {
        const int64_t lo = std::min<int64_t>(n, w * per), hi = std::min<int64_t>(n, lo + per);
        try {
            pool.emplace_back(run, w, lo, hi);
        } catch (...) {
            break;
        }
        started = w + 1;
    }
    run(0, 0, std::min<int64_t>(n, per));
    for (int w = started; w < nt; ++w) {
        const int64_t lo = std::min<int64_t>(n, w * per), hi = std::min<int64_t>(n, lo + per);
        run(w, lo, hi);
    }
    for (auto &t : pool) t.join();
    for (auto &e : errs)
        if (e) std::rethrow_exception(e);
}

double algorithmic_flops(const PendingProblem &p, Form form) {
    if (p.kind != PQG_KIND_WALK) return 0.0;
    const int nc = p.nc - p.padded_cols;
    double sum_cm = 0;
    for (int k = 0; k < nc; ++k) sum_cm += p.cm[k];
    if (form == Form::PLAIN) return p.S * (4.0 * nc + 6.0 * sum_cm + 4.0);
    // Laplace: updates, prefix and suffix products over the factors, one
    // combine per output and a weighted accumulation per output.
    return p.S * (4.0 * nc + 12.0 * sum_cm + 6.0 * nc + 4.0 * p.n_out);
}

namespace {

// One pool per host thread: the buffers of the last planner destroyed on the
// thread (up to a cap), handed to the next planner created on it.  A planner
// created while the pool is empty (another planner on the thread holds its
// buffers) allocates as usual.
thread_local bool t_pool_gone = false;  // trivially destructible: readable while the thread tears down

struct PlannerPool {
    std::vector<PendingProblem> pending;
    std::vector<PqgProblem> probs;
    std::vector<unsigned char> arena;
    std::vector<int32_t> idx_rows;
    ~PlannerPool() { t_pool_gone = true; }
};
thread_local PlannerPool t_pool;

constexpr size_t kPoolCapBytes = size_t(64) << 20;

template <typename T>
size_t capacity_bytes(const std::vector<T> &v) {
    return v.capacity() * sizeof(T);
}

}  // namespace

Planner::Planner(Precision prec, Form form, const PlanConfig &cfg) : prec_(prec), form_(form), cfg_(cfg) {
    if (t_pool_gone) return;
    PlannerPool &P = t_pool;
    pending.swap(P.pending);
    probs.swap(P.probs);
    arena.swap(P.arena);
    idx_rows_.swap(P.idx_rows);
    pending.clear();
    probs.clear();
    arena.clear();
    idx_rows_.clear();
}

Planner::~Planner() {
    if (t_pool_gone) return;  // a planner destroyed while its thread tears down: plain frees
    PlannerPool &P = t_pool;  // the destroying thread's pool (a plan handle may die on another thread)
    const size_t mine = capacity_bytes(pending) + capacity_bytes(probs) + capacity_bytes(arena) +
                        capacity_bytes(idx_rows_);
    const size_t pooled = capacity_bytes(P.pending) + capacity_bytes(P.probs) + capacity_bytes(P.arena) +
                          capacity_bytes(P.idx_rows);
    if (mine <= kPoolCapBytes && mine > pooled) {
        P.pending.swap(pending);
        P.probs.swap(probs);
        P.arena.swap(arena);
        P.idx_rows.swap(idx_rows_);
    }
}

void Planner::set_matrix(const double *a, int64_t nr, int64_t nc) {
    a_ = a;
    int_nr_ = nr;
    int_nc_ = nc;
}

int Planner::make_pending_(PendingProblem &p, const int32_t *rows, const int32_t *cols, std::string &err,
                           int64_t row_base, int64_t n_rows_local, bool &df_domain) const {
    const int64_t nr = n_rows_local >= 0 ? n_rows_local : int_nr_, nc = int_nc_;
    p = PendingProblem{};
    if (nr < 0 || nc < 0 || (nr > 0 && nc > 0 && a_ == nullptr) || (nr > 0 && !rows) || (nc > 0 && !cols) ||
        row_base < 0 || row_base + nr > int_nr_) {
        err = "invalid matrix or multiplicity buffers";
        return 2;
    }
    // one pass per side: validation, sums and (rows) the first index of the
    // smallest nonzero multiplicity, the row the reduction copies
    int64_t sr = 0, sc = 0;
    int32_t neg = 0;
    int64_t min_idx = 0;
    int minelem = 0;
    for (int64_t i = 0; i < nr; ++i) {
        const int32_t r = rows[i];
        neg |= r;
        sr += r;
        if (r != 0 && (minelem == 0 || r < minelem)) {
            minelem = r;
            min_idx = i;
        }
    }
    if (neg < 0) {
        err = "row multiplicities must be nonnegative";
        return 2;
    }
    neg = 0;
    for (int64_t j = 0; j < nc; ++j) {
        neg |= cols[j];
        sc += cols[j];
    }
    if (neg < 0) {
        err = "column multiplicities must be nonnegative";
        return 2;
    }

    if (form_ == Form::PLAIN) {
        // src/permanent.cpp:97-104 (the reduction keeps the row sum unchanged)
        if (sr != sc) {
            err = "Number of input and output states should be equal";
            return 1;
        }
        if (nr == 0 || nc == 0 || sr == 0) {  // src/permanent.cpp:106-108
            p.kind = PQG_KIND_CONSTANT;
            p.n_out = 1;
            return 0;
        }
    } else {
        if (nr == 0 || nc == 0 || sr == 0 || sc == 0) {  // src/permanent_laplace.cpp:52-57
            p.kind = PQG_KIND_CONSTANT;
            p.n_out = 1;
            return 0;
        }
    }
    if (sr > 250) {
        err = "too many particles";
        return 3;
    }
    if (int_nr_ > (1 << 30) || nc > (1 << 30)) {
        err = "matrix dimension above 2^30";
        return 3;
    }
    // the double-float kernel keeps typical terms (>= N^(-N/2) after column
    // scaling) far above the FP32 underflow threshold only for N <= 32
    if (sr > 32) df_domain = false;

    // columns with nonzero multiplicity (branch-free: a slot is written for
    // every column and kept only when its multiplicity is nonzero)
    int kept = 0;
    int32_t cmax = 0;
    {
        int32_t col[PQG_MAX_COLS + 1];  // one spare slot for the columns not kept
        uint8_t cm[PQG_MAX_COLS + 1];
        for (int64_t j = 0; j < nc; ++j) {
            const int32_t c = cols[j];
            col[kept] = static_cast<int32_t>(j);
            cm[kept] = static_cast<uint8_t>(c);
            cmax = c > cmax ? c : cmax;
            kept += c != 0;
            if (kept > PQG_MAX_COLS) {
                err = "more than 32 distinct columns with nonzero multiplicity";
                return 3;
            }
        }
        std::memcpy(p.col, col, sizeof(int32_t) * kept);
        std::memcpy(p.cm, cm, kept);
    }
    if (cmax > 255) {
        err = "column multiplicity above 255";
        return 3;
    }
    if (kept == 0) {
        err = "no column with nonzero multiplicity";
        return 2;
    }
    p.nc = kept;

    if (form_ == Form::LAPLACE) {
        // outputs: one per kept column; every zero-multiplicity column shares
        // one extra output (its exponent stays 0: permanent_laplace.cpp:180,210)
        p.laplace_full = static_cast<int64_t>(kept) < nc;
        p.n_out = p.nc + (p.laplace_full ? 1 : 0);
    }

    // row reduction (src/permanent.cpp:54-95): a copy of row min_idx (the
    // first row with the smallest nonzero multiplicity) becomes the
    // prepended row with multiplicity 1
    p.row0 = static_cast<int>(row_base + min_idx);
    double S = 1.0;
    // the binomial weights prod C(m_i, g_i) must stay exact integers in FP64
    // and in the kernels' int64 products (only multiplicities >= 2 add to it)
    double wmax = 1.0;
    int nd = 0;
    {
        uint8_t mm[PQG_MAX_OUTER + 1];  // branch-free like the columns
        int32_t rr[PQG_MAX_OUTER + 1];
        for (int64_t i = 0; i < nr; ++i) {
            const int m = rows[i] - (i == min_idx ? 1 : 0);
            mm[nd] = static_cast<uint8_t>(m);  // m <= 250
            rr[nd] = static_cast<int32_t>(row_base + i);
            S *= m > 0 ? m + 1 : 1;
            nd += m > 0;
            if (nd > PQG_MAX_OUTER) {  // every digit at least doubles S
                S = std::ldexp(1.0, 60);
                nd = PQG_MAX_OUTER;
                break;
            }
            if (m > 1) wmax *= binom_d(m, m / 2);
        }
        p.nd = nd;
        std::memcpy(p.m, mm, nd);
        std::memcpy(p.row, rr, sizeof(int32_t) * nd);
    }
    if (S > 1125899906842624.0) {  // 2^50
        err = "Gray-code space above 2^50 steps";
        return 3;
    }
    if (wmax > 9.0e15) {
        err = "binomial weights of the row multiplicities exceed 2^53";
        return 3;
    }
    p.S = S;
    p.scale_exp = static_cast<int>(sr - 1);
    return 0;
}

int Planner::add(const int32_t *rows, const int32_t *cols, std::string &err, int64_t row_base,
                 int64_t n_rows_local) {
    PendingProblem p;
    bool dom = true;
    const int st = make_pending_(p, rows, cols, err, row_base, n_rows_local, dom);
    if (st) return st;
    pending.push_back(p);
    if (!dom) df_ok_add_ = false;
    return 0;
}

int Planner::add_batch(const int32_t *rows, const int32_t *cols, int64_t batch, std::string &err,
                       int64_t *err_index) {
    const size_t base = pending.size();
    pending.resize(base + static_cast<size_t>(batch));
    const int nt = host_threads(batch);
    std::vector<int64_t> bad(static_cast<size_t>(nt), -1);
    std::vector<int> bad_st(static_cast<size_t>(nt), 0);
    std::vector<std::string> bad_err(static_cast<size_t>(nt));
    std::vector<char> dom(static_cast<size_t>(nt), 1);
    parallel_ranges(batch, nt, [&](int w, int64_t lo, int64_t hi) {
        for (int64_t b = lo; b < hi; ++b) {
            bool d = true;
            const int st = make_pending_(pending[base + static_cast<size_t>(b)], rows ? rows + b * int_nr_ : nullptr,
                                         cols ? cols + b * int_nc_ : nullptr, bad_err[static_cast<size_t>(w)], 0,
                                         -1, d);
            if (!d) dom[static_cast<size_t>(w)] = 0;
            if (st) {  // the range's first failure; later problems of the range are not needed
                bad[static_cast<size_t>(w)] = b;
                bad_st[static_cast<size_t>(w)] = st;
                return;
            }
        }
    });
    for (int w = 0; w < nt; ++w) {  // ranges are in order: the first failing range has the lowest index
        if (bad[static_cast<size_t>(w)] >= 0) {
            err = bad_err[static_cast<size_t>(w)];
            if (err_index) *err_index = bad[static_cast<size_t>(w)];
            pending.resize(base);
            return bad_st[static_cast<size_t>(w)];
        }
    }
    for (int w = 0; w < nt; ++w)
        if (!dom[static_cast<size_t>(w)]) df_ok_add_ = false;
    return 0;
}

void laplace_slots(const PendingProblem &p, int64_t n_cols, int *slot) {
    for (int64_t j = 0; j < n_cols; ++j) slot[j] = p.nc;  // the shared slot (only read when laplace_full)
    for (int k = 0; k < p.nc - p.padded_cols; ++k) slot[p.col[k]] = k;
}

int64_t Planner::align_(size_t al) {
    size_t n = arena.size();
    size_t r = (n + al - 1) / al * al;
    arena.resize(r, 0);
    return static_cast<int64_t>(r);
}

int64_t Planner::push_bytes_(const void *p, size_t n) {
    int64_t off = align_(16);
    arena.resize(arena.size() + n);
    std::memcpy(arena.data() + off, p, n);
    return off;
}

namespace {

// Steps per lane below which the per-lane seeding (about 2 x NC flops per
// nonzero outer digit, at 48 bits or more) stops being small next to the walk.
int64_t min_steps_per_seed(Precision prec) {
    switch (prec) {
        case Precision::C128: return 512;     // FP64 seed, FP64 steps
        case Precision::C128DF: return 256;   // double-float seed and steps
        default: return 1024;                 // double-float seed, FP32 steps
    }
}

// Signed binomial weights (-1)^sum(g) prod C(m, g) of the reflected
// mixed-radix Gray code over the inner digits (digit 0 fastest), from code 0.
std::vector<double> build_weights(const std::vector<int> &mm, int64_t P) {
    const size_t K = mm.size();
    std::vector<int> lim(K), chain(K, 0), code(K, 0);
    for (size_t k = 0; k < K; ++k) lim[k] = mm[k] + 1;
    std::vector<double> w(P, 1.0);
    int64_t bc = 1;
    int parity = 0;
    for (int64_t t = 1; t < P; ++t) {
        size_t k = 0;
        while (true) {
            if (chain[k] < lim[k] - 1) {
                chain[k]++;
                break;
            }
            chain[k] = 0;
            ++k;
        }
        int par = 0, ch = -1, prev = 0, val = 0;
        for (int i = static_cast<int>(K) - 1; i >= 0; --i) {
            const int c = par ? lim[i] - 1 - chain[i] : chain[i];
            par ^= (c & 1);
            if (c != code[i] && ch < 0) {
                ch = i;
                prev = code[i];
                val = c;
            }
        }
        code[ch] = val;
        parity ^= 1;
        bc = val > prev ? bc * (mm[ch] - prev) / val : bc * prev / (mm[ch] - val);
        w[t] = (parity ? -1.0 : 1.0) * static_cast<double>(bc);
    }
    return w;
}

}  // namespace

void Planner::finish() {
    const size_t np = pending.size();
    probs.assign(np, PqgProblem{});
    item_begin.assign(np + 1, 0);
    chunks.clear();
    arena.clear();
    table_cache_.clear();
    total_items = total_parts = total_outputs = 0;
    total_delta = 0;
    pdata_bytes = 0;
    matrix_off = 0;
    mat_rows = mat_cols = 0;
    total_steps = total_flops = 0.0;
    max_nc = 1;
    all_ones = true;
    df_ok = df_ok_add_;

    const bool c128 = prec_ == Precision::C128;
    const bool df = prec_ == Precision::C128DF;
    const bool laplace = form_ == Form::LAPLACE;

    // One walk kernel serves the whole plan and is compiled for an exact column
    // count, so every problem of a batch is padded to the largest column count
    // with neutral columns: multiplicity 1, column sum exactly 1 + 0i at every
    // step (zero rows), so each term is multiplied by 1 exactly.  In the
    // Laplace form a neutral column's own output is never read, and the shared
    // output of the zero-multiplicity columns moves behind the padded ones.
    bool any_walk = false;
    int ncmax = 1;
    {
        for (auto &p : pending)
            if (p.kind == PQG_KIND_WALK) {
                ncmax = std::max(ncmax, p.nc);
                any_walk = true;
            }
        for (auto &p : pending) {
            if (p.kind != PQG_KIND_WALK || p.nc == ncmax) continue;
            const int old = p.nc, add = ncmax - old;
            for (int k = old; k < ncmax; ++k) {
                p.cm[k] = 1;
                p.col[k] = -1;
            }
            p.nc = ncmax;
            p.padded_cols = add;
            if (laplace) p.n_out = ncmax + (p.laplace_full ? 1 : 0);
        }
    }
    // the matrix every problem indexes, once
    if (any_walk) {
        mat_rows = int_nr_;
        mat_cols = int_nc_;
        matrix_off = push_bytes_(a_, static_cast<size_t>(2 * int_nr_ * int_nc_) * sizeof(double));
    }

    // complex64 Laplace plans whose every walk problem has unit columns (the
    // exact sampler's) store their prefix tables as code pairs for the
    // two-code walk: each problem's table holds an even number of codes
    pairs = false;
    if (prec_ == Precision::C64 && laplace && any_walk && ncmax >= 2 && ncmax <= PQG_PAIRS_MAX_NC) {
        pairs = true;
        for (const auto &p : pending) {
            if (p.kind != PQG_KIND_WALK) continue;
            for (int k = 0; k < p.nc && pairs; ++k) pairs = p.cm[k] == 1;
            if (!pairs) break;
        }
    }

    // Steps per lane: about items_per_smsp warps of work per SM sub-partition
    // for balance, but at least enough steps to amortise the seeding.
    double S_tot = 0.0;
    for (auto &p : pending)
        if (p.kind == PQG_KIND_WALK) S_tot += p.S;
    const double resident_warps = 4.0 * cfg_.num_sms * 3.0;
    const int64_t items = cfg_.items_per_smsp > 0 ? cfg_.items_per_smsp : 16;
    const double balance = S_tot / (32.0 * 4.0 * cfg_.num_sms * static_cast<double>(items));
    const double seed_floor = std::min<double>(static_cast<double>(cfg_.seed_steps > 0 ? cfg_.seed_steps
                                                                                    : min_steps_per_seed(prec_)),
                                               S_tot / (32.0 * resident_warps));
    const double steps_per_lane = std::max({balance, seed_floor, 1.0});
    // longest inner walk: the problem's prefix table (P x nc elements) should
    // stay resident in L1 next to the other warps' tables; the FP64 walk is
    // bound by its arithmetic pipe and tolerates longer tables
    int64_t p_cap = prec_ == Precision::C128 ? 512 : 256;
    if (cfg_.p_max_user) p_cap = cfg_.p_max;
    int64_t p_max = laplace ? std::min<int64_t>(std::min<int64_t>(cfg_.p_max, p_cap), 512)
                            : std::min<int64_t>(cfg_.p_max, p_cap);
    // the complex64 plain walk of 17..24 columns stages each problem's table
    // in shared memory, which holds PQG_SMEM_TABLE_P codes (a hard limit, over
    // any tuning)
    if (prec_ == Precision::C64 && !laplace && ncmax >= PQG_SMEM_TABLE_NC_MIN && ncmax <= PQG_SMEM_TABLE_NC_MAX)
        p_max = std::min<int64_t>(p_max, PQG_SMEM_TABLE_P);
    // likewise the two-code Laplace walk's shared-memory table of code pairs
    if (pairs) p_max = std::min<int64_t>(p_max, PQG_PAIRS_TABLE_P);
    // per-problem device data (built by the prep kernel), by offset from the
    // start of that region; the region follows the uploaded arena
    auto pdata = [&](int64_t bytes) {
        const int64_t off = pdata_bytes;
        pdata_bytes += (bytes + 15) / 16 * 16;
        return off;
    };
    const int64_t d_elem = prec_ == Precision::C64 ? 8 : 16;  // one D element: float2, else double2 / float4
    // items a block takes at once: the complex64 plain walk and the two-code
    // Laplace walk hand out groups of PQG_ITEM_GROUP consecutive items (one
    // per warp of a block), so a block's warps walk one problem's prefix table
    // together (staged in shared memory or shared in L1); their problems then
    // come in whole groups of items
    const int64_t group = (prec_ == Precision::C64 && (form_ == Form::PLAIN || pairs)) ? PQG_ITEM_GROUP : 1;
    item_group = static_cast<int>(group);

    // Outputs stay in the caller's order; the work runs longest items first.
    // The device queue hands out items in problem order, so the problems are
    // laid out by descending steps per lane (an item's duration): the short
    // items come last and fill the end of the launch (longest-processing-
    // time-first), instead of a long item starting when the others are done.
    out_of.assign(np, 0);
    for (size_t b = 0; b < np; ++b) {
        out_of[b] = total_outputs;
        total_outputs += pending[b].n_out;
    }
    std::vector<double> key(np, 0.0);
    std::vector<int32_t> order(np);
    for (size_t b = 0; b < np; ++b) {
        order[b] = static_cast<int32_t>(b);
        if (pending[b].kind == PQG_KIND_WALK) key[b] = std::max(1.0, std::min(steps_per_lane, pending[b].S / 32.0));
    }
    std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) { return key[x] > key[y]; });

    // Per-problem work in two passes.  The first fills what depends on the
    // problem alone -- its split into inner and outer digits, the digit
    // tables, the matrix index rows for the prep kernel, the weight table's
    // key -- on several host threads for large batches; the second places the
    // problems in work order (offsets into items, partials, chunks, the arena,
    // the device-built data and the prefix tables).  The plan is the same
    // whatever the thread count.
    constexpr int IDX_STRIDE = 1 + PQG_MAX_OUTER + PQG_MAX_COLS;
    std::vector<int32_t> &idxv = idx_rows_;
    idxv.resize(np * IDX_STRIDE);  // reused capacity: every row's first n_idx entries are written below
    std::vector<int32_t> n_idx(np, 0);
    std::vector<std::pair<uint64_t, uint64_t>> tkey(np);
    std::vector<char> lap_too_wide(np, 0);
    std::vector<double> flops(np, 0.0);
    parallel_ranges(static_cast<int64_t>(np), host_threads(static_cast<int64_t>(np)), [&](int, int64_t lo,
                                                                                          int64_t hi) {
        for (int64_t ipl = lo; ipl < hi; ++ipl) {
            const size_t ip = static_cast<size_t>(ipl);
            const PendingProblem &p = pending[static_cast<size_t>(order[ip])];
            PqgProblem &q = probs[ip];
            q.kind = p.kind;
            q.index = order[ip];
            q.n_out = p.n_out;
            q.out_index = out_of[static_cast<size_t>(order[ip])];
            q.off_base64 = q.off_outer64 = q.off_base_df = q.off_outer_df = q.off_D = -1;
            if (p.kind == PQG_KIND_CONSTANT) {
                q.cval_re = p.cre;
                q.cval_im = p.cim;
                q.P = 1;
                q.R = 1;
                continue;
            }
            q.nc = p.nc;
            q.laplace = laplace ? 1 : 0;
            q.scale_exp = p.scale_exp;
            int cm_max = 1;
            for (int k = 0; k < p.nc; ++k) {
                q.cm[k] = static_cast<uint8_t>(p.cm[k]);
                cm_max = std::max<int>(cm_max, p.cm[k]);
            }
            q.cm_max = cm_max;
            if (df && laplace) {
                // the double-float Laplace walk folds the whole step weight
                // (inner times outer) into one FP32 value: its largest, the
                // product over every digit of C(m, m/2), must be exact in FP32
                double wmax = 1.0;
                for (int i = 0; i < p.nd; ++i) wmax *= binom_d(p.m[i], p.m[i] / 2);
                if (wmax > 16777216.0) lap_too_wide[ip] = 1;
            }

            // this problem's steps per lane: the plan's, but never so many
            // that the problem fills less than one warp
            const double lane_steps = std::max(1.0, std::min(steps_per_lane, p.S / 32.0));
            // inner digits: ascending multiplicity, greedily while the inner
            // walk fits both the lane's steps and the table limit
            const int nd = p.nd;
            int dorder[PQG_MAX_OUTER];
            for (int i = 0; i < nd; ++i) {  // stable insertion sort (nd <= 60; no allocation)
                int at = i;
                while (at > 0 && p.m[dorder[at - 1]] > p.m[i]) {
                    dorder[at] = dorder[at - 1];
                    --at;
                }
                dorder[at] = i;
            }
            const double p_target = std::min<double>(static_cast<double>(p_max), lane_steps);
            int inner[PQG_MAX_INNER], outer[PQG_MAX_OUTER];
            int K_ = 0, no = 0;
            double P = 1.0;
            for (int oi = 0; oi < nd; ++oi) {
                const int i = dorder[oi];
                if (no == 0 && K_ < PQG_MAX_INNER && P * (p.m[i] + 1) <= p_target) {
                    inner[K_++] = i;
                    P *= (p.m[i] + 1);
                } else {
                    outer[no++] = i;
                }
            }
            const size_t K = static_cast<size_t>(K_);
            q.P = static_cast<int32_t>(P);
            q.K = static_cast<int32_t>(K);
            q.n_outer = no;
            q.Q = static_cast<int64_t>(std::llround(p.S / P));
            q.R = std::max<int64_t>(1, static_cast<int64_t>(lane_steps / P));
            q.R = std::min<int64_t>(q.R, std::max<int64_t>(1, q.Q / (PQG_ITEM_LANES * group)));
            // whole warps (whole groups): the outer positions spread evenly
            // over the nearest count of item groups, so a problem's last item
            // is not mostly idle lanes (an item is one warp; its lanes all run
            // about R inner walks)
            {
                const int64_t per_group = PQG_ITEM_LANES * group * q.R;
                const int64_t n_grp = std::max<int64_t>(1, (q.Q + per_group / 2) / per_group);
                q.R = (q.Q + PQG_ITEM_LANES * group * n_grp - 1) / (PQG_ITEM_LANES * group * n_grp);
            }
            for (int o = 0; o < no; ++o) q.outer_m[o] = static_cast<uint8_t>(p.m[outer[o]]);
            for (size_t k = 0; k < K; ++k) q.inner_m[k] = static_cast<uint8_t>(p.m[inner[k]]);
            const int64_t lanes = (q.Q + q.R - 1) / q.R;
            q.n_items = (lanes + PQG_ITEM_LANES - 1) / PQG_ITEM_LANES;
            q.n_items = (q.n_items + group - 1) / group * group;  // trailing items of a group may be empty

            // matrix rows and columns for the device prep
            int32_t *idx = idxv.data() + ip * IDX_STRIDE;
            int c = 0;
            idx[c++] = p.row0;
            for (int o = 0; o < no; ++o) idx[c++] = p.row[outer[o]];
            for (size_t k = 0; k < K; ++k) idx[c++] = p.row[inner[k]];
            for (int k = 0; k < p.nc; ++k) idx[c++] = p.col[k];
            n_idx[ip] = c;
            // the weight table depends only on the inner multiplicities: K <= 16
            // of them, each below 256, packed into a 128-bit key
            std::pair<uint64_t, uint64_t> key{static_cast<uint64_t>(K), 0};
            for (size_t k = 0; k < K; ++k) {
                const uint64_t v = p.m[inner[k]];
                if (k < 7)
                    key.first |= v << (8 * (k + 1));
                else
                    key.second |= v << (8 * (k - 7));
            }
            tkey[ip] = key;
            flops[ip] = algorithmic_flops(p, form_);
        }
    });

    for (size_t ip = 0; ip < np; ++ip) {
        const PendingProblem &p = pending[static_cast<size_t>(order[ip])];
        PqgProblem &q = probs[ip];
        q.item_begin = total_items;
        q.part_begin = total_parts;
        q.chunk_begin = static_cast<int64_t>(chunks.size());
        q.delta_begin = total_delta;  // kept monotone for the device's binary search
        if (p.kind == PQG_KIND_CONSTANT) {
            item_begin[ip + 1] = total_items;
            continue;
        }
        max_nc = std::max(max_nc, p.nc);
        all_ones = all_ones && q.cm_max == 1;
        if (lap_too_wide[ip]) df_ok = false;
        const int no = q.n_outer;
        q.off_idx = push_bytes_(idxv.data() + ip * IDX_STRIDE, static_cast<size_t>(n_idx[ip]) * sizeof(int32_t));
        // device-built seeds and step rows in the walk's precision
        if (c128) {
            q.off_base64 = pdata(16 * p.nc);
            if (no) q.off_outer64 = pdata(16 * int64_t(no) * p.nc);
        } else {
            q.off_base_df = pdata(16 * p.nc);
            if (no) q.off_outer_df = pdata(16 * int64_t(no) * p.nc);
        }
        if (no) q.off_D = pdata(d_elem * 2 * int64_t(no) * p.nc);
        total_delta += static_cast<int64_t>(pairs ? (q.P + 1) & ~1 : q.P) * p.nc;

        auto it = table_cache_.find(tkey[ip]);
        if (it != table_cache_.end()) {
            q.off_tab = it->second;
        } else {
            std::vector<int> mm(static_cast<size_t>(q.K));
            for (int k = 0; k < q.K; ++k) mm[static_cast<size_t>(k)] = q.inner_m[k];
            const std::vector<double> w = build_weights(mm, q.P);
            std::vector<PqgStep> tab(q.P);
            for (int64_t t = 0; t < q.P; ++t) {
                tab[t].wd = w[t];
                tab[t].wf = static_cast<float>(w[t]);
                tab[t].pad = 0.0f;
                if (df && std::fabs(w[t]) > 16777216.0) df_ok = false;  // not exact in FP32
            }
            q.off_tab = push_bytes_(tab.data(), tab.size() * sizeof(PqgStep));
            table_cache_[tkey[ip]] = q.off_tab;
        }

        total_items += q.n_items;
        total_parts += q.n_items * q.n_out;
        item_begin[ip + 1] = total_items;
        // level-1 reduction chunks
        const int64_t per_chunk = PQG_CHUNK_ITEMS;
        for (int64_t lo = q.item_begin; lo < q.item_begin + q.n_items; lo += per_chunk) {
            PqgChunk c{};
            c.item_lo = lo;
            c.item_hi = std::min(lo + per_chunk, q.item_begin + q.n_items);
            c.problem = static_cast<int32_t>(ip);
            chunks.push_back(c);
        }
        q.n_chunks = static_cast<int64_t>(chunks.size()) - q.chunk_begin;
        total_steps += p.S;
        total_flops += flops[ip];
    }
    item_begin[np] = total_items;
    // the device data follows the uploaded arena: rebase its offsets (an
    // unused one points at the region's start and is never read)
    const int64_t pbase = align_(256);
    for (auto &q : probs) {
        if (q.kind != PQG_KIND_WALK) {
            q.off_base64 = q.off_outer64 = q.off_base_df = q.off_outer_df = q.off_D = pbase;
            continue;
        }
        for (int64_t *o : {&q.off_base64, &q.off_outer64, &q.off_base_df, &q.off_outer_df, &q.off_D})
            *o = *o < 0 ? pbase : pbase + *o;
        if (q.n_outer == 0) {  // never read: the seed is the base
            q.off_outer64 = q.off_base64;
            q.off_outer_df = q.off_base_df;
        }
    }
}

}  // namespace pqg
