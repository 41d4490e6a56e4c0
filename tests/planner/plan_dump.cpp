// Test program for the host planner (compiled with g++ by tests/test_planner_cpu.py;
// no CUDA): reads problems from stdin, plans them, prints the plan as JSON.
//
// The problems go through Planner::add_batch, which plans on several host
// threads from 2048 problems on (PQG_HOST_THREADS caps the count).
//
// stdin: prec form nr nc batch, then the matrix is all zeros except entry
// (0,0) = 1 (the planner copies it and never reads values), then batch lines
// of nr row multiplicities followed by nc column multiplicities.
// prec: 0 = C128, 1 = C64, 2 = C128DF; form: 0 = plain, 1 = Laplace.
#include <cstdint>
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "plan.hpp"

using namespace pqg;

int main() {
    int prec_i, form_i;
    long long nr, nc, batch;
    if (scanf("%d %d %lld %lld %lld", &prec_i, &form_i, &nr, &nc, &batch) != 5) return 2;
    const Precision prec = prec_i == 0 ? Precision::C128 : (prec_i == 1 ? Precision::C64 : Precision::C128DF);
    const Form form = form_i ? Form::LAPLACE : Form::PLAIN;
    std::vector<double> a(static_cast<size_t>(2 * nr * nc), 0.0);
    if (!a.empty()) a[0] = 1.0;
    std::vector<int32_t> rows(static_cast<size_t>(batch * nr)), cols(static_cast<size_t>(batch * nc));
    for (long long b = 0; b < batch; ++b) {
        for (long long i = 0; i < nr; ++i) scanf("%d", &rows[b * nr + i]);
        for (long long j = 0; j < nc; ++j) scanf("%d", &cols[b * nc + j]);
    }
    PlanConfig cfg;
    if (form == Form::LAPLACE) cfg.p_max = 512;
    if (std::getenv("PLAN_DUMP_WARM")) {
        // plan the problems in reverse order first and drop that plan: the
        // plan printed below then reuses its pooled (dirty) buffers
        std::vector<int32_t> rr(rows.size()), cr(cols.size());
        for (long long b = 0; b < batch; ++b) {
            std::copy(rows.begin() + b * nr, rows.begin() + (b + 1) * nr, rr.begin() + (batch - 1 - b) * nr);
            std::copy(cols.begin() + b * nc, cols.begin() + (b + 1) * nc, cr.begin() + (batch - 1 - b) * nc);
        }
        Planner warm(prec, form, cfg);
        warm.set_matrix(a.data(), nr, nc);
        std::string werr;
        int64_t wbad = -1;
        if (warm.add_batch(rr.data(), cr.data(), batch, werr, &wbad) == 0) warm.finish();
    }
    Planner pl(prec, form, cfg);
    pl.set_matrix(a.data(), nr, nc);
    std::string err;
    int64_t bad = -1;
    const int st = pl.add_batch(rows.data(), cols.data(), batch, err, &bad);
    if (st) {
        printf("{\"error\": %d, \"problem\": %lld, \"message\": \"%s\"}\n", st, static_cast<long long>(bad),
               err.c_str());
        return 0;
    }
    pl.finish();
    uint64_t h = 1469598103934665603ull;  // FNV-1a of the arena: tables, row/column indices, matrix
    for (unsigned char byte : pl.arena) h = (h ^ byte) * 1099511628211ull;
    uint64_t hp = 1469598103934665603ull;  // and of the problem records, byte for byte
    const unsigned char *pb = reinterpret_cast<const unsigned char *>(pl.probs.data());
    for (size_t i = 0; i < pl.probs.size() * sizeof(PqgProblem); ++i) hp = (hp ^ pb[i]) * 1099511628211ull;
    printf("{\"total_items\": %lld, \"total_outputs\": %lld, \"item_group\": %d, \"df_ok\": %d, \"all_ones\": %d, "
           "\"pairs\": %d, \"total_delta\": %lld, "
           "\"max_nc\": %d, \"arena_bytes\": %lld, \"arena_hash\": \"%016llx\", \"probs_hash\": \"%016llx\", \"out_of\": [",
           static_cast<long long>(pl.total_items), static_cast<long long>(pl.total_outputs), pl.item_group,
           pl.df_ok ? 1 : 0, pl.all_ones ? 1 : 0, pl.pairs ? 1 : 0, static_cast<long long>(pl.total_delta), pl.max_nc,
           static_cast<long long>(pl.arena.size()), static_cast<unsigned long long>(h),
           static_cast<unsigned long long>(hp));
    for (size_t b = 0; b < pl.out_of.size(); ++b) printf("%s%lld", b ? ", " : "", static_cast<long long>(pl.out_of[b]));
    printf("], \"item_begin\": [");
    for (size_t i = 0; i < pl.item_begin.size(); ++i)
        printf("%s%lld", i ? ", " : "", static_cast<long long>(pl.item_begin[i]));
    printf("], \"probs\": [");
    for (size_t i = 0; i < pl.probs.size(); ++i) {
        const PqgProblem &q = pl.probs[i];
        printf("%s{\"index\": %d, \"kind\": %d, \"n_out\": %d, \"out_index\": %lld, \"item_begin\": %lld, "
               "\"n_items\": %lld, \"P\": %d, \"K\": %d, \"n_outer\": %d, \"Q\": %lld, \"R\": %lld, \"nc\": %d, "
               "\"delta_begin\": %lld, \"S\": %.17g}",
               i ? ", " : "", q.index, q.kind, q.n_out, static_cast<long long>(q.out_index),
               static_cast<long long>(q.item_begin), static_cast<long long>(q.n_items), q.P, q.K, q.n_outer,
               static_cast<long long>(q.Q), static_cast<long long>(q.R), q.nc, static_cast<long long>(q.delta_begin),
               pl.pending[q.index].S);
    }
    printf("]}\n");
    return 0;
}
