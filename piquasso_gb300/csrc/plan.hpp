// Host-side planner: turns (matrix, row multiplicities, column multiplicities)
// problems into the device work plan described in pqg_plan.h.
//
// The planner only decides: the row reduction, which matrix rows and columns
// take part, the inner/outer split of the Gray-code digits, the per-problem
// data layout and the work items.  It copies no matrix data per problem: the
// plan carries the matrix once, and a device kernel (prep.cuh) builds every
// problem's seeds, step rows and prefix tables in device memory.
#pragma once
#include <functional>
#include <map>
#include <utility>
#include <string>
#include <vector>

#include "pqg_plan.h"

namespace pqg {

// C128: FP64 walk.  C64: FP32 walk.  C128DF: complex128 accuracy from
// double-float (FP32 pair) updates and products, FP64 seeds and sums.
enum class Precision { C128, C64, C128DF };
enum class Form { PLAIN, LAPLACE };

struct PlanConfig {
    int num_sms = 152;
    int64_t items_per_smsp = 0;   // work items per SM sub-partition the split aims for (0: per arithmetic)
    int64_t p_max = 2048;         // longest inner walk (table length)
    bool p_max_user = false;      // p_max was set explicitly (overrides the per-arithmetic cap)
    int64_t seed_steps = 0;       // steps per lane that amortise a seed; 0: per-precision default
    int blocks_per_sm = 0;        // walk blocks per SM; 0: as many as fit (occupancy)
};

// One reduced problem before its inner/outer split is fixed.  Fixed-size
// (no heap storage): a batch of thousands of problems is planned without
// per-problem allocations.
struct PendingProblem {
    int kind = PQG_KIND_WALK;
    double cre = 1.0, cim = 0.0;
    int nc = 0;                   // kept columns (padded to the plan's count by finish())
    int nd = 0;                   // digits (rows of nonzero multiplicity after the reduction)
    int row0 = 0;                 // matrix row of the prepended copy (multiplicity 1)
    int scale_exp = 0;
    int n_out = 1;
    int padded_cols = 0;          // neutral columns added to reach the plan's column count
    bool laplace_full = false;    // Laplace form with a zero-multiplicity column (shared output nc)
    double S = 1.0;               // Gray-code space size
    uint8_t cm[PQG_MAX_COLS];     // multiplicities of the kept columns
    int32_t col[PQG_MAX_COLS];    // matrix column of each kept column, ascending (-1: padding)
    uint8_t m[PQG_MAX_OUTER];     // digit multiplicities (>= 1)
    int32_t row[PQG_MAX_OUTER];   // matrix row of each digit
};

// Laplace outputs of a problem in the caller's column layout: original column
// j of the matrix (0 <= j < n_cols) reads output slot slot[j]: k for the k-th
// kept column, the shared zero-multiplicity slot nc otherwise
// (src/permanent_laplace.cpp:180,210 keeps those columns' exponent at 0).
void laplace_slots(const PendingProblem &p, int64_t n_cols, int *slot);

class Planner {
  public:
    // The large buffers (pending, probs, arena and finish()'s index rows)
    // come from a per-thread pool and go back to it on destruction, so that
    // repeated calls write into memory already mapped instead of faulting in
    // fresh pages (about half of the planning time of a 4096-problem batch).
    Planner(Precision prec, Form form, const PlanConfig &cfg);
    ~Planner();
    Planner(const Planner &) = delete;
    Planner &operator=(const Planner &) = delete;

    // The matrix every problem of this plan indexes: interleaved complex128,
    // row-major n_rows x n_cols (the complex64 entry points widen first).
    void set_matrix(const double *a, int64_t nr, int64_t nc);

    // Adds one problem over the plan's matrix.  Returns PQG_OK or an error
    // status with `err` set.  `rows` has one multiplicity per matrix row; or,
    // with n_rows_local >= 0, one per row of the n_rows_local-row block that
    // starts at matrix row row_base (problems over a stack of matrices).
    int add(const int32_t *rows, const int32_t *cols, std::string &err, int64_t row_base = 0,
            int64_t n_rows_local = -1);

    // Adds `batch` problems (rows: batch x n_rows, cols: batch x n_cols), on
    // several host threads for large batches; the same problems as `batch`
    // calls of add().  On failure *err_index receives the first failing
    // problem and nothing is added.
    int add_batch(const int32_t *rows, const int32_t *cols, int64_t batch, std::string &err, int64_t *err_index);

    // Fixes every problem's split and lays out the arena and the per-problem
    // device data.
    void finish();

    void set_config(const PlanConfig &cfg) { cfg_ = cfg; }
    const PlanConfig &config() const { return cfg_; }

    std::vector<PendingProblem> pending;
    std::vector<PqgProblem> probs;     // in work order (PqgProblem::index: the pending problem)
    std::vector<int64_t> out_of;       // first output slot of pending problem b (caller's order)
    std::vector<int64_t> item_begin;   // n_probs + 1
    std::vector<PqgChunk> chunks;
    std::vector<unsigned char> arena;  // weight tables and the matrix, by byte offset
    int64_t total_items = 0;
    int64_t total_parts = 0;           // dd-complex partial slots
    int64_t total_outputs = 0;
    int64_t total_delta = 0;           // prefix-table entries (delta buffer elements)
    int64_t pdata_bytes = 0;           // per-problem device data built by the prep kernel
    int64_t matrix_off = 0;            // byte offset of the matrix in the arena
    int64_t mat_rows = 0, mat_cols = 0;
    int max_nc = 0;
    int item_group = 1;                // items a walk block takes at once (total_items is a multiple)
    bool all_ones = true;              // every walk problem's columns have multiplicity 1
    bool pairs = false;                // complex64 Laplace, unit columns, <= PQG_PAIRS_MAX_NC columns:
                                       // prefix tables stored as code pairs (an even count per problem)
    double total_steps = 0.0;          // sum over problems of the Gray-code space
    double total_flops = 0.0;          // algorithmic flop count, see algorithmic_flops()

    Precision precision() const { return prec_; }
    void set_precision(Precision p) { prec_ = p; }
    Form form() const { return form_; }
    // C128DF plans only: false when some problem falls outside the double-float
    // kernel's validity domain (more than 32 particles, or an inner weight that
    // is not exact in FP32); the caller then plans in C128 instead.
    bool df_ok = true;

  private:
    Precision prec_;
    Form form_;
    PlanConfig cfg_;
    std::map<std::pair<uint64_t, uint64_t>, int64_t> table_cache_;  // packed inner multiplicities -> table
    bool df_ok_add_ = true;
    const double *a_ = nullptr;
    int64_t int_nr_ = 0, int_nc_ = 0;
    std::vector<int32_t> idx_rows_;  // finish(): index rows before they are packed into the arena
    int make_pending_(PendingProblem &p, const int32_t *rows, const int32_t *cols, std::string &err, int64_t row_base,
                      int64_t n_rows_local, bool &df_domain) const;
    int64_t align_(size_t a);
    int64_t push_bytes_(const void *p, size_t n);
};

// Algorithmic flops of one problem: S * (4*c + 6*sum(cols) + 4) for the plain
// permanent (c column-sum updates of 4 flops, one complex multiply of 6 flops
// per factor, 4 flops for the weighted accumulation).
double algorithmic_flops(const PendingProblem &p, Form form);

// Host threads the planner uses for n problems (1 below a few thousand), and
// a parallel loop over contiguous ranges [lo, hi) of 0..n (worker w).
int host_threads(int64_t n);
void parallel_ranges(int64_t n, int nt, const std::function<void(int, int64_t, int64_t)> &fn);

}  // namespace pqg
