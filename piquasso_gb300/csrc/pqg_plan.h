// Work plan shared by the host planner (plan.cpp) and the walk kernels.
//
// A permanent with repeated rows and columns is the signed, binomially weighted
// sum over a mixed-radix Gray code that walks the row multiplicities (the
// BB/FG-Glynn form, Eq. (8) of arXiv:2309.07027, as in the reference's
// src/permanent.cpp:49-264).  The planner splits the Gray-code digits of every
// problem into
//   * inner digits: walked by every lane of a warp in lock step, from the same
//     start, along one precomputed table of (changed row, signed weight) steps;
//   * outer digits: one assignment per lane, decoded from the lane's segment
//     index, seeded from scratch in FP64 at the segment start.
// A work item is one warp: 32 consecutive outer assignments of one problem.
#pragma once
#include <stdint.h>

#define PQG_MAX_COLS 32
#define PQG_MAX_OUTER 60
#define PQG_ITEM_LANES 32

enum PqgProblemKind : int32_t {
    PQG_KIND_WALK = 0,      // Gray-code walk on the device
    PQG_KIND_CONSTANT = 1,  // value known without a walk (empty input: 1)
};

struct PqgProblem {
    int32_t kind;       // PqgProblemKind
    int32_t nc;         // distinct columns with nonzero multiplicity (<= PQG_MAX_COLS)
    int32_t n_outer;    // outer digits
    int32_t P;          // inner walk length = table entries (>= 1)
    int32_t scale_exp;  // sum of multiplicities minus one: result = sum / 2^scale_exp
    int32_t cm_max;     // largest column multiplicity
    int32_t n_out;      // outputs of this problem (1, or nc for the Laplace form)
    int32_t pad0;
    int64_t Q;          // outer assignments (lanes)
    int64_t item_begin; // first work item
    int64_t n_items;    // ceil(Q / 32)
    int64_t off_base;   // byte offset: nc x double2, FP64 column sums with every digit at 0
    int64_t off_outer;  // byte offset: n_outer x nc x double2, FP64 rows of the outer digits
    int64_t off_D;      // byte offset: 2*K x nc complex in kernel precision (K inner digits);
                        //   row 2k = -2 a_k (digit k steps up), row 2k+1 = +2 a_k (steps down)
    int64_t off_tab;    // byte offset: P table entries
    int64_t out_index;  // first output slot of this problem
    int64_t part_begin; // first partial slot (n_out dd-complex slots per item)
    int64_t chunk_begin;// first level-1 reduction chunk
    int64_t n_chunks;   // level-1 chunks of this problem
    double cval_re, cval_im;          // PQG_KIND_CONSTANT value
    uint8_t cm[PQG_MAX_COLS];         // column multiplicities
    uint8_t outer_m[PQG_MAX_OUTER];   // outer digit multiplicities (radix m + 1)
    uint8_t pad1[4];
};

// One inner step, complex128 kernels: add row D[drow .. drow+nc) to the column
// sums, then accumulate w * product.  Entry 0 is the start (drow unused).
struct PqgStep128 {
    double w;
    int32_t drow;  // element offset into the problem's D block
    int32_t pad;
};

// One inner step, complex64 kernels.
struct PqgStep64 {
    float w;
    int32_t drow;
};

// Level-1 reduction chunk: items [item_lo, item_hi) of one problem.
struct PqgChunk {
    int64_t item_lo, item_hi;  // global item indices
    int32_t problem;
    int32_t pad;
};
