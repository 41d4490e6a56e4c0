// Work plan shared by the host planner (plan.cpp) and the walk kernels.
//
// A permanent with repeated rows and columns is the signed, binomially weighted
// sum over a mixed-radix Gray code that walks the row multiplicities (the
// BB/FG-Glynn form, Eq. (8) of arXiv:2309.07027, as in the reference's
// src/permanent.cpp:49-264).  The planner splits the Gray-code digits of every
// problem into
//   * K inner digits, whose reflected Gray code (P codes) all lanes of a warp
//     walk in lock step, forward from code 0 or backward from code P-1.  The
//     column sums at inner code t are seed + Delta(t), with the prefix table
//     Delta(t) = sum_k -2 g_k(t) a_k built once per problem on the device, so
//     a step is one addition per column and rounding errors never accumulate;
//   * outer digits: each lane owns R consecutive positions of the reflected
//     mixed-radix Gray code over the outer digits.  It seeds its column sums
//     from scratch at its first position, walks the inner codes, then moves to
//     the next outer position with a one-digit update of the seed and walks
//     the inner codes in the other direction, R times.
// A work item is one warp: 32 lanes x R outer positions of one problem.
#pragma once
#include <stdint.h>

#define PQG_MAX_COLS 32
#define PQG_MAX_OUTER 60
#define PQG_MAX_INNER 16
#define PQG_ITEM_LANES 32
// Level-1 reduction chunk: items per chunk = threads of its block.  Small
// chunks spread the double-double sums over every SM (the FP64 pipe of an SM
// completes about two lanes per clock).
#define PQG_CHUNK_ITEMS 64
#define PQG_ITEM_GROUP 4  // items (warps) a block of the complex64 plain walk takes at once
// complex64 plain walks of these column counts read the prefix table from
// shared memory, which holds at most PQG_SMEM_TABLE_P codes
#define PQG_SMEM_TABLE_NC_MIN 17
#define PQG_SMEM_TABLE_NC_MAX 24
#define PQG_SMEM_TABLE_P 256
// complex64 Laplace walks of unit columns up to this count take two inner
// codes per iteration, from prefix tables stored as code pairs
#define PQG_PAIRS_MAX_NC 24
// ... whose block stages the problem's table of at most this many codes in
// shared memory (a block takes PQG_ITEM_GROUP items of one problem)
#define PQG_PAIRS_TABLE_P 128

enum PqgProblemKind : int32_t {
    PQG_KIND_WALK = 0,      // Gray-code walk on the device
    PQG_KIND_CONSTANT = 1,  // value known without a walk (empty input: 1)
};

struct PqgProblem {
    int32_t kind;       // PqgProblemKind
    int32_t nc;         // columns (nonzero multiplicity, padded to the plan's count)
    int32_t n_outer;    // outer digits
    int32_t P;          // inner codes = table entries (>= 1)
    int32_t K;          // inner digits
    int32_t scale_exp;  // result = sum / 2^(scale_exp - col_shift); scale_exp = sum of multiplicities - 1
    int32_t cm_max;     // largest column multiplicity
    int32_t n_out;      // outputs of this problem (1, or the Laplace count)
    int32_t col_shift;  // sum_j e_j cm_j of the double-float column scales 2^-e_j (device-written)
    int32_t index;      // the caller's problem index (problems are laid out in work order)
    int64_t Q;          // outer positions
    int64_t R;          // outer positions per lane
    int64_t item_begin; // first work item
    int64_t n_items;    // ceil(Q / (32 R))
    // Byte offsets into the arena.  Uploaded by the host:
    int64_t off_idx;      //   int32 [row0, matrix row of each outer digit, of each inner
                          //   digit, matrix column of each column (-1: neutral padding)]
    int64_t off_tab;      //   P x PqgStep
    // Built on the device from the matrix (prep.cuh); FP64 walks read the
    // *64 seeds, FP32-pipe walks the *_df ones:
    int64_t off_base64;   //   nc x double2, column sums with every digit 0
    int64_t off_outer64;  //   n_outer x nc x double2, rows a_o of the outer digits
    int64_t off_base_df;  //   nc x float4 {re_hi, re_lo, im_hi, im_lo}, the same column sums
    int64_t off_outer_df; //   n_outer x nc x float4, the same rows
    int64_t off_D;        //   2 n_outer x nc elements in kernel precision: row 2o = -2 a_o
                          //   (outer digit o steps up), row 2o+1 = +2 a_o (steps down)
    int64_t delta_begin;  // first element of this problem's P x nc prefix table (delta buffer)
    int64_t out_index;  // first output slot of this problem
    int64_t part_begin; // first partial slot (n_out dd-complex slots per item)
    int64_t chunk_begin;// first level-1 reduction chunk
    int64_t n_chunks;   // level-1 chunks of this problem
    double cval_re, cval_im;          // PQG_KIND_CONSTANT value
    uint8_t cm[PQG_MAX_COLS];         // column multiplicities
    uint8_t outer_m[PQG_MAX_OUTER];   // outer digit multiplicities (radix m + 1)
    uint8_t inner_m[PQG_MAX_INNER];   // inner digit multiplicities
    int32_t laplace;                  // Laplace form: output k < nc lacks one factor of column k
    int16_t col_e[PQG_MAX_COLS];      // column scale exponents e_j (device-written; 0 unless double-float)
};

// Inner code t: its signed binomial weight (-1)^sum(g) prod C(m, g), in FP64
// and FP32.
struct PqgStep {
    double wd;
    float wf;
    float pad;
};

// Level-1 reduction chunk: items [item_lo, item_hi) of one problem (at most PQG_CHUNK_ITEMS).
struct PqgChunk {
    int64_t item_lo, item_hi;  // global item indices
    int32_t problem;
    int32_t pad;
};
