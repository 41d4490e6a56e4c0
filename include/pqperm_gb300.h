/*
 * pqperm_gb300 — C ABI of the GB300 permanent engine.
 *
 * Plain pointers and sizes only.  Complex numbers are interleaved (re, im)
 * pairs in row-major order, exactly numpy's complex128 / complex64 layout, so
 * a numpy array's data pointer can be passed as is.  Multiplicities are int32.
 *
 * Every entry point returns a status code (PQG_OK == 0); pqg_last_error()
 * returns a message for the calling thread's last failure.
 *
 * Each entry point replaces one function of the reference (piquasso 8.0.1,
 * paths relative to its repository):
 *   pqg_permanent_c128 / _c64          piquasso/_math/permanent.cpp:26-41,71-78
 *                                      (permanent_np<double>/<float> -> src/permanent.cpp:49-264)
 *   pqg_permanent_laplace_c128 / _c64  piquasso/_math/permanent.cpp:43-58,79-84
 *                                      (permanent_laplace_np -> src/permanent_laplace.cpp:43-240)
 *   pqg_permanent_batch_c128 / _c64    the per-pattern loop over permanent() in
 *                                      piquasso/_simulators/passive/utils.py:131-138 and
 *                                      probabilities.py:26-54 (many output patterns, one matrix)
 */
#ifndef PQPERM_GB300_H
#define PQPERM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define PQG_OK 0
#define PQG_ERR_SUM_MISMATCH 1 /* sum(rows) != sum(cols): src/permanent.cpp:100-104 throws */
#define PQG_ERR_INVALID 2      /* negative multiplicity, null pointer, bad size */
#define PQG_ERR_TOO_LARGE 3    /* > 32 distinct nonzero columns or > 2^50 Gray-code steps */
#define PQG_ERR_CUDA 4         /* a CUDA runtime call failed */
#define PQG_ERR_NO_DEVICE 5    /* no CUDA device visible */
#define PQG_ERR_HOST 6         /* host-side failure, e.g. out of host memory (no C++ exception leaves the library) */

/* precision modes for the complex128 entry points */
#define PQG_MODE_AUTO 0 /* default: PQG_MODE_DF where valid (<= 32 particles) and the plan
                           has more than 2^16 Gray-code steps, else FP64; the environment
                           variable PQG_C128_MODE=fp64 forces FP64 */
#define PQG_MODE_FP64 1 /* column sums, updates and products in FP64; double-double sums */
#define PQG_MODE_DF 2   /* double-float on the FP32 pipes: the column-scaled matrix rounded
                           once to 2^-47 per entry, then exact column sums and seed updates,
                           double-float products (~2^-48 relative each), double-double sums */

/* Host planning: a call with 2048 or more problems is planned on up to 8
 * host threads (the environment variable PQG_HOST_THREADS caps the count; 1
 * plans on the calling thread).  The plan does not depend on the count. */

/* Message describing the calling thread's last failure ("" if none). */
const char *pqg_last_error(void);

/* Library version string. */
const char *pqg_version(void);

/* Number of kernels this library launched since load (all entry points). */
uint64_t pqg_kernel_launches(void);

/* Permanent of an n_rows x n_cols complex128 matrix with row multiplicities
 * `rows` (n_rows) and column multiplicities `cols` (n_cols), as
 * permanent(matrix, rows, cols) in the reference.  `out` receives 2 doubles
 * (re, im).  `out_lo` (nullable) receives the low words of the double-double
 * result (re_lo, im_lo).  Host buffers; the call is synchronous. */
int pqg_permanent_c128(const double *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows,
                       const int32_t *cols, int32_t mode, double *out, double *out_lo);

/* complex64 variant: FP32 row-sum updates and products, FP32 TwoSum-compensated
 * partial sums folded into compensated FP32 lane sums (value and error word),
 * combined across lanes, items and blocks in double-double.  `out` receives 2
 * floats (re, im). */
int pqg_permanent_c64(const float *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows,
                      const int32_t *cols, float *out);

/* Many permanents of ONE matrix: problem b uses rows[b*n_rows ...] and
 * cols[b*n_cols ...].  `out` receives 2*batch values.  One work queue, one
 * walk launch and one reduction for the whole batch. */
int pqg_permanent_batch_c128(const double *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows,
                             const int32_t *cols, int64_t batch, int32_t mode, double *out);
int pqg_permanent_batch_c64(const float *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows,
                            const int32_t *cols, int64_t batch, float *out);

/* Laplace-expansion permanents: for every column l, the permanent with
 * cols[l] lowered by one (reference semantics, including a column with
 * multiplicity 0 contributing exponent 0).  `out` must hold 2*max(n_cols,1)
 * values; *n_out receives the count written (1 for the empty case, whose value
 * is 1, as src/permanent_laplace.cpp:52-57). */
int pqg_permanent_laplace_c128(const double *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows,
                               const int32_t *cols, double *out, int64_t *n_out);
int pqg_permanent_laplace_c64(const float *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows,
                              const int32_t *cols, float *out, int64_t *n_out);

/* Batched Laplace permanents of one matrix, one walk launch for the batch:
 * problem b uses rows[b*n_rows ...] and cols[b*n_cols ...] and writes
 * 2*max(n_cols,1) values at out + 2*max(n_cols,1)*b; n_out (nullable, batch
 * entries) receives each problem's count (1 for an empty problem, whose single
 * value is 1).  Replaces the per-step permanent_laplace calls of the
 * reference's sampler (piquasso/_simulators/passive/sampling.py:723-749),
 * batched over independent shots. */
int pqg_permanent_laplace_batch_c128(const double *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows,
                                     const int32_t *cols, int64_t batch, double *out, int64_t *n_out);
int pqg_permanent_laplace_batch_c64(const float *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows,
                                    const int32_t *cols, int64_t batch, float *out, int64_t *n_out);

/* One step of the batched exact boson sampler (Clifford & Clifford algorithm
 * B), fused on the device: for every shot b, the Laplace permanents L of
 * (rows[b*n_rows ...] = the output photons drawn so far, cols[b*n_cols ...] =
 * the input photons placed so far), then the pmf over the n_rows output modes
 * p_i = |sum_j cols_j L_j U[i, j]|^2 and the inverse-CDF draw
 * modes[b] = min(#{i : cdf_i < uniforms[b] * cdf_last}, n_rows - 1).
 * Replaces one iteration of the reference's sampling loop
 * (piquasso/_simulators/passive/sampling.py:723-749: permanent_laplace, the
 * pmf and the draw), batched over shots; the Laplace values stay on the device
 * and only the drawn modes are copied back.  Every shot needs at least one
 * output and one input photon (PQG_ERR_INVALID otherwise: the first step of a
 * shot, with no output photon, has pmf |U[i, j]|^2 and needs no permanent). */
int pqg_sampler_step_c128(const double *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows,
                          const int32_t *cols, int64_t batch, const double *uniforms, int32_t *modes);
int pqg_sampler_step_c64(const float *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows,
                         const int32_t *cols, int64_t batch, const double *uniforms, int32_t *modes);

/* Gradient of the permanent with respect to every matrix entry.
 * Replaces grad_perm (src/permanent.cpp:271-300 of the reference), reached
 * through the JAX FFI backward target PermBwd (src/jax_perm/jax_perm_core.cpp:
 * 139-208), whose batch loop over leading matrix dimensions this mirrors.
 * `matrices` holds `batch` row-major n_rows x n_cols interleaved complex
 * matrices; rows (batch x n_rows) and cols (batch x n_cols) their
 * multiplicities.  out[b][i][j] (interleaved complex, batch x n_rows x n_cols)
 * = rows_i cols_j perm(A_b; rows - e_i, cols - e_j), 0 where rows_i or cols_j
 * is 0.  PQG_ERR_SUM_MISMATCH when sum(rows) != sum(cols) and some entry has
 * rows_i > 0 and cols_j > 0 (where the reference's first minor throws).  The
 * reference returns an n_rows x n_rows array; this returns n_rows x n_cols,
 * the same for the square matrices it supports.  Computed as one batched
 * Laplace walk per row of nonzero multiplicity (FP64 walk for complex128,
 * FP32 for complex64). */
int pqg_permanent_grad_c128(const double *matrices, int64_t n_rows, int64_t n_cols, const int32_t *rows,
                            const int32_t *cols, int64_t batch, double *out);
int pqg_permanent_grad_c64(const float *matrices, int64_t n_rows, int64_t n_cols, const int32_t *rows,
                           const int32_t *cols, int64_t batch, float *out);

/* Exact binomial moments of ideal boson sampling on n_sets sets of k output
 * modes each (modes: n_sets x k indices), the generating-function dynamic
 * program of the reference's marginal probabilities
 * (piquasso/_simulators/passive/marginal.py:163-216, get_binomial_moments),
 * for every set in the same launches.  U: host d x d interleaved complex128
 * interferometer; input: d photon numbers (n = their sum <= 64).  moments
 * (host): n_sets x (n+1)^k doubles, b[alpha] = E[prod_j C(X_j, alpha_j)]
 * row-major over alpha (first mode slowest), 0 where |alpha| > n.  The
 * marginal probabilities follow by the binomial transform.
 * max_device_bytes > 0 refuses (PQG_ERR_TOO_LARGE) a call whose blocks
 * would need more device memory; the call allocates and frees its own. */
int pqg_binomial_moments_c128(const double *U, int64_t d, const int32_t *input, const int32_t *modes, int32_t k,
                              int32_t n_sets, double *moments, int64_t max_device_bytes);

/* Plan handles: plan and upload a batch once, then execute it many times as
 * one CUDA graph (queue reset, persistent walk, reductions) on the handle's
 * own stream — the form used for repeated batches (exact probabilities of a
 * fixed set of output patterns, benchmark loops).  `dtype`: 0 complex128, 1
 * complex64; `form`: 0 plain permanents (2 values per problem), 1 Laplace
 * permanents (2*max(n_cols,1) values per problem, laid out as
 * pqg_permanent_laplace_batch_*); `mode` as for the complex128 entry points.
 * pqg_plan_launch enqueues one execution and returns; pqg_plan_synchronize
 * waits for it and reports its device time; pqg_plan_read copies the results
 * of the last completed execution to host memory.  A handle is used by one
 * thread at a time. */
typedef struct pqg_plan_s pqg_plan_t;
int pqg_plan_create(const void *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows, const int32_t *cols,
                    int64_t batch, int32_t dtype, int32_t form, int32_t mode, pqg_plan_t **out_plan);
int pqg_plan_launch(pqg_plan_t *plan);
int pqg_plan_synchronize(pqg_plan_t *plan, double *device_ms);
int pqg_plan_read(pqg_plan_t *plan, void *out, int64_t *n_values);
int pqg_plan_info(pqg_plan_t *plan, double *steps, double *flops, int64_t *work_items, int64_t *h2d_bytes);
int pqg_plan_destroy(pqg_plan_t *plan);

/* Work-split knobs of the planner (process-wide; 0 restores a default):
 * items_per_smsp — warps of work per SM sub-partition the split aims for
 * (default 16); p_max — longest inner walk, i.e. step-table length (default
 * 2048, at most 32768); seed_steps — Gray-code steps per lane that amortise
 * one seed (default depends on the arithmetic).  The reference fixes its
 * split at 4 x hardware_concurrency contiguous segments
 * (src/permanent.cpp:144-155); these knobs replace it.  A knob set here
 * (nonzero) overrides the autotuned table below for every workload; the
 * autotuner (piquasso_gb300.autotune) sets them while it times candidates.
 * pqg_set_blocks_per_sm caps the walk's resident blocks per SM the same way
 * (0: as many as fit, or the autotuned value). */
int pqg_set_tuning(int64_t items_per_smsp, int64_t p_max, int64_t seed_steps);
int pqg_get_tuning(int64_t *items_per_smsp, int64_t *p_max, int64_t *seed_steps);
int pqg_set_blocks_per_sm(int32_t blocks);

/* Autotuned settings (no counterpart in the reference).  Each entry gives the
 * planner knobs (0: keep the default) for the workloads of one form (0 plain,
 * 1 Laplace) and arithmetic (0 FP64, 1 double-float, 2 complex64) whose
 * largest column count lies in [nc_lo, nc_hi], total Gray-code steps in
 * [steps_lo, steps_hi) and walk problems in [probs_lo, probs_hi].  Every
 * call's planner takes the first matching entry for each knob that
 * pqg_set_tuning leaves at 0.  The Python package fills this table at load
 * time from the tuning cache that piquasso_gb300.autotune writes (a JSON file
 * keyed by GPU name and library version); C callers add entries themselves.
 * pqg_plan_config reports the knobs a plan handle was planned with. */
int pqg_tuning_add(int32_t form, int32_t arith, int32_t nc_lo, int32_t nc_hi, double steps_lo, double steps_hi,
                   int64_t probs_lo, int64_t probs_hi, int64_t items_per_smsp, int64_t p_max, int64_t seed_steps,
                   int32_t blocks_per_sm);
int pqg_tuning_clear(void);
int pqg_tuning_count(int64_t *count);
int pqg_plan_config(pqg_plan_t *plan, int64_t *items_per_smsp, int64_t *p_max, int64_t *seed_steps,
                    int32_t *blocks_per_sm);

/* Name (NUL-terminated, at most name_len bytes with the NUL) and SM count of
 * the device the engine runs on. */
int pqg_device_info(char *name, int64_t name_len, int32_t *num_sms);

/* Measured FP64 / FP32 fused-multiply-add throughput of device 0 in TFLOP/s
 * (2 flops per FMA), from dependent-chain microkernels run over all SMs for
 * about `ms` milliseconds each.  out2 = {fp64_tflops, fp32_tflops}. */
int pqg_measure_vector_peaks(double ms, double *out2);

/* Timing of the calling thread's last plain/Laplace/batch call, measured with
 * CUDA events on the launching stream: `walk_ms` is the walk kernel alone,
 * `device_ms` the whole device pipeline (the prep kernel that builds the
 * problems' seeds, rows and prefix tables, queue reset, walk, both reductions;
 * excluding the host<->device copies).  `steps` is the number of Gray-code
 * steps walked, `flops` the algorithmic flop count of the call, and
 * `h2d_bytes` / `d2h_bytes` the bytes the call copied each way.  Any pointer
 * may be null. */
int pqg_last_timing(double *walk_ms, double *device_ms, double *steps, double *flops, double *h2d_bytes,
                    double *d2h_bytes);

/* Walk kernel of the calling thread's last plain/Laplace/batch/sampler call
 * (no counterpart in the reference, whose CPU loop has one form): `table`
 * receives one of PQG_WALK_* (-1 when the call needed no walk) and `n_cols`
 * the exact column count of the instantiation (1..32).  Every (table, column
 * count) pair is a separately compiled kernel; tests use this to show that
 * each one has run against the oracle.  Either pointer may be null. */
#define PQG_WALK_PLAIN_FP64 0        /* FP64 walk, repeated columns */
#define PQG_WALK_PLAIN_C64 1         /* complex64 walk, repeated columns */
#define PQG_WALK_LAPLACE_FP64 2      /* FP64 Laplace walk */
#define PQG_WALK_LAPLACE_C64 3       /* complex64 Laplace walk, repeated columns */
#define PQG_WALK_PLAIN_DF 4          /* double-float walk, repeated columns */
#define PQG_WALK_LAPLACE_C64_UNIT 5  /* complex64 Laplace walk, unit columns (<= 24; two codes per iteration) */
#define PQG_WALK_PLAIN_FP64_UNIT 6   /* FP64 walk, unit columns */
#define PQG_WALK_PLAIN_C64_UNIT 7    /* complex64 walk, unit columns */
#define PQG_WALK_PLAIN_DF_UNIT 8     /* double-float walk, unit columns */
#define PQG_WALK_LAPLACE_DF_UNIT 9   /* double-float Laplace walk, unit columns (<= 25) */
#define PQG_WALK_LAPLACE_DF 10       /* double-float Laplace walk, any columns */
int pqg_last_walk_kernel(int32_t *table, int32_t *n_cols);

/* Learned proposal (no counterpart in the reference): kernels of the
 * autoregressive MLP over output occupations used as the independence
 * proposal of the Metropolis boson sampler.  All pointers are DEVICE pointers;
 * `stream` is a cudaStream_t (NULL: legacy default stream); the calls enqueue
 * and return.
 *
 * pqg_mlp_gemm_tc: C[M x N] = A[M x K] . B[N x K]^T with BF16 operands, both
 * row-major with K contiguous (row strides lda, ldb >= K, multiples of 8;
 * 16-byte aligned base pointers), FP32 accumulation on the tcgen05 tensor
 * cores (TMA-staged operands, TMEM accumulator).  With N <= 256, K <= 256,
 * no split-K and at least two 128-row tiles per SM, a persistent kernel runs
 * instead (one CTA per SM, B resident in shared memory, two TMEM
 * accumulators); its results are bit-identical.  epilogue 0: C = acc; 1: C =
 * acc + bias (pre-activation), c_bf16 = GELU(C); 2: split-K over `splits`
 * ranges of K through `splitk_scratch` (splits*M*N floats), then a fixed-order
 * sum into C (weight gradients); 3: C = acc + bias; 4: C = acc * GELU'(pre)
 * (pre: M x N FP32), c_bf16 = BF16(C) (backward through the activation).
 * pqg_mlp_transpose_bf16: dst[c*ld_dst + r] = src[r*ld_src + c] (rows x cols
 * BF16), the K-major copies of backward operands.  pqg_mlp_tc_status: reads
 * (and clears) the GEMM's device error code: 0, or the bounded wait that ran
 * out (1: operand copy, 2: stage release, 3: accumulator); synchronising.
 * pqg_mlp_bias_grad: db = column sums of d (M x N), deterministic, through
 * `scratch` (ceil(M/256) * N floats).  pqg_mlp_softmax_xent:
 * per row m, softmax over classes lo[m]..hi[m] of logits (row stride ld),
 * loss = -log p(target), dlogits = (p - onehot) * scale (FP32, and BF16 when
 * dlogits_bf16 is not NULL).  pqg_mlp_adam: one Adam step on FP32 weights
 * (and their BF16 copy, nullable), bias-corrected with `step`.
 * pqg_mlp_adam_multi: the same step on `count` (1..16) row-major tensors of
 * rows[i] x cols[i] in one launch, with per tensor an optional BF16 copy
 * (w_bf16 NULL or w_bf16[i] NULL: none) and an optional transposed BF16 copy
 * (cols x rows); the arrays are host arrays of device pointers.  The FP32
 * results equal pqg_mlp_adam's bit for bit. */
int pqg_mlp_gemm_tc(const void *a, int64_t lda, const void *b, int64_t ldb, int64_t M, int64_t N, int64_t K,
                    int32_t epilogue, float *c, void *c_bf16, const float *bias, const float *pre,
                    float *splitk_scratch, int32_t splits, void *stream);
/* pqg_mlp_gemm_tc_t: pqg_mlp_gemm_tc with a BF16 epilogue (1 or 4) that also
 * writes the BF16 output transposed, c_bf16_t = c_bf16^T (N x M, row stride
 * ld_t >= M, a multiple of 8): the K-major operand of a weight gradient over
 * the rows; and, when col_sums is not NULL, the column sums of the FP32 output
 * c (the next layer's bias gradient) through col_scratch (4 ceil(M/128) N
 * floats), deterministic.  The persistent kernel writes both from its
 * epilogue; other shapes run the transpose and the bias-gradient kernels
 * after the GEMM.  The same bits of c, c_bf16 and c_bf16_t either way. */
int pqg_mlp_gemm_tc_t(const void *a, int64_t lda, const void *b, int64_t ldb, int64_t M, int64_t N, int64_t K,
                      int32_t epilogue, float *c, void *c_bf16, const float *bias, const float *pre, void *c_bf16_t,
                      int64_t ld_t, float *col_sums, float *col_scratch, void *stream);
int pqg_mlp_transpose_bf16(const void *src, int64_t rows, int64_t cols, int64_t ld_src, void *dst, int64_t ld_dst,
                           void *stream);
int pqg_mlp_tc_status(int32_t *code);
int pqg_mlp_bias_grad(const float *d, int64_t M, int64_t N, float *db, float *scratch, void *stream);
int pqg_mlp_softmax_xent(const float *logits, int64_t M, int32_t ld, int32_t classes, const int8_t *lo,
                         const int8_t *hi, const int8_t *target, float scale, float *loss, float *dlogits,
                         void *dlogits_bf16, void *stream);
int pqg_mlp_adam(float *w, void *w_bf16, const float *g, float *m1, float *m2, int64_t n, float lr, float b1,
                 float b2, float eps, int64_t step, void *stream);
int pqg_mlp_adam_multi(int32_t count, float *const *w, void *const *w_bf16, void *const *w_bf16_t,
                       const float *const *g, float *const *m1, float *const *m2, const int64_t *rows,
                       const int64_t *cols, float lr, float b1, float b2, float eps, int64_t step, void *stream);

/* Autoregressive proposal step for B chains at output mode j (d modes, n
 * photons): pqg_proposal_features writes the 16 BF16 features of mode j and
 * the feasible occupation range [lo, hi]; pqg_proposal_sample draws mode j's
 * occupation from the masked softmax of `logits` (row stride 8) with a
 * counter-based generator (seed, chain, j) — the seed read from device memory
 * at seed_dev when that is not null (so a captured CUDA graph of the whole
 * draw can be replayed with new seeds) — adds its log-probability to logq,
 * and updates samples, n_rem and the mean shifts of the later modes (C: d x d
 * mode covariances; mode_stats: 12 floats per mode: p(0..4), Pr(X >= 5), mean,
 * variance, suffix sum of the means, 3 pad).  Occupations 0..7. */
int pqg_proposal_features(int32_t j, int32_t B, int32_t d, int32_t n, const float *mode_stats, const int32_t *n_rem,
                          const float *shift, void *X_bf16, int8_t *lo, int8_t *hi, void *stream);
int pqg_proposal_sample(int32_t j, int32_t B, int32_t d, const float *logits, const int8_t *lo, const int8_t *hi,
                        uint64_t seed, const uint64_t *seed_dev, int8_t *samples, int32_t *n_rem, float *shift,
                        const float *C, const float *mode_stats, float *logq, void *stream);

/* The whole proposal step for mode j fused into one tensor-core kernel:
 * pqg_proposal_features, the four-layer MLP (W1^T 256x16, W2^T and W3^T
 * 256x256, W4^T 8x256: BF16, K-major; FP32 biases b1..b4; bias + GELU after
 * the hidden layers) and pqg_proposal_sample, with the same roundings, per
 * tile of 128 chains (TMA-streamed weights, TMEM accumulators, activations in
 * shared memory).  The same chain state and seed arguments as the separate
 * calls. */
int pqg_proposal_step_tc(int32_t j, int32_t B, int32_t d, int32_t n, const float *mode_stats, const void *w1t,
                         const void *w2t, const void *w3t, const void *w4t, const float *b1, const float *b2,
                         const float *b3, const float *b4, uint64_t seed, const uint64_t *seed_dev, int8_t *samples,
                         int32_t *n_rem, float *shift, const float *C, float *logq, void *stream);

/* Allocation-free permanent — no counterpart in the reference.
 *
 * For callers that cannot allocate device memory: applications whose own
 * allocator has already reserved the GPU, latency-critical code that cannot
 * afford an allocation's implicit synchronisation, code running while its
 * stream is being recorded.  Computes the permanent of an n x n complex128
 * matrix with every row and column taken once (rows = cols = 1) from DEVICE
 * pointers: `d_matrix` (n*n interleaved re/im, row-major) and `d_out` (2
 * doubles), enqueued on `stream` (a cudaStream_t; NULL is the legacy default
 * stream) and returning without waiting.  The FP64 walk is used.
 *
 * It allocates no device memory: all intermediate data lives in one
 * file-scope device array of PQG_NOALLOC_SCRATCH_BYTES, held by every GPU that
 * loads the library until the process exits.  With CUDA's lazy module loading
 * (the default) the array comes into being when the library's device code is
 * first loaded on a device, at the latest in the first call of this entry
 * point there: that first call looks the array's address up
 * (cudaGetSymbolAddress) with the device current, and it is the one call that
 * can need device memory.  Make it before your own allocator reserves the
 * device, and before any stream capture; later calls allocate nothing.  Every
 * call on a device shares
 * the array, so calls whose executions overlap on the GPU (different streams,
 * or threads) race and give wrong results: order them on one stream.
 * n must be between 1 and PQG_NOALLOC_MAX_N; larger sizes are rejected with
 * PQG_ERR_TOO_LARGE. */
#define PQG_NOALLOC_MAX_N 32
#define PQG_NOALLOC_SCRATCH_BYTES (4u << 20)
int pqg_permanent_unit_c128_noalloc(const double *d_matrix, int64_t n, double *d_out, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* PQPERM_GB300_H */
