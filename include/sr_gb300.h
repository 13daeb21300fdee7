/*
 * sr_gb300.h -- C ABI of the GB300 expression-fitting library (libsr_gb300.so).
 *
 * Plain pointers, sizes and strides only.  Every pointer argument named *_dev is
 * device memory owned by the caller; nothing here allocates device memory except
 * where a function says so.  `stream` is a cudaStream_t passed as void* (NULL =
 * legacy default stream).  Work is enqueued on that stream; functions return after
 * enqueueing, without synchronising.
 *
 * Return values: SR_OK (0) when the work was enqueued, a negative SR_ERR_* for an
 * API-level problem (sr_last_error() gives the text).  Data-dependent errors found
 * by the kernels (the reference's ErrorCode values 101, 102, 201, 204) are written
 * to the caller's device status word, which the caller reads once per call, as
 * the reference reads its error flag with .item().
 *
 * Layouts use the reference's user-facing (batch-first) view:
 *   X (N, n_x) row-major; Ops/C (B, M) addressed through (b, m) strides;
 *   Ch (B, M, 2) through (b, m, child) strides; cache and grad_out (B, M, N)
 *   contiguous; grad_C (B, M) contiguous; Y, Y_final (B, N) contiguous.
 * Staged tapes: desc (B, M) uint32 and meta (B, 4) int32 written by
 * sr_tape_compile (meta = {L_eff, root, n_const_to_root, n_const}).
 */
#ifndef SR_GB300_H
#define SR_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SR_OK 0
#define SR_ERR_INVALID_ARGUMENT (-1)
#define SR_ERR_CUDA (-2)
#define SR_ERR_UNSUPPORTED (-3)
#define SR_ERR_WORKSPACE (-4)

/* Largest tape (M) and variable count the node encoding holds. */
#define SR_MAX_NODES 4095
/* device status of the fit, screening and adjoint kernels: a tape exceeds the table
 * sizes the call was given (max_len, max_consts, max_operators) */
#define SR_TAPE_EXCEEDS_LAUNCH 602
#define SR_MAX_VARS 4095

/* Text of the last API-level error on this host thread ("" if none). */
const char *sr_last_error(void);

/* Library version string. */
const char *sr_version(void);

/*
 * Input validation: child index below the parent's (101) and child count equal to
 * the arity (102).  Replaces validate_inputs_cuda_impl
 * (reference src/evaluation_kernels_cuda.cu:13-49, 675-689) and the validation
 * half of validate_inputs (reference src/symbolic_evaluation.cpp:7-37).
 * status_dev is zeroed and then receives the first error found.
 */
int sr_validate(const int64_t *ops_dev, const int64_t *ch_dev, int64_t B, int64_t M,
                int64_t ops_sb, int64_t ops_sm, int64_t ch_sb, int64_t ch_sm, int64_t ch_si,
                int32_t *status_dev, void *stream);

/*
 * Validation plus staging of the tapes into the compact node encoding used by
 * every kernel here (one pass over Ops/Ch).  desc_dev (B, M) uint32 and
 * meta_dev (B, 4) int32 are outputs.  stats_dev is int32[8], zeroed by the call:
 * stats[0] = status as in sr_validate, stats[1] = largest L_eff, stats[2] = largest
 * root + 1, stats[3] = largest number of constants up to the root, stats[4] =
 * largest number of operator nodes (arity >= 1 or NO_OP) up to the root.
 * Covers the validation of validate_inputs (reference src/symbolic_evaluation.cpp:7-37)
 * and the root/constant-mask bookkeeping of optimize
 * (reference symbolic_torch/optimization.py:51-61).
 */
int sr_tape_compile(const int64_t *ops_dev, const int64_t *ch_dev, int64_t B, int64_t M,
                    int64_t ops_sb, int64_t ops_sm, int64_t ch_sb, int64_t ch_sm, int64_t ch_si,
                    int32_t n_vars, uint32_t *desc_dev, int32_t *meta_dev, int32_t *stats_dev,
                    void *stream);

/*
 * Forward evaluation: cache (B, M, N) of every node at every point; NO_OP nodes
 * and the padding after the last real node are NaN.  Replaces the reference's
 * host loop of M launches of evaluation_forward_step_k
 * (reference src/symbolic_evaluation.cpp:39-92, src/evaluation_kernels_cuda.cu:51-216,
 * 634-652).  One warp interprets one tape, lanes over data points, one grid per
 * class of tape lengths; the NaN padding rows are written by a kernel on a
 * library-owned side stream, forked from `stream` and joined back into it before the
 * call returns (a CUDA graph capture of `stream` records both).
 * max_len: largest meta[0] of the batch (stats[1] of sr_tape_compile), or 0 for M;
 * it sizes the per-warp shared-memory node tables, and a tape whose meta[0] exceeds
 * it is not evaluated: its whole (M, N) block is NaN.  order_dev (B) int32, or NULL:
 * the order in which the persistent warps take the tapes (longest first balances
 * the work).
 */
int sr_eval_forward_f32(const float *X_dev, int64_t N, int64_t n_x, const uint32_t *desc_dev,
                        const int32_t *meta_dev, const int32_t *order_dev, int64_t B, int64_t M,
                        int32_t max_len, const float *C_dev, int64_t c_sb, int64_t c_sm,
                        float *cache_dev, void *stream);
int sr_eval_forward_f64(const double *X_dev, int64_t N, int64_t n_x, const uint32_t *desc_dev,
                        const int32_t *meta_dev, const int32_t *order_dev, int64_t B, int64_t M,
                        int32_t max_len, const double *C_dev, int64_t c_sb, int64_t c_sm,
                        double *cache_dev, void *stream);

/*
 * Adjoint of the forward evaluation for a dense output gradient grad_out (B, M, N).
 * Node values are read from cache_dev, the (B, M, N) output of sr_eval_forward_f32 for
 * the same X, tapes and C, as the reference's backward reads its saved cache; with
 * cache_dev NULL they are recomputed from X and C (the same bits, more instructions).
 * Writes
 * grad_C (B, M) (zero at non-constant nodes) and, when grad_X_dev is not NULL,
 * accumulates into grad_X (N, n_x), which the caller zeroes first.  status_dev
 * is zeroed and then receives 201 (nonzero gradient on a NO_OP node) or 204
 * (a/b with b = 0 and a nonzero gradient; 201 is kept over 204).  Replaces
 * SymbolicEvaluation::backward and evaluation_backward_step_k (reference
 * src/symbolic_evaluation.cpp:94-168, src/evaluation_kernels_cuda.cu:218-632, 654-673).
 * order_dev, max_len and the side stream (here the padding-row check) as for the
 * forward; a tape whose meta[0] exceeds max_len is not adjoined and status_dev
 * receives SR_TAPE_EXCEEDS_LAUNCH (its grad_C row is left as it was).
 */
int sr_eval_backward_f32(const float *X_dev, int64_t N, int64_t n_x, const uint32_t *desc_dev,
                         const int32_t *meta_dev, const int32_t *order_dev, int64_t B, int64_t M,
                         int32_t max_len, const float *C_dev, int64_t c_sb, int64_t c_sm,
                         const float *cache_dev, const float *grad_out_dev, float *grad_C_dev, float *grad_X_dev,
                         int32_t *status_dev, void *stream);
int sr_eval_backward_f64(const double *X_dev, int64_t N, int64_t n_x, const uint32_t *desc_dev,
                         const int32_t *meta_dev, const int32_t *order_dev, int64_t B, int64_t M,
                         int32_t max_len, const double *C_dev, int64_t c_sb, int64_t c_sm,
                         const double *cache_dev, const double *grad_out_dev, double *grad_C_dev, double *grad_X_dev,
                         int32_t *status_dev, void *stream);

/* Options of sr_fit_lbfgs; mirrors optimize()/LBFGS_batch's arguments
 * (reference symbolic_torch/optimization.py:9-19, symbolic_torch/lbfgs_batch.py:15-23). */
typedef struct sr_fit_options {
  int32_t max_iter;             /* 100 */
  int32_t history_size;         /* 10 */
  double tolerance_grad;        /* 1e-7 */
  int32_t line_search;          /* 0 = strong Wolfe, 1 = Armijo backtracking */
  int32_t line_search_max_iter; /* 10 */
  double eps;                   /* 1e-10 */
  int32_t objective;            /* 0 = mean squared error vs Y, 1 = mean of the root value */
  int32_t warps_per_block;      /* warps sharing one problem's points (0 = automatic) */
  int32_t points_per_lane;      /* data points per lane per pass: 1, 2 or 4 (0 = automatic) */
  int32_t grid_blocks;          /* persistent CTAs (0 = one wave over all SMs) */
  int32_t max_operators;        /* largest number of operator nodes (arity >= 1 or NO_OP) up to a
                                   root, stats[4] of sr_tape_compile; sizes the node tables
                                   (0 = max_len) */
  int32_t max_live;             /* largest number of operator-node adjoints live at once in a
                                   reverse sweep, stats[5] after sr_tape_live_rows; sizes the
                                   adjoint tables (0 = max_operators) */
} sr_fit_options;

/* The fit kernel keeps the adjoint of an operator node in a table row only from the
 * moment its first parent is swept until the node itself is: rows are assigned by
 * liveness.  This writes into stats_dev[5] (atomic max) the largest number of rows a
 * tape of the batch needs (exact for tapes of up to 128 nodes to the root, else its
 * operator-node count, a bound), to be passed as sr_fit_options.max_live.  desc_dev
 * and meta_dev as written by sr_tape_compile.  No counterpart in the reference.
 * Returns 0 or an error code. */
int sr_tape_live_rows(const uint32_t *desc_dev, const int32_t *meta_dev, int64_t B, int64_t M, int32_t *stats_dev,
                      void *stream);

/*
 * Evaluation with K constant sets per tape (the reference's
 * evaluate_multiple_constant_backend, src/symbolic_evaluation.cpp:171-305, with the
 * per-position kernels src/evaluation_kernels_cuda.cu:761-1343, here one launch):
 * C (B, M, K) through (b, m, set) strides; cache (B, M, N, K) contiguous, NO_OP rows
 * NaN.  The adjoint takes grad_out (B, M, N, K) contiguous and the forward's cache
 * (B, M, N, K), or NULL to recompute the values, and writes grad_C (B, M, K)
 * contiguous and, if not NULL, adds into grad_X (N, n_x) summed over the sets; status
 * as for sr_eval_backward_f32.
 */
int sr_eval_forward_multi_f32(const float *X_dev, int64_t N, int64_t n_x, const uint32_t *desc_dev,
                              const int32_t *meta_dev, const int32_t *order_dev, int64_t B, int64_t M,
                              int32_t max_len, const float *C_dev, int64_t c_sb, int64_t c_sm, int64_t c_sk,
                              int64_t K, float *cache_dev, void *stream);
int sr_eval_forward_multi_f64(const double *X_dev, int64_t N, int64_t n_x, const uint32_t *desc_dev,
                              const int32_t *meta_dev, const int32_t *order_dev, int64_t B, int64_t M,
                              int32_t max_len, const double *C_dev, int64_t c_sb, int64_t c_sm, int64_t c_sk,
                              int64_t K, double *cache_dev, void *stream);
int sr_eval_backward_multi_f32(const float *X_dev, int64_t N, int64_t n_x, const uint32_t *desc_dev,
                               const int32_t *meta_dev, const int32_t *order_dev, int64_t B, int64_t M,
                               int32_t max_len, const float *C_dev, int64_t c_sb, int64_t c_sm, int64_t c_sk,
                               int64_t K, const float *cache_dev, const float *grad_out_dev, float *grad_C_dev,
                               float *grad_X_dev,
                               int32_t *status_dev, void *stream);
int sr_eval_backward_multi_f64(const double *X_dev, int64_t N, int64_t n_x, const uint32_t *desc_dev,
                               const int32_t *meta_dev, const int32_t *order_dev, int64_t B, int64_t M,
                               int32_t max_len, const double *C_dev, int64_t c_sb, int64_t c_sm, int64_t c_sk,
                               int64_t K, const double *cache_dev, const double *grad_out_dev, double *grad_C_dev,
                               double *grad_X_dev,
                               int32_t *status_dev, void *stream);

/* Bytes of device workspace sr_fit_lbfgs needs for this problem set
 * (B, N, M, max_len, max_consts and opt as passed to sr_fit_lbfgs). */
int64_t sr_fit_workspace_bytes(int64_t B, int64_t N, int64_t M, int32_t max_len, int32_t max_consts,
                               const sr_fit_options *opt);

/* Multi-start screening: the mean squared error (or, with opt->objective = 1, the
 * mean root value) of K candidate constant sets per problem, each measured as the
 * fit's first closure measures the loss, in one launch (the tape is staged once per
 * problem; forward passes only).  Candidate k of problem b is C_sets_dev + k c_sk +
 * b c_sb with slot m at + m c_sm; loss_dev is (B, K) row-major.  The other arguments
 * are sr_fit_lbfgs's; opt's launch-shape fields apply, its iteration fields are
 * ignored.  status_dev is zeroed, then receives SR_TAPE_EXCEEDS_LAUNCH for a
 * tape larger than max_len / max_consts (its losses are NaN).  No counterpart in
 * the reference (its optimize starts from one C).  Returns 0 or an error code. */
int sr_fit_screen(const float *X_dev, int64_t N, int64_t n_x, const float *Y_dev, const uint32_t *desc_dev,
                  const int32_t *meta_dev, int64_t B, int64_t M, const float *C_sets_dev, int64_t c_sk, int64_t c_sb,
                  int64_t c_sm, int64_t K, float *loss_dev, int32_t max_len, int32_t max_consts,
                  const sr_fit_options *opt, int32_t *status_dev, void *stream);

/* Launch shape sr_fit_lbfgs picks on the current device for these arguments (as
 * passed to it): shape[0] points per lane, shape[1] warps per problem, shape[2]
 * persistent CTAs (before any shrinking to fit a workspace).  The warps and points
 * per lane fix the order in which a fit sums over its points, so they are what a
 * bit-exact host restatement of a fit needs.  No counterpart in the reference.
 * Returns 0 or an error code. */
int sr_fit_launch_shape(int64_t B, int64_t N, int64_t n_x, int64_t M, int32_t max_len, int32_t max_consts,
                        const sr_fit_options *opt, int32_t *shape);

/*
 * Fused batched L-BFGS fit of the learnable constants of every tape: one
 * persistent kernel in which each CTA owns one problem at a time (its warps split
 * the data points) and runs the whole optimisation (closure = forward + adjoint over all N points, the
 * L-BFGS direction, strong-Wolfe or backtracking line search, history update) on chip.
 * Follows optimize() and LBFGS_batch per problem (reference
 * symbolic_torch/optimization.py:9-112, symbolic_torch/lbfgs_batch.py:61-326).
 * C_init/C_out (B, M) use (c_sb, c_sm) strides; Y and Y_final (B, N) are
 * contiguous (Y_final may be NULL); iters_out/loss_out/evals_out (B) may be NULL.
 * iters_out[b] is the number of L-BFGS iterations run, or -code when a closure
 * of problem b hit error 201/204 (status_dev then holds the first such code), or
 * -SR_TAPE_EXCEEDS_LAUNCH when its tape is longer than max_len, has more
 * constants than max_consts or more operator nodes than opt->max_operators: such a
 * problem is not fitted (C_out = C_init, Y_final and loss NaN).
 * order_dev (B) int32 gives the processing order (NULL = 0..B-1).
 * max_len: largest root + 1 (stats[2] of sr_tape_compile; 0 = M); max_consts:
 * largest meta[2] (stats[3]) or more.  max_consts also sets the constant-slot layout
 * (1, 2 or 4 slot registers per lane for up to 31, 63 or 127 constants), which with
 * the launch shape fixes the order of the direction's sums: slices of one batch
 * fitted separately give each problem the bits of the whole fit when each gets the
 * whole batch's max_consts and, through opt, its warps and points per lane
 * (sr_fit_launch_shape).  workspace_dev must hold sr_fit_workspace_bytes(...)
 * bytes; it is initialised by the call.
 */
int sr_fit_lbfgs(const float *X_dev, int64_t N, int64_t n_x, const float *Y_dev,
                 const uint32_t *desc_dev, const int32_t *meta_dev, int64_t B, int64_t M,
                 const float *C_init_dev, float *C_out_dev, int64_t c_sb, int64_t c_sm,
                 float *Y_final_dev, int32_t *iters_out_dev, float *loss_out_dev,
                 int32_t *evals_out_dev, const int32_t *order_dev, int32_t max_len,
                 int32_t max_consts, const sr_fit_options *opt, void *workspace_dev,
                 int64_t workspace_bytes, int32_t *status_dev, void *stream);

/*
 * sr_fit_lbfgs without a caller workspace.  No counterpart in the reference: it is
 * for callers that cannot allocate device memory for this library (a host whose
 * device memory is all owned by its own pool and forbids other cudaMalloc calls,
 * or a service that must not allocate on its request path).  The scratch (work
 * counter and the L-BFGS history of each CTA) is a fixed 16 MiB device array inside the
 * library, present on every device that loads it until the process exits.  The
 * persistent grid is shrunk until its history fits; when even one CTA does not fit
 * (very large history_size) the call fails with SR_ERR_WORKSPACE.  Every call looks
 * up the array's device address on the current device (cudaGetSymbolAddress: no
 * allocation, no synchronisation), so a device reset between calls leaves no stale
 * address; the first call on a device may load the library's device code, so make
 * it before any stream capture.  Every call uses the same array and resets
 * the work counter itself, so calls that overlap on the same GPU (for instance on
 * two streams) race on it and must be serialised by the caller; each device has
 * its own array.  Arguments and results are those of sr_fit_lbfgs; nothing is
 * allocated.
 */
int sr_fit_lbfgs_static_scratch(const float *X_dev, int64_t N, int64_t n_x, const float *Y_dev,
                                const uint32_t *desc_dev, const int32_t *meta_dev, int64_t B,
                                int64_t M, const float *C_init_dev, float *C_out_dev, int64_t c_sb,
                                int64_t c_sm, float *Y_final_dev, int32_t *iters_out_dev,
                                float *loss_out_dev, int32_t *evals_out_dev, const int32_t *order_dev,
                                int32_t max_len, int32_t max_consts, const sr_fit_options *opt,
                                int32_t *status_dev, void *stream);

/*
 * create_constants support (reference symbolic_torch/utils.py:7-41).
 * sr_const_offsets: for a 2-D Ops view (R, Cc) with strides (s0, s1), writes
 * offsets_dev (R + 1) int64: the exclusive prefix count of LEARNABLE_CONSTANT
 * entries in row-major order; offsets[R] is the total.
 * sr_const_scatter: out (R, Cc) contiguous float32 gets values[rank] at the k-th
 * LEARNABLE_CONSTANT entry in row-major order and 0 elsewhere.
 */
int sr_const_offsets(const int64_t *ops_dev, int64_t R, int64_t Cc, int64_t s0, int64_t s1,
                     int64_t *offsets_dev, void *stream);
int sr_const_scatter(const int64_t *ops_dev, int64_t R, int64_t Cc, int64_t s0, int64_t s1,
                     const int64_t *offsets_dev, const float *values_dev, float *out_dev,
                     void *stream);

/*
 * Child table of left-packed postfix tapes: ch (B, M, 2) int64 (-1 = no child) and
 * err (B) int64 per tape: 0, the reference's codes 404/405/406/407/408, or -1 / -2
 * when a symbol is negative / not below VAR_START_ID + n_vars.  Replaces
 * get_postfix_children (reference src/pcfg_cuda.cu:1228-1300, src/pcfg.cpp:957-986).
 * ops (B, M) int64 contiguous.
 */
int sr_postfix_children(const int64_t *ops_dev, int64_t B, int64_t M, int32_t n_vars, int64_t *ch_dev,
                        int64_t *err_dev, void *stream);

/*
 * Postfix tapes to infix token ids with parentheses: infix (B, M_out) int64, NO_OP
 * padded; "(" = VAR_START_ID + n_vars, ")" = "(" + 1.  err (B) int64: 0, the
 * reference's codes 501/504/505/506/508/509, or -1 / -2 as above.  Replaces
 * postfix_to_infix (reference src/pcfg_cuda.cu:502-701, src/pcfg.cpp:790-826).
 */
int sr_postfix_to_infix(const int64_t *ops_dev, int64_t B, int64_t M, int32_t n_vars, int64_t *infix_dev,
                        int64_t M_out, int64_t *err_dev, void *stream);

/* ---- Grammar sampling and infix parsing -------------------------------------------
 * Sample B infix expressions (B, max_length) int64, NO_OP padded, from a grammar in
 * the reference's CSR form: nt_rule_ptr (n_symbols + 1) int32, the rules of symbol s
 * being nt_rule_ptr[s] .. nt_rule_ptr[s + 1] - 1; nt_rule_cum_probs (rules) float32
 * cumulative per symbol, the last of each symbol 1.0; rhs_ptr (rules + 1) int32 and
 * rhs_concat int32, the right-hand sides.  A seed fixes every expression (a
 * SplitMix64 stream per expression).  err (B) int64: 0, 303 (max_tries exceeded) or
 * 304 (no rule for the drawn number).  max_length <= 128.  Symbol ids (start_symbol
 * and every rhs_concat entry) lie in [0, 32768); an id at or above n_symbols is a
 * terminal.  The tables are read as given: nt_rule_ptr nondecreasing within [0, rules]
 * and rhs_ptr within rhs_concat, as the grammar object builds them.  Replaces
 * sample_infix (reference src/pcfg.cpp:568-628, src/pcfg_cuda.cu:10-146).
 */
int sr_pcfg_sample_infix(const int32_t *nt_rule_ptr, const float *nt_rule_cum_probs, const int32_t *rhs_ptr,
                         const int32_t *rhs_concat, int32_t n_symbols, int32_t start_symbol, int64_t B,
                         int32_t max_length, int32_t max_tries, uint64_t seed, int64_t *out_dev,
                         int64_t *err_dev, void *stream);

/*
 * Infix token rows (B, M) int64 (M <= 128; "(" = VAR_START_ID + n_vars, ")" = "(" + 1)
 * to postfix (with the reference's tree check) or to prefix, (B, M) int64 NO_OP
 * padded; a row with an error is all NO_OP.  err (B) int64: 0, the reference's codes
 * 401..408, or -1 / -2 for a token below 0 / at or above the terminal limit.
 * Replace infix_to_postfix and infix_to_prefix (reference src/pcfg.cpp:660-746,
 * src/pcfg_cpu.cpp:121-448).
 */
int sr_infix_to_postfix(const int64_t *infix_dev, int64_t B, int64_t M, int32_t n_vars, int64_t *postfix_dev,
                        int64_t *err_dev, void *stream);
int sr_infix_to_prefix(const int64_t *infix_dev, int64_t B, int64_t M, int32_t n_vars, int64_t *prefix_dev,
                       int64_t *err_dev, void *stream);

/*
 * Prefix rows: to postfix, from postfix, to infix (M_out tokens), and the parent of
 * every node (-1 for the root and padding), all (B, M) int64, NO_OP padded; a row
 * with an error is all NO_OP (all -1 for parents).  err (B) int64: 0, the
 * reference's codes (404..408 for parents; 501..509 for the conversions), or -1 / -2
 * for a symbol below 0 / at or above VAR_START_ID + n_vars.  Replace
 * prefix_to_postfix, postfix_to_prefix, prefix_to_infix and get_prefix_parent
 * (reference src/pcfg.cpp:827-955, src/pcfg_cpu.cpp:637-1064).
 */
int sr_prefix_to_postfix(const int64_t *prefix_dev, int64_t B, int64_t M, int32_t n_vars, int64_t *postfix_dev,
                         int64_t *err_dev, void *stream);
int sr_postfix_to_prefix(const int64_t *postfix_dev, int64_t B, int64_t M, int32_t n_vars, int64_t *prefix_dev,
                         int64_t *err_dev, void *stream);
int sr_prefix_to_infix(const int64_t *prefix_dev, int64_t B, int64_t M, int32_t n_vars, int64_t *infix_dev,
                       int64_t M_out, int64_t *err_dev, void *stream);
int sr_prefix_parent(const int64_t *prefix_dev, int64_t B, int64_t M, int32_t n_vars, int64_t *parent_dev,
                     int64_t *err_dev, void *stream);

/* ---- Warm-start network ---------------------------------------------------------
 * No reference counterpart: the learned part of the fit.  A BF16 MLP with fp32
 * accumulation predicts starting constants from a tape (bag of tokens through a
 * 64-wide embedding) and 32 features of its target row.  bf16 tensors are passed
 * as uint16_t bit patterns.  Layer widths are padded to multiples of 64. */
#define SR_MLP_VOCAB 64  /* token bins: operator codes 0..63 (larger codes share bin 63) */
#define SR_MLP_EMB 64    /* embedding width */
#define SR_MLP_FEATS 32  /* target features: 4 moments + SR_MLP_PROJ projections */
#define SR_MLP_PROJ 28   /* random features of X */
#define SR_MLP_IN 128    /* first hidden layer input: embedding | features | zero padding */
#define SR_MLP_TIMEOUT 601 /* status: a GEMM wait on the tensor-core pipeline ran out */

#define SR_MLP_EPI_RELU 0       /* bf16 out = relu(acc + bias), row-major and/or transposed */
#define SR_MLP_EPI_LINEAR 1     /* bf16 out = acc + bias (bias may be NULL) */
#define SR_MLP_EPI_F32 2        /* fp32 out_f32 = acc + bias (bias may be NULL) */
#define SR_MLP_EPI_RELU_GRAD 3  /* bf16 out = acc where gate > 0, else 0 (ReLU adjoint) */
#define SR_MLP_EPI_SPLIT_F32 4  /* fp32 partial sums: the K range is cut into `splits` pieces,
                                   piece s written at out_f32 + s * split_stride (no bias) */

typedef struct {
  int32_t epilogue;         /* SR_MLP_EPI_* */
  int32_t splits;           /* SR_MLP_EPI_SPLIT_F32 only */
  const float *bias_dev;    /* [n] or NULL */
  const uint16_t *gate_dev; /* RELU_GRAD: bf16 [rows][ld_gate] */
  int64_t ld_gate;
  uint16_t *out_dev;        /* bf16 row-major: row r, column c at out[r * ld_out + out_col0 + c]; or NULL */
  int64_t ld_out, out_col0;
  uint16_t *out_t_dev;      /* bf16 transposed: out_t[(out_t_row0 + c) * ld_out_t + r]; or NULL */
  int64_t ld_out_t, out_t_row0;
  float *out_f32_dev;       /* fp32 row-major [rows][ld_out_f32] (per split) */
  int64_t ld_out_f32, split_stride;
} sr_mlp_epilogue;

/*
 * D[rows][n] = A[rows][k] . W[n][k]^T on the tensor cores (tcgen05, bf16 operands
 * staged by TMA, fp32 accumulation in TMEM), followed by the epilogue.  k a positive
 * multiple of 64; n 64, 128 or 256; lda, ldw >= k and multiples of 8; A and W
 * 16-byte aligned.  status_dev receives SR_MLP_TIMEOUT if a pipeline wait ran out.
 */
int sr_mlp_gemm(const uint16_t *A_dev, int64_t rows, int64_t k, int64_t lda, const uint16_t *W_dev, int64_t n,
                int64_t ldw, const sr_mlp_epilogue *epi, int32_t *status_dev, void *stream);

/* Number of K pieces sr_mlp_gemm uses for SR_MLP_EPI_SPLIT_F32 with this k and request. */
int sr_mlp_gemm_splits_used(int64_t k, int32_t splits);

/* phi (N, SR_MLP_PROJ) = sqrt(2) cos(omega_j . x_n + beta_j); omega (SR_MLP_PROJ, n_x), beta (SR_MLP_PROJ). */
int sr_mlp_random_features(const float *X_dev, int64_t N, int64_t n_x, const float *omega_dev,
                           const float *beta_dev, float *phi_dev, void *stream);

/*
 * Network inputs of B problems: hist (B, SR_MLP_VOCAB) bf16 token frequencies of each
 * tape (counts / number of non-NO_OP tokens) and its transpose hist_t (SR_MLP_VOCAB,
 * ld_t); columns SR_MLP_EMB.. of x0 (B, SR_MLP_IN) and rows SR_MLP_EMB.. of x0_t
 * (SR_MLP_IN, ld_t) get the 32 target features of Y (B, N) then zeros: asinh(mean),
 * log(std + 1e-3), skewness, asinh(excess kurtosis), and the means of the standardised
 * target times each random feature phi (N, SR_MLP_PROJ).  feats (B, 32) fp32 or NULL.
 */
int sr_mlp_features(const int64_t *ops_dev, int64_t B, int64_t M, int64_t ops_sb, int64_t ops_sm,
                    const float *Y_dev, int64_t N, const float *phi_dev, uint16_t *hist_dev,
                    uint16_t *hist_t_dev, int64_t ld_t, uint16_t *x0_dev, uint16_t *x0_t_dev,
                    float *feats_dev, void *stream);

/*
 * Squared-error loss on the first n_out output columns where mask > 0:
 * row_loss (rows) = sum_j mask (out - target)^2 (or NULL), and the bf16 output
 * gradient scale * 2 * mask * (out - target) into d_out (rows, ld_d) (zero in columns
 * n_out..ld_d-1) and, if not NULL, its transpose d_out_t (ld_d rows, ld_dt).
 */
int sr_mlp_loss(const float *out_dev, int64_t rows, int64_t ld_out, const float *target_dev,
                const float *mask_dev, int32_t n_out, float scale, float *row_loss_dev, uint16_t *d_out_dev,
                int64_t ld_d, uint16_t *d_out_t_dev, int64_t ld_dt, void *stream);

/*
 * An output gradient computed outside the network: d_out (rows, ld_d) bf16 =
 * scale * g (rows, n_out; row stride ld_g), zero in columns n_out..ld_d-1 and in rows
 * where g is not finite; its transpose into d_out_t (ld_d rows, ld_dt) if not NULL.
 */
int sr_mlp_output_grad(const float *g_dev, int64_t rows, int32_t n_out, int64_t ld_g, float scale,
                       uint16_t *d_out_dev, int64_t ld_d, uint16_t *d_out_t_dev, int64_t ld_dt, void *stream);

/* out (n) = row sums of the bf16 matrix xt (n, ld) over its first `rows` columns. */
int sr_mlp_colsum(const uint16_t *xt_dev, int64_t n, int64_t rows, int64_t ld, float *out_dev, void *stream);

/* out (count) = sum over s < splits of part[s * split_stride + i], in order. */
int sr_mlp_reduce_splits(const float *part_dev, int32_t splits, int64_t count, int64_t split_stride,
                         float *out_dev, void *stream);

/*
 * One Adam step (decoupled weight decay, bias correction for `step` >= 1) on fp32
 * weights w (rows, cols) with gradient g and moments m, v; then bf16 copies into
 * w_bf16 (rows, cols) and w_t_bf16 (cols, rows) where not NULL.  lr = 0 only
 * refreshes the bf16 copies (g, m, v unused).
 */
int sr_mlp_adam(float *w_dev, const float *g_dev, float *m_dev, float *v_dev, int64_t rows, int64_t cols,
                float lr, float beta1, float beta2, float eps, float weight_decay, int32_t step,
                uint16_t *w_bf16_dev, uint16_t *w_t_bf16_dev, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* SR_GB300_H */
