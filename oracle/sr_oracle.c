/*
 * sr_oracle.c -- CPU restatement of the reference's expression-fitting path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product links or calls this file:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it,
 * and only to check results (or as the timed stand-in for the reference's CPU
 * path).  Parity is pinned against outputs of the reference itself, run in the
 * development container and committed as fixtures under tests/golden/.
 *
 * It restates, in plain C and with the reference's own loop structure:
 *   - operator domain policies        include/operators.h:222-434
 *   - input validation (codes 101/102) src/evaluation_kernels_cpu.cpp:8-52
 *   - forward tape step                src/evaluation_kernels_cpu.cpp:55-219
 *     (NO_OP -> NaN; arity-0 unknown codes -> 0)
 *   - adjoint tape step (201/204)      src/evaluation_kernels_cuda.cu:218-632
 *     (the CUDA variant is followed where it differs from the CPU one:
 *      EXP uses the cached output, CUBE/FOURTH/FIFTH multiply (g*k)*a^n)
 *   - autograd host loops              src/symbolic_evaluation.cpp:39-168
 *   - optimize() closure               symbolic_torch/optimization.py:51-112
 *   - LBFGS_batch                      symbolic_torch/lbfgs_batch.py:61-326
 *   - grammar sampler (own stream)     src/pcfg_cpu.cpp:10-119
 *   - infix -> postfix / prefix        src/pcfg_cpu.cpp:121-448
 *   - notation conversions             src/pcfg_cpu.cpp:449-1142 (postfix/prefix ->
 *                                      infix, prefix <-> postfix, parents, children)
 *
 * Floating-point contraction must be off (-ffp-contract=off) so that x86 and
 * aarch64 hosts give the same bits.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* The library's own float sin, cos, exp and log (used by the kernel-arithmetic mode
 * below): the same source the kernels compile, a fixed sequence of IEEE operations. */
#include "../cudasymbolicregression_gb300/csrc/sr_fmath.h"

enum {
    OP_NO_OP = 0, OP_LEARNABLE = 1, OP_C1 = 2, OP_C2 = 3, OP_C3 = 4, OP_C4 = 5, OP_C5 = 6,
    OP_PI = 7, OP_E = 8,
    OP_SIN = 10, OP_COS, OP_EXP, OP_LOG, OP_SQUARE, OP_SQRT, OP_TAN, OP_ARCSIN, OP_ARCCOS,
    OP_ARCTAN, OP_SINH, OP_COSH, OP_TANH, OP_FLOOR, OP_CEIL, OP_LN, OP_LOG10, OP_NEG, OP_INV,
    OP_CUBE, OP_FOURTH, OP_FIFTH,
    OP_ADD = 40, OP_SUB, OP_MUL, OP_DIV, OP_POW,
    OP_VAR0 = 50
};

#define ERR_CHILD_GEQ_PARENT 101
#define ERR_ARITY 102
#define ERR_GRAD_NO_OP 201
#define ERR_DIV_ZERO 204

static int arity_of(int64_t op) {
    if (op >= OP_SIN && op <= OP_FIFTH) return 1;
    if (op >= OP_ADD && op <= OP_POW) return 2;
    return 0;
}

/* ---- validation (reference: evaluation_kernels_cpu.cpp:8-52) ------------------
 * ops/ch are addressed through (b, m) strides so both the (B,M) and (M,B) layouts
 * can be checked in place.  The lowest (m, b) offender wins (the reference lets
 * whichever thread writes last win; on a single offender both agree). */
int sro_validate(const int64_t *ops, const int64_t *ch, int64_t B, int64_t M,
                 int64_t ops_sb, int64_t ops_sm, int64_t ch_sb, int64_t ch_sm)
{
    for (int64_t m = 0; m < M; ++m)
        for (int64_t b = 0; b < B; ++b) {
            int64_t op = ops[b * ops_sb + m * ops_sm];
            int expected = arity_of(op), actual = 0;
            for (int i = 0; i < 2; ++i) {
                int64_t c = ch[b * ch_sb + m * ch_sm + i];
                if (c != -1) {
                    actual++;
                    if (c >= m) return ERR_CHILD_GEQ_PARENT;
                }
            }
            if (actual != expected) return ERR_ARITY;
        }
    return 0;
}

/* ---- scalar operator policies (operators.h:222-434) ---------------------------- */
#define DEFINE_SCALAR_OPS(T, SUF, SIN, COS, EXP, LOG, SQRT, TAN, ASIN, ACOS, ATAN, SINH, COSH, TANH, \
                          FLOOR, CEIL, LOG10, POW)                                                \
static T fwd_##SUF(int64_t op, T a, T b, T cval, const T *xrow, int64_t nx)                     \
{                                                                                                 \
    const T qnan = (T)NAN;                                                                        \
    switch (op) {                                                                                 \
    case OP_NO_OP: return qnan;                                                                   \
    case OP_LEARNABLE: return cval;                                                               \
    case OP_C1: return (T)1; case OP_C2: return (T)2; case OP_C3: return (T)3;                    \
    case OP_C4: return (T)4; case OP_C5: return (T)5;                                             \
    case OP_PI: return (T)3.14159265358979323846; case OP_E: return (T)2.7182818284590452354;     \
    case OP_SIN: return SIN(a); case OP_COS: return COS(a); case OP_EXP: return EXP(a);          \
    case OP_LOG: case OP_LN: return a <= (T)0 ? qnan : LOG(a);                                    \
    case OP_SQUARE: return a * a;                                                                 \
    case OP_SQRT: return a < (T)0 ? qnan : SQRT(a);                                               \
    case OP_TAN: return TAN(a);                                                                   \
    case OP_ARCSIN: return (a < (T)-1 || a > (T)1) ? qnan : ASIN(a);                              \
    case OP_ARCCOS: return (a < (T)-1 || a > (T)1) ? qnan : ACOS(a);                              \
    case OP_ARCTAN: return ATAN(a);                                                               \
    case OP_SINH: return SINH(a); case OP_COSH: return COSH(a); case OP_TANH: return TANH(a);    \
    case OP_FLOOR: return FLOOR(a); case OP_CEIL: return CEIL(a);                                 \
    case OP_LOG10: return a <= (T)0 ? qnan : LOG10(a);                                            \
    case OP_NEG: return -a;                                                                       \
    case OP_INV: return a == (T)0 ? qnan : (T)1 / a;                                              \
    case OP_CUBE: return a * a * a;                                                               \
    case OP_FOURTH: { T s = a * a; return s * s; }                                                \
    case OP_FIFTH: { T s = a * a; return s * s * a; }                                             \
    case OP_ADD: return a + b; case OP_SUB: return a - b; case OP_MUL: return a * b;              \
    case OP_DIV: return b == (T)0 ? qnan : a / b;                                                 \
    case OP_POW: return a < (T)0 ? qnan : POW(a, b);                                              \
    default:                                                                                      \
        if (op >= OP_VAR0 && op < OP_VAR0 + nx) return xrow[op - OP_VAR0];                        \
        return (T)0;                                                                              \
    }                                                                                             \
}                                                                                                 \
static T div_##SUF(T a, T b) { return b == (T)0 ? (T)NAN : a / b; }                              \
/* One adjoint step for node k at one point (evaluation_kernels_cuda.cu:218-632).              \
 * adj: per-node adjoints of this point; val: node values; returns an error code or 0.         \
 * gc/gx receive constant / variable contributions (may be NULL). */                            \
static int bwd_##SUF(int64_t op, int64_t c0, int64_t c1, T g, const T *val, T *adj, int64_t k,  \
                     T *gc, T *gx, int64_t nx)                                                    \
{                                                                                                 \
    const T qnan = (T)NAN;                                                                        \
    T a = 0, b = 0, o0, o1;                                                                       \
    if (op == OP_NO_OP) return g == (T)0 ? 0 : ERR_GRAD_NO_OP;                                    \
    int ar = arity_of(op);                                                                        \
    if (ar >= 1) a = val[c0];                                                                     \
    if (ar == 2) b = val[c1];                                                                     \
    switch (op) {                                                                                 \
    case OP_LEARNABLE: if (g != (T)0 && gc) *gc += g; return 0;                                   \
    case OP_SIN: if (g == (T)0) return 0; adj[c0] += g * COS(a); return 0;                        \
    case OP_COS: if (g == (T)0) return 0; adj[c0] += g * -SIN(a); return 0;                       \
    case OP_EXP: if (g == (T)0) return 0; adj[c0] += g * val[k]; return 0;                        \
    case OP_LOG: case OP_LN: if (g == (T)0) return 0; adj[c0] += div_##SUF(g, a); return 0;      \
    case OP_SQUARE: if (g == (T)0) return 0; adj[c0] += g * (T)2 * a; return 0;                   \
    case OP_SQRT:                                                                                 \
        if (a < (T)0) o0 = qnan;                                                                  \
        else if (g == (T)0) o0 = (T)0;                                                            \
        else o0 = div_##SUF(g * (T)0.5, a < (T)0 ? qnan : SQRT(a));                               \
        adj[c0] += o0; return 0;                                                                  \
    case OP_TAN: { if (g == (T)0) return 0; T cv = COS(a); adj[c0] += div_##SUF(g, cv * cv); return 0; } \
    case OP_ARCSIN: case OP_ARCCOS: {                                                             \
        if (g == (T)0) return 0;                                                                  \
        if (a < (T)-1 || a > (T)1) o0 = qnan;                                                     \
        else { T r = (T)1 - a * a; T d = r < (T)0 ? qnan : SQRT(r); o0 = div_##SUF(g, d); }       \
        adj[c0] += (op == OP_ARCSIN) ? o0 : -o0; return 0; }                                      \
    case OP_ARCTAN: if (g == (T)0) return 0; adj[c0] += div_##SUF(g, (T)1 + a * a); return 0;    \
    case OP_SINH: if (g == (T)0) return 0; adj[c0] += g * COSH(a); return 0;                      \
    case OP_COSH: if (g == (T)0) return 0; adj[c0] += g * SINH(a); return 0;                      \
    case OP_TANH: { if (g == (T)0) return 0; T t = TANH(a); adj[c0] += g * ((T)1 - t * t); return 0; } \
    case OP_FLOOR: case OP_CEIL: return 0;                                                        \
    case OP_LOG10: if (g == (T)0) return 0; adj[c0] += div_##SUF(g, a * LOG((T)10)); return 0;   \
    case OP_NEG: if (g == (T)0) return 0; adj[c0] += -g; return 0;                                \
    case OP_INV: if (g == (T)0) return 0; adj[c0] += (a == (T)0) ? qnan : -div_##SUF(g, a * a); return 0; \
    case OP_CUBE: if (g == (T)0) return 0; adj[c0] += g * (T)3 * (a * a); return 0;               \
    case OP_FOURTH: if (g == (T)0) return 0; adj[c0] += g * (T)4 * (a * a * a); return 0;         \
    case OP_FIFTH: { if (g == (T)0) return 0; T s = a * a; adj[c0] += g * (T)5 * (s * s); return 0; } \
    case OP_ADD: if (g == (T)0) return 0; adj[c0] += g; adj[c1] += g; return 0;                   \
    case OP_SUB: if (g == (T)0) return 0; adj[c0] += g; adj[c1] += -g; return 0;                  \
    case OP_MUL: if (g == (T)0) return 0; o0 = g * b; o1 = g * a; adj[c0] += o0; adj[c1] += o1; return 0; \
    case OP_DIV: {                                                                                \
        int err = 0;                                                                              \
        if (g == (T)0) return 0;                                                                  \
        if (b == (T)0) { err = ERR_DIV_ZERO; o0 = 0; o1 = 0; }                                    \
        else { o0 = div_##SUF(g, b); o1 = -div_##SUF(g * a, b * b); }                             \
        adj[c0] += o0; adj[c1] += o1; return err; }                                               \
    case OP_POW:                                                                                  \
        if (a < (T)0) { o0 = qnan; o1 = qnan; }                                                   \
        else {                                                                                    \
            if (g == (T)0) return 0;                                                              \
            T pm1 = POW(a, b - (T)1), pw = POW(a, b), lg = a <= (T)0 ? qnan : LOG(a);             \
            o0 = g * (pm1 * b); o1 = g * (lg * pw);                                               \
        }                                                                                         \
        adj[c0] += o0; adj[c1] += o1; return 0;                                                   \
    default:                                                                                      \
        if (g == (T)0) return 0;                                                                  \
        if (op >= OP_VAR0 && op < OP_VAR0 + nx && gx) gx[op - OP_VAR0] += g;                      \
        return 0;                                                                                 \
    }                                                                                             \
}

DEFINE_SCALAR_OPS(float, f32, sinf, cosf, expf, logf, sqrtf, tanf, asinf, acosf, atanf, sinhf, coshf, tanhf,
                  floorf, ceilf, log10f, powf)
DEFINE_SCALAR_OPS(double, f64, sin, cos, exp, log, sqrt, tan, asin, acos, atan, sinh, cosh, tanh,
                  floor, ceil, log10, pow)
/* The fused kernels' float operators: sin, cos, exp and log from sr_fmath.h. */
DEFINE_SCALAR_OPS(float, kf32, sr_sinf, sr_cosf, sr_expf, sr_logf, sqrtf, tanf, asinf, acosf, atanf, sinhf, coshf,
                  tanhf, floorf, ceilf, log10f, powf)

/* ---- forward / backward over a batch ------------------------------------------
 * Layouts (user-facing, B first): X (N,nx), ops (B,M), ch (B,M,2), C (B,M),
 * cache / grad_out (B,M,N), gC (B,M), gX (N,nx).  Per point the node order is
 * k = 0..M-1 forward and M-1..0 backward, children ch0 then ch1: the same per
 * point order as the reference's one-launch-per-k loops. */
#define DEFINE_BATCH(T, SUF)                                                                      \
void sro_eval_fwd_##SUF(const T *X, int64_t N, int64_t nx, const int64_t *ops, const int64_t *ch, \
                        const T *C, int64_t B, int64_t M, T *cache)                               \
{                                                                                                 \
    _Pragma("omp parallel for schedule(dynamic, 1)")                                              \
    for (int64_t b = 0; b < B; ++b) {                                                             \
        T *val = (T *)malloc(sizeof(T) * (size_t)(M > 0 ? M : 1));                                \
        for (int64_t n = 0; n < N; ++n) {                                                         \
            for (int64_t k = 0; k < M; ++k) {                                                     \
                int64_t op = ops[b * M + k];                                                      \
                int ar = arity_of(op);                                                            \
                T a = 0, bb = 0;                                                                  \
                if (op != OP_NO_OP) {                                                             \
                    if (ar >= 1) a = val[ch[(b * M + k) * 2 + 0]];                                \
                    if (ar == 2) bb = val[ch[(b * M + k) * 2 + 1]];                               \
                }                                                                                 \
                val[k] = fwd_##SUF(op, a, bb, C[b * M + k], X + n * nx, nx);                      \
                cache[(b * M + k) * N + n] = val[k];                                              \
            }                                                                                     \
        }                                                                                         \
        free(val);                                                                                \
    }                                                                                             \
}                                                                                                 \
/* Returns 0 or the error code; gC is (B,M) and gX is (N,nx) (either may be NULL). */          \
int sro_eval_bwd_##SUF(const T *X, int64_t N, int64_t nx, const int64_t *ops, const int64_t *ch, \
                       const T *C, int64_t B, int64_t M, const T *gout, T *gC, T *gX)            \
{                                                                                                 \
    int err = 0;                                                                                  \
    int *errs = (int *)calloc((size_t)(B > 0 ? B : 1), sizeof(int));                              \
    if (gC) memset(gC, 0, sizeof(T) * (size_t)(B * M));                                           \
    if (gX) memset(gX, 0, sizeof(T) * (size_t)(N * nx));                                          \
    T *gxall = gX ? (T *)calloc((size_t)(B * N * nx), sizeof(T)) : NULL;                          \
    _Pragma("omp parallel for schedule(dynamic, 1)")                                              \
    for (int64_t b = 0; b < B; ++b) {                                                             \
        T *val = (T *)malloc(sizeof(T) * (size_t)(M > 0 ? M : 1));                                \
        T *adj = (T *)malloc(sizeof(T) * (size_t)(M > 0 ? M : 1));                                \
        for (int64_t n = 0; n < N; ++n) {                                                         \
            for (int64_t k = 0; k < M; ++k) {                                                     \
                int64_t op = ops[b * M + k];                                                      \
                int ar = arity_of(op);                                                            \
                T a = 0, bb = 0;                                                                  \
                if (op != OP_NO_OP) {                                                             \
                    if (ar >= 1) a = val[ch[(b * M + k) * 2 + 0]];                                \
                    if (ar == 2) bb = val[ch[(b * M + k) * 2 + 1]];                               \
                }                                                                                 \
                val[k] = fwd_##SUF(op, a, bb, C[b * M + k], X + n * nx, nx);                      \
                adj[k] = (T)0 + gout[(b * M + k) * N + n];                                        \
            }                                                                                     \
            for (int64_t k = M - 1; k >= 0; --k) {                                                \
                int64_t op = ops[b * M + k];                                                      \
                T gcl = 0;                                                                        \
                int e = bwd_##SUF(op, ch[(b * M + k) * 2], ch[(b * M + k) * 2 + 1], adj[k], val,  \
                                  adj, k, &gcl, gxall ? gxall + (b * N + n) * nx : NULL, nx);      \
                if (op == OP_LEARNABLE && gC) gC[b * M + k] += gcl;                               \
                if (e && (!errs[b] || e < errs[b])) errs[b] = e;                                  \
            }                                                                                     \
        }                                                                                         \
        free(val); free(adj);                                                                     \
    }                                                                                             \
    if (gX) for (int64_t b = 0; b < B; ++b) for (int64_t i = 0; i < N * nx; ++i)                  \
        gX[i] += gxall[b * N * nx + i];                                                           \
    free(gxall);                                                                                  \
    for (int64_t b = 0; b < B && !err; ++b) err = errs[b];                                        \
    free(errs);                                                                                   \
    return err;                                                                                   \
}

DEFINE_BATCH(float, f32)
DEFINE_BATCH(double, f64)
/* The same loops with the kernels' sin, cos, exp and log (sr_fmath.h): forward values
 * the device reproduces bit for bit on tapes whose other operators are IEEE-exact. */
DEFINE_BATCH(float, kf32)

static int ladj_f32(int64_t op, float g, float a, float b, float v, int *add0, float *o0, int *add1, float *o1);

/* grad_C of the evaluation adjoint in the device kernel's summation order
 * (csrc/sr_eval.cu eval_backward_kernel, one point per lane): per point the leaf
 * adjoints as sro_eval_bwd_kf32 forms them; per constant node, lane l (0..31) sums
 * its nonzero adjoints at the points l, l + 32, l + 64, ... in that order, then the 32
 * lane sums are added by an xor butterfly (offsets 16, 8, 4, 2, 1).  gC (B, M) gets
 * the constant nodes' sums and 0 elsewhere; returns the first error code.
 *
 * The variable gradient is an atomic float sum over tapes and variable nodes on the
 * device, in no fixed order, so it has no single right answer; what it must satisfy is
 * the error bound of a float sum of its terms in any order.  When gx_sum is not NULL,
 * the terms are described per (point, variable), each (N, nx): gx_sum the sum of the
 * nonzero variable-node adjoints (the device's terms, bit for bit) in double, gx_abs the
 * sum of their magnitudes, gx_cnt their number, gx_flags bit 0 a NaN term, bit 1 a +inf
 * term, bit 2 a -inf term (non-finite terms are left out of the sums). */
int sro_eval_bwd_gc_kernel_order_f32(const float *X, int64_t N, int64_t nx, const int64_t *ops, const int64_t *ch,
                                     const float *C, int64_t B, int64_t M, const float *gout, float *gC,
                                     double *gx_sum, double *gx_abs, int32_t *gx_cnt, int32_t *gx_flags)
{
    int err = 0;
    int *errs = (int *)calloc((size_t)(B > 0 ? B : 1), sizeof(int));
    const int64_t NX = N * nx;
    /* per tape, then added over the tapes in order below (the threads own whole tapes) */
    double *tsum = NULL, *tabs = NULL;
    int32_t *tcnt = NULL, *tflg = NULL;
    if (gx_sum) {
        tsum = (double *)calloc((size_t)(B * NX > 0 ? B * NX : 1), sizeof(double));
        tabs = (double *)calloc((size_t)(B * NX > 0 ? B * NX : 1), sizeof(double));
        tcnt = (int32_t *)calloc((size_t)(B * NX > 0 ? B * NX : 1), sizeof(int32_t));
        tflg = (int32_t *)calloc((size_t)(B * NX > 0 ? B * NX : 1), sizeof(int32_t));
    }
    _Pragma("omp parallel for schedule(dynamic, 1)")
    for (int64_t b = 0; b < B; ++b) {
        float *val = (float *)malloc(sizeof(float) * (size_t)(M > 0 ? M : 1));
        float *adj = (float *)malloc(sizeof(float) * (size_t)(M > 0 ? M : 1));
        float *lanes = (float *)calloc((size_t)(M > 0 ? M : 1) * 32, sizeof(float));
        const int64_t *o = ops + b * M, *c = ch + b * M * 2;
        for (int64_t n = 0; n < N; ++n) {
            for (int64_t k = 0; k < M; ++k) {
                int64_t op = o[k];
                int ar = arity_of(op);
                float a = 0, bb = 0;
                if (op != OP_NO_OP) {
                    if (ar >= 1) a = val[c[k * 2]];
                    if (ar == 2) bb = val[c[k * 2 + 1]];
                }
                val[k] = fwd_kf32(op, a, bb, C[b * M + k], X + n * nx, nx);
                adj[k] = gout[(b * M + k) * N + n];
            }
            for (int64_t k = M - 1; k >= 0; --k) {
                int64_t op = o[k];
                if (op == OP_LEARNABLE) {
                    float g = adj[k];
                    float *d = lanes + k * 32 + (n & 31);
                    if (g != 0.0f) *d = *d + g;
                    continue;
                }
                if (op >= OP_VAR0 && op < OP_VAR0 + nx && tsum) {
                    /* every parent has a larger index: adj[k] is this node's whole adjoint */
                    const float g = adj[k];
                    const int64_t i = b * NX + n * nx + (op - OP_VAR0);
                    if (g != 0.0f) {
                        if (isnan(g)) tflg[i] |= 1;
                        else if (isinf(g)) tflg[i] |= g > 0.0f ? 2 : 4;
                        else { tsum[i] += (double)g; tabs[i] += fabs((double)g); }
                        tcnt[i] += 1;
                    }
                }
                if (op != OP_NO_OP && arity_of(op) == 0) continue;
                int a0, a1;
                float o0, o1;
                int ar = arity_of(op);
                float a = ar >= 1 ? val[c[k * 2]] : 0.0f, bb = ar == 2 ? val[c[k * 2 + 1]] : 0.0f;
                int e = ladj_f32(op, adj[k], a, bb, val[k], &a0, &o0, &a1, &o1);
                if (e && !errs[b]) errs[b] = e;
                if (a0) adj[c[k * 2]] = adj[c[k * 2]] + o0;
                if (a1) adj[c[k * 2 + 1]] = adj[c[k * 2 + 1]] + o1;
            }
        }
        for (int64_t k = 0; k < M; ++k) {
            float v[32], t[32];
            for (int l = 0; l < 32; ++l) v[l] = lanes[k * 32 + l];
            for (int off = 16; off > 0; off >>= 1) {
                for (int l = 0; l < 32; ++l) t[l] = v[l] + v[l ^ off];
                memcpy(v, t, sizeof(v));
            }
            gC[b * M + k] = o[k] == OP_LEARNABLE ? v[0] : 0.0f;
        }
        free(val); free(adj); free(lanes);
    }
    if (gx_sum) {
        for (int64_t i = 0; i < NX; ++i) {
            gx_sum[i] = 0.0; gx_abs[i] = 0.0; gx_cnt[i] = 0; gx_flags[i] = 0;
        }
        for (int64_t b = 0; b < B; ++b)
            for (int64_t i = 0; i < NX; ++i) {
                gx_sum[i] += tsum[b * NX + i];
                gx_abs[i] += tabs[b * NX + i];
                gx_cnt[i] += tcnt[b * NX + i];
                gx_flags[i] |= tflg[b * NX + i];
            }
        free(tsum); free(tabs); free(tcnt); free(tflg);
    }
    for (int64_t b = 0; b < B && !err; ++b) err = errs[b];
    free(errs);
    return err;
}

/* Elementwise forward of single nodes: out[i] = op[i](a[i], b[i]) with constant
 * c[i] and variable value x[i] (for VAR nodes pass op = OP_VAR0 and nx = 1).
 * Used to check a device result node by node from the device's own child values. */
void sro_node_fwd_f32(int64_t n, const int64_t *op, const float *a, const float *b, const float *c,
                      const float *x, float *out)
{
    for (int64_t i = 0; i < n; ++i) {
        int64_t o = op[i] >= OP_VAR0 ? OP_VAR0 : op[i];
        out[i] = fwd_f32(o, a[i], b[i], c[i], x + i, 1);
    }
}

/* The same with the kernels' own sin, cos, exp and log (sr_fmath.h). */
void sro_node_fwd_kf32(int64_t n, const int64_t *op, const float *a, const float *b, const float *c,
                       const float *x, float *out)
{
    for (int64_t i = 0; i < n; ++i) {
        int64_t o = op[i] >= OP_VAR0 ? OP_VAR0 : op[i];
        out[i] = fwd_kf32(o, a[i], b[i], c[i], x + i, 1);
    }
}

/* ---- optimize(): per-problem batched L-BFGS --------------------------------------
 *
 * Every problem (column) of the reference's LBFGS_batch evolves independently:
 * all reductions are per column and the batch-wide tests (done.all(), all(done)
 * in the line searches) only stop loops early for columns whose state no longer
 * changes.  So this restatement runs one problem at a time, with the reference's
 * control flow (strong_wolfe, zoom, backtracking and the outer loop below follow
 * lbfgs_batch.py:105-326 line by line) and one of three arithmetics:
 *
 * dot_mode 0 follows the reference arithmetic: float32 vectors over the D = M
 * parameter slots, float32 dots summed in slot order, float32 scalars.
 * dot_mode 1 approximates the fused kernel's arithmetic with double dots and
 * two-loop scalars and per-constant gradients summed over the points in double.
 * dot_mode 2 is the fused kernel's arithmetic exactly (see "the fused kernel's
 * arithmetic" below): its slot vectors (the real constants and one virtual slot
 * for all other slots), its per-lane point sums and lane/warp reduction order for a
 * given launch shape, its float-pair (Sum2/Dot2, Dekker) dots and direction (the
 * compact representation of the inverse Hessian for histories of at most 32 pairs,
 * the two-loop recursion for longer ones, both with float-pair scalars), and the
 * closures it evaluates (it reuses points the reference evaluates twice).
 * Its sin, cos, exp and log are the kernels' own (sr_fmath.h), so on tapes over
 * the IEEE-exact operators (+ - * /, square, sqrt, neg, inv, cube, fourth, fifth)
 * and sin, cos, exp, log this mode and the kernel give the same bits; the other
 * transcendental operators are CUDA's on the device and the host's here.
 */
typedef struct {
    const float *X; int64_t N, nx;
    const float *Y;                 /* (N) target row, or NULL for raw-objective mode */
    const int64_t *ops, *ch;        /* (M), (M,2) rows of this problem */
    int64_t M, root;
    float *val, *adj;
    double *gacc;                   /* per-slot gradient sums (dot_mode 1 sums in double) */
    int dmode;
    long n_evals;
    int err;
} problem_t;

/* closure(): loss = mean_n (y_root - Y)^2 and its gradient w.r.t. the M slots
 * (optimization.py:72-99).  The root adjoint is (2 (f - y)) * (1/N) in float, as
 * autograd's mse_loss/mean backward computes it.  Without Y the objective is the
 * mean of the root value itself (used for the raw-objective known-answer tests). */
static float closure_f32(problem_t *P, const float *x, float *g)
{
    const int64_t M = P->M, N = P->N;
    const float invN = 1.0f / (float)N;
    double acc = 0.0;
    for (int64_t j = 0; j < M; ++j) { g[j] = 0.0f; P->gacc[j] = 0.0; }
    for (int64_t n = 0; n < N; ++n) {
        for (int64_t k = 0; k < M; ++k) {
            int64_t op = P->ops[k];
            int ar = arity_of(op);
            float a = 0, bb = 0;
            if (op != OP_NO_OP) {
                if (ar >= 1) a = P->val[P->ch[k * 2]];
                if (ar == 2) bb = P->val[P->ch[k * 2 + 1]];
            }
            P->val[k] = fwd_f32(op, a, bb, x[k], P->X + n * P->nx, P->nx);
            P->adj[k] = 0.0f;
        }
        float f = P->val[P->root];
        float groot;
        if (P->Y) {
            float r = f - P->Y[n];
            acc += (double)(r * r);
            groot = (r * 2.0f) * invN;
        } else {
            acc += (double)f;
            groot = invN;
        }
        P->adj[P->root] = groot;
        for (int64_t k = M - 1; k >= 0; --k) {
            int64_t op = P->ops[k];
            float gcl = 0.0f;
            int e = bwd_f32(op, P->ch[k * 2], P->ch[k * 2 + 1], P->adj[k], P->val, P->adj, k, &gcl,
                            NULL, P->nx);
            if (op == OP_LEARNABLE) {
                if (P->dmode) P->gacc[k] += (double)gcl;
                else g[k] += gcl;
            }
            if (e && !P->err) P->err = e;
        }
    }
    for (int64_t k = 0; k < M; ++k) {
        if (P->dmode) g[k] = (float)P->gacc[k];
        if (P->ops[k] != OP_LEARNABLE) g[k] = 0.0f;
    }
    P->n_evals++;
    return (float)(acc / (double)N);
}

/* ---- the fused kernel's arithmetic (dot_mode 2) ------------------------------------
 *
 * Float pairs.  f2_add is Knuth's TwoSum of the high parts with the low parts summed
 * (Ogita, Rump and Oishi's cascaded Sum2); f2_val is hi + lo for a finite hi and hi
 * otherwise; f2_norm renormalises a cascaded pair; f2_mul / f2_div are Dekker's
 * double-float product and quotient with FMA.  Every operation is a single IEEE
 * float32 operation (the file is compiled with -ffp-contract=off; fmaf is the
 * correctly rounded fused multiply-add). */
typedef struct { float hi, lo; } f2_t;

static f2_t f2_mk(float hi, float lo) { f2_t r; r.hi = hi; r.lo = lo; return r; }

static f2_t f2_add(f2_t a, f2_t b)
{
    float s = a.hi + b.hi;
    float bv = s - a.hi;
    float e = (a.hi - (s - bv)) + (b.hi - bv);
    return f2_mk(s, (a.lo + b.lo) + e);
}

static float f2_val(f2_t a) { return isfinite(a.hi) ? a.hi + a.lo : a.hi; }

static f2_t f2_norm(f2_t a)
{
    if (!isfinite(a.hi)) return f2_mk(a.hi, 0.0f);
    float s = a.hi + a.lo;
    float bv = s - a.hi;
    return f2_mk(s, (a.hi - (s - bv)) + (a.lo - bv));
}

static f2_t f2_mul(f2_t a, f2_t b)
{
    float p = a.hi * b.hi;
    if (!isfinite(p)) return f2_mk(p, 0.0f);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    float s = p + e;
    return f2_mk(s, e - (s - p));
}

static f2_t f2_sub(f2_t a, f2_t b) { return f2_norm(f2_add(a, f2_mk(-b.hi, -b.lo))); }

static f2_t f2_div(f2_t a, f2_t b)
{
    float q1 = a.hi / b.hi;
    if (!isfinite(q1)) return f2_mk(q1, 0.0f);
    float ph = q1 * b.hi;
    float pl = fmaf(q1, b.hi, -ph);
    float r = (a.hi - ph) - pl;
    r = fmaf(-q1, b.lo, r + a.lo);
    float q2 = r / b.hi;
    float sum = q1 + q2;
    return f2_mk(sum, q2 - (sum - q1));
}

static f2_t f2_of_double(double d)
{
    float hi = (float)d;
    return f2_mk(hi, isfinite(hi) ? (float)(d - (double)hi) : 0.0f);
}

/* Local adjoint of one operator node at one point, as (add0, o0, add1, o1): the
 * same rules as bwd_f32 (evaluation_kernels_cuda.cu:218-632), in the form in which
 * the fused kernel adds them to their destinations, with its sin, cos and log. */
static int ladj_f32(int64_t op, float g, float a, float b, float v, int *add0, float *o0, int *add1, float *o1)
{
    const float qnan = (float)NAN;
    const int zero = g == 0.0f;
    *add0 = *add1 = 0;
    *o0 = *o1 = 0.0f;
    switch (op) {
    case OP_NO_OP: return zero ? 0 : ERR_GRAD_NO_OP;
    case OP_SIN: if (zero) return 0; *o0 = g * sr_cosf(a); *add0 = 1; return 0;
    case OP_COS: if (zero) return 0; *o0 = g * -sr_sinf(a); *add0 = 1; return 0;
    case OP_EXP: if (zero) return 0; *o0 = g * v; *add0 = 1; return 0;
    case OP_LOG: case OP_LN: if (zero) return 0; *o0 = div_f32(g, a); *add0 = 1; return 0;
    case OP_SQUARE: if (zero) return 0; *o0 = g * 2.0f * a; *add0 = 1; return 0;
    case OP_SQRT:
        *add0 = 1;
        if (a < 0.0f) *o0 = qnan;
        else if (zero) *o0 = 0.0f;
        else *o0 = div_f32(g * 0.5f, sqrtf(a));
        return 0;
    case OP_TAN: { if (zero) return 0; float cv = sr_cosf(a); *o0 = div_f32(g, cv * cv); *add0 = 1; return 0; }
    case OP_ARCSIN: case OP_ARCCOS: {
        if (zero) return 0;
        *add0 = 1;
        if (a < -1.0f || a > 1.0f) { *o0 = qnan; return 0; }
        float r = 1.0f - a * a;
        float den = r < 0.0f ? qnan : sqrtf(r);
        *o0 = div_f32(g, den);
        if (op == OP_ARCCOS) *o0 = -*o0;
        return 0; }
    case OP_ARCTAN: if (zero) return 0; *o0 = div_f32(g, 1.0f + a * a); *add0 = 1; return 0;
    case OP_SINH: if (zero) return 0; *o0 = g * coshf(a); *add0 = 1; return 0;
    case OP_COSH: if (zero) return 0; *o0 = g * sinhf(a); *add0 = 1; return 0;
    case OP_TANH: { if (zero) return 0; float t = tanhf(a); *o0 = g * (1.0f - t * t); *add0 = 1; return 0; }
    case OP_LOG10: if (zero) return 0; *o0 = div_f32(g, a * sr_logf(10.0f)); *add0 = 1; return 0;
    case OP_NEG: if (zero) return 0; *o0 = -g; *add0 = 1; return 0;
    case OP_INV: if (zero) return 0; *o0 = (a == 0.0f) ? qnan : -div_f32(g, a * a); *add0 = 1; return 0;
    case OP_CUBE: if (zero) return 0; *o0 = g * 3.0f * (a * a); *add0 = 1; return 0;
    case OP_FOURTH: if (zero) return 0; *o0 = g * 4.0f * (a * a * a); *add0 = 1; return 0;
    case OP_FIFTH: { if (zero) return 0; float s = a * a; *o0 = g * 5.0f * (s * s); *add0 = 1; return 0; }
    case OP_ADD: if (zero) return 0; *o0 = g; *o1 = g; *add0 = *add1 = 1; return 0;
    case OP_SUB: if (zero) return 0; *o0 = g; *o1 = -g; *add0 = *add1 = 1; return 0;
    case OP_MUL: if (zero) return 0; *o0 = g * b; *o1 = g * a; *add0 = *add1 = 1; return 0;
    case OP_DIV:
        if (zero) return 0;
        *add0 = *add1 = 1;
        if (b == 0.0f) return ERR_DIV_ZERO;
        *o0 = div_f32(g, b);
        *o1 = -div_f32(g * a, b * b);
        return 0;
    case OP_POW:
        if (a < 0.0f) { *o0 = qnan; *o1 = qnan; *add0 = *add1 = 1; return 0; }
        if (zero) return 0;
        {
            float pm1 = powf(a, b - 1.0f), pw = powf(a, b), lg = a <= 0.0f ? qnan : sr_logf(a);
            *o0 = g * (pm1 * b);
            *o1 = g * (lg * pw);
        }
        *add0 = *add1 = 1;
        return 0;
    default: return 0;  /* FLOOR, CEIL */
    }
}

static int is_operator_node(int64_t op) { return op == OP_NO_OP || arity_of(op) >= 1; }

/* State of one problem in the fused kernel's arithmetic (one CTA of W warps, V
 * points per lane).  Slot vectors hold D = 32 spl entries: the K learnable
 * constants up to the root in tape order, then, when M > K, one virtual slot that
 * stands for all other slots (its gradient is always 0; it only carries the NaN
 * that 0 * NaN spreads into them); the rest are inactive zeros. */
typedef struct {
    int W, V, spl, D;
    int K, nslots, has_virtual;
    int objective;
    int *slot_of;                   /* (M) slot of a learnable node up to the root, else -1 */
    int64_t *slot_node;             /* (K) */
    float *vals, *adjs;             /* (V, 32, M) node values / adjoints of one chunk */
    float *gl;                      /* (K, 32 V) per-point-row gradient partials of one warp */
    f2_t *red_g, *red_l;            /* (W, K), (W) */
    int *lane_err;                  /* (32 W) first error each thread met, over the whole fit */
    int hist, h, head;
    float *ringS, *ringY;           /* (hist, D) */
    f2_t *rho, *alph;               /* (hist) rho per ring slot, alpha per position */
    int compact;                    /* hist <= 32: the compact representation (else the two-loop) */
    int pending;                    /* ring slot of the pair whose compact update is pending */
    int split;                      /* compact with hist <= 16 and one slot register: two lanes per pair */
    f2_t *cd, *Rinv, *YY;           /* (hist), (hist, hist), (hist, hist): c = s.y + eps, R^-1, Y^T Y by slot */
    f2_t u[32], w[32], tpart[32];   /* by position: S^T g, Y^T g, t over the older pairs */
    f2_t last_sy, last_yy, eps2;
    int poison;
} kern_t;

/* Sum over the 32 lanes of a warp of x[lane][0..KP) (per-slot partials, the loss
 * partial at K) by recursive halving (the kernel's reduce_slots): at each step a lane
 * keeps half of its values and adds its partner's partial sums of that half; the
 * lowest lane of each group then holds one slot's total. */
static void reduce_lanes(int KP, int K, f2_t x[32][32], f2_t *out_g, f2_t *out_l)
{
    int slot[32] = { 0 };
    int n = KP;
    f2_t t[32][32];
    for (int o = 16; o > 0; o >>= 1) {
        if (n > 1) {
            int h = n >> 1;
            for (int l = 0; l < 32; ++l) {
                int p = l ^ o, up = (l & o) != 0;
                for (int q = 0; q < h; ++q) {
                    f2_t keep = up ? x[l][q + h] : x[l][q];
                    f2_t recv = up ? x[p][q + h] : x[p][q];  /* the half the partner gives away */
                    t[l][q] = f2_add(keep, recv);
                }
                slot[l] = slot[l] * 2 + up;
            }
            for (int l = 0; l < 32; ++l) for (int q = 0; q < h; ++q) x[l][q] = t[l][q];
            n = h;
        } else {
            for (int l = 0; l < 32; ++l) t[l][0] = f2_add(x[l][0], x[l ^ o][0]);
            for (int l = 0; l < 32; ++l) x[l][0] = t[l][0];
        }
    }
    int group = 32 / KP;
    for (int l = 0; l < 32; ++l) {
        if (l & (group - 1)) continue;
        if (slot[l] < K) out_g[slot[l]] = x[l][0];
        else if (slot[l] == K) *out_l = x[l][0];
    }
}

/* xor butterfly over groups of `width` lanes: every lane ends with its group's total. */
static void lane_butterfly(f2_t acc[32], int width)
{
    f2_t t[32];
    for (int o = width >> 1; o > 0; o >>= 1) {
        for (int l = 0; l < 32; ++l) t[l] = f2_add(acc[l], acc[l ^ o]);
        memcpy(acc, t, sizeof(t));
    }
}

/* The fused kernel's closure (sr_fit.cu tape_pass + reduce_slots + closure): warp w
 * takes the chunks of 32 V points starting at w 32 V, W 32 V apart; lane l of a chunk
 * holds points base + v 32 + l.  Per thread: the loss is a float sum over its points,
 * each constant's gradient a float sum per point row, the contributions of a point
 * added in the order of the reverse sweep (parents last to first, child 0 first). */
static float kclosure(problem_t *P, kern_t *k, const float *xt, float *g)
{
    const int64_t N = P->N, M = P->M, root = P->root;
    const int W = k->W, V = k->V, RW = 32 * k->V, K = k->K;
    const float invN = 1.0f / (float)N;
    for (int w = 0; w < W; ++w) {
        float lpart[32];
        for (int l = 0; l < 32; ++l) lpart[l] = 0.0f;
        for (int64_t i = 0; i < (int64_t)K * RW; ++i) k->gl[i] = 0.0f;
        for (int64_t base = (int64_t)w * RW; base < N; base += (int64_t)W * RW) {
            /* forward and residuals, point by point */
            for (int v = 0; v < V; ++v)
                for (int l = 0; l < 32; ++l) {
                    int64_t n = base + v * 32 + l;
                    if (n >= N) continue;
                    float *val = k->vals + ((int64_t)v * 32 + l) * M, *adj = k->adjs + ((int64_t)v * 32 + l) * M;
                    for (int64_t kk = 0; kk <= root; ++kk) {
                        int64_t op = P->ops[kk];
                        int ar = arity_of(op);
                        float a = 0, bb = 0;
                        if (op != OP_NO_OP) {
                            if (ar >= 1) a = val[P->ch[kk * 2]];
                            if (ar == 2) bb = val[P->ch[kk * 2 + 1]];
                        }
                        float cval = k->slot_of[kk] >= 0 ? xt[k->slot_of[kk]] : 0.0f;
                        val[kk] = fwd_kf32(op, a, bb, cval, P->X + n * P->nx, P->nx);
                        adj[kk] = 0.0f;
                    }
                    float f = val[root], groot;
                    if (k->objective == 0) {
                        float rr = f - P->Y[n];
                        lpart[l] = lpart[l] + rr * rr;
                        groot = (rr * 2.0f) * invN;
                    } else {
                        lpart[l] = lpart[l] + f;
                        groot = invN;
                    }
                    if (is_operator_node(P->ops[root])) adj[root] = groot;
                    else if (groot != 0.0f && k->slot_of[root] >= 0) {
                        float *d = k->gl + (int64_t)k->slot_of[root] * RW + v * 32 + l;
                        *d = *d + groot;
                    }
                }
            /* reverse sweep: node by node, the points of a node in row order */
            for (int64_t kk = root; kk >= 0; --kk) {
                int64_t op = P->ops[kk];
                if (!is_operator_node(op)) continue;
                int64_t c0 = P->ch[kk * 2], c1 = P->ch[kk * 2 + 1];
                for (int v = 0; v < V; ++v)
                    for (int l = 0; l < 32; ++l) {
                        int64_t n = base + v * 32 + l;
                        if (n >= N) continue;
                        float *val = k->vals + ((int64_t)v * 32 + l) * M, *adj = k->adjs + ((int64_t)v * 32 + l) * M;
                        int ar = arity_of(op), a0, a1;
                        float o0, o1;
                        float a = ar >= 1 ? val[c0] : 0.0f, bb = ar == 2 ? val[c1] : 0.0f;
                        int e = ladj_f32(op, adj[kk], a, bb, val[kk], &a0, &o0, &a1, &o1);
                        int *te = k->lane_err + w * 32 + l;
                        if (e && !*te) *te = e;
                        for (int side = 0; side < 2; ++side) {
                            if (!(side ? a1 : a0)) continue;
                            int64_t c = side ? c1 : c0;
                            float o = side ? o1 : o0;
                            float *d = NULL;
                            if (is_operator_node(P->ops[c])) d = adj + c;
                            else if (k->slot_of[c] >= 0) d = k->gl + (int64_t)k->slot_of[c] * RW + v * 32 + l;
                            if (d) *d = *d + o;
                        }
                    }
            }
        }
        /* lanes, then warps */
        if (K < 32) {
            int KP = K < 1 ? 1 : K < 2 ? 2 : K < 4 ? 4 : K < 8 ? 8 : K < 16 ? 16 : 32;
            f2_t x[32][32];
            for (int l = 0; l < 32; ++l)
                for (int j = 0; j < KP; ++j) {
                    float part = 0.0f;
                    if (j < K) {
                        part = k->gl[(int64_t)j * RW + l];
                        for (int v = 1; v < V; ++v) part = part + k->gl[(int64_t)j * RW + v * 32 + l];
                    } else if (j == K) {
                        part = lpart[l];
                    }
                    x[l][j] = f2_mk(part, 0.0f);
                }
            reduce_lanes(KP, K, x, k->red_g + (int64_t)w * K, k->red_l + w);
        } else {
            f2_t acc[32];
            for (int l = 0; l < 32; ++l) acc[l] = f2_mk(lpart[l], 0.0f);
            lane_butterfly(acc, 32);
            k->red_l[w] = acc[0];
            for (int j = 0; j < K; ++j) {
                for (int l = 0; l < 32; ++l) {
                    float part = k->gl[(int64_t)j * RW + l];
                    for (int v = 1; v < V; ++v) part = part + k->gl[(int64_t)j * RW + v * 32 + l];
                    acc[l] = f2_mk(part, 0.0f);
                }
                lane_butterfly(acc, 32);
                k->red_g[(int64_t)w * K + j] = acc[0];
            }
        }
    }
    for (int j = 0; j < k->D; ++j) {
        f2_t acc = f2_mk(0.0f, 0.0f);
        if (j < K)
            for (int w = 0; w < W; ++w) acc = f2_add(acc, k->red_g[(int64_t)w * K + j]);
        g[j] = f2_val(acc);
    }
    f2_t lt = f2_mk(0.0f, 0.0f);
    for (int w = 0; w < W; ++w) lt = f2_add(lt, k->red_l[w]);
    P->n_evals++;
    return f2_val(lt) / (float)N;
}

/* Per-lane float-pair terms of a slot-vector dot (TwoProduct by FMA). */
static void lane_terms(const kern_t *k, const float *a, const float *b, f2_t acc[32])
{
    for (int l = 0; l < 32; ++l) {
        acc[l] = f2_mk(0.0f, 0.0f);
        for (int s = 0; s < k->spl; ++s) {
            int j = s * 32 + l;
            if (j >= k->nslots) continue;
            float pr = a[j] * b[j];
            acc[l] = f2_add(acc[l], f2_mk(pr, fmaf(a[j], b[j], -pr)));
        }
    }
}

/* Line-search slopes and the gradient norm (the kernel's dot_f2, Dot2 rounded to float). */
static float kdot_f2(const kern_t *k, const float *a, const float *b)
{
    f2_t acc[32];
    lane_terms(k, a, b, acc);
    lane_butterfly(acc, 32);
    return f2_val(acc[0]);
}

/* Curvature dots of the two-loop recursion (the kernel's dot_pair, a normalised pair). */
static f2_t kdot_pair(const kern_t *k, const float *a, const float *b)
{
    f2_t acc[32];
    lane_terms(k, a, b, acc);
    if (k->spl == 1 && k->nslots <= 16)
        lane_butterfly(acc, k->nslots <= 4 ? 4 : (k->nslots <= 8 ? 8 : 16));
    else
        lane_butterfly(acc, 32);
    return f2_norm(acc[0]);
}

/* acc + a b for float pairs and for floats, as cascaded pair sums (the kernel's f2_mad
 * and f2_madf). */
static f2_t f2_mad(f2_t acc, f2_t a, f2_t b)
{
    float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return f2_add(acc, f2_mk(p, e));
}

static f2_t f2_madf(f2_t acc, float a, float b)
{
    float p = a * b;
    return f2_add(acc, f2_mk(p, fmaf(a, b, -p)));
}

/* Sums of the compact form as the kernel splits them (sr_fit.cu sum_part, join_parts):
 * with two lanes per pair (split: histories of at most 16 pairs, one slot register) a
 * sum over n terms is the f2_add of the in-order sum of its first (n + 1) / 2 terms and
 * the in-order sum of the rest; otherwise one in-order sum.  Terms outside the
 * predicate are skipped in place.  term_f / term_p give the j-th product (floats / pairs). */
static f2_t ksplit_dot(int split, int n, const float *a, const float *b)
{
    int mid = split ? (n + 1) >> 1 : n;
    f2_t p0 = f2_mk(0.0f, 0.0f), p1 = f2_mk(0.0f, 0.0f);
    for (int j = 0; j < mid; ++j) p0 = f2_madf(p0, a[j], b[j]);
    if (!split) return p0;
    for (int j = mid; j < n; ++j) p1 = f2_madf(p1, a[j], b[j]);
    return f2_add(p0, p1);
}

/* sum over positions j < n of M[j] x[j] where take(j); M[j], x[j] pairs. */
static f2_t ksplit_matvec(int split, int n, const f2_t *m, const f2_t *x, int lo_ok, int hi_ok)
{
    int mid = split ? (n + 1) >> 1 : n;
    f2_t p0 = f2_mk(0.0f, 0.0f), p1 = f2_mk(0.0f, 0.0f);
    for (int j = 0; j < mid; ++j)
        if (j >= lo_ok && j <= hi_ok) p0 = f2_mad(p0, m[j], x[j]);
    if (!split) return p0;
    for (int j = mid; j < n; ++j)
        if (j >= lo_ok && j <= hi_ok) p1 = f2_mad(p1, m[j], x[j]);
    return f2_add(p0, p1);
}

/* The kernel's history update for the newest pair (ring slot `slot`, position h - 1),
 * done in compact_update_direction (sr_fit.cu) just before the direction: its dots with
 * every pair in the ring, c and rho, its row and column of Y^T Y and its column of R^-1
 * (-rho times R^-1 r over the older pairs; rho on the diagonal).  The dropped pair's slot
 * is the new one, so what R^-1 keeps of the others is the inverse of R's trailing block
 * (Byrd, Nocedal and Schnabel 1994).  The partial sum of t over the older pairs is kept
 * in k->tpart for the direction (the kernel forms both in one loop). */
static void kpush_compact(kern_t *k, int slot, const float *g)
{
    const int h = k->h, hs = k->hist, D = k->D, head = k->head, split = k->split;
    const float *yn = k->ringY + (int64_t)slot * D;
    f2_t r[32], q[32], m[32];
    int sl[32];
    for (int i = 0; i < h; ++i) {
        sl[i] = (head + i) % hs;
        const float *si = k->ringS + (int64_t)sl[i] * D, *yi = k->ringY + (int64_t)sl[i] * D;
        r[i] = f2_norm(ksplit_dot(split, k->nslots, si, yn));
        q[i] = f2_norm(ksplit_dot(split, k->nslots, yi, yn));
        k->u[i] = f2_norm(ksplit_dot(split, k->nslots, si, g));
        k->w[i] = f2_norm(ksplit_dot(split, k->nslots, yi, g));
    }
    k->last_sy = r[h - 1];
    k->last_yy = q[h - 1];
    f2_t cn = f2_norm(f2_add(k->last_sy, k->eps2));
    f2_t rho = f2_div(f2_mk(1.0f, 0.0f), cn);
    for (int i = 0; i < h; ++i) {
        for (int j = 0; j < h - 1; ++j) m[j] = k->Rinv[sl[i] * hs + sl[j]];
        f2_t acc = ksplit_matvec(split, h - 1, m, r, i, h - 1);
        k->tpart[i] = ksplit_matvec(split, h - 1, m, k->u, i, h - 1);
        k->YY[sl[i] * hs + slot] = q[i];
        k->YY[slot * hs + sl[i]] = q[i];
        f2_t col = f2_mul(rho, f2_norm(acc));
        k->Rinv[sl[i] * hs + slot] = i == h - 1 ? rho : f2_mk(-col.hi, -col.lo);
    }
    k->rho[slot] = rho;
    k->cd[slot] = cn;
}

/* The kernel's compact direction (after kpush_compact): q = gamma g + S z - gamma Y t
 * with u = S^T g, w = Y^T g, t = R^-1 u, v = c t + gamma (Y^T Y t - w), z = R^-T v;
 * every sum split as the kernel splits it, the vector formed per slot in float. */
static void kdirection_compact(kern_t *k, const float *g, float *q)
{
    const int h = k->h, hs = k->hist, D = k->D, head = k->head, split = k->split;
    f2_t t[32], z[32], bb[32], v[32], m[32];
    int sl[32];
    for (int i = 0; i < h; ++i) sl[i] = (head + i) % hs;
    for (int i = 0; i < h; ++i)
        t[i] = f2_norm(f2_mad(k->tpart[i], k->Rinv[sl[i] * hs + sl[h - 1]], k->u[h - 1]));
    f2_t gam = f2_div(k->last_sy, f2_norm(f2_add(k->last_yy, k->eps2)));
    for (int i = 0; i < h; ++i) {
        for (int j = 0; j < h; ++j) m[j] = k->YY[sl[i] * hs + sl[j]];
        f2_t yt = f2_norm(ksplit_matvec(split, h, m, t, 0, h - 1));
        v[i] = f2_norm(f2_add(f2_mul(k->cd[sl[i]], t[i]), f2_mul(gam, f2_sub(yt, k->w[i]))));
    }
    for (int i = 0; i < h; ++i) {
        for (int j = 0; j < h; ++j) m[j] = k->Rinv[sl[j] * hs + sl[i]];
        z[i] = f2_norm(ksplit_matvec(split, h, m, v, 0, i));
        bb[i] = f2_mul(gam, t[i]);
    }
    for (int j = 0; j < D; ++j) {
        float qs = fmaf(g[j], gam.lo, g[j] * gam.hi), qy = 0.0f;
        for (int i = 0; i < h; ++i) {
            float sv = k->ringS[(int64_t)sl[i] * D + j], yv = k->ringY[(int64_t)sl[i] * D + j];
            qs = fmaf(z[i].lo, sv, fmaf(z[i].hi, sv, qs));
            qy = fmaf(bb[i].lo, yv, fmaf(bb[i].hi, yv, qy));
        }
        q[j] = qs - qy;
    }
}

/* The kernel's direction over its history ring (oldest pair at `head`): the compact
 * representation for histories of at most 32 pairs, else the two-loop recursion. */
static void kdirection(kern_t *k, const float *g, float *q, float *p)
{
    const int D = k->D;
    for (int j = 0; j < D; ++j) q[j] = g[j];
    if (k->h > 0 && k->compact) {
        kpush_compact(k, k->pending, g);
        kdirection_compact(k, g, q);
    } else if (k->h > 0) {
        for (int i = k->h - 1; i >= 0; --i) {
            int sl = (k->head + i) % k->hist;
            const float *si = k->ringS + (int64_t)sl * D, *yi = k->ringY + (int64_t)sl * D;
            f2_t a = f2_mul(k->rho[sl], kdot_pair(k, si, q));
            for (int j = 0; j < D; ++j) q[j] = fmaf(-a.lo, yi[j], fmaf(-a.hi, yi[j], q[j]));
            k->alph[i] = a;
        }
        f2_t gam = f2_div(k->last_sy, f2_norm(f2_add(k->last_yy, k->eps2)));
        for (int j = 0; j < D; ++j) q[j] = fmaf(q[j], gam.lo, q[j] * gam.hi);
        for (int i = 0; i < k->h; ++i) {
            int sl = (k->head + i) % k->hist;
            const float *si = k->ringS + (int64_t)sl * D, *yi = k->ringY + (int64_t)sl * D;
            f2_t be = f2_mul(k->rho[sl], kdot_pair(k, yi, q));
            f2_t coef = f2_sub(k->alph[i], be);
            for (int j = 0; j < D; ++j) q[j] = fmaf(coef.lo, si[j], fmaf(coef.hi, si[j], q[j]));
        }
    }
    for (int j = 0; j < D; ++j) p[j] = j < k->nslots ? -q[j] : 0.0f;
}

/* The fused kernel's search direction for a given history, for tests of its arithmetic:
 * npairs (s, y) pairs (rows of 32 spl floats, oldest first) go through the kernel's
 * history ring of `hist` pairs (the oldest dropped when it is full) and its updates,
 * then p = -H g.  two_loop = 1 forces the two-loop recursion (the kernel's choice for
 * histories above 32 pairs); otherwise the kernel's choice for `hist`.  nslots slots are
 * active (the rest of each row is ignored and p is 0 there). */
void sro_direction_f32(int hist, int two_loop, int spl, int nslots, int npairs, const float *S, const float *Y,
                       const float *g, double eps, float *p)
{
    kern_t K;
    memset(&K, 0, sizeof(K));
    K.spl = spl; K.D = 32 * spl; K.nslots = nslots; K.K = nslots; K.hist = hist;
    K.compact = !two_loop && hist <= 32;
    K.split = K.compact && hist <= 16 && spl == 1;
    K.ringS = calloc((size_t)hist * K.D, sizeof(float));
    K.ringY = calloc((size_t)hist * K.D, sizeof(float));
    K.rho = calloc((size_t)hist, sizeof(f2_t));
    K.alph = calloc((size_t)hist, sizeof(f2_t));
    K.cd = calloc((size_t)hist, sizeof(f2_t));
    K.Rinv = calloc((size_t)hist * hist, sizeof(f2_t));
    K.YY = calloc((size_t)hist * hist, sizeof(f2_t));
    K.eps2 = f2_of_double(eps);
    float *q = malloc(sizeof(float) * (size_t)K.D);
    for (int n = 0; n < npairs; ++n) {
        int slot;
        if (K.h < K.hist) { slot = (K.head + K.h) % K.hist; K.h++; }
        else { slot = K.head; K.head = (K.head + 1) % K.hist; }
        const float *sv = S + (int64_t)n * K.D, *yv = Y + (int64_t)n * K.D;
        for (int j = 0; j < K.D; ++j) {
            K.ringS[(int64_t)slot * K.D + j] = j < nslots ? sv[j] : 0.0f;
            K.ringY[(int64_t)slot * K.D + j] = j < nslots ? yv[j] : 0.0f;
        }
        if (K.compact) {
            /* each pair's update runs before the direction that follows it */
            K.pending = slot;
            if (n + 1 < npairs) kpush_compact(&K, slot, g);
        } else {
            K.last_sy = kdot_pair(&K, K.ringY + (int64_t)slot * K.D, K.ringS + (int64_t)slot * K.D);
            K.last_yy = kdot_pair(&K, K.ringY + (int64_t)slot * K.D, K.ringY + (int64_t)slot * K.D);
            K.rho[slot] = f2_div(f2_mk(1.0f, 0.0f), f2_norm(f2_add(K.last_sy, K.eps2)));
        }
    }
    kdirection(&K, g, q, p);
    free(q); free(K.ringS); free(K.ringY); free(K.rho); free(K.alph); free(K.cd); free(K.Rinv); free(K.YY);
}

/* One problem's fit: the closure and dots of the chosen arithmetic behind the
 * reference's control flow.  kevals counts the closures the fused kernel
 * evaluates: it reuses phi(0), phi(alpha_lo) and the accepted trial point, which
 * the reference evaluates again (bit-identical, both being deterministic). */
typedef struct {
    problem_t *P;
    kern_t *k;          /* dot_mode 2 */
    int mode;
    double eps;
    int64_t D;          /* vector length */
    long kevals;
} fit_t;

static float fit_closure(fit_t *F, const float *x, float *g, int counted)
{
    if (F->mode == 2) {
        if (counted) F->kevals++;
        return kclosure(F->P, F->k, x, g);
    }
    return closure_f32(F->P, x, g);
}

static double dotv(const fit_t *F, const float *a, const float *b, int64_t D)
{
    if (F->mode == 0) {
        float s = 0.0f;
        for (int64_t j = 0; j < D; ++j) s += a[j] * b[j];
        return (double)s;
    }
    double s = 0.0;
    for (int64_t j = 0; j < D; ++j) s += (double)a[j] * (double)b[j];
    return s;
}

static float dotf(const fit_t *F, const float *a, const float *b)
{
    if (F->mode == 2) return kdot_f2(F->k, a, b);
    return (float)dotv(F, a, b, F->D);
}

/* Two-loop recursion (lbfgs_batch.py:65-103) in dot_mode 0 / 1; writes p = -z. */
static void direction(const fit_t *F, const float *g, float *const *S, float *const *Yh, int h,
                      int64_t D, float *q, float *p, double *alph)
{
    for (int64_t j = 0; j < D; ++j) q[j] = g[j];
    if (h == 0) { for (int64_t j = 0; j < D; ++j) p[j] = -q[j]; return; }
    if (F->mode == 0) {
        float eps = (float)F->eps;
        for (int i = h - 1; i >= 0; --i) {
            float rho = 1.0f / ((float)dotv(F, Yh[i], S[i], D) + eps);
            float al = rho * (float)dotv(F, S[i], q, D);
            for (int64_t j = 0; j < D; ++j) q[j] = q[j] - al * Yh[i][j];
            alph[i] = al;
        }
        float gam = (float)dotv(F, S[h - 1], Yh[h - 1], D) / ((float)dotv(F, Yh[h - 1], Yh[h - 1], D) + eps);
        for (int64_t j = 0; j < D; ++j) q[j] = gam * q[j];
        for (int i = 0; i < h; ++i) {
            float rho = 1.0f / ((float)dotv(F, Yh[i], S[i], D) + eps);
            float be = rho * (float)dotv(F, Yh[i], q, D);
            float coef = (float)alph[i] - be;
            for (int64_t j = 0; j < D; ++j) q[j] = q[j] + S[i][j] * coef;
        }
    } else {
        double eps = F->eps;
        for (int i = h - 1; i >= 0; --i) {
            double rho = 1.0 / (dotv(F, Yh[i], S[i], D) + eps);
            double al = rho * dotv(F, S[i], q, D);
            for (int64_t j = 0; j < D; ++j) q[j] = (float)((double)q[j] - al * (double)Yh[i][j]);
            alph[i] = al;
        }
        double gam = dotv(F, S[h - 1], Yh[h - 1], D) / (dotv(F, Yh[h - 1], Yh[h - 1], D) + eps);
        for (int64_t j = 0; j < D; ++j) q[j] = (float)(gam * (double)q[j]);
        for (int i = 0; i < h; ++i) {
            double rho = 1.0 / (dotv(F, Yh[i], S[i], D) + eps);
            double be = rho * dotv(F, Yh[i], q, D);
            for (int64_t j = 0; j < D; ++j) q[j] = (float)((double)q[j] + (double)S[i][j] * (alph[i] - be));
        }
    }
    for (int64_t j = 0; j < D; ++j) p[j] = -q[j];
}

static void trial_point(const float *x, const float *p, float al, float *xt, int64_t D)
{
    for (int64_t j = 0; j < D; ++j) xt[j] = x[j] + al * p[j];
}

/* Zoom (lbfgs_batch.py:204-264) for one problem.  phi0/dphi0 are re-evaluated
 * by the reference at x; they equal the bracket phase's values.  lo_counted: the
 * fused kernel evaluates phi(alpha_lo) itself (alpha_lo = 0 and x + 0 p differs
 * from x in its bits); otherwise it holds that point already. */
static float zoom(fit_t *F, const float *x, const float *p, float lo, float hi,
                  float phi0, float dphi0, float *xt, float *gt, int lo_counted)
{
    const float c1 = 1e-4f, c2 = 0.9f;
    const int64_t D = F->D;
    trial_point(x, p, lo, xt, D);
    float phi_lo = fit_closure(F, xt, gt, lo_counted);
    float alpha = 0.0f;
    int zdone = 0;
    for (int it = 0; it < 10; ++it) {
        if (zdone) break;
        float aj = (lo + hi) / 2.0f;
        trial_point(x, p, aj, xt, D);
        float phij = fit_closure(F, xt, gt, 1);
        float dphij = dotf(F, gt, p);
        int bad = (phij > phi0 + (c1 * aj) * dphi0) || (phij >= phi_lo);
        int good = fabsf(dphij) <= c2 * fabsf(dphi0);
        if (good) { alpha = aj; zdone = 1; }
        if (!zdone) {
            float thi = bad ? aj : hi;
            int cond3 = dphij * (thi - lo) >= 0.0f;
            hi = (!bad && cond3) ? lo : thi;
            if (!bad) { lo = aj; phi_lo = phij; }
        }
        if (!zdone && fabsf(hi - lo) < 1e-9f) { alpha = aj; zdone = 1; }
    }
    if (!zdone) alpha = lo;
    return alpha;
}

/* Strong-Wolfe bracketing (lbfgs_batch.py:138-202) for one problem.  *known: the
 * returned step was evaluated (found by the bracket or the zoom), not the next
 * extrapolated step of an unfinished bracket. */
static float strong_wolfe(fit_t *F, const float *x, const float *p, float phi0,
                          float dphi0, int ls_max, float *xt, float *gt, int *known)
{
    const float c1 = 1e-4f, c2 = 0.9f, amax = 20.0f;
    const int64_t D = F->D;
    float a_prev = 0.0f, phi_prev = phi0, a_i = 1.0f, fin = 0.0f;
    int done = 0;
    for (int i = 0; i < ls_max; ++i) {
        if (done) break;
        trial_point(x, p, a_i, xt, D);
        float phii = fit_closure(F, xt, gt, 1);
        float dphii = dotf(F, gt, p);
        int bad = (phii > phi0 + (c1 * a_i) * dphi0) || (i > 0 && phii >= phi_prev);
        int good = fabsf(dphii) <= c2 * fabsf(dphi0);
        int passed = dphii >= 0.0f;
        if (good) { fin = a_i; done = 1; }
        else if (bad || passed) {
            float lo = bad ? a_prev : a_i, hi = bad ? a_i : a_prev;
            int lo_counted = 0;
            if (F->mode == 2 && bad && i == 0) {  /* alpha_lo = 0: is x + 0 p bit-identical to x? */
                for (int j = 0; j < F->k->K; ++j) {
                    float z = x[j] + 0.0f * p[j];
                    if (memcmp(&z, &x[j], sizeof(float)) != 0) lo_counted = 1;
                }
            }
            fin = zoom(F, x, p, lo, hi, phi0, dphi0, xt, gt, lo_counted);
            done = 1;
        }
        if (!done) {
            a_prev = a_i; phi_prev = phii;
            a_i = a_i + (amax - a_i) * 0.8f;
        }
    }
    *known = done;
    return done ? fin : a_i;
}

/* Armijo backtracking (lbfgs_batch.py:105-136) for one problem: alpha halves
 * after every failed try, including the last. */
static float backtracking(fit_t *F, const float *x, const float *p, float fk,
                          const float *gk, int ls_max, float *xt, float *gt, int *known)
{
    float gfp = dotf(F, gk, p);
    float al = 1.0f;
    for (int t = 0; t < ls_max; ++t) {
        trial_point(x, p, al, xt, F->D);
        float ft = fit_closure(F, xt, gt, 1);
        if (ft <= fk + (1e-4f * al) * gfp) { *known = 1; return al; }
        al = al * 0.5f;
    }
    *known = 0;
    return al;
}

static void final_forward(const float *X, int64_t N, int64_t nx, problem_t *P, const float *cvals, float *Yrow,
                          int kernel_math)
{
    for (int64_t n = 0; n < N; ++n) {
        for (int64_t k = 0; k < P->M; ++k) {
            int64_t op = P->ops[k];
            int ar = arity_of(op);
            float a = 0, bb = 0;
            if (op != OP_NO_OP) {
                if (ar >= 1) a = P->val[P->ch[k * 2]];
                if (ar == 2) bb = P->val[P->ch[k * 2 + 1]];
            }
            P->val[k] = kernel_math ? fwd_kf32(op, a, bb, cvals[k], X + n * nx, nx)
                                    : fwd_f32(op, a, bb, cvals[k], X + n * nx, nx);
        }
        Yrow[n] = P->val[P->root];
    }
}

/* One problem in dot_mode 0 / 1 (reference slot vectors, D = M). */
static void fit_problem_ref(problem_t *P, fit_t *F, const float *C_init, int max_iter, int history, double tol,
                            int ls_kind, int ls_max, float *C_out, int *iters_out, float *loss_out)
{
    const int64_t D = P->M;
    const int dot_mode = F->mode;
    size_t vb = sizeof(float) * (size_t)D;
    float *x = malloc(vb), *g = malloc(vb), *p = malloc(vb), *q = malloc(vb), *xt = malloc(vb),
          *gt = malloc(vb), *gn = malloc(vb);
    float **S = malloc(sizeof(float *) * (size_t)(history + 1)), **Yh = malloc(sizeof(float *) * (size_t)(history + 1));
    double *alph = malloc(sizeof(double) * (size_t)(history + 1));
    for (int i = 0; i <= history; ++i) { S[i] = malloc(vb); Yh[i] = malloc(vb); }
    int h = 0, it = 0, known = 0;
    memcpy(x, C_init, vb);
    float f = fit_closure(F, x, g, 1);
    for (it = 0; it < max_iter; ++it) {
        double gn2 = 0.0;
        if (dot_mode == 0) { float s = 0.0f; for (int64_t j = 0; j < D; ++j) s += g[j] * g[j]; gn2 = (double)s; }
        else for (int64_t j = 0; j < D; ++j) gn2 += (double)g[j] * (double)g[j];
        double gnorm = dot_mode == 0 ? (double)sqrtf((float)gn2) : sqrt(gn2);
        if (gnorm < (dot_mode == 0 ? (double)(float)tol : tol)) break;
        direction(F, g, S, Yh, h, D, q, p, alph);
        float al;
        if (ls_kind == 0) {
            float dphi0 = dotf(F, g, p);
            al = strong_wolfe(F, x, p, f, dphi0, ls_max, xt, gt, &known);
        } else {
            al = backtracking(F, x, p, f, g, ls_max, xt, gt, &known);
        }
        /* s = alpha p ; x += s ; closure at the new x (lbfgs_batch.py:305-312) */
        float *s_new = S[h], *y_new = Yh[h];
        for (int64_t j = 0; j < D; ++j) { s_new[j] = al * p[j]; x[j] = x[j] + s_new[j]; }
        float fn = fit_closure(F, x, gn, 1);
        for (int64_t j = 0; j < D; ++j) y_new[j] = gn[j] - g[j];
        if (h < history) h++;
        else {  /* drop the oldest pair; the slot just written becomes the newest */
            float *s0 = S[0], *y0 = Yh[0];
            for (int i = 0; i < history; ++i) { S[i] = S[i + 1]; Yh[i] = Yh[i + 1]; }
            S[history] = s0; Yh[history] = y0;
        }
        memcpy(g, gn, vb);
        f = fn;
    }
    memcpy(C_out, x, vb);
    *iters_out = it;
    *loss_out = f;
    for (int i = 0; i <= history; ++i) { free(S[i]); free(Yh[i]); }
    free(S); free(Yh); free(alph);
    free(x); free(g); free(p); free(q); free(xt); free(gt); free(gn);
}

/* One problem in dot_mode 2 (the fused kernel's slot vectors, history ring and
 * end-of-fit rules).  C_out gets the fitted constants in their tape slots and
 * C_init in the others (NaN everywhere when the virtual slot was poisoned). */
static void fit_problem_kernel(problem_t *P, fit_t *F, const float *C_init, int max_iter, double tol,
                               int ls_kind, int ls_max, float *C_out, int *iters_out, float *loss_out)
{
    kern_t *k = F->k;
    const int D = k->D;
    size_t vb = sizeof(float) * (size_t)D;
    float *x = calloc((size_t)D, sizeof(float)), *g = malloc(vb), *p = malloc(vb), *q = malloc(vb),
          *xt = malloc(vb), *gt = malloc(vb), *gn = malloc(vb), *sv = malloc(vb), *yv = malloc(vb);
    const float tolf = (float)tol;
    int it = 0, known = 0;
    for (int j = 0; j < k->K; ++j) x[j] = C_init[k->slot_node[j]];
    float f = fit_closure(F, x, g, 1);
    for (it = 0; it < max_iter;) {
        if (sqrtf(kdot_f2(k, g, g)) < tolf) break;
        kdirection(k, g, q, p);
        float al;
        if (ls_kind == 0) al = strong_wolfe(F, x, p, f, kdot_f2(k, g, p), ls_max, xt, gt, &known);
        else al = backtracking(F, x, p, f, g, ls_max, xt, gt, &known);
        for (int j = 0; j < D; ++j) {
            sv[j] = j < k->nslots ? al * p[j] : 0.0f;
            x[j] = x[j] + sv[j];
        }
        float fn = fit_closure(F, x, gn, !known);
        if (k->has_virtual && isnan(sv[k->K])) k->poison = 1;
        int slot;
        if (k->h < k->hist) { slot = (k->head + k->h) % k->hist; k->h++; }
        else { slot = k->head; k->head = (k->head + 1) % k->hist; }
        for (int j = 0; j < D; ++j) yv[j] = j < k->nslots ? gn[j] - g[j] : 0.0f;
        memcpy(k->ringS + (int64_t)slot * D, sv, vb);
        memcpy(k->ringY + (int64_t)slot * D, yv, vb);
        if (k->compact) {
            k->pending = slot;  /* the kernel updates the compact history with the next direction */
        } else {
            k->last_sy = kdot_pair(k, yv, sv);
            k->last_yy = kdot_pair(k, yv, yv);
            k->rho[slot] = f2_div(f2_mk(1.0f, 0.0f), f2_norm(f2_add(k->last_sy, k->eps2)));
        }
        memcpy(g, gn, vb);
        f = fn;
        ++it;
        /* every real slot NaN and the others poisoned: nothing changes any more */
        int allnan = 1;
        for (int j = 0; j < k->K; ++j) if (!isnan(x[j])) allnan = 0;
        if (k->K > 0 && allnan && (k->poison || !k->has_virtual)) { it = max_iter; break; }
    }
    for (int64_t m = 0; m < P->M; ++m) C_out[m] = k->poison ? (float)NAN : C_init[m];
    for (int j = 0; j < k->K; ++j) C_out[k->slot_node[j]] = x[j];
    *iters_out = it;
    *loss_out = f;
    free(x); free(g); free(p); free(q); free(xt); free(gt); free(gn); free(sv); free(yv);
}

/* Runs optimize() for problems [0, B).  Layouts: X (N,nx), Y (B,N) or NULL,
 * ops (B,M), ch (B,M,2), C_init/C_out (B,M), Y_out (B,N) or NULL.
 * iters_out/evals_out/loss_out (B) may be NULL; iters_out[b] = -code for a
 * problem whose closures raised an error.  dot_mode 2 takes the fused kernel's
 * launch shape (warps W, points per lane V) and slot registers per lane (spl:
 * 1, 2 or 4, from the batch's largest constant count); its evals are the kernel's
 * closure count.  Returns 0 or an error code. */
int sro_optimize_shape_f32(const float *X, int64_t N, int64_t nx, const float *Y, const int64_t *ops,
                           const int64_t *ch, const float *C_init, int64_t B, int64_t M, int max_iter,
                           int history, double tol, int ls_kind, int ls_max, int dot_mode, int warps,
                           int points_per_lane, int spl, float *C_out, float *Y_out, int *iters_out,
                           long *evals_out, float *loss_out)
{
    int err_all = 0;
    if (dot_mode == 2 && (warps < 1 || points_per_lane < 1 || spl < 1 || history < 1)) return -1;
    _Pragma("omp parallel for schedule(dynamic, 1)")
    for (int64_t b = 0; b < B; ++b) {
        problem_t P;
        memset(&P, 0, sizeof(P));
        P.X = X; P.N = N; P.nx = nx; P.Y = Y ? Y + b * N : NULL;
        P.ops = ops + b * M; P.ch = ch + b * M * 2; P.M = M;
        int64_t cnt = 0;
        for (int64_t k = 0; k < M; ++k) cnt += P.ops[k] != OP_NO_OP;
        P.root = cnt > 0 ? cnt - 1 : 0;
        P.val = (float *)malloc(sizeof(float) * (size_t)M);
        P.adj = (float *)malloc(sizeof(float) * (size_t)M);
        P.gacc = (double *)malloc(sizeof(double) * (size_t)M);
        P.dmode = dot_mode == 1;
        fit_t F;
        memset(&F, 0, sizeof(F));
        F.P = &P; F.mode = dot_mode; F.eps = 1e-10; F.D = M;
        int it = 0;
        float f = 0.0f;
        float *cout = C_out + b * M;
        if (dot_mode == 2) {
            kern_t K;
            memset(&K, 0, sizeof(K));
            K.W = warps; K.V = points_per_lane; K.spl = spl; K.D = 32 * spl;
            K.objective = Y ? 0 : 1;
            K.slot_of = malloc(sizeof(int) * (size_t)M);
            K.slot_node = malloc(sizeof(int64_t) * (size_t)M);
            for (int64_t k = 0; k < M; ++k) {
                K.slot_of[k] = -1;
                if (k <= P.root && P.ops[k] == OP_LEARNABLE) { K.slot_node[K.K] = k; K.slot_of[k] = K.K++; }
            }
            K.has_virtual = M > K.K;
            K.nslots = K.K + K.has_virtual;
            int RW = 32 * K.V;
            K.vals = malloc(sizeof(float) * (size_t)RW * (size_t)M);
            K.adjs = malloc(sizeof(float) * (size_t)RW * (size_t)M);
            K.gl = malloc(sizeof(float) * (size_t)RW * (size_t)(K.K > 0 ? K.K : 1));
            K.red_g = malloc(sizeof(f2_t) * (size_t)K.W * (size_t)(K.K > 0 ? K.K : 1));
            K.red_l = malloc(sizeof(f2_t) * (size_t)K.W);
            K.lane_err = calloc((size_t)32 * K.W, sizeof(int));
            K.hist = history;
            K.ringS = calloc((size_t)history * K.D, sizeof(float));
            K.ringY = calloc((size_t)history * K.D, sizeof(float));
            K.rho = calloc((size_t)history, sizeof(f2_t));
            K.alph = calloc((size_t)history, sizeof(f2_t));
            K.compact = history <= 32;
            K.split = K.compact && history <= 16 && spl == 1;
            K.cd = calloc((size_t)history, sizeof(f2_t));
            K.Rinv = K.compact ? calloc((size_t)history * history, sizeof(f2_t)) : NULL;
            K.YY = K.compact ? calloc((size_t)history * history, sizeof(f2_t)) : NULL;
            K.eps2 = f2_of_double(F.eps);
            F.k = &K; F.D = K.D;
            if (K.nslots <= K.D)
                fit_problem_kernel(&P, &F, C_init + b * M, max_iter, tol, ls_kind, ls_max, cout, &it, &f);
            else
                P.err = -1;
            for (int t = 0; t < 32 * K.W; ++t) if (K.lane_err[t] > P.err) P.err = K.lane_err[t];
            free(K.slot_of); free(K.slot_node); free(K.vals); free(K.adjs); free(K.gl); free(K.red_g);
            free(K.red_l); free(K.lane_err); free(K.ringS); free(K.ringY); free(K.rho); free(K.alph);
            free(K.cd); free(K.Rinv); free(K.YY);
        } else {
            fit_problem_ref(&P, &F, C_init + b * M, max_iter, history, tol, ls_kind, ls_max, cout, &it, &f);
        }
        if (iters_out) iters_out[b] = it;
        if (Y_out) final_forward(X, N, nx, &P, cout, Y_out + b * N, dot_mode == 2);
        if (loss_out) loss_out[b] = f;
        if (evals_out) evals_out[b] = dot_mode == 2 ? F.kevals : P.n_evals;
        if (P.err && iters_out) iters_out[b] = -P.err;
        if (P.err) {
            _Pragma("omp critical")
            { if (!err_all) err_all = P.err; }
        }
        free(P.val); free(P.adj); free(P.gacc);
    }
    return err_all;
}

int sro_optimize_f32(const float *X, int64_t N, int64_t nx, const float *Y, const int64_t *ops,
                     const int64_t *ch, const float *C_init, int64_t B, int64_t M, int max_iter,
                     int history, double tol, int ls_kind, int ls_max, int dot_mode,
                     float *C_out, float *Y_out, int *iters_out, long *evals_out, float *loss_out)
{
    return sro_optimize_shape_f32(X, N, nx, Y, ops, ch, C_init, B, M, max_iter, history, tol, ls_kind, ls_max,
                                  dot_mode, 1, 1, 1, C_out, Y_out, iters_out, evals_out, loss_out);
}

int sro_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Threads of the parallel loops from now on (a launcher may have set OMP_NUM_THREADS=1
 * before the OpenMP runtime was loaded); returns the count now in effect. */
int sro_set_num_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
    return sro_num_threads();
}

/* ---- grammar sampling and infix parsing --------------------------------------------
 * Restates the reference's sampler (src/pcfg_cpu.cpp:10-119, the same derivation as
 * src/pcfg_cuda.cu:10-118) and shunting-yard parsers (src/pcfg_cpu.cpp:121-448).
 * The random numbers are the library's own SplitMix64 stream per expression
 * (Steele, Lea and Flood, OOPSLA 2014), restated here so that the device sampler is
 * checked token for token; the reference draws from curand instead, so against the
 * reference the sampler is checked by frequencies.
 */
#define SRO_HARD_MAX 128

static uint64_t sro_mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static float sro_uniform(uint64_t *s)
{
    *s += 0x9E3779B97F4A7C15ull;
    return (float)((sro_mix64(*s) >> 40) + 1ull) * (1.0f / 16777216.0f);
}

void sro_pcfg_sample(const int32_t *nt_ptr, const float *cum, const int32_t *rhs_ptr, const int32_t *rhs,
                     int32_t n_symbols, int32_t start, int64_t B, int32_t max_len, int32_t max_tries,
                     uint64_t seed, int64_t *out, int64_t *errors)
{
    #pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < B; ++b) {
        uint64_t s = sro_mix64(seed ^ sro_mix64((uint64_t)b + 0x9E3779B97F4A7C15ull));
        int32_t stack[SRO_HARD_MAX];
        int64_t *row = out + b * max_len;
        int err = 0, done = 0, len = 0;
        for (int tr = 0; tr < max_tries && !done && !err; ++tr) {
            int restart = 0, sp = 0;
            len = 0;
            stack[sp++] = start;
            while (sp > 0) {
                const int sym = stack[--sp];
                const int has_rules = (unsigned)sym < (unsigned)n_symbols;
                const int r0 = has_rules ? nt_ptr[sym] : 0;
                const int r1 = has_rules ? nt_ptr[sym + 1] : 0;
                if (r0 != r1) {
                    const float u = sro_uniform(&s);
                    int chosen = -1;
                    for (int r = r0; r < r1; ++r)
                        if (u <= cum[r]) { chosen = r; break; }
                    if (chosen < 0) { err = 304; break; }
                    for (int i = rhs_ptr[chosen + 1] - 1; i >= rhs_ptr[chosen]; --i) {
                        if (sp >= SRO_HARD_MAX) { restart = 1; break; }
                        stack[sp++] = rhs[i];
                    }
                    if (restart) break;
                } else {
                    if (len >= max_len) { restart = 1; break; }
                    row[len++] = sym;
                }
            }
            if (!restart && !err && len > 0) done = 1;
        }
        if (!done && !err) err = 303;
        if (!done) len = 0;
        for (int i = len; i < max_len; ++i) row[i] = OP_NO_OP;
        errors[b] = err;
    }
}

static int sro_precedence(int64_t tok, int64_t lp, int64_t rp)
{
    if (tok == OP_ADD || tok == OP_SUB) return 1;
    if (tok == OP_MUL || tok == OP_DIV) return 2;
    if (tok == OP_POW) return 3;
    if ((tok >= OP_SIN && tok <= OP_FIFTH) || tok == lp || tok == rp) return 4;
    return 0;
}

static int sro_token_arity(int64_t tok)
{
    if (tok >= OP_SIN && tok <= OP_FIFTH) return 1;
    if (tok >= OP_ADD && tok <= OP_POW) return 2;
    return 0;
}

/* prefix = 0: infix -> postfix with the tree check; 1: infix -> prefix.  errors: 0,
 * the reference's 401..408, or -1 / -2 for a token below 0 / at or above the
 * terminal limit (the reference rejects those before parsing). */
void sro_infix_parse(const int64_t *infix, int64_t B, int64_t M, int32_t n_vars, int32_t prefix, int64_t *outp,
                     int64_t *errors)
{
    const int64_t lp = OP_VAR0 + n_vars, rp = lp + 1, limit = rp + 1;
    #pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < B; ++b) {
        const int64_t *in = infix + b * M;
        int64_t *o = outp + b * M;
        int64_t ops[SRO_HARD_MAX], queue[SRO_HARD_MAX];
        int bad = 0, err = 0, len = 0, ended = 0, sp = 0, n_out = 0;
        for (int64_t i = 0; i < M; ++i) {
            if (in[i] < 0) bad = -1;
            else if (in[i] >= limit && bad == 0) bad = -2;
        }
        for (int64_t i = 0; i < M && !err; ++i) {
            if (in[i] == OP_NO_OP) ended = 1;
            else if (ended) err = 408;
            else ++len;
        }
        const int64_t open = prefix ? rp : lp, close = prefix ? lp : rp;
        for (int step = 0; step < len && !err && !bad; ++step) {
            const int64_t tok = in[prefix ? len - 1 - step : step];
            const int pt = sro_precedence(tok, lp, rp);
            if (pt == 0) {
                if (n_out >= SRO_HARD_MAX) { err = 401; break; }
                queue[n_out++] = tok;
            } else if (tok == open) {
                if (sp >= SRO_HARD_MAX) { err = 402; break; }
                ops[sp++] = tok;
            } else if (tok == close) {
                while (sp > 0 && ops[sp - 1] != open) {
                    if (n_out >= SRO_HARD_MAX) { err = 401; break; }
                    queue[n_out++] = ops[--sp];
                }
                if (err) break;
                if (sp == 0) { err = 403; break; }
                --sp;
            } else {
                const int ra = tok == OP_POW || (tok >= OP_SIN && tok <= OP_FIFTH);
                while (sp > 0 && ops[sp - 1] != open) {
                    const int ptop = sro_precedence(ops[sp - 1], lp, rp);
                    const int pop = prefix ? (ra ? ptop >= pt : ptop > pt) : (ra ? ptop > pt : ptop >= pt);
                    if (!pop) break;
                    if (n_out >= SRO_HARD_MAX) { err = 401; break; }
                    queue[n_out++] = ops[--sp];
                }
                if (err) break;
                if (sp >= SRO_HARD_MAX) { err = 402; break; }
                ops[sp++] = tok;
            }
        }
        while (!err && !bad && sp > 0) {
            if (ops[sp - 1] == open) { err = 403; break; }
            if (n_out >= SRO_HARD_MAX) { err = 401; break; }
            queue[n_out++] = ops[--sp];
        }
        if (!prefix && !err && !bad && n_out > 0) {
            int depth = 0;
            for (int i = 0; i < n_out && !err; ++i) {
                if (sro_precedence(queue[i], lp, rp) == 0) {
                    ++depth;
                } else {
                    const int ar = sro_token_arity(queue[i]);
                    if (depth < ar) err = ar == 1 ? 404 : 405;
                    depth = depth - ar + 1;
                }
            }
            if (!err && depth != 1) err = 407;
        }
        if (err || bad) n_out = 0;
        for (int64_t i = 0; i < M; ++i)
            o[i] = i < n_out ? queue[prefix ? n_out - 1 - i : i] : OP_NO_OP;
        errors[b] = bad ? bad : err;
    }
}

/* Child table of postfix rows (src/pcfg_cpu.cpp:1066-1142): ch (B, M, 2), -1 where a
 * node has no such child; errors 0 or 404..408. */
void sro_postfix_children(const int64_t *post, int64_t B, int64_t M, int64_t *ch, int64_t *errors)
{
    #pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < B; ++b) {
        const int64_t *row = post + b * M;
        int64_t *c = ch + b * M * 2;
        int32_t st[SRO_HARD_MAX];
        int sp = 0, ended = 0, len = 0, err = 0;
        for (int64_t i = 0; i < 2 * M; ++i) c[i] = -1;
        for (int64_t i = 0; i < M && !err; ++i) {
            const int64_t t = row[i];
            if (t == OP_NO_OP) { ended = 1; continue; }
            ++len;
            if (ended) { err = 408; break; }
            const int ar = sro_token_arity(t);
            if (ar == 1) {
                if (sp < 1) { err = 404; break; }
                c[2 * i] = st[--sp];
            } else if (ar == 2) {
                if (sp < 2) { err = 405; break; }
                c[2 * i + 1] = st[--sp];
                c[2 * i] = st[--sp];
            }
            if (sp >= SRO_HARD_MAX) { err = 406; break; }
            st[sp++] = (int32_t)i;
        }
        if (!err && len > 0 && sp != 1) err = 407;
        errors[b] = err;
    }
}

/* ---- the remaining notation conversions ------------------------------------------
 * postfix -> infix (src/pcfg_cpu.cpp:449-635), prefix -> infix (637-811), prefix <->
 * postfix (812-993) and the parent table of prefix rows (995-1064).  Symbols are
 * checked first as the reference's wrappers do (src/pcfg.cpp:644-657): -1 for a symbol
 * below 0, -2 for one at or above VAR_START_ID + n_vars.  A row with an error is left
 * all NO_OP (parents: all -1); the reference raises for the batch instead. */
static int sro_functional(int64_t op)
{
    return (op >= OP_SIN && op <= OP_LOG) || (op >= OP_SQRT && op <= OP_NEG);
}

static int sro_symbols(const int64_t *row, int64_t M, int64_t n_ops)
{
    int flag = 0;
    for (int64_t i = 0; i < M; ++i) {
        if (row[i] < 0) return -1;
        if (row[i] >= n_ops) flag = -2;
    }
    return flag;
}

/* Shape of a row read from the right (postfix) or from the left (prefix): its length,
 * 509 for a token after the padding, 508 for several roots. */
static int sro_shape(const int64_t *row, int64_t M, int from_right, int *len)
{
    int started = 0, ended = 0, balance = 0, roots = 0;
    *len = 0;
    for (int64_t s = 0; s < M; ++s) {
        const int64_t t = row[from_right ? M - 1 - s : s];
        if (t == OP_NO_OP) {
            if (from_right) { if (started) return 509; }
            else ended = 1;
            continue;
        }
        if (!from_right && ended) return 509;
        started = 1;
        ++*len;
        balance += sro_token_arity(t) - 1;
        if (balance == -1) ++roots;
    }
    return roots > 1 ? 508 : 0;
}

void sro_postfix_to_infix(const int64_t *post, int64_t B, int64_t M, int32_t n_vars, int64_t *infix, int64_t M_out,
                          int64_t *errors)
{
    const int64_t lp = OP_VAR0 + n_vars, rp = lp + 1;
    #pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < B; ++b) {
        const int64_t *row = post + b * M;
        int64_t *o = infix + b * M_out;
        int64_t buf[3 * SRO_HARD_MAX];
        int32_t ops[SRO_HARD_MAX];
        int waiting_left[SRO_HARD_MAX];
        int top = 3 * SRO_HARD_MAX - 1, sp = 0, len = 0, err;
        for (int64_t i = 0; i < M_out; ++i) o[i] = OP_NO_OP;
        err = sro_symbols(row, M, OP_VAR0 + n_vars);
        if (!err) err = sro_shape(row, M, 1, &len);
        for (int k = len - 1; k >= 0 && !err; --k) {   /* the rendering is built from its end */
            const int64_t t = row[k];
            if (sro_token_arity(t) == 0) {
                if (top < 0) { err = 504; break; }
                buf[top--] = t;
                int done = 1;
                while (done && sp > 0 && !err) {
                    const int32_t parent = ops[sp - 1];
                    if (sro_token_arity(parent) == 1) {
                        if (sro_functional(parent)) {
                            if (top - 1 < 0) { err = 504; break; }
                            buf[top--] = lp;
                            buf[top--] = parent;
                        } else {
                            if (top < 0) { err = 504; break; }
                            buf[top--] = lp;
                        }
                        --sp;
                    } else if (!waiting_left[sp - 1]) {
                        if (top < 0) { err = 504; break; }
                        buf[top--] = parent;
                        waiting_left[sp - 1] = 1;
                        done = 0;
                    } else {
                        if (top < 0) { err = 504; break; }
                        buf[top--] = lp;
                        --sp;
                    }
                }
            } else {
                if (sp >= SRO_HARD_MAX) { err = 504; break; }
                ops[sp] = (int32_t)t;
                waiting_left[sp] = 0;
                if (sro_token_arity(t) == 1 && !sro_functional(t)) {
                    if (top < 0) { err = 504; break; }
                    buf[top--] = t;
                }
                if (top < 0) { err = 504; break; }
                buf[top--] = rp;
                ++sp;
            }
        }
        if (!err && sp > 0) err = sro_token_arity(ops[sp - 1]) == 1 ? 505 : 506;
        if (!err && len > 0) {
            const int n = 3 * SRO_HARD_MAX - 1 - top;
            if (n > M_out) err = 501;
            else for (int i = 0; i < n; ++i) o[i] = buf[top + 1 + i];
        }
        errors[b] = err;
    }
}

void sro_prefix_to_infix(const int64_t *pre, int64_t B, int64_t M, int32_t n_vars, int64_t *infix, int64_t M_out,
                         int64_t *errors)
{
    const int64_t lp = OP_VAR0 + n_vars, rp = lp + 1;
    #pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < B; ++b) {
        const int64_t *row = pre + b * M;
        int64_t *o = infix + b * M_out;
        int32_t ops[SRO_HARD_MAX];
        int waiting_right[SRO_HARD_MAX];
        int64_t n = 0;
        int sp = 0, len = 0, err;
        for (int64_t i = 0; i < M_out; ++i) o[i] = OP_NO_OP;
        err = sro_symbols(row, M, OP_VAR0 + n_vars);
        if (!err) err = sro_shape(row, M, 0, &len);
        for (int k = 0; k < len && !err; ++k) {       /* left to right */
            const int64_t t = row[k];
            const int ar = sro_token_arity(t);
            if (ar == 0) {
                if (n >= M_out) { err = 501; break; }
                o[n++] = t;
                int done = 1;
                while (done && sp > 0 && !err) {
                    const int32_t parent = ops[sp - 1];
                    if (sro_token_arity(parent) == 1) {
                        if (n >= M_out) { err = 501; break; }
                        o[n++] = rp;
                        if (!sro_functional(parent)) {
                            if (n >= M_out) { err = 501; break; }
                            o[n++] = parent;
                        }
                        --sp;
                    } else if (!waiting_right[sp - 1]) {
                        if (n >= M_out) { err = 501; break; }
                        o[n++] = parent;
                        waiting_right[sp - 1] = 1;
                        done = 0;
                    } else {
                        if (n >= M_out) { err = 501; break; }
                        o[n++] = rp;
                        --sp;
                    }
                }
            } else {
                if (sp >= SRO_HARD_MAX) { err = 504; break; }
                ops[sp] = (int32_t)t;
                waiting_right[sp] = 0;
                if (ar == 1 && sro_functional(t)) {
                    if (n + 2 > M_out) { err = 501; break; }
                    o[n++] = t;
                    o[n++] = lp;
                } else {
                    if (n >= M_out) { err = 501; break; }
                    o[n++] = lp;
                }
                ++sp;
            }
        }
        if (!err && sp > 0) err = sro_token_arity(ops[sp - 1]) == 1 ? 505 : 506;
        if (err) for (int64_t i = 0; i < M_out; ++i) o[i] = OP_NO_OP;
        errors[b] = err;
    }
}

/* from_prefix = 1: prefix -> postfix; 0: postfix -> prefix. */
void sro_prefix_reorder(const int64_t *in, int64_t B, int64_t M, int32_t n_vars, int32_t from_prefix, int64_t *out,
                        int64_t *errors)
{
    #pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < B; ++b) {
        const int64_t *row = in + b * M;
        int64_t *o = out + b * M;
        int32_t node[SRO_HARD_MAX], missing[SRO_HARD_MAX];
        int sp = 0, n = 0, balance = 0, roots = 0, seen = 0, err;
        for (int64_t i = 0; i < M; ++i) o[i] = OP_NO_OP;
        err = sro_symbols(row, M, OP_VAR0 + n_vars);
        for (int64_t s = 0; s < M && !err; ++s) {
            const int64_t i = from_prefix ? s : M - 1 - s;
            const int64_t t = row[i];
            if (t == OP_NO_OP) {
                if (from_prefix) seen = 1;
                else if (seen) err = 509;
                continue;
            }
            if (from_prefix && seen) { err = 509; break; }
            if (!from_prefix) seen = 1;
            const int ar = sro_token_arity(t);
            balance += ar - 1;
            if (balance == -1) ++roots;
            if (sp >= SRO_HARD_MAX) { err = 504; break; }
            node[sp] = (int32_t)i;
            missing[sp++] = ar;
            while (sp > 0 && missing[sp - 1] == 0) {
                --sp;
                if (n >= M) { err = from_prefix ? 502 : 503; break; }
                o[n++] = row[node[sp]];
                if (sp > 0) --missing[sp - 1];
            }
        }
        if (!err && sp != 0) err = sro_token_arity(row[node[sp - 1]]) == 1 ? 505 : 506;
        if (!err && roots != 1 && n > 0) err = 508;
        if (!err && !from_prefix)
            for (int i = 0, j = n - 1; i < j; ++i, --j) { const int64_t x = o[i]; o[i] = o[j]; o[j] = x; }
        if (err) for (int64_t i = 0; i < M; ++i) o[i] = OP_NO_OP;
        errors[b] = err;
    }
}

void sro_prefix_parent(const int64_t *pre, int64_t B, int64_t M, int32_t n_vars, int64_t *parent, int64_t *errors)
{
    #pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < B; ++b) {
        const int64_t *row = pre + b * M;
        int64_t *par = parent + b * M;
        int32_t st[SRO_HARD_MAX];
        int sp = 0, started = 0, err;
        for (int64_t i = 0; i < M; ++i) par[i] = -1;
        err = sro_symbols(row, M, OP_VAR0 + n_vars);
        for (int64_t i = M - 1; i >= 0 && !err; --i) {   /* from the right */
            const int64_t t = row[i];
            if (t == OP_NO_OP) {
                if (started) err = 408;
                continue;
            }
            started = 1;
            const int ar = sro_token_arity(t);
            if (ar == 1) {
                if (sp < 1) { err = 404; break; }
                par[st[--sp]] = i;
            } else if (ar == 2) {
                if (sp < 2) { err = 405; break; }
                par[st[--sp]] = i;
                par[st[--sp]] = i;
            }
            if (sp >= SRO_HARD_MAX) { err = 406; break; }
            st[sp++] = (int32_t)i;
        }
        if (!err && started && sp != 1) err = 407;
        if (err) for (int64_t i = 0; i < M; ++i) par[i] = -1;
        errors[b] = err;
    }
}

/* ---- the library's float math (sr_fmath.h) -----------------------------------------
 * fn: 0 sin, 1 cos, 2 exp, 3 log. */
static float fmath_eval(int fn, float x)
{
    switch (fn) {
    case 0: return sr_sinf(x);
    case 1: return sr_cosf(x);
    case 2: return sr_expf(x);
    default: return sr_logf(x);
    }
}

static double fmath_ref(int fn, double x)
{
    switch (fn) {
    case 0: return sin(x);
    case 1: return cos(x);
    case 2: return exp(x);
    default: return log(x);
    }
}

void sro_fmath_f32(int fn, int64_t n, const float *x, float *y)
{
    _Pragma("omp parallel for schedule(static)")
    for (int64_t i = 0; i < n; ++i) y[i] = fmath_eval(fn, x[i]);
}

/* Error of fn over the float inputs whose bit patterns are lo, lo + step, ... <= hi,
 * against the double-precision function: out[0] = largest error in units of the last
 * place of the float result (the spacing of floats at the exact value), out[1] = the
 * input where it occurs, out[2] = inputs whose special-value class (NaN, +-inf, +-0)
 * differs from the correctly rounded result, out[3] = inputs checked. */
void sro_fmath_error(int fn, uint32_t lo, uint32_t hi, uint32_t step, double *out)
{
    double worst = 0.0, worst_x = 0.0, bad = 0.0, count = 0.0;
    int64_t n = ((int64_t)hi - (int64_t)lo) / (int64_t)step + 1;
    _Pragma("omp parallel")
    {
        double w = 0.0, wx = 0.0, b = 0.0, c = 0.0;
        _Pragma("omp for schedule(static)")
        for (int64_t i = 0; i < n; ++i) {
            uint32_t bits = lo + (uint32_t)(i * (int64_t)step);
            float x = srm_i2f((int32_t)bits);
            if (x != x) continue;
            float y = fmath_eval(fn, x);
            double v = fmath_ref(fn, (double)x);
            float vf = (float)v;
            c += 1.0;
            int cy = (y != y) ? 1 : isinf(y) ? 2 + (y < 0) : (y == 0.0f) ? 4 : 0;
            int cv = (vf != vf) ? 1 : isinf(vf) ? 2 + (vf < 0) : (vf == 0.0f) ? 4 : 0;
            if (cy != cv) {
                /* a result at the overflow or underflow edge may round either way */
                double ulp0 = ldexp(1.0, -149);
                if (!(cy == 4 && fabs(v) <= ulp0) && !(cv == 4 && fabs((double)y) <= ulp0) &&
                    !(cy >= 2 && cy <= 3 && fabs(v) >= 3.4028234e38) && !(cv >= 2 && cv <= 3 && fabs((double)y) >= 3.4028234e38))
                    b += 1.0;
                continue;
            }
            if (cy) continue;
            int e;
            frexp(v, &e);                               /* |v| in [2^(e-1), 2^e) */
            double ulp = ldexp(1.0, (e - 1 - 23) < -149 ? -149 : e - 1 - 23);
            double err = fabs((double)y - v) / ulp;
            if (err > w) { w = err; wx = (double)x; }
        }
        _Pragma("omp critical")
        {
            if (w > worst) { worst = w; worst_x = wx; }
            bad += b;
            count += c;
        }
    }
    out[0] = worst; out[1] = worst_x; out[2] = bad; out[3] = count;
}
