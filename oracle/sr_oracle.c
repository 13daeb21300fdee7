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

/* ---- optimize(): per-problem batched L-BFGS --------------------------------------
 *
 * Every problem (column) of the reference's LBFGS_batch evolves independently:
 * all reductions are per column and the batch-wide tests (done.all(), all(done)
 * in the line searches) only stop loops early for columns whose state no longer
 * changes.  So this restatement runs one problem at a time, with the reference's
 * D = M parameter slots (non-constant slots get zero gradient, optimization.py:95-97).
 *
 * dot_mode 0 follows the reference arithmetic: float32 vectors, float32 dots
 * summed in slot order, float32 scalars.
 * dot_mode 1 approximates the fused kernel's arithmetic: dots and two-loop scalars
 * in double (s.y, y.y, the alphas, beta, gamma, rho), vector updates rounded once
 * to float, line-search scalars in float, and the per-constant gradient summed
 * over the points in double.  The kernel carries all of these as float pairs
 * (about 44 significant bits; no FP64 in its iteration) and its sums as cascaded
 * float pairs, so the two agree to far below a float ulp on well-conditioned
 * problems.
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

typedef struct { int mode; double eps; } lb_cfg_t;

static double dotv(const lb_cfg_t *cf, const float *a, const float *b, int64_t D)
{
    if (cf->mode == 0) {
        float s = 0.0f;
        for (int64_t j = 0; j < D; ++j) s += a[j] * b[j];
        return (double)s;
    }
    double s = 0.0;
    for (int64_t j = 0; j < D; ++j) s += (double)a[j] * (double)b[j];
    return s;
}

/* Two-loop recursion (lbfgs_batch.py:65-103); writes p = -z. */
static void direction(const lb_cfg_t *cf, const float *g, float *const *S, float *const *Yh, int h,
                      int64_t D, float *q, float *p, double *alph)
{
    for (int64_t j = 0; j < D; ++j) q[j] = g[j];
    if (h == 0) { for (int64_t j = 0; j < D; ++j) p[j] = -q[j]; return; }
    if (cf->mode == 0) {
        float eps = (float)cf->eps;
        for (int i = h - 1; i >= 0; --i) {
            float rho = 1.0f / ((float)dotv(cf, Yh[i], S[i], D) + eps);
            float al = rho * (float)dotv(cf, S[i], q, D);
            for (int64_t j = 0; j < D; ++j) q[j] = q[j] - al * Yh[i][j];
            alph[i] = al;
        }
        float gam = (float)dotv(cf, S[h - 1], Yh[h - 1], D) / ((float)dotv(cf, Yh[h - 1], Yh[h - 1], D) + eps);
        for (int64_t j = 0; j < D; ++j) q[j] = gam * q[j];
        for (int i = 0; i < h; ++i) {
            float rho = 1.0f / ((float)dotv(cf, Yh[i], S[i], D) + eps);
            float be = rho * (float)dotv(cf, Yh[i], q, D);
            float coef = (float)alph[i] - be;
            for (int64_t j = 0; j < D; ++j) q[j] = q[j] + S[i][j] * coef;
        }
    } else {
        double eps = cf->eps;
        for (int i = h - 1; i >= 0; --i) {
            double rho = 1.0 / (dotv(cf, Yh[i], S[i], D) + eps);
            double al = rho * dotv(cf, S[i], q, D);
            for (int64_t j = 0; j < D; ++j) q[j] = (float)((double)q[j] - al * (double)Yh[i][j]);
            alph[i] = al;
        }
        double gam = dotv(cf, S[h - 1], Yh[h - 1], D) / (dotv(cf, Yh[h - 1], Yh[h - 1], D) + eps);
        for (int64_t j = 0; j < D; ++j) q[j] = (float)(gam * (double)q[j]);
        for (int i = 0; i < h; ++i) {
            double rho = 1.0 / (dotv(cf, Yh[i], S[i], D) + eps);
            double be = rho * dotv(cf, Yh[i], q, D);
            for (int64_t j = 0; j < D; ++j) q[j] = (float)((double)q[j] + (double)S[i][j] * (alph[i] - be));
        }
    }
    for (int64_t j = 0; j < D; ++j) p[j] = -q[j];
}

static float dotf(const lb_cfg_t *cf, const float *a, const float *b, int64_t D)
{
    return (float)dotv(cf, a, b, D);
}

static void trial_point(const float *x, const float *p, float al, float *xt, int64_t D)
{
    for (int64_t j = 0; j < D; ++j) xt[j] = x[j] + al * p[j];
}

/* Zoom (lbfgs_batch.py:204-264) for one problem.  phi0/dphi0 are re-evaluated
 * by the reference at x; they equal the bracket phase's values. */
static float zoom(problem_t *P, const lb_cfg_t *cf, const float *x, const float *p, float lo, float hi,
                  float phi0, float dphi0, float *xt, float *gt, int64_t D)
{
    const float c1 = 1e-4f, c2 = 0.9f;
    trial_point(x, p, lo, xt, D);
    float phi_lo = closure_f32(P, xt, gt);
    float alpha = 0.0f;
    int zdone = 0;
    for (int it = 0; it < 10; ++it) {
        if (zdone) break;
        float aj = (lo + hi) / 2.0f;
        trial_point(x, p, aj, xt, D);
        float phij = closure_f32(P, xt, gt);
        float dphij = dotf(cf, gt, p, D);
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

/* Strong-Wolfe bracketing (lbfgs_batch.py:138-202) for one problem. */
static float strong_wolfe(problem_t *P, const lb_cfg_t *cf, const float *x, const float *p, float phi0,
                          float dphi0, int ls_max, float *xt, float *gt, int64_t D)
{
    const float c1 = 1e-4f, c2 = 0.9f, amax = 20.0f;
    float a_prev = 0.0f, phi_prev = phi0, a_i = 1.0f, fin = 0.0f;
    int done = 0;
    for (int i = 0; i < ls_max; ++i) {
        if (done) break;
        trial_point(x, p, a_i, xt, D);
        float phii = closure_f32(P, xt, gt);
        float dphii = dotf(cf, gt, p, D);
        int bad = (phii > phi0 + (c1 * a_i) * dphi0) || (i > 0 && phii >= phi_prev);
        int good = fabsf(dphii) <= c2 * fabsf(dphi0);
        int passed = dphii >= 0.0f;
        if (good) { fin = a_i; done = 1; }
        else if (bad || passed) {
            float lo = bad ? a_prev : a_i, hi = bad ? a_i : a_prev;
            fin = zoom(P, cf, x, p, lo, hi, phi0, dphi0, xt, gt, D);
            done = 1;
        }
        if (!done) {
            a_prev = a_i; phi_prev = phii;
            a_i = a_i + (amax - a_i) * 0.8f;
        }
    }
    return done ? fin : a_i;
}

/* Armijo backtracking (lbfgs_batch.py:105-136) for one problem: alpha halves
 * after every failed try, including the last. */
static float backtracking(problem_t *P, const lb_cfg_t *cf, const float *x, const float *p, float fk,
                          const float *gk, int ls_max, float *xt, float *gt, int64_t D)
{
    float gfp = dotf(cf, gk, p, D);
    float al = 1.0f;
    for (int t = 0; t < ls_max; ++t) {
        trial_point(x, p, al, xt, D);
        float ft = closure_f32(P, xt, gt);
        if (ft <= fk + (1e-4f * al) * gfp) return al;
        al = al * 0.5f;
    }
    return al;
}

/* Runs optimize() for problems [0, B).  Layouts: X (N,nx), Y (B,N) or NULL,
 * ops (B,M), ch (B,M,2), C_init/C_out (B,M), Y_out (B,N) or NULL.
 * iters_out/evals_out/loss_out (B) may be NULL; iters_out[b] = -code for a
 * problem whose closures raised an error.  Returns 0 or an error code. */
int sro_optimize_f32(const float *X, int64_t N, int64_t nx, const float *Y, const int64_t *ops,
                     const int64_t *ch, const float *C_init, int64_t B, int64_t M, int max_iter,
                     int history, double tol, int ls_kind, int ls_max, int dot_mode,
                     float *C_out, float *Y_out, int *iters_out, long *evals_out, float *loss_out)
{
    int err_all = 0;
    lb_cfg_t cf = { dot_mode, 1e-10 };
    const int64_t D = M;
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
        P.dmode = dot_mode;
        size_t vb = sizeof(float) * (size_t)D;
        float *x = malloc(vb), *g = malloc(vb), *p = malloc(vb), *q = malloc(vb), *xt = malloc(vb),
              *gt = malloc(vb), *gn = malloc(vb);
        float **S = malloc(sizeof(float *) * (size_t)(history + 1)), **Yh = malloc(sizeof(float *) * (size_t)(history + 1));
        double *alph = malloc(sizeof(double) * (size_t)(history + 1));
        for (int i = 0; i <= history; ++i) { S[i] = malloc(vb); Yh[i] = malloc(vb); }
        int h = 0, it = 0;
        memcpy(x, C_init + b * M, vb);
        float f = closure_f32(&P, x, g);
        for (it = 0; it < max_iter; ++it) {
            double gn2 = 0.0;
            if (dot_mode == 0) { float s = 0.0f; for (int64_t j = 0; j < D; ++j) s += g[j] * g[j]; gn2 = (double)s; }
            else for (int64_t j = 0; j < D; ++j) gn2 += (double)g[j] * (double)g[j];
            double gnorm = dot_mode == 0 ? (double)sqrtf((float)gn2) : sqrt(gn2);
            if (gnorm < (dot_mode == 0 ? (double)(float)tol : tol)) break;
            direction(&cf, g, S, Yh, h, D, q, p, alph);
            float al;
            if (ls_kind == 0) {
                float dphi0 = dotf(&cf, g, p, D);
                al = strong_wolfe(&P, &cf, x, p, f, dphi0, ls_max, xt, gt, D);
            } else {
                al = backtracking(&P, &cf, x, p, f, g, ls_max, xt, gt, D);
            }
            /* s = alpha p ; x += s ; closure at the new x (lbfgs_batch.py:305-312) */
            float *s_new = S[h], *y_new = Yh[h];
            for (int64_t j = 0; j < D; ++j) { s_new[j] = al * p[j]; x[j] = x[j] + s_new[j]; }
            float fn = closure_f32(&P, x, gn);
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
        memcpy(C_out + b * M, x, vb);
        if (iters_out) iters_out[b] = it;
        if (Y_out) {  /* final forward pass at the optimized constants */
            for (int64_t n = 0; n < N; ++n) {
                for (int64_t k = 0; k < M; ++k) {
                    int64_t op = P.ops[k];
                    int ar = arity_of(op);
                    float a = 0, bb = 0;
                    if (op != OP_NO_OP) {
                        if (ar >= 1) a = P.val[P.ch[k * 2]];
                        if (ar == 2) bb = P.val[P.ch[k * 2 + 1]];
                    }
                    P.val[k] = fwd_f32(op, a, bb, x[k], X + n * nx, nx);
                }
                Y_out[b * N + n] = P.val[P.root];
            }
        }
        if (loss_out) loss_out[b] = f;
        if (evals_out) evals_out[b] = P.n_evals;
        if (P.err && iters_out) iters_out[b] = -P.err;
        if (P.err) {
            _Pragma("omp critical")
            { if (!err_all) err_all = P.err; }
        }
        for (int i = 0; i <= history; ++i) { free(S[i]); free(Yh[i]); }
        free(S); free(Yh); free(alph);
        free(x); free(g); free(p); free(q); free(xt); free(gt); free(gn);
        free(P.val); free(P.adj); free(P.gacc);
    }
    return err_all;
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
                const int r0 = sym < n_symbols ? nt_ptr[sym] : 0;
                const int r1 = sym < n_symbols ? nt_ptr[sym + 1] : 0;
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
