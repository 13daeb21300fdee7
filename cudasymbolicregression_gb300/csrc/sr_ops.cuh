// sr_ops.cuh -- postfix-tape node encoding and per-point operator semantics.
//
// Tapes are staged once per call from the reference's int64 Ops/Ch tensors into
// one 32-bit word per node:
//
//     bits  0.. 7  opcode (the reference's Operator code; VAR for X_i, ZERO for codes
//                  the reference evaluates to 0: unknown codes, X_i with i >= n_x)
//     bits  8..19  first child index, or the variable index for VAR
//     bits 20..31  second child index
//
// so a tape of at most 4095 nodes fits.  The operator policies (NaN for log of
// x <= 0, sqrt of x < 0, a/0, pow of a < 0, asin/acos outside [-1,1], inv(0)) follow
// include/operators.h:222-434 of the reference.  The per-point adjoint rules follow
// the reference's CUDA backward (src/evaluation_kernels_cuda.cu:218-632): most
// rules skip a zero incoming adjoint, SQRT and POW emit NaN for a negative base
// even then, EXP uses the node's own value, and a/0 with a nonzero adjoint is
// reported as error 204.  Adjoint accumulation is written with explicit
// round-to-nearest adds so it is never fused with the product that feeds it,
// exactly like the reference's separate atomicAdd.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "sr_fmath.h"

namespace sr {

enum Op : int {
  NO_OP = 0, LEARNABLE = 1, C1 = 2, C2 = 3, C3 = 4, C4 = 5, C5 = 6, PI_ = 7, E_ = 8,
  ZERO = 9,  // internal: evaluates to 0 (the reference's default branch)
  SIN = 10, COS, EXP, LOG, SQUARE, SQRT, TAN, ARCSIN, ARCCOS, ARCTAN, SINH, COSH, TANH,
  FLOOR, CEIL, LN, LOG10, NEG, INV, CUBE, FOURTH, FIFTH,
  ADD = 40, SUB, MUL, DIV, POW,
  VAR = 50
};

enum Status : int {
  OK = 0,
  ERR_CHILD_GEQ_PARENT = 101,
  ERR_ARITY = 102,
  ERR_GRAD_ON_NO_OP = 201,
  ERR_DIV_BY_ZERO = 204,
};

constexpr int kMaxNodes = 4095;

__host__ __device__ __forceinline__ int arity_of(int64_t op) {
  if (op >= SIN && op <= FIFTH) return 1;
  if (op >= ADD && op <= POW) return 2;
  return 0;
}

__host__ __device__ __forceinline__ uint32_t pack(int code, uint32_t c0, uint32_t c1) {
  return uint32_t(code) | (c0 << 8) | (c1 << 20);
}
__device__ __forceinline__ int code_of(uint32_t d) { return int(d & 0xffu); }
__device__ __forceinline__ int child0(uint32_t d) { return int((d >> 8) & 0xfffu); }
__device__ __forceinline__ int child1(uint32_t d) { return int(d >> 20); }

// ---- math per scalar type --------------------------------------------------------
template <typename T> struct M_;
template <> struct M_<float> {
  static __device__ __forceinline__ float nan() { return __int_as_float(0x7fffffff); }
  // sin, cos, exp and log: the library's own functions (sr_fmath.h), which the
  // oracle reproduces bit for bit; the other functions are CUDA's
  static __device__ __forceinline__ float sin(float x) { return sr_sinf(x); }
  static __device__ __forceinline__ float cos(float x) { return sr_cosf(x); }
  static __device__ __forceinline__ float exp(float x) { return sr_expf(x); }
  static __device__ __forceinline__ float log(float x) { return sr_logf(x); }
  static __device__ __forceinline__ float sqrt(float x) { return ::sqrtf(x); }
  static __device__ __forceinline__ float tan(float x) { return ::tanf(x); }
  static __device__ __forceinline__ float asin(float x) { return ::asinf(x); }
  static __device__ __forceinline__ float acos(float x) { return ::acosf(x); }
  static __device__ __forceinline__ float atan(float x) { return ::atanf(x); }
  static __device__ __forceinline__ float sinh(float x) { return ::sinhf(x); }
  static __device__ __forceinline__ float cosh(float x) { return ::coshf(x); }
  static __device__ __forceinline__ float tanh(float x) { return ::tanhf(x); }
  static __device__ __forceinline__ float floor(float x) { return ::floorf(x); }
  static __device__ __forceinline__ float ceil(float x) { return ::ceilf(x); }
  static __device__ __forceinline__ float log10(float x) { return ::log10f(x); }
  static __device__ __forceinline__ float pow(float a, float b) { return ::powf(a, b); }
  static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
};
template <> struct M_<double> {
  static __device__ __forceinline__ double nan() { return __longlong_as_double(0x7fffffffffffffffLL); }
  static __device__ __forceinline__ double sin(double x) { return ::sin(x); }
  static __device__ __forceinline__ double cos(double x) { return ::cos(x); }
  static __device__ __forceinline__ double exp(double x) { return ::exp(x); }
  static __device__ __forceinline__ double log(double x) { return ::log(x); }
  static __device__ __forceinline__ double sqrt(double x) { return ::sqrt(x); }
  static __device__ __forceinline__ double tan(double x) { return ::tan(x); }
  static __device__ __forceinline__ double asin(double x) { return ::asin(x); }
  static __device__ __forceinline__ double acos(double x) { return ::acos(x); }
  static __device__ __forceinline__ double atan(double x) { return ::atan(x); }
  static __device__ __forceinline__ double sinh(double x) { return ::sinh(x); }
  static __device__ __forceinline__ double cosh(double x) { return ::cosh(x); }
  static __device__ __forceinline__ double tanh(double x) { return ::tanh(x); }
  static __device__ __forceinline__ double floor(double x) { return ::floor(x); }
  static __device__ __forceinline__ double ceil(double x) { return ::ceil(x); }
  static __device__ __forceinline__ double log10(double x) { return ::log10(x); }
  static __device__ __forceinline__ double pow(double a, double b) { return ::pow(a, b); }
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
};

// Division with the reference's policy: NaN when the divisor is exactly zero.
template <typename T>
__device__ __forceinline__ T pdiv(T a, T b) { return b == T(0) ? M_<T>::nan() : a / b; }

// ---- forward value of one node at one point ---------------------------------------
// a, b: values of the children; c: the node's learnable constant; xv: X[n][var].
template <typename T>
__device__ __forceinline__ T node_value(int code, T a, T b, T c, T xv) {
  using F = M_<T>;
  switch (code) {
    case NO_OP: return F::nan();
    case LEARNABLE: return c;
    case C1: return T(1);
    case C2: return T(2);
    case C3: return T(3);
    case C4: return T(4);
    case C5: return T(5);
    case PI_: return T(3.14159265358979323846);
    case E_: return T(2.7182818284590452354);
    case SIN: return F::sin(a);
    case COS: return F::cos(a);
    case EXP: return F::exp(a);
    case LOG:
    case LN: return a <= T(0) ? F::nan() : F::log(a);
    case SQUARE: return a * a;
    case SQRT: return a < T(0) ? F::nan() : F::sqrt(a);
    case TAN: return F::tan(a);
    case ARCSIN: return (a < T(-1) || a > T(1)) ? F::nan() : F::asin(a);
    case ARCCOS: return (a < T(-1) || a > T(1)) ? F::nan() : F::acos(a);
    case ARCTAN: return F::atan(a);
    case SINH: return F::sinh(a);
    case COSH: return F::cosh(a);
    case TANH: return F::tanh(a);
    case FLOOR: return F::floor(a);
    case CEIL: return F::ceil(a);
    case LOG10: return a <= T(0) ? F::nan() : F::log10(a);
    case NEG: return -a;
    case INV: return a == T(0) ? F::nan() : T(1) / a;
    case CUBE: return a * a * a;
    case FOURTH: { T s = a * a; return s * s; }
    case FIFTH: { T s = a * a; return s * s * a; }
    case ADD: return a + b;
    case SUB: return a - b;
    case MUL: return a * b;
    case DIV: return pdiv(a, b);
    case POW: return a < T(0) ? F::nan() : F::pow(a, b);
    case VAR: return xv;
    default: return T(0);
  }
}

// ---- adjoint of one node at one point ---------------------------------------------
// g: the node's adjoint; a, b: child values; v: the node's own value.
// On return, (add0, o0) / (add1, o1) say what to add to the children's adjoints.
// Returns 0 or a Status (201 / 204).  LEARNABLE and VAR nodes are handled by the
// caller (their adjoint goes to dC / dX); leaves and FLOOR/CEIL propagate nothing.
template <typename T>
__device__ __forceinline__ int node_adjoint(int code, T g, T a, T b, T v, bool& add0, T& o0, bool& add1,
                                            T& o1) {
  using F = M_<T>;
  add0 = false;
  add1 = false;
  o0 = T(0);
  o1 = T(0);
  const bool zero = (g == T(0));
  switch (code) {
    case NO_OP: return zero ? 0 : ERR_GRAD_ON_NO_OP;
    case SIN: if (zero) return 0; o0 = g * F::cos(a); add0 = true; return 0;
    case COS: if (zero) return 0; o0 = g * -F::sin(a); add0 = true; return 0;
    case EXP: if (zero) return 0; o0 = g * v; add0 = true; return 0;
    case LOG:
    case LN: if (zero) return 0; o0 = pdiv(g, a); add0 = true; return 0;
    case SQUARE: if (zero) return 0; o0 = g * T(2) * a; add0 = true; return 0;
    case SQRT:
      add0 = true;
      if (a < T(0)) o0 = F::nan();
      else if (zero) o0 = T(0);
      else o0 = pdiv(g * T(0.5), F::sqrt(a));
      return 0;
    case TAN: { if (zero) return 0; T cv = F::cos(a); o0 = pdiv(g, cv * cv); add0 = true; return 0; }
    case ARCSIN:
    case ARCCOS: {
      if (zero) return 0;
      add0 = true;
      if (a < T(-1) || a > T(1)) { o0 = F::nan(); return 0; }
      T r = T(1) - a * a;
      T den = r < T(0) ? F::nan() : F::sqrt(r);
      o0 = pdiv(g, den);
      if (code == ARCCOS) o0 = -o0;
      return 0;
    }
    case ARCTAN: if (zero) return 0; o0 = pdiv(g, T(1) + a * a); add0 = true; return 0;
    case SINH: if (zero) return 0; o0 = g * F::cosh(a); add0 = true; return 0;
    case COSH: if (zero) return 0; o0 = g * F::sinh(a); add0 = true; return 0;
    case TANH: { if (zero) return 0; T t = F::tanh(a); o0 = g * (T(1) - t * t); add0 = true; return 0; }
    case LOG10: if (zero) return 0; o0 = pdiv(g, a * F::log(T(10))); add0 = true; return 0;
    case NEG: if (zero) return 0; o0 = -g; add0 = true; return 0;
    case INV: if (zero) return 0; o0 = (a == T(0)) ? F::nan() : -pdiv(g, a * a); add0 = true; return 0;
    case CUBE: if (zero) return 0; o0 = g * T(3) * (a * a); add0 = true; return 0;
    case FOURTH: if (zero) return 0; o0 = g * T(4) * (a * a * a); add0 = true; return 0;
    case FIFTH: { if (zero) return 0; T s = a * a; o0 = g * T(5) * (s * s); add0 = true; return 0; }
    case ADD: if (zero) return 0; o0 = g; o1 = g; add0 = add1 = true; return 0;
    case SUB: if (zero) return 0; o0 = g; o1 = -g; add0 = add1 = true; return 0;
    case MUL: if (zero) return 0; o0 = g * b; o1 = g * a; add0 = add1 = true; return 0;
    case DIV:
      if (zero) return 0;
      add0 = add1 = true;
      if (b == T(0)) return ERR_DIV_BY_ZERO;  // adds 0 to both, as the reference does
      o0 = pdiv(g, b);
      o1 = -pdiv(g * a, b * b);
      return 0;
    case POW:
      if (a < T(0)) { o0 = F::nan(); o1 = F::nan(); add0 = add1 = true; return 0; }
      if (zero) return 0;
      {
        T pm1 = a < T(0) ? F::nan() : F::pow(a, b - T(1));
        T pw = a < T(0) ? F::nan() : F::pow(a, b);
        T lg = a <= T(0) ? F::nan() : F::log(a);
        o0 = g * (pm1 * b);
        o1 = g * (lg * pw);
      }
      add0 = add1 = true;
      return 0;
    default: return 0;
  }
}

// ---- dense dispatch for operator nodes ---------------------------------------------
// The interpreters' programs hold operator nodes only (NO_OP and arity >= 1), coded
// densely: 0 = NO_OP, 1..22 = SIN..FIFTH, 23..27 = ADD..POW, so the per-node switch
// has contiguous cases.  Each case calls the scalar rule above with a constant code,
// which folds to that one rule.
constexpr int kDenseOps = 28;

__host__ __device__ __forceinline__ int dense_op(int code) {
  return code == NO_OP ? 0 : (code >= ADD ? code - ADD + 23 : code - SIN + 1);
}

__host__ __device__ constexpr int op_of_dense(int d) { return d == 0 ? NO_OP : (d >= 23 ? ADD + d - 23 : SIN + d - 1); }

#define SR_DENSE_CASES(X) \
  X(0) X(1) X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12) X(13) X(14) X(15) X(16) X(17) X(18) \
  X(19) X(20) X(21) X(22) X(23) X(24) X(25) X(26) X(27)

template <typename T>
__device__ __forceinline__ T op_value(int d, T a, T b) {
  switch (d) {
#define SR_VALUE_CASE(i) \
  case i: return node_value<T>(op_of_dense(i), a, b, T(0), T(0));
    SR_DENSE_CASES(SR_VALUE_CASE)
#undef SR_VALUE_CASE
    default: return T(0);
  }
}

template <typename T>
__device__ __forceinline__ int op_adjoint(int d, T g, T a, T b, T v, bool& add0, T& o0, bool& add1, T& o1) {
  switch (d) {
#define SR_ADJOINT_CASE(i) \
  case i: return node_adjoint<T>(op_of_dense(i), g, a, b, v, add0, o0, add1, o1);
    SR_DENSE_CASES(SR_ADJOINT_CASE)
#undef SR_ADJOINT_CASE
    default: add0 = add1 = false; o0 = o1 = T(0); return 0;
  }
}

// V points at once: one dispatch, then the rule for every point (the operands are in
// registers, so the points' chains interleave).
template <typename T, int V>
__device__ __forceinline__ void op_value_v(int d, const T (&a)[V], const T (&b)[V], T (&r)[V]) {
  switch (d) {
#define SR_VALUE_V_CASE(i)                                                           \
  case i:                                                                            \
    _Pragma("unroll") for (int q = 0; q < V; ++q) r[q] = node_value<T>(op_of_dense(i), a[q], b[q], T(0), T(0)); \
    break;
    SR_DENSE_CASES(SR_VALUE_V_CASE)
#undef SR_VALUE_V_CASE
    default:
      _Pragma("unroll") for (int q = 0; q < V; ++q) r[q] = T(0);
  }
}

template <typename T, int V>
__device__ __forceinline__ void op_adjoint_v(int d, const T (&g)[V], const T (&a)[V], const T (&b)[V],
                                             const T (&v)[V], bool (&add0)[V], T (&o0)[V], bool (&add1)[V],
                                             T (&o1)[V], int (&e)[V]) {
  switch (d) {
#define SR_ADJOINT_V_CASE(i)                                                                               \
  case i:                                                                                                  \
    _Pragma("unroll") for (int q = 0; q < V; ++q) e[q] =                                                   \
        node_adjoint<T>(op_of_dense(i), g[q], a[q], b[q], v[q], add0[q], o0[q], add1[q], o1[q]);           \
    break;
    SR_DENSE_CASES(SR_ADJOINT_V_CASE)
#undef SR_ADJOINT_V_CASE
    default:
      _Pragma("unroll") for (int q = 0; q < V; ++q) {
        add0[q] = add1[q] = false;
        o0[q] = o1[q] = T(0);
        e[q] = 0;
      }
  }
}

}  // namespace sr
