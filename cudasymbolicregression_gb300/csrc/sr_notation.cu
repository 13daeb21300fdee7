// sr_notation.cu -- integer tape conversions of the grammar object:
//   * child table of left-packed postfix tapes   (reference get_postfix_children,
//     src/pcfg_cuda.cu:1228-1300, src/pcfg.cpp:957-986)
//   * postfix -> infix token ids with parentheses (reference postfix_to_infix,
//     src/pcfg_cuda.cu:502-701, src/pcfg.cpp:790-826)
//   * prefix -> postfix, postfix -> prefix, prefix -> infix and the parent table of
//     prefix rows (reference src/pcfg_cpu.cpp:637-1064, src/pcfg.cpp:827-955)
// All are bit-exact integer transformations with the reference's error codes and
// stack limits (128 entries, 3 x 128 output tokens).  One thread owns one tape; a
// warp's 32 tapes are read with 8-byte loads that stay in L1 across the row.
#include <cstdint>

#include "sr_common.cuh"
#include "sr_ops.cuh"

namespace sr {

constexpr int kStackLimit = 128;  // the reference's HARD_MAX_LENGTH

enum NotationCode : int64_t {
  SYM_NEGATIVE = -1,  // a symbol < 0
  SYM_TOO_LARGE = -2, // a symbol >= n_operators
  PARSE_UNEXPECTED_TOKEN = 408,
  PARSE_UNARY_MISSING = 404,
  PARSE_BINARY_MISSING = 405,
  PARSE_STACK_OVERFLOW = 406,
  PARSE_MALFORMED = 407,
  CONV_TOO_LONG = 501,
  CONV_POSTFIX_TOO_LONG = 502,
  CONV_PREFIX_TOO_LONG = 503,
  CONV_STACK_OVERFLOW = 504,
  CONV_UNARY_MISSING = 505,
  CONV_BINARY_MISSING = 506,
  CONV_MULTIPLE_ROOTS = 508,
  CONV_UNEXPECTED_TOKEN = 509,
};

// Symbols must lie in [0, n_operators): -1 / -2 flag the two ways to fail.
__device__ __forceinline__ int64_t symbol_check(const int64_t* row, int64_t M, int64_t n_operators) {
  int64_t flag = 0;
  for (int64_t i = 0; i < M; ++i) {
    const int64_t t = row[i];
    if (t < 0) return SYM_NEGATIVE;
    if (t >= n_operators) flag = SYM_TOO_LARGE;
  }
  return flag;
}

// Unary operators written f(x); the others (^2, ^3, ^4, ^5, ^-1) are written (x)^k.
__device__ __forceinline__ bool functional_style(int64_t op) {
  return (op >= SIN && op <= LOG) || (op >= SQRT && op <= NEG);
}

__global__ void postfix_children_kernel(const int64_t* __restrict__ ops, int64_t B, int64_t M, int64_t n_operators,
                                        int64_t* __restrict__ ch, int64_t* __restrict__ err) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const int64_t* row = ops + b * M;
  int64_t* out = ch + b * M * 2;
  for (int64_t i = 0; i < 2 * M; ++i) out[i] = -1;
  int64_t e = symbol_check(row, M, n_operators);
  if (e) {
    err[b] = e;
    return;
  }
  int stack[kStackLimit];
  int sp = 0;
  bool ended = false;
  for (int64_t i = 0; i < M; ++i) {
    const int64_t t = row[i];
    if (t == NO_OP) {
      ended = true;
      continue;
    }
    if (ended) { e = PARSE_UNEXPECTED_TOKEN; break; }
    const int ar = arity_of(t);
    if (ar == 1) {
      if (sp < 1) { e = PARSE_UNARY_MISSING; break; }
      out[i * 2] = stack[--sp];
    } else if (ar == 2) {
      if (sp < 2) { e = PARSE_BINARY_MISSING; break; }
      const int right = stack[--sp];
      const int left = stack[--sp];
      out[i * 2] = left;
      out[i * 2 + 1] = right;
    }
    if (sp >= kStackLimit) { e = PARSE_STACK_OVERFLOW; break; }
    stack[sp++] = (int)i;
  }
  if (!e && sp != 1) e = PARSE_MALFORMED;
  err[b] = e;
}

// The same child table for rows of 1..128 tokens and token ids below 32768, with the
// CTA's rows staged through shared memory: the CTA reads its 128 rows and writes their
// child tables with coalesced 8-byte accesses (consecutive threads, consecutive
// elements), and each thread's stack and table sit in shared memory instead of local
// memory (an M-token row never holds more than M entries on the stack).  Symbols are
// staged as -1 (negative) or -2 (too large) when they fail the check.  The left child of
// position i replaces its token once the token has been read; positions the scan does
// not reach (after an error) are set to -1 at the end, as the table starts all -1.
constexpr int kChildThreads = 128;

__global__ void __launch_bounds__(kChildThreads) postfix_children_staged_kernel(
    const int64_t* __restrict__ ops, int64_t B, int64_t M, int64_t n_operators, int64_t* __restrict__ ch,
    int64_t* __restrict__ err) {
  extern __shared__ int16_t csm[];
  const int t = threadIdx.x, Mi = (int)M;
  int16_t* in = csm;                            // [M][kChildThreads]: tokens, then left children
  int16_t* rt = csm + Mi * kChildThreads;       // [M][kChildThreads]: right children
  int16_t* stk = csm + 2 * Mi * kChildThreads;  // [M][kChildThreads]
  const int64_t b0 = (int64_t)blockIdx.x * kChildThreads;
  const int rows = (int)(B - b0 < kChildThreads ? B - b0 : kChildThreads);
  // element j of the block is token j % M of row j / M; (row, token) advance by
  // (kChildThreads / M, kChildThreads % M) with a carry
  {
    const int total = rows * Mi, dr = kChildThreads / Mi, di = kChildThreads % Mi;
    int r = t / Mi, i = t - r * Mi;
#pragma unroll 4
    for (int j = t; j < total; j += kChildThreads) {
      const int64_t tok = ops[b0 * M + j];
      in[i * kChildThreads + r] = (int16_t)(tok < 0 ? -1 : (tok >= n_operators ? -2 : tok));
      r += dr;
      i += di;
      if (i >= Mi) {
        i -= Mi;
        ++r;
      }
    }
  }
  __syncthreads();
  if (t < rows) {
    int64_t e = 0;
    for (int i = 0; i < Mi; ++i) {
      const int v = in[i * kChildThreads + t];
      if (v == -1) {
        e = SYM_NEGATIVE;
        break;
      }
      if (v == -2) e = SYM_TOO_LARGE;
    }
    int stop = 0;  // positions from here on keep no children
    if (!e) {
      int sp = 0;
      bool ended = false;
      int i = 0;
      for (; i < Mi; ++i) {
        const int tok = in[i * kChildThreads + t];
        int16_t left = -1, right = -1;
        if (tok == NO_OP) {
          ended = true;
        } else {
          if (ended) { e = PARSE_UNEXPECTED_TOKEN; break; }
          const int ar = arity_of(tok);
          if (ar == 1) {
            if (sp < 1) { e = PARSE_UNARY_MISSING; break; }
            left = stk[(--sp) * kChildThreads + t];
          } else if (ar == 2) {
            if (sp < 2) { e = PARSE_BINARY_MISSING; break; }
            right = stk[(--sp) * kChildThreads + t];
            left = stk[(--sp) * kChildThreads + t];
          }
          stk[(sp++) * kChildThreads + t] = (int16_t)i;  // sp <= i + 1 <= M <= kStackLimit
        }
        in[i * kChildThreads + t] = left;
        rt[i * kChildThreads + t] = right;
      }
      stop = i;
      if (!e && sp != 1) e = PARSE_MALFORMED;
    }
    for (int i = stop; i < Mi; ++i) {
      in[i * kChildThreads + t] = -1;
      rt[i * kChildThreads + t] = -1;
    }
    err[b0 + t] = e;
  }
  __syncthreads();
  {
    const int M2 = 2 * Mi, total = rows * M2, dr = kChildThreads / M2, di = kChildThreads % M2;
    int r = t / M2, i = t - r * M2;
#pragma unroll 4
    for (int j = t; j < total; j += kChildThreads) {
      const int16_t* src = (i & 1) ? rt : in;
      ch[b0 * 2 * M + j] = src[(i >> 1) * kChildThreads + r];
      r += dr;
      i += di;
      if (i >= M2) {
        i -= M2;
        ++r;
      }
    }
  }
}

// Right-to-left rendering: the output is built backwards from the end of a
// 3 x 128 buffer.  An operator first emits ")" (and, for (x)^k forms, its own
// token); once its right operand is complete a binary operator emits itself, once
// its left operand is complete it emits "(".  A unary f emits "( f" when its operand
// is complete, a (x)^k form emits "(".
__global__ void postfix_to_infix_kernel(const int64_t* __restrict__ ops, int64_t B, int64_t M, int64_t n_operators,
                                        int64_t lparen, int64_t rparen, int64_t* __restrict__ infix, int64_t M_out,
                                        int64_t* __restrict__ err) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const int64_t* row = ops + b * M;
  int64_t* out = infix + b * M_out;
  for (int64_t i = 0; i < M_out; ++i) out[i] = NO_OP;
  int64_t e = symbol_check(row, M, n_operators);
  if (e) {
    err[b] = e;
    return;
  }
  // shape check from the right: padding only at the end, one root
  bool started = false;
  int len = 0, balance = 0, roots = 0;
  for (int64_t k = M - 1; k >= 0; --k) {
    const int64_t t = row[k];
    if (t == NO_OP) {
      if (started) { err[b] = CONV_UNEXPECTED_TOKEN; return; }
    } else {
      started = true;
      ++len;
      balance += arity_of(t) - 1;
      if (balance == -1) ++roots;
    }
  }
  if (len == 0) { err[b] = 0; return; }
  if (roots > 1) { err[b] = CONV_MULTIPLE_ROOTS; return; }

  constexpr int kBuf = 3 * kStackLimit;
  int32_t buf[kBuf];
  int32_t opst[kStackLimit];
  int8_t waiting_left[kStackLimit];
  int top = kBuf - 1;  // next free slot, filled downwards
  int sp = 0;
#define SR_EMIT(tok)                                \
  do {                                              \
    if (top < 0) { err[b] = CONV_STACK_OVERFLOW; return; } \
    buf[top--] = (int32_t)(tok);                    \
  } while (0)
  for (int k = len - 1; k >= 0; --k) {
    const int64_t t = row[k];
    const int ar = arity_of(t);
    if (ar == 0) {
      SR_EMIT(t);
      bool done = true;
      while (done && sp > 0) {
        const int32_t parent = opst[sp - 1];
        if (arity_of(parent) == 1) {
          if (functional_style(parent)) {
            if (top - 1 < 0) { err[b] = CONV_STACK_OVERFLOW; return; }
            buf[top--] = (int32_t)lparen;
            buf[top--] = parent;
          } else {
            SR_EMIT(lparen);
          }
          --sp;
        } else if (!waiting_left[sp - 1]) {
          SR_EMIT(parent);
          waiting_left[sp - 1] = 1;
          done = false;
        } else {
          SR_EMIT(lparen);
          --sp;
        }
      }
    } else {
      if (sp >= kStackLimit) { err[b] = CONV_STACK_OVERFLOW; return; }
      opst[sp] = (int32_t)t;
      waiting_left[sp] = 0;
      if (ar == 1 && !functional_style(t)) SR_EMIT(t);
      SR_EMIT(rparen);
      ++sp;
    }
  }
#undef SR_EMIT
  if (sp > 0) {
    err[b] = arity_of(opst[sp - 1]) == 1 ? CONV_UNARY_MISSING : CONV_BINARY_MISSING;
    return;
  }
  const int n = kBuf - 1 - top;
  if (n > M_out) { err[b] = CONV_TOO_LONG; return; }
  for (int i = 0; i < n; ++i) out[i] = buf[top + 1 + i];
  err[b] = 0;
}

// ---- prefix conversions ---------------------------------------------------------
// prefix <-> postfix (src/pcfg_cpu.cpp:812-993): a stack of (node, children still
// missing); a node is emitted once all its children are.  postfix -> prefix walks the
// row from the right and reverses what it emits.  Rows with an error are all NO_OP.
template <bool kFromPrefix>
__global__ void reorder_kernel(const int64_t* __restrict__ in, int64_t B, int64_t M, int64_t n_operators,
                               int64_t* __restrict__ outp, int64_t* __restrict__ err) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const int64_t* row = in + b * M;
  int64_t* out = outp + b * M;
  for (int64_t i = 0; i < M; ++i) out[i] = NO_OP;
  int64_t e = symbol_check(row, M, n_operators);
  if (e) {
    err[b] = e;
    return;
  }
  int32_t node[kStackLimit];
  int8_t missing[kStackLimit];
  int sp = 0, n_out = 0, balance = 0, roots = 0;
  bool seen = false;  // prefix: past the end; postfix: the expression has started
  for (int64_t s = 0; s < M; ++s) {
    const int64_t i = kFromPrefix ? s : M - 1 - s;
    const int64_t t = row[i];
    if (t == NO_OP) {
      if (kFromPrefix) seen = true;
      else if (seen) { err[b] = CONV_UNEXPECTED_TOKEN; return; }
      continue;
    }
    if (kFromPrefix && seen) { err[b] = CONV_UNEXPECTED_TOKEN; return; }
    if (!kFromPrefix) seen = true;
    const int ar = arity_of(t);
    balance += ar - 1;
    if (balance == -1) ++roots;
    if (sp >= kStackLimit) { err[b] = CONV_STACK_OVERFLOW; return; }
    node[sp] = (int32_t)i;
    missing[sp++] = (int8_t)ar;
    while (sp > 0 && missing[sp - 1] == 0) {
      --sp;
      if (n_out >= M) { err[b] = kFromPrefix ? CONV_POSTFIX_TOO_LONG : CONV_PREFIX_TOO_LONG; return; }
      out[n_out++] = row[node[sp]];
      if (sp > 0) --missing[sp - 1];
    }
  }
  if (sp != 0) {
    for (int64_t i = 0; i < M; ++i) out[i] = NO_OP;
    err[b] = arity_of(row[node[sp - 1]]) == 1 ? CONV_UNARY_MISSING : CONV_BINARY_MISSING;
    return;
  }
  if (roots != 1 && n_out > 0) {
    for (int64_t i = 0; i < M; ++i) out[i] = NO_OP;
    err[b] = CONV_MULTIPLE_ROOTS;
    return;
  }
  if (!kFromPrefix) {  // emitted from the right: reverse into prefix order
    for (int i = 0, j = n_out - 1; i < j; ++i, --j) {
      const int64_t x = out[i];
      out[i] = out[j];
      out[j] = x;
    }
  }
  err[b] = 0;
}

// Parent of every node of a prefix row (src/pcfg_cpu.cpp:995-1064): from the right,
// a stack of finished subtrees; an operator adopts the top one or two.  Roots and
// padding keep -1.
__global__ void prefix_parent_kernel(const int64_t* __restrict__ in, int64_t B, int64_t M, int64_t n_operators,
                                     int64_t* __restrict__ parent, int64_t* __restrict__ err) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const int64_t* row = in + b * M;
  int64_t* par = parent + b * M;
  for (int64_t i = 0; i < M; ++i) par[i] = -1;
  int64_t e = symbol_check(row, M, n_operators);
  if (e) {
    err[b] = e;
    return;
  }
  int32_t st[kStackLimit];
  int sp = 0;
  bool started = false;
  for (int64_t i = M - 1; i >= 0; --i) {
    const int64_t t = row[i];
    if (t == NO_OP) {
      if (started) { err[b] = PARSE_UNEXPECTED_TOKEN; return; }
      continue;
    }
    started = true;
    const int ar = arity_of(t);
    if (ar == 1) {
      if (sp < 1) { err[b] = PARSE_UNARY_MISSING; return; }
      par[st[--sp]] = i;
    } else if (ar == 2) {
      if (sp < 2) { err[b] = PARSE_BINARY_MISSING; return; }
      par[st[--sp]] = i;
      par[st[--sp]] = i;
    }
    if (sp >= kStackLimit) { err[b] = PARSE_STACK_OVERFLOW; return; }
    st[sp++] = (int32_t)i;
  }
  err[b] = (started && sp != 1) ? PARSE_MALFORMED : 0;
}

// Prefix -> infix token ids with parentheses (src/pcfg_cpu.cpp:637-811): the same
// rendering as postfix -> infix, produced left to right by a stack of operators that
// wait for their left or right operand.
__global__ void prefix_to_infix_kernel(const int64_t* __restrict__ in, int64_t B, int64_t M, int64_t n_operators,
                                       int64_t lparen, int64_t rparen, int64_t* __restrict__ infix, int64_t M_out,
                                       int64_t* __restrict__ err) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const int64_t* row = in + b * M;
  int64_t* out = infix + b * M_out;
  for (int64_t i = 0; i < M_out; ++i) out[i] = NO_OP;
  int64_t e = symbol_check(row, M, n_operators);
  if (e) {
    err[b] = e;
    return;
  }
  int len = 0, balance = 0, roots = 0;
  bool ended = false;
  for (int64_t i = 0; i < M; ++i) {
    if (row[i] == NO_OP) {
      ended = true;
    } else {
      if (ended) { err[b] = CONV_UNEXPECTED_TOKEN; return; }
      ++len;
      balance += arity_of(row[i]) - 1;
      if (balance == -1) ++roots;
    }
  }
  if (len == 0) { err[b] = 0; return; }
  if (roots > 1) { err[b] = CONV_MULTIPLE_ROOTS; return; }
  int32_t opst[kStackLimit];
  int8_t waiting_right[kStackLimit];
  int sp = 0;
  int64_t n = 0;
#define SR_PUT(tok)                                            \
  do {                                                         \
    if (n >= M_out) { err[b] = CONV_TOO_LONG; goto fail; }     \
    out[n++] = (tok);                                          \
  } while (0)
  for (int k = 0; k < len; ++k) {
    const int64_t t = row[k];
    const int ar = arity_of(t);
    if (ar == 0) {
      SR_PUT(t);
      bool done = true;
      while (done && sp > 0) {
        const int32_t parent = opst[sp - 1];
        if (arity_of(parent) == 1) {
          SR_PUT(rparen);
          if (!functional_style(parent)) SR_PUT(parent);
          --sp;
        } else if (!waiting_right[sp - 1]) {
          SR_PUT(parent);
          waiting_right[sp - 1] = 1;
          done = false;
        } else {
          SR_PUT(rparen);
          --sp;
        }
      }
    } else {
      if (sp >= kStackLimit) { err[b] = CONV_STACK_OVERFLOW; goto fail; }
      opst[sp] = (int32_t)t;
      waiting_right[sp] = 0;
      if (ar == 1 && functional_style(t)) {
        if (n + 2 > M_out) { err[b] = CONV_TOO_LONG; goto fail; }
        out[n++] = t;
        out[n++] = lparen;
      } else {
        SR_PUT(lparen);
      }
      ++sp;
    }
  }
#undef SR_PUT
  if (sp != 0) {
    err[b] = arity_of(opst[sp - 1]) == 1 ? CONV_UNARY_MISSING : CONV_BINARY_MISSING;
    goto fail;
  }
  err[b] = 0;
  return;
fail:
  for (int64_t i = 0; i < M_out; ++i) out[i] = NO_OP;
}

}  // namespace sr

extern "C" {

int sr_postfix_children(const int64_t* ops, int64_t B, int64_t M, int32_t n_vars, int64_t* ch, int64_t* err,
                        void* stream) {
  using namespace sr;
  if (B < 0 || M < 0 || n_vars < 0 || (B > 0 && (!ops || !ch || !err))) {
    set_error("invalid arguments");
    return SR_ERR_INVALID_ARGUMENT;
  }
  if (B == 0) return SR_OK;
  const int64_t n_operators = (int64_t)VAR + n_vars;
  if (M >= 1 && M <= kStackLimit && n_operators <= 32767) {
    const size_t smem = (size_t)3 * M * kChildThreads * sizeof(int16_t);
    int rc = cuda_check(cudaFuncSetAttribute(postfix_children_staged_kernel,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                        "smem");
    if (rc) return rc;
    postfix_children_staged_kernel<<<(unsigned)((B + kChildThreads - 1) / kChildThreads), kChildThreads, smem,
                                     as_stream(stream)>>>(ops, B, M, n_operators, ch, err);
    return launch_check("postfix_children_staged_kernel");
  }
  const int threads = 128;
  postfix_children_kernel<<<(unsigned)((B + threads - 1) / threads), threads, 0, as_stream(stream)>>>(
      ops, B, M, n_operators, ch, err);
  return launch_check("postfix_children_kernel");
}

int sr_postfix_to_infix(const int64_t* ops, int64_t B, int64_t M, int32_t n_vars, int64_t* infix, int64_t M_out,
                        int64_t* err, void* stream) {
  using namespace sr;
  if (B < 0 || M < 0 || M_out < 0 || n_vars < 0 || (B > 0 && (!ops || !err || (M_out > 0 && !infix)))) {
    set_error("invalid arguments");
    return SR_ERR_INVALID_ARGUMENT;
  }
  if (B == 0) return SR_OK;
  const int threads = 128;
  const int64_t lparen = (int64_t)VAR + n_vars, rparen = lparen + 1;
  postfix_to_infix_kernel<<<(unsigned)((B + threads - 1) / threads), threads, 0, as_stream(stream)>>>(
      ops, B, M, (int64_t)VAR + n_vars, lparen, rparen, infix, M_out, err);
  return launch_check("postfix_to_infix_kernel");
}

static int notation_args_ok(const int64_t* in, int64_t B, int64_t M, int32_t n_vars, const void* out,
                            const int64_t* err) {
  if (B < 0 || M < 0 || n_vars < 0 || (B > 0 && (!in || !out || !err))) {
    sr::set_error("invalid arguments");
    return 0;
  }
  return 1;
}

int sr_prefix_to_postfix(const int64_t* prefix, int64_t B, int64_t M, int32_t n_vars, int64_t* postfix, int64_t* err,
                         void* stream) {
  using namespace sr;
  if (!notation_args_ok(prefix, B, M, n_vars, postfix, err)) return SR_ERR_INVALID_ARGUMENT;
  if (B == 0) return SR_OK;
  reorder_kernel<true><<<(unsigned)((B + 127) / 128), 128, 0, as_stream(stream)>>>(prefix, B, M, (int64_t)VAR + n_vars,
                                                                                postfix, err);
  return launch_check("reorder_kernel<prefix>");
}

int sr_postfix_to_prefix(const int64_t* postfix, int64_t B, int64_t M, int32_t n_vars, int64_t* prefix, int64_t* err,
                         void* stream) {
  using namespace sr;
  if (!notation_args_ok(postfix, B, M, n_vars, prefix, err)) return SR_ERR_INVALID_ARGUMENT;
  if (B == 0) return SR_OK;
  reorder_kernel<false><<<(unsigned)((B + 127) / 128), 128, 0, as_stream(stream)>>>(postfix, B, M,
                                                                                 (int64_t)VAR + n_vars, prefix, err);
  return launch_check("reorder_kernel<postfix>");
}

int sr_prefix_parent(const int64_t* prefix, int64_t B, int64_t M, int32_t n_vars, int64_t* parent, int64_t* err,
                     void* stream) {
  using namespace sr;
  if (!notation_args_ok(prefix, B, M, n_vars, parent, err)) return SR_ERR_INVALID_ARGUMENT;
  if (B == 0) return SR_OK;
  prefix_parent_kernel<<<(unsigned)((B + 127) / 128), 128, 0, as_stream(stream)>>>(prefix, B, M, (int64_t)VAR + n_vars,
                                                                                 parent, err);
  return launch_check("prefix_parent_kernel");
}

int sr_prefix_to_infix(const int64_t* prefix, int64_t B, int64_t M, int32_t n_vars, int64_t* infix, int64_t M_out,
                       int64_t* err, void* stream) {
  using namespace sr;
  if (!notation_args_ok(prefix, B, M, n_vars, M_out > 0 ? (const void*)infix : (const void*)err, err) || M_out < 0)
    return SR_ERR_INVALID_ARGUMENT;
  if (B == 0) return SR_OK;
  const int64_t lparen = (int64_t)VAR + n_vars, rparen = lparen + 1;
  prefix_to_infix_kernel<<<(unsigned)((B + 127) / 128), 128, 0, as_stream(stream)>>>(
      prefix, B, M, (int64_t)VAR + n_vars, lparen, rparen, infix, M_out, err);
  return launch_check("prefix_to_infix_kernel");
}

}  // extern "C"
