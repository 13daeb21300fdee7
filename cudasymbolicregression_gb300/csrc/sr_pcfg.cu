// sr_pcfg.cu -- grammar sampling and infix parsing on the GPU.
//
// The sampler draws expressions from a probabilistic context-free grammar given as
// the reference's CSR tables (src/pcfg.cpp:364-451): rules sorted by left-hand
// side, nt_rule_ptr[s] .. nt_rule_ptr[s + 1] the rules of symbol s, their cumulative
// probabilities, and the concatenated right-hand sides.  A lane derives one expression
// at a time (the derivation is sequential; persistent warps hand a finished lane the
// next expression), leftmost first with an explicit stack,
// exactly as the reference's sample_infix_kernel (src/pcfg_cuda.cu:10-118) does: a
// try restarts when the stack would exceed 128 symbols or the output would exceed
// the padded length, and after max_tries failed tries the expression reports 303.
// The random numbers come from a counter-based SplitMix64 stream per expression
// (Steele, Lea and Flood, "Fast splittable pseudorandom number generators", OOPSLA
// 2014), seeded from the caller's seed, so a seed fixes every expression; the
// oracle restates the same stream, so samples are checked token for token.
//
// The parser is the reference's shunting-yard (src/pcfg_cpu.cpp:121-448, the CUDA
// kernels at src/pcfg_cuda.cu:150-480 are the same): precedence 1 for + -, 2 for
// * /, 3 for ^, 4 for functions and parentheses, 0 (an operand) for everything
// else; ^ and the functions associate to the right.  To postfix it then checks
// that every operator has its operands and exactly one tree remains; to prefix it
// runs the mirrored algorithm from the right end.  One thread per expression; the
// stacks and the CTA's rows sit in shared memory, and rows are read and written by
// the whole CTA in coalesced order.
#include <cstdint>

#include "sr_common.cuh"
#include "sr_ops.cuh"

namespace sr {
namespace pcfg {

constexpr int kHardMax = 128;  // the reference's HARD_MAX_LENGTH (include/pcfg_kernels.h:4)
constexpr int kThreads = 128;  // expressions per CTA

enum : int {
  GEN_MAX_TRIES = 303,
  GEN_NO_RULE = 304,
  PARSE_QUEUE_OVERFLOW = 401,
  PARSE_STACK_OVERFLOW = 402,
  PARSE_PAREN = 403,
  PARSE_UNARY_MISSING = 404,
  PARSE_BINARY_MISSING = 405,
  PARSE_MALFORMED = 407,
  PARSE_UNEXPECTED = 408,
  BAD_NEGATIVE = -1,  // a token below 0
  BAD_RANGE = -2,     // a token at or above the grammar's terminal limit
};

// SplitMix64 finaliser and stream (see the file comment).
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

struct Stream {
  uint64_t s;
  __device__ Stream(uint64_t seed, uint64_t index) : s(mix64(seed ^ mix64(index + 0x9E3779B97F4A7C15ull))) {}
  // uniform in (0, 1], 24 bits: the range the reference's curand_uniform draws from
  __device__ float uniform() {
    s += 0x9E3779B97F4A7C15ull;
    return (float)((mix64(s) >> 40) + 1ull) * (1.0f / 16777216.0f);
  }
};

__global__ void __launch_bounds__(kThreads) sample_infix_kernel(
    const int32_t* __restrict__ nt_ptr, const float* __restrict__ cum, const int32_t* __restrict__ rhs_ptr,
    const int32_t* __restrict__ rhs, int32_t n_symbols, int32_t start, int64_t B, int32_t max_len,
    int32_t max_tries, uint64_t seed, int64_t* __restrict__ out, int64_t* __restrict__ errors) {
  // Persistent warps: warp w owns expressions [w per, (w + 1) per).  Every lane works on
  // one expression and advances it by one symbol per loop turn (the same few branches in
  // every lane); a lane whose expression is finished writes its row and takes the next
  // expression of the warp's range.  So a warp pays for the sum of its lanes' work, not for
  // 32 times its longest derivation (its tries included).  The draws of expression b come
  // from its own stream, so the assignment of expressions to lanes changes no output.
  extern __shared__ int16_t sm[];
  const int t = threadIdx.x, lane = t & 31;
  int16_t* stack = sm;                      // [kHardMax][kThreads]
  int16_t* buf = sm + kHardMax * kThreads;  // [max_len][kThreads]
  const int64_t nwarps = (int64_t)gridDim.x * (kThreads / 32);
  const int64_t w = (int64_t)blockIdx.x * (kThreads / 32) + (t >> 5);
  const int64_t per = (B + nwarps - 1) / nwarps;
  const int64_t wbeg = w * per < B ? w * per : B, wend = wbeg + per < B ? wbeg + per : B;
  const unsigned below = (1u << lane) - 1u;
  int64_t b = wbeg + lane;
  int64_t next = wbeg + 32;
  bool active = b < wend;
  Stream rng(seed, (uint64_t)(active ? b : 0));
  int tries = 0, sp = 0, len = 0, err = 0;
  bool fin = false;
  // a new expression: its first try (or 303 at once when no try is allowed)
  auto begin = [&]() {
    rng = Stream(seed, (uint64_t)b);
    tries = 0;
    err = 0;
    len = 0;
    sp = 0;
    fin = false;
    if (max_tries <= 0) {
      err = GEN_MAX_TRIES;
      fin = true;
    } else {
      stack[t] = (int16_t)start;
      sp = 1;
    }
  };
  if (active) begin();
  while (__any_sync(0xffffffffu, active)) {
    if (active && !fin) {
      // one symbol of the derivation, leftmost first
      bool restart = false;
      const int sym = stack[(--sp) * kThreads + t];
      // an id outside [0, n_symbols) has no rules (a terminal): no table read for it
      const bool has_rules = (unsigned)sym < (unsigned)n_symbols;
      const int r0 = has_rules ? nt_ptr[sym] : 0;
      const int r1 = has_rules ? nt_ptr[sym + 1] : 0;
      if (r0 != r1) {  // a non-terminal: choose a rule, push its right-hand side reversed
        const float u = rng.uniform();
        int chosen = -1;
        for (int r = r0; r < r1; ++r) {
          if (u <= cum[r]) {
            chosen = r;
            break;
          }
        }
        if (chosen < 0) {
          err = GEN_NO_RULE;
          len = 0;
          fin = true;
        } else {
          for (int i = rhs_ptr[chosen + 1] - 1; i >= rhs_ptr[chosen]; --i) {
            if (sp >= kHardMax) {
              restart = true;
              break;
            }
            stack[(sp++) * kThreads + t] = (int16_t)rhs[i];
          }
        }
      } else if (len >= max_len) {  // a terminal past the padded length
        restart = true;
      } else {  // a terminal: emit it
        buf[(len++) * kThreads + t] = (int16_t)sym;
      }
      // a try ends: restarted, or derived completely (an empty derivation fails too)
      if (!fin && (restart || sp == 0)) {
        if (!restart && len > 0) {
          fin = true;
        } else if (++tries >= max_tries) {
          err = GEN_MAX_TRIES;
          len = 0;
          fin = true;
        } else {
          stack[t] = (int16_t)start;
          sp = 1;
          len = 0;
        }
      }
    }
    const bool done = active && fin;
    const unsigned m = __ballot_sync(0xffffffffu, done);
    // the warp writes the rows finished in this turn together, one row at a time, its
    // lanes on consecutive tokens (coalesced), while no lane waits on another's row
    if (m) __syncwarp();  // the finished rows' tokens, written by their lanes
    for (unsigned mm = m; mm; mm &= mm - 1) {
      const int src = __ffs(mm) - 1;
      const int64_t bs = __shfl_sync(0xffffffffu, b, src);
      const int ls = __shfl_sync(0xffffffffu, len, src);
      const int es = __shfl_sync(0xffffffffu, err, src);
      const int ts = (t & ~31) + src;
      for (int i = lane; i < max_len; i += 32) out[bs * max_len + i] = i < ls ? (int64_t)buf[i * kThreads + ts] : NO_OP;
      if (lane == 0) errors[bs] = es;
    }
    if (m) __syncwarp();  // read before their lanes start the next expressions
    if (done) {
      b = next + __popc(m & below);
      active = b < wend;
      if (active) begin();
    }
    next += __popc(m);
  }
}

__device__ __forceinline__ int precedence(int64_t tok, int64_t lp, int64_t rp) {
  if (tok == ADD || tok == SUB) return 1;
  if (tok == MUL || tok == DIV) return 2;
  if (tok == POW) return 3;
  if ((tok >= SIN && tok <= FIFTH) || tok == lp || tok == rp) return 4;
  return 0;
}

__device__ __forceinline__ bool right_assoc(int tok) { return tok == POW || (tok >= SIN && tok <= FIFTH); }

// kPrefix: infix -> prefix (src/pcfg_cpu.cpp:121-259); else infix -> postfix with the
// tree check (src/pcfg_cpu.cpp:261-448).
template <bool kPrefix>
__global__ void __launch_bounds__(kThreads) infix_parse_kernel(const int64_t* __restrict__ infix, int64_t B,
                                                               int64_t M, int32_t n_vars,
                                                               int64_t* __restrict__ outp,
                                                               int64_t* __restrict__ errors) {
  // An M-token row never holds more than M operators on the stack or M tokens in the
  // queue, so both are sized by M (the reference's 128-entry limits cannot be reached
  // for M <= 128; their checks stay).
  extern __shared__ int16_t sm[];
  const int cap = (int)M;
  int16_t* row = sm;                    // [M][kThreads]: the input, then the output
  int16_t* ops = sm + M * kThreads;     // [M][kThreads] operator stack
  // [M][kThreads] output queue.  To postfix the queue lives in the row itself: every
  // queued token was read before (operands when read, operators after, parentheses
  // never), so the queue never holds more tokens than the scan has read and each write
  // lands on a token already consumed.  To prefix the scan runs from the right end and
  // the queue from the left, so it has its own array.
  int16_t* queue = kPrefix ? ops + M * kThreads : row;
  const int t = threadIdx.x;
  const int64_t b0 = (int64_t)blockIdx.x * kThreads;
  const int64_t rows = B - b0 < kThreads ? B - b0 : kThreads;
  const int64_t lp = VAR + n_vars, rp = lp + 1, limit = rp + 1;
  // tokens outside [0, limit) are staged as -1 (negative) or -2 (too large).  Element j
  // of the CTA's block is token i = j % M of row r = j / M; j advances by kThreads, so
  // (r, i) advance by (kThreads / M, kThreads % M) with a carry (no division per token).
  int bad = 0;
  const int Mi = M > 0 ? (int)M : 1, total = (int)(rows * M);  // M = 0: no element
  const int dr = kThreads / Mi, di = kThreads % Mi;
  int r = t / Mi, i = t - (t / Mi) * Mi;
#pragma unroll 4
  for (int j = t; j < total; j += kThreads) {
    const int64_t tok = infix[b0 * M + j];
    int16_t v = (int16_t)tok;
    if (tok < 0 || tok >= limit) v = (int16_t)(tok < 0 ? -1 : -2);
    row[i * kThreads + r] = v;
    r += dr;
    i += di;
    if (i >= Mi) {
      i -= Mi;
      ++r;
    }
  }
  __syncthreads();
  const int64_t b = b0 + t;
  int n_out = 0;
  int err = 0;
  if (b < B) {
    for (int i = 0; i < M; ++i) {
      const int v = row[i * kThreads + t];
      if (v == -1) bad = BAD_NEGATIVE;  // reported before an out-of-range token, as the reference checks
      else if (v == -2 && bad == 0) bad = BAD_RANGE;
    }
    // a token after the first NO_OP
    int len = 0;
    bool ended = false;
    for (int i = 0; i < M && !err; ++i) {
      if (row[i * kThreads + t] == NO_OP) {
        ended = true;
      } else if (ended) {
        err = PARSE_UNEXPECTED;
      } else {
        ++len;
      }
    }
    int sp = 0;
    for (int step = 0; step < len && !err && !bad; ++step) {
      const int tok = row[(kPrefix ? len - 1 - step : step) * kThreads + t];
      const int open = (int)(kPrefix ? rp : lp), close = (int)(kPrefix ? lp : rp);
      const int pt = precedence(tok, lp, rp);
      if (pt == 0) {
        if (n_out >= cap) { err = PARSE_QUEUE_OVERFLOW; break; }
        queue[(n_out++) * kThreads + t] = (int16_t)tok;
      } else if (tok == open) {
        if (sp >= cap) { err = PARSE_STACK_OVERFLOW; break; }
        ops[(sp++) * kThreads + t] = (int16_t)tok;
      } else if (tok == close) {
        while (sp > 0 && ops[(sp - 1) * kThreads + t] != open) {
          if (n_out >= cap) { err = PARSE_QUEUE_OVERFLOW; break; }
          queue[(n_out++) * kThreads + t] = ops[(--sp) * kThreads + t];
        }
        if (err) break;
        if (sp == 0) { err = PARSE_PAREN; break; }
        --sp;
      } else {
        const bool ra = right_assoc(tok);
        while (sp > 0) {
          const int top = ops[(sp - 1) * kThreads + t];
          if (top == open) break;
          const int ptop = precedence(top, lp, rp);
          // to postfix: pop while the top binds at least as tightly (left-assoc) or
          // more tightly (right-assoc); to prefix the two conditions swap
          const bool pop = kPrefix ? (ra ? ptop >= pt : ptop > pt) : (ra ? ptop > pt : ptop >= pt);
          if (!pop) break;
          if (n_out >= cap) { err = PARSE_QUEUE_OVERFLOW; break; }
          queue[(n_out++) * kThreads + t] = (int16_t)top;
          --sp;
        }
        if (err) break;
        if (sp >= cap) { err = PARSE_STACK_OVERFLOW; break; }
        ops[(sp++) * kThreads + t] = (int16_t)tok;
      }
    }
    while (!err && !bad && sp > 0) {
      const int top = ops[(sp - 1) * kThreads + t];
      if (top == (int)(kPrefix ? rp : lp)) { err = PARSE_PAREN; break; }
      if (n_out >= cap) { err = PARSE_QUEUE_OVERFLOW; break; }
      queue[(n_out++) * kThreads + t] = (int16_t)top;
      --sp;
    }
    if (!kPrefix && !err && !bad && n_out > 0) {
      int depth = 0;
      for (int i = 0; i < n_out && !err; ++i) {
        const int tok = queue[i * kThreads + t];
        if (precedence(tok, lp, rp) == 0) {
          ++depth;
        } else {
          const int ar = arity_of(tok);
          if (depth < ar) err = ar == 1 ? PARSE_UNARY_MISSING : PARSE_BINARY_MISSING;
          depth = depth - ar + 1;
        }
      }
      if (!err && depth != 1) err = PARSE_MALFORMED;
    }
    if (err || bad) n_out = 0;
    errors[b] = bad ? bad : err;
  }
  __syncthreads();  // every thread is done with the staged rows
  if (b < B) {
    for (int i = 0; i < M; ++i) {
      int16_t v = (int16_t)NO_OP;
      if (i < n_out) v = queue[(kPrefix ? n_out - 1 - i : i) * kThreads + t];
      row[i * kThreads + t] = v;
    }
  }
  __syncthreads();
  r = t / Mi;
  i = t - r * Mi;
#pragma unroll 4
  for (int j = t; j < total; j += kThreads) {
    outp[b0 * M + j] = row[i * kThreads + r];
    r += dr;
    i += di;
    if (i >= Mi) {
      i -= Mi;
      ++r;
    }
  }
}

static int max_smem_optin() {
  int dev = 0, v = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 48 * 1024;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 48 * 1024;
  return v;
}

template <bool kPrefix>
static int launch_parse(const int64_t* infix, int64_t B, int64_t M, int32_t n_vars, int64_t* outp, int64_t* errors,
                        void* stream) {
  if (B < 0 || M < 0) { set_error("negative size"); return SR_ERR_INVALID_ARGUMENT; }
  if (M > kHardMax) {
    set_error("M must be less than or equal to HARD_MAX_LENGTH, but got %lld > %d.", (long long)M, kHardMax);
    return SR_ERR_UNSUPPORTED;
  }
  if (n_vars < 0 || n_vars > SR_MAX_VARS) { set_error("n_vars out of range (%d)", n_vars); return SR_ERR_UNSUPPORTED; }
  if (B == 0) return SR_OK;
  if (!errors || (M > 0 && (!infix || !outp))) { set_error("null pointer argument"); return SR_ERR_INVALID_ARGUMENT; }
  const int64_t arrays = kPrefix ? 3 : 2;  // row, operator stack (, queue)
  const size_t smem = (size_t)(arrays * M > 0 ? arrays * M : 1) * kThreads * sizeof(int16_t);
  auto kern = infix_parse_kernel<kPrefix>;
  int rc = cuda_check(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "smem");
  if (rc) return rc;
  const int64_t blocks = (B + kThreads - 1) / kThreads;
  kern<<<(unsigned)blocks, kThreads, smem, as_stream(stream)>>>(infix, B, M, n_vars, outp, errors);
  return launch_check(kPrefix ? "infix_parse_kernel<prefix>" : "infix_parse_kernel<postfix>");
}

}  // namespace pcfg
}  // namespace sr

extern "C" {

int sr_pcfg_sample_infix(const int32_t* nt_rule_ptr, const float* nt_rule_cum_probs, const int32_t* rhs_ptr,
                         const int32_t* rhs_concat, int32_t n_symbols, int32_t start_symbol, int64_t B,
                         int32_t max_length, int32_t max_tries, uint64_t seed, int64_t* out, int64_t* errors,
                         void* stream) {
  using namespace sr;
  using namespace sr::pcfg;
  if (B < 0 || max_length < 1 || max_length > kHardMax || max_tries < 0) {
    set_error("bad sampling request: B=%lld max_length=%d max_tries=%d", (long long)B, max_length, max_tries);
    return SR_ERR_INVALID_ARGUMENT;
  }
  if (n_symbols < 1 || n_symbols >= 32768 || start_symbol < 0 || start_symbol >= 32768) {
    set_error("grammar symbol ids must lie in [0, 32768) (n_symbols=%d, start=%d)", n_symbols, start_symbol);
    return SR_ERR_UNSUPPORTED;
  }
  if (B == 0) return SR_OK;
  if (!nt_rule_ptr || !nt_rule_cum_probs || !rhs_ptr || !rhs_concat || !out || !errors) {
    set_error("null pointer argument");
    return SR_ERR_INVALID_ARGUMENT;
  }
  const size_t smem = (size_t)(kHardMax + max_length) * kThreads * sizeof(int16_t);
  if ((int)smem > max_smem_optin()) { set_error("sampling tables do not fit in shared memory"); return SR_ERR_UNSUPPORTED; }
  int rc = cuda_check(cudaFuncSetAttribute(sample_infix_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                      "smem");
  if (rc) return rc;
  // persistent grid: the CTAs that fit at once, or fewer when B is small
  int dev = 0, sms = 0, per_sm = 0;
  rc = cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  if (!rc) rc = cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
  if (!rc)
    rc = cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sample_infix_kernel, kThreads, smem),
                    "occupancy");
  if (rc) return rc;
  int64_t blocks = (int64_t)sms * (per_sm > 0 ? per_sm : 1);
  const int64_t need = (B + kThreads - 1) / kThreads;
  if (blocks > need) blocks = need;
  sample_infix_kernel<<<(unsigned)blocks, kThreads, smem, as_stream(stream)>>>(
      nt_rule_ptr, nt_rule_cum_probs, rhs_ptr, rhs_concat, n_symbols, start_symbol, B, max_length, max_tries, seed,
      out, errors);
  return launch_check("sample_infix_kernel");
}

int sr_infix_to_postfix(const int64_t* infix, int64_t B, int64_t M, int32_t n_vars, int64_t* postfix,
                        int64_t* errors, void* stream) {
  return sr::pcfg::launch_parse<false>(infix, B, M, n_vars, postfix, errors, stream);
}

int sr_infix_to_prefix(const int64_t* infix, int64_t B, int64_t M, int32_t n_vars, int64_t* prefix, int64_t* errors,
                       void* stream) {
  return sr::pcfg::launch_parse<true>(infix, B, M, n_vars, prefix, errors, stream);
}

}  // extern "C"
