// sr_eval.cu -- tape validation/staging, forward evaluation and adjoint kernels.
//
// Design (sm_103a): one warp interprets one tape; its lanes cover data points, so
// opcode dispatch is warp-uniform and every cache row segment a warp writes is a
// contiguous 128-byte line.  The tape words of a warp and the node values of the
// points it is working on live in shared memory; children are read from there,
// never from HBM.  The forward pass writes each (node, point) value once with a
// streaming store, which makes it bound by HBM write bandwidth; the adjoint pass
// recomputes node values instead of reading the saved cache and reads the dense
// output gradient once.
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "sr_common.cuh"
#include "sr_ops.cuh"

namespace sr {

static thread_local char g_err[512];

__host__ __device__ __forceinline__ size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

// ------------------------------------------------------------------------------------
// Validation + staging.  One warp per tape row; lanes over nodes.
// Validation follows the reference (src/evaluation_kernels_cuda.cu:13-49): a child
// that is not NULL_CHILD counts towards the arity and must be below its parent
// (101); the count must equal the arity (102).  Inputs the reference accepts but
// then reads out of bounds (a counted child < 0, or a unary node whose only child
// sits in the second slot) are reported as 101 here.
// ------------------------------------------------------------------------------------
template <bool kStage>
__global__ void __launch_bounds__(256) tape_compile_kernel(const int64_t* __restrict__ ops,
                                                           const int64_t* __restrict__ ch, int64_t B,
                                                           int64_t M, int64_t ops_sb, int64_t ops_sm,
                                                           int64_t ch_sb, int64_t ch_sm, int64_t ch_si,
                                                           int32_t n_vars, uint32_t* __restrict__ desc,
                                                           int32_t* __restrict__ meta,
                                                           int32_t* __restrict__ status) {
  const int lane = threadIdx.x & 31;
  const int64_t warps_total = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t b = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); b < B; b += warps_total) {
    int count = 0, last = -1;
    int err = 0;
    for (int64_t m0 = 0; m0 < M; m0 += 32) {
      const int64_t m = m0 + lane;
      const bool in = m < M;
      int64_t op = 0;
      if (in) {
        op = ops[b * ops_sb + m * ops_sm];
        const int64_t c0 = ch[b * ch_sb + m * ch_sm];
        const int64_t c1 = ch[b * ch_sb + m * ch_sm + ch_si];
        const int ar = arity_of(op);
        int actual = 0;
        int e = 0;
        if (c0 != -1) { actual++; if (c0 >= m) e = ERR_CHILD_GEQ_PARENT; }
        if (!e && c1 != -1) { actual++; if (c1 >= m) e = ERR_CHILD_GEQ_PARENT; }
        if (!e && actual != ar) e = ERR_ARITY;
        if (!e && ar >= 1 && c0 < 0) e = ERR_CHILD_GEQ_PARENT;
        if (!e && ar == 2 && c1 < 0) e = ERR_CHILD_GEQ_PARENT;
        err = err ? err : e;
        if (kStage) {
          int code;
          uint32_t f0 = 0, f1 = 0;
          if (op == NO_OP || (op >= LEARNABLE && op <= E_) || (op >= SIN && op <= FIFTH) ||
              (op >= ADD && op <= POW)) {
            code = (int)op;
            if (ar >= 1 && !e) f0 = (uint32_t)c0;
            if (ar == 2 && !e) f1 = (uint32_t)c1;
          } else if (op >= VAR && op < VAR + (int64_t)n_vars) {
            code = VAR;
            f0 = (uint32_t)(op - VAR);
          } else {
            code = ZERO;
          }
          desc[b * M + m] = pack(code, f0, f1);
        }
      }
      const unsigned real = __ballot_sync(0xffffffffu, in && op != NO_OP);
      count += __popc(real);
      if (real) last = (int)m0 + 31 - __clz((int)real);
    }
    if (err) report(status, err);
    if (kStage) {
      const int root = count > 0 ? count - 1 : 0;
      int kroot = 0, kall = 0, nops = 0;
      for (int64_t m0 = 0; m0 < M; m0 += 32) {
        const int64_t m = m0 + lane;
        const int64_t op = m < M ? ops[b * ops_sb + m * ops_sm] : -1;
        const bool lc = op == LEARNABLE;
        kall += __popc(__ballot_sync(0xffffffffu, lc));
        kroot += __popc(__ballot_sync(0xffffffffu, lc && m <= root));
        nops += __popc(__ballot_sync(0xffffffffu, m <= root && (op == NO_OP || arity_of(op) >= 1)));
      }
      if (lane == 0) {
        meta[b * 4 + 0] = last + 1;
        meta[b * 4 + 1] = root;
        meta[b * 4 + 2] = kroot;
        meta[b * 4 + 3] = kall;
        // batch summary: stats[1] = max L_eff, stats[2] = max root + 1, stats[3] = max constants to root
        atomicMax(status + 1, last + 1);
        atomicMax(status + 2, root + 1);
        atomicMax(status + 3, kroot);
        atomicMax(status + 4, nops);
      }
    }
  }
}

// ------------------------------------------------------------------------------------
// Forward.  Work unit = (tape, slice of at most kSlice points); units are taken in
// grid-stride order over the tapes sorted longest first, so every warp of the
// persistent grid gets a similar mix of long and short tapes.  One point per lane:
// the per-warp node table is L_max * 128 bytes, which keeps ~24 warps per SM.
// ------------------------------------------------------------------------------------
constexpr int kSlice = 256;

// Fill count values at p with NaN, 16-byte vector stores in the aligned middle;
// threads tid = 0 .. nthreads - 1 share the range.
template <typename T>
__device__ __forceinline__ void fill_nan(T* p, size_t count, int tid, int nthreads) {
  const T qnan = M_<T>::nan();
  constexpr int kVec = 16 / sizeof(T);
  size_t head = (size_t)((16 - (reinterpret_cast<uintptr_t>(p) & 15)) & 15) / sizeof(T);
  if (reinterpret_cast<uintptr_t>(p) % sizeof(T)) head = count;  // unaligned element type: scalar path
  if (head > count) head = count;
  for (size_t i = tid; i < head; i += nthreads) __stcs(p + i, qnan);
  const size_t nvec = (count - head) / kVec;
  float4 v4;
  if (sizeof(T) == 4) {
    const float f = __int_as_float(0x7fffffff);
    v4 = make_float4(f, f, f, f);
  } else {
    const float lo = __int_as_float(0xffffffff), hi = __int_as_float(0x7fffffff);
    v4 = make_float4(lo, hi, lo, hi);
  }
  float4* q = reinterpret_cast<float4*>(p + head);
  for (size_t i = tid; i < nvec; i += nthreads) __stcs(q + i, v4);
  for (size_t i = head + nvec * kVec + tid; i < count; i += nthreads) __stcs(p + i, qnan);
}

// Rows L..M-1 of every tape's cache block are NaN.  They form one contiguous range per
// tape, streamed by one CTA per tape (grid-stride) on a side stream, concurrently with
// the forward kernel, which writes only the real rows: the forward is bound by
// instruction latency and leaves most of the HBM write bandwidth to this kernel.
// A tape longer than the max_len the call was given is evaluated by no class grid: its
// whole block is NaN, so no row keeps what the buffer held before.
template <typename T>
__global__ void __launch_bounds__(256) pad_fill_kernel(const int32_t* __restrict__ meta, int64_t B, int64_t M,
                                                       int64_t NK, int Lmax, T* __restrict__ cache) {
  for (int64_t b = blockIdx.x; b < B; b += gridDim.x) {
    int64_t L = meta[b * 4];
    if (L > Lmax) L = 0;
    fill_nan(cache + (size_t)b * M * NK + (size_t)L * NK, (size_t)(M - L) * NK, (int)threadIdx.x, (int)blockDim.x);
  }
}

// Shared-memory layout of one warp of the forward kernel: the tape words, the
// operator program (dense code | node << 8, two operand source words), the lists of
// variable leaves and of broadcast leaves (learnable, fixed, codes that evaluate to
// 0), the broadcast entries (entry 0 = 0, entry 1 + k = value of leaf k) and one
// value row of 32 points per node.
struct FwdLayout {
  uint32_t pw, psa, psb, lvar, lbc, bc, vals, bytes;
};

template <typename T>
__host__ __device__ __forceinline__ FwdLayout forward_layout(int Lmax) {
  const uint32_t lb = (uint32_t)align16((size_t)Lmax * 4);
  FwdLayout l;
  l.pw = lb;  // the tape words sit at offset 0
  l.psa = 2 * lb;
  l.psb = 3 * lb;
  l.lvar = 4 * lb;
  l.lbc = 5 * lb;
  l.bc = 6 * lb;
  l.vals = l.bc + (uint32_t)align16((size_t)(Lmax + 1) * sizeof(T));
  l.bytes = l.vals + (uint32_t)Lmax * 32u * (uint32_t)sizeof(T);
  return l;
}

template <typename T>
__device__ __forceinline__ T lds_operand(const unsigned char* wb, uint32_t w, int li) {
  return *reinterpret_cast<const T*>(wb + (w & 0xffffffu) + (uint32_t)li * (w >> 24));
}

template <typename T>
__device__ __forceinline__ T* row_at(unsigned char* wb, uint32_t off, int li) {
  return reinterpret_cast<T*>(wb + off) + li;
}

// Per unit the warp compiles its tape into an operator program whose operands are
// precomputed addresses (the value row of an operator node or variable leaf, or the
// broadcast entry of any other leaf), so the point loop runs the leaves as plain
// loads and stores and dispatches on the opcode for operator nodes only.
template <typename T, bool kMulti>
__global__ void __launch_bounds__(256) eval_forward_kernel(const T* __restrict__ X, int64_t N, int64_t n_x,
                                                           const uint32_t* __restrict__ desc,
                                                           const int32_t* __restrict__ meta,
                                                           const int32_t* __restrict__ order, int64_t B,
                                                           int64_t M, int Llo, int Lhi, const T* __restrict__ C,
                                                           int64_t c_sb, int64_t c_sm, int64_t c_sk, int64_t K_,
                                                           T* __restrict__ cache) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int64_t K = kMulti ? K_ : 1;  // one constant set: the strides fold at compile time
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  constexpr uint32_t RB = 32u * (uint32_t)sizeof(T);
  constexpr uint32_t kRowStride = (uint32_t)sizeof(T) << 24;
  const FwdLayout ly = forward_layout<T>(Lhi);
  unsigned char* wb = smem + (size_t)warp * ly.bytes;
  uint32_t* tape = reinterpret_cast<uint32_t*>(wb);
  uint32_t* pw = reinterpret_cast<uint32_t*>(wb + ly.pw);
  uint32_t* psa = reinterpret_cast<uint32_t*>(wb + ly.psa);
  uint32_t* psb = reinterpret_cast<uint32_t*>(wb + ly.psb);
  int* lvar = reinterpret_cast<int*>(wb + ly.lvar);
  int* lbc = reinterpret_cast<int*>(wb + ly.lbc);
  T* bc = reinterpret_cast<T*>(wb + ly.bc);
  T* vals = reinterpret_cast<T*>(wb + ly.vals);
  const unsigned below = (1u << lane) - 1u;
  const int64_t nslices = (N + kSlice - 1) / kSlice;
  const int64_t units = B * nslices;
  for (int64_t u = (int64_t)blockIdx.x * nwarp + warp; u < units; u += (int64_t)gridDim.x * nwarp) {
    const int64_t ti = u / nslices, sl = u - ti * nslices;
    const int64_t b = order ? (int64_t)order[ti] : ti;
    const int L = meta[b * 4];
    if (L <= Llo || L > Lhi) continue;  // another class's grid takes it (warp-uniform)
    for (int k = lane; k < L; k += 32) tape[k] = desc[b * M + k];
    if (lane == 0) bc[0] = T(0);
    __syncwarp();
    auto src_word = [&](int c) -> uint32_t {
      const int cc = code_of(tape[c]);
      if (cc == NO_OP || cc == VAR || arity_of(cc) >= 1) return (ly.vals + (uint32_t)c * RB) | kRowStride;
      return ly.bc + (uint32_t)(1 + c) * (uint32_t)sizeof(T);
    };
    int nop = 0, nvar = 0, nbc = 0;
    for (int k0 = 0; k0 < L; k0 += 32) {
      const int k = k0 + lane;
      const uint32_t d = k < L ? tape[k] : 0u;
      const int code = k < L ? code_of(d) : -1;
      const bool isop = k < L && (code == NO_OP || arity_of(code) >= 1);
      const bool isvar = code == VAR;
      const bool isbc = k < L && !isop && !isvar;
      const unsigned mo = __ballot_sync(0xffffffffu, isop);
      const unsigned mv = __ballot_sync(0xffffffffu, isvar);
      const unsigned mb = __ballot_sync(0xffffffffu, isbc);
      if (isop) {
        const int ar = arity_of(code);
        const int pos = nop + __popc(mo & below);
        pw[pos] = (uint32_t)dense_op(code) | ((uint32_t)k << 8);
        psa[pos] = ar >= 1 ? src_word(child0(d)) : ly.bc;
        psb[pos] = ar == 2 ? src_word(child1(d)) : ly.bc;
      }
      if (isvar) lvar[nvar + __popc(mv & below)] = k;
      if (isbc) {
        lbc[nbc + __popc(mb & below)] = k;
        if (code != LEARNABLE) bc[1 + k] = node_value<T>(code, T(0), T(0), T(0), T(0));
      }
      nop += __popc(mo);
      nvar += __popc(mv);
      nbc += __popc(mb);
    }
    // K constant sets: the cache is (B, M, N, K), set kk of node k, point n at
    // ((b M + k) N + n) K + kk
    T* out = cache + (size_t)b * M * N * K;
    const int64_t rs = N * K;
    const int64_t n0 = sl * kSlice, n1 = min(N, n0 + kSlice);
    for (int64_t kk = 0; kk < K; ++kk) {
      __syncwarp();  // every lane is done with the previous set's broadcast entries
      const T* Crow = C + b * c_sb + kk * c_sk;
      for (int j = lane; j < nbc; j += 32) {
        const int k = lbc[j];
        if (code_of(tape[k]) == LEARNABLE) bc[1 + k] = __ldg(Crow + (int64_t)k * c_sm);
      }
      __syncwarp();
      for (int64_t base = n0; base < n1; base += 32) {
        const int64_t n = base + lane;
        const bool valid = n < n1;
        const int64_t nn = valid ? n : n1 - 1;
        T* o = out + kk + nn * K;  // node k of this point at o[k * rs]
        for (int j = 0; j < nvar; ++j) {
          const int k = lvar[j];
          const T x = __ldg(X + nn * n_x + child0(tape[k]));
          vals[k * 32 + lane] = x;
          if (valid) __stcs(o + (int64_t)k * rs, x);
        }
        if (valid) {
          for (int j = 0; j < nbc; ++j) {
            const int k = lbc[j];
            __stcs(o + (int64_t)k * rs, bc[1 + k]);
          }
        }
        for (int i = 0; i < nop; ++i) {
          const uint32_t w = pw[i];
          const int k = (int)(w >> 8);
          const T r = op_value<T>((int)(w & 0xffu), lds_operand<T>(wb, psa[i], lane), lds_operand<T>(wb, psb[i], lane));
          vals[k * 32 + lane] = r;
          if (valid) __stcs(o + (int64_t)k * rs, r);
        }
      }
    }
    // rows after the last real node are filled with NaN by pad_fill_kernel
    __syncwarp();
  }
}

// ------------------------------------------------------------------------------------
// Adjoint for a dense grad_out: the padding-row check and the adjoint proper, run
// concurrently (the check streams the padding rows from HBM, the adjoint is bound by
// instruction latency).
// ------------------------------------------------------------------------------------

// Error precedence of the adjoint: a gradient on a NO_OP row (201) is reported over a
// zero denominator (204) whichever kernel finds it first, as in the reference, whose
// reverse loop meets the padding rows first.
__device__ __forceinline__ void report_adjoint(int* status, int code) {
  if (!code) return;
  const int prev = atomicCAS(status, 0, code);
  if (code == ERR_GRAD_ON_NO_OP && prev == ERR_DIV_BY_ZERO) atomicCAS(status, ERR_DIV_BY_ZERO, code);
}

// ---- padding rows: any nonzero output gradient on a NO_OP row is error 201 ----------
// One CTA per tape (grid-stride): rows L..M-1 of its (M, N) gradient block are one
// contiguous range, read with 16-byte streaming loads, four in flight per thread.
// A tape longer than the max_len the call was given is adjoined by no class grid: it
// is reported (status 602) instead of being skipped silently.
template <typename T>
__global__ void __launch_bounds__(256) padding_check_kernel(const T* __restrict__ gout,
                                                            const int32_t* __restrict__ meta, int64_t B,
                                                            int64_t M, int64_t N, int Lmax,
                                                            int32_t* __restrict__ status) {
  constexpr int kVec = 16 / sizeof(T);
  for (int64_t b = blockIdx.x; b < B; b += gridDim.x) {
    // the whole CTA stops once a 201 is recorded (uniform decision)
    if (__syncthreads_or(threadIdx.x == 0 && *reinterpret_cast<volatile int32_t*>(status) == ERR_GRAD_ON_NO_OP))
      return;
    const int64_t L = meta[b * 4];
    if (L > Lmax) {
      if (threadIdx.x == 0) report(status, SR_TAPE_EXCEEDS_LAUNCH);
      continue;
    }
    const T* p = gout + (size_t)b * M * N + (size_t)L * N;
    const size_t count = (size_t)(M - L) * N;
    size_t head = (size_t)((16 - (reinterpret_cast<uintptr_t>(p) & 15)) & 15) / sizeof(T);
    if (reinterpret_cast<uintptr_t>(p) % sizeof(T)) head = count;  // unaligned element type: scalar path
    if (head > count) head = count;
    bool nz = false;
    for (size_t i = threadIdx.x; i < head; i += blockDim.x) nz |= __ldcs(p + i) != T(0);
    const size_t nvec = (count - head) / kVec;
    const float4* q = reinterpret_cast<const float4*>(p + head);
    size_t i = threadIdx.x;
    for (; i + 3 * blockDim.x < nvec; i += 4 * blockDim.x) {
      float4 v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) v[u] = __ldcs(q + i + u * blockDim.x);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (sizeof(T) == 4) {
          nz |= (v[u].x != 0.f) | (v[u].y != 0.f) | (v[u].z != 0.f) | (v[u].w != 0.f);
        } else {
          const double* d = reinterpret_cast<const double*>(&v[u]);
          nz |= (d[0] != 0.0) | (d[1] != 0.0);
        }
      }
    }
    for (; i < nvec; i += blockDim.x) {
      const float4 v = __ldcs(q + i);
      if (sizeof(T) == 4) {
        nz |= (v.x != 0.f) | (v.y != 0.f) | (v.z != 0.f) | (v.w != 0.f);
      } else {
        const double* d = reinterpret_cast<const double*>(&v);
        nz |= (d[0] != 0.0) | (d[1] != 0.0);
      }
    }
    for (size_t j = head + nvec * kVec + threadIdx.x; j < count; j += blockDim.x) nz |= __ldcs(p + j) != T(0);
    if (__syncthreads_or(nz) && threadIdx.x == 0) report_adjoint(status, ERR_GRAD_ON_NO_OP);
  }
}

// ---- asynchronous staging of output-gradient rows -----------------------------------

__device__ __forceinline__ void cp_async(void* dst_smem, const void* src, int cp_bytes, int src_bytes) {
  const uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(dst_smem));
  if (cp_bytes == 16) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(src), "r"(src_bytes) : "memory");
  } else if (cp_bytes == 8) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(d), "l"(src), "r"(src_bytes) : "memory");
  } else {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(src), "r"(src_bytes) : "memory");
  }
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int kPending>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(kPending) : "memory"); }

// Copies rows 0..L-1, points base..base+32V-1 of the gradient block G (node k, point
// n at G[k * rs + n * es]) into buf[k][32 V] (zero beyond N).  vec16 (es == 1, rows
// 16-byte aligned): each lane moves 16 bytes (E = 16 / sizeof(T) points), 32 E / (32 V)
// rows per instruction; otherwise one element per lane, point and row.
template <typename T, int V>
__device__ __forceinline__ void stage_rows(T* buf, const T* G, int L, int64_t N, int64_t rs, int64_t es,
                                           int64_t base, int lane, bool vec16) {
  constexpr int RW = 32 * V;
  if (vec16) {
    constexpr int E = 16 / sizeof(T);
    constexpr int kLanesPerRow = RW / E;
    static_assert(kLanesPerRow <= 32 && 32 % kLanesPerRow == 0, "row width");
    constexpr int kRowsPerStep = 32 / kLanesPerRow;
    const int r0 = lane / kLanesPerRow, p = (lane % kLanesPerRow) * E;
    const int64_t left = N - (base + p);
    const int bytes = left >= E ? 16 : (left > 0 ? (int)left * (int)sizeof(T) : 0);
    for (int k = r0; k < L; k += kRowsPerStep) {
      const T* src = bytes ? G + (size_t)k * rs + base + p : G;
      cp_async(buf + k * RW + p, src, 16, bytes);
    }
  } else {
#pragma unroll
    for (int v = 0; v < V; ++v) {
      const int64_t n = base + v * 32 + lane;
      const int bytes = n < N ? (int)sizeof(T) : 0;
      for (int k = 0; k < L; ++k) {
        const T* src = bytes ? G + (size_t)k * rs + n * es : G;
        cp_async(buf + k * RW + v * 32 + lane, src, (int)sizeof(T), bytes);
      }
    }
  }
  cp_async_commit();
}

// Copies the value rows of this chunk from the forward cache Cc (node k, point n at
// Cc[k * rs + n * es]) into vals[k][32 V] for the operator nodes (rows at byte offsets
// prow[0..nop) from vals_off) and the variable leaves lvar[0..nvar); the rows of the
// learnable leaves hold their gradient partial sums and are not touched.  Same copy
// shapes as stage_rows.
template <typename T, int V>
__device__ __forceinline__ void stage_value_rows(T* vals, const T* Cc, const uint32_t* prow, uint32_t vals_off,
                                                 int nop, const int* lvar, int nvar, int64_t N, int64_t rs,
                                                 int64_t es, int64_t base, int lane, bool vec16) {
  constexpr int RW = 32 * V;
  constexpr uint32_t RB = RW * (uint32_t)sizeof(T);
  const int nrows = nop + nvar;
  auto node_of = [&](int r) -> int { return r < nop ? (int)((prow[r] - vals_off) / RB) : lvar[r - nop]; };
  if (vec16) {
    constexpr int E = 16 / sizeof(T);
    constexpr int kLanesPerRow = RW / E;
    constexpr int kRowsPerStep = 32 / kLanesPerRow;
    const int r0 = lane / kLanesPerRow, p = (lane % kLanesPerRow) * E;
    const int64_t left = N - (base + p);
    const int bytes = left >= E ? 16 : (left > 0 ? (int)left * (int)sizeof(T) : 0);
    for (int r = r0; r < nrows; r += kRowsPerStep) {
      const int k = node_of(r);
      const T* src = bytes ? Cc + (size_t)k * rs + base + p : Cc;
      cp_async(vals + k * RW + p, src, 16, bytes);
    }
  } else {
#pragma unroll
    for (int v = 0; v < V; ++v) {
      const int64_t n = base + v * 32 + lane;
      const int bytes = n < N ? (int)sizeof(T) : 0;
      for (int r = 0; r < nrows; ++r) {
        const int k = node_of(r);
        const T* src = bytes ? Cc + (size_t)k * rs + n * es : Cc;
        cp_async(vals + k * RW + v * 32 + lane, src, (int)sizeof(T), bytes);
      }
    }
  }
  cp_async_commit();
}

// ------------------------------------------------------------------------------------
// Adjoint.  One warp per tape, 32 V points per chunk (V points per lane: the per-node
// decode and dispatch serve V points).  The host launches one persistent grid per
// class of tape lengths (Llo, Lhi], each sized for its class's shared memory, so short
// tapes run at the occupancy their size allows; every grid scans the whole work order
// and takes the tapes of its class.  Per tape the warp compiles its nodes into an
// operator program (NO_OP nodes included: their value NaN and their adjoint check
// matter) whose operands are precomputed addresses in the warp's shared memory:
//   source word = byte offset (bits 0..23) | lane stride in bytes (bits 24..31): the
//                 value row of an operator node or a variable leaf (stride sizeof(T))
//                 or the broadcast entry of any other leaf (stride 0);
//   adjoint destination = byte offset of the child's adjoint row.
// Every node has an adjoint row.  Per chunk the output-gradient rows are staged into
// them with cp.async.  With the forward cache (kCached: the reference's backward reads
// it too) the value rows of the operator nodes and variables are staged from it in the
// same way, the cache holding exactly the values the forward kernel computed; without
// it the operator nodes are recomputed while the copies are in flight.  The reverse
// sweep then adds the contributions into the children's rows in the
// reference's order (parents from the last to the first, child 0 before child 1), and
// the leaves are reduced afterwards.  A learnable constant's operand is a broadcast
// entry, so its value row is free and holds its per-lane gradient sums over the
// chunks; one butterfly per constant and set ends the sum (a fixed order: grad_C is
// deterministic).
// ------------------------------------------------------------------------------------
struct BwdLayout {
  uint32_t pcode, psa, psb, prow, pda, pdb, lcon, lvar, bc, vals, adj, bytes;
};

template <typename T, int V>
__host__ __device__ __forceinline__ BwdLayout backward_layout(int Lmax) {
  const uint32_t lb = (uint32_t)align16((size_t)Lmax * 4);
  BwdLayout l;
  l.pcode = lb;  // the tape words sit at offset 0
  l.psa = 2 * lb;
  l.psb = 3 * lb;
  l.prow = 4 * lb;
  l.pda = 5 * lb;
  l.pdb = 6 * lb;
  l.lcon = 7 * lb;
  l.lvar = 8 * lb;
  l.bc = 9 * lb;
  l.vals = l.bc + (uint32_t)align16((size_t)(Lmax + 1) * sizeof(T));
  const uint32_t rows = (uint32_t)Lmax * 32u * V * (uint32_t)sizeof(T);
  l.adj = l.vals + rows;
  l.bytes = l.adj + rows;
  return l;
}

template <typename T, bool kMulti, int V, bool kCached>
__global__ void __launch_bounds__(256, 4) eval_backward_kernel(
    const T* __restrict__ X, int64_t N, int64_t n_x, const uint32_t* __restrict__ desc,
    const int32_t* __restrict__ meta, const int32_t* __restrict__ order, int64_t B, int64_t M, int Llo, int Lhi,
    const T* __restrict__ C, int64_t c_sb, int64_t c_sm, int64_t c_sk, int64_t K_, const T* __restrict__ cache,
    const T* __restrict__ gout, T* __restrict__ gC, T* __restrict__ gX, int32_t* __restrict__ status, bool vec16,
    bool cvec16) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int64_t K = kMulti ? K_ : 1;  // one constant set: the strides fold at compile time
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  constexpr uint32_t RW = 32u * V;                       // elements per row
  constexpr uint32_t RB = RW * (uint32_t)sizeof(T);      // bytes per row
  constexpr uint32_t kRowStride = (uint32_t)sizeof(T) << 24;
  const BwdLayout ly = backward_layout<T, V>(Lhi);
  unsigned char* wb = smem + (size_t)warp * ly.bytes;
  uint32_t* tape = reinterpret_cast<uint32_t*>(wb);
  uint32_t* pcode = reinterpret_cast<uint32_t*>(wb + ly.pcode);
  uint32_t* psa = reinterpret_cast<uint32_t*>(wb + ly.psa);
  uint32_t* psb = reinterpret_cast<uint32_t*>(wb + ly.psb);
  uint32_t* prow = reinterpret_cast<uint32_t*>(wb + ly.prow);
  uint32_t* pda = reinterpret_cast<uint32_t*>(wb + ly.pda);
  uint32_t* pdb = reinterpret_cast<uint32_t*>(wb + ly.pdb);
  int* lcon = reinterpret_cast<int*>(wb + ly.lcon);
  int* lvar = reinterpret_cast<int*>(wb + ly.lvar);
  T* bc = reinterpret_cast<T*>(wb + ly.bc);
  T* vals = reinterpret_cast<T*>(wb + ly.vals);
  T* adj = reinterpret_cast<T*>(wb + ly.adj);
  const uint32_t adj_delta = ly.adj - ly.vals;
  const unsigned below = (1u << lane) - 1u;
  for (int64_t ti = (int64_t)blockIdx.x * nwarp + warp; ti < B; ti += (int64_t)gridDim.x * nwarp) {
    const int64_t b = order ? (int64_t)order[ti] : ti;
    const int L = meta[b * 4];
    if (L <= Llo || L > Lhi) continue;  // another class's grid takes it (warp-uniform)
    for (int k = lane; k < L; k += 32) tape[k] = desc[b * M + k];
    if (lane == 0) bc[0] = T(0);
    __syncwarp();
    // source word of operand node c: its value row, or its broadcast entry
    auto src_word = [&](int c) -> uint32_t {
      const int cc = code_of(tape[c]);
      if (cc == NO_OP || cc == VAR || arity_of(cc) >= 1) return (ly.vals + (uint32_t)c * RB) | kRowStride;
      return ly.bc + (uint32_t)(1 + c) * (uint32_t)sizeof(T);
    };
    // compaction: operator nodes, learnable and variable leaves; the broadcast
    // entries of fixed leaves (and of codes that evaluate to 0) now
    int nop = 0, ncon = 0, nvar = 0;
    for (int k0 = 0; k0 < L; k0 += 32) {
      const int k = k0 + lane;
      const uint32_t d = k < L ? tape[k] : 0u;
      const int code = k < L ? code_of(d) : -1;
      const bool isop = k < L && (code == NO_OP || arity_of(code) >= 1);
      const bool iscon = code == LEARNABLE, isvar = code == VAR;
      const unsigned mo = __ballot_sync(0xffffffffu, isop);
      const unsigned mc = __ballot_sync(0xffffffffu, iscon);
      const unsigned mv = __ballot_sync(0xffffffffu, isvar);
      if (isop) {
        const int ar = arity_of(code);
        const int pos = nop + __popc(mo & below);
        const uint32_t own = ly.adj + (uint32_t)k * RB;  // never written through (arity < 2)
        uint32_t sa = ly.bc, sb = ly.bc, da = own, db = own;
        if (ar >= 1) {
          sa = src_word(child0(d));
          da = ly.adj + (uint32_t)child0(d) * RB;
        }
        if (ar == 2) {
          sb = src_word(child1(d));
          db = ly.adj + (uint32_t)child1(d) * RB;
        }
        pcode[pos] = (uint32_t)dense_op(code);
        psa[pos] = sa;
        psb[pos] = sb;
        prow[pos] = ly.vals + (uint32_t)k * RB;
        pda[pos] = da;
        pdb[pos] = db;
      } else if (k < L && !iscon && !isvar) {
        bc[1 + k] = node_value<T>(code, T(0), T(0), T(0), T(0));
      }
      if (iscon) lcon[ncon + __popc(mc & below)] = k;
      if (isvar) lvar[nvar + __popc(mv & below)] = k;
      nop += __popc(mo);
      ncon += __popc(mc);
      nvar += __popc(mv);
    }
    int err = 0;
    const int64_t nchunks = (N + RW - 1) / RW;
    // K constant sets, one after the other: grad_out is (B, M, N, K), set kk of
    // node k, point n at ((b M + k) N + n) K + kk
    for (int64_t kk = 0; kk < K; ++kk) {
      const T* Crow = C + b * c_sb + kk * c_sk;
      for (int j = lane; j < ncon; j += 32) bc[1 + lcon[j]] = __ldg(Crow + (int64_t)lcon[j] * c_sm);
      for (int j = 0; j < ncon; ++j) {
#pragma unroll
        for (int v = 0; v < V; ++v) vals[lcon[j] * RW + v * 32 + lane] = T(0);
      }
      const T* G = gout + (size_t)b * M * N * K + kk;
      const T* Cc = kCached ? cache + (size_t)b * M * N * K + kk : nullptr;
      const int64_t rs = N * K;
      __syncwarp();
      for (int64_t c = 0; c < nchunks; ++c) {
        const int64_t base = c * RW;
        int64_t nn[V];
        bool valid[V];
#pragma unroll
        for (int v = 0; v < V; ++v) {
          const int64_t n = base + v * 32 + lane;
          valid[v] = n < N;
          nn[v] = valid[v] ? n : N - 1;
        }
        // the adjoint seeds (grad_out rows of this chunk) are in flight while the node
        // values are recomputed.  Seeding with the raw values instead of 0 + grad_out
        // (the reference's zeros_like(cache).add_(grad_output)) can only flip the sign
        // of a zero seed, which no output can see: a zero adjoint contributes nothing
        stage_rows<T, V>(adj, G, L, N, rs, K, base, lane, vec16);
        if constexpr (kCached) {
          stage_value_rows<T, V>(vals, Cc, prow, ly.vals, nop, lvar, nvar, N, rs, K, base, lane, cvec16);
        } else {
          for (int j = 0; j < nvar; ++j) {
            const int k = lvar[j];
            const int var = child0(tape[k]);
#pragma unroll
            for (int v = 0; v < V; ++v) vals[k * RW + v * 32 + lane] = __ldg(X + nn[v] * n_x + var);
          }
          __syncwarp();
          for (int i = 0; i < nop; ++i) {
            const int code = (int)pcode[i];
            const uint32_t sa = psa[i], sb = psb[i], pr = prow[i];
            T a[V], bb[V], r[V];
#pragma unroll
            for (int v = 0; v < V; ++v) {
              a[v] = lds_operand<T>(wb, sa, v * 32 + lane);
              bb[v] = lds_operand<T>(wb, sb, v * 32 + lane);
            }
            op_value_v<T, V>(code, a, bb, r);
#pragma unroll
            for (int v = 0; v < V; ++v) *row_at<T>(wb, pr, v * 32 + lane) = r[v];
          }
        }
        cp_async_wait<0>();
        __syncwarp();
        for (int i = nop - 1; i >= 0; --i) {
          const int code = (int)pcode[i];
          const uint32_t sa = psa[i], sb = psb[i], pr = prow[i], da = pda[i], db = pdb[i];
          T g[V], a[V], bb[V], vv[V], o0[V], o1[V];
          bool a0[V], a1[V];
          int e[V];
#pragma unroll
          for (int v = 0; v < V; ++v) {
            const int li = v * 32 + lane;
            g[v] = *row_at<T>(wb, pr + adj_delta, li);
            a[v] = lds_operand<T>(wb, sa, li);
            bb[v] = lds_operand<T>(wb, sb, li);
            vv[v] = *row_at<T>(wb, pr, li);
          }
          op_adjoint_v<T, V>(code, g, a, bb, vv, a0, o0, a1, o1, e);
#pragma unroll
          for (int v = 0; v < V; ++v) {
            if (valid[v]) {
              const int li = v * 32 + lane;
              if (e[v] && !err) err = e[v];
              if (a0[v]) { T* d = row_at<T>(wb, da, li); *d = M_<T>::add(*d, o0[v]); }
              if (a1[v]) { T* d = row_at<T>(wb, db, li); *d = M_<T>::add(*d, o1[v]); }
            }
          }
        }
        // leaves: every contribution from the parents has arrived
        for (int j = 0; j < ncon; ++j) {
          const int k = lcon[j];
#pragma unroll
          for (int v = 0; v < V; ++v) {
            const T g = adj[k * RW + v * 32 + lane];
            if (valid[v] && g != T(0)) vals[k * RW + v * 32 + lane] = M_<T>::add(vals[k * RW + v * 32 + lane], g);
          }
        }
        if (gX) {
          for (int j = 0; j < nvar; ++j) {
            const int k = lvar[j];
            const int var = child0(tape[k]);
#pragma unroll
            for (int v = 0; v < V; ++v) {
              const T g = adj[k * RW + v * 32 + lane];
              if (valid[v] && g != T(0)) atomicAdd(gX + nn[v] * n_x + var, g);
            }
          }
        }
        __syncwarp();  // every lane is done with the seeds before the next chunk's land
      }
      // the constants' sums (lane partials in point order, then a butterfly) replace
      // their values in the broadcast entries
      for (int j = 0; j < ncon; ++j) {
        const int k = lcon[j];
        T part = vals[k * RW + lane];
#pragma unroll
        for (int v = 1; v < V; ++v) part = M_<T>::add(part, vals[k * RW + v * 32 + lane]);
        part = warp_sum(part);
        if (lane == 0) bc[1 + k] = part;
      }
      __syncwarp();
      // gradient row of this set: constant nodes get their sums, everything else 0
      T* gCrow = gC + (size_t)b * M * K + kk;
      for (int64_t k = lane; k < M; k += 32) {
        T val = T(0);
        if (k < L && code_of(tape[k]) == LEARNABLE) val = bc[1 + k];
        gCrow[k * K] = val;
      }
      __syncwarp();
    }  // sets
    err = __reduce_max_sync(0xffffffffu, err);
    if (err && lane == 0) report_adjoint(status, err);
    __syncwarp();
  }
}

// ------------------------------------------------------------------------------------
// Host launchers
// ------------------------------------------------------------------------------------
static int device_sm_count() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 148;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 148;
  return sms;
}

static int max_dyn_smem() {
  int dev = 0, v = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 48 * 1024;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 48 * 1024;
  return v;
}

static int check_tape_args(int64_t B, int64_t M) {
  if (B < 0 || M < 0) { set_error("negative size"); return SR_ERR_INVALID_ARGUMENT; }
  if (M > kMaxNodes) {
    set_error("tapes longer than %d nodes are not supported (M=%lld)", kMaxNodes, (long long)M);
    return SR_ERR_UNSUPPORTED;
  }
  return SR_OK;
}

// Side stream and fork/join events per device, created on first use and kept for the
// life of the process.
struct Aux {
  std::mutex mu;
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
};

static Aux* aux_for_current_device() {
  constexpr int kMaxDevices = 64;
  static Aux aux[kMaxDevices];
  static std::mutex create_mu;
  int dev = 0;
  if (cuda_check(cudaGetDevice(&dev), "cudaGetDevice")) return nullptr;
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("device index %d out of range", dev);
    return nullptr;
  }
  std::lock_guard<std::mutex> hold(create_mu);
  Aux& a = aux[dev];
  if (!a.stream) {
    // created into locals and published together, so a failure leaves nothing behind
    cudaStream_t s = nullptr;
    cudaEvent_t f = nullptr, j = nullptr;
    int rc = cuda_check(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "side stream");
    if (!rc) rc = cuda_check(cudaEventCreateWithFlags(&f, cudaEventDisableTiming), "fork event");
    if (!rc) rc = cuda_check(cudaEventCreateWithFlags(&j, cudaEventDisableTiming), "join event");
    if (rc) {
      if (j) cudaEventDestroy(j);
      if (f) cudaEventDestroy(f);
      if (s) cudaStreamDestroy(s);
      return nullptr;
    }
    a.fork = f;
    a.join = j;
    a.stream = s;
  }
  return &a;
}

template <bool kStage>
static int launch_compile(const int64_t* ops, const int64_t* ch, int64_t B, int64_t M, int64_t ops_sb,
                          int64_t ops_sm, int64_t ch_sb, int64_t ch_sm, int64_t ch_si, int32_t n_vars,
                          uint32_t* desc, int32_t* meta, int32_t* status, void* stream) {
  int rc = check_tape_args(B, M);
  if (rc) return rc;
  if (!status || (B > 0 && M > 0 && (!ops || !ch)) || (kStage && B > 0 && (!meta || (M > 0 && !desc)))) {
    set_error("null pointer argument");
    return SR_ERR_INVALID_ARGUMENT;
  }
  if (n_vars < 0 || n_vars > SR_MAX_VARS) {
    set_error("n_vars out of range (%d)", n_vars);
    return SR_ERR_UNSUPPORTED;
  }
  cudaStream_t st = as_stream(stream);
  rc = cuda_check(cudaMemsetAsync(status, 0, (kStage ? 8 : 1) * sizeof(int32_t), st), "status reset");
  if (rc || B == 0) return rc;
  const int threads = 256;
  int64_t blocks = (B + 7) / 8;
  const int64_t cap = (int64_t)device_sm_count() * 16;
  if (blocks > cap) blocks = cap;
  tape_compile_kernel<kStage><<<(unsigned)blocks, threads, 0, st>>>(ops, ch, B, M, ops_sb, ops_sm, ch_sb, ch_sm,
                                                                    ch_si, n_vars, desc, meta, status);
  return launch_check("tape_compile_kernel");
}

// Persistent grid for an interpreter kernel: warps per CTA and CTAs from the
// per-warp shared memory and the occupancy the kernel reaches.
struct Shape {
  int warps;
  size_t smem;
  int64_t blocks;
};

static bool pick_shape(const void* kern, size_t per_warp, int64_t work_items, Shape& sh) {
  const int limit = max_dyn_smem();
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, limit) != cudaSuccess) return false;
  // the CTA size (8, 4, 2 or 1 warps) that keeps the most warps resident per SM
  int w = 0, per_sm = 0, best = 0;
  for (int cand = 8; cand >= 1; cand >>= 1) {
    if (per_warp * cand > (size_t)limit) continue;
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kern, cand * 32, per_warp * cand) != cudaSuccess)
      continue;
    if (blocks * cand > best) {
      best = blocks * cand;
      w = cand;
      per_sm = blocks;
    }
  }
  if (w == 0) return false;
  sh.warps = w;
  sh.smem = per_warp * w;
  int64_t blocks = (int64_t)device_sm_count() * per_sm;
  const int64_t need = (work_items + w - 1) / w;
  sh.blocks = blocks < need ? blocks : need;
  if (sh.blocks < 1) sh.blocks = 1;
  return true;
}

template <typename T>
static int launch_forward(const T* X, int64_t N, int64_t n_x, const uint32_t* desc, const int32_t* meta,
                          const int32_t* order, int64_t B, int64_t M, int32_t max_len, const T* C, int64_t c_sb,
                          int64_t c_sm, int64_t c_sk, int64_t K, T* cache, void* stream) {
  int rc = check_tape_args(B, M);
  if (rc) return rc;
  if (N < 0 || n_x < 0 || K < 0) { set_error("negative size"); return SR_ERR_INVALID_ARGUMENT; }
  if (B == 0 || M == 0 || N == 0 || K == 0) return SR_OK;
  if (!X && n_x > 0) { set_error("null X"); return SR_ERR_INVALID_ARGUMENT; }
  if (!desc || !meta || !C || !cache) { set_error("null pointer argument"); return SR_ERR_INVALID_ARGUMENT; }
  const int Lmax = (max_len > 0 && max_len < M) ? max_len : (int)M;
  auto kern = K == 1 ? eval_forward_kernel<T, false> : eval_forward_kernel<T, true>;
  const int64_t units = B * ((N + kSlice - 1) / kSlice);
  cudaStream_t st = as_stream(stream);
  Aux* aux = aux_for_current_device();
  if (!aux) return SR_ERR_CUDA;
  std::lock_guard<std::mutex> hold(aux->mu);
  rc = cuda_check(cudaEventRecord(aux->fork, st), "fork event");
  if (!rc) rc = cuda_check(cudaStreamWaitEvent(aux->stream, aux->fork, 0), "fork wait");
  if (rc) return rc;
  // one persistent grid per class of tape lengths, as in launch_backward
  int cls[3][2], nc = 0;
  if (Lmax > 32) { cls[nc][0] = 32; cls[nc][1] = Lmax; ++nc; }
  if (Lmax > 16) { cls[nc][0] = 16; cls[nc][1] = Lmax < 32 ? Lmax : 32; ++nc; }
  cls[nc][0] = -1; cls[nc][1] = Lmax < 16 ? Lmax : 16; ++nc;
  for (int ci = 0; ci < nc && !rc; ++ci) {
    Shape sh;
    if (!pick_shape(reinterpret_cast<const void*>(kern), forward_layout<T>(cls[ci][1]).bytes, units, sh)) {
      set_error("tape of %d nodes does not fit in shared memory", cls[ci][1]);
      rc = SR_ERR_UNSUPPORTED;
      break;
    }
    kern<<<(unsigned)sh.blocks, sh.warps * 32, sh.smem, st>>>(X, N, n_x, desc, meta, order, B, M, cls[ci][0],
                                                             cls[ci][1], C, c_sb, c_sm, c_sk, K, cache);
    rc = launch_check("eval_forward_kernel");
    if (!rc && ci == 0) {
      // enqueued after the first forward grid, whose CTAs are placed first (see
      // launch_backward); eight CTAs per SM: at two the fill streamed too slowly to hide
      // (3.75 against 3.65 ms for the forward of 65536 tapes, N = 1024)
      int64_t fblocks = (int64_t)device_sm_count() * 8;
      if (fblocks > B) fblocks = B;
      pad_fill_kernel<T><<<(unsigned)fblocks, 256, 0, aux->stream>>>(meta, B, M, N * K, Lmax, cache);
      rc = launch_check("pad_fill_kernel");
    }
  }
  const int rj = cuda_check(cudaEventRecord(aux->join, aux->stream), "join event");
  const int rw = rj ? rj : cuda_check(cudaStreamWaitEvent(st, aux->join, 0), "join wait");
  return rc ? rc : rw;
}

template <typename T, bool kMulti, int V, bool kCached>
static int launch_backward_v(const T* X, int64_t N, int64_t n_x, const uint32_t* desc, const int32_t* meta,
                             const int32_t* order, int64_t B, int64_t M, int Llo, int Lhi, const T* C, int64_t c_sb,
                             int64_t c_sm, int64_t c_sk, int64_t K, const T* cache, const T* gout, T* gC, T* gX,
                             int32_t* status, bool vec16, bool cvec16, cudaStream_t st) {
  const size_t per_warp = backward_layout<T, V>(Lhi).bytes;
  Shape sh;
  auto kern = eval_backward_kernel<T, kMulti, V, kCached>;
  if (!pick_shape(reinterpret_cast<const void*>(kern), per_warp, B, sh)) {
    set_error("tape of %d nodes does not fit in shared memory", Lhi);
    return SR_ERR_UNSUPPORTED;
  }
  kern<<<(unsigned)sh.blocks, sh.warps * 32, sh.smem, st>>>(X, N, n_x, desc, meta, order, B, M, Llo, Lhi, C, c_sb,
                                                           c_sm, c_sk, K, cache, gout, gC, gX, status, vec16, cvec16);
  return launch_check("eval_backward_kernel");
}

// One point per lane: two points per lane (one dispatch for both, their chains
// interleaved in registers) ran at half the resident warps, and the adjoint took 1.4x as
// long on a GB300 (10.3 ms against 7.1 ms for 65536 tapes of mean length 20, N = 1024),
// so only the one-point kernels are instantiated.
template <typename T>
static int launch_backward_class(const T* X, int64_t N, int64_t n_x, const uint32_t* desc, const int32_t* meta,
                                 const int32_t* order, int64_t B, int64_t M, int Llo, int Lhi, const T* C,
                                 int64_t c_sb, int64_t c_sm, int64_t c_sk, int64_t K, const T* cache, const T* gout,
                                 T* gC, T* gX, int32_t* status, bool vec16, bool cvec16, cudaStream_t st) {
#define SR_BWD_ARGS X, N, n_x, desc, meta, order, B, M, Llo, Lhi, C, c_sb, c_sm, c_sk, K, cache, gout, gC, gX, status, \
                    vec16, cvec16, st
  if (K == 1)
    return cache ? launch_backward_v<T, false, 1, true>(SR_BWD_ARGS) : launch_backward_v<T, false, 1, false>(SR_BWD_ARGS);
  return cache ? launch_backward_v<T, true, 1, true>(SR_BWD_ARGS) : launch_backward_v<T, true, 1, false>(SR_BWD_ARGS);
#undef SR_BWD_ARGS
}

template <typename T>
static int launch_backward(const T* X, int64_t N, int64_t n_x, const uint32_t* desc, const int32_t* meta,
                           const int32_t* order, int64_t B, int64_t M, int32_t max_len, const T* C, int64_t c_sb,
                           int64_t c_sm, int64_t c_sk, int64_t K, const T* cache, const T* gout, T* gC, T* gX,
                           int32_t* status, void* stream) {
  int rc = check_tape_args(B, M);
  if (rc) return rc;
  if (N < 0 || n_x < 0 || K < 0) { set_error("negative size"); return SR_ERR_INVALID_ARGUMENT; }
  if (!status) { set_error("null status"); return SR_ERR_INVALID_ARGUMENT; }
  cudaStream_t st = as_stream(stream);
  rc = cuda_check(cudaMemsetAsync(status, 0, sizeof(int32_t), st), "status reset");
  if (rc) return rc;
  if (B == 0 || M == 0 || K == 0) return SR_OK;
  if (!desc || !meta || !C || !gC || (N > 0 && !gout)) { set_error("null pointer argument"); return SR_ERR_INVALID_ARGUMENT; }
  if (N == 0) return cuda_check(cudaMemsetAsync(gC, 0, sizeof(T) * B * M * K, st), "grad_C reset");
  const int Lmax = (max_len > 0 && max_len < M) ? max_len : (int)M;
  // the padding check runs on a side stream, forked from and joined back into the
  // caller's stream (a CUDA graph capture records the same fork and join)
  Aux* aux = aux_for_current_device();
  if (!aux) return SR_ERR_CUDA;
  std::lock_guard<std::mutex> hold(aux->mu);
  rc = cuda_check(cudaEventRecord(aux->fork, st), "fork event");
  if (!rc) rc = cuda_check(cudaStreamWaitEvent(aux->stream, aux->fork, 0), "fork wait");
  if (rc) return rc;
  // 16-byte staging needs every (tape, row, chunk) start 16-byte aligned
  const bool vec16 =
      K == 1 && (reinterpret_cast<uintptr_t>(gout) % 16 == 0) && (N % (16 / (int64_t)sizeof(T)) == 0);
  const bool cvec16 =
      K == 1 && (reinterpret_cast<uintptr_t>(cache) % 16 == 0) && (N % (16 / (int64_t)sizeof(T)) == 0);
  // one persistent grid per class of tape lengths (Llo, Lhi]: (48, Lmax], (32, 48],
  // (16, 32], [0, 16], as far as Lmax reaches.  The longest class is bound by the
  // warps its shared memory lets reside (1.5x its tables cost 23% of the adjoint's time
  // on a GB300, the same for the middle class 5%, the shortest nothing): splitting it at
  // 48 gained 2%, further splits at 40, 56 or 24 lost more to the extra grids' tails.
  const int bound[3] = {48, 32, 16};
  int cls[4][2], nc = 0, hi = Lmax;
  for (int j = 0; j < 3; ++j) {
    if (hi > bound[j]) {
      cls[nc][0] = bound[j];
      cls[nc][1] = hi;
      ++nc;
      hi = bound[j];
    }
  }
  cls[nc][0] = -1;
  cls[nc][1] = hi;
  ++nc;
  for (int ci = 0; ci < nc; ++ci) {
    rc = launch_backward_class<T>(X, N, n_x, desc, meta, order, B, M, cls[ci][0], cls[ci][1], C, c_sb, c_sm, c_sk, K,
                                  cache, gout, gC, gX, status, vec16, cvec16, st);
    if (rc) break;
    if (ci == 0) {
      // enqueued after the first adjoint grid, so that grid's CTAs are placed first and
      // the check's CTAs take the registers and warp slots they leave
      int64_t pblocks = (int64_t)device_sm_count() * 2;
      if (pblocks > B) pblocks = B;
      padding_check_kernel<T><<<(unsigned)pblocks, 256, 0, aux->stream>>>(gout, meta, B, M, N * K, Lmax, status);
      rc = launch_check("padding_check_kernel");
      if (rc) break;
    }
  }
  // join (also after a failed launch: the side stream must not outlive the call)
  const int rj = cuda_check(cudaEventRecord(aux->join, aux->stream), "join event");
  const int rw = rj ? rj : cuda_check(cudaStreamWaitEvent(st, aux->join, 0), "join wait");
  return rc ? rc : rw;
}

}  // namespace sr

// ------------------------------------------------------------------------------------
// C ABI
// ------------------------------------------------------------------------------------
extern "C" {

const char* sr_last_error(void) { return sr::g_err; }

const char* sr_version(void) { return "sr_gb300 0.1 (sm_103a)"; }

int sr_validate(const int64_t* ops, const int64_t* ch, int64_t B, int64_t M, int64_t ops_sb, int64_t ops_sm,
                int64_t ch_sb, int64_t ch_sm, int64_t ch_si, int32_t* status, void* stream) {
  return sr::launch_compile<false>(ops, ch, B, M, ops_sb, ops_sm, ch_sb, ch_sm, ch_si, 0, nullptr, nullptr, status,
                                   stream);
}

int sr_tape_compile(const int64_t* ops, const int64_t* ch, int64_t B, int64_t M, int64_t ops_sb, int64_t ops_sm,
                    int64_t ch_sb, int64_t ch_sm, int64_t ch_si, int32_t n_vars, uint32_t* desc, int32_t* meta,
                    int32_t* stats, void* stream) {
  return sr::launch_compile<true>(ops, ch, B, M, ops_sb, ops_sm, ch_sb, ch_sm, ch_si, n_vars, desc, meta, stats,
                                  stream);
}

int sr_eval_forward_f32(const float* X, int64_t N, int64_t n_x, const uint32_t* desc, const int32_t* meta,
                        const int32_t* order, int64_t B, int64_t M, int32_t max_len, const float* C, int64_t c_sb,
                        int64_t c_sm, float* cache, void* stream) {
  return sr::launch_forward<float>(X, N, n_x, desc, meta, order, B, M, max_len, C, c_sb, c_sm, 0, 1, cache, stream);
}

int sr_eval_forward_f64(const double* X, int64_t N, int64_t n_x, const uint32_t* desc, const int32_t* meta,
                        const int32_t* order, int64_t B, int64_t M, int32_t max_len, const double* C, int64_t c_sb,
                        int64_t c_sm, double* cache, void* stream) {
  return sr::launch_forward<double>(X, N, n_x, desc, meta, order, B, M, max_len, C, c_sb, c_sm, 0, 1, cache, stream);
}

int sr_eval_backward_f32(const float* X, int64_t N, int64_t n_x, const uint32_t* desc, const int32_t* meta,
                         const int32_t* order, int64_t B, int64_t M, int32_t max_len, const float* C, int64_t c_sb,
                         int64_t c_sm, const float* cache, const float* gout, float* gC, float* gX, int32_t* status,
                         void* stream) {
  return sr::launch_backward<float>(X, N, n_x, desc, meta, order, B, M, max_len, C, c_sb, c_sm, 0, 1, cache, gout, gC,
                                    gX, status, stream);
}

int sr_eval_backward_f64(const double* X, int64_t N, int64_t n_x, const uint32_t* desc, const int32_t* meta,
                         const int32_t* order, int64_t B, int64_t M, int32_t max_len, const double* C, int64_t c_sb,
                         int64_t c_sm, const double* cache, const double* gout, double* gC, double* gX,
                         int32_t* status, void* stream) {
  return sr::launch_backward<double>(X, N, n_x, desc, meta, order, B, M, max_len, C, c_sb, c_sm, 0, 1, cache, gout, gC,
                                     gX, status, stream);
}

int sr_eval_forward_multi_f32(const float* X, int64_t N, int64_t n_x, const uint32_t* desc, const int32_t* meta,
                              const int32_t* order, int64_t B, int64_t M, int32_t max_len, const float* C,
                              int64_t c_sb, int64_t c_sm, int64_t c_sk, int64_t K, float* cache, void* stream) {
  return sr::launch_forward<float>(X, N, n_x, desc, meta, order, B, M, max_len, C, c_sb, c_sm, c_sk, K, cache, stream);
}

int sr_eval_forward_multi_f64(const double* X, int64_t N, int64_t n_x, const uint32_t* desc, const int32_t* meta,
                              const int32_t* order, int64_t B, int64_t M, int32_t max_len, const double* C,
                              int64_t c_sb, int64_t c_sm, int64_t c_sk, int64_t K, double* cache, void* stream) {
  return sr::launch_forward<double>(X, N, n_x, desc, meta, order, B, M, max_len, C, c_sb, c_sm, c_sk, K, cache,
                                    stream);
}

int sr_eval_backward_multi_f32(const float* X, int64_t N, int64_t n_x, const uint32_t* desc, const int32_t* meta,
                               const int32_t* order, int64_t B, int64_t M, int32_t max_len, const float* C,
                               int64_t c_sb, int64_t c_sm, int64_t c_sk, int64_t K, const float* cache,
                               const float* gout, float* gC, float* gX, int32_t* status, void* stream) {
  return sr::launch_backward<float>(X, N, n_x, desc, meta, order, B, M, max_len, C, c_sb, c_sm, c_sk, K, cache, gout,
                                    gC, gX, status, stream);
}

int sr_eval_backward_multi_f64(const double* X, int64_t N, int64_t n_x, const uint32_t* desc, const int32_t* meta,
                               const int32_t* order, int64_t B, int64_t M, int32_t max_len, const double* C,
                               int64_t c_sb, int64_t c_sm, int64_t c_sk, int64_t K, const double* cache,
                               const double* gout, double* gC, double* gX, int32_t* status, void* stream) {
  return sr::launch_backward<double>(X, N, n_x, desc, meta, order, B, M, max_len, C, c_sb, c_sm, c_sk, K, cache, gout,
                                     gC, gX, status, stream);
}

}  // extern "C"
