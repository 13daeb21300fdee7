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
      int kroot = 0, kall = 0;
      for (int64_t m0 = 0; m0 < M; m0 += 32) {
        const int64_t m = m0 + lane;
        const bool lc = m < M && ops[b * ops_sb + m * ops_sm] == LEARNABLE;
        kall += __popc(__ballot_sync(0xffffffffu, lc));
        kroot += __popc(__ballot_sync(0xffffffffu, lc && m <= root));
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
      }
    }
  }
}

// ------------------------------------------------------------------------------------
// Forward.  V points per lane per pass (point = base + v*32 + lane).
// Shared memory per warp: M tape words + L_max * 32V node values.
// ------------------------------------------------------------------------------------
template <typename T, int V>
__device__ __forceinline__ void forward_pass(const uint32_t* __restrict__ tape, int L, T* __restrict__ vals,
                                             const T* __restrict__ X, int64_t n_x, const int64_t* nn,
                                             const T* __restrict__ Crow, int64_t c_sm, int lane) {
  for (int k = 0; k < L; ++k) {
    const uint32_t d = tape[k];
    const int code = code_of(d);
    T* out = vals + (size_t)k * (32 * V);
    if (code == VAR) {
      const int var = child0(d);
#pragma unroll
      for (int v = 0; v < V; ++v) out[v * 32 + lane] = __ldg(X + nn[v] * n_x + var);
    } else if (code == LEARNABLE) {
      const T c = __ldg(Crow + (int64_t)k * c_sm);
#pragma unroll
      for (int v = 0; v < V; ++v) out[v * 32 + lane] = c;
    } else {
      const T* A = vals + (size_t)child0(d) * (32 * V);
      const T* Bv = vals + (size_t)child1(d) * (32 * V);
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const T a = A[v * 32 + lane];
        const T b = Bv[v * 32 + lane];
        out[v * 32 + lane] = node_value<T>(code, a, b, T(0), T(0));
      }
    }
  }
}

// Fill count values at p with NaN, 16-byte vector stores in the aligned middle.
template <typename T>
__device__ __forceinline__ void warp_fill_nan(T* p, size_t count, int lane) {
  const T qnan = M_<T>::nan();
  constexpr int kVec = 16 / sizeof(T);
  size_t head = (size_t)((16 - (reinterpret_cast<uintptr_t>(p) & 15)) & 15) / sizeof(T);
  if (reinterpret_cast<uintptr_t>(p) % sizeof(T)) head = count;  // unaligned element type: scalar path
  if (head > count) head = count;
  for (size_t i = lane; i < head; i += 32) __stcs(p + i, qnan);
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
  for (size_t i = lane; i < nvec; i += 32) __stcs(q + i, v4);
  for (size_t i = head + nvec * kVec + lane; i < count; i += 32) __stcs(p + i, qnan);
}

template <typename T, int V>
__global__ void __launch_bounds__(256) eval_forward_kernel(const T* __restrict__ X, int64_t N, int64_t n_x,
                                                           const uint32_t* __restrict__ desc,
                                                           const int32_t* __restrict__ meta, int64_t B,
                                                           int64_t M, int Lmax, const T* __restrict__ C,
                                                           int64_t c_sb, int64_t c_sm, T* __restrict__ cache) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  const size_t tbytes = align16((size_t)Lmax * 4);
  const size_t per_warp = tbytes + (size_t)Lmax * 32 * V * sizeof(T);
  uint32_t* tape = reinterpret_cast<uint32_t*>(smem + warp * per_warp);
  T* vals = reinterpret_cast<T*>(smem + warp * per_warp + tbytes);
  for (int64_t b = (int64_t)blockIdx.x * nwarp + warp; b < B; b += (int64_t)gridDim.x * nwarp) {
    const int L = meta[b * 4];
    for (int k = lane; k < L; k += 32) tape[k] = desc[b * M + k];
    __syncwarp();
    const T* Crow = C + b * c_sb;
    T* out = cache + (size_t)b * M * N;
    for (int64_t base = 0; base < N; base += 32 * V) {
      int64_t nn[V];
      bool valid[V];
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const int64_t n = base + v * 32 + lane;
        valid[v] = n < N;
        nn[v] = valid[v] ? n : N - 1;
      }
      // each node's values go to the cache as soon as they exist (streaming stores,
      // 128 contiguous bytes per warp and v), interleaving compute with HBM writes
      for (int k = 0; k < L; ++k) {
        const uint32_t d = tape[k];
        const int code = code_of(d);
        T* o = vals + (size_t)k * (32 * V);
        T r[V];
        if (code == VAR) {
          const int var = child0(d);
#pragma unroll
          for (int v = 0; v < V; ++v) r[v] = __ldg(X + nn[v] * n_x + var);
        } else if (code == LEARNABLE) {
          const T c = __ldg(Crow + (int64_t)k * c_sm);
#pragma unroll
          for (int v = 0; v < V; ++v) r[v] = c;
        } else {
          const T* A = vals + (size_t)child0(d) * (32 * V);
          const T* Bv = vals + (size_t)child1(d) * (32 * V);
#pragma unroll
          for (int v = 0; v < V; ++v) r[v] = node_value<T>(code, A[v * 32 + lane], Bv[v * 32 + lane], T(0), T(0));
        }
#pragma unroll
        for (int v = 0; v < V; ++v) {
          o[v * 32 + lane] = r[v];
          if (valid[v]) __stcs(out + (size_t)k * N + nn[v], r[v]);
        }
      }
    }
    // rows after the last real node are one contiguous block of (M - L) * N values
    warp_fill_nan(out + (size_t)L * N, (size_t)(M - L) * N, lane);
    __syncwarp();
  }
}

// ------------------------------------------------------------------------------------
// Adjoint for a dense grad_out.  Per warp shared memory: tape, node values,
// node adjoints (L_max * 32V each) and the per-node constant gradient sums.
// ------------------------------------------------------------------------------------
// True in every lane when one of count values at p is nonzero (NaN counts as nonzero).
template <typename T>
__device__ __forceinline__ bool warp_any_nonzero(const T* p, size_t count, int lane) {
  bool nz = false;
  constexpr int kVec = 16 / sizeof(T);
  size_t head = (size_t)((16 - (reinterpret_cast<uintptr_t>(p) & 15)) & 15) / sizeof(T);
  if (reinterpret_cast<uintptr_t>(p) % sizeof(T)) head = count;
  if (head > count) head = count;
  for (size_t i = lane; i < head; i += 32) nz |= __ldcs(p + i) != T(0);
  const size_t nvec = (count - head) / kVec;
  const float4* q = reinterpret_cast<const float4*>(p + head);
  for (size_t i = lane; i < nvec; i += 32) {
    const float4 v = __ldcs(q + i);
    if (sizeof(T) == 4) {
      nz |= (v.x != 0.f) | (v.y != 0.f) | (v.z != 0.f) | (v.w != 0.f);
    } else {
      const double* d = reinterpret_cast<const double*>(&v);
      nz |= (d[0] != 0.0) | (d[1] != 0.0);
    }
  }
  for (size_t i = head + nvec * kVec + lane; i < count; i += 32) nz |= __ldcs(p + i) != T(0);
  return __any_sync(0xffffffffu, nz);
}

template <typename T, int V>
__global__ void __launch_bounds__(256) eval_backward_kernel(
    const T* __restrict__ X, int64_t N, int64_t n_x, const uint32_t* __restrict__ desc,
    const int32_t* __restrict__ meta, int64_t B, int64_t M, int Lmax, const T* __restrict__ C, int64_t c_sb,
    int64_t c_sm, const T* __restrict__ gout, T* __restrict__ gC, T* __restrict__ gX,
    int32_t* __restrict__ status) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  const size_t tbytes = align16((size_t)Lmax * 4);
  const size_t vbytes = (size_t)Lmax * 32 * V * sizeof(T);
  const size_t per_warp = tbytes + 2 * vbytes + align16((size_t)Lmax * sizeof(T));
  unsigned char* base_ptr = smem + warp * per_warp;
  uint32_t* tape = reinterpret_cast<uint32_t*>(base_ptr);
  T* vals = reinterpret_cast<T*>(base_ptr + tbytes);
  T* adj = reinterpret_cast<T*>(base_ptr + tbytes + vbytes);
  T* gsum = reinterpret_cast<T*>(base_ptr + tbytes + 2 * vbytes);
  for (int64_t b = (int64_t)blockIdx.x * nwarp + warp; b < B; b += (int64_t)gridDim.x * nwarp) {
    const int L = meta[b * 4];
    for (int k = lane; k < L; k += 32) {
      tape[k] = desc[b * M + k];
      gsum[k] = T(0);
    }
    __syncwarp();
    const T* Crow = C + b * c_sb;
    const T* G = gout + (size_t)b * M * N;
    int err = 0;
    for (int64_t base = 0; base < N; base += 32 * V) {
      int64_t nn[V];
      bool valid[V];
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const int64_t n = base + v * 32 + lane;
        valid[v] = n < N;
        nn[v] = valid[v] ? n : N - 1;
      }
      forward_pass<T, V>(tape, L, vals, X, n_x, nn, Crow, c_sm, lane);
      // adjoint seeds: 0 + grad_out, as the reference's zeros_like(cache).add_(grad_output)
      for (int k = 0; k < L; ++k) {
#pragma unroll
        for (int v = 0; v < V; ++v)
          adj[(size_t)k * 32 * V + v * 32 + lane] = valid[v] ? M_<T>::add(T(0), __ldcs(G + (size_t)k * N + nn[v])) : T(0);
      }
      __syncwarp();
      for (int k = L - 1; k >= 0; --k) {
        const uint32_t d = tape[k];
        const int code = code_of(d);
        const T* gk = adj + (size_t)k * 32 * V;
        if (code == LEARNABLE) {
          T part = T(0);
#pragma unroll
          for (int v = 0; v < V; ++v) {
            const T g = gk[v * 32 + lane];
            if (valid[v] && g != T(0)) part = M_<T>::add(part, g);
          }
          part = warp_sum(part);
          if (lane == 0) gsum[k] = M_<T>::add(gsum[k], part);
          continue;
        }
        if (code == VAR) {
          if (gX) {
            const int var = child0(d);
#pragma unroll
            for (int v = 0; v < V; ++v) {
              const T g = gk[v * 32 + lane];
              if (valid[v] && g != T(0)) atomicAdd(gX + nn[v] * n_x + var, g);
            }
          }
          continue;
        }
        const int c0 = child0(d), c1 = child1(d);
        T* A = adj + (size_t)c0 * 32 * V;
        T* Bb = adj + (size_t)c1 * 32 * V;
        const T* av = vals + (size_t)c0 * 32 * V;
        const T* bv = vals + (size_t)c1 * 32 * V;
        const T* kv = vals + (size_t)k * 32 * V;
#pragma unroll
        for (int v = 0; v < V; ++v) {
          const int i = v * 32 + lane;
          bool a0, a1;
          T o0, o1;
          const int e = node_adjoint<T>(code, gk[i], av[i], bv[i], kv[i], a0, o0, a1, o1);
          if (valid[v]) {
            if (e && !err) err = e;
            if (a0) A[i] = M_<T>::add(A[i], o0);
            if (a1) Bb[i] = M_<T>::add(Bb[i], o1);
          }
        }
      }
      __syncwarp();
    }
    // rows after the last real node are NO_OP nodes: any nonzero gradient there is error 201
    if (warp_any_nonzero(G + (size_t)L * N, (size_t)(M - L) * N, lane)) err = ERR_GRAD_ON_NO_OP;
    if (err) report(status, err);
    // gradient row: constant nodes get their sums, everything else 0
    T* gCrow = gC + (size_t)b * M;
    for (int64_t k = lane; k < M; k += 32) {
      T val = T(0);
      if (k < L && code_of(tape[k]) == LEARNABLE) val = gsum[k];
      gCrow[k] = val;
    }
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
  rc = cuda_check(cudaMemsetAsync(status, 0, (kStage ? 4 : 1) * sizeof(int32_t), st), "status reset");
  if (rc || B == 0) return rc;
  const int threads = 256;
  int64_t blocks = (B + 7) / 8;
  const int64_t cap = (int64_t)device_sm_count() * 16;
  if (blocks > cap) blocks = cap;
  tape_compile_kernel<kStage><<<(unsigned)blocks, threads, 0, st>>>(ops, ch, B, M, ops_sb, ops_sm, ch_sb, ch_sm,
                                                                    ch_si, n_vars, desc, meta, status);
  return launch_check("tape_compile_kernel");
}

// Warps per CTA and points per lane for the interpreter kernels, given the
// per-warp shared memory they need.
template <typename T>
static bool pick_shape(int Lmax, size_t per_point_bytes, bool with_sums, int& V, int& warps, size_t& smem) {
  const int limit = max_dyn_smem();
  const size_t fixed = align16((size_t)Lmax * 4) + (with_sums ? align16((size_t)Lmax * sizeof(T)) : 0);
  // one point per lane keeps the per-warp table small, so more warps fit on an SM
  for (int v : {1}) {
    const size_t per_warp = fixed + (size_t)Lmax * 32 * v * per_point_bytes;
    for (int w : {8, 4, 2, 1}) {
      if (per_warp * w <= (size_t)limit && per_warp * w <= 72 * 1024) {
        V = v;
        warps = w;
        smem = per_warp * w;
        return true;
      }
    }
  }
  const size_t per_warp = fixed + (size_t)Lmax * 32 * per_point_bytes;
  if (per_warp <= (size_t)limit) {
    V = 1;
    warps = 1;
    smem = per_warp;
    return true;
  }
  return false;
}

template <typename T, int V>
static int launch_forward_v(const T* X, int64_t N, int64_t n_x, const uint32_t* desc, const int32_t* meta,
                            int64_t B, int64_t M, int Lmax, const T* C, int64_t c_sb, int64_t c_sm, T* cache,
                            int warps, size_t smem, cudaStream_t st) {
  auto kern = eval_forward_kernel<T, V>;
  int rc = cuda_check(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                      "forward smem attribute");
  if (rc) return rc;
  int64_t blocks = (B + warps - 1) / warps;
  const int64_t cap = (int64_t)device_sm_count() * 64;
  if (blocks > cap) blocks = cap;
  kern<<<(unsigned)blocks, warps * 32, smem, st>>>(X, N, n_x, desc, meta, B, M, Lmax, C, c_sb, c_sm, cache);
  return launch_check("eval_forward_kernel");
}

template <typename T>
static int launch_forward(const T* X, int64_t N, int64_t n_x, const uint32_t* desc, const int32_t* meta,
                          int64_t B, int64_t M, int32_t max_len, const T* C, int64_t c_sb, int64_t c_sm, T* cache,
                          void* stream) {
  int rc = check_tape_args(B, M);
  if (rc) return rc;
  if (N < 0 || n_x < 0) { set_error("negative size"); return SR_ERR_INVALID_ARGUMENT; }
  if (B == 0 || M == 0 || N == 0) return SR_OK;
  if (!X && n_x > 0) { set_error("null X"); return SR_ERR_INVALID_ARGUMENT; }
  if (!desc || !meta || !C || !cache) { set_error("null pointer argument"); return SR_ERR_INVALID_ARGUMENT; }
  const int Lmax = (max_len > 0 && max_len < M) ? max_len : (int)M;
  int V = 1, warps = 1;
  size_t smem = 0;
  if (!pick_shape<T>(Lmax, sizeof(T), false, V, warps, smem)) {
    set_error("tape of %lld nodes does not fit in shared memory", (long long)M);
    return SR_ERR_UNSUPPORTED;
  }
  cudaStream_t st = as_stream(stream);
  switch (V) {
    case 4: return launch_forward_v<T, 4>(X, N, n_x, desc, meta, B, M, Lmax, C, c_sb, c_sm, cache, warps, smem, st);
    case 2: return launch_forward_v<T, 2>(X, N, n_x, desc, meta, B, M, Lmax, C, c_sb, c_sm, cache, warps, smem, st);
    default: return launch_forward_v<T, 1>(X, N, n_x, desc, meta, B, M, Lmax, C, c_sb, c_sm, cache, warps, smem, st);
  }
}

template <typename T, int V>
static int launch_backward_v(const T* X, int64_t N, int64_t n_x, const uint32_t* desc, const int32_t* meta,
                             int64_t B, int64_t M, int Lmax, const T* C, int64_t c_sb, int64_t c_sm,
                             const T* gout, T* gC, T* gX, int32_t* status, int warps, size_t smem,
                             cudaStream_t st) {
  auto kern = eval_backward_kernel<T, V>;
  int rc = cuda_check(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                      "backward smem attribute");
  if (rc) return rc;
  int64_t blocks = (B + warps - 1) / warps;
  const int64_t cap = (int64_t)device_sm_count() * 64;
  if (blocks > cap) blocks = cap;
  kern<<<(unsigned)blocks, warps * 32, smem, st>>>(X, N, n_x, desc, meta, B, M, Lmax, C, c_sb, c_sm, gout, gC, gX,
                                                     status);
  return launch_check("eval_backward_kernel");
}

template <typename T>
static int launch_backward(const T* X, int64_t N, int64_t n_x, const uint32_t* desc, const int32_t* meta,
                           int64_t B, int64_t M, int32_t max_len, const T* C, int64_t c_sb, int64_t c_sm,
                           const T* gout, T* gC, T* gX, int32_t* status, void* stream) {
  int rc = check_tape_args(B, M);
  if (rc) return rc;
  if (N < 0 || n_x < 0) { set_error("negative size"); return SR_ERR_INVALID_ARGUMENT; }
  if (!status) { set_error("null status"); return SR_ERR_INVALID_ARGUMENT; }
  cudaStream_t st = as_stream(stream);
  rc = cuda_check(cudaMemsetAsync(status, 0, sizeof(int32_t), st), "status reset");
  if (rc) return rc;
  if (B == 0 || M == 0) return SR_OK;
  if (!desc || !meta || !C || !gC || (N > 0 && !gout)) { set_error("null pointer argument"); return SR_ERR_INVALID_ARGUMENT; }
  if (N == 0) return cuda_check(cudaMemsetAsync(gC, 0, sizeof(T) * B * M, st), "grad_C reset");
  const int Lmax = (max_len > 0 && max_len < M) ? max_len : (int)M;
  int V = 1, warps = 1;
  size_t smem = 0;
  if (!pick_shape<T>(Lmax, 2 * sizeof(T), true, V, warps, smem)) {
    set_error("tape of %lld nodes does not fit in shared memory", (long long)M);
    return SR_ERR_UNSUPPORTED;
  }
  switch (V) {
    case 4: return launch_backward_v<T, 4>(X, N, n_x, desc, meta, B, M, Lmax, C, c_sb, c_sm, gout, gC, gX, status, warps, smem, st);
    case 2: return launch_backward_v<T, 2>(X, N, n_x, desc, meta, B, M, Lmax, C, c_sb, c_sm, gout, gC, gX, status, warps, smem, st);
    default: return launch_backward_v<T, 1>(X, N, n_x, desc, meta, B, M, Lmax, C, c_sb, c_sm, gout, gC, gX, status, warps, smem, st);
  }
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

int sr_eval_forward_f32(const float* X, int64_t N, int64_t n_x, const uint32_t* desc, const int32_t* meta, int64_t B,
                        int64_t M, int32_t max_len, const float* C, int64_t c_sb, int64_t c_sm, float* cache,
                        void* stream) {
  return sr::launch_forward<float>(X, N, n_x, desc, meta, B, M, max_len, C, c_sb, c_sm, cache, stream);
}

int sr_eval_forward_f64(const double* X, int64_t N, int64_t n_x, const uint32_t* desc, const int32_t* meta,
                        int64_t B, int64_t M, int32_t max_len, const double* C, int64_t c_sb, int64_t c_sm,
                        double* cache, void* stream) {
  return sr::launch_forward<double>(X, N, n_x, desc, meta, B, M, max_len, C, c_sb, c_sm, cache, stream);
}

int sr_eval_backward_f32(const float* X, int64_t N, int64_t n_x, const uint32_t* desc, const int32_t* meta,
                         int64_t B, int64_t M, int32_t max_len, const float* C, int64_t c_sb, int64_t c_sm,
                         const float* gout, float* gC, float* gX, int32_t* status, void* stream) {
  return sr::launch_backward<float>(X, N, n_x, desc, meta, B, M, max_len, C, c_sb, c_sm, gout, gC, gX, status,
                                    stream);
}

int sr_eval_backward_f64(const double* X, int64_t N, int64_t n_x, const uint32_t* desc, const int32_t* meta,
                         int64_t B, int64_t M, int32_t max_len, const double* C, int64_t c_sb, int64_t c_sm,
                         const double* gout, double* gC, double* gX, int32_t* status, void* stream) {
  return sr::launch_backward<double>(X, N, n_x, desc, meta, B, M, max_len, C, c_sb, c_sm, gout, gC, gX, status,
                                     stream);
}

}  // extern "C"
