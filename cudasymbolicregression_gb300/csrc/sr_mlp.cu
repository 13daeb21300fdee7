// sr_mlp.cu -- kernels of the warm-start network: a small BF16 MLP that predicts
// starting constants for the fit from a tape and a summary of its target.
//
// The GEMMs run on the 5th-generation tensor cores: a CTA of 4 warps owns a
// 128-row tile of D = A . W^T.  Warp 0 (one lane) streams 64-wide K slices of A and
// W into a 4-stage shared-memory ring with TMA (128-byte swizzle), warp 1 (one
// lane) issues tcgen05.mma (M=128, N=64..256, K=16, bf16 x bf16 -> fp32) into a
// TMEM accumulator and releases each stage with tcgen05.commit, and then all four
// warps read their 32 TMEM lanes (one row each) with tcgen05.ld and apply the
// layer's epilogue (bias, ReLU or ReLU' gate, bf16 rounding, a row-major and a
// transposed copy, or fp32 partial sums of a split reduction).  Every wait on an
// mbarrier gives up after about a second, records SR_MLP_TIMEOUT in the status
// word and lets the CTA finish (TMEM is always released).
//
// Around the GEMMs: the input features (bag of tokens, moments of Y, projections of
// Y on random features of X), the loss and its gradient, bias gradients, the split
// reduction, and an Adam step that also refreshes the bf16 weight copies.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <cmath>
#include <mutex>

#include "sr_common.cuh"

namespace sr {
namespace mlp {

constexpr int kTileM = 128;  // rows of D per CTA = TMEM lanes
constexpr int kTileK = 64;   // bf16 elements per 128-byte swizzled smem row
constexpr int kStages = 4;
constexpr int kThreads = 128;
constexpr long long kWaitCycles = 2000000000LL;  // about one second at 2 GHz

struct Epi {
  int mode;
  const float* bias;
  const __nv_bfloat16* gate;
  long long ld_gate;
  __nv_bfloat16* out;
  long long ld_out, out_col0;
  __nv_bfloat16* out_t;
  long long ld_out_t, out_t_row0;
  float* out_f32;
  long long ld_out_f32, split_stride;
};

struct GemmParams {
  int rows;              // valid rows of D
  int k_chunks;          // 64-wide slices of the reduction
  int chunks_per_split;  // slices per blockIdx.y
  Epi e;
  int* status;
};

// ---- PTX wrappers ------------------------------------------------------------------

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}

// Waits until the phase of the given parity has completed; false after about a second.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  if (mbar_test(bar, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_test(bar, parity)) {
    if (clock64() - t0 > kWaitCycles) return false;
  }
  return true;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, uint32_t bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
          dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(x), "r"(y)
      : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor of a K-major tile stored as 128-byte rows with the
// 128-byte swizzle (what TMA writes with CU_TENSOR_MAP_SWIZZLE_128B): 8-row groups
// 1024 bytes apart, fixed field 0b001 at bit 46, swizzle mode 2 at bits 61-63.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// Instruction descriptor of kind::f16: fp32 accumulator (bits 4-5 = 1), bf16 A and
// B (bits 7-9 and 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 32 consecutive fp32 columns of this thread's TMEM lane; the wait is part of the
// same statement, so no use of the registers can be scheduled before it.
__device__ __forceinline__ void tmem_load32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// ---- epilogue ---------------------------------------------------------------------

__device__ __forceinline__ void store_bf16_row(__nv_bfloat16* dst, const float (&h)[32]) {
  uint4* d = reinterpret_cast<uint4*>(dst);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    uint32_t w[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const __nv_bfloat162 pr = __floats2bfloat162_rn(h[q * 8 + 2 * t], h[q * 8 + 2 * t + 1]);
      w[t] = *reinterpret_cast<const uint32_t*>(&pr);
    }
    d[q] = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

__device__ __forceinline__ void epilogue(const GemmParams& p, int r, int col0, int split, float (&v)[32]) {
  const Epi& e = p.e;
  if (r >= p.rows) return;
  if (e.mode == SR_MLP_EPI_F32 || e.mode == SR_MLP_EPI_SPLIT_F32) {
    float* o = e.out_f32 + (e.mode == SR_MLP_EPI_SPLIT_F32 ? (long long)split * e.split_stride : 0LL) +
               (long long)r * e.ld_out_f32 + col0;
    if (e.bias) {
#pragma unroll
      for (int j = 0; j < 32; ++j) v[j] += e.bias[col0 + j];
    }
    float4* o4 = reinterpret_cast<float4*>(o);
#pragma unroll
    for (int q = 0; q < 8; ++q) o4[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
    return;
  }
  float h[32];
  if (e.mode == SR_MLP_EPI_RELU_GRAD) {
    const uint4* g4 = reinterpret_cast<const uint4*>(e.gate + (long long)r * e.ld_gate + col0);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint4 w = g4[q];
      const uint32_t ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const __nv_bfloat162 pr = *reinterpret_cast<const __nv_bfloat162*>(&ws[t]);
        h[q * 8 + 2 * t] = __bfloat162float(pr.x) > 0.f ? v[q * 8 + 2 * t] : 0.f;
        h[q * 8 + 2 * t + 1] = __bfloat162float(pr.y) > 0.f ? v[q * 8 + 2 * t + 1] : 0.f;
      }
    }
  } else {
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      const float z = v[j] + (e.bias ? e.bias[col0 + j] : 0.f);
      h[j] = (e.mode == SR_MLP_EPI_RELU) ? fmaxf(z, 0.f) : z;
    }
  }
  if (e.out) store_bf16_row(e.out + (long long)r * e.ld_out + e.out_col0 + col0, h);
  if (e.out_t) {
    __nv_bfloat16* t = e.out_t + (e.out_t_row0 + col0) * e.ld_out_t + r;
#pragma unroll
    for (int j = 0; j < 32; ++j) t[(long long)j * e.ld_out_t] = __float2bfloat16_rn(h[j]);
  }
}

// ---- the GEMM ---------------------------------------------------------------------

template <int BN>
__global__ void __launch_bounds__(kThreads, 1)
    gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, GemmParams p) {
  extern __shared__ unsigned char smem_raw[];
  constexpr uint32_t kABytes = kTileM * kTileK * 2;
  constexpr uint32_t kBBytes = BN * kTileK * 2;
  constexpr uint32_t kStageBytes = kABytes + kBBytes;
  constexpr uint32_t kCols = BN;  // 64, 128 or 256 TMEM columns (fp32 accumulator)
  const uint32_t raw = smem_addr(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  const uint32_t bar_full = base + kStages * kStageBytes;
  const uint32_t bar_empty = bar_full + 8 * kStages;
  const uint32_t bar_acc = bar_empty + 8 * kStages;
  const uint32_t tmem_slot = bar_acc + 8;
  const volatile uint32_t* tmem_slot_ptr =
      reinterpret_cast<const volatile uint32_t*>(smem_raw + (tmem_slot - raw));

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int split = blockIdx.y;
  const int c0 = split * p.chunks_per_split;
  const int c1 = min(p.k_chunks, c0 + p.chunks_per_split);
  const int nk = max(0, c1 - c0);
  const int row0 = blockIdx.x * kTileM;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(bar_full + 8 * s, 1);
      mbar_init(bar_empty + 8 * s, 1);
    }
    mbar_init(bar_acc, 1);
    mbar_fence_init();
  }
  if (warp == 1) tmem_alloc(tmem_slot, kCols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot_ptr;

  bool fail = false;
  int issued = 0;
  if (nk > 0 && warp == 0 && lane == 0) {
    // TMA producer: stage s is reused once the MMAs that read it have completed
    for (int i = 0; i < nk; ++i) {
      const int s = i % kStages;
      if (i >= kStages && !mbar_wait(bar_empty + 8 * s, ((i / kStages) - 1) & 1)) {
        fail = true;
        break;
      }
      const uint32_t a = base + s * kStageBytes;
      mbar_arrive_expect_tx(bar_full + 8 * s, kStageBytes);
      tma_load_2d(a, &tmA, bar_full + 8 * s, (c0 + i) * kTileK, row0);
      tma_load_2d(a + kABytes, &tmB, bar_full + 8 * s, (c0 + i) * kTileK, 0);
      ++issued;
    }
  } else if (nk > 0 && warp == 1 && lane == 0) {
    // MMA issuer: 4 MMAs of K=16 per 64-wide slice, 32 bytes apart in the swizzled rows
    constexpr uint32_t idesc = idesc_bf16(kTileM, BN);
    for (int i = 0; i < nk; ++i) {
      const int s = i % kStages;
      if (!mbar_wait(bar_full + 8 * s, (i / kStages) & 1)) {
        fail = true;
        break;
      }
      tc_fence_after();
      const uint32_t a = base + s * kStageBytes;
      const uint64_t ad = sw128_desc(a), bd = sw128_desc(a + kABytes);
#pragma unroll
      for (int kk = 0; kk < kTileK / 16; ++kk)
        mma_bf16(tmem, ad + 2 * kk, bd + 2 * kk, idesc, (i > 0 || kk > 0) ? 1u : 0u);
      mma_commit(bar_empty + 8 * s);
    }
    mma_commit(bar_acc);
  }
  __syncwarp();

  // epilogue: warp w reads TMEM lanes 32w..32w+31 (= rows of the tile)
  bool ok = nk > 0 && mbar_wait(bar_acc, 0);
  ok = __all_sync(0xffffffffu, ok);
  tc_fence_after();
  const int r = row0 + warp * 32 + lane;
  const uint32_t t_row = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
  for (int cc = 0; cc < BN / 32; ++cc) {
    float v[32];
    if (ok) {
      tmem_load32(t_row + cc * 32, v);
    } else {
#pragma unroll
      for (int j = 0; j < 32; ++j) v[j] = 0.f;
    }
    epilogue(p, r, cc * 32, split, v);
  }
  if (nk > 0 && !ok && threadIdx.x == 0) fail = true;

  // the producer makes sure none of its copies is still in flight before the CTA ends
  if (warp == 0 && lane == 0) {
    for (int i = max(0, issued - kStages); i < issued; ++i)
      if (!mbar_wait(bar_full + 8 * (i % kStages), (i / kStages) & 1)) fail = true;
  }
  if (fail) report(p.status, SR_MLP_TIMEOUT);
  tc_fence_before();
  __syncthreads();
  if (warp == 1) tmem_dealloc(tmem, kCols);
}

// ---- features ----------------------------------------------------------------------

// phi[n][j] = sqrt(2) cos(omega_j . x_n + beta_j)
__global__ void random_features_kernel(const float* __restrict__ X, int64_t N, int64_t n_x,
                                       const float* __restrict__ omega, const float* __restrict__ beta,
                                       float* __restrict__ phi) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N * SR_MLP_PROJ) return;
  const int64_t n = i / SR_MLP_PROJ;
  const int j = (int)(i % SR_MLP_PROJ);
  float a = beta[j];
  for (int64_t d = 0; d < n_x; ++d) a = fmaf(omega[j * n_x + d], X[n * n_x + d], a);
  phi[i] = 1.41421356f * cosf(a);
}

// One warp per problem: bag of tokens (token counts / tape length) and the 32 target
// features (asinh(mean), log(std + 1e-3), skewness, asinh(excess kurtosis), and the
// mean of the standardised target times each random feature).
__global__ void __launch_bounds__(256) features_kernel(const int64_t* __restrict__ ops, int64_t B, int64_t M,
                                                       int64_t ops_sb, int64_t ops_sm, const float* __restrict__ Y,
                                                       int64_t N, const float* __restrict__ phi,
                                                       __nv_bfloat16* __restrict__ hist,
                                                       __nv_bfloat16* __restrict__ hist_t, int64_t ld_t,
                                                       __nv_bfloat16* __restrict__ x0,
                                                       __nv_bfloat16* __restrict__ x0_t,
                                                       float* __restrict__ feats) {
  __shared__ int cnt[8][SR_MLP_VOCAB];
  const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
  const int64_t b = (int64_t)blockIdx.x * 8 + wl;
  if (b >= B) return;
  for (int v = lane; v < SR_MLP_VOCAB; v += 32) cnt[wl][v] = 0;
  __syncwarp();
  int L = 0;
  for (int64_t m = lane; m < M; m += 32) {
    const int64_t t = ops[b * ops_sb + m * ops_sm];
    if (t != 0) {
      ++L;
      atomicAdd(&cnt[wl][(t >= 0 && t < SR_MLP_VOCAB) ? (int)t : SR_MLP_VOCAB - 1], 1);
    }
  }
  L = warp_sum(L);
  __syncwarp();
  const float invL = L > 0 ? 1.f / (float)L : 0.f;
  for (int v = lane; v < SR_MLP_VOCAB; v += 32) {
    const __nv_bfloat16 h = __float2bfloat16_rn((float)cnt[wl][v] * invL);
    hist[b * SR_MLP_VOCAB + v] = h;
    hist_t[(int64_t)v * ld_t + b] = h;
  }
  // moments of Y (two passes over the row)
  const float* y = Y + b * N;
  float s1 = 0.f;
  for (int64_t n = lane; n < N; n += 32) s1 += y[n];
  const float mu = warp_sum(s1) / (float)N;
  float s2 = 0.f, s3 = 0.f, s4 = 0.f;
  for (int64_t n = lane; n < N; n += 32) {
    const float d = y[n] - mu, d2 = d * d;
    s2 += d2;
    s3 += d2 * d;
    s4 += d2 * d2;
  }
  const float m2 = warp_sum(s2) / (float)N, m3 = warp_sum(s3) / (float)N, m4 = warp_sum(s4) / (float)N;
  const float sd = sqrtf(m2);
  const bool flat = !(sd > 1e-12f);
  const float inv_sd = flat ? 0.f : 1.f / sd;
  float proj[SR_MLP_PROJ];
#pragma unroll
  for (int j = 0; j < SR_MLP_PROJ; ++j) proj[j] = 0.f;
  for (int64_t n = lane; n < N; n += 32) {
    const float z = (y[n] - mu) * inv_sd;
    const float* ph = phi + n * SR_MLP_PROJ;
#pragma unroll
    for (int j = 0; j < SR_MLP_PROJ; ++j) proj[j] = fmaf(z, ph[j], proj[j]);
  }
  float f[SR_MLP_FEATS];
  f[0] = asinhf(mu);
  f[1] = logf(sd + 1e-3f);
  f[2] = flat ? 0.f : fminf(fmaxf(m3 * inv_sd * inv_sd * inv_sd, -50.f), 50.f);
  f[3] = flat ? 0.f : asinhf(m4 * inv_sd * inv_sd * inv_sd * inv_sd - 3.f);
#pragma unroll
  for (int j = 0; j < SR_MLP_PROJ; ++j) f[4 + j] = warp_sum(proj[j]) / (float)N;
  // lane j writes feature j (and zeros in the padding columns)
  float mine = 0.f;
#pragma unroll
  for (int j = 0; j < SR_MLP_FEATS; ++j)
    if (lane == j) mine = f[j];
  if (!isfinite(mine)) mine = 0.f;
  if (feats) feats[b * SR_MLP_FEATS + lane] = mine;
  const __nv_bfloat16 hb = __float2bfloat16_rn(mine);
  x0[b * SR_MLP_IN + SR_MLP_EMB + lane] = hb;
  x0[b * SR_MLP_IN + SR_MLP_EMB + SR_MLP_FEATS + lane] = __float2bfloat16_rn(0.f);
  x0_t[(int64_t)(SR_MLP_EMB + lane) * ld_t + b] = hb;
  x0_t[(int64_t)(SR_MLP_EMB + SR_MLP_FEATS + lane) * ld_t + b] = __float2bfloat16_rn(0.f);
}

// ---- loss, reductions, optimiser ----------------------------------------------------

// Thread per row: squared error against the targets where mask > 0, and the bf16
// output gradient scale * 2 (out - target) * mask (zero in the padding columns).
__global__ void loss_kernel(const float* __restrict__ out, int64_t rows, int64_t ld_out,
                            const float* __restrict__ target, const float* __restrict__ mask, int n_out,
                            float scale, float* __restrict__ row_loss, __nv_bfloat16* __restrict__ d_out,
                            int64_t ld_d, __nv_bfloat16* __restrict__ d_out_t, int64_t ld_dt) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  float acc = 0.f;
  for (int64_t j = 0; j < ld_d; ++j) {
    float g = 0.f;
    if (j < n_out) {
      const float mk = mask[r * n_out + j];
      const float d = out[r * ld_out + j] - target[r * n_out + j];
      if (mk > 0.f) {
        acc = fmaf(mk * d, d, acc);
        g = scale * 2.f * mk * d;
      }
    }
    const __nv_bfloat16 gb = __float2bfloat16_rn(g);
    d_out[r * ld_d + j] = gb;
    if (d_out_t) d_out_t[j * ld_dt + r] = gb;
  }
  if (row_loss) row_loss[r] = acc;
}

// Thread per row: an externally computed output gradient, scaled, in bf16; rows with
// a non-finite entry contribute nothing.
__global__ void output_grad_kernel(const float* __restrict__ g, int64_t rows, int n_out, int64_t ld_g, float scale,
                                   __nv_bfloat16* __restrict__ d_out, int64_t ld_d, __nv_bfloat16* __restrict__ d_out_t,
                                   int64_t ld_dt) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  bool finite = true;
  for (int j = 0; j < n_out; ++j) finite = finite && isfinite(g[r * ld_g + j]);
  for (int64_t j = 0; j < ld_d; ++j) {
    const float v = (finite && j < n_out) ? scale * g[r * ld_g + j] : 0.f;
    const __nv_bfloat16 b = __float2bfloat16_rn(v);
    d_out[r * ld_d + j] = b;
    if (d_out_t) d_out_t[j * ld_dt + r] = b;
  }
}

// Warp per output row: out[j] = sum over the row of xt[j][:] (bias gradients).
__global__ void colsum_kernel(const __nv_bfloat16* __restrict__ xt, int64_t n, int64_t rows, int64_t ld,
                              float* __restrict__ out) {
  const int64_t j = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (j >= n) return;
  float s = 0.f;
  for (int64_t r = lane; r < rows; r += 32) s += __bfloat162float(xt[j * ld + r]);
  s = warp_sum(s);
  if (lane == 0) out[j] = s;
}

__global__ void reduce_splits_kernel(const float* __restrict__ part, int splits, int64_t count,
                                     int64_t split_stride, float* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  float s = 0.f;
  for (int k = 0; k < splits; ++k) s += part[k * split_stride + i];
  out[i] = s;
}

// Adam with decoupled weight decay on fp32 master weights (rows x cols), then the
// bf16 copies used by the GEMMs: row-major and (optionally) transposed.
__global__ void adam_kernel(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, int64_t rows, int64_t cols, float lr, float beta1, float beta2,
                            float eps, float weight_decay, float bc1, float bc2, __nv_bfloat16* __restrict__ w_bf16,
                            __nv_bfloat16* __restrict__ w_t_bf16) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows * cols) return;
  float wi = w[i];
  if (lr != 0.f) {
    const float gi = g[i];
    const float mi = beta1 * m[i] + (1.f - beta1) * gi;
    const float vi = beta2 * v[i] + (1.f - beta2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    wi -= lr * ((mi / bc1) / (sqrtf(vi / bc2) + eps) + weight_decay * wi);
    w[i] = wi;
  }
  const __nv_bfloat16 wb = __float2bfloat16_rn(wi);
  if (w_bf16) w_bf16[i] = wb;
  if (w_t_bf16) w_t_bf16[(i % cols) * rows + i / cols] = wb;
}

// ---- host --------------------------------------------------------------------------

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* ptr = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
  });
  return fn;
}

// 2-D bf16 tensor of `rows` rows of `cols` elements, `ld` elements apart; boxes of
// 64 x box_rows with the 128-byte swizzle; out-of-range elements read as zero.
static int make_map(CUtensorMap* map, const void* ptr, int64_t rows, int64_t cols, int64_t ld, int box_rows) {
  auto fn = encode_fn();
  if (!fn) {
    set_error("cuTensorMapEncodeTiled is not available from the driver");
    return SR_ERR_CUDA;
  }
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  cuuint32_t box[2] = {(cuuint32_t)kTileK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
    return SR_ERR_CUDA;
  }
  return SR_OK;
}

template <int BN>
static size_t gemm_smem() {
  return 1024 + (size_t)kStages * (kTileM * kTileK * 2 + BN * kTileK * 2) + 8 * (2 * kStages + 1) + 16;
}

template <int BN>
static int launch_gemm(const CUtensorMap& ma, const CUtensorMap& mb, const GemmParams& p, int grid_x, int splits,
                       cudaStream_t st) {
  static std::once_flag once;
  static cudaError_t attr = cudaSuccess;
  std::call_once(once, [] {
    attr = cudaFuncSetAttribute(gemm_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gemm_smem<BN>());
  });
  if (attr != cudaSuccess) return cuda_check(attr, "mlp gemm shared memory attribute");
  gemm_kernel<BN><<<dim3(grid_x, splits), kThreads, gemm_smem<BN>(), st>>>(ma, mb, p);
  return launch_check("mlp gemm_kernel");
}

static bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace mlp
}  // namespace sr

extern "C" {

int sr_mlp_gemm(const uint16_t* A, int64_t rows, int64_t k, int64_t lda, const uint16_t* W, int64_t n, int64_t ldw,
                const sr_mlp_epilogue* epi, int32_t* status, void* stream) {
  using namespace sr;
  using namespace sr::mlp;
  if (!epi || rows < 0) {
    set_error("sr_mlp_gemm: invalid arguments");
    return SR_ERR_INVALID_ARGUMENT;
  }
  if (rows == 0) return SR_OK;
  if (k <= 0 || k % kTileK || !(n == 64 || n == 128 || n == 256) || lda < k || ldw < k || lda % 8 || ldw % 8 ||
      !A || !W || !aligned16(A) || !aligned16(W) || rows > (int64_t)1 << 30 || !status) {
    set_error("sr_mlp_gemm: k must be a positive multiple of 64, n one of 64/128/256, lda/ldw >= k and multiples "
              "of 8, A and W 16-byte aligned (rows=%lld k=%lld n=%lld lda=%lld ldw=%lld)",
              (long long)rows, (long long)k, (long long)n, (long long)lda, (long long)ldw);
    return SR_ERR_INVALID_ARGUMENT;
  }
  const int mode = epi->epilogue;
  Epi e{};
  e.mode = mode;
  e.bias = epi->bias_dev;
  e.gate = reinterpret_cast<const __nv_bfloat16*>(epi->gate_dev);
  e.ld_gate = epi->ld_gate;
  e.out = reinterpret_cast<__nv_bfloat16*>(epi->out_dev);
  e.ld_out = epi->ld_out;
  e.out_col0 = epi->out_col0;
  e.out_t = reinterpret_cast<__nv_bfloat16*>(epi->out_t_dev);
  e.ld_out_t = epi->ld_out_t;
  e.out_t_row0 = epi->out_t_row0;
  e.out_f32 = epi->out_f32_dev;
  e.ld_out_f32 = epi->ld_out_f32;
  e.split_stride = epi->split_stride;
  bool bad = false;
  switch (mode) {
    case SR_MLP_EPI_RELU:
    case SR_MLP_EPI_LINEAR:
    case SR_MLP_EPI_RELU_GRAD:
      if (!e.out && !e.out_t) bad = true;
      if (e.out && (!aligned16(e.out) || e.ld_out % 8 || e.out_col0 % 8 || e.out_col0 < 0 || e.ld_out < e.out_col0 + n))
        bad = true;
      if (e.out_t && (e.ld_out_t < rows || e.out_t_row0 < 0)) bad = true;
      if (mode == SR_MLP_EPI_RELU_GRAD && (!e.gate || !aligned16(e.gate) || e.ld_gate % 8 || e.ld_gate < n))
        bad = true;
      break;
    case SR_MLP_EPI_F32:
    case SR_MLP_EPI_SPLIT_F32:
      if (!e.out_f32 || !aligned16(e.out_f32) || e.ld_out_f32 % 4 || e.ld_out_f32 < n) bad = true;
      if (mode == SR_MLP_EPI_SPLIT_F32 && (e.split_stride < rows * e.ld_out_f32 || e.split_stride % 4 || e.bias))
        bad = true;
      break;
    default:
      bad = true;
  }
  if (bad) {
    set_error("sr_mlp_gemm: epilogue %d has missing, misaligned or too small outputs", mode);
    return SR_ERR_INVALID_ARGUMENT;
  }
  GemmParams p{};
  p.rows = (int)rows;
  p.k_chunks = (int)(k / kTileK);
  int splits = 1;
  if (mode == SR_MLP_EPI_SPLIT_F32) splits = epi->splits < 1 ? 1 : (epi->splits > p.k_chunks ? p.k_chunks : epi->splits);
  p.chunks_per_split = (p.k_chunks + splits - 1) / splits;
  splits = (p.k_chunks + p.chunks_per_split - 1) / p.chunks_per_split;  // every split has work
  p.e = e;
  p.status = status;
  CUtensorMap ma, mb;
  int rc = make_map(&ma, A, rows, k, lda, kTileM);
  if (rc) return rc;
  rc = make_map(&mb, W, n, k, ldw, (int)n);
  if (rc) return rc;
  const int grid_x = (int)((rows + kTileM - 1) / kTileM);
  cudaStream_t st = as_stream(stream);
  switch (n) {
    case 64: return launch_gemm<64>(ma, mb, p, grid_x, splits, st);
    case 128: return launch_gemm<128>(ma, mb, p, grid_x, splits, st);
    default: return launch_gemm<256>(ma, mb, p, grid_x, splits, st);
  }
}

int sr_mlp_gemm_splits_used(int64_t k, int32_t splits) {
  const int kc = (int)(k / sr::mlp::kTileK);
  if (kc <= 0) return 0;
  int s = splits < 1 ? 1 : (splits > kc ? kc : splits);
  const int cps = (kc + s - 1) / s;
  return (kc + cps - 1) / cps;
}

int sr_mlp_random_features(const float* X, int64_t N, int64_t n_x, const float* omega, const float* beta, float* phi,
                           void* stream) {
  using namespace sr;
  if (N < 0 || n_x < 0 || (N > 0 && (!X || !omega || !beta || !phi))) {
    set_error("sr_mlp_random_features: invalid arguments");
    return SR_ERR_INVALID_ARGUMENT;
  }
  if (N == 0) return SR_OK;
  const int64_t total = N * SR_MLP_PROJ;
  mlp::random_features_kernel<<<(unsigned)((total + 255) / 256), 256, 0, as_stream(stream)>>>(X, N, n_x, omega, beta,
                                                                                              phi);
  return launch_check("random_features_kernel");
}

int sr_mlp_features(const int64_t* ops, int64_t B, int64_t M, int64_t ops_sb, int64_t ops_sm, const float* Y,
                    int64_t N, const float* phi, uint16_t* hist, uint16_t* hist_t, int64_t ld_t, uint16_t* x0,
                    uint16_t* x0_t, float* feats, void* stream) {
  using namespace sr;
  if (B < 0 || M < 0 || N <= 0 || ld_t < B ||
      (B > 0 && (!ops || !Y || !phi || !hist || !hist_t || !x0 || !x0_t))) {
    set_error("sr_mlp_features: invalid arguments");
    return SR_ERR_INVALID_ARGUMENT;
  }
  if (B == 0) return SR_OK;
  mlp::features_kernel<<<(unsigned)((B + 7) / 8), 256, 0, as_stream(stream)>>>(
      ops, B, M, ops_sb, ops_sm, Y, N, phi, reinterpret_cast<__nv_bfloat16*>(hist),
      reinterpret_cast<__nv_bfloat16*>(hist_t), ld_t, reinterpret_cast<__nv_bfloat16*>(x0),
      reinterpret_cast<__nv_bfloat16*>(x0_t), feats);
  return launch_check("features_kernel");
}

int sr_mlp_loss(const float* out, int64_t rows, int64_t ld_out, const float* target, const float* mask,
                int32_t n_out, float scale, float* row_loss, uint16_t* d_out, int64_t ld_d, uint16_t* d_out_t,
                int64_t ld_dt, void* stream) {
  using namespace sr;
  if (rows < 0 || n_out < 0 || ld_out < n_out || ld_d < n_out ||
      (rows > 0 && (!out || !target || !mask || !d_out || (d_out_t && ld_dt < rows)))) {
    set_error("sr_mlp_loss: invalid arguments");
    return SR_ERR_INVALID_ARGUMENT;
  }
  if (rows == 0) return SR_OK;
  mlp::loss_kernel<<<(unsigned)((rows + 255) / 256), 256, 0, as_stream(stream)>>>(
      out, rows, ld_out, target, mask, n_out, scale, row_loss, reinterpret_cast<__nv_bfloat16*>(d_out), ld_d,
      reinterpret_cast<__nv_bfloat16*>(d_out_t), ld_dt);
  return launch_check("loss_kernel");
}

int sr_mlp_output_grad(const float* g, int64_t rows, int32_t n_out, int64_t ld_g, float scale, uint16_t* d_out,
                       int64_t ld_d, uint16_t* d_out_t, int64_t ld_dt, void* stream) {
  using namespace sr;
  if (rows < 0 || n_out < 0 || ld_g < n_out || ld_d < n_out || (rows > 0 && (!g || !d_out || (d_out_t && ld_dt < rows)))) {
    set_error("sr_mlp_output_grad: invalid arguments");
    return SR_ERR_INVALID_ARGUMENT;
  }
  if (rows == 0) return SR_OK;
  mlp::output_grad_kernel<<<(unsigned)((rows + 255) / 256), 256, 0, as_stream(stream)>>>(
      g, rows, n_out, ld_g, scale, reinterpret_cast<__nv_bfloat16*>(d_out), ld_d,
      reinterpret_cast<__nv_bfloat16*>(d_out_t), ld_dt);
  return launch_check("output_grad_kernel");
}

int sr_mlp_colsum(const uint16_t* xt, int64_t n, int64_t rows, int64_t ld, float* out, void* stream) {
  using namespace sr;
  if (n < 0 || rows < 0 || ld < rows || (n > 0 && (!xt || !out))) {
    set_error("sr_mlp_colsum: invalid arguments");
    return SR_ERR_INVALID_ARGUMENT;
  }
  if (n == 0) return SR_OK;
  mlp::colsum_kernel<<<(unsigned)((n * 32 + 255) / 256), 256, 0, as_stream(stream)>>>(
      reinterpret_cast<const __nv_bfloat16*>(xt), n, rows, ld, out);
  return launch_check("colsum_kernel");
}

int sr_mlp_reduce_splits(const float* part, int32_t splits, int64_t count, int64_t split_stride, float* out,
                         void* stream) {
  using namespace sr;
  if (splits < 1 || count < 0 || split_stride < count || (count > 0 && (!part || !out))) {
    set_error("sr_mlp_reduce_splits: invalid arguments");
    return SR_ERR_INVALID_ARGUMENT;
  }
  if (count == 0) return SR_OK;
  mlp::reduce_splits_kernel<<<(unsigned)((count + 255) / 256), 256, 0, as_stream(stream)>>>(part, splits, count,
                                                                                            split_stride, out);
  return launch_check("reduce_splits_kernel");
}

int sr_mlp_adam(float* w, const float* g, float* m, float* v, int64_t rows, int64_t cols, float lr, float beta1,
                float beta2, float eps, float weight_decay, int32_t step, uint16_t* w_bf16, uint16_t* w_t_bf16,
                void* stream) {
  using namespace sr;
  if (rows < 0 || cols < 0 || (rows * cols > 0 && (!w || (lr != 0.f && (!g || !m || !v || step < 1))))) {
    set_error("sr_mlp_adam: invalid arguments");
    return SR_ERR_INVALID_ARGUMENT;
  }
  const int64_t count = rows * cols;
  if (count == 0) return SR_OK;
  const float bc1 = step > 0 ? 1.f - powf(beta1, (float)step) : 1.f;
  const float bc2 = step > 0 ? 1.f - powf(beta2, (float)step) : 1.f;
  mlp::adam_kernel<<<(unsigned)((count + 255) / 256), 256, 0, as_stream(stream)>>>(
      w, g, m, v, rows, cols, lr, beta1, beta2, eps, weight_decay, bc1, bc2, reinterpret_cast<__nv_bfloat16*>(w_bf16),
      reinterpret_cast<__nv_bfloat16*>(w_t_bf16));
  return launch_check("adam_kernel");
}

}  // extern "C"
