// sr_consts.cu -- create_constants: row-major rank of every LEARNABLE_CONSTANT entry
// of an Ops view and the scatter of drawn values into a dense constant table.
// (reference symbolic_torch/utils.py:7-41: output[const_mask] = constants_flat)
#include <cstdint>

#include "sr_common.cuh"
#include "sr_ops.cuh"

namespace sr {

// One warp per row: number of LEARNABLE entries.
__global__ void const_count_kernel(const int64_t* __restrict__ ops, int64_t R, int64_t Cc, int64_t s0, int64_t s1,
                                   int64_t* __restrict__ counts) {
  const int lane = threadIdx.x & 31;
  const int64_t wstride = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < R; r += wstride) {
    int c = 0;
    for (int64_t j0 = 0; j0 < Cc; j0 += 32) {
      const int64_t j = j0 + lane;
      c += __popc(__ballot_sync(0xffffffffu, j < Cc && ops[r * s0 + j * s1] == LEARNABLE));
    }
    if (lane == 0) counts[r + 1] = c;
  }
}

// Single CTA: in-place inclusive scan of counts[1..R], counts[0] = 0.
__global__ void const_scan_kernel(int64_t* __restrict__ off, int64_t R) {
  __shared__ int64_t warp_tot[32];
  __shared__ int64_t carry;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  if (tid == 0) { carry = 0; off[0] = 0; }
  __syncthreads();
  for (int64_t base = 0; base < R; base += blockDim.x) {
    const int64_t i = base + tid;
    int64_t v = i < R ? off[i + 1] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t t = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += t;
    }
    if (lane == 31) warp_tot[w] = v;
    __syncthreads();
    if (w == 0) {
      int64_t t = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int64_t u = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += u;
      }
      if (lane < (int)(blockDim.x >> 5)) warp_tot[lane] = t;
    }
    __syncthreads();
    const int64_t add = carry + (w > 0 ? warp_tot[w - 1] : 0);
    if (i < R) off[i + 1] = v + add;
    __syncthreads();
    if (tid == blockDim.x - 1) carry = add + v;
    __syncthreads();
  }
}

__global__ void const_scatter_kernel(const int64_t* __restrict__ ops, int64_t R, int64_t Cc, int64_t s0, int64_t s1,
                                     const int64_t* __restrict__ off, const float* __restrict__ values,
                                     float* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t wstride = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < R; r += wstride) {
    int64_t rank = off[r];
    for (int64_t j0 = 0; j0 < Cc; j0 += 32) {
      const int64_t j = j0 + lane;
      const bool lc = j < Cc && ops[r * s0 + j * s1] == LEARNABLE;
      const unsigned m = __ballot_sync(0xffffffffu, lc);
      if (j < Cc) out[r * Cc + j] = lc ? values[rank + __popc(m & ((1u << lane) - 1u))] : 0.f;
      rank += __popc(m);
    }
  }
}

}  // namespace sr

extern "C" {

int sr_const_offsets(const int64_t* ops, int64_t R, int64_t Cc, int64_t s0, int64_t s1, int64_t* off, void* stream) {
  using namespace sr;
  if (R < 0 || Cc < 0 || !off || (R > 0 && Cc > 0 && !ops)) { set_error("invalid arguments"); return SR_ERR_INVALID_ARGUMENT; }
  cudaStream_t st = as_stream(stream);
  int rc = cuda_check(cudaMemsetAsync(off, 0, sizeof(int64_t) * (R + 1), st), "offsets reset");
  if (rc || R == 0 || Cc == 0) return rc;
  int64_t blocks = (R + 7) / 8;
  if (blocks > 65535) blocks = 65535;
  const_count_kernel<<<(unsigned)blocks, 256, 0, st>>>(ops, R, Cc, s0, s1, off);
  rc = launch_check("const_count_kernel");
  if (rc) return rc;
  const_scan_kernel<<<1, 1024, 0, st>>>(off, R);
  return launch_check("const_scan_kernel");
}

int sr_const_scatter(const int64_t* ops, int64_t R, int64_t Cc, int64_t s0, int64_t s1, const int64_t* off,
                     const float* values, float* out, void* stream) {
  using namespace sr;
  if (R < 0 || Cc < 0 || (R > 0 && Cc > 0 && (!ops || !off || !out))) { set_error("invalid arguments"); return SR_ERR_INVALID_ARGUMENT; }
  if (R == 0 || Cc == 0) return SR_OK;
  cudaStream_t st = as_stream(stream);
  int64_t blocks = (R + 7) / 8;
  if (blocks > 65535) blocks = 65535;
  const_scatter_kernel<<<(unsigned)blocks, 256, 0, st>>>(ops, R, Cc, s0, s1, off, values, out);
  return launch_check("const_scatter_kernel");
}

}  // extern "C"
