// sr_common.cuh -- host-side helpers shared by the C-ABI translation units.
#pragma once
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cuda_runtime.h>

#include "../../include/sr_gb300.h"

namespace sr {

// Thread-local text of the last API-level failure (sr_last_error()).
void set_error(const char* fmt, ...);

inline int cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return SR_OK;
  set_error("%s: %s", what, cudaGetErrorString(e));
  return SR_ERR_CUDA;
}

inline int launch_check(const char* what) { return cuda_check(cudaGetLastError(), what); }

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

__device__ __forceinline__ void report(int* status, int code) {
  if (code) atomicCAS(status, 0, code);
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

}  // namespace sr
