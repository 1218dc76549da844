// Shared device helpers for the GB300 gridder kernels.
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <stdint.h>

namespace gg {

// Largest KB table the kernels stage in shared memory; the reference stages
// its table in `__shared__ float locKer[1000]` (gpuForwardProject.cu:26).
constexpr int kMaxKerSize = 1000;

// Storage-type loads (read-only path) returning FP32.
__device__ __forceinline__ float ld_f32(const float *p) { return __ldg(p); }
__device__ __forceinline__ float ld_f32(const __half *p) { return __half2float(__ldg(p)); }
__device__ __forceinline__ float ld_f32(const __nv_bfloat16 *p) { return __bfloat162float(__ldg(p)); }

template <typename T> __device__ __forceinline__ T from_f32(float x);
template <> __device__ __forceinline__ float from_f32<float>(float x) { return x; }
template <> __device__ __forceinline__ __half from_f32<__half>(float x) { return __float2half_rn(x); }
template <> __device__ __forceinline__ __nv_bfloat16 from_f32<__nv_bfloat16>(float x) { return __float2bfloat16_rn(x); }

} // namespace gg
