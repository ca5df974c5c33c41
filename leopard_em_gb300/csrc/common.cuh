// Shared definitions for the GB300 2DTM kernels: status codes, complex helpers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/leopard_gb300.h"

namespace lgb {

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// a * conj(b)
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }

// float -> double with integer operations (exponent re-bias, mantissa shift):
// exact for normal floats, which leaves the FP64 pipe (about one operation per
// SM per clock on this GPU, conversions included) to the additions.  Zero,
// subnormal, inf and nan go through the converter.
__device__ __forceinline__ double f2d_bits(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned ex = (u >> 23) & 0xffu;
  if (ex == 0u || ex == 0xffu) return (double)f;
  const unsigned hi = (u & 0x80000000u) | ((ex + 896u) << 20) | ((u & 0x7fffffu) >> 3);
  return __hiloint2double((int)hi, (int)(u << 29));
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// multiply by DIR*i  (DIR = +1: i, DIR = -1: -i)
template <int DIR>
__device__ __forceinline__ float2 mul_i(float2 a) {
  return DIR > 0 ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// Status codes returned by every C-ABI entry point (see include/leopard_gb300.h).
#define LGB_CUDA_TRY(expr)                                   \
  do {                                                       \
    cudaError_t _e = (expr);                                 \
    if (_e != cudaSuccess) return LGB_ERR_CUDA;              \
  } while (0)

}  // namespace lgb
