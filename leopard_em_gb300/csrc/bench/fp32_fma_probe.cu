// FP32 FMA throughput probe: the non-tensor FP32 peak of this GPU (the
// denominator of the FFT kernels' compute roofline), measured with
// independent FMA chains in registers.  Measurement only: it is linked into
// its own library (_build/libleopard_gb300_probe.so), which the benchmark
// loads; the product library does not carry it.
#include "../common.cuh"

namespace lgb {

__global__ void __launch_bounds__(256) fma_probe_kernel(int iters, float seed, float* out) {
  // 8 independent chains per thread hide the FMA latency
  float a0 = seed + threadIdx.x, a1 = a0 + 1.f, a2 = a0 + 2.f, a3 = a0 + 3.f;
  float a4 = a0 + 4.f, a5 = a0 + 5.f, a6 = a0 + 6.f, a7 = a0 + 7.f;
  const float m = 0.999999f, c = 1e-7f;
#pragma unroll 1
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      a0 = fmaf(a0, m, c); a1 = fmaf(a1, m, c); a2 = fmaf(a2, m, c); a3 = fmaf(a3, m, c);
      a4 = fmaf(a4, m, c); a5 = fmaf(a5, m, c); a6 = fmaf(a6, m, c); a7 = fmaf(a7, m, c);
    }
  }
  const float s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == 12345.678f) out[0] = s;  // keeps the chains alive, never true in practice
}

}  // namespace lgb

using namespace lgb;

extern "C" int lgb_fp32_fma_probe(int blocks, int iters, float* out, void* stream) {
  if (blocks < 1 || iters < 1 || !out) return LGB_ERR_INVALID_ARGUMENT;
  fma_probe_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(iters, 0.5f, out);
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}
