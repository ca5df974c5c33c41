// C-ABI entry of the split-precision tcgen05 GEMM with a plain FP32 store
// epilogue (the building block of the precision form, exposed for its tests).
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "tc_gemm.cuh"

namespace lgb {

struct EpiStore {
  struct Params {
    float* d;
    int ldd;
    int m_valid;
    int n_valid;
  };
  static __device__ __forceinline__ void apply(int row, int col0, const float* v, const Params& p) {
    if (row >= p.m_valid) return;
    float* out = p.d + (size_t)row * p.ldd;
#pragma unroll
    for (int i = 0; i < 32; ++i)
      if (col0 + i < p.n_valid) out[col0 + i] = v[i];
  }
};

template <int BN, bool F16>
static int tc_gemm_t(int m_tiles, int n_tiles, const TcGemmArgs& g, const EpiStore::Params& ep, cudaStream_t s) {
  constexpr int SMEM = TcSmem<BN>::BYTES;
  if (cudaFuncSetAttribute(tc_gemm_kernel<EpiStore, BN, F16>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM) !=
      cudaSuccess)
    return LGB_ERR_CUDA;
  tc_gemm_kernel<EpiStore, BN, F16><<<dim3(n_tiles, m_tiles), kTcThreads, SMEM, s>>>(g, ep);
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

// Wait-timeout self-test: one thread waits on an mbarrier phase that nothing
// completes, with a bounded number of polls, and reports the timeout through
// the device status word -- the path every bounded wait takes on expiry.
__global__ void wait_timeout_selftest_kernel(unsigned polls, int* status) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    if (!mbar_wait(&bar, 0, polls)) atomicExch(status, LGB_ERR_DEVICE_TIMEOUT);
  }
}

}  // namespace lgb

using namespace lgb;

extern "C" int lgb_wait_timeout_selftest(unsigned polls, int* device_status, void* stream) {
  if (!device_status || polls == 0 || polls > kTcSpinLimit) return LGB_ERR_INVALID_ARGUMENT;
  wait_timeout_selftest_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(polls, device_status);
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

extern "C" int lgb_tc_gemm(int m_tiles, int n_tiles, int k_chunks, int bn, int f16, int terms, const void* a_hi,
                           const void* a_lo, const void* b_hi, const void* b_lo, float* d, int ldd, int m_valid,
                           int n_valid, int* err, void* stream) {
  if (m_tiles < 1 || n_tiles < 1 || k_chunks < 1 || (bn != 128 && bn != 256) || (terms != 1 && terms != 3) ||
      !a_hi || !b_hi || (terms == 3 && (!a_lo || !b_lo)) || !d || !err || ldd < 1 || m_valid < 0 || n_valid < 0 ||
      m_valid > m_tiles * kTcM || n_valid > n_tiles * bn || n_valid > ldd)
    return LGB_ERR_INVALID_ARGUMENT;
  // every block is read with 16-byte bulk copies
  const uintptr_t al = reinterpret_cast<uintptr_t>(a_hi) | reinterpret_cast<uintptr_t>(b_hi) |
                       reinterpret_cast<uintptr_t>(a_lo) | reinterpret_cast<uintptr_t>(b_lo);
  if (al & 15) return LGB_ERR_INVALID_ARGUMENT;
  TcGemmArgs g{static_cast<const uint16_t*>(a_hi), static_cast<const uint16_t*>(a_lo),
               static_cast<const uint16_t*>(b_hi), static_cast<const uint16_t*>(b_lo), k_chunks, terms, err};
  EpiStore::Params ep{d, ldd, m_valid, n_valid};
  cudaStream_t s = (cudaStream_t)stream;
  if (bn == 256) return f16 ? tc_gemm_t<256, true>(m_tiles, n_tiles, g, ep, s) : tc_gemm_t<256, false>(m_tiles, n_tiles, g, ep, s);
  return f16 ? tc_gemm_t<128, true>(m_tiles, n_tiles, g, ep, s) : tc_gemm_t<128, false>(m_tiles, n_tiles, g, ep, s);
}
