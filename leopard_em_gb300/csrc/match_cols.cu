// Launcher: the fused column pass (forward FFT, cross power, inverse FFT) for
// image height H.
#include "match_fused.cuh"
#include "match_kernels.cuh"
#include "match_launch.h"

namespace lgb {

#define LGB_COL_SIZES(X) \
  X(48) X(64) X(128) X(256) X(288) X(512) X(576) X(1024) X(2048) X(2880) X(3072) X(3840) X(4096) X(5760)

bool supported_col(int H) {
  switch (H) {
#define X(n) case n:
    LGB_COL_SIZES(X)
#undef X
    return true;
    default:
      return false;
  }
}

// Split the correlogram loop of each column group over grid.y until the grid
// covers about `waves` x the SM count; returns the split and the correlograms
// per CTA.
static int colpass_split(int groups, int n_c, int waves, int* per) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (waves <= 0) waves = 4;
  int split = 1;
  while (split < n_c && groups * split < waves * sms) split *= 2;
  if (split > n_c) split = n_c;
  *per = (n_c + split - 1) / split;
  return (n_c + *per - 1) / *per;
}

template <int HN>
static int colpass_tab_t(const void* A, const void* Ip, int h, int Wcp, int n_c, int cpi, int y_rows, int waves,
                         void* Y, cudaStream_t s) {
  using CT = ColTab<HN>;
  if (cudaFuncSetAttribute(colpass_tab_kernel<HN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CT::SMEM) !=
      cudaSuccess)
    return LGB_ERR_CUDA;
  int per = 1;
  const int groups = (Wcp + CT::G - 1) / CT::G;
  const int split = colpass_split(groups, n_c, waves, &per);
  colpass_tab_kernel<HN><<<dim3(groups, split), CT::G * CT::NT, CT::SMEM, s>>>(
      static_cast<const float2*>(A), static_cast<const float2*>(Ip), h, Wcp, n_c, per, cpi, y_rows,
      static_cast<float2*>(Y));
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

template <int R, int P>
static int colpass_fused_t(const void* A, const void* Ip, int h, int Wcp, int n_c, int cpi, int y_rows, int waves,
                           void* Y, cudaStream_t s) {
  using CF = ColFused<R, P>;
  if (cudaFuncSetAttribute(colpass_fused_kernel<R, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CF::SMEM) !=
      cudaSuccess)
    return LGB_ERR_CUDA;
  int per = 1;
  const int groups = Wcp / kColGroup;
  const int split = colpass_split(groups, n_c, waves, &per);
  dim3 grid(groups, split);
  colpass_fused_kernel<R, P><<<grid, CF::THREADS, CF::SMEM, s>>>(
      static_cast<const float2*>(A), static_cast<const float2*>(Ip), h, Wcp, n_c, per, cpi, y_rows,
      static_cast<float2*>(Y));
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

template <int R1, int R2>
static int colpass_pair_t(const void* A, const void* Ip, int h, int Wcp, int n_c, int cpi, int y_rows, int waves,
                          void* Y, cudaStream_t s, const float2* norm, int norm_stride, int norm_w) {
  using CP = ColPair<R1, R2>;
  if (cudaFuncSetAttribute(colpass_pair_kernel<R1, R2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CP::SMEM) !=
      cudaSuccess)
    return LGB_ERR_CUDA;
  int per = 1;
  const int groups = (Wcp + CP::G - 1) / CP::G;
  const int split = colpass_split(groups, n_c, waves, &per);
  colpass_pair_kernel<R1, R2><<<dim3(groups, split), CP::THREADS, CP::SMEM, s>>>(
      static_cast<const float2*>(A), static_cast<const float2*>(Ip), h, Wcp, n_c, per, cpi, y_rows,
      static_cast<float2*>(Y), norm, norm_stride, norm_w);
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

int launch_colpass(int H, const void* A, const void* Ip, int h, int Wcp, int n_c, int cpi, int y_rows, int waves,
                   void* Y, cudaStream_t s, const float2* norm, int norm_stride, int norm_w) {
  if (cpi < 1 || y_rows < 1 || y_rows > H || Wcp % kColGroup) return LGB_ERR_INVALID_ARGUMENT;
  if (norm && (H != 288 || norm_w < 2 || norm_w / 2 + 1 > Wcp || norm_stride < 1)) return LGB_ERR_UNSUPPORTED_SIZE;
  switch (H) {
    case 4096:
      return colpass_fused_t<16, 3>(A, Ip, h, Wcp, n_c, cpi, y_rows, waves, Y, s);
    case 512:
      return colpass_fused_t<8, 3>(A, Ip, h, Wcp, n_c, cpi, y_rows, waves, Y, s);
    case 256:
      return colpass_fused_t<16, 2>(A, Ip, h, Wcp, n_c, cpi, y_rows, waves, Y, s);
    case 64:
      return colpass_fused_t<8, 2>(A, Ip, h, Wcp, n_c, cpi, y_rows, waves, Y, s);
    case 288:
      return colpass_pair_t<16, 18>(A, Ip, h, Wcp, n_c, cpi, y_rows, waves, Y, s, norm, norm_stride, norm_w);
    default:
      break;
  }
  switch (H) {
#define X(n) \
  case n:    \
    return colpass_tab_t<n>(A, Ip, h, Wcp, n_c, cpi, y_rows, waves, Y, s);
    LGB_COL_SIZES(X)
#undef X
    default:
      return LGB_ERR_UNSUPPORTED_SIZE;
  }
}

}  // namespace lgb
