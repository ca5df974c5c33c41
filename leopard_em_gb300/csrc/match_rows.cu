// Launchers: zero-padded projection rfft and the row c2r + statistics pass
// (image width W).
#include "match_fused.cuh"
#include "match_kernels.cuh"
#include "match_launch.h"

namespace lgb {

// One warp per correlogram: the normalisation constants (edge mean e, scale
// s) from the h row moments, stored as a float2 over rowstats[c][0][0] (row
// 0's moments are not needed afterwards), so that every pad_rfft or column
// pass CTA reads them instead of reducing all rows again.
__global__ void norm_constants_kernel(double* __restrict__ rowstats, int n_c, int h, int norm_h, int norm_w) {
  const int c = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  if (c >= n_c) return;
  double* rs = rowstats + (size_t)c * h * 3;
  float e = 0.f, s = 0.f;
  projection_norm_constants(rs, h, norm_h, norm_w, &e, &s);
  __syncwarp();
  if ((threadIdx.x & 31) == 0) *reinterpret_cast<float2*>(rs) = make_float2(e, s);
}

int launch_norm_constants(double* rowstats, int n_c, int h, int norm_h, int norm_w, cudaStream_t s) {
  norm_constants_kernel<<<(n_c + 7) / 8, 256, 0, s>>>(rowstats, n_c, h, norm_h, norm_w);
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}


// W/2 values
#define LGB_ROW_SIZES(X) \
  X(24) X(32) X(40) X(64) X(128) X(144) X(256) X(288) X(512) X(1024) X(1440) X(1536) X(1920) X(2048) X(2880)

bool supported_row(int W) {
  if (W % 2) return false;
  switch (W / 2) {
#define X(n) case n:
    LGB_ROW_SIZES(X)
#undef X
    return true;
    default:
      return false;
  }
}

template <int WH>
static int pad_rfft_t(const float* proj, const double* rowstats, int h, int norm_h, int norm_w, int Wcp, int n_c,
                      void* A, cudaStream_t s) {
  constexpr int NT = FftThreads<WH>::value;
  if constexpr (WH >= 1024) {
    // long rows: tables in dynamic shared memory, 32 rows per CTA, constants precomputed
    constexpr int ROWS = 2, RPC = 32;
    using PR = PadRows<WH, ROWS>;
    int st = launch_norm_constants(const_cast<double*>(rowstats), n_c, h, norm_h, norm_w, s);
    if (st) return st;
    if (cudaFuncSetAttribute(pad_rfft_rows_kernel<WH, ROWS, RPC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)PR::SMEM) != cudaSuccess)
      return LGB_ERR_CUDA;
    pad_rfft_rows_kernel<WH, ROWS, RPC><<<dim3((h + RPC - 1) / RPC, n_c), ROWS * NT, PR::SMEM, s>>>(
        proj, rowstats, h, Wcp, static_cast<float2*>(A));
    return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
  } else {
    // at least one full warp: the normalisation reduction shuffles across warp 0
    constexpr int ROWS0 = NT >= 128 ? 2 : (NT >= 32 ? 4 : (NT >= 16 ? 8 : 16));
    constexpr int ROWS1 = ROWS0 * NT >= 32 ? ROWS0 : (32 + NT - 1) / NT;
    // static shared memory (ROWS rows of the padded transform) stays under 40 KB
    constexpr int ROWS = ROWS1 * (IdxPad16::pad(WH) + 2) * 8 <= 40960 ? ROWS1 : 1;
    static_assert(ROWS * NT >= 32, "pad_rfft CTA must hold a full warp");
    const int ctas = (h + ROWS - 1) / ROWS;
    // precompute the constants when many CTAs share a correlogram (each would
    // otherwise reduce all h rows in FP64); a few CTAs do it themselves
    const int ready = ctas >= 16;
    if (ready) {
      const int st = launch_norm_constants(const_cast<double*>(rowstats), n_c, h, norm_h, norm_w, s);
      if (st) return st;
    }
    dim3 grid(ctas, n_c);
    // shared twiddle tables where a CTA transforms >= 4 rows
    pad_rfft_kernel<WH, ROWS, (ROWS >= 4)><<<grid, ROWS * NT, 0, s>>>(proj, rowstats, h, norm_h, norm_w, Wcp,
                                                                      ready, static_cast<float2*>(A));
    return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
  }
}

template <int WH>
static int rowpass_t(const void* Y, int H, int y_rows, int Wcp, int n_c, int nb, int n_orient, int o0,
                     const int* o0_dev, float* mip, int* best, double* s1, double* s2, cudaStream_t s) {
  constexpr int NT = row_threads(WH);
  constexpr size_t SMEM = RowGeneric<WH>::SMEM;
  if (cudaFuncSetAttribute(rowpass_kernel<WH, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM) !=
      cudaSuccess)
    return LGB_ERR_CUDA;
  const float scale = 1.0f / ((float)H * (float)(2 * WH));
  rowpass_kernel<WH, NT><<<y_rows, NT, SMEM, s>>>(static_cast<const float2*>(Y), y_rows, Wcp, n_c, nb, n_orient,
                                                  o0, o0_dev, scale, mip, best, s1, s2);
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

int launch_pad_rfft(int W, const float* proj, const double* rowstats, int h, int norm_h, int norm_w, int Wcp,
                    int n_c, void* A, cudaStream_t s) {
  if (W % 2 || norm_w > W || norm_w < h || norm_h < h) return LGB_ERR_UNSUPPORTED_SIZE;
  if (!supported_row(W)) return LGB_ERR_UNSUPPORTED_SIZE;
  switch (W / 2) {
#define X(n) \
  case n:    \
    return pad_rfft_t<n>(proj, rowstats, h, norm_h, norm_w, Wcp, n_c, A, s);
    LGB_ROW_SIZES(X)
#undef X
    default:
      return LGB_ERR_UNSUPPORTED_SIZE;
  }
}

template <int WH, int NT, class RL, int MINB = 3>
static int rowpass_fused_t(const void* Y, int H, int y_rows, int Wcp, int n_c, int nb, int n_orient, int o0,
                           const int* o0_dev, float* mip, int* best, double* s1, double* s2, cudaStream_t s) {
  using RF = RowFused<WH, NT, RL>;
  if (n_c > 0xffff) return LGB_ERR_INVALID_ARGUMENT;  // batch indices are kept in 16 bits
  const size_t smem = RF::smem(Wcp);
  if (cudaFuncSetAttribute(rowpass_fused_kernel<WH, NT, RL, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess ||
      cudaFuncSetAttribute(rowpass_fused_kernel<WH, NT, RL, MINB>, cudaFuncAttributePreferredSharedMemoryCarveout,
                           cudaSharedmemCarveoutMaxShared) != cudaSuccess)
    return LGB_ERR_CUDA;
  const float scale = 1.0f / ((float)H * (float)(2 * WH));
  rowpass_fused_kernel<WH, NT, RL, MINB><<<y_rows, NT, smem, s>>>(static_cast<const float2*>(Y), y_rows, Wcp, n_c, nb,
                                                            n_orient, o0, o0_dev, scale, mip, best, s1, s2);
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

int launch_rowpass(int W, const void* Y, int H, int y_rows, int Wcp, int n_c, int nb, int n_orient, int o0,
                   const int* o0_dev, float* mip, int* best, double* s1, double* s2, cudaStream_t s) {
  if (W % 2 || y_rows < 1 || y_rows > H) return LGB_ERR_INVALID_ARGUMENT;
  switch (W / 2) {
    case 2048:
      return rowpass_fused_t<2048, 256, Radices<8, 8, 8, 4>>(Y, H, y_rows, Wcp, n_c, nb, n_orient, o0, o0_dev, mip,
                                                             best, s1, s2, s);
    case 2880:  // 5760-wide grids (e.g. a 5760 x 4092 micrograph searched transposed): one CTA per SM at
                // 157 registers without spills (two CTAs at 80 registers spill 324 B and run 9 % slower)
      return rowpass_fused_t<2880, 360, Radices<8, 9, 5, 8>, 1>(Y, H, y_rows, Wcp, n_c, nb, n_orient, o0, o0_dev,
                                                                mip, best, s1, s2, s);
    case 1024:
      return rowpass_fused_t<1024, 256, Radices<8, 8, 4, 4>>(Y, H, y_rows, Wcp, n_c, nb, n_orient, o0, o0_dev, mip,
                                                             best, s1, s2, s);
    case 256:
      return rowpass_fused_t<256, 64, Radices<8, 8, 4>>(Y, H, y_rows, Wcp, n_c, nb, n_orient, o0, o0_dev, mip, best,
                                                        s1, s2, s);
    default:
      break;
  }
  switch (W / 2) {
#define X(n) \
  case n:    \
    return rowpass_t<n>(Y, H, y_rows, Wcp, n_c, nb, n_orient, o0, o0_dev, mip, best, s1, s2, s);
    LGB_ROW_SIZES(X)
#undef X
    default:
      return LGB_ERR_UNSUPPORTED_SIZE;
  }
}

}  // namespace lgb
