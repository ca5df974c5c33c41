// Launchers: Fourier slice, projection column/row passes (template size h).
#include "match_kernels.cuh"
#include "match_launch.h"

namespace lgb {

// ---------------------------------------------------------------------------
// Fourier-slice extraction with trilinear interpolation.
// Output slices[b][r][kx], r in fft order (the reference's ifftshift of the
// fftshifted slice), DC set to 0, multiplied by -1.
// ---------------------------------------------------------------------------
__global__ void slice_kernel(const float2* __restrict__ vol, int d, const float* __restrict__ euler, int o0,
                             const int* __restrict__ o0_dev, const float* __restrict__ rotations,
                             float2* __restrict__ slices) {
  const int b = blockIdx.y;
  __shared__ float R[9];
  if (threadIdx.x == 0) {
    if (rotations) {
      for (int i = 0; i < 9; ++i) R[i] = rotations[9 * (size_t)b + i];
    } else {
      const int o = o0 + (o0_dev ? *o0_dev : 0) + b;
      euler_zyz_to_rotmat(euler + 3 * (size_t)o, R);
    }
  }
  __syncthreads();
  const int wc = d / 2 + 1;
  const int n_el = d * wc;
  const float fd = (float)d;
  const int half = d / 2;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n_el; e += gridDim.x * blockDim.x) {
    const int r = e / wc, kx = e - (e / wc) * wc;
    const float fy = (float)(r < (d + 1) / 2 ? r : r - d) / fd;
    const float fx = (float)kx / fd;
    float X = R[0] * fx + R[1] * fy;
    float Y = R[3] * fx + R[4] * fy;
    float Z = R[6] * fx + R[7] * fy;
    const bool cj = X < 0.f;
    if (cj) { X = -X; Y = -Y; Z = -Z; }
    const float cz = Z * fd + (float)half, cy = Y * fd + (float)half, cx = X * fd;
    float2 val = make_float2(0.f, 0.f);
    if (cz >= 0.f && cz <= (float)(d - 1) && cy >= 0.f && cy <= (float)(d - 1) && cx >= 0.f &&
        cx <= (float)(wc - 1)) {
      const int z0 = (int)floorf(cz), y0 = (int)floorf(cy), x0 = (int)floorf(cx);
      const float tz = cz - (float)z0, ty = cy - (float)y0, tx = cx - (float)x0;
      const int z1 = min(z0 + 1, d - 1), y1 = min(y0 + 1, d - 1), x1 = min(x0 + 1, wc - 1);
      const int zz[2] = {z0, z1}, yy[2] = {y0, y1}, xx[2] = {x0, x1};
      const float wz[2] = {1.f - tz, tz}, wy[2] = {1.f - ty, ty}, wx[2] = {1.f - tx, tx};
#pragma unroll
      for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int bb = 0; bb < 2; ++bb)
#pragma unroll
          for (int cc = 0; cc < 2; ++cc) {
            const float w = wz[a] * wy[bb] * wx[cc];
            const float2 s = __ldg(vol + ((size_t)zz[a] * d + yy[bb]) * wc + xx[cc]);
            val.x = fmaf(s.x, w, val.x);
            val.y = fmaf(s.y, w, val.y);
          }
    }
    if (cj) val.y = -val.y;
    if (e == 0) val = make_float2(0.f, 0.f);
    slices[(size_t)b * n_el + e] = make_float2(-val.x, -val.y);
  }
}


#define LGB_TEMPLATE_SIZES(X) X(16) X(32) X(48) X(64) X(96) X(128) X(192) X(256) X(288) X(384) X(512)

bool supported_template(int h) {
  switch (h) {
#define X(n) case n:
    LGB_TEMPLATE_SIZES(X)
#undef X
    return true;
    default:
      return false;
  }
}

int launch_slice(const void* vol, int d, const float* euler, int o0, const int* o0_dev, int nb,
                 const float* rotations, void* slices, cudaStream_t s) {
  const int n_el = d * (d / 2 + 1);
  dim3 grid((n_el + 255) / 256, nb);
  slice_kernel<<<grid, 256, 0, s>>>(static_cast<const float2*>(vol), d, euler, o0, o0_dev, rotations,
                                    static_cast<float2*>(slices));
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

constexpr int kProjCols = 8;
constexpr int kProjRows = 8;

template <int HT>
static int proj_col_t(const void* slices, const float* pf, int nb, int n_cd, int n_c, void* T, cudaStream_t s) {
  constexpr int WC = HT / 2 + 1;
  if constexpr (HT == 256) {
    // two register passes (16 x 16), 8 columns per CTA
    using PC = ProjColPair<16, 16>;
    dim3 pgrid((WC + PC::G - 1) / PC::G, n_c);
    proj_col_pair_kernel<16, 16><<<pgrid, PC::G * PC::NT, 0, s>>>(static_cast<const float2*>(slices), pf, nb, n_cd,
                                                                  static_cast<float2*>(T));
    return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
  }
  dim3 grid((WC + kProjCols - 1) / kProjCols, n_c);
  proj_col_kernel<HT, kProjCols><<<grid, kProjCols * FftThreads<HT>::value, 0, s>>>(
      static_cast<const float2*>(slices), pf, nb, n_cd, static_cast<float2*>(T));
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

template <int HT>
static int proj_row_t(const void* T, int n_c, float* proj, double* rowstats, cudaStream_t s) {
  static_assert(HT % kProjRows == 0, "rows per CTA must divide the template size");
  dim3 grid(HT / kProjRows, n_c);
  if constexpr (HT == 256) {
    // two register passes (16 x 8) of the 128-point c2r, 16 threads per row
    proj_row_pair_kernel<16, 8, kProjRows><<<grid, kProjRows * 16, 0, s>>>(static_cast<const float2*>(T), proj,
                                                                           rowstats);
    return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
  }
  proj_row_kernel<HT, kProjRows><<<grid, kProjRows * FftThreads<HT / 2>::value, 0, s>>>(
      static_cast<const float2*>(T), proj, rowstats);
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

bool supported_proj_row_rfft(int h, int W) { return h == 256 && W == 288; }

int launch_proj_row_rfft(int h, int W, const void* T, int n_c, double* rowstats, int Wcp, void* A, cudaStream_t s) {
  if (!supported_proj_row_rfft(h, W) || Wcp < W / 2 + 1) return LGB_ERR_UNSUPPORTED_SIZE;
  // 16 rows per CTA: the twiddle tables are built once per 16 rows
  proj_row_rfft_kernel<16><<<dim3(256 / 16, n_c), 16 * 16, 0, s>>>(
      static_cast<const float2*>(T), rowstats, Wcp, static_cast<float2*>(A));
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

int launch_proj_col(int h, const void* slices, const float* pf, int nb, int n_cd, int n_c, void* T, cudaStream_t s) {
  switch (h) {
#define X(n) \
  case n:    \
    return proj_col_t<n>(slices, pf, nb, n_cd, n_c, T, s);
    LGB_TEMPLATE_SIZES(X)
#undef X
    default:
      return LGB_ERR_UNSUPPORTED_SIZE;
  }
}

int launch_proj_row(int h, const void* T, int n_c, float* proj, double* rowstats, cudaStream_t s) {
  switch (h) {
#define X(n) \
  case n:    \
    return proj_row_t<n>(T, n_c, proj, rowstats, s);
    LGB_TEMPLATE_SIZES(X)
#undef X
    default:
      return LGB_ERR_UNSUPPORTED_SIZE;
  }
}

}  // namespace lgb
