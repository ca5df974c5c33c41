// Cross-correlation of a particle stack with one template projection per
// particle (backend/core_refine_template.py:771-895,
// cross_correlate_particle_stack): per particle, the Fourier slice at its
// rotation times its projective filter, irfft2, ifftshift, the padded-variance
// normalisation, the padded rfft, particle * conj(projection) and irfft2,
// returned whole ("same") or cropped to the valid positions ("valid",
// utils/cross_correlation.py:8-40).  Unlike the search, the DC bin of the
// projection is not zeroed here; the column pass (shared with the search)
// zeroes it, and the row kernel adds the DC term back:
// Re(I[0,0] conj(P[0,0])) / (H W), with P[0,0] = sum over the projection rows
// of their rfft DC bins.
#include "match_kernels.cuh"
#include "match_launch.h"

namespace lgb {

__global__ void repack_stack_kernel(const float2* __restrict__ src, long long n_particles, int H, int wc, int wcp,
                                    float2* __restrict__ dst) {
  const long long n = n_particles * H * wcp;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const long long row = i / wcp;
    const int k = (int)(i - row * wcp);
    dst[i] = k < wc ? src[row * wc + k] : make_float2(0.f, 0.f);
  }
}

// one warp per particle: offset[p] = Re(I00 * conj(P00)) * scale
__global__ void dc_offset_kernel(int n_particles, int H, int d, int wcp, const float2* __restrict__ Ip,
                                 const float2* __restrict__ A, float scale, float* __restrict__ offset) {
  const int p = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (p >= n_particles) return;
  double pr = 0.0, pi = 0.0;
  for (int y = lane; y < d; y += 32) {
    const float2 a = A[((size_t)p * d + y) * wcp];
    pr += a.x;
    pi += a.y;
  }
  for (int o = 16; o > 0; o >>= 1) {
    pr += __shfl_down_sync(0xffffffffu, pr, o);
    pi += __shfl_down_sync(0xffffffffu, pi, o);
  }
  if (lane == 0) {
    const float2 I = Ip[(size_t)p * H * wcp];
    offset[p] = (float)(((double)I.x * pr + (double)I.y * pi) * (double)scale);
  }
}

// row y of particle p: c2r of length W = 2*WH, scale, DC term, crop
template <int WH, int NT>
__global__ void __launch_bounds__(NT) rowstore_kernel(const float2* __restrict__ Y, int y_rows, int Wcp, float scale,
                                                      const float* __restrict__ offset, int out_w,
                                                      float* __restrict__ out) {
  constexpr int ZS = IdxPad16::pad(WH) + 2;
  __shared__ float2 xr[WH + 4];
  __shared__ float2 z[ZS];
  const int y = blockIdx.x, p = blockIdx.y, t = threadIdx.x;
  const float2* row = Y + ((size_t)p * y_rows + y) * Wcp;
  for (int k = t; k <= WH; k += NT) xr[k] = row[k];
  __syncthreads();
  for (int k = t; k < WH; k += NT) {
    float2 A = xr[k];
    float2 B = xr[WH - k];
    if (k == 0) {
      A.y = 0.f;
      B.y = 0.f;
    }
    B.y = -B.y;
    const float2 xe = cadd(A, B);
    float sn, cs;
    sincospif((float)k / (float)WH, &sn, &cs);
    const float2 xo = cmul(csub(A, B), make_float2(cs, sn));
    z[IdxPad16::f(k)] = cadd(xe, mul_i<1>(xo));
  }
  __syncthreads();
  block_fft_outline<WH, NT, +1, IdxPad16>(z, t);
  const float off = offset[p];
  float* o = out + ((size_t)p * y_rows + y) * out_w;
  for (int m = t; m < WH; m += NT) {
    const float2 v = z[IdxPad16::f(m)];
    if (2 * m < out_w) o[2 * m] = fmaf(v.x, scale, off);
    if (2 * m + 1 < out_w) o[2 * m + 1] = fmaf(v.y, scale, off);
  }
}

#define LGB_XCORR_ROWS(X) X(24) X(32) X(40) X(64) X(128) X(144) X(256) X(288) X(512) X(1024) X(2048)

static bool xcorr_row_supported(int W) {
  if (W % 2) return false;
  switch (W / 2) {
#define X(n) case n:
    LGB_XCORR_ROWS(X)
#undef X
    return true;
    default:
      return false;
  }
}

template <int WH>
static int rowstore_t(const void* Y, int y_rows, int Wcp, int P, float scale, const float* off, int out_w, float* out,
                      cudaStream_t s) {
  constexpr int NT = row_threads(WH) > FftThreads<WH>::value ? row_threads(WH) : FftThreads<WH>::value;
  rowstore_kernel<WH, NT><<<dim3(y_rows, P), NT, 0, s>>>(static_cast<const float2*>(Y), y_rows, Wcp, scale, off,
                                                         out_w, out);
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

static int launch_rowstore(int W, const void* Y, int y_rows, int Wcp, int P, float scale, const float* off, int out_w,
                           float* out, cudaStream_t s) {
  switch (W / 2) {
#define X(n) \
  case n:    \
    return rowstore_t<n>(Y, y_rows, Wcp, P, scale, off, out_w, out, s);
    LGB_XCORR_ROWS(X)
#undef X
    default:
      return LGB_ERR_UNSUPPORTED_SIZE;
  }
}

struct XcorrLayout {
  size_t ip, slices, t, proj, rowstats, a, y, off, total;
  int wc, wcp, wc_t, out_h, out_w;
};

static size_t al256(size_t n) { return (n + 255) & ~(size_t)255; }

static XcorrLayout xcorr_layout(int G, int H, int W, int d, int mode) {
  XcorrLayout L{};
  L.wc = W / 2 + 1;
  L.wcp = pad4(L.wc);
  L.wc_t = d / 2 + 1;
  L.out_h = mode == 0 ? H - d + 1 : H;
  L.out_w = mode == 0 ? W - d + 1 : W;
  size_t off = 0;
  L.ip = off; off += al256((size_t)G * H * L.wcp * sizeof(float2));
  L.slices = off; off += al256((size_t)G * d * L.wc_t * sizeof(float2));
  L.t = off; off += al256((size_t)G * d * L.wc_t * sizeof(float2));
  L.proj = off; off += al256((size_t)G * d * d * sizeof(float));
  L.rowstats = off; off += al256((size_t)G * d * 3 * sizeof(double));
  L.a = off; off += al256((size_t)G * d * L.wcp * sizeof(float2));
  L.y = off; off += al256((size_t)G * L.out_h * L.wcp * sizeof(float2));
  L.off = off; off += al256((size_t)G * sizeof(float));
  L.total = off;
  return L;
}

static bool xcorr_valid(int G, int H, int W, int d, int mode) {
  return G > 0 && H > 0 && W > 0 && d > 1 && d % 2 == 0 && d <= H && d <= W && (mode == 0 || mode == 1) &&
         supported_template(d) && supported_col(H) && supported_row(W) && xcorr_row_supported(W);
}

}  // namespace lgb

using namespace lgb;

extern "C" {

int lgb_xcorr_stack_supported(int H, int W, int d) { return xcorr_valid(1, H, W, d, 0); }

int lgb_xcorr_stack_workspace_size(int group, int H, int W, int d, int mode, size_t* bytes) {
  if (!bytes) return LGB_ERR_INVALID_ARGUMENT;
  if (!xcorr_valid(group, H, W, d, mode)) return LGB_ERR_UNSUPPORTED_SIZE;
  *bytes = xcorr_layout(group, H, W, d, mode).total;
  return LGB_OK;
}

int lgb_xcorr_stack(int n_particles, int group, int H, int W, int d, int mode, const void* particle_dft,
                    const void* template_dft, const float* rotations, const float* projective_filters, float* out,
                    void* workspace, size_t workspace_bytes, void* stream) {
  if (n_particles < 0 || !particle_dft || !template_dft || !rotations || !projective_filters || !out ||
      !workspace)
    return LGB_ERR_INVALID_ARGUMENT;
  if (!xcorr_valid(group, H, W, d, mode)) return LGB_ERR_UNSUPPORTED_SIZE;
  const XcorrLayout L = xcorr_layout(group, H, W, d, mode);
  if (workspace_bytes < L.total) return LGB_ERR_WORKSPACE_TOO_SMALL;
  cudaStream_t s = (cudaStream_t)stream;
  char* ws = static_cast<char*>(workspace);
  float2* ip = reinterpret_cast<float2*>(ws + L.ip);
  void* A = ws + L.a;
  void* Y = ws + L.y;
  float* off = reinterpret_cast<float*>(ws + L.off);
  const float scale = 1.0f / ((float)H * (float)W);
  int st;
  for (int p0 = 0; p0 < n_particles; p0 += group) {
    const int G = n_particles - p0 < group ? n_particles - p0 : group;
    const float2* src = static_cast<const float2*>(particle_dft) + (size_t)p0 * H * L.wc;
    const long long n = (long long)G * H * L.wcp;
    long long blocks = (n + 255) / 256;
    if (blocks > 65535LL * 8) blocks = 65535LL * 8;
    repack_stack_kernel<<<(int)blocks, 256, 0, s>>>(src, G, H, L.wc, L.wcp, ip);
    if (cudaGetLastError() != cudaSuccess) return LGB_ERR_CUDA;
    if ((st = launch_slice(template_dft, d, nullptr, 0, nullptr, G, rotations + (size_t)p0 * 9, ws + L.slices, s)))
      return st;
    // per particle one slice (nb = 1) and one filter (n_cd = 1): c = p
    if ((st = launch_proj_col(d, ws + L.slices, projective_filters + (size_t)p0 * d * L.wc_t, 1, 1, G, ws + L.t, s)))
      return st;
    if ((st = launch_proj_row(d, ws + L.t, G, reinterpret_cast<float*>(ws + L.proj),
                              reinterpret_cast<double*>(ws + L.rowstats), s)))
      return st;
    if ((st = launch_pad_rfft(W, reinterpret_cast<float*>(ws + L.proj), reinterpret_cast<double*>(ws + L.rowstats), d,
                              H, W, L.wcp, G, A, s)))
      return st;
    // correlogram p against particle image p (one image per correlogram)
    if ((st = launch_colpass(H, A, ip, d, L.wcp, G, 1, L.out_h, 0, Y, s))) return st;
    dc_offset_kernel<<<(G + 7) / 8, 256, 0, s>>>(G, H, d, L.wcp, ip, static_cast<const float2*>(A), scale, off);
    if (cudaGetLastError() != cudaSuccess) return LGB_ERR_CUDA;
    if ((st = launch_rowstore(W, Y, L.out_h, L.wcp, G, scale, off, L.out_w,
                              out + (size_t)p0 * L.out_h * L.out_w, s)))
      return st;
  }
  return LGB_OK;
}

}  // extern "C"
