// Pre-processing of the search inputs on the device: the CTF filter stack of
// an optics group, the whitening filter (radially averaged spectrum, inverted
// and normalised), the bandpass filter and the filter-and-normalise step of
// the image spectrum.  Once per micrograph, outside the orientation loop.
//
// Reference: utils/ctf_utils.py:19-116 (calculate_ctf_filter_stack),
// pydantic_models/config/correlation_filters.py:16-410 (whitening and
// bandpass filters through torch-fourier-filter), utils/image_processing.py:
// 16-75 (preprocess_image).  Frequencies are those of torch.fft.fftfreq /
// rfftfreq and numpy.fft.fftfreq (cycles per pixel): index times the FP64
// reciprocal of the length, squared and summed without contraction, so that
// the nearest-bin assignment of |k| -- which has exact ties, e.g. |k| = 97.5
// bins on a 256 x 288 grid -- rounds the way a host evaluation does.
#include <math.h>

#include "common.cuh"

namespace lgb {

__device__ __forceinline__ double fftfreq_d(int i, int n) {
  return __dmul_rn((double)(i < (n + 1) / 2 ? i : i - n), __ddiv_rn(1.0, (double)n));
}
// |k| of rfft bin (y, x) of an h x w real grid, cycles per pixel
__device__ __forceinline__ double rfft_radius(int y, int x, int h, int w) {
  const double ky = fftfreq_d(y, h), kx = __dmul_rn((double)x, __ddiv_rn(1.0, (double)w));
  return sqrt(__dadd_rn(__dmul_rn(kx, kx), __dmul_rn(ky, ky)));
}
__device__ __forceinline__ int radial_bin(double r, double fmax, int nb) {
  const double t = rint(__dmul_rn(__ddiv_rn(r, fmax), (double)(nb - 1)));
  return t < 0.0 ? 0 : (t > (double)(nb - 1) ? nb - 1 : (int)t);
}

// out[cs][df][y][x], CTF = -sin(chi) exp(-B k^2 / 4) on the d x (d/2+1) rfft
// grid at pixel size px: chi = -pi lambda k^2 df(theta) + pi/2 Cs lambda^3 k^4
// - phase - atan(A / sqrt(1 - A^2)); df(theta) = mean defocus + offset +
// astigmatism cos(2 (theta - angle)); Cs = Cs0 / ((px + off) / px)^4.
__global__ void ctf_stack_kernel(int d, double du, double dv, double ang_deg, const float* __restrict__ dfo, int D,
                                 const float* __restrict__ pxo, int C, lgb_ctf_params prm, double lambda,
                                 float* __restrict__ out) {
  const int wc = d / 2 + 1;
  const long long plane = (long long)d * wc;
  const long long n = (long long)C * D * plane;
  const double pi = 3.14159265358979323846;
  const double k5 = atan(prm.amplitude_contrast / sqrt(1.0 - prm.amplitude_contrast * prm.amplitude_contrast));
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const int xy = (int)(e % plane);
    const int df = (int)((e / plane) % D);
    const int cs = (int)(e / (plane * D));
    const int y = xy / wc, x = xy % wc;
    const double ky = fftfreq_d(y, d) / prm.pixel_size;
    const double kx = __dmul_rn((double)x, __ddiv_rn(1.0, (double)d)) / prm.pixel_size;  // rfftfreq: x >= 0
    const double k2 = kx * kx + ky * ky;
    const double ang = atan2(ky, kx);
    const double defocus = (double)dfo[df] + 0.5 * (du + dv);
    const double astig = 0.5 * fabs(du - dv);
    const double dfe = defocus + astig * cos(2.0 * (ang - ang_deg * pi / 180.0));
    const double rel = (prm.pixel_size + (double)pxo[cs]) / prm.pixel_size;
    const double csA = prm.spherical_aberration_mm / (rel * rel * rel * rel) * 1e7;
    const double chi = -pi * lambda * k2 * dfe + 0.5 * pi * csA * lambda * lambda * lambda * k2 * k2 -
                       prm.phase_shift_deg * pi / 180.0 - k5;
    out[e] = (float)(-sin(chi) * exp(-prm.b_factor * k2 / 4.0));
  }
}

// Radial sums of |F|^2 (power) or |F| per image: each thread walks a
// contiguous run of one row, where the bin index is monotone, and flushes a
// bin's partial sum to the shared histogram when the bin changes; the CTA then
// adds its histogram to the image's global one.
constexpr int kRadialThreads = 256;
constexpr int kRadialRows = 16;  // rows per CTA

__global__ void __launch_bounds__(kRadialThreads) radial_spectrum_kernel(const float2* __restrict__ F, int H, int W,
                                                                         int nb, double fmax, int power,
                                                                         double* __restrict__ sum,
                                                                         double* __restrict__ count) {
  extern __shared__ double hist[];  // [2][nb]
  const int wc = W / 2 + 1;
  const int img = blockIdx.y;
  for (int b = threadIdx.x; b < 2 * nb; b += blockDim.x) hist[b] = 0.0;
  __syncthreads();
  const float2* f = F + (size_t)img * H * wc;
  const int per = (wc + blockDim.x - 1) / blockDim.x;
  for (int y = blockIdx.x * kRadialRows; y < min(H, (blockIdx.x + 1) * kRadialRows); ++y) {
    const int x0 = threadIdx.x * per, x1 = min(wc, x0 + per);
    int cur = -1;
    double acc = 0.0, cnt = 0.0;
    for (int x = x0; x < x1; ++x) {
      const int bin = radial_bin(rfft_radius(y, x, H, W), fmax, nb);
      const float2 v = f[(size_t)y * wc + x];
      const double m = (double)hypotf(v.x, v.y);
      if (bin != cur) {
        if (cur >= 0) {
          atomicAdd(&hist[cur], acc);
          atomicAdd(&hist[nb + cur], cnt);
        }
        cur = bin;
        acc = 0.0;
        cnt = 0.0;
      }
      acc += power ? m * m : m;
      cnt += 1.0;
    }
    if (cur >= 0) {
      atomicAdd(&hist[cur], acc);
      atomicAdd(&hist[nb + cur], cnt);
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    if (hist[nb + b] != 0.0) {
      atomicAdd(&sum[(size_t)img * nb + b], hist[b]);
      atomicAdd(&count[(size_t)img * nb + b], hist[nb + b]);
    }
  }
}

// One CTA per image: spectrum = sum / max(count, 1) (square root for power),
// filter = 1 / spectrum where positive else 0, normalised to its maximum.
// Written over `sum` (FP64).
__global__ void whitening_curve_kernel(int nb, int power, double* __restrict__ sum, const double* __restrict__ count) {
  __shared__ double red[32];
  double* s = sum + (size_t)blockIdx.x * nb;
  const double* c = count + (size_t)blockIdx.x * nb;
  double mx = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    double spec = s[b] / fmax(c[b], 1.0);
    if (power) spec = sqrt(spec);
    const double f = spec > 0.0 ? 1.0 / spec : 0.0;
    s[b] = f;
    mx = fmax(mx, f);
  }
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x + 31) / 32 ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (threadIdx.x == 0) red[0] = v;
  }
  __syncthreads();
  const double m = red[0];
  for (int b = threadIdx.x; b < nb; b += blockDim.x) s[b] = m > 0.0 ? s[b] / m : s[b];
}

// out[img][y][x] = curve[img][bin of |k| on the out_h x out_w rfft grid]
__global__ void radial_map_kernel(int n_img, int nb, double fmax, const double* __restrict__ curve, int h, int w,
                                  float* __restrict__ out) {
  const int wc = w / 2 + 1;
  const long long plane = (long long)h * wc;
  const long long n = plane * n_img;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const int img = (int)(e / plane);
    const int xy = (int)(e % plane);
    out[e] = (float)curve[(size_t)img * nb + radial_bin(rfft_radius(xy / wc, xy % wc, h, w), fmax, nb)];
  }
}

// Band [lo, hi] cycles/pixel with raised-cosine edges of width fo (hard band for fo = 0).
__global__ void bandpass_kernel(int h, int w, double lo, double hi, double fo, float* __restrict__ out) {
  const int wc = w / 2 + 1;
  const long long n = (long long)h * wc;
  const double pi = 3.14159265358979323846;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const double r = rfft_radius((int)(e / wc), (int)(e % wc), h, w);
    double f;
    if (fo > 0.0) {
      f = 1.0;
      if (r < lo) f = 0.5 * (1.0 + cos(pi * fmin(fmax((lo - r) / fo, 0.0), 1.0)));
      if (r > hi) f = 0.5 * (1.0 + cos(pi * fmin(fmax((r - hi) / fo, 0.0), 1.0)));
    } else {
      f = (r >= lo && r <= hi) ? 1.0 : 0.0;
    }
    out[e] = (float)f;
  }
}

// Pass 1 of preprocess_image: per image sum over the filtered spectrum of
// |F f|^2 with the interior rfft columns counted twice; blockIdx.y = image
// (image == n_img: the same weighted sum of the bandpass filter).
__global__ void filtered_power_kernel(const float2* __restrict__ F, int H, int wc, const float* __restrict__ filt,
                                      long long filt_stride, const float* __restrict__ band, int n_img,
                                      double* __restrict__ acc) {
  __shared__ double red[32];
  const int img = blockIdx.y;
  const long long plane = (long long)H * wc;
  double s = 0.0;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < plane; e += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(e % wc);
    const double wgt = (x == 0 || x == wc - 1) ? 1.0 : 2.0;
    if (img < n_img) {
      const float2 v = F[(size_t)img * plane + e];
      const float g = filt[(size_t)img * filt_stride + e];
      const float a = hypotf(v.x * g, v.y * g);
      s += wgt * (double)(a * a);
    } else {
      s += wgt * (double)band[e];
    }
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x + 31) / 32 ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) atomicAdd(&acc[img], v);
  }
}

// Pass 2: out = F f / sqrt(power) * sqrt(dimensionality) * sqrt(area ratio).
__global__ void normalise_spectrum_kernel(const float2* __restrict__ F, int H, int wc, const float* __restrict__ filt,
                                          long long filt_stride, int n_img, const double* __restrict__ acc,
                                          double area_ratio, float2* __restrict__ out) {
  const long long plane = (long long)H * wc;
  const long long n = plane * n_img;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const int img = (int)(e / plane);
    const long long xy = e % plane;
    const float g = filt[(size_t)img * filt_stride + xy];
    const float2 v = F[e];
    const float sc = (float)(sqrt(acc[n_img]) * sqrt(area_ratio) / sqrt(acc[img]));
    out[e] = make_float2(v.x * g * sc, v.y * g * sc);
  }
}

static int grid_for_pp(long long n) {
  long long g = (n + 255) / 256;
  if (g > 65535LL * 16) g = 65535LL * 16;
  return (int)(g < 1 ? 1 : g);
}

static double electron_wavelength_pp(double kv) {
  const double v = kv * 1e3, h = 6.62607015e-34, m0 = 9.1093837015e-31, e = 1.602176634e-19, c = 299792458.0;
  return h / sqrt(2 * m0 * e * v * (1 + e * v / (2 * m0 * c * c))) * 1e10;
}

}  // namespace lgb

using namespace lgb;

extern "C" {

int lgb_ctf_filter_stack(int template_size, double defocus_u, double defocus_v, double astigmatism_angle_deg,
                         const lgb_ctf_params* ctf, const float* defocus_offsets, int n_defocus,
                         const float* pixel_size_offsets, int n_pixel_sizes, float* out, void* stream) {
  if (template_size < 2 || !ctf || !defocus_offsets || n_defocus < 1 || !pixel_size_offsets || n_pixel_sizes < 1 ||
      !out || ctf->pixel_size <= 0.0 || ctf->voltage_kv <= 0.0 || ctf->amplitude_contrast < 0.0 ||
      ctf->amplitude_contrast >= 1.0)
    return LGB_ERR_INVALID_ARGUMENT;
  const long long n = (long long)n_pixel_sizes * n_defocus * template_size * (template_size / 2 + 1);
  ctf_stack_kernel<<<grid_for_pp(n), 256, 0, (cudaStream_t)stream>>>(
      template_size, defocus_u, defocus_v, astigmatism_angle_deg, defocus_offsets, n_defocus, pixel_size_offsets,
      n_pixel_sizes, *ctf, electron_wavelength_pp(ctf->voltage_kv), out);
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

int lgb_radial_spectrum(int n_images, int image_h, int image_w, const void* image_dft, int n_bins, double max_freq,
                        int power, double* bin_sum, double* bin_count, void* stream) {
  if (n_images < 1 || image_h < 1 || image_w < 2 || (image_w % 2) || !image_dft || n_bins < 2 ||
      n_bins > 8192 || !(max_freq > 0.0) || !bin_sum || !bin_count)
    return LGB_ERR_INVALID_ARGUMENT;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemsetAsync(bin_sum, 0, sizeof(double) * (size_t)n_images * n_bins, s) != cudaSuccess ||
      cudaMemsetAsync(bin_count, 0, sizeof(double) * (size_t)n_images * n_bins, s) != cudaSuccess)
    return LGB_ERR_CUDA;
  const size_t smem = sizeof(double) * 2 * (size_t)n_bins;
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(radial_spectrum_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
          cudaSuccess)
    return LGB_ERR_CUDA;
  dim3 grid((image_h + kRadialRows - 1) / kRadialRows, n_images);
  radial_spectrum_kernel<<<grid, kRadialThreads, smem, s>>>(static_cast<const float2*>(image_dft), image_h, image_w,
                                                            n_bins, max_freq, power, bin_sum, bin_count);
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

int lgb_whitening_filter(int n_images, int n_bins, double max_freq, int power, double* bin_sum,
                         const double* bin_count, int out_h, int out_w, float* out, void* stream) {
  if (n_images < 1 || n_bins < 2 || !(max_freq > 0.0) || !bin_sum || !bin_count || out_h < 1 || out_w < 2 ||
      (out_w % 2) || !out)
    return LGB_ERR_INVALID_ARGUMENT;
  cudaStream_t s = (cudaStream_t)stream;
  whitening_curve_kernel<<<n_images, 256, 0, s>>>(n_bins, power, bin_sum, bin_count);
  if (cudaGetLastError() != cudaSuccess) return LGB_ERR_CUDA;
  const long long n = (long long)n_images * out_h * (out_w / 2 + 1);
  radial_map_kernel<<<grid_for_pp(n), 256, 0, s>>>(n_images, n_bins, max_freq, bin_sum, out_h, out_w, out);
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

int lgb_bandpass_filter(int h, int w, double low, double high, double falloff, float* out, void* stream) {
  if (h < 1 || w < 2 || (w % 2) || !out || falloff < 0.0) return LGB_ERR_INVALID_ARGUMENT;
  bandpass_kernel<<<grid_for_pp((long long)h * (w / 2 + 1)), 256, 0, (cudaStream_t)stream>>>(h, w, low, high,
                                                                                            falloff, out);
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

int lgb_preprocess_image(int n_images, int image_h, int image_w, const void* image_dft, const float* filters,
                         long long filter_stride, const float* bandpass, double area_ratio, double* scratch,
                         void* out, void* stream) {
  if (n_images < 1 || image_h < 1 || image_w < 2 || (image_w % 2) || !image_dft || !filters || filter_stride < 0 ||
      !bandpass || !(area_ratio > 0.0) || !scratch || !out)
    return LGB_ERR_INVALID_ARGUMENT;
  cudaStream_t s = (cudaStream_t)stream;
  const int wc = image_w / 2 + 1;
  if (cudaMemsetAsync(scratch, 0, sizeof(double) * (size_t)(n_images + 1), s) != cudaSuccess) return LGB_ERR_CUDA;
  const long long plane = (long long)image_h * wc;
  int bx = (int)((plane + 255) / 256);
  if (bx > 1024) bx = 1024;
  filtered_power_kernel<<<dim3(bx, n_images + 1), 256, 0, s>>>(static_cast<const float2*>(image_dft), image_h, wc,
                                                               filters, filter_stride, bandpass, n_images, scratch);
  if (cudaGetLastError() != cudaSuccess) return LGB_ERR_CUDA;
  normalise_spectrum_kernel<<<grid_for_pp(plane * n_images), 256, 0, s>>>(
      static_cast<const float2*>(image_dft), image_h, wc, filters, filter_stride, n_images, scratch, area_ratio,
      static_cast<float2*>(out));
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

}  // extern "C"
