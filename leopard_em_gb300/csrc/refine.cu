// Plain local-grid refinement (Leopard-EM core_refine_template) on the GPU.
//
// One call refines P particles over K Euler-angle offsets x D defocus offsets
// x C pixel-size offsets.  Per offset batch (B offsets, n_cpp = C*D*B
// correlograms per particle, c = (cs*D + df)*B + b):
//   refine_rotations_kernel  R = R(offset) @ R(particle)            (FP64)
//   slice / proj_col / proj_row / pad_rfft / colpass                (shared with the search;
//                            288^2 crops with d = 256: proj_row + pad_rfft fused, the
//                            normalisation applied by the column pass)
//   refine_rowpass_kernel    rows y < crop_h only: c2r, valid crop, z = (cc - mean)/std,
//   (_pair for W = 288)      packed (z, pixel-major flat index) arg-max and max cc per particle
//   refine_commit_kernel     strict '>' against the particle's best so far
// The filters (per-particle projective filter x CTF stack with B envelope) are
// built once per call by refine_filters_kernel.
// Reference: backend/core_refine_template.py:555-767, utils/ctf_utils.py:19-116.
#include <math.h>

#include "profiler.h"
#include "match_kernels.cuh"
#include "match_launch.h"

namespace lgb {

__device__ inline void euler_zyz_d(const float* e, double* R) {
  const double k = 3.14159265358979323846 / 180.0;
  double sp, cp, st, ct, ss, cs;
  sincos((double)e[0] * k, &sp, &cp);
  sincos((double)e[1] * k, &st, &ct);
  sincos((double)e[2] * k, &ss, &cs);
  R[0] = cp * ct * cs - sp * ss;
  R[1] = -cp * ct * ss - sp * cs;
  R[2] = cp * st;
  R[3] = sp * ct * cs + cp * ss;
  R[4] = -sp * ct * ss + cp * cs;
  R[5] = sp * st;
  R[6] = -st * cs;
  R[7] = st * ss;
  R[8] = ct;
}

// rot[(p*nb + b)*9] = R(offsets[o0 + b]) @ R(euler[p])
__global__ void refine_rotations_kernel(const float* __restrict__ euler, const float* __restrict__ offsets, int o0,
                                        int nb, int n_particles, float* __restrict__ rot) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_particles * nb) return;
  const int p = i / nb, b = i % nb;
  double A[9], B[9];
  euler_zyz_d(offsets + 3 * (size_t)(o0 + b), A);
  euler_zyz_d(euler + 3 * (size_t)p, B);
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c)
      rot[9 * (size_t)i + 3 * r + c] = (float)(A[3 * r] * B[c] + A[3 * r + 1] * B[3 + c] + A[3 * r + 2] * B[6 + c]);
}

// out[p][cs][df][y][x] = pf[p][y][x] * CTF(p, cs, df; y, x) * exp(-B k^2 / 4)
// CTF = -sin(chi), chi = -pi lambda k^2 df(theta) + pi/2 Cs lambda^3 k^4 - phase - atan(A / sqrt(1 - A^2)),
// df(theta) = defocus + astig cos(2 (theta - angle)), Cs = Cs0 / ((px + off)/px)^4.
// The phase is a polynomial in (kx, ky) evaluated in FP64 without transcendental
// calls: k^2 cos(2 (theta - a)) = (kx^2 - ky^2) cos 2a + 2 kx ky sin 2a.  It is
// reduced to [-pi, pi] in FP64 and its sine (and the B envelope) taken in FP32,
// which keeps the FP64 phase accuracy at a small fraction of the cost of FP64
// atan2 / cos / sin / exp per filter element.
__global__ void refine_filters_kernel(const float* __restrict__ pf, const float* __restrict__ du,
                                      const float* __restrict__ dv, const float* __restrict__ dang,
                                      const float* __restrict__ dfo, const float* __restrict__ pxo, int P, int C,
                                      int D, int d, lgb_ctf_params prm, double lambda, float* __restrict__ out) {
  const int wc = d / 2 + 1;
  const long long plane = (long long)d * wc;
  const long long n = (long long)P * C * D * plane;
  const double pi = 3.14159265358979323846;
  const double k5 = atan(prm.amplitude_contrast / sqrt(1.0 - prm.amplitude_contrast * prm.amplitude_contrast));
  const double phase0 = prm.phase_shift_deg * pi / 180.0 + k5;
  const double lam3 = lambda * lambda * lambda;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const int xy = (int)(e % plane);
    const long long r = e / plane;
    const int df = (int)(r % D);
    const int cs = (int)((r / D) % C);
    const int p = (int)(r / ((long long)D * C));
    const int y = xy / wc, x = xy % wc;
    const double ky = (double)(y < (d + 1) / 2 ? y : y - d) / d / prm.pixel_size;
    const double kx = (double)x / d / prm.pixel_size;
    const double k2 = kx * kx + ky * ky;
    float s2a, c2a;  // 2 * angle, in units of pi: angle / 90
    sincospif(dang[p] / 90.0f, &s2a, &c2a);
    const double defocus = (double)dfo[df] + 0.5 * ((double)du[p] + (double)dv[p]);
    const double astig = 0.5 * fabs((double)du[p] - (double)dv[p]);
    const double dfk2 = defocus * k2 + astig * ((kx * kx - ky * ky) * (double)c2a + 2.0 * kx * ky * (double)s2a);
    const double rel = ((double)prm.pixel_size + (double)pxo[cs]) / prm.pixel_size;
    const double csA = prm.spherical_aberration_mm / (rel * rel * rel * rel) * 1e7;
    const double chi = -pi * lambda * dfk2 + 0.5 * pi * csA * lam3 * k2 * k2 - phase0;
    const double red = chi - 2.0 * pi * rint(chi / (2.0 * pi));
    const float ctf = -sinf((float)red);
    const float env = expf((float)(-prm.b_factor * k2 / 4.0));
    out[e] = pf[(size_t)p * plane + xy] * (ctf * env);
  }
}

__device__ __forceinline__ unsigned ord_f(float f) {
  const unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float unord_f(unsigned u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// Row y (< crop_h) of every correlogram of particle p = blockIdx.y.  The packed
// key is (ordered z) << 32 | ~flat with flat = (y*crop_w + x)*n_cpp + c, so the
// largest key is the largest z and, among equal z, the first pixel in
// row-major order and then the first correlogram: the order in which the
// reference's torch.max over correlograms and then over pixels resolves ties.
template <int WH, int NT>
__global__ void __launch_bounds__(NT)
    refine_rowpass_kernel(const float2* __restrict__ Y, int y_rows, int Wcp, int n_cpp, int c_per_block,
                          int crop_w, float scale, const float* __restrict__ corr_mean,
                          const float* __restrict__ corr_std, int crop_h, unsigned long long* __restrict__ slot_key,
                          unsigned* __restrict__ slot_cc) {
  constexpr int ZS = IdxPad16::pad(WH) + 2;
  __shared__ float2 xr[WH + 4];
  __shared__ float2 z[ZS];
  // c2r pre-twiddles and FFT twiddles, filled once and reused by every correlogram
  __shared__ float2 pre[WH];
  __shared__ float2 tab[FftTable<WH>::SIZE + 1];
  __shared__ unsigned long long red_key[1];
  __shared__ unsigned red_cc[1];
  const int y = blockIdx.x, p = blockIdx.y, t = threadIdx.x;
  fill_fft_table<WH>(tab, t, NT);
  for (int k = t; k < WH; k += NT) {
    float sn, cs;
    sincospif((float)k / (float)WH, &sn, &cs);
    pre[k] = make_float2(cs, sn);
  }
  unsigned long long best_key = 0ull;
  unsigned best_cc = 0u;
  const float* mrow = corr_mean + ((size_t)p * crop_h + y) * crop_w;
  const float* srow = corr_std + ((size_t)p * crop_h + y) * crop_w;
  // this CTA's share of the particle's correlograms (blockIdx.z); the slots
  // combine the shares with atomicMax
  const int c_begin = blockIdx.z * c_per_block;
  const int c_end = min(n_cpp, c_begin + c_per_block);
  for (int c = c_begin; c < c_end; ++c) {
    const float2* row = Y + (((size_t)p * n_cpp + c) * y_rows + y) * Wcp;
    for (int k = t; k <= WH; k += NT) xr[k] = row[k];
    __syncthreads();
    for (int k = t; k < WH; k += NT) {
      float2 A = xr[k];
      float2 B = xr[WH - k];
      if (k == 0) { A.y = 0.f; B.y = 0.f; }
      B.y = -B.y;
      const float2 xo = cmul(csub(A, B), pre[k]);
      z[IdxPad16::f(k)] = cadd(cadd(A, B), mul_i<1>(xo));
    }
    __syncthreads();
    block_fft_tab<WH, NT, +1, IdxPad16>(z, tab, t);
    for (int m = t; 2 * m < crop_w; m += NT) {
      const float2 v = z[IdxPad16::f(m)];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int x = 2 * m + h;
        if (x >= crop_w) break;
        const float cc = (h ? v.y : v.x) * scale;
        const float zz = (cc - mrow[x]) / srow[x];
        const unsigned flat = (unsigned)((y * crop_w + x) * n_cpp + c);
        const unsigned long long key = ((unsigned long long)ord_f(zz) << 32) | (unsigned long long)(~flat);
        best_key = key > best_key ? key : best_key;
        const unsigned oc = ord_f(cc);
        best_cc = oc > best_cc ? oc : best_cc;
      }
    }
    __syncthreads();
  }
  // block reduction through shared atomics (NT need not be a multiple of 32)
  if (t == 0) {
    red_key[0] = 0ull;
    red_cc[0] = 0u;
  }
  __syncthreads();
  atomicMax(&red_key[0], best_key);
  atomicMax(&red_cc[0], best_cc);
  __syncthreads();
  if (t == 0) {
    atomicMax(slot_key + p, red_key[0]);
    atomicMax(slot_cc + p, red_cc[0]);
  }
}

// The same row pass for WH = R1*R2 (144 = 16*9) in two register passes, ROWS
// correlograms of one crop row per CTA (R1 threads each): the c2r
// pre-twiddle is applied while loading the radix-R1 inputs k = t + R2*q from
// the staged row; shared transpose M1[t][q]; radix R2 with twiddles w^(r*t)
// leaves pixel pairs m = t + R1*r in thread t.  Same keys and reduction as
// refine_rowpass_kernel.
template <int R1, int R2, int ROWS>
__global__ void __launch_bounds__(ROWS* R1, 3)
    refine_rowpass_pair_kernel(const float2* __restrict__ Y, int y_rows, int Wcp, int n_cpp, int c_per_block,
                               int crop_w, float scale, const float* __restrict__ corr_mean,
                               const float* __restrict__ corr_std, int crop_h,
                               unsigned long long* __restrict__ slot_key, unsigned* __restrict__ slot_cc) {
  constexpr int WH = R1 * R2, NT = R1, S1 = R1 + 1, NROOT = (R1 - 1) * (R2 - 1) + 1;
  static_assert(R1 >= R2, "second pass uses every thread of the row");
  // row strides 9 (mod 16) float2: the first pass packs rows two to a
  // half-warp, and this stride keeps their loads and stores conflict free
  constexpr int XS = WH + 1 + ((9 - (WH + 1) % 16) + 16) % 16;
  constexpr int ZS = R2 * S1 + ((9 - (R2 * S1) % 16) + 16) % 16;
  __shared__ float2 xr[ROWS][XS];
  __shared__ float2 zb[ROWS][ZS];
  __shared__ float2 pre[WH];      // exp(+i pi k / WH)
  __shared__ float2 root[NROOT];  // exp(+2 pi i m / WH)
  __shared__ unsigned long long red_key[1];
  __shared__ unsigned red_cc[1];
  for (int k = threadIdx.x; k < WH; k += blockDim.x) {
    float sn, cs;
    sincospif((float)k / (float)WH, &sn, &cs);
    pre[k] = make_float2(cs, sn);
  }
  for (int m = threadIdx.x; m < NROOT; m += blockDim.x) {
    float sn, cs;
    sincospif(2.0f * (float)m / (float)WH, &sn, &cs);
    root[m] = make_float2(cs, sn);
  }
  if (threadIdx.x == 0) {
    red_key[0] = 0ull;
    red_cc[0] = 0u;
  }
  const int y = blockIdx.x, p = blockIdx.y;
  const int g = threadIdx.x / NT, t = threadIdx.x - (threadIdx.x / NT) * NT;
  unsigned long long best_key = 0ull;
  unsigned best_cc = 0u;
  const float* mrow = corr_mean + ((size_t)p * crop_h + y) * crop_w;
  const float* srow = corr_std + ((size_t)p * crop_h + y) * crop_w;
  const int c_begin = blockIdx.z * c_per_block;
  const int c_end = min(n_cpp, c_begin + c_per_block);
  for (int cb = c_begin; cb < c_end; cb += ROWS) {
    const int c = cb + g;
    const bool act = c < c_end;
    __syncthreads();  // tables filled / the previous rows fully read
    if (act) {
      const float2* row = Y + (((size_t)p * n_cpp + c) * y_rows + y) * Wcp;
      for (int k = t; k <= WH; k += NT) xr[g][k] = row[k];
    }
    __syncthreads();
    // first pass: R2 (< R1) DFTs per row, the (row, DFT) tasks packed densely
    // onto the CTA's threads so that whole warps idle instead of lanes
    if (threadIdx.x < ROWS * R2 && cb + (int)threadIdx.x / R2 < c_end) {
      const int gg = threadIdx.x / R2, tt = threadIdx.x - (threadIdx.x / R2) * R2;
      float2 v[R1];
#pragma unroll
      for (int q = 0; q < R1; ++q) {
        const int k = tt + q * R2;
        float2 A = xr[gg][k];
        float2 B = xr[gg][WH - k];
        if (k == 0) { A.y = 0.f; B.y = 0.f; }
        B.y = -B.y;
        const float2 xo = cmul(csub(A, B), pre[k]);
        v[q] = cadd(cadd(A, B), mul_i<1>(xo));
      }
      Dft<R1, +1>::run(v);
#pragma unroll
      for (int q = 0; q < R1; ++q) zb[gg][tt * S1 + q] = v[q];
    }
    __syncthreads();
    if (act) {
      float2 w[R2];
#pragma unroll
      for (int r = 0; r < R2; ++r) w[r] = cmul(zb[g][r * S1 + t], root[r * t]);
      Dft<R2, +1>::run(w);
#pragma unroll
      for (int r = 0; r < R2; ++r) {
        const int m = t + r * R1;
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
          const int x = 2 * m + hh;
          if (x < crop_w) {
            const float cc = (hh ? w[r].y : w[r].x) * scale;
            const float zz = (cc - mrow[x]) / srow[x];
            const unsigned flat = (unsigned)((y * crop_w + x) * n_cpp + c);
            const unsigned long long key = ((unsigned long long)ord_f(zz) << 32) | (unsigned long long)(~flat);
            best_key = key > best_key ? key : best_key;
            const unsigned oc = ord_f(cc);
            best_cc = oc > best_cc ? oc : best_cc;
          }
        }
      }
    }
  }
  __syncthreads();
  atomicMax(&red_key[0], best_key);
  atomicMax(&red_cc[0], best_cc);
  __syncthreads();
  if (threadIdx.x == 0) {
    atomicMax(slot_key + p, red_key[0]);
    atomicMax(slot_cc + p, red_cc[0]);
  }
}

// Strict '>' update of each particle's best (core_refine_template.py:725),
// then reset of the batch slots.
__global__ void refine_commit_kernel(int P, unsigned long long* slot_key, unsigned* slot_cc, int o0, int nb,
                                     float* best_z, float* best_cc, int* best_flat, int* best_o0, int* best_nb) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  const unsigned long long key = slot_key[p];
  if (key != 0ull) {
    const float zb = unord_f((unsigned)(key >> 32));
    if (zb > best_z[p]) {
      best_z[p] = zb;
      best_cc[p] = unord_f(slot_cc[p]);
      best_flat[p] = (int)(~(unsigned)(key & 0xffffffffull));
      best_o0[p] = o0;
      best_nb[p] = nb;
    }
  }
  slot_key[p] = 0ull;
  slot_cc[p] = 0u;
}

__global__ void refine_init_kernel(int P, float* best_z, float* best_cc, int* best_flat, int* best_o0, int* best_nb,
                                   unsigned long long* slot_key, unsigned* slot_cc) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  best_z[p] = -1e9f;
  best_cc[p] = -1e9f;
  best_flat[p] = -1;
  best_o0[p] = 0;
  best_nb[p] = 1;
  slot_key[p] = 0ull;
  slot_cc[p] = 0u;
}

#define LGB_REFINE_ROW_SIZES(X) X(24) X(32) X(64) X(128) X(144) X(256)

bool supported_refine_row(int W) {
  if (W % 2) return false;
  switch (W / 2) {
#define X(n) case n:
    LGB_REFINE_ROW_SIZES(X)
#undef X
    return true;
    default:
      return false;
  }
}

template <int WH>
static int refine_rowpass_t(const void* Y, int y_rows, int Wcp, int n_cpp, int P, int crop_h, int crop_w,
                            float scale, const float* mean, const float* std_, unsigned long long* key, unsigned* cc,
                            cudaStream_t s) {
  if constexpr (WH == 144) {
    // two register passes (16 x 9), 16 correlograms per step, two steps per CTA
    constexpr int ROWS = 16;
    const int per = 2 * ROWS;
    dim3 grid(crop_h, P, (n_cpp + per - 1) / per);
    refine_rowpass_pair_kernel<16, 9, ROWS><<<grid, ROWS * 16, 0, s>>>(
        static_cast<const float2*>(Y), y_rows, Wcp, n_cpp, per, crop_w, scale, mean, std_, crop_h, key, cc);
    return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
  }
  constexpr int NT = row_threads(WH);
  // split each particle's correlograms until the grid covers ~4 waves of the SMs
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int split = 1;
  while (split < n_cpp && crop_h * P * split < 4 * sms) split *= 2;
  if (split > n_cpp) split = n_cpp;
  const int per = (n_cpp + split - 1) / split;
  split = (n_cpp + per - 1) / per;
  dim3 grid(crop_h, P, split);
  refine_rowpass_kernel<WH, NT><<<grid, NT, 0, s>>>(static_cast<const float2*>(Y), y_rows, Wcp, n_cpp, per, crop_w,
                                                    scale, mean, std_, crop_h, key, cc);
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

int launch_refine_rowpass(int W, const void* Y, int y_rows, int Wcp, int n_cpp, int P, int crop_h, int crop_w,
                          float scale, const float* mean, const float* std_, unsigned long long* key, unsigned* cc,
                          cudaStream_t s) {
  if (W % 2) return LGB_ERR_UNSUPPORTED_SIZE;
  switch (W / 2) {
#define X(n) \
  case n:    \
    return refine_rowpass_t<n>(Y, y_rows, Wcp, n_cpp, P, crop_h, crop_w, scale, mean, std_, key, cc, s);
    LGB_REFINE_ROW_SIZES(X)
#undef X
    default:
      return LGB_ERR_UNSUPPORTED_SIZE;
  }
}

struct RefineLayout {
  size_t ip, filt, rot, slices, t, proj, rowstats, a, y, key, cc, total;
  int wcp, wc_t, crop_h, crop_w, n_cd, n_c;
};

static size_t al256(size_t n) { return (n + 255) & ~(size_t)255; }

static bool valid_refine(const lgb_refine_problem* p) {
  return p && p->image_h > 0 && p->image_w > 0 && p->image_w % 2 == 0 && p->template_size > 1 &&
         p->template_size % 2 == 0 && p->template_size <= p->image_h && p->template_size <= p->image_w &&
         p->n_pixel_sizes > 0 && p->n_defocus > 0 && p->n_offsets > 0 && p->offset_batch > 0 &&
         p->n_particles > 0;
}

// 288^2 crops with a 256 template: the projection row pass and the padded
// rfft run fused (no projection buffer) and the column pass normalises
static bool refine_fused_rfft(int d, int W, int H) { return supported_proj_row_rfft(d, W) && H == 288; }

static RefineLayout refine_layout(const lgb_refine_problem* p) {
  RefineLayout L{};
  const size_t H = p->image_h, W = p->image_w, d = p->template_size, P = p->n_particles;
  L.wcp = pad4((int)(W / 2 + 1));
  L.wc_t = (int)(d / 2 + 1);
  L.crop_h = (int)(H - d + 1);
  L.crop_w = (int)(W - d + 1);
  L.n_cd = p->n_pixel_sizes * p->n_defocus;
  L.n_c = (int)P * L.n_cd * p->offset_batch;
  const size_t nc = L.n_c;
  size_t off = 0;
  L.ip = off;
  off += al256(P * H * L.wcp * sizeof(float2));
  L.filt = off;
  off += al256(P * L.n_cd * d * L.wc_t * sizeof(float));
  L.rot = off;
  off += al256(P * p->offset_batch * 9 * sizeof(float));
  L.slices = off;
  off += al256(P * p->offset_batch * d * L.wc_t * sizeof(float2));
  L.t = off;
  off += al256(nc * d * L.wc_t * sizeof(float2));
  L.proj = off;
  off += refine_fused_rfft((int)d, (int)W, (int)H) ? 0 : al256(nc * d * d * sizeof(float));
  L.rowstats = off;
  off += al256(nc * d * 3 * sizeof(double));
  L.a = off;
  off += al256(nc * d * L.wcp * sizeof(float2));
  L.y = off;
  off += al256(nc * L.crop_h * L.wcp * sizeof(float2));
  L.key = off;
  off += al256(P * sizeof(unsigned long long));
  L.cc = off;
  off += al256(P * sizeof(unsigned));
  L.total = off;
  return L;
}

__global__ void repack_stack_kernel(const float2* __restrict__ src, long long rows, int wc, int wcp,
                                    float2* __restrict__ dst) {
  const long long n = rows * wcp;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const long long y = i / wcp;
    const int k = (int)(i % wcp);
    dst[i] = k < wc ? src[y * wc + k] : make_float2(0.f, 0.f);
  }
}

static double electron_wavelength_angstrom(double kv) {
  const double v = kv * 1e3, h = 6.62607015e-34, m0 = 9.1093837015e-31, e = 1.602176634e-19, c = 299792458.0;
  return h / sqrt(2 * m0 * e * v * (1 + e * v / (2 * m0 * c * c))) * 1e10;
}

static int grid256(long long n) {
  long long g = (n + 255) / 256;
  if (g > 65535LL * 16) g = 65535LL * 16;
  return (int)(g < 1 ? 1 : g);
}

}  // namespace lgb

using namespace lgb;

extern "C" {

int lgb_refine_supported(const lgb_refine_problem* p) {
  if (!valid_refine(p)) return 0;
  return supported_template(p->template_size) && supported_row(p->image_w) && supported_col(p->image_h) &&
         supported_refine_row(p->image_w);
}

int lgb_refine_workspace_size(const lgb_refine_problem* p, size_t* bytes) {
  if (!valid_refine(p) || !bytes) return LGB_ERR_INVALID_ARGUMENT;
  *bytes = refine_layout(p).total;
  return LGB_OK;
}

int lgb_refine_search(const lgb_refine_problem* p, const lgb_ctf_params* ctf, const void* particle_stack_dft,
                      const void* template_dft, const float* euler_angles, const float* euler_offsets,
                      const float* defocus_u, const float* defocus_v, const float* defocus_angle,
                      const float* defocus_offsets, const float* pixel_size_offsets, const float* corr_mean,
                      const float* corr_std, const float* projective_filters, float* best_z, float* best_cc,
                      int* best_flat, int* best_offset_begin, int* best_batch_len, void* workspace,
                      size_t workspace_bytes, void* stream) {
  if (!valid_refine(p) || !ctf || !particle_stack_dft || !template_dft || !euler_angles || !euler_offsets ||
      !defocus_u || !defocus_v || !defocus_angle || !defocus_offsets || !pixel_size_offsets || !corr_mean ||
      !corr_std || !projective_filters || !best_z || !best_cc || !best_flat || !best_offset_begin ||
      !best_batch_len || !workspace)
    return LGB_ERR_INVALID_ARGUMENT;
  if (ctf->pixel_size <= 0.0 || ctf->voltage_kv <= 0.0 || ctf->amplitude_contrast < 0.0 ||
      ctf->amplitude_contrast >= 1.0)
    return LGB_ERR_INVALID_ARGUMENT;
  if (!lgb_refine_supported(p)) return LGB_ERR_UNSUPPORTED_SIZE;
  const RefineLayout L = refine_layout(p);
  if (workspace_bytes < L.total) return LGB_ERR_WORKSPACE_TOO_SMALL;
  if ((long long)L.crop_h * L.crop_w * (long long)L.n_cd * p->offset_batch >= 4294967295LL)
    return LGB_ERR_INVALID_ARGUMENT;  // packed flat index is 32 bits
  cudaStream_t s = (cudaStream_t)stream;
  char* ws = static_cast<char*>(workspace);
  float2* ip = reinterpret_cast<float2*>(ws + L.ip);
  float* filt = reinterpret_cast<float*>(ws + L.filt);
  float* rot = reinterpret_cast<float*>(ws + L.rot);
  void* slices = ws + L.slices;
  void* T = ws + L.t;
  float* proj = reinterpret_cast<float*>(ws + L.proj);
  double* rowstats = reinterpret_cast<double*>(ws + L.rowstats);
  void* A = ws + L.a;
  void* Y = ws + L.y;
  unsigned long long* key = reinterpret_cast<unsigned long long*>(ws + L.key);
  unsigned* cc = reinterpret_cast<unsigned*>(ws + L.cc);
  const int P = p->n_particles, H = p->image_h, W = p->image_w, d = p->template_size;
  const int C = p->n_pixel_sizes, D = p->n_defocus;

  repack_stack_kernel<<<grid256((long long)P * H * L.wcp), 256, 0, s>>>(
      static_cast<const float2*>(particle_stack_dft), (long long)P * H, W / 2 + 1, L.wcp, ip);
  refine_filters_kernel<<<grid256((long long)P * C * D * d * L.wc_t), 256, 0, s>>>(
      projective_filters, defocus_u, defocus_v, defocus_angle, defocus_offsets, pixel_size_offsets, P, C, D, d, *ctf,
      electron_wavelength_angstrom(ctf->voltage_kv), filt);
  refine_init_kernel<<<(P + 127) / 128, 128, 0, s>>>(P, best_z, best_cc, best_flat, best_offset_begin,
                                                       best_batch_len, key, cc);
  if (cudaGetLastError() != cudaSuccess) return LGB_ERR_CUDA;
  const float scale = 1.0f / ((float)H * (float)W);
  const bool prof = profiling_on();
  const bool fused_rfft = refine_fused_rfft(d, W, H);
  int st;
  for (int o0 = 0; o0 < p->n_offsets; o0 += p->offset_batch) {
    const int nb = (p->n_offsets - o0) < p->offset_batch ? (p->n_offsets - o0) : p->offset_batch;
    const int n_cpp = L.n_cd * nb;
    const int n_c = P * n_cpp;
    refine_rotations_kernel<<<(P * nb + 127) / 128, 128, 0, s>>>(euler_angles, euler_offsets, o0, nb, P, rot);
    if (cudaGetLastError() != cudaSuccess) return LGB_ERR_CUDA;
    {
      StageScope sc(LGB_STAGE_SLICE, s, prof);
      if ((st = launch_slice(template_dft, d, nullptr, 0, nullptr, P * nb, rot, slices, s))) return st;
    }
    {
      StageScope sc(LGB_STAGE_PROJ_COL, s, prof);
      if ((st = launch_proj_col(d, slices, filt, nb, L.n_cd, n_c, T, s))) return st;
    }
    if (fused_rfft) {
      // the projection stays on chip: row c2r + padded rfft of the raw row, and
      // the normalisation s (A - e U) applied by the column pass
      {
        StageScope sc(LGB_STAGE_PROJ_ROW, s, prof);
        if ((st = launch_proj_row_rfft(d, W, T, n_c, rowstats, L.wcp, A, s))) return st;
      }
      {
        StageScope sc(LGB_STAGE_PAD_RFFT, s, prof);
        if ((st = launch_norm_constants(rowstats, n_c, d, H, W, s))) return st;
      }
      {
        StageScope sc(LGB_STAGE_COLPASS, s, prof);
        // (e, s) of correlogram c: float2 at rowstats[c][0][0], d * 3 doubles apart
        if ((st = launch_colpass(H, A, ip, d, L.wcp, n_c, n_cpp, L.crop_h, 0, Y, s,
                                 reinterpret_cast<const float2*>(rowstats), d * 3, W)))
          return st;
      }
    } else {
      {
        StageScope sc(LGB_STAGE_PROJ_ROW, s, prof);
        if ((st = launch_proj_row(d, T, n_c, proj, rowstats, s))) return st;
      }
      {
        StageScope sc(LGB_STAGE_PAD_RFFT, s, prof);
        if ((st = launch_pad_rfft(W, proj, rowstats, d, H, W, L.wcp, n_c, A, s))) return st;
      }
      {
        StageScope sc(LGB_STAGE_COLPASS, s, prof);
        if ((st = launch_colpass(H, A, ip, d, L.wcp, n_c, n_cpp, L.crop_h, 0, Y, s))) return st;
      }
    }
    {
      StageScope sc(LGB_STAGE_ROWPASS, s, prof);
      if ((st = launch_refine_rowpass(W, Y, L.crop_h, L.wcp, n_cpp, P, L.crop_h, L.crop_w, scale, corr_mean,
                                      corr_std, key, cc, s)))
        return st;
    }
    refine_commit_kernel<<<(P + 127) / 128, 128, 0, s>>>(P, key, cc, o0, nb, best_z, best_cc, best_flat,
                                                           best_offset_begin, best_batch_len);
    if (cudaGetLastError() != cudaSuccess) return LGB_ERR_CUDA;
  }
  return LGB_OK;
}

}  // extern "C"
