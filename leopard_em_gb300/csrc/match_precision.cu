// Precision form of the whole-orientation search: the two inverse DFT stages
// of each correlogram (the column inverse transform of the cross power and
// the row c2r transform, cross_correlation.py:137-142) run as split-precision
// DFT-GEMMs on the tcgen05 tensor cores; the statistics update
// (backend/utils.py:191-255) is fused into the second GEMM's epilogue.  The
// forward half (slice, projection, normalisation, padded row rfft and the
// pruned forward column FFT with the cross power) stays FP32 on the CUDA
// cores, as do the sums (FP64 maps).
//
// Per batch of n_c correlograms (H x W grid, Wc = W/2 + 1, Wq = Wc rounded up
// to 32, n_cp = n_c rounded up to a power of two <= 32):
//
//   colfwd            X[c][ky][kx] = I[ky][kx] conj(P_c[ky][kx]) (P[0,0] = 0)
//                     written as the split operand B1: row n = c*Wq + kx,
//                     k = 2*ky + (re, im)                       [n_c*Wq, 2H]
//   GEMM 1 (tcgen05)  D1[2y + ri][n] = sum_k F1[2y + ri][k] B1[n][k]
//                     F1 = the inverse DFT exp(+2 pi i ky y / H) as a real
//                     2H x 2H matrix; the epilogue writes D1 as the split
//                     operand B2: row y*n_cp + c, k = 2*kx + ri   [H*n_cp, 2Wc]
//   GEMM 2 (tcgen05)  D2[x][y*n_cp + c] = sum_k F2[x][k] B2[y*n_cp + c][k]
//                     F2 = the c2r transform (weights 1, 2, ..., 2, 1; the
//                     imaginary parts of the DC and Nyquist bins ignored); the
//                     epilogue scales by 1/(H W) and folds the n_c values of
//                     each pixel into the maps: batch maximum with the first
//                     correlogram winning ties, strict '>' MIP update, global
//                     index, FP64 sums.
//
// Modes: 1 = BF16 hi + lo operands, 2 = FP16 hi + lo (the cross power is
// scaled by 2^-10 before the split to stay inside FP16's range; the epilogue
// undoes it).  All waits inside the GEMM kernel are bounded and report
// LGB_ERR_DEVICE_TIMEOUT through *device_status.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "match_launch.h"
#include "match_layout.h"
#include "profiler.h"
#include "tc_gemm.cuh"

namespace lgb {

constexpr int kPrecBN = 256;         // N tile of both GEMMs
constexpr int kPrecMaxNc = 32;       // correlograms per batch (one 32-column TMEM load holds whole pixels)
constexpr float kF16Scale = 1.0f / 1024.0f;

struct PrecLayout {
  MatchLayout base;
  int wq, n_cp, kc1, kc2, n1_tiles, n2_tiles, m1_tiles, m2_tiles;
  size_t b1_hi, b1_lo, b2_hi, b2_lo, f1_hi, f1_lo, f2_hi, f2_lo, total;
  size_t b1_bytes, b2_bytes;
};

static int next_pow2(int n) {
  int p = 1;
  while (p < n) p <<= 1;
  return p;
}

static bool prec_supported(const lgb_match_problem* p) {
  if (!valid_problem(p) || !lgb_match_supported(p)) return false;
  const int H = p->image_h, W = p->image_w;
  const int n_c = p->n_pixel_sizes * p->n_defocus * p->orientation_batch;
  // GEMM tiles: 2H and W multiples of 128; the DFT matrices grow as H^2 and W^2
  return mic_h(p) == H && mic_w(p) == W && (2 * H) % kTcM == 0 && W % kTcM == 0 && H <= 1024 && W <= 1024 &&
         n_c <= kPrecMaxNc;
}

static PrecLayout prec_layout(const lgb_match_problem* p) {
  PrecLayout L{};
  L.base = layout_of(p);
  const int H = p->image_h, W = p->image_w;
  const int wc = W / 2 + 1;
  const int n_c = p->n_pixel_sizes * p->n_defocus * p->orientation_batch;
  L.wq = (wc + 31) / 32 * 32;
  L.n_cp = next_pow2(n_c);
  L.kc1 = 2 * H / kTcKC;
  L.kc2 = (2 * wc + kTcKC - 1) / kTcKC;
  L.m1_tiles = 2 * H / kTcM;
  L.m2_tiles = W / kTcM;
  L.n1_tiles = (n_c * L.wq + kPrecBN - 1) / kPrecBN;
  L.n2_tiles = (H * L.n_cp + kPrecBN - 1) / kPrecBN;
  L.b1_bytes = (size_t)L.n1_tiles * kPrecBN * L.kc1 * kTcKC * 2;
  L.b2_bytes = (size_t)L.n2_tiles * kPrecBN * L.kc2 * kTcKC * 2;
  const size_t f1 = (size_t)L.m1_tiles * kTcM * L.kc1 * kTcKC * 2;
  const size_t f2 = (size_t)L.m2_tiles * kTcM * L.kc2 * kTcKC * 2;
  size_t off = L.base.total;
  L.b1_hi = off; off += align256(L.b1_bytes);
  L.b1_lo = off; off += align256(L.b1_bytes);
  L.b2_hi = off; off += align256(L.b2_bytes);
  L.b2_lo = off; off += align256(L.b2_bytes);
  L.f1_hi = off; off += align256(f1);
  L.f1_lo = off; off += align256(f1);
  L.f2_hi = off; off += align256(f2);
  L.f2_lo = off; off += align256(f2);
  L.total = off;
  return L;
}

template <bool F16>
__device__ __forceinline__ void split_store8(const float* x, uint16_t* hi, uint16_t* lo) {
  uint16_t h[8], l[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) Split16<F16>::run(x[i], &h[i], &l[i]);
  uint4 vh, vl;
  vh.x = h[0] | ((uint32_t)h[1] << 16); vh.y = h[2] | ((uint32_t)h[3] << 16);
  vh.z = h[4] | ((uint32_t)h[5] << 16); vh.w = h[6] | ((uint32_t)h[7] << 16);
  vl.x = l[0] | ((uint32_t)l[1] << 16); vl.y = l[2] | ((uint32_t)l[3] << 16);
  vl.z = l[4] | ((uint32_t)l[5] << 16); vl.w = l[6] | ((uint32_t)l[7] << 16);
  *reinterpret_cast<uint4*>(hi) = vh;
  *reinterpret_cast<uint4*>(lo) = vl;
}

// ----------------------------------------------------------------------------
// DFT matrices (FP64 angles, reduced mod the length before the sine/cosine)
// ----------------------------------------------------------------------------
template <bool F16>
__global__ void f1_kernel(int H, int kc, uint16_t* hi, uint16_t* lo) {
  const int M = 2 * H, K = 2 * H;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)M * K;
       e += (long long)gridDim.x * blockDim.x) {
    const int m = (int)(e / K), k = (int)(e % K);
    const int y = m >> 1, ro = m & 1, ky = k >> 1, ri = k & 1;
    const long long t = ((long long)ky * y) % H;
    double s, c;
    sincospi(2.0 * (double)t / (double)H, &s, &c);
    // [Yr; Yi] = [[cos, -sin], [sin, cos]] [Xr; Xi]   (exp(+i theta))
    const double v = ro == 0 ? (ri == 0 ? c : -s) : (ri == 0 ? s : c);
    uint16_t h, l;
    Split16<F16>::run((float)v, &h, &l);
    const size_t o = tc_offset(m, k, kTcM, kc);
    hi[o] = h;
    lo[o] = l;
  }
}

template <bool F16>
__global__ void f2_kernel(int W, int kc, uint16_t* hi, uint16_t* lo) {
  const int M = W, K = kc * kTcKC, wc = W / 2 + 1;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)M * K;
       e += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(e / K), k = (int)(e % K);
    const int kx = k >> 1, ri = k & 1;
    double v = 0.0;
    if (kx < wc) {
      const bool edge = kx == 0 || 2 * kx == W;
      if (!(edge && ri == 1)) {
        const long long t = ((long long)kx * x) % W;
        double s, c;
        sincospi(2.0 * (double)t / (double)W, &s, &c);
        const double w = edge ? 1.0 : 2.0;
        v = ri == 0 ? w * c : -w * s;  // Re(Y exp(+i phi)) = Yr cos - Yi sin
      }
    }
    uint16_t h, l;
    Split16<F16>::run((float)v, &h, &l);
    const size_t o = tc_offset(x, k, kTcM, kc);
    hi[o] = h;
    lo[o] = l;
  }
}

// ----------------------------------------------------------------------------
// colfwd: pruned forward column FFT of the padded projection rows, cross
// power with the image spectrum, written as the split operand B1.
// ----------------------------------------------------------------------------
// Eight columns per CTA: the eight operand rows (c, kx0..kx0+7) of one
// 8-element k group form one 128-byte core matrix, written by eight
// consecutive threads.
constexpr int kColfwdG = 8;

template <int HN, bool F16>
__global__ void __launch_bounds__(kColfwdG* FftThreads<HN>::value, 1)
    colfwd_kernel(const float2* __restrict__ A, const float2* __restrict__ Ip, int h, int Wcp, int wc, int wq,
                  int n_c, int c_per_block, int kc1, float xscale, uint16_t* __restrict__ b1_hi,
                  uint16_t* __restrict__ b1_lo) {
  constexpr int NT = FftThreads<HN>::value;
  constexpr int G = kColfwdG;
  constexpr int STRIDE = IdxPad16::pad(HN) + 4;
  constexpr int NTH = G * NT;
  extern __shared__ float2 cbuf[];
  const int kx0 = blockIdx.x * G;
  const int c_begin = blockIdx.y * c_per_block;
  const int c_end = min(n_c, c_begin + c_per_block);
  const int g = threadIdx.x / NT, t = threadIdx.x - (threadIdx.x / NT) * NT;
#pragma unroll 1
  for (int c = c_begin; c < c_end; ++c) {
    const float2* a = A + (size_t)c * h * Wcp + kx0;
    for (int e = threadIdx.x; e < h * G; e += NTH) {
      const int y = e / G, i = e % G;
      cbuf[i * STRIDE + IdxPad16::f(y)] = kx0 + i < wc ? a[(size_t)y * Wcp + i] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    block_fft_pruned_outline<HN, NT, -1, IdxPad16>(cbuf + g * STRIDE, t, h);
    // cross power, 4 rows x 1 column per item -> 8 consecutive k of row n;
    // the column index runs fastest (coalesced image reads, whole core matrices)
    for (int e = threadIdx.x; e < G * (HN / 4); e += NTH) {
      const int i = e % G, q = e / G;
      const int kx = kx0 + i;
      if (kx >= wc) continue;
      float v[8];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int ky = 4 * q + r;
        const float2 I = __ldg(Ip + (size_t)ky * Wcp + kx);
        float2 X = cmulc(I, cbuf[i * STRIDE + IdxPad16::f(ky)]);
        if (ky == 0 && kx == 0) X = make_float2(0.f, 0.f);
        v[2 * r] = X.x * xscale;
        v[2 * r + 1] = X.y * xscale;
      }
      const size_t o = tc_offset(c * wq + kx, 8 * q, kPrecBN, kc1);
      split_store8<F16>(v, b1_hi + o, b1_lo + o);
    }
    __syncthreads();
  }
}

// ----------------------------------------------------------------------------
// GEMM 1 epilogue: D1 rows (2y + ri) x columns (c*Wq + kx) -> B2 operand
// ----------------------------------------------------------------------------
template <bool F16>
struct EpiColToRow {
  struct Params {
    uint16_t* b2_hi;
    uint16_t* b2_lo;
    int wc, wq, n_c, n_cp, kc2;
  };
  static __device__ __forceinline__ void apply(int row, int col0, const float* v, const Params& p) {
    // lanes 2j and 2j+1 hold the real and imaginary rows of the same y
    float o[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) o[j] = __shfl_xor_sync(0xffffffffu, v[j], 1);
    const int y = row >> 1, ri = row & 1;
    const int c = col0 / p.wq, kxb = col0 - c * p.wq;  // kxb multiple of 32
    if (c >= p.n_c) return;
    const size_t rowb = (size_t)y * p.n_cp + c;
    // even lane: kx offsets 0..15, odd lane 16..31; 4 groups of 4 kx = 8 k each
#pragma unroll
    for (int gq = 0; gq < 4; ++gq) {
      const int kx = kxb + (ri ? 16 : 0) + 4 * gq;
      if (kx >= p.wc) continue;
      float x8[8];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        // compile-time indices only (the values stay in registers)
        const float mine = ri ? v[16 + 4 * gq + r] : v[4 * gq + r];
        const float other = ri ? o[16 + 4 * gq + r] : o[4 * gq + r];
        const float re = ri ? other : mine;
        const float im = ri ? mine : other;
        const bool ok = kx + r < p.wc;
        x8[2 * r] = ok ? re : 0.f;
        x8[2 * r + 1] = ok ? im : 0.f;
      }
      const size_t off = tc_offset((int)rowb, 2 * kx, kPrecBN, p.kc2);
      split_store8<F16>(x8, p.b2_hi + off, p.b2_lo + off);
    }
  }
};

// ----------------------------------------------------------------------------
// GEMM 2 epilogue: D2 rows x (pixel column) by columns (y*n_cp + c) -> maps
// ----------------------------------------------------------------------------
struct EpiRowStats {
  struct Params {
    float* mip;
    int* best;
    double* s1;
    double* s2;
    int H, W, n_c, n_cp, nb, n_orient, o0;
    float scale;
  };
  // NCP = n_cp as a compile-time constant keeps v[] in registers
  template <int NCP>
  static __device__ __forceinline__ void fold(int x, int col0, const float* v, const Params& p) {
#pragma unroll
    for (int gi = 0; gi < 32 / NCP; ++gi) {
      const int y = col0 / NCP + gi;
      if (y >= p.H) break;
      float bmax = -INFINITY, bs = 0.f, bss = 0.f;
      int barg = 0;
#pragma unroll
      for (int c = 0; c < NCP; ++c) {
        if (c >= p.n_c) break;
        const float a = v[gi * NCP + c] * p.scale;
        if (a > bmax) {
          bmax = a;
          barg = c;
        }
        bs += a;
        bss = fmaf(a, a, bss);
      }
      const size_t idx = (size_t)y * p.W + x;
      if (bmax > p.mip[idx]) {
        p.mip[idx] = bmax;
        p.best[idx] = (barg / p.nb) * p.n_orient + p.o0 + (barg - (barg / p.nb) * p.nb);
      }
      p.s1[idx] += (double)bs;
      p.s2[idx] += (double)bss;
    }
  }
  static __device__ __forceinline__ void apply(int row, int col0, const float* v, const Params& p) {
    if (row >= p.W) return;
    switch (p.n_cp) {
      case 1: fold<1>(row, col0, v, p); break;
      case 2: fold<2>(row, col0, v, p); break;
      case 4: fold<4>(row, col0, v, p); break;
      case 8: fold<8>(row, col0, v, p); break;
      case 16: fold<16>(row, col0, v, p); break;
      default: fold<32>(row, col0, v, p); break;
    }
  }
};

template <class Epi, bool F16>
static int launch_gemm(int m_tiles, int n_tiles, const TcGemmArgs& g, const typename Epi::Params& ep,
                       cudaStream_t s) {
  constexpr int SMEM = TcSmem<kPrecBN>::BYTES;
  if (cudaFuncSetAttribute(tc_gemm_kernel<Epi, kPrecBN, F16>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM) !=
      cudaSuccess)
    return LGB_ERR_CUDA;
  tc_gemm_kernel<Epi, kPrecBN, F16><<<dim3(n_tiles, m_tiles), kTcThreads, SMEM, s>>>(g, ep);
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

template <int HN, bool F16>
static int colfwd_t(const void* A, const void* Ip, int h, int Wcp, int wc, int wq, int n_c, int kc1, float xs,
                    uint16_t* hi, uint16_t* lo, cudaStream_t s) {
  constexpr int NT = FftThreads<HN>::value;
  constexpr int G = kColfwdG;
  static_assert(G * NT <= 1024, "colfwd CTA size");
  const size_t smem = sizeof(float2) * G * (IdxPad16::pad(HN) + 4);
  if (cudaFuncSetAttribute(colfwd_kernel<HN, F16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return LGB_ERR_CUDA;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int groups = (wc + G - 1) / G;
  int split = 1;
  while (split < n_c && groups * split < 4 * sms) split *= 2;
  if (split > n_c) split = n_c;
  const int per = (n_c + split - 1) / split;
  split = (n_c + per - 1) / per;
  colfwd_kernel<HN, F16><<<dim3(groups, split), G * NT, smem, s>>>(
      static_cast<const float2*>(A), static_cast<const float2*>(Ip), h, Wcp, wc, wq, n_c, per, kc1, xs, hi, lo);
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

template <bool F16>
static int launch_colfwd(int H, const void* A, const void* Ip, int h, int Wcp, int wc, int wq, int n_c, int kc1,
                         float xs, uint16_t* hi, uint16_t* lo, cudaStream_t s) {
  switch (H) {
#define X(n) \
  case n:    \
    return colfwd_t<n, F16>(A, Ip, h, Wcp, wc, wq, n_c, kc1, xs, hi, lo, s);
    X(64) X(128) X(256) X(512) X(1024)
#undef X
    default:
      return LGB_ERR_UNSUPPORTED_SIZE;
  }
}

template <bool F16>
static int precision_search(const lgb_match_problem* p, const void* template_dft, const float* pf,
                            const float* euler, int begin, int end, float* mip, int* best, double* s1, double* s2,
                            char* ws, const PrecLayout& L, int* dstatus, cudaStream_t s) {
  const int H = p->image_h, W = p->image_w, h = p->template_size;
  const int wc = W / 2 + 1;
  const int n_cd = p->n_pixel_sizes * p->n_defocus;
  auto u16 = [&](size_t off) { return reinterpret_cast<uint16_t*>(ws + off); };
  // zero padding rows / columns of the operands (never written below)
  LGB_CUDA_TRY(cudaMemsetAsync(ws + L.b1_hi, 0, L.b1_bytes, s));
  LGB_CUDA_TRY(cudaMemsetAsync(ws + L.b1_lo, 0, L.b1_bytes, s));
  LGB_CUDA_TRY(cudaMemsetAsync(ws + L.b2_hi, 0, L.b2_bytes, s));
  LGB_CUDA_TRY(cudaMemsetAsync(ws + L.b2_lo, 0, L.b2_bytes, s));
  f1_kernel<F16><<<1024, 256, 0, s>>>(H, L.kc1, u16(L.f1_hi), u16(L.f1_lo));
  f2_kernel<F16><<<512, 256, 0, s>>>(W, L.kc2, u16(L.f2_hi), u16(L.f2_lo));
  if (cudaGetLastError() != cudaSuccess) return LGB_ERR_CUDA;
  const MatchLayout& B = L.base;
  void* ip = ws + B.ip;
  void* slices = ws + B.slices;
  void* T = ws + B.t;
  float* proj = reinterpret_cast<float*>(ws + B.proj);
  double* rowstats = reinterpret_cast<double*>(ws + B.rowstats);
  void* A = ws + B.a;
  const float xs = F16 ? kF16Scale : 1.0f;
  const float out_scale = 1.0f / ((float)H * (float)W) / xs;
  int st;
  for (int o0 = begin; o0 < end; o0 += p->orientation_batch) {
    const int nb = (end - o0) < p->orientation_batch ? (end - o0) : p->orientation_batch;
    const int n_c = n_cd * nb;
    const bool prof = profiling_on();
    {
      StageScope sc(LGB_STAGE_SLICE, s, prof);
      if ((st = launch_slice(template_dft, h, euler, o0, nullptr, nb, nullptr, slices, s))) return st;
    }
    {
      StageScope sc(LGB_STAGE_PROJ_COL, s, prof);
      if ((st = launch_proj_col(h, slices, pf, nb, n_cd, n_c, T, s))) return st;
    }
    {
      StageScope sc(LGB_STAGE_PROJ_ROW, s, prof);
      if ((st = launch_proj_row(h, T, n_c, proj, rowstats, s))) return st;
    }
    {
      StageScope sc(LGB_STAGE_PAD_RFFT, s, prof);
      if ((st = launch_pad_rfft(W, proj, rowstats, h, H, W, B.wcp, n_c, A, s))) return st;
    }
    {
      StageScope sc(LGB_STAGE_COLFWD, s, prof);
      if ((st = launch_colfwd<F16>(H, A, ip, h, B.wcp, wc, L.wq, n_c, L.kc1, xs, u16(L.b1_hi), u16(L.b1_lo), s)))
        return st;
    }
    const int n1_tiles = (n_c * L.wq + kPrecBN - 1) / kPrecBN;
    {
      StageScope sc(LGB_STAGE_DFT_COL, s, prof);
      TcGemmArgs g1{u16(L.f1_hi), u16(L.f1_lo), u16(L.b1_hi), u16(L.b1_lo), L.kc1, 3, dstatus};
      typename EpiColToRow<F16>::Params e1{u16(L.b2_hi), u16(L.b2_lo), wc, L.wq, n_c, L.n_cp, L.kc2};
      if ((st = launch_gemm<EpiColToRow<F16>, F16>(L.m1_tiles, n1_tiles, g1, e1, s))) return st;
    }
    {
      StageScope sc(LGB_STAGE_DFT_ROW, s, prof);
      TcGemmArgs g2{u16(L.f2_hi), u16(L.f2_lo), u16(L.b2_hi), u16(L.b2_lo), L.kc2, 3, dstatus};
      EpiRowStats::Params e2{mip, best, s1, s2, H, W, n_c, L.n_cp, nb, p->n_orientations, o0, out_scale};
      if ((st = launch_gemm<EpiRowStats, F16>(L.m2_tiles, L.n2_tiles, g2, e2, s))) return st;
    }
  }
  return LGB_OK;
}

}  // namespace lgb

using namespace lgb;

extern "C" {

int lgb_match_precision_supported(const lgb_match_problem* p, int mode) {
  return (mode == 1 || mode == 2) && prec_supported(p);
}

int lgb_match_precision_workspace_size(const lgb_match_problem* p, size_t* bytes) {
  if (!bytes || !prec_supported(p)) return !bytes ? LGB_ERR_INVALID_ARGUMENT : LGB_ERR_UNSUPPORTED_SIZE;
  *bytes = prec_layout(p).total;
  return LGB_OK;
}

int lgb_match_search_precision(const lgb_match_problem* p, int mode, const void* template_dft,
                               const float* projective_filters, const float* euler_angles, int orientation_begin,
                               int orientation_end, float* mip, int* best_index, double* corr_sum,
                               double* corr_sq_sum, void* workspace, size_t workspace_bytes, int* device_status,
                               void* stream) {
  if (!valid_problem(p) || (mode != 1 && mode != 2) || !template_dft || !projective_filters || !euler_angles ||
      !mip || !best_index || !corr_sum || !corr_sq_sum || !workspace || !device_status)
    return LGB_ERR_INVALID_ARGUMENT;
  if (orientation_begin < 0 || orientation_end > p->n_orientations || orientation_begin > orientation_end)
    return LGB_ERR_INVALID_ARGUMENT;
  if (!prec_supported(p)) return LGB_ERR_UNSUPPORTED_SIZE;
  const long long total_idx = (long long)p->n_orientations * p->n_defocus * p->n_pixel_sizes;
  if (total_idx > 2147483647LL) return LGB_ERR_INVALID_ARGUMENT;
  const PrecLayout L = prec_layout(p);
  if (workspace_bytes < L.total) return LGB_ERR_WORKSPACE_TOO_SMALL;
  if (reinterpret_cast<uintptr_t>(workspace) & 255) return LGB_ERR_INVALID_ARGUMENT;
  char* ws = static_cast<char*>(workspace);
  cudaStream_t s = (cudaStream_t)stream;
  if (mode == 2)
    return precision_search<true>(p, template_dft, projective_filters, euler_angles, orientation_begin,
                                  orientation_end, mip, best_index, corr_sum, corr_sq_sum, ws, L, device_status, s);
  return precision_search<false>(p, template_dft, projective_filters, euler_angles, orientation_begin,
                                 orientation_end, mip, best_index, corr_sum, corr_sq_sum, ws, L, device_status, s);
}

}  // extern "C"
