// Kernels of the plain FP32 whole-orientation search.
//
// Per orientation batch (B orientations, C*D projective filters, n_c = C*D*B
// correlograms, c = (cs*D + df)*B + b):
//   slice_kernel      Fourier slice of the template at R(phi,theta,psi),
//                     rows un-shifted, DC zeroed, contrast flipped
//                     (cross_correlation.py:76-92)                     [B, d, d/2+1]
//   proj_col_kernel   x projective filter, inverse FFT along y          [n_c, d, d/2+1]
//   proj_row_kernel   c2r along x, 1/d^2, ifftshift, per-row moments    [n_c, d, d]
//   pad_rfft_kernel   edge-mean/variance normalisation (utils.py:106-188)
//                     and the zero-padded row rfft of length W          [n_c, d, Wcp]
//   column pass       per column: pruned FFT along y (length H), cross power
//                     image * conj(P) with P[0,0]=0, inverse FFT along y
//                     (colpass_fused_kernel / colpass_tab_kernel)      [n_c, H, Wcp]
//   rowpass_kernel    per row: c2r of length W (1/(H W)) and the fused
//                     statistics update (utils.py:191-255): max over the
//                     batch, strict '>' MIP update, global index, FP64 sums
// Two-register-pass forms for the refinement crops (288^2, d = 256):
// proj_col_pair_kernel (256 = 16 x 16) and proj_row_rfft_kernel (row c2r
// 16 x 8 and the padded rfft 16 x 9 in one kernel; the normalisation moves to
// the column pass, colpass_pair_kernel in match_fused.cuh).
#pragma once

#include "fft.cuh"

namespace lgb {

constexpr int kColGroup = 4;  // columns per colpass CTA: 4 x 8 B = one 32 B sector per row

__host__ __device__ inline int pad4(int n) { return (n + 3) & ~3; }

// ---------------------------------------------------------------------------
// Euler (ZYZ, degrees) -> R = Rz(phi) Ry(theta) Rz(psi), in FP64.
// ---------------------------------------------------------------------------
__device__ inline void euler_zyz_to_rotmat(const float* e, float* R) {
  const double k = 3.14159265358979323846 / 180.0;
  double sp, cp, st, ct, ss, cs;
  sincos((double)e[0] * k, &sp, &cp);
  sincos((double)e[1] * k, &st, &ct);
  sincos((double)e[2] * k, &ss, &cs);
  R[0] = (float)(cp * ct * cs - sp * ss);
  R[1] = (float)(-cp * ct * ss - sp * cs);
  R[2] = (float)(cp * st);
  R[3] = (float)(sp * ct * cs + cp * ss);
  R[4] = (float)(-sp * ct * ss + cp * cs);
  R[5] = (float)(sp * st);
  R[6] = (float)(-st * cs);
  R[7] = (float)(st * ss);
  R[8] = (float)ct;
}

// ---------------------------------------------------------------------------
// proj_col: T[c][y][kx] = IFFT_y( slice_b[y][kx] * pf[cd][y][kx] )   (unscaled)
// ---------------------------------------------------------------------------
template <int HT, int COLS>
__global__ void __launch_bounds__(COLS* FftThreads<HT>::value)
    proj_col_kernel(const float2* __restrict__ slices, const float* __restrict__ pf, int nb, int n_cd,
                    float2* __restrict__ T) {
  constexpr int NT = FftThreads<HT>::value;
  constexpr int WC = HT / 2 + 1;
  constexpr int STRIDE = IdxPad16::pad(HT) + 2;
  __shared__ float2 buf[COLS * STRIDE];
  // c = (p*n_cd + cd)*nb + b: slices are per (p, b), filters per (p, cd)
  const int c = blockIdx.y;
  const int pc = c / nb, b = c - (c / nb) * nb;
  const int p = pc / n_cd;
  const float2* sl = slices + ((size_t)p * nb + b) * HT * WC;
  const float* f = pf + (size_t)pc * HT * WC;
  const int kx0 = blockIdx.x * COLS;
  for (int e = threadIdx.x; e < HT * COLS; e += blockDim.x) {
    const int y = e / COLS, i = e % COLS, kx = kx0 + i;
    float2 v = make_float2(0.f, 0.f);
    if (kx < WC) {
      v = sl[y * WC + kx];
      const float w = f[y * WC + kx];
      v.x *= w;
      v.y *= w;
    }
    buf[i * STRIDE + IdxPad16::f(y)] = v;
  }
  __syncthreads();
  const int g = threadIdx.x / NT, t = threadIdx.x - (threadIdx.x / NT) * NT;
  block_fft<HT, NT, +1, IdxPad16>(buf + g * STRIDE, t);
  float2* out = T + (size_t)c * HT * WC;
  for (int e = threadIdx.x; e < HT * COLS; e += blockDim.x) {
    const int y = e / COLS, i = e % COLS, kx = kx0 + i;
    if (kx < WC) out[y * WC + kx] = buf[i * STRIDE + IdxPad16::f(y)];
  }
}

// proj_col for HT = R1*R2 (256 = 16*16) in two register passes: radix R1
// over rows t + R2*q of slice x filter straight from global memory ->
// shared transpose M1[t][q] (odd stride R1+1; column stride 2 mod 16) ->
// radix R2 with twiddles w^(r*t), w = exp(+2 pi i / HT) -> rows t + R1*r of T.
// G columns per CTA (lane bits 0-2), one thread per butterfly.
template <int R1, int R2>
struct ProjColPair {
  static constexpr int HT = R1 * R2;
  static constexpr int NT = R1 > R2 ? R1 : R2;
  static constexpr int G = 8;
  static constexpr int S1 = R1 + 1;
  static constexpr int CB = R2 * S1;
  static constexpr int STRIDE = CB + (18 - CB % 16) % 16;  // = 2 (mod 16)
  static constexpr int NROOT = (R1 - 1) * (R2 - 1) + 1;
};

template <int R1, int R2>
__global__ void __launch_bounds__(ProjColPair<R1, R2>::G* ProjColPair<R1, R2>::NT)
    proj_col_pair_kernel(const float2* __restrict__ slices, const float* __restrict__ pf, int nb, int n_cd,
                         float2* __restrict__ T) {
  using PC = ProjColPair<R1, R2>;
  constexpr int HT = PC::HT, WC = HT / 2 + 1, G = PC::G, S1 = PC::S1;
  __shared__ float2 buf[G * PC::STRIDE];
  __shared__ float2 root[PC::NROOT];  // exp(+2 pi i m / HT)
  for (int m = threadIdx.x; m < PC::NROOT; m += blockDim.x) {
    float sn, cs;
    sincospif(2.0f * (float)m / (float)HT, &sn, &cs);
    root[m] = make_float2(cs, sn);
  }
  // c = (p*n_cd + cd)*nb + b: slices are per (p, b), filters per (p, cd)
  const int c = blockIdx.y;
  const int pc = c / nb, b = c - (c / nb) * nb;
  const int p = pc / n_cd;
  const float2* sl = slices + ((size_t)p * nb + b) * HT * WC;
  const float* f = pf + (size_t)pc * HT * WC;
  const int g = threadIdx.x % G, t = threadIdx.x / G;
  const int kx = blockIdx.x * G + g;
  const bool col_ok = kx < WC;
  float2* x = buf + g * PC::STRIDE;
  if (t < R2) {
    float2 v[R1];
#pragma unroll
    for (int q = 0; q < R1; ++q) {
      const int y = t + q * R2;
      v[q] = make_float2(0.f, 0.f);
      if (col_ok) {
        const float2 s = __ldg(sl + (size_t)y * WC + kx);
        const float w = __ldg(f + (size_t)y * WC + kx);
        v[q] = make_float2(s.x * w, s.y * w);
      }
    }
    Dft<R1, +1>::run(v);
#pragma unroll
    for (int q = 0; q < R1; ++q) x[t * S1 + q] = v[q];
  }
  __syncthreads();
  if (t < R1) {
    float2 w[R2];
#pragma unroll
    for (int r = 0; r < R2; ++r) w[r] = cmul(x[r * S1 + t], root[r * t]);
    Dft<R2, +1>::run(w);
    if (col_ok) {
      float2* out = T + (size_t)c * HT * WC + (size_t)t * WC + kx;
#pragma unroll
      for (int r = 0; r < R2; ++r) out[(size_t)r * R1 * WC] = w[r];
    }
  }
}

// ---------------------------------------------------------------------------
// proj_row: c2r along x of each row of T[c] (length HT via an HT/2 complex
// inverse FFT), scale 1/HT^2, ifftshift both axes, and per-row moments
// rowstats[c][py] = (sum, sum of squares, edge sum) in FP64.
// Imaginary parts of the DC and Nyquist bins are ignored (c2r convention).
// ---------------------------------------------------------------------------
template <int HT, int ROWS>
__global__ void __launch_bounds__(ROWS* FftThreads<HT / 2>::value)
    proj_row_kernel(const float2* __restrict__ T, float* __restrict__ proj, double* __restrict__ rowstats) {
  constexpr int M = HT / 2;
  constexpr int WC = HT / 2 + 1;
  constexpr int NT = FftThreads<M>::value;
  constexpr int ZS = IdxPad16::pad(M) + 2;
  __shared__ float2 xin[ROWS][WC];
  __shared__ float2 z[ROWS][ZS];
  __shared__ float part[ROWS * NT][3];
  const int c = blockIdx.y;
  const int g = threadIdx.x / NT, t = threadIdx.x - (threadIdx.x / NT) * NT;
  const int row0 = blockIdx.x * ROWS;
  const float2* src = T + ((size_t)c * HT + row0) * WC;
  for (int e = threadIdx.x; e < ROWS * WC; e += blockDim.x) xin[e / WC][e % WC] = src[e];
  __syncthreads();
  for (int k = t; k < M; k += NT) {
    float2 A = xin[g][k];
    float2 B = xin[g][M - k];
    if (k == 0) { A.y = 0.f; B.y = 0.f; }  // DC and Nyquist: real parts only
    B.y = -B.y;                            // conj
    const float2 xe = cadd(A, B);
    float s, co;
    sincospif(2.0f * (float)k / (float)HT, &s, &co);
    const float2 xo = cmul(csub(A, B), make_float2(co, s));
    z[g][IdxPad16::f(k)] = cadd(xe, mul_i<1>(xo));
  }
  __syncthreads();
  block_fft<M, NT, +1, IdxPad16>(z[g], t);
  const int y = row0 + g;
  const int py = (y + HT - HT / 2) % HT;
  const float scale = 1.0f / ((float)HT * (float)HT);
  const bool edge_row = (py == 0) || (py == HT - 1);
  // partial moments in FP32, per thread and then across the row's threads;
  // FP64 only for the stored row moments (FP64 arithmetic, conversions
  // included, runs at about one operation per SM per clock on this GPU); the
  // cross-row reduction is FP64
  float s1 = 0.f, s2 = 0.f, se = 0.f;
  float* prow = proj + ((size_t)c * HT + py) * HT;
  for (int m = t; m < M; m += NT) {
    const float2 v = z[g][IdxPad16::f(m)];
    const float a = v.x * scale, b = v.y * scale;
    const int px0 = (2 * m + HT - HT / 2) % HT, px1 = (2 * m + 1 + HT - HT / 2) % HT;
    prow[px0] = a;
    prow[px1] = b;
    s1 += a + b;
    s2 = fmaf(a, a, fmaf(b, b, s2));
    if (edge_row) {
      se += a + b;
    } else {
      if (px0 == 0 || px0 == HT - 1) se += a;
      if (px1 == 0 || px1 == HT - 1) se += b;
    }
  }
  part[threadIdx.x][0] = s1;
  part[threadIdx.x][1] = s2;
  part[threadIdx.x][2] = se;
  __syncthreads();
  if (t == 0) {
    float a = 0.f, b = 0.f, e = 0.f;
    for (int i = 0; i < NT; ++i) {
      a += part[g * NT + i][0];
      b += part[g * NT + i][1];
      e += part[g * NT + i][2];
    }
    double* rs = rowstats + ((size_t)c * HT + py) * 3;
    rs[0] = (double)a;
    rs[1] = (double)b;
    rs[2] = (double)e;
  }
}

// proj_row for HT/2 = R1*R2 (128 = 16*8) in two register passes: the c2r
// pre-twiddle is applied while loading the radix-R1 inputs k = t + R2*q from
// the staged row; shared transpose M1[t][q]; radix R2 with twiddles w^(r*t)
// leaves pixel pairs m = t + R1*r in thread t.  Same outputs, ifftshift and
// moments as proj_row_kernel; R1 threads per row, ROWS rows per CTA.
template <int R1, int R2, int ROWS>
struct ProjRowPair {
  static constexpr int M = R1 * R2;
  static constexpr int NT = R1;
  static constexpr int S1 = R1 + 1;
  static constexpr int ZR = R2 * S1 + 1;
  static constexpr int NROOT = (R1 - 1) * (R2 - 1) + 1;
  static_assert(R1 >= R2, "second pass uses every thread of the row");
};

template <int R1, int R2, int ROWS>
__global__ void __launch_bounds__(ROWS* R1)
    proj_row_pair_kernel(const float2* __restrict__ T, float* __restrict__ proj, double* __restrict__ rowstats) {
  using PR = ProjRowPair<R1, R2, ROWS>;
  constexpr int M = PR::M, HT = 2 * M, WC = M + 1, NT = PR::NT, S1 = PR::S1;
  __shared__ float2 xin[ROWS][WC + 1];
  __shared__ float2 zb[ROWS][PR::ZR];
  __shared__ float2 pre[M];            // exp(+i pi k / M)
  __shared__ float2 root[PR::NROOT];   // exp(+2 pi i m / M)
  static_assert(32 % R1 == 0, "rows must be lane aligned for the shuffle reduction");
  for (int k = threadIdx.x; k < M; k += blockDim.x) {
    float sn, cs;
    sincospif((float)k / (float)M, &sn, &cs);
    pre[k] = make_float2(cs, sn);
  }
  for (int m = threadIdx.x; m < PR::NROOT; m += blockDim.x) {
    float sn, cs;
    sincospif(2.0f * (float)m / (float)M, &sn, &cs);
    root[m] = make_float2(cs, sn);
  }
  const int c = blockIdx.y;
  const int g = threadIdx.x / NT, t = threadIdx.x - (threadIdx.x / NT) * NT;
  const int row0 = blockIdx.x * ROWS;
  const float2* src = T + ((size_t)c * HT + row0) * WC;
  for (int e = threadIdx.x; e < ROWS * WC; e += blockDim.x) xin[e / WC][e % WC] = src[e];
  __syncthreads();
  // ---- pass 1 (radix R1, stride 1) on the pre-twiddled z[k], k = t + R2*q
  if (t < R2) {
    float2 v[R1];
#pragma unroll
    for (int q = 0; q < R1; ++q) {
      const int k = t + q * R2;
      float2 A = xin[g][k];
      float2 B = xin[g][M - k];
      if (k == 0) { A.y = 0.f; B.y = 0.f; }  // DC and Nyquist: real parts only
      B.y = -B.y;                            // conj
      const float2 xo = cmul(csub(A, B), pre[k]);
      v[q] = cadd(cadd(A, B), mul_i<1>(xo));
    }
    Dft<R1, +1>::run(v);
#pragma unroll
    for (int q = 0; q < R1; ++q) zb[g][t * S1 + q] = v[q];
  }
  __syncthreads();
  // ---- pass 2 (radix R2, stride R1): w[r] = z[t + R1*r]
  float2 w[R2];
#pragma unroll
  for (int r = 0; r < R2; ++r) w[r] = cmul(zb[g][r * S1 + t], root[r * t]);
  Dft<R2, +1>::run(w);
  const int y = row0 + g;
  const int py = (y + HT - HT / 2) % HT;
  const float scale = 1.0f / ((float)HT * (float)HT);
  const bool edge_row = (py == 0) || (py == HT - 1);
  float s1 = 0.f, s2 = 0.f, se = 0.f;
  float* prow = proj + ((size_t)c * HT + py) * HT;
#pragma unroll
  for (int r = 0; r < R2; ++r) {
    const int m = t + r * R1;
    const float a = w[r].x * scale, b = w[r].y * scale;
    const int px0 = (2 * m + HT - HT / 2) % HT;  // even: px0 + 1 does not wrap
    *reinterpret_cast<float2*>(prow + px0) = make_float2(a, b);
    s1 += a + b;
    s2 = fmaf(a, a, fmaf(b, b, s2));
    if (edge_row) {
      se += a + b;
    } else {
      if (px0 == 0) se += a;
      if (px0 + 1 == HT - 1) se += b;
    }
  }
  // row reduction across the row's R1 lanes in FP32 (R1 divides 32, rows are
  // lane aligned); FP64 only for the stored row moments: this GPU's FP64 pipe
  // retires about one operation per SM per clock, conversions included
#pragma unroll
  for (int o = R1 / 2; o > 0; o >>= 1) {
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    se += __shfl_xor_sync(0xffffffffu, se, o);
  }
  if (t == 0) {
    double* rs = rowstats + ((size_t)c * HT + py) * 3;
    rs[0] = (double)s1;
    rs[1] = (double)s2;
    rs[2] = (double)se;
  }
}

// proj_row and the zero-padded row rfft in one kernel, for d = 256 templates
// and rows of W = 288 (the refinement crops).  Per row y of T[c]: the 256-point
// c2r as in proj_row_pair_kernel<16, 8> (pixel pairs m = t + 16r in thread t),
// the row moments, the ifftshift (pair m -> m' = (m + 64) mod 128), then the
// rfft of the un-normalised row zero padded to W in two register passes
// (144 = 16 x 9) and the real post-process:
//   A[c][py][k] = sum_{px < d} p[py][px] exp(-2 pi i k px / W),  k <= W/2.
// The projection never goes to memory.  Its normalisation (p - e) s
// (utils.py:106-188) is affine, rfft((p - e) s) = s (A - e U) with
// U[k] = sum_{px < d} exp(-2 pi i k px / W), and is applied by the column pass.
template <int ROWS>
__global__ void __launch_bounds__(ROWS * 16)
    proj_row_rfft_kernel(const float2* __restrict__ T, double* __restrict__ rowstats, int Wcp,
                         float2* __restrict__ A) {
  constexpr int HT = 256, M = 128, WC = M + 1, NT = 16, S1 = 17;
  constexpr int WH = 144;  // W / 2
  constexpr int C2 = 8;    // c2r: M = 16 x 8
  constexpr int R2 = 9;    // rfft: WH = 16 x 9
  // Row strides of the shared buffers, chosen for the densely packed first
  // passes below, where two rows share a half-warp: 152 float2 (xz) and
  // 153 = R2 * S1 (zb) keep those loads and stores at the fewest bank
  // conflicts the index maps allow (per-row passes are conflict free at any
  // stride).
  constexpr int ZR = 152;
  static_assert(ZR >= IdxPad16::pad(WH) - 1 && ZR >= WC + 1, "staged row and padded rfft input fit");
  // xin (the staged row of T, read only by c2r pass 1) and zr (the rfft input,
  // written from c2r pass 2 on, then Z) share one buffer per row
  __shared__ float2 xz[ROWS][ZR];
  __shared__ float2 zb[ROWS][R2 * S1];  // c2r transpose (8 x 17), then rfft transpose (9 x 17)
  float2(*xin)[ZR] = xz;
  float2(*zr)[ZR] = xz;
  __shared__ float2 pre[M];                 // exp(+i pi k / M)
  __shared__ float2 rootc[15 * (C2 - 1) + 1];  // exp(+2 pi i m / M)
  __shared__ float2 rootr[15 * (R2 - 1) + 1];  // exp(-2 pi i m / WH)
  __shared__ float2 post[WH + 1];              // exp(-i pi k / WH)
  for (int k = threadIdx.x; k < M; k += blockDim.x) {
    float sn, cs;
    sincospif((float)k / (float)M, &sn, &cs);
    pre[k] = make_float2(cs, sn);
  }
  for (int k = threadIdx.x; k <= WH; k += blockDim.x) {
    float sn, cs;
    sincospif((float)k / (float)WH, &sn, &cs);
    post[k] = make_float2(cs, -sn);
  }
  const int c = blockIdx.y;
  const int g = threadIdx.x / NT, t = threadIdx.x - (threadIdx.x / NT) * NT;
  const int row0 = blockIdx.x * ROWS;
  const float2* src = T + ((size_t)c * HT + row0) * WC;
  for (int e = threadIdx.x; e < ROWS * WC; e += blockDim.x) xin[e / WC][e % WC] = src[e];
  __syncthreads();
  // the radix roots are the pre- and post-twiddles at even angles:
  // exp(+2 pi i m / M) = +-pre[2m mod M], exp(-2 pi i m / WH) = +-post[2m mod WH]
  // (read from the next pass on, after a barrier)
  for (int m = threadIdx.x; m < 15 * (C2 - 1) + 1; m += blockDim.x) {
    const float2 v = pre[(2 * m) & (M - 1)];
    rootc[m] = 2 * m < M ? v : make_float2(-v.x, -v.y);
  }
  for (int m = threadIdx.x; m < 15 * (R2 - 1) + 1; m += blockDim.x) {
    const float2 v = post[2 * m <= WH ? 2 * m : 2 * m - WH];
    rootr[m] = 2 * m <= WH ? v : make_float2(-v.x, -v.y);
  }
  // The two radix-16 passes have fewer DFTs per row (8 and 9) than a row has
  // threads (16): their (row, DFT) tasks are packed densely onto the CTA's
  // threads, so whole warps idle instead of half of every warp's lanes.
  // ---- c2r pass 1 (radix 16) on the pre-twiddled z[k], k = tt + 8q
  if (threadIdx.x < ROWS * C2) {
    const int gg = threadIdx.x / C2, tt = threadIdx.x - (threadIdx.x / C2) * C2;
    float2 v[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int k = tt + q * C2;
      float2 a = xin[gg][k];
      float2 b = xin[gg][M - k];
      if (k == 0) { a.y = 0.f; b.y = 0.f; }  // DC and Nyquist: real parts only
      b.y = -b.y;
      const float2 xo = cmul(csub(a, b), pre[k]);
      v[q] = cadd(cadd(a, b), mul_i<1>(xo));
    }
    Dft<16, +1>::run(v);
#pragma unroll
    for (int q = 0; q < 16; ++q) zb[gg][tt * S1 + q] = v[q];
  }
  __syncthreads();
  // ---- c2r pass 2 (radix 8): pixel pairs m = t + 16r, moments, shifted rfft input
  const int y = row0 + g;
  const int py = (y + HT - HT / 2) % HT;
  {
    float2 w[C2];
#pragma unroll
    for (int r = 0; r < C2; ++r) w[r] = cmul(zb[g][r * S1 + t], rootc[r * t]);
    Dft<C2, +1>::run(w);
    const float scale = 1.0f / ((float)HT * (float)HT);
    const bool edge_row = (py == 0) || (py == HT - 1);
    float s1 = 0.f, s2 = 0.f, se = 0.f;
#pragma unroll
    for (int r = 0; r < C2; ++r) {
      const int m = t + r * 16;
      const float a = w[r].x * scale, b = w[r].y * scale;
      const int mp = (m + M / 2) & (M - 1);  // ifftshift: px = 2 mp, 2 mp + 1
      zr[g][IdxPad16::f(mp)] = make_float2(a, b);
      s1 += a + b;
      s2 = fmaf(a, a, fmaf(b, b, s2));
      if (edge_row) {
        se += a + b;
      } else {
        if (mp == 0) se += a;
        if (mp == M - 1) se += b;
      }
    }
    zr[g][IdxPad16::f(M + t)] = make_float2(0.f, 0.f);  // zero padding m' = 128..143
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) {
      s1 += __shfl_xor_sync(0xffffffffu, s1, o);
      s2 += __shfl_xor_sync(0xffffffffu, s2, o);
      se += __shfl_xor_sync(0xffffffffu, se, o);
    }
    if (t == 0) {
      double* rs = rowstats + ((size_t)c * HT + py) * 3;
      rs[0] = (double)s1;
      rs[1] = (double)s2;
      rs[2] = (double)se;
    }
  }
  __syncthreads();
  // ---- rfft pass 1 (radix 16) over m' = tt + 9q, tasks packed as above
  if (threadIdx.x < ROWS * R2) {
    const int gg = threadIdx.x / R2, tt = threadIdx.x - (threadIdx.x / R2) * R2;
    float2 v[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = zr[gg][IdxPad16::f(tt + q * R2)];
    Dft<16, -1>::run(v);
#pragma unroll
    for (int q = 0; q < 16; ++q) zb[gg][tt * S1 + q] = v[q];
  }
  __syncthreads();
  // ---- rfft pass 2 (radix 9): Z[t + 16r]
  {
    float2 u[R2];
#pragma unroll
    for (int r = 0; r < R2; ++r) u[r] = cmul(zb[g][r * S1 + t], rootr[r * t]);
    Dft<R2, -1>::run(u);
#pragma unroll
    for (int r = 0; r < R2; ++r) zr[g][IdxPad16::f(t + 16 * r)] = u[r];
  }
  __syncthreads();
  float2* out = A + ((size_t)c * HT + py) * Wcp;
  for (int k = t; k <= WH; k += NT) {
    const float2 Zk = zr[g][IdxPad16::f(k == WH ? 0 : k)];
    const float2 Zm = cconj(zr[g][IdxPad16::f(k == 0 ? 0 : WH - k)]);
    const float2 xe = cscale(cadd(Zk, Zm), 0.5f);
    const float2 xo = mul_i<-1>(cscale(csub(Zk, Zm), 0.5f));
    out[k] = cadd(xe, cmul(post[k], xo));
  }
  for (int k = WH + 1 + t; k < Wcp; k += NT) out[k] = make_float2(0.f, 0.f);
}

// Normalisation constants of utils.py:106-188 from the per-row moments:
// returns edge mean e and scale s such that normalised = (p - e) * s.
// Called by all 32 lanes of warp 0 (the launcher guarantees a full warp).
__device__ inline void projection_norm_constants(const double* rs, int h, int H, int W, float* e_out,
                                                 float* s_out) {
  // warp 0 reduces h rows
  double s1 = 0, s2 = 0, se = 0;
  const int lane = threadIdx.x & 31;
  for (int r = lane; r < h; r += 32) {
    s1 += rs[3 * r];
    s2 += rs[3 * r + 1];
    se += rs[3 * r + 2];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s1 += __shfl_down_sync(0xffffffffu, s1, o);
    s2 += __shfl_down_sync(0xffffffffu, s2, o);
    se += __shfl_down_sync(0xffffffffu, se, o);
  }
  if (lane == 0) {
    const double n = (double)h * (double)h;
    const double e = se / (double)(4 * h - 4);
    const double S1 = s1 - n * e;                  // sum of (p - e)
    const double S2 = s2 - 2.0 * e * s1 + n * e * e;  // sum of (p - e)^2
    const double rel = n / ((double)H * (double)W);
    const double mean = (S1 / n) * rel * rel;
    double var = S2 - 2.0 * mean * S1 + n * mean * mean;
    var += (double)(H - h) * (double)(W - h) * mean * mean;
    if (var < 1e-8) var = 1e-8;
    *e_out = (float)e;
    *s_out = (float)(sqrt((double)H * (double)W) / sqrt(var));
  }
}

// ---------------------------------------------------------------------------
// pad_rfft: A[c][y][k] = rfft_W( normalised projection row y, zero padded )
// for k = 0..W/2, zeros up to Wcp.  The normalisation is that of a
// norm_h x norm_w micrograph (W may exceed norm_w when the micrograph was
// zero padded to a supported FFT length).  Real FFT of length W = 2*WH through a
// WH-point complex FFT (first pass pruned to the ceil(h/2) non-zero inputs).
// ---------------------------------------------------------------------------
// TAB: twiddles and post-twiddles from shared tables filled once per CTA (for
// small transforms, where a CTA holds many rows to amortise the fill).
template <int WH, int ROWS, bool TAB>
__global__ void __launch_bounds__(ROWS* FftThreads<WH>::value)
    pad_rfft_kernel(const float* __restrict__ proj, const double* __restrict__ rowstats, int h, int norm_h,
                    int norm_w, int Wcp, int norm_ready, float2* __restrict__ A) {
  constexpr int NT = FftThreads<WH>::value;
  constexpr int ZS = IdxPad16::pad(WH) + 2;
  __shared__ float2 z[ROWS][ZS];
  __shared__ float2 post[TAB ? WH + 1 : 1];  // exp(-i pi k / WH)
  __shared__ float2 tab[TAB ? FftTable<WH>::SIZE + 1 : 1];
  if (TAB) {
    fill_fft_table<WH>(tab, threadIdx.x, blockDim.x);
    for (int k = threadIdx.x; k <= WH; k += blockDim.x) {
      float sn, cs;
      sincospif((float)k / (float)WH, &sn, &cs);
      post[k] = make_float2(cs, -sn);
    }
  }
  const int c = blockIdx.y;
  // norm_ready: constants (e, s) precomputed by norm_constants_kernel as a
  // float2 over rowstats[c][0][0]; otherwise warp 0 reduces the row moments here
  __shared__ float norm[2];
  if (norm_ready) {
    if (threadIdx.x == 0) {
      const float2 es = *reinterpret_cast<const float2*>(rowstats + (size_t)c * h * 3);
      norm[0] = es.x;
      norm[1] = es.y;
    }
  } else if (threadIdx.x < 32) {
    projection_norm_constants(rowstats + (size_t)c * h * 3, h, norm_h, norm_w, &norm[0], &norm[1]);
  }
  __syncthreads();
  const float e = norm[0], s = norm[1];
  const int g = threadIdx.x / NT, t = threadIdx.x - (threadIdx.x / NT) * NT;
  const int y = blockIdx.x * ROWS + g;
  const bool active = y < h;
  const int nz = (h + 1) / 2;
  if (active) {
    const float* p = proj + ((size_t)c * h + y) * h;
    for (int m = t; m < nz; m += NT) {
      const float a = (p[2 * m] - e) * s;
      const float b = (2 * m + 1 < h) ? (p[2 * m + 1] - e) * s : 0.f;
      z[g][IdxPad16::f(m)] = make_float2(a, b);
    }
  }
  __syncthreads();
  if (TAB)
    block_fft_pruned_tab<WH, NT, -1, IdxPad16>(z[g], tab, t, nz);
  else
    block_fft_pruned<WH, NT, -1, IdxPad16>(z[g], t, nz);
  if (!active) return;
  float2* out = A + ((size_t)c * h + y) * Wcp;
  for (int k = t; k <= WH; k += NT) {
    const float2 Zk = z[g][IdxPad16::f(k == WH ? 0 : k)];
    const float2 Zm = cconj(z[g][IdxPad16::f(k == 0 ? 0 : WH - k)]);
    const float2 xe = cscale(cadd(Zk, Zm), 0.5f);
    const float2 xo = mul_i<-1>(cscale(csub(Zk, Zm), 0.5f));
    float2 w;
    if (TAB) {
      w = post[k];
    } else {
      float sn, cs;
      sincospif((float)k / (float)WH, &sn, &cs);
      w = make_float2(cs, -sn);
    }
    out[k] = cadd(xe, cmul(w, xo));
  }
  for (int k = WH + 1 + t; k < Wcp; k += NT) out[k] = make_float2(0.f, 0.f);
}

// pad_rfft for long rows (WH >= 1024, where a CTA holds too few rows for the
// static form to carry twiddle tables): the CTA fills the FFT and post-twiddle
// tables once in dynamic shared memory and walks RPC rows of one correlogram,
// ROWS at a time.  The normalisation constants come precomputed (norm_constants_kernel).
template <int WH, int ROWS>
struct PadRows {
  static constexpr int NT = FftThreads<WH>::value;
  static constexpr int ZS = IdxPad16::pad(WH) + 2;
  static constexpr size_t SMEM = sizeof(float2) * ((size_t)ROWS * ZS + FftTable<WH>::SIZE + 1 + WH + 1);
  static constexpr int MINB = 3 * SMEM <= 227 * 1024 ? 3 : 2;  // CTAs per SM the shared memory allows
};

template <int WH, int ROWS, int RPC>
__global__ void __launch_bounds__(ROWS* FftThreads<WH>::value, (PadRows<WH, ROWS>::MINB))
    pad_rfft_rows_kernel(const float* __restrict__ proj, const double* __restrict__ rowstats, int h, int Wcp,
                         float2* __restrict__ A) {
  using PR = PadRows<WH, ROWS>;
  constexpr int NT = PR::NT, ZS = PR::ZS;
  extern __shared__ float2 prsm[];
  float2* z = prsm;                            // [ROWS][ZS]
  float2* tab = z + ROWS * ZS;                 // FftTable<WH>::SIZE
  float2* post = tab + FftTable<WH>::SIZE + 1;  // exp(-i pi k / WH), k = 0..WH
  fill_fft_table<WH>(tab, threadIdx.x, blockDim.x);
  for (int k = threadIdx.x; k <= WH; k += blockDim.x) {
    float sn, cs;
    sincospif((float)k / (float)WH, &sn, &cs);
    post[k] = make_float2(cs, -sn);
  }
  const int c = blockIdx.y;
  const float2 es = *reinterpret_cast<const float2*>(rowstats + (size_t)c * h * 3);
  const float e = es.x, s = es.y;
  const int g = threadIdx.x / NT, t = threadIdx.x - (threadIdx.x / NT) * NT;
  float2* zg = z + g * ZS;
  const int nz = (h + 1) / 2;
  const int y_end = min(h, (int)blockIdx.x * RPC + RPC);
#pragma unroll 1
  for (int y0 = blockIdx.x * RPC; y0 < y_end; y0 += ROWS) {
    const int y = y0 + g;
    const bool active = y < y_end;
    if (active) {
      const float* p = proj + ((size_t)c * h + y) * h;
      for (int m = t; m < nz; m += NT) {
        const float a = (p[2 * m] - e) * s;
        const float b = (2 * m + 1 < h) ? (p[2 * m + 1] - e) * s : 0.f;
        zg[IdxPad16::f(m)] = make_float2(a, b);
      }
    }
    __syncthreads();  // rows staged; tables filled (first iteration)
    block_fft_pruned_tab<WH, NT, -1, IdxPad16>(zg, tab, t, nz);
    if (active) {
      float2* out = A + ((size_t)c * h + y) * Wcp;
      for (int k = t; k <= WH; k += NT) {
        const float2 Zk = zg[IdxPad16::f(k == WH ? 0 : k)];
        const float2 Zm = cconj(zg[IdxPad16::f(k == 0 ? 0 : WH - k)]);
        const float2 xe = cscale(cadd(Zk, Zm), 0.5f);
        const float2 xo = mul_i<-1>(cscale(csub(Zk, Zm), 0.5f));
        out[k] = cadd(xe, cmul(post[k], xo));
      }
      for (int k = WH + 1 + t; k < Wcp; k += NT) out[k] = make_float2(0.f, 0.f);
    }
    __syncthreads();  // this pass's rows are read before the next ones are staged
  }
}

// Columns per colpass CTA: kColGroup, or 2 where four transforms of length HN
// would need more than 1024 threads (HN = 5760).
template <int HN>
struct ColGroupOf {
  static constexpr int value = kColGroup * FftThreads<HN>::value <= 1024 ? kColGroup : 2;
};

// ---------------------------------------------------------------------------
// rowpass: row y of every correlogram in the batch: c2r of length W = 2*WH
// (imaginary parts of DC / Nyquist ignored), scale 1/(H W) (passed in), then the fused
// statistics update of utils.py:191-255 (max over the batch in c order with
// strict '>', MIP update with strict '>', global index, FP64 sums).
// ---------------------------------------------------------------------------
constexpr int kRowThreads = 256;

template <int WH>
struct RowGeneric {
  static constexpr size_t SMEM = sizeof(float2) * ((size_t)WH + 4 + IdxPad16::pad(WH) + 2 + WH +
                                                   FftTable<WH>::SIZE + 1);
};

// Largest divisor of WH that is <= kRowThreads (threads of one rowpass CTA).
constexpr int row_threads(int wh, int cand = kRowThreads) {
  return cand <= 1 ? 1 : (wh % cand == 0 ? cand : row_threads(wh, cand - 1));
}

template <int WH, int NT>
__global__ void __launch_bounds__(NT, 2)
    rowpass_kernel(const float2* __restrict__ Y, int y_rows, int Wcp, int n_c, int nb, int n_orient, int o0,
                   const int* __restrict__ o0_dev, float scale, float* __restrict__ mip, int* __restrict__ best,
                   double* __restrict__ s1, double* __restrict__ s2) {
  static_assert(NT >= FftThreads<WH>::value, "row FFT needs more threads");
  static_assert(WH % NT == 0, "row length must be a multiple of the CTA size");
  constexpr int PIX = WH / NT;
  constexpr int ZS = IdxPad16::pad(WH) + 2;
  // dynamic shared memory (RowGeneric<WH>::SMEM): row, transform, c2r
  // pre-twiddles and FFT twiddle table (filled once, reused by every correlogram)
  extern __shared__ float2 rgsm[];
  float2* xr = rgsm;
  float2* z = xr + WH + 4;
  float2* pre = z + ZS;
  float2* tab = pre + WH;
  const int y = blockIdx.x;
  const int t = threadIdx.x;
  fill_fft_table<WH>(tab, t, NT);
  for (int k = t; k < WH; k += NT) {
    float sn, cs;
    sincospif((float)k / (float)WH, &sn, &cs);
    pre[k] = make_float2(cs, sn);
  }
  float bmax[2 * PIX], bs[2 * PIX], bss[2 * PIX];
  int barg[2 * PIX];
#pragma unroll
  for (int i = 0; i < 2 * PIX; ++i) {
    bmax[i] = -INFINITY;
    barg[i] = 0;
    bs[i] = 0.f;
    bss[i] = 0.f;
  }
  for (int c = 0; c < n_c; ++c) {
    const float2* row = Y + ((size_t)c * y_rows + y) * Wcp;
    for (int k = t; k <= WH; k += NT) xr[k] = row[k];
    __syncthreads();
    for (int k = t; k < WH; k += NT) {
      float2 A = xr[k];
      float2 B = xr[WH - k];
      if (k == 0) { A.y = 0.f; B.y = 0.f; }
      B.y = -B.y;
      const float2 xe = cadd(A, B);
      const float2 xo = cmul(csub(A, B), pre[k]);
      z[IdxPad16::f(k)] = cadd(xe, mul_i<1>(xo));
    }
    __syncthreads();
    block_fft_tab<WH, NT, +1, IdxPad16>(z, tab, t);
#pragma unroll
    for (int r = 0; r < PIX; ++r) {
      const float2 v = z[IdxPad16::f(t + r * NT)];
      const float a = v.x * scale, b = v.y * scale;
      if (a > bmax[2 * r]) { bmax[2 * r] = a; barg[2 * r] = c; }
      if (b > bmax[2 * r + 1]) { bmax[2 * r + 1] = b; barg[2 * r + 1] = c; }
      bs[2 * r] += a;
      bss[2 * r] = fmaf(a, a, bss[2 * r]);
      bs[2 * r + 1] += b;
      bss[2 * r + 1] = fmaf(b, b, bss[2 * r + 1]);
    }
    __syncthreads();
  }
  const size_t W = 2 * (size_t)WH;
  if (o0_dev) o0 += *o0_dev;
#pragma unroll
  for (int r = 0; r < PIX; ++r) {
    const size_t idx = (size_t)y * W + 2 * (size_t)(t + r * NT);
    float2 m = *reinterpret_cast<float2*>(mip + idx);
    int2 bi = *reinterpret_cast<int2*>(best + idx);
    double2 a = *reinterpret_cast<double2*>(s1 + idx);
    double2 q = *reinterpret_cast<double2*>(s2 + idx);
    if (bmax[2 * r] > m.x) {
      m.x = bmax[2 * r];
      const int cc = barg[2 * r];
      bi.x = (cc / nb) * n_orient + o0 + (cc - (cc / nb) * nb);
    }
    if (bmax[2 * r + 1] > m.y) {
      m.y = bmax[2 * r + 1];
      const int cc = barg[2 * r + 1];
      bi.y = (cc / nb) * n_orient + o0 + (cc - (cc / nb) * nb);
    }
    a.x += f2d_bits(bs[2 * r]);
    a.y += f2d_bits(bs[2 * r + 1]);
    q.x += f2d_bits(bss[2 * r]);
    q.y += f2d_bits(bss[2 * r + 1]);
    *reinterpret_cast<float2*>(mip + idx) = m;
    *reinterpret_cast<int2*>(best + idx) = bi;
    *reinterpret_cast<double2*>(s1 + idx) = a;
    *reinterpret_cast<double2*>(s2 + idx) = q;
  }
}

}  // namespace lgb
