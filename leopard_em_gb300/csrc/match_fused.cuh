// Register-fused column and row passes of the plain FP32 search.
//
// colpass_fused_kernel<R, P>  (H = R^P, one butterfly per thread per pass)
//   The forward FFT's last Stockham pass leaves element j + q*H/R of the
//   column in thread j, and the inverse FFT's first pass consumes exactly those
//   elements in the same thread: forward-last -> cross power -> inverse-first
//   run in registers.  The pruned forward first pass reads its (at most two)
//   non-zero inputs straight from global memory, the inverse last pass writes
//   its outputs straight to global memory, so each correlogram column costs
//   four shared-memory round trips instead of eight.  Twiddles come from a
//   per-CTA shared table (built once with sincospif).  Thread layout: lane
//   bits 0-1 select one of four adjacent columns, so each warp touches 8 rows
//   x 32 B: whole sectors.
//
// rowpass_fused_kernel<WH, NT, Plan>  (W = 2*WH)
//   The c2r pre-twiddle (X[k], conj X[WH-k] -> Z[k]) is applied while the
//   first pass loads from the staged row; the last pass's outputs stay in
//   registers and feed the statistics directly.  Rows are staged with
//   cp.async double buffering (the next correlogram's row is in flight while
//   the current one is transformed).  Waits are cp.async.wait_group: no spins.
#pragma once

#include <type_traits>

#include "fft.cuh"
#include "match_kernels.cuh"

namespace lgb {

// ---- async copy helpers (16-byte cp.async, completion via wait_group) -------
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// L2 placement: measured, neither an evict_last policy on the image-spectrum
// loads nor streaming stores of the intermediate help -- both take L2 away
// from the correlogram rows that the row pass re-reads right after.

// exp(-2 pi i r / 16), r = 0..15 (roots for the sparse first pass; R | 16)
static __constant__ float2 kRootsFwd16[16] = {
    {1.0f, 0.0f},
    {0.92387953251128674f, -0.38268343236508977f},
    {0.70710678118654752f, -0.70710678118654752f},
    {0.38268343236508977f, -0.92387953251128674f},
    {0.0f, -1.0f},
    {-0.38268343236508977f, -0.92387953251128674f},
    {-0.70710678118654752f, -0.70710678118654752f},
    {-0.92387953251128674f, -0.38268343236508977f},
    {-1.0f, 0.0f},
    {-0.92387953251128674f, 0.38268343236508977f},
    {-0.70710678118654752f, 0.70710678118654752f},
    {-0.38268343236508977f, 0.92387953251128674f},
    {0.0f, 1.0f},
    {0.38268343236508977f, 0.92387953251128674f},
    {0.70710678118654752f, 0.70710678118654752f},
    {0.92387953251128674f, 0.38268343236508977f},
};

// Value of v that the compiler cannot treat as loop invariant: keeps per-row
// address arithmetic inside the loop instead of holding 16 hoisted addresses.
__device__ __forceinline__ int opaque(int v) {
  int r;
  asm volatile("mov.b32 %0, %1;" : "=r"(r) : "r"(v));
  return r;
}

// ---------------------------------------------------------------------------
// Fused column pass for H = R^P.
// ---------------------------------------------------------------------------
template <int R, int P>
struct UniformPlan;
template <int R>
struct UniformPlan<R, 2> {
  using type = Radices<R, R>;
  static constexpr int N = R * R;
};
template <int R>
struct UniformPlan<R, 3> {
  using type = Radices<R, R, R>;
  static constexpr int N = R * R * R;
};

template <int R, int P>
struct ColFused {
  using RL = typename UniformPlan<R, P>::type;
  static constexpr int N = UniformPlan<R, P>::N;
  static constexpr int NB = N / R;                    // butterflies per pass = threads per column
  static constexpr int THREADS = kColGroup * NB;
  static constexpr int STRIDE = IdxPad16::pad(N) + 4; // column stride in shared memory (float2)
  static constexpr int TAB = TableSize<1, RL>::value; // twiddle entries of passes 2..P
  static constexpr size_t SMEM = sizeof(float2) * (size_t)(kColGroup * STRIDE + TAB);
};

template <int R, int P>
__global__ void __launch_bounds__(ColFused<R, P>::THREADS, 1)
    colpass_fused_kernel(const float2* __restrict__ A, const float2* __restrict__ Ip, int h, int Wcp, int n_c,
                         int c_per_block, int c_per_image, int y_rows, float2* __restrict__ Y) {
  using CF = ColFused<R, P>;
  using RL = typename CF::RL;
  constexpr int N = CF::N, NB = CF::NB, STRIDE = CF::STRIDE;
  constexpr int NS_LAST = N / R;
  extern __shared__ float2 csm[];
  float2* tab = csm + kColGroup * STRIDE;
  FillTables<N, 1, RL>::run(tab, threadIdx.x, CF::THREADS);
  // twiddle sub-table of the last pass (stride NS_LAST)
  const float2* tab_last = tab + TableSize<1, typename DropLast<RL>::type>::value;
  const float2* tab_mid = tab;  // middle passes start at stride R (first pass has none)

  const int lane = threadIdx.x & 31;
  const int g = lane & 3;                             // column within the group
  const int j = (threadIdx.x >> 5) * 8 + (lane >> 2); // butterfly index
  float2* x = csm + g * STRIDE;
  const int kx = blockIdx.x * kColGroup + g;
  const int c_begin = blockIdx.y * c_per_block;
  const int c_end = min(n_c, c_begin + c_per_block);
  // first-pass sparse form: at most two non-zero inputs per butterfly when h <= 2*NB
  const bool sparse = h <= 2 * NB;
  __syncthreads();

  const int fj = IdxPad16::f(j);
  const int f1 = padded_first<R>(j);
  // sparse inputs of the first correlogram; later ones are prefetched one
  // correlogram ahead, while the current one runs its middle passes
  float2 nx0 = make_float2(0.f, 0.f), nx1 = make_float2(0.f, 0.f);
  if (sparse && c_begin < c_end) {
    const float2* a = A + (size_t)c_begin * h * Wcp + kx;
    if (j < h) nx0 = __ldg(a + (size_t)j * Wcp);
    if (j + NB < h) nx1 = __ldg(a + (size_t)(j + NB) * Wcp);
  }
#pragma unroll 1
  for (int c = c_begin; c < c_end; ++c) {
    float2 v[R];
    const size_t ws = (size_t)opaque(Wcp);  // row stride, re-derived per correlogram
    const float2* a = A + (size_t)c * h * ws + kx;
    // ---- forward pass 1 (stride 1, inputs from global, rows >= h are zero)
    if (sparse) {
      const float2 x0 = nx0, x1 = nx1;
      if (c + 1 < c_end) {
        const float2* an = a + (size_t)h * ws;
        nx0 = j < h ? __ldg(an + (size_t)j * ws) : make_float2(0.f, 0.f);
        nx1 = j + NB < h ? __ldg(an + (size_t)(j + NB) * ws) : make_float2(0.f, 0.f);
      }
      // y[r] = x0 + x1 * exp(-2 pi i r / R)
      static_assert(16 % R == 0, "sparse first pass needs R | 16");
#pragma unroll
      for (int r = 0; r < R; ++r) v[r] = cadd(x0, cmul(x1, kRootsFwd16[r * (16 / R)]));
    } else {
      const float2* ar = a + (size_t)j * ws;
#pragma unroll
      for (int q = 0; q < R; ++q) {
        v[q] = j + q * NB < h ? __ldg(ar) : make_float2(0.f, 0.f);
        ar += NB * ws;
      }
      Dft<R, -1>::run(v);
    }
#pragma unroll
    for (int q = 0; q < R; ++q) x[f1 + q] = v[q];
    __syncthreads();
    // ---- forward middle passes
    TablePasses<N, NB, -1, IdxPad16, R, typename Middle<RL>::type>::run(x, tab_mid, j);
    // ---- forward last pass -> registers
#pragma unroll
    for (int q = 0; q < R; ++q) v[q] = x[padded_at<IdxPad16, NB>(fj, j, q)];
    twiddle_from_table<R, -1, NS_LAST>(v, tab_last, j);
    Dft<R, -1>::run(v);
    // v[q] = P[row j + q*NB]; cross power with the image spectrum, P[0,0] = 0
    {
      const float2* ip = Ip + (size_t)(c / c_per_image) * N * ws + (size_t)j * ws + kx;
#pragma unroll
      for (int q = 0; q < R; ++q) {
        const float2 I = __ldg(ip);
        ip += NB * ws;
        v[q] = (q == 0 && j == 0 && kx == 0) ? make_float2(0.f, 0.f) : cmulc(I, v[q]);
      }
    }
    // ---- inverse pass 1 in registers (stride 1, no twiddles)
    Dft<R, +1>::run(v);
    __syncthreads();  // everyone has read the forward last pass inputs
#pragma unroll
    for (int q = 0; q < R; ++q) x[f1 + q] = v[q];
    __syncthreads();
    TablePasses<N, NB, +1, IdxPad16, R, typename Middle<RL>::type>::run(x, tab_mid, j);
    // ---- inverse last pass -> global
#pragma unroll
    for (int q = 0; q < R; ++q) v[q] = x[padded_at<IdxPad16, NB>(fj, j, q)];
    twiddle_from_table<R, +1, NS_LAST>(v, tab_last, j);
    Dft<R, +1>::run(v);
    float2* yo = Y + (size_t)c * y_rows * ws + (size_t)j * ws + kx;
#pragma unroll
    for (int q = 0; q < R; ++q) {
      if (j + q * NB < y_rows) *yo = v[q];
      yo += NB * ws;
    }
    __syncthreads();  // before the next correlogram's first-pass stores
  }
}

// ---------------------------------------------------------------------------
// Column pass for the mixed-radix lengths (those without a uniform R^P plan):
// the generic Stockham schedule of Plan<HN> with the twiddles of every pass
// after the first read from one shared table (filled once per CTA) instead
// of sincospif per butterfly.  The forward first pass is pruned to the h
// non-zero inputs.  G columns per CTA (ColGroupOf).
// ---------------------------------------------------------------------------
template <int HN>
struct ColTab {
  using RL = typename Plan<HN>::type;
  static constexpr int NT = FftThreads<HN>::value;
  // 288 (the refinement crops, 18 threads per column): 8 columns per CTA and
  // up to 4 CTAs per SM measured 3 % faster than 4 columns at one CTA
  static constexpr int G = HN == 288 ? 8 : ColGroupOf<HN>::value;
  static constexpr int MIN_BLOCKS = HN == 288 ? 4 : 1;
  static constexpr int STRIDE = IdxPad16::pad(HN) + 4;
  static constexpr int TAB = TableSize<1, RL>::value;
  static constexpr size_t SMEM = sizeof(float2) * ((size_t)G * STRIDE + TAB);
};

template <int HN>
__global__ void __launch_bounds__(ColTab<HN>::G* ColTab<HN>::NT, ColTab<HN>::MIN_BLOCKS)
    colpass_tab_kernel(const float2* __restrict__ A, const float2* __restrict__ Ip, int h, int Wcp, int n_c,
                       int c_per_block, int c_per_image, int y_rows, float2* __restrict__ Y) {
  using CT = ColTab<HN>;
  using RL = typename CT::RL;
  constexpr int NT = CT::NT, G = CT::G, STRIDE = CT::STRIDE, NTH = G * NT;
  constexpr int R1 = Head<RL>::value;
  extern __shared__ float2 ctsm[];
  float2* tab = ctsm + G * STRIDE;
  FillTables<HN, 1, RL>::run(tab, threadIdx.x, NTH);
  const int kx0 = blockIdx.x * G;
  const int c_begin = blockIdx.y * c_per_block;
  const int c_end = min(n_c, c_begin + c_per_block);
  const int g = threadIdx.x / NT, t = threadIdx.x - (threadIdx.x / NT) * NT;
  float2* x = ctsm + g * STRIDE;
  __syncthreads();
#pragma unroll 1
  for (int c = c_begin; c < c_end; ++c) {
    const float2* a = A + (size_t)c * h * Wcp + kx0;
    for (int e = threadIdx.x; e < h * G; e += NTH) {
      const int y = e / G, i = e % G;
      // the last group may run past Wcp when G does not divide it
      ctsm[i * STRIDE + IdxPad16::f(y)] = kx0 + i < Wcp ? a[(size_t)y * Wcp + i] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    // forward: pruned first pass (no twiddles), then the table passes
    stockham_pass<HN, R1, 1, NT, -1, IdxPad16, true>(x, t, h);
    TablePasses<HN, NT, -1, IdxPad16, R1, typename Tail<RL>::type>::run(x, tab, t);
    const float2* ipc = Ip + (size_t)(c / c_per_image) * HN * Wcp;
    for (int e = threadIdx.x; e < HN * G; e += NTH) {
      const int y = e / G, i = e % G;
      const float2 I = kx0 + i < Wcp ? __ldg(ipc + (size_t)y * Wcp + kx0 + i) : make_float2(0.f, 0.f);
      const int si = i * STRIDE + IdxPad16::f(y);
      float2 X = cmulc(I, ctsm[si]);
      if (y == 0 && kx0 + i == 0) X = make_float2(0.f, 0.f);
      ctsm[si] = X;
    }
    __syncthreads();
    TablePasses<HN, NT, +1, IdxPad16, 1, RL>::run(x, tab, t);
    float2* yo = Y + (size_t)c * y_rows * Wcp + kx0;
    for (int e = threadIdx.x; e < y_rows * G; e += NTH) {
      const int y = e / G, i = e % G;
      if (kx0 + i < Wcp) yo[(size_t)y * Wcp + i] = ctsm[i * STRIDE + IdxPad16::f(y)];
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Column pass for H = R1*R2 (288 = 16*18) in two register passes per
// direction.  Forward (Stockham): radix R1 over rows b + R2*q (pruned to the h
// non-zero rows, read from global) -> shared transpose M1[b][q] -> radix R2
// with twiddles w^(r*b), which leaves P[b + R1*r] in thread b; the cross
// power and the inverse's first pass (radix R2, stride 1: the same elements)
// stay in registers -> shared transpose M2[b][r] -> inverse radix R1 with
// twiddles w^(-q*b) -> rows b + R2*q to global.  Two shared round trips per
// column and correlogram; twiddle roots exp(-2 pi i m / H) for m = r*b <=
// (R1-1)(R2-1) from one shared table.  Odd transpose row strides and a column
// stride of 2 (mod 16) float2 make both transposes conflict free for the
// lane layout (8 columns x consecutive butterflies).
// ---------------------------------------------------------------------------
template <int R1, int R2>
struct ColPair {
  static constexpr int N = R1 * R2;
  static constexpr int NT = R1 > R2 ? R1 : R2;  // threads per column
  static constexpr int G = 8;                   // columns per CTA: 64 B row segments
  static constexpr int THREADS = G * NT;
  static constexpr int S1 = R1 + 1, S2 = R2 + 1;  // transpose row strides
  static_assert(S1 % 2 == 1 && S2 % 2 == 1, "odd transpose strides");
  static constexpr int CB = R2 * S1 > R1 * S2 ? R2 * S1 : R1 * S2;
  static constexpr int STRIDE = CB + (18 - CB % 16) % 16;  // = 2 (mod 16)
  static constexpr int NROOT = (R1 - 1) * (R2 - 1) + 1;
  static constexpr size_t SMEM = sizeof(float2) * ((size_t)G * STRIDE + NROOT);
};

template <int R1, int R2>
__global__ void __launch_bounds__(ColPair<R1, R2>::THREADS, 4)
    colpass_pair_kernel(const float2* __restrict__ A, const float2* __restrict__ Ip, int h, int Wcp, int n_c,
                        int c_per_block, int c_per_image, int y_rows, float2* __restrict__ Y,
                        const float2* __restrict__ norm, int norm_stride, int norm_w) {
  using CP = ColPair<R1, R2>;
  constexpr int N = CP::N, G = CP::G, S1 = CP::S1, S2 = CP::S2;
  extern __shared__ float2 psm[];
  float2* root = psm + G * CP::STRIDE;  // root[m] = exp(-2 pi i m / N)
  for (int m = threadIdx.x; m < CP::NROOT; m += CP::THREADS) {
    float sn, cs;
    sincospif(2.0f * (float)m / (float)N, &sn, &cs);
    root[m] = make_float2(cs, -sn);
  }
  const int g = threadIdx.x % G, b = threadIdx.x / G;
  const int kx = blockIdx.x * G + g;
  const bool col_ok = kx < Wcp;  // the last group may run past Wcp
  float2* x = psm + g * CP::STRIDE;
  const int c_begin = blockIdx.y * c_per_block;
  const int c_end = min(n_c, c_begin + c_per_block);
  // deferred normalisation: rfft_W((p - e) s) = s (A - e U), U[k] = sum_{x<h} w^(k x)
  // = exp(-i pi k (h-1) / W) sin(pi k h / W) / sin(pi k / W), w = exp(-2 pi i / W)
  float2 U = make_float2(0.f, 0.f);
  if (norm && col_ok && kx <= norm_w / 2) {
    if (kx == 0) {
      U = make_float2((float)h, 0.f);
    } else {
      const int w2 = 2 * norm_w;
      float sa, ca, sn, cn, sd, cd;
      sincospif((float)((kx * (h - 1)) % w2) / (float)norm_w, &sa, &ca);
      sincospif((float)((kx * h) % w2) / (float)norm_w, &sn, &cn);
      sincospif((float)kx / (float)norm_w, &sd, &cd);
      const float mag = sn / sd;
      U = make_float2(ca * mag, -sa * mag);
    }
  }
  __syncthreads();
#pragma unroll 1
  for (int c = c_begin; c < c_end; ++c) {
    // ---- forward pass 1 (radix R1, stride 1): rows b + R2*q, rows >= h are zero
    if (b < R2) {
      float2 v[R1];
      const float2* a = A + ((size_t)c * h + b) * Wcp + kx;
#pragma unroll
      for (int q = 0; q < R1; ++q)
        v[q] = (col_ok && b + q * R2 < h) ? __ldg(a + (size_t)q * R2 * Wcp) : make_float2(0.f, 0.f);
      if (norm) {
        const float2 es = __ldg(norm + (size_t)c * norm_stride);
        const float2 eU = make_float2(es.x * U.x, es.x * U.y);
#pragma unroll
        for (int q = 0; q < R1; ++q)
          if (b + q * R2 < h) v[q] = make_float2(es.y * (v[q].x - eU.x), es.y * (v[q].y - eU.y));
      }
      Dft<R1, -1>::run(v);
#pragma unroll
      for (int q = 0; q < R1; ++q) x[b * S1 + q] = v[q];
    }
    __syncthreads();
    float2 w[R2];
    if (b < R1) {
      // ---- forward pass 2 (radix R2, stride R1): w[r] = P[row b + R1*r]
#pragma unroll
      for (int r = 0; r < R2; ++r) w[r] = cmul(x[r * S1 + b], root[r * b]);
      Dft<R2, -1>::run(w);
      // ---- cross power with the image spectrum, P[0,0] = 0
      const float2* ip = Ip + ((size_t)(c / c_per_image) * N + b) * Wcp + kx;
#pragma unroll
      for (int r = 0; r < R2; ++r) {
        const float2 I = col_ok ? __ldg(ip + (size_t)r * R1 * Wcp) : make_float2(0.f, 0.f);
        w[r] = (r == 0 && b == 0 && kx == 0) ? make_float2(0.f, 0.f) : cmulc(I, w[r]);
      }
      // ---- inverse pass 1 (radix R2, stride 1) on the same elements
      Dft<R2, +1>::run(w);
    }
    __syncthreads();  // every read of M1 is done
    if (b < R1) {
#pragma unroll
      for (int r = 0; r < R2; ++r) x[b * S2 + r] = w[r];
    }
    __syncthreads();
    // ---- inverse pass 2 (radix R1, stride R2) -> rows b + R2*q
    if (b < R2) {
      float2 v[R1];
#pragma unroll
      for (int q = 0; q < R1; ++q) v[q] = cmulc(x[q * S2 + b], root[q * b]);
      Dft<R1, +1>::run(v);
      if (col_ok) {
        float2* yo = Y + ((size_t)c * y_rows + b) * Wcp + kx;
#pragma unroll
        for (int q = 0; q < R1; ++q)
          if (b + q * R2 < y_rows) yo[(size_t)q * R2 * Wcp] = v[q];
      }
    }
    __syncthreads();  // before the next correlogram's pass-1 stores
  }
}

// ---------------------------------------------------------------------------
// Fused row pass (c2r of length 2*WH + statistics).
// ---------------------------------------------------------------------------
template <int WH, int NT, class RL>
struct RowFused {
  static constexpr int R1 = Head<RL>::value;
  static constexpr int RLAST = Last<RL>::value;
  static constexpr int NB1 = WH / R1;
  static constexpr int PER1 = (NB1 + NT - 1) / NT;
  static constexpr int NBL = WH / RLAST;
  static constexpr int PERL = NBL / NT;
  // the 8, 8 middle passes of 2048 = 8 8 8 4 store / load through the 16x2 layout
  static constexpr bool MID88 = std::is_same<typename Middle<RL>::type, Radices<8, 8>>::value;
  static constexpr int ZS = (MID88 ? IdxPad16x2::pad(WH) : IdxPad16::pad(WH)) + 2;
  static constexpr int TAB = TableSize<1, RL>::value;
  static_assert(NBL % NT == 0, "last pass must give every thread whole butterflies");
  static_assert(NB1 <= NT * PER1, "first pass coverage");
  static_assert(16 % (2 * R1) == 0, "pre-twiddle roots exp(i pi q / R1) come from the 16th roots");
  static size_t smem(int wcp) { return sizeof(float2) * (size_t)(2 * wcp + ZS + TAB); }
};

template <int WH, int NT, class RL, int MINB = 3>
__global__ void __launch_bounds__(NT, MINB)
    rowpass_fused_kernel(const float2* __restrict__ Y, int y_rows, int Wcp, int n_c, int nb, int n_orient, int o0,
                         const int* __restrict__ o0_dev, float scale, float* __restrict__ mip,
                         int* __restrict__ best, double* __restrict__ s1, double* __restrict__ s2) {
  using RF = RowFused<WH, NT, RL>;
  constexpr int R1 = RF::R1, RLAST = RF::RLAST, NB1 = RF::NB1, PER1 = RF::PER1, NBL = RF::NBL, PERL = RF::PERL;
  constexpr int OUT = PERL * RLAST;  // complex outputs (pixel pairs) per thread
  extern __shared__ float2 rsm[];
  float2* xr0 = rsm;
  float2* xr1 = rsm + Wcp;
  float2* z = rsm + 2 * Wcp;
  float2* tab = z + RF::ZS;
  const int y = blockIdx.x;
  const int t = threadIdx.x;
  const int n16 = Wcp / 2;  // 16-byte chunks per row

  // stage row 0 while the tables are built
  {
    const float2* src = Y + (size_t)y * Wcp;
    for (int i = t; i < n16; i += NT) cp_async16(xr0 + 2 * i, src + 2 * i);
    cp_async_commit();
  }
  FillTables<WH, 1, RL>::run(tab, t, NT);
  // c2r pre-twiddle exp(+i pi k / WH) at k = j + q*NB1 factors into
  // exp(+i pi j / WH) (per thread, kept in registers) x exp(+i pi q / R1)
  float2 prej[PER1];
#pragma unroll
  for (int p = 0; p < PER1; ++p) {
    float sn, cs;
    sincospif((float)(t + p * NT) / (float)WH, &sn, &cs);
    prej[p] = make_float2(cs, sn);
  }
  const float2* tab_last = tab + TableSize<1, typename DropLast<RL>::type>::value;

  float bmax[2 * OUT], bs[2 * OUT], bss[2 * OUT];
  unsigned barg[OUT];  // batch index of each pixel pair's maxima: low / high 16 bits
#pragma unroll
  for (int i = 0; i < 2 * OUT; ++i) {
    bmax[i] = -INFINITY;
    bs[i] = 0.f;
    bss[i] = 0.f;
  }
#pragma unroll
  for (int i = 0; i < OUT; ++i) barg[i] = 0u;

#pragma unroll 1
  for (int c = 0; c < n_c; ++c) {
    const float2* xr = (c & 1) ? xr1 : xr0;
    if (c + 1 < n_c) {
      float2* nxt = (c & 1) ? xr0 : xr1;
      const float2* src = Y + ((size_t)(c + 1) * y_rows + y) * Wcp;
      for (int i = t; i < n16; i += NT) cp_async16(nxt + 2 * i, src + 2 * i);
      cp_async_commit();
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    // ---- pass 1: pre-twiddle while loading, no twiddles (stride 1)
    {
      float2 v[PER1][R1];
#pragma unroll
      for (int p = 0; p < PER1; ++p) {
        const int j = t + p * NT;
        if ((NB1 % NT == 0) || j < NB1) {
#pragma unroll
          for (int q = 0; q < R1; ++q) {
            const int k = j + q * NB1;
            float2 a = xr[k];
            float2 b = xr[WH - k];
            if (k == 0) {
              a.y = 0.f;
              b.y = 0.f;
            }
            b.y = -b.y;
            float2 xo = cmul(csub(a, b), prej[p]);
            if (q) xo = cmulc(xo, kRootsFwd16[q * (16 / (2 * R1))]);
            v[p][q] = cadd(cadd(a, b), mul_i<1>(xo));
          }
          Dft<R1, +1>::run(v[p]);
        }
      }
#pragma unroll
      for (int p = 0; p < PER1; ++p) {
        const int j = t + p * NT;
        if ((NB1 % NT == 0) || j < NB1) {
#pragma unroll
          for (int q = 0; q < R1; ++q) z[IdxPad16::f(j * R1 + q)] = v[p][q];
        }
      }
    }
    __syncthreads();
    if constexpr (RF::MID88) {
      // stride-8 radix-8 stores into the 16x2 layout, read back by the
      // stride-64 pass, which stores the plain padded layout again
      table_pass_io<WH, 8, R1, NT, +1, IdxPad16, IdxPad16x2>(z, tab, t);
      table_pass_io<WH, 8, R1 * 8, NT, +1, IdxPad16x2, IdxPad16>(z, tab + R1 * 7, t);
    } else {
      TablePasses<WH, NT, +1, IdxPad16, R1, typename Middle<RL>::type>::run(z, tab, t);
    }
    // ---- last pass -> registers -> statistics
#pragma unroll
    for (int p = 0; p < PERL; ++p) {
      const int j = t + p * NT;
      float2 v[RLAST];
#pragma unroll
      for (int q = 0; q < RLAST; ++q) v[q] = z[IdxPad16::f(j + q * NBL)];
      twiddle_from_table<RLAST, +1, NBL>(v, tab_last, j);
      Dft<RLAST, +1>::run(v);
#pragma unroll
      for (int q = 0; q < RLAST; ++q) {
        const int o = 2 * (p * RLAST + q);
        const float a = v[q].x * scale, b = v[q].y * scale;
        const int k = p * RLAST + q;
        if (a > bmax[o]) { bmax[o] = a; barg[k] = (barg[k] & 0xffff0000u) | (unsigned)c; }
        if (b > bmax[o + 1]) { bmax[o + 1] = b; barg[k] = (barg[k] & 0xffffu) | ((unsigned)c << 16); }
        bs[o] += a;
        bss[o] = fmaf(a, a, bss[o]);
        bs[o + 1] += b;
        bss[o + 1] = fmaf(b, b, bss[o + 1]);
      }
    }
    __syncthreads();
  }

  const size_t W = 2 * (size_t)WH;
  if (o0_dev) o0 += *o0_dev;
#pragma unroll
  for (int p = 0; p < PERL; ++p) {
#pragma unroll
    for (int q = 0; q < RLAST; ++q) {
      const int o = 2 * (p * RLAST + q);
      const int m = t + p * NT + q * NBL;
      const size_t idx = (size_t)y * W + 2 * (size_t)m;
      float2 mm = *reinterpret_cast<float2*>(mip + idx);
      int2 bi = *reinterpret_cast<int2*>(best + idx);
      double2 sa = *reinterpret_cast<double2*>(s1 + idx);
      double2 sq = *reinterpret_cast<double2*>(s2 + idx);
      if (bmax[o] > mm.x) {
        mm.x = bmax[o];
        const int cc = (int)(barg[p * RLAST + q] & 0xffffu);
        bi.x = (cc / nb) * n_orient + o0 + (cc - (cc / nb) * nb);
      }
      if (bmax[o + 1] > mm.y) {
        mm.y = bmax[o + 1];
        const int cc = (int)(barg[p * RLAST + q] >> 16);
        bi.y = (cc / nb) * n_orient + o0 + (cc - (cc / nb) * nb);
      }
      sa.x += f2d_bits(bs[o]);
      sa.y += f2d_bits(bs[o + 1]);
      sq.x += f2d_bits(bss[o]);
      sq.y += f2d_bits(bss[o + 1]);
      *reinterpret_cast<float2*>(mip + idx) = mm;
      *reinterpret_cast<int2*>(best + idx) = bi;
      *reinterpret_cast<double2*>(s1 + idx) = sa;
      *reinterpret_cast<double2*>(s2 + idx) = sq;
    }
  }
}

}  // namespace lgb
