// Block-cooperative mixed-radix Stockham FFT in shared memory.
//
// A length-N transform lives in shared memory (optionally with a padded index
// map to break bank conflicts).  Each pass of radix R loads R strided values
// per butterfly into registers, applies the twiddles w^(t*k) with
// w = exp(DIR * 2*pi*i / (Ns*R)), k = j mod Ns, does an in-register R-point
// DFT and writes the results to their autosorted positions
// (j/Ns)*Ns*R + k + q*Ns.  After the last pass the data is in natural order.
// All passes are separated by __syncthreads(), so every thread of the CTA must
// call the transform (threads with no butterfly simply idle).
//
// DIR = -1 is the forward transform exp(-2*pi*i*k*n/N); DIR = +1 the unscaled
// inverse.  Twiddle bases come from sincospif (accurate to ~1 ulp) and their
// powers from a short multiplication chain.
#pragma once

#include <type_traits>

#include "common.cuh"

namespace lgb {

// ---------------------------------------------------------------------------
// In-register DFTs:  y[q] = sum_t x[t] * exp(DIR*2*pi*i*t*q/R)
// ---------------------------------------------------------------------------

template <int DIR>
__device__ __forceinline__ void dft2(float2& a, float2& b) {
  float2 t = a;
  a = cadd(t, b);
  b = csub(t, b);
}

template <int DIR>
__device__ __forceinline__ void dft4(float2& x0, float2& x1, float2& x2, float2& x3) {
  float2 a = cadd(x0, x2), b = csub(x0, x2);
  float2 c = cadd(x1, x3), d = mul_i<DIR>(csub(x1, x3));
  x0 = cadd(a, c);
  x2 = csub(a, c);
  x1 = cadd(b, d);
  x3 = csub(b, d);
}

template <int R, int DIR>
struct Dft;

template <int DIR>
struct Dft<2, DIR> {
  static __device__ __forceinline__ void run(float2* v) { dft2<DIR>(v[0], v[1]); }
};

template <int DIR>
struct Dft<3, DIR> {
  static __device__ __forceinline__ void run(float2* v) {
    const float s3 = 0.86602540378443865f;
    float2 t1 = cadd(v[1], v[2]);
    float2 t2 = make_float2(fmaf(-0.5f, t1.x, v[0].x), fmaf(-0.5f, t1.y, v[0].y));
    float2 t3 = mul_i<DIR>(cscale(csub(v[1], v[2]), s3));
    v[0] = cadd(v[0], t1);
    v[1] = cadd(t2, t3);
    v[2] = csub(t2, t3);
  }
};

template <int DIR>
struct Dft<4, DIR> {
  static __device__ __forceinline__ void run(float2* v) { dft4<DIR>(v[0], v[1], v[2], v[3]); }
};

template <int DIR>
struct Dft<5, DIR> {
  static __device__ __forceinline__ void run(float2* v) {
    const float c1 = 0.30901699437494742f, c2 = -0.80901699437494742f;
    const float s1 = 0.95105651629515357f, s2 = 0.58778525229247313f;
    float2 p14 = cadd(v[1], v[4]), m14 = csub(v[1], v[4]);
    float2 p23 = cadd(v[2], v[3]), m23 = csub(v[2], v[3]);
    float2 x0 = v[0];
    float2 a1 = make_float2(x0.x + c1 * p14.x + c2 * p23.x, x0.y + c1 * p14.y + c2 * p23.y);
    float2 a2 = make_float2(x0.x + c2 * p14.x + c1 * p23.x, x0.y + c2 * p14.y + c1 * p23.y);
    float2 b1 = mul_i<DIR>(make_float2(s1 * m14.x + s2 * m23.x, s1 * m14.y + s2 * m23.y));
    float2 b2 = mul_i<DIR>(make_float2(s2 * m14.x - s1 * m23.x, s2 * m14.y - s1 * m23.y));
    v[0] = cadd(x0, cadd(p14, p23));
    v[1] = cadd(a1, b1);
    v[4] = csub(a1, b1);
    v[2] = cadd(a2, b2);
    v[3] = csub(a2, b2);
  }
};

template <int DIR>
struct Dft<8, DIR> {
  // y[2k] = DFT4(x_i + x_{i+4})[k];  y[2k+1] = DFT4((x_i - x_{i+4}) w8^i)[k]
  static __device__ __forceinline__ void run(float2* v) {
    const float r2 = 0.70710678118654752f;
    float2 a0 = cadd(v[0], v[4]), a1 = cadd(v[1], v[5]), a2 = cadd(v[2], v[6]), a3 = cadd(v[3], v[7]);
    float2 b0 = csub(v[0], v[4]), b1 = csub(v[1], v[5]), b2 = csub(v[2], v[6]), b3 = csub(v[3], v[7]);
    // w8^1 = (1 + DIR i)/sqrt2, w8^2 = DIR i, w8^3 = (-1 + DIR i)/sqrt2
    b1 = cscale(cadd(b1, mul_i<DIR>(b1)), r2);
    b2 = mul_i<DIR>(b2);
    b3 = cscale(csub(mul_i<DIR>(b3), b3), r2);
    dft4<DIR>(a0, a1, a2, a3);
    dft4<DIR>(b0, b1, b2, b3);
    v[0] = a0; v[2] = a1; v[4] = a2; v[6] = a3;
    v[1] = b0; v[3] = b1; v[5] = b2; v[7] = b3;
  }
};

template <int DIR>
struct Dft<16, DIR> {
  // 4 x 4:  u_i = DFT4(x_i, x_{i+4}, x_{i+8}, x_{i+12});
  //         y[q1 + 4 q2] = DFT4_i(u_i[q1] * w16^(i q1))[q2]
  static __device__ __forceinline__ void run(float2* v) {
    const float c1 = 0.92387953251128674f, s1 = 0.38268343236508977f, r2 = 0.70710678118654752f;
#pragma unroll
    for (int i = 0; i < 4; ++i) dft4<DIR>(v[i], v[i + 4], v[i + 8], v[i + 12]);
    // now v[i + 4*q1] = u_i[q1]; twiddle by w16^(i*q1), w16^m = (cos(2pi m/16), DIR sin(2pi m/16))
    auto tw = [](float2 a, float c, float s) {  // a * (c + DIR*i*s)
      float ss = DIR > 0 ? s : -s;
      return make_float2(a.x * c - a.y * ss, a.x * ss + a.y * c);
    };
    v[5] = tw(v[5], c1, s1);     // i=1,q1=1: m=1
    v[9] = tw(v[9], r2, r2);     // i=1,q1=2: m=2
    v[13] = tw(v[13], s1, c1);   // i=1,q1=3: m=3
    v[6] = tw(v[6], r2, r2);     // i=2,q1=1: m=2
    v[10] = mul_i<DIR>(v[10]);   // i=2,q1=2: m=4
    v[14] = tw(v[14], -r2, r2);  // i=2,q1=3: m=6
    v[7] = tw(v[7], s1, c1);     // i=3,q1=1: m=3
    v[11] = tw(v[11], -r2, r2);  // i=3,q1=2: m=6
    v[15] = tw(v[15], -c1, -s1); // i=3,q1=3: m=9
#pragma unroll
    for (int q1 = 0; q1 < 4; ++q1) dft4<DIR>(v[4 * q1], v[4 * q1 + 1], v[4 * q1 + 2], v[4 * q1 + 3]);
    // v[4*q1 + q2] = y[q1 + 4*q2]; transpose 4x4 into natural order
    float2 t[16];
#pragma unroll
    for (int q1 = 0; q1 < 4; ++q1)
#pragma unroll
      for (int q2 = 0; q2 < 4; ++q2) t[q1 + 4 * q2] = v[4 * q1 + q2];
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = t[i];
  }
};

template <int DIR>
struct Dft<9, DIR> {
  // 3 x 3:  u_i = DFT3(x_i, x_{i+3}, x_{i+6});
  //         y[q1 + 3 q2] = DFT3_i(u_i[q1] * w9^(i q1))[q2]
  static __device__ __forceinline__ void run(float2* v) {
    // w9^m = (cos(2 pi m/9), DIR sin(2 pi m/9)), m = 1, 2, 4
    const float c1 = 0.76604444311897804f, s1 = 0.64278760968653933f;
    const float c2 = 0.17364817766693035f, s2 = 0.98480775301220806f;
    const float c4 = -0.93969262078590838f, s4 = 0.34202014332566873f;
    auto tw = [](float2 a, float c, float s) {  // a * (c + DIR*i*s)
      float ss = DIR > 0 ? s : -s;
      return make_float2(a.x * c - a.y * ss, a.x * ss + a.y * c);
    };
    float2 u[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      u[i][0] = v[i];
      u[i][1] = v[i + 3];
      u[i][2] = v[i + 6];
      Dft<3, DIR>::run(u[i]);
    }
    u[1][1] = tw(u[1][1], c1, s1);
    u[1][2] = tw(u[1][2], c2, s2);
    u[2][1] = tw(u[2][1], c2, s2);
    u[2][2] = tw(u[2][2], c4, s4);
#pragma unroll
    for (int q1 = 0; q1 < 3; ++q1) {
      float2 t[3] = {u[0][q1], u[1][q1], u[2][q1]};
      Dft<3, DIR>::run(t);
      v[q1] = t[0];
      v[q1 + 3] = t[1];
      v[q1 + 6] = t[2];
    }
  }
};

template <int DIR>
struct Dft<18, DIR> {
  // Prime-factor (Good-Thomas) 2 x 9, no twiddles: input n = (9 n1 + 2 n2) mod 18,
  // output k = (9 k1 + 10 k2) mod 18 (CRT map: 9 = 1 mod 2, 10 = 1 mod 9).
  static __device__ __forceinline__ void run(float2* v) {
    float2 a[9], b[9];
#pragma unroll
    for (int n2 = 0; n2 < 9; ++n2) {
      const float2 x0 = v[(2 * n2) % 18], x1 = v[(9 + 2 * n2) % 18];
      a[n2] = cadd(x0, x1);
      b[n2] = csub(x0, x1);
    }
    Dft<9, DIR>::run(a);
    Dft<9, DIR>::run(b);
#pragma unroll
    for (int k2 = 0; k2 < 9; ++k2) {
      v[(10 * k2) % 18] = a[k2];
      v[(9 + 10 * k2) % 18] = b[k2];
    }
  }
};

// ---------------------------------------------------------------------------
// Twiddles w^t, t = 1..R-1, w = exp(DIR*2*pi*i*k/L)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 unit_root(float frac, int dir) {  // exp(dir * i * pi * frac)
  float s, c;
  sincospif(frac, &s, &c);
  return make_float2(c, dir > 0 ? s : -s);
}

// Few live registers: w1, w2 = w1^2, w3 = w2 w1 from one sincospif, w4 from a
// second accurate sincospif; w^(4a+b) = (w4)^a * w^b.  Longest product chain
// is 4 multiplies, so twiddle error stays within a few ulp.
template <int R, int DIR>
__device__ __forceinline__ void apply_twiddles(float2* v, int k, int L) {
  const float frac = 2.0f * (float)k / (float)L;
  const float2 w1 = unit_root(frac, DIR);
  v[1] = cmul(v[1], w1);
  if (R == 2) return;
  const float2 w2 = cmul(w1, w1);
  v[2] = cmul(v[2], w2);
  if (R == 3) return;
  const float2 w3 = cmul(w2, w1);
  v[3] = cmul(v[3], w3);
  if (R == 4) return;
  if (R == 5) {
    v[4] = cmul(v[4], cmul(w2, w2));
    return;
  }
  const float2 w4 = unit_root(4.0f * frac, DIR);
  float2 wa = w4;
#pragma unroll
  for (int a = 1; a < R / 4; ++a) {
    if (a > 1) wa = cmul(wa, w4);
    v[4 * a] = cmul(v[4 * a], wa);
    v[4 * a + 1] = cmul(v[4 * a + 1], cmul(wa, w1));
    v[4 * a + 2] = cmul(v[4 * a + 2], cmul(wa, w2));
    v[4 * a + 3] = cmul(v[4 * a + 3], cmul(wa, w3));
  }
}

// Index maps for the shared-memory buffer.
struct IdxPlain {
  __host__ __device__ static constexpr int pad(int n) { return n; }
  static __device__ __forceinline__ int f(int i) { return i; }
};
// one float2 of padding per 16 elements: stride-16 accesses become conflict free
struct IdxPad16 {
  __host__ __device__ static constexpr int pad(int n) { return n + n / 16; }
  static __device__ __forceinline__ int f(int i) { return i + (i >> 4); }
};

// two float2 of padding per 16 elements: the layout between the two radix-8
// middle passes of a 2048-point transform, where the stride-8 stores of the
// first and the stride-256 loads of the second are both conflict free
struct IdxPad16x2 {
  __host__ __device__ static constexpr int pad(int n) { return n + 2 * (n / 16); }
  static __device__ __forceinline__ int f(int i) { return i + 2 * (i >> 4); }
};

// One Stockham pass.  NZ >= 0 marks a pruned first pass whose inputs at index
// >= nz are known zeros (nz given at run time); they are not read.
template <int N, int R, int NS, int NT, int DIR, class IDX, bool PRUNED>
__device__ __forceinline__ void stockham_pass(float2* __restrict__ x, int t, int nz) {
  constexpr int NB = N / R;
  constexpr int PER = (NB + NT - 1) / NT;
  float2 v[PER][R];
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int j = t + p * NT;
    if ((NB % NT == 0) || j < NB) {
#pragma unroll
      for (int q = 0; q < R; ++q) {
        const int src = j + q * NB;
        if (PRUNED)
          v[p][q] = (src < nz) ? x[IDX::f(src)] : make_float2(0.f, 0.f);
        else
          v[p][q] = x[IDX::f(src)];
      }
      if (NS > 1) apply_twiddles<R, DIR>(v[p], j % NS, NS * R);
      Dft<R, DIR>::run(v[p]);
    }
  }
  __syncthreads();
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int j = t + p * NT;
    if ((NB % NT == 0) || j < NB) {
      const int k = j % NS;
      const int base = (j / NS) * NS * R + k;
#pragma unroll
      for (int q = 0; q < R; ++q) x[IDX::f(base + q * NS)] = v[p][q];
    }
  }
  __syncthreads();
}

template <int... Rs>
struct Radices {};

// Radix plans (product must equal N).  Larger radices first.
template <int N>
struct Plan;
#define LGB_PLAN(N, ...)                    \
  template <>                               \
  struct Plan<N> {                          \
    using type = Radices<__VA_ARGS__>;      \
  };
LGB_PLAN(8, 8)
LGB_PLAN(16, 16)
LGB_PLAN(20, 5, 4)
LGB_PLAN(24, 8, 3)
LGB_PLAN(32, 8, 4)
LGB_PLAN(40, 8, 5)
LGB_PLAN(48, 16, 3)
LGB_PLAN(64, 8, 8)
LGB_PLAN(72, 8, 3, 3)
LGB_PLAN(80, 16, 5)
LGB_PLAN(96, 8, 4, 3)
LGB_PLAN(128, 16, 8)
LGB_PLAN(144, 16, 3, 3)
LGB_PLAN(160, 8, 4, 5)
LGB_PLAN(192, 16, 4, 3)
LGB_PLAN(256, 16, 16)
LGB_PLAN(288, 16, 2, 3, 3)
LGB_PLAN(384, 16, 8, 3)
LGB_PLAN(512, 8, 8, 8)
LGB_PLAN(576, 16, 4, 3, 3)
LGB_PLAN(768, 16, 16, 3)
LGB_PLAN(1024, 16, 8, 8)
LGB_PLAN(1440, 16, 5, 3, 3, 2)
LGB_PLAN(1536, 16, 8, 4, 3)
LGB_PLAN(1920, 16, 8, 5, 3)
LGB_PLAN(2048, 8, 16, 16)
LGB_PLAN(2880, 16, 4, 5, 3, 3)
LGB_PLAN(3072, 16, 16, 4, 3)
LGB_PLAN(3840, 16, 16, 5, 3)
LGB_PLAN(4096, 16, 16, 16)
LGB_PLAN(5760, 16, 8, 5, 3, 3)
#undef LGB_PLAN

template <int N, int NT, int DIR, class IDX, int NS, bool PRUNED, class RL>
struct Passes;
template <int N, int NT, int DIR, class IDX, int NS, bool PRUNED>
struct Passes<N, NT, DIR, IDX, NS, PRUNED, Radices<>> {
  static __device__ __forceinline__ void run(float2*, int, int) {}
};
template <int N, int NT, int DIR, class IDX, int NS, bool PRUNED, int R, int... Rs>
struct Passes<N, NT, DIR, IDX, NS, PRUNED, Radices<R, Rs...>> {
  static __device__ __forceinline__ void run(float2* x, int t, int nz) {
    stockham_pass<N, R, NS, NT, DIR, IDX, PRUNED && NS == 1>(x, t, nz);
    Passes<N, NT, DIR, IDX, NS * R, PRUNED, Radices<Rs...>>::run(x, t, nz);
  }
};

template <class RL>
struct MinRadix;
template <int R>
struct MinRadix<Radices<R>> {
  static constexpr int value = R;
};
template <int R, int R2, int... Rs>
struct MinRadix<Radices<R, R2, Rs...>> {
  static constexpr int value = R < MinRadix<Radices<R2, Rs...>>::value ? R : MinRadix<Radices<R2, Rs...>>::value;
};
template <class RL>
struct MaxRadix;
template <int R>
struct MaxRadix<Radices<R>> {
  static constexpr int value = R;
};
template <int R, int R2, int... Rs>
struct MaxRadix<Radices<R, R2, Rs...>> {
  static constexpr int value = R > MaxRadix<Radices<R2, Rs...>>::value ? R : MaxRadix<Radices<R2, Rs...>>::value;
};

// Threads that make every pass of the plan one butterfly per thread at most
// for the largest radix (smaller radices loop).
template <int N>
struct FftThreads {
  static constexpr int value = N / MaxRadix<typename Plan<N>::type>::value;
};

// In-place transform of x[IDX::f(0..N-1)], cooperatively by NT threads (t in [0,NT)).
template <int N, int NT, int DIR, class IDX = IdxPlain>
__device__ __forceinline__ void block_fft(float2* x, int t) {
  Passes<N, NT, DIR, IDX, 1, false, typename Plan<N>::type>::run(x, t, N);
}
// Out-of-line variants: a separate register allocation for the transform, so
// that a caller with a tight register budget (1024-thread CTAs) does not keep
// hoisted twiddles of both directions live across its own loop.
template <int N, int NT, int DIR, class IDX = IdxPlain>
__device__ __noinline__ void block_fft_outline(float2* x, int t) {
  Passes<N, NT, DIR, IDX, 1, false, typename Plan<N>::type>::run(x, t, N);
}
template <int N, int NT, int DIR, class IDX = IdxPlain>
__device__ __noinline__ void block_fft_pruned_outline(float2* x, int t, int nz) {
  Passes<N, NT, DIR, IDX, 1, true, typename Plan<N>::type>::run(x, t, nz);
}
// Same, with inputs at index >= nz known to be zero (first pass skips them).
template <int N, int NT, int DIR, class IDX = IdxPlain>
__device__ __forceinline__ void block_fft_pruned(float2* x, int t, int nz) {
  Passes<N, NT, DIR, IDX, 1, true, typename Plan<N>::type>::run(x, t, nz);
}

// ---- radix-list helpers ----------------------------------------------------
template <class RL>
struct Head;
template <int R, int... Rs>
struct Head<Radices<R, Rs...>> {
  static constexpr int value = R;
};
template <class RL>
struct Last;
template <int R>
struct Last<Radices<R>> {
  static constexpr int value = R;
};
template <int R, int R2, int... Rs>
struct Last<Radices<R, R2, Rs...>> {
  static constexpr int value = Last<Radices<R2, Rs...>>::value;
};
template <int R, class RL>
struct Prepend;
template <int R, int... Rs>
struct Prepend<R, Radices<Rs...>> {
  using type = Radices<R, Rs...>;
};
template <class RL>
struct DropLast;
template <int R>
struct DropLast<Radices<R>> {
  using type = Radices<>;
};
template <int R, int R2, int... Rs>
struct DropLast<Radices<R, R2, Rs...>> {
  using type = typename Prepend<R, typename DropLast<Radices<R2, Rs...>>::type>::type;
};
template <class RL>
struct Tail;
template <int R, int... Rs>
struct Tail<Radices<R, Rs...>> {
  using type = Radices<Rs...>;
};
// middle passes: drop first and last
template <class RL>
struct Middle {
  using type = typename DropLast<typename Tail<RL>::type>::type;
};

// Padded shared-memory access at base + q*STEP.  With IdxPad16 and STEP a
// multiple of 16, f(base + q*STEP) = f(base) + q*(STEP + STEP/16): one index
// computation and compile-time offsets for the whole butterfly.
template <class IDX, int STEP>
__device__ __forceinline__ int padded_at(int fbase, int base, int q) {
  if constexpr (std::is_same<IDX, IdxPad16>::value && STEP % 16 == 0) {
    return fbase + q * (STEP + STEP / 16);
  } else if constexpr (std::is_same<IDX, IdxPad16x2>::value && STEP % 16 == 0) {
    return fbase + q * (STEP + 2 * (STEP / 16));
  } else {
    return IDX::f(base + q * STEP);
  }
}
// f(R*j + q) for q < R <= 16 and R | 16: R*j + (R*j >> 4) + q.
template <int R>
__device__ __forceinline__ int padded_first(int j) {
  static_assert(16 % R == 0, "radix must divide 16");
  return R * j + ((R * j) >> 4);
}

// ---- twiddles from a shared table ------------------------------------------
// table row for k: w^t = exp(-2 pi i k t / L), t = 1..R-1 (forward sign);
// the inverse uses the conjugates.
// Table of one Stockham pass (stride NS, radix R): entry (t, k) =
// exp(-2 pi i k t / (NS R)) at tab[(t-1)*NS + k], t = 1..R-1, k < NS.  Lanes
// reading consecutive k hit consecutive addresses (no bank conflicts); lanes
// sharing k broadcast.  The inverse uses the conjugates.
template <int R, int DIR, int NS>
__device__ __forceinline__ void twiddle_from_table(float2* v, const float2* tab, int k) {
#pragma unroll
  for (int t = 1; t < R; ++t) {
    const float2 w = tab[(t - 1) * NS + k];
    v[t] = DIR < 0 ? cmul(v[t], w) : cmulc(v[t], w);
  }
}

template <int NS, int R>
__device__ __forceinline__ void fill_twiddles(float2* tab, int tid, int nthreads) {
  constexpr int L = NS * R;
  for (int e = tid; e < NS * (R - 1); e += nthreads) {
    const int t = e / NS + 1, k = e % NS;
    float s, c;
    sincospif(2.0f * (float)((k * t) % L) / (float)L, &s, &c);
    tab[e] = make_float2(c, -s);
  }
}

// Shared-memory Stockham pass with table twiddles (in place, two barriers).
template <int N, int R, int NS, int NT, int DIR, class IDX>
__device__ __forceinline__ void table_pass(float2* __restrict__ x, const float2* __restrict__ tab, int t) {
  constexpr int NB = N / R;
  constexpr int PER = (NB + NT - 1) / NT;
  float2 v[PER][R];
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int j = t + p * NT;
    if ((NB % NT == 0) || j < NB) {
      const int fj = IDX::f(j);
#pragma unroll
      for (int q = 0; q < R; ++q) v[p][q] = x[padded_at<IDX, NB>(fj, j, q)];
      if (NS > 1) twiddle_from_table<R, DIR, NS>(v[p], tab, j % NS);
      Dft<R, DIR>::run(v[p]);
    }
  }
  __syncthreads();
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int j = t + p * NT;
    if ((NB % NT == 0) || j < NB) {
      const int base = (j / NS) * NS * R + (j % NS);
      const int fb = IDX::f(base);
#pragma unroll
      for (int q = 0; q < R; ++q) x[padded_at<IDX, NS>(fb, base, q)] = v[p][q];
    }
  }
  __syncthreads();
}

// The same pass reading with one index map and writing with another (the
// buffer then changes layout between passes).
template <int N, int R, int NS, int NT, int DIR, class IDX_LD, class IDX_ST>
__device__ __forceinline__ void table_pass_io(float2* __restrict__ x, const float2* __restrict__ tab, int t) {
  constexpr int NB = N / R;
  constexpr int PER = (NB + NT - 1) / NT;
  float2 v[PER][R];
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int j = t + p * NT;
    if ((NB % NT == 0) || j < NB) {
      const int fj = IDX_LD::f(j);
#pragma unroll
      for (int q = 0; q < R; ++q) v[p][q] = x[padded_at<IDX_LD, NB>(fj, j, q)];
      if (NS > 1) twiddle_from_table<R, DIR, NS>(v[p], tab, j % NS);
      Dft<R, DIR>::run(v[p]);
    }
  }
  __syncthreads();
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int j = t + p * NT;
    if ((NB % NT == 0) || j < NB) {
      const int base = (j / NS) * NS * R + (j % NS);
      const int fb = IDX_ST::f(base);
#pragma unroll
      for (int q = 0; q < R; ++q) x[padded_at<IDX_ST, NS>(fb, base, q)] = v[p][q];
    }
  }
  __syncthreads();
}

// Table offsets: pass with stride NS starts at sum over earlier passes of NS'*(R'-1).
template <int NS, class RL>
struct TableSize;
template <int NS>
struct TableSize<NS, Radices<>> {
  static constexpr int value = 0;
};
template <int NS, int R, int... Rs>
struct TableSize<NS, Radices<R, Rs...>> {
  static constexpr int value = (NS > 1 ? NS * (R - 1) : 0) + TableSize<NS * R, Radices<Rs...>>::value;
};

template <int N, int NS, class RL>
struct FillTables;
template <int N, int NS>
struct FillTables<N, NS, Radices<>> {
  static __device__ __forceinline__ void run(float2*, int, int) {}
};
template <int N, int NS, int R, int... Rs>
struct FillTables<N, NS, Radices<R, Rs...>> {
  static __device__ __forceinline__ void run(float2* tab, int tid, int nt) {
    if (NS > 1) fill_twiddles<NS, R>(tab, tid, nt);
    FillTables<N, NS * R, Radices<Rs...>>::run(tab + (NS > 1 ? NS * (R - 1) : 0), tid, nt);
  }
};

// Run a list of middle passes (shared memory in place), starting at stride NS,
// with twiddles from `tab` (laid out by TableSize/FillTables from stride NS0).
template <int N, int NT, int DIR, class IDX, int NS, class RL>
struct TablePasses;
template <int N, int NT, int DIR, class IDX, int NS>
struct TablePasses<N, NT, DIR, IDX, NS, Radices<>> {
  static __device__ __forceinline__ void run(float2*, const float2*, int) {}
};
template <int N, int NT, int DIR, class IDX, int NS, int R, int... Rs>
struct TablePasses<N, NT, DIR, IDX, NS, Radices<R, Rs...>> {
  static __device__ __forceinline__ void run(float2* x, const float2* tab, int t) {
    table_pass<N, R, NS, NT, DIR, IDX>(x, tab, t);
    TablePasses<N, NT, DIR, IDX, NS * R, Radices<Rs...>>::run(x, tab + (NS > 1 ? NS * (R - 1) : 0), t);
  }
};

// Whole transform with table twiddles: every pass after the first reads its
// twiddles from `tab` (FftTable<N>::SIZE entries filled by fill_fft_table).
template <int N>
struct FftTable {
  static constexpr int SIZE = TableSize<1, typename Plan<N>::type>::value;
};
template <int N>
__device__ __forceinline__ void fill_fft_table(float2* tab, int tid, int nthreads) {
  FillTables<N, 1, typename Plan<N>::type>::run(tab, tid, nthreads);
}
template <int N, int NT, int DIR, class IDX = IdxPlain>
__device__ __forceinline__ void block_fft_tab(float2* x, const float2* tab, int t) {
  TablePasses<N, NT, DIR, IDX, 1, typename Plan<N>::type>::run(x, tab, t);
}
// Same, with inputs at index >= nz known to be zero (the first pass skips them).
template <int N, int NT, int DIR, class IDX = IdxPlain>
__device__ __forceinline__ void block_fft_pruned_tab(float2* x, const float2* tab, int t, int nz) {
  using RL = typename Plan<N>::type;
  stockham_pass<N, Head<RL>::value, 1, NT, DIR, IDX, true>(x, t, nz);
  TablePasses<N, NT, DIR, IDX, Head<RL>::value, typename Tail<RL>::type>::run(x, tab, t);
}

}  // namespace lgb
