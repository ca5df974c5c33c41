// Convolutions and linear layers of the proposal network on the tensor cores:
// each pass is a GEMM (for the 3x3 convolutions an implicit GEMM) run by the
// tcgen05 GEMM of tc_gemm.cuh (BF16 operands, FP32 accumulation in TMEM), with
// gather kernels that write the operands directly in the GEMM's blocked
// core-matrix layout and epilogues that scatter the accumulator to the
// network's NCHW / [N][features] tensors.
//
//   forward      y[p][co]   = sum_k  im2col(x)[p][k] * w[co][k]        k = ci*9 + tap
//   input grad   dx[q][ci]  = sum_k' col(g)[q][k'] * wT[ci][k']        k' = co*9 + tap
//   weight grad  dw[co][k]  = sum_p  im2col(x)[p][k] * g[p][co]        as [k][co], split over p, atomic adds
//
// p runs over output pixels (n, oy, ox), q over input pixels (n, iy, ix).  The
// linear layers run the same three products with x [N][In], w [Out][In], in
// transposed form (outputs as rows) so the epilogue's stores are coalesced.  The
// output gradient g (FP32) enters the tensor cores rounded to BF16, like the
// activations; accumulation stays FP32.  The bias gradient is one more column
// of the weight-gradient GEMM (a row of ones in its operand).  No reference
// counterpart (Leopard-EM has no learned component).
#include <cuda_bf16.h>

#include "tc_gemm.cuh"

namespace lgb {

using bf16t = __nv_bfloat16;

struct ConvShape {
  int N, Cin, H, W, Cout, s, Ho, Wo;
  int P, Q, K, Kt;  // output pixels, input pixels, Cin*9, Cout*9 (P, Q < 2^23: checked by the entry points)
};

static ConvShape conv_shape(int N, int Cin, int H, int W, int Cout, int s) {
  ConvShape c{N, Cin, H, W, Cout, s, (H - 1) / s + 1, (W - 1) / s + 1, 0, 0, 0, 0};
  c.P = N * c.Ho * c.Wo;
  c.Q = N * H * W;
  c.K = Cin * 9;
  c.Kt = Cout * 9;
  return c;
}

__host__ __device__ constexpr int round_up(int a, int b) { return (a + b - 1) / b * b; }

// N tile (B rows per CTA) for a GEMM N extent: 32, 64 or 128 (TMEM columns are a power of two)
static int bn_for(int n) { return n <= 32 ? 32 : (n <= 64 ? 64 : 128); }

// ---- operand writers: 8 consecutive K elements (one 16-byte core-matrix row) per thread ----
__device__ __forceinline__ void store8(uint16_t* dst, const float* v) {
  uint4 u;
  uint16_t* h = reinterpret_cast<uint16_t*>(&u);
#pragma unroll
  for (int e = 0; e < 8; ++e) h[e] = __bfloat16_as_ushort(__float2bfloat16_rn(v[e]));
  *reinterpret_cast<uint4*>(dst) = u;
}

// Threads walk the operand in its memory order, one 16-byte unit (8 K values of
// one row) each, so the stores are fully coalesced: unit u of a blocked operand
// with TR-row tiles and KC chunks holds row r, K elements [k0, k0 + 8).
__device__ __forceinline__ void unit_rk(long long u, int TR, int KC, int& r, int& k0) {
  const int r8 = (int)(u & 7), kg = (int)((u >> 3) & 7);
  const long long rest = u >> 6;
  const int rg = (int)(rest % (TR / 8));
  const long long tc = rest / (TR / 8);
  r = (int)(tc / KC) * TR + rg * 8 + r8;
  k0 = (int)(tc % KC) * kTcKC + kg * 8;
}

// A of the forward and of the weight gradient: im2col(x) [rows p][k], rows
// padded to TR, K padded to 64 (zeros).  transpose_k = false: rows are pixels
// and K runs over ci*9+tap; true: rows are ci*9+tap and K runs over pixels,
// plus row Cin*9 of ones, whose product with g is the bias gradient.
__global__ void im2col_kernel(ConvShape c, const bf16t* __restrict__ x, int rows_pad, int k_pad, int TR,
                              bool transpose_k, uint16_t* __restrict__ out) {
  const long long n8 = (long long)rows_pad * (k_pad / 8);
  const int KC = k_pad / kTcKC;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n8; e += (long long)gridDim.x * blockDim.x) {
    int r, k0;
    unit_rk(e, TR, KC, r, k0);
    float v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int p = transpose_k ? k0 + i : r;
      const int k = transpose_k ? r : k0 + i;
      float val = (transpose_k && k == c.K && p < c.P) ? 1.f : 0.f;  // ones row: sums g into db
      if (p < c.P && k < c.K) {
        const int n = p / (c.Ho * c.Wo), pix = p % (c.Ho * c.Wo);
        const int oy = pix / c.Wo, ox = pix % c.Wo;
        const int ci = k / 9, tap = k % 9;
        const int iy = oy * c.s - 1 + tap / 3, ix = ox * c.s - 1 + tap % 3;
        if (iy >= 0 && iy < c.H && ix >= 0 && ix < c.W)
          val = __bfloat162float(x[(((size_t)n * c.Cin + ci) * c.H + iy) * c.W + ix]);
      }
      v[i] = val;
    }
    store8(out + e * 8, v);
  }
}

// B of the forward: w[co][k] (bf16 [Cout][Cin*9])
__global__ void weights_kernel(int rows, int cols, const bf16t* __restrict__ w, int rows_pad, int k_pad, int TR,
                               uint16_t* __restrict__ out) {
  const long long n8 = (long long)rows_pad * (k_pad / 8);
  const int KC = k_pad / kTcKC;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n8; e += (long long)gridDim.x * blockDim.x) {
    int r, k0;
    unit_rk(e, TR, KC, r, k0);
    float v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
      v[i] = (r < rows && k0 + i < cols) ? __bfloat162float(w[(size_t)r * cols + k0 + i]) : 0.f;
    store8(out + e * 8, v);
  }
}

// B of the input gradient: wT[ci][co*9 + tap] = w[co][ci][tap]
__global__ void weights_t_kernel(ConvShape c, const bf16t* __restrict__ w, int rows_pad, int k_pad, int TR,
                                 uint16_t* __restrict__ out) {
  const long long n8 = (long long)rows_pad * (k_pad / 8);
  const int KC = k_pad / kTcKC;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n8; e += (long long)gridDim.x * blockDim.x) {
    int ci, k0;
    unit_rk(e, TR, KC, ci, k0);
    float v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int kt = k0 + i;
      v[i] = (ci < c.Cin && kt < c.Kt)
                 ? __bfloat162float(w[((size_t)(kt / 9) * c.Cin + ci) * 9 + kt % 9])
                 : 0.f;
    }
    store8(out + e * 8, v);
  }
}

// A of the input gradient: col(g)[q][co*9 + tap] = g[n][co][oy][ox] for the
// output pixel whose tap covers input pixel q (zero where none does)
__global__ void gcol_kernel(ConvShape c, const float* __restrict__ g, int rows_pad, int k_pad,
                            uint16_t* __restrict__ out) {
  const long long n8 = (long long)rows_pad * (k_pad / 8);
  const int KC = k_pad / kTcKC;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n8; e += (long long)gridDim.x * blockDim.x) {
    int q, k0;
    unit_rk(e, kTcM, KC, q, k0);
    float v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int kt = k0 + i;
      float val = 0.f;
      if (q < c.Q && kt < c.Kt) {
        const int n = q / (c.H * c.W), pix = q % (c.H * c.W);
        const int iy = pix / c.W, ix = pix % c.W;
        const int co = kt / 9, tap = kt % 9;
        const int ty = iy + 1 - tap / 3, tx = ix + 1 - tap % 3;
        if (ty >= 0 && tx >= 0 && ty % c.s == 0 && tx % c.s == 0) {
          const int oy = ty / c.s, ox = tx / c.s;
          if (oy < c.Ho && ox < c.Wo) val = g[(((size_t)n * c.Cout + co) * c.Ho + oy) * c.Wo + ox];
        }
      }
      v[i] = val;
    }
    store8(out + e * 8, v);
  }
}

// B of the weight gradient: gT[co][p] = g[n][co][oy][ox]
__global__ void gT_kernel(ConvShape c, const float* __restrict__ g, int rows_pad, int k_pad, int TR,
                          uint16_t* __restrict__ out) {
  const long long n8 = (long long)rows_pad * (k_pad / 8);
  const int KC = k_pad / kTcKC;
  const int HoWo = c.Ho * c.Wo;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n8; e += (long long)gridDim.x * blockDim.x) {
    int co, p0;
    unit_rk(e, TR, KC, co, p0);
    float v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int p = p0 + i;
      v[i] = (co < c.Cout && p < c.P) ? g[((size_t)(p / HoWo) * c.Cout + co) * HoWo + p % HoWo] : 0.f;
    }
    store8(out + e * 8, v);
  }
}

// Linear-layer operands: (r, k) = src[r*sr + k*sk] for r < R, k < Kv; row
// ones_row (if >= R) holds ones for k < Kv; zeros elsewhere.
__device__ __forceinline__ float to_f(bf16t v) { return __bfloat162float(v); }
__device__ __forceinline__ float to_f(float v) { return v; }

template <class T>
__global__ void pack_kernel(const T* __restrict__ src, long long sr, long long sk, int R, int Kv, int ones_row,
                            int rows_pad, int k_pad, int TR, uint16_t* __restrict__ out) {
  const long long n8 = (long long)rows_pad * (k_pad / 8);
  const int KC = k_pad / kTcKC;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n8; e += (long long)gridDim.x * blockDim.x) {
    int r, k0;
    unit_rk(e, TR, KC, r, k0);
    float v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int k = k0 + i;
      v[i] = k >= Kv ? 0.f : (r < R ? to_f(src[r * sr + k * sk]) : (r == ones_row ? 1.f : 0.f));
    }
    store8(out + e * 8, v);
  }
}

// ---- epilogues ----------------------------------------------------------------
struct EpiConvFwd {
  struct Params {
    bf16t* y;
    const float* bias;
    int Cout, HoWo, P, relu;
  };
  static __device__ __forceinline__ void apply(int row, int col0, const float* v, const Params& p) {
    if (row >= p.P) return;
    const int n = row / p.HoWo, pix = row % p.HoWo;
#pragma unroll
    for (int i = 0; i < 32; ++i) {
      const int co = col0 + i;
      if (co < p.Cout) {
        float a = v[i] + (p.bias ? p.bias[co] : 0.f);
        if (p.relu && a < 0.f) a = 0.f;
        p.y[((size_t)n * p.Cout + co) * p.HoWo + pix] = __float2bfloat16(a);
      }
    }
  }
};

struct EpiConvDx {
  struct Params {
    float* dx;
    int Cin, HW, Q;
  };
  static __device__ __forceinline__ void apply(int row, int col0, const float* v, const Params& p) {
    if (row >= p.Q) return;
    const int n = row / p.HW, pix = row % p.HW;
#pragma unroll
    for (int i = 0; i < 32; ++i)
      if (col0 + i < p.Cin) p.dx[((size_t)n * p.Cin + col0 + i) * p.HW + pix] = v[i];
  }
};

// rows: k = ci*9 + tap (row Cin*9: the bias), columns: co.  Adjacent threads
// add to adjacent words of dw.
struct EpiConvDw {
  struct Params {
    float* dw;
    float* db;  // optional
    int Cout, K;
  };
  static __device__ __forceinline__ void apply(int row, int col0, const float* v, const Params& p) {
    if (row > p.K || (row == p.K && !p.db)) return;
    float* dst = row < p.K ? p.dw + row : p.db;
    const int stride = row < p.K ? p.K : 1;
#pragma unroll
    for (int i = 0; i < 32; ++i)
      if (col0 + i < p.Cout) atomicAdd(dst + (size_t)(col0 + i) * stride, v[i]);
  }
};

// linear forward as y^T: rows o, columns n (adjacent threads write adjacent outputs)
struct EpiLinFwd {
  struct Params {
    bf16t* y;
    float* yf;
    const float* bias;
    int Out, N, relu;
  };
  static __device__ __forceinline__ void apply(int row, int col0, const float* v, const Params& p) {
    if (row >= p.Out) return;
    const float b = p.bias ? p.bias[row] : 0.f;
#pragma unroll
    for (int i = 0; i < 32; ++i) {
      const int n = col0 + i;
      if (n < p.N) {
        float a = v[i] + b;
        if (p.relu && a < 0.f) a = 0.f;
        if (p.y) p.y[(size_t)n * p.Out + row] = __float2bfloat16(a);
        if (p.yf) p.yf[(size_t)n * p.Out + row] = a;
      }
    }
  }
};

// linear input gradient as dx^T: rows i, columns n
struct EpiLinDx {
  struct Params {
    float* dx;
    int In, N;
  };
  static __device__ __forceinline__ void apply(int row, int col0, const float* v, const Params& p) {
    if (row >= p.In) return;
#pragma unroll
    for (int i = 0; i < 32; ++i)
      if (col0 + i < p.N) p.dx[(size_t)(col0 + i) * p.In + row] = v[i];
  }
};

template <class Epi, int BN>
static int run_gemm(int m_tiles, int n_tiles, int k_chunks, int splits, const uint16_t* a, const uint16_t* b,
                    int* status, const typename Epi::Params& ep, cudaStream_t s) {
  constexpr int SMEM = TcSmem<BN, false>::BYTES;  // single BF16 term: no lo buffers
  if (cudaFuncSetAttribute(tc_gemm_kernel<Epi, BN, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           SMEM) != cudaSuccess)
    return LGB_ERR_CUDA;
  const int per = (k_chunks + splits - 1) / splits;
  const int z = (k_chunks + per - 1) / per;
  TcGemmArgs g{a, nullptr, b, nullptr, k_chunks, 1, status, splits > 1 ? per : 0};
  tc_gemm_kernel<Epi, BN, false, false><<<dim3(n_tiles, m_tiles, z), kTcThreads, SMEM, s>>>(g, ep);
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

template <class Epi>
static int run_gemm_bn(int bn, int m_tiles, int n_tiles, int k_chunks, int splits, const uint16_t* a,
                       const uint16_t* b, int* status, const typename Epi::Params& ep, cudaStream_t s) {
  switch (bn) {
    case 32:
      return run_gemm<Epi, 32>(m_tiles, n_tiles, k_chunks, splits, a, b, status, ep, s);
    case 64:
      return run_gemm<Epi, 64>(m_tiles, n_tiles, k_chunks, splits, a, b, status, ep, s);
    default:
      return run_gemm<Epi, 128>(m_tiles, n_tiles, k_chunks, splits, a, b, status, ep, s);
  }
}

static int grid256(long long n) {
  long long g = (n + 255) / 256;
  if (g > 65535LL * 16) g = 65535LL * 16;
  return (int)(g < 1 ? 1 : g);
}

// Operand sizes (bytes) of each pass, 256-byte aligned.
struct ConvWs {
  size_t fwd_a, fwd_b, dx_a, dx_b, dw_a, dw_b, total_fwd, total_bwd;
};
static size_t al256(size_t n) { return (n + 255) & ~(size_t)255; }
static ConvWs conv_ws(const ConvShape& c) {
  ConvWs w{};
  const int bnf = bn_for(c.Cout), bnx = bn_for(c.Cin);
  w.fwd_a = al256((size_t)round_up(c.P, kTcM) * round_up(c.K, kTcKC) * 2);
  w.fwd_b = al256((size_t)round_up(c.Cout, bnf) * round_up(c.K, kTcKC) * 2);
  w.dx_a = al256((size_t)round_up(c.Q, kTcM) * round_up(c.Kt, kTcKC) * 2);
  w.dx_b = al256((size_t)round_up(c.Cin, bnx) * round_up(c.Kt, kTcKC) * 2);
  w.dw_a = al256((size_t)round_up(c.K + 1, kTcM) * round_up(c.P, kTcKC) * 2);
  w.dw_b = al256((size_t)round_up(c.Cout, bnf) * round_up(c.P, kTcKC) * 2);
  w.total_fwd = w.fwd_a + w.fwd_b;
  w.total_bwd = w.dx_a + w.dx_b > w.dw_a + w.dw_b ? w.dx_a + w.dx_b : w.dw_a + w.dw_b;
  return w;
}

struct LinWs {
  size_t fwd_a, fwd_b, dx_a, dx_b, dw_a, dw_b, total;
};
static LinWs lin_ws(int N, int In, int Out) {
  LinWs w{};
  const int bnN = bn_for(N), bnO = bn_for(Out);
  w.fwd_a = al256((size_t)round_up(Out, kTcM) * round_up(In, kTcKC) * 2);
  w.fwd_b = al256((size_t)round_up(N, bnN) * round_up(In, kTcKC) * 2);
  w.dx_a = al256((size_t)round_up(In, kTcM) * round_up(Out, kTcKC) * 2);
  w.dx_b = al256((size_t)round_up(N, bnN) * round_up(Out, kTcKC) * 2);
  w.dw_a = al256((size_t)round_up(In + 1, kTcM) * round_up(N, kTcKC) * 2);
  w.dw_b = al256((size_t)round_up(Out, bnO) * round_up(N, kTcKC) * 2);
  size_t t = w.fwd_a + w.fwd_b;
  if (w.dx_a + w.dx_b > t) t = w.dx_a + w.dx_b;
  if (w.dw_a + w.dw_b > t) t = w.dw_a + w.dw_b;
  w.total = t;
  return w;
}

static int sm_count() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 1;
}

}  // namespace lgb

using namespace lgb;

extern "C" {

int lgb_nn_conv3x3_workspace_size(int N, int Cin, int H, int W, int Cout, int stride, size_t* bytes) {
  if (N < 1 || Cin < 1 || H < 1 || W < 1 || Cout < 1 || Cout > 128 || Cin > 128 || (stride != 1 && stride != 2) ||
      !bytes)
    return LGB_ERR_INVALID_ARGUMENT;
  const ConvShape c = conv_shape(N, Cin, H, W, Cout, stride);
  if ((long long)N * H * W > 65535LL * kTcM) return LGB_ERR_INVALID_ARGUMENT;  // M tiles on grid y
  const ConvWs w = conv_ws(c);
  *bytes = w.total_fwd > w.total_bwd ? w.total_fwd : w.total_bwd;
  return LGB_OK;
}

int lgb_nn_conv3x3_forward(int N, int Cin, int H, int W, int Cout, int stride, int relu, const void* x, const void* w,
                           const float* b, void* y, void* workspace, size_t workspace_bytes, int* device_status,
                           void* stream) {
  size_t need = 0;
  if (lgb_nn_conv3x3_workspace_size(N, Cin, H, W, Cout, stride, &need) != LGB_OK || !x || !w || !y || !workspace ||
      !device_status)
    return LGB_ERR_INVALID_ARGUMENT;
  if (workspace_bytes < need) return LGB_ERR_WORKSPACE_TOO_SMALL;
  if (reinterpret_cast<uintptr_t>(workspace) & 255) return LGB_ERR_INVALID_ARGUMENT;
  cudaStream_t s = (cudaStream_t)stream;
  const ConvShape c = conv_shape(N, Cin, H, W, Cout, stride);
  const ConvWs ws = conv_ws(c);
  uint16_t* a = static_cast<uint16_t*>(workspace);
  uint16_t* bm = reinterpret_cast<uint16_t*>(static_cast<char*>(workspace) + ws.fwd_a);
  const int bn = bn_for(Cout);
  const int kp = round_up(c.K, kTcKC), pp = round_up(c.P, kTcM), cp = round_up(Cout, bn);
  im2col_kernel<<<grid256((long long)pp * kp / 8), 256, 0, s>>>(c, static_cast<const bf16t*>(x), pp, kp, kTcM, false,
                                                                 a);
  weights_kernel<<<grid256((long long)cp * kp / 8), 256, 0, s>>>(Cout, c.K, static_cast<const bf16t*>(w), cp, kp, bn,
                                                                 bm);
  if (cudaGetLastError() != cudaSuccess) return LGB_ERR_CUDA;
  EpiConvFwd::Params ep{static_cast<bf16t*>(y), b, Cout, c.Ho * c.Wo, c.P, relu};
  return run_gemm_bn<EpiConvFwd>(bn, pp / kTcM, cp / bn, kp / kTcKC, 1, a, bm, device_status, ep, s);
}

int lgb_nn_conv3x3_backward(int N, int Cin, int H, int W, int Cout, int stride, const void* x, const void* w,
                            const float* g, float* dx, float* dw, float* db, void* workspace, size_t workspace_bytes,
                            int* device_status, void* stream) {
  size_t need = 0;
  if (lgb_nn_conv3x3_workspace_size(N, Cin, H, W, Cout, stride, &need) != LGB_OK || !x || !w || !g || !dw ||
      !workspace || !device_status)
    return LGB_ERR_INVALID_ARGUMENT;
  if (workspace_bytes < need) return LGB_ERR_WORKSPACE_TOO_SMALL;
  if (reinterpret_cast<uintptr_t>(workspace) & 255) return LGB_ERR_INVALID_ARGUMENT;
  cudaStream_t s = (cudaStream_t)stream;
  const ConvShape c = conv_shape(N, Cin, H, W, Cout, stride);
  const ConvWs ws = conv_ws(c);
  char* base = static_cast<char*>(workspace);
  int st;
  if (dx) {  // input gradient
    uint16_t* a = reinterpret_cast<uint16_t*>(base);
    uint16_t* bm = reinterpret_cast<uint16_t*>(base + ws.dx_a);
    const int bn = bn_for(Cin);
    const int kp = round_up(c.Kt, kTcKC), qp = round_up(c.Q, kTcM), cp = round_up(Cin, bn);
    gcol_kernel<<<grid256((long long)qp * kp / 8), 256, 0, s>>>(c, g, qp, kp, a);
    weights_t_kernel<<<grid256((long long)cp * kp / 8), 256, 0, s>>>(c, static_cast<const bf16t*>(w), cp, kp, bn, bm);
    if (cudaGetLastError() != cudaSuccess) return LGB_ERR_CUDA;
    EpiConvDx::Params ep{dx, Cin, H * W, c.Q};
    if ((st = run_gemm_bn<EpiConvDx>(bn, qp / kTcM, cp / bn, kp / kTcKC, 1, a, bm, device_status, ep, s)))
      return st;
  }
  {  // weight and bias gradients: [Cin*9 + 1] x [Cout] over K = output pixels, split across CTAs
     // (atomic adds into zeroed dw, db)
    uint16_t* a = reinterpret_cast<uint16_t*>(base);
    uint16_t* bm = reinterpret_cast<uint16_t*>(base + ws.dw_a);
    const int bn = bn_for(Cout);
    const int pk = round_up(c.P, kTcKC), kr = round_up(c.K + 1, kTcM), cp = round_up(Cout, bn);
    im2col_kernel<<<grid256((long long)kr * pk / 8), 256, 0, s>>>(c, static_cast<const bf16t*>(x), kr, pk, kTcM, true,
                                                                  a);
    gT_kernel<<<grid256((long long)cp * pk / 8), 256, 0, s>>>(c, g, cp, pk, bn, bm);
    if (cudaGetLastError() != cudaSuccess) return LGB_ERR_CUDA;
    if (cudaMemsetAsync(dw, 0, sizeof(float) * (size_t)Cout * c.K, s) != cudaSuccess) return LGB_ERR_CUDA;
    if (db && cudaMemsetAsync(db, 0, sizeof(float) * (size_t)Cout, s) != cudaSuccess) return LGB_ERR_CUDA;
    const int m_tiles = kr / kTcM, k_chunks = pk / kTcKC;
    int splits = (2 * sm_count() + m_tiles - 1) / m_tiles;
    if (splits > k_chunks) splits = k_chunks;
    EpiConvDw::Params ep{dw, db, Cout, c.K};
    if ((st = run_gemm_bn<EpiConvDw>(bn, m_tiles, cp / bn, k_chunks, splits, a, bm, device_status, ep, s))) return st;
  }
  return LGB_OK;
}

int lgb_nn_linear_workspace_size(int N, int In, int Out, size_t* bytes) {
  if (N < 1 || In < 1 || Out < 1 || !bytes || (long long)round_up(In + 1, kTcM) / kTcM > 65535 ||
      (long long)round_up(Out, kTcM) / kTcM > 65535)
    return LGB_ERR_INVALID_ARGUMENT;
  *bytes = lin_ws(N, In, Out).total;
  return LGB_OK;
}

int lgb_nn_linear_forward(int N, int In, int Out, int relu, const void* x, const void* w, const float* b, void* y_bf16,
                          float* y_f32, void* workspace, size_t workspace_bytes, int* device_status, void* stream) {
  size_t need = 0;
  if (lgb_nn_linear_workspace_size(N, In, Out, &need) != LGB_OK || !x || !w || (!y_bf16 && !y_f32) || !workspace ||
      !device_status)
    return LGB_ERR_INVALID_ARGUMENT;
  if (workspace_bytes < need) return LGB_ERR_WORKSPACE_TOO_SMALL;
  if (reinterpret_cast<uintptr_t>(workspace) & 255) return LGB_ERR_INVALID_ARGUMENT;
  cudaStream_t s = (cudaStream_t)stream;
  const LinWs ws = lin_ws(N, In, Out);
  uint16_t* a = static_cast<uint16_t*>(workspace);
  uint16_t* bm = reinterpret_cast<uint16_t*>(static_cast<char*>(workspace) + ws.fwd_a);
  const int bn = bn_for(N);
  const int kp = round_up(In, kTcKC), op = round_up(Out, kTcM), np = round_up(N, bn);
  pack_kernel<bf16t><<<grid256((long long)op * kp / 8), 256, 0, s>>>(static_cast<const bf16t*>(w), In, 1, Out, In, -1,
                                                                      op, kp, kTcM, a);
  pack_kernel<bf16t><<<grid256((long long)np * kp / 8), 256, 0, s>>>(static_cast<const bf16t*>(x), In, 1, N, In, -1,
                                                                      np, kp, bn, bm);
  if (cudaGetLastError() != cudaSuccess) return LGB_ERR_CUDA;
  EpiLinFwd::Params ep{static_cast<bf16t*>(y_bf16), y_f32, b, Out, N, relu};
  return run_gemm_bn<EpiLinFwd>(bn, op / kTcM, np / bn, kp / kTcKC, 1, a, bm, device_status, ep, s);
}

int lgb_nn_linear_backward(int N, int In, int Out, const void* x, const void* w, const float* g, float* dx, float* dw,
                           float* db, void* workspace, size_t workspace_bytes, int* device_status, void* stream) {
  size_t need = 0;
  if (lgb_nn_linear_workspace_size(N, In, Out, &need) != LGB_OK || !x || !w || !g || !dw || !workspace ||
      !device_status)
    return LGB_ERR_INVALID_ARGUMENT;
  if (workspace_bytes < need) return LGB_ERR_WORKSPACE_TOO_SMALL;
  if (reinterpret_cast<uintptr_t>(workspace) & 255) return LGB_ERR_INVALID_ARGUMENT;
  cudaStream_t s = (cudaStream_t)stream;
  const LinWs ws = lin_ws(N, In, Out);
  char* base = static_cast<char*>(workspace);
  int st;
  if (dx) {  // dx^T[i][n] = sum_o w[o][i] g[n][o]
    uint16_t* a = reinterpret_cast<uint16_t*>(base);
    uint16_t* bm = reinterpret_cast<uint16_t*>(base + ws.dx_a);
    const int bn = bn_for(N);
    const int kp = round_up(Out, kTcKC), ip = round_up(In, kTcM), np = round_up(N, bn);
    pack_kernel<bf16t><<<grid256((long long)ip * kp / 8), 256, 0, s>>>(static_cast<const bf16t*>(w), 1, In, In, Out,
                                                                        -1, ip, kp, kTcM, a);
    pack_kernel<float><<<grid256((long long)np * kp / 8), 256, 0, s>>>(g, Out, 1, N, Out, -1, np, kp, bn, bm);
    if (cudaGetLastError() != cudaSuccess) return LGB_ERR_CUDA;
    EpiLinDx::Params ep{dx, In, N};
    if ((st = run_gemm_bn<EpiLinDx>(bn, ip / kTcM, np / bn, kp / kTcKC, 1, a, bm, device_status, ep, s))) return st;
  }
  {  // [dw^T; db][i][o] = sum_n [x; 1][n][i] g[n][o], split over n with atomic adds
    uint16_t* a = reinterpret_cast<uint16_t*>(base);
    uint16_t* bm = reinterpret_cast<uint16_t*>(base + ws.dw_a);
    const int bn = bn_for(Out);
    const int kp = round_up(N, kTcKC), ip = round_up(In + 1, kTcM), op = round_up(Out, bn);
    pack_kernel<bf16t><<<grid256((long long)ip * kp / 8), 256, 0, s>>>(static_cast<const bf16t*>(x), 1, In, In, N, In,
                                                                        ip, kp, kTcM, a);
    pack_kernel<float><<<grid256((long long)op * kp / 8), 256, 0, s>>>(g, 1, Out, Out, N, -1, op, kp, bn, bm);
    if (cudaGetLastError() != cudaSuccess) return LGB_ERR_CUDA;
    if (cudaMemsetAsync(dw, 0, sizeof(float) * (size_t)Out * In, s) != cudaSuccess) return LGB_ERR_CUDA;
    if (db && cudaMemsetAsync(db, 0, sizeof(float) * (size_t)Out, s) != cudaSuccess) return LGB_ERR_CUDA;
    const int m_tiles = ip / kTcM, n_tiles = op / bn, k_chunks = kp / kTcKC;
    int splits = (2 * sm_count() + m_tiles * n_tiles - 1) / (m_tiles * n_tiles);
    if (splits > k_chunks) splits = k_chunks;
    EpiConvDw::Params ep{dw, db, Out, In};
    if ((st = run_gemm_bn<EpiConvDw>(bn, m_tiles, n_tiles, k_chunks, splits, a, bm, device_status, ep, s))) return st;
  }
  return LGB_OK;
}

}  // extern "C"
