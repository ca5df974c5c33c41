// Hand-written kernels of the refinement proposal network (no reference
// counterpart: Leopard-EM has no learned component; the closest analogue is
// backend/core_differentiable_refine.py).
//
// Storage: activations and forward weights BF16; accumulation FP32; gradients,
// master weights and Adam moments FP32.  Layout NCHW; conv weights
// [Cout][Cin][3][3]; linear weights [Out][In].  The convolutions and linear
// layers run on the tensor cores (nn_tc.cu); this file holds the ReLU
// gradient, the loss, Adam and the input builder.
//
// Also: the network's input builder (lgb_nn_make_inputs): a low-frequency band
// of each particle spectrum and the template's central slice at the particle's
// starting pose on the same band, CTF-filtered, inverse transformed with the
// block FFT and standardised.
#include <cuda_bf16.h>
#include <math.h>

#include "match_kernels.cuh"

namespace lgb {

using bf16 = __nv_bfloat16;


__global__ void relu_bwd_kernel(long long n, const bf16* __restrict__ y, const float* __restrict__ dy,
                                float* __restrict__ g) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    g[i] = __bfloat162float(y[i]) > 0.f ? dy[i] : 0.f;
}

__global__ void mse_kernel(int N, int D, const float* __restrict__ pred, const float* __restrict__ tgt,
                           const float* __restrict__ wd, float* __restrict__ dpred, float* __restrict__ loss) {
  __shared__ float red[256];
  float acc = 0.f;
  for (int i = threadIdx.x; i < N * D; i += blockDim.x) {
    const float w = wd ? wd[i % D] : 1.f;
    const float e = pred[i] - tgt[i];
    acc += w * e * e;
    dpred[i] = 2.f * w * e / (float)N;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *loss = red[0] / (float)N;
}

__global__ void adam_kernel(long long n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, bf16* __restrict__ pbf, float lr, float b1, float b2, float eps,
                            float wd, float c1, float c2) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i] + wd * p[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    p[i] = pi;
    if (pbf) pbf[i] = __float2bfloat16(pi);
  }
}

__global__ void f32_to_bf16_kernel(long long n, const float* __restrict__ s, bf16* __restrict__ d) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    d[i] = __float2bfloat16(s[i]);
}

// ---- network inputs --------------------------------------------------------
// Band of G x (G/2+1) frequencies (G = 2*GH): rows ky in [0, GH) and [H-GH, H) of the
// particle's H x (W/2+1) spectrum, columns [0, GH]; the template's central
// slice at rotation R sampled at the same physical frequencies (f = k / H on
// the particle grid, cubic template of edge d), multiplied by the particle's
// CTF; each irfft2'd to G x G and standardised (zero mean, unit std) into
// channel 0 (particle) and 1 (reference) of out[p][2][G][G].
struct NnCtf {
  double lambda, cs_A, amp_phase, pixel_size, b_factor;
};

// Network input channels (G = 64 band of the particle's H x W spectrum, frequencies
// f = (kx/W, ky/H), ky in [-G/2, G/2), kx in [0, G/2]):
//   0  particle band, re-centred from the crop centre to the frame origin and
//      shifted onto the reference by the integer+parabolic peak of their band
//      cross-correlation (|shift| <= G/4), standardised by itself
//   1  reference: central slice at R0 times the particle's CTF (contrast flipped)
//   2-4  (slice at D_a(1 deg) R0 - reference) / 1 deg, D_a = rotation about the
//      image-frame x, y, z axis (finite-difference derivatives)
//   5  derivative of the reference w.r.t. defocus, times 100 A (analytic, via chi)
// Channels 1-5 are mean-subtracted and divided by the reference's std.
// Inverse transforms by direct separable DFT in shared memory, one image at a
// time (G = 64: ~0.5 MFLOP per image).
constexpr int kNnChannels = 6;

__device__ float2 slice_sample(const float2* __restrict__ vol, int d, const float* R, float fx, float fy) {
  const int wcv = d / 2 + 1;
  float X = R[0] * fx + R[1] * fy, Y = R[3] * fx + R[4] * fy, Z = R[6] * fx + R[7] * fy;
  const bool cj = X < 0.f;
  if (cj) { X = -X; Y = -Y; Z = -Z; }
  const float cz = Z * d + d / 2, cy = Y * d + d / 2, cx = X * d;
  float2 val = make_float2(0.f, 0.f);
  if (cz >= 0.f && cz <= (float)(d - 1) && cy >= 0.f && cy <= (float)(d - 1) && cx >= 0.f &&
      cx <= (float)(wcv - 1)) {
    const int z0 = (int)floorf(cz), y0 = (int)floorf(cy), x0 = (int)floorf(cx);
    const float tz = cz - z0, ty = cy - y0, tx = cx - x0;
    const int z1 = min(z0 + 1, d - 1), y1 = min(y0 + 1, d - 1), x1 = min(x0 + 1, wcv - 1);
    const int zz[2] = {z0, z1}, yy[2] = {y0, y1}, xx[2] = {x0, x1};
    const float wz[2] = {1.f - tz, tz}, wy[2] = {1.f - ty, ty}, wx[2] = {1.f - tx, tx};
    for (int a = 0; a < 2; ++a)
      for (int bq = 0; bq < 2; ++bq)
        for (int c = 0; c < 2; ++c) {
          const float w = wz[a] * wy[bq] * wx[c];
          const float2 sv = vol[((size_t)zz[a] * d + yy[bq]) * wcv + xx[c]];
          val.x = fmaf(sv.x, w, val.x);
          val.y = fmaf(sv.y, w, val.y);
        }
  }
  if (cj) val.y = -val.y;
  return val;
}

// spec [G][GC] -> img [G*G] (unnormalised inverse, c2r semantics)
template <int G>
__device__ void band_irfft2(const float2* spec, float2* cols, float* img, const float2* tw) {
  constexpr int GH = G / 2, GC = GH + 1;
  for (int e = threadIdx.x; e < G * GC; e += blockDim.x) {
    const int y = e / GC, kx = e % GC;
    float2 acc = make_float2(0.f, 0.f);
    for (int r = 0; r < G; ++r) acc = cadd(acc, cmul(spec[r * GC + kx], tw[(y * r) % G]));
    cols[e] = acc;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < G * G; e += blockDim.x) {
    const int y = e / G, x = e % G;
    const float2* cr = cols + y * GC;
    float acc = cr[0].x + ((x & 1) ? -cr[GH].x : cr[GH].x);
    for (int kx = 1; kx < GH; ++kx) {
      const float2 w = tw[(x * kx) % G];
      acc += 2.f * (cr[kx].x * w.x - cr[kx].y * w.y);
    }
    img[e] = acc;
  }
  __syncthreads();
}

// block mean and 1/std of img[G*G] (FP64 sums)
template <int G>
__device__ void image_moments(const float* img, double (*red)[8], float* mean_out, float* inv_out) {
  double s1 = 0.0, s2 = 0.0;
  for (int e = threadIdx.x; e < G * G; e += blockDim.x) {
    const double v = img[e];
    s1 += v;
    s2 += v * v;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s1 += __shfl_down_sync(0xffffffffu, s1, o);
    s2 += __shfl_down_sync(0xffffffffu, s2, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = s1;
    red[1][threadIdx.x >> 5] = s2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w8 = 0; w8 < (int)(blockDim.x >> 5); ++w8) {
      a += red[0][w8];
      b += red[1][w8];
    }
    const double n = (double)G * G, m = a / n, var = b / n - m * m;
    *mean_out = (float)m;
    *inv_out = (float)(var > 1e-30 ? 1.0 / sqrt(var) : 0.0);
  }
  __syncthreads();
}

template <int G>
__global__ void __launch_bounds__(256)
    make_inputs_kernel(const float2* __restrict__ pdft, int H, int W, const float2* __restrict__ vol, int d,
                       const float* __restrict__ rot, const float* __restrict__ du, const float* __restrict__ dv,
                       const float* __restrict__ dang, NnCtf ctf, int out_channels, bf16* __restrict__ out) {
  constexpr int GH = G / 2, GC = GH + 1;
  extern __shared__ float2 nsm[];
  float2* pspec = nsm;              // [G][GC] particle band
  float2* rspec = pspec + G * GC;   // [G][GC] reference slice (no CTF)
  float2* spec = rspec + G * GC;    // [G][GC] scratch spectrum
  float2* cols = spec + G * GC;     // [G][GC]
  float* ctfv = reinterpret_cast<float*>(cols + G * GC);  // [G][GC] CTF
  float* dctf = ctfv + G * GC;                            // [G][GC] dCTF/ddf * 100 A
  float* img = dctf + G * GC;                             // [G*G]
  float2* tw = reinterpret_cast<float2*>(img + G * G);    // [G]
  __shared__ float Rm[4][9];
  __shared__ double red[2][8];
  __shared__ float ref_mean, ref_inv, p_mean, p_inv;
  __shared__ unsigned long long best_key;
  const int p = blockIdx.x;
  const int t = threadIdx.x;
  const int wc = W / 2 + 1;
  const double pi = 3.14159265358979323846;
  if (t == 0) {
    // R0 and D_a(1 deg) R0 for a = x, y, z (image frame: left multiplication)
    const double dl = pi / 180.0, c = cos(dl), sn = sin(dl);
    double R0[9];
    for (int i = 0; i < 9; ++i) R0[i] = rot[9 * p + i];
    double D[3][9] = {{1, 0, 0, 0, c, -sn, 0, sn, c}, {c, 0, sn, 0, 1, 0, -sn, 0, c}, {c, -sn, 0, sn, c, 0, 0, 0, 1}};
    for (int i = 0; i < 9; ++i) Rm[0][i] = (float)R0[i];
    for (int a = 0; a < 3; ++a)
      for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q)
          Rm[a + 1][3 * r + q] =
              (float)(D[a][3 * r] * R0[q] + D[a][3 * r + 1] * R0[3 + q] + D[a][3 * r + 2] * R0[6 + q]);
    best_key = 0ull;
  }
  for (int k = t; k < G; k += blockDim.x) {
    float sn, cs;
    sincospif(2.0f * (float)k / (float)G, &sn, &cs);
    tw[k] = make_float2(cs, sn);
  }
  __syncthreads();
  for (int e = t; e < G * GC; e += blockDim.x) {
    const int r = e / GC, kx = e % GC;
    const int ky = r < GH ? r : r - G;
    const int prow = ky >= 0 ? ky : H + ky;
    const bool dc = (r == 0 && kx == 0);
    // particles sit at the crop centre (H/2, W/2); the reference slice is a
    // projection centred on the frame origin: re-centre the particle with
    // exp(+2 pi i (ky/2 + kx/2)) = (-1)^(ky + kx)
    float2 pv = pdft[((size_t)p * H + prow) * wc + kx];
    if ((ky + kx) & 1) pv = make_float2(-pv.x, -pv.y);
    pspec[e] = dc ? make_float2(0.f, 0.f) : pv;
    const float fx = (float)kx / (float)W, fy = (float)ky / (float)H;
    const float2 s0 = slice_sample(vol, d, Rm[0], fx, fy);
    rspec[e] = dc ? make_float2(0.f, 0.f) : make_float2(-s0.x, -s0.y);
    const double kyA = (double)ky / H / ctf.pixel_size, kxA = (double)kx / W / ctf.pixel_size;
    const double k2 = kxA * kxA + kyA * kyA;
    const double ang = atan2(kyA, kxA);
    const double dfm = 0.5 * ((double)du[p] + (double)dv[p]), ast = 0.5 * fabs((double)du[p] - (double)dv[p]);
    const double dfe = dfm + ast * cos(2.0 * (ang - (double)dang[p] * pi / 180.0));
    const double chi = -pi * ctf.lambda * k2 * dfe +
                       0.5 * pi * ctf.cs_A * ctf.lambda * ctf.lambda * ctf.lambda * k2 * k2 - ctf.amp_phase;
    const double env = exp(-ctf.b_factor * k2 / 4.0);
    ctfv[e] = (float)(-sin(chi) * env);
    dctf[e] = (float)(-cos(chi) * (-pi * ctf.lambda * k2) * 100.0 * env);
  }
  __syncthreads();
  // ---- shift of the particle w.r.t. the reference: peak of the band cross-correlation
  for (int e = t; e < G * GC; e += blockDim.x) spec[e] = cmulc(pspec[e], cscale(rspec[e], ctfv[e]));
  __syncthreads();
  band_irfft2<G>(spec, cols, img, tw);
  for (int e = t; e < G * G; e += blockDim.x) {
    const int y = e / G, x = e % G;
    const int sy = y < GH ? y : y - G, sx = x < GH ? x : x - G;
    if (abs(sy) > G / 4 || abs(sx) > G / 4) continue;
    const unsigned u = __float_as_uint(img[e]);
    const unsigned o = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    atomicMax(&best_key, ((unsigned long long)o << 32) | (unsigned)e);
  }
  __syncthreads();
  __shared__ float shift_y, shift_x;
  if (t == 0) {
    const int e = (int)(best_key & 0xffffffffull);
    const int y = e / G, x = e % G;
    auto at = [&](int yy, int xx) { return img[((yy + G) % G) * G + (xx + G) % G]; };
    const float c0 = at(y, x);
    const float ym = at(y - 1, x), yp = at(y + 1, x), xm = at(y, x - 1), xp = at(y, x + 1);
    float dy = 0.f, dx = 0.f;
    const float deny = ym - 2.f * c0 + yp, denx = xm - 2.f * c0 + xp;
    if (deny < 0.f) dy = fminf(0.5f, fmaxf(-0.5f, 0.5f * (ym - yp) / deny));
    if (denx < 0.f) dx = fminf(0.5f, fmaxf(-0.5f, 0.5f * (xm - xp) / denx));
    shift_y = (float)(y < GH ? y : y - G) + dy;
    shift_x = (float)(x < GH ? x : x - G) + dx;
  }
  __syncthreads();
  // ---- channel 0: particle moved back by the shift (phase ramp), standardised by itself
  for (int e = t; e < G * GC; e += blockDim.x) {
    const int r = e / GC, kx = e % GC;
    const int ky = r < GH ? r : r - G;
    float sn, cs;
    sincospif(2.0f * ((float)ky * shift_y + (float)kx * shift_x) / (float)G, &sn, &cs);
    spec[e] = cmul(pspec[e], make_float2(cs, sn));
  }
  __syncthreads();
  band_irfft2<G>(spec, cols, img, tw);
  image_moments<G>(img, red, &p_mean, &p_inv);
  bf16* o = out + (size_t)p * out_channels * G * G;
  for (int e = t; e < G * G; e += blockDim.x) o[e] = __float2bfloat16((img[e] - p_mean) * p_inv);
  __syncthreads();
  // ---- channel 1: reference
  for (int e = t; e < G * GC; e += blockDim.x) spec[e] = cscale(rspec[e], ctfv[e]);
  __syncthreads();
  band_irfft2<G>(spec, cols, img, tw);
  image_moments<G>(img, red, &ref_mean, &ref_inv);
  for (int e = t; e < G * G; e += blockDim.x) o[G * G + e] = __float2bfloat16((img[e] - ref_mean) * ref_inv);
  __syncthreads();
  // ---- channels 2-4: rotation derivatives; 5: defocus derivative
  for (int ch = 2; ch < kNnChannels; ++ch) {
    for (int e = t; e < G * GC; e += blockDim.x) {
      if (ch < 5) {
        const int r = e / GC, kx = e % GC;
        const int ky = r < GH ? r : r - G;
        const float2 sa = slice_sample(vol, d, Rm[ch - 1], (float)kx / (float)W, (float)ky / (float)H);
        const float2 ra = (r == 0 && kx == 0) ? make_float2(0.f, 0.f) : make_float2(-sa.x, -sa.y);
        spec[e] = cscale(csub(ra, rspec[e]), ctfv[e]);
      } else {
        spec[e] = cscale(rspec[e], dctf[e]);
      }
    }
    __syncthreads();
    band_irfft2<G>(spec, cols, img, tw);
    float m_unused, i_unused;
    image_moments<G>(img, red, &m_unused, &i_unused);
    for (int e = t; e < G * G; e += blockDim.x)
      o[(size_t)ch * G * G + e] = __float2bfloat16((img[e] - m_unused) * ref_inv);
    __syncthreads();
  }
}

// Gauss-Newton step on the input channels of one particle (CTA per particle):
// J = [d/dx, d/dy (central differences of the reference), the three rotation
// derivatives, the defocus derivative]; amplitude a = <P,R>/<R,R>;
// residual r = P - a R; solve (J^T J) delta = J^T r / a in FP64 (Gaussian
// elimination with partial pivoting).  delta = (shift x, y in band pixels,
// rotation about x, y, z in degrees, defocus in 100 A).  Writes
// gn[p] = (delta[0..5], a, |r|^2/|P|^2) and, when out_channels >= 12, fills
// channels 6..11 of the input with constant maps of delta (rotation / 3 deg,
// shifts / 2, defocus / 4).
template <int G>
__global__ void __launch_bounds__(256) gauss_newton_kernel(bf16* __restrict__ x, int channels, float* __restrict__ gn) {
  constexpr int NJ = 6;
  constexpr int NS = NJ * (NJ + 1) / 2 + 2 * NJ + 3;  // Gram upper triangle, J^T P, J^T R, <P,R>, <R,R>, <P,P>
  const int p = blockIdx.x, t = threadIdx.x;
  const bf16* P = x + (size_t)p * channels * G * G;
  const bf16* R = P + G * G;
  double acc[NS];
#pragma unroll
  for (int i = 0; i < NS; ++i) acc[i] = 0.0;
  for (int e = t; e < G * G; e += blockDim.x) {
    const int y = e / G, xx = e % G;
    const float pv = __bfloat162float(P[e]), rv = __bfloat162float(R[e]);
    float j[NJ];
    j[0] = 0.5f * (__bfloat162float(R[y * G + (xx + 1) % G]) - __bfloat162float(R[y * G + (xx + G - 1) % G]));
    j[1] = 0.5f * (__bfloat162float(R[((y + 1) % G) * G + xx]) - __bfloat162float(R[((y + G - 1) % G) * G + xx]));
#pragma unroll
    for (int a = 0; a < 4; ++a) j[2 + a] = __bfloat162float(P[(size_t)(2 + a) * G * G + e]);
    int k = 0;
#pragma unroll
    for (int a = 0; a < NJ; ++a)
#pragma unroll
      for (int b = a; b < NJ; ++b) acc[k++] += (double)j[a] * j[b];
#pragma unroll
    for (int a = 0; a < NJ; ++a) acc[k + a] += (double)j[a] * pv;
    k += NJ;
#pragma unroll
    for (int a = 0; a < NJ; ++a) acc[k + a] += (double)j[a] * rv;
    k += NJ;
    acc[k] += (double)pv * rv;
    acc[k + 1] += (double)rv * rv;
    acc[k + 2] += (double)pv * pv;
  }
  __shared__ double red[NS][8];
#pragma unroll
  for (int i = 0; i < NS; ++i) {
    double v = acc[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((t & 31) == 0) red[i][t >> 5] = v;
  }
  __syncthreads();
  __shared__ float delta_s[NJ];
  if (t == 0) {
    double S[NS];
    for (int i = 0; i < NS; ++i) {
      S[i] = 0.0;
      for (int w8 = 0; w8 < (int)(blockDim.x >> 5); ++w8) S[i] += red[i][w8];
    }
    double A[NJ][NJ + 1];
    int k = 0;
    for (int a = 0; a < NJ; ++a)
      for (int b = a; b < NJ; ++b) {
        A[a][b] = S[k];
        A[b][a] = S[k];
        ++k;
      }
    const double pr = S[k + 2 * NJ], rr = S[k + 2 * NJ + 1], pp = S[k + 2 * NJ + 2];
    const double amp = rr > 0.0 ? pr / rr : 0.0;
    for (int a = 0; a < NJ; ++a) A[a][NJ] = S[k + a] - amp * S[k + NJ + a];  // J^T (P - a R)
    for (int a = 0; a < NJ; ++a) A[a][a] += 1e-6 * (A[a][a] + 1e-12);
    for (int c = 0; c < NJ; ++c) {
      int piv = c;
      for (int r2 = c + 1; r2 < NJ; ++r2)
        if (fabs(A[r2][c]) > fabs(A[piv][c])) piv = r2;
      if (piv != c)
        for (int q = 0; q <= NJ; ++q) {
          const double tmp = A[c][q];
          A[c][q] = A[piv][q];
          A[piv][q] = tmp;
        }
      const double dg = A[c][c];
      if (fabs(dg) < 1e-30) continue;
      for (int r2 = 0; r2 < NJ; ++r2) {
        if (r2 == c) continue;
        const double f = A[r2][c] / dg;
        for (int q = c; q <= NJ; ++q) A[r2][q] -= f * A[c][q];
      }
    }
    float* o = gn + (size_t)p * 8;
    for (int a = 0; a < NJ; ++a) {
      const double dl = (fabs(A[a][a]) > 1e-30 && amp != 0.0) ? A[a][NJ] / A[a][a] / amp : 0.0;
      o[a] = (float)dl;
      delta_s[a] = (float)dl;
    }
    o[6] = (float)amp;
    o[7] = (float)(pp > 0.0 ? (pp - 2.0 * amp * pr + amp * amp * rr) / pp : 1.0);
  }
  __syncthreads();
  if (channels >= 12) {
    const float scale[NJ] = {0.5f, 0.5f, 1.f / 3.f, 1.f / 3.f, 1.f / 3.f, 0.25f};
    for (int a = 0; a < NJ; ++a) {
      const bf16 v = __float2bfloat16(delta_s[a] * scale[a]);
      bf16* c = x + ((size_t)p * channels + 6 + a) * G * G;
      for (int e = t; e < G * G; e += blockDim.x) c[e] = v;
    }
  }
}

static int g256(long long n) {
  long long g = (n + 255) / 256;
  if (g > 65535LL * 16) g = 65535LL * 16;
  return (int)(g < 1 ? 1 : g);
}

}  // namespace lgb

using namespace lgb;

extern "C" {

int lgb_nn_relu_backward(long long n, const void* y, const float* dy, float* g, void* stream) {
  if (n < 1 || !y || !dy || !g) return LGB_ERR_INVALID_ARGUMENT;
  relu_bwd_kernel<<<g256(n), 256, 0, (cudaStream_t)stream>>>(n, static_cast<const bf16*>(y), dy, g);
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

int lgb_nn_mse(int N, int D, const float* pred, const float* target, const float* weights, float* dpred, float* loss,
               void* stream) {
  if (N < 1 || D < 1 || !pred || !target || !dpred || !loss) return LGB_ERR_INVALID_ARGUMENT;
  mse_kernel<<<1, 256, 0, (cudaStream_t)stream>>>(N, D, pred, target, weights, dpred, loss);
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

int lgb_nn_adam(long long n, float* param, const float* grad, float* m, float* v, void* param_bf16, float lr,
                float beta1, float beta2, float eps, float weight_decay, int step, void* stream) {
  if (n < 1 || !param || !grad || !m || !v || step < 1) return LGB_ERR_INVALID_ARGUMENT;
  const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  adam_kernel<<<g256(n), 256, 0, (cudaStream_t)stream>>>(n, param, grad, m, v, static_cast<bf16*>(param_bf16), lr,
                                                         beta1, beta2, eps, weight_decay, c1, c2);
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

int lgb_nn_to_bf16(long long n, const float* src, void* dst, void* stream) {
  if (n < 1 || !src || !dst) return LGB_ERR_INVALID_ARGUMENT;
  f32_to_bf16_kernel<<<g256(n), 256, 0, (cudaStream_t)stream>>>(n, src, static_cast<bf16*>(dst));
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

int lgb_nn_make_inputs(int n_particles, int image_h, int image_w, const void* particle_dft, const void* template_dft,
                       int template_size, const float* rotations, const float* defocus_u, const float* defocus_v,
                       const float* defocus_angle, const lgb_ctf_params* ctf, int band, int out_channels, void* out,
                       void* stream) {
  if (n_particles < 1 || image_h < 2 * 64 || image_w < 2 * 64 || !particle_dft || !template_dft ||
      template_size < 2 || !rotations || !defocus_u || !defocus_v || !defocus_angle || !ctf || !out ||
      out_channels < kNnChannels)
    return LGB_ERR_INVALID_ARGUMENT;
  if (band != 64) return LGB_ERR_UNSUPPORTED_SIZE;
  const double v = ctf->voltage_kv * 1e3, hP = 6.62607015e-34, m0 = 9.1093837015e-31, e = 1.602176634e-19,
               c = 299792458.0;
  NnCtf k;
  k.lambda = hP / sqrt(2 * m0 * e * v * (1 + e * v / (2 * m0 * c * c))) * 1e10;
  k.cs_A = ctf->spherical_aberration_mm * 1e7;
  k.amp_phase = ctf->phase_shift_deg * 3.14159265358979323846 / 180.0 +
                atan(ctf->amplitude_contrast / sqrt(1.0 - ctf->amplitude_contrast * ctf->amplitude_contrast));
  k.pixel_size = ctf->pixel_size;
  k.b_factor = ctf->b_factor;
  constexpr int G = 64;
  const size_t smem = sizeof(float2) * (size_t)(4 * G * (G / 2 + 1) + G) +
                      sizeof(float) * (size_t)(2 * G * (G / 2 + 1) + G * G);
  if (cudaFuncSetAttribute(make_inputs_kernel<G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return LGB_ERR_CUDA;
  make_inputs_kernel<G><<<n_particles, 256, smem, (cudaStream_t)stream>>>(
      static_cast<const float2*>(particle_dft), image_h, image_w, static_cast<const float2*>(template_dft),
      template_size, rotations, defocus_u, defocus_v, defocus_angle, k, out_channels, static_cast<bf16*>(out));
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

int lgb_nn_gauss_newton(int n_particles, int band, int channels, void* inputs, float* gn, void* stream) {
  if (n_particles < 1 || channels < kNnChannels || !inputs || !gn) return LGB_ERR_INVALID_ARGUMENT;
  if (band != 64) return LGB_ERR_UNSUPPORTED_SIZE;
  gauss_newton_kernel<64><<<n_particles, 256, 0, (cudaStream_t)stream>>>(static_cast<bf16*>(inputs), channels, gn);
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

}  // extern "C"
