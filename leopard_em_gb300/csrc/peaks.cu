// Peak picking on the z-score map on the device: candidates above a cutoff,
// greedy suppression within a radius in descending order of value
// (analysis/zscore_metric.py:43-84 find_peaks_from_zscore with
// analysis/utils.py:6-50 filter_peaks_by_distance).
//
// The reference sorts the candidates and walks them in order, picking a peak
// unless an already picked one lies closer than the radius.  That recursive
// rule has a unique solution, which is computed here without a global sort:
// a candidate is decided once every higher-ranked candidate within the radius
// is decided -- picked if none of them was picked, suppressed otherwise.
// Rounds of one kernel over the map settle the candidates chain by chain
// (status transitions are final, so in-place updates are safe).  Rank order:
// larger value first, equal values in row-major order (the order of
// torch.nonzero, kept by a stable sort).  Distances are sqrtf(dy^2 + dx^2) <
// radius in FP32, as torch.norm on the float coordinates.
#include "common.cuh"

namespace lgb {

enum : unsigned char { kNotCand = 0, kUndecided = 1, kPicked = 2, kSuppressed = 3 };

__global__ void peaks_init_kernel(long long n, const float* __restrict__ z, float cutoff,
                                  unsigned char* __restrict__ status) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    status[i] = z[i] > cutoff ? kUndecided : kNotCand;
}

__global__ void peaks_round_kernel(int H, int W, const float* __restrict__ z, float radius, int R,
                                   unsigned char* status, int* counters, int round) {
  if (round > 0 && *((volatile int*)&counters[round - 1]) == 0) return;  // settled already
  int remaining = 0;
  const long long n = (long long)H * W;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    if (*((volatile unsigned char*)&status[p]) != kUndecided) continue;
    const int y = (int)(p / W), x = (int)(p - (long long)y * W);
    const float zp = z[p];
    bool blocked = false, suppressed = false;
    for (int dy = -R; dy <= R && !suppressed; ++dy) {
      const int yy = y + dy;
      if (yy < 0 || yy >= H) continue;
      for (int dx = -R; dx <= R; ++dx) {
        const int xx = x + dx;
        if (xx < 0 || xx >= W || (dy == 0 && dx == 0)) continue;
        if (!(sqrtf((float)(dy * dy + dx * dx)) < radius)) continue;
        const long long q = (long long)yy * W + xx;
        const unsigned char sq = *((volatile unsigned char*)&status[q]);
        if (sq == kNotCand) continue;
        const float zq = z[q];
        const bool higher = zq > zp || (zq == zp && q < p);
        if (!higher) continue;
        if (sq == kPicked) {
          suppressed = true;
          break;
        }
        if (sq == kUndecided) blocked = true;
      }
    }
    if (suppressed)
      status[p] = kSuppressed;
    else if (!blocked)
      status[p] = kPicked;
    else
      ++remaining;
  }
  // warp-aggregated count of the candidates still undecided
  for (int o = 16; o > 0; o >>= 1) remaining += __shfl_down_sync(0xffffffffu, remaining, o);
  if ((threadIdx.x & 31) == 0 && remaining) atomicAdd(&counters[round], remaining);
}

__global__ void peaks_collect_kernel(long long n, const unsigned char* __restrict__ status, int max_peaks,
                                     int* __restrict__ out, int* __restrict__ count) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    if (status[i] != kPicked) continue;
    const int k = atomicAdd(count, 1);
    if (k < max_peaks) out[k] = (int)i;
  }
}

static int grid_of(long long n) {
  long long g = (n + 255) / 256;
  if (g > 8192) g = 8192;
  return (int)(g < 1 ? 1 : g);
}

}  // namespace lgb

using namespace lgb;

extern "C" {

size_t lgb_peaks_scratch_size(int H, int W, int max_rounds) {
  if (H < 1 || W < 1 || max_rounds < 1) return 0;
  return (((size_t)H * W + 255) & ~(size_t)255) + sizeof(int) * (size_t)(max_rounds + 2);
}

int lgb_peaks_find(int H, int W, const float* zscore, float cutoff, float radius, int max_rounds, void* scratch,
                   size_t scratch_bytes, int max_peaks, int* peak_index, int* n_peaks, int* rounds_used,
                   void* stream) {
  if (H < 1 || W < 1 || !zscore || !(radius > 0.f) || radius > 256.f || max_rounds < 1 || !scratch ||
      max_peaks < 0 || (max_peaks > 0 && !peak_index) || !n_peaks || !rounds_used)
    return LGB_ERR_INVALID_ARGUMENT;
  if (scratch_bytes < lgb_peaks_scratch_size(H, W, max_rounds)) return LGB_ERR_WORKSPACE_TOO_SMALL;
  cudaStream_t s = (cudaStream_t)stream;
  const long long n = (long long)H * W;
  unsigned char* status = static_cast<unsigned char*>(scratch);
  int* counters = reinterpret_cast<int*>(static_cast<char*>(scratch) + (((size_t)n + 255) & ~(size_t)255));
  int* d_count = counters + max_rounds + 1;
  LGB_CUDA_TRY(cudaMemsetAsync(counters, 0, sizeof(int) * (size_t)(max_rounds + 2), s));
  peaks_init_kernel<<<grid_of(n), 256, 0, s>>>(n, zscore, cutoff, status);
  const int R = (int)ceilf(radius);
  // rounds in groups of 8 between host checks of the undecided count
  int used = 0, left = -1;
  while (used < max_rounds) {
    const int group = max_rounds - used < 8 ? max_rounds - used : 8;
    for (int r = 0; r < group; ++r)
      peaks_round_kernel<<<grid_of(n), 256, 0, s>>>(H, W, zscore, radius, R, status, counters, used + r);
    used += group;
    LGB_CUDA_TRY(cudaGetLastError());
    LGB_CUDA_TRY(cudaMemcpyAsync(&left, counters + used - 1, sizeof(int), cudaMemcpyDeviceToHost, s));
    LGB_CUDA_TRY(cudaStreamSynchronize(s));
    if (left == 0) break;
  }
  *rounds_used = used;
  if (left != 0) return LGB_ERR_DEVICE_TIMEOUT;  // did not settle within max_rounds
  peaks_collect_kernel<<<grid_of(n), 256, 0, s>>>(n, status, max_peaks, peak_index, d_count);
  LGB_CUDA_TRY(cudaGetLastError());
  LGB_CUDA_TRY(cudaMemcpyAsync(n_peaks, d_count, sizeof(int), cudaMemcpyDeviceToHost, s));
  LGB_CUDA_TRY(cudaStreamSynchronize(s));
  return LGB_OK;
}

}  // extern "C"
