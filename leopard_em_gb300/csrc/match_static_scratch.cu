// Whole-orientation search that allocates no device memory.
//
// Who needs it: callers that cannot call cudaMalloc -- code embedded in a host
// application that owns every byte of device memory through its own pool and
// forbids outside allocations (an acquisition or processing pipeline running
// under a fixed memory budget), and code that must not trigger the implicit
// device synchronisation cudaMalloc / cudaFree can cause while other streams
// are busy.  Such callers still pass every input and output buffer; the
// kernels' scratch (the padded image spectrum and the per-batch projection
// and correlogram intermediates) lives in the fixed-size device array below.
//
// Contract:
//   * capacity is kStaticScratchBytes (32 MiB).  Problems whose scratch need
//     (lgb_match_workspace_size) is larger are rejected with
//     LGB_ERR_WORKSPACE_TOO_SMALL before any GPU work;
//   * the array is part of the library image: every GPU that loads the
//     library holds these 32 MiB until the process exits;
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (with that device current) and caches it; make that
//     first call before any stream capture on the device.  The cached address
//     belongs to the device's primary context: the library must not be used
//     again on a device after cudaDeviceReset (which destroys that context and
//     the array with it);
//   * every argument is checked before any GPU work: a rejected call leaves
//     the array untouched;
//   * all calls share the one array, which keeps the last call's contents.
//     Every byte the kernels read is rewritten earlier in the same call (the
//     image spectrum is repacked, zero padding included, at the start of each
//     call), so nothing has to start at zero.  Calls whose GPU work overlaps
//     (different streams, or different host threads without ordering) race on
//     the array; serialise them.
#include <mutex>

#include "match_kernels.cuh"
#include "match_launch.h"

namespace lgb {

constexpr size_t kStaticScratchBytes = size_t(32) << 20;
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
static void* g_static_scratch_ptr[kMaxDevices] = {};
static std::mutex g_static_scratch_mu;

// Device address of g_static_scratch on the current device (cached per device).
static int static_scratch_address(void** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return LGB_ERR_CUDA;
  if (dev >= kMaxDevices) return LGB_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(g_static_scratch_mu);
  if (!g_static_scratch_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_static_scratch) != cudaSuccess || p == nullptr) return LGB_ERR_CUDA;
    g_static_scratch_ptr[dev] = p;
  }
  *out = g_static_scratch_ptr[dev];
  return LGB_OK;
}

}  // namespace lgb

extern "C" {

size_t lgb_static_scratch_capacity(void) { return lgb::kStaticScratchBytes; }

int lgb_match_search_static_scratch(const lgb_match_problem* problem, const void* image_dft,
                                    const void* template_dft, const float* projective_filters,
                                    const float* euler_angles, int orientation_begin, int orientation_end,
                                    float* mip, int* best_index, double* corr_sum, double* corr_sq_sum,
                                    void* stream) {
  size_t need = 0;
  int st = lgb_match_workspace_size(problem, &need);
  if (st != LGB_OK) return st;
  if (need > lgb::kStaticScratchBytes) return LGB_ERR_WORKSPACE_TOO_SMALL;
  if (!image_dft) return LGB_ERR_INVALID_ARGUMENT;
  // all of lgb_match_search's checks before the image repack touches the array
  if ((st = lgb::check_search_args(problem, template_dft, projective_filters, euler_angles, orientation_begin,
                                   orientation_end, mip, best_index, corr_sum, corr_sq_sum)) != LGB_OK)
    return st;
  void* scratch = nullptr;
  if ((st = lgb::static_scratch_address(&scratch)) != LGB_OK) return st;
  if ((st = lgb_match_prepare_image(problem, image_dft, scratch, lgb::kStaticScratchBytes, stream)) != LGB_OK)
    return st;
  return lgb_match_search(problem, template_dft, projective_filters, euler_angles, orientation_begin, orientation_end,
                          mip, best_index, corr_sum, corr_sq_sum, scratch, lgb::kStaticScratchBytes, stream);
}

}  // extern "C"
