// C-ABI entry points of the GB300 2DTM search (declared in include/leopard_gb300.h).
#include <math.h>

#include <mutex>
#include <vector>

#include "match_kernels.cuh"
#include "match_launch.h"
#include "match_layout.h"
#include "profiler.h"

namespace lgb {

__global__ void init_stats_kernel(long long n, float* mip, int* best, double* s1, double* s2) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    mip[i] = -INFINITY;
    best[i] = -1;
    s1[i] = 0.0;
    s2[i] = 0.0;
  }
}

__global__ void repack_image_kernel(const float2* __restrict__ src, int H, int wc, int wcp, float2* __restrict__ dst) {
  const long long n = (long long)H * wcp;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(i / wcp), k = (int)(i % wcp);
    dst[i] = k < wc ? src[(size_t)y * wc + k] : make_float2(0.f, 0.f);
  }
}

__global__ void filters_kernel(const float* __restrict__ ctf, const float* __restrict__ wf, long long n_filters,
                               int plane, float* __restrict__ out) {
  const long long n = n_filters * plane;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = ctf[i] * wf[i % plane];
}

__global__ void finalize_kernel(long long n, int W, long long total, int n_orient, int n_defocus,
                                const float* __restrict__ mip, const int* __restrict__ best,
                                const double* __restrict__ s1, const double* __restrict__ s2,
                                const float* __restrict__ euler, const float* __restrict__ defocus, float* scaled,
                                float* phi, float* theta, float* psi, float* dfo, float* mean_out, float* std_out) {
  const long long stride_cs = (long long)n_orient * n_defocus;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double mean = s1[i] / (double)total;
    double var = s2[i] / (double)total - mean * mean;
    const double sd = sqrt(var > 0.0 ? var : 0.0);
    const float m = mip[i];
    scaled[i] = sd != 0.0 ? (float)(((double)m - mean) / sd) : 0.0f;
    mean_out[i] = (float)mean;
    std_out[i] = (float)sd;
    // python-style modulo: -1 (never updated) maps to the last index
    long long g = best[i];
    long long rem = g % stride_cs;
    if (rem < 0) rem += stride_cs;
    const int df = (int)(rem / n_orient);
    const int o = (int)(rem % n_orient);
    phi[i] = euler[3 * (size_t)o];
    theta[i] = euler[3 * (size_t)o + 1];
    psi[i] = euler[3 * (size_t)o + 2];
    dfo[i] = defocus[df];
  }
}

// ---------------------------------------------------------------------------
// Stage profiler: while enabled, every stage launch of lgb_match_search is
// bracketed by two CUDA events recorded on the launching stream.
// ---------------------------------------------------------------------------
struct StageEvent {
  int stage;
  cudaEvent_t start, stop;
};
static std::mutex g_prof_mu;
static bool g_prof_on = false;
static std::vector<StageEvent> g_prof_events;

bool profiling_on() { return g_prof_on; }
void profile_record(int stage, cudaEvent_t a, cudaEvent_t b) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_prof_events.push_back({stage, a, b});
}

static int grid_for(long long n) {
  long long g = (n + 255) / 256;
  if (g > 65535LL * 16) g = 65535LL * 16;
  return (int)(g < 1 ? 1 : g);
}

__global__ void set_cursor_kernel(int* cursor, int value) { *cursor = value; }
__global__ void advance_cursor_kernel(int* cursor, int step) { *cursor += step; }

// Validated pointers and layout of one search call.
struct SearchArgs {
  const lgb_match_problem* p;
  MatchLayout L;
  char* ws;
  const void* template_dft;
  const float* pf;
  const float* euler;
  float* mip;
  int* best;
  double* s1;
  double* s2;
};

int check_search_args(const lgb_match_problem* p, const void* template_dft, const float* pf, const float* euler,
                      int begin, int end, const float* mip, const int* best, const double* s1, const double* s2) {
  if (!valid_problem(p) || !template_dft || !pf || !euler || !mip || !best || !s1 || !s2)
    return LGB_ERR_INVALID_ARGUMENT;
  if (begin < 0 || end > p->n_orientations || begin > end) return LGB_ERR_INVALID_ARGUMENT;
  if (!lgb_match_supported(p)) return LGB_ERR_UNSUPPORTED_SIZE;
  const long long total_idx = (long long)p->n_orientations * p->n_defocus * p->n_pixel_sizes;
  if (total_idx > 2147483647LL) return LGB_ERR_INVALID_ARGUMENT;  // int32 global index, as the reference
  // the row pass keeps each pixel's batch argmax in 16 bits
  if ((long long)p->n_pixel_sizes * p->n_defocus * p->orientation_batch > 0xffff) return LGB_ERR_INVALID_ARGUMENT;
  return LGB_OK;
}

static int search_args(const lgb_match_problem* p, const void* template_dft, const float* pf, const float* euler,
                       int begin, int end, float* mip, int* best, double* s1, double* s2, void* workspace,
                       size_t workspace_bytes, SearchArgs* a) {
  const int st = check_search_args(p, template_dft, pf, euler, begin, end, mip, best, s1, s2);
  if (st != LGB_OK) return st;
  if (!workspace) return LGB_ERR_INVALID_ARGUMENT;
  a->p = p;
  a->L = layout_of(p);
  if (workspace_bytes < a->L.total) return LGB_ERR_WORKSPACE_TOO_SMALL;
  a->ws = static_cast<char*>(workspace);
  a->template_dft = template_dft;
  a->pf = pf;
  a->euler = euler;
  a->mip = mip;
  a->best = best;
  a->s1 = s1;
  a->s2 = s2;
  return LGB_OK;
}

// The six kernels of one orientation batch: orientations o0 (+ *o0_dev when
// given) .. + nb.  `profile` brackets each launch with the stage profiler's
// events (off while a graph is being captured).
static int run_batch(const SearchArgs& a, int o0, const int* o0_dev, int nb, bool profile, cudaStream_t s) {
  const lgb_match_problem* p = a.p;
  const MatchLayout& L = a.L;
  void* ip = a.ws + L.ip;
  void* slices = a.ws + L.slices;
  void* T = a.ws + L.t;
  float* proj = reinterpret_cast<float*>(a.ws + L.proj);
  double* rowstats = reinterpret_cast<double*>(a.ws + L.rowstats);
  void* A = a.ws + L.a;
  void* Y = a.ws + L.y;
  const int h = p->template_size, H = p->image_h, W = p->image_w;
  const int y_rows = mic_h(p);
  const int n_cd = p->n_pixel_sizes * p->n_defocus;
  const int n_c = n_cd * nb;
  const bool prof = profile && profiling_on();
  int st;
  {
    StageScope sc(LGB_STAGE_SLICE, s, prof);
    if ((st = launch_slice(a.template_dft, h, a.euler, o0, o0_dev, nb, nullptr, slices, s))) return st;
  }
  {
    StageScope sc(LGB_STAGE_PROJ_COL, s, prof);
    if ((st = launch_proj_col(h, slices, a.pf, nb, n_cd, n_c, T, s))) return st;
  }
  {
    StageScope sc(LGB_STAGE_PROJ_ROW, s, prof);
    if ((st = launch_proj_row(h, T, n_c, proj, rowstats, s))) return st;
  }
  {
    StageScope sc(LGB_STAGE_PAD_RFFT, s, prof);
    if ((st = launch_pad_rfft(W, proj, rowstats, h, mic_h(p), mic_w(p), L.wcp, n_c, A, s))) return st;
  }
  {
    StageScope sc(LGB_STAGE_COLPASS, s, prof);
    if ((st = launch_colpass(H, A, ip, h, L.wcp, n_c, n_c, y_rows, p->col_waves, Y, s))) return st;
  }
  {
    StageScope sc(LGB_STAGE_ROWPASS, s, prof);
    if ((st = launch_rowpass(W, Y, H, y_rows, L.wcp, n_c, nb, p->n_orientations, o0, o0_dev, a.mip, a.best, a.s1,
                             a.s2, s)))
      return st;
  }
  return LGB_OK;
}

}  // namespace lgb

using namespace lgb;

extern "C" {

const char* lgb_status_string(int status) {
  switch (status) {
    case LGB_OK:
      return "ok";
    case LGB_ERR_INVALID_ARGUMENT:
      return "invalid argument";
    case LGB_ERR_UNSUPPORTED_SIZE:
      return "unsupported FFT size";
    case LGB_ERR_WORKSPACE_TOO_SMALL:
      return "workspace too small";
    case LGB_ERR_CUDA:
      return "CUDA error";
    case LGB_ERR_DEVICE_TIMEOUT:
      return "device-side wait timed out";
    default:
      return "unknown status";
  }
}

int lgb_version(void) { return 100; }

int lgb_profile_begin(void) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  for (auto& e : g_prof_events) {
    cudaEventDestroy(e.start);
    cudaEventDestroy(e.stop);
  }
  g_prof_events.clear();
  g_prof_on = true;
  return LGB_OK;
}

int lgb_profile_end(double* stage_ms, long long* stage_launches, int n_stages) {
  if (!stage_ms || !stage_launches || n_stages < LGB_N_STAGES) return LGB_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_prof_on = false;
  for (int i = 0; i < n_stages; ++i) {
    stage_ms[i] = 0.0;
    stage_launches[i] = 0;
  }
  int st = LGB_OK;
  for (auto& e : g_prof_events) {
    float ms = 0.f;
    if (cudaEventSynchronize(e.stop) != cudaSuccess || cudaEventElapsedTime(&ms, e.start, e.stop) != cudaSuccess)
      st = LGB_ERR_CUDA;
    stage_ms[e.stage] += ms;
    stage_launches[e.stage] += 1;
    cudaEventDestroy(e.start);
    cudaEventDestroy(e.stop);
  }
  g_prof_events.clear();
  return st;
}

int lgb_match_supported(const lgb_match_problem* p) {
  if (!valid_problem(p)) return 0;
  return supported_template(p->template_size) && supported_row(p->image_w) && supported_col(p->image_h);
}

int lgb_match_fft_size(int n, int axis) {
  if (n < 1 || (axis != 0 && axis != 1)) return 0;
  for (int m = n; m <= 2 * n + 64; ++m)
    if (axis == 0 ? supported_col(m) : supported_row(m)) return m;
  return 0;
}

int lgb_match_workspace_size(const lgb_match_problem* p, size_t* bytes) {
  if (!valid_problem(p) || !bytes) return LGB_ERR_INVALID_ARGUMENT;
  *bytes = layout_of(p).total;
  return LGB_OK;
}

int lgb_match_init_stats(long long n_pixels, float* mip, int* best_index, double* corr_sum, double* corr_sq_sum,
                         void* stream) {
  if (n_pixels < 0 || (n_pixels > 0 && (!mip || !best_index || !corr_sum || !corr_sq_sum)))
    return LGB_ERR_INVALID_ARGUMENT;
  if (n_pixels == 0) return LGB_OK;
  init_stats_kernel<<<grid_for(n_pixels), 256, 0, (cudaStream_t)stream>>>(n_pixels, mip, best_index, corr_sum,
                                                                           corr_sq_sum);
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

int lgb_match_prepare_image(const lgb_match_problem* p, const void* image_dft, void* workspace,
                            size_t workspace_bytes, void* stream) {
  if (!valid_problem(p) || !image_dft || !workspace) return LGB_ERR_INVALID_ARGUMENT;
  const MatchLayout L = layout_of(p);
  if (workspace_bytes < L.total) return LGB_ERR_WORKSPACE_TOO_SMALL;
  float2* ip = reinterpret_cast<float2*>(static_cast<char*>(workspace) + L.ip);
  repack_image_kernel<<<grid_for((long long)p->image_h * L.wcp), 256, 0, (cudaStream_t)stream>>>(
      static_cast<const float2*>(image_dft), p->image_h, L.wc_img, L.wcp, ip);
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

int lgb_match_filters(const lgb_match_problem* p, const float* ctf_filters, const float* whitening,
                      float* projective_filters, void* stream) {
  if (!valid_problem(p) || !ctf_filters || !whitening || !projective_filters) return LGB_ERR_INVALID_ARGUMENT;
  const int plane = p->template_size * (p->template_size / 2 + 1);
  const long long nf = (long long)p->n_pixel_sizes * p->n_defocus;
  filters_kernel<<<grid_for(nf * plane), 256, 0, (cudaStream_t)stream>>>(ctf_filters, whitening, nf, plane,
                                                                         projective_filters);
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

int lgb_match_search(const lgb_match_problem* p, const void* template_dft, const float* projective_filters,
                     const float* euler_angles, int orientation_begin, int orientation_end, float* mip,
                     int* best_index, double* corr_sum, double* corr_sq_sum, void* workspace, size_t workspace_bytes,
                     void* stream) {
  SearchArgs a{};
  int st = search_args(p, template_dft, projective_filters, euler_angles, orientation_begin, orientation_end, mip,
                       best_index, corr_sum, corr_sq_sum, workspace, workspace_bytes, &a);
  if (st != LGB_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  for (int o0 = orientation_begin; o0 < orientation_end; o0 += p->orientation_batch) {
    const int nb = (orientation_end - o0) < p->orientation_batch ? (orientation_end - o0) : p->orientation_batch;
    if ((st = run_batch(a, o0, nullptr, nb, true, s))) return st;
  }
  return LGB_OK;
}

int lgb_match_search_graph(const lgb_match_problem* p, const void* template_dft, const float* projective_filters,
                           const float* euler_angles, int orientation_begin, int orientation_end,
                           int batches_per_graph, float* mip, int* best_index, double* corr_sum,
                           double* corr_sq_sum, void* workspace, size_t workspace_bytes, void* stream) {
  if (batches_per_graph < 1) return LGB_ERR_INVALID_ARGUMENT;
  SearchArgs a{};
  int st = search_args(p, template_dft, projective_filters, euler_angles, orientation_begin, orientation_end, mip,
                       best_index, corr_sum, corr_sq_sum, workspace, workspace_bytes, &a);
  if (st != LGB_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const long long chunk = (long long)batches_per_graph * p->orientation_batch;
  const long long replays = (orientation_end - orientation_begin) / chunk;
  if (replays > 0) {
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone)
      return LGB_ERR_INVALID_ARGUMENT;
    int* cursor = reinterpret_cast<int*>(a.ws + a.L.cursor);
    cudaStream_t cs = nullptr;
    if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) return LGB_ERR_CUDA;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    st = LGB_OK;
    if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      st = LGB_ERR_CUDA;
    } else {
      for (int m = 0; m < batches_per_graph && st == LGB_OK; ++m)
        st = run_batch(a, m * p->orientation_batch, cursor, p->orientation_batch, false, cs);
      if (st == LGB_OK) {
        advance_cursor_kernel<<<1, 1, 0, cs>>>(cursor, (int)chunk);
        if (cudaGetLastError() != cudaSuccess) st = LGB_ERR_CUDA;
      }
      if (cudaStreamEndCapture(cs, &graph) != cudaSuccess && st == LGB_OK) st = LGB_ERR_CUDA;
    }
    if (st == LGB_OK && cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) st = LGB_ERR_CUDA;
    if (st == LGB_OK) {
      set_cursor_kernel<<<1, 1, 0, s>>>(cursor, orientation_begin);
      if (cudaGetLastError() != cudaSuccess) st = LGB_ERR_CUDA;
      for (long long r = 0; r < replays && st == LGB_OK; ++r)
        if (cudaGraphLaunch(exec, s) != cudaSuccess) st = LGB_ERR_CUDA;
    }
    // in-flight launches complete before the executable graph is freed
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cs);
    if (st != LGB_OK) return st;
  }
  for (long long o0 = orientation_begin + replays * chunk; o0 < orientation_end; o0 += p->orientation_batch) {
    const int nb = (int)((orientation_end - o0) < p->orientation_batch ? (orientation_end - o0) : p->orientation_batch);
    if ((st = run_batch(a, (int)o0, nullptr, nb, true, s))) return st;
  }
  return LGB_OK;
}

int lgb_match_finalize(const lgb_match_problem* p, long long total_positions, const float* mip,
                       const int* best_index, const double* corr_sum, const double* corr_sq_sum,
                       const float* euler_angles, const float* defocus_values, float* scaled_mip, float* best_phi,
                       float* best_theta, float* best_psi, float* best_defocus, float* corr_mean, float* corr_std,
                       void* stream) {
  if (!valid_problem(p) || total_positions <= 0 || !mip || !best_index || !corr_sum || !corr_sq_sum ||
      !euler_angles || !defocus_values || !scaled_mip || !best_phi || !best_theta || !best_psi || !best_defocus ||
      !corr_mean || !corr_std)
    return LGB_ERR_INVALID_ARGUMENT;
  const long long n = (long long)p->image_h * p->image_w;
  finalize_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(
      n, p->image_w, total_positions, p->n_orientations, p->n_defocus, mip, best_index, corr_sum, corr_sq_sum,
      euler_angles, defocus_values, scaled_mip, best_phi, best_theta, best_psi, best_defocus, corr_mean, corr_std);
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

}  // extern "C"
