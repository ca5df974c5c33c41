// Plan-based form of the search ABI: one handle owns the device workspace,
// the projective-filter stack and the four statistics maps of one search
// shape, so a host program (C, C++, or any FFI) drives a micrograph with
// create -> set_filters -> set_image -> search (any number of orientation
// ranges) -> finalize -> destroy, without managing scratch memory itself.
// Every call is asynchronous on the given stream except create/destroy.
#include <new>

#include "match_layout.h"

namespace lgb {

struct MatchPlan {
  lgb_match_problem problem;
  int device;
  void* workspace = nullptr;
  size_t workspace_bytes = 0;
  float* filters = nullptr;
  float* mip = nullptr;
  int* best = nullptr;
  double* s1 = nullptr;
  double* s2 = nullptr;
  long long searched = 0;  // orientations folded into the maps
};

static void plan_free(MatchPlan* p) {
  if (!p) return;
  int cur = -1;
  cudaGetDevice(&cur);
  if (cur != p->device) cudaSetDevice(p->device);
  cudaFree(p->workspace);
  cudaFree(p->filters);
  cudaFree(p->mip);
  cudaFree(p->best);
  cudaFree(p->s1);
  cudaFree(p->s2);
  if (cur >= 0 && cur != p->device) cudaSetDevice(cur);
  delete p;
}

}  // namespace lgb

using namespace lgb;

extern "C" {

lgb_match_plan* lgb_match_plan_create(const lgb_match_problem* problem, int* status) {
  int st = LGB_OK;
  MatchPlan* p = nullptr;
  if (!problem || !valid_problem(problem)) {
    st = LGB_ERR_INVALID_ARGUMENT;
  } else if (!lgb_match_supported(problem)) {
    st = LGB_ERR_UNSUPPORTED_SIZE;
  } else {
    p = new (std::nothrow) MatchPlan();
    if (!p) {
      st = LGB_ERR_CUDA;
    } else {
      p->problem = *problem;
      cudaGetDevice(&p->device);
      const size_t n = (size_t)problem->image_h * problem->image_w;
      const size_t nf = (size_t)problem->n_pixel_sizes * problem->n_defocus * problem->template_size *
                        (problem->template_size / 2 + 1);
      if (lgb_match_workspace_size(problem, &p->workspace_bytes) != LGB_OK ||
          cudaMalloc(&p->workspace, p->workspace_bytes) != cudaSuccess ||
          cudaMalloc(reinterpret_cast<void**>(&p->filters), nf * sizeof(float)) != cudaSuccess ||
          cudaMalloc(reinterpret_cast<void**>(&p->mip), n * sizeof(float)) != cudaSuccess ||
          cudaMalloc(reinterpret_cast<void**>(&p->best), n * sizeof(int)) != cudaSuccess ||
          cudaMalloc(reinterpret_cast<void**>(&p->s1), n * sizeof(double)) != cudaSuccess ||
          cudaMalloc(reinterpret_cast<void**>(&p->s2), n * sizeof(double)) != cudaSuccess) {
        plan_free(p);
        p = nullptr;
        st = LGB_ERR_CUDA;
      }
    }
  }
  if (status) *status = st;
  return reinterpret_cast<lgb_match_plan*>(p);
}

void lgb_match_plan_destroy(lgb_match_plan* plan) { plan_free(reinterpret_cast<MatchPlan*>(plan)); }

int lgb_match_plan_set_filters(lgb_match_plan* plan, const float* ctf_filters, const float* whitening,
                               void* stream) {
  MatchPlan* p = reinterpret_cast<MatchPlan*>(plan);
  if (!p) return LGB_ERR_INVALID_ARGUMENT;
  return lgb_match_filters(&p->problem, ctf_filters, whitening, p->filters, stream);
}

int lgb_match_plan_set_image(lgb_match_plan* plan, const void* image_dft, void* stream) {
  MatchPlan* p = reinterpret_cast<MatchPlan*>(plan);
  if (!p) return LGB_ERR_INVALID_ARGUMENT;
  int st = lgb_match_prepare_image(&p->problem, image_dft, p->workspace, p->workspace_bytes, stream);
  if (st != LGB_OK) return st;
  p->searched = 0;
  return lgb_match_init_stats((long long)p->problem.image_h * p->problem.image_w, p->mip, p->best, p->s1, p->s2,
                              stream);
}

int lgb_match_plan_search(lgb_match_plan* plan, const void* template_dft, const float* euler_angles,
                          int orientation_begin, int orientation_end, void* stream) {
  MatchPlan* p = reinterpret_cast<MatchPlan*>(plan);
  if (!p) return LGB_ERR_INVALID_ARGUMENT;
  const int st = lgb_match_search(&p->problem, template_dft, p->filters, euler_angles, orientation_begin,
                                  orientation_end, p->mip, p->best, p->s1, p->s2, p->workspace, p->workspace_bytes,
                                  stream);
  if (st == LGB_OK) p->searched += orientation_end - orientation_begin;
  return st;
}

int lgb_match_plan_maps(lgb_match_plan* plan, float** mip, int** best_index, double** corr_sum,
                        double** corr_sq_sum) {
  MatchPlan* p = reinterpret_cast<MatchPlan*>(plan);
  if (!p || !mip || !best_index || !corr_sum || !corr_sq_sum) return LGB_ERR_INVALID_ARGUMENT;
  *mip = p->mip;
  *best_index = p->best;
  *corr_sum = p->s1;
  *corr_sq_sum = p->s2;
  return LGB_OK;
}

int lgb_match_plan_finalize(lgb_match_plan* plan, const float* euler_angles, const float* defocus_values,
                            float* scaled_mip, float* best_phi, float* best_theta, float* best_psi,
                            float* best_defocus, float* corr_mean, float* corr_std, void* stream) {
  MatchPlan* p = reinterpret_cast<MatchPlan*>(plan);
  if (!p || p->searched <= 0) return LGB_ERR_INVALID_ARGUMENT;
  const long long total = p->searched * p->problem.n_defocus * p->problem.n_pixel_sizes;
  return lgb_match_finalize(&p->problem, total, p->mip, p->best, p->s1, p->s2, euler_angles, defocus_values,
                            scaled_mip, best_phi, best_theta, best_psi, best_defocus, corr_mean, corr_std, stream);
}

}  // extern "C"
