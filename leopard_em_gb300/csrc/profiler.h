// Stage profiler shared by the search drivers: while lgb_profile_begin is in
// effect, every stage launch wrapped in a StageScope is bracketed by two CUDA
// events recorded on the launching stream (collected by lgb_profile_end).
#pragma once

#include <cuda_runtime.h>

namespace lgb {

bool profiling_on();
void profile_record(int stage, cudaEvent_t a, cudaEvent_t b);

struct StageScope {
  int stage;
  cudaStream_t s;
  cudaEvent_t a = nullptr, b = nullptr;
  StageScope(int st, cudaStream_t str, bool on) : stage(st), s(str) {
    if (!on) return;
    if (cudaEventCreate(&a) == cudaSuccess && cudaEventCreate(&b) == cudaSuccess) cudaEventRecord(a, s);
  }
  ~StageScope() {
    if (!a || !b) return;
    cudaEventRecord(b, s);
    profile_record(stage, a, b);
  }
};

}  // namespace lgb
