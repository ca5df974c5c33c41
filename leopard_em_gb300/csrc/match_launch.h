// Internal launchers of the plain FP32 search kernels (one translation unit
// per kernel family so the size instantiations compile in parallel).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

namespace lgb {

// Each returns an lgb_status; LGB_ERR_UNSUPPORTED_SIZE when the FFT length is
// not instantiated.
int launch_slice(const void* vol, int d, const float* euler, int o0, int nb, void* slices, cudaStream_t s);
int launch_proj_col(int h, const void* slices, const float* pf, int nb, int n_c, void* T, cudaStream_t s);
int launch_proj_row(int h, const void* T, int n_c, float* proj, double* rowstats, cudaStream_t s);
int launch_pad_rfft(int W, const float* proj, const double* rowstats, int h, int H, int Wcp, int n_c, void* A,
                    cudaStream_t s);
int launch_colpass(int H, const void* A, const void* Ip, int h, int Wcp, int n_c, void* Y, cudaStream_t s);
int launch_rowpass(int W, const void* Y, int H, int Wcp, int n_c, int nb, int n_orient, int o0, float* mip,
                   int* best, double* s1, double* s2, cudaStream_t s);

bool supported_template(int h);
bool supported_row(int W);
bool supported_col(int H);

}  // namespace lgb
