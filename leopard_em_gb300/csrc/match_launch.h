// Internal launchers of the plain FP32 search kernels (one translation unit
// per kernel family so the size instantiations compile in parallel).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include "../../include/leopard_gb300.h"

namespace lgb {

// Each returns an lgb_status; LGB_ERR_UNSUPPORTED_SIZE when the FFT length is
// not instantiated.
// Slices for nb rotations: from Euler angles euler[o0 + *o0_dev + b] (rotations
// == nullptr; o0_dev may be null) or from row-major 3x3 matrices rotations[9*b].
int launch_slice(const void* vol, int d, const float* euler, int o0, const int* o0_dev, int nb,
                 const float* rotations, void* slices, cudaStream_t s);
// Refine row pass (valid crop, z-score, per-particle packed arg-max); see refine.cu.
int launch_refine_rowpass(int W, const void* Y, int y_rows, int Wcp, int n_cpp, int n_particles, int crop_h,
                          int crop_w, float scale, const float* corr_mean, const float* corr_std,
                          unsigned long long* slot_key, unsigned* slot_cc, cudaStream_t s);
bool supported_refine_row(int W);
// c = (p*n_cd + cd)*nb + b; slices [P][nb], filters [P][n_cd] (P = n_c / (n_cd*nb))
int launch_proj_col(int h, const void* slices, const float* pf, int nb, int n_cd, int n_c, void* T, cudaStream_t s);
int launch_proj_row(int h, const void* T, int n_c, float* proj, double* rowstats, cudaStream_t s);
// proj_row and the zero-padded row rfft of the un-normalised projection in one
// kernel (h = 256, W = 288 only): A[c][py][k] = rfft_W(p[py])[k], row moments
// in rowstats.  The column pass then applies the normalisation (norm below).
bool supported_proj_row_rfft(int h, int W);
int launch_proj_row_rfft(int h, int W, const void* T, int n_c, double* rowstats, int Wcp, void* A, cudaStream_t s);
// Per-correlogram normalisation constants (e, s) from the row moments, stored
// as a float2 over rowstats[c][0][0].
int launch_norm_constants(double* rowstats, int n_c, int h, int norm_h, int norm_w, cudaStream_t s);
// Projections normalised for a norm_h x norm_w micrograph (utils.py:106-188),
// rfft'd at length W (W >= norm_w: zero padding beyond the micrograph).
int launch_pad_rfft(int W, const float* proj, const double* rowstats, int h, int norm_h, int norm_w, int Wcp,
                    int n_c, void* A, cudaStream_t s);
// Ip holds one padded spectrum per image; correlogram c uses image c / c_per_image.
// Only rows y < y_rows of each inverse column transform are stored (Y is [n_c][y_rows][Wcp]).
// waves: the correlogram range is split until the grid covers about waves x
// the SM count (0 = 4).
// norm (H = 288 only; null otherwise): A holds un-normalised row spectra of
// length norm_w rows and correlogram c is normalised on load as
// s (A - e U[kx]), (e, s) = norm[c * norm_stride], U[k] = sum_{x < h} exp(-2 pi i k x / norm_w).
int launch_colpass(int H, const void* A, const void* Ip, int h, int Wcp, int n_c, int c_per_image, int y_rows,
                   int waves, void* Y, cudaStream_t s, const float2* norm = nullptr, int norm_stride = 0,
                   int norm_w = 0);
// Rows y < y_rows of the H x W correlograms (Y is [n_c][y_rows][Wcp]); global
// index base o0 + *o0_dev (o0_dev may be null).
int launch_rowpass(int W, const void* Y, int H, int y_rows, int Wcp, int n_c, int nb, int n_orient, int o0,
                   const int* o0_dev, float* mip, int* best, double* s1, double* s2, cudaStream_t s);

// Every argument check of lgb_match_search except the workspace; LGB_OK or
// the status lgb_match_search would return.  Runs no GPU work.
int check_search_args(const lgb_match_problem* p, const void* template_dft, const float* pf, const float* euler,
                      int begin, int end, const float* mip, const int* best, const double* s1, const double* s2);

bool supported_template(int h);
bool supported_row(int W);
bool supported_col(int H);

}  // namespace lgb
