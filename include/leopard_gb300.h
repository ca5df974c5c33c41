/*
 * leopard_gb300.h -- C ABI of the GB300 (sm_103a) 2DTM search library.
 *
 * Plain pointers and sizes only; every pointer argument marked "device" must
 * point to memory on the current CUDA device, and `stream` is a cudaStream_t
 * (NULL = legacy default stream).  All calls are asynchronous on `stream`
 * unless stated otherwise and return an lgb_status (0 = success).
 *
 * Reference interfaces these entry points replace (Leopard-EM, paths inside
 * the Leopard-EM source tree):
 *   lgb_match_init_stats      core_match_template.py:472-486
 *                             (mip=-inf, best index=-1, sums=0 in
 *                             _core_match_template_single_gpu)
 *   lgb_match_prepare_image   core_match_template.py:446 (image_dft.to(device))
 *   lgb_match_filters         core_match_template.py:274
 *                             (projective_filters = ctf * whitening)
 *   lgb_match_search          core_match_template.py:492-550, the orientation
 *                             loop: roma.euler_to_rotmat (:506-508), the
 *                             cross-correlation of cross_correlation.py:13-154
 *                             and do_iteration_statistics_updates
 *                             (backend/utils.py:191-255), fused
 *   lgb_match_search_graph    the same loop, replayed as a CUDA graph (the
 *                             reference launches every kernel of every batch
 *                             from Python, cross_correlation.py:60-154)
 *   lgb_match_finalize        core_match_template.py:337-349 ->
 *                             process_results.py:67-183
 *                             (decode_global_search_index, scale_mip)
 */
#ifndef LEOPARD_GB300_H
#define LEOPARD_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum lgb_status {
  LGB_OK = 0,
  LGB_ERR_INVALID_ARGUMENT = 1, /* null pointer, negative count, bad range   */
  LGB_ERR_UNSUPPORTED_SIZE = 2, /* an FFT length outside the compiled set    */
  LGB_ERR_WORKSPACE_TOO_SMALL = 3,
  LGB_ERR_CUDA = 4,             /* a CUDA runtime call or launch failed      */
  LGB_ERR_DEVICE_TIMEOUT = 5    /* a bounded device-side wait ran out        */
} lgb_status;

/* Shape of one whole-orientation search (one micrograph). */
typedef struct lgb_match_problem {
  int image_h;            /* H: rows of the correlation grid (image spectrum, maps) */
  int image_w;            /* W: columns of the correlation grid (even)              */
  int template_size;      /* d: cubic template edge; projections are d x d        */
  int n_pixel_sizes;      /* C: leading axis of the projective-filter stack       */
  int n_defocus;          /* D: second axis of the projective-filter stack        */
  int n_orientations;     /* N: rows of the Euler-angle table                     */
  int orientation_batch;  /* B: orientations correlated per statistics update     */
  /* Micrograph size when the image was zero padded to the H x W grid (0 = H or
   * W): projections are normalised for a micrograph_h x micrograph_w image
   * (utils.py:106-188) and only map rows < micrograph_h are computed.  With
   * padding, correlations at valid positions (y <= micrograph_h - d,
   * x <= micrograph_w - d) equal those of the unpadded search. */
  int micrograph_h;
  int micrograph_w;
  /* Column-pass launch shape: split correlograms over CTAs until the grid
   * covers about col_waves x the SM count (0 = 4).  Results do not depend on
   * it. */
  int col_waves;
} lgb_match_problem;

/* Kernel stages of one orientation batch inside lgb_match_search. */
enum {
  LGB_STAGE_SLICE = 0,    /* Fourier slice extraction                          */
  LGB_STAGE_PROJ_COL = 1, /* projective filter + inverse FFT along y           */
  LGB_STAGE_PROJ_ROW = 2, /* c2r along x, ifftshift, projection moments        */
  LGB_STAGE_PAD_RFFT = 3, /* normalisation + zero-padded row rfft              */
  LGB_STAGE_COLPASS = 4,  /* column FFT, cross power, inverse column FFT       */
  LGB_STAGE_ROWPASS = 5,  /* row c2r + MIP / index / sum statistics            */
  LGB_STAGE_COLFWD = 6,   /* precision form: column FFT + cross power -> operand */
  LGB_STAGE_DFT_COL = 7,  /* precision form: inverse column DFT-GEMM (tcgen05)   */
  LGB_STAGE_DFT_ROW = 8,  /* precision form: row c2r DFT-GEMM + statistics       */
  LGB_N_STAGES = 9
};

/* Human-readable text of a status code (static storage). */
const char* lgb_status_string(int status);

/* Library version, major*10000 + minor*100 + patch. */
int lgb_version(void);

/* Stage profiler (no reference counterpart; measurement only).  Between
 * lgb_profile_begin and lgb_profile_end every stage launch made by
 * lgb_match_search on any stream is bracketed by CUDA events on that stream.
 * lgb_profile_end waits for the recorded events and writes, per stage, the
 * summed device milliseconds and the launch count (arrays of n_stages >=
 * LGB_N_STAGES entries). */
int lgb_profile_begin(void);
int lgb_profile_end(double* stage_ms, long long* stage_launches, int n_stages);

/* 1 if every FFT length this problem needs is compiled in, else 0. */
int lgb_match_supported(const lgb_match_problem* problem);

/* Smallest compiled correlation-grid length >= n along an axis (0 = rows,
 * image_h; 1 = columns, image_w), or 0 if there is none.  A micrograph whose
 * size is not compiled is searched on the zero-padded grid (see
 * micrograph_h / micrograph_w).  No reference counterpart: torch.fft accepts
 * every length. */
int lgb_match_fft_size(int n, int axis);

/* Bytes of device scratch that lgb_match_search needs for `problem`. */
int lgb_match_workspace_size(const lgb_match_problem* problem, size_t* bytes);

/* mip <- -inf, best_index <- -1, corr_sum <- 0, corr_sq_sum <- 0 over n_pixels. */
int lgb_match_init_stats(long long n_pixels, float* mip, int* best_index, double* corr_sum,
                         double* corr_sq_sum, void* stream);

/* Copy the image spectrum (device, complex64 [H][W/2+1], row-major) into the
 * workspace's padded layout.  Must precede lgb_match_search on a workspace.
 * For a zero-padded micrograph this is the spectrum of the padded H x W image. */
int lgb_match_prepare_image(const lgb_match_problem* problem, const void* image_dft, void* workspace,
                            size_t workspace_bytes, void* stream);

/* projective_filters[c][d][y][x] = ctf_filters[c][d][y][x] * whitening[y][x]
 * over C x D x d x (d/2+1) floats (device pointers). */
int lgb_match_filters(const lgb_match_problem* problem, const float* ctf_filters, const float* whitening,
                      float* projective_filters, void* stream);

/* Correlate orientations [orientation_begin, orientation_end) in batches of
 * problem->orientation_batch against the prepared image and fold every
 * correlogram into the four per-pixel statistics maps (device, H x W):
 *   mip          running maximum (strict '>' across batches, first index wins)
 *   best_index   global search index  cs*D*N + df*N + orientation  (int32)
 *   corr_sum     running sum (FP64)
 *   corr_sq_sum  running sum of squares (FP64)
 * template_dft: device complex64 [d][d][d/2+1], fftshifted over the first two
 *   axes (volume_to_rfft_fourier_slice layout).
 * projective_filters: device float [C][D][d][d/2+1].
 * euler_angles: device float [N][3], ZYZ (phi, theta, psi) in degrees. */
int lgb_match_search(const lgb_match_problem* problem, const void* template_dft, const float* projective_filters,
                     const float* euler_angles, int orientation_begin, int orientation_end, float* mip,
                     int* best_index, double* corr_sum, double* corr_sq_sum, void* workspace,
                     size_t workspace_bytes, void* stream);

/* lgb_match_search through a CUDA graph: the kernels of batches_per_graph
 * orientation batches are captured once (on a private stream) with their
 * orientation offset read from a cursor in the workspace, and the graph is
 * replayed on `stream`, each replay advancing the cursor, until fewer than
 * batches_per_graph full batches remain; the rest runs as in
 * lgb_match_search.  Same results as lgb_match_search bit for bit.  The host
 * enqueues ceil(range / (B * batches_per_graph)) graph launches instead of
 * 6 kernel launches per batch; the graph is destroyed before returning (after
 * the launches are enqueued).  `stream` must not be capturing. */
int lgb_match_search_graph(const lgb_match_problem* problem, const void* template_dft,
                           const float* projective_filters, const float* euler_angles, int orientation_begin,
                           int orientation_end, int batches_per_graph, float* mip, int* best_index,
                           double* corr_sum, double* corr_sq_sum, void* workspace, size_t workspace_bytes,
                           void* stream);

/* Plan form of the same search: an opaque handle owning the workspace, the
 * projective filters and the four maps (device memory of the device current
 * at creation).  create/destroy allocate and free (synchronously); the others
 * are asynchronous on `stream`.  set_image (re)initialises the maps;
 * finalize divides by the orientations searched since then x D x C.
 * Replaces the per-device worker state of _core_match_template_single_gpu
 * (core_match_template.py:369-562). */
typedef struct lgb_match_plan lgb_match_plan;
lgb_match_plan* lgb_match_plan_create(const lgb_match_problem* problem, int* status);
void lgb_match_plan_destroy(lgb_match_plan* plan);
int lgb_match_plan_set_filters(lgb_match_plan* plan, const float* ctf_filters, const float* whitening, void* stream);
int lgb_match_plan_set_image(lgb_match_plan* plan, const void* image_dft, void* stream);
int lgb_match_plan_search(lgb_match_plan* plan, const void* template_dft, const float* euler_angles,
                          int orientation_begin, int orientation_end, void* stream);
int lgb_match_plan_maps(lgb_match_plan* plan, float** mip, int** best_index, double** corr_sum,
                        double** corr_sq_sum);
int lgb_match_plan_finalize(lgb_match_plan* plan, const float* euler_angles, const float* defocus_values,
                            float* scaled_mip, float* best_phi, float* best_theta, float* best_psi,
                            float* best_defocus, float* corr_mean, float* corr_std, void* stream);

/* lgb_match_search without any device allocation: no reference counterpart
 * (the reference always allocates through PyTorch).  For callers that cannot
 * call cudaMalloc -- code inside a host application that owns all device
 * memory through its own pool, or that must avoid the implicit device
 * synchronisation of cudaMalloc/cudaFree.  The caller passes every input and
 * output (image_dft: device complex64 [H][W/2+1]; the rest as in
 * lgb_match_search); scratch comes from a fixed array of
 * lgb_static_scratch_capacity() bytes (32 MiB) compiled into the library and
 * held by every GPU that loads it until the process exits.  Problems needing
 * more scratch (see lgb_match_workspace_size) fail with
 * LGB_ERR_WORKSPACE_TOO_SMALL.  The first call on a device resolves the
 * array's device address (cudaGetSymbolAddress): make it before any stream
 * capture.  All calls share the array and its contents persist between calls;
 * calls whose GPU work overlaps race on it and must be serialised. */
size_t lgb_static_scratch_capacity(void);
int lgb_match_search_static_scratch(const lgb_match_problem* problem, const void* image_dft,
                                    const void* template_dft, const float* projective_filters,
                                    const float* euler_angles, int orientation_begin, int orientation_end,
                                    float* mip, int* best_index, double* corr_sum, double* corr_sq_sum,
                                    void* stream);

/* Decode the best index and turn the sums into mean, standard deviation and
 * z-score (FP64 arithmetic, FP32 outputs; all maps device, H x W):
 *   corr_mean = S/total, corr_std = sqrt(max(S2/total - mean^2, 0)),
 *   scaled_mip = (mip - mean)/std, or 0 where std == 0.
 * `total_positions` is N*D*C of the whole search. */
int lgb_match_finalize(const lgb_match_problem* problem, long long total_positions, const float* mip,
                       const int* best_index, const double* corr_sum, const double* corr_sq_sum,
                       const float* euler_angles, const float* defocus_values, float* scaled_mip,
                       float* best_phi, float* best_theta, float* best_psi, float* best_defocus,
                       float* corr_mean, float* corr_std, void* stream);

/* ------------------------------------------------------------------------ */
/* Local-grid refinement (core_refine_template.py:33-202, :555-767)          */
/* ------------------------------------------------------------------------ */

/* Shape of one refinement call: P particle crops of H x W against a cubic
 * template of edge d, over K Euler-angle offsets (in batches of B), D defocus
 * offsets and C pixel-size offsets.  The valid crop is (H-d+1) x (W-d+1). */
typedef struct lgb_refine_problem {
  int image_h;
  int image_w;
  int template_size;
  int n_pixel_sizes;
  int n_defocus;
  int n_offsets;
  int offset_batch;
  int n_particles;
} lgb_refine_problem;

/* Microscope parameters of the CTF (ctf_utils.py:19-116 ctf_kwargs). */
typedef struct lgb_ctf_params {
  double voltage_kv;
  double spherical_aberration_mm;
  double amplitude_contrast;
  double b_factor;          /* B envelope exp(-B k^2 / 4), A^2 */
  double phase_shift_deg;
  double pixel_size;        /* A; the CTF grid and the Cs <-> pixel-size relation */
} lgb_ctf_params;

/* 1 if every FFT length of this refinement is compiled in, else 0. */
int lgb_refine_supported(const lgb_refine_problem* problem);

/* Bytes of device scratch lgb_refine_search needs. */
int lgb_refine_workspace_size(const lgb_refine_problem* problem, size_t* bytes);

/* Replaces _core_refine_template_single_thread (core_refine_template.py:555-767)
 * for P particles at once.  Device inputs: particle_stack_dft complex64
 * [P][H][W/2+1]; template_dft complex64 [d][d][d/2+1] (fftshifted); euler_angles
 * [P][3] and euler_offsets [K][3] (ZYZ degrees); defocus_u/v/angle [P] (A, A,
 * degrees); defocus_offsets [D] (A); pixel_size_offsets [C] (A); corr_mean /
 * corr_std [P][H-d+1][W-d+1]; projective_filters [P][d][d/2+1].  Per particle
 * the CTF stack (C x D, from `ctf`) times the projective filter filters each
 * slice; rotations are R(offset) @ R(particle).  Outputs (device, [P]): best
 * z-score and the largest correlation of the batch that produced it, the
 * winning flat index f = (y*(W-d+1) + x)*C*D*n + c (c = (cs*D + df)*n + b within
 * that batch of n offsets starting at best_offset_begin), or -1 if no batch
 * beat the initial -1e9. */
int lgb_refine_search(const lgb_refine_problem* problem, const lgb_ctf_params* ctf, const void* particle_stack_dft,
                      const void* template_dft, const float* euler_angles, const float* euler_offsets,
                      const float* defocus_u, const float* defocus_v, const float* defocus_angle,
                      const float* defocus_offsets, const float* pixel_size_offsets, const float* corr_mean,
                      const float* corr_std, const float* projective_filters, float* best_z, float* best_cc,
                      int* best_flat, int* best_offset_begin, int* best_batch_len, void* workspace,
                      size_t workspace_bytes, void* stream);

/* Precision form of lgb_match_search (mode 1: BF16 hi + lo, mode 2: FP16 hi +
 * lo operands): the inverse column DFT of the cross power and the row c2r
 * DFT run as split-precision DFT-GEMMs on the tcgen05 tensor cores with FP32
 * accumulation (cross_correlation.py:137-142), the statistics update
 * (utils.py:191-255) in the second GEMM's epilogue; everything else as in
 * lgb_match_search, same inputs, maps and index convention.  Supported when
 * the plain search is, the grid has no zero padding, 2H and W are multiples of
 * 128, H, W <= 1024, and C*D*B <= 32 (lgb_match_precision_supported).  The
 * workspace (lgb_match_precision_workspace_size bytes, 256-byte aligned) must
 * be prepared with lgb_match_prepare_image like the plain one.
 * device_status (device int, caller-zeroed) receives LGB_ERR_DEVICE_TIMEOUT if
 * a bounded device-side wait ran out. */
int lgb_match_precision_supported(const lgb_match_problem* problem, int mode);
int lgb_match_precision_workspace_size(const lgb_match_problem* problem, size_t* bytes);
int lgb_match_search_precision(const lgb_match_problem* problem, int mode, const void* template_dft,
                               const float* projective_filters, const float* euler_angles, int orientation_begin,
                               int orientation_end, float* mip, int* best_index, double* corr_sum,
                               double* corr_sq_sum, void* workspace, size_t workspace_bytes, int* device_status,
                               void* stream);

/* Cross-correlation of a particle stack with one projection per particle
 * (core_refine_template.py:771-895, cross_correlate_particle_stack).  Device
 * inputs: particle_dft complex64 [P][H][W/2+1] (filtered, un-shifted rfft2 of
 * the particles); template_dft complex64 [d][d][d/2+1] (fftshifted);
 * rotations [P][3][3] row-major; projective_filters [P][d][d/2+1].  Output
 * out [P][H-d+1][W-d+1] (mode 0, "valid") or [P][H][W] (mode 1, "same").
 * Particles are processed `group` at a time in a workspace of
 * lgb_xcorr_stack_workspace_size(group, ...) bytes. */
int lgb_xcorr_stack_supported(int H, int W, int d);
int lgb_xcorr_stack_workspace_size(int group, int H, int W, int d, int mode, size_t* bytes);
int lgb_xcorr_stack(int n_particles, int group, int H, int W, int d, int mode, const void* particle_dft,
                    const void* template_dft, const float* rotations, const float* projective_filters, float* out,
                    void* workspace, size_t workspace_bytes, void* stream);

/* ------------------------------------------------------------------------ */
/* Peak picking on the z-score map (analysis/zscore_metric.py:43-84,        */
/* analysis/utils.py:6-50).                                                  */
/* ------------------------------------------------------------------------ */

/* Scratch bytes lgb_peaks_find needs for an H x W map. */
size_t lgb_peaks_scratch_size(int H, int W, int max_rounds);

/* Candidates z > cutoff of the H x W map `zscore` (device, FP32, row-major);
 * a candidate is picked unless a picked candidate of higher rank (larger z;
 * equal z: smaller row-major index) lies at distance sqrtf(dy^2+dx^2) <
 * radius -- the reference's greedy walk in descending order.  Writes the flat
 * indices of the picked peaks (unordered, device int[max_peaks]) and their
 * number (host int, may exceed max_peaks: then only max_peaks were written),
 * and the rounds used (host int).  Synchronises `stream`.  Returns
 * LGB_ERR_DEVICE_TIMEOUT if the candidates did not settle in max_rounds. */
int lgb_peaks_find(int H, int W, const float* zscore, float cutoff, float radius, int max_rounds, void* scratch,
                   size_t scratch_bytes, int max_peaks, int* peak_index, int* n_peaks, int* rounds_used,
                   void* stream);

/* ------------------------------------------------------------------------ */
/* Split-precision tensor-core GEMM (tcgen05), the DFT building block of the  */
/* precision form; no reference counterpart (the reference's DFTs are        */
/* cuFFT calls inside torch.fft).                                            */
/* ------------------------------------------------------------------------ */

/* D[m][n] = sum_k A[m][k] B[n][k] with FP32 accumulation, where A = a_hi +
 * a_lo and B = b_hi + b_lo are 16-bit (BF16, or FP16 if f16) splits of FP32
 * matrices; terms = 3 accumulates hi*hi + lo*hi + hi*lo, terms = 1 hi*hi only.
 * A has m_tiles*128 rows, B n_tiles*bn rows (bn = 128 or 256), both
 * k_chunks*64 columns, in the blocked core-matrix layout: element (r, k) of a
 * matrix cut into TR-row tiles (TR = 128 for A, bn for B) is at
 *   (((r/TR)*k_chunks + k/64)*(TR/8) + (r%TR)/8)*512 + ((k%64)/8)*64 + (r%8)*8 + k%8.
 * D (device, FP32, row stride ldd) receives rows < m_valid, columns < n_valid.
 * Device pointers 16-byte aligned.  *err (device int) is set to
 * LGB_ERR_DEVICE_TIMEOUT if a bounded device wait ran out. */
/* Self-test of the bounded device waits: one thread polls an mbarrier phase
 * that never completes at most `polls` times (<= 2^22) and then writes
 * LGB_ERR_DEVICE_TIMEOUT to *device_status -- the same expiry path as the
 * waits inside lgb_tc_gemm and lgb_match_search_precision.  No GPU fault, no
 * trap; the context stays usable. */
int lgb_wait_timeout_selftest(unsigned polls, int* device_status, void* stream);

int lgb_tc_gemm(int m_tiles, int n_tiles, int k_chunks, int bn, int f16, int terms, const void* a_hi,
                const void* a_lo, const void* b_hi, const void* b_lo, float* d, int ldd, int m_valid, int n_valid,
                int* err, void* stream);

/* ------------------------------------------------------------------------ */
/* Pre-processing of the search inputs (once per micrograph).                */
/* ------------------------------------------------------------------------ */

/* CTF filter stack of one optics group, out float32 (device)
 * [n_pixel_sizes][n_defocus][d][d/2+1] on the unshifted rfft grid of a d x d
 * template: -sin(chi) exp(-B k^2 / 4) with defocus (defocus_u + defocus_v)/2 +
 * offset, astigmatism |defocus_u - defocus_v|/2 at astigmatism_angle_deg, and
 * Cs scaled for the pixel-size offsets, FP64 arithmetic.  Replaces
 * calculate_ctf_filter_stack (utils/ctf_utils.py:19-116, torch-ctf's
 * calculate_ctf_2d with torch-fourier-filter's b_envelope). */
int lgb_ctf_filter_stack(int template_size, double defocus_u, double defocus_v, double astigmatism_angle_deg,
                         const lgb_ctf_params* ctf, const float* defocus_offsets, int n_defocus,
                         const float* pixel_size_offsets, int n_pixel_sizes, float* out, void* stream);

/* Radially binned spectrum of n_images rfft images (complex64 device
 * [n][H][W/2+1]): bin of |k| = round(|k| / max_freq * (n_bins - 1)) clamped
 * to the last bin (|k| in cycles/pixel); bin_sum[n][n_bins] = sum of |F|^2
 * (power = 1) or |F| (power = 0), bin_count[n][n_bins] = samples (FP64,
 * device).  First half of the whitening filter of
 * correlation_filters.py:49-108 (torch-fourier-filter's whitening_filter). */
int lgb_radial_spectrum(int n_images, int image_h, int image_w, const void* image_dft, int n_bins, double max_freq,
                        int power, double* bin_sum, double* bin_count, void* stream);

/* Second half: per image the 1-D filter 1/spectrum (square root of the mean
 * power when power = 1), 0 where the spectrum is 0, normalised to maximum 1
 * (written over bin_sum), sampled by nearest bin onto the rfft grid of an
 * out_h x out_w real image: out float32 [n][out_h][out_w/2+1] (device). */
int lgb_whitening_filter(int n_images, int n_bins, double max_freq, int power, double* bin_sum,
                         const double* bin_count, int out_h, int out_w, float* out, void* stream);

/* Bandpass [low, high] cycles/pixel with raised-cosine edges of width falloff
 * (a hard band when 0) on the rfft grid of an h x w real image, out float32
 * [h][w/2+1] (device).  Replaces BandpassFilterConfig.calculate_bandpass_filter
 * (correlation_filters.py:234-271). */
int lgb_bandpass_filter(int h, int w, double low, double high, double falloff, float* out, void* stream);

/* out[n] = F[n] f[n] / sqrt(P[n]) * sqrt(D) * sqrt(area_ratio), where P[n] =
 * sum |F f|^2 with interior rfft columns counted twice, D the same weighted sum
 * of the bandpass filter and area_ratio = (image area) / (box area).  F, out
 * complex64 [n][H][W/2+1]; filters float32, image n at filters + n *
 * filter_stride (0: one filter for all); scratch >= n_images + 1 doubles
 * (device).  Replaces preprocess_image (utils/image_processing.py:16-75). */
int lgb_preprocess_image(int n_images, int image_h, int image_w, const void* image_dft, const float* filters,
                         long long filter_stride, const float* bandpass, double area_ratio, double* scratch,
                         void* out, void* stream);

/* ------------------------------------------------------------------------ */
/* Refinement proposal network (no reference counterpart: Leopard-EM has no  */
/* learned component; closest analogue core_differentiable_refine.py).       */
/* Activations and forward weights are BF16 (device), accumulation FP32,     */
/* gradients FP32.  NCHW; conv weights [Cout][Cin][3][3]; linear [Out][In]. */
/* ------------------------------------------------------------------------ */

/* 3x3 convolutions (pad 1, stride 1|2, 1 <= Cin, Cout <= 128) as implicit
 * GEMMs on the tcgen05 tensor cores: BF16 operands, FP32 accumulation.
 * workspace (device, 256-byte aligned) holds the gathered operands; its size
 * for one layer shape (forward or backward) comes from
 * lgb_nn_conv3x3_workspace_size.  device_status (device int, caller-zeroed)
 * receives LGB_ERR_DEVICE_TIMEOUT if a bounded device wait ran out. */
int lgb_nn_conv3x3_workspace_size(int N, int Cin, int H, int W, int Cout, int stride, size_t* bytes);
/* y = act(conv3x3(x, w) + b) in BF16; act = ReLU if relu; b optional. */
int lgb_nn_conv3x3_forward(int N, int Cin, int H, int W, int Cout, int stride, int relu, const void* x,
                           const void* w, const float* b, void* y, void* workspace, size_t workspace_bytes,
                           int* device_status, void* stream);
/* From g = dLoss/d(pre-activation output): dx (optional), dw, db (optional). */
int lgb_nn_conv3x3_backward(int N, int Cin, int H, int W, int Cout, int stride, const void* x, const void* w,
                            const float* g, float* dx, float* dw, float* db, void* workspace, size_t workspace_bytes,
                            int* device_status, void* stream);
/* Linear layers on the tcgen05 tensor cores (BF16 operands, FP32
 * accumulation), with the same workspace and device_status contract as the
 * convolutions; lgb_nn_linear_workspace_size covers forward and backward.
 * y[n][o] = act(sum_i x[n][i] w[o][i] + b[o]) into y_bf16 and/or y_f32. */
int lgb_nn_linear_workspace_size(int N, int In, int Out, size_t* bytes);
int lgb_nn_linear_forward(int N, int In, int Out, int relu, const void* x, const void* w, const float* b,
                          void* y_bf16, float* y_f32, void* workspace, size_t workspace_bytes, int* device_status,
                          void* stream);
/* From g = dLoss/dy (pre-activation): dx (optional), dw, db (optional). */
int lgb_nn_linear_backward(int N, int In, int Out, const void* x, const void* w, const float* g, float* dx,
                           float* dw, float* db, void* workspace, size_t workspace_bytes, int* device_status,
                           void* stream);
/* g = dy * (y > 0) for a ReLU output y (bf16). */
int lgb_nn_relu_backward(long long n, const void* y, const float* dy, float* g, void* stream);
/* loss = mean_n sum_d w_d (pred - target)^2 and its gradient (weights optional). */
int lgb_nn_mse(int N, int D, const float* pred, const float* target, const float* weights, float* dpred,
               float* loss, void* stream);
/* Adam with bias correction (step >= 1) and decoupled-as-L2 weight decay; also
 * refreshes the bf16 copy of the parameters when param_bf16 is not NULL. */
int lgb_nn_adam(long long n, float* param, const float* grad, float* m, float* v, void* param_bf16, float lr,
                float beta1, float beta2, float eps, float weight_decay, int step, void* stream);
int lgb_nn_to_bf16(long long n, const float* src, void* dst, void* stream);
/* Network input per particle p, on the band of `band` x (band/2+1) lowest
 * frequencies of particle_dft[p] (complex64 [H][W/2+1]); out bf16
 * [P][6][band][band], band = 64:
 *   0    the particle band (particle centred in its crop), moved onto the
 *        reference by the peak of their band cross-correlation, standardised;
 *   1    the template's central slice at rotations[p] (row-major 3x3) on the
 *        same physical frequencies times the particle's CTF (the reference);
 *   2-4  finite-difference derivatives of the reference for 1-degree rotations
 *        about the image x, y, z axes;
 *   5    derivative of the reference with respect to defocus (per 100 A);
 *   channels 1-5 mean-subtracted and scaled by the reference's std;
 *   out has out_channels >= 6 channels per particle (channels 0-5 written). */
int lgb_nn_make_inputs(int n_particles, int image_h, int image_w, const void* particle_dft,
                       const void* template_dft, int template_size, const float* rotations,
                       const float* defocus_u, const float* defocus_v, const float* defocus_angle,
                       const lgb_ctf_params* ctf, int band, int out_channels, void* out, void* stream);
/* Gauss-Newton step from input channels 0-5 (out [P][channels][band][band]):
 * gn[p][0..7] = (shift x, y in band pixels, rotation about x, y, z in degrees,
 * defocus in 100 A, amplitude <P,R>/<R,R>, residual fraction); with
 * channels >= 12 also writes channels 6-11 as constant maps of the step. */
int lgb_nn_gauss_newton(int n_particles, int band, int channels, void* inputs, float* gn, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* LEOPARD_GB300_H */
