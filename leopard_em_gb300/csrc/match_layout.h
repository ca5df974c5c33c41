// Workspace layout of the whole-orientation search (shared by the plain and
// the precision drivers).
#pragma once

#include <stddef.h>

#include "match_kernels.cuh"

namespace lgb {

struct MatchLayout {
  size_t ip, slices, t, proj, rowstats, a, y, cursor, total;
  int wc_img, wcp, wc_t, n_c_max;
};

inline size_t align256(size_t n) { return (n + 255) & ~(size_t)255; }

// Micrograph size inside the (possibly zero-padded) correlation grid.
inline int mic_h(const lgb_match_problem* p) { return p->micrograph_h > 0 ? p->micrograph_h : p->image_h; }
inline int mic_w(const lgb_match_problem* p) { return p->micrograph_w > 0 ? p->micrograph_w : p->image_w; }

inline bool valid_problem(const lgb_match_problem* p) {
  return p && p->image_h > 0 && p->image_w > 0 && (p->image_w % 2) == 0 && p->template_size > 1 &&
         (p->template_size % 2) == 0 && p->n_pixel_sizes > 0 && p->n_defocus > 0 && p->n_orientations > 0 &&
         p->orientation_batch > 0 && p->template_size <= p->image_h && p->template_size <= p->image_w &&
         p->micrograph_h >= 0 && p->micrograph_w >= 0 && p->col_waves >= 0 && mic_h(p) <= p->image_h &&
         mic_w(p) <= p->image_w && p->template_size <= mic_h(p) && p->template_size <= mic_w(p);
}

inline MatchLayout layout_of(const lgb_match_problem* p) {
  MatchLayout L{};
  const size_t H = p->image_h, W = p->image_w, h = p->template_size;
  const size_t y_rows = mic_h(p);
  L.wc_img = (int)(W / 2 + 1);
  L.wcp = pad4(L.wc_img);
  L.wc_t = (int)(h / 2 + 1);
  L.n_c_max = p->n_pixel_sizes * p->n_defocus * p->orientation_batch;
  const size_t nc = (size_t)L.n_c_max;
  size_t off = 0;
  L.ip = off;
  off += align256(H * L.wcp * sizeof(float2));
  L.slices = off;
  off += align256((size_t)p->orientation_batch * h * L.wc_t * sizeof(float2));
  L.t = off;
  off += align256(nc * h * L.wc_t * sizeof(float2));
  L.proj = off;
  off += align256(nc * h * h * sizeof(float));
  L.rowstats = off;
  off += align256(nc * h * 3 * sizeof(double));
  L.a = off;
  off += align256(nc * h * L.wcp * sizeof(float2));
  L.y = off;
  off += align256(nc * y_rows * L.wcp * sizeof(float2));
  L.cursor = off;  // orientation cursor of graph replays
  off += 256;
  L.total = off;
  return L;
}

}  // namespace lgb
