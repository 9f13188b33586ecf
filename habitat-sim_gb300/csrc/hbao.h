// Horizon-based ambient occlusion kernels and their host-side parameters
// (shared by the renderer's gbr_hbao_draw and the standalone gbr_hbao_apply).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/gbr_hbao.h"

namespace gbr {

// One image: its rectangle in the planes, projection info and radius.
struct HbaoScene {
  long long offset;  // element index of pixel (0, 0) (bottom-left)
  long long pitch;   // elements per row
  int w, h;
  float pi[4];       // view position = ((u, v) * pi.xy + pi.zw) * z (z = 1 if orthographic)
  float radius_to_screen;
  float far_plane;   // depth given to background pixels (linear depth 0)
  int ortho;
  int block0;        // first block of the scene in the launch grid (256 pixels per block)
  int qw, qh;        // quarter resolution of the cache-aware algorithm: ceil(w / 4) x ceil(h / 4)
  float inv_qw, inv_qh;  // 1 / qw, 1 / qh
};

struct HbaoParams {
  float neg_inv_r2, bias, ao_mult, pow_exp, sharpness;
  int no_blur;
  int special;       // AO and view depth kept as two halves per pixel, blurred with that depth
  int cache_aware;   // the deinterleaved algorithm
  float jitter[64];  // 4 x 4 texels of (cos, sin, start offset, 0), 16-bit snorm (classic)
  float jitter_f[64];  // the same, unquantized (cache-aware: one per deinterleaved layer)
  float dirs[16];    // 8 unit directions (cos, sin)
};

void hbao_jitter_unquantized(float out[64]);
// Validates the configuration and fills the per-call constants.
bool hbao_params(const gbr_hbao_config& c, HbaoParams& p, std::string& err);
// Per-image constants from a column-major projection (Hbao.cpp:761-786, 874-895).
HbaoScene hbao_scene(const float* projection, int w, int h, long long offset, long long pitch,
                     float radius);
// Bytes per pixel of each of the two intermediate planes: an 8-bit AO, or
// with the special blur an (AO, view depth) pair of halves.
inline int hbao_plane_bytes(const HbaoParams& p) { return p.special ? 4 : 1; }
// Three launches on `stream`: AO (into q1, or straight into colour without
// blur), blur along x (q1 -> q2), blur along y and the colour multiply.
// q1 / q2 have the colour plane's layout, hbao_plane_bytes(p) per pixel.
cudaError_t hbao_launch(const HbaoScene* d_scenes, int count, int blocks, const float* depth,
                        uint32_t* color, void* q1, void* q2, const HbaoParams& p,
                        cudaStream_t stream);

}  // namespace gbr
