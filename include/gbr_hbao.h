/* gbr_hbao.h -- C ABI of horizon-based ambient occlusion on the GPU.
 *
 * A drop-in for habitat-sim's esp::gfx_batch::Hbao (src/esp/gfx_batch/
 * Hbao.h:30-190, Hbao.cpp:595-1038, shaders src/shaders/gfx_batch/hbao/):
 * per pixel, the view position from linear depth, a normal from the nearest
 * neighbours, 8 jittered directions x 4 steps of occlusion within a
 * world-space radius, stored as 8-bit AO, a depth-aware 7-tap blur along x
 * then y, and the colour multiplied by the result.  HbaoType::CacheAware
 * computes the same on 16 deinterleaved quarter-resolution layers of the
 * depth (normals through an RGBA8 store, per-layer jitter); the special blur
 * (HbaoFlag::UseAoSpecialBlur) keeps AO and view depth as two halves and
 * blurs with that depth.  The GL version draws on the classic renderer's
 * render target; here it runs as three kernels over every scene of a batch
 * renderer (or on one caller image).  Conventions as gbr.h.
 */
#ifndef GBR_HBAO_H
#define GBR_HBAO_H

#include "gbr.h"

#ifdef __cplusplus
extern "C" {
#endif

/* HbaoType (Hbao.h:135). */
#define GBR_HBAO_CLASSIC 0
#define GBR_HBAO_CACHE_AWARE 1

/* HbaoConfiguration (Hbao.h:30-141) and the algorithm of drawEffect. */
typedef struct gbr_hbao_config {
  float intensity;      /* power exponent, default 0.732                    */
  float bias;           /* N.V bias, default 0.05                           */
  float radius;         /* metres, default 1.84                             */
  float blur_sharpness; /* default 10                                       */
  int32_t no_blur;      /* HbaoFlag::NoBlur: raw AO multiplied in           */
  int32_t special_blur; /* HbaoFlag::UseAoSpecialBlur (not with no_blur)    */
  int32_t algorithm;    /* GBR_HBAO_CLASSIC (default) or GBR_HBAO_CACHE_AWARE */
} gbr_hbao_config;

void gbr_hbao_config_init(gbr_hbao_config* config);

/* Hbao::drawEffect(projection, algorithm, depth, output)
 * (Hbao.cpp:874-1038) on every enabled scene of the renderer's last draw:
 * each scene's colour plane is darkened in place using its linear depth and
 * the projection of its last updateCamera.  Needs the colour and
 * linear-depth planes; asynchronous on stream (ordered after the draw). */
gbr_status gbr_hbao_draw(gbr_renderer* r, const gbr_hbao_config* config, void* stream);

/* The same on one caller image: RGBA8 colour and linear depth in metres
 * (0 = background, read as the far plane), both device arrays of
 * width x height with `pitch` elements per row; returns when done. */
gbr_status gbr_hbao_apply(const gbr_hbao_config* config, const float projection[16],
                          const float* linear_depth, uint32_t* color, int32_t width,
                          int32_t height, int64_t pitch, void* stream);

/* The 4 x 4 jitter table (cos, sin, start offset, 0 per texel; Hbao.cpp:
 * 603-617 with std::mt19937's default seed), host only. */
gbr_status gbr_hbao_jitter_table(float out[64]);

#ifdef __cplusplus
}
#endif

#endif /* GBR_HBAO_H */
