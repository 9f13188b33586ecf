/* gbr_replay.h -- C ABI of the batch replay renderer driven by gfx-replay
 * keyframes.
 *
 * A drop-in for habitat-sim's esp::sim::BatchReplayRenderer
 * (src/esp/sim/BatchReplayRenderer.cpp:22-213, AbstractReplayRenderer.h:
 * 67-186), its per-environment esp::gfx::replay::Player
 * (src/esp/gfx/replay/Player.cpp:103-370) and the BatchPlayerImplementation
 * that turns keyframes into batch-renderer calls
 * (src/esp/sim/BatchPlayerImplementation.cpp:51-170).  Each entry point
 * names the member it replaces.  The driver owns one gbr_renderer (the
 * batch renderer of include/gbr.h) with one scene per environment.
 *
 * Conventions are those of gbr.h: every call returns gbr_status with
 * gbr_last_error() set on failure; matrices are column-major 4x4 floats;
 * images have row 0 at the bottom.  Quaternions are {x, y, z, w}.
 */
#ifndef GBR_REPLAY_H
#define GBR_REPLAY_H

#include "gbr.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gbr_replay gbr_replay;

/* ReplayRendererConfiguration (AbstractReplayRenderer.h:24-63) with its one
 * CameraSensorSpec (sensor/CameraSensor.h:14-30, VisualSensor.h:36-63). */
typedef struct gbr_replay_config {
  uint32_t num_environments;   /* default 1                                   */
  int32_t gpu_device_id;       /* default 0                                   */
  int32_t standalone;          /* must be 1: no GL framebuffer to draw into   */
  int32_t enable_frustum_culling; /* accepted; culling is always exact        */
  int32_t enable_hbao;         /* 1: ambient occlusion on the colour images
                                  (gbr_hbao.h, default configuration)          */
  const char* sensor_uuid;     /* sensor name, default "rgba_camera"          */
  int32_t resolution[2];       /* {height, width}, default {128, 128}         */
  float hfov_degrees;          /* default 90                                  */
  float near_plane, far_plane; /* default 0.01, 1000                          */
  int32_t orthographic;        /* 0 pinhole (default), 1 orthographic         */
  float ortho_scale;           /* default 0.1                                 */
  /* Batch renderer options (gfx_batch::RendererConfiguration, which the
   * reference leaves at its defaults here). */
  uint32_t max_light_count;    /* default 0 (flat shading)                    */
  float ambient_factor;        /* default 0.1                                 */
  uint32_t draw_mode;          /* GBR_DRAW_*, default GBR_DRAW_BATCHED        */
  uint32_t quiet;              /* 1: no warnings on stderr                    */
} gbr_replay_config;

void gbr_replay_config_init(gbr_replay_config* config);

/* BatchReplayRenderer::BatchReplayRenderer (BatchReplayRenderer.cpp:22-54):
 * tile size = sensor resolution, tile grid = environment_grid_size. */
gbr_status gbr_replay_create(const gbr_replay_config* config, gbr_replay** out);
void gbr_replay_destroy(gbr_replay* r);
/* AbstractReplayRenderer::close (BatchReplayRenderer.cpp:60-71); safe to
 * call more than once.  Every later call except destroy fails. */
gbr_status gbr_replay_close(gbr_replay* r);
/* The batch renderer the driver draws with (valid until close/destroy), for
 * DLPack views, plane pointers and statistics. */
gbr_status gbr_replay_renderer(gbr_replay* r, gbr_renderer** out);

/* AbstractReplayRenderer::environmentGridSize (AbstractReplayRenderer.cpp:
 * 26-31): {ceil(sqrt(n)), ceil(n / x)}. */
gbr_status gbr_replay_environment_grid_size(int32_t environment_count, int32_t out[2]);
/* preloadFile (BatchReplayRenderer.cpp:73-75): a composite glTF whose
 * hierarchies keyframe creations then name. */
gbr_status gbr_replay_preload_file(gbr_replay* r, const char* filename);
/* environmentCount / sensorSize ({width, height}) (:77-86). */
gbr_status gbr_replay_environment_count(gbr_replay* r, uint32_t* out);
gbr_status gbr_replay_sensor_size(gbr_replay* r, uint32_t env, int32_t out[2]);
/* clearEnvironment (AbstractReplayRenderer.cpp:55-59): drops the
 * environment's keyframes and instances. */
gbr_status gbr_replay_clear_environment(gbr_replay* r, uint32_t env);

/* setEnvironmentKeyframe (AbstractReplayRenderer.cpp:61-66): json is a
 * serialized {"keyframe": {...}} as Recorder::keyframeToString writes it;
 * the environment's player holds that one keyframe and applies it. */
gbr_status gbr_replay_set_environment_keyframe(gbr_replay* r, uint32_t env, const char* json,
                                               uint64_t length);
/* setEnvironmentKeyframeUnwrapped (:68-73): the keyframe object itself. */
gbr_status gbr_replay_set_environment_keyframe_unwrapped(gbr_replay* r, uint32_t env,
                                                         const char* json, uint64_t length);
/* setEnvironmentKeyframe for environments first_env .. first_env + count - 1
 * in one call (json[i], length[i] go to environment first_env + i), followed,
 * when sensor_prefix is not NULL, by setSensorTransformsFromKeyframe(env,
 * sensor_prefix) for each (AbstractReplayRenderer.cpp:61-66, 83-92).  All documents
 * are parsed before any is applied: a malformed one returns
 * GBR_ERROR_INVALID_ARGUMENT naming its environment and changes nothing.
 * Errors while applying (a missing asset, a missing sensor transform) stop
 * at that environment with the per-environment call's status; earlier
 * environments keep their new keyframes.  Large batches are parsed on
 * several host threads.  Same results as the per-environment calls in
 * environment order. */
gbr_status gbr_replay_set_environment_keyframes(gbr_replay* r, uint32_t first_env, uint32_t count,
                                                const char* const* json, const uint64_t* length,
                                                const char* sensor_prefix);
/* Player::readKeyframesFromJsonDocument + setKeyframeIndex(-1)
 * (Player.cpp:103-106, 142-152): a {"keyframes": [...]} document for the
 * environment's player; nothing is applied until gbr_replay_set_keyframe_index. */
gbr_status gbr_replay_set_keyframes(gbr_replay* r, uint32_t env, const char* json,
                                    uint64_t length);
/* Player::setKeyframeIndex (Player.cpp:142-152): -1 clears the environment;
 * going back clears and re-applies from the first keyframe. */
gbr_status gbr_replay_set_keyframe_index(gbr_replay* r, uint32_t env, int32_t index);
/* Player::getNumKeyframes / getKeyframeIndex (Player.cpp:134-140). */
gbr_status gbr_replay_keyframe_count(gbr_replay* r, uint32_t env, int32_t* count, int32_t* index);
/* Player::getUserTransform (Player.cpp:154-170) of the current keyframe;
 * *found = 0 when the keyframe has no such name. */
gbr_status gbr_replay_user_transform(gbr_replay* r, uint32_t env, const char* name,
                                     float translation[3], float rotation[4], int32_t* found);

/* setSensorTransform (BatchReplayRenderer.cpp:92-99): camera view =
 * transform^-1 with the sensor's projection.  sensor_name is not checked
 * (one sensor per environment, as the reference). */
gbr_status gbr_replay_set_sensor_transform(gbr_replay* r, uint32_t env, const char* sensor_name,
                                           const float transform[16]);
/* setSensorTransformsFromKeyframe (BatchReplayRenderer.cpp:101-115): uses
 * the user transform named prefix + sensor uuid of the environment's
 * keyframe; GBR_ERROR_NOT_FOUND if absent, GBR_ERROR_STATE if the
 * environment holds no single keyframe (AbstractReplayRenderer.cpp:83-92). */
gbr_status gbr_replay_set_sensor_transforms_from_keyframe(gbr_replay* r, uint32_t env,
                                                          const char* prefix);

/* render(colorImageViews, depthImageViews) (BatchReplayRenderer.cpp:117-151,
 * AbstractReplayRenderer.cpp:94-110): draws every environment on `stream`
 * and copies environment i's RGBA8 image to color[i] and its depth in
 * metres (0 where nothing is drawn; the reference's depthImageInto +
 * unprojectDepth) to depth[i].  Either count may be 0 (skip that output);
 * otherwise it must equal the environment count.  Destinations may be host
 * or device memory; the call returns when the copies are complete. */
gbr_status gbr_replay_render(gbr_replay* r, void* stream, uint32_t color_count,
                             void* const* color, uint64_t color_row_bytes, uint32_t depth_count,
                             void* const* depth, uint64_t depth_row_bytes);

/* unproject (AbstractReplayRenderer.cpp:134-139): the ray through the
 * viewport pixel (x from the left, y from the top) of the environment's
 * camera, origin at the camera, direction normalised (the classic renderer's
 * RenderCamera::unproject, gfx/RenderCamera.cpp:186-216). */
gbr_status gbr_replay_unproject(gbr_replay* r, uint32_t env, int32_t x, int32_t y,
                                float origin[3], float direction[3]);

#ifdef __cplusplus
}
#endif

#endif /* GBR_REPLAY_H */
