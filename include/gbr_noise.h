/* gbr_noise.h -- C ABI of the depth-sensor noise model on the GPU.
 *
 * A drop-in for habitat-sim's esp::sensor::RedwoodNoiseModelGPUImpl
 * (src/esp/sensor/RedwoodNoiseModel.h:37-95, RedwoodNoiseModel.cpp:37-95,
 * RedwoodNoiseModel.cu:20-200): the Redwood / CLAMS PrimeSense depth model —
 * pixel jitter, 2x downsampling, per-pixel distortion from an 80 x 80 x 5
 * table, disparity quantisation with high-frequency noise, nothing beyond
 * 10 m.  Conventions as gbr.h (status codes, gbr_last_error()).
 *
 * Random numbers: the reference draws curand XORWOW normals from per-thread
 * states seeded by rand(); here each pixel's three normals come from one
 * Philox4x32-10 block (Salmon et al., SC'11) of the counter (pixel, image,
 * call) under a 64-bit seed, mapped through a 4097-knot table of the
 * normal quantile function.  Results are reproducible for a given seed and
 * call counter, independent of launch shapes.
 */
#ifndef GBR_NOISE_H
#define GBR_NOISE_H

#include "gbr.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gbr_redwood_noise gbr_redwood_noise;

/* Knots of the normal quantile table: knot k = Phi^-1((k + 0.5) / 4097). */
#define GBR_NORMAL_TABLE_SIZE 4097u

/* RedwoodNoiseModelGPUImpl::RedwoodNoiseModelGPUImpl (RedwoodNoiseModel.cpp:37-63):
 * model is the distortion table as rows x cols floats, 80 x 400 (80 x 80 x 5
 * flattened), as habitat-sim's redwood-depth-dist-model.npy. */
gbr_status gbr_redwood_noise_create(const float* model, int32_t model_rows, int32_t model_cols,
                                    int32_t gpu_device_id, float noise_multiplier, uint64_t seed,
                                    gbr_redwood_noise** out);
void gbr_redwood_noise_destroy(gbr_redwood_noise* m);

/* simulateFromGPU (RedwoodNoiseModel.cpp:85-93): depth and noisy are device
 * arrays of rows x cols floats (metres, row-major); asynchronous on stream. */
gbr_status gbr_redwood_noise_simulate_device(gbr_redwood_noise* m, const float* depth, int32_t rows,
                                             int32_t cols, float* noisy, void* stream);
/* simulateFromCPU (RedwoodNoiseModel.cpp:73-83): host arrays; returns when done. */
gbr_status gbr_redwood_noise_simulate_host(gbr_redwood_noise* m, const float* depth, int32_t rows,
                                           int32_t cols, float* noisy);
/* Batched form (no reference counterpart): `count` images of tile_w x tile_h
 * pixels laid out as the tiles of a plane with `pitch` floats per row, image
 * i at ((i % tiles_x) * tile_w, (i / tiles_x) * tile_h) -- the renderer's
 * linear-depth plane -- noised in one launch from src into dst (device). */
gbr_status gbr_redwood_noise_simulate_tiles(gbr_redwood_noise* m, const float* src, float* dst,
                                            int64_t pitch, int32_t tile_w, int32_t tile_h,
                                            int32_t tiles_x, int32_t count, void* stream);
/* Batched form for any plane layout (no reference counterpart): `count`
 * images, image i at src + layout[4i] with row pitch layout[4i+1] floats,
 * layout[4i+2] x layout[4i+3] pixels (the renderer's ragged framebuffer:
 * gbr_scene_viewport of every scene), noised in one launch into the same
 * places of dst (device).  layout is a host array; image i draws the same
 * noise as image i of gbr_redwood_noise_simulate_tiles. */
gbr_status gbr_redwood_noise_simulate_images(gbr_redwood_noise* m, const float* src, float* dst,
                                             const int64_t* layout, int32_t count, void* stream);
/* Seed and call counter: every simulate call uses the counter's value and
 * then increments it. */
gbr_status gbr_redwood_noise_set_state(gbr_redwood_noise* m, uint64_t seed, uint64_t counter);
gbr_status gbr_redwood_noise_get_state(gbr_redwood_noise* m, uint64_t* seed, uint64_t* counter);

/* The normal quantile knots the kernel interpolates (host only, no GPU). */
gbr_status gbr_normal_quantile_table(float* out, uint32_t n);

#ifdef __cplusplus
}
#endif

#endif /* GBR_NOISE_H */
