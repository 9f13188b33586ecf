// Launch interface of the batch renderer's sm_103a kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "records.h"

namespace gbr {

struct Planes {
  uint32_t* color;
  float* depth;
  float* linear;
  uint32_t* semantic;
};

// Prepare: per scene, absolute node transforms, per-draw MVP and view-z row,
// frustum culling of each draw's bounding box, compaction of the visible
// draws with the running triangle ordinal, and the order in which the
// raster kernel walks them (nearest first, so that near geometry hides the
// chunks behind it early).  One CTA per scene.
struct PrepareParams {
  const SceneRec* scenes;
  const CameraRec* cameras;
  const DrawRec* draws;
  const int32_t* parents;
  const float* local;
  const MeshRec* meshes;
  VisibleRec* visible;
  uint2* order;        // per visible draw: (draw, first cluster) in processing order
  uint32_t* vis_count;
  uint32_t* vis_tris;
  uint32_t* vis_clusters;
  uint32_t* status;
  uint32_t scene_base;
  const LightSrc* light_src;  // [scene][max_lights] (lit renderers)
  WorldLight* lights;         // [scene][max_lights] (lit renderers)
  ModelRec* model;            // per visible draw (lit renderers, else null)
  uint32_t max_lights;
};

// Raster: per work item (scene, region), warps take 32-triangle chunks,
// cull them by bounding box, set up + clip + rasterise their triangles into a
// shared-memory (depth, ordinal) z-buffer; then deferred shading and plane
// writes.
struct RasterParams {
  const SceneRec* scenes;
  const CameraRec* cameras;   // binding of each scene (vis_base, enabled)
  const VisibleRec* visible;
  const uint2* order;         // processing order of the visible draws (see PrepareParams)
  const uint32_t* vis_count;
  const uint32_t* vis_tris;
  const uint32_t* vis_clusters;
  void* spill;                // per CTA (blockIdx) `threads` queue entries of spill space, or null
  const ChunkBox* boxes;      // chunk and cluster boxes (null: no box culling)
  const float4* pos;
  const float4* color;
  const float2* uv;
  const uint32_t* indices;
  const MaterialRec* materials;
  const TextureRec* textures;
  const uint32_t* texels;
  int32_t texture_count;
  uint32_t flags;  // 1 = no textures
  const WorkItem* items;
  uint32_t item_base;
  uint32_t item_count;
  // Persistent form: the items in use this launch (at most item_count), read
  // from device memory so that a captured graph follows a list that changes
  // from step to step; null: item_count.
  const uint32_t* item_count_dev;
  uint32_t* counter;  // persistent mode: next item
  int32_t persistent;
  Planes out;
  int32_t region_px;   // capacity of the shared z-buffer, pixels
  int32_t prefix_cap;  // visible draws whose ordinals are cached in shared memory
  int32_t small_area;  // boxes up to this many pixels are rasterised by one lane
  int32_t occlusion;   // skip chunks hidden behind the depths written so far
  uint32_t flush_at;   // the queue is rasterised once it holds this many triangles (1..threads)
  // Lighting (max_lights > 0): lights per scene, per-draw model data, normals.
  const WorldLight* lights;
  const ModelRec* model;
  const float4* normals;
  uint32_t max_lights;
  float ambient_factor;
  int any_lod;  // some texture has mip levels or a minification filter of its own
};

cudaError_t launch_prepare(const PrepareParams& p, uint32_t scene_count, cudaStream_t stream);
size_t raster_smem_bytes(int threads, int region_px, int prefix_cap);
// Bytes of the queue spill area for `grid` CTAs of `threads` threads.
size_t raster_spill_bytes(int threads, uint32_t grid);
// Raises the kernel's dynamic shared-memory limit to the device maximum and
// returns that maximum and the kernel's static shared memory.
cudaError_t raster_configure(int threads, size_t* max_dynamic, size_t* static_bytes);
cudaError_t launch_raster(const RasterParams& p, int threads, uint32_t grid, size_t smem,
                          cudaStream_t stream);
cudaError_t raster_max_ctas_per_sm(int threads, size_t smem, int* out);
cudaError_t launch_unproject(float a, float b, float* depth, uint64_t rows, uint64_t cols,
                             uint64_t row_stride, cudaStream_t stream);
// Packs scenes [first, first + count) of a tile-grid plane of 4-byte
// elements (row pitch `pitch` elements, tiles w x h, tiles_x per row) into
// dst, one scene after another.
cudaError_t launch_gather_tiles(const void* src, int64_t pitch, int w, int h, int tiles_x, uint32_t first,
                                uint32_t count, void* dst, cudaStream_t stream);

}  // namespace gbr
