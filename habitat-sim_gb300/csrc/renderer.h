// Host runtime of the GB300 batch renderer: the C++ counterpart of
// esp::gfx_batch::Renderer / RendererStandalone (src/esp/gfx_batch/Renderer.h,
// RendererStandalone.h) with device-resident scene data.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <map>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/gbr.h"
#include "../../include/gbr_hbao.h"
#include "kernels.h"
#include "records.h"

namespace gbr {

// Device bytes a renderer's buffers may hold (0: no limit) and hold now.
struct DeviceBudget {
  uint64_t limit = 0;
  uint64_t held = 0;
};

// A growable device allocation, charged to a budget when it has one.
struct DeviceBuffer {
  void* ptr = nullptr;
  size_t bytes = 0;
  DeviceBudget* budget = nullptr;
  ~DeviceBuffer();
  bool reserve(size_t n, bool keep, cudaStream_t stream = nullptr);
  template <class T>
  T* as() const { return static_cast<T*>(ptr); }
};

struct PinnedBuffer {
  void* ptr = nullptr;
  size_t bytes = 0;
  ~PinnedBuffer();
  bool reserve(size_t n);
};

// Offsets into one of the device arrays (vertices, indices, texels, chunk
// boxes): first-fit reuse of released ranges, else growth at the end.
struct RangePool {
  uint64_t end = 0;                   // one past the highest range ever handed out
  uint64_t free_total = 0;
  std::map<uint64_t, uint64_t> free;  // offset -> size, coalesced
  uint64_t alloc(uint64_t n);
  void release(uint64_t offset, uint64_t n);
  uint64_t live() const { return end - free_total; }
};

struct MeshView {
  uint32_t mesh, index_offset, index_count, material;
  float transform[16];
  float bbox[6];
  uint32_t box_base;     // first chunk box of this view (its cluster boxes follow)
  uint32_t chunk_count;  // 32-triangle chunks of this view
  bool live;             // false once its template was removed
};

struct HostDraw {
  uint32_t batch, node, top, mesh, index_offset, index_count, material, semantic;
  float bbox[6];
  uint32_t box_base, chunk_count;
  uint32_t view;  // index into the renderer's mesh views
};

struct BatchKey {
  uint32_t flags, mesh, texture;
};

struct SceneState {
  std::vector<int32_t> parents;
  std::vector<float> transforms;  // 16 per node
  std::vector<HostDraw> draws;    // add order
  std::vector<BatchKey> batches;
  float pv[16];
  float view[16];
  float proj[16] = {};
  float unprojection[2] = {0, 0};
  int32_t width = 0, height = 0;
  int64_t fb_offset = 0, pitch = 0;
  bool transforms_dirty = true;
  uint32_t node_base = 0;  // in the flattened device arrays
  uint32_t draw_count = 0; // draws in the flattened device arrays (at the last rebuild)
  uint64_t tris = 0;       // triangles of those draws
  uint32_t source = 0;     // scene whose nodes and draws this scene renders
  uint32_t vis_base = 0;   // first visible record (from the current bindings)
  bool enabled = true;
  // lights (Renderer.cpp:990-1121): node, type, colour (3 floats), range
  std::vector<int32_t> light_nodes, light_types;
  std::vector<float> light_colors, light_ranges;
};

class Renderer {
 public:
  static Renderer* create(const gbr_config& cfg, std::string& err);
  ~Renderer();

  std::atomic<int> refs{1};
  void retain() { refs.fetch_add(1); }
  void release() {
    if (refs.fetch_sub(1) == 1) delete this;
  }

  // -- resources
  gbr_status add_file(const char* filename, uint32_t flags, const char* name);
  gbr_status add_mesh(const gbr_mesh_data& m, uint32_t* id);
  gbr_status add_texture(const gbr_texture_data& t, uint32_t* id);
  gbr_status add_material(const gbr_material_data& m, uint32_t* id);
  gbr_status add_template(const char* name, uint32_t count, const gbr_mesh_view* views);
  gbr_status remove_mesh(uint32_t mesh);
  gbr_status remove_texture(uint32_t texture);
  gbr_status remove_template(const char* name);
  gbr_status memory_usage(uint64_t* live, uint64_t* reserved) const;

  // -- scenes
  bool has_hierarchy(const char* name) const { return names_.count(name) != 0; }
  gbr_status add_node_hierarchy(uint32_t scene, const char* name, const float* bake, uint64_t* id);
  gbr_status add_empty_node(uint32_t scene, uint64_t* id);
  gbr_status clear(uint32_t scene);
  gbr_status set_semantic_id(uint32_t scene, uint64_t node, uint32_t id);
  gbr_status update_camera(uint32_t scene, const float* p, const float* v);
  gbr_status update_cameras(uint32_t first, uint32_t count, const float* p, const float* v);
  gbr_status camera(uint32_t scene, float* out) const;
  gbr_status unprojection(uint32_t scene, float* out) const;
  gbr_status transformations(uint32_t scene, float** out, uint64_t* count);
  gbr_status stats(uint32_t scene, gbr_scene_stats_info* out) const;
  gbr_status set_sources(uint32_t first, uint32_t count, const uint32_t* sources);
  gbr_status add_light(uint32_t scene, uint64_t node, uint32_t type, uint64_t* id);
  gbr_status clear_lights(uint32_t scene);
  gbr_status light_colors(uint32_t scene, float** out, uint64_t* count);
  gbr_status light_ranges(uint32_t scene, float** out, uint64_t* count);
  gbr_status set_enabled(uint32_t scene, bool enabled);

  // -- drawing
  gbr_status draw(cudaStream_t stream, uint32_t mode, bool use_graph);
  // Ambient occlusion on the colour plane of every enabled scene of the last draw.
  gbr_status hbao(const gbr_hbao_config& c, cudaStream_t stream);
  gbr_status image_into(uint32_t plane, const int32_t* rect, void* dst, uint64_t row_bytes);
  gbr_status image_into_async(uint32_t plane, const int32_t* rect, void* dst, uint64_t row_bytes);
  gbr_status readback_wait();
  // Scenes [first, first + count) of a plane packed one after another into
  // dst (host or device), asynchronously on the copy stream.
  gbr_status scenes_into_async(uint32_t plane, uint32_t first, uint32_t count, void* dst);
  gbr_status scene_image_into(uint32_t plane, uint32_t scene, void* dst, uint64_t row_bytes);
  gbr_status plane_pointer(uint32_t plane, void** out, uint64_t* bytes);
  gbr_status plane_dlpack(uint32_t plane, void** out);
  gbr_status get_tuning(gbr_tuning* t) const;
  gbr_status set_tuning(const gbr_tuning& t);
  gbr_status last_stats(gbr_draw_stats* out);
  gbr_status set_kernel_timing(bool on);
  gbr_status set_memory_limit(uint64_t bytes);
  gbr_status device_memory(uint64_t* held, uint64_t* limit) const;
  gbr_status debug_corrupt_parent(uint32_t scene, uint64_t node, int32_t parent);

  uint32_t scene_count() const { return uint32_t(scenes_.size()); }
  const gbr_config& config() const { return cfg_; }
  bool ragged() const { return ragged_; }
  int64_t fb_width() const { return fb_w_; }
  int64_t fb_height() const { return fb_h_; }
  const SceneState& scene(uint32_t s) const { return scenes_[s]; }

 private:
  Renderer() = default;
  gbr_status fail(gbr_status s, const std::string& msg);
  gbr_status cuda_fail(cudaError_t e, const char* what);
  gbr_status check_scene(uint32_t scene, const char* fn) const;
  gbr_status upload_tables();
  gbr_status rebuild(cudaStream_t stream);
  gbr_status upload_step(cudaStream_t stream);
  gbr_status enqueue_step(cudaStream_t stream, uint32_t mode);
  gbr_status ensure_raster_config();
  void build_chunk_boxes(uint32_t first_view, uint32_t last_view);
  void* plane_ptr(uint32_t plane, size_t* elem) const;
  gbr_status sync_and_check();
  gbr_status quiesce();
  size_t camera_block_bytes() const;  // cameras then light sources, per step
  bool texture_removed(uint32_t t) const { return t < texture_live_.size() && !texture_live_[t]; }
  void order_items();

  gbr_config cfg_{};
  std::vector<int32_t> viewports_;
  bool ragged_ = false;
  int64_t fb_w_ = 0, fb_h_ = 0, fb_px_ = 0;
  int device_ = 0;
  int sm_count_ = 0;

  // resources (host mirrors)
  std::vector<MeshRec> meshes_;
  std::vector<bool> mesh_live_;
  std::vector<float> host_pos_;                    // xyz per vertex, for view bounding boxes
  std::vector<uint32_t> host_indices_;
  std::vector<TextureRec> textures_;
  std::vector<bool> texture_live_;
  std::vector<MaterialRec> materials_;
  std::vector<MeshView> views_;
  std::vector<ChunkBox> boxes_;
  // Boxes written since the last upload: [boxes_lo_, boxes_hi_) of boxes_.
  size_t boxes_lo_ = SIZE_MAX, boxes_hi_ = 0;
  std::unordered_map<std::string, std::pair<uint32_t, uint32_t>> names_;
  RangePool vertex_pool_, index_pool_, texel_pool_, box_pool_;
  bool tables_dirty_ = true;

  std::vector<SceneState> scenes_;
  bool structure_dirty_ = true;

  // device (every buffer below is charged to budget_, declared first so that
  // it outlives them)
  DeviceBudget budget_;
  void attach_budget();
  DeviceBuffer d_pos_, d_color_, d_uv_, d_indices_, d_texels_, d_normal_;
  DeviceBuffer d_lights_, d_model_;  // lit renderers: world lights, per-draw model data
  DeviceBuffer d_spill_;  // raster queue spill area, per CTA
  DeviceBuffer d_gather_;  // packed scenes on their way to host memory
  DeviceBuffer d_hbao_scenes_, d_hbao_ao_;  // ambient occlusion: per-scene records, two 8-bit planes
  uint32_t max_lights_ = 0;
  DeviceBuffer d_meshes_, d_materials_, d_textures_, d_boxes_;
  DeviceBuffer d_scenes_, d_parents_, d_local_, d_draws_, d_cameras_;
  DeviceBuffer d_visible_, d_order_, d_vis_count_, d_vis_tris_, d_vis_clusters_, d_status_, d_items_,
      d_items_lpt_, d_counter_;
  DeviceBuffer d_planes_[2][4];  // output planes; two sets when double-buffered
  bool double_buffer_ = false;
  int front_ = 0;                // set written by the last draw
  int draw_set_ = 0;             // set the draw being enqueued writes
  gbr_status wait_uploads();     // both slots idle
  cudaStream_t copy_stream_ = nullptr;
  cudaEvent_t copy_done_[2] = {nullptr, nullptr};
  bool copy_pending_[2] = {false, false};
  // Host staging of the per-step uploads, two slots used by alternate draws so
  // that the host stages draw k + 1 while draw k runs; upload_done_[slot]
  // follows the whole step that last used the slot.
  PinnedBuffer h_stage_[2];
  PinnedBuffer h_mesh_stage_;  // addMesh uploads
  cudaEvent_t upload_done_[2] = {nullptr, nullptr};
  bool upload_pending_[2] = {false, false};
  int slot_ = 1;  // slot of the last draw (the next draw takes the other)
  cudaStream_t last_stream_ = nullptr;
  cudaStream_t own_stream_ = nullptr;

  uint32_t total_nodes_ = 0, total_draws_ = 0;
  uint64_t total_tris_ = 0;
  std::vector<uint32_t> scene_item_base_, scene_item_count_;
  uint32_t item_count_ = 0;
  uint32_t lpt_count_ = 0;  // batched form: capacity of the item list (every scene at its finest split)
  uint32_t lpt_items_ = 0;  // batched form: items in the current list
  bool bindings_dirty_ = true;           // sources or enabled flags changed
  bool items_staged_ = false;            // a new item order waits in the staging buffer
  uint64_t vis_needed_ = 0;              // visible records the current bindings need

  gbr_tuning tuning_{1024, 128, 128, 1, 1, 16, 32, 1, 75};
  size_t smem_bytes_ = 0, smem_plain_ = 0;
  int prefix_cap_ = 0;
  bool raster_configured_ = false;
  int ctas_per_sm_ = 1;

  // CUDA graphs of the batched step, one per plane set
  cudaGraphExec_t graph_exec_[2] = {nullptr, nullptr};
  cudaStream_t graph_stream_[2] = {nullptr, nullptr};
  bool graph_built_[2] = {false, false};
  bool graph_valid_ = false;  // false: every graph must be re-captured

  gbr_draw_stats last_stats_{};
  bool timing_ = false;
  bool timed_ = false;
  cudaEvent_t ev_[3] = {nullptr, nullptr, nullptr};
  uint64_t launches_ = 0;
};

void set_last_error(const std::string& msg);
const char* last_error_cstr();

}  // namespace gbr
