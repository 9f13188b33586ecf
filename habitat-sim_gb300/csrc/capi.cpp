// extern "C" boundary of the GB300 batch renderer (declared in include/gbr.h).
#include <cuda_runtime.h>

#include <cstring>
#include <new>
#include <string>

#include "../../include/gbr.h"
#include "kernels.h"
#include "renderer.h"

namespace gbr {
const char* last_error_cstr();
}

using gbr::Renderer;

namespace {

Renderer* R(gbr_renderer* r) { return reinterpret_cast<Renderer*>(r); }

gbr_status null_handle() {
  gbr::set_last_error("null renderer handle");
  return GBR_ERROR_INVALID_ARGUMENT;
}

gbr_status null_arg(const char* what) {
  gbr::set_last_error(std::string("null argument: ") + what);
  return GBR_ERROR_INVALID_ARGUMENT;
}

template <class F>
gbr_status guarded(F&& f) {
  try {
    gbr::set_last_error("");
    return f();
  } catch (const std::bad_alloc&) {
    gbr::set_last_error("host allocation failed");
    return GBR_ERROR_OUT_OF_MEMORY;
  } catch (const std::exception& e) {
    gbr::set_last_error(e.what());
    return GBR_ERROR_STATE;
  }
}

}  // namespace

#define GBR_HANDLE(r) \
  if (!(r)) return null_handle()
#define GBR_ARG(p) \
  if (!(p)) return null_arg(#p)

extern "C" {

void gbr_config_init(gbr_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->tile_size[0] = c->tile_size[1] = 128;
  c->tile_count[0] = c->tile_count[1] = 1;
  c->ambient_factor = 0.1f;
  c->planes = GBR_PLANE_ALL;
  c->draw_mode = GBR_DRAW_PER_SCENE;
}

gbr_status gbr_create(const gbr_config* config, gbr_renderer** out) {
  GBR_ARG(config);
  GBR_ARG(out);
  return guarded([&] {
    std::string err;
    Renderer* r = Renderer::create(*config, err);
    if (!r) {
      gbr::set_last_error(err);
      *out = nullptr;
      return err.find("memory") != std::string::npos ? GBR_ERROR_OUT_OF_MEMORY
             : err.find("cuda") != std::string::npos ? GBR_ERROR_CUDA
                                                      : GBR_ERROR_INVALID_ARGUMENT;
    }
    *out = reinterpret_cast<gbr_renderer*>(r);
    return GBR_OK;
  });
}

void gbr_destroy(gbr_renderer* r) {
  if (r) R(r)->release();
}

const char* gbr_last_error(void) { return gbr::last_error_cstr(); }

gbr_status gbr_tile_size_count(gbr_renderer* r, int32_t ts[2], int32_t tc[2]) {
  GBR_HANDLE(r);
  const gbr_config& c = R(r)->config();
  if (ts) {
    ts[0] = c.tile_size[0];
    ts[1] = c.tile_size[1];
  }
  if (tc) {
    tc[0] = c.tile_count[0];
    tc[1] = c.tile_count[1];
  }
  return GBR_OK;
}

gbr_status gbr_scene_count(gbr_renderer* r, uint32_t* count) {
  GBR_HANDLE(r);
  GBR_ARG(count);
  *count = R(r)->scene_count();
  return GBR_OK;
}

gbr_status gbr_framebuffer_size(gbr_renderer* r, int64_t size[2]) {
  GBR_HANDLE(r);
  GBR_ARG(size);
  size[0] = R(r)->fb_width();
  size[1] = R(r)->fb_height();
  return GBR_OK;
}

gbr_status gbr_scene_viewport(gbr_renderer* r, uint32_t scene, int64_t out[4]) {
  GBR_HANDLE(r);
  GBR_ARG(out);
  if (scene >= R(r)->scene_count()) {
    gbr::set_last_error("sceneViewport: scene out of range");
    return GBR_ERROR_INVALID_ARGUMENT;
  }
  const gbr::SceneState& s = R(r)->scene(scene);
  out[0] = s.fb_offset;
  out[1] = s.pitch;
  out[2] = s.width;
  out[3] = s.height;
  return GBR_OK;
}

gbr_status gbr_add_file(gbr_renderer* r, const char* filename, uint32_t flags, const char* name) {
  GBR_HANDLE(r);
  GBR_ARG(filename);
  return guarded([&] { return R(r)->add_file(filename, flags, name); });
}

gbr_status gbr_add_mesh(gbr_renderer* r, const gbr_mesh_data* mesh, uint32_t* out) {
  GBR_HANDLE(r);
  GBR_ARG(mesh);
  GBR_ARG(out);
  return guarded([&] { return R(r)->add_mesh(*mesh, out); });
}

gbr_status gbr_add_texture(gbr_renderer* r, const gbr_texture_data* t, uint32_t* out) {
  GBR_HANDLE(r);
  GBR_ARG(t);
  GBR_ARG(out);
  return guarded([&] { return R(r)->add_texture(*t, out); });
}

gbr_status gbr_add_material(gbr_renderer* r, const gbr_material_data* m, uint32_t* out) {
  GBR_HANDLE(r);
  GBR_ARG(m);
  GBR_ARG(out);
  return guarded([&] { return R(r)->add_material(*m, out); });
}

gbr_status gbr_add_node_hierarchy_template(gbr_renderer* r, const char* name, uint32_t count,
                                           const gbr_mesh_view* views) {
  GBR_HANDLE(r);
  GBR_ARG(name);
  if (count) GBR_ARG(views);
  return guarded([&] { return R(r)->add_template(name, count, views); });
}

gbr_status gbr_add_light(gbr_renderer* r, uint32_t scene, uint64_t node, uint32_t type,
                         uint64_t* out) {
  GBR_HANDLE(r);
  GBR_ARG(out);
  return guarded([&] { return R(r)->add_light(scene, node, type, out); });
}

gbr_status gbr_clear_lights(gbr_renderer* r, uint32_t scene) {
  GBR_HANDLE(r);
  return guarded([&] { return R(r)->clear_lights(scene); });
}

gbr_status gbr_light_colors(gbr_renderer* r, uint32_t scene, float** out, uint64_t* count) {
  GBR_HANDLE(r);
  GBR_ARG(out);
  GBR_ARG(count);
  return guarded([&] { return R(r)->light_colors(scene, out, count); });
}

gbr_status gbr_light_ranges(gbr_renderer* r, uint32_t scene, float** out, uint64_t* count) {
  GBR_HANDLE(r);
  GBR_ARG(out);
  GBR_ARG(count);
  return guarded([&] { return R(r)->light_ranges(scene, out, count); });
}

gbr_status gbr_set_scene_sources(gbr_renderer* r, uint32_t first, uint32_t count,
                                 const uint32_t* sources) {
  GBR_HANDLE(r);
  return guarded([&] { return R(r)->set_sources(first, count, sources); });
}

gbr_status gbr_set_scene_enabled(gbr_renderer* r, uint32_t scene, int32_t enabled) {
  GBR_HANDLE(r);
  return guarded([&] { return R(r)->set_enabled(scene, enabled != 0); });
}

gbr_status gbr_remove_mesh(gbr_renderer* r, uint32_t mesh) {
  GBR_HANDLE(r);
  return guarded([&] { return R(r)->remove_mesh(mesh); });
}

gbr_status gbr_remove_texture(gbr_renderer* r, uint32_t texture) {
  GBR_HANDLE(r);
  return guarded([&] { return R(r)->remove_texture(texture); });
}

gbr_status gbr_remove_node_hierarchy_template(gbr_renderer* r, const char* name) {
  GBR_HANDLE(r);
  GBR_ARG(name);
  return guarded([&] { return R(r)->remove_template(name); });
}

gbr_status gbr_memory_usage(gbr_renderer* r, uint64_t* live_bytes, uint64_t* reserved_bytes) {
  GBR_HANDLE(r);
  return guarded([&] { return R(r)->memory_usage(live_bytes, reserved_bytes); });
}

gbr_status gbr_has_node_hierarchy(gbr_renderer* r, const char* name, int32_t* out) {
  GBR_HANDLE(r);
  GBR_ARG(name);
  GBR_ARG(out);
  *out = R(r)->has_hierarchy(name) ? 1 : 0;
  return GBR_OK;
}

gbr_status gbr_add_node_hierarchy(gbr_renderer* r, uint32_t scene, const char* name,
                                  const float bake[16], uint64_t* out) {
  GBR_HANDLE(r);
  GBR_ARG(name);
  GBR_ARG(out);
  return guarded([&] { return R(r)->add_node_hierarchy(scene, name, bake, out); });
}

gbr_status gbr_add_empty_node(gbr_renderer* r, uint32_t scene, uint64_t* out) {
  GBR_HANDLE(r);
  GBR_ARG(out);
  return guarded([&] { return R(r)->add_empty_node(scene, out); });
}

gbr_status gbr_clear(gbr_renderer* r, uint32_t scene) {
  GBR_HANDLE(r);
  return guarded([&] { return R(r)->clear(scene); });
}

gbr_status gbr_set_semantic_id(gbr_renderer* r, uint32_t scene, uint64_t node, uint32_t id) {
  GBR_HANDLE(r);
  return guarded([&] { return R(r)->set_semantic_id(scene, node, id); });
}

gbr_status gbr_update_camera(gbr_renderer* r, uint32_t scene, const float p[16], const float v[16]) {
  GBR_HANDLE(r);
  GBR_ARG(p);
  GBR_ARG(v);
  return R(r)->update_camera(scene, p, v);
}

gbr_status gbr_update_cameras(gbr_renderer* r, uint32_t first, uint32_t count, const float* p,
                              const float* v) {
  GBR_HANDLE(r);
  if (count) {
    GBR_ARG(p);
    GBR_ARG(v);
  }
  return R(r)->update_cameras(first, count, p, v);
}

gbr_status gbr_camera(gbr_renderer* r, uint32_t scene, float out[16]) {
  GBR_HANDLE(r);
  GBR_ARG(out);
  return R(r)->camera(scene, out);
}

gbr_status gbr_camera_depth_unprojection(gbr_renderer* r, uint32_t scene, float out[2]) {
  GBR_HANDLE(r);
  GBR_ARG(out);
  return R(r)->unprojection(scene, out);
}

gbr_status gbr_transformations(gbr_renderer* r, uint32_t scene, float** out, uint64_t* count) {
  GBR_HANDLE(r);
  GBR_ARG(out);
  GBR_ARG(count);
  return R(r)->transformations(scene, out, count);
}

gbr_status gbr_draw(gbr_renderer* r, void* stream) {
  GBR_HANDLE(r);
  return guarded([&] {
    return R(r)->draw(static_cast<cudaStream_t>(stream), R(r)->config().draw_mode, false);
  });
}

gbr_status gbr_draw_mode(gbr_renderer* r, void* stream, uint32_t mode, int32_t use_graph) {
  GBR_HANDLE(r);
  if (mode != GBR_DRAW_PER_SCENE && mode != GBR_DRAW_BATCHED) {
    gbr::set_last_error("drawMode: unknown mode");
    return GBR_ERROR_INVALID_ARGUMENT;
  }
  return guarded(
      [&] { return R(r)->draw(static_cast<cudaStream_t>(stream), mode, use_graph != 0); });
}

gbr_status gbr_scene_stats(gbr_renderer* r, uint32_t scene, gbr_scene_stats_info* out) {
  GBR_HANDLE(r);
  GBR_ARG(out);
  return R(r)->stats(scene, out);
}

gbr_status gbr_image_into(gbr_renderer* r, uint32_t plane, const int32_t rect[4], void* dst,
                          uint64_t row_bytes) {
  GBR_HANDLE(r);
  GBR_ARG(rect);
  GBR_ARG(dst);
  return guarded([&] { return R(r)->image_into(plane, rect, dst, row_bytes); });
}

gbr_status gbr_image_into_async(gbr_renderer* r, uint32_t plane, const int32_t rect[4], void* dst,
                                uint64_t row_bytes) {
  GBR_HANDLE(r);
  GBR_ARG(rect);
  GBR_ARG(dst);
  return guarded([&] { return R(r)->image_into_async(plane, rect, dst, row_bytes); });
}

gbr_status gbr_readback_wait(gbr_renderer* r) {
  GBR_HANDLE(r);
  return guarded([&] { return R(r)->readback_wait(); });
}

gbr_status gbr_color_image_into(gbr_renderer* r, const int32_t rect[4], void* dst,
                                uint64_t row_bytes) {
  return gbr_image_into(r, GBR_PLANE_COLOR, rect, dst, row_bytes);
}

gbr_status gbr_depth_image_into(gbr_renderer* r, const int32_t rect[4], void* dst,
                                uint64_t row_bytes) {
  return gbr_image_into(r, GBR_PLANE_DEPTH, rect, dst, row_bytes);
}

gbr_status gbr_semantic_image_into(gbr_renderer* r, const int32_t rect[4], void* dst,
                                   uint64_t row_bytes) {
  return gbr_image_into(r, GBR_PLANE_SEMANTIC, rect, dst, row_bytes);
}

gbr_status gbr_linear_depth_image_into(gbr_renderer* r, const int32_t rect[4], void* dst,
                                       uint64_t row_bytes) {
  return gbr_image_into(r, GBR_PLANE_LINEAR_DEPTH, rect, dst, row_bytes);
}

gbr_status gbr_scene_image_into(gbr_renderer* r, uint32_t plane, uint32_t scene, void* dst,
                                uint64_t row_bytes) {
  GBR_HANDLE(r);
  GBR_ARG(dst);
  return guarded([&] { return R(r)->scene_image_into(plane, scene, dst, row_bytes); });
}

gbr_status gbr_plane_device_pointer(gbr_renderer* r, uint32_t plane, void** out, uint64_t* bytes) {
  GBR_HANDLE(r);
  GBR_ARG(out);
  return R(r)->plane_pointer(plane, out, bytes);
}

gbr_status gbr_plane_dlpack(gbr_renderer* r, uint32_t plane, void** out) {
  GBR_HANDLE(r);
  GBR_ARG(out);
  return guarded([&] { return R(r)->plane_dlpack(plane, out); });
}

gbr_status gbr_unproject_depth(const float u[2], float* depth, uint64_t rows, uint64_t cols,
                               uint64_t stride) {
  GBR_ARG(u);
  if (rows && cols) GBR_ARG(depth);
  if (stride < cols) {
    gbr::set_last_error("unprojectDepth: row stride smaller than the row");
    return GBR_ERROR_INVALID_ARGUMENT;
  }
  // unprojectDepth (DepthUnprojection.cpp:107-129).
  const float a = u[0], b = u[1];
  for (uint64_t y = 0; y < rows; ++y)
    for (uint64_t x = 0; x < cols; ++x) {
      float& d = depth[y * stride + x];
      d = b / (d + a);
    }
  const float far_depth = b / (1.0f + a);
  for (uint64_t y = 0; y < rows; ++y)
    for (uint64_t x = 0; x < cols; ++x) {
      float& d = depth[y * stride + x];
      if (d == far_depth) d = 0.0f;
    }
  return GBR_OK;
}

gbr_status gbr_unproject_depth_device(const float u[2], float* depth, uint64_t rows, uint64_t cols,
                                      uint64_t stride, void* stream) {
  GBR_ARG(u);
  if (stride < cols) {
    gbr::set_last_error("unprojectDepthDevice: row stride smaller than the row");
    return GBR_ERROR_INVALID_ARGUMENT;
  }
  cudaError_t e =
      gbr::launch_unproject(u[0], u[1], depth, rows, cols, stride, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) {
    gbr::set_last_error(std::string("unprojectDepthDevice: ") + cudaGetErrorString(e));
    return GBR_ERROR_CUDA;
  }
  return GBR_OK;
}

gbr_status gbr_get_tuning(gbr_renderer* r, gbr_tuning* out) {
  GBR_HANDLE(r);
  GBR_ARG(out);
  return R(r)->get_tuning(out);
}

gbr_status gbr_set_tuning(gbr_renderer* r, const gbr_tuning* t) {
  GBR_HANDLE(r);
  GBR_ARG(t);
  return R(r)->set_tuning(*t);
}

gbr_status gbr_last_draw_stats(gbr_renderer* r, gbr_draw_stats* out) {
  GBR_HANDLE(r);
  GBR_ARG(out);
  return guarded([&] { return R(r)->last_stats(out); });
}

gbr_status gbr_set_kernel_timing(gbr_renderer* r, int32_t enabled) {
  GBR_HANDLE(r);
  return R(r)->set_kernel_timing(enabled != 0);
}

gbr_status gbr_set_device_memory_limit(gbr_renderer* r, uint64_t bytes) {
  GBR_HANDLE(r);
  return R(r)->set_memory_limit(bytes);
}

gbr_status gbr_device_memory(gbr_renderer* r, uint64_t* held, uint64_t* limit) {
  GBR_HANDLE(r);
  return R(r)->device_memory(held, limit);
}

gbr_status gbr_debug_corrupt_parent(gbr_renderer* r, uint32_t scene, uint64_t node, int32_t parent) {
  GBR_HANDLE(r);
  return guarded([&] { return R(r)->debug_corrupt_parent(scene, node, parent); });
}

gbr_status gbr_scenes_into_async(gbr_renderer* r, uint32_t plane, uint32_t first, uint32_t count,
                                 void* dst) {
  GBR_HANDLE(r);
  GBR_ARG(dst);
  return guarded([&] { return R(r)->scenes_into_async(plane, first, count, dst); });
}

gbr_status gbr_hbao_draw(gbr_renderer* r, const gbr_hbao_config* config, void* stream) {
  GBR_HANDLE(r);
  GBR_ARG(config);
  return guarded([&] { return R(r)->hbao(*config, static_cast<cudaStream_t>(stream)); });
}

}  // extern "C"
