// Host runtime of the GB300 batch renderer.
//
// Scene bookkeeping follows esp::gfx_batch::Renderer
// (src/esp/gfx_batch/Renderer.cpp): reserved white texture and material
// (:287-304), file import offsets (:410-415), addNodeHierarchy's root node
// plus one child per mesh view with bake * view transform and draw-batch ids
// keyed by (vertex-colour flag, mesh, texture) (:880-961, :136-152), the
// stable counting sort of draws by batch (:1139-1196), camera P*V and depth
// unprojection (:1077-1088).  What the reference does on the CPU every frame
// -- the transform hierarchy and per-draw uniform gathering (:1203-1290) --
// and everything it asks of GL runs on the device (kernels.cu).
#include "renderer.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <numeric>

#include "hbao.h"
#include "importer.h"
#include "mips.h"
#include "pool.h"
#include "trace.h"
#include "work_items.h"

namespace gbr {

namespace {
thread_local std::string g_last_error;

constexpr size_t kCameraBytes = sizeof(CameraRec);
constexpr int kPrefixCapMax = 4096;

const float kIdentity[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};

size_t plane_elem(uint32_t plane) { return 4; }

int plane_slot(uint32_t plane) {
  switch (plane) {
    case GBR_PLANE_COLOR: return 0;
    case GBR_PLANE_DEPTH: return 1;
    case GBR_PLANE_LINEAR_DEPTH: return 2;
    case GBR_PLANE_SEMANTIC: return 3;
    default: return -1;
  }
}
}  // namespace

void set_last_error(const std::string& msg) { g_last_error = msg; }
const char* last_error_cstr() { return g_last_error.c_str(); }

// ------------------------------------------------------------- buffers
DeviceBuffer::~DeviceBuffer() {
  if (ptr) cudaFree(ptr);
  if (budget) budget->held -= bytes;
}

bool DeviceBuffer::reserve(size_t n, bool keep, cudaStream_t stream) {
  if (n <= bytes) return true;
  size_t cap = std::max(n, bytes + bytes / 2);
  cap = (cap + 255) & ~size_t(255);
  if (budget && budget->limit) {
    // Within the limit: the usual growth, else exactly what is asked, else fail.
    if (budget->held - bytes + cap > budget->limit) cap = (n + 255) & ~size_t(255);
    if (budget->held - bytes + cap > budget->limit) return false;
  }
  void* p = nullptr;
  if (cudaMalloc(&p, cap) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (keep && ptr && bytes) {
    if (cudaMemcpy(p, ptr, bytes, cudaMemcpyDeviceToDevice) != cudaSuccess) {
      cudaFree(p);
      return false;
    }
  }
  if (ptr) cudaFree(ptr);
  if (budget) budget->held = budget->held - bytes + cap;
  ptr = p;
  bytes = cap;
  return true;
}

uint64_t RangePool::alloc(uint64_t n) {
  if (n == 0) return 0;
  for (auto it = free.begin(); it != free.end(); ++it) {
    if (it->second < n) continue;
    const uint64_t off = it->first, rest = it->second - n;
    free.erase(it);
    if (rest) free.emplace(off + n, rest);
    free_total -= n;
    return off;
  }
  const uint64_t off = end;
  end += n;
  return off;
}

void RangePool::release(uint64_t offset, uint64_t n) {
  if (n == 0) return;
  auto it = free.emplace(offset, n).first;
  free_total += n;
  auto next = std::next(it);
  if (next != free.end() && it->first + it->second == next->first) {
    it->second += next->second;
    free.erase(next);
  }
  if (it != free.begin()) {
    auto prev = std::prev(it);
    if (prev->first + prev->second == it->first) {
      prev->second += it->second;
      free.erase(it);
      it = prev;
    }
  }
  if (it->first + it->second == end) {  // the tail is free: shrink
    end = it->first;
    free_total -= it->second;
    free.erase(it);
  }
}

PinnedBuffer::~PinnedBuffer() {
  if (ptr) cudaFreeHost(ptr);
}

bool PinnedBuffer::reserve(size_t n) {
  if (n <= bytes) return true;
  size_t cap = std::max(n, bytes * 2);
  void* p = nullptr;
  if (cudaMallocHost(&p, cap) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (ptr) cudaFreeHost(ptr);
  ptr = p;
  bytes = cap;
  return true;
}

// -------------------------------------------------------------- errors
gbr_status Renderer::fail(gbr_status s, const std::string& msg) {
  set_last_error(msg);
  return s;
}

gbr_status Renderer::cuda_fail(cudaError_t e, const char* what) {
  set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
  cudaGetLastError();
  return e == cudaErrorMemoryAllocation ? GBR_ERROR_OUT_OF_MEMORY : GBR_ERROR_CUDA;
}

gbr_status Renderer::check_scene(uint32_t scene, const char* fn) const {
  if (scene >= scenes_.size()) {
    set_last_error(std::string(fn) + ": index " + std::to_string(scene) + " out of range for " +
                   std::to_string(scenes_.size()) + " scenes");
    return GBR_ERROR_INVALID_ARGUMENT;
  }
  return GBR_OK;
}

#define GBR_CUDA(call, what)                         \
  do {                                               \
    cudaError_t e_ = (call);                         \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

// -------------------------------------------------------------- create
Renderer* Renderer::create(const gbr_config& cfg, std::string& err) {
  if (cfg.max_light_count > 64) {
    err = "max_light_count above 64 is not supported";
    return nullptr;
  }
  if (cfg.scene_count == 0 &&
      (cfg.tile_size[0] <= 0 || cfg.tile_size[1] <= 0 || cfg.tile_count[0] <= 0 ||
       cfg.tile_count[1] <= 0)) {
    err = "tile size and count must be positive";
    return nullptr;
  }
  if (cfg.scene_count > 0 && !cfg.viewports) {
    err = "scene_count > 0 needs viewports";
    return nullptr;
  }
  std::unique_ptr<Renderer> r(new Renderer());
  r->attach_budget();
  r->cfg_ = cfg;
  r->max_lights_ = cfg.max_light_count;
  if (r->cfg_.planes == 0) r->cfg_.planes = GBR_PLANE_ALL;
  r->device_ = cfg.cuda_device;
  cudaError_t e = cudaSetDevice(r->device_);
  if (e != cudaSuccess) {
    err = std::string("cudaSetDevice: ") + cudaGetErrorString(e);
    cudaGetLastError();
    return nullptr;
  }
  cudaDeviceGetAttribute(&r->sm_count_, cudaDevAttrMultiProcessorCount, r->device_);
  uint32_t n;
  if (cfg.scene_count > 0) {
    r->ragged_ = true;
    n = cfg.scene_count;
    r->viewports_.assign(cfg.viewports, cfg.viewports + 2 * n);
    r->cfg_.viewports = nullptr;
    r->scenes_.resize(n);
    int64_t off = 0;
    for (uint32_t s = 0; s < n; ++s) {
      const int32_t w = r->viewports_[2 * s], h = r->viewports_[2 * s + 1];
      if (w <= 0 || h <= 0 || w > 16384 || h > 16384) {
        err = "viewport sizes must be in [1, 16384]";
        return nullptr;
      }
      SceneState& sc = r->scenes_[s];
      sc.width = w;
      sc.height = h;
      sc.fb_offset = off;
      sc.pitch = w;
      off += int64_t(w) * h;
    }
    r->fb_w_ = off;
    r->fb_h_ = 1;
    r->fb_px_ = off;
  } else {
    const int tw = cfg.tile_size[0], th = cfg.tile_size[1];
    if (tw > 16384 || th > 16384) {
      err = "tile sizes must be at most 16384";
      return nullptr;
    }
    n = uint32_t(cfg.tile_count[0]) * uint32_t(cfg.tile_count[1]);
    r->scenes_.resize(n);
    r->fb_w_ = int64_t(tw) * cfg.tile_count[0];
    r->fb_h_ = int64_t(th) * cfg.tile_count[1];
    r->fb_px_ = r->fb_w_ * r->fb_h_;
    for (uint32_t s = 0; s < n; ++s) {
      SceneState& sc = r->scenes_[s];
      const int x = int(s % uint32_t(cfg.tile_count[0])), y = int(s / uint32_t(cfg.tile_count[0]));
      sc.width = tw;
      sc.height = th;
      sc.pitch = r->fb_w_;
      sc.fb_offset = int64_t(y) * th * r->fb_w_ + int64_t(x) * tw;
    }
  }
  for (uint32_t s = 0; s < n; ++s) {
    SceneState& sc = r->scenes_[s];
    std::memcpy(sc.pv, kIdentity, 64);
    std::memcpy(sc.view, kIdentity, 64);
    sc.source = s;
  }
  r->double_buffer_ = (cfg.standalone_flags & GBR_STANDALONE_DOUBLE_BUFFER) != 0;
  for (int set = 0; set < (r->double_buffer_ ? 2 : 1); ++set)
    for (int i = 0; i < 4; ++i)
      if (r->cfg_.planes & (1u << i))
        if (!r->d_planes_[set][i].reserve(size_t(r->fb_px_) * 4, false)) {
          err = "out of device memory for the framebuffer";
          return nullptr;
        }
  for (auto& e : r->upload_done_)
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
      err = "cudaEventCreate failed";
      return nullptr;
    }
  // A blocking stream (ordered with the legacy default stream) for graph
  // capture when the caller passes the default stream, which cannot be captured.
  if (cudaStreamCreate(&r->own_stream_) != cudaSuccess) {
    err = "cudaStreamCreate failed";
    return nullptr;
  }
  // Texture 0: one white texel; material 0: white, untextured
  // (Renderer.cpp:287-304).
  const uint8_t white[4] = {255, 255, 255, 255};
  gbr_texture_data wt{1, 1, 1, white, 0, 0, 0};
  uint32_t id;
  if (r->add_texture(wt, &id) != GBR_OK) {
    err = g_last_error;
    return nullptr;
  }
  gbr_material_data wm{{1, 1, 1, 1}, 0, 0, {1, 0, 0, 0, 1, 0, 0, 0, 1}};
  r->add_material(wm, &id);
  return r.release();
}

void Renderer::attach_budget() {
  DeviceBuffer* all[] = {&d_pos_, &d_color_, &d_uv_, &d_indices_, &d_texels_, &d_normal_, &d_lights_,
                         &d_model_, &d_spill_, &d_gather_, &d_hbao_scenes_, &d_hbao_ao_, &d_meshes_,
                         &d_materials_, &d_textures_, &d_boxes_, &d_scenes_, &d_parents_, &d_local_,
                         &d_draws_, &d_cameras_, &d_visible_, &d_order_, &d_vis_count_, &d_vis_tris_,
                         &d_vis_clusters_, &d_status_, &d_items_, &d_items_lpt_, &d_counter_};
  for (DeviceBuffer* b : all) b->budget = &budget_;
  for (auto& set : d_planes_)
    for (DeviceBuffer& b : set) b.budget = &budget_;
}

gbr_status Renderer::set_memory_limit(uint64_t bytes) {
  budget_.limit = bytes;
  return GBR_OK;
}

gbr_status Renderer::device_memory(uint64_t* held, uint64_t* limit) const {
  if (held) *held = budget_.held;
  if (limit) *limit = budget_.limit;
  return GBR_OK;
}

// Fault injection: the parent of `node` replaced in device memory only,
// after the host validated and uploaded the scene (the host copy stays
// right, and is uploaded again once the device reports the bad record).
gbr_status Renderer::debug_corrupt_parent(uint32_t scene, uint64_t node, int32_t parent) {
  if (gbr_status st = check_scene(scene, "debugCorruptParent")) return st;
  if (node >= scenes_[scene].parents.size())
    return fail(GBR_ERROR_INVALID_ARGUMENT, "debugCorruptParent: node out of range");
  if (structure_dirty_)
    if (gbr_status st = rebuild(last_stream_)) return st;
  cudaSetDevice(device_);
  GBR_CUDA(cudaStreamSynchronize(last_stream_), "debugCorruptParent: synchronise");
  const size_t at = size_t(scenes_[scene].node_base) + size_t(node);
  GBR_CUDA(cudaMemcpy(d_parents_.as<int32_t>() + at, &parent, 4, cudaMemcpyHostToDevice),
           "debugCorruptParent: write");
  return GBR_OK;
}

Renderer::~Renderer() {
  cudaSetDevice(device_);
  if (last_stream_ || upload_pending_[0] || upload_pending_[1]) cudaDeviceSynchronize();
  if (copy_stream_) cudaStreamSynchronize(copy_stream_);
  for (auto& g : graph_exec_)
    if (g) cudaGraphExecDestroy(g);
  for (auto& e : copy_done_)
    if (e) cudaEventDestroy(e);
  if (copy_stream_) cudaStreamDestroy(copy_stream_);
  for (auto& e : upload_done_)
    if (e) cudaEventDestroy(e);
  if (own_stream_) cudaStreamDestroy(own_stream_);
  for (auto& e : ev_)
    if (e) cudaEventDestroy(e);
}

// ----------------------------------------------------------- resources
gbr_status Renderer::add_mesh(const gbr_mesh_data& m, uint32_t* id) {
  TraceRange trace_("gbr.add_mesh");
  if (!m.positions || (m.index_count && !m.indices))
    return fail(GBR_ERROR_INVALID_ARGUMENT, "addMesh: positions and indices are required");
  // Every index below the vertex count (large meshes checked on the host pool;
  // the first bad index is then looked up for the message).
  std::atomic<bool> bad_index{false};
  const std::function<void(uint32_t, uint32_t)> check = [&](uint32_t a, uint32_t b) {
    uint32_t hi = 0;
    for (uint32_t i = a; i < b; ++i) hi = std::max(hi, m.indices[i]);
    if (b > a && hi >= m.vertex_count) bad_index.store(true);
  };
  if (m.index_count >= (1u << 18))
    shared_pool().run(m.index_count, 1u << 16, check);
  else
    check(0, m.index_count);
  if (bad_index.load())
    for (uint32_t i = 0; i < m.index_count; ++i)
      if (m.indices[i] >= m.vertex_count)
        return fail(GBR_ERROR_INVALID_ARGUMENT, "addMesh: index " + std::to_string(i) +
                                                    " out of range for " +
                                                    std::to_string(m.vertex_count) + " vertices");
  cudaSetDevice(device_);
  const size_t nv = m.vertex_count;
  const uint64_t vb = vertex_pool_.alloc(nv), ib = index_pool_.alloc(m.index_count);
  auto undo = [&]() {
    vertex_pool_.release(vb, nv);
    index_pool_.release(ib, m.index_count);
  };
  if (vb + nv > 0xffffffffull || ib + m.index_count > 0xffffffffull) {
    undo();
    return fail(GBR_ERROR_INVALID_ARGUMENT, "addMesh: more than 2^32 vertices or indices");
  }
  const size_t ve = vertex_pool_.end, ie = index_pool_.end;
  if (!d_pos_.reserve(ve * 16, true) || !d_color_.reserve(ve * 16, true) ||
      !d_uv_.reserve(ve * 8, true) || !d_indices_.reserve(std::max<size_t>(ie, 1) * 4, true)) {
    undo();
    return fail(GBR_ERROR_OUT_OF_MEMORY, "addMesh: out of device memory");
  }
  const bool normals = max_lights_ > 0 && m.normals;
  if (normals && !d_normal_.reserve(ve * 16, true)) {
    undo();
    return fail(GBR_ERROR_OUT_OF_MEMORY, "addMesh: out of device memory");
  }
  // Device layouts (position + object id, colour, texture coordinate,
  // normal) written straight into pinned staging and copied at full link
  // speed, in pieces of at most kStageBytes so that a large mesh does not
  // keep a large pinned buffer.  The copies go on the legacy stream, as
  // cudaMemcpy's would (ordered after earlier work on blocking streams); the
  // staging is free again once a piece is drained.
  constexpr size_t kStageBytes = size_t(32) << 20;
  const size_t vbytes = normals ? 56 : 40;
  const size_t piece_v = kStageBytes / vbytes;
  const size_t need = std::min(nv, piece_v) * vbytes;
  if (!h_mesh_stage_.reserve(std::max<size_t>(need, 16))) {
    undo();
    return fail(GBR_ERROR_OUT_OF_MEMORY, "addMesh: out of pinned host memory");
  }
  char* stage = static_cast<char*>(h_mesh_stage_.ptr);
  for (size_t p0 = 0; p0 < nv; p0 += piece_v) {
    const size_t n = std::min(piece_v, nv - p0);
    float* pos = reinterpret_cast<float*>(stage);
    float* col = reinterpret_cast<float*>(stage + n * 16);
    float* uv = reinterpret_cast<float*>(stage + n * 32);
    float* nrm = reinterpret_cast<float*>(stage + n * 40);
    const std::function<void(uint32_t, uint32_t)> fill = [&](uint32_t a, uint32_t b) {
      for (size_t i = a; i < b; ++i) {
        const size_t v = p0 + i;
        pos[i * 4 + 0] = m.positions[v * 3 + 0];
        pos[i * 4 + 1] = m.positions[v * 3 + 1];
        pos[i * 4 + 2] = m.positions[v * 3 + 2];
        const uint32_t oid = m.object_ids ? m.object_ids[v] : 0u;
        std::memcpy(&pos[i * 4 + 3], &oid, 4);
        for (int c = 0; c < 4; ++c) col[i * 4 + c] = m.colors ? m.colors[v * 4 + c] : 1.0f;
        uv[i * 2] = m.texcoords ? m.texcoords[v * 2] : 0.0f;
        uv[i * 2 + 1] = m.texcoords ? m.texcoords[v * 2 + 1] : 0.0f;
        if (normals) {
          for (int c = 0; c < 3; ++c) nrm[i * 4 + c] = m.normals[v * 3 + c];
          nrm[i * 4 + 3] = 0.0f;
        }
      }
    };
    if (n >= (1u << 16))
      shared_pool().run(uint32_t(n), 8192, fill);
    else
      fill(0, uint32_t(n));
    const size_t v = vb + p0;
    GBR_CUDA(cudaMemcpyAsync(d_pos_.as<char>() + v * 16, pos, n * 16, cudaMemcpyHostToDevice, 0),
             "addMesh upload");
    GBR_CUDA(cudaMemcpyAsync(d_color_.as<char>() + v * 16, col, n * 16, cudaMemcpyHostToDevice, 0),
             "addMesh upload");
    GBR_CUDA(cudaMemcpyAsync(d_uv_.as<char>() + v * 8, uv, n * 8, cudaMemcpyHostToDevice, 0),
             "addMesh upload");
    if (normals)
      GBR_CUDA(cudaMemcpyAsync(d_normal_.as<char>() + v * 16, nrm, n * 16, cudaMemcpyHostToDevice, 0),
               "addMesh upload");
    GBR_CUDA(cudaStreamSynchronize(0), "addMesh upload");
  }
  // The indices need no repacking: one copy from the caller's memory.
  if (m.index_count)
    GBR_CUDA(cudaMemcpy(d_indices_.as<char>() + size_t(ib) * 4, m.indices, size_t(m.index_count) * 4,
                        cudaMemcpyHostToDevice),
             "addMesh upload");
  MeshRec rec{};
  rec.vertex_base = uint32_t(vb);
  rec.vertex_count = m.vertex_count;
  rec.index_base = uint32_t(ib);
  rec.index_count = m.index_count;
  rec.flags = (m.colors ? kMeshVertexColor : 0u) | (m.object_ids ? kMeshObjectId : 0u) |
              (m.texcoords ? kMeshTexcoords : 0u) | (normals ? kMeshNormals : 0u);
  meshes_.push_back(rec);
  mesh_live_.push_back(true);
  if (host_pos_.size() < ve * 3) host_pos_.resize(ve * 3);
  if (host_indices_.size() < ie) host_indices_.resize(ie);
  // Host mirrors (positions and indices, for the views' bounding boxes).
  float* hp = host_pos_.data() + vb * 3;
  uint32_t* hi = host_indices_.data() + ib;
  const uint64_t pos_words = uint64_t(nv) * 3, words = pos_words + m.index_count;
  const std::function<void(uint32_t, uint32_t)> mirror = [&](uint32_t a, uint32_t b) {
    const uint64_t w0 = uint64_t(a) << 12, w1 = std::min<uint64_t>(words, uint64_t(b) << 12);
    if (w0 < pos_words)
      std::memcpy(hp + w0, m.positions + w0, (std::min(w1, pos_words) - w0) * 4);
    if (w1 > pos_words) {
      const uint64_t i0 = std::max(w0, pos_words) - pos_words, i1 = w1 - pos_words;
      std::memcpy(hi + i0, m.indices + i0, (i1 - i0) * 4);
    }
  };
  const uint32_t blocks = uint32_t((words + 4095) >> 12);
  if (words >= (1u << 20))
    shared_pool().run(blocks, 64, mirror);
  else
    mirror(0, blocks);
  tables_dirty_ = true;
  graph_valid_ = false;
  *id = uint32_t(meshes_.size() - 1);
  return GBR_OK;
}

gbr_status Renderer::add_texture(const gbr_texture_data& t, uint32_t* id) {
  TraceRange trace_("gbr.add_texture");
  if (t.width <= 0 || t.height <= 0 || t.layers <= 0 || !t.rgba8)
    return fail(GBR_ERROR_INVALID_ARGUMENT, "addTexture: empty texture");
  if (t.filter < 0 || t.filter > 1 || t.wrap_s < 0 || t.wrap_s > 2 || t.wrap_t < 0 || t.wrap_t > 2 ||
      t.min_filter < 0 || t.min_filter > 2 || t.mip_filter < 0 || t.mip_filter > 2)
    return fail(GBR_ERROR_INVALID_ARGUMENT, "addTexture: bad filter or wrap mode");
  int levels = std::max(1, t.levels);
  if (levels > mip_max_levels(t.width, t.height))
    return fail(GBR_ERROR_INVALID_ARGUMENT, "addTexture: more levels than the size allows");
  std::vector<uint8_t> chain;
  const uint8_t* data = t.rgba8;
  if (t.generate_mipmap && levels == 1) {
    levels = mip_chain_levels(t.width, t.height);
    chain = generate_mips(t.rgba8, t.width, t.height, t.layers, levels);
    data = chain.data();
  }
  cudaSetDevice(device_);
  const size_t n = mip_texels(t.width, t.height, t.layers, levels);
  const uint64_t off = texel_pool_.alloc(n);
  if (!d_texels_.reserve(texel_pool_.end * 4, true)) {
    texel_pool_.release(off, n);
    return fail(GBR_ERROR_OUT_OF_MEMORY, "addTexture: out of device memory");
  }
  GBR_CUDA(cudaMemcpy(d_texels_.as<char>() + off * 4, data, n * 4, cudaMemcpyHostToDevice),
           "addTexture upload");
  TextureRec rec{};
  rec.offset = off;
  rec.width = t.width;
  rec.height = t.height;
  rec.layers = t.layers;
  rec.filter = t.filter;
  rec.wrap_s = t.wrap_s;
  rec.wrap_t = t.wrap_t;
  rec.min_filter = t.min_filter == 0 ? t.filter : t.min_filter - 1;
  rec.mip_filter = t.mip_filter;
  rec.levels = levels;
  textures_.push_back(rec);
  texture_live_.push_back(true);
  tables_dirty_ = true;
  graph_valid_ = false;
  *id = uint32_t(textures_.size() - 1);
  return GBR_OK;
}

gbr_status Renderer::add_material(const gbr_material_data& m, uint32_t* id) {
  MaterialRec rec{};
  std::memcpy(rec.color, m.color, 16);
  rec.texture = int32_t(m.texture);
  rec.layer = int32_t(m.layer);
  std::memcpy(rec.m, m.matrix, 36);
  // Lit only when lights are enabled (Renderer.cpp:579-620: every material is
  // flat otherwise).
  rec.phong = (m.shaded && max_lights_ > 0) ? 1 : 0;
  materials_.push_back(rec);
  tables_dirty_ = true;
  graph_valid_ = false;
  *id = uint32_t(materials_.size() - 1);
  return GBR_OK;
}

gbr_status Renderer::add_template(const char* name, uint32_t count, const gbr_mesh_view* views) {
  if (!name) return fail(GBR_ERROR_INVALID_ARGUMENT, "addNodeHierarchyTemplate: null name");
  if (names_.count(name))
    return fail(GBR_ERROR_INVALID_ARGUMENT,
                std::string("addNodeHierarchyTemplate: node name ") + name + " already exists");
  const uint32_t begin = uint32_t(views_.size());
  for (uint32_t i = 0; i < count; ++i) {
    const gbr_mesh_view& v = views[i];
    if (v.mesh >= meshes_.size() || v.material >= materials_.size())
      return fail(GBR_ERROR_INVALID_ARGUMENT, "addNodeHierarchyTemplate: bad mesh or material id");
    if (!mesh_live_[v.mesh])
      return fail(GBR_ERROR_STATE, "addNodeHierarchyTemplate: mesh " + std::to_string(v.mesh) +
                                       " was removed");
    const MeshRec& m = meshes_[v.mesh];
    if (uint64_t(v.index_offset) + v.index_count > m.index_count)
      return fail(GBR_ERROR_INVALID_ARGUMENT, "addNodeHierarchyTemplate: index range out of mesh");
  }
  for (uint32_t i = 0; i < count; ++i) {
    const gbr_mesh_view& v = views[i];
    MeshView mv{};
    mv.mesh = v.mesh;
    mv.index_offset = v.index_offset;
    mv.index_count = v.index_count;
    mv.material = v.material;
    std::memcpy(mv.transform, v.transform, 64);
    mv.chunk_count = (v.index_count / 3 + kChunkTris - 1) / kChunkTris;
    mv.box_base = uint32_t(box_pool_.alloc(mv.chunk_count + cluster_count(mv.chunk_count)));
    boxes_lo_ = std::min<size_t>(boxes_lo_, mv.box_base);
    boxes_hi_ = std::max<size_t>(boxes_hi_, mv.box_base + mv.chunk_count + cluster_count(mv.chunk_count));
    mv.live = true;
    views_.push_back(mv);
  }
  if (boxes_.size() < box_pool_.end) boxes_.resize(box_pool_.end);
  build_chunk_boxes(begin, uint32_t(views_.size()));
  names_[name] = {begin, uint32_t(views_.size())};
  tables_dirty_ = true;
  graph_valid_ = false;
  return GBR_OK;
}

// Object-space bounding box of every kChunkTris consecutive triangles of the
// views [first, last), of every kClusterChunks consecutive chunks, and of each
// whole view (every index of its range, also a trailing partial triangle)
// into its bbox {lo xyz, hi xyz}.  The clusters of all the views are one
// range of work for the host pool when they hold many triangles.
void Renderer::build_chunk_boxes(uint32_t first, uint32_t last) {
  auto extend = [](ChunkBox& b, const float* p) {
    for (int c = 0; c < 3; ++c) {
      b.lo[c] = std::min(b.lo[c], p[c]);
      b.hi[c] = std::max(b.hi[c], p[c]);
    }
  };
  auto empty = []() {
    ChunkBox b{};
    for (int k = 0; k < 3; ++k) {
      b.lo[k] = INFINITY;
      b.hi[k] = -INFINITY;
    }
    return b;
  };
  // Work units: (view, cluster) in view order.
  std::vector<uint32_t> unit_base(last - first + 1, 0);
  uint64_t tris_all = 0;
  for (uint32_t v = first; v < last; ++v) {
    unit_base[v - first + 1] = unit_base[v - first] + cluster_count(views_[v].chunk_count);
    tris_all += views_[v].index_count / 3;
  }
  const std::function<void(uint32_t, uint32_t)> fn = [&](uint32_t u0, uint32_t u1) {
    uint32_t v = uint32_t(std::upper_bound(unit_base.begin(), unit_base.end(), u0) - unit_base.begin()) - 1;
    for (uint32_t u = u0; u < u1; ++u) {
      while (u >= unit_base[v + 1]) ++v;
      const MeshView& mv = views_[first + v];
      const MeshRec& m = meshes_[mv.mesh];
      const uint32_t* idx = host_indices_.data() + size_t(m.index_base) + mv.index_offset;
      const float* pos = host_pos_.data() + size_t(m.vertex_base) * 3;
      const uint32_t tris = mv.index_count / 3, chunks = mv.chunk_count, cl = u - unit_base[v];
      ChunkBox c = empty();
      const uint32_t ch1 = std::min(chunks, (cl + 1) * kClusterChunks);
      for (uint32_t ch = cl * kClusterChunks; ch < ch1; ++ch) {
        ChunkBox b = empty();
        const uint32_t k1 = std::min(tris, (ch + 1) * kChunkTris) * 3;
        for (uint32_t k = ch * kChunkTris * 3; k < k1; ++k) extend(b, pos + size_t(idx[k]) * 3);
        boxes_[mv.box_base + ch] = b;
        for (int k = 0; k < 3; ++k) {
          c.lo[k] = std::min(c.lo[k], b.lo[k]);
          c.hi[k] = std::max(c.hi[k], b.hi[k]);
        }
      }
      boxes_[mv.box_base + chunks + cl] = c;
    }
  };
  const uint32_t units = unit_base.back();
  if (tris_all >= (1u << 16))
    shared_pool().run(units, 4, fn);
  else
    fn(0, units);
  for (uint32_t v = first; v < last; ++v) {
    MeshView& mv = views_[v];
    const MeshRec& m = meshes_[mv.mesh];
    const uint32_t* idx = host_indices_.data() + size_t(m.index_base) + mv.index_offset;
    const float* pos = host_pos_.data() + size_t(m.vertex_base) * 3;
    ChunkBox all = empty();
    for (uint32_t cl = 0; cl < cluster_count(mv.chunk_count); ++cl) {
      const ChunkBox& u = boxes_[mv.box_base + mv.chunk_count + cl];
      for (int k = 0; k < 3; ++k) {
        all.lo[k] = std::min(all.lo[k], u.lo[k]);
        all.hi[k] = std::max(all.hi[k], u.hi[k]);
      }
    }
    for (uint32_t k = mv.index_count / 3 * 3; k < mv.index_count; ++k) extend(all, pos + size_t(idx[k]) * 3);
    for (int c = 0; c < 3; ++c) {
      mv.bbox[c] = all.lo[c];
      mv.bbox[3 + c] = all.hi[c];
    }
  }
}

gbr_status Renderer::add_file(const char* filename, uint32_t flags, const char* name) {
  TraceRange trace_("gbr.add_file");
  if (!filename) return fail(GBR_ERROR_INVALID_ARGUMENT, "addFile: null filename");
  ImportedFile f;
  std::string err;
  const bool no_textures = cfg_.flags & GBR_FLAG_NO_TEXTURES;
  if (!import_gltf(filename, flags & GBR_FILE_WHOLE, name ? name : "", no_textures, f, err))
    return fail(GBR_ERROR_IO, "Renderer::addFile(): " + err);
  for (auto& t : f.templates)
    if (names_.count(t.name))
      return fail(GBR_ERROR_INVALID_ARGUMENT,
                  "Renderer::addFile(): node name " + t.name + " in " + filename + " already exists");
  const uint32_t texture_offset = uint32_t(textures_.size());
  const uint32_t mesh_offset = uint32_t(meshes_.size());
  const uint32_t material_offset = uint32_t(materials_.size());
  // GenerateMipmap: a full chain for single-level images that were not block
  // compressed (Renderer.cpp:445-477); the sampler's minification and mipmap
  // filters come from the file.
  for (auto& t : f.textures) {
    const int gen = (flags & GBR_FILE_GENERATE_MIPMAP) && !t.compressed ? 1 : 0;
    gbr_texture_data td{t.width, t.height, t.layers, t.rgba.data(), t.filter, t.wrap_s, t.wrap_t,
                        t.min_filter + 1, t.mip_filter, 1, gen};
    uint32_t id;
    gbr_status s = add_texture(td, &id);
    if (s != GBR_OK) return s;
  }
  for (auto& m : f.meshes) {
    gbr_mesh_data md{m.vertex_count,
                     m.positions.data(),
                     m.colors.empty() ? nullptr : m.colors.data(),
                     m.texcoords.empty() ? nullptr : m.texcoords.data(),
                     m.object_ids.empty() ? nullptr : m.object_ids.data(),
                     uint32_t(m.indices.size()),
                     m.indices.data(),
                     m.normals.empty() ? nullptr : m.normals.data()};
    uint32_t id;
    gbr_status s = add_mesh(md, &id);
    if (s != GBR_OK) return s;
  }
  for (auto& m : f.materials) {
    gbr_material_data md{};
    std::memcpy(md.color, m.color, 16);
    md.shaded = m.flat ? 0 : 1;
    if (m.texture < 0) {
      md.texture = 0;
      md.layer = 0;
      const float id3[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
      std::memcpy(md.matrix, id3, 36);
    } else {
      md.texture = uint32_t(m.texture) + texture_offset;
      md.layer = uint32_t(m.layer);
      std::memcpy(md.matrix, m.matrix, 36);
    }
    uint32_t id;
    add_material(md, &id);
  }
  for (auto& t : f.templates) {
    std::vector<gbr_mesh_view> views;
    for (uint32_t i = t.begin; i < t.end; ++i) {
      const ImportedView& v = f.views[i];
      gbr_mesh_view mv{};
      mv.mesh = v.mesh + mesh_offset;
      mv.index_offset = v.index_offset_bytes / 4;
      mv.index_count = v.index_count;
      mv.material = v.material < 0 ? 0u : uint32_t(v.material) + material_offset;
      std::memcpy(mv.transform, v.transform, 64);
      views.push_back(mv);
    }
    gbr_status s = add_template(t.name.c_str(), uint32_t(views.size()), views.data());
    if (s != GBR_OK) return s;
  }
  return GBR_OK;
}

// --------------------------------------------------------------- scenes
gbr_status Renderer::add_node_hierarchy(uint32_t scene, const char* name, const float* bake,
                                        uint64_t* id) {
  if (gbr_status s = check_scene(scene, "Renderer::addNodeHierarchy()")) return s;
  auto found = names_.find(name ? name : "");
  if (found == names_.end())
    return fail(GBR_ERROR_NOT_FOUND,
                std::string("Renderer::add(): name ") + (name ? name : "") + " not found");
  for (uint32_t i = found->second.first; i < found->second.second; ++i) {
    const MeshView& v = views_[i];
    if (!mesh_live_[v.mesh] || texture_removed(uint32_t(materials_[v.material].texture)))
      return fail(GBR_ERROR_STATE, std::string("Renderer::add(): ") + name +
                                       " uses a removed mesh or texture");
  }
  SceneState& sc = scenes_[scene];
  const uint32_t top = uint32_t(sc.parents.size());
  sc.parents.push_back(-1);
  sc.transforms.insert(sc.transforms.end(), kIdentity, kIdentity + 16);
  const float* b = bake ? bake : kIdentity;
  for (uint32_t i = found->second.first; i < found->second.second; ++i) {
    const MeshView& v = views_[i];
    const uint32_t nid = uint32_t(sc.parents.size());
    sc.parents.push_back(int32_t(top));
    float t[16];
    mat4_mul(b, v.transform, t);
    sc.transforms.insert(sc.transforms.end(), t, t + 16);
    const BatchKey key{meshes_[v.mesh].flags & kMeshVertexColor, v.mesh,
                       uint32_t(materials_[v.material].texture)};
    uint32_t batch = 0;
    while (batch < sc.batches.size() &&
           !(sc.batches[batch].flags == key.flags && sc.batches[batch].mesh == key.mesh &&
             sc.batches[batch].texture == key.texture))
      ++batch;
    if (batch == sc.batches.size()) sc.batches.push_back(key);
    HostDraw d{batch, nid, top, v.mesh, v.index_offset, v.index_count, v.material, 0u, {},
               v.box_base, v.chunk_count, i};
    std::memcpy(d.bbox, v.bbox, 24);
    sc.draws.push_back(d);
  }
  sc.transforms_dirty = true;
  structure_dirty_ = true;
  *id = top;
  return GBR_OK;
}

gbr_status Renderer::add_empty_node(uint32_t scene, uint64_t* id) {
  if (gbr_status s = check_scene(scene, "Renderer::addEmptyNode()")) return s;
  SceneState& sc = scenes_[scene];
  *id = sc.parents.size();
  sc.parents.push_back(-1);
  sc.transforms.insert(sc.transforms.end(), kIdentity, kIdentity + 16);
  sc.transforms_dirty = true;
  structure_dirty_ = true;
  return GBR_OK;
}

gbr_status Renderer::clear(uint32_t scene) {
  if (gbr_status s = check_scene(scene, "Renderer::clear()")) return s;
  SceneState& sc = scenes_[scene];
  sc.parents.clear();
  sc.transforms.clear();
  sc.draws.clear();
  sc.batches.clear();
  sc.light_nodes.clear();
  sc.light_types.clear();
  sc.light_colors.clear();
  sc.light_ranges.clear();
  structure_dirty_ = true;
  return GBR_OK;
}

gbr_status Renderer::add_light(uint32_t scene, uint64_t node, uint32_t type, uint64_t* id) {
  if (max_lights_ == 0) return fail(GBR_ERROR_STATE, "Renderer::addLight(): max light count is zero");
  if (gbr_status s = check_scene(scene, "Renderer::addLight()")) return s;
  SceneState& sc = scenes_[scene];
  if (node >= sc.parents.size())
    return fail(GBR_ERROR_INVALID_ARGUMENT, "Renderer::addLight(): index " + std::to_string(node) +
                                                " out of range for " +
                                                std::to_string(sc.parents.size()) + " nodes");
  if (type > 1) return fail(GBR_ERROR_INVALID_ARGUMENT, "Renderer::addLight(): bad light type");
  *id = sc.light_nodes.size();
  sc.light_nodes.push_back(int32_t(node));
  sc.light_types.push_back(int32_t(type));
  sc.light_colors.insert(sc.light_colors.end(), {1.0f, 1.0f, 1.0f});
  sc.light_ranges.push_back(INFINITY);
  return GBR_OK;
}

gbr_status Renderer::clear_lights(uint32_t scene) {
  if (gbr_status s = check_scene(scene, "Renderer::clearLights()")) return s;
  SceneState& sc = scenes_[scene];
  sc.light_nodes.clear();
  sc.light_types.clear();
  sc.light_colors.clear();
  sc.light_ranges.clear();
  return GBR_OK;
}

gbr_status Renderer::light_colors(uint32_t scene, float** out, uint64_t* count) {
  if (gbr_status s = check_scene(scene, "Renderer::lightColors()")) return s;
  SceneState& sc = scenes_[scene];
  *out = sc.light_colors.empty() ? nullptr : sc.light_colors.data();
  *count = sc.light_nodes.size();
  return GBR_OK;
}

gbr_status Renderer::light_ranges(uint32_t scene, float** out, uint64_t* count) {
  if (gbr_status s = check_scene(scene, "Renderer::lightRanges()")) return s;
  SceneState& sc = scenes_[scene];
  *out = sc.light_ranges.empty() ? nullptr : sc.light_ranges.data();
  *count = sc.light_nodes.size();
  return GBR_OK;
}

size_t Renderer::camera_block_bytes() const {
  return scenes_.size() * (kCameraBytes + size_t(max_lights_) * sizeof(LightSrc));
}

gbr_status Renderer::set_semantic_id(uint32_t scene, uint64_t node, uint32_t id) {
  if (gbr_status s = check_scene(scene, "Renderer::setSemanticId()")) return s;
  SceneState& sc = scenes_[scene];
  if (node >= sc.parents.size())
    return fail(GBR_ERROR_INVALID_ARGUMENT, "Renderer::setSemanticId(): node out of range");
  for (auto& d : sc.draws)
    if (d.top == node) d.semantic = id;
  structure_dirty_ = true;
  return GBR_OK;
}

gbr_status Renderer::update_camera(uint32_t scene, const float* p, const float* v) {
  if (gbr_status s = check_scene(scene, "Renderer::updateCamera()")) return s;
  SceneState& sc = scenes_[scene];
  mat4_mul(p, v, sc.pv);
  std::memcpy(sc.view, v, 64);
  std::memcpy(sc.proj, p, 64);
  // calculateDepthUnprojection (DepthUnprojection.cpp:98-101)
  sc.unprojection[0] = (p[2 * 4 + 2] - 1.0f) * 0.5f;
  sc.unprojection[1] = p[3 * 4 + 2] * 0.5f;
  return GBR_OK;
}

gbr_status Renderer::update_cameras(uint32_t first, uint32_t count, const float* p,
                                    const float* v) {
  if (uint64_t(first) + count > scenes_.size())
    return fail(GBR_ERROR_INVALID_ARGUMENT, "updateCameras: scene range out of bounds");
  for (uint32_t i = 0; i < count; ++i) update_camera(first + i, p + 16 * size_t(i), v + 16 * size_t(i));
  return GBR_OK;
}

gbr_status Renderer::camera(uint32_t scene, float* out) const {
  if (gbr_status s = check_scene(scene, "Renderer::camera()")) return s;
  std::memcpy(out, scenes_[scene].pv, 64);
  return GBR_OK;
}

gbr_status Renderer::unprojection(uint32_t scene, float* out) const {
  if (gbr_status s = check_scene(scene, "Renderer::cameraDepthUnprojection()")) return s;
  out[0] = scenes_[scene].unprojection[0];
  out[1] = scenes_[scene].unprojection[1];
  return GBR_OK;
}

gbr_status Renderer::transformations(uint32_t scene, float** out, uint64_t* count) {
  if (gbr_status s = check_scene(scene, "Renderer::transformations()")) return s;
  SceneState& sc = scenes_[scene];
  *out = sc.transforms.empty() ? nullptr : sc.transforms.data();
  *count = sc.parents.size();
  sc.transforms_dirty = true;
  return GBR_OK;
}

gbr_status Renderer::stats(uint32_t scene, gbr_scene_stats_info* out) const {
  if (gbr_status s = check_scene(scene, "Renderer::sceneStats()")) return s;
  const SceneState& sc = scenes_[scene];
  out->node_count = sc.parents.size();
  out->draw_count = sc.draws.size();
  out->draw_batch_count = sc.batches.size();
  return GBR_OK;
}

gbr_status Renderer::set_sources(uint32_t first, uint32_t count, const uint32_t* sources) {
  if (uint64_t(first) + count > scenes_.size())
    return fail(GBR_ERROR_INVALID_ARGUMENT, "setSceneSources: scene range out of bounds");
  if (count && !sources) return fail(GBR_ERROR_INVALID_ARGUMENT, "setSceneSources: null sources");
  for (uint32_t i = 0; i < count; ++i)
    if (sources[i] >= scenes_.size())
      return fail(GBR_ERROR_INVALID_ARGUMENT, "setSceneSources: source " +
                                                  std::to_string(sources[i]) + " out of range");
  for (uint32_t i = 0; i < count; ++i)
    if (scenes_[first + i].source != sources[i]) {
      scenes_[first + i].source = sources[i];
      bindings_dirty_ = true;
    }
  return GBR_OK;
}

gbr_status Renderer::set_enabled(uint32_t scene, bool enabled) {
  if (gbr_status s = check_scene(scene, "setSceneEnabled()")) return s;
  if (scenes_[scene].enabled != enabled) {
    scenes_[scene].enabled = enabled;
    bindings_dirty_ = true;
  }
  return GBR_OK;
}

// ------------------------------------------------------------- removal
// Device ranges of a removed resource are reused by later adds, so nothing
// the GPU may still be reading (the last draw) can be released early.
gbr_status Renderer::quiesce() {
  cudaSetDevice(device_);
  return wait_uploads();  // upload_done_ follows the whole step that used each slot
}

gbr_status Renderer::wait_uploads() {
  for (int s = 0; s < 2; ++s)
    if (upload_pending_[s]) {
      GBR_CUDA(cudaEventSynchronize(upload_done_[s]), "wait for previous steps");
      upload_pending_[s] = false;
    }
  return GBR_OK;
}

gbr_status Renderer::remove_mesh(uint32_t mesh) {
  if (mesh >= meshes_.size() || !mesh_live_[mesh])
    return fail(GBR_ERROR_INVALID_ARGUMENT, "removeMesh: no mesh " + std::to_string(mesh));
  if (gbr_status s = quiesce()) return s;
  const MeshRec& m = meshes_[mesh];
  vertex_pool_.release(m.vertex_base, m.vertex_count);
  index_pool_.release(m.index_base, m.index_count);
  mesh_live_[mesh] = false;
  structure_dirty_ = true;  // the next draw checks that no scene uses it
  return GBR_OK;
}

gbr_status Renderer::remove_texture(uint32_t texture) {
  if (texture == 0)
    return fail(GBR_ERROR_INVALID_ARGUMENT, "removeTexture: texture 0 is reserved");
  if (texture >= textures_.size() || !texture_live_[texture])
    return fail(GBR_ERROR_INVALID_ARGUMENT, "removeTexture: no texture " + std::to_string(texture));
  if (gbr_status s = quiesce()) return s;
  const TextureRec& t = textures_[texture];
  texel_pool_.release(t.offset, mip_texels(t.width, t.height, t.layers, t.levels));
  texture_live_[texture] = false;
  structure_dirty_ = true;
  return GBR_OK;
}

gbr_status Renderer::remove_template(const char* name) {
  auto found = names_.find(name ? name : "");
  if (found == names_.end())
    return fail(GBR_ERROR_NOT_FOUND,
                std::string("removeNodeHierarchyTemplate: name ") + (name ? name : "") + " not found");
  if (gbr_status s = quiesce()) return s;
  for (uint32_t i = found->second.first; i < found->second.second; ++i) {
    MeshView& v = views_[i];
    box_pool_.release(v.box_base, v.chunk_count + cluster_count(v.chunk_count));
    v.live = false;
  }
  names_.erase(found);
  structure_dirty_ = true;
  return GBR_OK;
}

gbr_status Renderer::memory_usage(uint64_t* live, uint64_t* reserved) const {
  // Bytes per element: vertices 16 position + 16 colour + 8 texcoord,
  // indices and texels 4, chunk and cluster boxes 32.
  constexpr uint64_t kV = 40, kI = 4, kT = 4, kB = sizeof(ChunkBox);
  if (live)
    *live = vertex_pool_.live() * kV + index_pool_.live() * kI + texel_pool_.live() * kT +
            box_pool_.live() * kB;
  if (reserved)
    *reserved = vertex_pool_.end * kV + index_pool_.end * kI + texel_pool_.end * kT +
                box_pool_.end * kB;
  return GBR_OK;
}

// -------------------------------------------------------------- drawing
gbr_status Renderer::upload_tables() {
  if (!tables_dirty_) return GBR_OK;
  if (!d_meshes_.reserve(std::max<size_t>(1, meshes_.size()) * sizeof(MeshRec), false) ||
      !d_materials_.reserve(materials_.size() * sizeof(MaterialRec), false) ||
      !d_textures_.reserve(textures_.size() * sizeof(TextureRec), false) ||
      !d_boxes_.reserve(std::max<size_t>(1, boxes_.size()) * sizeof(ChunkBox), true))
    return fail(GBR_ERROR_OUT_OF_MEMORY, "draw: out of device memory for tables");
  // Only the boxes written since the last upload (the device copy keeps the
  // rest, also across growth): a scene loaded into a large resident set
  // costs its own boxes, not the whole table.
  if (boxes_hi_ > boxes_lo_) {
    GBR_CUDA(cudaMemcpy(d_boxes_.as<ChunkBox>() + boxes_lo_, boxes_.data() + boxes_lo_,
                        (boxes_hi_ - boxes_lo_) * sizeof(ChunkBox), cudaMemcpyHostToDevice),
             "table upload");
    boxes_lo_ = SIZE_MAX;
    boxes_hi_ = 0;
  }
  if (!meshes_.empty())
    GBR_CUDA(cudaMemcpy(d_meshes_.ptr, meshes_.data(), meshes_.size() * sizeof(MeshRec),
                        cudaMemcpyHostToDevice), "table upload");
  GBR_CUDA(cudaMemcpy(d_materials_.ptr, materials_.data(), materials_.size() * sizeof(MaterialRec),
                      cudaMemcpyHostToDevice), "table upload");
  GBR_CUDA(cudaMemcpy(d_textures_.ptr, textures_.data(), textures_.size() * sizeof(TextureRec),
                      cudaMemcpyHostToDevice), "table upload");
  tables_dirty_ = false;
  return GBR_OK;
}

gbr_status Renderer::rebuild(cudaStream_t stream) {
  GBR_CUDA(cudaStreamSynchronize(stream), "draw: synchronise before rebuild");
  if (gbr_status st = wait_uploads()) return st;
  const uint32_t S = uint32_t(scenes_.size());
  std::vector<SceneRec> recs(S);
  std::vector<int32_t> parents;
  std::vector<DrawRec> draws;
  std::vector<uint64_t> cost(S, 0);
  uint32_t nodes = 0;
  for (uint32_t s = 0; s < S; ++s) {
    SceneState& sc = scenes_[s];
    SceneRec& r = recs[s];
    r.width = sc.width;
    r.height = sc.height;
    r.fb_offset = sc.fb_offset;
    r.pitch = sc.pitch;
    r.node_base = nodes;
    r.node_count = uint32_t(sc.parents.size());
    sc.node_base = nodes;
    r.draw_base = uint32_t(draws.size());
    r.draw_count = uint32_t(sc.draws.size());
    nodes += r.node_count;
    parents.insert(parents.end(), sc.parents.begin(), sc.parents.end());
    // Stable counting sort of the draws by batch id (Renderer.cpp:1139-1196).
    std::vector<uint32_t> order(sc.draws.size());
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
      return sc.draws[a].batch < sc.draws[b].batch;
    });
    uint64_t tris = 0;
    for (uint32_t k : order) {
      const HostDraw& d = sc.draws[k];
      if (!mesh_live_[d.mesh] || !views_[d.view].live ||
          texture_removed(uint32_t(materials_[d.material].texture)))
        return fail(GBR_ERROR_STATE, "draw: scene " + std::to_string(s) +
                                         " uses a removed mesh, texture or hierarchy template;"
                                         " clear it first");
      DrawRec dr{};
      dr.node = d.node;
      dr.mesh = d.mesh;
      dr.first_index = meshes_[d.mesh].index_base + d.index_offset;
      dr.tri_count = d.index_count / 3;
      dr.material = d.material;
      dr.semantic_id = d.semantic;
      std::memcpy(dr.bbox, d.bbox, 24);
      dr.box_base = d.box_base;
      dr.chunk_count = d.chunk_count;
      draws.push_back(dr);
      tris += dr.tri_count;
    }
    if (tris >= (1ull << 31))
      return fail(GBR_ERROR_INVALID_ARGUMENT, "draw: 2^31 or more triangles in one scene");
    cost[s] = tris;
    sc.draw_count = r.draw_count;
    sc.tris = tris;
  }
  total_nodes_ = nodes;
  total_draws_ = uint32_t(draws.size());
  total_tris_ = std::accumulate(cost.begin(), cost.end(), uint64_t(0));

  // Work items: each scene's viewport cut into regions.  The per-scene form
  // uses small regions so that one scene spreads over several CTAs; the
  // batched form uses large ones (fewer redundant triangle setups), ordered
  // longest-processing-time first for the persistent grid by order_items().
  std::vector<WorkItem> items;
  scene_item_base_.assign(S, 0);
  scene_item_count_.assign(S, 0);
  auto tile = [&](uint32_t s, int rwm, int rhm, std::vector<WorkItem>& out) {
    const SceneState& sc = scenes_[s];
    for (int y = 0; y < sc.height; y += rhm)
      for (int x = 0; x < sc.width; x += rwm) {
        WorkItem it{};
        it.scene = s;
        it.x0 = uint16_t(x);
        it.y0 = uint16_t(y);
        it.w = uint16_t(std::min(rwm, sc.width - x));
        it.h = uint16_t(std::min(rhm, sc.height - y));
        out.push_back(it);
      }
  };
  std::vector<ItemScene> info(S);
  for (uint32_t s = 0; s < S; ++s) {
    scene_item_base_[s] = uint32_t(items.size());
    tile(s, tuning_.plain_region_width, tuning_.plain_region_height, items);
    scene_item_count_[s] = uint32_t(items.size()) - scene_item_base_[s];
    info[s].width = scenes_[s].width;
    info[s].height = scenes_[s].height;
  }
  // Every scene at its finest split, whichever are enabled, and the last
  // wave's halves (at most one per resident CTA, 8 per SM).
  const uint64_t capacity =
      work_item_capacity(info, tuning_.region_width, tuning_.region_height, uint64_t(sm_count_) * 8);
  if (capacity > 0xffffffffull) return fail(GBR_ERROR_INVALID_ARGUMENT, "draw: too many work items");
  item_count_ = uint32_t(items.size());
  lpt_count_ = uint32_t(capacity);

  cudaSetDevice(device_);
  if (gbr_status st = upload_tables()) return st;
  const size_t S1 = std::max<size_t>(S, 1);
  if (!d_scenes_.reserve(S1 * sizeof(SceneRec), false) ||
      !d_parents_.reserve(std::max<size_t>(nodes, 1) * 4, false) ||
      !d_local_.reserve(std::max<size_t>(nodes, 1) * 64, false) ||
      !d_draws_.reserve(std::max<size_t>(draws.size(), 1) * sizeof(DrawRec), false) ||
      !d_cameras_.reserve(std::max<size_t>(camera_block_bytes(), 1), false) ||
      !d_lights_.reserve(std::max<size_t>(size_t(S) * max_lights_ * sizeof(WorldLight), 16), false) ||
      !d_visible_.reserve(std::max<size_t>(draws.size(), 1) * sizeof(VisibleRec), false) ||
      !d_order_.reserve(std::max<size_t>(draws.size(), 1) * sizeof(uint2), false) ||
      !d_vis_count_.reserve(S1 * 4, false) || !d_vis_tris_.reserve(S1 * 4, false) ||
      !d_vis_clusters_.reserve(S1 * 4, false) ||
      !d_status_.reserve(4, false) || !d_counter_.reserve(4, false) ||
      !d_items_.reserve(std::max<size_t>(items.size(), 1) * sizeof(WorkItem), false) ||
      !d_items_lpt_.reserve((size_t(lpt_count_) + 1) * sizeof(WorkItem), false) ||
      !h_stage_[0].reserve(std::max<size_t>(camera_block_bytes(), 1) +
                           std::max<size_t>(nodes, 1) * 64 +
                           (size_t(lpt_count_) + 1) * sizeof(WorkItem)) ||
      !h_stage_[1].reserve(h_stage_[0].bytes))
    return fail(GBR_ERROR_OUT_OF_MEMORY, "draw: out of memory for scene data");
  GBR_CUDA(cudaMemcpy(d_scenes_.ptr, recs.data(), S * sizeof(SceneRec), cudaMemcpyHostToDevice),
           "scene upload");
  if (nodes)
    GBR_CUDA(cudaMemcpy(d_parents_.ptr, parents.data(), nodes * 4, cudaMemcpyHostToDevice),
             "scene upload");
  if (!draws.empty())
    GBR_CUDA(cudaMemcpy(d_draws_.ptr, draws.data(), draws.size() * sizeof(DrawRec),
                        cudaMemcpyHostToDevice), "scene upload");
  if (!items.empty())
    GBR_CUDA(cudaMemcpy(d_items_.ptr, items.data(), items.size() * sizeof(WorkItem),
                        cudaMemcpyHostToDevice), "scene upload");
  GBR_CUDA(cudaMemset(d_status_.ptr, 0, 4), "scene upload");
  for (auto& sc : scenes_) sc.transforms_dirty = true;
  structure_dirty_ = false;
  bindings_dirty_ = true;  // item order and visible-record bases follow the new draws
  graph_valid_ = false;
  return GBR_OK;
}

gbr_status Renderer::ensure_raster_config() {
  if (raster_configured_) return GBR_OK;
  const int region_px = tuning_.region_width * tuning_.region_height;
  const int plain_px = tuning_.plain_region_width * tuning_.plain_region_height;
  size_t max_dyn = 0, static_smem = 0;
  GBR_CUDA(raster_configure(tuning_.threads, &max_dyn, &static_smem), "raster configure");
  // Room for the requested CTAs per SM: the SM's shared memory less the
  // per-CTA reservation and static part, shared by ctas_per_sm CTAs.
  int per_sm = 0, reserved = 0;
  cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, device_);
  cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, device_);
  const int want = std::max(1, tuning_.ctas_per_sm);
  size_t budget = max_dyn;
  if (want > 1 && per_sm > 0) {
    const size_t share = size_t(per_sm) / size_t(want);
    const size_t fixed = size_t(reserved) + static_smem;
    budget = std::min(budget, share > fixed ? share - fixed : size_t(0));
  }
  int cap = kPrefixCapMax;
  size_t smem = raster_smem_bytes(tuning_.threads, std::max(region_px, plain_px), cap);
  while (smem > budget && cap > 64) {
    cap /= 2;
    smem = raster_smem_bytes(tuning_.threads, std::max(region_px, plain_px), cap);
  }
  if (smem > max_dyn)
    return fail(GBR_ERROR_INVALID_ARGUMENT, "tuning: region does not fit in shared memory");
  smem = raster_smem_bytes(tuning_.threads, region_px, cap);
  int occ = 0;
  GBR_CUDA(raster_max_ctas_per_sm(tuning_.threads, smem, &occ), "raster occupancy");
  if (occ < 1) return fail(GBR_ERROR_INVALID_ARGUMENT, "tuning: raster kernel cannot be resident");
  ctas_per_sm_ = std::min(occ, std::max(1, tuning_.ctas_per_sm));
  smem_bytes_ = smem;
  smem_plain_ = raster_smem_bytes(tuning_.threads, plain_px, cap);
  prefix_cap_ = cap;
  raster_configured_ = true;
  return GBR_OK;
}

gbr_status Renderer::upload_step(cudaStream_t stream) {
  // Cameras always, local transforms of scenes whose view was taken.
  const uint32_t S = uint32_t(scenes_.size());
  if (upload_pending_[slot_]) {  // the step that last used this staging slot
    GBR_CUDA(cudaEventSynchronize(upload_done_[slot_]), "draw: wait for previous upload");
    upload_pending_[slot_] = false;
  }
  char* stage = static_cast<char*>(h_stage_[slot_].ptr);
  if (bindings_dirty_) {
    // Visible records: each enabled scene gets room for its source's draws.
    uint64_t base = 0;
    for (uint32_t s = 0; s < S; ++s) {
      SceneState& sc = scenes_[s];
      sc.vis_base = uint32_t(base);
      if (sc.enabled) base += scenes_[sc.source].draw_count;
      if (base > 0xffffffffull) return fail(GBR_ERROR_INVALID_ARGUMENT, "draw: too many draws");
    }
    vis_needed_ = base;
    void* before = d_visible_.ptr;
    void* before_order = d_order_.ptr;
    void* before_model = d_model_.ptr;
    if (!d_visible_.reserve(std::max<uint64_t>(base, 1) * sizeof(VisibleRec), false) ||
        !d_order_.reserve(std::max<uint64_t>(base, 1) * sizeof(uint2), false) ||
        (max_lights_ > 0 &&
         !d_model_.reserve(std::max<uint64_t>(base, 1) * sizeof(ModelRec), false)))
      return fail(GBR_ERROR_OUT_OF_MEMORY, "draw: out of device memory for visible draws");
    if (d_visible_.ptr != before || d_order_.ptr != before_order || d_model_.ptr != before_model)
      graph_valid_ = false;
    order_items();
    bindings_dirty_ = false;
  }
  CameraRec* cams = reinterpret_cast<CameraRec*>(stage);
  for (uint32_t s = 0; s < S; ++s) {
    const SceneState& sc = scenes_[s];
    std::memcpy(cams[s].pv, sc.pv, 64);
    for (int k = 0; k < 4; ++k) cams[s].vrow[k] = sc.view[k * 4 + 2];
    cams[s].source = sc.source;
    cams[s].vis_base = sc.vis_base;
    cams[s].enabled = sc.enabled ? 1u : 0u;
    cams[s].light_count = uint32_t(std::min<size_t>(sc.light_nodes.size(), max_lights_));
  }
  if (max_lights_ > 0) {
    // Light sources (colours and ranges are host-writable views): re-staged
    // every step after the cameras, uploaded with them.
    LightSrc* ls = reinterpret_cast<LightSrc*>(stage + S * kCameraBytes);
    for (uint32_t s = 0; s < S; ++s) {
      const SceneState& sc = scenes_[s];
      for (uint32_t j = 0; j < max_lights_; ++j) {
        LightSrc& d = ls[size_t(s) * max_lights_ + j];
        if (j < sc.light_nodes.size()) {
          d.node = sc.light_nodes[j];
          d.type = sc.light_types[j];
          for (int c = 0; c < 3; ++c) d.color[c] = sc.light_colors[j * 3 + c];
          d.range = sc.light_ranges[j];
        } else {
          d = LightSrc{};
        }
      }
    }
  }
  if (items_staged_) {
    WorkItem* istage = reinterpret_cast<WorkItem*>(stage + camera_block_bytes() +
                                                   size_t(total_nodes_) * 64);
    if (lpt_items_)
      GBR_CUDA(cudaMemcpyAsync(d_items_lpt_.ptr, istage, size_t(lpt_items_) * sizeof(WorkItem),
                               cudaMemcpyHostToDevice, stream), "work item upload");
    GBR_CUDA(cudaMemcpyAsync(d_items_lpt_.as<WorkItem>() + lpt_count_, istage + lpt_count_, 4,
                             cudaMemcpyHostToDevice, stream), "work item upload");
    items_staged_ = false;
  }
  float* tstage = reinterpret_cast<float*>(stage + camera_block_bytes());
  // Coalesce runs of dirty scenes into single copies.
  uint32_t s = 0;
  while (s < S) {
    if (!scenes_[s].transforms_dirty || scenes_[s].parents.empty()) {
      scenes_[s].transforms_dirty = false;
      ++s;
      continue;
    }
    const uint32_t begin = s;
    while (s < S && (scenes_[s].transforms_dirty || scenes_[s].parents.empty())) {
      SceneState& sc = scenes_[s];
      if (!sc.parents.empty())
        std::memcpy(tstage + size_t(sc.node_base) * 16, sc.transforms.data(), sc.parents.size() * 64);
      sc.transforms_dirty = false;
      ++s;
    }
    const size_t nb = scenes_[begin].node_base;
    const size_t ne = s < S ? scenes_[s].node_base : total_nodes_;
    if (ne > nb)
      GBR_CUDA(cudaMemcpyAsync(d_local_.as<float>() + nb * 16, tstage + nb * 16, (ne - nb) * 64,
                               cudaMemcpyHostToDevice, stream), "transform upload");
  }
  return GBR_OK;
}

// The batched form's work items of the enabled scenes (build_work_items:
// longest first, costly regions split, the last wave halved), staged for
// upload_step() with their count.
void Renderer::order_items() {
  std::vector<ItemScene> info(scenes_.size());
  for (size_t s = 0; s < scenes_.size(); ++s) {
    const SceneState& sc = scenes_[s];
    const SceneState& src = scenes_[sc.source];
    ItemScene& it = info[s];
    it.width = sc.width;
    it.height = sc.height;
    it.tris = src.tris;
    it.enabled = sc.enabled;
    // Geometry of the source: the mesh of its largest draw.
    uint32_t best = 0;
    it.geometry = 0xffffffffu;
    for (const HostDraw& d : src.draws)
      if (d.index_count > best) {
        best = d.index_count;
        it.geometry = d.mesh;
      }
  }
  const uint64_t grid = std::max<uint64_t>(1, uint64_t(sm_count_) * uint64_t(ctas_per_sm_));
  const std::vector<WorkItem> items = build_work_items(info, tuning_.region_width, tuning_.region_height, grid);
  WorkItem* istage = reinterpret_cast<WorkItem*>(static_cast<char*>(h_stage_[slot_].ptr) +
                                                 camera_block_bytes() +
                                                 size_t(total_nodes_) * 64);
  std::copy(items.begin(), items.end(), istage);
  lpt_items_ = uint32_t(items.size());
  std::memcpy(istage + lpt_count_, &lpt_items_, 4);
  items_staged_ = true;
}

gbr_status Renderer::enqueue_step(cudaStream_t stream, uint32_t mode) {
  const uint32_t S = uint32_t(scenes_.size());
  PrepareParams pp{};
  pp.scenes = d_scenes_.as<SceneRec>();
  pp.cameras = d_cameras_.as<CameraRec>();
  pp.draws = d_draws_.as<DrawRec>();
  pp.parents = d_parents_.as<int32_t>();
  pp.local = d_local_.as<float>();
  pp.meshes = d_meshes_.as<MeshRec>();
  pp.visible = d_visible_.as<VisibleRec>();
  pp.order = d_order_.as<uint2>();
  pp.max_lights = max_lights_;
  if (max_lights_ > 0) {
    pp.light_src = reinterpret_cast<const LightSrc*>(d_cameras_.as<char>() + S * kCameraBytes);
    pp.lights = d_lights_.as<WorldLight>();
    pp.model = d_model_.as<ModelRec>();
  }
  pp.vis_count = d_vis_count_.as<uint32_t>();
  pp.vis_tris = d_vis_tris_.as<uint32_t>();
  pp.vis_clusters = d_vis_clusters_.as<uint32_t>();
  pp.status = d_status_.as<uint32_t>();
  RasterParams rp{};
  rp.scenes = pp.scenes;
  rp.cameras = pp.cameras;
  rp.visible = pp.visible;
  rp.order = pp.order;
  rp.vis_count = pp.vis_count;
  rp.vis_tris = pp.vis_tris;
  rp.vis_clusters = pp.vis_clusters;
  rp.boxes = d_boxes_.as<ChunkBox>();
  rp.pos = d_pos_.as<float4>();
  rp.color = d_color_.as<float4>();
  rp.uv = d_uv_.as<float2>();
  rp.indices = d_indices_.as<uint32_t>();
  rp.materials = d_materials_.as<MaterialRec>();
  rp.textures = d_textures_.as<TextureRec>();
  rp.texels = d_texels_.as<uint32_t>();
  rp.texture_count = int32_t(textures_.size());
  rp.flags = (cfg_.flags & GBR_FLAG_NO_TEXTURES) ? 1u : 0u;
  rp.counter = d_counter_.as<uint32_t>();
  DeviceBuffer* planes = d_planes_[draw_set_];
  rp.out.color = (cfg_.planes & GBR_PLANE_COLOR) ? planes[0].as<uint32_t>() : nullptr;
  rp.out.depth = (cfg_.planes & GBR_PLANE_DEPTH) ? planes[1].as<float>() : nullptr;
  rp.out.linear = (cfg_.planes & GBR_PLANE_LINEAR_DEPTH) ? planes[2].as<float>() : nullptr;
  rp.out.semantic = (cfg_.planes & GBR_PLANE_SEMANTIC) ? planes[3].as<uint32_t>() : nullptr;
  rp.prefix_cap = prefix_cap_;
  rp.spill = d_spill_.ptr;
  rp.small_area = tuning_.small_area;
  rp.occlusion = tuning_.occlusion_culling;
  rp.flush_at = uint32_t(std::max(1, tuning_.threads * tuning_.queue_fill_percent / 100));
  rp.max_lights = max_lights_;
  rp.ambient_factor = cfg_.ambient_factor;
  rp.any_lod = 0;
  for (size_t i = 0; i < textures_.size(); ++i)
    if (texture_live_[i] && (textures_[i].mip_filter != 0 || textures_[i].min_filter != textures_[i].filter))
      rp.any_lod = 1;
  if (max_lights_ > 0) {
    rp.lights = pp.lights;
    rp.model = pp.model;
    rp.normals = d_normal_.as<float4>();
  }
  uint64_t launches = 0;
  if (mode == GBR_DRAW_BATCHED) {
    pp.scene_base = 0;
    if (timing_) GBR_CUDA(cudaEventRecordWithFlags(ev_[0], stream, cudaEventRecordExternal), "timing event");
    GBR_CUDA(launch_prepare(pp, S, stream), "prepare launch");
    GBR_CUDA(cudaMemsetAsync(d_counter_.ptr, 0, 4, stream), "counter reset");
    if (timing_) GBR_CUDA(cudaEventRecordWithFlags(ev_[1], stream, cudaEventRecordExternal), "timing event");
    rp.items = d_items_lpt_.as<WorkItem>();
    rp.item_base = 0;
    rp.item_count = lpt_count_;
    rp.item_count_dev = reinterpret_cast<const uint32_t*>(d_items_lpt_.as<WorkItem>() + lpt_count_);
    rp.persistent = 1;
    rp.region_px = tuning_.region_width * tuning_.region_height;
    const uint32_t grid =
        std::min<uint32_t>(lpt_count_, uint32_t(sm_count_) * uint32_t(ctas_per_sm_));
    GBR_CUDA(launch_raster(rp, tuning_.threads, grid, smem_bytes_, stream), "raster launch");
    if (timing_) GBR_CUDA(cudaEventRecordWithFlags(ev_[2], stream, cudaEventRecordExternal), "timing event");
    launches = 2;
  } else {
    rp.items = d_items_.as<WorkItem>();
    rp.persistent = 0;
    rp.region_px = tuning_.plain_region_width * tuning_.plain_region_height;
    for (uint32_t s = 0; s < S; ++s) {
      if (!scenes_[s].enabled) continue;
      pp.scene_base = s;
      GBR_CUDA(launch_prepare(pp, 1, stream), "prepare launch");
      rp.item_base = scene_item_base_[s];
      rp.item_count = scene_item_count_[s];
      GBR_CUDA(launch_raster(rp, tuning_.threads, scene_item_count_[s], smem_plain_, stream),
               "raster launch");
      launches += 2;
    }
  }
  launches_ = launches;
  return GBR_OK;
}

gbr_status Renderer::draw(cudaStream_t stream, uint32_t mode, bool use_graph) {
  TraceRange trace_("gbr.draw");
  cudaSetDevice(device_);
  if (use_graph && mode == GBR_DRAW_BATCHED && stream == nullptr) stream = own_stream_;
  if (structure_dirty_)
    if (gbr_status s = rebuild(stream)) return s;
  if (gbr_status s = ensure_raster_config()) return s;
  if (tables_dirty_)
    if (gbr_status s = upload_tables()) return s;
  {
    // Queue spill space for every CTA of the largest launch (allocated
    // before any graph capture).
    uint32_t grid = uint32_t(sm_count_) * uint32_t(ctas_per_sm_);
    if (mode != GBR_DRAW_BATCHED)
      for (uint32_t c : scene_item_count_) grid = std::max(grid, c);
    void* before = d_spill_.ptr;
    if (!d_spill_.reserve(raster_spill_bytes(tuning_.threads, grid), false))
      return fail(GBR_ERROR_OUT_OF_MEMORY, "draw: out of device memory for the raster queue");
    if (d_spill_.ptr != before) graph_valid_ = false;
  }
  const int prev_slot = slot_;
  slot_ ^= 1;  // this draw's staging slot (and plane set when double-buffered)
  if (gbr_status s = upload_step(stream)) {
    slot_ = prev_slot;
    return s;
  }
  const uint32_t S = uint32_t(scenes_.size());
  const size_t cam_bytes = camera_block_bytes();
  // The plane set this draw writes; with double buffering, the one the last
  // draw did not write, once the readbacks of its previous contents are done.
  const int set = double_buffer_ ? slot_ : 0;
  draw_set_ = set;
  if (copy_pending_[set]) {
    GBR_CUDA(cudaStreamWaitEvent(stream, copy_done_[set], 0), "wait for readback");
    copy_pending_[set] = false;
  }
  if (!graph_valid_) {
    graph_built_[0] = graph_built_[1] = false;
    graph_valid_ = true;
  }
  const int gi = slot_;  // graphs by staging slot (and with it the plane set)
  if (mode == GBR_DRAW_BATCHED && use_graph) {
    if (!graph_built_[gi] || graph_stream_[gi] != stream) {
      if (graph_exec_[gi]) {
        cudaGraphExecDestroy(graph_exec_[gi]);
        graph_exec_[gi] = nullptr;
      }
      cudaGraph_t g;
      GBR_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "graph capture");
      cudaError_t e = cudaMemcpyAsync(d_cameras_.ptr, h_stage_[gi].ptr, cam_bytes,
                                      cudaMemcpyHostToDevice, stream);
      gbr_status st = e == cudaSuccess ? enqueue_step(stream, mode) : cuda_fail(e, "graph camera copy");
      cudaError_t e2 = cudaStreamEndCapture(stream, &g);
      if (st != GBR_OK) return st;
      GBR_CUDA(e2, "graph capture");
      e = cudaGraphInstantiate(&graph_exec_[gi], g, 0);
      cudaGraphDestroy(g);
      GBR_CUDA(e, "graph instantiate");
      graph_built_[gi] = true;
      graph_stream_[gi] = stream;
    }
    GBR_CUDA(cudaGraphLaunch(graph_exec_[gi], stream), "graph launch");
  } else {
    GBR_CUDA(cudaMemcpyAsync(d_cameras_.ptr, h_stage_[slot_].ptr, cam_bytes,
                             cudaMemcpyHostToDevice, stream),
             "camera upload");
    if (gbr_status s = enqueue_step(stream, mode)) return s;
  }
  GBR_CUDA(cudaEventRecord(upload_done_[slot_], stream), "event record");
  upload_pending_[slot_] = true;
  last_stream_ = stream;
  front_ = set;
  last_stats_.scenes = S;
  last_stats_.draws = total_draws_;
  last_stats_.kernel_launches = launches_;
  timed_ = timing_ && mode == GBR_DRAW_BATCHED;
  return GBR_OK;
}

gbr_status Renderer::sync_and_check() {
  cudaSetDevice(device_);
  GBR_CUDA(cudaStreamSynchronize(last_stream_), "synchronise");
  if (d_status_.ptr) {
    uint32_t status = 0;
    GBR_CUDA(cudaMemcpy(&status, d_status_.ptr, 4, cudaMemcpyDeviceToHost), "status read");
    if (status) {
      // The host's scene records are authoritative: upload them again at the
      // next draw, so that a record damaged on the device does not persist.
      cudaMemset(d_status_.ptr, 0, 4);
      structure_dirty_ = true;
      return fail(GBR_ERROR_DEVICE, "draw: the device reported bad scene data (status " +
                                        std::to_string(status) +
                                        ((status & kStatusBadNode) ? ": a node's parent is out of range" : "") +
                                        ((status & kStatusHierarchyTooDeep) ? ": a hierarchy deeper than 64 or a cycle" : "") +
                                        "); the scene records are uploaded again at the next draw");
    }
  }
  return GBR_OK;
}

void* Renderer::plane_ptr(uint32_t plane, size_t* elem) const {
  const int slot = plane_slot(plane);
  if (slot < 0 || !(cfg_.planes & plane)) return nullptr;
  *elem = plane_elem(plane);
  return d_planes_[front_][slot].ptr;
}

gbr_status Renderer::image_into_async(uint32_t plane, const int32_t* rect, void* dst,
                                      uint64_t row_bytes) {
  TraceRange trace_("gbr.image_into");
  size_t elem;
  const char* src = static_cast<const char*>(plane_ptr(plane, &elem));
  if (!src) return fail(GBR_ERROR_INVALID_ARGUMENT, "imageIntoAsync: plane not enabled");
  if (!(rect[0] >= 0 && rect[1] >= 0 && rect[2] <= fb_w_ && rect[3] <= fb_h_ && rect[0] <= rect[2] &&
        rect[1] <= rect[3]))
    return fail(GBR_ERROR_INVALID_ARGUMENT, "imageIntoAsync: rectangle doesn't fit in the framebuffer");
  const size_t w = size_t(rect[2] - rect[0]), h = size_t(rect[3] - rect[1]);
  if (row_bytes < w * elem)
    return fail(GBR_ERROR_INVALID_ARGUMENT, "imageIntoAsync: row pitch too small");
  cudaSetDevice(device_);
  if (!copy_stream_) {
    GBR_CUDA(cudaStreamCreateWithFlags(&copy_stream_, cudaStreamNonBlocking), "copy stream");
    for (auto& e : copy_done_)
      GBR_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "copy event");
  }
  if (upload_pending_[slot_])
    GBR_CUDA(cudaStreamWaitEvent(copy_stream_, upload_done_[slot_], 0), "wait for draw");
  if (w && h)
    GBR_CUDA(cudaMemcpy2DAsync(dst, row_bytes, src + (size_t(rect[1]) * fb_w_ + rect[0]) * elem,
                               size_t(fb_w_) * elem, w * elem, h, cudaMemcpyDefault,
                               copy_stream_),
             "imageIntoAsync copy");
  GBR_CUDA(cudaEventRecord(copy_done_[front_], copy_stream_), "copy event");
  copy_pending_[front_] = true;
  return GBR_OK;
}

// Hbao::drawEffect, classic (src/esp/gfx_batch/Hbao.cpp:874-935), over all
// enabled scenes at once (three launches, csrc/hbao.cu).
gbr_status Renderer::hbao(const gbr_hbao_config& c, cudaStream_t stream) {
  TraceRange trace_("gbr.hbao");
  if (!(cfg_.planes & GBR_PLANE_COLOR) || !(cfg_.planes & GBR_PLANE_LINEAR_DEPTH))
    return fail(GBR_ERROR_STATE, "Hbao: the renderer needs its colour and linear-depth planes");
  HbaoParams params;
  std::string err;
  if (!hbao_params(c, params, err)) return fail(GBR_ERROR_INVALID_ARGUMENT, err);
  std::vector<HbaoScene> recs;
  long long blocks = 0;  // one per 256 pixels of each scene
  for (const SceneState& sc : scenes_) {
    if (!sc.enabled || sc.width <= 0 || sc.height <= 0) continue;
    recs.push_back(hbao_scene(sc.proj, sc.width, sc.height, sc.fb_offset, sc.pitch, c.radius));
    recs.back().block0 = int(blocks);
    blocks += (static_cast<long long>(sc.width) * sc.height + 255) / 256;
  }
  if (blocks > 0x7fffffffLL) return fail(GBR_ERROR_INVALID_ARGUMENT, "Hbao: too many pixels in one call");
  if (recs.empty()) return GBR_OK;
  cudaSetDevice(device_);
  const size_t fb = size_t(fb_w_) * size_t(fb_h_) * size_t(hbao_plane_bytes(params));
  if (!d_hbao_scenes_.reserve(recs.size() * sizeof(HbaoScene), false) || !d_hbao_ao_.reserve(2 * fb, false))
    return fail(GBR_ERROR_OUT_OF_MEMORY, "Hbao: device allocation failed");
  if (upload_pending_[slot_])  // after the last draw, whatever stream it ran on
    GBR_CUDA(cudaStreamWaitEvent(stream, upload_done_[slot_], 0), "Hbao: wait for draw");
  GBR_CUDA(cudaMemcpyAsync(d_hbao_scenes_.ptr, recs.data(), recs.size() * sizeof(HbaoScene),
                           cudaMemcpyHostToDevice, stream),
           "Hbao: records");
  size_t elem;
  uint32_t* color = static_cast<uint32_t*>(plane_ptr(GBR_PLANE_COLOR, &elem));
  const float* depth = static_cast<const float*>(plane_ptr(GBR_PLANE_LINEAR_DEPTH, &elem));
  uint8_t* q = static_cast<uint8_t*>(d_hbao_ao_.ptr);
  GBR_CUDA(hbao_launch(d_hbao_scenes_.as<HbaoScene>(), int(recs.size()), int(blocks), depth, color, q, q + fb,
                       params, stream),
           "Hbao launch");
  // Readbacks of this draw now follow the effect.
  GBR_CUDA(cudaEventRecord(upload_done_[slot_], stream), "Hbao: event");
  upload_pending_[slot_] = true;
  last_stream_ = stream;
  return GBR_OK;
}

gbr_status Renderer::scenes_into_async(uint32_t plane, uint32_t first, uint32_t count, void* dst) {
  TraceRange trace_("gbr.scenes_into");
  size_t elem;
  const char* src = static_cast<const char*>(plane_ptr(plane, &elem));
  if (!src) return fail(GBR_ERROR_INVALID_ARGUMENT, "scenesIntoAsync: plane not enabled");
  if (uint64_t(first) + count > scenes_.size())
    return fail(GBR_ERROR_INVALID_ARGUMENT, "scenesIntoAsync: scene range out of bounds");
  if (count == 0) return GBR_OK;
  const SceneState& s0 = scenes_[first];
  for (uint32_t i = first; i < first + count; ++i)
    if (scenes_[i].width != s0.width || scenes_[i].height != s0.height)
      return fail(GBR_ERROR_INVALID_ARGUMENT, "scenesIntoAsync: the scenes differ in size");
  const size_t bytes = size_t(count) * size_t(s0.width) * size_t(s0.height) * elem;
  cudaSetDevice(device_);
  if (!copy_stream_) {
    GBR_CUDA(cudaStreamCreateWithFlags(&copy_stream_, cudaStreamNonBlocking), "copy stream");
    for (auto& e : copy_done_)
      GBR_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "copy event");
  }
  if (upload_pending_[slot_])
    GBR_CUDA(cudaStreamWaitEvent(copy_stream_, upload_done_[slot_], 0), "wait for draw");
  if (ragged_) {  // scenes are consecutive blocks: one copy
    GBR_CUDA(cudaMemcpyAsync(dst, src + size_t(s0.fb_offset) * elem, bytes, cudaMemcpyDefault, copy_stream_),
             "scenesIntoAsync copy");
  } else {
    cudaPointerAttributes attr{};
    const bool device_dst = cudaPointerGetAttributes(&attr, dst) == cudaSuccess &&
                            attr.type == cudaMemoryTypeDevice && attr.device == device_;
    cudaGetLastError();  // a host pointer is not an error
    void* packed = dst;
    if (!device_dst) {
      if (!d_gather_.reserve(bytes, false)) return fail(GBR_ERROR_OUT_OF_MEMORY, "scenesIntoAsync: staging");
      packed = d_gather_.ptr;
    }
    GBR_CUDA(launch_gather_tiles(src, fb_w_, cfg_.tile_size[0], cfg_.tile_size[1], cfg_.tile_count[0], first,
                                 count, packed, copy_stream_),
             "scenesIntoAsync gather");
    if (!device_dst)
      GBR_CUDA(cudaMemcpyAsync(dst, packed, bytes, cudaMemcpyDeviceToHost, copy_stream_), "scenesIntoAsync copy");
  }
  GBR_CUDA(cudaEventRecord(copy_done_[front_], copy_stream_), "copy event");
  copy_pending_[front_] = true;
  return GBR_OK;
}

gbr_status Renderer::readback_wait() {
  TraceRange trace_("gbr.readback_wait");
  if (!copy_stream_) return GBR_OK;
  cudaSetDevice(device_);
  GBR_CUDA(cudaStreamSynchronize(copy_stream_), "readback wait");
  return GBR_OK;
}

gbr_status Renderer::image_into(uint32_t plane, const int32_t* rect, void* dst, uint64_t row_bytes) {
  size_t elem;
  const char* src = static_cast<const char*>(plane_ptr(plane, &elem));
  if (!src) return fail(GBR_ERROR_INVALID_ARGUMENT, "imageInto: plane not enabled");
  if (!(rect[0] >= 0 && rect[1] >= 0 && rect[2] <= fb_w_ && rect[3] <= fb_h_ && rect[0] <= rect[2] &&
        rect[1] <= rect[3]))
    return fail(GBR_ERROR_INVALID_ARGUMENT, "imageInto: rectangle doesn't fit in the framebuffer");
  const size_t w = size_t(rect[2] - rect[0]), h = size_t(rect[3] - rect[1]);
  if (row_bytes < w * elem) return fail(GBR_ERROR_INVALID_ARGUMENT, "imageInto: row pitch too small");
  if (gbr_status s = sync_and_check()) return s;
  if (!w || !h) return GBR_OK;
  GBR_CUDA(cudaMemcpy2D(dst, row_bytes, src + (size_t(rect[1]) * fb_w_ + rect[0]) * elem,
                        size_t(fb_w_) * elem, w * elem, h, cudaMemcpyDefault),
           "imageInto copy");
  return GBR_OK;
}

gbr_status Renderer::scene_image_into(uint32_t plane, uint32_t scene, void* dst, uint64_t row_bytes) {
  if (gbr_status s = check_scene(scene, "sceneImageInto()")) return s;
  size_t elem;
  const char* src = static_cast<const char*>(plane_ptr(plane, &elem));
  if (!src) return fail(GBR_ERROR_INVALID_ARGUMENT, "sceneImageInto: plane not enabled");
  const SceneState& sc = scenes_[scene];
  if (row_bytes < size_t(sc.width) * elem)
    return fail(GBR_ERROR_INVALID_ARGUMENT, "sceneImageInto: row pitch too small");
  if (gbr_status s = sync_and_check()) return s;
  GBR_CUDA(cudaMemcpy2D(dst, row_bytes, src + size_t(sc.fb_offset) * elem, size_t(sc.pitch) * elem,
                        size_t(sc.width) * elem, size_t(sc.height), cudaMemcpyDefault),
           "sceneImageInto copy");
  return GBR_OK;
}

gbr_status Renderer::plane_pointer(uint32_t plane, void** out, uint64_t* bytes) {
  size_t elem;
  void* p = plane_ptr(plane, &elem);
  if (!p) return fail(GBR_ERROR_INVALID_ARGUMENT, "planeDevicePointer: plane not enabled");
  *out = p;
  if (bytes) *bytes = uint64_t(fb_px_) * elem;
  return GBR_OK;
}

// ------------------------------------------------------------- DLPack
namespace {
struct DLDevice_ {
  int32_t device_type;
  int32_t device_id;
};
struct DLDataType_ {
  uint8_t code;
  uint8_t bits;
  uint16_t lanes;
};
struct DLTensor_ {
  void* data;
  DLDevice_ device;
  int32_t ndim;
  DLDataType_ dtype;
  int64_t* shape;
  int64_t* strides;
  uint64_t byte_offset;
};
struct DLManagedTensor_ {
  DLTensor_ dl_tensor;
  void* manager_ctx;
  void (*deleter)(DLManagedTensor_*);
};
struct DLHolder {
  DLManagedTensor_ t;
  int64_t shape[3];
  Renderer* owner;
};
void dl_deleter(DLManagedTensor_* t) {
  DLHolder* h = static_cast<DLHolder*>(t->manager_ctx);
  h->owner->release();
  delete h;
}
}  // namespace

gbr_status Renderer::plane_dlpack(uint32_t plane, void** out) {
  size_t elem;
  void* p = plane_ptr(plane, &elem);
  if (!p) return fail(GBR_ERROR_INVALID_ARGUMENT, "planeDlpack: plane not enabled");
  DLHolder* h = new DLHolder();
  h->owner = this;
  retain();
  h->t.manager_ctx = h;
  h->t.deleter = dl_deleter;
  DLTensor_& t = h->t.dl_tensor;
  t.data = p;
  t.device = {2 /* kDLCUDA */, device_};
  t.byte_offset = 0;
  t.strides = nullptr;
  int nd = 0;
  if (ragged_) {
    h->shape[nd++] = fb_px_;
  } else {
    h->shape[nd++] = fb_h_;
    h->shape[nd++] = fb_w_;
  }
  if (plane == GBR_PLANE_COLOR) {
    h->shape[nd++] = 4;
    t.dtype = {1 /* uint */, 8, 1};
  } else if (plane == GBR_PLANE_SEMANTIC) {
    t.dtype = {1, 32, 1};
  } else {
    t.dtype = {2 /* float */, 32, 1};
  }
  t.ndim = nd;
  t.shape = h->shape;
  *out = &h->t;
  return GBR_OK;
}

gbr_status Renderer::set_kernel_timing(bool on) {
  cudaSetDevice(device_);
  for (auto& e : ev_)
    if (!e) GBR_CUDA(cudaEventCreate(&e), "timing events");
  if (on != timing_) graph_valid_ = false;
  timing_ = on;
  return GBR_OK;
}

gbr_status Renderer::get_tuning(gbr_tuning* t) const {
  *t = tuning_;
  return GBR_OK;
}

gbr_status Renderer::set_tuning(const gbr_tuning& t) {
  if ((t.threads != 256 && t.threads != 512 && t.threads != 1024) || t.region_width < 4 ||
      t.region_height < 1 || t.region_width > 1024 || t.region_height > 1024 ||
      t.region_width * t.region_height > 32768 || t.small_area < 1 || t.ctas_per_sm < 1 ||
      t.plain_region_width < 4 || t.plain_region_height < 1 || t.plain_region_width > 1024 ||
      t.plain_region_height > 1024 || t.plain_region_width * t.plain_region_height > 32768 ||
      t.occlusion_culling < 0 || t.occlusion_culling > 1 || t.queue_fill_percent < 25 ||
      t.queue_fill_percent > 100)
    return fail(GBR_ERROR_INVALID_ARGUMENT, "setTuning: out of range");
  tuning_ = t;
  raster_configured_ = false;
  structure_dirty_ = true;  // regions change
  return GBR_OK;
}

gbr_status Renderer::last_stats(gbr_draw_stats* out) {
  if (gbr_status s = sync_and_check()) return s;
  const uint32_t S = uint32_t(scenes_.size());
  std::vector<uint32_t> cnt(S), tris(S);
  if (S && d_vis_count_.ptr) {
    GBR_CUDA(cudaMemcpy(cnt.data(), d_vis_count_.ptr, S * 4, cudaMemcpyDeviceToHost), "stats");
    GBR_CUDA(cudaMemcpy(tris.data(), d_vis_tris_.ptr, S * 4, cudaMemcpyDeviceToHost), "stats");
  }
  last_stats_.prepare_ms = last_stats_.raster_ms = -1.0f;
  if (timed_) {
    GBR_CUDA(cudaEventElapsedTime(&last_stats_.prepare_ms, ev_[0], ev_[1]), "timing");
    GBR_CUDA(cudaEventElapsedTime(&last_stats_.raster_ms, ev_[1], ev_[2]), "timing");
  }
  last_stats_.visible_draws = std::accumulate(cnt.begin(), cnt.end(), uint64_t(0));
  last_stats_.triangles = std::accumulate(tris.begin(), tris.end(), uint64_t(0));
  *out = last_stats_;
  return GBR_OK;
}

}  // namespace gbr
