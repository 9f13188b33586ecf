// gbr.hpp -- C++ API of the GB300 batch renderer.
//
// The classes of habitat-sim's esp::gfx_batch draw path with the same member
// names and argument meaning, for C++ callers that switch from the reference:
//   RendererConfiguration            src/esp/gfx_batch/Renderer.h:45-113
//   Renderer                         src/esp/gfx_batch/Renderer.h:437-743
//   SceneStats                       src/esp/gfx_batch/Renderer.h:750-771
//   RendererStandaloneConfiguration  src/esp/gfx_batch/RendererStandalone.h:47-100
//   RendererStandalone               src/esp/gfx_batch/RendererStandalone.h:120-241
// Header only: every member forwards to the C ABI of gbr.h (link libgbr.so).
//
// Differences a caller sees:
//  - Magnum's math and image types are replaced by the small value types
//    below (Vector2i, Vector2, Matrix4 column-major, Range2Di, Color3,
//    MutableImageView2D, Image2D) with the same memory layout and meaning.
//  - Where the reference asserts (an out-of-range scene or node id,
//    Renderer.cpp:883-895) a member throws gbr::gfx_batch::Error carrying the
//    C ABI's status and message.  addFile() returns false and prints the
//    message, as the reference does (Renderer.cpp:405-427).
//  - draw() takes an optional cudaStream_t (as void*) and is asynchronous on
//    it; colorImage()/depthImage() and the *Into() readbacks wait for it.
//  - The CUDA device pointers are the live framebuffer planes (no copy).
#ifndef GBR_HPP
#define GBR_HPP

#include <cstddef>
#include <cstdint>
#include <cstring>
#include <iostream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "gbr.h"

namespace gbr {
namespace gfx_batch {

// ------------------------------------------------------------------ errors
class Error : public std::runtime_error {
 public:
  Error(gbr_status status, const std::string& what) : std::runtime_error(what), status_(status) {}
  gbr_status status() const { return status_; }

 private:
  gbr_status status_;
};

namespace detail {
inline void check(gbr_status s, const char* where) {
  if (s != GBR_OK) throw Error(s, std::string(where) + ": " + gbr_last_error());
}
}  // namespace detail

// ------------------------------------------------------------ value types
struct Vector2i {
  int32_t x = 0, y = 0;
  Vector2i() = default;
  Vector2i(int32_t x_, int32_t y_) : x(x_), y(y_) {}
  bool operator==(const Vector2i& o) const { return x == o.x && y == o.y; }
  bool operator!=(const Vector2i& o) const { return !(*this == o); }
};

struct Vector2 {
  float x = 0.0f, y = 0.0f;
};

struct Color3 {
  float r = 1.0f, g = 1.0f, b = 1.0f;
};

// 4x4 float matrix, column-major (data[col * 4 + row]), identity by default.
struct Matrix4 {
  float data[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  float* operator[](int col) { return data + 4 * col; }
  const float* operator[](int col) const { return data + 4 * col; }
  bool operator==(const Matrix4& o) const { return std::memcmp(data, o.data, sizeof data) == 0; }
  bool operator!=(const Matrix4& o) const { return !(*this == o); }
  static Matrix4 translation(float x, float y, float z) {
    Matrix4 m;
    m.data[12] = x;
    m.data[13] = y;
    m.data[14] = z;
    return m;
  }
  static Matrix4 scaling(float x, float y, float z) {
    Matrix4 m;
    m.data[0] = x;
    m.data[5] = y;
    m.data[10] = z;
    return m;
  }
};
static_assert(sizeof(Matrix4) == 64, "Matrix4 is 16 tightly packed floats");
static_assert(sizeof(Color3) == 12, "Color3 is 3 tightly packed floats");

// Pixel rectangle [min, max) of the framebuffer, origin bottom-left.
struct Range2Di {
  Vector2i min, max;
  Range2Di() = default;
  Range2Di(const Vector2i& lo, const Vector2i& hi) : min(lo), max(hi) {}
  Vector2i size() const { return {max.x - min.x, max.y - min.y}; }
};

enum class PixelFormat { RGBA8Unorm, Depth32F, R32F, R32UI };

inline std::size_t pixelSize(PixelFormat) { return 4; }

// Caller-owned destination of a readback: `size` pixels of `format`, rows
// bottom-up, `rowStride` bytes apart (0: tightly packed).
struct MutableImageView2D {
  PixelFormat format = PixelFormat::RGBA8Unorm;
  Vector2i size;
  void* data = nullptr;
  std::size_t rowStride = 0;
  MutableImageView2D() = default;
  MutableImageView2D(PixelFormat f, const Vector2i& s, void* d, std::size_t stride = 0)
      : format(f), size(s), data(d), rowStride(stride) {}
  std::size_t stride() const { return rowStride ? rowStride : std::size_t(size.x) * pixelSize(format); }
};

// An owned image, rows bottom-up, tightly packed.
struct Image2D {
  PixelFormat format = PixelFormat::RGBA8Unorm;
  Vector2i size;
  std::vector<unsigned char> bytes;
  // pixels<T>()[y][x] as in Magnum: row y from the bottom, column x.
  template <class T>
  const T* row(int y) const {
    return reinterpret_cast<const T*>(bytes.data() + std::size_t(y) * std::size_t(size.x) * sizeof(T));
  }
  template <class T>
  const T& pixel(int y, int x) const {
    return row<T>(y)[x];
  }
};

// A writable view of renderer-owned host memory (the reference's
// StridedArrayView1D), valid until the next add or clear on that scene.
template <class T>
class ArrayView {
 public:
  ArrayView(T* data, std::size_t size) : data_(data), size_(size) {}
  std::size_t size() const { return size_; }
  T& operator[](std::size_t i) const {
    if (i >= size_) throw Error(GBR_ERROR_INVALID_ARGUMENT, "gfx_batch view: index out of range");
    return data_[i];
  }
  T* begin() const { return data_; }
  T* end() const { return data_ + size_; }
  T* data() const { return data_; }

 private:
  T* data_;
  std::size_t size_;
};

// ------------------------------------------------------------------ flags
template <class E>
class EnumSet {
 public:
  EnumSet() = default;
  EnumSet(E e) : bits_(static_cast<uint32_t>(e)) {}
  explicit EnumSet(uint32_t bits) : bits_(bits) {}
  EnumSet operator|(EnumSet o) const { return EnumSet(bits_ | o.bits_); }
  EnumSet& operator|=(EnumSet o) {
    bits_ |= o.bits_;
    return *this;
  }
  bool operator>=(EnumSet o) const { return (bits_ & o.bits_) == o.bits_; }  // contains
  bool operator==(EnumSet o) const { return bits_ == o.bits_; }
  explicit operator uint32_t() const { return bits_; }

 private:
  uint32_t bits_ = 0;
};

// RendererFlag (Renderer.h:20-30).
enum class RendererFlag : uint32_t { NoTextures = GBR_FLAG_NO_TEXTURES };
using RendererFlags = EnumSet<RendererFlag>;
inline RendererFlags operator|(RendererFlag a, RendererFlag b) { return RendererFlags(a) | b; }

// RendererFileFlag (Renderer.h:120-154).
enum class RendererFileFlag : uint32_t {
  Whole = GBR_FILE_WHOLE,
  GenerateMipmap = GBR_FILE_GENERATE_MIPMAP
};
using RendererFileFlags = EnumSet<RendererFileFlag>;
inline RendererFileFlags operator|(RendererFileFlag a, RendererFileFlag b) {
  return RendererFileFlags(a) | b;
}

// RendererLightType (Renderer.h:170-173).
enum class RendererLightType : uint32_t {
  Directional = GBR_LIGHT_DIRECTIONAL,
  Point = GBR_LIGHT_POINT
};

// RendererStandaloneFlag (RendererStandalone.h:21-36); DoubleBuffer is an
// extension (two sets of planes, so a readback overlaps the next draw).
enum class RendererStandaloneFlag : uint32_t {
  QuietLog = GBR_STANDALONE_QUIET_LOG,
  DoubleBuffer = GBR_STANDALONE_DOUBLE_BUFFER
};
using RendererStandaloneFlags = EnumSet<RendererStandaloneFlag>;
inline RendererStandaloneFlags operator|(RendererStandaloneFlag a, RendererStandaloneFlag b) {
  return RendererStandaloneFlags(a) | b;
}

// Renderer::sceneStats (Renderer.cpp:1356-1375).
struct SceneStats {
  std::size_t nodeCount = 0;
  std::size_t drawCount = 0;
  std::size_t drawBatchCount = 0;
};

// ---------------------------------------------------------- configuration
// RendererConfiguration (Renderer.h:45-113), plus the output planes, the
// draw form and per-scene viewports of this implementation.
class RendererConfiguration {
 public:
  RendererConfiguration() { gbr_config_init(&c_); }
  RendererConfiguration& setFlags(RendererFlags flags) {
    c_.flags = uint32_t(flags);
    return *this;
  }
  RendererConfiguration& setTileSizeCount(const Vector2i& tileSize, const Vector2i& tileCount) {
    c_.tile_size[0] = tileSize.x;
    c_.tile_size[1] = tileSize.y;
    c_.tile_count[0] = tileCount.x;
    c_.tile_count[1] = tileCount.y;
    return *this;
  }
  RendererConfiguration& setMaxLightCount(uint32_t count) {
    c_.max_light_count = count;
    return *this;
  }
  RendererConfiguration& setAmbientFactor(float factor) {
    c_.ambient_factor = factor;
    return *this;
  }
  // Extensions: GBR_PLANE_* mask, GBR_DRAW_* form, and the ragged layout
  // (scene i renders viewports[i].x x viewports[i].y pixels).
  RendererConfiguration& setPlanes(uint32_t planes) {
    c_.planes = planes;
    return *this;
  }
  RendererConfiguration& setDrawMode(uint32_t mode) {
    c_.draw_mode = mode;
    return *this;
  }
  RendererConfiguration& setViewports(const std::vector<Vector2i>& viewports) {
    viewports_.clear();
    for (const Vector2i& v : viewports) {
      viewports_.push_back(v.x);
      viewports_.push_back(v.y);
    }
    return *this;
  }
  RendererFlags flags() const { return RendererFlags(c_.flags); }
  // The C ABI configuration (viewports point into this object).
  gbr_config raw() const {
    gbr_config c = c_;
    c.scene_count = uint32_t(viewports_.size() / 2);
    c.viewports = viewports_.empty() ? nullptr : viewports_.data();
    return c;
  }

 private:
  gbr_config c_;
  std::vector<int32_t> viewports_;
};

// RendererStandaloneConfiguration (RendererStandalone.h:47-100).
class RendererStandaloneConfiguration {
 public:
  RendererStandaloneConfiguration& setCudaDevice(uint32_t id) {
    device_ = id;
    return *this;
  }
  RendererStandaloneConfiguration& setFlags(RendererStandaloneFlags flags) {
    flags_ = flags;
    return *this;
  }
  uint32_t cudaDevice() const { return device_; }
  RendererStandaloneFlags flags() const { return flags_; }

 private:
  uint32_t device_ = 0;
  RendererStandaloneFlags flags_;
};

// --------------------------------------------------------------- renderer
// Renderer (Renderer.h:437-743).  Constructed through RendererStandalone,
// which owns the framebuffer planes on the GPU.
class Renderer {
 public:
  Renderer(const Renderer&) = delete;
  Renderer& operator=(const Renderer&) = delete;
  Renderer(Renderer&& o) noexcept : r_(std::exchange(o.r_, nullptr)), flags_(o.flags_) {}
  virtual ~Renderer() {
    if (r_) gbr_destroy(r_);
  }

  RendererFlags flags() const { return flags_; }
  Vector2i tileSize() const {
    int32_t s[2], c[2];
    detail::check(gbr_tile_size_count(r_, s, c), "Renderer::tileSize()");
    return {s[0], s[1]};
  }
  Vector2i tileCount() const {
    int32_t s[2], c[2];
    detail::check(gbr_tile_size_count(r_, s, c), "Renderer::tileCount()");
    return {c[0], c[1]};
  }
  std::size_t sceneCount() const {
    uint32_t n = 0;
    detail::check(gbr_scene_count(r_, &n), "Renderer::sceneCount()");
    return n;
  }
  uint32_t maxLightCount() const { return max_lights_; }

  // Renderer::addFile (Renderer.cpp:337-867): false with a message on failure.
  bool addFile(const std::string& filename, RendererFileFlags flags = {},
               const std::string& name = {}) {
    const gbr_status s =
        gbr_add_file(r_, filename.c_str(), uint32_t(flags), name.empty() ? nullptr : name.c_str());
    if (s != GBR_OK) {
      std::cerr << "Renderer::addFile(): " << gbr_last_error() << "\n";
      return false;
    }
    return true;
  }
  // The overload that names an importer plugin: glTF is the only format
  // this implementation imports, under either of the reference's names.
  bool addFile(const std::string& filename, const std::string& importerPlugin, RendererFileFlags flags,
               const std::string& name = {}) {
    if (importerPlugin != "GltfImporter" && importerPlugin != "AnySceneImporter") {
      std::cerr << "Renderer::addFile(): unsupported importer " << importerPlugin << "\n";
      return false;
    }
    return addFile(filename, flags, name);
  }

  // Renderer::hasNodeHierarchy (Renderer.cpp:869-878).
  bool hasNodeHierarchy(const std::string& name) const {
    int32_t out = 0;
    detail::check(gbr_has_node_hierarchy(r_, name.c_str(), &out), "Renderer::hasNodeHierarchy()");
    return out != 0;
  }
  // Renderer::addNodeHierarchy (Renderer.cpp:880-961): the root node's id.
  std::size_t addNodeHierarchy(uint32_t sceneId, const std::string& name,
                               const Matrix4& bakeTransformation = Matrix4{}) {
    uint64_t id = 0;
    detail::check(gbr_add_node_hierarchy(r_, sceneId, name.c_str(), bakeTransformation.data, &id),
                  "Renderer::addNodeHierarchy()");
    return std::size_t(id);
  }
  // Renderer::addEmptyNode (Renderer.cpp:968-988).
  std::size_t addEmptyNode(uint32_t sceneId) {
    uint64_t id = 0;
    detail::check(gbr_add_empty_node(r_, sceneId, &id), "Renderer::addEmptyNode()");
    return std::size_t(id);
  }
  // Renderer::addLight (Renderer.cpp:990-1015).
  std::size_t addLight(uint32_t sceneId, std::size_t nodeId, RendererLightType type) {
    uint64_t id = 0;
    detail::check(gbr_add_light(r_, sceneId, nodeId, uint32_t(type), &id), "Renderer::addLight()");
    return std::size_t(id);
  }
  // Renderer::clear / clearLights (Renderer.cpp:1017-1054).
  void clear(uint32_t sceneId) { detail::check(gbr_clear(r_, sceneId), "Renderer::clear()"); }
  void clearLights(uint32_t sceneId) {
    detail::check(gbr_clear_lights(r_, sceneId), "Renderer::clearLights()");
  }
  // Renderer::camera / cameraDepthUnprojection / updateCamera
  // (Renderer.cpp:1056-1088).
  Matrix4 camera(uint32_t sceneId) const {
    Matrix4 m;
    detail::check(gbr_camera(r_, sceneId, m.data), "Renderer::camera()");
    return m;
  }
  Vector2 cameraDepthUnprojection(uint32_t sceneId) const {
    float ab[2];
    detail::check(gbr_camera_depth_unprojection(r_, sceneId, ab), "Renderer::cameraDepthUnprojection()");
    return {ab[0], ab[1]};
  }
  void updateCamera(uint32_t sceneId, const Matrix4& projection, const Matrix4& view) {
    detail::check(gbr_update_camera(r_, sceneId, projection.data, view.data), "Renderer::updateCamera()");
  }
  // Renderer::transformations / lightColors / lightRanges
  // (Renderer.cpp:1090-1121): writable views, valid until the next add or
  // clear on the scene.
  ArrayView<Matrix4> transformations(uint32_t sceneId) {
    float* p = nullptr;
    uint64_t n = 0;
    detail::check(gbr_transformations(r_, sceneId, &p, &n), "Renderer::transformations()");
    return {reinterpret_cast<Matrix4*>(p), std::size_t(n)};
  }
  ArrayView<Color3> lightColors(uint32_t sceneId) {
    float* p = nullptr;
    uint64_t n = 0;
    detail::check(gbr_light_colors(r_, sceneId, &p, &n), "Renderer::lightColors()");
    return {reinterpret_cast<Color3*>(p), std::size_t(n)};
  }
  ArrayView<float> lightRanges(uint32_t sceneId) {
    float* p = nullptr;
    uint64_t n = 0;
    detail::check(gbr_light_ranges(r_, sceneId, &p, &n), "Renderer::lightRanges()");
    return {p, std::size_t(n)};
  }
  SceneStats sceneStats(uint32_t sceneId) const {
    gbr_scene_stats_info s{};
    detail::check(gbr_scene_stats(r_, sceneId, &s), "Renderer::sceneStats()");
    return {std::size_t(s.node_count), std::size_t(s.draw_count), std::size_t(s.draw_batch_count)};
  }

  // The C ABI handle, for the extensions of gbr.h.
  gbr_renderer* handle() const { return r_; }

 protected:
  Renderer(const RendererConfiguration& configuration,
           const RendererStandaloneConfiguration& standalone)
      : flags_(configuration.flags()) {
    gbr_config c = configuration.raw();
    c.cuda_device = int32_t(standalone.cudaDevice());
    c.standalone_flags = uint32_t(standalone.flags());
    max_lights_ = c.max_light_count;
    detail::check(gbr_create(&c, &r_), "RendererStandalone");
  }
  gbr_renderer* r_ = nullptr;

 private:
  RendererFlags flags_;
  uint32_t max_lights_ = 0;
};

// RendererStandalone (RendererStandalone.h:120-241): the renderer with its
// framebuffer planes in device memory.
class RendererStandalone : public Renderer {
 public:
  RendererStandalone(const RendererConfiguration& configuration,
                     const RendererStandaloneConfiguration& standaloneConfiguration)
      : Renderer(configuration, standaloneConfiguration), standalone_flags_(standaloneConfiguration.flags()) {}

  RendererStandaloneFlags standaloneFlags() const { return standalone_flags_; }
  PixelFormat colorFramebufferFormat() const { return PixelFormat::RGBA8Unorm; }
  PixelFormat depthFramebufferFormat() const { return PixelFormat::Depth32F; }

  // RendererStandalone::draw (RendererStandalone.cpp:155-159): clear and
  // draw every scene, asynchronously on `cudaStream` (null: default stream).
  void draw(void* cudaStream = nullptr) { detail::check(gbr_draw(r_, cudaStream), "RendererStandalone::draw()"); }

  // colorImage / colorImageInto / depthImage / depthImageInto
  // (RendererStandalone.cpp:161-202): window depth for the depth plane.
  Image2D colorImage() { return image(GBR_PLANE_COLOR, PixelFormat::RGBA8Unorm); }
  void colorImageInto(const Range2Di& rectangle, const MutableImageView2D& image) {
    into(GBR_PLANE_COLOR, rectangle, image, "RendererStandalone::colorImageInto()");
  }
  Image2D depthImage() { return image(GBR_PLANE_DEPTH, PixelFormat::Depth32F); }
  void depthImageInto(const Range2Di& rectangle, const MutableImageView2D& image) {
    into(GBR_PLANE_DEPTH, rectangle, image, "RendererStandalone::depthImageInto()");
  }
  // Extensions: linear depth in metres and the semantic-id plane.
  Image2D linearDepthImage() { return image(GBR_PLANE_LINEAR_DEPTH, PixelFormat::R32F); }
  Image2D semanticImage() { return image(GBR_PLANE_SEMANTIC, PixelFormat::R32UI); }
  void linearDepthImageInto(const Range2Di& rectangle, const MutableImageView2D& image) {
    into(GBR_PLANE_LINEAR_DEPTH, rectangle, image, "RendererStandalone::linearDepthImageInto()");
  }
  void semanticImageInto(const Range2Di& rectangle, const MutableImageView2D& image) {
    into(GBR_PLANE_SEMANTIC, rectangle, image, "RendererStandalone::semanticImageInto()");
  }
  void imageInto(uint32_t plane, const Range2Di& rectangle, const MutableImageView2D& image) {
    into(plane, rectangle, image, "RendererStandalone::imageInto()");
  }

  // colorCudaBufferDevicePointer / depthCudaBufferDevicePointer
  // (RendererStandalone.cpp:204-263): the live planes, owned by the renderer.
  const void* colorCudaBufferDevicePointer() { return plane_pointer(GBR_PLANE_COLOR); }
  const void* depthCudaBufferDevicePointer() { return plane_pointer(GBR_PLANE_DEPTH); }

 private:
  Vector2i framebuffer_size() const {
    int64_t s[2];
    detail::check(gbr_framebuffer_size(r_, s), "RendererStandalone: framebuffer size");
    return {int32_t(s[0]), int32_t(s[1])};
  }
  Image2D image(uint32_t plane, PixelFormat format) {
    Image2D img;
    img.format = format;
    img.size = framebuffer_size();
    img.bytes.resize(std::size_t(img.size.x) * std::size_t(img.size.y) * 4);
    const int32_t rect[4] = {0, 0, img.size.x, img.size.y};
    detail::check(gbr_image_into(r_, plane, rect, img.bytes.data(), uint64_t(img.size.x) * 4),
                  "RendererStandalone: image readback");
    return img;
  }
  void into(uint32_t plane, const Range2Di& rectangle, const MutableImageView2D& image, const char* where) {
    if (!(image.size == rectangle.size()))
      throw Error(GBR_ERROR_INVALID_ARGUMENT, std::string(where) + ": image size differs from the rectangle");
    const int32_t rect[4] = {rectangle.min.x, rectangle.min.y, rectangle.max.x, rectangle.max.y};
    detail::check(gbr_image_into(r_, plane, rect, image.data, uint64_t(image.stride())), where);
  }
  const void* plane_pointer(uint32_t plane) {
    void* p = nullptr;
    uint64_t bytes = 0;
    detail::check(gbr_plane_device_pointer(r_, plane, &p, &bytes), "RendererStandalone: device pointer");
    return p;
  }
  RendererStandaloneFlags standalone_flags_;
};

}  // namespace gfx_batch
}  // namespace gbr

#endif  // GBR_HPP
