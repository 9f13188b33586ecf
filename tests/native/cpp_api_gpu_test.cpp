// The C++ API (include/gbr.hpp) on the GPU: the reference's singleMesh test
// (src/tests/GfxBatchRendererTest.cpp:1524-1600) written against
// gbr::gfx_batch::RendererStandalone the way a reference caller writes it
// against esp::gfx_batch::RendererStandalone.
//
//   cpp_api_gpu_test <scenes dir> <colour image out>
//
// Checks the hierarchy queries, returned node id, scene stats, the
// transformation view, the known-answer pixels and depths of the reference
// test, a colorImageInto sub-rectangle against colorImage, and the error
// paths; writes the colour image (128 x 96 RGBA8, rows bottom-up) for the
// caller to compare with the reference's golden screenshot.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gbr.hpp"

namespace gb = gbr::gfx_batch;

static int failures = 0;
#define CHECK(c)                                                             \
  do {                                                                       \
    if (!(c)) {                                                              \
      std::fprintf(stderr, "%s:%d: check failed: %s\n", __FILE__, __LINE__, #c); \
      ++failures;                                                            \
    }                                                                        \
  } while (0)

// Magnum's Matrix4::orthographicProjection(size, near, far), in float.
static gb::Matrix4 orthographic(float sx, float sy, float near, float far) {
  gb::Matrix4 m;
  m.data[0] = 2.0f / sx;
  m.data[5] = 2.0f / sy;
  const float zs = 2.0f / (near - far);
  m.data[10] = zs;
  m.data[14] = near * zs - 1.0f;
  return m;
}

int main(int argc, char** argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s <scenes dir> <colour image out>\n", argv[0]);
    return 2;
  }
  const std::string scenes = argv[1];
  try {
    gb::RendererStandalone renderer{
        gb::RendererConfiguration{}.setTileSizeCount({128, 96}, {1, 1}),
        gb::RendererStandaloneConfiguration{}.setFlags(gb::RendererStandaloneFlag::QuietLog)};
    CHECK(renderer.tileSize() == gb::Vector2i(128, 96));
    CHECK(renderer.tileCount() == gb::Vector2i(1, 1));
    CHECK(renderer.sceneCount() == 1);
    CHECK(renderer.addFile(scenes + "/batch.gltf"));
    CHECK(!renderer.addFile(scenes + "/does-not-exist.gltf"));

    // Undo the aspect ratio, move the camera back.
    renderer.updateCamera(0, orthographic(2.0f * (4.0f / 3.0f), 2.0f, 0.1f, 10.0f),
                          gb::Matrix4::translation(0.0f, 0.0f, -1.0f));
    CHECK(renderer.hasNodeHierarchy("square"));
    CHECK(!renderer.hasNodeHierarchy("squares"));
    CHECK(!renderer.hasNodeHierarchy(""));
    CHECK(renderer.addNodeHierarchy(0, "square", gb::Matrix4::scaling(0.4f, 0.4f, 0.4f)) == 0);

    const gb::SceneStats stats = renderer.sceneStats(0);
    CHECK(stats.nodeCount == 2);
    CHECK(stats.drawCount == 1);
    CHECK(stats.drawBatchCount == 1);
    CHECK(renderer.transformations(0).size() == 2);
    CHECK(renderer.transformations(0)[0] == gb::Matrix4{});
    renderer.transformations(0)[0] = gb::Matrix4::scaling(2.0f, 2.0f, 2.0f);

    renderer.draw();
    const gb::Image2D color = renderer.colorImage();
    CHECK(color.size == gb::Vector2i(128, 96));
    CHECK(color.format == gb::PixelFormat::RGBA8Unorm);
    const unsigned char* grey = reinterpret_cast<const unsigned char*>(&color.pixel<uint32_t>(75, 35));
    const unsigned char* red = reinterpret_cast<const unsigned char*>(&color.pixel<uint32_t>(20, 38));
    CHECK(grey[0] == 0xcc && grey[1] == 0xcc && grey[2] == 0xcc);
    CHECK(red[0] == 0x99 && red[1] == 0x00 && red[2] == 0x00);

    const gb::Image2D depth = renderer.depthImage();
    CHECK(depth.format == gb::PixelFormat::Depth32F);
    CHECK(depth.pixel<float>(0, 0) == 1.0f);
    CHECK(depth.pixel<float>(95, 127) == 1.0f);
    CHECK(std::fabs(depth.pixel<float>(64, 48) - 0.0909091f) < 1e-6f);

    // A sub-rectangle through colorImageInto with a padded row stride.
    const gb::Range2Di rect{{30, 10}, {70, 80}};
    const size_t stride = 40 * 4 + 16;
    std::vector<unsigned char> sub(stride * 70);
    renderer.colorImageInto(rect, gb::MutableImageView2D{gb::PixelFormat::RGBA8Unorm, rect.size(),
                                                         sub.data(), stride});
    bool same = true;
    for (int y = 0; y < 70; ++y)
      for (int x = 0; x < 40; ++x)
        same = same && std::memcmp(&sub[y * stride + x * 4], &color.pixel<uint32_t>(y + 10, x + 30), 4) == 0;
    CHECK(same);
    std::vector<float> dsub(40 * 70);
    renderer.depthImageInto(rect, gb::MutableImageView2D{gb::PixelFormat::Depth32F, rect.size(), dsub.data()});
    CHECK(dsub[(64 - 10) * 40 + (48 - 30)] == depth.pixel<float>(64, 48));
    // The extension planes' sub-rectangles against their whole images.
    const gb::Image2D ids = renderer.semanticImage();
    const gb::Image2D linear = renderer.linearDepthImage();
    std::vector<uint32_t> idsub(40 * 70);
    std::vector<float> lsub(40 * 70);
    renderer.semanticImageInto(rect, gb::MutableImageView2D{gb::PixelFormat::R32UI, rect.size(), idsub.data()});
    renderer.linearDepthImageInto(rect, gb::MutableImageView2D{gb::PixelFormat::R32F, rect.size(), lsub.data()});
    same = true;
    for (int y = 0; y < 70; ++y)
      for (int x = 0; x < 40; ++x)
        same = same && idsub[y * 40 + x] == ids.pixel<uint32_t>(y + 10, x + 30) &&
               std::memcmp(&lsub[y * 40 + x], &linear.pixel<float>(y + 10, x + 30), 4) == 0;
    CHECK(same);
    CHECK(ids.pixel<uint32_t>(0, 0) == 0 && linear.pixel<float>(0, 0) == 0.0f);
    CHECK(linear.pixel<float>(48, 64) > 0.0f);
    CHECK(renderer.colorCudaBufferDevicePointer() != nullptr);
    CHECK(renderer.depthCudaBufferDevicePointer() != nullptr);

    // Where the reference asserts, the C++ API throws with the status.
    bool threw = false;
    try {
      renderer.addNodeHierarchy(3, "square");
    } catch (const gb::Error& e) {
      threw = e.status() == GBR_ERROR_INVALID_ARGUMENT;
    }
    CHECK(threw);
    threw = false;
    try {
      renderer.addNodeHierarchy(0, "squares");
    } catch (const gb::Error& e) {
      threw = e.status() == GBR_ERROR_NOT_FOUND;
    }
    CHECK(threw);

    std::FILE* f = std::fopen(argv[2], "wb");
    CHECK(f != nullptr);
    if (f) {
      CHECK(std::fwrite(color.bytes.data(), 1, color.bytes.size(), f) == color.bytes.size());
      std::fclose(f);
    }
  } catch (const std::exception& e) {
    std::fprintf(stderr, "exception: %s\n", e.what());
    return 1;
  }
  if (failures) {
    std::fprintf(stderr, "%d failures\n", failures);
    return 1;
  }
  std::printf("ok\n");
  return 0;
}
