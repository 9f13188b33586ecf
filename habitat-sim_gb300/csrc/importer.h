// glTF 2.0 importer for Renderer::addFile.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace gbr {

struct ImportedTexture {
  int width = 0, height = 0, layers = 1;
  std::vector<uint8_t> rgba;  // layers*height*width*4, row 0 = bottom
  int filter = 1;             // 0 nearest, 1 linear (the magnification filter)
  int wrap_s = 0, wrap_t = 0; // 0 repeat, 1 clamp, 2 mirrored repeat
  int min_filter = 1;         // minification within a level: 0 nearest, 1 linear
  int mip_filter = 2;         // 0 base level only, 1 nearest level, 2 linear
  bool compressed = false;    // decoded from a block-compressed image (no generated mips)
};

struct ImportedMesh {
  std::vector<float> positions;   // 3 per vertex
  std::vector<float> colors;      // 4 per vertex, empty if absent
  std::vector<float> texcoords;   // 2 per vertex (Y-up), empty if absent
  std::vector<uint32_t> object_ids;
  std::vector<float> normals;     // 3 per vertex, empty if absent
  std::vector<uint32_t> indices;  // triangle list
  uint32_t vertex_count = 0;
};

struct ImportedMaterial {
  float color[4] = {1, 1, 1, 1};
  int texture = -1;  // file-local texture id, -1 = none
  int layer = 0;
  float matrix[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  bool flat = false;  // KHR_materials_unlit
};

struct ImportedView {
  uint32_t mesh = 0;
  uint32_t index_offset_bytes = 0;
  uint32_t index_count = 0;
  int32_t material = -1;
  float transform[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
};

struct ImportedTemplate {
  std::string name;
  uint32_t begin = 0, end = 0;
};

struct ImportedFile {
  std::vector<ImportedTexture> textures;
  std::vector<ImportedMesh> meshes;
  std::vector<ImportedMaterial> materials;
  std::vector<ImportedView> views;
  std::vector<ImportedTemplate> templates;
};

// Imports `path`.  whole: flatten the file under one name (`name`, or the
// path when empty).  no_textures: skip image decoding but keep texture ids.
bool import_gltf(const std::string& path, bool whole, const std::string& name, bool no_textures,
                 ImportedFile& out, std::string& error);

// Decoders, exposed for tests of the importer.
bool decode_png(const uint8_t* data, size_t size, ImportedTexture& out, std::string& error);
bool decode_ktx2(const uint8_t* data, size_t size, ImportedTexture& out, std::string& error);

// Column-major 4x4 product, each entry summed left to right without fusing.
void mat4_mul(const float* a, const float* b, float* c);

}  // namespace gbr
