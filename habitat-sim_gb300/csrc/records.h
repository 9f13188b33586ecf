// Device-resident records shared by the host runtime and the kernels.
//
// HBM layout (all arrays renderer-owned, 256-byte aligned allocations):
//   geometry   pos[v]    float4 (x, y, z, object-id bits)   16 B / vertex
//              normal[v] float4 (lit renderers only)        16 B / vertex
//              color[v]  float4 RGBA                        16 B / vertex
//              uv[v]     float2                              8 B / vertex
//              index[i]  uint32                              4 B / index
//   textures   texel[t]  uint32 RGBA8, level-major then layer-major, row 0 bottom
//   tables     MeshRec, MaterialRec, TextureRec
//   scenes     SceneRec[s]; per node parent (int32) + local 4x4 (64 B);
//              DrawRec[] (64 B) in draw-batch order; CameraRec[s] (96 B) followed
//              by LightSrc[s][max lights] (24 B); WorldLight[s][max lights] (32 B)
//   per step   VisibleRec[] (128 B, written by the prepare kernel) and its
//              processing order uint2[] (8 B per visible draw); ModelRec[]
//              (96 B per visible draw, lit renderers only),
//              vis_count[s], vis_tris[s], vis_chunks[s]; WorkItem[] (capacity for
//              every scene at its finest split) + the count in use + one counter
//   views      ChunkBox[] (32 B per 32 triangles of every mesh view, then
//              32 B per 1024 triangles: the cluster boxes)
//   output     colour u32, window depth f32, linear depth f32, id u32
//              planes, one element per framebuffer pixel.
#pragma once
#include <cstddef>
#include <cstdint>

namespace gbr {

enum : uint32_t {
  kMeshVertexColor = 1u,
  kMeshObjectId = 2u,
  kMeshTexcoords = 4u,
  kMeshNormals = 8u,  // normals stored (lighting enabled)
};
// VisibleRec::flags bit: the draw's bounding box lies inside the frustum.
constexpr uint32_t kDrawInsideFrustum = 0x100u;

struct MeshRec {
  uint32_t vertex_base;
  uint32_t vertex_count;
  uint32_t index_base;
  uint32_t index_count;
  uint32_t flags;
  uint32_t pad[3];
};

struct MaterialRec {
  float color[4];
  int32_t texture;  // 0 = white
  int32_t layer;
  float m[9];       // 3x3 column-major texture matrix
  int32_t phong;    // lit: ambient = color * ambient factor, diffuse = color
};

struct TextureRec {
  uint64_t offset;     // in texels: level 0 of every layer, then level 1, ...
  int32_t width, height, layers;
  int32_t filter;      // magnification: 0 nearest, 1 linear
  int32_t wrap_s, wrap_t;
  int32_t min_filter;  // minification within a level: 0 nearest, 1 linear
  int32_t mip_filter;  // 0 base level only, 1 nearest level, 2 linear between levels
  int32_t levels;
  int32_t pad;
};
static_assert(sizeof(TextureRec) == 48, "TextureRec layout");

struct SceneRec {
  int32_t width, height;
  int64_t fb_offset;   // pixel index of (0,0) in each plane
  int64_t pitch;       // pixels per row
  uint32_t node_base, node_count;
  uint32_t draw_base, draw_count;
};

struct DrawRec {
  uint32_t node;         // scene-local node index
  uint32_t mesh;
  uint32_t first_index;  // absolute index into the index array
  uint32_t tri_count;
  uint32_t material;
  uint32_t semantic_id;
  float bbox[6];         // object-space min xyz, max xyz of the view
  uint32_t box_base;     // first chunk box of the view
  uint32_t chunk_count;  // 32-triangle chunks of the view
  uint32_t pad[2];
};

// Per-scene state uploaded every step: the camera and the scene's binding
// (which scene's nodes and draws it renders, where its visible records go,
// whether it is drawn at all).
struct CameraRec {
  float pv[16];       // projection * view
  float vrow[4];      // row 2 of the view matrix
  uint32_t source;    // scene whose nodes and draws are rendered
  uint32_t vis_base;  // first visible record of this scene
  uint32_t enabled;   // 0: not drawn, framebuffer rectangle untouched
  uint32_t light_count;  // this scene's lights in use (at most the maximum)
};
static_assert(sizeof(CameraRec) == 96, "CameraRec layout");

// A light as the host keeps it (uploaded with the camera block): node of
// the scene it follows, type (0 directional, 1 point), colour, range.
struct LightSrc {
  int32_t node;
  int32_t type;
  float color[3];
  float range;
};
static_assert(sizeof(LightSrc) == 24, "LightSrc layout");

// A light in world space, written by the prepare kernel: position (w = 1)
// or direction towards the light (w = 0), colour, range.
struct WorldLight {
  float pos[4];
  float color[3];
  float range;
};

// Per visible draw of a lit renderer: the draw's absolute transform (rows
// 0-2 of columns 0-3) and its normal matrix (cofactor of the upper-left
// 3x3, column-major).
struct ModelRec {
  float a[12];   // a[col * 3 + row]
  float nm[9];   // nm[col * 3 + row]
  float pad[3];
};
static_assert(sizeof(ModelRec) == 96, "ModelRec layout");

// 16-byte aligned: the raster kernel reads the matrix with float4 loads.
struct alignas(16) VisibleRec {
  float mvp[16];
  float zrow[4];       // row 2 of view * model
  uint32_t vertex_base;
  uint32_t first_index;
  uint32_t tri_count;
  uint32_t material;
  uint32_t semantic_id;
  uint32_t ordinal;    // index of this draw's first triangle in the scene
  uint32_t flags;      // mesh flags
  uint32_t cluster;    // index of this draw's first cluster in the scene (draw order)
  uint32_t box_base;   // first chunk box of the draw's view; its cluster boxes follow
  uint32_t chunk_count;
  uint32_t pad[2];
};
static_assert(sizeof(VisibleRec) == 128, "VisibleRec layout");
// The raster kernel loads the record as 16-byte vectors by these offsets.
static_assert(offsetof(VisibleRec, zrow) == 64 && offsetof(VisibleRec, vertex_base) == 80 &&
                  offsetof(VisibleRec, semantic_id) == 96 && offsetof(VisibleRec, flags) == 104,
              "VisibleRec vector layout");

// Triangles per chunk: the unit of work a warp takes and of bounding-box culling.
constexpr uint32_t kChunkTris = 32;
// Chunks per cluster: the coarser culling level.  A mesh view's boxes are
// its chunk_count chunk boxes followed by ceil(chunk_count / 32) cluster boxes.
constexpr uint32_t kClusterChunks = 32;
__host__ __device__ inline uint32_t cluster_count(uint32_t chunks) {
  return (chunks + kClusterChunks - 1) / kClusterChunks;
}

// Object-space bounding box of one chunk of a mesh view.
struct ChunkBox {
  float lo[4];
  float hi[4];
};


struct WorkItem {
  uint32_t scene;
  uint16_t x0, y0, w, h;   // region of the scene's viewport
};

// Device status bits (atomicOr into one word).
enum : uint32_t {
  kStatusHierarchyTooDeep = 1u,
  kStatusBadNode = 2u,
};

}  // namespace gbr
