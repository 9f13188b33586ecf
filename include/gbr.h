/* gbr.h -- C ABI of the GB300 batch renderer.
 *
 * A drop-in for the draw path of habitat-sim's esp::gfx_batch::Renderer /
 * RendererStandalone (src/esp/gfx_batch/Renderer.h:437-743,
 * src/esp/gfx_batch/RendererStandalone.h:120-241).  The reference has no C
 * ABI; each entry point below names the C++ member it replaces.  Plain
 * pointers and sizes only: no CUDA, torch or STL types cross the boundary.
 *
 * Conventions
 *  - Every call returns gbr_status; on failure gbr_last_error() holds a
 *    message for the calling thread (the reference asserts or returns false
 *    with a message: Renderer.cpp:405-427, 883-895).
 *  - Matrices are 4x4 float, column-major (m[col*4 + row]), as Magnum's
 *    Matrix4.
 *  - Images have row 0 at the bottom (GL window origin), as the reference's
 *    colorImage()/depthImage().
 *  - One renderer per host thread; gbr_draw is asynchronous on the given
 *    CUDA stream, the *_image_into readbacks synchronise that stream.
 */
#ifndef GBR_H
#define GBR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gbr_status {
  GBR_OK = 0,
  GBR_ERROR_INVALID_ARGUMENT = 1, /* out-of-range scene/node id, bad size  */
  GBR_ERROR_NOT_FOUND = 2,        /* unknown hierarchy name                */
  GBR_ERROR_IO = 3,               /* file cannot be opened or parsed       */
  GBR_ERROR_CUDA = 4,             /* a CUDA runtime call failed            */
  GBR_ERROR_OUT_OF_MEMORY = 5,    /* device or host allocation failed      */
  GBR_ERROR_DEVICE = 6,           /* a kernel reported a bad input         */
  GBR_ERROR_STATE = 7             /* call not valid in the current state   */
} gbr_status;

typedef struct gbr_renderer gbr_renderer;

/* RendererFlag (Renderer.h:20-30). */
#define GBR_FLAG_NO_TEXTURES 1u
/* RendererFileFlag (Renderer.h:120-154). */
#define GBR_FILE_WHOLE 1u
#define GBR_FILE_GENERATE_MIPMAP 2u
/* RendererStandaloneFlag::QuietLog (RendererStandalone.h:21-36). */
#define GBR_STANDALONE_QUIET_LOG 1u
/* Two sets of output planes: each draw renders into the set the previous
 * draw did not, so an asynchronous readback of one draw
 * (gbr_image_into_async) overlaps the next draw.  Plane pointers and DLPack
 * views refer to the set of the last draw at the time of the call. */
#define GBR_STANDALONE_DOUBLE_BUFFER 2u

/* Output planes of the framebuffer. */
#define GBR_PLANE_COLOR 1u        /* RGBA8, background (31,31,31,255)       */
#define GBR_PLANE_DEPTH 2u        /* window depth [0,1], D32F, cleared 1.0  */
#define GBR_PLANE_LINEAR_DEPTH 4u /* metres along -z_eye, background 0      */
#define GBR_PLANE_SEMANTIC 8u     /* uint32 object id, background 0         */
#define GBR_PLANE_ALL 15u

/* Draw modes for gbr_draw_mode. */
#define GBR_DRAW_PER_SCENE 0u /* one prepare + one raster launch per scene */
#define GBR_DRAW_BATCHED 1u   /* one prepare + one persistent raster launch */

/* RendererConfiguration (Renderer.h:45-113) + RendererStandaloneConfiguration
 * (RendererStandalone.h:47-100, setCudaDevice at :67), plus the per-scene viewport extension. */
typedef struct gbr_config {
  uint32_t flags;            /* GBR_FLAG_*                                  */
  int32_t tile_size[2];      /* default {128,128}                           */
  int32_t tile_count[2];     /* default {1,1}                               */
  uint32_t max_light_count;  /* lights used per scene; 0 = every material
                                flat (Renderer.cpp:579-620)                 */
  float ambient_factor;      /* default 0.1, used by lit materials only     */
  int32_t cuda_device;       /* default 0                                   */
  uint32_t standalone_flags; /* GBR_STANDALONE_*                            */
  uint32_t planes;           /* GBR_PLANE_* mask, default GBR_PLANE_ALL     */
  uint32_t draw_mode;        /* GBR_DRAW_*, default GBR_DRAW_PER_SCENE      */
  /* Ragged layout: if scene_count > 0, scene i renders viewports[2i] x
   * viewports[2i+1] pixels into its own contiguous block (row pitch = width)
   * instead of a tile of the tile_size x tile_count grid. */
  uint32_t scene_count;
  const int32_t* viewports;
} gbr_config;

/* Fills *config with the reference defaults. */
void gbr_config_init(gbr_config* config);

/* RendererStandalone::RendererStandalone (RendererStandalone.cpp:115-135). */
gbr_status gbr_create(const gbr_config* config, gbr_renderer** out);
/* RendererStandalone::~RendererStandalone. */
void gbr_destroy(gbr_renderer* renderer);
/* Message of the last failed call on this thread ("" if none). */
const char* gbr_last_error(void);

/* Renderer::tileSize / tileCount / sceneCount (Renderer.cpp:321-331). */
gbr_status gbr_tile_size_count(gbr_renderer* r, int32_t tile_size[2], int32_t tile_count[2]);
gbr_status gbr_scene_count(gbr_renderer* r, uint32_t* count);
/* Framebuffer geometry: for the tile grid {width, height} of the whole image;
 * for the ragged layout {total pixels, 1}. */
gbr_status gbr_framebuffer_size(gbr_renderer* r, int64_t size[2]);
/* Scene rectangle inside its plane: {pixel offset of (0,0), row pitch, width, height}. */
gbr_status gbr_scene_viewport(gbr_renderer* r, uint32_t scene, int64_t out[4]);

/* Renderer::addFile (Renderer.cpp:337-867): glTF 2.0 (.gltf/.glb) with the
 * MAGNUMX_mesh_views extras, KHR_texture_ktx (KTX2 RGB8/RGBA8/BC1),
 * KHR_texture_transform, KHR_materials_unlit, PNG images.  name may be NULL. */
gbr_status gbr_add_file(gbr_renderer* r, const char* filename, uint32_t file_flags,
                        const char* name);

/* Procedural resources: the pieces addFile creates from a file, for callers
 * that generate geometry (no reference counterpart; they mirror the imported
 * MeshData / TextureData / MaterialData of Renderer.cpp:410-633). */
typedef struct gbr_mesh_data {
  uint32_t vertex_count;
  const float* positions;     /* 3 per vertex                               */
  const float* colors;        /* 4 per vertex (RGBA in [0,1]) or NULL       */
  const float* texcoords;     /* 2 per vertex (Y-up texture space) or NULL  */
  const uint32_t* object_ids; /* 1 per vertex or NULL                       */
  uint32_t index_count;
  const uint32_t* indices;    /* triangle list                              */
  const float* normals;       /* 3 per vertex or NULL (kept only when
                                 max_light_count > 0)                       */
} gbr_mesh_data;
gbr_status gbr_add_mesh(gbr_renderer* r, const gbr_mesh_data* mesh, uint32_t* out_mesh_id);

typedef struct gbr_texture_data {
  int32_t width, height, layers;
  const uint8_t* rgba8;       /* RGBA8, row 0 bottom: level 0 of every layer,
                                 then level 1 of every layer, ...            */
  int32_t filter;             /* magnification: 0 nearest, 1 bilinear       */
  int32_t wrap_s, wrap_t;     /* 0 repeat, 1 clamp to edge, 2 mirrored      */
  int32_t min_filter;         /* minification within a level: 0 = as filter,
                                 1 nearest, 2 linear                        */
  int32_t mip_filter;         /* 0 base level only, 1 nearest level,
                                 2 linear between levels                    */
  int32_t levels;             /* levels in rgba8 (0 or 1: one); level k is
                                 max(1, w >> k) x max(1, h >> k)            */
  int32_t generate_mipmap;    /* 1 with one level: derive the chain down to
                                 min(w, h) = 1 (RendererFileFlag::
                                 GenerateMipmap, Renderer.cpp:445-477)       */
} gbr_texture_data;
gbr_status gbr_add_texture(gbr_renderer* r, const gbr_texture_data* texture,
                           uint32_t* out_texture_id);

typedef struct gbr_material_data {
  float color[4];             /* flat base colour                           */
  uint32_t texture;           /* texture id, 0 = the reserved white texel   */
  uint32_t layer;             /* array layer                                */
  float matrix[9];            /* 3x3 texture matrix, column-major           */
  int32_t shaded;             /* 1: lit when max_light_count > 0 (ambient =
                                 colour * ambient_factor, diffuse = colour);
                                 0: flat (unlit)                            */
} gbr_material_data;
gbr_status gbr_add_material(gbr_renderer* r, const gbr_material_data* material,
                            uint32_t* out_material_id);

typedef struct gbr_mesh_view {
  uint32_t mesh;
  uint32_t index_offset;      /* in indices (the reference stores bytes)    */
  uint32_t index_count;
  uint32_t material;
  float transform[16];
} gbr_mesh_view;
/* Registers a named node-hierarchy template, as a named root node of a
 * composite file does (Renderer.cpp:750-790). */
gbr_status gbr_add_node_hierarchy_template(gbr_renderer* r, const char* name,
                                           uint32_t view_count, const gbr_mesh_view* views);

/* Renderer::hasNodeHierarchy (Renderer.cpp:869-878). */
gbr_status gbr_has_node_hierarchy(gbr_renderer* r, const char* name, int32_t* out);
/* Renderer::addNodeHierarchy (Renderer.cpp:880-961); bake may be NULL. */
gbr_status gbr_add_node_hierarchy(gbr_renderer* r, uint32_t scene, const char* name,
                                  const float bake[16], uint64_t* out_node_id);
/* Renderer::addEmptyNode (Renderer.cpp:968-988). */
gbr_status gbr_add_empty_node(gbr_renderer* r, uint32_t scene, uint64_t* out_node_id);
/* Renderer::clear (Renderer.cpp:1017-1040). */
gbr_status gbr_clear(gbr_renderer* r, uint32_t scene);
/* Semantic id of every draw added by the addNodeHierarchy call that
 * returned node (no reference counterpart: gfx_batch draws no ids; the
 * classic renderer's per-draw object id, src/esp/gfx/GenericDrawable.cpp:112). */
gbr_status gbr_set_semantic_id(gbr_renderer* r, uint32_t scene, uint64_t node, uint32_t id);

/* Renderer::updateCamera (Renderer.cpp:1077-1088). */
gbr_status gbr_update_camera(gbr_renderer* r, uint32_t scene, const float projection[16],
                             const float view[16]);
/* updateCamera for scenes first..first+count-1 in one call: projections
 * and views hold 16 floats per scene (the batched form's per-step poses). */
gbr_status gbr_update_cameras(gbr_renderer* r, uint32_t first, uint32_t count,
                              const float* projections, const float* views);
/* Renderer::camera (Renderer.cpp:1056-1064): P*V. */
gbr_status gbr_camera(gbr_renderer* r, uint32_t scene, float out[16]);
/* Renderer::cameraDepthUnprojection (Renderer.cpp:1066-1075). */
gbr_status gbr_camera_depth_unprojection(gbr_renderer* r, uint32_t scene, float out[2]);
/* Renderer::transformations (Renderer.cpp:1090-1099): a writable view of
 * the scene's local node transforms (16 floats each), valid until the next
 * add/clear on that scene.  Taking the view marks the scene's transforms
 * for upload at the next draw. */
gbr_status gbr_transformations(gbr_renderer* r, uint32_t scene, float** out, uint64_t* count);

/* RendererStandalone::draw (RendererStandalone.cpp:155-159) + Renderer::draw
 * (Renderer.cpp:1123-1354).  stream is a cudaStream_t (NULL = default). */
gbr_status gbr_draw(gbr_renderer* r, void* stream);
/* Same with an explicit GBR_DRAW_* mode; use_graph captures the batched
 * step into a CUDA graph and replays it while the scene structure and the
 * stream stay the same. */
gbr_status gbr_draw_mode(gbr_renderer* r, void* stream, uint32_t mode, int32_t use_graph);

/* Lights: Renderer::addLight / clearLights / lightColors / lightRanges
 * (Renderer.h:600-720, Renderer.cpp:990-1121).  A light takes the node's
 * translation (point) or negative backward axis (directional) every draw;
 * colour defaults to white, range to infinity.  Needs max_light_count > 0;
 * a scene uses its first max_light_count lights.  The colour (3 floats per
 * light) and range views are writable and valid until the next
 * add/clear on that scene. */
typedef enum gbr_light_type { GBR_LIGHT_DIRECTIONAL = 0, GBR_LIGHT_POINT = 1 } gbr_light_type;
gbr_status gbr_add_light(gbr_renderer* r, uint32_t scene, uint64_t node, uint32_t type,
                         uint64_t* out_light_id);
gbr_status gbr_clear_lights(gbr_renderer* r, uint32_t scene);
gbr_status gbr_light_colors(gbr_renderer* r, uint32_t scene, float** out_rgb, uint64_t* out_count);
gbr_status gbr_light_ranges(gbr_renderer* r, uint32_t scene, float** out_ranges,
                            uint64_t* out_count);

/* Serving and batching extensions (no counterpart in the reference).
 * gbr_set_scene_sources: scene first+i renders the nodes and draws of scene
 * sources[i] with its own camera and viewport (by default every scene is its
 * own source).  Cheap: re-binding takes effect at the next draw without
 * rebuilding the scene records, so a request loop can point render slots at
 * resident scenes every step. */
gbr_status gbr_set_scene_sources(gbr_renderer* r, uint32_t first, uint32_t count,
                                 const uint32_t* sources);
/* A disabled scene is not drawn (its framebuffer rectangle keeps its
 * contents); use it for scenes that only hold content for other scenes. */
gbr_status gbr_set_scene_enabled(gbr_renderer* r, uint32_t scene, int32_t enabled);
/* Release a mesh, a texture or a hierarchy template: their device ranges go
 * back to a free list reused by later adds.  A draw that still uses a
 * removed mesh or texture fails with GBR_ERROR_STATE; clear those scenes
 * first. */
gbr_status gbr_remove_mesh(gbr_renderer* r, uint32_t mesh);
gbr_status gbr_remove_texture(gbr_renderer* r, uint32_t texture);
gbr_status gbr_remove_node_hierarchy_template(gbr_renderer* r, const char* name);
/* Device bytes of live geometry, textures and chunk boxes, and the bytes
 * currently reserved for them (live + free ranges). */
gbr_status gbr_memory_usage(gbr_renderer* r, uint64_t* live_bytes, uint64_t* reserved_bytes);

/* Asynchronous readback (no counterpart in the reference): enqueue the copy
 * of rect {x0, y0, x1, y1} of a plane of the last draw into host memory on
 * the renderer's copy stream, after that draw, and return at once.  dst must
 * stay valid until gbr_readback_wait (pinned memory copies at full speed).
 * The ragged layout is one row ({total pixels, 1}). */
gbr_status gbr_image_into_async(gbr_renderer* r, uint32_t plane, const int32_t rect[4], void* dst,
                                uint64_t dst_row_bytes);
/* Wait for every readback enqueued so far (not for later draws). */
gbr_status gbr_readback_wait(gbr_renderer* r);
/* Asynchronous batched readback: scenes [first, first + count) of a plane
 * of the last draw, all of one size, packed one after another (scene after
 * scene, rows bottom-up, width elements per row) into dst -- host memory
 * (through one device-side gather and one copy) or device memory on the
 * renderer's GPU (gathered in place).  Same lifetime rule as
 * gbr_image_into_async. */
gbr_status gbr_scenes_into_async(gbr_renderer* r, uint32_t plane, uint32_t first, uint32_t count,
                                 void* dst);

/* Renderer::sceneStats (Renderer.cpp:1356-1375). */
typedef struct gbr_scene_stats_info {
  uint64_t node_count, draw_count, draw_batch_count;
} gbr_scene_stats_info;
gbr_status gbr_scene_stats(gbr_renderer* r, uint32_t scene, gbr_scene_stats_info* out);

/* RendererStandalone::colorImageInto / depthImageInto
 * (RendererStandalone.cpp:168-180, 189-202): copy rect {x0, y0, x1, y1} of a plane
 * of the tile-grid framebuffer into host memory with the given row pitch.
 * plane is one GBR_PLANE_* bit.  The ragged layout is one row of all
 * scenes' pixels ({total pixels, 1}, scene after scene); single scenes are
 * easier read with gbr_scene_image_into. */
gbr_status gbr_image_into(gbr_renderer* r, uint32_t plane, const int32_t rect[4], void* dst,
                          uint64_t dst_row_bytes);
gbr_status gbr_color_image_into(gbr_renderer* r, const int32_t rect[4], void* dst,
                                uint64_t dst_row_bytes);
gbr_status gbr_depth_image_into(gbr_renderer* r, const int32_t rect[4], void* dst,
                                uint64_t dst_row_bytes);
/* The same for the planes the reference does not have: the semantic id
 * (uint32, 0 = background) and linear depth (float metres, 0 = background). */
gbr_status gbr_semantic_image_into(gbr_renderer* r, const int32_t rect[4], void* dst,
                                   uint64_t dst_row_bytes);
gbr_status gbr_linear_depth_image_into(gbr_renderer* r, const int32_t rect[4], void* dst,
                                       uint64_t dst_row_bytes);
/* One scene's rectangle of a plane (either layout), rows bottom-up. */
gbr_status gbr_scene_image_into(gbr_renderer* r, uint32_t plane, uint32_t scene, void* dst,
                                uint64_t dst_row_bytes);

/* RendererStandalone::colorCudaBufferDevicePointer / depthCudaBufferDevicePointer
 * (RendererStandalone.cpp:205-263): the device address of a whole plane,
 * owned by the renderer, valid until it is destroyed.  Unlike the reference
 * this is the live framebuffer (no copy) and the depth call returns depth. */
gbr_status gbr_plane_device_pointer(gbr_renderer* r, uint32_t plane, void** out,
                                    uint64_t* bytes);

/* DLPack export of a plane (DLManagedTensor*, dlpack v0.x ABI): a kDLCUDA
 * tensor of shape [H, W] (tile grid) or [N] (ragged); colour as uint8
 * [H, W, 4] / [N, 4].  The tensor keeps the renderer alive. */
gbr_status gbr_plane_dlpack(gbr_renderer* r, uint32_t plane, void** out_managed_tensor);

/* unprojectDepth (src/esp/gfx_batch/DepthUnprojection.cpp:107-129) on host
 * memory, and its device counterpart on the given stream. */
gbr_status gbr_unproject_depth(const float unprojection[2], float* depth, uint64_t rows,
                               uint64_t cols, uint64_t row_stride);
gbr_status gbr_unproject_depth_device(const float unprojection[2], float* depth, uint64_t rows,
                                      uint64_t cols, uint64_t row_stride, void* stream);

/* Tuning of the raster kernel (chosen by the autotuner). */
typedef struct gbr_tuning {
  int32_t threads;        /* threads per CTA: 256, 512 or 1024              */
  int32_t region_width;   /* batched form: max pixels per CTA region, x     */
  int32_t region_height;  /* batched form: max pixels per CTA region, y     */
  int32_t small_area;     /* bounding boxes up to this many pixels are
                             rasterised by one lane, larger ones by the
                             whole warp                                    */
  int32_t ctas_per_sm;    /* persistent grid = SMs x this (capped by
                             occupancy)                                    */
  int32_t plain_region_width;  /* per-scene form: region size, so that one */
  int32_t plain_region_height; /* scene spreads over several CTAs          */
  int32_t occlusion_culling;   /* 1: skip 32-triangle chunks hidden behind
                                  the depths already written (exact: the
                                  output does not change); 0: off           */
  int32_t queue_fill_percent;  /* bin capacity in use: the CTA rasterises
                                  its shared triangle queue once it holds
                                  this share of its `threads` entries,
                                  25..100 (default 75)                      */
} gbr_tuning;
gbr_status gbr_get_tuning(gbr_renderer* r, gbr_tuning* out);
gbr_status gbr_set_tuning(gbr_renderer* r, const gbr_tuning* tuning);

/* Counters of the last draw (host-read after the stream is synchronised). */
typedef struct gbr_draw_stats {
  uint64_t scenes, draws, visible_draws, triangles; /* triangles of visible draws */
  uint64_t kernel_launches;
  float prepare_ms, raster_ms; /* CUDA-event times on the draw's stream when
                                  kernel timing is on (batched mode), else -1 */
} gbr_draw_stats;
/* Records CUDA events around the prepare and raster launches of each
 * batched draw (also inside a captured graph). */
gbr_status gbr_set_kernel_timing(gbr_renderer* r, int32_t enabled);
gbr_status gbr_last_draw_stats(gbr_renderer* r, gbr_draw_stats* out);

/* Device-memory limit of one renderer (no counterpart in the reference):
 * an add, draw or readback whose device allocation would take the
 * renderer's buffers above `bytes` fails with GBR_ERROR_OUT_OF_MEMORY and
 * leaves the renderer usable; 0 (the default) is no limit.  Lowering the
 * limit below what the renderer holds frees nothing. */
gbr_status gbr_set_device_memory_limit(gbr_renderer* r, uint64_t bytes);
/* Device bytes the renderer's buffers hold now, and the limit. */
gbr_status gbr_device_memory(gbr_renderer* r, uint64_t* held, uint64_t* limit);

/* Fault injection for tests (no counterpart in the reference): replaces, in
 * device memory only, the parent index of `node` of `scene` after the host
 * has validated and uploaded the scene's records.  The next draw's prepare
 * kernel finds the bad record and sets the device status word, and the next
 * readback or gbr_last_draw_stats returns GBR_ERROR_DEVICE; the host's
 * records are then uploaded again at the following draw.  An out-of-range
 * parent reports a bad node, a parent cycle a hierarchy deeper than 64. */
gbr_status gbr_debug_corrupt_parent(gbr_renderer* r, uint32_t scene, uint64_t node, int32_t parent);

/* Renders one triangle mesh into caller-owned device planes without
 * allocating any memory.  No counterpart in the reference: it is for callers
 * that must not call cudaMalloc -- code running inside another framework's
 * memory pool or under a strict device-memory budget, real-time loops where
 * an allocation could stall or fail, plugins whose host owns every
 * allocation.  It runs the same raster kernel as gbr_draw on one scene whose
 * mesh sits under identity transforms, with flat white material (vertex
 * colours if `colors` is not NULL) and no texture.
 *
 *  positions   device, float4 per vertex (x, y, z, object-id bits), 16-B aligned
 *  colors      device, float4 RGBA per vertex, 16-B aligned, or NULL
 *  indices     device, 3 uint32 per triangle (an index >= vertex_count makes
 *              the call render only background; the call still returns
 *              GBR_OK, since it does not wait for the GPU)
 *  triangle_count  at most 1431655765 (3 x triangle_count indices are
 *              addressed in 32 bits); more is rejected
 *  projection, view   host, column-major 4x4 (as gbr_update_camera)
 *  semantic_id id of every pixel the mesh covers, unless use_vertex_ids,
 *              then the last vertex's id from positions[].w
 *  width, height      1..4096 each; larger viewports are rejected
 *  color, depth, linear_depth, semantic   device planes of width*height
 *              elements, row pitch = width, row 0 at the bottom; any may be NULL
 *
 * Its per-call scratch is one fixed 16 KiB __device__ array in the library
 * (held by every GPU that loads it until the process exits); each call
 * rewrites what must start fresh.  All calls share that array, so calls that
 * may overlap on the GPU (different streams without ordering) race: order
 * them on one stream.  The call looks up the array's device address in the
 * current context (cudaGetSymbolAddress) whenever its stream is not
 * capturing; the first call on a device does this set-up, so it should come
 * before any stream capture, and a first call after a device reset does it
 * again.  Asynchronous on `stream`. */
gbr_status gbr_render_mesh_no_alloc(const void* positions, const void* colors,
                                    const uint32_t* indices, uint32_t vertex_count,
                                    uint32_t triangle_count, const float projection[16],
                                    const float view[16], uint32_t semantic_id,
                                    int32_t use_vertex_ids, int32_t width, int32_t height,
                                    uint32_t* color, float* depth, float* linear_depth,
                                    uint32_t* semantic, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* GBR_H */
