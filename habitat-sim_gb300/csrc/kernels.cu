// sm_103a kernels of the batch renderer.
//
// Replaces the GPU half of esp::gfx_batch::Renderer::draw
// (src/esp/gfx_batch/Renderer.cpp:1203-1351): the per-frame transform
// hierarchy and per-draw uniforms (:1203-1290) become prepare_kernel; the
// per-tile multi-draw through PhongGL and the GL fixed-function pipeline
// (:1292-1351) become raster_kernel.
//
// Arithmetic: this translation unit is compiled with --fmad=false, so no
// multiply-add is fused unless written as __fmaf_rn.  Every operation that
// decides a pixel (transform, clip, snap, edge functions, depth, barycentric
// interpolation, texel fetch, unorm conversion) is written out in a fixed
// order so that the results are reproducible bit for bit on any IEEE-754
// machine that evaluates the same sequence.
//
// Rasterisation method (GL leaves the exact rules to the implementation):
//   - clip-space trivial reject; homogeneous clipping only for triangles
//     that cross the near plane z = -w or a guard band |x|,|y| <= G*w
//     (Sutherland & Hodgman 1974), fan re-triangulation;
//   - window coordinates snapped to 1/256 pixel, round half to even;
//   - integer edge functions (Pineda 1988) in 64-bit with the top-left
//     fill rule, pixel centres at (x+0.5, y+0.5), origin bottom-left;
//   - depth interpolated linearly in window space, LESS semantics realised
//     as an atomic minimum of (depth bits << 32 | triangle ordinal) in a
//     shared-memory z-buffer: the smallest depth wins, ties go to the
//     earliest submitted triangle, as with a sequential GL depth test;
//   - deferred shading of the winner only, with homogeneous barycentrics of
//     the unclipped triangle (Olano & Greer 1997).
#include <cuda_runtime.h>

#include <algorithm>

#include <cstdint>

#include "kernels.h"

namespace gbr {
namespace {

constexpr uint64_t kEmptyKey = ~0ull;
constexpr uint32_t kBackground = 0xFF1F1F1Fu;
constexpr int kMaxHierarchyDepth = 64;
// Capacity of the raster kernel's ring of chunks that passed culling: a
// power of two >= 31 + the CTA size (a cull pass starts with fewer than 32
// chunks waiting and adds at most one per thread).
__host__ __device__ constexpr uint32_t ring_capacity(int threads) {
  return threads > 512 ? 2048u : (threads > 256 ? 1024u : 512u);
}
// Capacity of the ring of clusters that passed culling (a power of two); a
// cluster pass tests at most as many clusters as there is room for.
constexpr uint32_t kClusterRing = 256;

__device__ __forceinline__ float fma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// C = A * B, column-major 4x4.
__device__ __forceinline__ void matmul(const float* a, const float* b, float* c) {
#pragma unroll
  for (int col = 0; col < 4; ++col) {
#pragma unroll
    for (int row = 0; row < 4; ++row) {
      float t = __fmul_rn(a[row], b[col * 4 + 0]);
      t = fma_(a[4 + row], b[col * 4 + 1], t);
      t = fma_(a[8 + row], b[col * 4 + 2], t);
      t = fma_(a[12 + row], b[col * 4 + 3], t);
      c[col * 4 + row] = t;
    }
  }
}

__device__ __forceinline__ float mrow(const float* m, int row, float x, float y, float z) {
  float r = m[12 + row];
  r = fma_(m[row], x, r);
  r = fma_(m[4 + row], y, r);
  r = fma_(m[8 + row], z, r);
  return r;
}

// ------------------------------------------------------------ block scan
template <int T>
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* s_warp,
                                                         uint32_t* s_total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t n = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += n;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    constexpr int kWarps = T / 32;
    uint32_t w = lane < kWarps ? s_warp[lane] : 0u;
    uint32_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t n = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += n;
    }
    if (lane < kWarps) s_warp[lane] = wi - w;
    if (lane == kWarps - 1) *s_total = wi;
  }
  __syncthreads();
  uint32_t out = s_warp[warp] + incl - v;
  __syncthreads();
  return out;
}

// Clip-plane outcode of an object-space point, with a relative margin: a
// bit is set only when the point is beyond that plane by more than rounding
// could move it, so every culling decision built on it is conservative.
__device__ __forceinline__ uint32_t outcode(const float* mvp, float x, float y, float z) {
  const float cx = mrow(mvp, 0, x, y, z), cy = mrow(mvp, 1, x, y, z), cz = mrow(mvp, 2, x, y, z),
              cw = mrow(mvp, 3, x, y, z);
  const float ax = 1e-5f * (fabsf(cx) + fabsf(cw)), ay = 1e-5f * (fabsf(cy) + fabsf(cw)),
              az = 1e-5f * (fabsf(cz) + fabsf(cw));
  uint32_t out = 0;
  out |= (cx - cw > ax) ? 1u : 0u;
  out |= (-cx - cw > ax) ? 2u : 0u;
  out |= (cy - cw > ay) ? 4u : 0u;
  out |= (-cy - cw > ay) ? 8u : 0u;
  out |= (cz - cw > az) ? 16u : 0u;
  out |= (-cz - cw > az) ? 32u : 0u;
  return out;
}

// True when the point is inside all six clip planes by a relative margin.
__device__ __forceinline__ bool inside_frustum(const float* mvp, float x, float y, float z) {
  const float cx = mrow(mvp, 0, x, y, z), cy = mrow(mvp, 1, x, y, z), cz = mrow(mvp, 2, x, y, z),
              cw = mrow(mvp, 3, x, y, z);
  const float m = 1e-5f * (fabsf(cx) + fabsf(cy) + fabsf(cz) + fabsf(cw));
  return cx + m < cw && -cx + m < cw && cy + m < cw && -cy + m < cw && cz + m < cw &&
         -cz + m < cw;
}

// ================================================================ prepare
// Absolute transform of a scene-local node: L_root * ... * L_node (parents
// precede children), the order of the reference's transform pass
// (Renderer.cpp:1214-1220).  False (and a status bit) for a bad node or a
// chain deeper than kMaxHierarchyDepth.
__device__ bool node_transform(const PrepareParams& p, const SceneRec& sc, int32_t node, float a[16]) {
  uint32_t chain[kMaxHierarchyDepth];
  int depth = 0;
  int32_t n = node;
  bool ok = n >= 0 && uint32_t(n) < sc.node_count;
  while (ok && n >= 0 && depth < kMaxHierarchyDepth) {
    chain[depth++] = uint32_t(n);
    n = p.parents[sc.node_base + n];
    if (n >= 0 && uint32_t(n) >= sc.node_count) ok = false;
  }
  if (!ok) {
    atomicOr(p.status, kStatusBadNode);
    return false;
  }
  if (n >= 0) {
    atomicOr(p.status, kStatusHierarchyTooDeep);
    return false;
  }
  const float* l = p.local + size_t(sc.node_base + chain[depth - 1]) * 16;
  for (int i = 0; i < 16; ++i) a[i] = l[i];
  for (int k = depth - 2; k >= 0; --k) {
    const float* lk = p.local + size_t(sc.node_base + chain[k]) * 16;
    float b[16], t[16];
    for (int i = 0; i < 16; ++i) b[i] = lk[i];
    matmul(a, b, t);
    for (int i = 0; i < 16; ++i) a[i] = t[i];
  }
  return true;
}

// Normal matrix: the cofactor of the upper-left 3x3 (columns c1 x c2,
// c2 x c0, c0 x c1), column-major, each entry a difference of two products.
__device__ __forceinline__ void normal_matrix(const float a[16], float nm[9]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float* u = a + 4 * ((k + 1) % 3);
    const float* v = a + 4 * ((k + 2) % 3);
    nm[k * 3 + 0] = __fsub_rn(__fmul_rn(u[1], v[2]), __fmul_rn(u[2], v[1]));
    nm[k * 3 + 1] = __fsub_rn(__fmul_rn(u[2], v[0]), __fmul_rn(u[0], v[2]));
    nm[k * 3 + 2] = __fsub_rn(__fmul_rn(u[0], v[1]), __fmul_rn(u[1], v[0]));
  }
}
// Scenes with at most this many visible draws get a nearest-first
// processing order; larger ones keep the draw order.
constexpr uint32_t kSortCap = 2048;

template <int T>
__global__ void __launch_bounds__(T) prepare_kernel(const PrepareParams p) {
  __shared__ uint32_t s_warp[T / 32], s_total, s_count, s_tris, s_clusters;
  __shared__ float s_key[kSortCap];
  __shared__ uint16_t s_idx[kSortCap];
  const uint32_t s = p.scene_base + blockIdx.x;
  const CameraRec& cam = p.cameras[s];
  const uint32_t vis_base = cam.vis_base;
  if (!cam.enabled) {
    if (threadIdx.x == 0) p.vis_count[s] = p.vis_tris[s] = p.vis_clusters[s] = 0;
    return;
  }
  // The scene renders the nodes and draws of its source scene.
  const SceneRec sc = p.scenes[cam.source];
  if (threadIdx.x == 0) {
    s_count = 0;
    s_tris = 0;
    s_clusters = 0;
  }
  float pv[16], vrow[4];
#pragma unroll
  for (int i = 0; i < 16; ++i) pv[i] = cam.pv[i];
#pragma unroll
  for (int i = 0; i < 4; ++i) vrow[i] = cam.vrow[i];
  __syncthreads();
  for (uint32_t base = 0; base < sc.draw_count; base += T) {
    const uint32_t j = base + threadIdx.x;
    uint32_t vis = 0, tris = 0, clusters = 0;
    float far = 0.0f;  // distance of the bounding box's farthest corner along the view axis
    VisibleRec rec;
    ModelRec model;
    if (j < sc.draw_count) {
      const DrawRec d = p.draws[sc.draw_base + j];
      // Absolute transform: abs = L_root * ... * L_node (parents precede children).
      uint32_t chain[kMaxHierarchyDepth];
      int depth = 0;
      int32_t n = int32_t(d.node);
      bool ok = n >= 0 && uint32_t(n) < sc.node_count;
      while (ok && n >= 0 && depth < kMaxHierarchyDepth) {
        chain[depth++] = uint32_t(n);
        n = p.parents[sc.node_base + n];
        if (n >= 0 && uint32_t(n) >= sc.node_count) ok = false;
      }
      if (!ok) atomicOr(p.status, kStatusBadNode);
      if (ok && n >= 0) {
        atomicOr(p.status, kStatusHierarchyTooDeep);
        ok = false;
      }
      if (ok) {
        float a[16], t[16];
        const float* l = p.local + size_t(sc.node_base + chain[depth - 1]) * 16;
#pragma unroll
        for (int i = 0; i < 16; ++i) a[i] = l[i];
        for (int k = depth - 2; k >= 0; --k) {
          const float* lk = p.local + size_t(sc.node_base + chain[k]) * 16;
          float b[16];
#pragma unroll
          for (int i = 0; i < 16; ++i) b[i] = lk[i];
          matmul(a, b, t);
#pragma unroll
          for (int i = 0; i < 16; ++i) a[i] = t[i];
        }
        matmul(pv, a, rec.mvp);
        if (p.model) {
#pragma unroll
          for (int col = 0; col < 4; ++col)
#pragma unroll
            for (int row = 0; row < 3; ++row) model.a[col * 3 + row] = a[col * 4 + row];
          normal_matrix(a, model.nm);
          model.pad[0] = model.pad[1] = model.pad[2] = 0.0f;
        }
#pragma unroll
        for (int col = 0; col < 4; ++col) {
          float z = __fmul_rn(vrow[0], a[col * 4 + 0]);
          z = fma_(vrow[1], a[col * 4 + 1], z);
          z = fma_(vrow[2], a[col * 4 + 2], z);
          z = fma_(vrow[3], a[col * 4 + 3], z);
          rec.zrow[col] = z;
        }
        // Frustum test of the view's bounding box: culled only when all
        // eight corners lie beyond the same clip plane by a relative margin,
        // so rounding can never drop a triangle that would cover a pixel.
        uint32_t all_out = 0x3fu;
        bool inside = true;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          const float x = d.bbox[(c & 1) ? 3 : 0], y = d.bbox[(c & 2) ? 4 : 1],
                      z = d.bbox[(c & 4) ? 5 : 2];
          all_out &= outcode(rec.mvp, x, y, z);
          inside = inside && inside_frustum(rec.mvp, x, y, z);
          float ze = fma_(rec.zrow[2], z, fma_(rec.zrow[1], y, fma_(rec.zrow[0], x, rec.zrow[3])));
          far = fmaxf(far, -ze);
        }
        if (all_out == 0 && d.tri_count > 0) {
          const MeshRec m = p.meshes[d.mesh];
          vis = 1;
          tris = d.tri_count;
          clusters = cluster_count(d.chunk_count);
          rec.vertex_base = m.vertex_base;
          rec.first_index = d.first_index;
          rec.tri_count = d.tri_count;
          rec.material = d.material;
          rec.semantic_id = d.semantic_id;
          rec.flags = m.flags | (inside ? kDrawInsideFrustum : 0u);
          rec.box_base = d.box_base;
          rec.chunk_count = d.chunk_count;
          rec.pad[0] = rec.pad[1] = 0;
        }
      }
    }
    const uint32_t vo = block_exclusive_scan<T>(vis, s_warp, &s_total);
    const uint32_t vtot = s_total;
    __syncthreads();
    const uint32_t to = block_exclusive_scan<T>(tris, s_warp, &s_total);
    const uint32_t ttot = s_total;
    __syncthreads();
    const uint32_t co = block_exclusive_scan<T>(clusters, s_warp, &s_total);
    const uint32_t ctot = s_total;
    if (vis) {
      rec.ordinal = s_tris + to;
      rec.cluster = s_clusters + co;
      p.visible[vis_base + s_count + vo] = rec;
      if (p.model) p.model[vis_base + s_count + vo] = model;
      if (s_count + vo < kSortCap) s_key[s_count + vo] = far == far ? far : INFINITY;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      s_count += vtot;
      s_tris += ttot;
      s_clusters += ctot;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    p.vis_count[s] = s_count;
    p.vis_tris[s] = s_tris;
    p.vis_clusters[s] = s_clusters;
  }
  // Lights of the source scene in world space (Renderer.cpp:1263-1289): a
  // point light at its node's translation, a directional light towards the
  // node's negative backward axis.
  if (p.lights) {
    const uint32_t nl = min(p.cameras[cam.source].light_count, p.max_lights);
    for (uint32_t j = threadIdx.x; j < nl; j += T) {
      const LightSrc src = p.light_src[size_t(cam.source) * p.max_lights + j];
      float a[16];
      WorldLight w{};
      if (node_transform(p, sc, src.node, a)) {
        if (src.type == 0) {
          w.pos[0] = -a[8];
          w.pos[1] = -a[9];
          w.pos[2] = -a[10];
          w.pos[3] = 0.0f;
        } else {
          w.pos[0] = a[12];
          w.pos[1] = a[13];
          w.pos[2] = a[14];
          w.pos[3] = 1.0f;
        }
      }
      w.color[0] = src.color[0];
      w.color[1] = src.color[1];
      w.color[2] = src.color[2];
      w.range = src.range;
      p.lights[size_t(s) * p.max_lights + j] = w;
    }
  }

  // Processing order: visible draws by the distance of their farthest
  // corner, nearest first (a draw around the camera, like a room shell,
  // goes last); ties by draw order.  The raster kernel's results do not
  // depend on this order, only how much it can cull.
  if (!p.order) return;
  const uint32_t n = s_count;
  uint2* order = p.order + vis_base;
  const VisibleRec* visible = p.visible + vis_base;  // written above by this CTA: plain loads
  if (n > kSortCap) {
    for (uint32_t k = threadIdx.x; k < n; k += T) order[k] = make_uint2(k, visible[k].cluster);
    return;
  }
  uint32_t m = 1;
  while (m < n) m <<= 1;
  for (uint32_t i = threadIdx.x; i < m; i += T) {
    if (i >= n) s_key[i] = INFINITY;
    s_idx[i] = uint16_t(i);
  }
  __syncthreads();
  for (uint32_t k = 2; k <= m; k <<= 1)
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      for (uint32_t i = threadIdx.x; i < m; i += T) {
        const uint32_t l = i ^ j;
        if (l > i) {
          const float ki = s_key[i], kl = s_key[l];
          const uint16_t ii = s_idx[i], il = s_idx[l];
          const bool greater = ki > kl || (ki == kl && ii > il);
          if (greater == ((i & k) == 0)) {
            s_key[i] = kl;
            s_key[l] = ki;
            s_idx[i] = il;
            s_idx[l] = ii;
          }
        }
      }
      __syncthreads();
    }
  uint32_t running = 0;
  for (uint32_t base = 0; base < n; base += T) {
    const uint32_t k = base + threadIdx.x;
    const uint32_t d = k < n ? s_idx[k] : 0u;
    const uint32_t cnt = k < n ? cluster_count(visible[d].chunk_count) : 0u;
    const uint32_t off = block_exclusive_scan<T>(cnt, s_warp, &s_total);
    if (k < n) order[k] = make_uint2(d, running + off);
    running += s_total;
    __syncthreads();
  }
}

// ================================================================= raster
struct QEntry {
  int32_t X[3], Y[3];
  float zw0, d1, d2, inva;
  uint32_t ordinal;
  uint32_t bias;  // bit i: edge i owns its pixels (top-left)
  int16_t x0, y0, x1, y1;
};

// Dynamic shared-memory layout of raster_kernel; every section starts on a
// 16-byte boundary.
struct SmemLayout {
  size_t queue, qoff, prefix, chunks, clusters, tiles, coarse, total;
};

// Depth tiles of the occlusion test: kTile x kTile pixels of the region,
// and coarse tiles of kCoarse x kCoarse tiles.
constexpr int kTile = 8, kCoarse = 4;
__host__ __device__ __forceinline__ int tile_capacity(int region_px, int side) {
  // ceil(w / s) * ceil(h / s) <= w h / s^2 + (w + h) / s + 1 with w, h <= 1024
  return region_px / (side * side) + 2 * 1024 / side + 1;
}
__host__ __device__ __forceinline__ size_t align16(size_t x) { return (x + 15) & ~size_t(15); }
__host__ __device__ __forceinline__ SmemLayout smem_layout(int threads, int region_px,
                                                           int prefix_cap) {
  SmemLayout l;
  l.queue = align16(size_t(region_px) * 8);
  l.qoff = align16(l.queue + size_t(threads) * sizeof(QEntry));
  l.prefix = align16(l.qoff + size_t(threads + 1) * 4);
  l.chunks = align16(l.prefix + size_t(prefix_cap + 1) * 4);
  l.clusters = align16(l.chunks + size_t(ring_capacity(threads)) * sizeof(uint2));
  l.tiles = align16(l.clusters + size_t(kClusterRing) * sizeof(uint2));
  l.coarse = align16(l.tiles + size_t(tile_capacity(region_px, kTile)) * 4);
  l.total = align16(l.coarse + size_t(tile_capacity(region_px, kTile * kCoarse)) * 4);
  return l;
}

struct Setup {
  int32_t X[3], Y[3];
  float zw0, d1, d2, inva;
  float zmin;  // nearest window depth of the three vertices
  uint32_t bias;
  int x0, y0, x1, y1;
};

struct Ctx {
  uint64_t* keys;
  QEntry* queue;
  QEntry* spill;  // this CTA's global spill area (qcap more entries), or null
  uint32_t* qcount;
  int qcap;
  int rx0, ry0, rw, rh;  // region
  int W, H;              // viewport
  int small_area;
  float hw, hh;          // half the viewport size
  float gx, gy;          // guard band in NDC: 32768 / W, 32768 / H
  // Deepest depth of each 8x8 depth tile and 32x32 coarse tile of the region
  // (null when occlusion culling is off).  Refreshed from the z-buffer from
  // time to time; depths only decrease, so a stale value is conservative.
  const uint32_t* tiles;
  const uint32_t* coarse;
  int tcols, ccols;
};

__device__ __forceinline__ void set_viewport(Ctx& c, int W, int H) {
  c.W = W;
  c.H = H;
  c.hw = __fmul_rn(0.5f, float(W));
  c.hh = __fmul_rn(0.5f, float(H));
  c.gx = __fdiv_rn(32768.0f, float(W));
  c.gy = __fdiv_rn(32768.0f, float(H));
}

// Project, snap, orient and bound one (sub)triangle.  False if it covers
// no pixel centre of the region.
__device__ __forceinline__ bool setup_sub(const float4* q, const Ctx& c, Setup& st) {
  const float hw = c.hw, hh = c.hh;
  float zw[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float iw = __frcp_rn(q[i].w);
    const float nx = __fmul_rn(q[i].x, iw), ny = __fmul_rn(q[i].y, iw),
                nz = __fmul_rn(q[i].z, iw);
    const float xw = fma_(nx, hw, hw), yw = fma_(ny, hh, hh);
    zw[i] = fma_(nz, 0.5f, 0.5f);
    st.X[i] = __float2int_rn(__fmul_rn(xw, 256.0f));
    st.Y[i] = __float2int_rn(__fmul_rn(yw, 256.0f));
  }
  // A box without a pixel centre first: most sub-pixel triangles leave here,
  // before the area and the fill rule.
  const int minX = min(st.X[0], min(st.X[1], st.X[2])), maxX = max(st.X[0], max(st.X[1], st.X[2]));
  const int minY = min(st.Y[0], min(st.Y[1], st.Y[2])), maxY = max(st.Y[0], max(st.Y[1], st.Y[2]));
  st.x0 = max((minX - 128 + 255) >> 8, c.rx0);
  st.x1 = min((maxX - 128) >> 8, c.rx0 + c.rw - 1);
  st.y0 = max((minY - 128 + 255) >> 8, c.ry0);
  st.y1 = min((maxY - 128) >> 8, c.ry0 + c.rh - 1);
  if (st.x0 > st.x1 || st.y0 > st.y1) return false;
  const int64_t area = int64_t(st.X[1] - st.X[0]) * int64_t(st.Y[2] - st.Y[0]) -
                       int64_t(st.X[2] - st.X[0]) * int64_t(st.Y[1] - st.Y[0]);
  if (area <= 0) return false;
  uint32_t bias = 0;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const int a = (i + 1) % 3, b = (i + 2) % 3;
    const int dx = st.X[b] - st.X[a], dy = st.Y[b] - st.Y[a];
    if (dy < 0 || (dy == 0 && dx < 0)) bias |= 1u << i;
  }
  st.bias = bias;
  st.inva = __frcp_rn(__ll2float_rn(area));
  st.zmin = fminf(zw[0], fminf(zw[1], zw[2]));
  st.zw0 = zw[0];
  st.d1 = __fsub_rn(zw[1], zw[0]);
  st.d2 = __fsub_rn(zw[2], zw[0]);
  return true;
}

// Coverage and depth of pixel (px, py); false if not covered or beyond far.
__device__ __forceinline__ bool cover(const int32_t* X, const int32_t* Y, uint32_t bias,
                                      float zw0, float d1, float d2, float inva, int px, int py,
                                      float& z) {
  const int32_t Px = px * 256 + 128, Py = py * 256 + 128;
  int64_t e[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const int a = (i + 1) % 3, b = (i + 2) % 3;
    e[i] = int64_t(X[b] - X[a]) * int64_t(Py - Y[a]) - int64_t(Y[b] - Y[a]) * int64_t(Px - X[a]);
    if (e[i] + ((bias >> i) & 1u ? 0 : -1) < 0) return false;
  }
  const float b1 = __fmul_rn(__ll2float_rn(e[1]), inva), b2 = __fmul_rn(__ll2float_rn(e[2]), inva);
  float zz = fma_(b2, d2, fma_(b1, d1, zw0));
  if (!(zz > 0.0f)) zz = 0.0f;
  if (!(zz < 1.0f)) return false;
  z = zz;
  return true;
}

__device__ __forceinline__ void depth_write(uint64_t* keys, int idx, float z, uint32_t ordinal) {
  const uint64_t key = (uint64_t(__float_as_uint(z)) << 32) | ordinal;
  if (key < *reinterpret_cast<volatile uint64_t*>(keys + idx))
    atomicMin(reinterpret_cast<unsigned long long*>(keys + idx), (unsigned long long)key);
}

__device__ __forceinline__ void raster_setup(const Setup& st, uint32_t ordinal, const Ctx& c) {
  for (int py = st.y0; py <= st.y1; ++py)
    for (int px = st.x0; px <= st.x1; ++px) {
      float z;
      if (cover(st.X, st.Y, st.bias, st.zw0, st.d1, st.d2, st.inva, px, py, z))
        depth_write(c.keys, (py - c.ry0) * c.rw + (px - c.rx0), z, ordinal);
    }
}

__device__ __forceinline__ void store_entry(QEntry& e, const Setup& st, uint32_t ordinal) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    e.X[i] = st.X[i];
    e.Y[i] = st.Y[i];
  }
  e.zw0 = st.zw0;
  e.d1 = st.d1;
  e.d2 = st.d2;
  e.inva = st.inva;
  e.ordinal = ordinal;
  e.bias = st.bias;
  e.x0 = int16_t(st.x0);
  e.y0 = int16_t(st.y0);
  e.x1 = int16_t(st.x1);
  e.y1 = int16_t(st.y1);
}

// Triangle-level occlusion test: true when every fragment the (sub)triangle
// could produce loses the depth test against the z-buffer.  A fragment's
// depth is interpolated from the vertices' window depths with barycentrics
// in [0, 1], so it is at least their minimum less a few units of rounding;
// with a margin far above that rounding, if that bound is deeper than the
// deepest depth of every tile the bounding box touches, no fragment passes
// (the z-buffer's depths only decrease).  The tile values may be stale,
// which only makes the test keep more.
__device__ __forceinline__ bool hidden(const Setup& st, const Ctx& c) {
  const float zm = __fsub_rn(st.zmin, 4e-6f);
  if (!c.tiles || !(zm > 0.0f)) return false;
  const uint32_t zbits = __float_as_uint(zm);
  int tx0 = (st.x0 - c.rx0) / kTile, tx1 = (st.x1 - c.rx0) / kTile;
  int ty0 = (st.y0 - c.ry0) / kTile, ty1 = (st.y1 - c.ry0) / kTile;
  const uint32_t* t = c.tiles;
  int cols = c.tcols;
  if ((tx1 - tx0 + 1) * (ty1 - ty0 + 1) > 16) {  // large footprint: coarse tiles
    tx0 /= kCoarse;
    tx1 /= kCoarse;
    ty0 /= kCoarse;
    ty1 /= kCoarse;
    t = c.coarse;
    cols = c.ccols;
  }
  for (int ty = ty0; ty <= ty1; ++ty)
    for (int tx = tx0; tx <= tx1; ++tx)
      if (t[ty * cols + tx] >= zbits) return false;
  return true;
}

__device__ __forceinline__ void emit(const float4* q, uint32_t ordinal, const Ctx& c) {
  Setup st;
  if (!setup_sub(q, c, st)) return;
  const int area = (st.x1 - st.x0 + 1) * (st.y1 - st.y0 + 1);
  if (area > c.small_area) {
    // Only triangles bound for the shared queue are tested: their pixels
    // cost the whole CTA; a small one is cheaper to rasterise than to test.
    if (hidden(st, c)) return;
    const uint32_t slot = atomicAdd(c.qcount, 1u);
    if (slot < uint32_t(c.qcap)) {
      store_entry(c.queue[slot], st, ordinal);
      return;
    }
    if (c.spill && slot < 2u * uint32_t(c.qcap)) {
      store_entry(c.spill[slot - c.qcap], st, ordinal);
      return;
    }
  }
  raster_setup(st, ordinal, c);
}

__device__ __forceinline__ float plane_dist(const float4& v, int p, float gx, float gy) {
  switch (p) {
    case 0: return __fadd_rn(v.z, v.w);
    case 1: return __fsub_rn(__fmul_rn(gx, v.w), v.x);
    case 2: return __fadd_rn(__fmul_rn(gx, v.w), v.x);
    case 3: return __fsub_rn(__fmul_rn(gy, v.w), v.y);
    default: return __fadd_rn(__fmul_rn(gy, v.w), v.y);
  }
}

__device__ __forceinline__ float4 lerp_clip(const float4& in, const float4& out, float din,
                                            float dout) {
  const float t = __fdiv_rn(din, __fsub_rn(din, dout));
  return make_float4(fma_(t, __fsub_rn(out.x, in.x), in.x), fma_(t, __fsub_rn(out.y, in.y), in.y),
                     fma_(t, __fsub_rn(out.z, in.z), in.z), fma_(t, __fsub_rn(out.w, in.w), in.w));
}

// Out of line, the vertices taken by value: an array address passed to the
// call would place the caller's vertices in local memory for every triangle,
// not only for the few that are clipped.  (The context stays a reference: it
// is stored once per work item, and copying it for the call costs registers.)
__device__ __noinline__ void clip_general(float4 v0, float4 v1, float4 v2, uint32_t ordinal,
                                          const Ctx& c) {
  const float gx = c.gx, gy = c.gy;
  float4 poly[9], next[9];
  int n = 3;
  poly[0] = v0;
  poly[1] = v1;
  poly[2] = v2;
  for (int p = 0; p < 5 && n >= 3; ++p) {
    int m = 0;
    for (int i = 0; i < n; ++i) {
      const float4 a = poly[i];
      const float4 b = poly[(i + 1) % n];
      const float da = plane_dist(a, p, gx, gy), db = plane_dist(b, p, gx, gy);
      const bool ina = da >= 0.0f, inb = db >= 0.0f;
      if (ina) next[m++] = a;
      if (ina != inb) next[m++] = ina ? lerp_clip(a, b, da, db) : lerp_clip(b, a, db, da);
    }
    n = m;
    for (int i = 0; i < n; ++i) poly[i] = next[i];
  }
  for (int i = 1; i + 1 < n; ++i) {
    const float4 sub[3] = {poly[0], poly[i], poly[i + 1]};
    emit(sub, ordinal, c);
  }
}

__device__ __forceinline__ bool inside_guard(const float4& v, float gx, float gy) {
  return plane_dist(v, 1, gx, gy) >= 0.0f && plane_dist(v, 2, gx, gy) >= 0.0f &&
         plane_dist(v, 3, gx, gy) >= 0.0f && plane_dist(v, 4, gx, gy) >= 0.0f;
}

// Clipping of a triangle that needs it.  The common case -- the near plane
// cuts it and its clipped polygon lies inside the guard band -- is done in
// registers: the polygon is the one Sutherland-Hodgman makes for the near
// plane (same vertices, same order, same intersection arithmetic), which the
// guard-band planes then leave unchanged, so the fan triangles are those of
// the general path.  Any other case runs the general path.
__device__ __noinline__ void clip_and_emit(float4 v0, float4 v1, float4 v2, uint32_t ordinal,
                                           const Ctx& c) {
  const float gx = c.gx, gy = c.gy;
  const float d0 = plane_dist(v0, 0, gx, gy), d1 = plane_dist(v1, 0, gx, gy),
              d2 = plane_dist(v2, 0, gx, gy);
  const uint32_t out = (d0 >= 0.0f ? 0u : 1u) | (d1 >= 0.0f ? 0u : 2u) | (d2 >= 0.0f ? 0u : 4u);
  float4 q0, q1, q2, q3;
  int n = 4;
  switch (out) {
    case 0: q0 = v0; q1 = v1; q2 = v2; n = 3; break;
    case 1: q0 = lerp_clip(v1, v0, d1, d0); q1 = v1; q2 = v2; q3 = lerp_clip(v2, v0, d2, d0); break;
    case 2: q0 = v0; q1 = lerp_clip(v0, v1, d0, d1); q2 = lerp_clip(v2, v1, d2, d1); q3 = v2; break;
    case 4: q0 = v0; q1 = v1; q2 = lerp_clip(v1, v2, d1, d2); q3 = lerp_clip(v0, v2, d0, d2); break;
    case 3: q0 = lerp_clip(v2, v1, d2, d1); q1 = v2; q2 = lerp_clip(v2, v0, d2, d0); n = 3; break;
    case 6: q0 = v0; q1 = lerp_clip(v0, v1, d0, d1); q2 = lerp_clip(v0, v2, d0, d2); n = 3; break;
    case 5: q0 = lerp_clip(v1, v0, d1, d0); q1 = v1; q2 = lerp_clip(v1, v2, d1, d2); n = 3; break;
    default: return;  // all three behind the near plane
  }
  if (!inside_guard(q0, gx, gy) || !inside_guard(q1, gx, gy) || !inside_guard(q2, gx, gy) ||
      (n == 4 && !inside_guard(q3, gx, gy))) {
    clip_general(v0, v1, v2, ordinal, c);
    return;
  }
  {
    const float4 sub[3] = {q0, q1, q2};
    emit(sub, ordinal, c);
  }
  if (n == 4) {
    const float4 sub[3] = {q0, q2, q3};
    emit(sub, ordinal, c);
  }
}

__device__ __forceinline__ void triangle(const float4* cv, uint32_t ordinal, const Ctx& c) {
  // Trivial reject: all three vertices beyond one frustum plane.
  if ((cv[0].x > cv[0].w && cv[1].x > cv[1].w && cv[2].x > cv[2].w) ||
      (cv[0].x < -cv[0].w && cv[1].x < -cv[1].w && cv[2].x < -cv[2].w) ||
      (cv[0].y > cv[0].w && cv[1].y > cv[1].w && cv[2].y > cv[2].w) ||
      (cv[0].y < -cv[0].w && cv[1].y < -cv[1].w && cv[2].y < -cv[2].w) ||
      (cv[0].z > cv[0].w && cv[1].z > cv[1].w && cv[2].z > cv[2].w) ||
      (cv[0].z < -cv[0].w && cv[1].z < -cv[1].w && cv[2].z < -cv[2].w))
    return;
  const float gx = c.gx, gy = c.gy;
  bool need_clip = false;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int p = 0; p < 5; ++p) need_clip |= plane_dist(cv[i], p, gx, gy) < 0.0f;
  if (!need_clip)
    emit(cv, ordinal, c);
  else
    clip_and_emit(cv[0], cv[1], cv[2], ordinal, c);
}

// Largest d in [0, n) with ordinal(d) <= g.
__device__ __forceinline__ uint32_t find_draw(const uint32_t* prefix, const VisibleRec* vis,
                                              bool cached, uint32_t n, uint32_t g) {
  uint32_t lo = 0, hi = n;  // invariant: ord(lo) <= g < ord(hi)
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    const uint32_t o = cached ? prefix[mid] : __ldg(&vis[mid].ordinal);
    if (o <= g)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

__device__ __forceinline__ int wrap(int i, int n, int mode) {
  if (mode == 0) {
    int m = i % n;
    return m < 0 ? m + n : m;
  }
  if (mode == 1) return i < 0 ? 0 : (i >= n ? n - 1 : i);
  const int p = 2 * n;
  int m = i % p;
  if (m < 0) m += p;
  return m >= n ? p - 1 - m : m;
}

__device__ __forceinline__ float clampc(float f) {
  const float lim = 16777216.0f;
  if (!(f > -lim)) return -lim;
  if (!(f < lim)) return lim;
  return f;
}

// Channel c of an RGBA8 texel as a float, v / 255 correctly rounded.  1/255
// is held as the unevaluated sum of two floats, hi = fl(1/255) and
// lo = fl(1/255 - hi); fl(v hi + fl(v lo)), the sum taken by one fused
// multiply-add, is the correctly rounded v / 255 for every v in [0, 255]
// (multiplication by a constant in double-word form: Brisebarre and Muller,
// "Correctly rounded multiplication by arbitrary precision constants", IEEE
// Trans. Computers 57(2), 2008; checked here for all 256 v in exact rational
// arithmetic).  v becomes a float exactly in the mantissa of 2^23.
__device__ __forceinline__ float chan(uint32_t t, int c) {
  const float v = __fsub_rn(__uint_as_float(0x4b000000u | ((t >> (8 * c)) & 255u)), 8388608.0f);
  return __fmaf_rn(v, 0x1.010102p-8f, __fmul_rn(v, -0x1.fdfdfep-33f));
}

// One level of a texture (level k is max(1, w >> k) x max(1, h >> k); the
// levels follow one another, each holding every layer), filtered nearest (0)
// or bilinear (1) at texel centres with the texture's wrap modes.
__device__ __forceinline__ void sample_level(const TextureRec& t, const uint32_t* texels, int L, int level, int filter,
                             float s, float u, float out[4]) {
  const int tw = max(1, t.width >> level), th = max(1, t.height >> level);
  size_t off = t.offset;
  for (int k = 0; k < level; ++k) off += size_t(max(1, t.width >> k)) * size_t(max(1, t.height >> k)) * t.layers;
  const float fw = float(tw), fh = float(th);
  const uint32_t* base = texels + off + size_t(L) * th * tw;
  if (filter == 0) {
    const int x = wrap(int(floorf(clampc(__fmul_rn(s, fw)))), tw, t.wrap_s);
    const int y = wrap(int(floorf(clampc(__fmul_rn(u, fh)))), th, t.wrap_t);
    const uint32_t v = __ldg(base + size_t(y) * tw + x);
#pragma unroll
    for (int c = 0; c < 4; ++c) out[c] = chan(v, c);
    return;
  }
  const float fx = clampc(__fsub_rn(__fmul_rn(s, fw), 0.5f));
  const float fy = clampc(__fsub_rn(__fmul_rn(u, fh), 0.5f));
  const float flx = floorf(fx), fly = floorf(fy);
  const float a = __fsub_rn(fx, flx), b = __fsub_rn(fy, fly);
  const int x0 = wrap(int(flx), tw, t.wrap_s), x1 = wrap(int(flx) + 1, tw, t.wrap_s);
  const int y0 = wrap(int(fly), th, t.wrap_t), y1 = wrap(int(fly) + 1, th, t.wrap_t);
  const uint32_t v00 = __ldg(base + size_t(y0) * tw + x0);
  const uint32_t v10 = __ldg(base + size_t(y0) * tw + x1);
  const uint32_t v01 = __ldg(base + size_t(y1) * tw + x0);
  const uint32_t v11 = __ldg(base + size_t(y1) * tw + x1);
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const float t00 = chan(v00, c), t10 = chan(v10, c), t01 = chan(v01, c), t11 = chan(v11, c);
    const float lo = fma_(a, __fsub_rn(t10, t00), t00);
    const float hi = fma_(a, __fsub_rn(t11, t01), t01);
    out[c] = fma_(b, __fsub_rn(hi, lo), lo);
  }
}

__device__ __forceinline__ int clamp_layer(const TextureRec& t, int layer) {
  return layer < 0 ? 0 : (layer >= t.layers ? t.layers - 1 : layer);
}

// Level-0 sampling with the magnification filter (textures whose
// minification is the same and that have no mip levels).
__device__ __forceinline__ void sample(const TextureRec& t, const uint32_t* texels, int layer, float s, float u,
                                       float out[4]) {
  sample_level(t, texels, clamp_layer(t, layer), 0, t.filter, s, u, out);
}

// log2 by the atanh series of the mantissa normalised to [sqrt(1/2), sqrt(2))
// (every operation one float rounding, so the oracle reproduces it).
__device__ __forceinline__ float series_log2(float x) {
  int e;
  float m = frexpf(x, &e);
  if (m < 0.7071067690849304f) {
    m = __fmul_rn(m, 2.0f);
    e -= 1;
  }
  const float t = __fdiv_rn(__fsub_rn(m, 1.0f), __fadd_rn(m, 1.0f));
  const float t2 = __fmul_rn(t, t);
  float q = 0.1111111119389534f;
  q = __fadd_rn(__fmul_rn(q, t2), 0.1428571492433548f);
  q = __fadd_rn(__fmul_rn(q, t2), 0.20000000298023224f);
  q = __fadd_rn(__fmul_rn(q, t2), 0.3333333432674408f);
  q = __fadd_rn(__fmul_rn(q, t2), 1.0f);
  return __fadd_rn(float(e), __fmul_rn(__fmul_rn(t, q), 2.885390043258667f));
}

// Texture lookup at level-of-detail lambda = log2(rho) (OpenGL 4.6, 8.14):
// magnification (level 0, magnification filter) up to c = 0.5 for a linear
// magnification with a nearest-mipmap minification, else 0; then the base
// level, the nearest level ceil(lambda + 1/2) - 1, or the two levels around
// lambda blended by its fraction, each with the minification filter.
__device__ __forceinline__ void sample_lod(const TextureRec& t, const uint32_t* texels, int layer, float s, float u,
                           float lambda, float out[4]) {
  const int L = clamp_layer(t, layer);
  const float c = (t.filter == 1 && t.min_filter == 0 && t.mip_filter != 0) ? 0.5f : 0.0f;
  if (!(lambda > c)) {
    sample_level(t, texels, L, 0, t.filter, s, u, out);
    return;
  }
  const int q = t.levels - 1;
  if (t.mip_filter == 0) {
    sample_level(t, texels, L, 0, t.min_filter, s, u, out);
  } else if (t.mip_filter == 1) {
    int d = lambda <= 0.5f ? 0 : int(ceilf(__fadd_rn(lambda, 0.5f))) - 1;
    if (d > q) d = q;
    sample_level(t, texels, L, d, t.min_filter, s, u, out);
  } else if (lambda >= float(q)) {
    sample_level(t, texels, L, q, t.min_filter, s, u, out);
  } else {
    const float fl = floorf(lambda);
    const int d1 = int(fl);
    const float f = __fsub_rn(lambda, fl);
    float hi[4];
    sample_level(t, texels, L, d1, t.min_filter, s, u, out);
    sample_level(t, texels, L, d1 + 1, t.min_filter, s, u, hi);
#pragma unroll
    for (int k = 0; k < 4; ++k) out[k] = fma_(f, __fsub_rn(hi[k], out[k]), out[k]);
  }
}

// Float -> unorm8: round to nearest, values within 1e-4 above a tie rounded
// down (the rounding of the reference's images).
__device__ __forceinline__ uint32_t unorm8(float c) {
  if (!(c > 0.0f)) c = 0.0f;
  if (c > 1.0f) c = 1.0f;
  float t = __fmul_rn(c, 255.0f);
  t = __fadd_rn(t, 0.4999f);
  return __float2uint_rz(t);
}

// Lit colour (Phong without a specular term, the reference's shader
// configuration): ambient + sum over lights of diffuse * light colour *
// max(0, N.L) * attenuation, attenuation = clamp(1 - (d / range)^4, 0, 1)^2
// / (1 + d^2), d = distance to a point light (0 for directional lights);
// N = the normalised interpolation of the vertices' normal-matrix normals,
// the fragment's world position the interpolation of theirs.  Alpha is the
// diffuse alpha.
// Out of line (the unlit path keeps its registers) and taking its inputs by
// value: an address passed to a call would place the caller's arrays in
// local memory for every shaded pixel.
__device__ __noinline__ uint32_t lit_color(const float4* __restrict__ vertex_normals, float ambient_factor,
                                           const MaterialRec& mat, float4 tc4, float4 vc4,
                                           const WorldLight* lights, uint32_t nl,
                                           const ModelRec* model, uint32_t v0, uint32_t v1, uint32_t v2,
                                           float4 q0, float4 q1, float4 q2, float b0, float b1, float b2,
                                           bool normals) {
#define GBR_INTERP(a0, a1, a2) fma_(b2, (a2), fma_(b1, (a1), __fmul_rn(b0, (a0))))
  const float tc[4] = {tc4.x, tc4.y, tc4.z, tc4.w}, vc[4] = {vc4.x, vc4.y, vc4.z, vc4.w};
  const uint32_t v[3] = {v0, v1, v2};
  const float4 q[3] = {q0, q1, q2};
  float amb[4], dif[4], rgb[3];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    amb[c] = __fmul_rn(__fmul_rn(__fmul_rn(mat.color[c], ambient_factor), tc[c]), vc[c]);
    dif[c] = __fmul_rn(__fmul_rn(mat.color[c], tc[c]), vc[c]);
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) rgb[c] = amb[c];
  if (nl > 0 && normals) {
    float A[12], NM[9];
#pragma unroll
    for (int i = 0; i < 12; ++i) A[i] = __ldg(&model->a[i]);
#pragma unroll
    for (int i = 0; i < 9; ++i) NM[i] = __ldg(&model->nm[i]);
    float wp[3][3], wn[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float4 n = __ldg(&vertex_normals[v[k]]);
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        float t = A[9 + r];
        t = fma_(A[r], q[k].x, t);
        t = fma_(A[3 + r], q[k].y, t);
        t = fma_(A[6 + r], q[k].z, t);
        wp[k][r] = t;
        wn[k][r] = fma_(NM[6 + r], n.z, fma_(NM[3 + r], n.y, __fmul_rn(NM[r], n.x)));
      }
    }
    float P[3], N[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      P[r] = GBR_INTERP(wp[0][r], wp[1][r], wp[2][r]);
      N[r] = GBR_INTERP(wn[0][r], wn[1][r], wn[2][r]);
    }
    const float len2 = fma_(N[2], N[2], fma_(N[1], N[1], __fmul_rn(N[0], N[0])));
    const float inv = __frcp_rn(__fsqrt_rn(len2));
    const float n0 = __fmul_rn(N[0], inv), n1 = __fmul_rn(N[1], inv), n2 = __fmul_rn(N[2], inv);
    for (uint32_t j = 0; j < nl; ++j) {
      const WorldLight L = lights[j];
      const float l0 = __fsub_rn(L.pos[0], __fmul_rn(P[0], L.pos[3]));
      const float l1 = __fsub_rn(L.pos[1], __fmul_rn(P[1], L.pos[3]));
      const float l2 = __fsub_rn(L.pos[2], __fmul_rn(P[2], L.pos[3]));
      const float d2 = fma_(l2, l2, fma_(l1, l1, __fmul_rn(l0, l0)));
      const float len = __fsqrt_rn(d2);
      if (!(len > 0.0f)) continue;
      const float dist = __fmul_rn(len, L.pos[3]);
      const float qd = __fdiv_rn(dist, fmaxf(L.range, 0.0001f));
      const float q2 = __fmul_rn(qd, qd);
      float a = __fsub_rn(1.0f, __fmul_rn(q2, q2));
      a = a < 0.0f ? 0.0f : (a > 1.0f ? 1.0f : a);
      const float att = __fdiv_rn(__fmul_rn(a, a), __fadd_rn(1.0f, __fmul_rn(dist, dist)));
      const float il = __frcp_rn(len);
      const float ndl = fma_(n2, __fmul_rn(l2, il),
                             fma_(n1, __fmul_rn(l1, il), __fmul_rn(n0, __fmul_rn(l0, il))));
      const float intensity = __fmul_rn(ndl > 0.0f ? ndl : 0.0f, att);
#pragma unroll
      for (int c = 0; c < 3; ++c) rgb[c] = fma_(__fmul_rn(dif[c], L.color[c]), intensity, rgb[c]);
    }
  }
#undef GBR_INTERP
  return unorm8(rgb[0]) | (unorm8(rgb[1]) << 8) | (unorm8(rgb[2]) << 16) | (unorm8(dif[3]) << 24);
}

// Shade the winning triangle `t` of visible draw `rec` at pixel (px, py).
// Mode 0: every texture sampled at level 0 with its magnification filter
// (no texture of the launch needs a level of detail).  Mode 1: textures that
// need one (mip levels or a minification filter other than the magnification
// one) are not sampled and the call returns false; the caller shades those
// pixels again with Mode 2, the level-of-detail path, in a separate loop, so
// that the derivative code does not add to the common path's registers.
template <int Mode>
__device__ __forceinline__ bool shade(const RasterParams& p, int W, int H, const VisibleRec* rec, uint32_t t,
                                      int px, int py, const WorldLight* lights, uint32_t nl,
                                      const ModelRec* model, uint32_t& color, float& lin, uint32_t& sid) {
  // The record in 16-byte loads: mvp, zrow, (vertex_base, first_index,
  // tri_count, material), (semantic_id, ordinal, flags, chunk).
  const float4* r4 = reinterpret_cast<const float4*>(rec);
  float mvp[16], zr[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float4 v = __ldg(r4 + i);
    mvp[4 * i] = v.x;
    mvp[4 * i + 1] = v.y;
    mvp[4 * i + 2] = v.z;
    mvp[4 * i + 3] = v.w;
  }
  const float4 z4 = __ldg(r4 + 4);
  zr[0] = z4.x;
  zr[1] = z4.y;
  zr[2] = z4.z;
  zr[3] = z4.w;
  const uint4 u5 = __ldg(reinterpret_cast<const uint4*>(rec) + 5);
  const uint4 u6 = __ldg(reinterpret_cast<const uint4*>(rec) + 6);
  const uint32_t flags = u6.z;
  const uint32_t vb = u5.x;
  const uint32_t fi = u5.y + 3u * t;
  uint32_t v[3];
  float4 c[3], q[3];
  float d[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    v[k] = vb + __ldg(&p.indices[fi + k]);
    q[k] = __ldg(&p.pos[v[k]]);
    c[k] = make_float4(mrow(mvp, 0, q[k].x, q[k].y, q[k].z), mrow(mvp, 1, q[k].x, q[k].y, q[k].z),
                       mrow(mvp, 2, q[k].x, q[k].y, q[k].z), mrow(mvp, 3, q[k].x, q[k].y, q[k].z));
    float ze = zr[3];
    ze = fma_(zr[0], q[k].x, ze);
    ze = fma_(zr[1], q[k].y, ze);
    ze = fma_(zr[2], q[k].z, ze);
    d[k] = -ze;
  }
  const float sx = __fdiv_rn(float(2 * px + 1 - W), float(W));
  const float sy = __fdiv_rn(float(2 * py + 1 - H), float(H));
  float l[3], ex[3], ey[3], ez[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float4 a = c[(i + 1) % 3];
    const float4 b = c[(i + 2) % 3];
    ex[i] = __fsub_rn(__fmul_rn(a.y, b.w), __fmul_rn(a.w, b.y));
    ey[i] = __fsub_rn(__fmul_rn(a.w, b.x), __fmul_rn(a.x, b.w));
    ez[i] = __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x));
    l[i] = fma_(ex[i], sx, fma_(ey[i], sy, ez[i]));
  }
  const float s = __fadd_rn(__fadd_rn(l[0], l[1]), l[2]);
  const float inv = __frcp_rn(s);
  const float b0 = __fmul_rn(l[0], inv), b1 = __fmul_rn(l[1], inv), b2 = __fmul_rn(l[2], inv);
#define GBR_INTERP(a0, a1, a2) fma_(b2, (a2), fma_(b1, (a1), __fmul_rn(b0, (a0))))
  lin = GBR_INTERP(d[0], d[1], d[2]);
  float vc[4] = {1.0f, 1.0f, 1.0f, 1.0f};
  if (flags & kMeshVertexColor) {
    const float4 c0 = __ldg(&p.color[v[0]]), c1 = __ldg(&p.color[v[1]]),
                 c2 = __ldg(&p.color[v[2]]);
    vc[0] = GBR_INTERP(c0.x, c1.x, c2.x);
    vc[1] = GBR_INTERP(c0.y, c1.y, c2.y);
    vc[2] = GBR_INTERP(c0.z, c1.z, c2.z);
    vc[3] = GBR_INTERP(c0.w, c1.w, c2.w);
  }
  const uint32_t mi = u5.w;
  const MaterialRec& mat = p.materials[mi];
  float tc[4] = {1.0f, 1.0f, 1.0f, 1.0f};
  const int tex = mat.texture;
  if (!(p.flags & 1u) && tex > 0 && tex < p.texture_count) {
    float u = 0.0f, w = 0.0f;
    float2 t0 = make_float2(0.0f, 0.0f), t1 = t0, t2 = t0;
    if (flags & kMeshTexcoords) {
      t0 = __ldg(&p.uv[v[0]]);
      t1 = __ldg(&p.uv[v[1]]);
      t2 = __ldg(&p.uv[v[2]]);
      u = GBR_INTERP(t0.x, t1.x, t2.x);
      w = GBR_INTERP(t0.y, t1.y, t2.y);
    }
    float ts = mat.m[6];
    ts = fma_(mat.m[0], u, ts);
    ts = fma_(mat.m[3], w, ts);
    float tt = mat.m[7];
    tt = fma_(mat.m[1], u, tt);
    tt = fma_(mat.m[4], w, tt);
    const TextureRec& tr = p.textures[tex];
    if (Mode == 0 || (tr.mip_filter == 0 && tr.min_filter == tr.filter)) {
      sample(tr, p.texels, mat.layer, ts, tt, tc);
    } else if (Mode == 1) {
      return false;
    } else {
      // Level of detail from the derivatives of the level-0 texel coordinates
      // across the pixel's 2x2 quad: the quad's pixel pair in this row (x)
      // and in this column (y), each evaluated like the pixel itself.
      auto st_at = [&](int x, int y, float& os, float& ot) {
        const float qx = __fdiv_rn(float(2 * x + 1 - W), float(W));
        const float qy = __fdiv_rn(float(2 * y + 1 - H), float(H));
        const float a0 = fma_(ex[0], qx, fma_(ey[0], qy, ez[0]));
        const float a1 = fma_(ex[1], qx, fma_(ey[1], qy, ez[1]));
        const float a2 = fma_(ex[2], qx, fma_(ey[2], qy, ez[2]));
        const float is = __frcp_rn(__fadd_rn(__fadd_rn(a0, a1), a2));
        const float c0 = __fmul_rn(a0, is), c1 = __fmul_rn(a1, is), c2 = __fmul_rn(a2, is);
        const float uu = fma_(c2, t2.x, fma_(c1, t1.x, __fmul_rn(c0, t0.x)));
        const float ww = fma_(c2, t2.y, fma_(c1, t1.y, __fmul_rn(c0, t0.y)));
        os = fma_(mat.m[3], ww, fma_(mat.m[0], uu, mat.m[6]));
        ot = fma_(mat.m[4], ww, fma_(mat.m[1], uu, mat.m[7]));
      };
      float sa, ta, sb, tb, sc, tcc, sd, td;
      st_at(px & ~1, py, sa, ta);
      st_at((px & ~1) + 1, py, sb, tb);
      st_at(px, py & ~1, sc, tcc);
      st_at(px, (py & ~1) + 1, sd, td);
      const float fw = float(tr.width), fh = float(tr.height);
      const float dux = __fmul_rn(__fsub_rn(sb, sa), fw), dvx = __fmul_rn(__fsub_rn(tb, ta), fh);
      const float duy = __fmul_rn(__fsub_rn(sd, sc), fw), dvy = __fmul_rn(__fsub_rn(td, tcc), fh);
      const float rx = __fsqrt_rn(__fadd_rn(__fmul_rn(dux, dux), __fmul_rn(dvx, dvx)));
      const float ry = __fsqrt_rn(__fadd_rn(__fmul_rn(duy, duy), __fmul_rn(dvy, dvy)));
      const float rho = fmaxf(rx, ry);
      const float lambda = rho > 0.0f ? (rho < 3.0e38f ? series_log2(rho) : 128.0f) : -1.0f;
      sample_lod(tr, p.texels, mat.layer, ts, tt, lambda, tc);
    }
  }
#undef GBR_INTERP
  if (p.max_lights > 0 && mat.phong) {
    color = lit_color(p.normals, p.ambient_factor, mat, make_float4(tc[0], tc[1], tc[2], tc[3]),
                      make_float4(vc[0], vc[1], vc[2], vc[3]), lights, nl, model, v[0], v[1], v[2], q[0],
                      q[1], q[2], b0, b1, b2, (flags & kMeshNormals) != 0u);
  } else {
    uint32_t packed = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float val = __fmul_rn(__fmul_rn(mat.color[k], tc[k]), vc[k]);
      packed |= unorm8(val) << (8 * k);
    }
    color = packed;
  }
  sid = (flags & kMeshObjectId) ? __float_as_uint(__ldg(&p.pos[v[2]]).w) : u6.x;
  return true;
}

// Largest k in [0, n) with order[k].y (first cluster in processing order) <= g.
__device__ __forceinline__ uint32_t find_cluster_draw(const uint2* order, uint32_t n, uint32_t g) {
  uint32_t lo = 0, hi = n;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(&order[mid].y) <= g)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// Culling of a 32-triangle chunk or a 1024-triangle cluster by its
// object-space box, decided by the thread that owns it.  Rejected when
//  * frustum: all eight corners lie beyond one clip plane (outcode margins);
//  * region: the box projects (two pixels of margin) outside the region;
//  * occlusion: every fragment it could produce loses the depth test against
//    what the z-buffer already holds -- the box lies in front of the camera,
//    and its nearest window depth, minus a margin far above the rounding of
//    either computation, is beyond the deepest value of every depth tile its
//    projection (plus one pixel) touches.  Depths only decrease, so the
//    chunk stays hidden.
// Every test is conservative: a rejected chunk has no fragment in the final
// image.
__device__ __forceinline__ bool chunk_keep(const float* mvp, const ChunkBox& b, const Ctx& c,
                                           bool frustum, bool region, const uint32_t* tiles,
                                           const uint32_t* coarse, int tcols, int ccols) {
  uint32_t all_out = 0x3fu;
  bool all_w = true, front = true;
  float x0 = 3.0e38f, x1 = -3.0e38f, y0 = 3.0e38f, y1 = -3.0e38f, zmin = 3.0e38f;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const float x = (k & 1) ? b.hi[0] : b.lo[0], y = (k & 2) ? b.hi[1] : b.lo[1],
                z = (k & 4) ? b.hi[2] : b.lo[2];
    const float cx = mrow(mvp, 0, x, y, z), cy = mrow(mvp, 1, x, y, z), cz = mrow(mvp, 2, x, y, z),
                cw = mrow(mvp, 3, x, y, z);
    const float ax = 1e-5f * (fabsf(cx) + fabsf(cw)), ay = 1e-5f * (fabsf(cy) + fabsf(cw)),
                az = 1e-5f * (fabsf(cz) + fabsf(cw));
    uint32_t out = 0;
    out |= (cx - cw > ax) ? 1u : 0u;
    out |= (-cx - cw > ax) ? 2u : 0u;
    out |= (cy - cw > ay) ? 4u : 0u;
    out |= (-cy - cw > ay) ? 8u : 0u;
    out |= (cz - cw > az) ? 16u : 0u;
    out |= (-cz - cw > az) ? 32u : 0u;
    all_out &= out;
    if (cw > 1e-6f && cw < 1e30f) {
      // An approximate reciprocal (relative error ~2^-22; w is bounded so it
      // cannot underflow): the decisions below compare against margins of
      // 1-2 pixels and 4e-6 in depth, far above the error it adds at values
      // near those thresholds.
      const float iw = __fdividef(1.0f, cw);
      const float sx = (cx * iw * 0.5f + 0.5f) * float(c.W);
      const float sy = (cy * iw * 0.5f + 0.5f) * float(c.H);
      x0 = fminf(x0, sx);
      x1 = fmaxf(x1, sx);
      y0 = fminf(y0, sy);
      y1 = fmaxf(y1, sy);
      zmin = fminf(zmin, cz * iw * 0.5f + 0.5f);
      front = front && cz >= -cw;
    } else {
      all_w = false;
    }
  }
  if (frustum && all_out) return false;
  if (!all_w) return true;
  if (region && (x1 + 2.0f < float(c.rx0) || x0 - 2.0f > float(c.rx0 + c.rw) ||
                 y1 + 2.0f < float(c.ry0) || y0 - 2.0f > float(c.ry0 + c.rh)))
    return false;
  if (!tiles || !front) return true;
  zmin -= 4e-6f;
  if (!(zmin > 0.0f)) return true;
  // Pixel range of the box in region coordinates, one pixel of margin.
  const float fx0 = fmaxf(x0 - 1.0f - float(c.rx0), 0.0f), fy0 = fmaxf(y0 - 1.0f - float(c.ry0), 0.0f);
  const float fx1 = fminf(x1 + 1.0f - float(c.rx0), float(c.rw - 1));
  const float fy1 = fminf(y1 + 1.0f - float(c.ry0), float(c.rh - 1));
  if (!(fx0 <= fx1 && fy0 <= fy1)) return false;  // no pixel of the region
  const uint32_t zbits = __float_as_uint(zmin);
  int tx0 = int(fx0) / kTile, tx1 = int(fx1) / kTile, ty0 = int(fy0) / kTile, ty1 = int(fy1) / kTile;
  const uint32_t* t = tiles;
  int cols = tcols;
  if ((tx1 - tx0 + 1) * (ty1 - ty0 + 1) > 16) {  // large footprint: coarse tiles
    tx0 /= kCoarse;
    tx1 /= kCoarse;
    ty0 /= kCoarse;
    ty1 /= kCoarse;
    t = coarse;
    cols = ccols;
  }
  for (int ty = ty0; ty <= ty1; ++ty)
    for (int tx = tx0; tx <= tx1; ++tx)
      if (t[ty * cols + tx] >= zbits) return true;
  return false;
}

template <int T, bool Lod>
__global__ void __launch_bounds__(T, 1024 / T) raster_kernel(const RasterParams p) {
  extern __shared__ __align__(16) unsigned char smem[];
  const SmemLayout L = smem_layout(T, p.region_px, p.prefix_cap);
  uint64_t* keys = reinterpret_cast<uint64_t*>(smem);
  QEntry* queue = reinterpret_cast<QEntry*>(smem + L.queue);
  uint32_t* qoff = reinterpret_cast<uint32_t*>(smem + L.qoff);
  uint32_t* prefix = reinterpret_cast<uint32_t*>(smem + L.prefix);
  uint2* chunks = reinterpret_cast<uint2*>(smem + L.chunks);
  uint2* cring = reinterpret_cast<uint2*>(smem + L.clusters);
  uint32_t* tiles = reinterpret_cast<uint32_t*>(smem + L.tiles);
  uint32_t* coarse = reinterpret_cast<uint32_t*>(smem + L.coarse);
  __shared__ uint32_t s_item, s_qcount, s_total, s_rd, s_wr, s_crd, s_cwr, s_next;
  __shared__ uint32_t s_warp[T / 32];
  const uint32_t item_count = p.item_count_dev ? min(p.item_count, *p.item_count_dev) : p.item_count;

  for (uint32_t iter = 0;; ++iter) {
    __syncthreads();
    if (threadIdx.x == 0)
      s_item = p.persistent ? atomicAdd(p.counter, 1u) : (iter == 0 ? blockIdx.x : item_count);
    __syncthreads();
    const uint32_t item = s_item;
    if (item >= item_count) return;
    const WorkItem wi = p.items[p.item_base + item];
    const uint32_t vis_base = p.cameras[wi.scene].vis_base;
    if (!p.cameras[wi.scene].enabled) continue;  // disabled scene: pixels untouched
    const SceneRec sc = p.scenes[wi.scene];
    Ctx c;
    c.keys = keys;
    c.queue = queue;
    c.spill = p.spill ? static_cast<QEntry*>(p.spill) + size_t(blockIdx.x) * T : nullptr;
    c.qcount = &s_qcount;
    c.qcap = T;
    c.rx0 = wi.x0;
    c.ry0 = wi.y0;
    c.rw = wi.w;
    c.rh = wi.h;
    set_viewport(c, sc.width, sc.height);
    c.small_area = p.small_area;
    const int npx = c.rw * c.rh;
    for (int i = threadIdx.x; i < npx; i += T) keys[i] = kEmptyKey;
    const uint32_t nvis = p.vis_count[wi.scene];
    const uint32_t total = p.vis_tris[wi.scene];
    const VisibleRec* vis = p.visible + vis_base;
    const bool cached = nvis <= uint32_t(p.prefix_cap);
    if (cached)
      for (uint32_t i = threadIdx.x; i < nvis; i += T) prefix[i] = vis[i].ordinal;
    if (threadIdx.x == 0) s_qcount = 0;
    __syncthreads();

    // Clusters (1024 triangles) and chunks (32 triangles) of the visible
    // draws, in processing order (nearest draws first).  Cull passes test
    // boxes with chunk_keep (frustum, region, occlusion against the depth
    // tiles): a cluster pass tests one cluster per thread and appends the
    // survivors to the cluster ring; a chunk pass gives each warp one
    // surviving cluster, tests its 32 chunks (one per lane) and appends the
    // survivors to the chunk ring.  Rounds: each warp takes one chunk of the
    // ring and its lanes set up one triangle each; triangles covering more
    // than small_area pixels are queued.  The queue is rasterised by the
    // whole CTA (flush) once it holds flush_at entries, before a cull pass and at the
    // end.  A cull pass runs whenever fewer chunks than warps wait in the
    // chunk ring, after the depth tiles are refreshed from the z-buffer.
    const uint32_t nclusters = p.vis_clusters[wi.scene];
    const uint2* order = p.order + vis_base;
    const bool whole = c.rw == c.W && c.rh == c.H;
    const bool occlusion = p.occlusion && p.boxes;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int tcols = (c.rw + kTile - 1) / kTile, trows = (c.rh + kTile - 1) / kTile;
    const int ccols = (tcols + kCoarse - 1) / kCoarse, crows = (trows + kCoarse - 1) / kCoarse;
    c.tiles = occlusion ? tiles : nullptr;  // filled by the first cull pass, before any round
    c.coarse = coarse;
    c.tcols = tcols;
    c.ccols = ccols;
    if (threadIdx.x == 0) {
      s_rd = s_wr = s_crd = s_cwr = s_next = 0;
    }
    (void)total;
    bool tiles_stale = true;  // uniform: the z-buffer changed since the last refresh
    __syncthreads();
    for (;;) {
      const uint32_t rd = s_rd, wr = s_wr, crd = s_crd, cwr = s_cwr, next = s_next,
                     queued = min(s_qcount, uint32_t(c.spill ? 2 * T : T)),
                     nq = min(queued, uint32_t(T));
      __syncthreads();  // everyone has read the counters
      const bool low = wr - rd < uint32_t(T / 32);
      const bool clusters_left = next < nclusters, have_clusters = cwr != crd;
      const bool need_cull = low && (clusters_left || have_clusters);
      // A round adds at most T entries to fewer than flush_at <= T: the queue and the
      // spill area (T each) hold them.
      if (nq > 0 && (nq >= p.flush_at || need_cull || wr == rd)) {
        // ---- flush: every thread takes a contiguous run of the queued
        // triangles' bounding-box pixels.
        uint32_t area = 0;
        if (threadIdx.x < nq) {
          const QEntry& e = queue[threadIdx.x];
          area = uint32_t(e.x1 - e.x0 + 1) * uint32_t(e.y1 - e.y0 + 1);
        }
        const uint32_t off = block_exclusive_scan<T>(area, s_warp, &s_total);
        const uint32_t tot = s_total;
        if (threadIdx.x < nq) qoff[threadIdx.x] = off;
        if (threadIdx.x == 0) qoff[nq] = tot;
        __syncthreads();
        const uint32_t per = (tot + T - 1) / T;
        const uint32_t q0 = min(tot, threadIdx.x * per), q1 = min(tot, q0 + per);
        if (q0 < q1) {
          uint32_t lo = 0, hi = nq;  // entry holding pixel q0: qoff[lo] <= q0 < qoff[lo + 1]
          while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (qoff[mid] <= q0)
              lo = mid;
            else
              hi = mid;
          }
          const QEntry* e = &queue[lo];
          int w = e->x1 - e->x0 + 1;
          int px = e->x0 + int(q0 - qoff[lo]) % w, py = e->y0 + int(q0 - qoff[lo]) / w;
          uint32_t end = qoff[lo + 1];
          for (uint32_t q = q0; q < q1; ++q) {
            if (q == end) {  // next entry (areas are >= 1, so one step)
              ++lo;
              e = &queue[lo];
              w = e->x1 - e->x0 + 1;
              px = e->x0;
              py = e->y0;
              end = qoff[lo + 1];
            }
            float z;
            if (cover(e->X, e->Y, e->bias, e->zw0, e->d1, e->d2, e->inva, px, py, z))
              depth_write(keys, (py - c.ry0) * c.rw + (px - c.rx0), z, e->ordinal);
            if (++px > e->x1) {
              px = e->x0;
              ++py;
            }
          }
        }
        if (threadIdx.x == 0) s_qcount = 0;
        tiles_stale = true;
        __syncthreads();
        if (queued > nq) {
          // A round queued more than the shared queue holds: the rest went to
          // this CTA's spill area; move it into the emptied queue.
          for (uint32_t i = threadIdx.x; i < queued - nq; i += T) queue[i] = c.spill[i];
          if (threadIdx.x == 0) s_qcount = queued - nq;
          __syncthreads();
        }
        continue;
      }
      if (need_cull) {
        if (occlusion && tiles_stale) {
          // Deepest depth (as ordered bits; empty pixels are all ones) of
          // each tile and coarse tile; pixels outside the region count as 0.
          // One warp per coarse tile: lane x reads column x of its 32 rows
          // (a warp reads 32 consecutive keys, free of bank conflicts), every
          // 8 rows groups of 8 lanes give the 4 tiles of that band, and the
          // whole warp gives the coarse tile.
          for (int u = warp; u < ccols * crows; u += T / 32) {
            const int x = (u % ccols) * (kTile * kCoarse) + lane, y0 = (u / ccols) * (kTile * kCoarse);
            uint32_t band = 0, all = 0;
            for (int r = 0; r < kTile * kCoarse && y0 + r < c.rh; ++r) {
              if (x < c.rw) band = max(band, uint32_t(keys[(y0 + r) * c.rw + x] >> 32));
              if ((r & (kTile - 1)) == kTile - 1 || y0 + r == c.rh - 1) {
                uint32_t b = band;
                b = max(b, __shfl_xor_sync(0xffffffffu, b, 1));
                b = max(b, __shfl_xor_sync(0xffffffffu, b, 2));
                b = max(b, __shfl_xor_sync(0xffffffffu, b, 4));
                const int tx = (u % ccols) * kCoarse + (lane >> 3), ty = (y0 + r) / kTile;
                if ((lane & 7) == 0 && tx < tcols) tiles[ty * tcols + tx] = b;
                all = max(all, band);
                band = 0;
              }
            }
            all = __reduce_max_sync(0xffffffffu, all);
            if (lane == 0) coarse[u] = all;
          }
          __syncthreads();
          tiles_stale = false;
        }
        if (have_clusters && (cwr - crd >= uint32_t(T / 32) || !clusters_left)) {
          // ---- chunk pass: warp w tests the chunks of surviving cluster w.
          const uint32_t n = min(cwr - crd, uint32_t(T / 32));
          bool keep = false;
          uint2 out = make_uint2(0u, 0u);
          if (uint32_t(warp) < n) {
            const uint2 cl = cring[(crd + warp) & (kClusterRing - 1)];  // (draw, cluster in draw)
            const VisibleRec* rec = vis + cl.x;
            const uint32_t nch = __ldg(&rec->chunk_count);
            const uint32_t chunk = cl.y * kClusterChunks + lane;
            if (chunk < nch) {
              keep = true;
              const bool inside = __ldg(&rec->flags) & kDrawInsideFrustum;
              if (p.boxes && (occlusion || !(inside && whole))) {
                float mvp[16];
                const float4* m4 = reinterpret_cast<const float4*>(rec->mvp);
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                  const float4 v = __ldg(m4 + i);
                  mvp[4 * i] = v.x;
                  mvp[4 * i + 1] = v.y;
                  mvp[4 * i + 2] = v.z;
                  mvp[4 * i + 3] = v.w;
                }
                keep = chunk_keep(mvp, p.boxes[__ldg(&rec->box_base) + chunk], c, !inside, !whole,
                                  occlusion ? tiles : nullptr, coarse, tcols, ccols);
              }
              out = make_uint2(cl.x, chunk);
            }
          }
          const uint32_t pos = block_exclusive_scan<T>(keep ? 1u : 0u, s_warp, &s_total);
          if (keep) chunks[(wr + pos) & (ring_capacity(T) - 1)] = out;
          if (threadIdx.x == 0) {
            s_wr = wr + s_total;
            s_crd = crd + n;
          }
        } else {
          // ---- cluster pass: one cluster per thread, as many as the ring holds.
          const uint32_t m = min(min(uint32_t(T), kClusterRing - (cwr - crd)), nclusters - next);
          const uint32_t g = next + threadIdx.x;
          bool keep = false;
          uint2 od = make_uint2(0u, 0u);
          if (threadIdx.x < m) {
            const uint32_t k = find_cluster_draw(order, nvis, g);
            od = __ldg(&order[k]);
            const VisibleRec* rec = vis + od.x;
            const bool inside = __ldg(&rec->flags) & kDrawInsideFrustum;
            keep = true;
            if (p.boxes && (occlusion || !(inside && whole))) {
              float mvp[16];
              const float4* m4 = reinterpret_cast<const float4*>(rec->mvp);
#pragma unroll
              for (int i = 0; i < 4; ++i) {
                const float4 v = __ldg(m4 + i);
                mvp[4 * i] = v.x;
                mvp[4 * i + 1] = v.y;
                mvp[4 * i + 2] = v.z;
                mvp[4 * i + 3] = v.w;
              }
              const uint32_t nch = __ldg(&rec->chunk_count);
              keep = chunk_keep(mvp, p.boxes[__ldg(&rec->box_base) + nch + (g - od.y)], c, !inside,
                                !whole, occlusion ? tiles : nullptr, coarse, tcols, ccols);
            }
          }
          const uint32_t pos = block_exclusive_scan<T>(keep ? 1u : 0u, s_warp, &s_total);
          if (keep) cring[(cwr + pos) & (kClusterRing - 1)] = make_uint2(od.x, g - od.y);
          if (threadIdx.x == 0) {
            s_cwr = cwr + s_total;
            s_next = next + m;
          }
        }
        __syncthreads();
        continue;
      }
      if (wr == rd) break;  // every chunk culled or drawn

      // ---- round: each warp takes chunks from the ring, one at a time, until
      // the ring is empty or the queue holds flush_at entries
      // (a chunk adds at most 32 triangles, or a few more when clipped; the
      // spill area and, beyond it, rasterisation by the lane itself take the
      // excess).  Chunks are claimed by compare-and-swap, so the read position
      // never passes the ring's write position.
      for (;;) {
        uint32_t slot = wr;
        if (lane == 0 && *reinterpret_cast<volatile uint32_t*>(&s_qcount) < p.flush_at) {
          uint32_t cur = *reinterpret_cast<volatile uint32_t*>(&s_rd);
          while (cur < wr) {
            const uint32_t prev = atomicCAS(&s_rd, cur, cur + 1u);
            if (prev == cur) {
              slot = cur;
              break;
            }
            cur = prev;
          }
        }
        slot = __shfl_sync(0xffffffffu, slot, 0);
        if (slot >= wr) break;
        const uint2 ch = chunks[slot & (ring_capacity(T) - 1)];
        const VisibleRec* rec = vis + ch.x;
        const uint32_t t = ch.y * kChunkTris + lane;
        if (t < __ldg(&rec->tri_count)) {
          float mvp[16];
          const float4* m4 = reinterpret_cast<const float4*>(rec->mvp);
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const float4 v = __ldg(m4 + i);
            mvp[4 * i] = v.x;
            mvp[4 * i + 1] = v.y;
            mvp[4 * i + 2] = v.z;
            mvp[4 * i + 3] = v.w;
          }
          const uint32_t vb = __ldg(&rec->vertex_base);
          const uint32_t fi = __ldg(&rec->first_index) + 3u * t;
          float4 cv[3];
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            const float4 q = __ldg(&p.pos[vb + __ldg(&p.indices[fi + k])]);
            cv[k] = make_float4(mrow(mvp, 0, q.x, q.y, q.z), mrow(mvp, 1, q.x, q.y, q.z),
                                mrow(mvp, 2, q.x, q.y, q.z), mrow(mvp, 3, q.x, q.y, q.z));
          }
          triangle(cv, __ldg(&rec->ordinal) + t, c);
        }
      }
      tiles_stale = true;
      __syncthreads();
    }
    __syncthreads();

    // Resolve + shade + write the planes.
    const uint32_t nlights =
        p.lights ? min(p.cameras[p.cameras[wi.scene].source].light_count, p.max_lights) : 0u;
    const WorldLight* lights = p.lights ? p.lights + size_t(wi.scene) * p.max_lights : nullptr;
    // Pixels whose texture needs a level of detail are marked in their key
    // (bit 63: depth bits of a drawn pixel are below 0x3f800000) and shaded in
    // a second loop by the same thread.
    constexpr uint64_t kDeferred = 1ull << 63;
    bool deferred = false;
    for (int i = threadIdx.x; i < npx; i += T) {
      const int px = c.rx0 + i % c.rw, py = c.ry0 + i / c.rw;
      const uint64_t key = keys[i];
      const int64_t o = sc.fb_offset + int64_t(py) * sc.pitch + px;
      uint32_t col = kBackground, sid = 0;
      float dep = 1.0f, lin = 0.0f;
      if (key != kEmptyKey) {
        const uint32_t ord = uint32_t(key);
        dep = __uint_as_float(uint32_t(key >> 32));
        const uint32_t di = find_draw(prefix, vis, cached, nvis, ord);
        if (!shade<Lod ? 1 : 0>(p, c.W, c.H, vis + di, ord - __ldg(&vis[di].ordinal), px, py,
                                lights, nlights, p.model ? p.model + vis_base + di : nullptr, col, lin, sid)) {
          keys[i] = key | kDeferred;
          deferred = true;
          continue;
        }
      }
      if (p.out.color) p.out.color[o] = col;
      if (p.out.depth) p.out.depth[o] = dep;
      if (p.out.linear) p.out.linear[o] = lin;
      if (p.out.semantic) p.out.semantic[o] = sid;
    }
    if (Lod && __syncthreads_or(deferred)) {
      for (int i = threadIdx.x; i < npx; i += T) {
        const uint64_t key = keys[i];
        if (key == kEmptyKey || !(key & kDeferred)) continue;
        const int px = c.rx0 + i % c.rw, py = c.ry0 + i / c.rw;
        const int64_t o = sc.fb_offset + int64_t(py) * sc.pitch + px;
        const uint32_t ord = uint32_t(key);
        const float dep = __uint_as_float(uint32_t((key & ~kDeferred) >> 32));
        const uint32_t di = find_draw(prefix, vis, cached, nvis, ord);
        uint32_t col, sid;
        float lin;
        shade<2>(p, c.W, c.H, vis + di, ord - __ldg(&vis[di].ordinal), px, py, lights, nlights,
                 p.model ? p.model + vis_base + di : nullptr, col, lin, sid);
        if (p.out.color) p.out.color[o] = col;
        if (p.out.depth) p.out.depth[o] = dep;
        if (p.out.linear) p.out.linear[o] = lin;
        if (p.out.semantic) p.out.semantic[o] = sid;
      }
    }
  }
}

__global__ void unproject_kernel(float a, float b, float* depth, uint64_t rows, uint64_t cols,
                                 uint64_t stride) {
  const float far_depth = __fdiv_rn(b, __fadd_rn(1.0f, a));
  const uint64_t n = rows * cols;
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n;
       i += uint64_t(gridDim.x) * blockDim.x) {
    float& d = depth[(i / cols) * stride + (i % cols)];
    const float v = __fdiv_rn(b, __fadd_rn(d, a));
    d = v == far_depth ? 0.0f : v;
  }
}

// Tiles of a plane packed one after another: scene i of the tile grid
// (tile (i % tiles_x, i / tiles_x), w x h elements of 4 bytes) goes to
// dst[i * w * h ...], rows kept in order.  One thread per 16 bytes when the
// rows are 16-byte multiples, else per element.
template <int Vec>
__global__ void gather_tiles_kernel(const uint32_t* __restrict__ src, int64_t pitch, int w, int h,
                                    int tiles_x, uint32_t first, uint64_t units, uint32_t* dst) {
  const int per_row = w / Vec;
  for (uint64_t u = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; u < units;
       u += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t row = u / per_row;            // scene-major rows
    const int c = int(u % per_row) * Vec;
    const uint32_t scene = first + uint32_t(row / h);
    const int y = int(row % h);
    const int64_t sx = int64_t(scene % uint32_t(tiles_x)) * w, sy = int64_t(scene / uint32_t(tiles_x)) * h;
    const uint32_t* from = src + (sy + y) * pitch + sx + c;
    uint32_t* to = dst + row * uint64_t(w) + c;
    if (Vec == 4)
      *reinterpret_cast<uint4*>(to) = __ldg(reinterpret_cast<const uint4*>(from));
    else
      *to = __ldg(from);
  }
}

}  // namespace

cudaError_t launch_gather_tiles(const void* src, int64_t pitch, int w, int h, int tiles_x, uint32_t first,
                                uint32_t count, void* dst, cudaStream_t stream) {
  const bool vec = (w % 4 == 0) && (pitch % 4 == 0) && (reinterpret_cast<uintptr_t>(src) % 16 == 0) &&
                   (reinterpret_cast<uintptr_t>(dst) % 16 == 0);
  const uint64_t units = uint64_t(count) * h * (vec ? w / 4 : w);
  if (units == 0) return cudaSuccess;
  const unsigned blocks = unsigned(std::min<uint64_t>((units + 255) / 256, 152ull * 32));
  if (vec)
    gather_tiles_kernel<4><<<blocks, 256, 0, stream>>>(static_cast<const uint32_t*>(src), pitch, w, h,
                                                       tiles_x, first, units, static_cast<uint32_t*>(dst));
  else
    gather_tiles_kernel<1><<<blocks, 256, 0, stream>>>(static_cast<const uint32_t*>(src), pitch, w, h,
                                                       tiles_x, first, units, static_cast<uint32_t*>(dst));
  return cudaGetLastError();
}

cudaError_t launch_prepare(const PrepareParams& p, uint32_t scene_count, cudaStream_t stream) {
  if (scene_count == 0) return cudaSuccess;
  prepare_kernel<128><<<scene_count, 128, 0, stream>>>(p);
  return cudaGetLastError();
}

size_t raster_smem_bytes(int threads, int region_px, int prefix_cap) {
  return smem_layout(threads, region_px, prefix_cap).total;
}

size_t raster_spill_bytes(int threads, uint32_t grid) {
  return size_t(grid) * size_t(threads) * sizeof(QEntry);
}

#define GBR_RASTER_SWITCH(threads, F) \
  switch (threads) {                  \
    case 256: F(256); break;          \
    case 512: F(512); break;          \
    case 1024: F(1024); break;        \
    default: return cudaErrorInvalidValue; \
  }

cudaError_t raster_configure(int threads, size_t* max_dynamic, size_t* static_bytes) {
  int optin = 0, dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
#define GBR_CFG(T)                                                                             \
  {                                                                                            \
    cudaFuncAttributes fa;                                                                     \
    e = cudaFuncGetAttributes(&fa, raster_kernel<T, false>);                                   \
    if (e != cudaSuccess) return e;                                                            \
    const size_t dyn = size_t(optin) > fa.sharedSizeBytes ? size_t(optin) - fa.sharedSizeBytes : 0; \
    e = cudaFuncSetAttribute(raster_kernel<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                             int(dyn));                                                        \
    if (e != cudaSuccess) return e;                                                            \
    e = cudaFuncSetAttribute(raster_kernel<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                             int(dyn));                                                        \
    if (e != cudaSuccess) return e;                                                            \
    *max_dynamic = dyn;                                                                        \
    *static_bytes = fa.sharedSizeBytes;                                                        \
  }
  GBR_RASTER_SWITCH(threads, GBR_CFG)
#undef GBR_CFG
  return cudaSuccess;
}

cudaError_t raster_max_ctas_per_sm(int threads, size_t smem, int* out) {
#define GBR_OCC(T)                                                                                \
  {                                                                                               \
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, raster_kernel<T, false>, T, smem); \
    if (e != cudaSuccess) return e;                                                               \
  }
  GBR_RASTER_SWITCH(threads, GBR_OCC)
#undef GBR_OCC
  return cudaSuccess;
}

cudaError_t launch_raster(const RasterParams& p, int threads, uint32_t grid, size_t smem,
                          cudaStream_t stream) {
  if (grid == 0) return cudaSuccess;
#define GBR_LAUNCH(T)                                           \
  if (p.any_lod)                                                \
    raster_kernel<T, true><<<grid, T, smem, stream>>>(p);       \
  else                                                          \
    raster_kernel<T, false><<<grid, T, smem, stream>>>(p);
  GBR_RASTER_SWITCH(threads, GBR_LAUNCH)
#undef GBR_LAUNCH
  return cudaGetLastError();
}

cudaError_t launch_unproject(float a, float b, float* depth, uint64_t rows, uint64_t cols,
                             uint64_t row_stride, cudaStream_t stream) {
  const uint64_t n = rows * cols;
  if (n == 0) return cudaSuccess;
  uint64_t blocks = (n + 255) / 256;
  if (blocks > 65535) blocks = 65535;
  unproject_kernel<<<unsigned(blocks), 256, 0, stream>>>(a, b, depth, rows, cols, row_stride);
  return cudaGetLastError();
}

}  // namespace gbr

// ======================================================================
// Rendering one mesh without allocating device memory.
//
// For callers that must not allocate: code running inside another
// framework's memory pool or under a strict device-memory budget, real-time
// loops where an allocation could stall or fail, and plugins whose host
// application owns every allocation.  They pass their own device buffers for
// the mesh and the output planes; the few hundred bytes of per-call scratch
// this path needs (scene and visible-draw records, the work-item list and
// counter of the persistent raster kernel, a bad-index flag) live in the
// fixed array below, which every GPU that loads this library keeps until
// the process exits.
// ======================================================================
#include <algorithm>
#include <mutex>
#include <string>

#include "../../include/gbr.h"

namespace gbr {
void set_last_error(const std::string& msg);
void mat4_mul(const float* a, const float* b, float* c);

namespace {

constexpr int kNoAllocMaxSide = 4096;  // largest viewport side the scratch can tile
constexpr int kNoAllocRegion = 128;    // region side of one work item
constexpr int kNoAllocMaxItems =
    (kNoAllocMaxSide / kNoAllocRegion) * (kNoAllocMaxSide / kNoAllocRegion);
constexpr size_t kNoAllocScratchBytes = 16384;
constexpr uint32_t kNoAllocMaxTriangles = 0xFFFFFFFFu / 3;
constexpr int kNoAllocMaxDevices = 64;

struct NoAllocScratch {
  CameraRec camera;
  uint2 order;
  SceneRec scene;
  VisibleRec visible;
  MaterialRec material;
  uint32_t vis_count, vis_tris, vis_clusters, counter, bad_index;
  WorkItem items[kNoAllocMaxItems];
};
static_assert(sizeof(NoAllocScratch) <= kNoAllocScratchBytes, "no-alloc scratch too small");

// The scratch.  Shared by every call on a device; calls that overlap on the
// GPU (different streams, no ordering between them) race on it.
static __device__ __align__(256) unsigned char g_no_alloc_scratch[kNoAllocScratchBytes];

std::mutex g_no_alloc_mutex;
void* g_no_alloc_ptr[kNoAllocMaxDevices] = {};

__global__ void no_alloc_check_indices(const uint32_t* indices, uint64_t n, uint32_t vertex_count,
                                       NoAllocScratch* s) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n;
       i += uint64_t(gridDim.x) * blockDim.x)
    if (indices[i] >= vertex_count) s->bad_index = 1u;
}

struct NoAllocSetup {
  float pv[16];
  float vrow[4];
  int32_t width, height;
  uint32_t triangles, semantic_id, flags, items;
};

// Fills the scene, visible-draw, material and work-item records and resets
// the work counter (everything the raster kernel must find fresh).
__global__ void no_alloc_setup(const NoAllocSetup a, NoAllocScratch* s) {
  if (threadIdx.x == 0) {
    SceneRec sc{};
    sc.width = a.width;
    sc.height = a.height;
    sc.fb_offset = 0;
    sc.pitch = a.width;
    sc.node_base = 0;
    sc.node_count = 2;
    sc.draw_base = 0;
    sc.draw_count = 1;
    s->scene = sc;
    CameraRec cam{};
    for (int i = 0; i < 16; ++i) cam.pv[i] = a.pv[i];
    for (int i = 0; i < 4; ++i) cam.vrow[i] = a.vrow[i];
    cam.source = 0;
    cam.vis_base = 0;
    cam.enabled = 1;
    s->camera = cam;
    s->order = make_uint2(0u, 0u);
    // The mesh sits under an identity root and an identity child, as a
    // hierarchy added without a bake transform: abs = I * I, MVP = PV * abs.
    float ident[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    float absm[16], mvp[16];
    matmul(ident, ident, absm);
    matmul(a.pv, absm, mvp);
    VisibleRec v{};
    for (int i = 0; i < 16; ++i) v.mvp[i] = mvp[i];
    for (int col = 0; col < 4; ++col) {
      float z = __fmul_rn(a.vrow[0], absm[col * 4 + 0]);
      z = fma_(a.vrow[1], absm[col * 4 + 1], z);
      z = fma_(a.vrow[2], absm[col * 4 + 2], z);
      z = fma_(a.vrow[3], absm[col * 4 + 3], z);
      v.zrow[col] = z;
    }
    const bool ok = s->bad_index == 0u;
    v.vertex_base = 0;
    v.first_index = 0;
    v.tri_count = a.triangles;
    v.material = 0;
    v.semantic_id = a.semantic_id;
    v.ordinal = 0;
    v.flags = a.flags;
    v.cluster = 0;
    v.chunk_count = (a.triangles + kChunkTris - 1) / kChunkTris;
    v.box_base = 0;
    s->visible = v;
    MaterialRec m{};
    m.color[0] = m.color[1] = m.color[2] = m.color[3] = 1.0f;
    m.texture = 0;
    m.layer = 0;
    m.m[0] = m.m[4] = m.m[8] = 1.0f;
    s->material = m;
    s->vis_count = ok && a.triangles ? 1u : 0u;
    s->vis_tris = ok ? a.triangles : 0u;
    s->vis_clusters = ok ? cluster_count((a.triangles + kChunkTris - 1) / kChunkTris) : 0u;
    s->counter = 0u;
  }
  const int cols = (a.width + kNoAllocRegion - 1) / kNoAllocRegion;
  for (uint32_t i = threadIdx.x; i < a.items; i += blockDim.x) {
    WorkItem w{};
    w.scene = 0;
    w.x0 = uint16_t((i % cols) * kNoAllocRegion);
    w.y0 = uint16_t((i / cols) * kNoAllocRegion);
    w.w = uint16_t(min(kNoAllocRegion, a.width - int(w.x0)));
    w.h = uint16_t(min(kNoAllocRegion, a.height - int(w.y0)));
    s->items[i] = w;
  }
}

gbr_status no_alloc_fail(gbr_status s, const std::string& m) {
  set_last_error("gbr_render_mesh_no_alloc: " + m);
  return s;
}

}  // namespace
}  // namespace gbr

extern "C" gbr_status gbr_render_mesh_no_alloc(
    const void* positions, const void* colors, const uint32_t* indices, uint32_t vertex_count,
    uint32_t triangle_count, const float projection[16], const float view[16],
    uint32_t semantic_id, int32_t use_vertex_ids, int32_t width, int32_t height, uint32_t* color,
    float* depth, float* linear_depth, uint32_t* semantic, void* stream) {
  using namespace gbr;
  if (!projection || !view) return no_alloc_fail(GBR_ERROR_INVALID_ARGUMENT, "null camera matrix");
  if (width < 1 || height < 1 || width > kNoAllocMaxSide || height > kNoAllocMaxSide)
    return no_alloc_fail(GBR_ERROR_INVALID_ARGUMENT,
                         "viewport " + std::to_string(width) + "x" + std::to_string(height) +
                             " is outside 1..4096 x 1..4096, the limit of its fixed scratch");
  // The raster kernel addresses index 3 * t + k of the mesh in 32 bits.
  if (triangle_count > kNoAllocMaxTriangles)
    return no_alloc_fail(GBR_ERROR_INVALID_ARGUMENT,
                         std::to_string(triangle_count) + " triangles: more than " +
                             std::to_string(kNoAllocMaxTriangles) +
                             " (3 x triangles indices must be addressable in 32 bits)");
  if (triangle_count && (!positions || !indices || vertex_count == 0))
    return no_alloc_fail(GBR_ERROR_INVALID_ARGUMENT, "positions, indices and vertices are required");
  if ((reinterpret_cast<uintptr_t>(positions) | reinterpret_cast<uintptr_t>(colors)) & 15u)
    return no_alloc_fail(GBR_ERROR_INVALID_ARGUMENT, "positions and colours must be 16-byte aligned");
  if ((reinterpret_cast<uintptr_t>(color) | reinterpret_cast<uintptr_t>(depth) |
       reinterpret_cast<uintptr_t>(linear_depth) | reinterpret_cast<uintptr_t>(semantic) |
       reinterpret_cast<uintptr_t>(indices)) & 3u)
    return no_alloc_fail(GBR_ERROR_INVALID_ARGUMENT, "indices and planes must be 4-byte aligned");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices)
    return no_alloc_fail(GBR_ERROR_CUDA, "no usable current device");
  void* scratch = nullptr;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  {
    // The device address of the fixed scratch (the host-side name of a
    // __device__ array is not a device address).  It belongs to the current
    // context, which a device reset or a caller's own driver-API context
    // replaces, so it is looked up again on every call whose stream is not
    // capturing; the first call on a device must come before any stream
    // capture.
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &capture) != cudaSuccess) {
      cudaGetLastError();
      capture = cudaStreamCaptureStatusActive;  // unknown: do not call into the runtime's symbol table
    }
    std::lock_guard<std::mutex> lock(g_no_alloc_mutex);
    if (capture == cudaStreamCaptureStatusNone) {
      void* ptr = nullptr;
      e = cudaGetSymbolAddress(&ptr, g_no_alloc_scratch);
      if (e != cudaSuccess) {
        cudaGetLastError();
        return no_alloc_fail(GBR_ERROR_CUDA, std::string("cudaGetSymbolAddress: ") +
                                                 cudaGetErrorString(e));
      }
      g_no_alloc_ptr[dev] = ptr;
    } else if (!g_no_alloc_ptr[dev]) {
      return no_alloc_fail(GBR_ERROR_INVALID_ARGUMENT,
                           "the first call on a device must come before any stream capture");
    }
    scratch = g_no_alloc_ptr[dev];
  }
  NoAllocScratch* s = static_cast<NoAllocScratch*>(scratch);
  const int cols = (width + kNoAllocRegion - 1) / kNoAllocRegion;
  const int rows = (height + kNoAllocRegion - 1) / kNoAllocRegion;
  NoAllocSetup a{};
  mat4_mul(projection, view, a.pv);
  for (int k = 0; k < 4; ++k) a.vrow[k] = view[k * 4 + 2];
  a.width = width;
  a.height = height;
  a.triangles = triangle_count;
  a.semantic_id = semantic_id;
  a.flags = (colors ? kMeshVertexColor : 0u) | (use_vertex_ids ? kMeshObjectId : 0u);
  a.items = uint32_t(cols * rows);
  e = cudaMemsetAsync(&s->bad_index, 0, sizeof(uint32_t), st);
  if (e == cudaSuccess && triangle_count) {
    const uint64_t n = uint64_t(triangle_count) * 3;
    const unsigned blocks = unsigned(std::min<uint64_t>((n + 255) / 256, 1024));
    no_alloc_check_indices<<<blocks, 256, 0, st>>>(indices, n, vertex_count, s);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    no_alloc_setup<<<1, 256, 0, st>>>(a, s);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess)
    return no_alloc_fail(GBR_ERROR_CUDA, std::string("setup: ") + cudaGetErrorString(e));
  constexpr int kThreads = 1024;
  size_t max_dyn = 0, static_bytes = 0;
  e = raster_configure(kThreads, &max_dyn, &static_bytes);
  const size_t smem = raster_smem_bytes(kThreads, kNoAllocRegion * kNoAllocRegion, 1);
  int occ = 0, sms = 0;
  if (e == cudaSuccess) e = raster_max_ctas_per_sm(kThreads, smem, &occ);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess || smem > max_dyn || occ < 1)
    return no_alloc_fail(GBR_ERROR_CUDA, "raster kernel configuration failed");
  RasterParams p{};
  p.scenes = &s->scene;
  p.cameras = &s->camera;
  p.order = &s->order;
  p.visible = &s->visible;
  p.vis_count = &s->vis_count;
  p.vis_tris = &s->vis_tris;
  p.vis_clusters = &s->vis_clusters;
  p.boxes = nullptr;
  p.pos = static_cast<const float4*>(positions);
  p.color = static_cast<const float4*>(colors);
  p.uv = nullptr;
  p.indices = indices;
  p.materials = &s->material;
  p.textures = nullptr;
  p.texels = nullptr;
  p.texture_count = 1;
  p.flags = 0;
  p.items = s->items;
  p.item_base = 0;
  p.item_count = a.items;
  p.counter = &s->counter;
  p.persistent = 1;
  p.out.color = color;
  p.out.depth = depth;
  p.out.linear = linear_depth;
  p.out.semantic = semantic;
  p.region_px = kNoAllocRegion * kNoAllocRegion;
  p.prefix_cap = 1;
  p.small_area = 1;
  p.flush_at = 3 * kThreads / 4;
  const uint32_t grid = std::min<uint32_t>(a.items, uint32_t(sms) * uint32_t(occ));
  e = launch_raster(p, kThreads, grid, smem, st);
  if (e != cudaSuccess)
    return no_alloc_fail(GBR_ERROR_CUDA, std::string("raster launch: ") + cudaGetErrorString(e));
  return GBR_OK;
}
