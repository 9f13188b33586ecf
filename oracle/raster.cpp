// CPU oracle for the batch renderer's draw path -- TEST INFRASTRUCTURE ONLY.
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline load this
// library; the product (habitat-sim_gb300/) never does.  It is a sequential,
// forward-shading restatement of what habitat-sim's batch renderer draws:
//
//   * scene graph: abs[i] = abs[parent[i]] * local[i], parents[i] < i
//     (src/esp/gfx_batch/Renderer.cpp:1214-1220); a root's absolute
//     transform is its local transform;
//   * camera: updateCamera stores P*V (Renderer.cpp:1077-1088); the vertex
//     stage is clip = (P*V*abs) * position (PhongGL's projection *
//     transformation, configured at Renderer.cpp:835-860), with the matrix
//     product formed once per draw;
//   * per scene, draws in draw-batch order then add order
//     (Renderer.cpp:1139-1196 counting sort, 1324-1349 submission) -- the
//     caller passes them already sorted;
//   * GL fixed function: clipping at the near plane, back faces culled with
//     CCW front faces (Renderer.cpp:307), depth test LESS against a depth
//     buffer cleared to 1.0 (Renderer.cpp:308, RendererStandalone.cpp:155-159),
//     pixel centres at (x+0.5, y+0.5), window origin bottom-left;
//   * flat shading when no lights are enabled: colour = base colour *
//     texture(layer, M * uv) * vertex colour (Renderer.cpp:579-620), written
//     as RGBA8 with round-to-nearest (see unorm8); background (31,31,31,255)
//     (GfxBatchRendererTest.cpp:1514-1521);
//   * linear depth = perspective-correct interpolation of -z_eye, the method
//     of src/shaders/gfx_batch/depth.vert:15-17, 0 where nothing was drawn
//     (DepthUnprojection.cpp:116-128); window depth as D32F;
//   * lit shading when lights are enabled (max_lights > 0) and the material
//     is not unlit: ambient = colour * ambient factor, diffuse = colour
//     (Renderer.cpp:579-620), both times texture and vertex colour; every
//     light of the scene (at most max_lights, world space from its node:
//     translation for point lights, negative backward axis for directional
//     ones, Renderer.cpp:1263-1289) adds diffuse * light colour * max(0, N.L)
//     * attenuation, attenuation = clamp(1 - (d/range)^4, 0, 1)^2 / (1 + d^2);
//     no specular term (the reference compiles its shaders with NoSpecular);
//     N = normalize(cofactor(abs) * normal) interpolated per fragment;
//   * semantic ID: the provoking (last) vertex's object ID when the mesh has
//     per-vertex IDs, else the draw's ID; 0 where nothing was drawn
//     (src/esp/gfx/RenderTarget.cpp:189-190).
//
// The rasterisation rules (GL leaves them to the implementation) are fixed
// here so that the device kernels can match them bit for bit:
//   - homogeneous clip of the triangle against z >= -w (near) and a guard
//     band |x| <= G*w, |y| <= G*w (Sutherland & Hodgman 1974), fan
//     re-triangulation;
//   - window coordinates snapped to 1/256 pixel (round half to even);
//   - 64-bit integer edge functions (Pineda 1988) with the top-left fill
//     rule (a left edge or a top edge owns its pixels);
//   - window depth interpolated linearly in screen space from the snapped
//     edge functions; fragments with depth >= 1 dropped (far plane);
//   - attributes from homogeneous barycentrics of the unclipped triangle at
//     the pixel centre (Olano & Greer 1997), so clipped triangles shade
//     exactly like unclipped ones;
//   - bilinear / nearest texel fetch on texel centres with GL wrap modes.
// Build with -ffp-contract=off so that a*b+c never fuses; every fused
// multiply-add is written as std::fmaf.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

extern "C" {

struct OracleTexture {
  const uint8_t* data;  // level 0 of every layer (layers * h * w * 4), then level 1, ...; row 0 = bottom
  int32_t width, height, layers;
  int32_t filter;       // magnification: 0 nearest, 1 linear
  int32_t wrap_s, wrap_t;  // 0 repeat, 1 clamp to edge, 2 mirrored repeat
  int32_t min_filter;   // minification within a level: 0 nearest, 1 linear
  int32_t mip_filter;   // 0 base level only, 1 nearest level, 2 linear between levels
  int32_t levels;
};

struct OracleMesh {
  const float* positions;   // 3 per vertex
  const float* colors;      // 4 per vertex or null
  const float* texcoords;   // 2 per vertex or null
  const uint32_t* object_ids;  // 1 per vertex or null
  const uint32_t* indices;
  uint32_t vertex_count, index_count;
  const float* normals;     // 3 per vertex or null
};

struct OracleMaterial {
  float color[4];
  int32_t texture;   // renderer texture id, 0 = white
  int32_t layer;
  float matrix[9];   // 3x3, [col][row]
  int32_t phong;     // 1: lit (ambient = color * ambient factor, diffuse = color)
};

struct OracleLight {
  int32_t node;
  int32_t type;      // 0 directional (along -backward of the node), 1 point
  float color[3];
  float range;
};

struct OracleDraw {
  int32_t node;
  int32_t mesh;
  uint32_t index_offset;  // in indices
  uint32_t index_count;
  int32_t material;
  uint32_t semantic_id;
};

struct OracleScene {
  int32_t width, height;
  int64_t fb_offset;  // pixel index of (0,0)
  int64_t pitch;      // pixels per row
  float pv[16];
  float view[16];
  int32_t node_count;
  const int32_t* parents;
  const float* transforms;  // 16 per node
  int32_t draw_count;
  const OracleDraw* draws;
  int32_t light_count;
  const OracleLight* lights;
};

struct OracleOutput {
  uint32_t* color;
  float* depth;        // window depth, may be null
  float* linear_depth; // may be null
  uint32_t* semantic;  // may be null
};

}  // extern "C"

namespace {

constexpr uint32_t kBackground = 0xFF1F1F1Fu;
constexpr int kNoTextures = 1;

inline float fma_(float a, float b, float c) { return std::fmaf(a, b, c); }

struct V4 { float x, y, z, w; };

// C = A * B for column-major 4x4 (m[col*4+row]).
void matmul(const float* a, const float* b, float* c) {
  for (int col = 0; col < 4; ++col)
    for (int row = 0; row < 4; ++row) {
      float t = a[0 * 4 + row] * b[col * 4 + 0];
      t = fma_(a[1 * 4 + row], b[col * 4 + 1], t);
      t = fma_(a[2 * 4 + row], b[col * 4 + 2], t);
      t = fma_(a[3 * 4 + row], b[col * 4 + 3], t);
      c[col * 4 + row] = t;
    }
}

inline float mrow(const float* m, int row, float x, float y, float z) {
  float r = m[12 + row];
  r = fma_(m[0 + row], x, r);
  r = fma_(m[4 + row], y, r);
  r = fma_(m[8 + row], z, r);
  return r;
}

struct Frame {
  const OracleTexture* tex; int ntex;
  const OracleMesh* meshes;
  const OracleMaterial* mats;
  int flags;
  OracleOutput out;
  int max_lights;        // 0: every material flat
  float ambient_factor;
};

// A light in world space: position (w = 1) or direction towards the light
// (w = 0), colour, range.
struct WorldLight {
  float pos[4];
  float color[3];
  float range;
};

inline int wrap(int i, int n, int mode) {
  if (mode == 0) { int m = i % n; return m < 0 ? m + n : m; }
  if (mode == 1) return i < 0 ? 0 : (i >= n ? n - 1 : i);
  int p = 2 * n; int m = i % p; if (m < 0) m += p;
  return m >= n ? p - 1 - m : m;
}

inline float clampc(float f) {
  const float lim = 16777216.0f;
  if (!(f > -lim)) return -lim;
  if (!(f < lim)) return lim;
  return f;
}

// Texel of level `level` (level k is max(1, w >> k) x max(1, h >> k); the
// levels follow one another, each holding every layer).
inline float texel(const OracleTexture& t, size_t level_off, int tw, int th, int layer, int x, int y, int c) {
  size_t i = level_off + ((size_t(layer) * th + y) * tw + x) * 4 + c;
  return float(t.data[i]) / 255.0f;
}

void sample_level(const OracleTexture& t, int L, int level, int filter, float s, float u, float out[4]) {
  const int tw = std::max(1, t.width >> level), th = std::max(1, t.height >> level);
  size_t off = 0;
  for (int k = 0; k < level; ++k)
    off += size_t(std::max(1, t.width >> k)) * size_t(std::max(1, t.height >> k)) * t.layers * 4;
  float fw = float(tw), fh = float(th);
  if (filter == 0) {
    int x = wrap(int(std::floor(clampc(s * fw))), tw, t.wrap_s);
    int y = wrap(int(std::floor(clampc(u * fh))), th, t.wrap_t);
    for (int c = 0; c < 4; ++c) out[c] = texel(t, off, tw, th, L, x, y, c);
    return;
  }
  float fx = clampc(s * fw - 0.5f), fy = clampc(u * fh - 0.5f);
  float flx = std::floor(fx), fly = std::floor(fy);
  float a = fx - flx, b = fy - fly;
  int x0 = wrap(int(flx), tw, t.wrap_s), x1 = wrap(int(flx) + 1, tw, t.wrap_s);
  int y0 = wrap(int(fly), th, t.wrap_t), y1 = wrap(int(fly) + 1, th, t.wrap_t);
  for (int c = 0; c < 4; ++c) {
    float t00 = texel(t, off, tw, th, L, x0, y0, c), t10 = texel(t, off, tw, th, L, x1, y0, c);
    float t01 = texel(t, off, tw, th, L, x0, y1, c), t11 = texel(t, off, tw, th, L, x1, y1, c);
    float lo = fma_(a, t10 - t00, t00);
    float hi = fma_(a, t11 - t01, t01);
    out[c] = fma_(b, hi - lo, lo);
  }
}

inline int clamp_layer(const OracleTexture& t, int layer) {
  return layer < 0 ? 0 : (layer >= t.layers ? t.layers - 1 : layer);
}

void sample(const OracleTexture& t, int layer, float s, float u, float out[4]) {
  sample_level(t, clamp_layer(t, layer), 0, t.filter, s, u, out);
}

// log2 by the atanh series of the mantissa normalised to [sqrt(1/2), sqrt(2)).
float series_log2(float x) {
  int e;
  float m = std::frexp(x, &e);
  if (m < 0.7071067690849304f) {
    m = m * 2.0f;
    e -= 1;
  }
  const float t = (m - 1.0f) / (m + 1.0f);
  const float t2 = t * t;
  float q = 0.1111111119389534f;
  q = q * t2 + 0.1428571492433548f;
  q = q * t2 + 0.20000000298023224f;
  q = q * t2 + 0.3333333432674408f;
  q = q * t2 + 1.0f;
  return float(e) + (t * q) * 2.885390043258667f;
}

// Level-of-detail selection of OpenGL 4.6, 8.14 (see the kernel's sample_lod).
void sample_lod(const OracleTexture& t, int layer, float s, float u, float lambda, float out[4]) {
  const int L = clamp_layer(t, layer);
  const float c = (t.filter == 1 && t.min_filter == 0 && t.mip_filter != 0) ? 0.5f : 0.0f;
  if (!(lambda > c)) {
    sample_level(t, L, 0, t.filter, s, u, out);
    return;
  }
  const int q = t.levels - 1;
  if (t.mip_filter == 0) {
    sample_level(t, L, 0, t.min_filter, s, u, out);
  } else if (t.mip_filter == 1) {
    int d = lambda <= 0.5f ? 0 : int(std::ceil(lambda + 0.5f)) - 1;
    if (d > q) d = q;
    sample_level(t, L, d, t.min_filter, s, u, out);
  } else if (lambda >= float(q)) {
    sample_level(t, L, q, t.min_filter, s, u, out);
  } else {
    const float fl = std::floor(lambda);
    const int d1 = int(fl);
    const float f = lambda - fl;
    float hi[4];
    sample_level(t, L, d1, t.min_filter, s, u, out);
    sample_level(t, L, d1 + 1, t.min_filter, s, u, hi);
    for (int k = 0; k < 4; ++k) out[k] = fma_(f, hi[k] - out[k], out[k]);
  }
}

// Float -> unorm8: round to nearest, with values within 1e-4 above a tie
// rounded down.  The reference's images round that way (its shaders land a
// hair below this restatement's values: e.g. an ambient 0.1 is stored as 25,
// not 26); every golden image of the flat path matches either way.
inline uint32_t unorm8(float c) {
  if (!(c > 0.0f)) c = 0.0f;
  if (c > 1.0f) c = 1.0f;
  float t = c * 255.0f;
  t = t + 0.4999f;
  return uint32_t(t);
}

struct Tri {
  V4 c[3];        // clip coordinates
  float d[3];     // -z_eye
  uint32_t vi[3]; // vertex indices
  float wp[3][3]; // world positions (lit draws)
  float wn[3][3]; // normals times the normal matrix (lit draws)
};

// Lit shading (Phong without a specular term, the reference's shader
// configuration): every light adds diffuse * light colour * max(0, N.L) *
// attenuation, attenuation = clamp(1 - (d / range)^4, 0, 1)^2 / (1 + d^2)
// with d the distance to a point light (0 for directional lights).
void light_rgb(const float n_in[3], const float P[3], const WorldLight* lights, int nl,
               const float dif[4], float rgb[3]) {
  float len2 = fma_(n_in[2], n_in[2], fma_(n_in[1], n_in[1], n_in[0] * n_in[0]));
  float inv = 1.0f / std::sqrt(len2);
  float n[3] = {n_in[0] * inv, n_in[1] * inv, n_in[2] * inv};
  for (int j = 0; j < nl; ++j) {
    const WorldLight& L = lights[j];
    float l[3];
    for (int k = 0; k < 3; ++k) l[k] = L.pos[k] - P[k] * L.pos[3];
    float d2 = fma_(l[2], l[2], fma_(l[1], l[1], l[0] * l[0]));
    float len = std::sqrt(d2);
    if (!(len > 0.0f)) continue;
    float dist = len * L.pos[3];
    float q = dist / std::max(L.range, 0.0001f);
    float q2 = q * q;
    float a = 1.0f - q2 * q2;
    a = a < 0.0f ? 0.0f : (a > 1.0f ? 1.0f : a);
    float att = (a * a) / (1.0f + dist * dist);
    float il = 1.0f / len;
    float ndl = fma_(n[2], l[2] * il, fma_(n[1], l[1] * il, n[0] * (l[0] * il)));
    float intensity = (ndl > 0.0f ? ndl : 0.0f) * att;
    for (int c = 0; c < 3; ++c) rgb[c] = fma_(dif[c] * L.color[c], intensity, rgb[c]);
  }
}

// Shade the fragment of `tri` at pixel (px, py): returns colour, linear depth, id.
void shade(const Frame& f, const OracleScene& sc, const OracleDraw& dr, const Tri& tri,
           const WorldLight* lights, int nl, int px, int py, uint32_t* color, float* lin,
           uint32_t* sid) {
  const OracleMesh& m = f.meshes[dr.mesh];
  const float sx = float(2 * px + 1 - sc.width) / float(sc.width);
  const float sy = float(2 * py + 1 - sc.height) / float(sc.height);
  float l[3];
  for (int i = 0; i < 3; ++i) {
    const V4& a = tri.c[(i + 1) % 3];
    const V4& b = tri.c[(i + 2) % 3];
    float ex = a.y * b.w - a.w * b.y;
    float ey = a.w * b.x - a.x * b.w;
    float ez = a.x * b.y - a.y * b.x;
    l[i] = fma_(ex, sx, fma_(ey, sy, ez));
  }
  float s = (l[0] + l[1]) + l[2];
  float inv = 1.0f / s;
  float b0 = l[0] * inv, b1 = l[1] * inv, b2 = l[2] * inv;
  auto interp = [&](float a0, float a1, float a2) {
    return fma_(b2, a2, fma_(b1, a1, b0 * a0));
  };
  *lin = interp(tri.d[0], tri.d[1], tri.d[2]);

  float vc[4] = {1.0f, 1.0f, 1.0f, 1.0f};
  if (m.colors)
    for (int c = 0; c < 4; ++c)
      vc[c] = interp(m.colors[tri.vi[0] * 4 + c], m.colors[tri.vi[1] * 4 + c],
                     m.colors[tri.vi[2] * 4 + c]);
  const OracleMaterial& mat = f.mats[dr.material];
  float tc[4] = {1.0f, 1.0f, 1.0f, 1.0f};
  if (!(f.flags & kNoTextures) && mat.texture > 0 && mat.texture < f.ntex) {
    float u = 0.0f, v = 0.0f;
    if (m.texcoords) {
      u = interp(m.texcoords[tri.vi[0] * 2], m.texcoords[tri.vi[1] * 2],
                 m.texcoords[tri.vi[2] * 2]);
      v = interp(m.texcoords[tri.vi[0] * 2 + 1], m.texcoords[tri.vi[1] * 2 + 1],
                 m.texcoords[tri.vi[2] * 2 + 1]);
    }
    const float* M = mat.matrix;
    float ts = M[6]; ts = fma_(M[0], u, ts); ts = fma_(M[3], v, ts);
    float tt = M[7]; tt = fma_(M[1], u, tt); tt = fma_(M[4], v, tt);
    const OracleTexture& tex = f.tex[mat.texture];
    if (tex.mip_filter == 0 && tex.min_filter == tex.filter) {
      sample(tex, mat.layer, ts, tt, tc);
    } else {
      // Level of detail from the texel-coordinate derivatives across the
      // pixel's 2x2 quad: the quad's pixel pair in this row (x) and column (y).
      float ex[3], ey[3], ez[3];
      for (int i = 0; i < 3; ++i) {
        const V4& a = tri.c[(i + 1) % 3];
        const V4& b = tri.c[(i + 2) % 3];
        ex[i] = a.y * b.w - a.w * b.y;
        ey[i] = a.w * b.x - a.x * b.w;
        ez[i] = a.x * b.y - a.y * b.x;
      }
      float t0[2] = {0, 0}, t1[2] = {0, 0}, t2[2] = {0, 0};
      if (m.texcoords)
        for (int k = 0; k < 2; ++k) {
          t0[k] = m.texcoords[tri.vi[0] * 2 + k];
          t1[k] = m.texcoords[tri.vi[1] * 2 + k];
          t2[k] = m.texcoords[tri.vi[2] * 2 + k];
        }
      auto st_at = [&](int x, int y, float& os, float& ot) {
        const float qx = float(2 * x + 1 - sc.width) / float(sc.width);
        const float qy = float(2 * y + 1 - sc.height) / float(sc.height);
        const float a0 = fma_(ex[0], qx, fma_(ey[0], qy, ez[0]));
        const float a1 = fma_(ex[1], qx, fma_(ey[1], qy, ez[1]));
        const float a2 = fma_(ex[2], qx, fma_(ey[2], qy, ez[2]));
        const float is = 1.0f / ((a0 + a1) + a2);
        const float c0 = a0 * is, c1 = a1 * is, c2 = a2 * is;
        const float uu = fma_(c2, t2[0], fma_(c1, t1[0], c0 * t0[0]));
        const float ww = fma_(c2, t2[1], fma_(c1, t1[1], c0 * t0[1]));
        os = fma_(M[3], ww, fma_(M[0], uu, M[6]));
        ot = fma_(M[4], ww, fma_(M[1], uu, M[7]));
      };
      float sa, ta, sb, tb, scc, tcc, sd, td;
      st_at(px & ~1, py, sa, ta);
      st_at((px & ~1) + 1, py, sb, tb);
      st_at(px, py & ~1, scc, tcc);
      st_at(px, (py & ~1) + 1, sd, td);
      const float fw = float(tex.width), fh = float(tex.height);
      const float dux = (sb - sa) * fw, dvx = (tb - ta) * fh;
      const float duy = (sd - scc) * fw, dvy = (td - tcc) * fh;
      const float rx = std::sqrt(dux * dux + dvx * dvx), ry = std::sqrt(duy * duy + dvy * dvy);
      const float rho = std::fmax(rx, ry);
      const float lambda = rho > 0.0f ? (rho < 3.0e38f ? series_log2(rho) : 128.0f) : -1.0f;
      sample_lod(tex, mat.layer, ts, tt, lambda, tc);
    }
  }
  uint32_t packed = 0;
  if (mat.phong && f.max_lights > 0) {
    float amb[4], dif[4], rgb[3];
    for (int c = 0; c < 4; ++c) {
      amb[c] = ((mat.color[c] * f.ambient_factor) * tc[c]) * vc[c];
      dif[c] = (mat.color[c] * tc[c]) * vc[c];
    }
    for (int c = 0; c < 3; ++c) rgb[c] = amb[c];
    if (nl > 0 && m.normals) {
      float P[3], N[3];
      for (int c = 0; c < 3; ++c) {
        P[c] = interp(tri.wp[0][c], tri.wp[1][c], tri.wp[2][c]);
        N[c] = interp(tri.wn[0][c], tri.wn[1][c], tri.wn[2][c]);
      }
      light_rgb(N, P, lights, nl, dif, rgb);
    }
    for (int c = 0; c < 3; ++c) packed |= unorm8(rgb[c]) << (8 * c);
    packed |= unorm8(dif[3]) << 24;
  } else {
    for (int c = 0; c < 4; ++c) {
      float v = (mat.color[c] * tc[c]) * vc[c];
      packed |= unorm8(v) << (8 * c);
    }
  }
  *color = packed;
  *sid = m.object_ids ? m.object_ids[tri.vi[2]] : dr.semantic_id;
}

// Distance of a clip-space vertex to clip plane p (>= 0 is inside).
inline float plane_dist(const V4& v, int p, float gx, float gy) {
  switch (p) {
    case 0: return v.z + v.w;
    case 1: return gx * v.w - v.x;
    case 2: return gx * v.w + v.x;
    case 3: return gy * v.w - v.y;
    default: return gy * v.w + v.y;
  }
}

inline V4 lerp_clip(const V4& in, const V4& out, float din, float dout) {
  float t = din / (din - dout);
  return {fma_(t, out.x - in.x, in.x), fma_(t, out.y - in.y, in.y),
          fma_(t, out.z - in.z, in.z), fma_(t, out.w - in.w, in.w)};
}

struct SceneRaster {
  const Frame& f;
  const OracleScene& sc;
  std::vector<float> zbuf;
  std::vector<WorldLight> lights;

  SceneRaster(const Frame& f_, const OracleScene& sc_) : f(f_), sc(sc_) {
    zbuf.assign(size_t(sc.width) * sc.height, 1.0f);
  }

  void raster_sub(const V4* q, const OracleDraw& dr, const Tri& tri) {
    const float hw = 0.5f * float(sc.width), hh = 0.5f * float(sc.height);
    int32_t X[3], Y[3];
    float zw[3];
    for (int i = 0; i < 3; ++i) {
      float iw = 1.0f / q[i].w;
      float nx = q[i].x * iw, ny = q[i].y * iw, nz = q[i].z * iw;
      float xw = fma_(nx, hw, hw), yw = fma_(ny, hh, hh);
      zw[i] = fma_(nz, 0.5f, 0.5f);
      X[i] = int32_t(std::lrintf(xw * 256.0f));
      Y[i] = int32_t(std::lrintf(yw * 256.0f));
    }
    int64_t area = int64_t(X[1] - X[0]) * (Y[2] - Y[0]) - int64_t(X[2] - X[0]) * (Y[1] - Y[0]);
    if (area <= 0) return;  // back-facing or degenerate
    int64_t bias[3];
    for (int i = 0; i < 3; ++i) {
      int a = (i + 1) % 3, b = (i + 2) % 3;
      int dx = X[b] - X[a], dy = Y[b] - Y[a];
      bias[i] = (dy < 0 || (dy == 0 && dx < 0)) ? 0 : -1;
    }
    int minX = std::min({X[0], X[1], X[2]}), maxX = std::max({X[0], X[1], X[2]});
    int minY = std::min({Y[0], Y[1], Y[2]}), maxY = std::max({Y[0], Y[1], Y[2]});
    int x0 = (minX - 128 + 255) >> 8, x1 = (maxX - 128) >> 8;
    int y0 = (minY - 128 + 255) >> 8, y1 = (maxY - 128) >> 8;
    x0 = std::max(x0, 0); y0 = std::max(y0, 0);
    x1 = std::min(x1, sc.width - 1); y1 = std::min(y1, sc.height - 1);
    if (x0 > x1 || y0 > y1) return;
    const float inva = 1.0f / float(area);
    const float d1 = zw[1] - zw[0], d2 = zw[2] - zw[0];
    for (int py = y0; py <= y1; ++py) {
      const int64_t Py = int64_t(py) * 256 + 128;
      for (int px = x0; px <= x1; ++px) {
        const int64_t Px = int64_t(px) * 256 + 128;
        int64_t e[3];
        bool inside = true;
        for (int i = 0; i < 3; ++i) {
          int a = (i + 1) % 3, b = (i + 2) % 3;
          e[i] = int64_t(X[b] - X[a]) * (Py - Y[a]) - int64_t(Y[b] - Y[a]) * (Px - X[a]);
          if (e[i] + bias[i] < 0) { inside = false; break; }
        }
        if (!inside) continue;
        float b1 = float(e[1]) * inva, b2 = float(e[2]) * inva;
        float z = fma_(b2, d2, fma_(b1, d1, zw[0]));
        if (!(z > 0.0f)) z = 0.0f;
        if (!(z < 1.0f)) continue;
        float& zb = zbuf[size_t(py) * sc.width + px];
        if (!(z < zb)) continue;
        zb = z;
        const int64_t o = sc.fb_offset + int64_t(py) * sc.pitch + px;
        uint32_t col, sid;
        float lin;
        shade(f, sc, dr, tri, lights.data(), int(lights.size()), px, py, &col, &lin, &sid);
        f.out.color[o] = col;
        if (f.out.depth) f.out.depth[o] = z;
        if (f.out.linear_depth) f.out.linear_depth[o] = lin;
        if (f.out.semantic) f.out.semantic[o] = sid;
      }
    }
  }

  void triangle(const OracleDraw& dr, const Tri& tri) {
    const V4* c = tri.c;
    // Trivial reject: all three vertices outside the same frustum plane.
    if ((c[0].x > c[0].w && c[1].x > c[1].w && c[2].x > c[2].w) ||
        (c[0].x < -c[0].w && c[1].x < -c[1].w && c[2].x < -c[2].w) ||
        (c[0].y > c[0].w && c[1].y > c[1].w && c[2].y > c[2].w) ||
        (c[0].y < -c[0].w && c[1].y < -c[1].w && c[2].y < -c[2].w) ||
        (c[0].z > c[0].w && c[1].z > c[1].w && c[2].z > c[2].w) ||
        (c[0].z < -c[0].w && c[1].z < -c[1].w && c[2].z < -c[2].w))
      return;
    const float gx = 32768.0f / float(sc.width), gy = 32768.0f / float(sc.height);
    bool need_clip = false;
    for (int i = 0; i < 3 && !need_clip; ++i)
      for (int p = 0; p < 5; ++p)
        if (plane_dist(c[i], p, gx, gy) < 0.0f) { need_clip = true; break; }
    if (!need_clip) {
      raster_sub(c, dr, tri);
      return;
    }
    V4 poly[9], next[9];
    int n = 3;
    for (int i = 0; i < 3; ++i) poly[i] = c[i];
    for (int p = 0; p < 5 && n >= 3; ++p) {
      int m = 0;
      for (int i = 0; i < n; ++i) {
        const V4& a = poly[i];
        const V4& b = poly[(i + 1) % n];
        float da = plane_dist(a, p, gx, gy), db = plane_dist(b, p, gx, gy);
        bool ina = da >= 0.0f, inb = db >= 0.0f;
        if (ina) next[m++] = a;
        if (ina != inb) next[m++] = ina ? lerp_clip(a, b, da, db) : lerp_clip(b, a, db, da);
      }
      n = m;
      for (int i = 0; i < n; ++i) poly[i] = next[i];
    }
    for (int i = 1; i + 1 < n; ++i) {
      V4 sub[3] = {poly[0], poly[i], poly[i + 1]};
      raster_sub(sub, dr, tri);
    }
  }

  void run() {
    // Clear this scene's rectangle.
    for (int y = 0; y < sc.height; ++y)
      for (int x = 0; x < sc.width; ++x) {
        const int64_t o = sc.fb_offset + int64_t(y) * sc.pitch + x;
        f.out.color[o] = kBackground;
        if (f.out.depth) f.out.depth[o] = 1.0f;
        if (f.out.linear_depth) f.out.linear_depth[o] = 0.0f;
        if (f.out.semantic) f.out.semantic[o] = 0;
      }
    if (sc.draw_count == 0) return;
    // Absolute transforms.
    std::vector<float> abs(size_t(sc.node_count) * 16);
    for (int i = 0; i < sc.node_count; ++i) {
      const float* local = sc.transforms + size_t(i) * 16;
      if (sc.parents[i] < 0)
        std::memcpy(&abs[size_t(i) * 16], local, 64);
      else
        matmul(&abs[size_t(sc.parents[i]) * 16], local, &abs[size_t(i) * 16]);
    }
    // Lights in world space: the node's translation (point) or its negative
    // backward axis (directional); at most max_lights of them.
    const int nl = std::min(sc.light_count, f.max_lights);
    for (int j = 0; j < nl; ++j) {
      const OracleLight& L = sc.lights[j];
      const float* A = &abs[size_t(L.node) * 16];
      WorldLight w{};
      if (L.type == 0) {
        w.pos[0] = -A[8];
        w.pos[1] = -A[9];
        w.pos[2] = -A[10];
        w.pos[3] = 0.0f;
      } else {
        w.pos[0] = A[12];
        w.pos[1] = A[13];
        w.pos[2] = A[14];
        w.pos[3] = 1.0f;
      }
      for (int c = 0; c < 3; ++c) w.color[c] = L.color[c];
      w.range = L.range;
      lights.push_back(w);
    }
    for (int di = 0; di < sc.draw_count; ++di) {
      const OracleDraw& dr = sc.draws[di];
      const OracleMesh& m = f.meshes[dr.mesh];
      const float* A = &abs[size_t(dr.node) * 16];
      // Normal matrix: cofactor of the upper-left 3x3 (columns c1 x c2,
      // c2 x c0, c0 x c1), [col][row].
      const bool lit = f.max_lights > 0 && f.mats[dr.material].phong && m.normals;
      float NM[9];
      if (lit) {
        const float* c0 = A;
        const float* c1 = A + 4;
        const float* c2 = A + 8;
        const float* cols[3][2] = {{c1, c2}, {c2, c0}, {c0, c1}};
        for (int k = 0; k < 3; ++k) {
          const float* u = cols[k][0];
          const float* v = cols[k][1];
          NM[k * 3 + 0] = u[1] * v[2] - u[2] * v[1];
          NM[k * 3 + 1] = u[2] * v[0] - u[0] * v[2];
          NM[k * 3 + 2] = u[0] * v[1] - u[1] * v[0];
        }
      }
      float mvp[16], zrow[4];
      matmul(sc.pv, A, mvp);
      for (int col = 0; col < 4; ++col) {
        float t = sc.view[0 * 4 + 2] * A[col * 4 + 0];
        t = fma_(sc.view[1 * 4 + 2], A[col * 4 + 1], t);
        t = fma_(sc.view[2 * 4 + 2], A[col * 4 + 2], t);
        t = fma_(sc.view[3 * 4 + 2], A[col * 4 + 3], t);
        zrow[col] = t;
      }
      const uint32_t ntri = dr.index_count / 3;
      for (uint32_t t = 0; t < ntri; ++t) {
        Tri tri;
        for (int k = 0; k < 3; ++k) {
          uint32_t vi = m.indices[dr.index_offset + t * 3 + k];
          tri.vi[k] = vi;
          const float* p = m.positions + size_t(vi) * 3;
          tri.c[k] = {mrow(mvp, 0, p[0], p[1], p[2]), mrow(mvp, 1, p[0], p[1], p[2]),
                      mrow(mvp, 2, p[0], p[1], p[2]), mrow(mvp, 3, p[0], p[1], p[2])};
          float ze = zrow[3];
          ze = fma_(zrow[0], p[0], ze);
          ze = fma_(zrow[1], p[1], ze);
          ze = fma_(zrow[2], p[2], ze);
          tri.d[k] = -ze;
          if (lit) {
            for (int r = 0; r < 3; ++r) tri.wp[k][r] = mrow(A, r, p[0], p[1], p[2]);
            const float* nv = m.normals + size_t(vi) * 3;
            for (int r = 0; r < 3; ++r)
              tri.wn[k][r] = fma_(NM[6 + r], nv[2], fma_(NM[3 + r], nv[1], NM[r] * nv[0]));
          }
        }
        triangle(dr, tri);
      }
    }
  }
};

}  // namespace

extern "C" int oracle_render(const OracleTexture* textures, int32_t texture_count,
                             const OracleMesh* meshes, const OracleMaterial* materials,
                             const OracleScene* scenes, int32_t scene_count, int32_t flags,
                             OracleOutput out, int32_t threads, int32_t max_lights,
                             float ambient_factor) {
  Frame f{textures, texture_count, meshes, materials, flags, out, max_lights, ambient_factor};
  if (threads < 1) threads = 1;
  std::atomic<int> next{0};
  auto worker = [&]() {
    for (int s; (s = next.fetch_add(1)) < scene_count;) {
      SceneRaster r(f, scenes[s]);
      r.run();
    }
  };
  if (threads == 1) {
    worker();
  } else {
    std::vector<std::thread> pool;
    for (int i = 0; i < threads; ++i) pool.emplace_back(worker);
    for (auto& t : pool) t.join();
  }
  return 0;
}

// unprojectDepth restated (src/esp/gfx_batch/DepthUnprojection.cpp:107-129):
// d <- b/(d + a), then values equal to b/(1 + a) (the cleared far plane) -> 0.
extern "C" void oracle_unproject_depth(const float* unprojection, float* depth, int64_t rows,
                                       int64_t cols, int64_t row_stride) {
  const float a = unprojection[0], b = unprojection[1];
  for (int64_t y = 0; y < rows; ++y)
    for (int64_t x = 0; x < cols; ++x) {
      float& d = depth[y * row_stride + x];
      d = b / (d + a);
    }
  const float far_depth = b / (1.0f + a);
  for (int64_t y = 0; y < rows; ++y)
    for (int64_t x = 0; x < cols; ++x) {
      float& d = depth[y * row_stride + x];
      if (d == far_depth) d = 0.0f;
    }
}
