// Horizon-based ambient occlusion, classic algorithm (declared in
// include/gbr_hbao.h; restating src/esp/gfx_batch/Hbao.cpp:595-935 and the
// shaders src/shaders/gfx_batch/hbao/hbao.frag, bilateralblur.frag).
//
// Per pixel (x, y) of a w x h image with linear depth L (0 -> far plane),
// u = (x + 0.5) / w, v = (y + 0.5) / h:
//   P = ((u, v) * pi.xy + pi.zw) * z, z)         view position (z = 1 in x, y if orthographic)
//   N = -normalize(cross(dx, dy)), dx / dy the shorter of the forward and
//       backward differences to the neighbouring pixels (clamped at edges)
//   R = radius_to_screen / z pixels, step = R / 5, jitter J = table[y & 3][x & 3]
//   for 8 directions d rotated by J.xy, 4 steps from J.z * step + 1 pixels:
//       S = the view position at P's pixel + rint(ray * d) (clamped texel,
//           unclamped coordinates), V = S - P,
//       AO += clamp(N.V / |V| - bias, 0, 1) * clamp(1 - |V|^2 / r^2, 0, 1)
//   ao = clamp(1 - 2 AO / (1 - bias) / 32, 0, 1) ^ intensity, stored as unorm8
// then a 7-tap blur along x, stored as unorm8, along y, each tap weighted
// exp2(-t^2 / 4.5 - ((L_t - L_c) sharpness)^2), and colour rgb *= ao.
//
// pow and exp2 are evaluated by the polynomials below (exp2: Taylor series of
// 2^f on [0, 1) to degree 9 and exact scaling; log2: atanh series of the
// mantissa normalised to [sqrt(1/2), sqrt(2))), every operation one float
// rounding, so the result is a pure function of the inputs that the
// oracle reproduces bit for bit.  GLSL leaves pow/exp2 precision to the
// driver; this fixes it.
#include "hbao.h"

#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

namespace gbr {
void set_last_error(const std::string& msg);

namespace {

__device__ __forceinline__ float poly_exp2(float x) {
  if (x < -149.0f) return 0.0f;
  const float n = floorf(x);
  const float f = __fsub_rn(x, n);
  float p = 1.0178086284895471e-07f;
  p = __fadd_rn(__fmul_rn(p, f), 1.3215486660556053e-06f);
  p = __fadd_rn(__fmul_rn(p, f), 1.5252733646775596e-05f);
  p = __fadd_rn(__fmul_rn(p, f), 0.0001540352968731895f);
  p = __fadd_rn(__fmul_rn(p, f), 0.0013333557872101665f);
  p = __fadd_rn(__fmul_rn(p, f), 0.009618128649890423f);
  p = __fadd_rn(__fmul_rn(p, f), 0.05550410971045494f);
  p = __fadd_rn(__fmul_rn(p, f), 0.24022650718688965f);
  p = __fadd_rn(__fmul_rn(p, f), 0.6931471824645996f);
  p = __fadd_rn(__fmul_rn(p, f), 1.0f);
  return ldexpf(p, int(n));
}

__device__ __forceinline__ float poly_log2(float x) {
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

__device__ __forceinline__ float poly_pow(float a, float e) {
  if (!(a > 0.0f)) return e == 0.0f ? 1.0f : 0.0f;
  return poly_exp2(__fmul_rn(e, poly_log2(a)));
}

__device__ __forceinline__ float clamp01(float v) { return fminf(fmaxf(v, 0.0f), 1.0f); }

__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 sub(float3 a, float3 b) {
  return f3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z));
}
__device__ __forceinline__ float dot3(float3 a, float3 b) {
  return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
  return f3(__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)),
            __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)),
            __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}

__device__ __forceinline__ float depth_at(const HbaoScene& s, const float* __restrict__ depth, int tx, int ty) {
  tx = min(max(tx, 0), s.w - 1);
  ty = min(max(ty, 0), s.h - 1);
  const float z = __ldg(depth + s.offset + (long long)ty * s.pitch + tx);
  return z == 0.0f ? s.far_plane : z;
}

__device__ __forceinline__ float3 view_pos(const HbaoScene& s, float u, float v, float z) {
  const float k = s.ortho ? 1.0f : z;
  return f3(__fmul_rn(__fadd_rn(__fmul_rn(u, s.pi[0]), s.pi[2]), k),
            __fmul_rn(__fadd_rn(__fmul_rn(v, s.pi[1]), s.pi[3]), k), z);
}

__device__ __forceinline__ float3 min_diff(float3 p, float3 pr, float3 pl) {
  const float3 v1 = sub(pr, p), v2 = sub(p, pl);
  return dot3(v1, v1) < dot3(v2, v2) ? v1 : v2;
}

__device__ __forceinline__ uint8_t unorm8(float v) {
  return uint8_t(__fadd_rn(__fmul_rn(clamp01(v), 255.0f), 0.5f));
}

__device__ __forceinline__ uint32_t modulate(uint32_t c, float ao) {
  uint32_t out = c & 0xFF000000u;  // alpha: blend factor one
  for (int ch = 0; ch < 3; ++ch) {
    const float v = __fmul_rn(__fdiv_rn(float((c >> (8 * ch)) & 0xFFu), 255.0f), ao);
    out |= uint32_t(unorm8(v)) << (8 * ch);
  }
  return out;
}

// The grid has one block per 256 pixels of the batch: scene i owns blocks
// scenes[i].block0 .. scenes[i + 1].block0 - 1.  The block's scene, by a
// binary search of thread 0.
__device__ __forceinline__ int scene_of_block(const HbaoScene* scenes, int count) {
  __shared__ int s_si;
  if (threadIdx.x == 0) {
    int lo = 0, hi = count;  // scenes[lo].block0 <= blockIdx.x < scenes[hi].block0
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (scenes[mid].block0 <= int(blockIdx.x))
        lo = mid;
      else
        hi = mid;
    }
    s_si = lo;
  }
  __syncthreads();
  return s_si;
}

__device__ __forceinline__ float3 reconstruct_normal(const HbaoScene& s, const float* __restrict__ depth, int x, int y,
                                                     float u, float v, float inv_w, float inv_h, float3 P,
                                                     float& inv_len) {
  const float3 pr = view_pos(s, __fadd_rn(u, inv_w), v, depth_at(s, depth, x + 1, y));
  const float3 pl = view_pos(s, __fadd_rn(u, -inv_w), v, depth_at(s, depth, x - 1, y));
  const float3 pt = view_pos(s, u, __fadd_rn(v, inv_h), depth_at(s, depth, x, y + 1));
  const float3 pb = view_pos(s, u, __fadd_rn(v, -inv_h), depth_at(s, depth, x, y - 1));
  const float3 c = cross3(min_diff(P, pr, pl), min_diff(P, pt, pb));
  inv_len = __fdiv_rn(1.0f, __fsqrt_rn(dot3(c, c)));
  return c;
}

// Depth of the cache-aware sample: texel (tqx, tqy) of deinterleaved layer
// (ox, oy), i.e. full-resolution pixel (4 tqx + ox, 4 tqy + oy); texels of
// the quarter-resolution layer that fall beyond the image read as the far plane.
__device__ __forceinline__ float layer_depth(const HbaoScene& s, const float* __restrict__ depth, int tqx, int tqy,
                                             int ox, int oy) {
  tqx = min(max(tqx, 0), s.qw - 1);
  tqy = min(max(tqy, 0), s.qh - 1);
  const int fx = 4 * tqx + ox, fy = 4 * tqy + oy;
  if (fx >= s.w || fy >= s.h) return s.far_plane;
  const float z = __ldg(depth + s.offset + (long long)fy * s.pitch + fx);
  return z == 0.0f ? s.far_plane : z;
}

__device__ __forceinline__ uint32_t pack_half2(float a, float b) {
  return uint32_t(__half_as_ushort(__float2half_rn(a))) | (uint32_t(__half_as_ushort(__float2half_rn(b))) << 16);
}
__device__ __forceinline__ float half_lo(uint32_t v) { return __half2float(__ushort_as_half((unsigned short)(v & 0xFFFFu))); }
__device__ __forceinline__ float half_hi(uint32_t v) { return __half2float(__ushort_as_half((unsigned short)(v >> 16))); }

// AO per pixel.  Classic: the pixel's own view position and reconstructed
// normal, samples at full resolution, the 16-bit jitter of texel
// (x & 3, y & 3).  CacheAware: the pixel belongs to deinterleaved layer
// (x & 3, y & 3) at quarter-resolution texel (x >> 2, y >> 2); its uv is that
// texel's centre in the layer, its normal the reconstructed one through an
// RGBA8 store, its samples are texels of the same layer at quarter-resolution
// steps (radius / 4), its jitter the layer's unquantized one; the result
// lands at the pixel, which is the reinterleave.  Special: (AO, view depth)
// stored as two halves.
template <bool CacheAware, bool Special>
__global__ void __launch_bounds__(256) hbao_ao_kernel(const HbaoScene* __restrict__ scenes, int count,
                                                      const float* __restrict__ depth, uint32_t* color,
                                                      void* q1, const HbaoParams p) {
  {
    const HbaoScene s = scenes[scene_of_block(scenes, count)];
    const int pixels = s.w * s.h;
    const float inv_w = __fdiv_rn(1.0f, float(s.w)), inv_h = __fdiv_rn(1.0f, float(s.h));
    const int idx = (int(blockIdx.x) - s.block0) * 256 + int(threadIdx.x);
    if (idx < pixels) {
      const int x = idx % s.w, y = idx / s.w;
      float u = __fdiv_rn(__fadd_rn(float(x), 0.5f), float(s.w));
      float v = __fdiv_rn(__fadd_rn(float(y), 0.5f), float(s.h));
      float3 P = view_pos(s, u, v, depth_at(s, depth, x, y));
      float inv_len;
      const float3 c = reconstruct_normal(s, depth, x, y, u, v, inv_w, inv_h, P, inv_len);
      float3 N;
      float radius;
      const float* j;
      float su_scale = inv_w, sv_scale = inv_h;
      const int ox = x & 3, oy = y & 3, qx = x >> 2, qy = y >> 2;
      if (!CacheAware) {
        N = f3(-__fmul_rn(c.x, inv_len), -__fmul_rn(c.y, inv_len), -__fmul_rn(c.z, inv_len));
        radius = __fdiv_rn(s.radius_to_screen, s.ortho ? 1.0f : P.z);
        j = p.jitter + 4 * ((y & 3) * 4 + (x & 3));
      } else {
        const float e[3] = {c.x, c.y, c.z};
        float n[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const float enc = float(unorm8(__fadd_rn(__fmul_rn(__fmul_rn(e[k], inv_len), 0.5f), 0.5f)));
          n[k] = -__fsub_rn(__fmul_rn(__fdiv_rn(enc, 255.0f), 2.0f), 1.0f);
        }
        N = f3(n[0], n[1], n[2]);
        u = __fmul_rn(__fadd_rn(__fmul_rn(float(qx), 4.0f), __fadd_rn(float(ox), 0.5f)), __fdiv_rn(s.inv_qw, 4.0f));
        v = __fmul_rn(__fadd_rn(__fmul_rn(float(qy), 4.0f), __fadd_rn(float(oy), 0.5f)), __fdiv_rn(s.inv_qh, 4.0f));
        P = view_pos(s, u, v, P.z);
        radius = __fdiv_rn(__fdiv_rn(s.radius_to_screen, s.ortho ? 1.0f : P.z), 4.0f);
        j = p.jitter_f + 4 * (oy * 4 + ox);
        su_scale = s.inv_qw;
        sv_scale = s.inv_qh;
      }
      const float step = __fdiv_rn(radius, 5.0f);
      float ao = 0.0f;
#pragma unroll
      for (int d = 0; d < 8; ++d) {
        const float dc = p.dirs[2 * d], ds = p.dirs[2 * d + 1];
        const float dx = __fsub_rn(__fmul_rn(dc, j[0]), __fmul_rn(ds, j[1]));
        const float dy = __fadd_rn(__fmul_rn(dc, j[1]), __fmul_rn(ds, j[0]));
        float ray = __fadd_rn(__fmul_rn(j[2], step), 1.0f);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const float kx = rintf(__fmul_rn(ray, dx)), ky = rintf(__fmul_rn(ray, dy));
          const float su = __fadd_rn(__fmul_rn(kx, su_scale), u), sv = __fadd_rn(__fmul_rn(ky, sv_scale), v);
          // Offsets beyond the image only select the clamped edge texel.
          const int ix = int(fminf(fmaxf(kx, -65536.0f), 65536.0f)), iy = int(fminf(fmaxf(ky, -65536.0f), 65536.0f));
          const float zs = CacheAware ? layer_depth(s, depth, qx + ix, qy + iy, ox, oy)
                                      : depth_at(s, depth, x + ix, y + iy);
          const float3 S = view_pos(s, su, sv, zs);
          ray = __fadd_rn(ray, step);
          const float3 V = sub(S, P);
          const float vv = dot3(V, V);
          const float ndotv = __fdiv_rn(dot3(N, V), __fsqrt_rn(vv));
          ao = __fadd_rn(ao, __fmul_rn(clamp01(__fsub_rn(ndotv, p.bias)),
                                       clamp01(__fadd_rn(__fmul_rn(vv, p.neg_inv_r2), 1.0f))));
        }
      }
      ao = __fmul_rn(ao, __fdiv_rn(p.ao_mult, 32.0f));
      const float occl = poly_pow(clamp01(__fsub_rn(1.0f, __fmul_rn(ao, 2.0f))), p.pow_exp);
      const long long at = s.offset + (long long)y * s.pitch + x;
      if (p.no_blur) {
        // The cache-aware result reaches the colour through its 8-bit layers.
        color[at] = modulate(color[at], CacheAware ? __fdiv_rn(float(unorm8(occl)), 255.0f) : occl);
      } else if (Special) {
        static_cast<uint32_t*>(q1)[at] = pack_half2(occl, P.z);
      } else {
        static_cast<uint8_t*>(q1)[at] = unorm8(occl);
      }
    }
  }
}

// One 7-tap pass along x (axis 0) or y (axis 1).  Bilateral: 8-bit AO, the
// depths from the linear-depth plane.  Special: (AO, depth) halves, the
// first pass storing (blurred AO, centre depth) as halves again.
template <int Axis, bool Special>
__global__ void __launch_bounds__(256) hbao_blur_kernel(const HbaoScene* __restrict__ scenes, int count,
                                                        const float* __restrict__ depth,
                                                        const void* __restrict__ src_v, void* dst_v,
                                                        uint32_t* color, const HbaoParams p) {
  const float falloff = 1.0f / (2.0f * 1.5f * 1.5f);
  const uint8_t* src8 = static_cast<const uint8_t*>(src_v);
  const uint32_t* src32 = static_cast<const uint32_t*>(src_v);
  {
    const HbaoScene s = scenes[scene_of_block(scenes, count)];
    const int pixels = s.w * s.h;
    const int idx = (int(blockIdx.x) - s.block0) * 256 + int(threadIdx.x);
    if (idx < pixels) {
      const int x = idx % s.w, y = idx / s.w;
      const long long at = s.offset + (long long)y * s.pitch + x;
      float cd, ct;
      if (Special) {
        const uint32_t c0 = src32[at];
        ct = half_lo(c0);
        cd = half_hi(c0);
      } else {
        cd = depth_at(s, depth, x, y);
        ct = __fdiv_rn(float(src8[at]), 255.0f);
      }
      float wt = 1.0f;
#pragma unroll
      for (int side = 0; side < 2; ++side) {
#pragma unroll
        for (int r = 1; r <= 3; ++r) {
          const int o = side == 0 ? r : -r;
          const int tx = Axis == 0 ? min(max(x + o, 0), s.w - 1) : x;
          const int ty = Axis == 1 ? min(max(y + o, 0), s.h - 1) : y;
          const long long t_at = s.offset + (long long)ty * s.pitch + tx;
          float c, dz;
          if (Special) {
            const uint32_t t = src32[t_at];
            c = half_lo(t);
            dz = half_hi(t);
          } else {
            c = __fdiv_rn(float(src8[t_at]), 255.0f);
            dz = depth_at(s, depth, tx, ty);
          }
          const float dd = __fmul_rn(__fsub_rn(dz, cd), p.sharpness);
          const float rf = float(r);
          const float w = poly_exp2(__fsub_rn(__fmul_rn(__fmul_rn(-rf, rf), falloff), __fmul_rn(dd, dd)));
          wt = __fadd_rn(wt, w);
          ct = __fadd_rn(ct, __fmul_rn(c, w));
        }
      }
      const float out = __fdiv_rn(ct, wt);
      if (Axis == 0) {
        if (Special)
          static_cast<uint32_t*>(dst_v)[at] = pack_half2(out, cd);
        else
          static_cast<uint8_t*>(dst_v)[at] = unorm8(out);
      } else {
        color[at] = modulate(color[at], out);
      }
    }
  }
}

template <bool CacheAware, bool Special>
void hbao_launch_t(const HbaoScene* d_scenes, int count, const dim3& grid, const float* depth, uint32_t* color,
                   void* q1, void* q2, const HbaoParams& p, cudaStream_t stream) {
  hbao_ao_kernel<CacheAware, Special><<<grid, 256, 0, stream>>>(d_scenes, count, depth, color, q1, p);
  if (!p.no_blur) {
    hbao_blur_kernel<0, Special><<<grid, 256, 0, stream>>>(d_scenes, count, depth, q1, q2, color, p);
    hbao_blur_kernel<1, Special><<<grid, 256, 0, stream>>>(d_scenes, count, depth, q2, nullptr, color, p);
  }
}

}  // namespace

// The jitter table before its 16-bit storage: the values the cache-aware
// algorithm passes per layer as a uniform (Hbao.cpp:603-617, 1000).
void hbao_jitter_unquantized(float out[64]) {
  std::mt19937 rmt;  // default seed, as the reference
  for (int i = 0; i < 16; ++i) {
    const float r1 = float(rmt()) / 4294967296.0f;
    const float r2 = float(rmt()) / 4294967296.0f;
    const float angle = 6.28318530718f * r1 / 8.0f;
    out[4 * i + 0] = float(std::cos(double(angle)));
    out[4 * i + 1] = float(std::sin(double(angle)));
    out[4 * i + 2] = r2;
    out[4 * i + 3] = 0.0f;
  }
}

bool hbao_params(const gbr_hbao_config& c, HbaoParams& p, std::string& err) {
  if (c.special_blur && c.no_blur) {
    err = "Hbao: no_blur and special_blur exclude each other (HbaoConfiguration::setNoBlur / setUseSpecialBlur)";
    return false;
  }
  if (c.algorithm != GBR_HBAO_CLASSIC && c.algorithm != GBR_HBAO_CACHE_AWARE) {
    err = "Hbao: unknown algorithm";
    return false;
  }
  if (!std::isfinite(c.radius) || !(c.radius > 0.0f) || !std::isfinite(c.intensity) ||
      !std::isfinite(c.bias) || !(c.bias < 1.0f) || !std::isfinite(c.blur_sharpness)) {
    err = "Hbao: bad configuration";
    return false;
  }
  std::memset(&p, 0, sizeof p);
  const float r = c.radius;  // metres to view space: 1
  const float r2 = r * r;
  p.neg_inv_r2 = -1.0f / r2;
  p.pow_exp = std::max(c.intensity, 0.0f);
  p.bias = std::min(std::max(c.bias, 0.0f), 1.0f);
  p.ao_mult = 1.0f / (1.0f - p.bias);
  p.sharpness = c.blur_sharpness / 1.0f;
  p.no_blur = c.no_blur ? 1 : 0;
  p.special = c.special_blur ? 1 : 0;
  p.cache_aware = c.algorithm == GBR_HBAO_CACHE_AWARE ? 1 : 0;
  gbr_hbao_jitter_table(p.jitter);
  hbao_jitter_unquantized(p.jitter_f);
  for (int d = 0; d < 8; ++d) {
    const float a = 2.0f * 3.14159265f / 8.0f * float(d);
    p.dirs[2 * d] = float(std::cos(double(a)));
    p.dirs[2 * d + 1] = float(std::sin(double(a)));
  }
  return true;
}

HbaoScene hbao_scene(const float* m, int w, int h, long long offset, long long pitch, float radius) {
  HbaoScene s{};
  s.offset = offset;
  s.pitch = pitch;
  s.w = w;
  s.h = h;
  s.qw = (w + 3) / 4;
  s.qh = (h + 3) / 4;
  s.inv_qw = 1.0f / float(s.qw);
  s.inv_qh = 1.0f / float(s.qh);
  const float p00 = m[0], p11 = m[5], p20 = m[8], p21 = m[9], p22 = m[10], p30 = m[12], p31 = m[13],
              p32 = m[14];
  s.ortho = m[15] != 0.0f ? 1 : 0;
  s.pi[0] = 2.0f / p00;
  s.pi[1] = 2.0f / p11;
  if (s.ortho) {
    s.pi[2] = -(1.0f + p30) / p00;
    s.pi[3] = -(1.0f - p31) / p11;
    s.far_plane = (p32 - 1.0f) / p22;
    s.radius_to_screen = radius * 0.5f * (float(h) / s.pi[1]);
  } else {
    s.pi[2] = -(1.0f - p20) / p00;
    s.pi[3] = -(1.0f + p21) / p11;
    s.far_plane = p32 / (p22 + 1.0f);
    s.radius_to_screen = radius * 0.5f * (0.5f * float(h) * p00);
  }
  return s;
}

cudaError_t hbao_launch(const HbaoScene* d_scenes, int count, int blocks, const float* depth,
                        uint32_t* color, void* q1, void* q2, const HbaoParams& p, cudaStream_t stream) {
  if (count <= 0 || blocks <= 0) return cudaSuccess;
  const dim3 grid(blocks);
  if (p.cache_aware) {
    if (p.special)
      hbao_launch_t<true, true>(d_scenes, count, grid, depth, color, q1, q2, p, stream);
    else
      hbao_launch_t<true, false>(d_scenes, count, grid, depth, color, q1, q2, p, stream);
  } else {
    if (p.special)
      hbao_launch_t<false, true>(d_scenes, count, grid, depth, color, q1, q2, p, stream);
    else
      hbao_launch_t<false, false>(d_scenes, count, grid, depth, color, q1, q2, p, stream);
  }
  return cudaGetLastError();
}

}  // namespace gbr

extern "C" {

void gbr_hbao_config_init(gbr_hbao_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->intensity = 0.732f;
  c->bias = 0.05f;
  c->radius = 1.84f;
  c->blur_sharpness = 10.0f;
}

gbr_status gbr_hbao_jitter_table(float out[64]) {
  if (!out) {
    gbr::set_last_error("null argument: out");
    return GBR_ERROR_INVALID_ARGUMENT;
  }
  std::mt19937 rmt;  // default seed, as the reference
  for (int i = 0; i < 16; ++i) {
    const float r1 = float(rmt()) / 4294967296.0f;
    const float r2 = float(rmt()) / 4294967296.0f;
    const float angle = 6.28318530718f * r1 / 8.0f;
    // cos / sin evaluated in double and rounded (the reference uses the
    // float functions; the 16-bit storage below hides the difference).
    const float v[3] = {float(std::cos(double(angle))), float(std::sin(double(angle))), r2};
    // RGBA16 snorm storage: round(v * 32767) / 32767, halves away from zero.
    for (int k = 0; k < 3; ++k) out[4 * i + k] = float(std::round(v[k] * 32767.0f)) / 32767.0f;
    out[4 * i + 3] = 0.0f;
  }
  return GBR_OK;
}

gbr_status gbr_hbao_apply(const gbr_hbao_config* config, const float projection[16], const float* depth,
                          uint32_t* color, int32_t w, int32_t h, int64_t pitch, void* stream) {
  if (!config || !projection || !depth || !color) {
    gbr::set_last_error("null argument");
    return GBR_ERROR_INVALID_ARGUMENT;
  }
  if (w <= 0 || h <= 0 || pitch < w || int64_t(w) * h > (int64_t(1) << 31) - 1) {
    gbr::set_last_error("Hbao: bad image size");
    return GBR_ERROR_INVALID_ARGUMENT;
  }
  gbr::HbaoParams p;
  std::string err;
  if (!gbr::hbao_params(*config, p, err)) {
    gbr::set_last_error(err);
    return GBR_ERROR_INVALID_ARGUMENT;
  }
  const gbr::HbaoScene s = gbr::hbao_scene(projection, w, h, 0, pitch, config->radius);
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  gbr::HbaoScene* d_scene = nullptr;
  uint8_t* q = nullptr;
  const size_t plane = size_t(pitch) * size_t(h) * size_t(gbr::hbao_plane_bytes(p));
  cudaError_t e = cudaMalloc(&d_scene, sizeof s);
  if (!e) e = cudaMalloc(&q, 2 * plane);
  if (!e) e = cudaMemcpyAsync(d_scene, &s, sizeof s, cudaMemcpyHostToDevice, st);
  if (!e) e = gbr::hbao_launch(d_scene, 1, int((int64_t(w) * h + 255) / 256), depth, color, q, q + plane, p, st);
  if (!e) e = cudaStreamSynchronize(st);
  cudaFree(d_scene);
  cudaFree(q);
  if (e) {
    gbr::set_last_error(std::string("Hbao: ") + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? GBR_ERROR_OUT_OF_MEMORY : GBR_ERROR_CUDA;
  }
  return GBR_OK;
}

}  // extern "C"
