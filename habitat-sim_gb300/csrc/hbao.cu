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

__global__ void __launch_bounds__(256) hbao_ao_kernel(const HbaoScene* __restrict__ scenes, int count,
                                                      const float* __restrict__ depth, uint32_t* color,
                                                      uint8_t* q1, const HbaoParams p) {
  {
    const HbaoScene s = scenes[scene_of_block(scenes, count)];
    const int pixels = s.w * s.h;
    const float inv_w = __fdiv_rn(1.0f, float(s.w)), inv_h = __fdiv_rn(1.0f, float(s.h));
    const int idx = (int(blockIdx.x) - s.block0) * 256 + int(threadIdx.x);
    if (idx < pixels) {
      const int x = idx % s.w, y = idx / s.w;
      const float u = __fdiv_rn(__fadd_rn(float(x), 0.5f), float(s.w));
      const float v = __fdiv_rn(__fadd_rn(float(y), 0.5f), float(s.h));
      const float3 P = view_pos(s, u, v, depth_at(s, depth, x, y));
      const float3 pr = view_pos(s, __fadd_rn(u, inv_w), v, depth_at(s, depth, x + 1, y));
      const float3 pl = view_pos(s, __fadd_rn(u, -inv_w), v, depth_at(s, depth, x - 1, y));
      const float3 pt = view_pos(s, u, __fadd_rn(v, inv_h), depth_at(s, depth, x, y + 1));
      const float3 pb = view_pos(s, u, __fadd_rn(v, -inv_h), depth_at(s, depth, x, y - 1));
      const float3 c = cross3(min_diff(P, pr, pl), min_diff(P, pt, pb));
      const float inv_len = __fdiv_rn(1.0f, __fsqrt_rn(dot3(c, c)));
      const float3 N = f3(-__fmul_rn(c.x, inv_len), -__fmul_rn(c.y, inv_len), -__fmul_rn(c.z, inv_len));
      const float radius = __fdiv_rn(s.radius_to_screen, s.ortho ? 1.0f : P.z);
      const float step = __fdiv_rn(radius, 5.0f);
      const float* j = p.jitter + 4 * ((y & 3) * 4 + (x & 3));
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
          const float su = __fadd_rn(__fmul_rn(kx, inv_w), u), sv = __fadd_rn(__fmul_rn(ky, inv_h), v);
          // Offsets beyond the image only select the clamped edge texel.
          const int ox = int(fminf(fmaxf(kx, -65536.0f), 65536.0f)), oy = int(fminf(fmaxf(ky, -65536.0f), 65536.0f));
          const float3 S = view_pos(s, su, sv, depth_at(s, depth, x + ox, y + oy));
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
      if (p.no_blur)
        color[at] = modulate(color[at], occl);
      else
        q1[at] = unorm8(occl);
    }
  }
}

// One 7-tap pass along x (axis 0) or y (axis 1).
template <int Axis>
__global__ void __launch_bounds__(256) hbao_blur_kernel(const HbaoScene* __restrict__ scenes, int count,
                                                        const float* __restrict__ depth,
                                                        const uint8_t* __restrict__ src, uint8_t* dst,
                                                        uint32_t* color, const HbaoParams p) {
  const float falloff = 1.0f / (2.0f * 1.5f * 1.5f);
  {
    const HbaoScene s = scenes[scene_of_block(scenes, count)];
    const int pixels = s.w * s.h;
    const int idx = (int(blockIdx.x) - s.block0) * 256 + int(threadIdx.x);
    if (idx < pixels) {
      const int x = idx % s.w, y = idx / s.w;
      const long long at = s.offset + (long long)y * s.pitch + x;
      const float cd = depth_at(s, depth, x, y);
      float ct = __fdiv_rn(float(src[at]), 255.0f), wt = 1.0f;
#pragma unroll
      for (int side = 0; side < 2; ++side) {
#pragma unroll
        for (int r = 1; r <= 3; ++r) {
          const int o = side == 0 ? r : -r;
          const int tx = Axis == 0 ? min(max(x + o, 0), s.w - 1) : x;
          const int ty = Axis == 1 ? min(max(y + o, 0), s.h - 1) : y;
          const float c = __fdiv_rn(float(src[s.offset + (long long)ty * s.pitch + tx]), 255.0f);
          const float dd = __fmul_rn(__fsub_rn(depth_at(s, depth, tx, ty), cd), p.sharpness);
          const float rf = float(r);
          const float w = poly_exp2(__fsub_rn(__fmul_rn(__fmul_rn(-rf, rf), falloff), __fmul_rn(dd, dd)));
          wt = __fadd_rn(wt, w);
          ct = __fadd_rn(ct, __fmul_rn(c, w));
        }
      }
      const float out = __fdiv_rn(ct, wt);
      if (Axis == 0)
        dst[at] = unorm8(out);
      else
        color[at] = modulate(color[at], out);
    }
  }
}

}  // namespace

bool hbao_params(const gbr_hbao_config& c, HbaoParams& p, std::string& err) {
  if (c.special_blur) {
    err = "Hbao: the special blur variant is not available";
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
  gbr_hbao_jitter_table(p.jitter);
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
                        uint32_t* color, uint8_t* q1, uint8_t* q2, const HbaoParams& p, cudaStream_t stream) {
  if (count <= 0 || blocks <= 0) return cudaSuccess;
  const dim3 grid(blocks);
  hbao_ao_kernel<<<grid, 256, 0, stream>>>(d_scenes, count, depth, color, q1, p);
  if (!p.no_blur) {
    hbao_blur_kernel<0><<<grid, 256, 0, stream>>>(d_scenes, count, depth, q1, q2, color, p);
    hbao_blur_kernel<1><<<grid, 256, 0, stream>>>(d_scenes, count, depth, q2, nullptr, color, p);
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
  const size_t plane = size_t(pitch) * size_t(h);
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
