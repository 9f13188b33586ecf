// Mip levels of RGBA8 textures: level k of a w x h texture is
// max(1, w >> k) x max(1, h >> k); the texel array holds level 0 of every
// layer, then level 1 of every layer, and so on (rows bottom-up).
#pragma once
#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <vector>

namespace gbr {

// Levels of a generated chain: floor(log2(min(w, h))) + 1, the count
// Renderer::addFile allocates for RendererFileFlag::GenerateMipmap
// (src/esp/gfx_batch/Renderer.cpp:445-450, 493-498).
inline int mip_chain_levels(int w, int h) {
  int m = std::min(w, h), l = 1;
  while (m > 1) {
    m >>= 1;
    ++l;
  }
  return l;
}

// Most levels a texture may have: floor(log2(max(w, h))) + 1.
inline int mip_max_levels(int w, int h) {
  int m = std::max(w, h), l = 1;
  while (m > 1) {
    m >>= 1;
    ++l;
  }
  return l;
}

inline size_t mip_texels(int w, int h, int layers, int levels) {
  size_t n = 0;
  for (int k = 0; k < levels; ++k) n += size_t(std::max(1, w >> k)) * size_t(std::max(1, h >> k)) * size_t(layers);
  return n;
}

// Levels 1 .. levels - 1 from level 0: each texel the rounded mean
// ((a + b + c + d + 2) >> 2 per channel) of the 2 x 2 texels above it,
// indices clamped to the finer level (GL leaves glGenerateMipmap's filter to
// the implementation; this is the box filter).
inline std::vector<uint8_t> generate_mips(const uint8_t* level0, int w, int h, int layers, int levels) {
  std::vector<uint8_t> out(mip_texels(w, h, layers, levels) * 4);
  const size_t n0 = size_t(w) * h * layers * 4;
  std::copy(level0, level0 + n0, out.begin());
  size_t prev = 0, cur = n0;
  for (int k = 1; k < levels; ++k) {
    const int pw = std::max(1, w >> (k - 1)), ph = std::max(1, h >> (k - 1));
    const int nw = std::max(1, w >> k), nh = std::max(1, h >> k);
    for (int L = 0; L < layers; ++L)
      for (int y = 0; y < nh; ++y)
        for (int x = 0; x < nw; ++x) {
          const int x0 = std::min(2 * x, pw - 1), x1 = std::min(2 * x + 1, pw - 1);
          const int y0 = std::min(2 * y, ph - 1), y1 = std::min(2 * y + 1, ph - 1);
          auto at = [&](int xx, int yy) { return prev + ((size_t(L) * ph + yy) * pw + xx) * 4; };
          const size_t o = cur + ((size_t(L) * nh + y) * nw + x) * 4;
          for (int c = 0; c < 4; ++c)
            out[o + c] = uint8_t((unsigned(out[at(x0, y0) + c]) + out[at(x1, y0) + c] + out[at(x0, y1) + c] +
                                  out[at(x1, y1) + c] + 2u) >> 2);
        }
    prev = cur;
    cur += size_t(nw) * nh * layers * 4;
  }
  return out;
}

}  // namespace gbr
