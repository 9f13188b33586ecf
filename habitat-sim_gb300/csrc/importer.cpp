// glTF 2.0 importer for Renderer::addFile (src/esp/gfx_batch/Renderer.cpp:354-867).
//
// The reference delegates file parsing to Magnum's importer plugins; this
// file implements the subset the batch renderer consumes, following the
// published glTF 2.0, KHR_texture_transform, KHR_texture_ktx, KTX2, PNG
// (RFC 2083) and DEFLATE (RFC 1951) specifications, with the Magnum
// conventions the renderer relies on:
//   - images and texture coordinates use a bottom-left origin (PNG rows
//     flipped, KTX2 rows flipped unless KTXorientation says "u", v' = 1 - v),
//     KHR_texture_transform converted to that space;
//   - KHR_texture_ktx textures sharing one image and sampler import as one
//     2D array texture, the layer moves to the material;
//   - meshes become indexed triangle lists (fans and strips expanded);
//   - MAGNUMX_mesh_views extras give per-node index ranges and materials
//     (Renderer.cpp:700-738); named root nodes are hierarchy templates whose
//     immediate children are the mesh views (Renderer.cpp:750-790); the
//     Whole flag flattens the file with absolute transforms (:795-820);
//     a file without scenes holds exactly one mesh (:663-690).
#include "importer.h"
#include "json.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>

namespace gbr {
namespace {

// --------------------------------------------------------------- inflate
struct BitReader {
  const uint8_t* d;
  size_t n, pos = 0;
  uint32_t bitbuf = 0;
  int bitcnt = 0;
  bool bad = false;
  int bits(int k) {
    while (bitcnt < k) {
      if (pos >= n) { bad = true; return 0; }
      bitbuf |= uint32_t(d[pos++]) << bitcnt;
      bitcnt += 8;
    }
    int v = int(bitbuf & ((1u << k) - 1));
    bitbuf >>= k;
    bitcnt -= k;
    return v;
  }
};

struct Huffman {
  uint16_t count[16] = {0};
  uint16_t symbol[320] = {0};
  void build(const uint8_t* lengths, int n) {
    std::memset(count, 0, sizeof(count));
    for (int i = 0; i < n; ++i) count[lengths[i]]++;
    count[0] = 0;
    uint16_t offs[16];
    offs[1] = 0;
    for (int i = 1; i < 15; ++i) offs[i + 1] = offs[i] + count[i];
    for (int i = 0; i < n; ++i)
      if (lengths[i]) symbol[offs[lengths[i]]++] = uint16_t(i);
  }
  int decode(BitReader& br) const {
    int code = 0, first = 0, index = 0;
    for (int len = 1; len < 16; ++len) {
      code |= br.bits(1);
      int c = count[len];
      if (code - c < first) return symbol[index + (code - first)];
      index += c;
      first += c;
      first <<= 1;
      code <<= 1;
      if (br.bad) return -1;
    }
    return -1;
  }
};

bool inflate(const uint8_t* data, size_t size, std::vector<uint8_t>& out) {
  static const uint16_t lbase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27,
                                     31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
  static const uint8_t lext[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2,
                                   2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
  static const uint16_t dbase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129,
                                     193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097,
                                     6145, 8193, 12289, 16385, 24577};
  static const uint8_t dext[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6,
                                   6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
  BitReader br{data, size};
  int last;
  do {
    last = br.bits(1);
    int type = br.bits(2);
    if (br.bad) return false;
    if (type == 0) {
      br.bitbuf = 0;
      br.bitcnt = 0;
      if (br.pos + 4 > size) return false;
      uint16_t len = uint16_t(data[br.pos] | (data[br.pos + 1] << 8));
      br.pos += 4;
      if (br.pos + len > size) return false;
      out.insert(out.end(), data + br.pos, data + br.pos + len);
      br.pos += len;
      continue;
    }
    Huffman lit, dist;
    if (type == 1) {
      uint8_t l[288];
      for (int i = 0; i < 144; ++i) l[i] = 8;
      for (int i = 144; i < 256; ++i) l[i] = 9;
      for (int i = 256; i < 280; ++i) l[i] = 7;
      for (int i = 280; i < 288; ++i) l[i] = 8;
      lit.build(l, 288);
      uint8_t dl[30];
      for (int i = 0; i < 30; ++i) dl[i] = 5;
      dist.build(dl, 30);
    } else if (type == 2) {
      int hlit = br.bits(5) + 257, hdist = br.bits(5) + 1, hclen = br.bits(4) + 4;
      static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
      uint8_t cl[19] = {0};
      for (int i = 0; i < hclen; ++i) cl[order[i]] = uint8_t(br.bits(3));
      Huffman clh;
      clh.build(cl, 19);
      uint8_t lens[320] = {0};
      int idx = 0;
      while (idx < hlit + hdist) {
        int sym = clh.decode(br);
        if (sym < 0 || br.bad) return false;
        if (sym < 16) {
          lens[idx++] = uint8_t(sym);
        } else {
          int rep = 0;
          uint8_t val = 0;
          if (sym == 16) {
            if (idx == 0) return false;
            val = lens[idx - 1];
            rep = 3 + br.bits(2);
          } else if (sym == 17) {
            rep = 3 + br.bits(3);
          } else {
            rep = 11 + br.bits(7);
          }
          if (idx + rep > hlit + hdist) return false;
          while (rep--) lens[idx++] = val;
        }
      }
      lit.build(lens, hlit);
      dist.build(lens + hlit, hdist);
    } else {
      return false;
    }
    for (;;) {
      int sym = lit.decode(br);
      if (sym < 0 || br.bad) return false;
      if (sym < 256) {
        out.push_back(uint8_t(sym));
      } else if (sym == 256) {
        break;
      } else {
        sym -= 257;
        if (sym >= 29) return false;
        int len = lbase[sym] + br.bits(lext[sym]);
        int ds = dist.decode(br);
        if (ds < 0 || ds >= 30) return false;
        size_t d = dbase[ds] + br.bits(dext[ds]);
        if (br.bad || d > out.size()) return false;
        size_t from = out.size() - d;
        for (int i = 0; i < len; ++i) out.push_back(out[from + i]);
      }
    }
  } while (!last);
  return true;
}

uint32_t be32(const uint8_t* p) {
  return (uint32_t(p[0]) << 24) | (uint32_t(p[1]) << 16) | (uint32_t(p[2]) << 8) | p[3];
}
uint32_t le32(const uint8_t* p) {
  return uint32_t(p[0]) | (uint32_t(p[1]) << 8) | (uint32_t(p[2]) << 16) | (uint32_t(p[3]) << 24);
}
uint64_t le64(const uint8_t* p) { return uint64_t(le32(p)) | (uint64_t(le32(p + 4)) << 32); }

bool read_file(const std::string& path, std::vector<uint8_t>& out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  f.seekg(0, std::ios::end);
  std::streamoff n = f.tellg();
  if (n < 0) return false;
  f.seekg(0);
  out.resize(size_t(n));
  if (n) f.read(reinterpret_cast<char*>(out.data()), n);
  return bool(f);
}

std::string dirname(const std::string& p) {
  size_t s = p.find_last_of('/');
  return s == std::string::npos ? std::string() : p.substr(0, s + 1);
}

}  // namespace

void mat4_mul(const float* a, const float* b, float* c) {
  float r[16];
  for (int col = 0; col < 4; ++col)
    for (int row = 0; row < 4; ++row) {
      float s = a[row] * b[col * 4];
      for (int k = 1; k < 4; ++k) s = s + a[k * 4 + row] * b[col * 4 + k];
      r[col * 4 + row] = s;
    }
  std::memcpy(c, r, sizeof(r));
}

// ------------------------------------------------------------------- PNG
bool decode_png(const uint8_t* d, size_t n, ImportedTexture& out, std::string& err) {
  static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', 0x0d, 0x0a, 0x1a, 0x0a};
  if (n < 8 || std::memcmp(d, sig, 8)) { err = "not a PNG"; return false; }
  size_t pos = 8;
  uint32_t w = 0, h = 0;
  int depth = 0, ctype = 0, interlace = 0;
  std::vector<uint8_t> idat, palette, trns;
  while (pos + 12 <= n) {
    uint32_t len = be32(d + pos);
    const uint8_t* tag = d + pos + 4;
    const uint8_t* body = d + pos + 8;
    if (pos + 12 + size_t(len) > n) { err = "truncated PNG"; return false; }
    if (!std::memcmp(tag, "IHDR", 4)) {
      w = be32(body);
      h = be32(body + 4);
      depth = body[8];
      ctype = body[9];
      interlace = body[12];
    } else if (!std::memcmp(tag, "PLTE", 4)) {
      palette.assign(body, body + len);
    } else if (!std::memcmp(tag, "tRNS", 4)) {
      trns.assign(body, body + len);
    } else if (!std::memcmp(tag, "IDAT", 4)) {
      idat.insert(idat.end(), body, body + len);
    } else if (!std::memcmp(tag, "IEND", 4)) {
      break;
    }
    pos += 12 + len;
  }
  if (depth != 8 || interlace != 0) { err = "only 8-bit non-interlaced PNG is supported"; return false; }
  int ch;
  switch (ctype) {
    case 0: ch = 1; break;
    case 2: ch = 3; break;
    case 3: ch = 1; break;
    case 4: ch = 2; break;
    case 6: ch = 4; break;
    default: err = "bad PNG colour type"; return false;
  }
  if (idat.size() < 2) { err = "PNG without image data"; return false; }
  std::vector<uint8_t> raw;
  if (!inflate(idat.data() + 2, idat.size() - 2, raw)) { err = "corrupt PNG stream"; return false; }
  const size_t stride = size_t(w) * ch;
  if (raw.size() < (stride + 1) * h) { err = "short PNG stream"; return false; }
  std::vector<uint8_t> px(stride * h);
  for (uint32_t y = 0; y < h; ++y) {
    const uint8_t ft = raw[y * (stride + 1)];
    const uint8_t* line = &raw[y * (stride + 1) + 1];
    uint8_t* cur = &px[y * stride];
    const uint8_t* prev = y ? &px[(y - 1) * stride] : nullptr;
    for (size_t i = 0; i < stride; ++i) {
      int a = i >= size_t(ch) ? cur[i - ch] : 0;
      int b = prev ? prev[i] : 0;
      int c = (prev && i >= size_t(ch)) ? prev[i - ch] : 0;
      int pred = 0;
      switch (ft) {
        case 0: pred = 0; break;
        case 1: pred = a; break;
        case 2: pred = b; break;
        case 3: pred = (a + b) >> 1; break;
        case 4: {
          int pa = std::abs(b - c), pb = std::abs(a - c), pc = std::abs(a + b - 2 * c);
          pred = (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
          break;
        }
        default: err = "bad PNG filter"; return false;
      }
      cur[i] = uint8_t((line[i] + pred) & 255);
    }
  }
  out.width = int(w);
  out.height = int(h);
  out.layers = 1;
  out.rgba.resize(size_t(w) * h * 4);
  for (uint32_t y = 0; y < h; ++y)
    for (uint32_t x = 0; x < w; ++x) {
      const uint8_t* s = &px[y * stride + x * ch];
      uint8_t* o = &out.rgba[((size_t(h - 1 - y)) * w + x) * 4];  // flip: row 0 = bottom
      switch (ctype) {
        case 0: o[0] = o[1] = o[2] = s[0]; o[3] = 255; break;
        case 2: o[0] = s[0]; o[1] = s[1]; o[2] = s[2]; o[3] = 255; break;
        case 3: {
          size_t k = s[0];
          if (k * 3 + 2 >= palette.size()) { err = "bad palette index"; return false; }
          o[0] = palette[k * 3]; o[1] = palette[k * 3 + 1]; o[2] = palette[k * 3 + 2];
          o[3] = k < trns.size() ? trns[k] : 255;
          break;
        }
        case 4: o[0] = o[1] = o[2] = s[0]; o[3] = s[1]; break;
        default: std::memcpy(o, s, 4);
      }
    }
  return true;
}

// ------------------------------------------------------------------ KTX2
namespace {
void bc1_block(const uint8_t* b, uint8_t out[16][4]) {
  const uint32_t c0 = b[0] | (b[1] << 8), c1 = b[2] | (b[3] << 8);
  const uint32_t bits = le32(b + 4);
  int p[4][4];
  auto expand = [](uint32_t c, int* o) {
    int r = (c >> 11) & 31, g = (c >> 5) & 63, bl = c & 31;
    o[0] = (r << 3) | (r >> 2);
    o[1] = (g << 2) | (g >> 4);
    o[2] = (bl << 3) | (bl >> 2);
    o[3] = 255;
  };
  expand(c0, p[0]);
  expand(c1, p[1]);
  for (int k = 0; k < 3; ++k) {
    if (c0 > c1) {
      p[2][k] = (2 * p[0][k] + p[1][k]) / 3;
      p[3][k] = (p[0][k] + 2 * p[1][k]) / 3;
    } else {
      p[2][k] = (p[0][k] + p[1][k]) / 2;
      p[3][k] = 0;
    }
  }
  p[2][3] = p[3][3] = 255;
  for (int i = 0; i < 16; ++i) {
    int s = (bits >> (2 * i)) & 3;
    for (int k = 0; k < 4; ++k) out[i][k] = uint8_t(p[s][k]);
  }
}
}  // namespace

bool decode_ktx2(const uint8_t* d, size_t n, ImportedTexture& out, std::string& err) {
  static const uint8_t id[12] = {0xAB, 'K', 'T', 'X', ' ', '2', '0', 0xBB, '\r', '\n', 0x1A, '\n'};
  if (n < 104 || std::memcmp(d, id, 12)) { err = "not a KTX2 file"; return false; }
  const uint32_t vk = le32(d + 12), w = le32(d + 20), h0 = le32(d + 24), depth = le32(d + 28),
                 layers = le32(d + 32), faces = le32(d + 36), sc = le32(d + 44);
  if (sc != 0 || faces != 1 || depth > 1) { err = "unsupported KTX2 layout"; return false; }
  const uint32_t kvo = le32(d + 56), kvl = le32(d + 60);
  const uint64_t off = le64(d + 80), len = le64(d + 88);
  std::string orient = "rd";
  for (size_t p = kvo; p + 4 <= size_t(kvo) + kvl && p + 4 <= n;) {
    uint32_t el = le32(d + p);
    if (p + 4 + el > n) break;
    std::string entry(reinterpret_cast<const char*>(d + p + 4), el);
    size_t z = entry.find('\0');
    if (z != std::string::npos && entry.substr(0, z) == "KTXorientation") {
      std::string v = entry.substr(z + 1);
      v = v.substr(0, v.find('\0'));
      orient = v;
    }
    p += 4 + ((el + 3) & ~3u);
  }
  const uint32_t nl = std::max<uint32_t>(layers, 1), h = std::max<uint32_t>(h0, 1);
  if (off + len > n) { err = "truncated KTX2 level"; return false; }
  const uint8_t* lv = d + off;
  out.width = int(w);
  out.height = int(h);
  out.layers = int(nl);
  out.rgba.assign(size_t(nl) * h * w * 4, 0);
  if (vk == 23 || vk == 29 || vk == 37 || vk == 43) {
    const int ch = (vk == 23 || vk == 29) ? 3 : 4;
    if (len < uint64_t(nl) * h * w * ch) { err = "short KTX2 level"; return false; }
    for (size_t i = 0; i < size_t(nl) * h * w; ++i) {
      for (int k = 0; k < ch; ++k) out.rgba[i * 4 + k] = lv[i * ch + k];
      if (ch == 3) out.rgba[i * 4 + 3] = 255;
    }
  } else if (vk >= 131 && vk <= 134) {
    out.compressed = true;
    const uint32_t bw = (w + 3) / 4, bh = (h + 3) / 4;
    if (len < uint64_t(nl) * bw * bh * 8) { err = "short KTX2 BC1 level"; return false; }
    size_t q = 0;
    for (uint32_t L = 0; L < nl; ++L)
      for (uint32_t by = 0; by < bh; ++by)
        for (uint32_t bx = 0; bx < bw; ++bx, q += 8) {
          uint8_t blk[16][4];
          bc1_block(lv + q, blk);
          for (int i = 0; i < 16; ++i) {
            uint32_t x = bx * 4 + (i % 4), y = by * 4 + (i / 4);
            if (x < w && y < h) std::memcpy(&out.rgba[((size_t(L) * h + y) * w + x) * 4], blk[i], 4);
          }
        }
  } else {
    err = "unsupported KTX2 vkFormat " + std::to_string(vk);
    return false;
  }
  if (orient.size() > 1 && orient[1] == 'd') {
    std::vector<uint8_t> f(out.rgba.size());
    for (uint32_t L = 0; L < nl; ++L)
      for (uint32_t y = 0; y < h; ++y)
        std::memcpy(&f[((size_t(L) * h + y) * w) * 4], &out.rgba[((size_t(L) * h + (h - 1 - y)) * w) * 4],
                    size_t(w) * 4);
    out.rgba.swap(f);
  }
  return true;
}

// ------------------------------------------------------------------ glTF
namespace {

struct Doc {
  Json j;
  std::vector<std::vector<uint8_t>> buffers;
  std::string base;
  std::string err;

  bool viewBytes(int i, const uint8_t*& ptr, size_t& len, size_t& stride) {
    const Json* views = j.get("bufferViews");
    if (!views || i < 0 || size_t(i) >= views->size()) { err = "bad bufferView"; return false; }
    const Json& v = (*views)[i];
    size_t b = size_t(v.numberOr("buffer", 0));
    size_t off = size_t(v.numberOr("byteOffset", 0));
    len = size_t(v.numberOr("byteLength", 0));
    stride = size_t(v.numberOr("byteStride", 0));
    if (b >= buffers.size() || off + len > buffers[b].size()) { err = "bufferView out of range"; return false; }
    ptr = buffers[b].data() + off;
    return true;
  }

  // Reads accessor i as float (normalised ints mapped to [0,1]) or uint32.
  bool accessor(int i, int& ncomp, std::vector<double>& outv) {
    const Json* accs = j.get("accessors");
    if (!accs || i < 0 || size_t(i) >= accs->size()) { err = "bad accessor"; return false; }
    const Json& a = (*accs)[i];
    const int ct = int(a.numberOr("componentType", 0));
    const size_t count = size_t(a.numberOr("count", 0));
    const Json* type = a.get("type");
    std::string t = type ? type->str : "";
    ncomp = t == "SCALAR" ? 1 : t == "VEC2" ? 2 : t == "VEC3" ? 3 : t == "VEC4" ? 4 : t == "MAT4" ? 16 : 0;
    if (!ncomp) { err = "bad accessor type"; return false; }
    int cs = (ct == 5120 || ct == 5121) ? 1 : (ct == 5122 || ct == 5123) ? 2 : (ct == 5125 || ct == 5126) ? 4 : 0;
    if (!cs) { err = "bad componentType"; return false; }
    const Json* nj = a.get("normalized");
    const bool norm = nj && nj->type == Json::Bool && nj->b;
    outv.assign(count * ncomp, 0.0);
    const Json* bvj = a.get("bufferView");
    if (!bvj) return true;  // all zeros
    const uint8_t* p;
    size_t len, stride;
    if (!viewBytes(int(bvj->num), p, len, stride)) return false;
    const size_t aoff = size_t(a.numberOr("byteOffset", 0));
    const size_t elem = size_t(cs) * ncomp;
    if (!stride) stride = elem;
    if (count && aoff + (count - 1) * stride + elem > len) { err = "accessor out of range"; return false; }
    for (size_t k = 0; k < count; ++k)
      for (int c = 0; c < ncomp; ++c) {
        const uint8_t* e = p + aoff + k * stride + size_t(c) * cs;
        double v = 0;
        switch (ct) {
          case 5120: { int8_t x; std::memcpy(&x, e, 1); v = norm ? double(float(x) / 127.0f) : x; break; }
          case 5121: v = norm ? double(float(e[0]) / 255.0f) : e[0]; break;
          case 5122: { int16_t x; std::memcpy(&x, e, 2); v = norm ? double(float(x) / 32767.0f) : x; break; }
          case 5123: { uint16_t x; std::memcpy(&x, e, 2); v = norm ? double(float(x) / 65535.0f) : x; break; }
          case 5125: { uint32_t x; std::memcpy(&x, e, 4); v = x; break; }
          case 5126: { float x; std::memcpy(&x, e, 4); v = x; break; }
        }
        outv[k * ncomp + c] = v;
      }
    return true;
  }
};

void node_matrix(const Json& nd, float* m) {
  const Json* mat = nd.get("matrix");
  if (mat && mat->size() == 16) {
    for (int i = 0; i < 16; ++i) m[i] = float((*mat)[i].num);
    return;
  }
  double t[3] = {0, 0, 0}, q[4] = {0, 0, 0, 1}, s[3] = {1, 1, 1};
  if (const Json* tj = nd.get("translation"))
    for (int i = 0; i < 3 && size_t(i) < tj->size(); ++i) t[i] = (*tj)[i].num;
  if (const Json* rj = nd.get("rotation"))
    for (int i = 0; i < 4 && size_t(i) < rj->size(); ++i) q[i] = (*rj)[i].num;
  if (const Json* sj = nd.get("scale"))
    for (int i = 0; i < 3 && size_t(i) < sj->size(); ++i) s[i] = (*sj)[i].num;
  const double x = q[0], y = q[1], z = q[2], w = q[3];
  const double r[3][3] = {{1 - 2 * (y * y + z * z), 2 * (x * y + z * w), 2 * (x * z - y * w)},
                          {2 * (x * y - z * w), 1 - 2 * (x * x + z * z), 2 * (y * z + x * w)},
                          {2 * (x * z + y * w), 2 * (y * z - x * w), 1 - 2 * (x * x + y * y)}};
  for (int c = 0; c < 3; ++c) {
    for (int rr = 0; rr < 3; ++rr) m[c * 4 + rr] = float(r[c][rr] * s[c]);
    m[c * 4 + 3] = 0.0f;
  }
  m[12] = float(t[0]);
  m[13] = float(t[1]);
  m[14] = float(t[2]);
  m[15] = 1.0f;
}

void texture_transform(const Json& tt, float* out) {
  double off[2] = {0, 0}, sc[2] = {1, 1}, rot = tt.numberOr("rotation", 0.0);
  if (const Json* o = tt.get("offset"))
    for (int i = 0; i < 2 && size_t(i) < o->size(); ++i) off[i] = (*o)[i].num;
  if (const Json* s = tt.get("scale"))
    for (int i = 0; i < 2 && size_t(i) < s->size(); ++i) sc[i] = (*s)[i].num;
  const double c = std::cos(rot), s = std::sin(rot);
  // glTF (Y-down) matrix, row-major acting on column vectors: T * R * S.
  const double mg[3][3] = {{c * sc[0], s * sc[1], off[0]}, {-s * sc[0], c * sc[1], off[1]}, {0, 0, 1}};
  // Y-up: F * M * F with F = [[1,0,0],[0,-1,1],[0,0,1]].
  const double F[3][3] = {{1, 0, 0}, {0, -1, 1}, {0, 0, 1}};
  double t1[3][3], t2[3][3];
  for (int i = 0; i < 3; ++i)
    for (int k = 0; k < 3; ++k) {
      t1[i][k] = 0;
      for (int l = 0; l < 3; ++l) t1[i][k] += F[i][l] * mg[l][k];
    }
  for (int i = 0; i < 3; ++i)
    for (int k = 0; k < 3; ++k) {
      t2[i][k] = 0;
      for (int l = 0; l < 3; ++l) t2[i][k] += t1[i][l] * F[l][k];
    }
  for (int col = 0; col < 3; ++col)
    for (int row = 0; row < 3; ++row) out[col * 3 + row] = float(t2[row][col]);
}

}  // namespace

bool import_gltf(const std::string& path, bool whole, const std::string& name, bool no_textures,
                 ImportedFile& out, std::string& error) {
  std::vector<uint8_t> raw;
  if (!read_file(path, raw)) { error = "can't open the file " + path; return false; }
  Doc doc;
  doc.base = dirname(path);
  std::vector<uint8_t> bin_chunk;
  const uint8_t* jsonp = raw.data();
  size_t jsonn = raw.size();
  if (raw.size() >= 12 && !std::memcmp(raw.data(), "glTF", 4)) {
    size_t total = std::min<size_t>(le32(raw.data() + 8), raw.size());
    size_t p = 12;
    jsonn = 0;
    while (p + 8 <= total) {
      uint32_t cl = le32(raw.data() + p), ct = le32(raw.data() + p + 4);
      if (p + 8 + cl > total) break;
      if (ct == 0x4E4F534Au) { jsonp = raw.data() + p + 8; jsonn = cl; }
      if (ct == 0x004E4942u) bin_chunk.assign(raw.data() + p + 8, raw.data() + p + 8 + cl);
      p += 8 + cl;
    }
  }
  JsonParser jp{reinterpret_cast<const char*>(jsonp), reinterpret_cast<const char*>(jsonp) + jsonn, {}};
  if (!jp.parse(doc.j) || doc.j.type != Json::Object) {
    error = "can't parse " + path + ": " + jp.err;
    return false;
  }
  if (const Json* bufs = doc.j.get("buffers"))
    for (size_t i = 0; i < bufs->size(); ++i) {
      const Json* uri = (*bufs)[i].get("uri");
      std::vector<uint8_t> b;
      if (uri) {
        if (!read_file(doc.base + uri->str, b)) { error = "can't open buffer " + uri->str; return false; }
      } else {
        b = bin_chunk;
      }
      doc.buffers.push_back(std::move(b));
    }

  // ---- textures
  std::vector<std::pair<int, int>> texture_map;  // glTF texture -> (file texture id, layer)
  {
    std::map<std::pair<long, long>, int> dedup;
    const Json* texs = doc.j.get("textures");
    int next_id = 0;
    for (size_t ti = 0; texs && ti < texs->size(); ++ti) {
      const Json& tex = (*texs)[ti];
      const Json* ext = nullptr;
      if (const Json* e = tex.get("extensions")) ext = e->get("KHR_texture_ktx");
      const long src = long(ext ? ext->numberOr("source", 0) : tex.numberOr("source", 0));
      const int layer = ext ? int(ext->numberOr("layer", 0)) : 0;
      const long smp = long(tex.numberOr("sampler", -1));
      std::pair<long, long> key = ext ? std::make_pair(src, smp) : std::make_pair(-1L - long(ti), -1L);
      auto it = dedup.find(key);
      if (it == dedup.end()) {
        it = dedup.emplace(key, next_id++).first;
        if (!no_textures) {
          ImportedTexture t;
          const Json* imgs = doc.j.get("images");
          if (!imgs || src < 0 || size_t(src) >= imgs->size()) { error = "bad image index"; return false; }
          const Json& img = (*imgs)[size_t(src)];
          std::vector<uint8_t> blob;
          std::string mime;
          if (const Json* bv = img.get("bufferView")) {
            const uint8_t* p;
            size_t len, stride;
            if (!doc.viewBytes(int(bv->num), p, len, stride)) { error = doc.err; return false; }
            blob.assign(p, p + len);
            if (const Json* m = img.get("mimeType")) mime = m->str;
          } else if (const Json* uri = img.get("uri")) {
            if (!read_file(doc.base + uri->str, blob)) { error = "can't open image " + uri->str; return false; }
          }
          std::string err;
          bool ok;
          if (blob.size() >= 4 && blob[0] == 0xAB && blob[1] == 'K')
            ok = decode_ktx2(blob.data(), blob.size(), t, err);
          else
            ok = decode_png(blob.data(), blob.size(), t, err);
          if (!ok) { error = "can't import image of " + path + ": " + err; return false; }
          int mag = 9729, minf = 9987, ws = 10497, wt = 10497;
          const Json* smps = doc.j.get("samplers");
          if (smp >= 0 && smps && size_t(smp) < smps->size()) {
            const Json& s = (*smps)[size_t(smp)];
            mag = int(s.numberOr("magFilter", 9729));
            minf = int(s.numberOr("minFilter", 9987));
            ws = int(s.numberOr("wrapS", 10497));
            wt = int(s.numberOr("wrapT", 10497));
          }
          auto wrap = [](int g) { return g == 33071 ? 1 : g == 33648 ? 2 : 0; };
          t.filter = mag == 9728 ? 0 : 1;
          // minFilter: NEAREST / LINEAR, then {NEAREST, LINEAR}_MIPMAP_{NEAREST, LINEAR}.
          t.min_filter = (minf == 9728 || minf == 9984 || minf == 9986) ? 0 : 1;
          t.mip_filter = (minf == 9984 || minf == 9985) ? 1 : (minf == 9986 || minf == 9987) ? 2 : 0;
          t.wrap_s = wrap(ws);
          t.wrap_t = wrap(wt);
          out.textures.push_back(std::move(t));
        }
      }
      texture_map.emplace_back(it->second, layer);
    }
  }

  // ---- meshes (one per primitive)
  std::vector<std::vector<uint32_t>> mesh_ids;      // glTF mesh -> imported mesh ids
  std::vector<std::vector<int>> mesh_materials;     // glTF mesh -> primitive materials
  if (const Json* meshes = doc.j.get("meshes"))
    for (size_t mi = 0; mi < meshes->size(); ++mi) {
      mesh_ids.emplace_back();
      mesh_materials.emplace_back();
      const Json* prims = (*meshes)[mi].get("primitives");
      for (size_t pi = 0; prims && pi < prims->size(); ++pi) {
        const Json& prim = (*prims)[pi];
        const Json* attrs = prim.get("attributes");
        const Json* pa = attrs ? attrs->get("POSITION") : nullptr;
        if (!pa) { error = "mesh without positions in " + path; return false; }
        ImportedMesh m;
        int nc;
        std::vector<double> v;
        if (!doc.accessor(int(pa->num), nc, v) || nc != 3) { error = "bad POSITION: " + doc.err; return false; }
        m.vertex_count = uint32_t(v.size() / 3);
        m.positions.assign(v.begin(), v.end());
        if (const Json* cj = attrs->get("COLOR_0")) {
          if (!doc.accessor(int(cj->num), nc, v) || nc < 3) { error = "bad COLOR_0"; return false; }
          m.colors.assign(size_t(m.vertex_count) * 4, 1.0f);
          for (uint32_t k = 0; k < m.vertex_count; ++k)
            for (int c = 0; c < nc && c < 4; ++c) m.colors[k * 4 + c] = float(v[k * nc + c]);
        }
        if (const Json* tj = attrs->get("TEXCOORD_0")) {
          if (!doc.accessor(int(tj->num), nc, v) || nc != 2) { error = "bad TEXCOORD_0"; return false; }
          m.texcoords.resize(size_t(m.vertex_count) * 2);
          for (uint32_t k = 0; k < m.vertex_count; ++k) {
            m.texcoords[k * 2] = float(v[k * 2]);
            m.texcoords[k * 2 + 1] = 1.0f - float(v[k * 2 + 1]);
          }
        }
        if (const Json* nj = attrs->get("NORMAL")) {
          if (!doc.accessor(int(nj->num), nc, v) || nc != 3) { error = "bad NORMAL"; return false; }
          m.normals.assign(v.begin(), v.end());
        }
        if (const Json* oj = attrs->get("_OBJECT_ID")) {
          if (!doc.accessor(int(oj->num), nc, v) || nc != 1) { error = "bad _OBJECT_ID"; return false; }
          m.object_ids.resize(m.vertex_count);
          for (uint32_t k = 0; k < m.vertex_count; ++k) m.object_ids[k] = uint32_t(v[k]);
        }
        std::vector<uint32_t> idx;
        if (const Json* ij = prim.get("indices")) {
          if (!doc.accessor(int(ij->num), nc, v) || nc != 1) { error = "bad indices"; return false; }
          idx.assign(v.begin(), v.end());
        } else {
          idx.resize(m.vertex_count);
          for (uint32_t k = 0; k < m.vertex_count; ++k) idx[k] = k;
        }
        const int mode = int(prim.numberOr("mode", 4));
        if (mode == 6) {
          for (size_t k = 1; k + 1 < idx.size(); ++k) {
            m.indices.push_back(idx[0]);
            m.indices.push_back(idx[k]);
            m.indices.push_back(idx[k + 1]);
          }
        } else if (mode == 5) {
          for (size_t k = 0; k + 2 < idx.size(); ++k) {
            if (k % 2 == 0) {
              m.indices.push_back(idx[k]);
              m.indices.push_back(idx[k + 1]);
            } else {
              m.indices.push_back(idx[k + 1]);
              m.indices.push_back(idx[k]);
            }
            m.indices.push_back(idx[k + 2]);
          }
        } else if (mode == 4) {
          m.indices = std::move(idx);
        } else {
          error = "unsupported primitive mode in " + path;
          return false;
        }
        for (uint32_t i : m.indices)
          if (i >= m.vertex_count) { error = "index out of range in " + path; return false; }
        mesh_ids.back().push_back(uint32_t(out.meshes.size()));
        mesh_materials.back().push_back(int(prim.numberOr("material", -1)));
        out.meshes.push_back(std::move(m));
      }
    }

  // ---- materials
  if (const Json* mats = doc.j.get("materials"))
    for (size_t i = 0; i < mats->size(); ++i) {
      ImportedMaterial m;
      if (const Json* ex = (*mats)[i].get("extensions")) m.flat = ex->get("KHR_materials_unlit") != nullptr;
      const Json* pbr = (*mats)[i].get("pbrMetallicRoughness");
      if (pbr) {
        if (const Json* bc = pbr->get("baseColorFactor"))
          for (int c = 0; c < 4 && size_t(c) < bc->size(); ++c) m.color[c] = float((*bc)[c].num);
        if (const Json* bct = pbr->get("baseColorTexture")) {
          size_t ti = size_t(bct->numberOr("index", 0));
          if (ti >= texture_map.size()) { error = "bad texture index in " + path; return false; }
          m.texture = texture_map[ti].first;
          m.layer = texture_map[ti].second;
          if (const Json* ex = bct->get("extensions"))
            if (const Json* tt = ex->get("KHR_texture_transform")) texture_transform(*tt, m.matrix);
        }
      }
      out.materials.push_back(m);
    }

  // ---- scene
  const Json* nodes = doc.j.get("nodes");
  const Json* scenes = doc.j.get("scenes");
  const size_t scene_count = scenes ? scenes->size() : 0;
  if (scene_count == 0) {
    if (out.meshes.size() != 1 || !out.materials.empty()) {
      error = "expected exactly one mesh and no material for a scene-less file " + path;
      return false;
    }
    if (!whole) {
      error = "scene-less file " + path + " has to be added with RendererFileFlag::Whole";
      return false;
    }
    ImportedView v;
    v.mesh = 0;
    v.index_count = uint32_t(out.meshes[0].indices.size());
    out.views.push_back(v);
    out.templates.push_back({name.empty() ? path : name, 0, 1});
    return true;
  }
  if (scene_count != 1) { error = "expected exactly one scene in " + path; return false; }
  const size_t nn = nodes ? nodes->size() : 0;
  std::vector<long> parent(nn, -1);
  for (size_t i = 0; i < nn; ++i)
    if (const Json* ch = (*nodes)[i].get("children"))
      for (size_t k = 0; k < ch->size(); ++k) {
        size_t c = size_t((*ch)[k].num);
        if (c < nn) parent[c] = long(i);
      }
  bool has_views = false;
  for (size_t i = 0; i < nn; ++i)
    if (const Json* ex = (*nodes)[i].get("extras"))
      if (ex->get("meshViewIndexOffset")) has_views = true;
  std::vector<float> local(nn * 16);
  for (size_t i = 0; i < nn; ++i) node_matrix((*nodes)[i], &local[i * 16]);
  auto absolute = [&](size_t i, float* m) {
    std::vector<size_t> chain;
    for (long k = long(i); k >= 0 && chain.size() <= nn; k = parent[size_t(k)]) chain.push_back(size_t(k));
    float a[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    for (size_t k = chain.size(); k-- > 0;) mat4_mul(a, &local[chain[k] * 16], a);
    std::memcpy(m, a, sizeof(a));
  };
  for (size_t i = 0; i < nn; ++i) {
    const Json& nd = (*nodes)[i];
    const Json* mj = nd.get("mesh");
    if (!mj) continue;
    size_t gm = size_t(mj->num);
    if (gm >= mesh_ids.size()) { error = "bad mesh index in " + path; return false; }
    for (size_t k = 0; k < mesh_ids[gm].size(); ++k) {
      ImportedView v;
      v.mesh = mesh_ids[gm][k];
      if (has_views) {
        const Json* ex = nd.get("extras");
        if (!ex || !ex->get("meshViewIndexCount")) {
          error = "no meshViewIndexCount field in the scene in " + path;
          return false;
        }
        if (!ex->get("meshViewMaterial")) {
          error = "no meshViewMaterial field in the scene in " + path;
          return false;
        }
        v.index_offset_bytes = uint32_t(ex->numberOr("meshViewIndexOffset", 0));
        v.index_count = uint32_t(ex->numberOr("meshViewIndexCount", 0));
        v.material = int32_t(ex->numberOr("meshViewMaterial", -1));
      } else {
        v.index_offset_bytes = 0;
        v.index_count = uint32_t(out.meshes[v.mesh].indices.size());
        v.material = mesh_materials[gm][k];
      }
      if (v.material >= int32_t(out.materials.size())) { error = "bad material index in " + path; return false; }
      if (whole)
        absolute(i, v.transform);
      else
        std::memcpy(v.transform, &local[i * 16], 64);
      out.views.push_back(v);
    }
  }
  if (whole) {
    out.templates.push_back({name.empty() ? path : name, 0, uint32_t(out.views.size())});
  } else {
    uint32_t offset = 0;
    const Json* roots = (*scenes)[0].get("nodes");
    for (size_t r = 0; roots && r < roots->size(); ++r) {
      size_t root = size_t((*roots)[r].num);
      if (root >= nn) { error = "bad root node in " + path; return false; }
      const Json* nmj = (*nodes)[root].get("name");
      if (!nmj || nmj->str.empty()) {
        error = "node " + std::to_string(root) + " in " + path + " has no name";
        return false;
      }
      const Json* ch = (*nodes)[root].get("children");
      uint32_t count = ch ? uint32_t(ch->size()) : 0;
      out.templates.push_back({nmj->str, offset, offset + count});
      offset += count;
    }
    if (offset != out.views.size()) {
      error = "mesh views in " + path + " are not the immediate children of named root nodes";
      return false;
    }
  }
  return true;
}

}  // namespace gbr
