// Redwood depth-sensor noise on the GPU (declared in include/gbr_noise.h).
//
// Per output pixel (r, c) of an H x W depth image, restating
// src/esp/sensor/RedwoodNoiseModel.cu:20-101 (the model of
// http://redwood-data.org/indoor/data/simdepth.py):
//   1. jitter: y = int(clamp(r + 0.25 m n0, 0, H-1) + 0.5), x likewise with n1
//      (m = noise multiplier, n* standard normal variates);
//   2. 2x downsampling: d = depth[y - y%2][x - x%2]; d >= 10 m -> 0;
//   3. distortion: the pixel remapped to 640 x 480, the 80 x 80 x 5 table
//      interpolated between the depth bins around d, d / f (0 if f < 1e-5);
//   4. disparity quantisation: denom = round((35.130 / d' + 0.027778 m n2) * 8)
//      in double, kept as float; out = 35.130 * 8 / denom (0 if denom <= 1e-5).
// The float operations are written in the reference's order (the build has
// no multiply-add contraction), so the output is a pure function of the
// input, the seed, the call counter and the pixel.
//
// Normal variates: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel
// random numbers: as easy as 1, 2, 3", SC'11) of the counter
// (pixel, image, call lo, call hi) under the key (seed lo, seed hi); the top
// 24 bits of a word pick a segment of the 4096-segment piecewise-linear
// normal quantile function tabulated at (k + 0.5) / 4097.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gbr_noise.h"

namespace gbr {
void set_last_error(const std::string& msg);
}

namespace {

constexpr int kModelCols = 80, kModelDims = 5;
constexpr int kModelFloats = 80 * kModelCols * kModelDims;
constexpr int kKnots = int(GBR_NORMAL_TABLE_SIZE);

__host__ __device__ inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = uint64_t(0xD2511F53u) * c[0];
    const uint64_t p1 = uint64_t(0xCD9E8D57u) * c[2];
    const uint32_t n0 = uint32_t(p1 >> 32) ^ c[1] ^ k0;
    const uint32_t n2 = uint32_t(p0 >> 32) ^ c[3] ^ k1;
    c[1] = uint32_t(p1);
    c[3] = uint32_t(p0);
    c[0] = n0;
    c[2] = n2;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

__device__ __forceinline__ float normal_variate(uint32_t bits, const float* __restrict__ table) {
  const uint32_t u = bits >> 8;
  const uint32_t k = u >> 12;
  const float f = __fmul_rn(float(u & 4095u), 1.0f / 4096.0f);
  const float t0 = __ldg(table + k), t1 = __ldg(table + k + 1);
  return __fadd_rn(t0, __fmul_rn(f, __fsub_rn(t1, t0)));
}

struct TileArgs {
  const float* src;
  float* dst;
  const float* model;
  const float* table;
  long long pitch;
  int tw, th, tiles_x, count;
  float mult;
  uint32_t key0, key1, call0, call1;
};

// One output pixel (row-major index idx) of image img, whose top-left pixel
// is src / dst with `pitch` floats per row and tw x th pixels.
__device__ __forceinline__ void noise_pixel(const TileArgs& a, int img, int idx, const float* src, float* dst,
                                            long long pitch, int tw, int th) {
  const float ymax = float(th - 1), xmax = float(tw - 1);
  uint32_t c[4] = {uint32_t(idx), uint32_t(img), a.call0, a.call1};
  philox4x32_10(c, a.key0, a.key1);
  const float n0 = normal_variate(c[0], a.table), n1 = normal_variate(c[1], a.table),
              n2 = normal_variate(c[2], a.table);
  const int r = idx / tw, col = idx % tw;
  const int y = int(__fadd_rn(fminf(fmaxf(__fadd_rn(float(r), __fmul_rn(__fmul_rn(n0, 0.25f), a.mult)),
                                          0.0f),
                                    ymax),
                              0.5f));
  const int x = int(__fadd_rn(fminf(fmaxf(__fadd_rn(float(col), __fmul_rn(__fmul_rn(n1, 0.25f), a.mult)),
                                          0.0f),
                                    xmax),
                              0.5f));
  const float d = src[(long long)(y - y % 2) * pitch + (x - x % 2)];
  float out = 0.0f;
  if (!(d >= 10.0f)) {
    // Remap to the model's 640 x 480 sensor (a 1-pixel axis maps to 0).
    const int ux = xmax > 0.0f ? int(__fadd_rn(__fmul_rn(__fdiv_rn(float(x), xmax), 639.0f), 0.5f)) : 0;
    const int uy = ymax > 0.0f ? int(__fadd_rn(__fmul_rn(__fdiv_rn(float(y), ymax), 479.0f), 0.5f)) : 0;
    // v / 2 and v * 0.5 are the same correctly rounded value.
    const int i2 = int(__fmul_rn(__fadd_rn(d, 1.0f), 0.5f));
    const int i1 = i2 - 1;
    const float w = __fmul_rn(__fsub_rn(d, __fadd_rn(__fmul_rn(float(i1), 2.0f), 1.0f)), 0.5f);
    const float* cell = a.model + ((uy / 6) * kModelCols + ux / 8) * kModelDims;
    // Bins clamped to 0..4 (the reference clamps the upper bin only from
    // above: equal for every depth >= 0).
    const float f = __fadd_rn(__fmul_rn(__fsub_rn(1.0f, w), __ldg(cell + min(max(i1, 0), 4))),
                              __fmul_rn(w, __ldg(cell + min(max(i2, 0), 4))));
    const float ud = f < 1e-5f ? 0.0f : __fdiv_rn(d, f);
    if (ud != 0.0f) {
      // round((35.130 / d' + noise) * 8) is defined in double.  The float
      // evaluation differs from it by less than `margin` (three roundings
      // of at most 2^-24 relative each), so it rounds to the same integer
      // unless it lies within the margin of a half; only those pixels
      // take the double path (FP64 throughput is low on this part).
      const float nz = __fmul_rn(__fmul_rn(n2, 0.027778f), a.mult);
      const float inv = __fdiv_rn(35.130f, ud);
      const float qf = __fmul_rn(__fadd_rn(inv, nz), 8.0f);
      const float margin = __fmul_rn(1e-6f, __fadd_rn(fabsf(qf), __fmul_rn(8.0f, fabsf(nz))));
      const float frac = fabsf(__fsub_rn(qf, truncf(qf)));
      float denom;
      if (fabsf(__fsub_rn(frac, 0.5f)) > margin && isfinite(qf)) {
        denom = roundf(qf);
      } else {
        const double q = (double(35.130f) / double(ud) + double(nz)) * 8.0;
        denom = float(round(q));
      }
      out = denom > 1e-5f ? __fdiv_rn(35.130f * 8.0f, denom) : 0.0f;
    }
  }
  dst[(long long)r * pitch + col] = out;
}

// Images as the tiles of a grid: blockIdx.y walks images, x their pixels.
__global__ void __launch_bounds__(256) redwood_kernel(TileArgs a) {
  const int pixels = a.tw * a.th;
  for (int img = blockIdx.y; img < a.count; img += gridDim.y) {
    const long long base =
        (long long)(img / a.tiles_x) * a.th * a.pitch + (long long)(img % a.tiles_x) * a.tw;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < pixels; idx += gridDim.x * blockDim.x)
      noise_pixel(a, img, idx, a.src + base, a.dst + base, a.pitch, a.tw, a.th);
  }
}

// Images anywhere in the plane: layout[4i..4i+3] = {offset, pitch, width,
// height} of image i, and blocks[i] .. blocks[i+1]-1 are the 256-pixel
// blocks of image i (a prefix sum), so the grid has one block per 256
// pixels of the batch whatever the mix of sizes.
__global__ void __launch_bounds__(256) redwood_images_kernel(TileArgs a, const long long* layout,
                                                             const long long* blocks) {
  __shared__ int s_img;
  if (threadIdx.x == 0) {
    int lo = 0, hi = a.count;  // blocks[lo] <= blockIdx.x < blocks[hi]
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (blocks[mid] <= (long long)blockIdx.x)
        lo = mid;
      else
        hi = mid;
    }
    s_img = lo;
  }
  __syncthreads();
  const int img = s_img;
  const long long base = layout[4 * img], pitch = layout[4 * img + 1];
  const int tw = int(layout[4 * img + 2]), th = int(layout[4 * img + 3]);
  const int idx = int((long long)blockIdx.x - blocks[img]) * 256 + int(threadIdx.x);
  if (idx < tw * th) noise_pixel(a, img, idx, a.src + base, a.dst + base, pitch, tw, th);
}

// Standard normal quantile in double: Halley steps on erfc from the
// Abramowitz & Stegun 26.2.23 starting point.
double normal_quantile(double p) {
  const double q = p < 0.5 ? p : 1.0 - p;
  const double t = std::sqrt(-2.0 * std::log(q));
  double x = t - (2.515517 + 0.802853 * t + 0.010328 * t * t) /
                     (1.0 + 1.432788 * t + 0.189269 * t * t + 0.001308 * t * t * t);
  x = p < 0.5 ? -x : x;
  const double s2pi = std::sqrt(2.0 * 3.14159265358979323846);
  for (int i = 0; i < 50; ++i) {
    const double e = 0.5 * std::erfc(-x / std::sqrt(2.0)) - p;
    const double u = e * s2pi * std::exp(0.5 * x * x);
    const double step = u / (1.0 + 0.5 * x * u);
    x -= step;
    if (std::fabs(step) <= 1e-17 * (1.0 + std::fabs(x))) break;
  }
  return x;
}

void fill_table(float* out) {
  const int n = kKnots;
  for (int k = 0; k <= n / 2; ++k) {
    const float v = float(normal_quantile((double(k) + 0.5) / double(n)));
    out[k] = v;
    out[n - 1 - k] = -v;
  }
  out[n / 2] = 0.0f;
}

gbr_status fail(gbr_status s, const std::string& m) {
  gbr::set_last_error(m);
  return s;
}

gbr_status cuda_fail(cudaError_t e, const char* what) {
  gbr::set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? GBR_ERROR_OUT_OF_MEMORY : GBR_ERROR_CUDA;
}

}  // namespace

struct gbr_redwood_noise {
  int device = 0;
  float mult = 1.0f;
  uint64_t seed = 0, counter = 0;
  float* model = nullptr;
  float* table = nullptr;
  float* in = nullptr;
  float* out = nullptr;
  size_t cap = 0;  // floats in `in` and `out`
  long long* layout = nullptr;  // device copy of the last per-image layout
  size_t layout_cap = 0;        // int64 values it holds
  cudaEvent_t layout_read = nullptr;  // recorded after the launch that reads it
  int sms = 1;
};

namespace {

struct DeviceScope {
  int prev = -1;
  explicit DeviceScope(int d) {
    cudaGetDevice(&prev);
    if (prev != d) cudaSetDevice(d);
  }
  ~DeviceScope() {
    int cur;
    if (cudaGetDevice(&cur) == cudaSuccess && cur != prev && prev >= 0) cudaSetDevice(prev);
  }
};

TileArgs make_args(gbr_redwood_noise* m, const float* src, float* dst, long long pitch, int tw, int th,
                   int tiles_x, int count) {
  TileArgs a;
  a.src = src;
  a.dst = dst;
  a.model = m->model;
  a.table = m->table;
  a.pitch = pitch;
  a.tw = tw;
  a.th = th;
  a.tiles_x = tiles_x;
  a.count = count;
  a.mult = m->mult;
  a.key0 = uint32_t(m->seed);
  a.key1 = uint32_t(m->seed >> 32);
  a.call0 = uint32_t(m->counter);
  a.call1 = uint32_t(m->counter >> 32);
  ++m->counter;
  return a;
}

gbr_status launch(gbr_redwood_noise* m, const float* src, float* dst, long long pitch, int tw, int th,
                  int tiles_x, int count, cudaStream_t stream) {
  const TileArgs a = make_args(m, src, dst, pitch, tw, th, tiles_x, count);
  const int pixels = tw * th;
  const int per_image = std::max(1, std::min((pixels + 255) / 256, 8 * m->sms));
  const int images = std::max(1, std::min(count, 65535));
  redwood_kernel<<<dim3(per_image, images), 256, 0, stream>>>(a);
  if (cudaError_t e = cudaGetLastError()) return cuda_fail(e, "redwood noise launch");
  return GBR_OK;
}

}  // namespace

extern "C" {

gbr_status gbr_normal_quantile_table(float* out, uint32_t n) {
  if (!out) return fail(GBR_ERROR_INVALID_ARGUMENT, "null argument: out");
  if (n != GBR_NORMAL_TABLE_SIZE)
    return fail(GBR_ERROR_INVALID_ARGUMENT, "normal quantile table: n must be GBR_NORMAL_TABLE_SIZE");
  fill_table(out);
  return GBR_OK;
}

gbr_status gbr_redwood_noise_create(const float* model, int32_t rows, int32_t cols, int32_t device,
                                    float mult, uint64_t seed, gbr_redwood_noise** out) {
  if (!model || !out) return fail(GBR_ERROR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  if (rows <= 0 || cols <= 0 || int64_t(rows) * cols != kModelFloats)
    return fail(GBR_ERROR_INVALID_ARGUMENT, "RedwoodNoiseModel: the model must hold 80 x 80 x 5 floats");
  if (!(mult >= 0.0f) || !std::isfinite(mult))
    return fail(GBR_ERROR_INVALID_ARGUMENT, "RedwoodNoiseModel: bad noise multiplier");
  int n = 0;
  if (cudaError_t e = cudaGetDeviceCount(&n)) return cuda_fail(e, "RedwoodNoiseModel: no CUDA device");
  if (device < 0 || device >= n) return fail(GBR_ERROR_INVALID_ARGUMENT, "RedwoodNoiseModel: bad device id");
  DeviceScope scope(device);
  auto* m = new gbr_redwood_noise();
  m->device = device;
  m->mult = mult;
  m->seed = seed;
  cudaDeviceGetAttribute(&m->sms, cudaDevAttrMultiProcessorCount, device);
  std::vector<float> table(kKnots);
  fill_table(table.data());
  cudaError_t e = cudaMalloc(&m->model, kModelFloats * sizeof(float));
  if (!e) e = cudaMalloc(&m->table, kKnots * sizeof(float));
  if (!e) e = cudaMemcpy(m->model, model, kModelFloats * sizeof(float), cudaMemcpyHostToDevice);
  if (!e) e = cudaMemcpy(m->table, table.data(), kKnots * sizeof(float), cudaMemcpyHostToDevice);
  if (e) {
    gbr_redwood_noise_destroy(m);
    return cuda_fail(e, "RedwoodNoiseModel: upload");
  }
  *out = m;
  return GBR_OK;
}

void gbr_redwood_noise_destroy(gbr_redwood_noise* m) {
  if (!m) return;
  DeviceScope scope(m->device);
  cudaFree(m->model);
  cudaFree(m->table);
  cudaFree(m->in);
  cudaFree(m->out);
  cudaFree(m->layout);
  if (m->layout_read) cudaEventDestroy(m->layout_read);
  delete m;
}

gbr_status gbr_redwood_noise_simulate_tiles(gbr_redwood_noise* m, const float* src, float* dst, int64_t pitch,
                                            int32_t tw, int32_t th, int32_t tiles_x, int32_t count,
                                            void* stream) {
  if (!m || !src || !dst) return fail(GBR_ERROR_INVALID_ARGUMENT, "null argument");
  if (tw <= 0 || th <= 0 || tiles_x <= 0 || count < 0 || pitch < int64_t(tw) * tiles_x ||
      int64_t(tw) * th > (int64_t(1) << 31) - 1)
    return fail(GBR_ERROR_INVALID_ARGUMENT, "RedwoodNoiseModel: bad image layout");
  if (src == dst) return fail(GBR_ERROR_INVALID_ARGUMENT, "RedwoodNoiseModel: input and output must differ");
  if (count == 0) return GBR_OK;
  DeviceScope scope(m->device);
  return launch(m, src, dst, pitch, tw, th, tiles_x, count, static_cast<cudaStream_t>(stream));
}

gbr_status gbr_redwood_noise_simulate_images(gbr_redwood_noise* m, const float* src, float* dst,
                                             const int64_t* layout, int32_t count, void* stream) {
  if (!m || !src || !dst || (count > 0 && !layout)) return fail(GBR_ERROR_INVALID_ARGUMENT, "null argument");
  if (count < 0) return fail(GBR_ERROR_INVALID_ARGUMENT, "RedwoodNoiseModel: negative image count");
  if (src == dst) return fail(GBR_ERROR_INVALID_ARGUMENT, "RedwoodNoiseModel: input and output must differ");
  // Host copy: the layout, then the prefix sum of 256-pixel blocks per image.
  std::vector<long long> host(size_t(count) * 5 + 1);
  long long blocks = 0;
  for (int32_t i = 0; i < count; ++i) {
    const int64_t off = layout[4 * i], pitch = layout[4 * i + 1], w = layout[4 * i + 2], h = layout[4 * i + 3];
    if (off < 0 || w <= 0 || h <= 0 || pitch < w || w * h > (int64_t(1) << 31) - 1)
      return fail(GBR_ERROR_INVALID_ARGUMENT,
                  "RedwoodNoiseModel: bad layout of image " + std::to_string(i));
    for (int k = 0; k < 4; ++k) host[4 * size_t(i) + k] = layout[4 * i + k];
    host[4 * size_t(count) + i] = blocks;
    blocks += (w * h + 255) / 256;
  }
  host[5 * size_t(count)] = blocks;
  if (blocks > (1LL << 31) - 1)
    return fail(GBR_ERROR_INVALID_ARGUMENT, "RedwoodNoiseModel: too many pixels in one batch");
  if (count == 0) return GBR_OK;
  DeviceScope scope(m->device);
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!m->layout_read)
    if (cudaError_t e = cudaEventCreateWithFlags(&m->layout_read, cudaEventDisableTiming))
      return cuda_fail(e, "RedwoodNoiseModel: event");
  if (host.size() > m->layout_cap) {
    // The previous layout may still be read by a launch on another stream.
    if (cudaError_t e = cudaEventSynchronize(m->layout_read)) return cuda_fail(e, "RedwoodNoiseModel: wait");
    cudaFree(m->layout);
    m->layout = nullptr;
    m->layout_cap = 0;
    if (cudaError_t e = cudaMalloc(&m->layout, host.size() * sizeof(long long)))
      return cuda_fail(e, "RedwoodNoiseModel: layout allocation");
    m->layout_cap = host.size();
  }
  // Overwrite the device layout only after the last launch that read it.
  if (cudaError_t e = cudaStreamWaitEvent(s, m->layout_read, 0)) return cuda_fail(e, "RedwoodNoiseModel: wait");
  if (cudaError_t e = cudaMemcpyAsync(m->layout, host.data(), host.size() * sizeof(long long),
                                      cudaMemcpyHostToDevice, s))
    return cuda_fail(e, "RedwoodNoiseModel: layout upload");
  const TileArgs a = make_args(m, src, dst, 0, 1, 1, 1, count);
  redwood_images_kernel<<<unsigned(blocks), 256, 0, s>>>(a, m->layout, m->layout + 4 * size_t(count));
  if (cudaError_t e = cudaGetLastError()) return cuda_fail(e, "redwood noise launch");
  if (cudaError_t e = cudaEventRecord(m->layout_read, s)) return cuda_fail(e, "RedwoodNoiseModel: event");
  return GBR_OK;
}

gbr_status gbr_redwood_noise_simulate_device(gbr_redwood_noise* m, const float* depth, int32_t rows,
                                             int32_t cols, float* noisy, void* stream) {
  return gbr_redwood_noise_simulate_tiles(m, depth, noisy, cols, cols, rows, 1, 1, stream);
}

gbr_status gbr_redwood_noise_simulate_host(gbr_redwood_noise* m, const float* depth, int32_t rows,
                                           int32_t cols, float* noisy) {
  if (!m || !depth || !noisy) return fail(GBR_ERROR_INVALID_ARGUMENT, "null argument");
  if (rows <= 0 || cols <= 0) return fail(GBR_ERROR_INVALID_ARGUMENT, "RedwoodNoiseModel: bad image size");
  DeviceScope scope(m->device);
  const size_t n = size_t(rows) * size_t(cols);
  if (n > m->cap) {
    cudaFree(m->in);
    cudaFree(m->out);
    m->in = m->out = nullptr;
    m->cap = 0;
    cudaError_t e = cudaMalloc(&m->in, n * sizeof(float));
    if (!e) e = cudaMalloc(&m->out, n * sizeof(float));
    if (e) return cuda_fail(e, "RedwoodNoiseModel: scratch");
    m->cap = n;
  }
  if (cudaError_t e = cudaMemcpy(m->in, depth, n * sizeof(float), cudaMemcpyHostToDevice))
    return cuda_fail(e, "RedwoodNoiseModel: upload");
  if (gbr_status s = launch(m, m->in, m->out, cols, cols, rows, 1, 1, nullptr)) return s;
  if (cudaError_t e = cudaMemcpy(noisy, m->out, n * sizeof(float), cudaMemcpyDeviceToHost))
    return cuda_fail(e, "RedwoodNoiseModel: readback");
  return GBR_OK;
}

gbr_status gbr_redwood_noise_set_state(gbr_redwood_noise* m, uint64_t seed, uint64_t counter) {
  if (!m) return fail(GBR_ERROR_INVALID_ARGUMENT, "null argument");
  m->seed = seed;
  m->counter = counter;
  return GBR_OK;
}

gbr_status gbr_redwood_noise_get_state(gbr_redwood_noise* m, uint64_t* seed, uint64_t* counter) {
  if (!m || !seed || !counter) return fail(GBR_ERROR_INVALID_ARGUMENT, "null argument");
  *seed = m->seed;
  *counter = m->counter;
  return GBR_OK;
}

}  // extern "C"
