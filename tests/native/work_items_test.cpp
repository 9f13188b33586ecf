// The batched form's work items (work_items.h) on random scene sets: every
// enabled viewport covered exactly once, nothing for disabled scenes, regions
// within the batched form's region, longest first, the list within its
// capacity, and a small viewport bound to a large scene split.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "work_items.h"

using namespace gbr;

static int failures = 0;
#define CHECK(c)                                                   \
  do {                                                             \
    if (!(c)) {                                                    \
      std::fprintf(stderr, "%s:%d: %s\n", __FILE__, __LINE__, #c); \
      ++failures;                                                  \
    }                                                              \
  } while (0)

static void check_set(const std::vector<ItemScene>& scenes, int rw, int rh, uint64_t grid) {
  const std::vector<WorkItem> items = build_work_items(scenes, rw, rh, grid);
  CHECK(items.size() <= work_item_capacity(scenes, rw, rh, grid));
  std::vector<std::vector<uint8_t>> hits(scenes.size());
  for (size_t s = 0; s < scenes.size(); ++s) hits[s].assign(size_t(scenes[s].width) * scenes[s].height, 0);
  uint64_t prev = UINT64_MAX;
  for (const WorkItem& it : items) {
    CHECK(it.scene < scenes.size());
    const ItemScene& sc = scenes[it.scene];
    CHECK(sc.enabled);
    CHECK(it.w >= 1 && it.h >= 1 && it.w <= rw && it.h <= rh);
    CHECK(it.x0 + it.w <= sc.width && it.y0 + it.h <= sc.height);
    const uint64_t cost = item_cost(sc.tris, it.w, it.h, sc.width, sc.height);
    CHECK(cost <= prev);  // longest first
    prev = cost;
    for (int y = it.y0; y < it.y0 + it.h; ++y)
      for (int x = it.x0; x < it.x0 + it.w; ++x) ++hits[it.scene][size_t(y) * sc.width + x];
  }
  for (size_t s = 0; s < scenes.size(); ++s)
    for (uint8_t h : hits[s]) CHECK(h == (scenes[s].enabled ? 1 : 0));
}

int main() {
  std::mt19937_64 rng(42);
  const int shapes[][2] = {{128, 128}, {128, 64}, {64, 64}, {32, 32}};
  for (int trial = 0; trial < 300; ++trial) {
    const int n = 1 + int(rng() % 200);
    std::vector<ItemScene> scenes(n);
    for (ItemScene& sc : scenes) {
      sc.width = 1 + int(rng() % 300);
      sc.height = 1 + int(rng() % 300);
      sc.tris = uint64_t(std::exp(std::uniform_real_distribution<double>(0.0, 15.0)(rng)));
      sc.geometry = uint32_t(rng() % 7);
      sc.enabled = rng() % 5 != 0;
    }
    const int* shape = shapes[trial % 4];
    const uint64_t grids[] = {1, 152, 304, 608};
    check_set(scenes, shape[0], shape[1], grids[trial % 4]);
  }
  // A 64 x 64 viewport bound to a 1M-triangle scene beside 300 light scenes:
  // its region is split (two halvings: 32 x 32), the light scenes' are not,
  // and the last wave (the `grid` cheapest items) is halved where it can be.
  std::vector<ItemScene> scenes(301);
  scenes[0] = ItemScene{64, 64, 1000000, 0, true};
  for (int s = 1; s <= 300; ++s) scenes[s] = ItemScene{128, 128, 20000, 1, true};
  const std::vector<WorkItem> items = build_work_items(scenes, 128, 64, 152);
  int heavy = 0;
  for (const WorkItem& it : items)
    if (it.scene == 0) {
      ++heavy;
      CHECK(it.w == 32 && it.h == 32);
    }
  CHECK(heavy == 4);
  CHECK(items.size() == 4 + 300 * 2 + 152);  // 152 of the light items halved
  check_set(scenes, 128, 64, 152);
  if (failures) return 1;
  std::printf("ok\n");
  return 0;
}
