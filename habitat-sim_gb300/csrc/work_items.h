// Work items of the batched form: the regions of every enabled scene, in
// longest-processing-time order for the persistent raster grid.  Host code,
// shared by the renderer and its native tests.
#pragma once

#include <algorithm>
#include <cstdint>
#include <numeric>
#include <vector>

#include "records.h"

namespace gbr {

// What the ordering needs to know of a scene.
struct ItemScene {
  int width = 0, height = 0;  // viewport
  uint64_t tris = 0;          // triangles of the scene it renders (its source)
  uint32_t geometry = 0;      // groups items of equal cost (the mesh of the source's largest draw)
  bool enabled = true;
};

// Region halvings a costly scene's items may get.
constexpr int kMaxSplits = 2;

// Region of a scene's items after `level` splits of the batched form's
// region (clamped to the viewport): each split halves the longer side, down
// to 32 pixels.
inline void split_region(int width, int height, int region_w, int region_h, int level, int& rw, int& rh) {
  rw = std::max(1, std::min(region_w, width));
  rh = std::max(1, std::min(region_h, height));
  for (int l = 0; l < level; ++l) {
    if (rw >= rh && rw > 32)
      rw = (rw + 1) / 2;
    else if (rh > 32)
      rh = (rh + 1) / 2;
    else if (rw > 32)
      rw = (rw + 1) / 2;
  }
}

// Estimated cost of a w x h region of a W x H viewport: its share of the
// scene's triangles plus a quarter of them for the region's culling and setup.
inline uint64_t item_cost(uint64_t tris, int w, int h, int W, int H) {
  return (tris + 1) * uint64_t(w) * uint64_t(h) / (uint64_t(W) * uint64_t(H)) + tris / 4;
}

// Items the list can ever hold: every scene at its finest split, plus the
// halves of the last wave (one per resident CTA, at most `max_grid`).
inline uint64_t work_item_capacity(const std::vector<ItemScene>& scenes, int region_w, int region_h,
                                   uint64_t max_grid) {
  uint64_t capacity = max_grid;
  for (const ItemScene& sc : scenes) {
    if (sc.width <= 0 || sc.height <= 0) continue;
    int rw, rh;
    split_region(sc.width, sc.height, region_w, region_h, kMaxSplits, rw, rh);
    capacity += uint64_t((sc.width + rw - 1) / rw) * uint64_t((sc.height + rh - 1) / rh);
  }
  return capacity;
}

// The items of the enabled scenes for a persistent grid of `grid` CTAs,
// longest first.  A scene whose regions would each cost more than half a
// CTA's share of the whole step (a small viewport bound to a large scene)
// gets smaller regions (at most kMaxSplits halvings), so that no single item
// outlasts the others; then the cheapest `grid` items -- the last wave -- are
// halved (longer side, not below 32 px), so that the CTAs finishing the step
// wait for half an item at most.  Items of equal cost are grouped by
// geometry, so that the CTAs in flight read the same vertices from L2.
// Measured on the serving workload: splitting at half the share beat the
// whole share by 9 % and a quarter of it by 16 %; halving two waves or
// quartering the last one was slower than halving one.
inline std::vector<WorkItem> build_work_items(const std::vector<ItemScene>& scenes, int region_w, int region_h,
                                              uint64_t grid) {
  grid = std::max<uint64_t>(grid, 1);
  const uint32_t S = uint32_t(scenes.size());
  uint64_t total = 0;
  for (uint32_t s = 0; s < S; ++s) {
    const ItemScene& sc = scenes[s];
    if (!sc.enabled || sc.width <= 0 || sc.height <= 0) continue;
    int rw, rh;
    split_region(sc.width, sc.height, region_w, region_h, 0, rw, rh);
    const uint64_t n = uint64_t((sc.width + rw - 1) / rw) * uint64_t((sc.height + rh - 1) / rh);
    total += n * item_cost(sc.tris, rw, rh, sc.width, sc.height);
  }
  const uint64_t share = total / grid / 2;  // half a CTA's share of the step
  std::vector<WorkItem> items;
  std::vector<uint64_t> cost;
  std::vector<uint32_t> key;
  for (uint32_t s = 0; s < S; ++s) {
    const ItemScene& sc = scenes[s];
    if (!sc.enabled || sc.width <= 0 || sc.height <= 0) continue;
    int rw, rh, level = 0;
    split_region(sc.width, sc.height, region_w, region_h, 0, rw, rh);
    while (level < kMaxSplits && item_cost(sc.tris, rw, rh, sc.width, sc.height) > share) {
      int nw, nh;
      split_region(sc.width, sc.height, region_w, region_h, level + 1, nw, nh);
      if (nw == rw && nh == rh) break;
      rw = nw;
      rh = nh;
      ++level;
    }
    for (int y = 0; y < sc.height; y += rh)
      for (int x = 0; x < sc.width; x += rw) {
        WorkItem it{};
        it.scene = s;
        it.x0 = uint16_t(x);
        it.y0 = uint16_t(y);
        it.w = uint16_t(std::min(rw, sc.width - x));
        it.h = uint16_t(std::min(rh, sc.height - y));
        items.push_back(it);
        cost.push_back(item_cost(sc.tris, it.w, it.h, sc.width, sc.height));
        key.push_back(sc.geometry);
      }
  }
  std::vector<uint32_t> perm(items.size());
  std::iota(perm.begin(), perm.end(), 0u);
  auto by_cost = [&](uint32_t a, uint32_t b) {
    if (cost[a] != cost[b]) return cost[a] > cost[b];
    return key[a] < key[b];
  };
  std::stable_sort(perm.begin(), perm.end(), by_cost);
  if (items.size() > grid) {
    const size_t n0 = items.size();
    for (size_t i = n0 - grid; i < n0; ++i) {
      WorkItem& it = items[perm[i]];
      WorkItem b = it;
      if (it.w >= it.h && it.w > 32) {
        b.w = uint16_t(it.w / 2);
        b.x0 = uint16_t(it.x0 + (it.w - b.w));
        it.w = uint16_t(it.w - b.w);
      } else if (it.h > 32) {
        b.h = uint16_t(it.h / 2);
        b.y0 = uint16_t(it.y0 + (it.h - b.h));
        it.h = uint16_t(it.h - b.h);
      } else {
        continue;
      }
      const ItemScene& sc = scenes[it.scene];
      const uint32_t geometry = key[perm[i]];
      cost[perm[i]] = item_cost(sc.tris, it.w, it.h, sc.width, sc.height);
      const uint64_t bcost = item_cost(sc.tris, b.w, b.h, sc.width, sc.height);
      items.push_back(b);  // `it` is not used past this point
      cost.push_back(bcost);
      key.push_back(geometry);
    }
    perm.resize(items.size());
    std::iota(perm.begin(), perm.end(), 0u);
    std::stable_sort(perm.begin(), perm.end(), by_cost);
  }
  std::vector<WorkItem> out(items.size());
  for (size_t i = 0; i < items.size(); ++i) out[i] = items[perm[i]];
  return out;
}

}  // namespace gbr
