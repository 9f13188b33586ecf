// Native unit test of the replay renderer's host worker pool and of keyframe
// parsing (no GPU): every index of a range is visited exactly once per run,
// runs back to back reuse the same threads, and keyframes parsed on the pool
// equal keyframes parsed serially.
#include <sys/wait.h>
#include <unistd.h>

#include <atomic>
#include <cstdio>
#include <string>
#include <vector>

#include "json.h"
#include "pool.h"
#include "replay.h"

using gbr::Json;
using gbr::JsonParser;
using gbr::replay::Keyframe;
using gbr::WorkerPool;

static int failures = 0;
#define CHECK(c)                                                     \
  do {                                                               \
    if (!(c)) {                                                      \
      std::fprintf(stderr, "%s:%d: check failed: %s\n", __FILE__, __LINE__, #c); \
      ++failures;                                                    \
    }                                                                \
  } while (0)

static bool parse(const std::string& s, Keyframe& k) {
  Json doc;
  JsonParser jp{s.data(), s.data() + s.size(), {}};
  if (!jp.parse(doc)) return false;
  const Json* obj = doc.get("keyframe");
  std::string err;
  return obj && gbr::replay::parse_keyframe(*obj, k, err);
}

int main() {
  for (unsigned threads : {0u, 1u, 3u, 7u}) {
    WorkerPool pool(threads);
    CHECK(pool.size() == threads + 1);
    for (uint32_t count : {0u, 1u, 31u, 32u, 33u, 1000u, 4096u}) {
      for (uint32_t chunk : {1u, 7u, 32u, 5000u}) {
        std::vector<std::atomic<int>> hits(count);
        for (auto& h : hits) h.store(0);
        const std::function<void(uint32_t, uint32_t)> fn = [&](uint32_t b, uint32_t e) {
          CHECK(b < e && e <= count && e - b <= chunk);
          for (uint32_t i = b; i < e; ++i) hits[i].fetch_add(1);
        };
        pool.run(count, chunk, fn);
        for (uint32_t i = 0; i < count; ++i) CHECK(hits[i].load() == 1);
      }
    }
  }
  // Keyframes parsed on the pool equal the serial parse.
  std::vector<std::string> docs;
  for (int i = 0; i < 700; ++i) {
    docs.push_back("{\"keyframe\": {\"loads\": [], \"deletions\": [" + std::to_string(i) +
                   "], \"stateUpdates\": [{\"instanceKey\": " + std::to_string(i % 13) +
                   ", \"state\": {\"absTransform\": {\"translation\": [" + std::to_string(0.25 * i) +
                   ", -1.5e-3, 2], \"rotation\": [1, 0, 0, 0]}}}], \"userTransforms\": [{\"name\": "
                   "\"sensor_\\u0041\", \"transform\": {\"translation\": [1, 2, " +
                   std::to_string(i) + "], \"rotation\": [0.5, 0.5, 0.5, 0.5]}}]}}");
  }
  std::vector<Keyframe> serial(docs.size()), pooled(docs.size());
  for (size_t i = 0; i < docs.size(); ++i) CHECK(parse(docs[i], serial[i]));
  WorkerPool pool(5);
  const std::function<void(uint32_t, uint32_t)> fn = [&](uint32_t b, uint32_t e) {
    for (uint32_t i = b; i < e; ++i) CHECK(parse(docs[i], pooled[i]));
  };
  pool.run(uint32_t(docs.size()), 32, fn);
  for (size_t i = 0; i < docs.size(); ++i) {
    CHECK(pooled[i].deletions == serial[i].deletions);
    CHECK(pooled[i].state_updates.size() == 1 && serial[i].state_updates.size() == 1);
    CHECK(pooled[i].user_transforms.size() == 1);
    const auto it = pooled[i].user_transforms.find("sensor_A");
    CHECK(it != pooled[i].user_transforms.end());
    if (it != pooled[i].user_transforms.end()) CHECK(it->second.translation[2] == float(i));
  }
  // A forked child has the pool object but not its threads: run() must
  // still finish, on the calling thread alone.
  {
    std::vector<int> seen(5000, 0);
    const std::function<void(uint32_t, uint32_t)> mark = [&](uint32_t b, uint32_t e) {
      for (uint32_t i = b; i < e; ++i) ++seen[i];
    };
    pool.run(5000, 64, mark);  // the threads exist and have run
    const pid_t child = fork();
    if (child == 0) {
      std::vector<int> again(5000, 0);
      const std::function<void(uint32_t, uint32_t)> mark2 = [&](uint32_t b, uint32_t e) {
        for (uint32_t i = b; i < e; ++i) ++again[i];
      };
      pool.run(5000, 64, mark2);
      for (int v : again)
        if (v != 1) _exit(3);
      _exit(0);
    }
    int status = 0;
    CHECK(child > 0 && waitpid(child, &status, 0) == child);
    CHECK(WIFEXITED(status) && WEXITSTATUS(status) == 0);
    for (int v : seen) CHECK(v == 1);
  }
  if (failures) {
    std::fprintf(stderr, "%d failures\n", failures);
    return 1;
  }
  std::puts("worker pool ok");
  return 0;
}
