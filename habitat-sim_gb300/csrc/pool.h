// A small persistent pool of host worker threads, used for the host-side
// preparation that scales with content size (keyframe parsing of large
// batches, chunk bounding boxes of large meshes).
#pragma once

#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace gbr {

// Host worker threads that split an index range [0, count) into chunks
// taken from a shared counter; the calling thread works too.  Calls to run()
// from several host threads are served one after another.
class WorkerPool {
 public:
  explicit WorkerPool(unsigned threads);
  ~WorkerPool();
  WorkerPool(const WorkerPool&) = delete;
  WorkerPool& operator=(const WorkerPool&) = delete;
  unsigned size() const { return unsigned(threads_.size()) + 1; }
  // fn(begin, end) over chunks of `chunk` indices; returns when all are done.
  // fn must not throw and must not call run() itself.
  void run(uint32_t count, uint32_t chunk, const std::function<void(uint32_t, uint32_t)>& fn);

 private:
  void work();
  void drain();
  std::mutex run_m_;  // one run() at a time
  std::mutex m_;
  std::condition_variable start_, done_;
  std::vector<std::thread> threads_;
  const std::function<void(uint32_t, uint32_t)>* fn_ = nullptr;
  uint32_t count_ = 0, chunk_ = 1;
  std::atomic<uint64_t> next_{0};
  unsigned pending_ = 0;  // workers yet to finish the current generation
  uint64_t generation_ = 0;
  bool stop_ = false;
  int owner_pid_;  // the process whose threads these are
};

// The process-wide pool (hardware threads - 1 workers, at most 15), started
// on first use and kept for the life of the process.
WorkerPool& shared_pool();

}  // namespace gbr
