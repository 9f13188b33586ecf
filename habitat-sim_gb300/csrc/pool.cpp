// Host worker pool (declared in pool.h).
#include "pool.h"

#include <unistd.h>

#include <algorithm>

namespace gbr {

WorkerPool::WorkerPool(unsigned threads) : owner_pid_(getpid()) {
  for (unsigned t = 0; t < threads; ++t) threads_.emplace_back([this] { work(); });
}

WorkerPool::~WorkerPool() {
  {
    std::lock_guard<std::mutex> lk(m_);
    stop_ = true;
  }
  start_.notify_all();
  for (auto& t : threads_) t.join();
}

void WorkerPool::drain() {
  // A 64-bit counter: it cannot wrap below count_ however many threads
  // overshoot the end, so no chunk runs twice.
  for (;;) {
    const uint64_t b = next_.fetch_add(chunk_);
    if (b >= count_) return;
    (*fn_)(uint32_t(b), uint32_t(std::min<uint64_t>(count_, b + chunk_)));
  }
}

void WorkerPool::work() {
  uint64_t seen = 0;
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(m_);
      start_.wait(lk, [&] { return stop_ || generation_ != seen; });
      if (stop_) return;
      seen = generation_;
    }
    drain();
    {
      std::lock_guard<std::mutex> lk(m_);
      --pending_;
    }
    done_.notify_all();
  }
}

void WorkerPool::run(uint32_t count, uint32_t chunk, const std::function<void(uint32_t, uint32_t)>& fn) {
  if (getpid() != owner_pid_) {
    // A forked child inherits the pool but not its threads: work alone.
    const uint64_t step = std::max(1u, chunk);
    for (uint64_t b = 0; b < count; b += step) fn(uint32_t(b), uint32_t(std::min<uint64_t>(count, b + step)));
    return;
  }
  std::lock_guard<std::mutex> serial(run_m_);
  {
    std::lock_guard<std::mutex> lk(m_);
    fn_ = &fn;
    count_ = count;
    chunk_ = std::max(1u, chunk);
    next_.store(0);
    pending_ = unsigned(threads_.size());
    ++generation_;
  }
  start_.notify_all();
  drain();
  // Every worker takes part in every generation, so none can still be
  // reading fn_ once they have all reported back.
  std::unique_lock<std::mutex> lk(m_);
  done_.wait(lk, [&] { return pending_ == 0; });
  fn_ = nullptr;
}

WorkerPool& shared_pool() {
  // Never destroyed: its threads end with the process, and a forked child
  // (which has the object but not the threads) never joins them.
  static WorkerPool* pool = new WorkerPool(std::min(std::max(1u, std::thread::hardware_concurrency()), 16u) - 1);
  return *pool;
}

}  // namespace gbr
