// Host threads that copy one block of host memory in parallel parts: the
// CPU side of moving pageable host buffers through pinned staging pieces.
// Pure C++ (no CUDA), portable to every host the library builds on.
#pragma once

#include <algorithm>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <system_error>
#include <thread>
#include <vector>

namespace pwmgpu {

class CopyPool {
 public:
  // `threads` copiers in all, the calling thread included (fewer when the
  // system cannot start more: the copies then take fewer parts).
  explicit CopyPool(unsigned threads) : requested_(threads) {
    try {
      for (unsigned i = 1; i < std::max(1u, threads); ++i) workers_.emplace_back([this, i]() { run(i); });
    } catch (const std::system_error&) {
    }
  }
  ~CopyPool() {
    {
      std::lock_guard<std::mutex> lk(m_);
      stop_ = true;
    }
    go_.notify_all();
    for (auto& t : workers_) t.join();
  }
  CopyPool(const CopyPool&) = delete;
  CopyPool& operator=(const CopyPool&) = delete;

  unsigned threads() const { return unsigned(workers_.size()) + 1; }
  unsigned requested() const { return requested_; }

  // dst[0, bytes) = src[0, bytes); returns when every part is copied.
  void copy(void* dst, const void* src, uint64_t bytes) {
    if (workers_.empty() || bytes < (uint64_t(1) << 20)) {
      std::memcpy(dst, src, bytes);
      return;
    }
    {
      std::lock_guard<std::mutex> lk(m_);
      dst_ = static_cast<char*>(dst);
      src_ = static_cast<const char*>(src);
      bytes_ = bytes;
      pending_ = unsigned(workers_.size());
      ++job_;
    }
    go_.notify_all();
    part(0);
    std::unique_lock<std::mutex> lk(m_);
    done_.wait(lk, [this]() { return pending_ == 0; });
  }

 private:
  // part i of threads(): 4 KiB-aligned slices, the last one takes the rest
  void part(unsigned i) {
    const uint64_t n = threads();
    const uint64_t slice = ((bytes_ + n - 1) / n + 4095) & ~uint64_t(4095);
    const uint64_t a = std::min<uint64_t>(bytes_, slice * i), b = std::min<uint64_t>(bytes_, a + slice);
    if (b > a) std::memcpy(dst_ + a, src_ + a, b - a);
  }
  void run(unsigned i) {
    uint64_t seen = 0;
    for (;;) {
      std::unique_lock<std::mutex> lk(m_);
      go_.wait(lk, [&]() { return stop_ || job_ != seen; });
      if (stop_) return;
      seen = job_;
      lk.unlock();
      part(i);
      lk.lock();
      if (--pending_ == 0) done_.notify_one();
    }
  }

  unsigned requested_;
  std::vector<std::thread> workers_;
  std::mutex m_;
  std::condition_variable go_, done_;
  bool stop_ = false;
  uint64_t job_ = 0;
  unsigned pending_ = 0;
  char* dst_ = nullptr;
  const char* src_ = nullptr;
  uint64_t bytes_ = 0;
};

}  // namespace pwmgpu
