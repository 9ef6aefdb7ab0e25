// Stand-in for the gapbs SlidingQueue/QueueBuffer containers (interface used by gapbs/bfs.cc):
// a shared append-only array whose readable window [out_start, out_end) advances on slide_window(),
// and a per-thread buffer that appends its contents with one atomic fetch-add on flush().
// Test infrastructure for oracle/_ref only.
#ifndef ORACLE_SHIM_SLIDING_QUEUE_H_
#define ORACLE_SHIM_SLIDING_QUEUE_H_
#include <cstddef>
#include <cstdlib>
#include <cstring>

template <typename T>
class QueueBuffer;

template <typename T>
class SlidingQueue {
 public:
  explicit SlidingQueue(size_t cap) : buf_(static_cast<T *>(std::malloc(sizeof(T) * (cap ? cap : 1)))) {}
  ~SlidingQueue() { std::free(buf_); }
  SlidingQueue(const SlidingQueue &) = delete;
  SlidingQueue &operator=(const SlidingQueue &) = delete;
  void push_back(T v) { buf_[in_++] = v; }
  bool empty() const { return out_start_ == out_end_; }
  void reset() { in_ = out_start_ = out_end_ = 0; }
  void slide_window() { out_start_ = out_end_; out_end_ = in_; }
  T *begin() const { return buf_ + out_start_; }
  T *end() const { return buf_ + out_end_; }
  size_t size() const { return out_end_ - out_start_; }

 private:
  friend class QueueBuffer<T>;
  T *buf_;
  size_t in_ = 0, out_start_ = 0, out_end_ = 0;
};

template <typename T>
class QueueBuffer {
 public:
  explicit QueueBuffer(SlidingQueue<T> &q, size_t cap = 16384)
      : q_(q), cap_(cap), len_(0), local_(static_cast<T *>(std::malloc(sizeof(T) * cap))) {}
  ~QueueBuffer() { std::free(local_); }
  void push_back(T v) {
    if (len_ == cap_) flush();
    local_[len_++] = v;
  }
  void flush() {
    size_t at = __atomic_fetch_add(&q_.in_, len_, __ATOMIC_RELAXED);
    std::memcpy(q_.buf_ + at, local_, sizeof(T) * len_);
    len_ = 0;
  }

 private:
  SlidingQueue<T> &q_;
  size_t cap_, len_;
  T *local_;
};
#endif
