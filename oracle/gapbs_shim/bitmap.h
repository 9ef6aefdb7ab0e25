// Stand-in for the gapbs Bitmap container (interface used by gapbs/bfs.cc: Bitmap(n), reset,
// set_bit, set_bit_atomic, get_bit, swap).  Test infrastructure for oracle/_ref only.
#ifndef ORACLE_SHIM_BITMAP_H_
#define ORACLE_SHIM_BITMAP_H_
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <utility>

class Bitmap {
 public:
  explicit Bitmap(size_t n) : words_((n + 63) / 64), w_(static_cast<uint64_t *>(std::calloc(words_ ? words_ : 1, 8))) {}
  ~Bitmap() { std::free(w_); }
  Bitmap(const Bitmap &) = delete;
  Bitmap &operator=(const Bitmap &) = delete;
  void reset() { std::memset(w_, 0, words_ * 8); }
  void set_bit(size_t i) { w_[i >> 6] |= (1ull << (i & 63)); }
  void set_bit_atomic(size_t i) { __atomic_fetch_or(&w_[i >> 6], 1ull << (i & 63), __ATOMIC_RELAXED); }
  bool get_bit(size_t i) const { return (w_[i >> 6] >> (i & 63)) & 1ull; }
  void swap(Bitmap &o) { std::swap(w_, o.w_); std::swap(words_, o.words_); }

 private:
  size_t words_;
  uint64_t *w_;
};
#endif
