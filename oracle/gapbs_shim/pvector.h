// Stand-in for the gapbs container header that the ParHDE sources include but do not vendor.
// Written from the interface gapbs/bfs.cc and gapbs/sssp.cc use: pvector(n), pvector(n, init),
// operator[], data(), size(), move construction.  Test infrastructure for oracle/_ref only.
#ifndef ORACLE_SHIM_PVECTOR_H_
#define ORACLE_SHIM_PVECTOR_H_
#include <cstddef>
#include <cstdlib>

template <typename T>
class pvector {
 public:
  explicit pvector(size_t n) : n_(n), p_(static_cast<T *>(std::malloc(sizeof(T) * (n ? n : 1)))) {}
  pvector(size_t n, T init) : pvector(n) {
#pragma omp parallel for
    for (long i = 0; i < static_cast<long>(n); i++) p_[i] = init;
  }
  pvector(pvector &&o) noexcept : n_(o.n_), p_(o.p_) { o.p_ = nullptr; o.n_ = 0; }
  pvector(const pvector &) = delete;
  pvector &operator=(const pvector &) = delete;
  ~pvector() { std::free(p_); }
  T &operator[](size_t i) { return p_[i]; }
  const T &operator[](size_t i) const { return p_[i]; }
  T *data() { return p_; }
  const T *data() const { return p_; }
  size_t size() const { return n_; }
  T *begin() { return p_; }
  T *end() { return p_ + n_; }

 private:
  size_t n_;
  T *p_;
};
#endif
