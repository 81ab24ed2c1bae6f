// dbuf.cuh -- owning device buffer.
#ifndef NNPP_DBUF_CUH
#define NNPP_DBUF_CUH

#include <cuda_runtime.h>
#include <cstddef>
#include <utility>

namespace nnpp {

template <typename T>
class DBuf {
 public:
  DBuf() = default;
  ~DBuf() { reset(); }
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : p_(o.p_), n_(o.n_) {
    o.p_ = nullptr;
    o.n_ = 0;
  }
  DBuf& operator=(DBuf&& o) noexcept {
    if (this != &o) {
      reset();
      p_ = o.p_;
      n_ = o.n_;
      o.p_ = nullptr;
      o.n_ = 0;
    }
    return *this;
  }
  // (Re)allocate n elements; returns false on failure.  Contents are undefined.
  bool alloc(size_t n) {
    if (n == n_ && p_) return true;
    reset();
    if (n == 0) return true;
    void* q = nullptr;
    if (cudaMalloc(&q, n * sizeof(T)) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    p_ = static_cast<T*>(q);
    n_ = n;
    return true;
  }
  void reset() {
    if (p_) cudaFree(p_);
    p_ = nullptr;
    n_ = 0;
  }
  T* get() const { return p_; }
  size_t size() const { return n_; }
  size_t bytes() const { return n_ * sizeof(T); }
  void swap(DBuf& o) {
    std::swap(p_, o.p_);
    std::swap(n_, o.n_);
  }

 private:
  T* p_ = nullptr;
  size_t n_ = 0;
};

}  // namespace nnpp

#endif  // NNPP_DBUF_CUH
