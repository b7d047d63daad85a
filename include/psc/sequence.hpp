// psc/sequence.hpp — the subset of parlay::sequence<T> that the reference's
// public interfaces use (operator[], size, begin/end, data, cut, construction
// with a size or a size and a value, uninitialized, push_back, back).  The
// reference takes sequence<T> from ParlayLib (src/graph.hpp:39-42,
// src/scc.hpp:79); this is an API-level restatement so the drop-in headers
// need no ParlayLib.  Storage is contiguous: sequence<bool> holds one byte per
// element (unlike std::vector<bool>), so data() can be handed to the C ABI.
#pragma once
#include <algorithm>
#include <cstddef>
#include <cstring>
#include <memory>
#include <utility>

namespace psc {

template <class T>
class sequence {
 public:
  using value_type = T;
  sequence() = default;
  explicit sequence(size_t n) : n_(n), cap_(n), p_(n ? new T[n]() : nullptr) {}
  sequence(size_t n, const T& v) : sequence(n) { std::fill(begin(), end(), v); }
  sequence(const sequence& o) : sequence(o.n_) { std::copy(o.begin(), o.end(), begin()); }
  sequence(sequence&& o) noexcept { swap(o); }
  sequence& operator=(sequence o) noexcept {
    swap(o);
    return *this;
  }
  static sequence uninitialized(size_t n) {
    sequence s;
    s.n_ = s.cap_ = n;
    s.p_.reset(n ? new T[n] : nullptr);
    return s;
  }
  void swap(sequence& o) noexcept {
    std::swap(n_, o.n_);
    std::swap(cap_, o.cap_);
    std::swap(p_, o.p_);
  }
  T& operator[](size_t i) { return p_[i]; }
  const T& operator[](size_t i) const { return p_[i]; }
  size_t size() const { return n_; }
  bool empty() const { return n_ == 0; }
  T* begin() { return p_.get(); }
  T* end() { return p_.get() + n_; }
  const T* begin() const { return p_.get(); }
  const T* end() const { return p_.get() + n_; }
  T* data() { return p_.get(); }
  const T* data() const { return p_.get(); }
  T& back() { return p_[n_ - 1]; }
  void push_back(const T& v) {
    if (n_ == cap_) {
      size_t c = cap_ ? 2 * cap_ : 8;
      std::unique_ptr<T[]> q(new T[c]());
      std::copy(begin(), end(), q.get());
      p_ = std::move(q);
      cap_ = c;
    }
    p_[n_++] = v;
  }
  void clear() {
    n_ = cap_ = 0;
    p_.reset();
  }
  // A view [a, b) (parlay's slice, as used by centers.cut(...)).
  struct slice {
    T* b_;
    T* e_;
    T* begin() const { return b_; }
    T* end() const { return e_; }
    size_t size() const { return (size_t)(e_ - b_); }
    T& operator[](size_t i) const { return b_[i]; }
  };
  slice cut(size_t a, size_t b) { return slice{begin() + a, begin() + b}; }

 private:
  size_t n_ = 0, cap_ = 0;
  std::unique_ptr<T[]> p_;
};

}  // namespace psc

namespace parlay {
using psc::sequence;
}
