// A small stand-in for the part of the ParlayLib API that the reference's
// src/*.hpp headers call, so that those headers compile unmodified into the
// reference-built oracle under oracle/_ref/.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the product (libpsc_cuda.so,
// libpsc_host.so, the drivers) includes this file.
//
// The reference pins ParlayLib as a git submodule (.gitmodules:1-3,
// LottieWang/parlay_baseline, commit not recorded in the checkout) whose
// directory is empty, so this file restates the published behaviour of the
// calls it needs in this project's own code:
//   parallel_for / num_workers / worker_id   OpenMP loop, thread ids
//   sequence<T>, slice, make_slice          owning array / non-owning view
//   delayed_seq, tabulate                   index -> value functions
//   filter, pack, pack_index,
//   pack_into_uninitialized                 order-preserving selections
//   reduce, scan_inplace, count, count_if   sums and counts
//   sort_inplace                            std::sort (keys are total orders
//                                           at every call site)
//   hash32 / hash64                         the library's own mixers
//                                           (lowbias32, SplitMix64 finaliser)
//   random_shuffle / random_permutation     the library's Feistel bijection
//                                           (P[i] = In[perm(i)]), keyed by a
//                                           seed the bridge sets per call
// The hashes and permutations are NOT ParlayLib's (its constants are not in
// the checkout); they are the ones the CUDA library and the C oracle use, so
// that raw SCC labels and LE-lists are comparable bit for bit.
#pragma once

#include <omp.h>
#include <stddef.h>
#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <cassert>
#include <cmath>
#include <cstring>
#include <iostream>
#include <string>
#include <tuple>
#include <vector>
#include <functional>
#include <initializer_list>
#include <limits>
#include <new>
#include <type_traits>
#include <utility>

#include "../../parallel-strong-connectivity_gb300/csrc/psc_hash.h"

namespace parlay {

// ---------------------------------------------------------------- threads
inline size_t num_workers() { return (size_t)omp_get_max_threads(); }
inline size_t worker_id() { return (size_t)omp_get_thread_num(); }

// Iterations [s, e) in parallel; a call made inside a parallel loop runs its
// iterations on the calling thread (nested loops keep the outer worker id).
template <class F>
inline void parallel_for(size_t s, size_t e, F&& f, long granularity = 0) {
  if (e <= s) return;
  size_t n = e - s;
  if (omp_in_parallel() || n < 2 || num_workers() == 1) {
    for (size_t i = s; i < e; i++) f(i);
    return;
  }
  long g = granularity > 0 ? granularity : (long)std::max<size_t>(1, n / (8 * num_workers()));
  if (g > 4096 && granularity <= 0) g = 4096;
#pragma omp parallel for schedule(dynamic, g)
  for (size_t i = s; i < e; i++) f(i);
}

// ---------------------------------------------------------------- views
template <class T>
class slice {
 public:
  T* b;
  T* e;
  slice() : b(nullptr), e(nullptr) {}
  slice(T* b_, T* e_) : b(b_), e(e_) {}
  size_t size() const { return (size_t)(e - b); }
  T* begin() const { return b; }
  T* end() const { return e; }
  T& operator[](size_t i) const { return b[i]; }
  slice<T> cut(size_t i, size_t j) const { return slice<T>(b + i, b + j); }
};

// Owning array.  Storage is a plain T[] (never std::vector), so that
// sequence<bool> elements are addressable bytes that the reference's
// compare_and_swap can work on.
template <class T>
class sequence {
  T* p_ = nullptr;
  size_t n_ = 0, cap_ = 0;
  void grow(size_t want) {
    size_t c = std::max<size_t>(want, cap_ ? 2 * cap_ : 4);
    T* q = new T[c]();
    for (size_t i = 0; i < n_; i++) q[i] = std::move(p_[i]);
    delete[] p_;
    p_ = q;
    cap_ = c;
  }

 public:
  using value_type = T;
  using iterator = T*;
  sequence() {}
  // A sized sequence owns at least one zeroed element, so that the
  // reference's read of P[0] when trimming has removed every vertex
  // (src/scc.hpp:313, P empty) stays in bounds and reads vertex 0.
  explicit sequence(size_t n) : p_(new T[n ? n : 1]()), n_(n), cap_(n ? n : 1) {}
  sequence(size_t n, const T& v) : sequence(n) {
    for (size_t i = 0; i < n; i++) p_[i] = v;
  }
  sequence(std::initializer_list<T> l) : sequence(l.size()) {
    size_t i = 0;
    for (const T& x : l) p_[i++] = x;
  }
  sequence(const sequence& o) : sequence(o.n_) {
    for (size_t i = 0; i < n_; i++) p_[i] = o.p_[i];
  }
  sequence(sequence&& o) noexcept : p_(o.p_), n_(o.n_), cap_(o.cap_) {
    o.p_ = nullptr;
    o.n_ = o.cap_ = 0;
  }
  sequence& operator=(const sequence& o) {
    if (this != &o) {
      sequence t(o);
      swap(t);
    }
    return *this;
  }
  sequence& operator=(sequence&& o) noexcept {
    if (this != &o) {
      delete[] p_;
      p_ = o.p_;
      n_ = o.n_;
      cap_ = o.cap_;
      o.p_ = nullptr;
      o.n_ = o.cap_ = 0;
    }
    return *this;
  }
  ~sequence() { delete[] p_; }
  void swap(sequence& o) noexcept {
    std::swap(p_, o.p_);
    std::swap(n_, o.n_);
    std::swap(cap_, o.cap_);
  }
  // Contents are value-initialised here too: the callers overwrite them.
  static sequence uninitialized(size_t n) { return sequence(n); }

  size_t size() const { return n_; }
  bool empty() const { return n_ == 0; }
  T* begin() const { return p_; }
  T* end() const { return p_ + n_; }
  T* data() const { return p_; }
  T& operator[](size_t i) const { return p_[i]; }
  T& back() const { return p_[n_ - 1]; }
  slice<T> cut(size_t i, size_t j) const { return slice<T>(p_ + i, p_ + j); }
  slice<T> head(size_t k) const { return cut(0, k); }
  void push_back(const T& v) {
    if (n_ == cap_) grow(n_ + 1);
    p_[n_++] = v;
  }
  void clear() {
    delete[] p_;
    p_ = nullptr;
    n_ = cap_ = 0;
  }
};

template <class T>
inline slice<T> make_slice(const sequence<T>& s) { return slice<T>(s.begin(), s.end()); }
template <class T>
inline slice<T> make_slice(const slice<T>& s) { return s; }
template <class T>
inline slice<T> make_slice(T* b, T* e) { return slice<T>(b, e); }

// Read-only sequence of f(i), i in [0, n).
template <class T, class F>
class delayed_sequence {
 public:
  size_t n;
  F f;
  using value_type = T;
  delayed_sequence(size_t n_, F f_) : n(n_), f(std::move(f_)) {}
  size_t size() const { return n; }
  T operator[](size_t i) const { return (T)f(i); }
};
template <class T, class F>
inline delayed_sequence<T, F> delayed_seq(size_t n, F f) {
  return delayed_sequence<T, F>(n, std::move(f));
}

template <class R>
using range_value_t = std::decay_t<decltype(std::declval<R&>()[0])>;

template <class F>
inline auto tabulate(size_t n, F f) {
  using T = std::decay_t<decltype(f((size_t)0))>;
  sequence<T> out(n);
  parallel_for(0, n, [&](size_t i) { out[i] = f(i); });
  return out;
}

// ---------------------------------------------------------------- selections
// Order-preserving selection of in[i] where keep(i); writes into out, returns
// the count.  Two passes over blocks: counts, then placement.
template <class In, class Keep, class Out>
inline size_t pack_by(const In& in, size_t n, Keep keep, Out& out) {
  const size_t B = 1 << 14;
  size_t nb = (n + B - 1) / B;
  if (nb == 0) return 0;
  sequence<size_t> cnt(nb + 1);
  parallel_for(0, nb, [&](size_t b) {
    size_t c = 0, e = std::min(n, (b + 1) * B);
    for (size_t i = b * B; i < e; i++) c += keep(i) ? 1 : 0;
    cnt[b] = c;
  }, 1);
  size_t tot = 0;
  for (size_t b = 0; b < nb; b++) {
    size_t c = cnt[b];
    cnt[b] = tot;
    tot += c;
  }
  parallel_for(0, nb, [&](size_t b) {
    size_t o = cnt[b], e = std::min(n, (b + 1) * B);
    for (size_t i = b * B; i < e; i++)
      if (keep(i)) out[o++] = in[i];
  }, 1);
  return tot;
}

template <class In, class Flags, class Out>
inline size_t pack_into_uninitialized(const In& in, const Flags& flags, Out&& out) {
  return pack_by(in, in.size(), [&](size_t i) { return (bool)flags[i]; }, out);
}

template <class In, class Flags>
inline auto pack(const In& in, const Flags& flags) {
  using T = range_value_t<In>;
  size_t n = in.size();
  size_t k = 0;
  for (size_t i = 0; i < n; i++) k += flags[i] ? 1 : 0;
  sequence<T> out(k);
  pack_by(in, n, [&](size_t i) { return (bool)flags[i]; }, out);
  return out;
}

template <class Flags>
inline sequence<size_t> pack_index(const Flags& flags) {
  auto ids = delayed_seq<size_t>(flags.size(), [](size_t i) { return i; });
  return pack(ids, flags);
}

template <class In, class Pred>
inline auto filter(const In& in, Pred pred) {
  using T = range_value_t<In>;
  size_t n = in.size();
  sequence<uint8_t> keep(n);
  parallel_for(0, n, [&](size_t i) { keep[i] = pred(in[i]) ? 1 : 0; });
  return pack(in, keep);
}

// ---------------------------------------------------------------- sums
template <class T>
struct addm {
  using value_type = T;
  T identity = T(0);
  T f(T a, T b) const { return a + b; }
};
template <class T>
struct maxm {
  using value_type = T;
  T identity = std::numeric_limits<T>::lowest();
  T f(T a, T b) const { return a < b ? b : a; }
};
template <class T>
struct minm {
  using value_type = T;
  T identity = std::numeric_limits<T>::max();
  T f(T a, T b) const { return b < a ? b : a; }
};

template <class R, class M>
inline auto reduce(const R& r, M m) {
  using T = typename M::value_type;
  size_t n = r.size();
  T acc = m.identity;
  int nt = (int)num_workers();
  if (omp_in_parallel() || n < 4096 || nt == 1) {
    for (size_t i = 0; i < n; i++) acc = m.f(acc, (T)r[i]);
    return acc;
  }
  sequence<T> part((size_t)nt, m.identity);
#pragma omp parallel num_threads(nt)
  {
    int t = omp_get_thread_num();
    T a = m.identity;
#pragma omp for schedule(static)
    for (size_t i = 0; i < n; i++) a = m.f(a, (T)r[i]);
    part[(size_t)t] = a;
  }
  for (int t = 0; t < nt; t++) acc = m.f(acc, part[(size_t)t]);
  return acc;
}
template <class R>
inline auto reduce(const R& r) {
  using T = range_value_t<R>;
  return reduce(r, addm<T>());
}

// Exclusive prefix sum in place; returns the total.
template <class R>
inline auto scan_inplace(R&& r) {
  using T = range_value_t<R>;
  T acc = 0;
  for (size_t i = 0; i < r.size(); i++) {
    T v = r[i];
    r[i] = acc;
    acc += v;
  }
  return acc;
}

template <class R, class V>
inline size_t count(const R& r, const V& v) {
  auto eq = delayed_seq<size_t>(r.size(), [&](size_t i) { return r[i] == v ? 1 : 0; });
  return reduce(eq);
}
template <class R, class P>
inline size_t count_if(const R& r, P p) {
  auto hit = delayed_seq<size_t>(r.size(), [&](size_t i) { return p(r[i]) ? 1 : 0; });
  return reduce(hit);
}

template <class R>
inline void sort_inplace(R&& r) {
  std::sort(r.begin(), r.end());
}
template <class R, class C>
inline void sort_inplace(R&& r, C cmp) {
  std::sort(r.begin(), r.end(), cmp);
}

// ---------------------------------------------------------------- utilities
inline size_t log2_up(size_t x) {
  size_t k = 0;
  while (((size_t)1 << k) < x) k++;
  return k;
}
inline uint32_t hash32(uint32_t x) { return psc::hash32(x); }
inline uint64_t hash64(uint64_t x) { return psc::hash64(x); }
// Second, independent mixers (the reference declares them; the scc, reach,
// connectivity and LE-list paths do not call them).
inline uint32_t hash32_2(uint32_t x) { return psc::hash32(x ^ 0x9E3779B9u); }
inline uint64_t hash64_2(uint64_t x) { return psc::hash64(x ^ 0xD1B54A32D192ED03ull); }

// ---------------------------------------------------------------- random
// Seed of the permutations below; the bridge sets it before each call.
inline uint64_t& shim_seed() {
  static uint64_t s = 0;
  return s;
}
// An explicit permutation that random_permutation returns instead (LE-lists
// take theirs as an input); null when unset.
inline const uint32_t*& shim_perm() {
  static const uint32_t* p = nullptr;
  return p;
}

template <class R>
inline auto random_shuffle(const R& in) {
  using T = range_value_t<R>;
  size_t n = in.size();
  sequence<T> out(n);
  psc::FeistelKey k = psc::feistel_key(n, shim_seed());
  parallel_for(0, n, [&](size_t i) { out[i] = in[psc::feistel(k, i)]; });
  return out;
}

template <class T>
inline sequence<T> random_permutation(T n) {
  sequence<T> out((size_t)n);
  if (shim_perm()) {
    const uint32_t* p = shim_perm();
    parallel_for(0, (size_t)n, [&](size_t i) { out[i] = (T)p[i]; });
    return out;
  }
  psc::FeistelKey k = psc::feistel_key((uint64_t)n, shim_seed());
  parallel_for(0, (size_t)n, [&](size_t i) { out[i] = (T)psc::feistel(k, i); });
  return out;
}

}  // namespace parlay
