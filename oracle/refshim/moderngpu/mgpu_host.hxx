// Host (CPU) restatement of the ModernGPU 2.x API surface that the VEDAS
// reference sources call.  Test infrastructure only: it lets the reference's
// own src/*.cu files compile with g++ so that they can serve as a parity
// oracle.  ModernGPU is an un-vendored, unpinned submodule of the reference
// (its `moderngpu/` directory is empty), so this file restates the library's
// published semantics; nothing here is taken from ModernGPU's source.
//
// Semantics restated (ModernGPU 2.x documentation):
//   transform(f, n, ctx)            : f(i) for every i in [0, n)
//   sorted_search<lower|upper>(a,b) : for each a[i], lower/upper bound in b
//   transform_scan<T>(f, n, out, plus, reduction) : exclusive scan of f(i)
//   inner_join(a, na, b, nb, less)  : (i, j) for every a[i] == b[j], ordered
//                                     by i, then j (both inputs sorted)
// The join's restatement follows the reference's own in-repo restatement of
// the algorithm at src/JoinQueryJob.cu:68-101.
#ifndef VEDAS_ORACLE_MGPU_HOST_HXX
#define VEDAS_ORACLE_MGPU_HOST_HXX

#include <algorithm>
#include <cstddef>
#include <cstring>
#include <utility>
#include <vector>

#include "../cuda_host.h"

namespace mgpu {

enum bounds_t { bounds_lower, bounds_upper };

struct empty_t {};

template <typename T>
struct less_t {
  bool operator()(const T& a, const T& b) const { return a < b; }
};

template <typename T>
struct plus_t {
  T operator()(const T& a, const T& b) const { return a + b; }
};

class standard_context_t {
 public:
  explicit standard_context_t(bool print_prop = true, void* stream = nullptr) {
    (void)print_prop;
    (void)stream;
  }
};
typedef standard_context_t context_t;

template <typename T>
class mem_t {
 public:
  mem_t() = default;
  mem_t(size_t count, context_t& ctx) : v_(count) { (void)ctx; }
  mem_t(const mem_t&) = delete;
  mem_t& operator=(const mem_t&) = delete;
  mem_t(mem_t&& o) noexcept : v_(std::move(o.v_)) {}
  mem_t& operator=(mem_t&& o) noexcept {
    v_ = std::move(o.v_);
    return *this;
  }
  T* data() { return v_.data(); }
  const T* data() const { return v_.data(); }
  size_t size() const { return v_.size(); }

 private:
  std::vector<T> v_;
};

template <typename T>
std::vector<T> from_mem(const mem_t<T>& m) {
  return std::vector<T>(m.data(), m.data() + m.size());
}

template <typename F, typename I>
void transform(F f, I count, context_t& ctx) {
  (void)ctx;
  long long n = static_cast<long long>(count);
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < n; ++i) f(static_cast<I>(i));
}

template <bounds_t bounds, typename launch_arg_t = empty_t, typename A, typename B,
          typename O, typename C>
void sorted_search(const A* a, int a_count, const B* b, int b_count, O* out, C comp,
                   context_t& ctx) {
  (void)ctx;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < a_count; ++i) {
    const B* it = (bounds == bounds_lower) ? std::lower_bound(b, b + b_count, a[i], comp)
                                           : std::upper_bound(b, b + b_count, a[i], comp);
    out[i] = static_cast<O>(it - b);
  }
}

template <typename T, typename F, typename O, typename Op>
void transform_scan(F f, int count, O* out, Op op, T* reduction, context_t& ctx) {
  (void)ctx;
  T acc = T();
  for (int i = 0; i < count; ++i) {
    out[i] = acc;
    acc = op(acc, static_cast<T>(f(i)));
  }
  if (reduction) *reduction = acc;
}

// Sorted inner join, restated from the reference's description of the
// algorithm (src/JoinQueryJob.cu:68-101): lower and upper bounds of each a[i]
// in b give the matching range; pairs are emitted for i ascending, then j
// ascending within [lower, upper).
template <typename K, typename C>
mem_t<int2> inner_join(const K* a, int a_count, const K* b, int b_count, C comp,
                       context_t& ctx) {
  std::vector<int> lo(a_count), hi(a_count);
  std::vector<long long> start(a_count + 1);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < a_count; ++i) {
    lo[i] = static_cast<int>(std::lower_bound(b, b + b_count, a[i], comp) - b);
    hi[i] = static_cast<int>(std::upper_bound(b, b + b_count, a[i], comp) - b);
  }
  start[0] = 0;
  for (int i = 0; i < a_count; ++i) start[i + 1] = start[i] + (hi[i] - lo[i]);
  mem_t<int2> out(static_cast<size_t>(start[a_count]), ctx);
  int2* o = out.data();
#pragma omp parallel for schedule(dynamic, 1024)
  for (int i = 0; i < a_count; ++i) {
    long long k = start[i];
    for (int j = lo[i]; j < hi[i]; ++j, ++k) o[k] = make_int2(i, j);
  }
  return out;
}

}  // namespace mgpu

#endif
