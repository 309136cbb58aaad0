/*
 * hashinator_compat.h — drop-in C++ surface of Hashinator's accelerated API
 * over libhx (hx.h). Compile the including translation unit with nvcc and
 * link libhx.so.
 *
 *   Hashinator::Hashmap<K,V>      hashinator/hashinator.h:59-62  (K = V = uint32_t or uint64_t)
 *   Hashinator::hash_pair<K,V>    hashinator/hash_pair.h:30-75
 *   Hashinator::Info / status     hashinator/defaults.h:44-54, common.h:85
 *   split::SplitVector<T>         splitvector/splitvec.h:83 (managed memory, minimal surface)
 *   split::tools::copy_if, copy_keys_if, splitStackArena,
 *   estimateMemoryForCompaction   splitvector/split_tools.h:491-535, 1065-1223
 *   split::tools::split_prefix_scan  split_tools.h:363-418
 *   device API (upload/download, device_find/insert/erase, iterators,
 *   warpInsert/warpFind/warpErase)   hashinator.h:853-1126, 1417-1769
 *
 * Behaviour matches the reference's: every accelerated call blocks the host
 * until its stream is done (hashinator/hashers.h:55 and siblings), CUDA
 * errors abort with a message (splitvector/split_allocators.h:33-40), and a
 * full table is reported through peek_status() == status::fail. Rules are
 * either hx_pred descriptors (run inside libhx) or any __host__ __device__
 * functor bool(T&) (run by the header's kernels in this translation unit,
 * with offsets from libhx's scan).
 */
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <initializer_list>
#include <iterator>
#include <limits>
#include <new>
#include <stdexcept>
#include <type_traits>
#include <utility>
#include <vector>

#include "hx.h"
#include "hx_device_api.cuh"
#include "hx_stream.cuh"

namespace hxcompat {
inline void check(hx_status st, const char* what) {
  if (st != HX_OK) {
    std::fprintf(stderr, "hashinator_compat: %s failed: %s (cuda error %d)\n", what, hx_status_string(st),
                 hx_last_cuda_error());
    std::abort();
  }
}
inline void check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    std::fprintf(stderr, "hashinator_compat: %s failed: %s\n", what, cudaGetErrorString(e));
    std::abort();
  }
}
// A valid key: neither EMPTY nor TOMBSTONE (the rule of the reference's
// extractLoop / extractAllKeys); at namespace scope so kernels can take it.
template <typename P, typename K, K EMPTY, K TOMB>
struct ValidKeyRule {
  __host__ __device__ bool operator()(const P& p) const { return p.first != EMPTY && p.first != TOMB; }
};
}  // namespace hxcompat

namespace Hashinator {

enum status { success, fail, invalid };
enum targets { host, device, automatic };

template <typename T, typename U>
struct hash_pair {
  T first;
  U second;
  __host__ __device__ hash_pair() : first(T()), second(U()) {}
  __host__ __device__ hash_pair(const T& f, const U& s) : first(f), second(s) {}
  __host__ __device__ bool operator==(const hash_pair& y) const { return first == y.first && second == y.second; }
  __host__ __device__ bool operator!=(const hash_pair& y) const { return !(*this == y); }
};
template <class T, class U>
__host__ __device__ inline hash_pair<T, U> make_pair(T x, U y) {
  return hash_pair<T, U>(x, y);
}

struct Info {
  int sizePower;
  size_t fill;
  size_t currentMaxBucketOverflow;
  size_t tombstoneCounter;
  status err;
};

}  // namespace Hashinator

namespace split {

/* split_unified_allocator<T> (splitvector/split_allocators.h:62-129): the
 * reference's default allocator, managed memory. SplitVector below always
 * keeps its elements, size and capacity in managed memory, so the allocator
 * parameter only spells the reference's type. */
template <typename T>
struct split_unified_allocator {
  using value_type = T;
};

/* SplitInfo (splitvec.h:43-46): what copyMetadata copies out. */
typedef struct SplitVectorInfo {
  size_t size;
  size_t capacity;
} SplitInfo;

namespace detail {
template <typename T>
__global__ void k_fill(T* p, size_t n, T v) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) p[i] = v;
}
}  // namespace detail

/* SplitVector<T> (splitvector/splitvec.h:83-1560). Elements, size and
 * capacity live in managed memory, as in the reference, so that the host and
 * device code share one vector: upload() gives kernels a device copy of the
 * object, and device_push_back / device_resize / device_insert change the
 * size that the host reads after a synchronisation. The observable rules
 * follow the reference's, including its quirks:
 *   - SplitVector() has no storage; reserve(n) on it allocates exactly n
 *     elements (splitvec.h:850-856); otherwise reserve grows to twice the
 *     request unless eco is set;
 *   - device_push_back fills at most capacity - 1 elements (splitvec.h:1070-1078);
 *   - the iterator's postfix ++ and -- return the neighbour without moving
 *     the iterator (splitvec.h:1133-1136);
 *   - device_insert(it, first, last) writes the range at `it` and grows the
 *     size by its length without moving later elements (splitvec.h:1362-1384),
 *     and device_insert(it, n, val) leaves the first index + n elements in
 *     place and puts the n copies after them (splitvec.h:1432-1460);
 * where the reference would assert or write past the allocation (a full
 * vector, an index out of range), the device calls here do nothing and
 * device_push_back returns false. */
template <typename T, class Allocator = split_unified_allocator<T>>
class SplitVector {
  T* data_ = nullptr;
  size_t* meta_ = nullptr;  // managed: meta_[0] = size, meta_[1] = capacity
  SplitVector* d_vec_ = nullptr;

  static void fill_range(T* p, size_t n) {
    if (!n) return;
    if constexpr (std::is_trivially_copyable<T>::value) {
      const unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, 4096);
      detail::k_fill<<<blocks, 256>>>(p, n, T());
      hxcompat::check_cuda(cudaGetLastError(), "k_fill");
      hxcompat::check_cuda(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
    } else {
      for (size_t i = 0; i < n; ++i) new (&p[i]) T();
    }
  }
  static T* alloc_elems(size_t n) {
    T* p = nullptr;
    if (n) hxcompat::check_cuda(cudaMallocManaged(&p, n * sizeof(T)), "cudaMallocManaged");
    fill_range(p, n);
    return p;
  }
  void alloc_meta() {
    if (!meta_) {
      hxcompat::check_cuda(cudaMallocManaged(&meta_, 2 * sizeof(size_t)), "cudaMallocManaged");
      meta_[0] = meta_[1] = 0;
    }
  }
  // _allocate(size) (splitvec.h:181): size = capacity = n, elements T().
  void allocate(size_t n) {
    alloc_meta();
    data_ = alloc_elems(n);
    meta_[0] = meta_[1] = n;
  }
  void copy_elems(T* dst, const T* src, size_t n) {
    if (!n) return;
    hxcompat::check_cuda(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
    if constexpr (std::is_trivially_copyable<T>::value) {
      hxcompat::check_cuda(cudaMemcpy(dst, src, n * sizeof(T), cudaMemcpyDefault), "cudaMemcpy");
    } else {
      for (size_t i = 0; i < n; ++i) dst[i] = src[i];
    }
  }
  void reallocate(size_t cap) {
    T* p = alloc_elems(cap);
    copy_elems(p, data_, std::min(size(), cap));
    if (data_) cudaFree(data_);
    data_ = p;
    meta_[1] = cap;
  }

 public:
  using value_type = T;

  /* iterator (splitvec.h:1101-1162), postfix ++ / -- as in the reference. */
  class iterator {
    T* p_;

   public:
    using iterator_category = std::forward_iterator_tag;
    using value_type = T;
    using difference_type = int64_t;
    using pointer = T*;
    using reference = T&;
    __host__ __device__ iterator(T* p = nullptr) : p_(p) {}
    __host__ __device__ T* data() const { return p_; }
    __host__ __device__ T* operator->() const { return p_; }
    __host__ __device__ T& operator*() const { return *p_; }
    __host__ __device__ bool operator==(const iterator& o) const { return p_ == o.p_; }
    __host__ __device__ bool operator!=(const iterator& o) const { return p_ != o.p_; }
    __host__ __device__ iterator& operator++() {
      ++p_;
      return *this;
    }
    __host__ __device__ iterator operator++(int) const { return iterator(p_ + 1); }
    __host__ __device__ iterator& operator--() {
      --p_;
      return *this;
    }
    __host__ __device__ iterator operator--(int) const { return iterator(p_ - 1); }
    __host__ __device__ iterator& operator+=(int64_t d) {
      p_ += d;
      return *this;
    }
    __host__ __device__ iterator& operator-=(int64_t d) {
      p_ -= d;
      return *this;
    }
    __host__ __device__ iterator operator+(int64_t d) const { return iterator(p_ + d); }
    __host__ __device__ iterator operator-(int64_t d) const { return iterator(p_ - d); }
  };
  class const_iterator {
    const T* p_;

   public:
    using iterator_category = std::forward_iterator_tag;
    using value_type = T;
    using difference_type = int64_t;
    using pointer = const T*;
    using reference = const T&;
    __host__ __device__ const_iterator(const T* p = nullptr) : p_(p) {}
    __host__ __device__ const_iterator(const iterator& it) : p_(it.data()) {}
    __host__ __device__ const T* data() const { return p_; }
    __host__ __device__ const T* operator->() const { return p_; }
    __host__ __device__ const T& operator*() const { return *p_; }
    __host__ __device__ bool operator==(const const_iterator& o) const { return p_ == o.p_; }
    __host__ __device__ bool operator!=(const const_iterator& o) const { return p_ != o.p_; }
    __host__ __device__ const_iterator& operator++() {
      ++p_;
      return *this;
    }
    __host__ __device__ const_iterator operator++(int) const { return const_iterator(p_ + 1); }
    __host__ __device__ const_iterator& operator--() {
      --p_;
      return *this;
    }
    __host__ __device__ const_iterator operator--(int) const { return const_iterator(p_ - 1); }
    __host__ __device__ const_iterator operator+(int64_t d) const { return const_iterator(p_ + d); }
    __host__ __device__ const_iterator operator-(int64_t d) const { return const_iterator(p_ - d); }
  };

  // ---- construction (splitvec.h:200-300) ----
  SplitVector() { alloc_meta(); }
  explicit SplitVector(size_t n) { allocate(n); }
  SplitVector(size_t n, const T& v) {
    allocate(n);
    for (size_t i = 0; i < n; ++i) data_[i] = v;
  }
  SplitVector(std::initializer_list<T> init) {
    allocate(init.size());
    size_t i = 0;
    for (const T& v : init) data_[i++] = v;
  }
  explicit SplitVector(const std::vector<T>& v) {
    allocate(v.size());
    for (size_t i = 0; i < v.size(); ++i) data_[i] = v[i];
  }
  SplitVector(const SplitVector& o) {
    allocate(o.size());
    copy_elems(data_, o.data_, o.size());
  }
  SplitVector(SplitVector&& o) noexcept : data_(o.data_), meta_(o.meta_) {
    o.data_ = nullptr;
    o.meta_ = nullptr;
  }
  SplitVector& operator=(const SplitVector& o) {
    if (this != &o) {
      resize(o.size());
      copy_elems(data_, o.data_, o.size());
    }
    return *this;
  }
  SplitVector& operator=(SplitVector&& o) noexcept {
    if (this != &o) {
      std::swap(data_, o.data_);
      std::swap(meta_, o.meta_);
    }
    return *this;
  }
  ~SplitVector() {
    if (data_) cudaFree(data_);
    if (meta_) cudaFree(meta_);
    if (d_vec_) cudaFree(d_vec_);
  }

  // ---- access (host and device) ----
  __host__ __device__ T* data() noexcept { return data_; }
  __host__ __device__ const T* data() const noexcept { return data_; }
  __host__ __device__ const size_t& size() const noexcept { return meta_[0]; }
  __host__ __device__ size_t capacity() const noexcept { return meta_[1]; }
  __host__ __device__ bool empty() const noexcept { return size() == 0; }
  __host__ __device__ T& operator[](size_t i) noexcept { return data_[i]; }
  __host__ __device__ const T& operator[](size_t i) const noexcept { return data_[i]; }
  __host__ __device__ T& at(size_t i) { return data_[i]; }
  __host__ __device__ const T& at(size_t i) const { return data_[i]; }
  __host__ __device__ T& back() noexcept { return data_[size() - 1]; }
  __host__ __device__ const T& back() const noexcept { return data_[size() - 1]; }
  __host__ __device__ T& front() noexcept { return data_[0]; }
  __host__ __device__ const T& front() const noexcept { return data_[0]; }
  __host__ __device__ iterator begin() noexcept { return iterator(data_); }
  __host__ __device__ iterator end() noexcept { return iterator(data_ + size()); }
  __host__ __device__ const_iterator begin() const noexcept { return const_iterator(data_); }
  __host__ __device__ const_iterator end() const noexcept { return const_iterator(data_ + size()); }
  // size_t* of the size word (managed memory): libhx's compactions write a
  // count there on the device.
  size_t* size_word() { return meta_; }

  // ---- host-side changes (splitvec.h:720-930, 1032-1060, 1262-1360) ----
  void reserve(size_t n, bool eco = false, cudaStream_t = 0) {
    if (!data_) {
      allocate(n);
      meta_[0] = 0;
      return;
    }
    if (n <= capacity()) return;
    reallocate(eco ? n : 2 * n);
  }
  void resize(size_t n, bool eco = false, cudaStream_t s = 0) {
    if (n > size()) reserve(n, eco, s);
    meta_[0] = n;
  }
  void grow(cudaStream_t s = 0) { reserve(capacity() + 1, false, s); }
  void shrink_to_fit(cudaStream_t = 0) {
    if (data_ && capacity() != size()) reallocate(size());
  }
  __host__ __device__ void clear() noexcept { meta_[0] = 0; }
  __host__ __device__ void remove_from_back(size_t n) noexcept { meta_[0] = size() - n; }
  __host__ __device__ void pop_back() noexcept {
    if (size() > 0) remove_from_back(1);
  }
  void push_back(const T& v) {
    if (!data_) {
      allocate(1);
      data_[0] = v;
      return;
    }
    resize(size() + 1);
    data_[size() - 1] = v;
  }
  template <class... Args>
  void emplace_back(Args&&... args) {
    push_back(T(std::forward<Args>(args)...));
  }
  iterator insert(iterator it, const T& v) {
    const int64_t index = it.data() - data_;
    if (index < 0 || index > (int64_t)size()) throw std::out_of_range("Insert");
    const size_t n = size();
    resize(n + 1);
    for (int64_t i = (int64_t)n - 1; i >= index; --i) data_[i + 1] = data_[i];
    data_[index] = v;
    return iterator(data_ + index);
  }
  iterator insert(iterator it, size_t count, const T& v) {
    const int64_t index = it.data() - data_;
    if (index < 0 || index > (int64_t)size()) throw std::out_of_range("Insert");
    const size_t n = size();
    resize(n + count);
    for (int64_t i = (int64_t)n - 1; i >= index; --i) data_[i + count] = data_[i];
    for (size_t k = 0; k < count; ++k) data_[index + k] = v;
    return iterator(data_ + index);
  }
  template <typename InputIterator, class = typename std::enable_if<!std::is_integral<InputIterator>::value>::type>
  iterator insert(iterator it, InputIterator p0, InputIterator p1) {
    const int64_t index = it.data() - data_;
    if (index < 0 || index > (int64_t)size()) throw std::out_of_range("Insert");
    const size_t count = (size_t)std::distance(p0, p1);
    const size_t n = size();
    resize(n + count);
    for (int64_t i = (int64_t)n - 1; i >= index; --i) data_[i + count] = data_[i];
    size_t k = 0;
    for (auto p = p0; p != p1; ++p) data_[index + k++] = *p;
    return iterator(data_ + index);
  }
  /* erase(it) / erase(first, last) (splitvec.h:1472-1520), host and device. */
  __host__ __device__ iterator erase(iterator it) noexcept {
    const int64_t index = it.data() - data_;
    for (size_t i = (size_t)index; i + 1 < size(); ++i) data_[i] = data_[i + 1];
    meta_[0] = size() - 1;
    return iterator(data_ + index);
  }
  __host__ __device__ iterator erase(iterator p0, iterator p1) noexcept {
    const int64_t start = p0.data() - data_, stop = p1.data() - data_;
    const int64_t range = stop - start;
    const size_t sz = size();
    for (size_t i = (size_t)start; i + range < sz; ++i) data_[i] = data_[i + range];
    meta_[0] = sz - range;
    return iterator(data_ + start);
  }
  void swap(SplitVector& o) noexcept {
    std::swap(data_, o.data_);
    std::swap(meta_, o.meta_);
  }
  /* copyMetadata(SplitInfo*, s) (splitvec.h:568-571). */
  void copyMetadata(SplitInfo* dst, cudaStream_t s = 0) {
    hxcompat::check_cuda(cudaMemcpyAsync(&dst->size, &meta_[0], sizeof(size_t), cudaMemcpyDefault, s),
                         "cudaMemcpyAsync");
    hxcompat::check_cuda(cudaMemcpyAsync(&dst->capacity, &meta_[1], sizeof(size_t), cudaMemcpyDefault, s),
                         "cudaMemcpyAsync");
  }
  /* upload(s) (splitvec.h:481-491): a device copy of this object for kernels;
   * it shares the elements, size and capacity. Call it again after any host
   * call that may reallocate. device_pointer() (:497) returns the last one. */
  template <bool optimize = true>
  SplitVector* upload(cudaStream_t s = 0) {
    if (!d_vec_) hxcompat::check_cuda(cudaMalloc(&d_vec_, sizeof(SplitVector)), "cudaMalloc");
    hxcompat::check_cuda(cudaMemcpyAsync(d_vec_, this, sizeof(SplitVector), cudaMemcpyHostToDevice, s),
                         "cudaMemcpyAsync");
    return d_vec_;
  }
  const SplitVector* device_pointer() const noexcept { return d_vec_; }
  void optimizeGPU(cudaStream_t = 0) noexcept {}
  void optimizeCPU(cudaStream_t = 0) noexcept {}
  void memAdvise(cudaMemoryAdvise, int = -1, cudaStream_t = 0) {}
  void streamAttach(cudaStream_t, uint32_t = cudaMemAttachSingle) {}

  // ---- device-side changes (splitvec.h:902-915, 1070-1100, 1362-1460) ----
  /* device_push_back: a slot by an atomic increment of the size; fails (and
   * takes the increment back) when the slot is at capacity - 1 or beyond. */
  __device__ bool device_push_back(const T& v) {
    auto* sz = reinterpret_cast<unsigned long long*>(meta_);
    const unsigned long long old = atomicAdd(sz, 1ull);
    const size_t cap = meta_[1];
    if (cap == 0 || old >= cap - 1) {
      atomicAdd(sz, ~0ull);  // -1
      return false;
    }
    data_[old] = v;
    return true;
  }
  __device__ bool device_push_back(T&& v) {
    auto* sz = reinterpret_cast<unsigned long long*>(meta_);
    const unsigned long long old = atomicAdd(sz, 1ull);
    const size_t cap = meta_[1];
    if (cap == 0 || old >= cap - 1) {
      atomicAdd(sz, ~0ull);
      return false;
    }
    data_[old] = std::move(v);
    return true;
  }
  /* device_resize(n, construct): n beyond the capacity is ignored. */
  __device__ void device_resize(size_t n, bool construct = true) {
    if (n > capacity()) return;
    if (construct)
      for (size_t i = size(); i < n; ++i) data_[i] = T();
    meta_[0] = n;
  }
  template <typename InputIterator, class = typename std::enable_if<!std::is_integral<InputIterator>::value>::type>
  __device__ iterator device_insert(iterator it, InputIterator p0, InputIterator p1) noexcept {
    const int64_t count = p1.data() - p0.data();
    const int64_t index = it.data() - data_;
    if (count < 0 || index < 0 || index > (int64_t)size() || size() + (size_t)count > capacity()) return end();
    device_resize(size() + count, false);
    for (int64_t i = 0; i < count; ++i) data_[index + i] = *(p0.data() + i);
    return iterator(data_ + index + count);
  }
  __device__ iterator device_insert(iterator it, const T& v) noexcept {
    if (it == end()) {
      device_push_back(v);
      return iterator(data_ + size() - 1);
    }
    const int64_t index = it.data() - data_;
    const size_t n = size();
    if (index < 0 || index > (int64_t)n || n == capacity()) return end();
    device_resize(n + 1, false);
    for (int64_t i = (int64_t)n - 1; i >= index; --i) data_[i + 1] = data_[i];
    data_[index] = v;
    return iterator(data_ + index);
  }
  __device__ iterator device_insert(iterator it, const size_t count, const T& v) {
    const int64_t index = it.data() - data_;
    const size_t n = size();
    if (index < 0 || index > (int64_t)n || n + count > capacity()) return end();
    device_resize(n + count, false);
    // elements from index + count on move up by count (in the reference's
    // order, so a source is read before it is overwritten) ...
    for (int64_t c = (int64_t)n - 1; c > index && c >= index + (int64_t)count; --c) data_[c + count] = data_[c];
    // ... and the copies go to [index + count, index + 2 count), inside the new size
    for (size_t k = 0; k < count && index + count + k < n + count; ++k) data_[index + count + k] = v;
    return iterator(data_ + index);
  }
};

template <typename T, class A>
inline bool operator==(const SplitVector<T, A>& a, const SplitVector<T, A>& b) {
  if (a.size() != b.size()) return false;
  for (size_t i = 0; i < a.size(); ++i)
    if (!(a[i] == b[i])) return false;
  return true;
}
template <typename T, class A>
inline bool operator!=(const SplitVector<T, A>& a, const SplitVector<T, A>& b) {
  return !(a == b);
}

namespace tools {
namespace detail {

struct Identity {
  template <typename T>
  __device__ const T& operator()(const T& x) const {
    return x;
  }
};
struct KeyOf {
  template <typename T>
  __device__ auto operator()(const T& x) const -> decltype(x.first) {
    return x.first;
  }
};

// A caller's rule as the selector of the single-pass compaction
// (hx_stream.cuh). The reference's rules may take their argument by
// non-const reference, so each call gets a copy of the element (and of the
// rule, whose call operator need not be const).
template <typename Rule>
struct RuleSel {
  Rule rule;
  static constexpr bool kRewrites = false;
  static constexpr bool kIndexed = false;
  template <class T>
  __device__ __forceinline__ bool operator()(const T& x) const {
    Rule r = rule;
    T y = x;
    return r(y);
  }
  template <class T>
  __device__ __forceinline__ void rewrite(T*, uint64_t, const T&, bool) const {}
};

// The first elements of an input that does not start on a 16-byte boundary
// (fewer than 16 / sizeof(T)), compacted by one thread before the main pass:
// out[0..h) and the count h in *head, where the main pass starts counting.
template <typename T, typename O, typename Rule, typename Proj>
__global__ void k_head(const T* in, size_t n, Rule rule, Proj proj, O* out, size_t cap,
                       unsigned long long* head) {
  unsigned long long c = 0;
  for (size_t i = 0; i < n; ++i) {
    T y = in[i];
    Rule r = rule;
    if (r(y)) {
      if (c < cap) out[c] = proj(in[i]);
      ++c;
    }
  }
  *head = c;
}

// Generic path for element sizes that do not divide 16 bytes: per-block
// counts, libhx's exclusive scan of the counts, then an order-preserving
// scatter (each block ranks its elements with warp ballots and a warp scan).
template <typename T, typename Rule>
__global__ void k_count_blocks(const T* in, size_t n, Rule rule, uint32_t* counts) {
  __shared__ uint32_t s;
  if (threadIdx.x == 0) s = 0;
  __syncthreads();
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  bool sel = false;
  if (i < n) {
    T x = in[i];
    Rule r = rule;
    sel = r(x);
  }
  const unsigned b = __ballot_sync(0xffffffffu, sel);
  if ((threadIdx.x & 31) == 0 && b) atomicAdd(&s, (uint32_t)__popc(b));
  __syncthreads();
  if (threadIdx.x == 0) counts[blockIdx.x] = s;
}
template <typename T, typename O, typename Rule, typename Proj>
__global__ void k_scatter_blocks(const T* in, size_t n, Rule rule, const uint32_t* offsets, O* out, size_t cap,
                                 unsigned long long* total, unsigned long long total_max, size_t nblocks, Proj proj) {
  __shared__ uint32_t warp_base[32];
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  bool sel = false;
  T x;
  if (i < n) {
    x = in[i];
    T y = x;
    Rule r = rule;
    sel = r(y);
  }
  const unsigned b = __ballot_sync(0xffffffffu, sel);
  if (lane == 0) warp_base[warp] = __popc(b);
  __syncthreads();
  if (warp == 0) {
    const unsigned nw = blockDim.x / 32;
    const unsigned c = lane < (int)nw ? warp_base[lane] : 0u;
    const unsigned incl = hxs::warp_incl_scan(c, lane);
    if (lane < (int)nw) warp_base[lane] = incl - c;
    if (lane == 31 && blockIdx.x == nblocks - 1) {
      const unsigned long long t = (unsigned long long)offsets[blockIdx.x] + incl;
      *total = t < total_max ? t : total_max;
    }
  }
  __syncthreads();
  if (sel) {
    const size_t dst = (size_t)offsets[blockIdx.x] + warp_base[warp] + __popc(b & ((1u << lane) - 1u));
    if (dst < cap) out[dst] = proj(x);
  }
}

// Device scratch of one compaction of n elements of T. Layout: the kernels'
// scratch, then 256 bytes of count words at the end (a head count at
// need - 256, the result count at need - 248). The kernels' part is the
// single-pass kernel's count slots, or, for element sizes that do not divide
// 16, the block counts and offsets and libhx's scan scratch.
template <typename T>
inline size_t blocks_bytes(size_t n) {
  const size_t nb = (n + 255) / 256;
  return ((2 * nb * sizeof(uint32_t) + 255) / 256) * 256;
}
template <typename T>
inline size_t compaction_scratch_bytes(size_t n) {
  if constexpr (16 % sizeof(T) == 0) {
    return (((size_t)hxs::scratch_need(n, sizeof(T)) + 255) / 256) * 256 + 256;
  } else {
    const size_t nb = (n + 255) / 256;
    uint64_t sb = 0;
    hx_scratch_bytes(HX_SCRATCH_SCAN, nb ? nb : 1, &sb);
    return blocks_bytes<T>(n) + (((size_t)sb + 255) / 256) * 256 + 256;
  }
}
template <typename T>
inline size_t* result_word(void* scratch, size_t n) {
  return reinterpret_cast<size_t*>(static_cast<char*>(scratch) + compaction_scratch_bytes<T>(n) - 248);
}

// Stable compaction with a caller's rule, on the stream, with no host
// synchronisation: out[0..c) = proj(x) for the selected x in input order
// (writes at or beyond cap are dropped), and min(c, count_max) to *count.
// Scratch: `scratch` (at least compaction_scratch_bytes<T>(n) bytes) or, if
// it is null, a stream-ordered allocation freed on the stream afterwards.
template <typename T, typename O, typename Rule, typename Proj>
void compact(const T* in, O* out, size_t n, size_t cap, Rule rule, Proj proj, size_t* count, size_t count_max,
             void* scratch, cudaStream_t s) {
  static_assert(sizeof(size_t) == sizeof(unsigned long long), "counts are 64-bit");
  auto* cnt = reinterpret_cast<unsigned long long*>(count);
  if (n == 0) {
    hxcompat::check_cuda(cudaMemsetAsync(cnt, 0, sizeof(*cnt), s), "cudaMemsetAsync");
    return;
  }
  const size_t need = compaction_scratch_bytes<T>(n);
  void* owned = nullptr;
  if (!scratch) {
    hxcompat::check_cuda(cudaMallocAsync(&owned, need, s), "cudaMallocAsync");
    scratch = owned;
  }
  if constexpr (16 % sizeof(T) == 0) {
    auto* head = reinterpret_cast<unsigned long long*>(static_cast<char*>(scratch) + need - 256);
    const size_t mis = (size_t)(reinterpret_cast<uintptr_t>(in) % 16);
    if (mis % sizeof(T)) {
      std::fprintf(stderr, "hashinator_compat: copy_if input is not aligned to its element size\n");
      std::abort();
    }
    const size_t h = std::min(n, mis ? (16 - mis) / sizeof(T) : (size_t)0);
    if (h) {
      k_head<<<1, 1, 0, s>>>(in, h, rule, proj, out, cap, head);
      hxcompat::check_cuda(cudaGetLastError(), "k_head");
    }
    if (n > h) {
      hxs::Done done{cnt, nullptr, nullptr};
      done.count_max = count_max;
      done.base_from = h ? head : nullptr;
      hxcompat::check_cuda(hxs::launch<T, O, RuleSel<Rule>, false>(in + h, out, n - h, RuleSel<Rule>{rule}, cap,
                                                                  done, scratch, s),
                           "single-pass compaction");
    } else {  // fewer elements than one 16-byte group: the head is everything
      hxcompat::check_cuda(cudaMemcpyAsync(cnt, head, sizeof(*cnt), cudaMemcpyDeviceToDevice, s), "cudaMemcpyAsync");
    }
  } else {
    const unsigned block = 256;
    const size_t nb = (n + block - 1) / block;
    auto* counts = static_cast<uint32_t*>(scratch);
    uint32_t* offsets = counts + nb;
    void* scan_scratch = static_cast<char*>(scratch) + blocks_bytes<T>(n);
    uint64_t sb = 0;
    hx_scratch_bytes(HX_SCRATCH_SCAN, nb, &sb);
    k_count_blocks<<<(unsigned)nb, block, 0, s>>>(in, n, rule, counts);
    hxcompat::check(hx_exclusive_scan_u32(counts, offsets, nb, scan_scratch, sb, s), "hx_exclusive_scan_u32");
    k_scatter_blocks<<<(unsigned)nb, block, 0, s>>>(in, n, rule, offsets, out, cap, cnt, count_max, nb, proj);
    hxcompat::check_cuda(cudaGetLastError(), "k_scatter_blocks");
  }
  if (owned) hxcompat::check_cuda(cudaFreeAsync(owned, s), "cudaFreeAsync");
}

// The same with the count read back on the host (synchronises the stream,
// as the reference's copy_if does). With caller scratch no allocation is made.
template <typename T, typename O, typename Rule, typename Proj>
size_t compact_sync(const T* in, O* out, size_t n, size_t cap, Rule rule, Proj proj, void* scratch, cudaStream_t s) {
  const size_t need = compaction_scratch_bytes<T>(n);
  void* owned = nullptr;
  if (!scratch) {
    hxcompat::check_cuda(cudaMallocAsync(&owned, need, s), "cudaMallocAsync");
    scratch = owned;
  }
  size_t* d = result_word<T>(scratch, n);
  compact(in, out, n, cap, rule, proj, d, ~(size_t)0, scratch, s);
  size_t h = 0;
  hxcompat::check_cuda(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
  if (owned) hxcompat::check_cuda(cudaFreeAsync(owned, s), "cudaFreeAsync");
  hxcompat::check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
  return h;
}

template <typename T>
constexpr int elem_bytes() {
  return (int)sizeof(T);
}

}  // namespace detail

/* splitStackArena (split_tools.h:491-535): a bump allocator over one device
 * buffer, either allocated stream-ordered (and freed with the arena) or
 * borrowed from the caller. The copy_if / copy_keys_if overloads that take
 * an arena or a (stack, max_size) buffer take their device scratch from it
 * and allocate nothing; like the reference's, the arena aborts with a message
 * when it has too little room (size it with estimateMemoryForCompaction). */
class splitStackArena {
  void* base_ = nullptr;
  size_t cap_ = 0, used_ = 0;
  cudaStream_t s_ = 0;
  bool owned_ = false;

 public:
  explicit splitStackArena(size_t bytes, cudaStream_t s) : cap_(bytes), s_(s), owned_(true) {
    hxcompat::check_cuda(cudaMallocAsync(&base_, bytes, s), "cudaMallocAsync");
  }
  explicit splitStackArena(void* ptr, size_t bytes) : base_(ptr), cap_(bytes) {}
  splitStackArena() = delete;
  splitStackArena(const splitStackArena&) = delete;
  splitStackArena(splitStackArena&&) = delete;
  ~splitStackArena() {
    if (owned_ && base_) cudaFreeAsync(base_, s_);
  }
  void* allocate(size_t bytes) {
    if (used_ + bytes > cap_) {
      std::fprintf(stderr, "splitStackArena: %zu bytes requested, %zu free\n", bytes, cap_ - used_);
      std::abort();
    }
    void* p = static_cast<char*>(base_) + used_;
    used_ += bytes;
    return p;
  }
  void deallocate(size_t bytes) { used_ -= bytes; }
  void reset() { used_ = 0; }
  const size_t& fill() const { return used_; }
  const size_t& capacity() const { return cap_; }
  size_t free_space() const { return cap_ - used_; }
};

/* estimateMemoryForCompaction (split_tools.h:1065-1090): the device scratch
 * that one compaction of inputSize elements takes from an arena here — enough
 * for libhx's descriptor rules and for a functor rule over elements of 4, 8
 * or 16 bytes (the typed form also covers its own element size). */
template <int BLOCKSIZE = 1024>
[[nodiscard]] size_t estimateMemoryForCompaction(const size_t inputSize) noexcept {
  uint64_t b = 0;
  const size_t lib = hx_scratch_bytes(HX_SCRATCH_COPY_IF, inputSize, &b) == HX_OK ? (size_t)b : 0;
  const size_t fun = detail::compaction_scratch_bytes<uint32_t>(inputSize);
  return ((std::max(lib, fun) + 255) / 256) * 256 + 256;  // + room to align the piece taken from an arena
}
template <typename T, int BLOCKSIZE = 1024>
[[nodiscard]] size_t estimateMemoryForCompaction(const SplitVector<T>& input) noexcept {
  const size_t n = input.size();
  return std::max(estimateMemoryForCompaction<BLOCKSIZE>(n),
                  ((detail::compaction_scratch_bytes<T>(n) + 255) / 256) * 256 + 256);
}

namespace detail {
// One compaction of `input` into `output` (a SplitVector), the count written
// into output's size word on the device (at most count_max), from `scratch`
// (or stream-ordered scratch when it is null). Rules are functors (the
// kernel here) or hx_pred descriptors (libhx, then the count is copied into
// the size word).
template <int = 0>  // a template, so that every translation unit may define it
__global__ void k_set_size(const unsigned long long* c, size_t* size_word, size_t count_max) {
  const unsigned long long v = *c;
  *size_word = v < count_max ? (size_t)v : count_max;
}
template <typename T, typename O, typename Rule, typename Proj>
void compact_into(const T* in, size_t n, O* out, size_t cap, Rule rule, Proj proj, size_t* size_word,
                  size_t count_max, void* scratch, size_t scratch_bytes, cudaStream_t s) {
  if constexpr (std::is_same<Rule, hx_pred>::value) {
    static_assert(std::is_same<T, O>::value, "descriptor rules copy whole elements: use a functor for keys");
    uint64_t need = 0;
    hxcompat::check(hx_scratch_bytes(HX_SCRATCH_COPY_IF, n, &need), "hx_scratch_bytes");
    void* owned = nullptr;
    if (!scratch) {
      hxcompat::check_cuda(cudaMallocAsync(&owned, need + 256, s), "cudaMallocAsync");
      scratch = owned;
    } else if (scratch_bytes < need + 256) {
      std::fprintf(stderr, "hashinator_compat: %zu scratch bytes given, %zu needed\n", scratch_bytes,
                   (size_t)need + 256);
      std::abort();
    }
    auto* c = reinterpret_cast<uint64_t*>(static_cast<char*>(scratch) + need);
    const hx_status st = hx_copy_if(in, out, n, elem_bytes<T>(), &rule, cap, c, nullptr, scratch, need, s);
    hxcompat::check(st, "hx_copy_if");
    k_set_size<><<<1, 1, 0, s>>>(reinterpret_cast<const unsigned long long*>(c), size_word, count_max);
    hxcompat::check_cuda(cudaGetLastError(), "k_set_size");
    if (owned) hxcompat::check_cuda(cudaFreeAsync(owned, s), "cudaFreeAsync");
  } else {
    if (scratch && scratch_bytes < compaction_scratch_bytes<T>(n)) {
      std::fprintf(stderr, "hashinator_compat: %zu scratch bytes given, %zu needed\n", scratch_bytes,
                   compaction_scratch_bytes<T>(n));
      std::abort();
    }
    compact(in, out, n, cap, rule, proj, size_word, count_max, scratch, s);
  }
}
// A 256-byte-aligned piece of `need` bytes from an arena (it takes need + 256).
inline void* take_aligned(splitStackArena& pool, size_t need) {
  const uintptr_t p = reinterpret_cast<uintptr_t>(pool.allocate(need + 256));
  return reinterpret_cast<void*>((p + 255) / 256 * 256);
}
// Bytes one compaction of n elements of T with this rule takes from an arena.
template <typename T, typename Rule>
inline size_t scratch_for(size_t n) {
  if constexpr (std::is_same<Rule, hx_pred>::value) {
    uint64_t need = 0;
    hx_scratch_bytes(HX_SCRATCH_COPY_IF, n, &need);
    return (size_t)need + 256;
  } else {
    return compaction_scratch_bytes<T>(n);
  }
}
// The loop forms' compaction: the input's size is read on the device (its
// capacity bounds it), output written into its capacity, its size set on the
// device; no host synchronisation. Descriptor rules and element sizes that
// do not divide 16 take the input's size as the host sees it.
template <typename T, class A, typename U, class B, typename Rule, typename Proj>
void compact_loop(SplitVector<T, A>& in, SplitVector<U, B>& out, Rule rule, Proj proj, cudaStream_t s) {
  constexpr bool single_pass = !std::is_same<Rule, hx_pred>::value && (16 % sizeof(T) == 0);
  if constexpr (single_pass) {
    const size_t nmax = in.capacity();
    if (nmax == 0 || !in.data()) {
      hxcompat::check_cuda(cudaMemsetAsync(out.size_word(), 0, sizeof(size_t), s), "cudaMemsetAsync");
      return;
    }
    void* sc = nullptr;
    hxcompat::check_cuda(cudaMallocAsync(&sc, compaction_scratch_bytes<T>(nmax), s), "cudaMallocAsync");
    hxs::Done done{reinterpret_cast<unsigned long long*>(out.size_word()), nullptr, nullptr};
    done.count_max = out.capacity();
    done.n_from = reinterpret_cast<const unsigned long long*>(in.size_word());
    hxcompat::check_cuda(hxs::launch<T, U, RuleSel<Rule>, false>(in.data(), out.data(), nmax, RuleSel<Rule>{rule},
                                                                out.capacity(), done, sc, s),
                         "single-pass compaction");
    hxcompat::check_cuda(cudaFreeAsync(sc, s), "cudaFreeAsync");
  } else {
    compact_into(in.data(), in.size(), out.data(), out.capacity(), rule, proj, out.size_word(), out.capacity(),
                 nullptr, 0, s);
  }
}
}  // namespace detail

/* copy_if(in, out, rule, stream) (split_tools.h:1129): out gets the selected
 * elements in order and is resized to their count (out must hold them, as in
 * the reference); blocks until done, as the reference does. One pass over
 * the input (hx_stream.cuh) for a functor rule, libhx for an hx_pred. */
template <typename T, class A, typename Rule>
void copy_if(SplitVector<T, A>& input, SplitVector<T, A>& output, Rule rule, cudaStream_t s = 0) {
  detail::compact_into(input.data(), input.size(), output.data(), output.size(), rule, detail::Identity{},
                       output.size_word(), output.size(), nullptr, 0, s);
  hxcompat::check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
}
/* copy_if(in, out, rule, splitStackArena&&, stream) (split_tools.h:1162)
 * and copy_if(in, out, rule, stack, max_size, stream) (:1194): the scratch
 * comes from the arena or the caller's buffer; nothing is allocated. */
template <typename T, class A, typename Rule>
void copy_if(SplitVector<T, A>& input, SplitVector<T, A>& output, Rule rule, splitStackArena&& pool,
             cudaStream_t s = 0) {
  const size_t need = detail::scratch_for<T, Rule>(input.size());
  void* sc = detail::take_aligned(pool, need);
  detail::compact_into(input.data(), input.size(), output.data(), output.size(), rule, detail::Identity{},
                       output.size_word(), output.size(), sc, need, s);
  hxcompat::check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
  pool.deallocate(need + 256);
}
template <typename T, class A, typename Rule>
void copy_if(SplitVector<T, A>& input, SplitVector<T, A>& output, Rule rule, void* stack, size_t max_size,
             cudaStream_t s = 0) {
  copy_if(input, output, rule, splitStackArena(stack, max_size), s);
}
/* copy_if(T* in, T* out, size, rule, stack, max_size, stream)
 * (split_tools.h:1211): returns the count; scratch from the caller's buffer. */
template <typename T, typename Rule>
size_t copy_if(T* input, T* output, size_t size, Rule rule, void* stack, size_t max_size, cudaStream_t s = 0) {
  splitStackArena pool(stack, max_size);
  void* sc = detail::take_aligned(pool, detail::compaction_scratch_bytes<T>(size));
  return detail::compact_sync(input, output, size, size, rule, detail::Identity{}, sc, s);
}

/* copy_keys_if(in, out, rule, stream) (split_tools.h:1095) and its arena
 * (:1147) and stack (:1177) forms: the keys of the selected hash_pairs, in
 * order; out must hold the result and is resized to the count. */
template <typename T, class A, typename U, class B, typename Rule>
void copy_keys_if(SplitVector<T, A>& input, SplitVector<U, B>& output, Rule rule, cudaStream_t s = 0) {
  detail::compact_into(input.data(), input.size(), output.data(), output.size(), rule, detail::KeyOf{},
                       output.size_word(), output.size(), nullptr, 0, s);
  hxcompat::check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
}
template <typename T, class A, typename U, class B, typename Rule>
void copy_keys_if(SplitVector<T, A>& input, SplitVector<U, B>& output, Rule rule, splitStackArena&& pool,
                  cudaStream_t s = 0) {
  const size_t need = detail::compaction_scratch_bytes<T>(input.size());
  void* sc = detail::take_aligned(pool, need);
  detail::compact_into(input.data(), input.size(), output.data(), output.size(), rule, detail::KeyOf{},
                       output.size_word(), output.size(), sc, need, s);
  hxcompat::check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
  pool.deallocate(need + 256);
}
template <typename T, class A, typename U, class B, typename Rule>
void copy_keys_if(SplitVector<T, A>& input, SplitVector<U, B>& output, Rule rule, void* stack, size_t max_size,
                  cudaStream_t s = 0) {
  copy_keys_if(input, output, rule, splitStackArena(stack, max_size), s);
}

/* copy_if_loop / copy_if_keys_loop (split_tools.h:997-1020, the single-block
 * loop_compact of :719-799): no host synchronisation — the input's size is
 * read on the device, the selected elements (or keys) are written into the
 * output's capacity, and the output's size is set on the device to their
 * count (at most the capacity). Scratch is stream-ordered. */
template <typename T, class A, typename Rule>
void copy_if_loop(SplitVector<T, A>& input, SplitVector<T, A>& output, Rule rule, cudaStream_t s = 0) {
  detail::compact_loop(input, output, rule, detail::Identity{}, s);
}
template <typename T, class A, typename U, class B, typename Rule>
void copy_if_keys_loop(SplitVector<T, A>& input, SplitVector<U, B>& output, Rule rule, cudaStream_t s = 0) {
  detail::compact_loop(input, output, rule, detail::KeyOf{}, s);
}

/* split_prefix_scan(in, out, stream) (split_tools.h:363): exclusive sum of
 * uint32_t, any length (the reference asserts a power of two). */
template <class A>
inline void split_prefix_scan(SplitVector<uint32_t, A>& input, SplitVector<uint32_t, A>& output,
                              cudaStream_t s = 0) {
  output.resize(input.size());
  hxcompat::check(hx_exclusive_scan_u32(input.data(), output.data(), input.size(), nullptr, 0, s),
                  "hx_exclusive_scan_u32");
  hxcompat::check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
}

}  // namespace tools
}  // namespace split

namespace Hashinator {

template <typename KEY_TYPE, typename VAL_TYPE, KEY_TYPE EMPTYBUCKET = std::numeric_limits<KEY_TYPE>::max(),
          KEY_TYPE TOMBSTONE = EMPTYBUCKET - 1>
class Hashmap {
  static_assert(std::is_same<KEY_TYPE, VAL_TYPE>::value &&
                    (std::is_same<KEY_TYPE, uint32_t>::value || std::is_same<KEY_TYPE, uint64_t>::value),
                "libhx serves hash_pair<uint32_t,uint32_t> and hash_pair<uint64_t,uint64_t>");
  // libhx's tables use the reference's default sentinels (EMPTY = all ones,
  // TOMBSTONE = EMPTY - 1). Other sentinels may be named, and
  // get_emptybucket() / get_tombstone() report them (the reference's
  // EMPTY_TOMBSTONE_values test), but every operation on the table goes
  // through map() or view(), whose static_assert rejects them at compile time.
  static constexpr bool kDefaultSentinels =
      EMPTYBUCKET == std::numeric_limits<KEY_TYPE>::max() && TOMBSTONE == EMPTYBUCKET - 1;
  using pair_t = hash_pair<KEY_TYPE, VAL_TYPE>;
  using view_t = hx_device::MapView<KEY_TYPE, VAL_TYPE>;
  hx_map* m_ = nullptr;
  hx_device_view dv_{};      // what the device copy works on (refreshed by upload())
  Hashmap* d_self_ = nullptr;  // the device copy that upload() returns

  hx_map* map() const {
    static_assert(kDefaultSentinels, "libhx operates only on tables with the default sentinels");
    return m_;
  }
  // The rule of extractLoop / extractAllKeys (hashinator.h:1195-1197, 1239-1241).
  using ValidKey = hxcompat::ValidKeyRule<hash_pair<KEY_TYPE, VAL_TYPE>, KEY_TYPE, EMPTYBUCKET, TOMBSTONE>;
  // extractKeysByPattern's body: the keys of the selected buckets into
  // `elements`, resized to the count; scratch from (stack, max_size) if given.
  template <typename Rule>
  size_t extract_keys(split::SplitVector<KEY_TYPE>& elements, Rule rule, void* stack, size_t max_size,
                      cudaStream_t s) {
    void* b = nullptr;
    uint64_t nb = 0;
    hxcompat::check(hx_bucket_data(map(), &b, &nb), "hx_bucket_data");
    elements.resize(nb);
    if constexpr (std::is_same<Rule, hx_pred>::value) {
      uint64_t h = 0;
      const hx_status st = hx_extract_keys(map(), &rule, elements.data(), nb, nullptr, &h, s);
      if (st != HX_OK && st != HX_ERR_CAPACITY) hxcompat::check(st, "hx_extract_keys");
      elements.erase(elements.data() + h, elements.end());
      return (size_t)h;
    } else {
      void* sc = nullptr;
      const size_t need = split::tools::detail::compaction_scratch_bytes<pair_t>((size_t)nb);
      if (stack) {
        split::tools::splitStackArena pool(stack, max_size);
        sc = split::tools::detail::take_aligned(pool, need);
      }
      split::tools::detail::compact(static_cast<const pair_t*>(b), elements.data(), (size_t)nb, (size_t)nb, rule,
                                    split::tools::detail::KeyOf{}, elements.size_word(), (size_t)nb, sc, s);
      sync(s);
      return elements.size();
    }
  }
  // The loop forms' body: into `elements`' capacity, its size set on the device.
  template <typename Rule, typename Proj, typename U>
  void loop_into(split::SplitVector<U>& elements, Rule rule, Proj proj, cudaStream_t s) {
    void* b = nullptr;
    uint64_t nb = 0;
    hxcompat::check(hx_bucket_data(map(), &b, &nb), "hx_bucket_data");
    split::tools::detail::compact_into(static_cast<const pair_t*>(b), (size_t)nb, elements.data(),
                                       elements.capacity(), rule, proj, elements.size_word(), elements.capacity(),
                                       nullptr, 0, s);
  }
  __host__ __device__ view_t view() const {
    static_assert(kDefaultSentinels, "libhx operates only on tables with the default sentinels");
    return view_t::from(dv_);
  }
  __device__ pair_t* dbuckets() const {
    static_assert(kDefaultSentinels, "libhx operates only on tables with the default sentinels");
    return static_cast<pair_t*>(dv_.buckets);
  }
  __device__ size_t dsize() const { return (size_t)1 << dv_.size_power; }
  __device__ static bool valid(KEY_TYPE k) { return k != EMPTYBUCKET && k != TOMBSTONE; }

  void sync(cudaStream_t s) const { hxcompat::check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize"); }
  hx_info info(cudaStream_t s = 0) const {
    hx_info i;
    hxcompat::check(hx_get_info(map(), &i, s), "hx_get_info");
    return i;
  }

 public:
  Hashmap() : Hashmap(5) {}  // Hashmap() starts at size power 5 (hashinator.h:109-118)
  explicit Hashmap(int sizepower) {
    hxcompat::check(hx_map_create(&m_, (int)sizeof(KEY_TYPE), (int)sizeof(VAL_TYPE), sizepower, nullptr),
                    "hx_map_create");
  }
  Hashmap(const Hashmap&) = delete;
  Hashmap& operator=(const Hashmap&) = delete;
  ~Hashmap() {
    if (d_self_) cudaFree(d_self_);
    if (m_) hx_map_destroy(m_);
  }

  // ---- accelerated API (hashinator.h:1262-1409) ----
  template <bool prefetches = true>
  void insert(KEY_TYPE* keys, VAL_TYPE* vals, size_t len, float targetLF = 0.5, cudaStream_t s = 0) {
    hxcompat::check(hx_insert(map(), keys, vals, len, targetLF, s), "hx_insert");
    sync(s);
  }
  template <bool prefetches = true>
  void insert(pair_t* src, size_t len, float targetLF = 0.5, cudaStream_t s = 0) {
    hxcompat::check(hx_insert_pairs(map(), src, len, targetLF, s), "hx_insert_pairs");
    sync(s);
  }
  template <bool prefetches = true>
  void retrieve(KEY_TYPE* keys, VAL_TYPE* vals, size_t len, cudaStream_t s = 0) {
    hxcompat::check(hx_retrieve(map(), keys, vals, len, s), "hx_retrieve");
    sync(s);
  }
  template <bool prefetches = true>
  void retrieve(pair_t* src, size_t len, cudaStream_t s = 0) {
    hxcompat::check(hx_retrieve_pairs(map(), src, len, s), "hx_retrieve_pairs");
    sync(s);
  }
  template <bool prefetches = true>
  void erase(KEY_TYPE* keys, size_t len, cudaStream_t s = 0) {
    hxcompat::check(hx_erase(map(), keys, len, s), "hx_erase");
    sync(s);
  }
  template <bool prefetches = true>
  void clean_tombstones(cudaStream_t s = 0) {
    hxcompat::check(hx_clean_tombstones(map(), s), "hx_clean_tombstones");
    sync(s);
  }
  template <bool prefetches = true>
  void device_rehash(int newSizePower, cudaStream_t s = 0) {
    hxcompat::check(hx_resize(map(), newSizePower, s), "hx_resize");
    sync(s);
  }
  void resize(int newSizePower, targets = targets::device, cudaStream_t s = 0) { device_rehash(newSizePower, s); }
  template <bool prefetches = true>
  void clear(targets = targets::device, cudaStream_t s = 0, size_t = 0) {
    hxcompat::check(hx_clear(map(), s), "hx_clear");
    sync(s);
  }

  /* insertIndex(keys, len, targetLF, s) (hashinator.h:1339): keys[i] -> i. */
  template <bool prefetches = true>
  void insertIndex(KEY_TYPE* keys, size_t len, float targetLF = 0.5, cudaStream_t s = 0) {
    hxcompat::check(hx_insert_index(map(), keys, len, targetLF, s), "hx_insert_index");
    sync(s);
  }
  /* resize_to_lf(targetLF, targets, s) (hashinator.h:530). */
  void resize_to_lf(float targetLF = 0.5, targets = targets::device, cudaStream_t s = 0) {
    hxcompat::check(hx_resize_to_lf(map(), targetLF, s), "hx_resize_to_lf");
  }
  /* performCleanupTasks(s) (hashinator.h:643). */
  template <bool prefetches = true>
  void performCleanupTasks(cudaStream_t s = 0) {
    hxcompat::check(hx_perform_cleanup_tasks(map(), s), "hx_perform_cleanup_tasks");
  }

  /* extractKeysByPattern(SplitVector<KEY>&, Rule, s) (hashinator.h:1199):
   * the keys of the buckets where the rule holds, in bucket order; blocks.
   * A functor rule runs the single-pass compaction in this translation unit
   * (one read of the buckets); an hx_pred runs inside libhx. */
  template <bool prefetches = true, typename Rule>
  size_t extractKeysByPattern(split::SplitVector<KEY_TYPE>& elements, Rule rule, cudaStream_t s = 0) {
    return extract_keys(elements, rule, nullptr, 0, s);
  }
  /* extractKeysByPattern(keys, rule, stack, max_size, s) (hashinator.h:1218):
   * the scratch comes from the caller's buffer; nothing is allocated. */
  template <bool prefetches = true, typename Rule>
  size_t extractKeysByPattern(split::SplitVector<KEY_TYPE>& elements, Rule rule, void* stack, size_t max_size,
                              cudaStream_t s = 0) {
    return extract_keys(elements, rule, stack, max_size, s);
  }
  /* extractAllKeys(SplitVector<KEY>&, s) (hashinator.h:1236) and its stack form (:1244). */
  template <bool prefetches = true>
  size_t extractAllKeys(split::SplitVector<KEY_TYPE>& elements, cudaStream_t s = 0) {
    return extract_keys(elements, ValidKey{}, nullptr, 0, s);
  }
  template <bool prefetches = true>
  size_t extractAllKeys(split::SplitVector<KEY_TYPE>& elements, void* stack, size_t max_size, cudaStream_t s = 0) {
    return extract_keys(elements, ValidKey{}, stack, max_size, s);
  }

  /* extractPattern(hash_pair*, Rule, stream) (hashinator.h:1168): bucket
   * order; the output must hold the result; returns the count (blocks). */
  template <typename Rule>
  size_t extractPattern(pair_t* elements, Rule rule, cudaStream_t s = 0) {
    void* b = nullptr;
    uint64_t nb = 0;
    hxcompat::check(hx_bucket_data(map(), &b, &nb), "hx_bucket_data");
    if constexpr (std::is_same<Rule, hx_pred>::value) {
      uint64_t c = 0;
      const hx_status st = hx_extract_pattern(map(), &rule, elements, nb, nullptr, &c, s);
      if (st != HX_OK && st != HX_ERR_CAPACITY) hxcompat::check(st, "hx_extract_pattern");
      return (size_t)c;
    } else {
      return split::tools::detail::compact_sync(static_cast<const pair_t*>(b), elements, (size_t)nb, (size_t)nb,
                                                rule, split::tools::detail::Identity{}, nullptr, s);
    }
  }
  /* extractPattern(SplitVector&, Rule, stream) (hashinator.h:1155): resized
   * to the count. */
  template <bool prefetches = true, typename Rule>
  size_t extractPattern(split::SplitVector<pair_t>& elements, Rule rule, cudaStream_t s = 0) {
    void* b = nullptr;
    uint64_t nb = 0;
    hxcompat::check(hx_bucket_data(map(), &b, &nb), "hx_bucket_data");
    elements.resize(nb);
    const size_t c = extractPattern(elements.data(), rule, s);
    elements.erase(elements.data() + c, elements.end());
    return c;
  }

  // ---- metadata (hashinator.h:434-457, 611, 228) ----
  status peek_status() {
    int32_t v = 0;
    hxcompat::check(hx_peek_status(map(), &v, nullptr), "hx_peek_status");
    return static_cast<status>(v);
  }
  int getSizePower() const { return info().size_power; }
  size_t size() const { return info().fill; }
  size_t bucket_count() const { return info().bucket_count; }
  size_t tombstone_count() const { return info().tombstone_counter; }
  float load_factor() const {
    const hx_info i = info();
    return (float)i.fill / (float)i.bucket_count;
  }
  constexpr KEY_TYPE get_emptybucket() const { return EMPTYBUCKET; }
  constexpr KEY_TYPE get_tombstone() const { return TOMBSTONE; }
  void copyMetadata(Info* dst, cudaStream_t s = 0) {
    const hx_info i = info(s);
    *dst = Info{i.size_power, i.fill, i.current_max_bucket_overflow, i.tombstone_counter,
                static_cast<status>(i.err)};
  }
  template <bool warn = true>
  pair_t* expose_bucketdata() {
    void* b = nullptr;
    hxcompat::check(hx_bucket_data(map(), &b, nullptr), "hx_bucket_data");
    return static_cast<pair_t*>(b);
  }
  void optimizeGPU(cudaStream_t = 0) {}
  void optimizeCPU(cudaStream_t = 0) {}
  // The table is device resident, so unified-memory advice and stream
  // attachment (hashinator.h:1129, 1440) have nothing to act on.
  void memAdvise(cudaMemoryAdvise, int, cudaStream_t = 0) {}
  void streamAttach(cudaStream_t, uint32_t = cudaMemAttachSingle) {}
  hx_map* handle() { return map(); }

  /* rehash(newSizePower) (hashinator.h:236): the same result as
   * device_rehash — every valid pair in a table of 2^newSizePower buckets. */
  void rehash(int newSizePower) { device_rehash(newSizePower); }
  /* tombstone_ratio() (hashinator.h:614). */
  float tombstone_ratio() const {
    const hx_info i = info();
    return i.tombstone_counter ? (float)i.tombstone_counter / (float)i.bucket_count : 0.0f;
  }
  /* swap(other) (hashinator.h:622): exchanges the two tables. */
  void swap(Hashmap& other) noexcept {
    std::swap(m_, other.m_);
    std::swap(dv_, other.dv_);
    std::swap(d_self_, other.d_self_);
  }
  /* stats() and dump_buckets() (hashinator.h:591-611): metadata, and every
   * bucket with its distance from home, printed on the host. */
  void stats() const {
    const hx_info i = info();
    std::printf("Hashmap: 2^%d buckets, fill %llu (load factor %.4f), tombstones %llu, probe bound %llu\n",
                i.size_power, (unsigned long long)i.fill, (double)i.fill / (double)i.bucket_count,
                (unsigned long long)i.tombstone_counter, (unsigned long long)i.current_max_bucket_overflow);
  }
  void dump_buckets() const {
    stats();
    void* b = nullptr;
    uint64_t nb = 0;
    hxcompat::check(hx_bucket_data(map(), &b, &nb), "hx_bucket_data");
    std::vector<pair_t> h(nb);
    hxcompat::check_cuda(cudaMemcpy(h.data(), b, nb * sizeof(pair_t), cudaMemcpyDeviceToHost), "cudaMemcpy");
    const int sp = getSizePower();
    for (uint64_t j = 0; j < nb; ++j) {
      const KEY_TYPE k = h[j].first;
      if (k == EMPTYBUCKET) {
        std::printf(". ");
      } else if (k == TOMBSTONE) {
        std::printf("x ");
      } else {
        const uint64_t home = (uint64_t)hx_device::home(k, sp);
        std::printf("(%llu,%llu,+%llu) ", (unsigned long long)k, (unsigned long long)h[j].second,
                    (unsigned long long)((j - home) & (nb - 1)));
      }
    }
    std::printf("\n");
  }

  /* The single-block "loop" extractions (hashinator.h:1187-1260): no host
   * synchronisation. The selection is written into `elements`' capacity and
   * its size is set on the device to the count (at most the capacity), as
   * the reference's loop_compact does; read elements.size() after the stream
   * has finished. Scratch is stream-ordered. */
  template <typename Rule>
  void extractPatternLoop(split::SplitVector<pair_t>& elements, Rule rule, cudaStream_t s = 0) {
    loop_into(elements, rule, split::tools::detail::Identity{}, s);
  }
  void extractLoop(split::SplitVector<pair_t>& elements, cudaStream_t s = 0) {
    loop_into(elements, ValidKey{}, split::tools::detail::Identity{}, s);
  }
  template <typename Rule>
  void extractKeysByPatternLoop(split::SplitVector<KEY_TYPE>& elements, Rule rule, cudaStream_t s = 0) {
    loop_into(elements, rule, split::tools::detail::KeyOf{}, s);
  }
  void extractAllKeysLoop(split::SplitVector<KEY_TYPE>& elements, cudaStream_t s = 0) {
    loop_into(elements, ValidKey{}, split::tools::detail::KeyOf{}, s);
  }

  // ---- device API (hashinator.h:853-1126, 1417-1769) ----
  /* upload(s) (hashinator.h:1417): a device copy of this map for kernels;
   * call it again after any host call that may reallocate the table. */
  template <bool prefetches = true>
  Hashmap* upload(cudaStream_t s = 0) {
    hxcompat::check(hx_map_device_view(map(), &dv_), "hx_map_device_view");
    if (!d_self_) hxcompat::check_cuda(cudaMalloc(&d_self_, sizeof(Hashmap)), "cudaMalloc");
    hxcompat::check_cuda(cudaMemcpyAsync(d_self_, this, sizeof(Hashmap), cudaMemcpyHostToDevice, s),
                         "cudaMemcpyAsync");
    sync(s);
    return d_self_;
  }
  Hashmap* get_device_pointer() { return d_self_; }
  /* download(s) (hashinator.h:1458): after device-side work, grow if the probe
   * bound passed one 32-bucket window, else drop tombstones. */
  void download(cudaStream_t s = 0) {
    const hx_info i = info(s);
    if (i.current_max_bucket_overflow > 32) {
      device_rehash(i.size_power + 1, s);
    } else if (i.tombstone_counter > 0) {
      clean_tombstones(s);
    }
  }

  /* device_iterator (hashinator.h:1470): walks the valid buckets. */
  template <bool CONST>
  class iterator_t {
    using map_t = typename std::conditional<CONST, const Hashmap, Hashmap>::type;
    using ref_t = typename std::conditional<CONST, const pair_t&, pair_t&>::type;
    using ptr_t = typename std::conditional<CONST, const pair_t*, pair_t*>::type;
    size_t index = 0;
    map_t* table = nullptr;

   public:
    __device__ iterator_t() {}
    __device__ iterator_t(map_t& t, size_t i) : index(i), table(&t) {}
    __device__ size_t getIndex() { return index; }
    __device__ iterator_t& operator++() {
      ++index;
      while (index < table->dsize() && !valid(table->dbuckets()[index].first)) ++index;
      return *this;
    }
    __device__ iterator_t operator++(int) {
      iterator_t t = *this;
      ++(*this);
      return t;
    }
    __device__ bool operator==(iterator_t o) const { return table == o.table && index == o.index; }
    __device__ bool operator!=(iterator_t o) const { return !(*this == o); }
    __device__ ref_t operator*() const { return table->dbuckets()[index]; }
    __device__ ptr_t operator->() const { return &table->dbuckets()[index]; }
  };
  using device_iterator = iterator_t<false>;
  using const_device_iterator = iterator_t<true>;

  __device__ device_iterator device_end() { return device_iterator(*this, dsize()); }
  __device__ const_device_iterator device_end() const { return const_device_iterator(*this, dsize()); }
  __device__ device_iterator device_begin() {
    size_t i = 0;
    while (i < dsize() && !valid(dbuckets()[i].first)) ++i;
    return device_iterator(*this, i);
  }
  __device__ const_device_iterator device_begin() const {
    size_t i = 0;
    while (i < dsize() && !valid(dbuckets()[i].first)) ++i;
    return const_device_iterator(*this, i);
  }
  __device__ device_iterator device_find(KEY_TYPE key) {
    const int64_t i = view().device_find(key);
    return i < 0 ? device_end() : device_iterator(*this, (size_t)i);
  }
  __device__ const_device_iterator device_find(KEY_TYPE key) const {
    const int64_t i = view().device_find(key);
    return i < 0 ? device_end() : const_device_iterator(*this, (size_t)i);
  }
  __device__ size_t device_count(const KEY_TYPE& key) const { return view().device_count(key); }
  __device__ size_t device_erase(const KEY_TYPE& key) { return view().device_erase(key); }
  /* device_erase(iterator) (hashinator.h:1673): tombstone the bucket, return
   * the next valid one. */
  __device__ device_iterator device_erase(device_iterator pos) {
    pair_t* b = &dbuckets()[pos.getIndex()];
    const KEY_TYPE item = b->first;
    if (valid(item) && view().cas_key(reinterpret_cast<typename view_t::Bucket*>(b), item, TOMBSTONE)) {
      atomicAdd(dv_.fill, 0ull - 1ull);
      atomicAdd(dv_.tombstones, 1ull);
    }
    return ++pos;
  }
  template <bool skipOverWrites = false>
  __device__ bool set_element(const KEY_TYPE& key, VAL_TYPE val) {
    return view().template set_element<skipOverWrites>(key, val);
  }
  template <bool skipOverWrites = false>
  __device__ hash_pair<device_iterator, bool> device_insert(hash_pair<KEY_TYPE, VAL_TYPE> e) {
    const bool n = set_element<skipOverWrites>(e.first, e.second);
    return hash_pair<device_iterator, bool>(device_find(e.first), n);
  }
  /* read_element (hashinator.h:1750): the reference asserts on a missing key;
   * here the map's status becomes fail and a zero is returned. */
  __device__ const VAL_TYPE& read_element(const KEY_TYPE& key) const {
    const int64_t i = view().device_find(key);
    if (i >= 0) return dbuckets()[i].second;
    atomicExch(dv_.err, HX_STATUS_FAIL);
    return missing_value();
  }
  template <bool skipOverWrites = false>
  __device__ void warpInsert(const KEY_TYPE& key, const VAL_TYPE& val, const size_t w_tid) {
    view().template warp_insert<skipOverWrites>(key, val, (int)w_tid);
  }
  template <bool skipOverWrites = false>
  __device__ bool warpInsert_V(const KEY_TYPE& key, const VAL_TYPE& val, const size_t w_tid) {
    return view().template warp_insert<skipOverWrites>(key, val, (int)w_tid);
  }
  __device__ void warpFind(const KEY_TYPE& key, VAL_TYPE& val, const size_t w_tid) const {
    view().warp_find(key, val, (int)w_tid);
  }
  __device__ void warpErase(const KEY_TYPE& key, const size_t w_tid) { view().warp_erase(key, (int)w_tid); }

 private:
  __device__ static const VAL_TYPE& missing_value() {
    static VAL_TYPE zero = 0;
    return zero;
  }
};

}  // namespace Hashinator
