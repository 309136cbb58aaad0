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

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <limits>
#include <type_traits>
#include <utility>
#include <vector>

#include "hx.h"
#include "hx_device_api.cuh"

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

/* Managed-memory vector (the reference's default allocator is
 * cudaMallocManaged, split_allocators.h:62-129), with the subset of the
 * SplitVector surface the accelerated API and its tests use. */
template <typename T>
class SplitVector {
  T* d_ = nullptr;
  size_t size_ = 0, cap_ = 0;

  void reallocate(size_t cap) {
    T* p = nullptr;
    if (cap) hxcompat::check_cuda(cudaMallocManaged(&p, cap * sizeof(T)), "cudaMallocManaged");
    if (d_) {
      hxcompat::check_cuda(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
      for (size_t i = 0; i < size_ && i < cap; ++i) p[i] = d_[i];
      cudaFree(d_);
    }
    d_ = p;
    cap_ = cap;
  }

 public:
  using value_type = T;
  using iterator = T*;
  using const_iterator = const T*;
  SplitVector() = default;
  explicit SplitVector(size_t n) { resize(n); }
  SplitVector(size_t n, const T& v) {
    resize(n);
    for (size_t i = 0; i < n; ++i) d_[i] = v;
  }
  SplitVector(const SplitVector& o) {
    reserve(o.size_);
    hxcompat::check_cuda(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
    for (size_t i = 0; i < o.size_; ++i) d_[i] = o.d_[i];
    size_ = o.size_;
  }
  SplitVector& operator=(const SplitVector& o) {
    if (this != &o) {
      resize(o.size_);
      hxcompat::check_cuda(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
      for (size_t i = 0; i < o.size_; ++i) d_[i] = o.d_[i];
    }
    return *this;
  }
  ~SplitVector() {
    if (d_) cudaFree(d_);
  }
  T* data() { return d_; }
  const T* data() const { return d_; }
  size_t size() const { return size_; }
  size_t capacity() const { return cap_; }
  bool empty() const { return size_ == 0; }
  void reserve(size_t n) {
    if (n > cap_) reallocate(n);
  }
  void resize(size_t n, bool /*eco*/ = false) {
    reserve(n);
    size_ = n;
  }
  void clear() { size_ = 0; }
  void push_back(const T& v) {
    if (size_ == cap_) reallocate(cap_ ? 2 * cap_ : 8);
    d_[size_++] = v;
  }
  T& operator[](size_t i) { return d_[i]; }
  const T& operator[](size_t i) const { return d_[i]; }
  T& at(size_t i) { return d_[i]; }
  T* begin() { return d_; }
  T* end() { return d_ + size_; }
  const T* begin() const { return d_; }
  const T* end() const { return d_ + size_; }
  void erase(T* first, T* last) {  // erase(range) (splitvec.h:1499): only the tail form is used
    if (last == end()) size_ = (size_t)(first - d_);
  }
  void optimizeGPU(cudaStream_t = 0) {}
  void optimizeCPU(cudaStream_t = 0) {}
};

namespace tools {
namespace detail {

template <typename T, typename Rule>
__global__ void count_tiles(const T* in, size_t n, Rule rule, uint32_t* counts) {
  __shared__ uint32_t s;
  if (threadIdx.x == 0) s = 0;
  __syncthreads();
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  bool sel = false;
  if (i < n) {
    T x = in[i];
    sel = rule(x);
  }
  const unsigned b = __ballot_sync(0xffffffffu, sel);
  if ((threadIdx.x & 31) == 0 && b) atomicAdd(&s, (uint32_t)__popc(b));
  __syncthreads();
  if (threadIdx.x == 0) counts[blockIdx.x] = s;
}

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

template <typename T, typename O, typename Rule, typename Proj>
__global__ void scatter_tiles(const T* in, size_t n, Rule rule, const uint32_t* offsets, O* out, size_t cap,
                              unsigned long long* total, size_t nblocks, Proj proj) {
  __shared__ uint32_t warp_base[32];
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  bool sel = false;
  T x;
  if (i < n) {
    x = in[i];
    sel = rule(x);
  }
  const unsigned b = __ballot_sync(0xffffffffu, sel);
  if (lane == 0) warp_base[warp] = __popc(b);
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t acc = 0;
    for (unsigned w = 0; w < blockDim.x / 32; ++w) {
      const uint32_t c = warp_base[w];
      warp_base[w] = acc;
      acc += c;
    }
    if (blockIdx.x == nblocks - 1) *total = (unsigned long long)offsets[blockIdx.x] + acc;
  }
  __syncthreads();
  if (sel) {
    const size_t dst = (size_t)offsets[blockIdx.x] + warp_base[warp] + __popc(b & ((1u << lane) - 1u));
    if (dst < cap) out[dst] = proj(x);
  }
}

// Stable compaction with a user functor: per-block counts, libhx exclusive
// scan of the counts, order-preserving scatter of proj(x) (the element, or
// the key of a bucket pair).
template <typename T, typename O, typename Rule, typename Proj>
size_t copy_if_functor(const T* in, O* out, size_t n, size_t cap, Rule rule, Proj proj, cudaStream_t s) {
  if (n == 0) return 0;
  const unsigned block = 256;
  const size_t nb = (n + block - 1) / block;
  uint32_t* counts = nullptr;
  unsigned long long* total = nullptr;
  hxcompat::check_cuda(cudaMallocAsync(&counts, 2 * nb * sizeof(uint32_t) + 16, s), "cudaMallocAsync");
  uint32_t* offsets = counts + nb;
  total = reinterpret_cast<unsigned long long*>(counts + 2 * nb);  // 8-byte aligned: 2*nb words
  count_tiles<<<(unsigned)nb, block, 0, s>>>(in, n, rule, counts);
  hxcompat::check(hx_exclusive_scan_u32(counts, offsets, nb, nullptr, 0, s), "hx_exclusive_scan_u32");
  scatter_tiles<<<(unsigned)nb, block, 0, s>>>(in, n, rule, offsets, out, cap, total, nb, proj);
  unsigned long long h = 0;
  hxcompat::check_cuda(cudaMemcpyAsync(&h, total, sizeof(h), cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
  hxcompat::check_cuda(cudaFreeAsync(counts, s), "cudaFreeAsync");
  hxcompat::check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
  return (size_t)h;
}

template <typename T>
constexpr int elem_bytes() {
  return (int)sizeof(T);
}

}  // namespace detail

/* copy_if(in, out, rule, stream) (split_tools.h:1129): out gets the selected
 * elements in order and is resized to their count. */
template <typename T, typename Rule>
void copy_if(SplitVector<T>& input, SplitVector<T>& output, Rule rule, cudaStream_t s = 0) {
  size_t c;
  if constexpr (std::is_same<Rule, hx_pred>::value) {
    uint64_t h = 0;
    const hx_status st = hx_copy_if(input.data(), output.data(), input.size(), detail::elem_bytes<T>(), &rule,
                                    output.size(), nullptr, &h, nullptr, 0, s);
    if (st != HX_OK && st != HX_ERR_CAPACITY) hxcompat::check(st, "hx_copy_if");
    c = (size_t)h;
  } else {
    c = detail::copy_if_functor(input.data(), output.data(), input.size(), output.size(), rule, detail::Identity{},
                                s);
  }
  output.erase(output.data() + (c < output.size() ? c : output.size()), output.end());
}

/* copy_if(T* in, T* out, size, rule, stack, max_size, stream)
 * (split_tools.h:1211): returns the count. */
template <typename T, typename Rule>
size_t copy_if(T* input, T* output, size_t size, Rule rule, void* /*stack*/, size_t /*max_size*/, cudaStream_t s = 0) {
  return detail::copy_if_functor(input, output, size, size, rule, detail::Identity{}, s);
}

/* splitStackArena (split_tools.h:491-535): a bump allocator over one device
 * buffer, either allocated stream-ordered (and freed with the arena) or
 * borrowed from the caller. libhx's compaction takes its scratch from the
 * device's stream-ordered pool itself, so the copy_if / copy_keys_if
 * overloads below accept an arena or a (stack, max_size) buffer for source
 * compatibility and leave it untouched. */
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
 * that libhx's compaction of inputSize elements uses (hx_scratch_bytes). */
template <int BLOCKSIZE = 1024>
[[nodiscard]] size_t estimateMemoryForCompaction(const size_t inputSize) noexcept {
  uint64_t b = 0;
  return hx_scratch_bytes(HX_SCRATCH_COPY_IF, inputSize, &b) == HX_OK ? (size_t)b : 0;
}
template <typename T, int BLOCKSIZE = 1024>
[[nodiscard]] size_t estimateMemoryForCompaction(const SplitVector<T>& input) noexcept {
  return estimateMemoryForCompaction<BLOCKSIZE>(input.size());
}

/* copy_if(in, out, rule, splitStackArena&&, stream) (split_tools.h:1162)
 * and copy_if(in, out, rule, stack, max_size, stream) (:1194). */
template <typename T, typename Rule>
void copy_if(SplitVector<T>& input, SplitVector<T>& output, Rule rule, splitStackArena&& /*mPool*/,
             cudaStream_t s = 0) {
  copy_if(input, output, rule, s);
}
template <typename T, typename Rule>
void copy_if(SplitVector<T>& input, SplitVector<T>& output, Rule rule, void* /*stack*/, size_t /*max_size*/,
             cudaStream_t s = 0) {
  copy_if(input, output, rule, s);
}

/* copy_keys_if(in, out, rule, stream) (split_tools.h:1095) and its arena
 * (:1147) and stack (:1177) forms: the keys of the selected hash_pairs, in
 * order; out must hold the result and is resized to the count. The rule is
 * a functor over the pair. */
template <typename T, typename U, typename Rule>
void copy_keys_if(SplitVector<T>& input, SplitVector<U>& output, Rule rule, cudaStream_t s = 0) {
  const size_t c = detail::copy_if_functor(input.data(), output.data(), input.size(), output.size(), rule,
                                           detail::KeyOf{}, s);
  output.erase(output.data() + (c < output.size() ? c : output.size()), output.end());
}
template <typename T, typename U, typename Rule>
void copy_keys_if(SplitVector<T>& input, SplitVector<U>& output, Rule rule, splitStackArena&& /*mPool*/,
                  cudaStream_t s = 0) {
  copy_keys_if(input, output, rule, s);
}
template <typename T, typename U, typename Rule>
void copy_keys_if(SplitVector<T>& input, SplitVector<U>& output, Rule rule, void* /*stack*/, size_t /*max_size*/,
                  cudaStream_t s = 0) {
  copy_keys_if(input, output, rule, s);
}

/* copy_if_loop / copy_if_keys_loop (split_tools.h:995-1020): the reference's
 * single-block compactions, which write into the output's capacity and set
 * its size on the device. Here they run copy_if / copy_keys_if into the
 * output's capacity and set its size on the host; the elements and the size
 * are the same once the stream has finished. */
template <typename T, typename Rule>
void copy_if_loop(SplitVector<T>& input, SplitVector<T>& output, Rule rule, cudaStream_t s = 0) {
  output.resize(output.capacity());
  copy_if(input, output, rule, s);
}
template <typename T, typename U, typename Rule>
void copy_if_keys_loop(SplitVector<T>& input, SplitVector<U>& output, Rule rule, cudaStream_t s = 0) {
  output.resize(output.capacity());
  copy_keys_if(input, output, rule, s);
}

/* split_prefix_scan(in, out, stream) (split_tools.h:363): exclusive sum of
 * uint32_t, any length (the reference asserts a power of two). */
inline void split_prefix_scan(SplitVector<uint32_t>& input, SplitVector<uint32_t>& output, cudaStream_t s = 0) {
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
   * the keys of the buckets where the rule holds, in bucket order. */
  template <bool prefetches = true, typename Rule>
  size_t extractKeysByPattern(split::SplitVector<KEY_TYPE>& elements, Rule rule, cudaStream_t s = 0) {
    void* b = nullptr;
    uint64_t nb = 0;
    hxcompat::check(hx_bucket_data(map(), &b, &nb), "hx_bucket_data");
    elements.resize(nb);
    size_t c;
    if constexpr (std::is_same<Rule, hx_pred>::value) {
      uint64_t h = 0;
      const hx_status st = hx_extract_keys(map(), &rule, elements.data(), nb, nullptr, &h, s);
      if (st != HX_OK && st != HX_ERR_CAPACITY) hxcompat::check(st, "hx_extract_keys");
      c = (size_t)h;
    } else {
      c = split::tools::detail::copy_if_functor(static_cast<pair_t*>(b), elements.data(), nb, nb, rule,
                                                split::tools::detail::KeyOf{}, s);
    }
    elements.erase(elements.data() + c, elements.end());
    return c;
  }
  template <bool prefetches = true, typename Rule>
  size_t extractKeysByPattern(split::SplitVector<KEY_TYPE>& elements, Rule rule, void* /*stack*/,
                              size_t /*max_size*/, cudaStream_t s = 0) {
    return extractKeysByPattern<prefetches>(elements, rule, s);
  }
  /* extractAllKeys(SplitVector<KEY>&, s) (hashinator.h:1224). */
  template <bool prefetches = true>
  size_t extractAllKeys(split::SplitVector<KEY_TYPE>& elements, cudaStream_t s = 0) {
    hx_pred p{HX_PRED_VALID, HX_FIELD_KEY, 0, 0, 0, 0};
    return extractKeysByPattern<prefetches>(elements, p, s);
  }
  template <bool prefetches = true>
  size_t extractAllKeys(split::SplitVector<KEY_TYPE>& elements, void* /*stack*/, size_t /*max_size*/,
                        cudaStream_t s = 0) {
    return extractAllKeys<prefetches>(elements, s);
  }

  /* extractPattern(hash_pair*, Rule, stream) (hashinator.h:1168): bucket
   * order; the output must hold the result. */
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
      return split::tools::detail::copy_if_functor(static_cast<pair_t*>(b), elements, nb, nb, rule,
                                                   split::tools::detail::Identity{}, s);
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

  /* The single-block "loop" extractions (hashinator.h:1187-1260) keep their
   * count on the device in the reference; here they run the same selection
   * as extractPattern / extractKeysByPattern and size `elements` on the
   * host, so the elements are the same once the stream has finished. */
  template <typename Rule>
  void extractPatternLoop(split::SplitVector<pair_t>& elements, Rule rule, cudaStream_t s = 0) {
    extractPattern(elements, rule, s);
  }
  void extractLoop(split::SplitVector<pair_t>& elements, cudaStream_t s = 0) {
    extractPattern(elements, hx_pred{HX_PRED_VALID, HX_FIELD_KEY, 0, 0, 0, 0}, s);
  }
  template <typename Rule>
  void extractKeysByPatternLoop(split::SplitVector<KEY_TYPE>& elements, Rule rule, cudaStream_t s = 0) {
    extractKeysByPattern(elements, rule, s);
  }
  void extractAllKeysLoop(split::SplitVector<KEY_TYPE>& elements, cudaStream_t s = 0) { extractAllKeys(elements, s); }

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
