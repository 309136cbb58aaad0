// The device-side SplitVector surface of the drop-in header, and its
// compactions with caller scratch:
//   the reference's own device tests (gtest_vec_device/vec_test.cu):
//     VectorAddition :77-93, Resizing_Device :430-466, Insert_Device :399-410,
//     Insert_Device_N :412-421, PushBack_And_Erase_Device :388-397,
//     Test_CopyMetaData :468-481
//   concurrent device_push_back (both overloads) against a host model of the
//     reference's rule (splitvec.h:1070-1100): at most capacity - 1 elements,
//     the element multiset equal to the set of pushes that returned true
//   device_insert(it, val) in the middle (splitvec.h:1394-1420)
//   the preallocated compactions of stream_compaction/preallocated.cu:225-303:
//     many vectors compacted from several host threads on several streams,
//     each call's scratch taken from its slice of one caller buffer; the
//     device's default stream-ordered pool must see no allocation meanwhile
//   copy_if_loop on a vector filled on the device, without a host
//     synchronisation between (the size is read on the device)
//   functor copy_if against libhx's descriptor copy_if on 2^22 elements, and
//     on an input that does not start on a 16-byte boundary
// A tiny harness stands in for gtest (not installed). Exit code 0 = all pass.
#include <algorithm>
#include <array>
#include <cstdio>
#include <set>
#include <thread>
#include <vector>

#include "hashinator_compat.h"

static int g_fail = 0;
#define EXPECT_TRUE(c)                                                   \
  do {                                                                   \
    if (!(c)) {                                                          \
      std::printf("FAIL %s:%d: %s\n", __FILE__, __LINE__, #c);           \
      ++g_fail;                                                          \
    }                                                                    \
  } while (0)

typedef split::SplitVector<int, split::split_unified_allocator<int>> vec;

__global__ void add_vectors(vec* a, vec* b, vec* c) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < (int)a->size()) c->at(i) = a->at(i) + b->at(i);
}
__global__ void resize_vector(vec* a, int size) { a->device_resize(size); }
__global__ void push_back_kernel(vec* a) { a->device_push_back(blockIdx.x * blockDim.x + threadIdx.x); }
__global__ void merge_kernel(vec* a, vec* b) {
  if (blockIdx.x * blockDim.x + threadIdx.x == 0) a->device_insert(a->end(), b->begin(), b->end());
}
__global__ void merge_kernel_2(vec* a) {
  if (blockIdx.x * blockDim.x + threadIdx.x == 0) a->device_insert(a->begin()++, 3, 42);
}
__global__ void erase_kernel(vec* a) { a->erase(a->begin()); }
__global__ void insert_one(vec* a, int index, int v) { a->device_insert(a->begin() + index, v); }

static void test_reference_device_tests() {
  {  // VectorAddition
    const int N = 1 << 12;
    vec a(N, 1), b(N, 2), c(N, 0);
    vec* da = a.upload();
    vec* db = b.upload();
    vec* dc = c.upload();
    add_vectors<<<N, 32>>>(da, db, dc);
    cudaDeviceSynchronize();
    bool ok = true;
    for (const auto& e : c) ok = ok && e == 3;
    EXPECT_TRUE(ok);
  }
  {  // Resizing_Device
    vec a(32, 42);
    EXPECT_TRUE(a.size() == a.capacity());
    a.resize(16);
    EXPECT_TRUE(a.size() == 16 && a.capacity() == 32);
  }
  {
    vec a(32, 42);
    vec* da = a.upload();
    resize_vector<<<1, 1>>>(da, 16);
    cudaDeviceSynchronize();
    EXPECT_TRUE(a.size() == 16 && a.capacity() == 32);
  }
  {
    vec a(32, 42);
    a.reserve(100);
    EXPECT_TRUE(a.capacity() > 100);
    vec* da = a.upload();
    resize_vector<<<1, 1>>>(da, 64);
    cudaDeviceSynchronize();
    EXPECT_TRUE(a.size() == 64 && a.capacity() > 100);
    bool ok = true;
    for (size_t i = 0; i < 32; ++i) ok = ok && a.at(i) == 42;
    for (size_t i = 32; i < 64; ++i) ok = ok && a.at(i) == 0;  // device_resize constructs the new elements
    EXPECT_TRUE(ok);
  }
  {  // Insert_Device
    vec a{1, 2, 3, 4};
    a.reserve(20);
    vec b{5, 6, 7, 8};
    vec* da = a.upload();
    vec* db = b.upload();
    merge_kernel<<<1, 1>>>(da, db);
    cudaDeviceSynchronize();
    merge_kernel<<<1, 1>>>(da, db);
    cudaDeviceSynchronize();
    EXPECT_TRUE(a.size() == 12);
    const int want[12] = {1, 2, 3, 4, 5, 6, 7, 8, 5, 6, 7, 8};
    bool ok = true;
    for (int i = 0; i < 12; ++i) ok = ok && a[i] == want[i];
    EXPECT_TRUE(ok);
  }
  {  // Insert_Device_N
    vec a{0, 1, 2, 3, 4, 5, 6, 7, 8, 9};
    vec b{0, 1, 2, 3, 42, 42, 42, 4, 5, 6, 7, 8, 9};
    a.reserve(30);
    vec* da = a.upload();
    merge_kernel_2<<<1, 1>>>(da);
    cudaDeviceSynchronize();
    EXPECT_TRUE(a == b);
  }
  {  // PushBack_And_Erase_Device: reserve on a default-constructed vector allocates exactly 100 (size 0);
     // 32 device pushes fit; erase then drops the first element
    vec a;
    a.reserve(100);
    EXPECT_TRUE(a.size() == 0 && a.capacity() == 100);
    vec* da = a.upload();
    push_back_kernel<<<4, 8>>>(da);
    cudaDeviceSynchronize();
    EXPECT_TRUE(a.size() == 32);
    std::set<int> got(a.begin(), a.end()), want;
    for (int i = 0; i < 32; ++i) want.insert(i);
    EXPECT_TRUE(got == want);
    vec* db = a.upload();
    erase_kernel<<<1, 1>>>(db);
    cudaDeviceSynchronize();
    EXPECT_TRUE(a.size() == 31);
  }
  {  // Test_CopyMetaData
    vec a(32, 42);
    a.resize(16);
    split::SplitInfo* info = nullptr;
    cudaMallocHost(&info, sizeof(split::SplitInfo));
    a.copyMetadata(info);
    cudaDeviceSynchronize();
    EXPECT_TRUE(info->capacity == 32 && info->size == 16);
    cudaFreeHost(info);
  }
  {  // device_insert(it, val) in the middle
    vec a{10, 11, 12, 13};
    a.reserve(8);
    vec* da = a.upload();
    insert_one<<<1, 1>>>(da, 2, 99);
    cudaDeviceSynchronize();
    vec want{10, 11, 99, 12, 13};
    EXPECT_TRUE(a == want);
  }
}

typedef split::SplitVector<uint32_t> u32vec;
__global__ void push_many(u32vec* v, uint32_t n, uint8_t* ok, int moved) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  bool r;
  if (moved) {
    uint32_t x = i;
    r = v->device_push_back(std::move(x));
  } else {
    r = v->device_push_back(i);
  }
  ok[i] = r ? 1 : 0;
}

// Concurrent pushes from 2^16 + 5000 threads into capacity 2^16: exactly
// capacity - 1 succeed; the stored elements are exactly the successful pushes.
static void test_concurrent_push_back() {
  for (int moved = 0; moved < 2; ++moved) {
    const uint32_t cap = 1u << 16, n = cap + 5000;
    u32vec v(cap);
    v.clear();
    EXPECT_TRUE(v.size() == 0 && v.capacity() == cap);
    uint8_t* ok = nullptr;
    cudaMallocManaged(&ok, n);
    u32vec* dv = v.upload();
    push_many<<<(n + 255) / 256, 256>>>(dv, n, ok, moved);
    cudaDeviceSynchronize();
    std::multiset<uint32_t> got(v.begin(), v.end()), want;
    for (uint32_t i = 0; i < n; ++i)
      if (ok[i]) want.insert(i);
    EXPECT_TRUE(v.size() == cap - 1);
    EXPECT_TRUE(want.size() == cap - 1);
    EXPECT_TRUE(got == want);
    cudaFree(ok);
  }
}

struct test_t {
  uint32_t num;
  uint32_t flag;
  __host__ __device__ bool operator==(const test_t& o) const { return num == o.num && flag == o.flag; }
};
typedef split::SplitVector<test_t> tvec;

static void fill_vec(tvec& v, size_t n, size_t* count) {
  v.clear();
  *count = 0;
  uint32_t st = 0;
  while (v.size() < n) {
    const uint32_t val = ++st;
    v.push_back(test_t{val, val % 2 == 0});
    if (val % 2 == 0) ++*count;
  }
}

// preallocated.cu:225-303 with std::thread in place of OpenMP: 64 vectors of
// 2^12 elements, 4 host threads, 2 streams each, every compaction's scratch a
// slice of one caller buffer.
static void test_preallocated_compactions() {
  constexpr size_t N = 64, nThreads = 4, streamsPerThread = 2;
  const size_t len = 1u << 12;
  std::vector<tvec> vecs(N), out1(N), out2(N);
  size_t count = 0;
  for (auto& v : vecs) fill_vec(v, len, &count);
  for (auto& v : out1) v.resize(len);
  for (auto& v : out2) v.resize(len);
  auto on = [] __host__ __device__(test_t e) -> bool { return e.flag == 1; };
  auto off = [] __host__ __device__(test_t e) -> bool { return e.flag == 0; };
  const size_t bytes = split::tools::estimateMemoryForCompaction(vecs[0]);
  void* buffer = nullptr;
  cudaMalloc(&buffer, streamsPerThread * nThreads * bytes);
  cudaDeviceSynchronize();
  // nothing below may allocate from the device's stream-ordered pool
  cudaMemPool_t pool;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetDefaultMemPool(&pool, dev);
  uint64_t zero = 0, high = 0, used0 = 0;
  cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used0);
  cudaMemPoolSetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &zero);
  std::vector<std::thread> threads;
  for (size_t t = 0; t < nThreads; ++t) {
    threads.emplace_back([&, t] {
      cudaSetDevice(dev);
      cudaStream_t st[streamsPerThread];
      for (auto& s : st) cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
      void* s1 = static_cast<char*>(buffer) + t * streamsPerThread * bytes;
      void* s2 = static_cast<char*>(s1) + bytes;
      for (size_t i = t; i < N; i += nThreads) {
        split::tools::copy_if(vecs[i], out1[i], on, split::tools::splitStackArena{s1, bytes}, st[0]);
        split::tools::copy_if(vecs[i], out2[i], off, s2, bytes, st[1]);
      }
      for (auto& s : st) {
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
      }
    });
  }
  for (auto& th : threads) th.join();
  cudaDeviceSynchronize();
  cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &high);
  EXPECT_TRUE(high <= used0);  // no stream-ordered allocation happened meanwhile
  cudaFree(buffer);
  bool sane = true;
  for (size_t i = 0; i < N; ++i) {
    sane = sane && out1[i].size() == count && out2[i].size() == len - count;
    for (const auto& e : out1[i]) sane = sane && e.flag == 1;
    for (const auto& e : out2[i]) sane = sane && e.flag == 0;
    // order preserved: the selected elements are the odd / even positions in input order
    for (size_t k = 0; k < out1[i].size(); ++k) sane = sane && out1[i][k].num == 2 * (k + 1);
    for (size_t k = 0; k < out2[i].size(); ++k) sane = sane && out2[i][k].num == 2 * k + 1;
  }
  EXPECT_TRUE(sane);
}

__global__ void push_range(u32vec* v, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v->device_push_back(i);
}
struct Mod3 {
  __host__ __device__ bool operator()(const uint32_t& x) const { return x % 3 == 0; }
};

// copy_if_loop reads the input's size on the device: the input is filled by
// a kernel on the same stream and compacted with no host synchronisation
// between; the output's size is set on the device.
static void test_loop_reads_device_size() {
  const uint32_t n = 100000;
  u32vec in(n + 2), out(n + 2);
  in.clear();
  out.clear();
  cudaStream_t s;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  u32vec* din = in.upload(s);
  push_range<<<(n + 255) / 256, 256, 0, s>>>(din, n);
  split::tools::copy_if_loop(in, out, Mod3{}, s);
  cudaStreamSynchronize(s);
  EXPECT_TRUE(in.size() == n);
  std::multiset<uint32_t> pushed(in.begin(), in.end());
  std::vector<uint32_t> want;
  for (uint32_t x : in)
    if (x % 3 == 0) want.push_back(x);  // input order, whatever order the pushes landed in
  EXPECT_TRUE(out.size() == want.size() && std::equal(want.begin(), want.end(), out.begin()));
  cudaStreamDestroy(s);
}

struct ModLt {
  uint32_t a, b;
  __host__ __device__ bool operator()(const uint32_t& x) const { return x % a < b; }
};

// The header's functor compaction equals libhx's descriptor compaction, and
// the raw-pointer form handles an input that starts 4 bytes past a 16-byte
// boundary (the elements before the boundary are compacted first).
static void test_functor_matches_descriptor() {
  const size_t n = (1u << 22) + 3;
  u32vec in(n);
  uint32_t x = 12345;
  for (size_t i = 0; i < n; ++i) {
    x = x * 1664525u + 1013904223u;
    in[i] = x;
  }
  for (uint32_t s : {1u, 50u, 99u}) {
    u32vec a(n), b(n);
    split::tools::copy_if(in, a, ModLt{100, s});
    split::tools::copy_if(in, b, hx_pred{HX_PRED_MOD_LT, HX_FIELD_ELEM, 0, 0, 100, s});
    EXPECT_TRUE(a.size() == b.size() && a == b);
    size_t c = 0;
    for (size_t i = 0; i < n; ++i) c += in[i] % 100 < s;
    EXPECT_TRUE(a.size() == c);
  }
  // unaligned raw input: elements 1..n-1
  u32vec out(n);
  const size_t bytes = split::tools::estimateMemoryForCompaction<1024>(n);
  void* stack = nullptr;
  cudaMalloc(&stack, bytes);
  const size_t c = split::tools::copy_if(in.data() + 1, out.data(), n - 1, ModLt{7, 3}, stack, bytes);
  std::vector<uint32_t> want;
  for (size_t i = 1; i < n; ++i)
    if (in[i] % 7 < 3) want.push_back(in[i]);
  EXPECT_TRUE(c == want.size() && std::equal(want.begin(), want.end(), out.begin()));
  cudaFree(stack);
}

int main() {
  test_reference_device_tests();
  test_concurrent_push_back();
  test_preallocated_compactions();
  test_loop_reads_device_size();
  test_functor_matches_descriptor();
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    std::printf("CUDA error %s\n", cudaGetErrorString(e));
    return 2;
  }
  if (g_fail) {
    std::printf("%d FAILED\n", g_fail);
    return 1;
  }
  std::printf("PASSED\n");
  return 0;
}
