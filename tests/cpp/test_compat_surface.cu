// The rest of the reference's Hashmap and split::tools surface, written
// against the drop-in header (include/hashinator_compat.h):
//   Test_Copy_Metadata                    unit_tests/hashmap_unit_test/main.cu:1022-1037
//   EMPTY_TOMBSTONE_values (custom sentinels named)            main.cu:1087-1094
//   splitStackArena, estimateMemoryForCompaction, the arena and stack copy_if
//   forms, copy_keys_if, copy_if_loop / copy_if_keys_loop
//                                         splitvector/split_tools.h:491-535, 995-1223
//   swap, rehash, tombstone_ratio, stats, dump_buckets, memAdvise,
//   streamAttach and the loop extractions  hashinator/hashinator.h:236, 591-627,
//                                         1129, 1187-1260, 1440
// A tiny harness stands in for gtest (not installed). Exit code 0 = all pass.
#include <algorithm>
#include <cstdio>
#include <random>
#include <set>
#include <vector>

#include "hashinator_compat.h"

using namespace Hashinator;
typedef uint32_t key_type;
typedef uint32_t val_type;
typedef split::SplitVector<hash_pair<key_type, val_type>> vector;
typedef Hashmap<key_type, val_type> hashmap;

static int g_fail = 0;
#define EXPECT_TRUE(c)                                                   \
  do {                                                                   \
    if (!(c)) {                                                          \
      std::printf("FAIL %s:%d: %s\n", __FILE__, __LINE__, #c);           \
      ++g_fail;                                                          \
    }                                                                    \
  } while (0)

struct Predicate {  // hashmap_unit_test/main.cu:28-33
  __host__ __device__ bool operator()(hash_pair<key_type, val_type>& e) const { return e.second % 2 == 0; }
};
struct KeyBelow1000 {  // hashmap_unit_test/main.cu:975-981
  __host__ __device__ bool operator()(hash_pair<key_type, val_type>& e) const { return e.first < 1000; }
};

static void create_input(vector& src, uint32_t bias = 0) {
  for (size_t i = 0; i < src.size(); ++i) src.at(i) = hash_pair<key_type, val_type>(i + bias, i);
}

// Query every source key through retrieve(pairs) and compare values.
static bool recover(hashmap& h, vector& src, bool odd_only) {
  vector q(src.size());
  for (size_t i = 0; i < src.size(); ++i) q[i] = hash_pair<key_type, val_type>(src[i].first, 0xDEADBEEFu);
  h.retrieve(q.data(), q.size());
  for (size_t i = 0; i < src.size(); ++i) {
    const bool present = !odd_only || (src[i].second % 2 == 1);
    if (present && q[i].second != src[i].second) return false;
    if (!present && q[i].second != 0xDEADBEEFu) return false;
  }
  return true;
}

static void test_copy_metadata() {  // hashmap_unit_test/main.cu:1022-1037
  vector src(size_t(1) << 18);
  create_input(src);
  hashmap hmap;
  hmap.insert(src.data(), src.size());
  EXPECT_TRUE(recover(hmap, src, false));
  EXPECT_TRUE(hmap.peek_status() == status::success);
  Info info;
  hmap.copyMetadata(&info);
  EXPECT_TRUE((size_t(1) << info.sizePower) == hmap.bucket_count());
  EXPECT_TRUE(info.tombstoneCounter == hmap.tombstone_count());
  EXPECT_TRUE(info.fill == src.size());
}

static void test_custom_sentinels() {  // hashmap_unit_test/main.cu:1087-1094
  Hashmap<key_type, val_type, 42, 42> hmap;
  const auto tombstone = hmap.get_tombstone();
  const auto emptybucket = hmap.get_emptybucket();
  EXPECT_TRUE(tombstone == emptybucket && tombstone == 42);
  static_assert(tombstone == emptybucket, "the sentinels are compile-time constants");
}

// copy_if with an owned arena and with a caller stack, copy_keys_if in its
// three forms, and the arena's bump allocation (split_tools.h:491-535,
// 1065-1223; the arena use of stream_compaction/preallocated.cu).
static void test_arena_and_key_overloads() {
  const size_t N = 5000;
  vector src(N);
  create_input(src);  // (i, i): the even values sit at even i
  const size_t bytes = split::tools::estimateMemoryForCompaction(src);
  EXPECT_TRUE(bytes >= 64 && bytes == split::tools::estimateMemoryForCompaction<1024>(N));
  void* stack = nullptr;
  cudaMalloc(&stack, bytes);
  vector o1(N), o2(N);
  split::tools::copy_if(src, o1, Predicate(), split::tools::splitStackArena(bytes, 0));
  split::tools::copy_if(src, o2, Predicate(), stack, bytes);
  EXPECT_TRUE(o1.size() == N / 2 && o2.size() == N / 2);
  bool ok = true;
  for (size_t i = 0; i < o1.size() && i < o2.size(); ++i)
    ok = ok && o1[i].first == 2 * i && o1[i].second == 2 * i && o2[i] == o1[i];
  EXPECT_TRUE(ok);
  split::SplitVector<key_type> k1(N), k2(N), k3(N);
  split::tools::copy_keys_if(src, k1, Predicate());
  split::tools::copy_keys_if(src, k2, Predicate(), split::tools::splitStackArena(bytes, 0));
  split::tools::copy_keys_if(src, k3, Predicate(), stack, bytes);
  EXPECT_TRUE(k1.size() == N / 2 && k2.size() == N / 2 && k3.size() == N / 2);
  ok = true;
  for (size_t i = 0; i < k1.size() && i < k2.size() && i < k3.size(); ++i)
    ok = ok && k1[i] == 2 * i && k2[i] == 2 * i && k3[i] == 2 * i;
  EXPECT_TRUE(ok);
  vector o3;
  split::SplitVector<key_type> k4;
  o3.reserve(N);  // the loop forms fill the output's capacity
  k4.reserve(N);
  split::tools::copy_if_loop(src, o3, Predicate());
  split::tools::copy_if_keys_loop(src, k4, Predicate());
  cudaDeviceSynchronize();
  EXPECT_TRUE(o3.size() == N / 2 && k4.size() == N / 2);
  ok = true;
  for (size_t i = 0; i < o3.size() && i < k4.size() && i < o1.size(); ++i) ok = ok && o3[i] == o1[i] && k4[i] == 2 * i;
  EXPECT_TRUE(ok);
  split::tools::splitStackArena a(stack, bytes);
  char* p0 = static_cast<char*>(a.allocate(16));
  char* p1 = static_cast<char*>(a.allocate(32));
  EXPECT_TRUE(p0 == stack && p1 == p0 + 16 && a.fill() == 48 && a.free_space() == bytes - 48);
  a.deallocate(32);
  EXPECT_TRUE(a.fill() == 16);
  a.reset();
  EXPECT_TRUE(a.fill() == 0 && a.capacity() == bytes);
  cudaDeviceSynchronize();
  cudaFree(stack);
}

// swap, rehash, tombstone_ratio, the "loop" extractions, the no-op memory
// hints and the printing helpers (hashinator.h:236, 591-627, 1129,
// 1187-1260, 1440).
static void test_more_host_methods() {
  const size_t N = 1000;
  vector src(N);
  create_input(src);
  hashmap a(12), b(6);
  a.insert(src.data(), N, 1.0f);
  a.swap(b);
  EXPECT_TRUE(a.size() == 0 && a.getSizePower() == 6 && b.size() == N && b.getSizePower() == 12);
  b.rehash(13);
  EXPECT_TRUE(b.size() == N && b.getSizePower() == 13 && recover(b, src, false));
  split::SplitVector<key_type> evens;
  for (size_t i = 0; i < N; i += 2) evens.push_back((key_type)i);
  b.erase(evens.data(), evens.size());
  EXPECT_TRUE(b.tombstone_count() == N / 2);
  EXPECT_TRUE(b.tombstone_ratio() == (float)(N / 2) / (float)(1 << 13));
  EXPECT_TRUE(a.tombstone_ratio() == 0.0f);
  auto odd_valid = [] __host__ __device__(hash_pair<key_type, val_type> & e) -> bool {
    return e.first != 0xFFFFFFFFu && e.first != 0xFFFFFFFEu && e.second % 2 == 1;
  };
  // the loop forms write into the output's capacity (the reference's
  // loop_compact asserts that it suffices), so the outputs are sized first
  vector e1(N), e2(N);
  split::SplitVector<key_type> k1(N), k2(N);
  b.extractLoop(e1);
  b.extractPatternLoop(e2, odd_valid);
  b.extractAllKeysLoop(k1);
  b.extractKeysByPatternLoop(k2, odd_valid);
  cudaDeviceSynchronize();  // the loop forms set the sizes on the device, without a host synchronisation
  EXPECT_TRUE(e1.size() == N / 2 && e2.size() == N / 2 && k1.size() == N / 2 && k2.size() == N / 2);
  bool ok = true;
  for (auto& e : e1) ok = ok && e.first % 2 == 1 && e.second == e.first;
  for (size_t i = 0; i < e2.size() && i < e1.size(); ++i) ok = ok && e2[i] == e1[i];  // both in bucket order
  for (size_t i = 0; i < k1.size() && i < e1.size(); ++i) ok = ok && k1[i] == e1[i].first && k2[i] == k1[i];
  EXPECT_TRUE(ok);
  b.memAdvise(cudaMemAdviseSetPreferredLocation, 0);
  b.streamAttach(0);
  b.stats();
  hashmap tiny(4);
  tiny.insert(src.data(), 3, 1.0f);
  tiny.dump_buckets();
  EXPECT_TRUE(tiny.size() == 3);
}


int main() {
  test_copy_metadata();
  test_custom_sentinels();
  test_arena_and_key_overloads();
  test_more_host_methods();
  std::printf("%s (%d failures)\n", g_fail ? "FAILED" : "PASSED", g_fail);
  return g_fail ? 1 : 0;
}
