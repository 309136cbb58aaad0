// The reference's own hot-path unit tests, written against the drop-in
// header (include/hashinator_compat.h) instead of hashinator.h:
//   test_hashmap_4          unit_tests/hashmap_unit_test/main.cu:726-785
//   Test_Duplicate_Insertion                          main.cu:1064-1085
//   Test_ErrorCodes_ExtractKeysByPattern-style rule   main.cu:975-1019
//   Compaction_Tests_Linear / _Power_of_2   unit_tests/stream_compaction/unit.cu:133-153
//   prefix scan of input[i] = i             unit_tests/stream_compaction/race.cu:100-113
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

static void test_hashmap_4(int power) {
  const size_t N = size_t(1) << power;
  vector src(N);
  create_input(src);
  hashmap hmap;
  hmap.insert(src.data(), src.size());
  EXPECT_TRUE(recover(hmap, src, false));
  vector evenBuffer(src.size());
  split::tools::copy_if(src, evenBuffer, Predicate());
  split::SplitVector<key_type> keyBuffer;
  for (auto& i : evenBuffer) keyBuffer.push_back(i.first);
  EXPECT_TRUE(keyBuffer.size() == N / 2);
  hmap.erase(keyBuffer.data(), keyBuffer.size());
  EXPECT_TRUE(recover(hmap, src, true));
  EXPECT_TRUE(hmap.size() == N / 2 && hmap.tombstone_count() == N / 2);
  cudaStream_t s;
  cudaStreamCreate(&s);
  hmap.clean_tombstones(s);
  EXPECT_TRUE(hmap.tombstone_count() == 0 && hmap.size() == N / 2);
  EXPECT_TRUE(recover(hmap, src, true));
  hmap.insert(src.data(), src.size());
  EXPECT_TRUE(recover(hmap, src, false));
  EXPECT_TRUE(hmap.size() == N);
  cudaStreamDestroy(s);
}

static void test_duplicate_insertion() {
  const int sz = 10;
  std::mt19937 g(7);
  for (size_t duplicates = 2; duplicates <= (1u << sz); duplicates *= 2) {
    std::set<key_type> uniq;
    while (uniq.size() < (1u << sz)) uniq.insert(g() % 0xFFFFFF00u);
    std::vector<key_type> keys(uniq.begin(), uniq.end());
    for (size_t i = 0; i < duplicates; ++i) keys.push_back(keys[0]);
    std::shuffle(keys.begin(), keys.end(), g);
    vector src(keys.size());
    for (size_t i = 0; i < keys.size(); ++i) src[i] = hash_pair<key_type, val_type>(keys[i], keys[i]);
    hashmap hmap;
    hmap.insert(src.data(), src.size(), 1);
    EXPECT_TRUE(recover(hmap, src, false));
    EXPECT_TRUE(hmap.peek_status() == status::success);
    EXPECT_TRUE(hmap.size() == (1u << sz));
  }
}

static void test_extract_rules() {
  const size_t N = 1 << 12;
  vector src(N);
  create_input(src);
  hashmap hmap(13);
  hmap.insert(src.data(), src.size());
  vector out;
  const size_t c = hmap.extractPattern(out, KeyBelow1000());
  EXPECT_TRUE(c == 1000 && out.size() == 1000);
  std::vector<key_type> ks;
  for (auto& e : out) ks.push_back(e.first);
  std::sort(ks.begin(), ks.end());
  for (size_t i = 0; i < ks.size(); ++i) EXPECT_TRUE(ks[i] == i);
  // the same rule as a descriptor, run inside libhx: same pairs in the same (bucket) order
  hx_pred p{HX_PRED_LT, HX_FIELD_KEY, 0, 0, 1000, 0};
  vector out2;
  EXPECT_TRUE(hmap.extractPattern(out2, p) == 1000);
  bool same = out2.size() == out.size();
  for (size_t i = 0; same && i < out.size(); ++i) same = out[i] == out2[i];
  EXPECT_TRUE(same);
  // value-even rule (extractPattern on the map): every selected value even
  vector ev;
  const size_t ce = hmap.extractPattern(ev, Predicate());
  size_t even_valid = 0;
  for (auto& e : ev) even_valid += (e.first < N && e.second % 2 == 0);
  // the rule also sees EMPTY buckets (value 0, even), like the reference's rules
  EXPECT_TRUE(even_valid == N / 2 && ce >= N / 2);
}

struct test_t {
  uint32_t num, flag;
};

static bool compaction_flags(size_t size) {  // stream_compaction/unit.cu:36-107
  split::SplitVector<test_t> v;
  size_t count = 0;
  for (uint32_t st = 1; v.size() < size; ++st) {
    v.push_back(test_t{st, (uint32_t)(st % 2 == 0)});
    count += (st % 2 == 0);
  }
  auto on = [] __host__ __device__(test_t & e) -> bool { return e.flag == 1; };
  auto off = [] __host__ __device__(test_t & e) -> bool { return e.flag == 0; };
  split::SplitVector<test_t> o1(v.size()), o2(v.size());
  split::tools::copy_if(v, o1, on);
  split::tools::copy_if(v, o2, off);
  bool ok = o1.size() + o2.size() == v.size() && o1.size() == count && o2.size() == v.size() - count;
  for (auto& e : o1) ok = ok && e.flag == 1;
  for (auto& e : o2) ok = ok && e.flag == 0;
  for (size_t i = 1; i < o1.size(); ++i) ok = ok && o1[i].num > o1[i - 1].num;  // order kept
  return ok;
}

static bool scan_iota(size_t n) {  // stream_compaction/race.cu:100-113
  split::SplitVector<uint32_t> in(n), out(n);
  for (size_t i = 0; i < n; ++i) in[i] = (uint32_t)i;
  split::tools::split_prefix_scan(in, out);
  uint32_t acc = 0;
  for (size_t i = 0; i < n; ++i) {
    if (out[i] != acc) return false;
    acc += (uint32_t)i;
  }
  return true;
}

int main() {
  for (int p = 10; p <= 16; p += 3) test_hashmap_4(p);
  test_duplicate_insertion();
  test_extract_rules();
  for (size_t s = 32; s < 3000; s += 37) EXPECT_TRUE(compaction_flags(s));
  for (int p = 5; p < 20; p += 2) EXPECT_TRUE(compaction_flags(size_t(1) << p));
  for (int p = 2; p < 18; ++p) EXPECT_TRUE(scan_iota(size_t(1) << p));
  std::printf("%s (%d failures)\n", g_fail ? "FAILED" : "PASSED", g_fail);
  return g_fail ? 1 : 0;
}
