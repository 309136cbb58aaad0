// The reference's device-API unit tests (user kernels that take the map's
// device copy from upload()), written against include/hashinator_compat.h:
//   gpu_write / gpu_delete_even / gpu_recover_odd_elements
//       + upload/download           unit_tests/hashmap_unit_test/main.cu:66-135, 531-585
//   gpu_remove_insert               main.cu:75-89
//   warpInsert / warpInsert<1> / warpInsert_V / warpFind / warpErase
//                                   main.cu:217-310, 817-856
//   extractKeysByPattern / extractAllKeys   main.cu:984-1019
//   insertIndex, resize_to_lf, performCleanupTasks   hashinator.h:530, 643, 1339
// Where the reference asserts inside a kernel, these kernels count the
// failures in managed memory and the host checks the count.
#include <algorithm>
#include <cstdio>
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

struct Counters {
  unsigned bad, found, erased, inserted, evens_seen, walked;
};

static Counters* new_counters() {
  Counters* c = nullptr;
  cudaMallocManaged(&c, sizeof(Counters));
  *c = Counters{};
  return c;
}

static void make_input(vector& src, uint32_t bias = 0) {
  for (size_t i = 0; i < src.size(); ++i) src[i] = hash_pair<key_type, val_type>(uint32_t(i) * 7u + 1u + bias, i);
}

// ---- thread-level kernels ---------------------------------------------------
__global__ void k_write(hashmap* h, hash_pair<key_type, val_type>* src, size_t n) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) h->set_element(src[i].first, src[i].second);
}

__global__ void k_delete_even(hashmap* h, hash_pair<key_type, val_type>* src, size_t n, Counters* c) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  auto pos = h->device_find(src[i].first);
  if (pos == h->device_end()) {
    atomicAdd(&c->bad, 1u);
    return;
  }
  if (pos->second % 2 == 0) {
    const key_type k = pos->first;
    if (h->device_erase(k) != 1) atomicAdd(&c->bad, 1u);
    if (h->device_erase(k) != 0) atomicAdd(&c->bad, 1u);  // second erase finds nothing
    atomicAdd(&c->erased, 1u);
  }
}

__global__ void k_recover_odd(hashmap* h, hash_pair<key_type, val_type>* src, size_t n, Counters* c) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n && src[i].second % 2 != 0) {
    auto it = h->device_find(src[i].first);
    if (it == h->device_end() || it->first != src[i].first || it->second != src[i].second) atomicAdd(&c->bad, 1u);
    if (h->device_count(src[i].first) != 1) atomicAdd(&c->bad, 1u);
    if (h->read_element(src[i].first) != src[i].second) atomicAdd(&c->bad, 1u);
  }
  if (i == 0) {  // one thread walks every valid bucket
    for (auto it = h->device_begin(); it != h->device_end(); ++it) {
      ++c->walked;
      if (it->second % 2 == 0) ++c->evens_seen;
    }
  }
}

// one thread: read + erase every element of rm, then set every element of add
__global__ void k_remove_insert(hashmap* h, hash_pair<key_type, val_type>* rm, hash_pair<key_type, val_type>* add,
                                size_t n, Counters* c) {
  if (blockIdx.x * blockDim.x + threadIdx.x != 0) return;
  for (size_t i = 0; i < n; ++i) {
    if (h->read_element(rm[i].first) != rm[i].second) ++c->bad;
    h->device_erase(rm[i].first);
  }
  for (size_t i = 0; i < n; ++i) c->inserted += h->set_element(add[i].first, add[i].second) ? 1u : 0u;
}

// device_insert returns (position, is new); device_erase(iterator) returns the next valid position
__global__ void k_insert_and_erase_by_position(hashmap* h, hash_pair<key_type, val_type>* src, size_t n,
                                               Counters* c) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  auto r = h->device_insert(src[i]);
  if (!r.second || r.first == h->device_end() || r.first->first != src[i].first) atomicAdd(&c->bad, 1u);
  auto again = h->device_insert(src[i]);  // already there: not new
  if (again.second) atomicAdd(&c->bad, 1u);
  if (i % 3 == 0) {
    auto pos = h->device_find(src[i].first);
    h->device_erase(pos);
    if (h->device_count(src[i].first) != 0) atomicAdd(&c->bad, 1u);
  }
}

// ---- warp-level kernels (one key per 32 lanes) -------------------------------
template <int SKIP>
__global__ void k_warp_write(hashmap* h, hash_pair<key_type, val_type>* src, size_t n, uint32_t val_bias) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t wid = t / 32, w_tid = t % 32;
  if (wid < n) h->warpInsert<SKIP>(src[wid].first, src[wid].second + val_bias, w_tid);
}
__global__ void k_warp_write_v(hashmap* h, hash_pair<key_type, val_type>* src, size_t n, Counters* c) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t wid = t / 32, w_tid = t % 32;
  if (wid < n) {
    const bool isnew = h->warpInsert_V(src[wid].first, src[wid].second, w_tid);
    if (w_tid == 0 && isnew) atomicAdd(&c->inserted, 1u);
  }
}
__global__ void k_warp_find(hashmap* h, hash_pair<key_type, val_type>* src, size_t n, uint32_t val_bias,
                            Counters* c) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t wid = t / 32, w_tid = t % 32;
  if (wid < n) {
    val_type v = 0xFFFFu;
    h->warpFind(src[wid].first, v, w_tid);
    if (v != src[wid].second + val_bias) atomicAdd(&c->bad, 1u);
    val_type absent = 42;
    h->warpFind(0xFFFFFFF0u - (key_type)wid, absent, w_tid);  // never inserted: untouched
    if (absent != 42) atomicAdd(&c->bad, 1u);
  }
}
__global__ void k_warp_erase(hashmap* h, hash_pair<key_type, val_type>* src, size_t n) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t wid = t / 32, w_tid = t % 32;
  if (wid < n) h->warpErase(src[wid].first, w_tid);
}

static unsigned blocks_for(size_t threads) { return (unsigned)((threads + 255) / 256); }

// Values present through the host retrieve path (what a later host call sees).
static bool host_sees(hashmap& h, vector& src, bool odd_only, uint32_t val_bias = 0) {
  vector q(src.size());
  for (size_t i = 0; i < src.size(); ++i) q[i] = hash_pair<key_type, val_type>(src[i].first, 0xDEADBEEFu);
  h.retrieve(q.data(), q.size());
  for (size_t i = 0; i < src.size(); ++i) {
    const bool present = !odd_only || (src[i].second % 2 == 1);
    if (present && q[i].second != src[i].second + val_bias) return false;
    if (!present && q[i].second != 0xDEADBEEFu) return false;
  }
  return true;
}

static void test_upload_download(int power) {
  const size_t n = size_t(1) << power;
  vector src(n);
  make_input(src);
  hashmap hmap(power + 1);
  Counters* c = new_counters();
  hashmap* d = hmap.upload();
  k_write<<<blocks_for(n), 256>>>(d, src.data(), n);
  cudaDeviceSynchronize();
  hmap.download();
  EXPECT_TRUE(hmap.size() == n);
  EXPECT_TRUE(host_sees(hmap, src, false));
  d = hmap.upload();
  k_delete_even<<<blocks_for(n), 256>>>(d, src.data(), n, c);
  cudaDeviceSynchronize();
  EXPECT_TRUE(c->bad == 0 && c->erased == n / 2);
  EXPECT_TRUE(hmap.tombstone_count() == n / 2);
  hmap.download();  // drops the tombstones
  EXPECT_TRUE(hmap.tombstone_count() == 0 && hmap.size() == n / 2);
  d = hmap.upload();
  k_recover_odd<<<blocks_for(n), 256>>>(d, src.data(), n, c);
  cudaDeviceSynchronize();
  EXPECT_TRUE(c->bad == 0 && c->evens_seen == 0 && c->walked == n / 2);
  EXPECT_TRUE(host_sees(hmap, src, true));
  EXPECT_TRUE(hmap.peek_status() == status::success || hmap.peek_status() == status::invalid);
  cudaFree(c);
}

static void test_remove_insert() {
  const size_t n = 64;
  vector rm(n), add(n);
  make_input(rm);
  make_input(add, 1u << 20);
  hashmap hmap(10);
  hmap.insert(rm.data(), n);
  Counters* c = new_counters();
  k_remove_insert<<<1, 32>>>(hmap.upload(), rm.data(), add.data(), n, c);
  cudaDeviceSynchronize();
  EXPECT_TRUE(c->bad == 0 && c->inserted == n);
  EXPECT_TRUE(hmap.size() == n && hmap.tombstone_count() == n);
  EXPECT_TRUE(host_sees(hmap, add, false));
  cudaFree(c);
}

static void test_device_insert_positions(int power) {
  const size_t n = size_t(1) << power;
  vector src(n);
  make_input(src);
  hashmap hmap(power + 1);
  Counters* c = new_counters();
  k_insert_and_erase_by_position<<<blocks_for(n), 256>>>(hmap.upload(), src.data(), n, c);
  cudaDeviceSynchronize();
  EXPECT_TRUE(c->bad == 0);
  const size_t erased = (n + 2) / 3;
  EXPECT_TRUE(hmap.size() == n - erased && hmap.tombstone_count() == erased);
  cudaFree(c);
}

static void test_warp_accessors(int power) {
  const size_t n = size_t(1) << power;
  vector src(n);
  make_input(src);
  hashmap hmap(power + 1);
  Counters* c = new_counters();
  hashmap* d = hmap.upload();
  k_warp_write<0><<<blocks_for(32 * n), 256>>>(d, src.data(), n, 0);
  k_warp_find<<<blocks_for(32 * n), 256>>>(d, src.data(), n, 0, c);
  cudaDeviceSynchronize();
  EXPECT_TRUE(c->bad == 0 && hmap.size() == n);
  // warpInsert<1> (skip overwrites, the unordered-set form) keeps the stored values
  k_warp_write<1><<<blocks_for(32 * n), 256>>>(d, src.data(), n, 5);
  k_warp_find<<<blocks_for(32 * n), 256>>>(d, src.data(), n, 0, c);
  cudaDeviceSynchronize();
  EXPECT_TRUE(c->bad == 0);
  // warpInsert overwrites
  k_warp_write<0><<<blocks_for(32 * n), 256>>>(d, src.data(), n, 5);
  k_warp_find<<<blocks_for(32 * n), 256>>>(d, src.data(), n, 5, c);
  cudaDeviceSynchronize();
  EXPECT_TRUE(c->bad == 0 && hmap.size() == n);
  EXPECT_TRUE(host_sees(hmap, src, false, 5));
  k_warp_erase<<<blocks_for(32 * n), 256>>>(d, src.data(), n);
  cudaDeviceSynchronize();
  EXPECT_TRUE(hmap.size() == 0 && hmap.tombstone_count() == n);
  hmap.download();
  EXPECT_TRUE(hmap.tombstone_count() == 0);
  // warpInsert_V reports every key as new into the emptied map
  d = hmap.upload();
  k_warp_write_v<<<blocks_for(32 * n), 256>>>(d, src.data(), n, c);
  cudaDeviceSynchronize();
  EXPECT_TRUE(c->inserted == n && hmap.size() == n);
  EXPECT_TRUE(host_sees(hmap, src, false));
  cudaFree(c);
}

struct KeyBelow1000 {  // hashmap_unit_test/main.cu:975-981
  __host__ __device__ bool operator()(hash_pair<key_type, val_type>& e) const { return e.first < 1000; }
};

static void test_extract_keys() {
  const size_t n = 5000;
  vector src(n);
  make_input(src);
  hashmap hmap(14);
  hmap.insert(src.data(), n);
  split::SplitVector<key_type> out;
  const size_t c = hmap.extractKeysByPattern(out, KeyBelow1000{});
  size_t want = 0;
  for (size_t i = 0; i < n; ++i) want += src[i].first < 1000;
  EXPECT_TRUE(c == want && out.size() == want);
  bool all_below = true;
  for (size_t i = 0; i < out.size(); ++i) all_below &= out[i] < 1000;
  EXPECT_TRUE(all_below);
  split::SplitVector<key_type> all;
  EXPECT_TRUE(hmap.extractAllKeys(all) == n && all.size() == n);
  std::vector<key_type> got(all.data(), all.data() + all.size()), exp(n);
  for (size_t i = 0; i < n; ++i) exp[i] = src[i].first;
  std::sort(got.begin(), got.end());
  std::sort(exp.begin(), exp.end());
  EXPECT_TRUE(got == exp);
  // the descriptor form gives the same keys in the same (bucket) order
  split::SplitVector<key_type> out2;
  hx_pred below{HX_PRED_LT, HX_FIELD_KEY, 0, 0, 1000, 0};
  EXPECT_TRUE(hmap.extractKeysByPattern(out2, below) == want);
  bool same = out2.size() == out.size();
  for (size_t i = 0; same && i < out.size(); ++i) same = out[i] == out2[i];
  EXPECT_TRUE(same);
}

static void test_index_and_maintenance() {
  const size_t n = 3000;
  split::SplitVector<key_type> keys(n);
  for (size_t i = 0; i < n; ++i) keys[i] = uint32_t(i) * 13u + 5u;
  hashmap hmap(4);
  hmap.insertIndex(keys.data(), n);  // grows: ceil(log2(3000 / 0.5)) = 13
  EXPECT_TRUE(hmap.getSizePower() == 13 && hmap.size() == n);
  vector q(n);
  for (size_t i = 0; i < n; ++i) q[i] = hash_pair<key_type, val_type>(keys[i], 0xDEADBEEFu);
  hmap.retrieve(q.data(), n);
  bool ok = true;
  for (size_t i = 0; i < n; ++i) ok &= q[i].second == i;
  EXPECT_TRUE(ok);
  hmap.resize_to_lf(0.1f);  // 3000 / 2^15 <= 0.1
  EXPECT_TRUE(hmap.getSizePower() == 15 && hmap.size() == n);
  hmap.erase(keys.data(), n / 2);
  hmap.performCleanupTasks();  // tombstone ratio 1500 / 2^15 > 0.025: cleaned
  EXPECT_TRUE(hmap.tombstone_count() == 0 && hmap.size() == n - n / 2);
}

int main() {
  for (int p = 8; p <= 16; p += 4) test_upload_download(p);
  test_remove_insert();
  test_device_insert_positions(12);
  for (int p = 6; p <= 14; p += 4) test_warp_accessors(p);
  test_extract_keys();
  test_index_and_maintenance();
  EXPECT_TRUE(cudaGetLastError() == cudaSuccess);
  std::printf("%s (%d failures)\n", g_fail ? "FAILED" : "PASSED", g_fail);
  return g_fail ? 1 : 0;
}
