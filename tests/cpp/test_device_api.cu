// Element access from user kernels through include/hx_device_api.cuh, checked
// against the C-ABI bulk path on the same map: the reference's device API
// usage (unit_tests/delete_by_compaction/main.cu:83-141: set_element from a
// kernel, device_erase, then the host-side cleanup) plus the warp accessors.
#include <cstdio>
#include <vector>

#include "hx_device_api.cuh"

static int g_fail = 0;
#define EXPECT(c)                                                       \
  do {                                                                  \
    if (!(c)) {                                                         \
      std::printf("FAIL %s:%d: %s\n", __FILE__, __LINE__, #c);          \
      ++g_fail;                                                         \
    }                                                                   \
  } while (0)
#define CK(x) EXPECT((x) == HX_OK)

template <class K>
__host__ __device__ K key_of(uint64_t i) {  // distinct, never a sentinel
  return (K)(i * 2654435761ull % 0xFFFFFFF0ull + 1);
}

template <class K, class V>
__global__ void k_set(hx_device::MapView<K, V> m, uint64_t n, unsigned* news) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i < n && m.set_element(key_of<K>(i), (V)(i * 3 + 1))) atomicAdd(news, 1u);
}
template <class K, class V>
__global__ void k_check(hx_device::MapView<K, V> m, uint64_t n, unsigned* bad, bool evens_erased) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  V v = 0;
  const bool f = m.read_element(key_of<K>(i), v);
  const bool want = !(evens_erased && i % 2 == 0);
  if (f != want || (f && v != (V)(i * 3 + 1)) || m.device_count(key_of<K>(i)) != (want ? 1u : 0u)) atomicAdd(bad, 1u);
}
template <class K, class V>
__global__ void k_erase_evens(hx_device::MapView<K, V> m, uint64_t n, unsigned* erased) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i < n && i % 2 == 0) atomicAdd(erased, (unsigned)m.device_erase(key_of<K>(i)));
}
// one warp per key: insert a new key range, find it, erase every third
template <class K, class V>
__global__ void k_warp(hx_device::MapView<K, V> m, uint64_t base, uint64_t n, unsigned* counts) {
  const uint64_t w = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x & 31;
  if (w >= n) return;  // whole warps leave together
  const K key = key_of<K>(base + w);
  const bool isnew = m.warp_insert(key, (V)(w + 7), lane);
  V v = 0;
  const bool found = m.warp_find(key, v, lane);
  bool er = false;
  if (w % 3 == 0) er = m.warp_erase(key, lane);
  if (lane == 0) {
    if (isnew) atomicAdd(counts + 0, 1u);
    if (found && v == (V)(w + 7)) atomicAdd(counts + 1, 1u);
    if (er) atomicAdd(counts + 2, 1u);
  }
}

template <class K>
static void run(int key_bytes) {
  using V = K;
  const uint64_t n = 20000, nw = 3000;
  hx_map* m = nullptr;
  CK(hx_map_create(&m, key_bytes, key_bytes, 16, nullptr));
  hx_device_view dv;
  CK(hx_map_device_view(m, &dv));
  auto view = hx_device::MapView<K, V>::from(dv);
  unsigned* c = nullptr;
  cudaMallocManaged(&c, 16 * sizeof(unsigned));
  for (int i = 0; i < 16; ++i) c[i] = 0;
  k_set<K, V><<<(n + 255) / 256, 256>>>(view, n, c + 0);
  k_set<K, V><<<(n + 255) / 256, 256>>>(view, n, c + 1);  // all overwrites
  k_check<K, V><<<(n + 255) / 256, 256>>>(view, n, c + 2, false);
  cudaDeviceSynchronize();
  EXPECT(c[0] == n && c[1] == 0 && c[2] == 0);
  hx_info inf;
  CK(hx_get_info(m, &inf, nullptr));
  EXPECT(inf.fill == n);
  // bulk retrieve through the C ABI sees the device-inserted keys
  std::vector<K> hk(n);
  for (uint64_t i = 0; i < n; ++i) hk[i] = key_of<K>(i);
  K *dk, *dval;
  cudaMalloc(&dk, n * sizeof(K));
  cudaMalloc(&dval, n * sizeof(V));
  cudaMemcpy(dk, hk.data(), n * sizeof(K), cudaMemcpyHostToDevice);
  CK(hx_retrieve(m, dk, dval, n, nullptr));
  std::vector<V> hv(n);
  cudaMemcpy(hv.data(), dval, n * sizeof(V), cudaMemcpyDeviceToHost);
  for (uint64_t i = 0; i < n; ++i) EXPECT(hv[i] == (V)(i * 3 + 1));
  k_erase_evens<K, V><<<(n + 255) / 256, 256>>>(view, n, c + 3);
  k_check<K, V><<<(n + 255) / 256, 256>>>(view, n, c + 4, true);
  cudaDeviceSynchronize();
  EXPECT(c[3] == n / 2 && c[4] == 0);
  CK(hx_get_info(m, &inf, nullptr));
  EXPECT(inf.fill == n / 2 && inf.tombstone_counter == n / 2);
  CK(hx_clean_tombstones(m, nullptr));  // the host-side cleanup after device work (download())
  CK(hx_get_info(m, &inf, nullptr));
  EXPECT(inf.fill == n / 2 && inf.tombstone_counter == 0);
  k_check<K, V><<<(n + 255) / 256, 256>>>(view, n, c + 5, true);
  k_warp<K, V><<<(nw * 32 + 255) / 256, 256>>>(view, n, nw, c + 6);
  cudaDeviceSynchronize();
  EXPECT(c[5] == 0);
  EXPECT(c[6] == nw && c[7] == nw && c[8] == (nw + 2) / 3);
  CK(hx_get_info(m, &inf, nullptr));
  EXPECT(inf.fill == n / 2 + nw - (nw + 2) / 3);
  EXPECT(cudaGetLastError() == cudaSuccess);
  cudaFree(dk);
  cudaFree(dval);
  cudaFree(c);
  CK(hx_map_destroy(m));
}

int main() {
  run<uint32_t>(4);
  run<uint64_t>(8);
  std::printf("%s (%d failures)\n", g_fail ? "FAILED" : "PASSED", g_fail);
  return g_fail ? 1 : 0;
}
