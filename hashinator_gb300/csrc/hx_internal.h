// hx_internal.h — host-side internals shared by the libhx translation units:
// the map handle and its probe tuning.
#pragma once
#include <cstdint>
#include <mutex>
#include <cuda_runtime.h>
#include "../../include/hx.h"
#include "hx_probe.cuh"

namespace hx {

struct Tuning {
  int group = 0;   // lanes per key; 0 = automatic policy (auto_policy)
  int unroll = 1;  // keys in flight per thread when group == 1
  int block = 256;
  bool blind = true;  // thread-per-key insert: CAS the home bucket without reading it first
  bool wide = false;  // thread-per-key windows of 64 B instead of 32 B
};


}  // namespace hx

struct hx_map {
  int key_bytes = 0, val_bytes = 0;
  int sp = 0;
  int device = 0;
  void* buckets = nullptr;
  hx::DInfo* info = nullptr;
  uint64_t fill_ub = 0;  // host upper bound on fill (exact after a sync)
  void* scratch = nullptr;
  uint64_t scratch_bytes = 0;
  hx::Tuning tune;
  std::mutex mu;  // guards scratch growth; a map is not thread-safe otherwise
};


namespace hx {
// The plain per-map paths on a map handle (also used on views into a batch).
hx_status map_insert_view(hx_map* m, const void* keys, const void* vals, const void* pairs, uint64_t n,
                          cudaStream_t s);
hx_status map_find_view(hx_map* m, const void* keys, void* vals, void* pairs, uint64_t n, bool erase,
                        cudaStream_t s);
// device_rehash of the viewed table into a new cudaMallocAsync allocation of
// 2^new_sp buckets; the old bucket array is released stream-ordered.
hx_status map_rehash_view(hx_map* m, int new_sp, cudaStream_t s);
}  // namespace hx
