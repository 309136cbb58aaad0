/*
 * hx_device_api.cuh — element access to a libhx table from inside user
 * kernels: the replacement of Hashinator's device API
 * (hashinator/hashinator.h:853-1126 warp accessors, :1563-1769 element API).
 *
 * Obtain a view on the host with hx_map_device_view() and pass it to the
 * kernel by value. All functions keep the table's invariants and counters
 * exactly as the library's own kernels do: probe order from the Fibonacci
 * home bucket, upsert, TOMBSTONE never reused by insert, fill / tombstone
 * counts, and the probe bound (largest distance + 1) that lookups use.
 *
 *   thread-level        set_element, device_insert, device_find, read_element,
 *                       device_count, device_erase
 *   warp-cooperative    warp_insert, warp_find, warp_erase (all 32 lanes call
 *                       with the same key; the reference's warpInsert /
 *                       warpFind / warpErase, one key per warp)
 *
 * Keys equal to EMPTY or TOMBSTONE are ignored (insert/erase do nothing,
 * lookups miss). Do not mix these calls with a concurrent libhx launch on
 * the same map (the reference forbids the same).
 */
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "hx.h"

namespace hx_device {

template <class K>
struct Sentinels {
  static constexpr K EMPTY = ~K(0);
  static constexpr K TOMB = ~K(0) - 1;
};

template <class K>
__host__ __device__ __forceinline__ uint32_t home(K key, int sp) {
  if constexpr (sizeof(K) == 4) {
    uint32_t k = key;
    k ^= k >> (32 - sp);
    return (uint32_t)(((uint64_t)k * 2654435769ull) >> (32 - sp)) & ((1u << sp) - 1u);
  } else {
    uint64_t k = key;
    k ^= k >> (64 - sp);
    return (uint32_t)((k * 11400714819323198485ull) >> (64 - sp)) & ((1u << sp) - 1u);
  }
}

/* A device view of one map (hx_device_view from hx_map_device_view()). */
template <class K, class V>
struct MapView {
  struct Bucket {
    K first;
    V second;
  };
  Bucket* buckets;
  int size_power;
  unsigned long long* fill;
  unsigned long long* tombstones;
  unsigned int* max_probe;
  int* err;

  __host__ __device__ static MapView from(const hx_device_view& v) {
    return MapView{static_cast<Bucket*>(v.buckets), v.size_power, v.fill, v.tombstones, v.max_probe, v.err};
  }

  // ---- publication primitives --------------------------------------------
  __device__ __forceinline__ bool cas_pair(Bucket* b, K& ek, V& ev, K key, V val) const {
    if constexpr (sizeof(K) == 4) {
      unsigned long long e = (unsigned long long)ek | ((unsigned long long)ev << 32);
      unsigned long long d = (unsigned long long)key | ((unsigned long long)val << 32);
      unsigned long long o = atomicCAS(reinterpret_cast<unsigned long long*>(b), e, d);
      ek = (K)o;
      ev = (V)(o >> 32);
      return o == e;
    } else {
      const unsigned __int128 c = ((unsigned __int128)ev << 64) | ek;
      const unsigned __int128 n = ((unsigned __int128)val << 64) | key;
      unsigned __int128 o;
      asm volatile("atom.global.relaxed.gpu.cas.b128 %0, [%1], %2, %3;" : "=q"(o) : "l"(b), "q"(c), "q"(n) : "memory");
      ek = (K)o;
      ev = (V)(o >> 64);
      return o == c;
    }
  }
  __device__ __forceinline__ void store_value(Bucket* b, V val) const {
    if constexpr (sizeof(V) == 4) atomicExch(reinterpret_cast<unsigned*>(&b->second), (unsigned)val);
    else atomicExch(reinterpret_cast<unsigned long long*>(&b->second), (unsigned long long)val);
  }
  __device__ __forceinline__ bool cas_key(Bucket* b, K key, K to) const {
    if constexpr (sizeof(K) == 4) return atomicCAS(reinterpret_cast<unsigned*>(&b->first), key, to) == key;
    else
      return atomicCAS(reinterpret_cast<unsigned long long*>(&b->first), (unsigned long long)key,
                       (unsigned long long)to) == (unsigned long long)key;
  }
  __device__ __forceinline__ K load_key(const Bucket* b) const {
    if constexpr (sizeof(K) == 4) return __ldcg(reinterpret_cast<const unsigned*>(&b->first));
    else return __ldcg(reinterpret_cast<const unsigned long long*>(&b->first));
  }
  __device__ __forceinline__ V load_value(const Bucket* b) const {
    if constexpr (sizeof(V) == 4) return __ldcg(reinterpret_cast<const unsigned*>(&b->second));
    else return __ldcg(reinterpret_cast<const unsigned long long*>(&b->second));
  }
  static __device__ __forceinline__ bool sentinel(K k) { return k == Sentinels<K>::EMPTY || k == Sentinels<K>::TOMB; }

  // ---- thread-level API (hashinator.h:1623-1769) ---------------------------

  /* set_element(key, val) (hashinator.h:1715): insert or overwrite; true if
   * the key is new. */
  template <bool skipOverWrites = false>
  __device__ bool set_element(K key, V val) const {
    if (sentinel(key)) return false;
    const uint32_t mask = (1u << size_power) - 1u;
    const uint32_t h = home(key, size_power);
    for (uint32_t d = 0; d <= mask; ++d) {
      Bucket* b = buckets + ((h + d) & mask);
      K ek = Sentinels<K>::EMPTY;
      V ev = 0;
      for (int tries = 0; tries < 9; ++tries) {
        if (cas_pair(b, ek, ev, key, val)) {
          atomicAdd(fill, 1ull);
          atomicMax(max_probe, d + 1);
          return true;
        }
        if (ek != Sentinels<K>::EMPTY) break;  // EMPTY with another value: retry with it
      }
      if (ek == key) {
        if (!skipOverWrites) store_value(b, val);
        return false;
      }
    }
    atomicExch(err, HX_STATUS_FAIL);  // no EMPTY bucket left
    return false;
  }

  /* device_insert(pair) (hashinator.h:1707): (bucket index, is new). */
  template <bool skipOverWrites = false>
  __device__ bool device_insert(K key, V val, int64_t* index) const {
    const bool n = set_element<skipOverWrites>(key, val);
    if (index) *index = device_find(key);
    return n;
  }

  /* device_find(key) (hashinator.h:1564): bucket index, or -1. */
  __device__ int64_t device_find(K key) const {
    if (sentinel(key)) return -1;
    const uint32_t mask = (1u << size_power) - 1u;
    const uint32_t h = home(key, size_power);
    const uint32_t limit = *reinterpret_cast<volatile unsigned*>(max_probe);
    for (uint32_t d = 0; d < limit; ++d) {
      const uint32_t i = (h + d) & mask;
      const K k = load_key(buckets + i);
      if (k == key) return i;
      if (k == Sentinels<K>::EMPTY) return -1;
    }
    return -1;
  }

  /* read_element(key) (hashinator.h:1750), without the assert: false if absent. */
  __device__ bool read_element(K key, V& val) const {
    const int64_t i = device_find(key);
    if (i < 0) return false;
    val = load_value(buckets + i);
    return true;
  }

  __device__ size_t device_count(K key) const { return device_find(key) >= 0 ? 1 : 0; }

  /* device_erase(key) (hashinator.h:1651, :1672): 1 if erased. */
  __device__ size_t device_erase(K key) const {
    const int64_t i = device_find(key);
    if (i < 0) return 0;
    if (cas_key(buckets + i, key, Sentinels<K>::TOMB)) {
      atomicAdd(fill, 0ull - 1ull);
      atomicAdd(tombstones, 1ull);
      return 1;
    }
    return 0;
  }

  // ---- warp-cooperative API (hashinator.h:853-1126) ------------------------
  // One key per warp: lane l looks at bucket h + i + l of window i, the
  // lowest matching lane wins (the reference's decision rule).

  /* warpInsert / warpInsert_V (hashinator.h:854, :939): insert or overwrite
   * one key per warp; true on every lane if the key is new. */
  template <bool skipOverWrites = false>
  __device__ bool warp_insert(K key, V val, int w_tid) const {
    if (sentinel(key)) return false;
    const uint32_t mask = (1u << size_power) - 1u;
    const uint32_t h = home(key, size_power);
    for (uint32_t i = 0; i <= mask; i += 32) {
      Bucket* b = buckets + ((h + i + w_tid) & mask);
      const bool in = i + w_tid <= mask;
      const K k = in ? load_key(b) : Sentinels<K>::TOMB;
      const unsigned match = __ballot_sync(0xffffffffu, in && k == key);
      if (match) {
        if (!skipOverWrites && w_tid == __ffs(match) - 1) store_value(b, val);
        return false;
      }
      unsigned empty = __ballot_sync(0xffffffffu, in && k == Sentinels<K>::EMPTY);
      while (empty) {
        const int w = __ffs(empty) - 1;
        int res = 0;  // 0 continue, 1 inserted, 2 updated
        if (w_tid == w) {
          K ek = Sentinels<K>::EMPTY;
          V ev = load_value(b);
          for (int tries = 0; tries < 9; ++tries) {
            if (cas_pair(b, ek, ev, key, val)) {
              res = 1;
              atomicAdd(fill, 1ull);
              atomicMax(max_probe, i + w_tid + 1);
              break;
            }
            if (ek == key) {
              if (!skipOverWrites) store_value(b, val);
              res = 2;
              break;
            }
            if (ek != Sentinels<K>::EMPTY) break;
          }
        }
        res = __shfl_sync(0xffffffffu, res, w);
        if (res) return res == 1;
        empty &= ~(1u << w);
      }
    }
    if (w_tid == 0) atomicExch(err, HX_STATUS_FAIL);
    return false;
  }

  /* warpFind (hashinator.h:1028): true and the value on every lane if found. */
  __device__ bool warp_find(K key, V& val, int w_tid) const {
    if (sentinel(key)) return false;
    const uint32_t mask = (1u << size_power) - 1u;
    const uint32_t h = home(key, size_power);
    const uint32_t limit = *reinterpret_cast<volatile unsigned*>(max_probe);
    for (uint32_t i = 0; i < limit; i += 32) {
      Bucket* b = buckets + ((h + i + w_tid) & mask);
      const bool in = i + w_tid < limit;
      const K k = in ? load_key(b) : Sentinels<K>::TOMB;
      const unsigned match = __ballot_sync(0xffffffffu, in && k == key);
      if (match) {
        const int w = __ffs(match) - 1;
        V v = 0;
        if (w_tid == w) v = load_value(b);
        val = __shfl_sync(0xffffffffu, v, w);
        return true;
      }
      if (__ballot_sync(0xffffffffu, in && k == Sentinels<K>::EMPTY)) return false;
    }
    return false;
  }

  /* warpErase (hashinator.h:1078): true on every lane if erased. */
  __device__ bool warp_erase(K key, int w_tid) const {
    if (sentinel(key)) return false;
    const uint32_t mask = (1u << size_power) - 1u;
    const uint32_t h = home(key, size_power);
    const uint32_t limit = *reinterpret_cast<volatile unsigned*>(max_probe);
    for (uint32_t i = 0; i < limit; i += 32) {
      Bucket* b = buckets + ((h + i + w_tid) & mask);
      const bool in = i + w_tid < limit;
      const K k = in ? load_key(b) : Sentinels<K>::TOMB;
      const unsigned match = __ballot_sync(0xffffffffu, in && k == key);
      if (match) {
        const int w = __ffs(match) - 1;
        int ok = 0;
        if (w_tid == w && cas_key(b, key, Sentinels<K>::TOMB)) {
          ok = 1;
          atomicAdd(fill, 0ull - 1ull);
          atomicAdd(tombstones, 1ull);
        }
        return __shfl_sync(0xffffffffu, ok, w) != 0;
      }
      if (__ballot_sync(0xffffffffu, in && k == Sentinels<K>::EMPTY)) return false;
    }
    return false;
  }
};

}  // namespace hx_device
