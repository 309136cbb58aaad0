// hx_device.cuh — device building blocks shared by the libhx kernels:
// bucket layouts, the Fibonacci hash, vector bucket loads, packed atomics and
// the predicate descriptor. sm_103a only.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "../../include/hx.h"

namespace hx {

// hash_pair<K,V> (hashinator/hash_pair.h:30-75): {K first; V second;}.
// The 8-byte u32 pair is one 64-bit word (key low, value high) so that a
// single 64-bit CAS publishes key and value together. The 16-byte u64 pair
// is published with one 128-bit CAS.
struct alignas(8) P32 {
  uint32_t first, second;
};
struct alignas(16) P64 {
  uint64_t first, second;
};

template <class P>
struct PairTraits;
template <>
struct PairTraits<P32> {
  using K = uint32_t;
  using V = uint32_t;
  static constexpr K EMPTY = 0xFFFFFFFFu;  // std::numeric_limits<K>::max()
  static constexpr K TOMB = 0xFFFFFFFEu;   // EMPTY - 1
};
template <>
struct PairTraits<P64> {
  using K = uint64_t;
  using V = uint64_t;
  static constexpr K EMPTY = 0xFFFFFFFFFFFFFFFFull;
  static constexpr K TOMB = 0xFFFFFFFFFFFFFFFEull;
};

// Fibonacci hashing, bit-identical to HashFunctions::Fibonacci
// (hashinator/hashfunctions.h:39-43 for 32-bit keys, :52-56 for 64-bit keys):
// xor-fold the top bits down, multiply by 2^w / golden ratio, keep the top
// bits. The callers mask with 2^sp - 1 like the reference kernels
// (kernels_NVIDIA.h:350-351).
__host__ __device__ __forceinline__ uint32_t fib_hash(uint32_t key, int sp) {
  key ^= key >> (32 - sp);
  return (uint32_t)(((uint64_t)key * 2654435769ull) >> (32 - sp));
}
__host__ __device__ __forceinline__ uint64_t fib_hash(uint64_t key, int sp) {
  key ^= key >> (64 - sp);
  return (key * 11400714819323198485ull) >> (64 - sp);
}
template <class K>
__host__ __device__ __forceinline__ uint32_t home_slot(K key, int sp) {
  return (uint32_t)fib_hash(key, sp) & ((1u << sp) - 1u);
}

// ---- bucket loads: B consecutive buckets per lane in vector accesses ------
// 8 B (u32 pair, B=1), 16 B (B=2 u32 pairs or B=1 u64 pair), 32 B (B=4 u32
// pairs or B=2 u64 pairs, the sm_100+ 256-bit load) or 64 B (two of those).
template <int B>
__device__ __forceinline__ void load_buckets(const P32* p, uint32_t (&k)[B], uint32_t (&v)[B]) {
  if constexpr (B == 1) {
    uint2 x = __ldcg(reinterpret_cast<const uint2*>(p));
    k[0] = x.x; v[0] = x.y;
  } else if constexpr (B == 2) {
    uint4 x = __ldcg(reinterpret_cast<const uint4*>(p));
    k[0] = x.x; v[0] = x.y; k[1] = x.z; v[1] = x.w;
  } else {
    static_assert(B == 4 || B == 8, "B in {1,2,4,8}");
#pragma unroll
    for (int h = 0; h < B / 4; ++h) {
      unsigned long long a, b, c, d;
      asm volatile("ld.global.cg.v4.u64 {%0,%1,%2,%3}, [%4];"
                   : "=l"(a), "=l"(b), "=l"(c), "=l"(d) : "l"(p + 4 * h));
      k[4 * h + 0] = (uint32_t)a; v[4 * h + 0] = (uint32_t)(a >> 32);
      k[4 * h + 1] = (uint32_t)b; v[4 * h + 1] = (uint32_t)(b >> 32);
      k[4 * h + 2] = (uint32_t)c; v[4 * h + 2] = (uint32_t)(c >> 32);
      k[4 * h + 3] = (uint32_t)d; v[4 * h + 3] = (uint32_t)(d >> 32);
    }
  }
}
template <int B>
__device__ __forceinline__ void load_buckets(const P64* p, uint64_t (&k)[B], uint64_t (&v)[B]) {
  if constexpr (B == 1) {
    ulonglong2 x = __ldcg(reinterpret_cast<const ulonglong2*>(p));
    k[0] = x.x; v[0] = x.y;
  } else {
    static_assert(B == 2 || B == 4, "B in {1,2,4}");
#pragma unroll
    for (int h = 0; h < B / 2; ++h) {
      unsigned long long a, b, c, d;
      asm volatile("ld.global.cg.v4.u64 {%0,%1,%2,%3}, [%4];"
                   : "=l"(a), "=l"(b), "=l"(c), "=l"(d) : "l"(p + 2 * h));
      k[2 * h] = a; v[2 * h] = b; k[2 * h + 1] = c; v[2 * h + 1] = d;
    }
  }
}

// ---- atomics on buckets ----------------------------------------------------
// Publish (key, val) into a bucket expected to hold (ek, ev). Returns true on
// success; on failure (ek, ev) receive the bucket's current content.
__device__ __forceinline__ bool cas_pair(P32* p, uint32_t& ek, uint32_t& ev, uint32_t key, uint32_t val) {
  unsigned long long expect = (unsigned long long)ek | ((unsigned long long)ev << 32);
  unsigned long long desired = (unsigned long long)key | ((unsigned long long)val << 32);
  unsigned long long old = atomicCAS(reinterpret_cast<unsigned long long*>(p), expect, desired);
  ek = (uint32_t)old;
  ev = (uint32_t)(old >> 32);
  return old == expect;
}
__device__ __forceinline__ bool cas_pair(P64* p, uint64_t& ek, uint64_t& ev, uint64_t key, uint64_t val) {
  // 128-bit operands as "q" registers: the unpacking of the old value is
  // left to the compiler, so several CAS can be in flight per thread.
  const unsigned __int128 c = ((unsigned __int128)ev << 64) | ek;
  const unsigned __int128 n = ((unsigned __int128)val << 64) | key;
  unsigned __int128 o;
  asm volatile("atom.global.relaxed.gpu.cas.b128 %0, [%1], %2, %3;" : "=q"(o) : "l"(p), "q"(c), "q"(n) : "memory");
  ek = (uint64_t)o;
  ev = (uint64_t)(o >> 64);
  return o == c;
}
// Overwrite the value of a bucket that already holds the key (the
// reference's atomicExch on .second, kernels_NVIDIA.h:377,397).
__device__ __forceinline__ void store_value(P32* p, uint32_t val) { atomicExch(&p->second, val); }
__device__ __forceinline__ void store_value(P64* p, uint64_t val) {
  atomicExch(reinterpret_cast<unsigned long long*>(&p->second), (unsigned long long)val);
}
// key -> TOMBSTONE if the bucket still holds key.
__device__ __forceinline__ bool cas_key(P32* p, uint32_t key, uint32_t tomb) {
  return atomicCAS(&p->first, key, tomb) == key;
}
__device__ __forceinline__ bool cas_key(P64* p, uint64_t key, uint64_t tomb) {
  return atomicCAS(reinterpret_cast<unsigned long long*>(&p->first), (unsigned long long)key,
                   (unsigned long long)tomb) == (unsigned long long)key;
}

// ---- predicate descriptor (hx_pred) ---------------------------------------
__device__ __forceinline__ bool pred_on(const hx_pred& pr, uint64_t x) {
  switch (pr.op) {
    case HX_PRED_ALL: return true;
    case HX_PRED_MOD_LT: return (x % pr.a) < pr.b;
    case HX_PRED_LT: return x < pr.a;
    case HX_PRED_GE: return x >= pr.a;
    case HX_PRED_EQ: return x == pr.a;
    case HX_PRED_NE: return x != pr.a;
    case HX_PRED_MASK_EQ: return (x & pr.a) == pr.b;
    case HX_PRED_RANGE: return x >= pr.a && x < pr.b;
    default: return false;
  }
}
// 32-bit specialisation: MOD_LT on 32-bit data with a 32-bit divisor is the
// hot copy_if rule; keep it in 32-bit arithmetic.
__device__ __forceinline__ bool pred_on32(const hx_pred& pr, uint32_t x) {
  if (pr.op == HX_PRED_MOD_LT) return (x % (uint32_t)pr.a) < (uint32_t)pr.b;
  return pred_on(pr, (uint64_t)x);
}

// Context for pair predicates that look at the table (HX_PRED_NOT_HOME).
template <class P>
struct TableRef {
  const P* table;
  int sp;
};

template <class P>
__device__ __forceinline__ bool pred_pair(const hx_pred& pr, typename PairTraits<P>::K k,
                                          typename PairTraits<P>::V v, const TableRef<P>& t) {
  using Tr = PairTraits<P>;
  const bool sentinel = (k == Tr::EMPTY) || (k == Tr::TOMB);
  bool r;
  if (pr.op == HX_PRED_VALID) {
    r = !sentinel;
  } else if (pr.op == HX_PRED_NOT_HOME) {
    r = !sentinel && t.table != nullptr && t.table[home_slot(k, t.sp)].first != k;
  } else {
    const uint64_t x = (pr.field == HX_FIELD_VALUE) ? (uint64_t)v : (uint64_t)k;
    r = pred_on(pr, x);
    if ((pr.flags & HX_PRED_SKIP_SENTINELS) && sentinel) r = false;
  }
  if (pr.flags & HX_PRED_NEGATE) r = !r;
  return r;
}

// pred_pair for a bucket at index i of a table of 2^sp buckets: HX_PRED_NOT_HOME
// becomes "i is not the key's home bucket" — the same answer as reading the
// home bucket and finding another key there (every key occurs once), with no
// read of the table.
template <class P>
__device__ __forceinline__ bool pred_pair_at(const hx_pred& pr, typename PairTraits<P>::K k,
                                             typename PairTraits<P>::V v, uint64_t i, int sp) {
  if (pr.op != HX_PRED_NOT_HOME) return pred_pair<P>(pr, k, v, TableRef<P>{nullptr, sp});
  using Tr = PairTraits<P>;
  const bool sentinel = (k == Tr::EMPTY) || (k == Tr::TOMB);
  bool r = !sentinel && (uint64_t)home_slot(k, sp) != i;
  if (pr.flags & HX_PRED_NEGATE) r = !r;
  return r;
}

}  // namespace hx
