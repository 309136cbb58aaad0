// hx_map.cu — Hashinator::Hashmap accelerated API on device-resident tables.
//
// Kernels: insert (keys+values or pairs), retrieve (keys or pairs), erase,
// device rehash, clear, and the clean_tombstones pair (compaction in clean
// mode + re-insert). All hash kernels are persistent grid-stride kernels:
// a warp takes 32/G consecutive keys per step (one per probe group), so key
// loads are coalesced; fill / tombstone / probe-bound updates are reduced per
// warp and applied with one atomic per warp at kernel exit (the reference
// reduces per block, kernels_NVIDIA.h:411-440).
#include <cmath>
#include <cstring>
#include <mutex>
#include "hx_host.h"
#include "hx_internal.h"
#include "hx_probe.cuh"
#include "hx_scan.cuh"

namespace hx {

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

// Every bucket := (EMPTY, 0), 16 bytes per store.
template <class P>
__global__ void k_fill_empty(P* __restrict__ t, uint64_t nslots) {
  constexpr int PER = 16 / sizeof(P);
  const uint64_t n16 = nslots / PER;
  uint4 v;
  if constexpr (sizeof(P) == 8) v = make_uint4(0xFFFFFFFFu, 0u, 0xFFFFFFFFu, 0u);
  else v = make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u);
  uint4* p = reinterpret_cast<uint4*>(t);
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n16; i += (uint64_t)gridDim.x * blockDim.x)
    __stcs(p + i, v);
  // odd tail (nslots == 1 for an 8-byte pair table of size power 0 never
  // occurs: size power >= 1)
}

__global__ void k_info_reset(DInfo* info) {
  info->fill = 0;
  info->tombstones = 0;
  info->max_probe = 0;
  info->err = HX_STATUS_SUCCESS;
  info->moved = 0;
  info->skip = 0;
}

// clean_tombstones prologue: nothing to do without tombstones
// (hashinator.h:1264-1266); else tombstones := 0 and the probe bound restarts
// from the keys left in their home bucket (hashinator.h:1301).
__global__ void k_clean_prologue(DInfo* info) {
  const bool skip = info->tombstones == 0;
  info->skip = skip ? 1u : 0u;
  info->moved = 0;
  if (!skip) {
    info->tombstones = 0;
    info->max_probe = info->fill ? 1u : 0u;
  }
}

__device__ __forceinline__ void publish_counts(DInfo* info, unsigned ins, unsigned maxd, bool fail, int lane) {
  ins = __reduce_add_sync(0xffffffffu, ins);
  maxd = __reduce_max_sync(0xffffffffu, maxd);
  const bool anyfail = __any_sync(0xffffffffu, fail);
  if (lane == 0) {
    if (ins) atomicAdd(&info->fill, (unsigned long long)ins);
    if (maxd) atomicMax(&info->max_probe, maxd);
    if (anyfail) atomicExch(&info->err, HX_STATUS_FAIL);
  }
}

// insert(keys, vals) / insert(pairs) (kernels_NVIDIA.h:307-447, :143-283).
// n is read from *d_n when d_n is given (re-insert after clean_tombstones,
// whose count stays on the device).
template <class P, int G, int B, bool PAIRS>
__global__ void __launch_bounds__(256) k_insert(const typename PairTraits<P>::K* __restrict__ keys,
                                                const typename PairTraits<P>::V* __restrict__ vals,
                                                const P* __restrict__ pairs, uint64_t n,
                                                const unsigned long long* d_n, uint64_t n_cap, P* table, int sp,
                                                DInfo* info) {
  using K = typename PairTraits<P>::K;
  using V = typename PairTraits<P>::V;
  constexpr int GPW = 32 / G;
  if (d_n) {
    const uint64_t dn = *d_n;
    n = dn < n_cap ? dn : n_cap;
  }
  const int lane = threadIdx.x & 31;
  const unsigned gmask = group_mask<G>(lane);
  const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  unsigned ins = 0, maxd = 0;
  bool fail = false;
  for (uint64_t base = warp * GPW; base < n; base += nwarps * GPW) {
    const uint64_t i = base + (lane / G);
    if (i < n) {
      K key;
      V val;
      if constexpr (PAIRS) {
        const P pr = pairs[i];
        key = pr.first;
        val = pr.second;
      } else {
        key = keys[i];
        val = vals ? vals[i] : (V)i;  // no values: insertIndex
      }
      if (key != PairTraits<P>::EMPTY && key != PairTraits<P>::TOMB) {
        unsigned d1 = 0;
        const int r = probe_insert_live<P, G, B>(table, sp, key, val, lane, gmask, d1);
        if (d1) {
          ++ins;
          maxd = d1 > maxd ? d1 : maxd;
        }
        if (r == PR_FAIL && (lane & (G - 1)) == 0) fail = true;
      }
    }
  }
  publish_counts(info, ins, maxd, fail, lane);
}

// retrieve(keys, vals) / retrieve(pairs) (kernels_NVIDIA.h:727-774, :783-829).
// A missing key leaves its output untouched.
template <class P, int G, int B, bool PAIRS>
__global__ void __launch_bounds__(256) k_retrieve(const typename PairTraits<P>::K* __restrict__ keys,
                                                  typename PairTraits<P>::V* __restrict__ vals, P* pairs,
                                                  uint64_t n, const P* __restrict__ table, int sp,
                                                  const DInfo* __restrict__ info) {
  using K = typename PairTraits<P>::K;
  using V = typename PairTraits<P>::V;
  constexpr int GPW = 32 / G;
  const unsigned limit = info->max_probe;
  const int lane = threadIdx.x & 31;
  const unsigned gmask = group_mask<G>(lane);
  const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t base = warp * GPW; base < n; base += nwarps * GPW) {
    const uint64_t i = base + (lane / G);
    if (i < n) {
      K key;
      if constexpr (PAIRS) key = pairs[i].first;
      else key = keys[i];
      if (key != PairTraits<P>::EMPTY && key != PairTraits<P>::TOMB) {
        V v;
        const int w = probe_find_live<P, G, B>(table, sp, key, true, limit, lane, gmask, v);
        if (w >= 0 && (lane & (G - 1)) == w) {
          if constexpr (PAIRS) pairs[i].second = v;
          else vals[i] = v;
        }
      }
    }
  }
}

// erase(keys) (kernels_NVIDIA.h:622-718): key -> TOMBSTONE with a CAS, so a
// key repeated in one batch is erased and counted once.
template <class P, int G, int B>
__global__ void __launch_bounds__(256) k_erase(const typename PairTraits<P>::K* __restrict__ keys, uint64_t n,
                                               P* table, int sp, DInfo* info) {
  using K = typename PairTraits<P>::K;
  using V = typename PairTraits<P>::V;
  constexpr int GPW = 32 / G;
  const unsigned limit = info->max_probe;
  const int lane = threadIdx.x & 31;
  const unsigned gmask = group_mask<G>(lane);
  const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  unsigned erased = 0;
  for (uint64_t base = warp * GPW; base < n; base += nwarps * GPW) {
    const uint64_t i = base + (lane / G);
    if (i < n) {
      const K key = keys[i];
      if (key != PairTraits<P>::EMPTY && key != PairTraits<P>::TOMB) {
        uint32_t slot;
        V v;
        const int w = probe_find<P, G, B>(table, sp, key, limit, lane, gmask, slot, v);
        if (w >= 0 && (lane & (G - 1)) == w)
          if (cas_key(table + slot, key, PairTraits<P>::TOMB)) ++erased;
      }
    }
  }
  erased = __reduce_add_sync(0xffffffffu, erased);
  if (lane == 0 && erased) {
    atomicAdd(&info->tombstones, (unsigned long long)erased);
    atomicAdd(&info->fill, 0ull - (unsigned long long)erased);
  }
}

// ---- thread-per-key variants: U keys in flight per thread -----------------

// Publish (key, val) into bucket h, which is expected EMPTY. Every EMPTY
// bucket written by libhx holds value 0, so the first attempt needs no read
// of the bucket; a different stale value costs one retry.
template <class P>
__device__ __forceinline__ bool cas_empty(P* b, typename PairTraits<P>::K& ek, typename PairTraits<P>::V& ev,
                                          typename PairTraits<P>::K key, typename PairTraits<P>::V val) {
  ek = PairTraits<P>::EMPTY;
  ev = 0;
  return cas_pair(b, ek, ev, key, val);
}

// BLIND: CAS the home bucket first without reading it (EMPTY buckets hold
// (EMPTY, 0)); else load every key's first window, then CAS into it.
template <class P, int B, int U, bool PAIRS, bool BLIND>
__global__ void __launch_bounds__(256) k_insert_t1(const typename PairTraits<P>::K* __restrict__ keys,
                                                   const typename PairTraits<P>::V* __restrict__ vals,
                                                   const P* __restrict__ pairs, uint64_t n,
                                                   const unsigned long long* d_n, uint64_t n_cap, P* table,
                                                   int sp, DInfo* info) {
  using K = typename PairTraits<P>::K;
  using V = typename PairTraits<P>::V;
  constexpr K EMPTY = PairTraits<P>::EMPTY;
  if (d_n) {
    const uint64_t dn = *d_n;
    n = dn < n_cap ? dn : n_cap;
  }
  const int lane = threadIdx.x & 31;
  const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  unsigned ins = 0, maxd = 0;
  bool fail = false;
  for (uint64_t base = warp * 32 * U; base < n; base += nwarps * 32 * U) {
    K key[U];
    V val[U];
    bool act[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint64_t i = base + (uint64_t)u * 32 + lane;
      act[u] = i < n;
      if (act[u]) {
        if constexpr (PAIRS) {
          const P pr = pairs[i];
          key[u] = pr.first;
          val[u] = pr.second;
        } else {
          key[u] = keys[i];
          val[u] = vals ? vals[i] : (V)i;  // no values: insertIndex
        }
        act[u] = key[u] != EMPTY && key[u] != PairTraits<P>::TOMB;
      }
    }
    // A key repeated within the warp is inserted once, by its lowest lane: the
    // copies would only contend for the same bucket, and which of their values
    // wins is unspecified anyway (a batch with duplicate keys races in the
    // reference too). Measured: 2^20 keys plus 2^20 copies of one key insert
    // 10.9x faster, distinct keys at the same speed.
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const unsigned amask = __ballot_sync(0xffffffffu, act[u]);
      if (act[u]) {
        const unsigned same = __match_any_sync(amask, key[u]);
        if ((__ffs(same) - 1) != lane) act[u] = false;
      }
    }
    uint32_t h[U];
    if constexpr (!BLIND) {
      Window<P, B> w[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (act[u]) {
          h[u] = home_slot(key[u], sp);
          load_buckets<B>(table + (h[u] & ~(uint32_t)(B - 1)), w[u].k, w[u].v);
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (!act[u]) continue;
        unsigned d1 = 0;
        const int r = insert_t1_win<P, B>(table, sp, key[u], val[u], h[u], w[u], d1);
        if (r == PR_INSERTED) {
          ++ins;
          maxd = d1 > maxd ? d1 : maxd;
        } else if (r == PR_FAIL) {
          fail = true;
        }
      }
    } else {
      K ek[U];
      V ev[U];
      bool ok[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (act[u]) {
          h[u] = home_slot(key[u], sp);
          ok[u] = cas_empty<P>(table + h[u], ek[u], ev[u], key[u], val[u]);
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (!act[u]) continue;
        bool done = ok[u];
        if (done) {
          ++ins;
          maxd = maxd > 1u ? maxd : 1u;
          continue;
        }
        for (int tries = 0; tries < 8 && ek[u] == EMPTY; ++tries) {  // EMPTY with a stale value
          if (cas_pair(table + h[u], ek[u], ev[u], key[u], val[u])) {
            ++ins;
            maxd = maxd > 1u ? maxd : 1u;
            done = true;
            break;
          }
        }
        if (done) continue;
        if (ek[u] == key[u]) {
          store_value(table + h[u], val[u]);
          continue;
        }
        unsigned d1 = 0;
        const int r = insert_t1_rest<P, B>(table, sp, key[u], val[u], h[u], d1);
        if (r == PR_INSERTED) {
          ++ins;
          maxd = d1 > maxd ? d1 : maxd;
        } else if (r == PR_FAIL) {
          fail = true;
        }
      }
    }
  }
  publish_counts(info, ins, maxd, fail, lane);
}

template <class P, int B, int U, bool PAIRS, bool ERASE>
__global__ void __launch_bounds__(256) k_find_t1(const typename PairTraits<P>::K* __restrict__ keys,
                                                 typename PairTraits<P>::V* __restrict__ vals, P* pairs, uint64_t n,
                                                 P* table, int sp, DInfo* info) {
  using K = typename PairTraits<P>::K;
  using V = typename PairTraits<P>::V;
  const unsigned limit = info->max_probe;
  const int lane = threadIdx.x & 31;
  const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  unsigned erased = 0;
  if (limit) {
    for (uint64_t base = warp * 32 * U; base < n; base += nwarps * 32 * U) {
      K key[U];
      bool act[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const uint64_t i = base + (uint64_t)u * 32 + lane;
        act[u] = i < n;
        if (act[u]) {
          if constexpr (PAIRS) key[u] = pairs[i].first;
          else key[u] = keys[i];
          act[u] = key[u] != PairTraits<P>::EMPTY && key[u] != PairTraits<P>::TOMB;
        }
      }
      uint32_t h[U];
      Window<P, B> w[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (act[u]) {
          h[u] = home_slot(key[u], sp);
          load_buckets<B>(table + (h[u] & ~(uint32_t)(B - 1)), w[u].k, w[u].v);
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (!act[u]) continue;
        uint32_t slot;
        V v;
        if (find_t1<P, B>(table, sp, key[u], limit, h[u], w[u], slot, v)) {
          if constexpr (ERASE) {
            if (cas_key(table + slot, key[u], PairTraits<P>::TOMB)) ++erased;
          } else {
            const uint64_t i = base + (uint64_t)u * 32 + lane;
            if constexpr (PAIRS) pairs[i].second = v;
            else vals[i] = v;
          }
        }
      }
    }
  }
  if constexpr (ERASE) {
    erased = __reduce_add_sync(0xffffffffu, erased);
    if (lane == 0 && erased) {
      atomicAdd(&info->tombstones, (unsigned long long)erased);
      atomicAdd(&info->fill, 0ull - (unsigned long long)erased);
    }
  }
}

// device_rehash (hashinator.h:285-336) in one pass: one thread per old
// bucket inserts its valid pair into the new table.
template <class P, int B>
__global__ void __launch_bounds__(256) k_rehash(const P* __restrict__ old_t, uint64_t old_n, P* new_t, int new_sp,
                                                DInfo* info) {
  using K = typename PairTraits<P>::K;
  const int lane = threadIdx.x & 31;
  unsigned ins = 0, maxd = 0;
  bool fail = false;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t base = blockIdx.x * (uint64_t)blockDim.x; base < old_n; base += stride) {
    const uint64_t i = base + threadIdx.x;
    if (i < old_n) {
      const P pr = old_t[i];
      const K key = pr.first;
      if (key != PairTraits<P>::EMPTY && key != PairTraits<P>::TOMB) {
        unsigned d1 = 0;
        const int r = probe_insert<P, 1, B>(new_t, new_sp, key, pr.second, lane, 1u << lane, d1);
        if (d1) {
          ++ins;
          maxd = d1 > maxd ? d1 : maxd;
        }
        if (r == PR_FAIL) fail = true;
      }
    }
  }
  publish_counts(info, ins, maxd, fail, lane);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

}  // namespace hx

namespace hx {

static inline bool is_p32(const hx_map* m) { return m->key_bytes == 4; }
static inline uint64_t pair_bytes(const hx_map* m) { return is_p32(m) ? 8 : 16; }
static inline unsigned key_bytes(const hx_map* m) { return is_p32(m) ? 4u : 8u; }
static inline uint64_t nslots(const hx_map* m) { return 1ull << m->sp; }

// Automatic probe policy (tune.group == 0), from GB300 sweeps over
// G x keys-per-thread at load factors 0.5 - 0.9 (2^27 buckets, u32 and u64):
//   insert:  one thread per key, blind home CAS, 1 key per thread, unless
//            the insert ends above load factor 0.85: then 4-lane groups
//            (u32 11.9 vs 10.9, u64 7.1 vs 6.9 G keys/s at 0.9);
//   query:   probe groups with the single-exit probe loop: u32 tables use
//            4 lanes (64 B windows) below load factor 0.875 and 8 above (31.6
//            vs 29.8 G keys/s for thread-per-key at 0.5, 7.9 vs 6.7 for 32
//            lanes at 0.9); u64 tables 4 lanes below 0.8, 8 to 0.875, 16 above
//            (24.8 vs 21.1 G keys/s for thread-per-key at 0.5, 12.9 vs 10.6 for
//            16 lanes at 0.75);
//   erase:   one thread per key with 2 keys in flight at every load factor
//            (erased keys are usually present, so a probe ends at the key,
//            not at the end of a long run; 1.1-2.7x faster than groups).
enum class Op { INSERT, QUERY, ERASE };
struct Geo {
  int G, B;
};
struct Policy {
  int G, U;
};
static Policy auto_policy(const hx_map* m, Op op) {
  if (op == Op::INSERT) {
    // fill_ub already counts this call's keys: the load factor the insert ends at
    const double lf_end = (double)m->fill_ub / (double)nslots(m);
    return lf_end < 0.85 ? Policy{1, 1} : Policy{4, 1};
  }
  if (op == Op::ERASE) return {1, 2};
  const double lf = (double)m->fill_ub / (double)nslots(m);
  const bool p32 = is_p32(m);
  if (p32) return lf < 0.875 ? Policy{4, 1} : Policy{8, 1};
  if (lf < 0.8) return {4, 1};
  return lf < 0.875 ? Policy{8, 1} : Policy{16, 1};
}
static Policy policy(const hx_map* m, Op op) {
  if (m->tune.group == 0) return auto_policy(m, op);
  return {m->tune.group, m->tune.unroll};
}

// Probe-group geometry for a table: (G, B) with G*B <= table size.
static Geo pick_geo(const hx_map* m, int G) {
  const bool p32 = is_p32(m);
  if (G == 1) return {1, 0};  // thread-per-key kernels pick their own window
  int B = p32 ? 2 : 1;
  if ((uint64_t)G * B > nslots(m)) {
    // a window larger than the table: the smallest group window that fits
    if (p32 && nslots(m) >= 4) return {2, 2};
    return {2, 1};
  }
  return {G, B};
}

template <class F>
static unsigned grid_for(F kernel, uint64_t work_threads, int block) {
  const uint64_t want = (work_threads + block - 1) / block;
  const uint64_t cap = (uint64_t)sm_count() * blocks_per_sm(kernel, block);
  const uint64_t g = want < cap ? want : cap;
  return (unsigned)(g ? g : 1);
}

// Dispatch a probe-group kernel template over the compiled (G, B) variants
// (G >= 2; a table smaller than one window falls back to G = 2, B = 1).
#define HX_GEO_DISPATCH(P, geo, LAUNCH)                                        \
  do {                                                                         \
    if constexpr (sizeof(P) == 8) {                                            \
      if (geo.B == 1) { LAUNCH(P, 2, 1); }                                     \
      else if (geo.G == 2) { LAUNCH(P, 2, 2); }                                \
      else if (geo.G == 4) { LAUNCH(P, 4, 2); }                                \
      else if (geo.G == 8) { LAUNCH(P, 8, 2); }                                \
      else if (geo.G == 16) { LAUNCH(P, 16, 2); }                              \
      else { LAUNCH(P, 32, 2); }                                               \
    } else {                                                                   \
      if (geo.G == 2) { LAUNCH(P, 2, 1); }                                     \
      else if (geo.G == 4) { LAUNCH(P, 4, 1); }                                \
      else if (geo.G == 8) { LAUNCH(P, 8, 1); }                                \
      else if (geo.G == 16) { LAUNCH(P, 16, 1); }                              \
      else { LAUNCH(P, 32, 1); }                                               \
    }                                                                          \
  } while (0)

// Thread-per-key geometry: B buckets (32 B) per window, U keys per thread.
// A 2-bucket u32 table uses B = 2 with U = 1.
#define HX_T1_DISPATCH(P, tsize, U, WIDE, LAUNCH)                \
  do {                                                           \
    if constexpr (sizeof(P) == 8) {                              \
      if (tsize < 4) { LAUNCH(P, 2, 1); }                        \
      else if (WIDE && tsize >= 8) {                             \
        if (U >= 4) { LAUNCH(P, 8, 4); }                         \
        else if (U >= 2) { LAUNCH(P, 8, 2); }                    \
        else { LAUNCH(P, 8, 1); }                                \
      }                                                          \
      else if (U >= 8) { LAUNCH(P, 4, 8); }                      \
      else if (U >= 4) { LAUNCH(P, 4, 4); }                      \
      else if (U >= 2) { LAUNCH(P, 4, 2); }                      \
      else { LAUNCH(P, 4, 1); }                                  \
    } else {                                                     \
      if (WIDE && tsize >= 4) {                                  \
        if (U >= 4) { LAUNCH(P, 4, 4); }                         \
        else if (U >= 2) { LAUNCH(P, 4, 2); }                    \
        else { LAUNCH(P, 4, 1); }                                \
      }                                                          \
      else if (U >= 8) { LAUNCH(P, 2, 8); }                      \
      else if (U >= 4) { LAUNCH(P, 2, 4); }                      \
      else if (U >= 2) { LAUNCH(P, 2, 2); }                      \
      else { LAUNCH(P, 2, 1); }                                  \
    }                                                            \
  } while (0)

template <class P>
static hx_status launch_insert(hx_map* m, const void* keys, const void* vals, const void* pairs, uint64_t n,
                               const unsigned long long* d_n, cudaStream_t s) {
  using K = typename PairTraits<P>::K;
  using V = typename PairTraits<P>::V;
  // clean_tombstones re-inserts its moved keys (count on the device) into a
  // table whose fill bound still counts the erased keys: thread-per-key, and
  // reading the window before any CAS. A moved key left its home because the
  // home was taken, and mostly still is, so a blind first CAS at home would
  // mostly fail: window-first took clean on 2^27 buckets from 0.91 to 0.75 ms
  // (u32, LF 0.5), 2.05 to 1.62 ms (u32, LF 0.9) and 1.43 to 1.18 ms (u64, LF 0.5).
  const Policy pol = (d_n && m->tune.group == 0) ? Policy{1, 1} : policy(m, Op::INSERT);
  const bool blind = d_n ? false : m->tune.blind;
  const Geo geo = pick_geo(m, pol.G);
  const int block = m->tune.block;
  if (geo.G == 1) {
    const int U = pol.U;
#define HX_LAUNCH_INSERT_T1_B(PP, BB, UU, BL)                                                                     \
  {                                                                                                              \
    if (pairs) {                                                                                                 \
      auto kern = k_insert_t1<PP, BB, UU, true, BL>;                                                             \
      kern<<<grid_for(kern, (n + UU - 1) / UU, block), block, 0, s>>>(                                           \
          nullptr, nullptr, static_cast<const PP*>(pairs), n, d_n, n, static_cast<PP*>(m->buckets), m->sp,        \
          m->info);                                                                                              \
    } else {                                                                                                     \
      auto kern = k_insert_t1<PP, BB, UU, false, BL>;                                                            \
      kern<<<grid_for(kern, (n + UU - 1) / UU, block), block, 0, s>>>(                                           \
          static_cast<const K*>(keys), static_cast<const V*>(vals), nullptr, n, d_n, n,                          \
          static_cast<PP*>(m->buckets), m->sp, m->info);                                                         \
    }                                                                                                            \
  }
#define HX_LAUNCH_INSERT_T1(PP, BB, UU)                   \
  {                                                       \
    if (blind) HX_LAUNCH_INSERT_T1_B(PP, BB, UU, true)    \
    else HX_LAUNCH_INSERT_T1_B(PP, BB, UU, false)         \
  }
    HX_T1_DISPATCH(P, nslots(m), U, m->tune.wide, HX_LAUNCH_INSERT_T1);
#undef HX_LAUNCH_INSERT_T1
#undef HX_LAUNCH_INSERT_T1_B
    return after_launch();
  }
#define HX_LAUNCH_INSERT(PP, GG, BB)                                                                      \
  {                                                                                                       \
    if (pairs) {                                                                                          \
      auto kern = k_insert<PP, GG, BB, true>;                                                             \
      kern<<<grid_for(kern, n * GG, block), block, 0, s>>>(nullptr, nullptr, static_cast<const PP*>(pairs), \
                                                           n, d_n, n, static_cast<PP*>(m->buckets), m->sp,  \
                                                           m->info);                                      \
    } else {                                                                                              \
      auto kern = k_insert<PP, GG, BB, false>;                                                            \
      kern<<<grid_for(kern, n * GG, block), block, 0, s>>>(static_cast<const K*>(keys),                     \
                                                           static_cast<const V*>(vals), nullptr, n, d_n, n,  \
                                                           static_cast<PP*>(m->buckets), m->sp, m->info);    \
    }                                                                                                     \
  }
  HX_GEO_DISPATCH(P, geo, HX_LAUNCH_INSERT);
#undef HX_LAUNCH_INSERT
  return after_launch();
}

// retrieve (keys or pairs) and erase share the lookup kernels.
template <class P, bool ERASE>
static hx_status launch_find(hx_map* m, const void* keys, void* vals, void* pairs, uint64_t n, cudaStream_t s) {
  using K = typename PairTraits<P>::K;
  using V = typename PairTraits<P>::V;
  const Policy pol = policy(m, ERASE ? Op::ERASE : Op::QUERY);
  const Geo geo = pick_geo(m, pol.G);
  const int block = m->tune.block;
  if (geo.G == 1) {
    const int U = pol.U;
#define HX_LAUNCH_FIND_T1(PP, BB, UU)                                                                            \
  {                                                                                                              \
    if (pairs) {                                                                                                 \
      auto kern = k_find_t1<PP, BB, UU, true, ERASE>;                                                            \
      kern<<<grid_for(kern, (n + UU - 1) / UU, block), block, 0, s>>>(nullptr, nullptr, static_cast<PP*>(pairs), \
                                                                      n, static_cast<PP*>(m->buckets), m->sp,    \
                                                                      m->info);                                  \
    } else {                                                                                                     \
      auto kern = k_find_t1<PP, BB, UU, false, ERASE>;                                                           \
      kern<<<grid_for(kern, (n + UU - 1) / UU, block), block, 0, s>>>(                                           \
          static_cast<const K*>(keys), static_cast<V*>(vals), nullptr, n, static_cast<PP*>(m->buckets), m->sp,   \
          m->info);                                                                                              \
    }                                                                                                            \
  }
    HX_T1_DISPATCH(P, nslots(m), U, m->tune.wide, HX_LAUNCH_FIND_T1);
#undef HX_LAUNCH_FIND_T1
    return after_launch();
  }
  if constexpr (ERASE) {
#define HX_LAUNCH_ERASE(PP, GG, BB)                                                                        \
  {                                                                                                        \
    auto kern = k_erase<PP, GG, BB>;                                                                       \
    kern<<<grid_for(kern, n * GG, block), block, 0, s>>>(static_cast<const K*>(keys), n,                    \
                                                         static_cast<PP*>(m->buckets), m->sp, m->info);    \
  }
    HX_GEO_DISPATCH(P, geo, HX_LAUNCH_ERASE);
#undef HX_LAUNCH_ERASE
  } else {
#define HX_LAUNCH_RETRIEVE(PP, GG, BB)                                                                      \
  {                                                                                                         \
    if (pairs) {                                                                                            \
      auto kern = k_retrieve<PP, GG, BB, true>;                                                             \
      kern<<<grid_for(kern, n * GG, block), block, 0, s>>>(nullptr, nullptr, static_cast<PP*>(pairs), n,     \
                                                           static_cast<const PP*>(m->buckets), m->sp, m->info); \
    } else {                                                                                                \
      auto kern = k_retrieve<PP, GG, BB, false>;                                                            \
      kern<<<grid_for(kern, n * GG, block), block, 0, s>>>(static_cast<const K*>(keys), static_cast<V*>(vals), \
                                                           nullptr, n, static_cast<const PP*>(m->buckets),   \
                                                           m->sp, m->info);                                 \
    }                                                                                                       \
  }
    HX_GEO_DISPATCH(P, geo, HX_LAUNCH_RETRIEVE);
#undef HX_LAUNCH_RETRIEVE
  }
  return after_launch();
}

template <class P>
static hx_status launch_fill_empty(void* t, uint64_t n, cudaStream_t s) {
  auto kern = k_fill_empty<P>;
  const uint64_t n16 = n * sizeof(P) / 16;
  kern<<<grid_for(kern, n16, 256), 256, 0, s>>>(static_cast<P*>(t), n);
  return after_launch();
}

static hx_status fill_empty(hx_map* m, void* t, uint64_t n, cudaStream_t s) {
  if (n * pair_bytes(m) < 16) {  // a 2-bucket u32 table: 16 B, always >= 16
    return HX_ERR_INVALID_ARG;
  }
  return is_p32(m) ? launch_fill_empty<P32>(t, n, s) : launch_fill_empty<P64>(t, n, s);
}

static hx_status ensure_scratch(hx_map* m, uint64_t bytes, cudaStream_t s) {
  if (m->scratch_bytes >= bytes) return HX_OK;
  if (m->scratch) HX_CUDA(cudaFreeAsync(m->scratch, s));
  m->scratch = nullptr;
  m->scratch_bytes = 0;
  uint64_t b = 1;
  while (b < bytes) b <<= 1;
  HX_CUDA(cudaMallocAsync(&m->scratch, b, s));
  m->scratch_bytes = b;
  return HX_OK;
}

static hx_status read_info(hx_map* m, DInfo* out, cudaStream_t s) {
  HX_CUDA(cudaMemcpyAsync(out, m->info, sizeof(DInfo), cudaMemcpyDeviceToHost, s));
  HX_CUDA(cudaStreamSynchronize(s));
  m->fill_ub = out->fill;
  return HX_OK;
}

// device_rehash to new_sp: allocate, (EMPTY,0)-fill, one streaming re-insert
// pass, swap. fill is preserved; tombstones and the probe bound restart.
static hx_status rehash(hx_map* m, int new_sp, cudaStream_t s) {
  if (new_sp < 1 || new_sp > 31) return HX_ERR_INVALID_ARG;
  const uint64_t nn = 1ull << new_sp;
  void* nt = nullptr;
  HX_CUDA(cudaMallocAsync(&nt, nn * pair_bytes(m), s));
  hx_status st = fill_empty(m, nt, nn, s);
  if (st != HX_OK) return st;
  k_info_reset<<<1, 1, 0, s>>>(m->info);
  if ((st = after_launch()) != HX_OK) return st;
  const uint64_t on = nslots(m);
  if (is_p32(m)) {
    auto kern = k_rehash<P32, 4>;
    const bool small = nn < 4;
    if (small) {
      auto k1 = k_rehash<P32, 1>;
      k1<<<grid_for(k1, on, 256), 256, 0, s>>>(static_cast<const P32*>(m->buckets), on, static_cast<P32*>(nt),
                                               new_sp, m->info);
    } else {
      kern<<<grid_for(kern, on, 256), 256, 0, s>>>(static_cast<const P32*>(m->buckets), on, static_cast<P32*>(nt),
                                                   new_sp, m->info);
    }
  } else {
    auto kern = k_rehash<P64, 2>;
    kern<<<grid_for(kern, on, 256), 256, 0, s>>>(static_cast<const P64*>(m->buckets), on, static_cast<P64*>(nt),
                                                 new_sp, m->info);
  }
  if ((st = after_launch()) != HX_OK) return st;
  HX_CUDA(cudaFreeAsync(m->buckets, s));
  m->buckets = nt;
  m->sp = new_sp;
  return HX_OK;
}

// Growth rule of insert (hashinator.h:1329-1332):
// ceil(log2((fill + len) / targetLF)) > sizePower -> device_rehash.
// Decided on the host upper bound of fill; only when that bound asks for
// growth is the exact fill read back.
static hx_status maybe_grow(hx_map* m, uint64_t n, float target_lf, cudaStream_t s) {
  if (!(target_lf > 0.0f)) return HX_OK;
  auto needed = [&](uint64_t fill) -> long long {
    return (long long)std::ceil(std::log2((double)(fill + n) * (1.0 / (double)target_lf)));
  };
  if (needed(m->fill_ub) <= m->sp) return HX_OK;
  DInfo di;
  hx_status st = read_info(m, &di, s);
  if (st != HX_OK) return st;
  const long long want = needed(di.fill);
  if (want <= m->sp) return HX_OK;
  if (want > 31) return HX_ERR_INVALID_ARG;
  return rehash(m, (int)want, s);
}

static bool valid_map(const hx_map* m) { return m && m->buckets && m->info; }

hx_status map_rehash_view(hx_map* m, int new_sp, cudaStream_t s) { return rehash(m, new_sp, s); }

hx_status map_insert_view(hx_map* m, const void* keys, const void* vals, const void* pairs, uint64_t n,
                          cudaStream_t s) {
  m->fill_ub += n;
  return is_p32(m) ? launch_insert<P32>(m, keys, vals, pairs, n, nullptr, s)
                   : launch_insert<P64>(m, keys, vals, pairs, n, nullptr, s);
}

hx_status map_find_view(hx_map* m, const void* keys, void* vals, void* pairs, uint64_t n, bool erase,
                        cudaStream_t s) {
  if (erase)
    return is_p32(m) ? launch_find<P32, true>(m, keys, vals, pairs, n, s) : launch_find<P64, true>(m, keys, vals, pairs, n, s);
  return is_p32(m) ? launch_find<P32, false>(m, keys, vals, pairs, n, s)
                   : launch_find<P64, false>(m, keys, vals, pairs, n, s);
}

}  // namespace hx

using namespace hx;

// extractPattern (KEYS = false) and extractKeysByPattern (KEYS = true): one
// order-preserving compaction pass over the bucket array.
template <bool KEYS>
static hx_status extract(hx_map* m, const hx_pred* pred, void* d_out, uint64_t capacity, uint64_t* d_count,
                         uint64_t* h_count, hx_stream stream) {
  if (!valid_map(m) || !pred) return HX_ERR_INVALID_ARG;
  if (pred->op > HX_PRED_NOT_HOME || (pred->op == HX_PRED_MOD_LT && pred->a == 0)) return HX_ERR_INVALID_ARG;
  if (capacity && !d_out) return HX_ERR_INVALID_ARG;
  if (misaligned(d_out, KEYS ? key_bytes(m) : pair_bytes(m))) return HX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  std::lock_guard<std::mutex> g(m->mu);
  const uint64_t n = nslots(m);
  const bool p32 = is_p32(m);
  const uint64_t need = p32 ? compact_scratch_need<P32>(n) : compact_scratch_need<P64>(n);
  const uint64_t sc_bytes = (need + 255) / 256 * 256;
  hx_status st = ensure_scratch(m, sc_bytes + 256, s);
  if (st != HX_OK) return st;
  unsigned long long* cnt = d_count ? reinterpret_cast<unsigned long long*>(d_count)
                                    : reinterpret_cast<unsigned long long*>(static_cast<char*>(m->scratch) + sc_bytes);
  cudaError_t e;
  CleanArgs cl{nullptr, nullptr};
  bool sk = false;
  if (p32) {
    using O = typename std::conditional<KEYS, uint32_t, P32>::type;
    e = launch_compact<P32, false, O>(static_cast<const P32*>(m->buckets), static_cast<O*>(d_out), n, *pred,
                                      TableRef<P32>{static_cast<const P32*>(m->buckets), m->sp}, capacity, cnt,
                                      m->scratch, cl, s, &sk);
  } else {
    using O = typename std::conditional<KEYS, uint64_t, P64>::type;
    e = launch_compact<P64, false, O>(static_cast<const P64*>(m->buckets), static_cast<O*>(d_out), n, *pred,
                                      TableRef<P64>{static_cast<const P64*>(m->buckets), m->sp}, capacity, cnt,
                                      m->scratch, cl, s, &sk);
  }
  if (e != cudaSuccess) return cuda_status(e);
  if ((st = after_launch()) != HX_OK) return st;
  if (h_count) {
    unsigned long long c = 0;
    unsigned int err = 0;
    HX_CUDA(cudaMemcpyAsync(&c, cnt, sizeof(c), cudaMemcpyDeviceToHost, s));
    HX_CUDA(cudaMemcpyAsync(&err, scan_error_word(m->scratch, sk), sizeof(err), cudaMemcpyDeviceToHost, s));
    HX_CUDA(cudaStreamSynchronize(s));
    *h_count = c;
    if (err) return HX_ERR_TIMEOUT;
    if (c > capacity) return HX_ERR_CAPACITY;
  }
  return HX_OK;
}

extern "C" {

hx_status hx_map_create(hx_map** out, int key_bytes, int val_bytes, int size_power, hx_stream stream) {
  if (!out) return HX_ERR_INVALID_ARG;
  *out = nullptr;
  if (!((key_bytes == 4 && val_bytes == 4) || (key_bytes == 8 && val_bytes == 8))) return HX_ERR_INVALID_ARG;
  if (size_power < 1 || size_power > 31) return HX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  hx_map* m = new hx_map();
  m->key_bytes = key_bytes;
  m->val_bytes = val_bytes;
  m->sp = size_power;
  cudaGetDevice(&m->device);
  auto fail = [&](hx_status st) {
    if (m->buckets) cudaFree(m->buckets);
    if (m->info) cudaFree(m->info);
    delete m;
    return st;
  };
  cudaError_t e = cudaMalloc(&m->buckets, nslots(m) * pair_bytes(m));
  if (e != cudaSuccess) return fail(cuda_status(e));
  e = cudaMalloc(reinterpret_cast<void**>(&m->info), sizeof(DInfo));
  if (e != cudaSuccess) return fail(cuda_status(e));
  hx_status st = fill_empty(m, m->buckets, nslots(m), s);
  if (st != HX_OK) return fail(st);
  k_info_reset<<<1, 1, 0, s>>>(m->info);
  if ((st = after_launch()) != HX_OK) return fail(st);
  // A fresh map reports status::invalid until its first insert
  // (Info(int) constructor, defaults.h:47-49).
  int inv = HX_STATUS_INVALID;
  e = cudaMemcpyAsync(&m->info->err, &inv, sizeof(int), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(cuda_status(e));
  *out = m;
  return HX_OK;
}

hx_status hx_map_destroy(hx_map* m) {
  if (!m) return HX_ERR_INVALID_ARG;
  cudaError_t e = cudaDeviceSynchronize();
  if (m->buckets) cudaFree(m->buckets);
  if (m->info) cudaFree(m->info);
  if (m->scratch) cudaFree(m->scratch);
  delete m;
  return e == cudaSuccess ? HX_OK : cuda_status(e);
}

hx_status hx_insert(hx_map* m, const void* d_keys, const void* d_vals, uint64_t n, float target_lf,
                    hx_stream stream) {
  HX_RANGE("hx_insert");
  if (!valid_map(m)) return HX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  HX_CUDA(cudaMemsetAsync(&m->info->err, 0, sizeof(int), s));  // err = success (hashers.h:50)
  if (n == 0) return HX_OK;
  if (!d_keys || !d_vals) return HX_ERR_INVALID_ARG;
  if (misaligned(d_keys, key_bytes(m)) || misaligned(d_vals, key_bytes(m))) return HX_ERR_INVALID_ARG;
  hx_status st = maybe_grow(m, n, target_lf, s);
  if (st != HX_OK) return st;
  HX_CUDA(cudaMemsetAsync(&m->info->err, 0, sizeof(int), s));
  m->fill_ub += n;
  return is_p32(m) ? launch_insert<P32>(m, d_keys, d_vals, nullptr, n, nullptr, s)
                   : launch_insert<P64>(m, d_keys, d_vals, nullptr, n, nullptr, s);
}

hx_status hx_insert_index(hx_map* m, const void* d_keys, uint64_t n, float target_lf, hx_stream stream) {
  HX_RANGE("hx_insert_index");
  if (!valid_map(m)) return HX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  HX_CUDA(cudaMemsetAsync(&m->info->err, 0, sizeof(int), s));
  if (n == 0) return HX_OK;
  if (!d_keys) return HX_ERR_INVALID_ARG;
  if (misaligned(d_keys, key_bytes(m))) return HX_ERR_INVALID_ARG;
  hx_status st = maybe_grow(m, n, target_lf, s);
  if (st != HX_OK) return st;
  HX_CUDA(cudaMemsetAsync(&m->info->err, 0, sizeof(int), s));
  m->fill_ub += n;
  return is_p32(m) ? launch_insert<P32>(m, d_keys, nullptr, nullptr, n, nullptr, s)
                   : launch_insert<P64>(m, d_keys, nullptr, nullptr, n, nullptr, s);
}

hx_status hx_insert_pairs(hx_map* m, const void* d_pairs, uint64_t n, float target_lf, hx_stream stream) {
  HX_RANGE("hx_insert_pairs");
  if (!valid_map(m)) return HX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  HX_CUDA(cudaMemsetAsync(&m->info->err, 0, sizeof(int), s));
  if (n == 0) return HX_OK;
  if (!d_pairs) return HX_ERR_INVALID_ARG;
  if (misaligned(d_pairs, pair_bytes(m))) return HX_ERR_INVALID_ARG;
  hx_status st = maybe_grow(m, n, target_lf, s);
  if (st != HX_OK) return st;
  HX_CUDA(cudaMemsetAsync(&m->info->err, 0, sizeof(int), s));
  m->fill_ub += n;
  return is_p32(m) ? launch_insert<P32>(m, nullptr, nullptr, d_pairs, n, nullptr, s)
                   : launch_insert<P64>(m, nullptr, nullptr, d_pairs, n, nullptr, s);
}

hx_status hx_retrieve(hx_map* m, const void* d_keys, void* d_vals, uint64_t n, hx_stream stream) {
  HX_RANGE("hx_retrieve");
  if (!valid_map(m)) return HX_ERR_INVALID_ARG;
  if (n == 0) return HX_OK;
  if (!d_keys || !d_vals) return HX_ERR_INVALID_ARG;
  if (misaligned(d_keys, key_bytes(m)) || misaligned(d_vals, key_bytes(m))) return HX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return is_p32(m) ? launch_find<P32, false>(m, d_keys, d_vals, nullptr, n, s)
                   : launch_find<P64, false>(m, d_keys, d_vals, nullptr, n, s);
}

hx_status hx_retrieve_pairs(hx_map* m, void* d_pairs, uint64_t n, hx_stream stream) {
  HX_RANGE("hx_retrieve_pairs");
  if (!valid_map(m)) return HX_ERR_INVALID_ARG;
  if (n == 0) return HX_OK;
  if (!d_pairs) return HX_ERR_INVALID_ARG;
  if (misaligned(d_pairs, pair_bytes(m))) return HX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return is_p32(m) ? launch_find<P32, false>(m, nullptr, nullptr, d_pairs, n, s)
                   : launch_find<P64, false>(m, nullptr, nullptr, d_pairs, n, s);
}

hx_status hx_erase(hx_map* m, const void* d_keys, uint64_t n, hx_stream stream) {
  HX_RANGE("hx_erase");
  if (!valid_map(m)) return HX_ERR_INVALID_ARG;
  if (n == 0) return HX_OK;
  if (!d_keys) return HX_ERR_INVALID_ARG;
  if (misaligned(d_keys, key_bytes(m))) return HX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return is_p32(m) ? launch_find<P32, true>(m, d_keys, nullptr, nullptr, n, s)
                   : launch_find<P64, true>(m, d_keys, nullptr, nullptr, n, s);
}

hx_status hx_clean_tombstones(hx_map* m, hx_stream stream) {
  HX_RANGE("hx_clean_tombstones");
  if (!valid_map(m)) return HX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  std::lock_guard<std::mutex> g(m->mu);
  const uint64_t n = nslots(m);
  const bool p32 = is_p32(m);
  const uint64_t need = p32 ? compact_scratch_need<P32>(n) : compact_scratch_need<P64>(n);
  const uint64_t sc_bytes = (need + 255) / 256 * 256;
  const uint64_t cap = m->fill_ub < n ? m->fill_ub : n;  // moved keys <= fill <= fill_ub
  hx_status st = ensure_scratch(m, sc_bytes + (cap + 1) * pair_bytes(m), s);
  if (st != HX_OK) return st;
  void* scan_sc = m->scratch;
  void* list = static_cast<char*>(m->scratch) + sc_bytes;
  k_clean_prologue<<<1, 1, 0, s>>>(m->info);
  if ((st = after_launch()) != HX_OK) return st;
  hx_pred pr{};
  pr.op = HX_PRED_NOT_HOME;
  CleanArgs cl{&m->info->skip, &m->info->fill};
  cudaError_t e;
  if (p32) {
    e = launch_compact<P32, true>(static_cast<const P32*>(m->buckets), static_cast<P32*>(list), n, pr,
                                  TableRef<P32>{static_cast<const P32*>(m->buckets), m->sp}, cap, &m->info->moved,
                                  scan_sc, cl, s);
  } else {
    e = launch_compact<P64, true>(static_cast<const P64*>(m->buckets), static_cast<P64*>(list), n, pr,
                                  TableRef<P64>{static_cast<const P64*>(m->buckets), m->sp}, cap, &m->info->moved,
                                  scan_sc, cl, s);
  }
  if (e != cudaSuccess) return cuda_status(e);
  if ((st = after_launch()) != HX_OK) return st;
  // Re-insert the moved keys; their count stays on the device.
  return p32 ? launch_insert<P32>(m, nullptr, nullptr, list, cap, &m->info->moved, s)
             : launch_insert<P64>(m, nullptr, nullptr, list, cap, &m->info->moved, s);
}

hx_status hx_extract_pattern(hx_map* m, const hx_pred* pred, void* d_out, uint64_t capacity, uint64_t* d_count,
                             uint64_t* h_count, hx_stream stream) {
  HX_RANGE("hx_extract_pattern");
  return extract<false>(m, pred, d_out, capacity, d_count, h_count, stream);
}

hx_status hx_extract_keys(hx_map* m, const hx_pred* pred, void* d_out_keys, uint64_t capacity, uint64_t* d_count,
                          uint64_t* h_count, hx_stream stream) {
  HX_RANGE("hx_extract_keys");
  return extract<true>(m, pred, d_out_keys, capacity, d_count, h_count, stream);
}

hx_status hx_resize(hx_map* m, int new_size_power, hx_stream stream) {
  HX_RANGE("hx_resize");
  if (!valid_map(m)) return HX_ERR_INVALID_ARG;
  return rehash(m, new_size_power, static_cast<cudaStream_t>(stream));
}

hx_status hx_clear(hx_map* m, hx_stream stream) {
  HX_RANGE("hx_clear");
  if (!valid_map(m)) return HX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  hx_status st = fill_empty(m, m->buckets, nslots(m), s);
  if (st != HX_OK) return st;
  k_info_reset<<<1, 1, 0, s>>>(m->info);
  m->fill_ub = 0;
  return after_launch();
}

hx_status hx_resize_to_lf(hx_map* m, float target_lf, hx_stream stream) {
  HX_RANGE("hx_resize_to_lf");
  if (!valid_map(m) || !(target_lf > 0.0f)) return HX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  DInfo di;
  hx_status st = read_info(m, &di, s);
  if (st != HX_OK) return st;
  int sp = m->sp;
  while ((float)di.fill / (float)(1ull << sp) > target_lf) {  // load_factor() > targetLF
    if (++sp > 31) return HX_ERR_OOM;
  }
  return sp == m->sp ? HX_OK : rehash(m, sp, s);
}

hx_status hx_perform_cleanup_tasks(hx_map* m, hx_stream stream) {
  HX_RANGE("hx_perform_cleanup_tasks");
  if (!valid_map(m)) return HX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  DInfo di;
  hx_status st = read_info(m, &di, s);
  if (st != HX_OK) return st;
  if (di.tombstones && (float)di.tombstones / (float)nslots(m) > 0.025f) {  // tombstone_ratio() > 0.025
    if ((st = hx_clean_tombstones(m, stream)) != HX_OK) return st;
    if ((st = read_info(m, &di, s)) != HX_OK) return st;
  }
  // currentMaxBucketOverflow > BUCKET_OVERFLOW: grow until the probe bound fits one 32-bucket window
  while (di.max_probe > 32 && m->sp < 31) {
    if ((st = rehash(m, m->sp + 1, s)) != HX_OK) return st;
    if ((st = read_info(m, &di, s)) != HX_OK) return st;
  }
  return HX_OK;
}

hx_status hx_get_info(hx_map* m, hx_info* out, hx_stream stream) {
  HX_RANGE("hx_get_info");
  if (!valid_map(m) || !out) return HX_ERR_INVALID_ARG;
  DInfo di;
  hx_status st = read_info(m, &di, static_cast<cudaStream_t>(stream));
  if (st != HX_OK) return st;
  out->size_power = m->sp;
  out->err = di.err;
  out->fill = di.fill;
  out->tombstone_counter = di.tombstones;
  out->max_probe = di.max_probe;
  uint64_t r = di.max_probe;
  r = (r + 31) / 32 * 32;  // nextOverflow(overflow, 32), common.h:54-57
  out->current_max_bucket_overflow = r < 32 ? 32 : r;
  out->bucket_count = nslots(m);
  out->last_clean_moved = di.moved;
  return HX_OK;
}

hx_status hx_peek_status(hx_map* m, int32_t* out, hx_stream stream) {
  if (!valid_map(m) || !out) return HX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int v = 0, inv = HX_STATUS_INVALID;
  HX_CUDA(cudaMemcpyAsync(&v, &m->info->err, sizeof(int), cudaMemcpyDeviceToHost, s));
  HX_CUDA(cudaMemcpyAsync(&m->info->err, &inv, sizeof(int), cudaMemcpyHostToDevice, s));
  HX_CUDA(cudaStreamSynchronize(s));
  *out = v;
  return HX_OK;
}

hx_status hx_map_device_view(hx_map* m, hx_device_view* out) {
  if (!valid_map(m) || !out) return HX_ERR_INVALID_ARG;
  out->buckets = m->buckets;
  out->size_power = m->sp;
  out->reserved = 0;
  out->fill = &m->info->fill;
  out->tombstones = &m->info->tombstones;
  out->max_probe = &m->info->max_probe;
  out->err = &m->info->err;
  m->fill_ub = nslots(m);  // device-side inserts are invisible to the host bound
  return HX_OK;
}

hx_status hx_bucket_data(hx_map* m, void** d_buckets, uint64_t* bucket_count) {
  if (!valid_map(m)) return HX_ERR_INVALID_ARG;
  if (d_buckets) *d_buckets = m->buckets;
  if (bucket_count) *bucket_count = nslots(m);
  return HX_OK;
}

hx_status hx_map_set_insert_mode(hx_map* m, int blind_cas) {
  if (!m) return HX_ERR_INVALID_ARG;
  m->tune.blind = blind_cas != 0;
  return HX_OK;
}

hx_status hx_map_set_window_bytes(hx_map* m, int bytes) {
  if (!m || (bytes != 32 && bytes != 64)) return HX_ERR_INVALID_ARG;
  m->tune.wide = bytes == 64;
  return HX_OK;
}

hx_status hx_set_l2_fetch_granularity(int bytes) {
  if (bytes != 32 && bytes != 64 && bytes != 128) return HX_ERR_INVALID_ARG;
  HX_CUDA(cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, (size_t)bytes));
  return HX_OK;
}

hx_status hx_map_set_tuning(hx_map* m, int group_width, int keys_per_thread, int block_size) {
  if (!m) return HX_ERR_INVALID_ARG;
  if (group_width) {
    if (group_width != 1 && group_width != 2 && group_width != 4 && group_width != 8 && group_width != 16 &&
        group_width != 32)
      return HX_ERR_INVALID_ARG;
    m->tune.group = group_width;
  }
  if (keys_per_thread) {
    if (keys_per_thread != 1 && keys_per_thread != 2 && keys_per_thread != 4 && keys_per_thread != 8)
      return HX_ERR_INVALID_ARG;
    m->tune.unroll = keys_per_thread;
  }
  if (block_size) {
    if (block_size % 32 || block_size < 32 || block_size > 256) return HX_ERR_INVALID_ARG;
    m->tune.block = block_size;
  }
  return HX_OK;
}

}  // extern "C"
