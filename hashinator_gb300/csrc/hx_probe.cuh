// hx_probe.cuh — probe-group linear probing over a power-of-two bucket array.
//
// The reference probes one key per 32-lane warp over a 32-bucket window that
// starts at the key's home bucket (kernels_NVIDIA.h:356-408 insert, :665-689
// erase, :753-773 retrieve): 256 B (u32) or 512 B (u64) read for the one or
// two buckets a key needs at load factor 0.5. Here a probe group of G lanes
// (G in {1,2,4,8,16,32}) serves one key, each lane reading B adjacent buckets
// with one vector load, so a window is W = G*B buckets. Windows are aligned
// to W buckets: the first window covers the home bucket's aligned block, and
// lanes ignore the buckets before the home bucket in it. A 32-byte window is
// exactly one DRAM sector.
//
// The probe order is the reference's linear order h, h+1, h+2, ... (mod 2^sp)
// and the decisions per window are the reference's:
//   insert:   key present in the window -> overwrite its value; else CAS the
//             first EMPTY bucket in probe order; TOMBSTONE buckets are never
//             reused; the whole table is the search bound.
//   retrieve/ key present in the window -> hit; else an EMPTY bucket in the
//   erase:    window -> miss; the bound is the longest probe of any key.
// The distance of bucket b from home h is (b - h) mod 2^sp; max_probe holds
// the largest distance + 1 ever placed (the reference keeps the same bound
// rounded up to 32 in Info::currentMaxBucketOverflow, kernels_NVIDIA.h:436).
#pragma once
#include "hx_device.cuh"

namespace hx {

// Device-resident map metadata (the reference keeps Info in managed memory,
// hashinator/defaults.h:44-54, and migrates it on every call).
struct DInfo {
  unsigned long long fill;
  unsigned long long tombstones;
  unsigned int max_probe;  // exact: largest (distance + 1); 0 for an empty map
  int err;                 // HX_STATUS_*
  unsigned long long moved;  // clean_tombstones: number of keys taken out
  unsigned int skip;         // clean_tombstones: 1 when there were no tombstones
  unsigned int pad;
};

enum : int { PR_CONTINUE = 0, PR_INSERTED = 1, PR_UPDATED = 2, PR_FAIL = 3 };

template <int G>
__device__ __forceinline__ unsigned group_mask(int lane) {
  if constexpr (G == 32) return 0xffffffffu;
  else return ((1u << G) - 1u) << (lane & ~(G - 1));
}
// Ballot over the G lanes of this group, as bits 0..G-1.
template <int G>
__device__ __forceinline__ unsigned group_ballot(unsigned gmask, int lane, bool p) {
  if constexpr (G == 1) return p ? 1u : 0u;
  else if constexpr (G == 32) return __ballot_sync(gmask, p);
  else return (__ballot_sync(gmask, p) >> (lane & ~(G - 1))) & ((1u << G) - 1u);
}
template <int G, class T>
__device__ __forceinline__ T group_shfl(unsigned gmask, T v, int src) {
  if constexpr (G == 1) return v;
  else return __shfl_sync(gmask, v, src, G);
}

// Insert or update one key. All G lanes of the group call it with the same
// key. Returns PR_INSERTED / PR_UPDATED / PR_FAIL on every lane; `dist1`
// receives distance + 1 on the lane that placed a new key, 0 elsewhere.
template <class P, int G, int B>
__device__ __forceinline__ int probe_insert(P* __restrict__ table, int sp, typename PairTraits<P>::K key,
                                            typename PairTraits<P>::V val, int lane, unsigned gmask,
                                            unsigned& dist1) {
  using K = typename PairTraits<P>::K;
  using V = typename PairTraits<P>::V;
  constexpr K EMPTY = PairTraits<P>::EMPTY;
  constexpr int W = G * B;
  const int glane = lane & (G - 1);
  const uint32_t tmask = (1u << sp) - 1u;
  const long long tsize = (long long)tmask + 1;
  const uint32_t h = home_slot(key, sp);
  const uint32_t wstart = h & ~(uint32_t)(W - 1);
  const int first = (int)(h - wstart);
  for (uint32_t s = 0;; ++s) {
    const long long d0 = (long long)s * W - first;  // distance of window offset 0
    if (d0 >= tsize) return PR_FAIL;
    P* wp = table + ((wstart + s * (uint32_t)W) & tmask) + glane * B;
    K kk[B];
    V vv[B];
    load_buckets<B>(wp, kk, vv);
    unsigned mbits = 0, ebits = 0;
#pragma unroll
    for (int j = 0; j < B; ++j) {
      const long long d = d0 + glane * B + j;
      const bool cons = d >= 0 && d < tsize;
      if (cons && kk[j] == key) mbits |= 1u << j;
      if (cons && kk[j] == EMPTY) ebits |= 1u << j;
    }
    const unsigned gm = group_ballot<G>(gmask, lane, mbits != 0);
    if (gm) {
      if (glane == __ffs(gm) - 1) store_value(wp + (__ffs(mbits) - 1), val);
      return PR_UPDATED;
    }
    unsigned ge = group_ballot<G>(gmask, lane, ebits != 0);
    while (ge) {
      const int w = __ffs(ge) - 1;
      int res = PR_CONTINUE;
      if (glane == w) {
        const int j = __ffs(ebits) - 1;
        K ek = EMPTY;
        V ev = 0;
#pragma unroll
        for (int t = 0; t < B; ++t)
          if (t == j) ev = vv[t];
        for (int tries = 0;; ++tries) {
          if (cas_pair(wp + j, ek, ev, key, val)) {
            res = PR_INSERTED;
            dist1 = (unsigned)(d0 + glane * B + j) + 1u;
            break;
          }
          if (ek == key) {  // the same key won this bucket concurrently
            store_value(wp + j, val);
            res = PR_UPDATED;
            break;
          }
          if (ek != EMPTY || tries >= 8) {
            ebits &= ~(1u << j);
            break;
          }
          // still EMPTY but with another stale value: retry with it
        }
      }
      res = group_shfl<G>(gmask, res, w);
      if (res != PR_CONTINUE) return res;
      ge = group_ballot<G>(gmask, lane, ebits != 0);
    }
  }
}

// probe_insert with a single exit at the top of the step loop (the form the
// group insert kernel uses; at load factor 0.9 it measured 4-15% faster than
// probe_insert for 2-8-lane groups on GB300).
template <class P, int G, int B>
__device__ __forceinline__ int probe_insert_live(P* __restrict__ table, int sp, typename PairTraits<P>::K key,
                                                 typename PairTraits<P>::V val, int lane, unsigned gmask,
                                                 unsigned& dist1) {
  using K = typename PairTraits<P>::K;
  using V = typename PairTraits<P>::V;
  constexpr K EMPTY = PairTraits<P>::EMPTY;
  constexpr int W = G * B;
  const int glane = lane & (G - 1);
  const uint32_t tmask = (1u << sp) - 1u;
  const long long tsize = (long long)tmask + 1;
  const uint32_t h = home_slot(key, sp);
  const uint32_t wstart = h & ~(uint32_t)(W - 1);
  const int first = (int)(h - wstart);
  int res = PR_CONTINUE;
  for (uint32_t s = 0;; ++s) {
    const long long d0 = (long long)s * W - first;
    if (res == PR_CONTINUE && d0 >= tsize) res = PR_FAIL;
    if (res != PR_CONTINUE) return res;  // the same on every lane of the group
    P* wp = table + ((wstart + s * (uint32_t)W) & tmask) + glane * B;
    K kk[B];
    V vv[B];
    load_buckets<B>(wp, kk, vv);
    unsigned mbits = 0, ebits = 0;
#pragma unroll
    for (int j = 0; j < B; ++j) {
      const long long d = d0 + glane * B + j;
      const bool cons = d >= 0 && d < tsize;
      if (cons && kk[j] == key) mbits |= 1u << j;
      if (cons && kk[j] == EMPTY) ebits |= 1u << j;
    }
    const unsigned gm = group_ballot<G>(gmask, lane, mbits != 0);
    if (gm) {
      if (glane == __ffs(gm) - 1) store_value(wp + (__ffs(mbits) - 1), val);
      res = PR_UPDATED;
      continue;
    }
    unsigned ge = group_ballot<G>(gmask, lane, ebits != 0);
    while (ge) {
      const int w = __ffs(ge) - 1;
      int r = PR_CONTINUE;
      if (glane == w) {
        const int j = __ffs(ebits) - 1;
        K ek = EMPTY;
        V ev = 0;
#pragma unroll
        for (int t = 0; t < B; ++t)
          if (t == j) ev = vv[t];
        for (int tries = 0;; ++tries) {
          if (cas_pair(wp + j, ek, ev, key, val)) {
            r = PR_INSERTED;
            dist1 = (unsigned)(d0 + glane * B + j) + 1u;
            break;
          }
          if (ek == key) {
            store_value(wp + j, val);
            r = PR_UPDATED;
            break;
          }
          if (ek != EMPTY || tries >= 8) {
            ebits &= ~(1u << j);
            break;
          }
        }
      }
      r = group_shfl<G>(gmask, r, w);
      if (r != PR_CONTINUE) {
        res = r;
        break;
      }
      ge = group_ballot<G>(gmask, lane, ebits != 0);
    }
  }
}

// Find one key within `limit` buckets of its home. Returns the group lane
// holding it (its bucket index in `slot`, value in `val`) or -1.
template <class P, int G, int B>
__device__ __forceinline__ int probe_find(const P* __restrict__ table, int sp, typename PairTraits<P>::K key,
                                          unsigned limit, int lane, unsigned gmask, uint32_t& slot,
                                          typename PairTraits<P>::V& val) {
  using K = typename PairTraits<P>::K;
  using V = typename PairTraits<P>::V;
  constexpr K EMPTY = PairTraits<P>::EMPTY;
  constexpr int W = G * B;
  const int glane = lane & (G - 1);
  const uint32_t tmask = (1u << sp) - 1u;
  const uint32_t h = home_slot(key, sp);
  const uint32_t wstart = h & ~(uint32_t)(W - 1);
  const int first = (int)(h - wstart);
  for (uint32_t s = 0;; ++s) {
    const long long d0 = (long long)s * W - first;
    if (d0 >= (long long)limit) return -1;
    const uint32_t b0 = ((wstart + s * (uint32_t)W) & tmask) + glane * B;
    K kk[B];
    V vv[B];
    load_buckets<B>(table + b0, kk, vv);
    unsigned mbits = 0, ebits = 0;
#pragma unroll
    for (int j = 0; j < B; ++j) {
      const long long d = d0 + glane * B + j;
      const bool cons = d >= 0 && d < (long long)limit;
      if (cons && kk[j] == key) mbits |= 1u << j;
      if (cons && kk[j] == EMPTY) ebits |= 1u << j;
    }
    const unsigned gm = group_ballot<G>(gmask, lane, mbits != 0);
    if (gm) {
      const int w = __ffs(gm) - 1;
      if (glane == w) {
        const int j = __ffs(mbits) - 1;
        slot = b0 + j;
#pragma unroll
        for (int t = 0; t < B; ++t)
          if (t == j) val = vv[t];
      }
      return w;
    }
    if (group_ballot<G>(gmask, lane, ebits != 0)) return -1;
  }
}


// probe_find with a single exit at the top of the step loop (a key stays
// "live" until a match, an EMPTY bucket or the probe bound ends it). For 4-
// and 8-lane groups this form measured 6-49% faster than probe_find at load
// factor 0.5-0.9 on GB300 (u32 and u64 tables), which made small groups the
// fastest queries; the group query kernels use it. Returns the lane of the
// group that found the key (value in val on that lane) or -1.
template <class P, int G, int B>
__device__ __forceinline__ int probe_find_live(const P* __restrict__ table, int sp, typename PairTraits<P>::K key,
                                               bool act, unsigned limit, int lane, unsigned gmask,
                                               typename PairTraits<P>::V& val) {
  using K = typename PairTraits<P>::K;
  using V = typename PairTraits<P>::V;
  constexpr K EMPTY = PairTraits<P>::EMPTY;
  constexpr int W = G * B;
  const int glane = lane & (G - 1);
  const uint32_t tmask = (1u << sp) - 1u;
  const uint32_t h = act ? home_slot(key, sp) : 0u;
  const uint32_t wstart = h & ~(uint32_t)(W - 1);
  const int first = (int)(h - wstart);
  bool live = act;
  int who = -1;
  for (uint32_t s = 0;; ++s) {
    K kk[B];
    V vv[B];
    const long long d0 = (long long)s * W - first;
    if (live && d0 >= (long long)limit) live = false;  // past the probe bound: a miss
    const uint32_t b0 = ((wstart + s * (uint32_t)W) & tmask) + glane * B;
    if (!live) return who;  // the same on every lane of the group
    load_buckets<B>(table + b0, kk, vv);
    unsigned mbits = 0, ebits = 0;
#pragma unroll
    for (int j = 0; j < B; ++j) {
      const long long d = d0 + glane * B + j;
      const bool cons = d >= 0 && d < (long long)limit;
      if (cons && kk[j] == key) mbits |= 1u << j;
      if (cons && kk[j] == EMPTY) ebits |= 1u << j;
    }
    const unsigned gm = group_ballot<G>(gmask, lane, mbits != 0);
    if (gm) {
      const int w = __ffs(gm) - 1;
      if (glane == w) {
        const int j = __ffs(mbits) - 1;
#pragma unroll
        for (int t = 0; t < B; ++t)
          if (t == j) val = vv[t];
      }
      who = w;
      live = false;
    } else if (group_ballot<G>(gmask, lane, ebits != 0)) {
      live = false;
    }
  }
}

// ---------------------------------------------------------------------------
// Thread-per-key probing (probe group of one lane): a thread holds U keys
// and issues all their first-window loads (or, for insert, their home-bucket
// CAS) before resolving any of them, so U independent DRAM requests per
// thread are in flight. A window is B buckets (32 B: one DRAM sector).
// ---------------------------------------------------------------------------
template <class P, int B>
struct Window {
  typename PairTraits<P>::K k[B];
  typename PairTraits<P>::V v[B];
};

// Lookup with the first window (the aligned block holding the home bucket h)
// already in w. Returns true and the bucket / value on a hit.
template <class P, int B>
__device__ __forceinline__ bool find_t1(const P* __restrict__ table, int sp, typename PairTraits<P>::K key,
                                        unsigned limit, uint32_t h, Window<P, B>& w, uint32_t& slot,
                                        typename PairTraits<P>::V& val) {
  constexpr auto EMPTY = PairTraits<P>::EMPTY;
  const uint32_t tmask = (1u << sp) - 1u;
  const uint32_t wstart = h & ~(uint32_t)(B - 1);
  const int first = (int)(h - wstart);
  for (uint32_t s = 0;; ++s) {
    const long long d0 = (long long)s * B - first;
    if (d0 >= (long long)limit) return false;
    const uint32_t b0 = (wstart + s * (uint32_t)B) & tmask;
    if (s > 0) load_buckets<B>(table + b0, w.k, w.v);
    int hit = -1;
    bool empty = false;
#pragma unroll
    for (int j = B - 1; j >= 0; --j) {  // descending: hit ends on the lowest match
      const long long d = d0 + j;
      const bool cons = d >= 0 && d < (long long)limit;
      if (cons && w.k[j] == key) hit = j;
      if (cons && w.k[j] == EMPTY) empty = true;
    }
    if (hit >= 0) {
      slot = b0 + hit;
#pragma unroll
      for (int j = 0; j < B; ++j)
        if (j == hit) val = w.v[j];
      return true;
    }
    if (empty) return false;
  }
}

// Insert after the home bucket h was found taken by another key (or a
// TOMBSTONE): continue the linear probe at distance 1. Same decisions as
// probe_insert.
template <class P, int B>
__device__ __noinline__ int insert_t1_rest(P* __restrict__ table, int sp, typename PairTraits<P>::K key,
                                           typename PairTraits<P>::V val, uint32_t h, unsigned& dist1) {
  using K = typename PairTraits<P>::K;
  using V = typename PairTraits<P>::V;
  constexpr K EMPTY = PairTraits<P>::EMPTY;
  const uint32_t tmask = (1u << sp) - 1u;
  const long long tsize = (long long)tmask + 1;
  const uint32_t wstart = h & ~(uint32_t)(B - 1);
  const int first = (int)(h - wstart);
  for (uint32_t s = 0;; ++s) {
    const long long d0 = (long long)s * B - first;
    if (d0 >= tsize) return PR_FAIL;
    P* wp = table + ((wstart + s * (uint32_t)B) & tmask);
    K kk[B];
    V vv[B];
    load_buckets<B>(wp, kk, vv);
    unsigned mbits = 0, ebits = 0;
#pragma unroll
    for (int j = 0; j < B; ++j) {
      const long long d = d0 + j;
      const bool cons = d >= 1 && d < tsize;
      if (cons && kk[j] == key) mbits |= 1u << j;
      if (cons && kk[j] == EMPTY) ebits |= 1u << j;
    }
    if (mbits) {
      store_value(wp + (__ffs(mbits) - 1), val);
      return PR_UPDATED;
    }
    while (ebits) {
      const int j = __ffs(ebits) - 1;
      K ek = EMPTY;
      V ev = 0;
#pragma unroll
      for (int t = 0; t < B; ++t)
        if (t == j) ev = vv[t];
      for (int tries = 0;; ++tries) {
        if (cas_pair(wp + j, ek, ev, key, val)) {
          dist1 = (unsigned)(d0 + j) + 1u;
          return PR_INSERTED;
        }
        if (ek == key) {
          store_value(wp + j, val);
          return PR_UPDATED;
        }
        if (ek != EMPTY || tries >= 8) break;
      }
      ebits &= ~(1u << j);
    }
  }
}

// Insert with the first window (aligned block holding the home bucket h)
// already loaded into w: the same decisions as probe_insert, starting at
// distance 0, so the CAS usually lands on a line that is already in L2.
template <class P, int B>
__device__ __forceinline__ int insert_t1_win(P* __restrict__ table, int sp, typename PairTraits<P>::K key,
                                             typename PairTraits<P>::V val, uint32_t h, Window<P, B>& w,
                                             unsigned& dist1) {
  using K = typename PairTraits<P>::K;
  using V = typename PairTraits<P>::V;
  constexpr K EMPTY = PairTraits<P>::EMPTY;
  const uint32_t tmask = (1u << sp) - 1u;
  const long long tsize = (long long)tmask + 1;
  const uint32_t wstart = h & ~(uint32_t)(B - 1);
  const int first = (int)(h - wstart);
  for (uint32_t s = 0;; ++s) {
    const long long d0 = (long long)s * B - first;
    if (d0 >= tsize) return PR_FAIL;
    P* wp = table + ((wstart + s * (uint32_t)B) & tmask);
    if (s > 0) load_buckets<B>(wp, w.k, w.v);
    unsigned mbits = 0, ebits = 0;
#pragma unroll
    for (int j = 0; j < B; ++j) {
      const long long d = d0 + j;
      const bool cons = d >= 0 && d < tsize;
      if (cons && w.k[j] == key) mbits |= 1u << j;
      if (cons && w.k[j] == EMPTY) ebits |= 1u << j;
    }
    if (mbits) {
      store_value(wp + (__ffs(mbits) - 1), val);
      return PR_UPDATED;
    }
    while (ebits) {
      const int j = __ffs(ebits) - 1;
      K ek = EMPTY;
      V ev = 0;
#pragma unroll
      for (int t = 0; t < B; ++t)
        if (t == j) ev = w.v[t];
      for (int tries = 0;; ++tries) {
        if (cas_pair(wp + j, ek, ev, key, val)) {
          dist1 = (unsigned)(d0 + j) + 1u;
          return PR_INSERTED;
        }
        if (ek == key) {
          store_value(wp + j, val);
          return PR_UPDATED;
        }
        if (ek != EMPTY || tries >= 8) break;
      }
      ebits &= ~(1u << j);
    }
  }
}

// The rest of a thread-per-key insert once its first blind CAS at home has
// failed and left the bucket's content in (ek, ev): retry while the bucket is
// EMPTY with a stale value (nine attempts in all), overwrite the value if the
// bucket holds the key, else probe on.
template <class P, int B>
__device__ __forceinline__ void insert_t1_after_cas(P* tab, int sp, typename PairTraits<P>::K key,
                                                    typename PairTraits<P>::V val, uint32_t h,
                                                    typename PairTraits<P>::K ek, typename PairTraits<P>::V ev,
                                                    unsigned& ins, unsigned& maxd, bool& fail) {
  for (int tries = 1; tries < 9 && ek == PairTraits<P>::EMPTY; ++tries) {
    if (cas_pair(tab + h, ek, ev, key, val)) {
      ++ins;
      maxd = maxd > 1u ? maxd : 1u;
      return;
    }
  }
  if (ek == key) {
    store_value(tab + h, val);
    return;
  }
  unsigned d1 = 0;
  const int r = insert_t1_rest<P, B>(tab, sp, key, val, h, d1);
  if (r == PR_INSERTED) {
    ++ins;
    maxd = d1 > maxd ? d1 : maxd;
  } else if (r == PR_FAIL) {
    fail = true;
  }
}

// One key into one table, thread-per-key: blind CAS at home, then probe.
template <class P, int B>
__device__ __forceinline__ void insert_one_t1(P* tab, int sp, typename PairTraits<P>::K key,
                                                typename PairTraits<P>::V val, unsigned& ins, unsigned& maxd,
                                                bool& fail) {
  using K = typename PairTraits<P>::K;
  using V = typename PairTraits<P>::V;
  if (key == PairTraits<P>::EMPTY || key == PairTraits<P>::TOMB) return;
  const uint32_t h = home_slot(key, sp);
  K ek = PairTraits<P>::EMPTY;
  V ev = 0;
  if (cas_pair(tab + h, ek, ev, key, val)) {
    ++ins;
    maxd = maxd > 1u ? maxd : 1u;
    return;
  }
  insert_t1_after_cas<P, B>(tab, sp, key, val, h, ek, ev, ins, maxd, fail);
}

// One key into one table, thread-per-key, reading the home window before any
// CAS: for keys whose home is probably taken (clean_tombstones' moved keys).
template <class P, int B>
__device__ __forceinline__ void insert_one_t1_win(P* tab, int sp, typename PairTraits<P>::K key,
                                                  typename PairTraits<P>::V val, unsigned& ins, unsigned& maxd,
                                                  bool& fail) {
  if (key == PairTraits<P>::EMPTY || key == PairTraits<P>::TOMB) return;
  const uint32_t h = home_slot(key, sp);
  Window<P, B> w;
  load_buckets<B>(tab + (h & ~(uint32_t)(B - 1)), w.k, w.v);
  unsigned d1 = 0;
  const int r = insert_t1_win<P, B>(tab, sp, key, val, h, w, d1);
  if (r == PR_INSERTED) {
    ++ins;
    maxd = d1 > maxd ? d1 : maxd;
  } else if (r == PR_FAIL) {
    fail = true;
  }
}

// U keys per thread, elements first + u * stride (those below count), each
// loaded by load(i, key, val): their first CASes at home are issued together,
// so U atomics are in flight per thread, and each key is then finished as
// insert_one_t1 does.
template <class P, int B, int U, class Load>
__device__ __forceinline__ void insert_t1_many(P* tab, int sp, unsigned first, unsigned stride, unsigned count,
                                               const Load& load, unsigned& ins, unsigned& maxd, bool& fail) {
  using K = typename PairTraits<P>::K;
  using V = typename PairTraits<P>::V;
  K key[U], ek[U];
  V val[U], ev[U];
  uint32_t h[U];
  bool act[U], ok[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const unsigned i = first + u * stride;
    act[u] = i < count;
    if (act[u]) {
      load(i, key[u], val[u]);
      act[u] = key[u] != PairTraits<P>::EMPTY && key[u] != PairTraits<P>::TOMB;
    }
  }
#pragma unroll
  for (int u = 0; u < U; ++u) {
    ok[u] = false;
    if (act[u]) {
      h[u] = home_slot(key[u], sp);
      ek[u] = PairTraits<P>::EMPTY;
      ev[u] = 0;
      ok[u] = cas_pair(tab + h[u], ek[u], ev[u], key[u], val[u]);
    }
  }
#pragma unroll
  for (int u = 0; u < U; ++u) {
    if (!act[u]) continue;
    if (ok[u]) {
      ++ins;
      maxd = maxd > 1u ? maxd : 1u;
    } else {
      insert_t1_after_cas<P, B>(tab, sp, key[u], val[u], h[u], ek[u], ev[u], ins, maxd, fail);
    }
  }
}

}  // namespace hx
