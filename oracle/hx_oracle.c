/*
 * hx_oracle.c — TEST INFRASTRUCTURE ONLY: serial CPU restatement of the
 * Hashinator accelerated hot path, used to check libhx. Each function cites
 * the reference code (paths inside the Hashinator source tree, v1.0.1) whose
 * observable behaviour it restates. The GPU kernels process keys
 * concurrently; processed one at a time they reduce to the serial rules
 * below. Bucket layouts follow hash_pair<K,V> (hashinator/hash_pair.h:30-75).
 */
#include "hx_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

struct ox_map {
  int kb;         /* key bytes: 4 (u32/u32 pairs, 8 B) or 8 (u64/u64, 16 B) */
  int sp;         /* size power */
  uint64_t fill, tombstones, max_probe;
  void* b;        /* bucket array */
};

#define E32 0xFFFFFFFFu
#define T32 0xFFFFFFFEu
#define E64 0xFFFFFFFFFFFFFFFFull
#define T64 0xFFFFFFFFFFFFFFFEull

/* HashFunctions::Fibonacci (hashinator/hashfunctions.h:39-43, :52-56). */
uint32_t ox_fib_hash32(uint32_t key, int sp) {
  key ^= key >> (32 - sp);
  return (uint32_t)(((uint64_t)key * 2654435769ull) >> (32 - sp));
}
uint64_t ox_fib_hash64(uint64_t key, int sp) {
  key ^= key >> (64 - sp);
  return (key * 11400714819323198485ull) >> (64 - sp);
}

static inline uint64_t nb(const ox_map* m) { return 1ull << m->sp; }
static inline uint64_t empty_key(const ox_map* m) { return m->kb == 4 ? E32 : E64; }
static inline uint64_t tomb_key(const ox_map* m) { return m->kb == 4 ? T32 : T64; }
static inline uint64_t home(const ox_map* m, uint64_t k) {
  const uint64_t mask = nb(m) - 1;
  return m->kb == 4 ? (ox_fib_hash32((uint32_t)k, m->sp) & mask) : (ox_fib_hash64(k, m->sp) & mask);
}
static inline uint64_t getk(const ox_map* m, uint64_t i) {
  return m->kb == 4 ? ((const uint32_t*)m->b)[2 * i] : ((const uint64_t*)m->b)[2 * i];
}
static inline uint64_t getv(const ox_map* m, uint64_t i) {
  return m->kb == 4 ? ((const uint32_t*)m->b)[2 * i + 1] : ((const uint64_t*)m->b)[2 * i + 1];
}
static inline void setk(ox_map* m, uint64_t i, uint64_t k) {
  if (m->kb == 4) ((uint32_t*)m->b)[2 * i] = (uint32_t)k;
  else ((uint64_t*)m->b)[2 * i] = k;
}
static inline void setv(ox_map* m, uint64_t i, uint64_t v) {
  if (m->kb == 4) ((uint32_t*)m->b)[2 * i + 1] = (uint32_t)v;
  else ((uint64_t*)m->b)[2 * i + 1] = v;
}
static inline uint64_t ld(const void* p, int kb, uint64_t i) {
  return kb == 4 ? ((const uint32_t*)p)[i] : ((const uint64_t*)p)[i];
}
static inline void st(void* p, int kb, uint64_t i, uint64_t v) {
  if (kb == 4) ((uint32_t*)p)[i] = (uint32_t)v;
  else ((uint64_t*)p)[i] = v;
}

static void fill_empty(ox_map* m) {
  for (uint64_t i = 0; i < nb(m); ++i) {
    setk(m, i, empty_key(m));
    setv(m, i, 0);
  }
}

/* Hashmap(int sizepower) (hashinator.h:120-129): all buckets (EMPTY, V()). */
ox_map* ox_map_create(int key_bytes, int size_power) {
  if ((key_bytes != 4 && key_bytes != 8) || size_power < 1 || size_power > 31) return NULL;
  ox_map* m = (ox_map*)calloc(1, sizeof(ox_map));
  m->kb = key_bytes;
  m->sp = size_power;
  m->b = malloc((size_t)nb(m) * 2 * key_bytes);
  fill_empty(m);
  return m;
}

void ox_map_destroy(ox_map* m) {
  if (!m) return;
  free(m->b);
  free(m);
}

void* ox_buckets(ox_map* m) { return m->b; }

/* One key of insert_kernel (kernels_NVIDIA.h:307-447) on its own: walk from
 * the home bucket in linear order; an existing key gets its value
 * overwritten (:373-381); else the first EMPTY bucket takes the pair
 * (:383-407); TOMBSTONE buckets are passed over, never reused. The whole
 * table is the search bound (:356). Returns 1 if inserted, 0 if updated,
 * -1 if no bucket was found. */
static int insert_one(ox_map* m, uint64_t k, uint64_t v) {
  const uint64_t n = nb(m), mask = n - 1, h = home(m, k);
  for (uint64_t d = 0; d < n; ++d) {
    const uint64_t i = (h + d) & mask;
    const uint64_t bk = getk(m, i);
    if (bk == k) {
      setv(m, i, v);
      return 0;
    }
    if (bk == empty_key(m)) {
      setk(m, i, k);
      setv(m, i, v);
      m->fill++;
      if (d + 1 > m->max_probe) m->max_probe = d + 1;
      return 1;
    }
  }
  return -1;
}

/* Lookup bounded by the longest probe, stopping at EMPTY
 * (retrieve_kernel, kernels_NVIDIA.h:753-773; delete_kernel :665-689). */
static int64_t find_one(const ox_map* m, uint64_t k) {
  const uint64_t mask = nb(m) - 1, h = home(m, k);
  for (uint64_t d = 0; d < m->max_probe; ++d) {
    const uint64_t i = (h + d) & mask;
    const uint64_t bk = getk(m, i);
    if (bk == k) return (int64_t)i;
    if (bk == empty_key(m)) return -1;
  }
  return -1;
}

static int is_sentinel(const ox_map* m, uint64_t k) { return k == empty_key(m) || k == tomb_key(m); }

static void rehash_to(ox_map* m, int new_sp);

/* insert(keys, vals, len, targetLF) (hashinator.h:1319-1335): grow first if
 * ceil(log2((fill + len) / targetLF)) > sizePower, then insert each pair.
 * Keys equal to EMPTY or TOMBSTONE are skipped (libhx contract). */
int ox_insert(ox_map* m, const void* keys, const void* vals, uint64_t n, float target_lf) {
  if (n == 0) return 0;
  if (target_lf > 0.0f) {
    long long need = (long long)ceil(log2((double)(m->fill + n) * (1.0 / (double)target_lf)));
    if (need > m->sp) rehash_to(m, (int)need);
  }
  int err = 0;
  for (uint64_t i = 0; i < n; ++i) {
    const uint64_t k = ld(keys, m->kb, i);
    if (is_sentinel(m, k)) continue;
    if (insert_one(m, k, ld(vals, m->kb, i)) < 0) err = 1;
  }
  return err;
}

/* retrieve(keys, vals, len) (hashinator.h:1378-1384): hits write the value,
 * misses leave the output untouched (kernels_NVIDIA.h:765-771). */
void ox_retrieve(const ox_map* m, const void* keys, void* vals, uint64_t n) {
  for (uint64_t i = 0; i < n; ++i) {
    const uint64_t k = ld(keys, m->kb, i);
    if (is_sentinel(m, k)) continue;
    const int64_t s = find_one(m, k);
    if (s >= 0) st(vals, m->kb, i, getv(m, (uint64_t)s));
  }
}

/* erase(keys, len) (hashinator.h:1398-1409, delete_kernel
 * kernels_NVIDIA.h:622-718): present key -> TOMBSTONE, tombstones += 1,
 * fill -= 1. */
void ox_erase(ox_map* m, const void* keys, uint64_t n) {
  for (uint64_t i = 0; i < n; ++i) {
    const uint64_t k = ld(keys, m->kb, i);
    if (is_sentinel(m, k)) continue;
    const int64_t s = find_one(m, k);
    if (s >= 0) {
      setk(m, (uint64_t)s, tomb_key(m));
      m->tombstones++;
      m->fill--;
    }
  }
}

/* clean_tombstones (hashinator.h:1262-1315): nothing without tombstones;
 * else TOMBSTONE -> EMPTY, keys not in their home bucket are extracted in
 * bucket order (the isOverflown rule, :1285-1297) and emptied
 * (reset_to_empty, kernels_NVIDIA.h:68-138), then inserted again
 * (insert_kernel on pairs). */
void ox_clean_tombstones(ox_map* m) {
  if (m->tombstones == 0) return;
  m->tombstones = 0;
  const uint64_t n = nb(m);
  uint64_t* lk = (uint64_t*)malloc(sizeof(uint64_t) * (m->fill + 1));
  uint64_t* lv = (uint64_t*)malloc(sizeof(uint64_t) * (m->fill + 1));
  uint64_t c = 0;
  /* The rule sees the table as it is rewritten; its decision for a valid key
   * does not depend on that (a home bucket holding another key or EMPTY both
   * differ from the key), so decide on the unmodified table first. */
  for (uint64_t i = 0; i < n; ++i) {
    const uint64_t k = getk(m, i);
    if (is_sentinel(m, k)) continue;
    if (getk(m, home(m, k)) != k) {
      lk[c] = k;
      lv[c] = getv(m, i);
      ++c;
    }
  }
  /* Apply: TOMBSTONE -> EMPTY and moved keys -> EMPTY. */
  for (uint64_t i = 0; i < n; ++i) {
    const uint64_t k = getk(m, i);
    if (k == tomb_key(m)) {
      setk(m, i, empty_key(m));
      setv(m, i, 0);
    }
  }
  for (uint64_t j = 0; j < c; ++j) {
    /* the bucket holding lk[j] */
    const uint64_t mask = n - 1, h = home(m, lk[j]);
    for (uint64_t d = 0; d < n; ++d) {
      const uint64_t i = (h + d) & mask;
      if (getk(m, i) == lk[j]) {
        setk(m, i, empty_key(m));
        setv(m, i, 0);
        break;
      }
    }
  }
  m->fill -= c;
  m->max_probe = m->fill ? 1 : 0; /* keys left are all in their home bucket */
  for (uint64_t j = 0; j < c; ++j) insert_one(m, lk[j], lv[j]);
  free(lk);
  free(lv);
}

/* device_rehash (hashinator.h:285-336): every valid pair, in bucket order,
 * into a fresh table; tombstones dropped. */
static void rehash_to(ox_map* m, int new_sp) {
  ox_map* t = ox_map_create(m->kb, new_sp);
  for (uint64_t i = 0; i < nb(m); ++i) {
    const uint64_t k = getk(m, i);
    if (!is_sentinel(m, k)) insert_one(t, k, getv(m, i));
  }
  free(m->b);
  m->b = t->b;
  m->sp = t->sp;
  m->fill = t->fill;
  m->max_probe = t->max_probe;
  m->tombstones = 0;
  free(t);
}

int ox_resize(ox_map* m, int new_size_power) {
  if (new_size_power < 1 || new_size_power > 31) return -1;
  rehash_to(m, new_size_power);
  return 0;
}

static int pred_scalar(const ox_pred* p, uint64_t x) {
  switch (p->op) {
    case 0: return 1;
    case 1: return (x % p->a) < p->b;
    case 2: return x < p->a;
    case 3: return x >= p->a;
    case 4: return x == p->a;
    case 5: return x != p->a;
    case 6: return (x & p->a) == p->b;
    case 7: return x >= p->a && x < p->b;
    default: return 0;
  }
}

/* Rule evaluation on a bucket: the reference's functors see EMPTY and
 * TOMBSTONE buckets too (split_tools.h:541-550 applies the rule to every
 * element); HX_PRED_SKIP_SENTINELS (flag 1) hides them. */
static int pred_pair(const ox_pred* p, uint64_t k, uint64_t v, int kb, const ox_map* m) {
  const uint64_t E = kb == 4 ? E32 : E64, T = kb == 4 ? T32 : T64;
  const int sent = (k == E) || (k == T);
  int r;
  if (p->op == 8) r = !sent;
  else if (p->op == 9) r = !sent && m && getk(m, home(m, k)) != k;
  else {
    r = pred_scalar(p, p->field == 2 ? v : k);
    if ((p->flags & 1u) && sent) r = 0;
  }
  if (p->flags & 2u) r = !r;
  return r;
}

/* extractPattern(elements, rule) (hashinator.h:1155-1185): bucket-order
 * copy of the buckets the rule selects. Returns the full count; writes at
 * most capacity pairs. */
uint64_t ox_extract(const ox_map* m, const ox_pred* pred, void* out, uint64_t capacity) {
  uint64_t c = 0;
  for (uint64_t i = 0; i < nb(m); ++i) {
    const uint64_t k = getk(m, i), v = getv(m, i);
    if (pred_pair(pred, k, v, m->kb, m)) {
      if (c < capacity) {
        st(out, m->kb, 2 * c, k);
        st(out, m->kb, 2 * c + 1, v);
      }
      ++c;
    }
  }
  return c;
}

uint64_t ox_mapping(const ox_map* m, void* keys, void* vals, uint64_t capacity) {
  uint64_t c = 0;
  for (uint64_t i = 0; i < nb(m); ++i) {
    const uint64_t k = getk(m, i);
    if (is_sentinel(m, k)) continue;
    if (c < capacity) {
      st(keys, m->kb, c, k);
      st(vals, m->kb, c, getv(m, i));
    }
    ++c;
  }
  return c;
}

void ox_info(const ox_map* m, int* size_power, uint64_t* fill, uint64_t* tombstones, uint64_t* max_probe) {
  if (size_power) *size_power = m->sp;
  if (fill) *fill = m->fill;
  if (tombstones) *tombstones = m->tombstones;
  if (max_probe) *max_probe = m->max_probe;
}

/* split::tools::copy_if (split_tools.h:1129-1223): stable compaction. */
uint64_t ox_copy_if(const void* in, void* out, uint64_t n, int elem_bytes, const ox_pred* pred) {
  uint64_t c = 0;
  for (uint64_t i = 0; i < n; ++i) {
    int sel;
    if (elem_bytes == 4) {
      sel = pred_scalar(pred, ((const uint32_t*)in)[i]);
      if (pred->flags & 2u) sel = !sel;
    } else if (elem_bytes == 8) {
      const uint32_t* p = (const uint32_t*)in + 2 * i;
      sel = pred_pair(pred, p[0], p[1], 4, NULL);
    } else {
      const uint64_t* p = (const uint64_t*)in + 2 * i;
      sel = pred_pair(pred, p[0], p[1], 8, NULL);
    }
    if (sel) {
      memcpy((char*)out + c * elem_bytes, (const char*)in + i * elem_bytes, (size_t)elem_bytes);
      ++c;
    }
  }
  return c;
}

/* split::tools::split_prefix_scan (split_tools.h:363-418): exclusive sum,
 * wrapping modulo 2^32. */
void ox_exclusive_scan_u32(const uint32_t* in, uint32_t* out, uint64_t n) {
  uint32_t acc = 0;
  for (uint64_t i = 0; i < n; ++i) {
    const uint32_t x = in[i];
    out[i] = acc;
    acc += x;
  }
}
