// ref_driver.cpp — TEST INFRASTRUCTURE ONLY. Runs the reference Hashinator
// in its own CPU-only mode (HASHINATOR_CPU_ONLY_MODE, the reference's
// "hybrid" build, unit_tests/hybrid/main.cu) on an input script and writes
// the results, to pin the oracle (oracle/hx_oracle.c) and to produce the
// golden fixtures in tests/golden/. Compiled by oracle/Makefile against the
// reference headers where they lie; nothing of the reference is copied.
//
// Input (little-endian u64 header, then arrays of key_bytes-wide words):
//   magic 0x48584752, key_bytes, size_power, n_ins, n_q, n_e, fill_pattern
//   keys[n_ins] vals[n_ins] qkeys[n_q] ekeys[n_e]
// Operations (the reference's CPU-only API):
//   Hashmap<K,K> m(size_power); m.insert(keys, vals, n_ins)  [serial _at]
//   query 1: find(q) for every q (hit -> value, miss -> fill_pattern)
//   erase(e) for every e, summing the returned counts
//   query 2: the same queries again
//   dump: iterate the map (bucket order)
// (The op-script mode, below, runs any sequence of these operations.)
// Output: size_after_insert, size_after_erase, tombstones_after_erase,
//   n_erased, size_power_final, n_map (u64 each), then
//   q1_found[n_q] (u8), q1_vals[n_q], q2_found[n_q], q2_vals[n_q],
//   map_keys[n_map], map_vals[n_map].
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "hashinator/hashinator.h"

template <class K>
static int run(FILE* in, FILE* out, uint64_t sp, uint64_t n_ins, uint64_t n_q, uint64_t n_e, uint64_t fillpat) {
  std::vector<K> keys(n_ins), vals(n_ins), q(n_q), e(n_e);
  if (fread(keys.data(), sizeof(K), n_ins, in) != n_ins || fread(vals.data(), sizeof(K), n_ins, in) != n_ins ||
      fread(q.data(), sizeof(K), n_q, in) != n_q || fread(e.data(), sizeof(K), n_e, in) != n_e) {
    fprintf(stderr, "short input\n");
    return 2;
  }
  Hashinator::Hashmap<K, K> m((int)sp);
  m.insert(keys.data(), vals.data(), n_ins);
  const uint64_t size_ins = m.size();

  auto query = [&](std::vector<uint8_t>& found, std::vector<K>& v) {
    found.assign(n_q, 0);
    v.assign(n_q, (K)fillpat);
    for (uint64_t i = 0; i < n_q; ++i) {
      auto it = m.find(q[i]);
      if (it != m.end()) {
        found[i] = 1;
        v[i] = it->second;
      }
    }
  };
  std::vector<uint8_t> f1, f2;
  std::vector<K> v1, v2;
  query(f1, v1);
  uint64_t n_erased = 0;
  for (uint64_t i = 0; i < n_e; ++i) n_erased += m.erase(e[i]);
  const uint64_t size_er = m.size();
  const uint64_t tomb_er = m.tombstone_count();
  query(f2, v2);
  std::vector<K> mk, mv;
  for (auto it = m.begin(); it != m.end(); ++it) {
    mk.push_back(it->first);
    mv.push_back(it->second);
  }
  const uint64_t hdr[6] = {size_ins, size_er, tomb_er, n_erased, (uint64_t)m.getSizePower(), (uint64_t)mk.size()};
  fwrite(hdr, 8, 6, out);
  fwrite(f1.data(), 1, n_q, out);
  fwrite(v1.data(), sizeof(K), n_q, out);
  fwrite(f2.data(), 1, n_q, out);
  fwrite(v2.data(), sizeof(K), n_q, out);
  fwrite(mk.data(), sizeof(K), mk.size(), out);
  fwrite(mv.data(), sizeof(K), mv.size(), out);
  return 0;
}

// Op-script mode (magic 0x48584753): header key_bytes, size_power, n_ops,
// fill_pattern, then per op: code, n, payload. Codes and payloads:
//   1 INSERT  keys[n] vals[n]   -> size after                      (u64)
//   2 QUERY   keys[n]           -> found[n] (u8), vals[n]
//   3 ERASE   keys[n]           -> erased, size, tombstones        (u64 x3)
//   4 RESIZE  (n = size power)  -> size, size power                (u64 x2)
//   5 DUMP    (n = 0)           -> n_map, keys[n_map], vals[n_map]
// INSERT is insert(keys, vals, n), QUERY find() per key, ERASE erase(key)
// per key, RESIZE resize(sp) — the CPU path's rehash, which drops
// tombstones (the CPU analogue of clean_tombstones).
template <class K>
static int run_ops(FILE* in, FILE* out, uint64_t sp, uint64_t n_ops, uint64_t fillpat) {
  Hashinator::Hashmap<K, K> m((int)sp);
  for (uint64_t o = 0; o < n_ops; ++o) {
    uint64_t h[2];
    if (fread(h, 8, 2, in) != 2) return 2;
    const uint64_t code = h[0], n = h[1];
    if (code == 1 || code == 2 || code == 3) {
      std::vector<K> keys(n), vals(code == 1 ? n : 0);
      if (fread(keys.data(), sizeof(K), n, in) != n) return 2;
      if (code == 1 && fread(vals.data(), sizeof(K), n, in) != n) return 2;
      if (code == 1) {
        m.insert(keys.data(), vals.data(), n);
        const uint64_t sz = m.size();
        fwrite(&sz, 8, 1, out);
      } else if (code == 2) {
        std::vector<uint8_t> found(n, 0);
        std::vector<K> v(n, (K)fillpat);
        for (uint64_t i = 0; i < n; ++i) {
          auto it = m.find(keys[i]);
          if (it != m.end()) {
            found[i] = 1;
            v[i] = it->second;
          }
        }
        fwrite(found.data(), 1, n, out);
        fwrite(v.data(), sizeof(K), n, out);
      } else {
        uint64_t erased = 0;
        for (uint64_t i = 0; i < n; ++i) erased += m.erase(keys[i]);
        const uint64_t r[3] = {erased, (uint64_t)m.size(), (uint64_t)m.tombstone_count()};
        fwrite(r, 8, 3, out);
      }
    } else if (code == 4) {
      m.resize((int)n);
      const uint64_t r[2] = {(uint64_t)m.size(), (uint64_t)m.getSizePower()};
      fwrite(r, 8, 2, out);
    } else if (code == 5) {
      std::vector<K> mk, mv;
      for (auto it = m.begin(); it != m.end(); ++it) {
        mk.push_back(it->first);
        mv.push_back(it->second);
      }
      const uint64_t c = mk.size();
      fwrite(&c, 8, 1, out);
      fwrite(mk.data(), sizeof(K), c, out);
      fwrite(mv.data(), sizeof(K), c, out);
    } else {
      fprintf(stderr, "bad op %llu\n", (unsigned long long)code);
      return 2;
    }
  }
  return 0;
}

int main(int argc, char** argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: %s <input> <output>\n", argv[0]);
    return 2;
  }
  FILE* in = fopen(argv[1], "rb");
  FILE* out = fopen(argv[2], "wb");
  if (!in || !out) {
    fprintf(stderr, "cannot open files\n");
    return 2;
  }
  uint64_t magic = 0;
  if (fread(&magic, 8, 1, in) != 1) {
    fprintf(stderr, "bad header\n");
    return 2;
  }
  if (magic == 0x48584753ull) {  // op script
    uint64_t g[4];
    if (fread(g, 8, 4, in) != 4) return 2;
    const int rc = (g[0] == 4) ? run_ops<uint32_t>(in, out, g[1], g[2], g[3]) : run_ops<uint64_t>(in, out, g[1], g[2], g[3]);
    fclose(in);
    fclose(out);
    return rc;
  }
  uint64_t h[7];
  h[0] = magic;
  if (fread(h + 1, 8, 6, in) != 6 || h[0] != 0x48584752ull) {
    fprintf(stderr, "bad header\n");
    return 2;
  }
  int rc = (h[1] == 4) ? run<uint32_t>(in, out, h[2], h[3], h[4], h[5], h[6])
                       : run<uint64_t>(in, out, h[2], h[3], h[4], h[5], h[6]);
  fclose(in);
  fclose(out);
  return rc;
}
