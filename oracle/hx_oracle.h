/*
 * hx_oracle.h — TEST INFRASTRUCTURE ONLY. A serial CPU restatement of the
 * Hashinator hot path used as the parity oracle for libhx. Nothing in the
 * product links or calls it; only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py do.
 *
 * Pinned against the reference's own CPU-only build (HASHINATOR_CPU_ONLY_MODE)
 * through the golden fixtures in tests/golden/ (made by
 * tests/golden/make_golden.py from oracle/_ref/ref_driver).
 */
#ifndef HX_ORACLE_H
#define HX_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ox_map ox_map;

typedef struct ox_pred { /* same layout and meaning as hx_pred (include/hx.h) */
  uint32_t op, field, flags, reserved;
  uint64_t a, b;
} ox_pred;

ox_map* ox_map_create(int key_bytes, int size_power);
void ox_map_destroy(ox_map* m);
/* returns 0 = success, 1 = fail (a key found no bucket) */
int ox_insert(ox_map* m, const void* keys, const void* vals, uint64_t n, float target_lf);
void ox_retrieve(const ox_map* m, const void* keys, void* vals, uint64_t n);
void ox_erase(ox_map* m, const void* keys, uint64_t n);
void ox_clean_tombstones(ox_map* m);
int ox_resize(ox_map* m, int new_size_power);
uint64_t ox_extract(const ox_map* m, const ox_pred* pred, void* out_pairs, uint64_t capacity);
/* valid (key, value) pairs in bucket order */
uint64_t ox_mapping(const ox_map* m, void* keys, void* vals, uint64_t capacity);
void ox_info(const ox_map* m, int* size_power, uint64_t* fill, uint64_t* tombstones, uint64_t* max_probe);
void* ox_buckets(ox_map* m);

uint64_t ox_copy_if(const void* in, void* out, uint64_t n, int elem_bytes, const ox_pred* pred);
void ox_exclusive_scan_u32(const uint32_t* in, uint32_t* out, uint64_t n);

uint32_t ox_fib_hash32(uint32_t key, int sp);
uint64_t ox_fib_hash64(uint64_t key, int sp);

#ifdef __cplusplus
}
#endif
#endif
