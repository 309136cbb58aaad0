/*
 * hx.h — C ABI of the GB300-native Hashinator hot path (libhx.so).
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes and
 * returns an hx_status. Device pointers must be device-accessible memory
 * (cudaMalloc, cudaMallocAsync or managed), and an array of elements of
 * k bytes (4-byte keys or words, 8-byte keys, 8- or 16-byte pairs) must start
 * at a multiple of k: a misaligned array is rejected with
 * HX_ERR_INVALID_ARG before any device work. Streams are passed as opaque
 * `hx_stream` values (a cudaStream_t; NULL = the legacy default stream).
 *
 * Calls are stream-ordered and asynchronous unless their comment says they
 * synchronise. The reference blocks the host after every kernel
 * (hashinator/hashers.h:55,76,98,118,128,140,151,161); a caller that wants
 * that behaviour calls cudaStreamSynchronize, or hx_get_info, afterwards.
 *
 * Each declaration names the reference interface it replaces
 * (path:line inside the Hashinator source tree, version 1.0.1).
 */
#ifndef HX_H
#define HX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef void* hx_stream; /* cudaStream_t */

/* Return codes. The reference aborts on CUDA errors (SPLIT_CHECK_ERR,
 * splitvector/split_allocators.h:33-40) and reports a full table through
 * Info::err = status::fail (hashinator/kernels_NVIDIA.h:443-445). */
typedef enum hx_status {
  HX_OK = 0,
  HX_ERR_OVERFLOW = 1,    /* insert could not place every key: table full      */
  HX_ERR_OOM = 2,         /* device allocation failed                          */
  HX_ERR_INVALID_ARG = 3, /* bad pointer, size, type or size power             */
  HX_ERR_CUDA = 4,        /* a CUDA runtime call failed (see hx_last_cuda_error)*/
  HX_ERR_TIMEOUT = 5,     /* a bounded device-side wait ran out                */
  HX_ERR_CAPACITY = 6     /* the output buffer is smaller than the result      */
} hx_status;

/* Hashinator::status (common.h:85): values of hx_info.err. */
enum { HX_STATUS_SUCCESS = 0, HX_STATUS_FAIL = 1, HX_STATUS_INVALID = 2 };

/* Host copy of the map metadata, mirroring Hashinator::Info
 * (hashinator/defaults.h:44-54). current_max_bucket_overflow keeps the
 * reference's meaning (the probe bound rounded up to a multiple of 32,
 * never below 32, common.h:54-57); max_probe is the exact longest probe
 * (distance + 1) that the device kernels use as their search bound.
 * last_clean_moved has no reference counterpart; it sizes the moved-key term
 * of clean_tombstones' traffic. */
typedef struct hx_info {
  int32_t size_power;
  int32_t err;
  uint64_t fill;
  uint64_t current_max_bucket_overflow;
  uint64_t tombstone_counter;
  uint64_t max_probe;
  uint64_t bucket_count;
  uint64_t last_clean_moved; /* keys the last clean_tombstones took out and
                                inserted again (0 when it found no tombstones) */
} hx_info;

/* Predicate descriptor: the C-ABI stand-in for the reference's `Rule`
 * functors (split_tools.h:1129, hashinator.h:1155). A user functor cannot
 * cross a C ABI; the descriptor covers the rules the reference's own tests,
 * benchmarks and clean_tombstones use. Evaluated on one field x:
 *   HX_PRED_ALL      true
 *   HX_PRED_MOD_LT   (x % a) <  b            (a != 0)
 *   HX_PRED_LT       x <  a
 *   HX_PRED_GE       x >= a
 *   HX_PRED_EQ       x == a
 *   HX_PRED_NE       x != a
 *   HX_PRED_MASK_EQ  (x & a) == b            (even: a=1,b=0; odd: a=1,b=1)
 *   HX_PRED_RANGE    a <= x < b
 *   HX_PRED_VALID    key is neither EMPTY nor TOMBSTONE (field ignored)
 *   HX_PRED_NOT_HOME valid key that does not sit in its home bucket
 *                    (map extraction only; the clean_tombstones rule,
 *                    hashinator.h:1285-1297, without its side effect)
 * field: HX_FIELD_ELEM for scalar arrays, HX_FIELD_KEY / HX_FIELD_VALUE for
 * hash_pair arrays. flags: HX_PRED_SKIP_SENTINELS makes a pair predicate
 * false on EMPTY and TOMBSTONE buckets (the reference's rules see those
 * buckets too, so the default keeps them); HX_PRED_NEGATE inverts. */
enum {
  HX_PRED_ALL = 0,
  HX_PRED_MOD_LT = 1,
  HX_PRED_LT = 2,
  HX_PRED_GE = 3,
  HX_PRED_EQ = 4,
  HX_PRED_NE = 5,
  HX_PRED_MASK_EQ = 6,
  HX_PRED_RANGE = 7,
  HX_PRED_VALID = 8,
  HX_PRED_NOT_HOME = 9
};
enum { HX_FIELD_ELEM = 0, HX_FIELD_KEY = 1, HX_FIELD_VALUE = 2 };
enum { HX_PRED_SKIP_SENTINELS = 1u, HX_PRED_NEGATE = 2u };

typedef struct hx_pred {
  uint32_t op;
  uint32_t field;
  uint32_t flags;
  uint32_t reserved;
  uint64_t a;
  uint64_t b;
} hx_pred;

typedef struct hx_map hx_map;

/* ---- map lifetime ------------------------------------------------------ */

/* Hashmap(int sizepower) (hashinator.h:120-129): a table of 2^size_power
 * buckets, every bucket (EMPTY, 0). key_bytes/val_bytes in {4, 8}:
 * (4,4) and (8,8) are hash_pair<uint32_t,uint32_t> (8 B) and
 * hash_pair<uint64_t,uint64_t> (16 B). EMPTY = all ones, TOMBSTONE =
 * EMPTY - 1 (hashinator.h:59-60). 1 <= size_power <= 31. Synchronises. */
hx_status hx_map_create(hx_map** out, int key_bytes, int val_bytes, int size_power, hx_stream stream);

/* ~Hashmap() (hashinator.h:213-216). Synchronises the device. */
hx_status hx_map_destroy(hx_map* map);

/* ---- the accelerated API (hashinator.h:1262-1409) ----------------------- */

/* insert(KEY*, VAL*, size_t, float targetLF = 0.5, stream) (hashinator.h:1319-1335).
 * Upsert of n keys. Grows the table first, like the reference, when
 * ceil(log2((fill + n) / target_lf)) exceeds the size power (target_lf <= 0
 * disables growth). Sets err = success, or fail if a key found no bucket. */
hx_status hx_insert(hx_map* map, const void* d_keys, const void* d_vals, uint64_t n, float target_lf,
                    hx_stream stream);

/* insertIndex(keys, len, targetLF, s) (hashinator.h:1339-1355,
 * insert_index_kernel kernels_NVIDIA.h:468-612): insert keys[i] with the
 * value i (its index in this call), same growth rule and upsert as
 * hx_insert. */
hx_status hx_insert_index(hx_map* map, const void* d_keys, uint64_t n, float target_lf, hx_stream stream);

/* insert(hash_pair*, size_t, float targetLF = 0.5, stream) (hashinator.h:1359-1374). */
hx_status hx_insert_pairs(hx_map* map, const void* d_pairs, uint64_t n, float target_lf, hx_stream stream);

/* retrieve(KEY*, VAL*, size_t, stream) (hashinator.h:1378-1384): d_vals[i]
 * receives the value of d_keys[i]; a missing key leaves d_vals[i] as it was. */
hx_status hx_retrieve(hx_map* map, const void* d_keys, void* d_vals, uint64_t n, hx_stream stream);

/* retrieve(hash_pair*, size_t, stream) (hashinator.h:1388-1394): writes
 * pairs[i].second for every key found. */
hx_status hx_retrieve_pairs(hx_map* map, void* d_pairs, uint64_t n, hx_stream stream);

/* erase(KEY*, size_t, stream) (hashinator.h:1398-1409): present keys become
 * TOMBSTONE; fill drops and tombstone_counter grows by the number erased. */
hx_status hx_erase(hx_map* map, const void* d_keys, uint64_t n, hx_stream stream);

/* clean_tombstones(stream) (hashinator.h:1262-1315): every TOMBSTONE bucket
 * becomes EMPTY and every key that does not sit in its home bucket is taken
 * out and inserted again; fill is unchanged, tombstone_counter becomes 0.
 * Uses a map-owned device buffer (grown on demand) for the moved keys. */
hx_status hx_clean_tombstones(hx_map* map, hx_stream stream);

/* extractPattern(hash_pair*, Rule, stream) (hashinator.h:1168-1185) and
 * extractPattern(SplitVector&, Rule, stream) (:1155-1165): order-preserving
 * copy of the buckets for which pred holds, in bucket order. At most
 * `capacity` pairs are written. The count goes to *d_count (device memory,
 * stream-ordered) if d_count is not NULL, and to *h_count (host memory,
 * the call then synchronises) if h_count is not NULL. A synchronous call
 * returns HX_ERR_CAPACITY when the count exceeds capacity. */
hx_status hx_extract_pattern(hx_map* map, const hx_pred* pred, void* d_out, uint64_t capacity, uint64_t* d_count,
                             uint64_t* h_count, hx_stream stream);

/* extractKeysByPattern(keys, rule, s) / extractAllKeys(keys, s)
 * (hashinator.h:1199-1239): the same selection as hx_extract_pattern, writing
 * only the key of each selected bucket (key_bytes each) in bucket order.
 * extractAllKeys is the predicate {HX_PRED_VALID}. Counts and capacity as
 * for hx_extract_pattern. */
hx_status hx_extract_keys(hx_map* map, const hx_pred* pred, void* d_out_keys, uint64_t capacity, uint64_t* d_count,
                          uint64_t* h_count, hx_stream stream);

/* resize(newSizePower, targets::device, stream) = device_rehash
 * (hashinator.h:285-336, :552-566): every valid pair moves into a new table
 * of 2^new_size_power buckets in one streaming pass; tombstones are dropped.
 * Sets err = success if fill is preserved. */
hx_status hx_resize(hx_map* map, int new_size_power, hx_stream stream);

/* resize_to_lf(targetLF, targets::device, s) (hashinator.h:530-549): grow
 * (device rehash) to the smallest size power whose load factor is at most
 * target_lf; nothing happens when it already is. Synchronises. */
hx_status hx_resize_to_lf(hx_map* map, float target_lf, hx_stream stream);

/* performCleanupTasks(s) (hashinator.h:643-650): clean_tombstones when
 * tombstones / buckets > 0.025, then device-rehash to the next size power
 * while the probe bound exceeds one 32-bucket window. Synchronises. */
hx_status hx_perform_cleanup_tasks(hx_map* map, hx_stream stream);

/* clear(targets::device, stream) (hashinator.h:492-518): every bucket
 * becomes (EMPTY, 0); fill, tombstones and the probe bound go to zero. */
hx_status hx_clear(hx_map* map, hx_stream stream);

/* size(), bucket_count(), tombstone_count(), load_factor(), getSizePower(),
 * copyMetadata(Info*, stream) (hashinator.h:441-457, 611, 228-230).
 * Synchronises the stream. */
hx_status hx_get_info(hx_map* map, hx_info* out, hx_stream stream);

/* peek_status() (hashinator.h:434-438): returns err and resets it to
 * invalid. Synchronises the stream. */
hx_status hx_peek_status(hx_map* map, int32_t* out, hx_stream stream);

/* expose_bucketdata() (hashinator.h:477-483): the device bucket array. */
hx_status hx_bucket_data(hx_map* map, void** d_buckets, uint64_t* bucket_count);

/* Device view of a map for element access from user kernels
 * (include/hx_device_api.cuh): Hashmap::upload() / get_device_pointer()
 * (hashinator.h:1420-1470) and the device API they enable. The pointers stay
 * valid until the next call that reallocates the table (insert with growth,
 * resize, destroy). Because device-side inserts bypass the host, the map's
 * host-side fill bound becomes the table size until hx_get_info refreshes it. */
typedef struct hx_device_view {
  void* buckets;
  int32_t size_power;
  int32_t reserved;
  unsigned long long* fill;
  unsigned long long* tombstones;
  unsigned int* max_probe;
  int32_t* err;
} hx_device_view;
hx_status hx_map_device_view(hx_map* map, hx_device_view* out);

/* Probe tuning (no reference counterpart: the reference fixes one 32-lane
 * warp per key, hashinator/defaults.h:26-38). group_width in
 * {1,2,4,8,16,32} lanes per key (1 = one thread per key with
 * keys_per_thread in {1,2,4,8} keys in flight), applied to insert, retrieve
 * and erase alike; block_size a multiple of 32 up to 256. 0 keeps the
 * current value. Until a group width is set, each call picks its own: one
 * thread per key for erase, for the re-insert of clean_tombstones and for
 * an insert whose load factor ends below 0.85 (4-lane groups above); small
 * probe groups for retrieve (u32: 4 lanes below load factor 0.875, 8 above;
 * u64: 4 below 0.8, 8 to 0.875, 16 above). */
hx_status hx_map_set_tuning(hx_map* map, int group_width, int keys_per_thread, int block_size);

/* Thread-per-key insert mode (no reference counterpart): blind_cas != 0
 * publishes into the home bucket with one CAS before reading anything;
 * 0 loads each key's first window and CASes into it afterwards. */
hx_status hx_map_set_insert_mode(hx_map* map, int blind_cas);

/* Thread-per-key window: 32 (one DRAM sector) or 64 bytes of buckets per
 * probe step. No reference counterpart. */
hx_status hx_map_set_window_bytes(hx_map* map, int bytes);

/* Maximum L2 fetch granularity of the calling thread's current device
 * context, 32/64/128 bytes (cudaLimitMaxL2FetchGranularity; a per-process
 * hint that ends with the process). Random 32-byte bucket sectors waste half
 * of every 64-byte fetch. No reference counterpart. */
hx_status hx_set_l2_fetch_granularity(int bytes);

/* ---- split::tools (splitvector/split_tools.h) -------------------------- */

/* Device scratch bytes that hx_exclusive_scan_u32 (op 0) or hx_copy_if
 * (op 1) needs for n elements; the replacement of
 * estimateMemoryForCompaction (split_tools.h:1065-1090). */
enum { HX_SCRATCH_SCAN = 0, HX_SCRATCH_COPY_IF = 1 };
hx_status hx_scratch_bytes(int op, uint64_t n, uint64_t* bytes);

/* split_prefix_scan(in, out, stream) (split_tools.h:363-418) for uint32:
 * exclusive sum, wrapping modulo 2^32, any n (the reference asserts a power
 * of two). d_scratch may be NULL (then it is allocated stream-ordered) or a
 * caller buffer of hx_scratch_bytes(HX_SCRATCH_SCAN, n) bytes. In-place
 * (d_out == d_in) is allowed. */
hx_status hx_exclusive_scan_u32(const uint32_t* d_in, uint32_t* d_out, uint64_t n, void* d_scratch,
                                uint64_t scratch_bytes, hx_stream stream);

/* copy_if(in, out, Rule, stream) (split_tools.h:1129-1223): stable stream
 * compaction of n elements of elem_bytes in {4, 8, 16} (uint32_t,
 * hash_pair<u32,u32>, hash_pair<u64,u64>). Count reporting and capacity
 * as for hx_extract_pattern. */
hx_status hx_copy_if(const void* d_in, void* d_out, uint64_t n, int elem_bytes, const hx_pred* pred,
                     uint64_t capacity, uint64_t* d_count, uint64_t* h_count, void* d_scratch,
                     uint64_t scratch_bytes, hx_stream stream);

/* ---- batched maps ------------------------------------------------------- */
/* No reference counterpart as one call: the reference serves many small maps
 * with one Hashmap object and one launch sequence per map (its per-map
 * accelerated API above). A batch is a directory of n_maps independent maps
 * (table i has 2^size_powers[i] buckets, 2 <= size power <= 31) in one device
 * arena; a plan describes one round of work per map and runs it in a single
 * persistent launch whose per-map results equal the plain per-map calls. */
typedef struct hx_batch hx_batch;
typedef struct hx_batch_plan hx_batch_plan;

/* One round of work. Keys/values/outputs are device arrays; the offsets are
 * HOST arrays of n_maps + 1 entries (map i owns [off[i], off[i+1])). Any
 * section may be absent (NULL offsets). Order per map: insert (no growth),
 * retrieve, erase, then clean_tombstones if clean != 0. */
typedef struct hx_batch_work {
  const void* ins_keys;
  const void* ins_vals;
  const uint64_t* ins_offsets;
  const void* query_keys;
  void* query_out;
  const uint64_t* query_offsets;
  const void* erase_keys;
  const uint64_t* erase_offsets;
  int clean;
} hx_batch_work;

hx_status hx_batch_create(hx_batch** out, uint32_t n_maps, const int32_t* size_powers, int key_bytes,
                          int val_bytes, hx_stream stream);
hx_status hx_batch_destroy(hx_batch* batch);
/* clear(targets::device) for every map. */
hx_status hx_batch_clear(hx_batch* batch, hx_stream stream);
/* Metadata of one map (synchronises), as hx_get_info. */
hx_status hx_batch_map_info(hx_batch* batch, uint32_t map, hx_info* out, hx_stream stream);
hx_status hx_batch_bucket_data(hx_batch* batch, uint32_t map, void** d_buckets, uint64_t* bucket_count);

/* Builds the tile list (synchronises once). The plan keeps the pointers of
 * `work`; run it as many times as needed. */
hx_status hx_batch_plan_create(hx_batch* batch, const hx_batch_work* work, hx_batch_plan** out, hx_stream stream);
hx_status hx_batch_plan_destroy(hx_batch_plan* plan);
/* group_width in {1,4,8,16,32} lanes per key, block_size in {128,256,512},
 * tile_keys keys per tile (64..2^20); 0 keeps the current value. */
hx_status hx_batch_set_tuning(hx_batch_plan* plan, int group_width, int block_size, int tile_keys, hx_stream stream);
/* The fused persistent launch. */
hx_status hx_batch_run(hx_batch_plan* plan, hx_stream stream);
/* The same launch, captured once into a CUDA graph and replayed. */
hx_status hx_batch_run_graph(hx_batch_plan* plan, hx_stream stream);
/* The plain path: the per-map launches of hx_insert, hx_retrieve, hx_erase
 * and hx_clean_tombstones for every map in turn. */
hx_status hx_batch_run_per_map(hx_batch_plan* plan, hx_stream stream);
/* Autotuner (no reference counterpart): times the plan's captured-graph
 * replay (hx_batch_run_graph, the launch the product runs) over the grid
 * group_widths x block_sizes x tile_keys (NULL arrays: {1,4,8,16,32} x
 * {128,256,512} x {512,2048,8192}); for each point one warm-up replay and
 * then `reps` timed replays (CUDA events on `stream`), each after `reset`
 * has restored the maps to the state the round starts from (reset = NULL:
 * hx_batch_clear, for a round that starts from empty maps). Leaves the plan
 * on the fastest point and the maps reset; writes up to trials_capacity
 * trials (milliseconds = the fastest timed replay of each point) and the
 * best one. Synchronises. A trial whose bounded waits ran out ends the
 * search with HX_ERR_TIMEOUT. */
typedef struct hx_batch_trial {
  int32_t group_width;
  int32_t block_size;
  int32_t tile_keys;
  float ms;
} hx_batch_trial;
typedef hx_status (*hx_batch_reset_fn)(void* user, hx_stream stream);
hx_status hx_batch_autotune(hx_batch_plan* plan, const int32_t* group_widths, uint32_t n_groups,
                            const int32_t* block_sizes, uint32_t n_blocks, const int32_t* tile_keys, uint32_t n_tiles,
                            int reps, hx_batch_reset_fn reset, void* reset_user, hx_stream stream,
                            hx_batch_trial* trials, uint32_t trials_capacity, hx_batch_trial* best);
/* Error word of the last fused run (synchronises): 0 ok, 1 a bounded wait ran
 * out (HX_ERR_TIMEOUT), 2 a moved list overflowed (HX_ERR_CAPACITY). */
hx_status hx_batch_check(hx_batch_plan* plan, int32_t* error, hx_stream stream);
/* Failure-detection test hook (no reference counterpart): with enable != 0
 * the plan's counter of `phase` tiles for `map` starts one higher than the
 * tiles that exist, so every later-phase tile of that map waits in vain
 * until its bounded wait (about one second) runs out; the launch still
 * returns and hx_batch_check reports HX_ERR_TIMEOUT. enable = 0 undoes it.
 * Phases: 0 insert, 1 query, 2 erase, 3..5 clean_tombstones. Synchronises. */
hx_status hx_batch_inject_stall(hx_batch_plan* plan, uint32_t map, int phase, int enable, hx_stream stream);

/* ---- serving loop ------------------------------------------------------- */
/* No reference counterpart (the reference has no request loop). A server
 * keeps many maps resident and runs queued requests in rounds: one fused
 * launch per round, requests on different maps concurrently, requests on the
 * same map in admission order, several rounds in flight (the host forms the
 * next round while the GPU runs the current one). Before a round, a map
 * whose load factor would pass max_load_factor is grown by an on-device
 * rehash; tables are admitted against memory_budget_bytes, and an insert
 * that cannot grow its table within the budget completes with HX_ERR_OOM.
 * One host thread drives a server. Tables live in a stream-ordered memory
 * pool that the server creates for itself, with its release threshold at
 * the maximum, so that growth does not return memory to the driver at every
 * synchronisation; the process's other pools are left as they were, and
 * hx_server_destroy destroys the server's pool (it synchronises the device). */
typedef struct hx_server hx_server;
enum { HX_OP_INSERT = 0, HX_OP_QUERY = 1, HX_OP_ERASE = 2 };
typedef struct hx_request {
  uint32_t map;
  uint32_t op;       /* HX_OP_*: insert keys+vals, query keys -> out (misses untouched), erase keys */
  const void* keys;  /* device arrays, alive until the request completes */
  const void* vals;
  void* out;
  uint64_t n;
  uint64_t tag;      /* returned in the completion */
} hx_request;
typedef struct hx_completion {
  uint64_t tag;
  uint64_t complete_ns; /* host steady-clock ns of the end of the request's round */
  int32_t status;       /* HX_OK, HX_ERR_OOM (insert not admitted), HX_ERR_TIMEOUT */
  int32_t reserved;
} hx_completion;

hx_status hx_server_create(hx_server** out, int key_bytes, uint64_t memory_budget_bytes, float max_load_factor,
                           uint32_t max_maps, uint32_t max_round_requests, uint64_t max_round_keys,
                           uint32_t rounds_in_flight);
hx_status hx_server_destroy(hx_server* server);
/* A new empty map of 2^size_power buckets, if it fits the budget (else HX_ERR_OOM). */
hx_status hx_server_add_map(hx_server* server, int size_power, uint32_t* map_id);
hx_status hx_server_submit(hx_server* server, const hx_request* requests, uint32_t count);
/* Forms and launches one round from the queue if a round slot is free;
 * *launched = requests in it (0 if none). Never blocks on the GPU. */
hx_status hx_server_step(hx_server* server, uint32_t* launched);
/* Completions since the last poll (at most capacity). */
hx_status hx_server_poll(hx_server* server, hx_completion* out, uint32_t capacity, uint32_t* n_out);
/* Runs until the queue is empty and every round has completed. */
hx_status hx_server_drain(hx_server* server);
hx_status hx_server_map_info(hx_server* server, uint32_t map, hx_info* out);
hx_status hx_server_bucket_data(hx_server* server, uint32_t map, void** d_buckets, uint64_t* bucket_count);
hx_status hx_server_memory(hx_server* server, uint64_t* used, uint64_t* budget);
typedef struct hx_server_stats {
  uint64_t rounds, requests, keys;  /* launched */
  uint64_t growths, growth_bytes;   /* on-device rehashes and the bytes of their new tables */
  uint64_t rejected, timeouts;
  uint64_t host_ns_step;            /* host time spent forming and launching rounds */
  uint32_t max_stage_depth;         /* longest per-map dependency chain in a round */
  uint32_t reserved;
} hx_server_stats;
hx_status hx_server_get_stats(hx_server* server, hx_server_stats* out);
/* Replays a request trace in real time: request i is submitted once
 * arrival_ns[i] (ns after the start, non-decreasing) has passed; returns
 * when all requests completed, with complete_ns[i] (ns after the start) and
 * status[i]. The loop is native so arrivals are not limited by a caller. */
hx_status hx_server_run_trace(hx_server* server, const hx_request* requests, const uint64_t* arrival_ns,
                              uint32_t count, uint64_t* complete_ns, int32_t* status, uint64_t* t_start_ns);

/* Exclusive u32 scan that allocates nothing. No counterpart in the
 * reference: it is hx_exclusive_scan_u32 for callers that may not allocate
 * device memory when they scan (a host framework that owns all device memory,
 * a fixed-budget serving loop, a time-stepping loop where cudaMalloc would
 * synchronise the device). Its look-back scratch is a static device array of
 * HX_NOALLOC_SCAN_SCRATCH_BYTES compiled into libhx, held on every GPU that
 * loads the library until the process exits.
 * - n <= HX_NOALLOC_SCAN_MAX_N (2^28); a larger n returns HX_ERR_INVALID_ARG
 *   and launches nothing. In-place (d_out == d_in) is allowed.
 * - The first call on each device looks up the array's device address (with
 *   that device current); make that first call before any stream capture.
 *   The address is kept for the device's current context; after a
 *   cudaDeviceReset the next call looks it up again in the new context.
 * - Every call shares the one array and clears the part it uses. Calls that
 *   overlap on the GPU race on it and give wrong results: serialise them,
 *   for example on one stream.
 * - The scan's waits between tiles are bounded. If one runs out (which
 *   needs the GPU to stop scheduling the kernel's blocks), this entry point
 *   cannot report it: it returns before the kernel ends, and the array that
 *   would hold the error word is private and cleared by the next call. The
 *   allocating scan with caller scratch reports HX_ERR_TIMEOUT instead.
 * - No cudaMalloc, cudaFree or allocating library call is made. */
#define HX_NOALLOC_SCAN_MAX_N (1ull << 28)
#define HX_NOALLOC_SCAN_SCRATCH_BYTES (256ull + 8ull * (HX_NOALLOC_SCAN_MAX_N / 4096ull))
hx_status hx_exclusive_scan_u32_noalloc(const uint32_t* d_in, uint32_t* d_out, uint64_t n, hx_stream stream);

/* ---- diagnostics -------------------------------------------------------- */

const char* hx_status_string(hx_status status);
/* Random-access ceiling probe (no reference counterpart): mode 0 reads
 * n_ops random 32-byte sectors of d_buf, mode 1 does n_ops random 64-bit CAS
 * (0 -> nonzero) on word 0 of random sectors, so the buffer is modified.
 * d_buf is 32-byte aligned, bytes >= 64; the largest power-of-two number of
 * sectors that fits is used. Time it on the stream. */
hx_status hx_diag_random_access(void* d_buf, uint64_t bytes, uint64_t n_ops, int mode, hx_stream stream);
/* The last cudaError_t value seen by the library on this host thread. */
int hx_last_cuda_error(void);
/* Number of kernels libhx has launched in this process. */
uint64_t hx_kernel_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif /* HX_H */
