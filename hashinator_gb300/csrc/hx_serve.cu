// hx_serve.cu — serving loop: continuous batching of insert / query / erase
// requests over many resident maps.
//
// Requests are queued as they arrive. A step takes the requests at the head
// of the queue (up to a key and request budget) and runs them as one round:
// one fused persistent launch in which requests on different maps proceed
// concurrently, while requests on the same map are chained in admission
// order (a request's tiles wait, bounded, until its predecessor on that map
// is done — the same ticket argument as the batched kernel: predecessors are
// earlier in the ticket order, so only running CTAs are ever waited on).
// Several rounds are in flight at once: the host forms round k+1 while the
// GPU runs round k, and requests that arrive meanwhile join the next round.
//
// Every table stays resident. Before a round, a map whose occupancy (keys plus
// tombstones, which insert never reuses) would pass the load-factor limit is
// rehashed on the device (device_rehash, hashinator.h:285-336): tombstones
// are dropped and the table grows only if its live keys need it, allocated
// against the server's device-memory budget. An insert that cannot be given
// room within the budget is rejected and reported; the map's other requests
// proceed.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <vector>

#include "hx_host.h"
#include "hx_internal.h"
#include "hx_probe.cuh"

namespace hx {

enum : unsigned { SOP_INSERT = 0, SOP_QUERY = 1, SOP_ERASE = 2 };

struct SReq {
  const void* keys;
  const void* vals;
  void* out;
  unsigned long long n;
  unsigned map;
  unsigned op;
  int wait;        // stage this request waits for (the map's previous stage), or -1
  unsigned stage;  // stage whose counter this request's tiles count off
};
struct STile {
  unsigned req;
  unsigned count;
  unsigned long long begin;
};
struct SMap {
  void* table;
  int sp;
  int pad;
};

template <class P>
struct ServeArgs {
  const SMap* maps;
  DInfo* info;
  const SReq* reqs;
  const STile* tiles;
  unsigned n_tiles;
  unsigned* work;
  unsigned* error;
  unsigned* remaining;  // tiles left per stage
};

constexpr unsigned long long kServeWaitNs = 1000000000ull;

__device__ __forceinline__ bool serve_wait_zero(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  if (v == 0) return true;
  unsigned long long t0, t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  for (unsigned i = 0; i < (1u << 26); ++i) {
    __nanosleep(i < 32 ? 32 : 256);
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    if (v == 0) return true;
    if ((i & 63) == 63) {
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
      if (t - t0 > kServeWaitNs) return false;
    }
  }
  return false;
}

template <class P>
// A round is latency bound (random probes into many tables): a register cap
// for 32 resident warps per SM (74 registers gave 24) raised the saturated
// throughput from 11.8 to 13.0 G keys/s; 48 warps gave no more.
#ifndef HX_SERVE_MIN_WARPS
#define HX_SERVE_MIN_WARPS 32
#endif
__global__ void __launch_bounds__(256, HX_SERVE_MIN_WARPS / 8) k_serve(ServeArgs<P> a) {
  using K = typename PairTraits<P>::K;
  using V = typename PairTraits<P>::V;
  constexpr int BLOCK = 256;
  constexpr int BT = sizeof(P) == 8 ? 4 : 2;
  constexpr int U = 2;
  __shared__ STile s_t;
  __shared__ SReq s_r;
  __shared__ unsigned s_ok, s_ins, s_max, s_fail, s_erased, s_end;
  const int lane = threadIdx.x & 31;
  for (;;) {
    if (threadIdx.x == 0) {
      const unsigned idx = atomicAdd(a.work, 1u);
      s_end = idx >= a.n_tiles;
      s_ins = s_max = s_fail = s_erased = 0;
      s_ok = 1;
      if (!s_end) {
        s_t = a.tiles[idx];
        s_r = a.reqs[s_t.req];
        if (s_r.wait >= 0 && !serve_wait_zero(a.remaining + s_r.wait)) {
          s_ok = 0;
          atomicExch(a.error, 1u);
        }
      }
    }
    __syncthreads();
    if (s_end) break;
    __threadfence();
    const STile t = s_t;
    const SReq r = s_r;
    if (s_ok) {
      const SMap md = a.maps[r.map];
      P* tab = static_cast<P*>(md.table);
      const int sp = md.sp;
      DInfo* inf = a.info + r.map;
      unsigned ins = 0, maxd = 0, erased = 0;
      bool fail = false;
      const K* keys = static_cast<const K*>(r.keys);
      if (r.op == SOP_INSERT) {
        const V* vals = static_cast<const V*>(r.vals);
        for (unsigned k = threadIdx.x; k < t.count; k += BLOCK)
          insert_one_t1<P, BT>(tab, sp, keys[t.begin + k], vals[t.begin + k], ins, maxd, fail);
      } else {
        const bool erase = r.op == SOP_ERASE;
        V* out = static_cast<V*>(r.out);
        const unsigned limit = inf->max_probe;
        if (limit) {
          for (unsigned base = 0; base < t.count; base += BLOCK * U) {
            K key[U];
            bool act[U];
            uint32_t h[U];
            Window<P, BT> w[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
              const unsigned k = base + u * BLOCK + threadIdx.x;
              act[u] = k < t.count;
              if (act[u]) {
                key[u] = keys[t.begin + k];
                act[u] = key[u] != PairTraits<P>::EMPTY && key[u] != PairTraits<P>::TOMB;
              }
              if (act[u]) {
                h[u] = home_slot(key[u], sp);
                load_buckets<BT>(tab + (h[u] & ~(uint32_t)(BT - 1)), w[u].k, w[u].v);
              }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
              if (!act[u]) continue;
              uint32_t slot;
              V v;
              if (find_t1<P, BT>(tab, sp, key[u], limit, h[u], w[u], slot, v)) {
                if (erase) {
                  if (cas_key(tab + slot, key[u], PairTraits<P>::TOMB)) ++erased;
                } else {
                  out[t.begin + base + u * BLOCK + threadIdx.x] = v;
                }
              }
            }
          }
        }
      }
      ins = __reduce_add_sync(0xffffffffu, ins);
      maxd = __reduce_max_sync(0xffffffffu, maxd);
      erased = __reduce_add_sync(0xffffffffu, erased);
      const bool anyfail = __any_sync(0xffffffffu, fail);
      if (lane == 0) {
        if (ins) atomicAdd(&s_ins, ins);
        if (maxd) atomicMax(&s_max, maxd);
        if (erased) atomicAdd(&s_erased, erased);
        if (anyfail) atomicExch(&s_fail, 1u);
      }
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
      DInfo* inf = a.info + r.map;
      if (s_ins) atomicAdd(&inf->fill, (unsigned long long)s_ins);
      if (s_max) atomicMax(&inf->max_probe, s_max);
      if (s_fail) atomicExch(&inf->err, HX_STATUS_FAIL);
      if (s_erased) {
        atomicAdd(&inf->tombstones, (unsigned long long)s_erased);
        atomicAdd(&inf->fill, 0ull - (unsigned long long)s_erased);
      }
      __threadfence();
      atomicSub(a.remaining + r.stage, 1u);
    }
  }
}

// ---- batched rehash of the tables a round needs to grow or clean ----------
struct GrowTask {
  void* old_table;
  void* new_table;
  unsigned long long old_n;
  int new_sp;
  unsigned map;
};
struct GrowChunk {
  unsigned task;
  unsigned count;
  unsigned long long begin;
};

// (EMPTY, 0) into every bucket of the new tables; chunk 0 of a task also
// resets the map's metadata (a rehash drops tombstones and re-counts fill).
template <class P>
__global__ void __launch_bounds__(256) k_grow_fill(const GrowTask* tasks, const GrowChunk* chunks, unsigned n_chunks,
                                                   DInfo* info) {
  for (unsigned c = blockIdx.x; c < n_chunks; c += gridDim.x) {
    const GrowChunk ch = chunks[c];
    const GrowTask tk = tasks[ch.task];
    P* t = static_cast<P*>(tk.new_table);
    P e;
    e.first = PairTraits<P>::EMPTY;
    e.second = 0;
    for (unsigned k = threadIdx.x; k < ch.count; k += blockDim.x) t[ch.begin + k] = e;
    if (ch.begin == 0 && threadIdx.x == 0) {
      DInfo* inf = info + tk.map;
      inf->fill = 0;
      inf->tombstones = 0;
      inf->max_probe = 0;
    }
  }
}

// Every valid pair of the old tables into the new ones (thread per bucket).
template <class P>
__global__ void __launch_bounds__(256) k_grow_move(const GrowTask* tasks, const GrowChunk* chunks, unsigned n_chunks,
                                                   DInfo* info) {
  constexpr int BT = sizeof(P) == 8 ? 4 : 2;
  __shared__ unsigned s_ins, s_max, s_fail;
  const int lane = threadIdx.x & 31;
  for (unsigned c = blockIdx.x; c < n_chunks; c += gridDim.x) {
    if (threadIdx.x == 0) s_ins = s_max = s_fail = 0;
    __syncthreads();
    const GrowChunk ch = chunks[c];
    const GrowTask tk = tasks[ch.task];
    const P* o = static_cast<const P*>(tk.old_table);
    P* t = static_cast<P*>(tk.new_table);
    unsigned ins = 0, maxd = 0;
    bool fail = false;
    for (unsigned k = threadIdx.x; k < ch.count; k += blockDim.x) {
      const P pr = o[ch.begin + k];
      if (pr.first != PairTraits<P>::EMPTY && pr.first != PairTraits<P>::TOMB)
        insert_one_t1<P, BT>(t, tk.new_sp, pr.first, pr.second, ins, maxd, fail);
    }
    ins = __reduce_add_sync(0xffffffffu, ins);
    maxd = __reduce_max_sync(0xffffffffu, maxd);
    const bool anyfail = __any_sync(0xffffffffu, fail);
    if (lane == 0) {
      if (ins) atomicAdd(&s_ins, ins);
      if (maxd) atomicMax(&s_max, maxd);
      if (anyfail) atomicExch(&s_fail, 1u);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      DInfo* inf = info + tk.map;
      if (s_ins) atomicAdd(&inf->fill, (unsigned long long)s_ins);
      if (s_max) atomicMax(&inf->max_probe, s_max);
      if (s_fail) atomicExch(&inf->err, HX_STATUS_FAIL);
    }
    __syncthreads();
  }
}

static uint64_t now_ns() {
  return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

struct ServeMap {
  int sp = 0;
  void* table = nullptr;
  uint64_t bytes = 0;
  uint64_t fill_ub = 0;          // upper bound of fill once every launched round is done
  uint64_t tomb_ub = 0;          // upper bound of tombstones once every launched round is done
  uint64_t in_flight = 0;        // inserts launched in rounds not yet completed
  uint64_t in_flight_erase = 0;  // erase keys launched in rounds not yet completed
  uint64_t rehash_round = 0;     // first round that runs on the current table
};

struct Pending {
  hx_request r;
  uint64_t seq;
};

struct Slot {
  bool busy = false;
  uint64_t round_no = 0;  // launch order
  size_t n_maps = 0;      // maps covered by this round's metadata snapshot
  SReq* h_reqs = nullptr;
  STile* h_tiles = nullptr;
  unsigned* h_rem = nullptr;
  SMap* h_dir = nullptr;
  DInfo* h_info = nullptr;
  unsigned* h_err = nullptr;
  SReq* d_reqs = nullptr;
  STile* d_tiles = nullptr;
  unsigned* d_cnt = nullptr;  // work, error, remaining[]
  cudaEvent_t done = nullptr;
  std::vector<uint64_t> tags;
  std::vector<std::pair<unsigned, uint64_t>> inserts;  // (map, keys) launched in this round
  std::vector<std::pair<unsigned, uint64_t>> erases;   // (map, keys) launched in this round
  GrowTask* h_tasks = nullptr;
  GrowChunk* h_chunks = nullptr;
  GrowTask* d_tasks = nullptr;
  GrowChunk* d_chunks = nullptr;
  size_t chunk_cap = 0;
};

}  // namespace hx

struct hx_server {
  int kb = 8;
  uint64_t budget = 0, used = 0;
  float max_lf = 0.8f;
  uint32_t max_maps = 0;
  uint32_t max_round_requests = 0;
  uint64_t max_round_keys = 0;
  uint32_t tile_keys = 4096;
  std::vector<hx::ServeMap> maps;
  hx::SMap* d_maps = nullptr;
  hx::DInfo* d_info = nullptr;
  cudaStream_t s = nullptr;
  cudaMemPool_t pool = nullptr;  // the tables' stream-ordered pool
  std::deque<hx::Pending> queue;
  std::vector<hx::Slot> slots;
  uint64_t seq = 0;
  uint64_t rounds = 0;
  cudaEvent_t t0 = nullptr;
  uint64_t t0_ns = 0;
  bool t0_set = false;
  std::vector<hx_completion> done;  // completed since the last poll
  uint64_t timeouts = 0;
  hx_server_stats st{};
};

namespace hx {

static uint64_t pb(const hx_server* sv) { return sv->kb == 4 ? 8 : 16; }

static void view_of(hx_server* sv, unsigned i, hx_map* v) {
  v->key_bytes = sv->kb;
  v->val_bytes = sv->kb;
  v->sp = sv->maps[i].sp;
  v->buckets = sv->maps[i].table;
  v->info = sv->d_info + i;
  v->fill_ub = sv->maps[i].fill_ub;
}

// Completed rounds: completion times, fill bounds refreshed from the
// round's metadata snapshot.
static hx_status reap(hx_server* sv, bool wait_oldest) {
  // rounds run in launch order on one stream: reap them in that order
  std::vector<Slot*> busy;
  for (auto& sl : sv->slots)
    if (sl.busy) busy.push_back(&sl);
  std::sort(busy.begin(), busy.end(), [](const Slot* a, const Slot* b) { return a->round_no < b->round_no; });
  for (Slot* slp : busy) {
    Slot& sl = *slp;
    cudaError_t q = wait_oldest ? cudaEventSynchronize(sl.done) : cudaEventQuery(sl.done);
    wait_oldest = false;
    if (q == cudaErrorNotReady) break;
    if (q != cudaSuccess) return cuda_status(q);
    float ms = 0.f;
    if (sv->t0_set) cudaEventElapsedTime(&ms, sv->t0, sl.done);
    const uint64_t t_ns = sv->t0_ns + (uint64_t)((double)ms * 1e6);
    const int32_t st = *sl.h_err ? HX_ERR_TIMEOUT : HX_OK;
    if (*sl.h_err) {
      sv->timeouts++;
      sv->st.timeouts++;
    }
    for (uint64_t tag : sl.tags) sv->done.push_back(hx_completion{tag, t_ns, st, 0});
    for (auto& ins : sl.inserts) sv->maps[ins.first].in_flight -= ins.second;
    for (auto& er : sl.erases) sv->maps[er.first].in_flight_erase -= er.second;
    for (size_t i = 0; i < sl.n_maps && i < sv->maps.size(); ++i) {
      ServeMap& m = sv->maps[i];
      m.fill_ub = sl.h_info[i].fill + m.in_flight;  // a rehash keeps fill
      // tombstones of a snapshot taken before the map's last rehash are gone
      if (sl.round_no >= m.rehash_round) m.tomb_ub = sl.h_info[i].tombstones + m.in_flight_erase;
    }
    sl.busy = false;
    sl.tags.clear();
    sl.inserts.clear();
    sl.erases.clear();
  }
  return HX_OK;
}

}  // namespace hx

using namespace hx;

extern "C" {

hx_status hx_server_create(hx_server** out, int key_bytes, uint64_t memory_budget_bytes, float max_load_factor,
                           uint32_t max_maps, uint32_t max_round_requests, uint64_t max_round_keys,
                           uint32_t rounds_in_flight) {
  if (!out || (key_bytes != 4 && key_bytes != 8) || !(max_load_factor > 0.f && max_load_factor <= 1.f) ||
      max_maps == 0 || max_round_requests == 0 || max_round_keys == 0 || rounds_in_flight == 0 ||
      rounds_in_flight > 16)
    return HX_ERR_INVALID_ARG;
  *out = nullptr;
  hx_server* sv = new hx_server();
  sv->kb = key_bytes;
  sv->budget = memory_budget_bytes;
  sv->max_lf = max_load_factor;
  sv->max_maps = max_maps;
  sv->max_round_requests = max_round_requests;
  sv->max_round_keys = max_round_keys;
  const uint64_t max_tiles = max_round_requests + max_round_keys / 256 + 1;
  cudaError_t e = cudaStreamCreateWithFlags(&sv->s, cudaStreamNonBlocking);
  // Tables grow and shrink through the stream-ordered allocator, from a pool
  // of the server's own: freed tables stay in it (release threshold = max)
  // instead of going back to the driver at every synchronisation, and no
  // other allocation of the process (torch's, another library's) is affected.
  {
    int dev = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    if (e == cudaSuccess) e = cudaMemPoolCreate(&sv->pool, &props);
    uint64_t keep = ~0ull;
    if (e == cudaSuccess) e = cudaMemPoolSetAttribute(sv->pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&sv->d_maps), max_maps * sizeof(SMap));
  if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&sv->d_info), max_maps * sizeof(DInfo));
  if (e == cudaSuccess) e = cudaEventCreate(&sv->t0);
  sv->slots.resize(rounds_in_flight);
  for (auto& sl : sv->slots) {
    if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&sl.h_reqs), max_round_requests * sizeof(SReq));
    if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&sl.h_tiles), max_tiles * sizeof(STile));
    if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&sl.h_rem), max_round_requests * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&sl.h_dir), max_maps * sizeof(SMap));
    if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&sl.h_info), max_maps * sizeof(DInfo));
    if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&sl.h_err), sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&sl.d_reqs), max_round_requests * sizeof(SReq));
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&sl.d_tiles), max_tiles * sizeof(STile));
    if (e == cudaSuccess)
      e = cudaMalloc(reinterpret_cast<void**>(&sl.d_cnt), (2 + max_round_requests) * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, cudaEventDefault);
    sl.chunk_cap = 1 << 16;
    if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&sl.h_tasks), max_maps * sizeof(GrowTask));
    if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&sl.h_chunks), sl.chunk_cap * sizeof(GrowChunk));
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&sl.d_tasks), max_maps * sizeof(GrowTask));
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&sl.d_chunks), sl.chunk_cap * sizeof(GrowChunk));
  }
  if (e != cudaSuccess) {
    *out = sv;
    hx_server_destroy(sv);
    *out = nullptr;
    return cuda_status(e);
  }
  *out = sv;
  return HX_OK;
}

hx_status hx_server_destroy(hx_server* sv) {
  if (!sv) return HX_ERR_INVALID_ARG;
  if (sv->s) cudaStreamSynchronize(sv->s);
  for (auto& m : sv->maps) cudaFree(m.table);
  for (auto& sl : sv->slots) {
    cudaFreeHost(sl.h_reqs);
    cudaFreeHost(sl.h_tiles);
    cudaFreeHost(sl.h_rem);
    cudaFreeHost(sl.h_dir);
    cudaFreeHost(sl.h_info);
    cudaFreeHost(sl.h_err);
    cudaFree(sl.d_reqs);
    cudaFree(sl.d_tiles);
    cudaFree(sl.d_cnt);
    cudaFreeHost(sl.h_tasks);
    cudaFreeHost(sl.h_chunks);
    cudaFree(sl.d_tasks);
    cudaFree(sl.d_chunks);
    if (sl.done) cudaEventDestroy(sl.done);
  }
  cudaFree(sv->d_maps);
  cudaFree(sv->d_info);
  if (sv->t0) cudaEventDestroy(sv->t0);
  if (sv->s) cudaStreamDestroy(sv->s);
  if (sv->pool) {
    cudaDeviceSynchronize();  // every table's free has completed
    cudaMemPoolDestroy(sv->pool);
  }
  delete sv;
  return HX_OK;
}

hx_status hx_server_add_map(hx_server* sv, int size_power, uint32_t* map_id) {
  if (!sv || !map_id || size_power < 2 || size_power > 31) return HX_ERR_INVALID_ARG;
  if (sv->maps.size() >= sv->max_maps) return HX_ERR_CAPACITY;
  const uint64_t bytes = (1ull << size_power) * pb(sv);
  if (sv->used + bytes > sv->budget) return HX_ERR_OOM;  // admission against the budget
  ServeMap m;
  m.sp = size_power;
  m.bytes = bytes;
  HX_CUDA(cudaMallocFromPoolAsync(&m.table, bytes, sv->pool, sv->s));
  hx_map v;
  v.key_bytes = sv->kb;
  v.val_bytes = sv->kb;
  v.sp = size_power;
  v.buckets = m.table;
  const uint32_t id = (uint32_t)sv->maps.size();
  v.info = sv->d_info + id;
  hx_status st = hx_clear(&v, sv->s);
  if (st != HX_OK) {
    cudaFreeAsync(m.table, sv->s);
    return st;
  }
  sv->used += bytes;
  sv->maps.push_back(m);
  *map_id = id;
  return HX_OK;
}

hx_status hx_server_submit(hx_server* sv, const hx_request* reqs, uint32_t count) {
  if (!sv || (count && !reqs)) return HX_ERR_INVALID_ARG;
  for (uint32_t i = 0; i < count; ++i) {
    const hx_request& r = reqs[i];
    if (r.map >= sv->maps.size() || r.op > SOP_ERASE || (r.n && !r.keys) || (r.op == SOP_INSERT && r.n && !r.vals) ||
        (r.op == SOP_QUERY && r.n && !r.out) || misaligned(r.keys, (unsigned)sv->kb) ||
        misaligned(r.vals, (unsigned)sv->kb) || misaligned(r.out, (unsigned)sv->kb))
      return HX_ERR_INVALID_ARG;
  }
  for (uint32_t i = 0; i < count; ++i) sv->queue.push_back(Pending{reqs[i], sv->seq++});
  return HX_OK;
}

static hx_status server_step(hx_server* sv, uint32_t* launched);

hx_status hx_server_step(hx_server* sv, uint32_t* launched) {
  HX_RANGE("hx_server_step");
  if (!sv) return HX_ERR_INVALID_ARG;
  const uint64_t t0 = now_ns();
  hx_status st = server_step(sv, launched);
  sv->st.host_ns_step += now_ns() - t0;
  return st;
}

static hx_status server_step(hx_server* sv, uint32_t* launched) {
  if (launched) *launched = 0;
  hx_status st = reap(sv, false);
  if (st != HX_OK) return st;
  if (sv->queue.empty()) return HX_OK;
  Slot* sl = nullptr;
  for (auto& x : sv->slots)
    if (!x.busy) {
      sl = &x;
      break;
    }
  if (!sl) return HX_OK;  // every round slot is in flight
  if (!sv->t0_set) {
    HX_CUDA(cudaEventRecord(sv->t0, sv->s));
    sv->t0_ns = now_ns();
    sv->t0_set = true;
  }
  // Take requests from the head of the queue.
  std::vector<Pending> round;
  uint64_t keys = 0;
  while (!sv->queue.empty() && round.size() < sv->max_round_requests) {
    const Pending& p = sv->queue.front();
    if (!round.empty() && keys + p.r.n > sv->max_round_keys) break;
    keys += p.r.n;
    round.push_back(p);
    sv->queue.pop_front();
  }
  // Table maintenance and admission of inserts, in admission order. Insert
  // never reuses TOMBSTONE buckets (kernels_NVIDIA.h:383-407), so a map whose
  // fill + tombstones + incoming keys would pass the load-factor limit is
  // rehashed first: the rehash drops its tombstones and grows the table only
  // if the live keys need it. Bounds are upper bounds, so a map never fills.
  std::vector<uint64_t> add(sv->maps.size(), 0), era(sv->maps.size(), 0);
  std::vector<char> admitted(round.size(), 1);
  std::vector<int> grow_of(sv->maps.size(), -1);
  std::vector<GrowTask> tasks;
  std::vector<void*> old_tables;
  const uint64_t this_round = sv->rounds;
  for (size_t i = 0; i < round.size(); ++i) {
    const hx_request& r = round[i].r;
    if (r.op == SOP_ERASE) {
      era[r.map] += r.n;
      continue;
    }
    if (r.op != SOP_INSERT || r.n == 0) continue;
    ServeMap& m = sv->maps[r.map];
    const double lim = (double)sv->max_lf;
    const uint64_t occ = m.fill_ub + m.tomb_ub + add[r.map] + era[r.map] + r.n;
    if ((double)occ > lim * (double)(1ull << m.sp)) {
      // after a rehash: live keys (bound) + this round's erases and inserts so far + this insert
      const uint64_t after = m.fill_ub + add[r.map] + era[r.map] + r.n;
      int nsp = m.sp;
      while ((double)after > lim * (double)(1ull << nsp) && nsp < 31) ++nsp;
      const uint64_t nbytes = (1ull << nsp) * pb(sv);
      if ((double)after > lim * (double)(1ull << nsp) || sv->used - m.bytes + nbytes > sv->budget) {
        admitted[i] = 0;  // cannot make room within the budget: reject this insert
        continue;
      }
      // one batched rehash per map and round: a second need in the same round
      // replaces the pending target with the larger table
      int& slot_of = grow_of[r.map];
      void* nt = nullptr;
      HX_CUDA(cudaMallocFromPoolAsync(&nt, nbytes, sv->pool, sv->s));
      if (slot_of < 0) {
        slot_of = (int)tasks.size();
        tasks.push_back(GrowTask{m.table, nt, 1ull << m.sp, nsp, r.map});
        old_tables.push_back(m.table);
      } else {
        HX_CUDA(cudaFreeAsync(tasks[slot_of].new_table, sv->s));  // never used
        tasks[slot_of].new_table = nt;
        tasks[slot_of].new_sp = nsp;
      }
      sv->used = sv->used - m.bytes + nbytes;
      sv->st.growths++;
      sv->st.growth_bytes += nbytes;
      m.table = nt;
      m.sp = nsp;
      m.bytes = nbytes;
      m.tomb_ub = 0;
      m.rehash_round = this_round;
    }
    add[r.map] += r.n;
  }
  if (!tasks.empty()) {
    // chunk the old tables (move) and the new ones (fill) into pieces of 2048
    // buckets, 8 per thread: a move is a dependent chain of random CASes per
    // thread, so small chunks spread one table's rehash over many CTAs
    // (64K-bucket chunks made a round that grew a few tables run on a handful
    // of CTAs for hundreds of microseconds)
    constexpr uint64_t kChunk = 1 << 11;
    std::vector<GrowChunk> fillc, movec;
    for (unsigned i = 0; i < tasks.size(); ++i) {
      const uint64_t nn = 1ull << tasks[i].new_sp;
      for (uint64_t a0 = 0; a0 < nn; a0 += kChunk) fillc.push_back(GrowChunk{i, (unsigned)std::min<uint64_t>(kChunk, nn - a0), a0});
      for (uint64_t a0 = 0; a0 < tasks[i].old_n; a0 += kChunk)
        movec.push_back(GrowChunk{i, (unsigned)std::min<uint64_t>(kChunk, tasks[i].old_n - a0), a0});
    }
    if (fillc.size() + movec.size() > sl->chunk_cap) {
      cudaStreamSynchronize(sv->s);  // rare: grow the staging buffers
      cudaFreeHost(sl->h_chunks);
      cudaFree(sl->d_chunks);
      sl->chunk_cap = (fillc.size() + movec.size()) * 2;
      HX_CUDA(cudaMallocHost(reinterpret_cast<void**>(&sl->h_chunks), sl->chunk_cap * sizeof(GrowChunk)));
      HX_CUDA(cudaMalloc(reinterpret_cast<void**>(&sl->d_chunks), sl->chunk_cap * sizeof(GrowChunk)));
    }
    std::copy(tasks.begin(), tasks.end(), sl->h_tasks);
    std::copy(fillc.begin(), fillc.end(), sl->h_chunks);
    std::copy(movec.begin(), movec.end(), sl->h_chunks + fillc.size());
    cudaStream_t gs = sv->s;
    HX_CUDA(cudaMemcpyAsync(sl->d_tasks, sl->h_tasks, tasks.size() * sizeof(GrowTask), cudaMemcpyHostToDevice, gs));
    HX_CUDA(cudaMemcpyAsync(sl->d_chunks, sl->h_chunks, (fillc.size() + movec.size()) * sizeof(GrowChunk),
                            cudaMemcpyHostToDevice, gs));
    const unsigned g = (unsigned)std::min<size_t>((size_t)sm_count() * 8, std::max(fillc.size(), movec.size()));
    if (sv->kb == 4) {
      k_grow_fill<P32><<<g, 256, 0, gs>>>(sl->d_tasks, sl->d_chunks, (unsigned)fillc.size(), sv->d_info);
      k_grow_move<P32><<<g, 256, 0, gs>>>(sl->d_tasks, sl->d_chunks + fillc.size(), (unsigned)movec.size(), sv->d_info);
    } else {
      k_grow_fill<P64><<<g, 256, 0, gs>>>(sl->d_tasks, sl->d_chunks, (unsigned)fillc.size(), sv->d_info);
      k_grow_move<P64><<<g, 256, 0, gs>>>(sl->d_tasks, sl->d_chunks + fillc.size(), (unsigned)movec.size(), sv->d_info);
    }
    st = after_launch();
    if (st != HX_OK) return st;
    for (void* p : old_tables) HX_CUDA(cudaFreeAsync(p, gs));
  }
  // Stages per map, in admission order: a write (insert, erase) is a stage of
  // its own; consecutive queries share one stage. Every stage waits for the
  // map's previous stage, so reads never see later writes and writes never
  // overtake earlier reads, while queries between two writes run together.
  std::vector<int> cur_stage(sv->maps.size(), -1), cur_depth(sv->maps.size(), -1);
  std::vector<char> cur_is_query(sv->maps.size(), 0);
  std::vector<int> stage_depth, stage_wait;
  std::vector<std::pair<int, unsigned>> order;  // (stage depth, request index in round)
  unsigned nreq = 0;
  uint64_t round_keys = 0;
  sl->tags.clear();
  sl->inserts.clear();
  for (size_t i = 0; i < round.size(); ++i) {
    const hx_request& r = round[i].r;
    if (!admitted[i]) {
      sv->done.push_back(hx_completion{r.tag, now_ns(), HX_ERR_OOM, 0});
      sv->st.rejected++;
      continue;
    }
    const bool query = r.op == SOP_QUERY;
    int wait, stage;
    if (query && cur_stage[r.map] >= 0 && cur_is_query[r.map]) {
      stage = cur_stage[r.map];  // join the running group of queries
      wait = stage_wait[stage];
    } else {
      wait = cur_stage[r.map];
      stage = (int)stage_depth.size();
      stage_depth.push_back(cur_depth[r.map] + 1);
      stage_wait.push_back(wait);
      cur_stage[r.map] = stage;
      cur_depth[r.map] += 1;
      cur_is_query[r.map] = query ? 1 : 0;
    }
    SReq q;
    q.keys = r.keys;
    q.vals = r.vals;
    q.out = r.out;
    q.n = r.n;
    q.map = r.map;
    q.op = r.op;
    q.wait = wait;
    q.stage = (unsigned)stage;
    sl->h_reqs[nreq] = q;
    order.push_back({stage_depth[stage], nreq});
    sl->tags.push_back(r.tag);
    if (r.op == SOP_INSERT && r.n) sl->inserts.push_back({r.map, r.n});
    if (r.op == SOP_ERASE && r.n) sl->erases.push_back({r.map, r.n});
    round_keys += r.n;
    ++nreq;
  }
  if (nreq == 0) return HX_OK;
  std::stable_sort(order.begin(), order.end(),
                   [](const std::pair<int, unsigned>& a, const std::pair<int, unsigned>& b) { return a.first < b.first; });
  // Tile size: enough tiles to spread one round over every SM, 256..4096 keys.
  const uint64_t spread = (uint64_t)sm_count() * 8;
  uint64_t tile = 256;
  while (tile < 4096 && tile * spread < round_keys) tile *= 2;
  const unsigned nstages = (unsigned)stage_depth.size();
  for (unsigned j = 0; j < nstages; ++j) sl->h_rem[j] = 0;
  unsigned ntiles = 0;
  int max_depth = 0;
  for (auto& o : order) {
    const SReq& q = sl->h_reqs[o.second];
    max_depth = std::max(max_depth, o.first);
    unsigned nt = 0;
    for (uint64_t a0 = 0; a0 < q.n || nt == 0; a0 += tile) {
      const uint64_t c = q.n > a0 ? std::min<uint64_t>(tile, q.n - a0) : 0;
      sl->h_tiles[ntiles++] = STile{o.second, (unsigned)c, a0};
      ++nt;
      if (q.n == 0) break;
    }
    sl->h_rem[q.stage] += nt;
  }
  sv->st.rounds++;
  sv->st.requests += nreq;
  sv->st.keys += round_keys;
  sv->st.max_stage_depth = std::max<uint32_t>(sv->st.max_stage_depth, (uint32_t)max_depth);
  for (auto& x : sl->inserts) {
    sv->maps[x.first].in_flight += x.second;
    sv->maps[x.first].fill_ub += x.second;  // counted from launch until a snapshot covers it
  }
  for (auto& x : sl->erases) {
    sv->maps[x.first].in_flight_erase += x.second;
    sv->maps[x.first].tomb_ub += x.second;
  }
  for (size_t i = 0; i < sv->maps.size(); ++i) sl->h_dir[i] = SMap{sv->maps[i].table, sv->maps[i].sp, 0};
  cudaStream_t s = sv->s;
  HX_CUDA(cudaMemcpyAsync(sv->d_maps, sl->h_dir, sv->maps.size() * sizeof(SMap), cudaMemcpyHostToDevice, s));
  HX_CUDA(cudaMemcpyAsync(sl->d_reqs, sl->h_reqs, nreq * sizeof(SReq), cudaMemcpyHostToDevice, s));
  HX_CUDA(cudaMemcpyAsync(sl->d_tiles, sl->h_tiles, ntiles * sizeof(STile), cudaMemcpyHostToDevice, s));
  HX_CUDA(cudaMemsetAsync(sl->d_cnt, 0, 2 * sizeof(unsigned), s));
  HX_CUDA(cudaMemcpyAsync(sl->d_cnt + 2, sl->h_rem, nstages * sizeof(unsigned), cudaMemcpyHostToDevice, s));
  const unsigned tiles_grid = (unsigned)(sm_count() * blocks_per_sm(k_serve<P64>, 256));
  const unsigned grid = std::min<unsigned>(tiles_grid, ntiles);
  if (sv->kb == 4) {
    ServeArgs<P32> a{sv->d_maps, sv->d_info, sl->d_reqs, sl->d_tiles, ntiles, sl->d_cnt, sl->d_cnt + 1, sl->d_cnt + 2};
    k_serve<P32><<<grid, 256, 0, s>>>(a);
  } else {
    ServeArgs<P64> a{sv->d_maps, sv->d_info, sl->d_reqs, sl->d_tiles, ntiles, sl->d_cnt, sl->d_cnt + 1, sl->d_cnt + 2};
    k_serve<P64><<<grid, 256, 0, s>>>(a);
  }
  st = after_launch();
  if (st != HX_OK) return st;
  HX_CUDA(cudaMemcpyAsync(sl->h_info, sv->d_info, sv->maps.size() * sizeof(DInfo), cudaMemcpyDeviceToHost, s));
  HX_CUDA(cudaMemcpyAsync(sl->h_err, sl->d_cnt + 1, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  HX_CUDA(cudaEventRecord(sl->done, s));
  sl->busy = true;
  sl->round_no = sv->rounds++;
  sl->n_maps = sv->maps.size();
  if (launched) *launched = nreq;
  return HX_OK;
}

hx_status hx_server_poll(hx_server* sv, hx_completion* out, uint32_t capacity, uint32_t* n_out) {
  if (!sv || !n_out || (capacity && !out)) return HX_ERR_INVALID_ARG;
  hx_status st = reap(sv, false);
  if (st != HX_OK) return st;
  const uint32_t n = (uint32_t)std::min<size_t>(capacity, sv->done.size());
  for (uint32_t i = 0; i < n; ++i) out[i] = sv->done[i];
  sv->done.erase(sv->done.begin(), sv->done.begin() + n);
  *n_out = n;
  return HX_OK;
}

hx_status hx_server_drain(hx_server* sv) {
  if (!sv) return HX_ERR_INVALID_ARG;
  for (;;) {
    uint32_t launched = 0;
    hx_status st = hx_server_step(sv, &launched);
    if (st != HX_OK) return st;
    bool busy = false;
    for (auto& sl : sv->slots) busy |= sl.busy;
    if (sv->queue.empty() && !busy) return HX_OK;
    if (!launched) {
      st = reap(sv, true);
      if (st != HX_OK) return st;
    }
  }
}

hx_status hx_server_map_info(hx_server* sv, uint32_t map, hx_info* out) {
  if (!sv || !out || map >= sv->maps.size()) return HX_ERR_INVALID_ARG;
  hx_map v;
  view_of(sv, map, &v);
  return hx_get_info(&v, out, sv->s);
}

hx_status hx_server_bucket_data(hx_server* sv, uint32_t map, void** d_buckets, uint64_t* bucket_count) {
  if (!sv || map >= sv->maps.size()) return HX_ERR_INVALID_ARG;
  if (d_buckets) *d_buckets = sv->maps[map].table;
  if (bucket_count) *bucket_count = 1ull << sv->maps[map].sp;
  return HX_OK;
}

hx_status hx_server_get_stats(hx_server* sv, hx_server_stats* out) {
  if (!sv || !out) return HX_ERR_INVALID_ARG;
  *out = sv->st;
  return HX_OK;
}

hx_status hx_server_memory(hx_server* sv, uint64_t* used, uint64_t* budget) {
  if (!sv) return HX_ERR_INVALID_ARG;
  if (used) *used = sv->used;
  if (budget) *budget = sv->budget;
  return HX_OK;
}

hx_status hx_server_run_trace(hx_server* sv, const hx_request* reqs, const uint64_t* arrival_ns, uint32_t count,
                              uint64_t* complete_ns, int32_t* status, uint64_t* t_start_ns) {
  HX_RANGE("hx_server_run_trace");
  if (!sv || (count && (!reqs || !arrival_ns || !complete_ns || !status))) return HX_ERR_INVALID_ARG;
  for (uint32_t i = 0; i < count; ++i) {
    complete_ns[i] = 0;
    status[i] = -1;
  }
  // tags are trace indices
  std::vector<hx_request> rq(reqs, reqs + count);
  for (uint32_t i = 0; i < count; ++i) rq[i].tag = i;
  HX_CUDA(cudaStreamSynchronize(sv->s));
  HX_CUDA(cudaEventRecord(sv->t0, sv->s));
  sv->t0_ns = now_ns();
  sv->t0_set = true;
  const uint64_t start = sv->t0_ns;
  if (t_start_ns) *t_start_ns = start;
  uint32_t next = 0, completed = 0;
  std::vector<hx_completion> buf(4096);
  while (completed < count) {
    const uint64_t now = now_ns() - start;
    uint32_t first = next;
    while (next < count && arrival_ns[next] <= now) ++next;
    if (next > first) {
      hx_status st = hx_server_submit(sv, rq.data() + first, next - first);
      if (st != HX_OK) return st;
    }
    uint32_t launched = 0;
    hx_status st = hx_server_step(sv, &launched);
    if (st != HX_OK) return st;
    uint32_t n = 0;
    do {
      st = hx_server_poll(sv, buf.data(), (uint32_t)buf.size(), &n);
      if (st != HX_OK) return st;
      for (uint32_t i = 0; i < n; ++i) {
        const uint64_t tag = buf[i].tag;
        if (tag < count) {
          complete_ns[tag] = buf[i].complete_ns - start;
          status[tag] = buf[i].status;
          ++completed;
        }
      }
    } while (n == buf.size());
  }
  return HX_OK;
}

}  // extern "C"
