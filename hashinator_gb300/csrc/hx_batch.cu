// hx_batch.cu — thousands of independent maps served by one persistent launch.
//
// A batch is a directory of maps (size power, bucket offset, metadata) over one
// device arena of buckets — the per-cell velocity-block maps of a Vlasov mesh.
// A plan turns one round of work (insert, query, erase, clean_tombstones per
// map, each a contiguous segment of flat device arrays) into tiles, ordered
// phase by phase. The fused kernel is persistent: each CTA takes the next tile
// from an atomic ticket, waits until the earlier phases of that tile's map are
// done, runs it, and counts it off. Tiles are claimed strictly in order, so a
// tile only ever waits on tiles that running CTAs already hold: no grid-wide
// barrier and no co-residency assumption is needed. Every wait is bounded; a
// wait that runs out sets the plan's error word and the tile is skipped.
//
// Per map the semantics are the plain path's (hx_insert, hx_retrieve,
// hx_erase, hx_clean_tombstones): same probe order, same decisions, same
// counters, so results are identical to per-map launches.
#include <algorithm>
#include <cstring>
#include <vector>

#include "hx_autotune.h"
#include "hx_host.h"
#include "hx_internal.h"
#include "hx_probe.cuh"

namespace hx {

enum BatchPhase : unsigned {
  BP_INSERT = 0,
  BP_QUERY = 1,
  BP_ERASE = 2,
  BP_CLEAN_PRO = 3,
  BP_CLEAN_EXTRACT = 4,
  BP_CLEAN_REINSERT = 5,
  BP_NPHASES = 6
};

struct Tile {
  unsigned map;    // 0xffffffff: no more work
  unsigned phase;
  unsigned long long begin;  // first key (insert/query/erase), bucket (extract) or moved entry (reinsert)
  unsigned count;
  unsigned pad;
};

template <class P>
struct BatchArgs {
  using K = typename PairTraits<P>::K;
  using V = typename PairTraits<P>::V;
  P* arena;
  const unsigned long long* off;  // first bucket of each map
  const int* sp;
  DInfo* info;
  const Tile* tiles;
  unsigned n_tiles;
  unsigned n_maps;
  unsigned* work;       // ticket counter
  unsigned* remaining;  // [BP_NPHASES][n_maps] tiles left per phase and map
  unsigned* error;      // nonzero: a bounded wait ran out, or a moved list overflowed
  const K* ins_keys;
  const V* ins_vals;
  const K* q_keys;
  V* q_out;
  const K* e_keys;
  P* moved;                             // clean_tombstones: moved pairs, per-map regions
  const unsigned long long* moved_off;  // region start per map
  const unsigned long long* moved_cap;  // region size per map
};

constexpr unsigned long long kBatchWaitNs = 1000000000ull;  // one second of global time
constexpr unsigned kBatchSpinLimit = 1u << 26;                // backstop on the number of polls

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Waits until *p == 0, for about one second at most.
__device__ __forceinline__ bool wait_zero(const unsigned* p) {
  if (ld_acquire_u32(p) == 0) return true;
  const unsigned long long t0 = global_ns();
  for (unsigned i = 0; i < kBatchSpinLimit; ++i) {
    __nanosleep(i < 32 ? 32 : 256);
    if (ld_acquire_u32(p) == 0) return true;
    if ((i & 63) == 63 && global_ns() - t0 > kBatchWaitNs) return false;
  }
  return false;
}

template <class P, int G, int BLOCK>
// The round is bound by memory-level parallelism (random probes of many small
// tables), not by DRAM bytes: capping registers so that 48 warps fit per SM
// (some spills to L1) took it from about 4.5 to 3.2 ms against 20 warps at 96
// registers (sweep of 20/24/32/40/48/64 warps on GB300).
#ifndef HX_BATCH_MIN_WARPS
#define HX_BATCH_MIN_WARPS 48
#endif
// Inserts per thread whose first CAS is in flight at once. One key at a time
// measured fastest on GB300 (2.99 ms a round): 2 in flight at 48 warps per SM
// took 3.13 ms, 2 or 4 at 32 warps 3.34 / 3.41 ms.
#ifndef HX_BATCH_INSERTS_IN_FLIGHT
#define HX_BATCH_INSERTS_IN_FLIGHT 1
#endif
__global__ void __launch_bounds__(BLOCK, HX_BATCH_MIN_WARPS * 32 / BLOCK > 0 ? HX_BATCH_MIN_WARPS * 32 / BLOCK : 1)
    k_batch(BatchArgs<P> a) {
  using K = typename PairTraits<P>::K;
  using V = typename PairTraits<P>::V;
  constexpr K EMPTY = PairTraits<P>::EMPTY;
  constexpr K TOMB = PairTraits<P>::TOMB;
  constexpr int BT = sizeof(P) == 8 ? 4 : 2;  // thread-per-key window: 32 B
  constexpr int BG = sizeof(P) == 8 ? 2 : 1;  // group lane: 16 B
  constexpr int U = 4;                        // lookups in flight per thread
  constexpr int UI = HX_BATCH_INSERTS_IN_FLIGHT;  // inserts in flight per thread
  __shared__ Tile s_t;
  __shared__ unsigned s_ok, s_ins, s_max, s_fail, s_erased, s_moved;
  const int lane = threadIdx.x & 31;
  for (;;) {
    if (threadIdx.x == 0) {
      const unsigned idx = atomicAdd(a.work, 1u);
      Tile t;
      if (idx < a.n_tiles) t = a.tiles[idx];
      else t.map = 0xffffffffu;
      s_t = t;
      s_ins = s_max = s_fail = s_erased = s_moved = 0;
      unsigned ok = 1;
      if (t.map != 0xffffffffu) {
        for (int q = (int)t.phase - 1; q >= 0 && ok; --q) ok = wait_zero(a.remaining + q * a.n_maps + t.map);
        if (!ok) atomicExch(a.error, 1u);
      }
      s_ok = ok;
    }
    __syncthreads();
    const Tile t = s_t;
    if (t.map == 0xffffffffu) break;
    __threadfence();
    if (s_ok) {
      const unsigned map = t.map;
      const int sp = a.sp[map];
      P* tab = a.arena + a.off[map];
      DInfo* inf = a.info + map;
      unsigned ins = 0, maxd = 0, erased = 0, moved = 0;
      bool fail = false;
      // a group window larger than this table: the thread-per-key path
      const bool groups = G > 1 && (1ull << sp) >= (unsigned long long)(G * BG);
      switch (t.phase) {
        case BP_INSERT:
        case BP_CLEAN_REINSERT: {
          unsigned long long begin = t.begin, count = t.count;
          const P* src = nullptr;
          if (t.phase == BP_CLEAN_REINSERT) {
            const unsigned long long cap = a.moved_cap[map];
            unsigned long long nm = inf->moved;
            nm = nm < cap ? nm : cap;
            count = begin < nm ? (nm - begin < count ? nm - begin : count) : 0;
            src = a.moved + a.moved_off[map];
          }
          // inserts are thread-per-key whatever the tuned group width: on
          // GB300 they measured fastest at every load factor
          auto load = [&](unsigned k, K& key, V& val) {
            if (src) {
              const P pr = src[begin + k];
              key = pr.first;
              val = pr.second;
            } else {
              key = a.ins_keys[begin + k];
              val = a.ins_vals[begin + k];
            }
          };
          const unsigned cnt = (unsigned)count;
          if (src) {  // moved keys, whose homes are mostly taken: window first, as the single-map clean
            for (unsigned k = threadIdx.x; k < cnt; k += BLOCK) {
              K key;
              V val;
              load(k, key, val);
              insert_one_t1_win<P, BT>(tab, sp, key, val, ins, maxd, fail);
            }
          } else {
            for (unsigned base = 0; base < cnt; base += BLOCK * UI)
              insert_t1_many<P, BT, UI>(tab, sp, base + threadIdx.x, BLOCK, cnt, load, ins, maxd, fail);
          }
          break;
        }
        case BP_QUERY:
        case BP_ERASE: {
          const bool erase = t.phase == BP_ERASE;
          const K* keys = erase ? a.e_keys : a.q_keys;
          const unsigned limit = inf->max_probe;
          if (limit == 0) break;
          // the tuned group width applies to queries; erases are thread-per-key
          if (!groups || erase) {
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
                  act[u] = key[u] != EMPTY && key[u] != TOMB;
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
                    if (cas_key(tab + slot, key[u], TOMB)) ++erased;
                  } else {
                    a.q_out[t.begin + base + u * BLOCK + threadIdx.x] = v;
                  }
                }
              }
            }
          } else if constexpr (G > 1) {
            const unsigned gmask = group_mask<G>(lane);
            for (unsigned k = threadIdx.x / G; k < t.count; k += BLOCK / G) {
              const K key = keys[t.begin + k];
              if (key == EMPTY || key == TOMB) continue;
              V v;
              const int w = probe_find_live<P, G, BG>(tab, sp, key, true, limit, lane, gmask, v);
              if (w >= 0 && (lane & (G - 1)) == w) a.q_out[t.begin + k] = v;
            }
          }
          break;
        }
        case BP_CLEAN_PRO:
          // clean_tombstones prologue (hashinator.h:1264-1269, :1301)
          if (threadIdx.x == 0) {
            const bool skip = inf->tombstones == 0;
            inf->skip = skip ? 1u : 0u;
            inf->moved = 0;
            if (!skip) {
              inf->tombstones = 0;
              inf->max_probe = inf->fill ? 1u : 0u;
            }
          }
          break;
        case BP_CLEAN_EXTRACT: {
          if (inf->skip) break;
          const unsigned long long cap = a.moved_cap[map];
          P* dst = a.moved + a.moved_off[map];
          // whole warps iterate together so the append can be warp-aggregated
          for (unsigned base = 0; base < t.count; base += BLOCK) {
            const unsigned k = base + threadIdx.x;
            bool take = false, tomb = false;
            P pr;
            if (k < t.count) {
              pr = tab[t.begin + k];
              tomb = pr.first == TOMB;
              // not in its home bucket: decided from the bucket's index, which gives the
              // reference's answer (bucket[home] != key) because a key occurs once
              take = pr.first != EMPTY && !tomb && home_slot(pr.first, sp) != (uint32_t)(t.begin + k);
            }
            const unsigned bal = __ballot_sync(0xffffffffu, take);
            unsigned long long slot0 = 0;
            if (bal && lane == __ffs(bal) - 1) slot0 = atomicAdd(&inf->moved, (unsigned long long)__popc(bal));
            slot0 = __shfl_sync(0xffffffffu, slot0, bal ? __ffs(bal) - 1 : 0);
            if (take) {
              const unsigned long long slot = slot0 + __popc(bal & ((1u << lane) - 1u));
              if (slot < cap) {
                dst[slot] = pr;
                ++moved;
              } else {
                atomicExch(a.error, 2u);
                take = false;  // keep the key where it is
              }
            }
            if (take || tomb) {
              P e;
              e.first = EMPTY;
              e.second = 0;
              tab[t.begin + k] = e;
            }
          }
          break;
        }
        default:
          break;
      }
      // per-tile counters: warp reduce, then shared, then one global atomic each
      ins = __reduce_add_sync(0xffffffffu, ins);
      maxd = __reduce_max_sync(0xffffffffu, maxd);
      erased = __reduce_add_sync(0xffffffffu, erased);
      moved = __reduce_add_sync(0xffffffffu, moved);
      const bool anyfail = __any_sync(0xffffffffu, fail);
      if (lane == 0) {
        if (ins) atomicAdd(&s_ins, ins);
        if (maxd) atomicMax(&s_max, maxd);
        if (erased) atomicAdd(&s_erased, erased);
        if (moved) atomicAdd(&s_moved, moved);
        if (anyfail) atomicExch(&s_fail, 1u);
      }
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
      DInfo* inf = a.info + t.map;
      if (s_ins) atomicAdd(&inf->fill, (unsigned long long)s_ins);
      if (s_max) atomicMax(&inf->max_probe, s_max);
      if (s_fail) atomicExch(&inf->err, HX_STATUS_FAIL);
      if (s_erased) {
        atomicAdd(&inf->tombstones, (unsigned long long)s_erased);
        atomicAdd(&inf->fill, 0ull - (unsigned long long)s_erased);
      }
      if (s_moved) atomicAdd(&inf->fill, 0ull - (unsigned long long)s_moved);
      __threadfence();
      atomicSub(a.remaining + t.phase * a.n_maps + t.map, 1u);
    }
  }
}

template <class P>
__global__ void k_batch_fill_empty(P* arena, uint64_t n) {
  P e;
  e.first = PairTraits<P>::EMPTY;
  e.second = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    arena[i] = e;
}

__global__ void k_batch_info_reset(DInfo* info, unsigned n) {
  const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    info[i].fill = 0;
    info[i].tombstones = 0;
    info[i].max_probe = 0;
    info[i].err = HX_STATUS_SUCCESS;
    info[i].moved = 0;
    info[i].skip = 0;
  }
}

}  // namespace hx

struct hx_batch {
  int key_bytes = 4, val_bytes = 4;
  unsigned n_maps = 0;
  std::vector<int> sp;
  std::vector<unsigned long long> off;
  std::vector<uint64_t> fill_ub;
  uint64_t total_buckets = 0;
  void* arena = nullptr;
  unsigned long long* d_off = nullptr;
  int* d_sp = nullptr;
  hx::DInfo* d_info = nullptr;
  void* scratch = nullptr;  // per-map plain clean_tombstones scratch (shared)
  uint64_t scratch_bytes = 0;
};

struct hx_batch_plan {
  hx_batch* b = nullptr;
  hx_batch_work w{};
  std::vector<uint64_t> ins_off, q_off, e_off;
  int group = 1, block = 256, tile = 2048;
  unsigned n_tiles = 0;
  hx::Tile* d_tiles = nullptr;
  unsigned* d_counters = nullptr;  // [0]: ticket, [1]: error, [2..]: remaining
  unsigned* d_remaining_init = nullptr;
  void* moved = nullptr;
  unsigned long long* d_moved_off = nullptr;
  unsigned long long* d_moved_cap = nullptr;
  std::vector<unsigned long long> moved_cap;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  std::vector<unsigned> rem_host;  // initial tiles per (phase, map)
};

namespace hx {

static uint64_t pbytes(const hx_batch* b) { return b->key_bytes == 4 ? 8 : 16; }

static void free_plan_device(hx_batch_plan* p) {
  if (p->graph_exec) cudaGraphExecDestroy(p->graph_exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  p->graph_exec = nullptr;
  p->graph = nullptr;
  cudaFree(p->d_tiles);
  cudaFree(p->d_counters);
  cudaFree(p->d_remaining_init);
  p->d_tiles = nullptr;
  p->d_counters = nullptr;
  p->d_remaining_init = nullptr;
}

// Builds the tile list and the per-map phase counters on the host, uploads
// them. Phase-major order; inside a phase, larger maps first.
static hx_status build_tiles(hx_batch_plan* p, cudaStream_t s) {
  hx_batch* b = p->b;
  const unsigned nm = b->n_maps;
  free_plan_device(p);
  std::vector<Tile> tiles;
  std::vector<unsigned> rem((size_t)BP_NPHASES * nm, 0);
  std::vector<unsigned> order(nm);
  for (unsigned i = 0; i < nm; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](unsigned x, unsigned y) { return b->sp[x] > b->sp[y]; });
  const uint64_t T = (uint64_t)p->tile;
  // Maps in groups of consecutive maps (largest first) whose tables total
  // about kGroupBytes (24 MiB), and each group's phases software-pipelined across the
  // tile list: group g's inserts, then g-1's queries, g-2's erases, g-3's
  // clean prologue and extraction, g-4's re-inserts. A map's later phases run
  // while its table is still in L2 from the earlier ones, and they rarely wait,
  // because the tiles they depend on were claimed a group earlier. Every map's
  // phases still appear in phase order, so a tile only waits on earlier tiles.
#ifndef HX_BATCH_GROUP_MB
#define HX_BATCH_GROUP_MB 24
#endif
  constexpr uint64_t kGroupBytes = (uint64_t)HX_BATCH_GROUP_MB << 20;
  const uint64_t pair_bytes = (uint64_t)b->key_bytes * 2;
  std::vector<std::vector<unsigned>> groups;
  uint64_t acc = 0;
  for (unsigned i : order) {
    const uint64_t bytes = (1ull << b->sp[i]) * pair_bytes;
    if (!groups.empty() && acc + bytes <= kGroupBytes) {
      groups.back().push_back(i);
      acc += bytes;
    } else {
      groups.push_back({i});
      acc = bytes;
    }
  }
  auto add_segments = [&](unsigned phase, const std::vector<uint64_t>& offs, const std::vector<unsigned>& maps) {
    if (offs.empty()) return;
    for (unsigned i : maps) {
      for (uint64_t a0 = offs[i]; a0 < offs[i + 1]; a0 += T) {
        const uint64_t c = std::min<uint64_t>(T, offs[i + 1] - a0);
        tiles.push_back(Tile{i, phase, a0, (unsigned)c, 0});
        rem[(size_t)phase * nm + i]++;
      }
    }
  };
  const long ng = (long)groups.size();
  for (long step = 0; step < ng + 4; ++step) {
    if (step < ng) add_segments(BP_INSERT, p->ins_off, groups[step]);
    if (step - 1 >= 0 && step - 1 < ng) add_segments(BP_QUERY, p->q_off, groups[step - 1]);
    if (step - 2 >= 0 && step - 2 < ng) add_segments(BP_ERASE, p->e_off, groups[step - 2]);
    if (!p->w.clean) continue;
    if (step - 3 >= 0 && step - 3 < ng) {
      const auto& g = groups[step - 3];
      for (unsigned i : g) {
        tiles.push_back(Tile{i, BP_CLEAN_PRO, 0, 0, 0});
        rem[(size_t)BP_CLEAN_PRO * nm + i]++;
      }
      const uint64_t TB = 4 * T;  // buckets per extraction tile
      for (unsigned i : g) {
        const uint64_t nb = 1ull << b->sp[i];
        for (uint64_t a0 = 0; a0 < nb; a0 += TB) {
          tiles.push_back(Tile{i, BP_CLEAN_EXTRACT, a0, (unsigned)std::min<uint64_t>(TB, nb - a0), 0});
          rem[(size_t)BP_CLEAN_EXTRACT * nm + i]++;
        }
      }
    }
    if (step - 4 >= 0 && step - 4 < ng) {
      for (unsigned i : groups[step - 4]) {
        for (uint64_t a0 = 0; a0 < p->moved_cap[i]; a0 += T) {
          tiles.push_back(Tile{i, BP_CLEAN_REINSERT, a0, (unsigned)T, 0});
          rem[(size_t)BP_CLEAN_REINSERT * nm + i]++;
        }
      }
    }
  }
  if (tiles.size() > 0xFFFFFFF0ull) return HX_ERR_INVALID_ARG;
  p->n_tiles = (unsigned)tiles.size();
  const size_t cnt_words = 2 + rem.size();
  HX_CUDA(cudaMalloc(&p->d_tiles, std::max<size_t>(1, tiles.size()) * sizeof(Tile)));
  HX_CUDA(cudaMalloc(&p->d_counters, cnt_words * sizeof(unsigned)));
  HX_CUDA(cudaMalloc(&p->d_remaining_init, rem.size() * sizeof(unsigned)));
  if (!tiles.empty())
    HX_CUDA(cudaMemcpyAsync(p->d_tiles, tiles.data(), tiles.size() * sizeof(Tile), cudaMemcpyHostToDevice, s));
  HX_CUDA(cudaMemcpyAsync(p->d_remaining_init, rem.data(), rem.size() * sizeof(unsigned), cudaMemcpyHostToDevice, s));
  HX_CUDA(cudaStreamSynchronize(s));
  p->rem_host = rem;
  return HX_OK;
}

template <class P, int G>
static hx_status launch_batch_g(hx_batch_plan* p, cudaStream_t s) {
  hx_batch* b = p->b;
  using K = typename PairTraits<P>::K;
  using V = typename PairTraits<P>::V;
  BatchArgs<P> a;
  a.arena = static_cast<P*>(b->arena);
  a.off = b->d_off;
  a.sp = b->d_sp;
  a.info = b->d_info;
  a.tiles = p->d_tiles;
  a.n_tiles = p->n_tiles;
  a.n_maps = b->n_maps;
  a.work = p->d_counters;
  a.error = p->d_counters + 1;
  a.remaining = p->d_counters + 2;
  a.ins_keys = static_cast<const K*>(p->w.ins_keys);
  a.ins_vals = static_cast<const V*>(p->w.ins_vals);
  a.q_keys = static_cast<const K*>(p->w.query_keys);
  a.q_out = static_cast<V*>(p->w.query_out);
  a.e_keys = static_cast<const K*>(p->w.erase_keys);
  a.moved = static_cast<P*>(p->moved);
  a.moved_off = p->d_moved_off;
  a.moved_cap = p->d_moved_cap;
  const size_t rem_bytes = (size_t)BP_NPHASES * b->n_maps * sizeof(unsigned);
  HX_CUDA(cudaMemsetAsync(p->d_counters, 0, 2 * sizeof(unsigned), s));
  HX_CUDA(cudaMemcpyAsync(p->d_counters + 2, p->d_remaining_init, rem_bytes, cudaMemcpyDeviceToDevice, s));
#define HX_BATCH_LAUNCH(BL)                                                              \
  {                                                                                      \
    auto kern = k_batch<P, G, BL>;                                                       \
    const unsigned grid = (unsigned)(sm_count() * blocks_per_sm(kern, BL));              \
    kern<<<grid, BL, 0, s>>>(a);                                                         \
  }
  if (p->block == 128) HX_BATCH_LAUNCH(128)
  else if (p->block == 512) HX_BATCH_LAUNCH(512)
  else HX_BATCH_LAUNCH(256)
#undef HX_BATCH_LAUNCH
  return after_launch();
}

template <class P>
static hx_status launch_batch(hx_batch_plan* p, cudaStream_t s) {
  switch (p->group) {
    case 4: return launch_batch_g<P, 4>(p, s);
    case 8: return launch_batch_g<P, 8>(p, s);
    case 16: return launch_batch_g<P, 16>(p, s);
    case 32: return launch_batch_g<P, 32>(p, s);
    default: return launch_batch_g<P, 1>(p, s);
  }
}

// A map handle that views map i of a batch, for the plain per-map path.
static void make_view(hx_batch* b, unsigned i, hx_map* v) {
  v->key_bytes = b->key_bytes;
  v->val_bytes = b->val_bytes;
  v->sp = b->sp[i];
  v->buckets = static_cast<char*>(b->arena) + b->off[i] * pbytes(b);
  v->info = b->d_info + i;
  v->fill_ub = b->fill_ub[i];
  v->scratch = b->scratch;
  v->scratch_bytes = b->scratch_bytes;
}

}  // namespace hx

using namespace hx;

extern "C" {

hx_status hx_batch_create(hx_batch** out, uint32_t n_maps, const int32_t* size_powers, int key_bytes, int val_bytes,
                          hx_stream stream) {
  if (!out || !size_powers || n_maps == 0) return HX_ERR_INVALID_ARG;
  *out = nullptr;
  if (!((key_bytes == 4 && val_bytes == 4) || (key_bytes == 8 && val_bytes == 8))) return HX_ERR_INVALID_ARG;
  hx_batch* b = new hx_batch();
  b->key_bytes = key_bytes;
  b->val_bytes = val_bytes;
  b->n_maps = n_maps;
  b->sp.resize(n_maps);
  b->off.resize(n_maps);
  b->fill_ub.assign(n_maps, 0);
  uint64_t acc = 0;
  for (uint32_t i = 0; i < n_maps; ++i) {
    const int sp = size_powers[i];
    if (sp < 2 || sp > 31) {
      delete b;
      return HX_ERR_INVALID_ARG;
    }
    b->sp[i] = sp;
    b->off[i] = acc;  // every table is a power of two >= 4 buckets: 32-byte aligned
    acc += 1ull << sp;
  }
  b->total_buckets = acc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  auto fail = [&](cudaError_t e) {
    cudaFree(b->arena);
    cudaFree(b->d_off);
    cudaFree(b->d_sp);
    cudaFree(b->d_info);
    delete b;
    return cuda_status(e);
  };
  cudaError_t e;
  if ((e = cudaMalloc(&b->arena, acc * pbytes(b))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(reinterpret_cast<void**>(&b->d_off), n_maps * sizeof(unsigned long long))) != cudaSuccess)
    return fail(e);
  if ((e = cudaMalloc(reinterpret_cast<void**>(&b->d_sp), n_maps * sizeof(int))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(reinterpret_cast<void**>(&b->d_info), n_maps * sizeof(DInfo))) != cudaSuccess) return fail(e);
  if ((e = cudaMemcpyAsync(b->d_off, b->off.data(), n_maps * sizeof(unsigned long long), cudaMemcpyHostToDevice,
                           s)) != cudaSuccess)
    return fail(e);
  if ((e = cudaMemcpyAsync(b->d_sp, b->sp.data(), n_maps * sizeof(int), cudaMemcpyHostToDevice, s)) != cudaSuccess)
    return fail(e);
  *out = b;
  hx_status st = hx_batch_clear(b, stream);
  if (st == HX_OK && (e = cudaStreamSynchronize(s)) != cudaSuccess) st = cuda_status(e);
  if (st != HX_OK) {
    hx_batch_destroy(b);
    *out = nullptr;
  }
  return st;
}

hx_status hx_batch_destroy(hx_batch* b) {
  if (!b) return HX_ERR_INVALID_ARG;
  cudaError_t e = cudaDeviceSynchronize();
  cudaFree(b->arena);
  cudaFree(b->d_off);
  cudaFree(b->d_sp);
  cudaFree(b->d_info);
  cudaFree(b->scratch);
  delete b;
  return e == cudaSuccess ? HX_OK : cuda_status(e);
}

hx_status hx_batch_clear(hx_batch* b, hx_stream stream) {
  if (!b) return HX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const unsigned grid = (unsigned)(sm_count() * 8);
  if (b->key_bytes == 4) k_batch_fill_empty<P32><<<grid, 256, 0, s>>>(static_cast<P32*>(b->arena), b->total_buckets);
  else k_batch_fill_empty<P64><<<grid, 256, 0, s>>>(static_cast<P64*>(b->arena), b->total_buckets);
  hx_status st = after_launch();
  if (st != HX_OK) return st;
  k_batch_info_reset<<<(b->n_maps + 255) / 256, 256, 0, s>>>(b->d_info, b->n_maps);
  std::fill(b->fill_ub.begin(), b->fill_ub.end(), 0);
  return after_launch();
}

hx_status hx_batch_map_info(hx_batch* b, uint32_t map, hx_info* out, hx_stream stream) {
  if (!b || !out || map >= b->n_maps) return HX_ERR_INVALID_ARG;
  hx_map v;
  make_view(b, map, &v);
  hx_status st = hx_get_info(&v, out, stream);
  b->fill_ub[map] = v.fill_ub;
  return st;
}

hx_status hx_batch_bucket_data(hx_batch* b, uint32_t map, void** d_buckets, uint64_t* bucket_count) {
  if (!b || map >= b->n_maps) return HX_ERR_INVALID_ARG;
  if (d_buckets) *d_buckets = static_cast<char*>(b->arena) + b->off[map] * pbytes(b);
  if (bucket_count) *bucket_count = 1ull << b->sp[map];
  return HX_OK;
}

hx_status hx_batch_plan_create(hx_batch* b, const hx_batch_work* w, hx_batch_plan** out, hx_stream stream) {
  HX_RANGE("hx_batch_plan_create");
  if (!b || !w || !out) return HX_ERR_INVALID_ARG;
  *out = nullptr;
  const unsigned kb = (unsigned)b->key_bytes;
  if (misaligned(w->ins_keys, kb) || misaligned(w->ins_vals, kb) || misaligned(w->query_keys, kb) ||
      misaligned(w->query_out, kb) || misaligned(w->erase_keys, kb))
    return HX_ERR_INVALID_ARG;
  const unsigned nm = b->n_maps;
  hx_batch_plan* p = new hx_batch_plan();
  p->b = b;
  p->w = *w;
  auto copy_offs = [&](const uint64_t* src, const void* keys, std::vector<uint64_t>& dst) -> bool {
    if (!src) return keys == nullptr;
    dst.assign(src, src + nm + 1);
    for (unsigned i = 0; i < nm; ++i)
      if (dst[i + 1] < dst[i]) return false;
    return dst[nm] == dst[0] || keys != nullptr;
  };
  if (!copy_offs(w->ins_offsets, w->ins_keys, p->ins_off) || !copy_offs(w->query_offsets, w->query_keys, p->q_off) ||
      !copy_offs(w->erase_offsets, w->erase_keys, p->e_off) ||
      (w->ins_offsets && !w->ins_vals && p->ins_off[nm] != p->ins_off[0]) ||
      (w->query_offsets && !w->query_out && p->q_off[nm] != p->q_off[0])) {
    delete p;
    return HX_ERR_INVALID_ARG;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // Moved-list regions for clean_tombstones: at most fill <= min(table, fill
  // bound + this plan's inserts) pairs per map.
  p->moved_cap.assign(nm, 0);
  if (w->clean) {
    std::vector<unsigned long long> moff(nm);
    unsigned long long acc = 0;
    for (unsigned i = 0; i < nm; ++i) {
      const uint64_t ins = p->ins_off.empty() ? 0 : p->ins_off[i + 1] - p->ins_off[i];
      const uint64_t cap = std::min<uint64_t>(1ull << b->sp[i], b->fill_ub[i] + ins);
      p->moved_cap[i] = cap;
      moff[i] = acc;
      acc += cap;
    }
    cudaError_t e = cudaMalloc(&p->moved, std::max<unsigned long long>(1, acc) * pbytes(b));
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&p->d_moved_off), nm * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&p->d_moved_cap), nm * sizeof(unsigned long long));
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(p->d_moved_off, moff.data(), nm * sizeof(unsigned long long), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(p->d_moved_cap, p->moved_cap.data(), nm * sizeof(unsigned long long),
                          cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) {
      hx_batch_plan_destroy(p);
      return cuda_status(e);
    }
  }
  hx_status st = build_tiles(p, s);
  if (st != HX_OK) {
    hx_batch_plan_destroy(p);
    return st;
  }
  *out = p;
  return HX_OK;
}

hx_status hx_batch_plan_destroy(hx_batch_plan* p) {
  if (!p) return HX_ERR_INVALID_ARG;
  cudaDeviceSynchronize();
  free_plan_device(p);
  cudaFree(p->moved);
  cudaFree(p->d_moved_off);
  cudaFree(p->d_moved_cap);
  delete p;
  return HX_OK;
}

hx_status hx_batch_set_tuning(hx_batch_plan* p, int group_width, int block_size, int tile_keys, hx_stream stream) {
  if (!p) return HX_ERR_INVALID_ARG;
  if (group_width && group_width != 1 && group_width != 4 && group_width != 8 && group_width != 16 &&
      group_width != 32)
    return HX_ERR_INVALID_ARG;
  if (block_size && block_size != 128 && block_size != 256 && block_size != 512) return HX_ERR_INVALID_ARG;
  if (tile_keys && (tile_keys < 64 || tile_keys > (1 << 20))) return HX_ERR_INVALID_ARG;
  if (group_width) p->group = group_width;
  if (block_size) p->block = block_size;
  if (tile_keys && tile_keys != p->tile) {
    p->tile = tile_keys;
    return build_tiles(p, static_cast<cudaStream_t>(stream));
  }
  if (p->graph_exec) {  // the captured launch has the old tuning baked in
    cudaGraphExecDestroy(p->graph_exec);
    cudaGraphDestroy(p->graph);
    p->graph_exec = nullptr;
    p->graph = nullptr;
  }
  return HX_OK;
}

static void account_inserts(hx_batch_plan* p) {
  if (p->ins_off.empty()) return;
  for (unsigned i = 0; i < p->b->n_maps; ++i) {
    p->b->fill_ub[i] += p->ins_off[i + 1] - p->ins_off[i];
    const uint64_t nb = 1ull << p->b->sp[i];
    if (p->b->fill_ub[i] > nb) p->b->fill_ub[i] = nb;
  }
}

hx_status hx_batch_run(hx_batch_plan* p, hx_stream stream) {
  HX_RANGE("hx_batch_run");
  if (!p) return HX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  account_inserts(p);
  return p->b->key_bytes == 4 ? launch_batch<P32>(p, s) : launch_batch<P64>(p, s);
}

hx_status hx_batch_run_graph(hx_batch_plan* p, hx_stream stream) {
  HX_RANGE("hx_batch_run_graph");
  if (!p) return HX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!p->graph_exec) {
    // capture the counter reset + the fused launch on a private stream
    cudaStream_t cs;
    HX_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    hx_status st = HX_OK;
    if (e == cudaSuccess) st = p->b->key_bytes == 4 ? launch_batch<P32>(p, cs) : launch_batch<P64>(p, cs);
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(cs, &g);
    cudaStreamDestroy(cs);
    if (e != cudaSuccess) return cuda_status(e);
    if (st != HX_OK) return st;
    if (e2 != cudaSuccess) return cuda_status(e2);
    p->graph = g;
    HX_CUDA(cudaGraphInstantiate(&p->graph_exec, g, 0));
  }
  account_inserts(p);
  HX_CUDA(cudaGraphLaunch(p->graph_exec, s));
  return HX_OK;
}

hx_status hx_batch_autotune(hx_batch_plan* p, const int32_t* group_widths, uint32_t n_groups,
                            const int32_t* block_sizes, uint32_t n_blocks, const int32_t* tile_keys, uint32_t n_tiles,
                            int reps, hx_batch_reset_fn reset, void* reset_user, hx_stream stream,
                            hx_batch_trial* trials, uint32_t trials_capacity, hx_batch_trial* best) {
  HX_RANGE("hx_batch_autotune");
  if (!p || !best || reps < 1) return HX_ERR_INVALID_ARG;
  static const int32_t kGroups[] = {1, 4, 8, 16, 32}, kBlocks[] = {128, 256, 512}, kTiles[] = {512, 2048, 8192};
  if (!group_widths) {
    group_widths = kGroups;
    n_groups = 5;
  }
  if (!block_sizes) {
    block_sizes = kBlocks;
    n_blocks = 3;
  }
  if (!tile_keys) {
    tile_keys = kTiles;
    n_tiles = 3;
  }
  if (!n_groups || !n_blocks || !n_tiles) return HX_ERR_INVALID_ARG;
  std::vector<TunePoint> grid;
  for (uint32_t g = 0; g < n_groups; ++g)
    for (uint32_t b = 0; b < n_blocks; ++b)
      for (uint32_t t = 0; t < n_tiles; ++t) grid.push_back(TunePoint{group_widths[g], block_sizes[b], tile_keys[t]});
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  HX_CUDA(cudaEventCreate(&e0));
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return cuda_status(cudaGetLastError());
  }
  // One trial = one replay of the plan's captured graph (the launch the
  // product runs), timed with events on the caller's stream.
  struct Runner {
    hx_batch_plan* p;
    hx_batch_reset_fn reset_fn;
    void* user;
    hx_stream stream;
    cudaStream_t s;
    cudaEvent_t e0, e1;
    hx_status set(const TunePoint& t) { return hx_batch_set_tuning(p, t.group, t.block, t.tile, stream); }
    hx_status reset() { return reset_fn ? reset_fn(user, stream) : hx_batch_clear(p->b, stream); }
    hx_status timed_run(float* ms) {
      HX_CUDA(cudaEventRecord(e0, s));
      hx_status st = hx_batch_run_graph(p, stream);
      if (st != HX_OK) return st;
      HX_CUDA(cudaEventRecord(e1, s));
      HX_CUDA(cudaEventSynchronize(e1));
      HX_CUDA(cudaEventElapsedTime(ms, e0, e1));
      int32_t err = 0;
      if ((st = hx_batch_check(p, &err, stream)) != HX_OK) return st;
      return err == 1 ? HX_ERR_TIMEOUT : (err == 2 ? HX_ERR_CAPACITY : HX_OK);
    }
  } runner{p, reset, reset_user, stream, s, e0, e1};
  std::vector<float> ms(grid.size(), 0.f);
  TunePoint bp{};
  float bms = 0.f;
  const hx_status st = autotune_grid(runner, grid.data(), grid.size(), reps, ms.data(), &bp, &bms);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st != HX_OK) return st;
  for (size_t i = 0; i < grid.size() && trials && i < trials_capacity; ++i)
    trials[i] = hx_batch_trial{grid[i].group, grid[i].block, grid[i].tile, ms[i]};
  *best = hx_batch_trial{bp.group, bp.block, bp.tile, bms};
  return HX_OK;
}

hx_status hx_batch_run_per_map(hx_batch_plan* p, hx_stream stream) {
  HX_RANGE("hx_batch_run_per_map");
  if (!p) return HX_ERR_INVALID_ARG;
  hx_batch* b = p->b;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const uint64_t kb = (uint64_t)b->key_bytes;
  hx_map v;
  // The plain path in the reference's call order for every map: insert,
  // retrieve, erase, clean_tombstones — one launch sequence per map.
  for (unsigned i = 0; i < b->n_maps; ++i) {
    make_view(b, i, &v);
    hx_status st;
    if (!p->ins_off.empty() && p->ins_off[i + 1] > p->ins_off[i]) {
      const uint64_t a0 = p->ins_off[i], n = p->ins_off[i + 1] - a0;
      st = map_insert_view(&v, static_cast<const char*>(p->w.ins_keys) + a0 * kb,
                           static_cast<const char*>(p->w.ins_vals) + a0 * kb, nullptr, n, s);
      if (st != HX_OK) return st;
    }
    if (!p->q_off.empty() && p->q_off[i + 1] > p->q_off[i]) {
      const uint64_t a0 = p->q_off[i], n = p->q_off[i + 1] - a0;
      st = map_find_view(&v, static_cast<const char*>(p->w.query_keys) + a0 * kb,
                         static_cast<char*>(p->w.query_out) + a0 * kb, nullptr, n, false, s);
      if (st != HX_OK) return st;
    }
    if (!p->e_off.empty() && p->e_off[i + 1] > p->e_off[i]) {
      const uint64_t a0 = p->e_off[i], n = p->e_off[i + 1] - a0;
      st = map_find_view(&v, static_cast<const char*>(p->w.erase_keys) + a0 * kb, nullptr, nullptr, n, true, s);
      if (st != HX_OK) return st;
    }
    if (p->w.clean) {
      st = hx_clean_tombstones(&v, stream);
      if (st != HX_OK) return st;
    }
    b->fill_ub[i] = v.fill_ub;
    b->scratch = v.scratch;  // the views share one clean scratch buffer
    b->scratch_bytes = v.scratch_bytes;
  }
  return HX_OK;
}

hx_status hx_batch_inject_stall(hx_batch_plan* p, uint32_t map, int phase, int enable, hx_stream stream) {
  if (!p || map >= p->b->n_maps || phase < 0 || phase >= (int)BP_NPHASES) return HX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t at = (size_t)phase * p->b->n_maps + map;
  const unsigned v = p->rem_host[at] + (enable ? 1u : 0u);  // one tile more than will ever run
  HX_CUDA(cudaMemcpyAsync(p->d_remaining_init + at, &v, sizeof(v), cudaMemcpyHostToDevice, s));
  HX_CUDA(cudaStreamSynchronize(s));
  return HX_OK;
}

hx_status hx_batch_check(hx_batch_plan* p, int32_t* error, hx_stream stream) {
  if (!p || !error) return HX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned e = 0;
  HX_CUDA(cudaMemcpyAsync(&e, p->d_counters + 1, sizeof(e), cudaMemcpyDeviceToHost, s));
  HX_CUDA(cudaStreamSynchronize(s));
  *error = (int32_t)e;
  return e == 1 ? HX_ERR_TIMEOUT : (e ? HX_ERR_CAPACITY : HX_OK);
}

}  // extern "C"
