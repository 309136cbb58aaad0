// hx_scan.cuh — single-pass scan and stable stream compaction.
//
// Replaces the reference's three-kernel compaction (scan_reduce_raw ->
// split_prefix_scan_raw -> split_compact_raw, splitvector/split_tools.h:
// 541-550, 556-602, 444-482) and its two-level Blelloch scan
// (split_prescan + scan_add, split_tools.h:133-195, 78-88) with one pass over
// the input: each CTA takes the next tile from an atomic ticket, reads it with
// 128-bit loads, reduces it, publishes its aggregate, and resolves its
// exclusive prefix by decoupled look-back over the tiles before it
// (Merrill & Garland, "Single-pass Parallel Prefix Scan with Decoupled
// Look-back", NVIDIA tech report NVR-2016-002). Input is read once and the
// output written once: 8 B per element for the u32 scan, sizeof(T) * (n + c)
// for compaction.
//
// Every wait on another tile's status is bounded: after kSpinLimit polls the
// CTA records a timeout in the scratch error word and uses what it has; the
// host turns that word into HX_ERR_TIMEOUT.
#pragma once
#include "hx_device.cuh"
#include "../../include/hx_stream.cuh"
#include <mutex>
#include <set>
#include <atomic>
#include <type_traits>
#include <utility>

namespace hx {

// Tile status word: bits 63..62 = flag, bits 61..0 = value.
constexpr unsigned long long kStAgg = 1ull << 62;   // tile aggregate only
constexpr unsigned long long kStInc = 2ull << 62;   // inclusive prefix
constexpr unsigned long long kStVal = (1ull << 62) - 1;
constexpr unsigned kSpinLimit = 1u << 22;

// Scratch layout (hx_scratch_bytes): [ticket u32][error u32][pad .. 256 B]
// [status u64 x tiles]. The host zeroes the first 256 + 8*tiles bytes before
// each launch.
struct ScanScratch {
  unsigned int* ticket;
  unsigned int* error;
  unsigned long long* status;
};

__host__ __device__ inline uint64_t scan_scratch_bytes(uint64_t tiles) { return 256 + 8 * (tiles ? tiles : 1); }

__device__ __forceinline__ unsigned long long ld_status(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_status(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ unsigned warp_incl_scan(unsigned x, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  return x;
}

// Look-back by warp 0 of the CTA: returns the exclusive prefix of `tile`
// (sum of all earlier tiles, modulo 2^62 / 2^32 by caller) and publishes the
// inclusive prefix. Called by all 32 lanes of warp 0. Each step reads a
// window of 32 * kLookbackV predecessor statuses (lane l holds distances
// l*V+1 .. l*V+V) and waits for those nearer than the closest inclusive one.
#ifndef HX_LOOKBACK_V
#define HX_LOOKBACK_V 1
#endif
constexpr int kLookbackV = HX_LOOKBACK_V;

__device__ __forceinline__ unsigned long long lookback(const ScanScratch& sc, unsigned long long tile,
                                                       unsigned long long aggregate, int lane) {
  constexpr int V = kLookbackV;
  if (tile == 0) {
    if (lane == 0) st_status(sc.status, kStInc | (aggregate & kStVal));
    return 0;
  }
  if (lane == 0) st_status(sc.status + tile, kStAgg | (aggregate & kStVal));
  unsigned long long exclusive = 0;
  long long top = (long long)tile - 1;  // closest predecessor not yet summed
  unsigned spins = 0;
  bool timed_out = false;
  while (true) {
    unsigned long long st[V];
#pragma unroll
    for (int j = 0; j < V; ++j) {
      const long long idx = top - (lane * V + j);
      st[j] = (idx >= 0) ? ld_status(sc.status + idx) : kStInc;  // before tile 0: prefix 0
    }
    // Wait only for the statuses nearer than the closest inclusive prefix in
    // the window (all of them if there is none): the ones beyond it are never
    // summed. Waiting for the whole window meant waiting for the slowest of
    // 32 neighbours still loading their tiles, which dominated a CTA's life.
    while (true) {
      int first = V;  // this lane's nearest inclusive status
#pragma unroll
      for (int j = V - 1; j >= 0; --j)
        if ((st[j] >> 62) == 2) first = j;
      const unsigned inc = __ballot_sync(0xffffffffu, first < V);
      const int stop_lane = inc ? __ffs(inc) - 1 : 32;
      const int stop_j = __shfl_sync(0xffffffffu, first, stop_lane & 31);
      bool missing = false;
#pragma unroll
      for (int j = 0; j < V; ++j) {
        const bool needed = lane < stop_lane || (lane == stop_lane && j <= stop_j);
        missing |= needed && (st[j] >> 62) == 0;
      }
      if (!__any_sync(0xffffffffu, missing)) break;
      if (++spins > kSpinLimit) {
        timed_out = true;
        break;
      }
      if (spins > 64) __nanosleep(spins > 4096 ? 256 : 32);
#pragma unroll
      for (int j = 0; j < V; ++j)
        if ((st[j] >> 62) == 0) st[j] = ld_status(sc.status + (top - (lane * V + j)));
    }
    if (timed_out) {
      if (lane == 0) atomicExch(sc.error, 1u);
      break;
    }
    // Within the lane: sum up to and including its closest inclusive status.
    unsigned long long part = 0, full = 0;
    bool has_inc = false;
#pragma unroll
    for (int j = 0; j < V; ++j) {
      const long long idx = top - (lane * V + j);
      const unsigned long long v = idx >= 0 ? (st[j] & kStVal) : 0ull;
      full += v;
      if (!has_inc) part += v;
      has_inc |= (st[j] >> 62) == 2;
    }
    const unsigned inc_mask = __ballot_sync(0xffffffffu, has_inc);
    // Lanes below the lowest lane with an inclusive status contribute fully,
    // that lane up to its inclusive status, lanes above it nothing.
    const int stop = inc_mask ? (__ffs(inc_mask) - 1) : 32;
    unsigned long long v = lane < stop ? full : (lane == stop ? part : 0ull);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    exclusive += v;
    if (inc_mask) break;
    top -= 32 * V;
  }
  if (lane == 0) st_status(sc.status + tile, kStInc | ((exclusive + aggregate) & kStVal));
  return exclusive;
}

// ---------------------------------------------------------------------------
// Exclusive u32 sum scan. CTA = BLOCK threads; each warp owns a contiguous
// chunk of 32*R uint4 (128*R elements); the tile is BLOCK/32 chunks.
// Thread (warp w, lane l) holds uint4 number r*32+l of its chunk, r < R, so
// every load and store instruction of the warp covers 512 contiguous bytes.
// ---------------------------------------------------------------------------
template <int BLOCK, int R>
__global__ void __launch_bounds__(BLOCK) k_scan_u32(const uint32_t* in, uint32_t* out,
                                                   uint64_t n, ScanScratch sc, bool vec) {
  constexpr int WARPS = BLOCK / 32;
  constexpr uint64_t TILE = (uint64_t)BLOCK * R * 4;
  __shared__ unsigned s_warp[WARPS];
  __shared__ unsigned long long s_tile;
  __shared__ unsigned s_prefix;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_tile = atomicAdd(sc.ticket, 1u);
  __syncthreads();
  const unsigned long long tile = s_tile;
  const uint64_t chunk = tile * TILE + (uint64_t)warp * 32 * R * 4;

  uint32_t x[R][4];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const uint64_t e = chunk + ((uint64_t)r * 32 + lane) * 4;
    if (vec && e + 4 <= n) {
      uint4 q = __ldcs(reinterpret_cast<const uint4*>(in + e));
      x[r][0] = q.x; x[r][1] = q.y; x[r][2] = q.z; x[r][3] = q.w;
    } else {
#pragma unroll
      for (int q = 0; q < 4; ++q) x[r][q] = (e + q < n) ? in[e + q] : 0u;
    }
  }
  // Warp-level exclusive prefixes of each held uint4.
  unsigned pre[R];
  unsigned acc = 0;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const unsigned s = x[r][0] + x[r][1] + x[r][2] + x[r][3];
    const unsigned incl = warp_incl_scan(s, lane);
    pre[r] = acc + incl - s;
    acc += __shfl_sync(0xffffffffu, incl, 31);
  }
  if (lane == 0) s_warp[warp] = acc;
  __syncthreads();
  if (warp == 0) {
    unsigned wt = (lane < WARPS) ? s_warp[lane] : 0u;
    const unsigned wincl = warp_incl_scan(wt, lane);
    const unsigned aggregate = __shfl_sync(0xffffffffu, wincl, 31);
    const unsigned long long tp = lookback(sc, tile, aggregate, lane);
    if (lane < WARPS) s_warp[lane] = wincl - wt;  // exclusive warp offsets
    if (lane == 0) s_prefix = (unsigned)tp;
  }
  __syncthreads();
  const unsigned base = s_prefix + s_warp[warp];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const uint64_t e = chunk + ((uint64_t)r * 32 + lane) * 4;
    unsigned o0 = base + pre[r];
    unsigned o1 = o0 + x[r][0];
    unsigned o2 = o1 + x[r][1];
    unsigned o3 = o2 + x[r][2];
    if (vec && e + 4 <= n) {
      __stcs(reinterpret_cast<uint4*>(out + e), make_uint4(o0, o1, o2, o3));
    } else {
      const unsigned o[4] = {o0, o1, o2, o3};
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (e + q < n) out[e + q] = o[q];
    }
  }
}

// ---------------------------------------------------------------------------
// Stable compaction of T (uint32_t, P32 or P64): E = 16/sizeof(T) elements
// per uint4. Selected elements are staged in shared memory in output order
// and written out as one contiguous run per tile with coalesced stores.
// The count of the last tile's inclusive prefix goes to *d_count.
// ---------------------------------------------------------------------------
// Predicate kinds compiled into the compaction kernel; the launch picks one
// from hx_pred.op, so the hot rules cost a few instructions per element
// instead of a switch (and a division) per element.
enum : int { PK_GENERIC = 0, PK_MOD_LT32 = 1, PK_MASK_EQ = 2, PK_VALID = 3, PK_MOD_LT_THRESH = 4 };

// (x mod d) < s for 32-bit x and 2 <= d <= 2^31, 0 < s < d, from the high
// 32 bits of one product, derived from the direct-remainder method cited
// below: with M = ceil(2^64 / d) (at least 2^33), write x = q*d + r and
// M*d = 2^64 + e (0 <= e < d); then L = M*x mod 2^64 = r*M + q*e without
// wrapping, with 0 <= q*e < 2^32. If r >= s, L >= s*M. If r < s,
// L < (s-1)*M + 2^32 <= s*M - 2^32. So r < s exactly when
// floor(L / 2^32) < floor(s*M / 2^32), and floor(L / 2^32) is
// umulhi(M_lo, x) + M_hi*x mod 2^32: two 32-bit multiplies and a compare.
// The host computes the threshold floor(s*M / 2^32) (s*M < 2^64, as s < d).
__host__ __device__ inline bool mod_lt_thresh_ok(uint64_t d, uint64_t s) {
  return d >= 2 && d <= (1ull << 31) && s > 0 && s < d;
}

// x mod d for 32-bit x and 1 <= d < 2^32 by direct computation (D. Lemire,
// O. Kaser, N. Kurz, "Faster Remainder by Direct Computation: Applications to
// Compilers and Software Libraries", Software: Practice and Experience 2019):
// with M = floor((2^64 - 1) / d) + 1 (mod 2^64), x mod d is the high 64 bits
// of the 128-bit product (M * x mod 2^64) * d.
__host__ __device__ inline uint64_t fastmod_magic(uint32_t d) { return ~0ull / d + 1ull; }
__device__ __forceinline__ uint32_t fastmod_u32(uint32_t x, uint64_t magic, uint32_t d) {
  return (uint32_t)__umul64hi(magic * x, (uint64_t)d);
}

template <class T>
struct ElemOps;
template <>
struct ElemOps<uint32_t> {
  static constexpr int E = 4;
  struct Ctx {};
  template <int PK>
  __device__ static bool pred(const hx_pred& p, const uint32_t& x, const Ctx&, uint64_t magic) {
    bool r;
    if constexpr (PK == PK_MOD_LT32) r = fastmod_u32(x, magic, (uint32_t)p.a) < (uint32_t)p.b;  // as pred_on32
    else if constexpr (PK == PK_MASK_EQ) r = ((uint64_t)x & p.a) == p.b;
    else r = pred_on32(p, x);
    return (p.flags & HX_PRED_NEGATE) ? !r : r;
  }
};
template <class P>
struct PairOps {
  static constexpr int E = 16 / sizeof(P);
  using Ctx = TableRef<P>;
  template <int PK>
  __device__ static bool pred(const hx_pred& p, const P& x, const Ctx& c, uint64_t magic) {
    if constexpr (PK == PK_GENERIC) {
      return pred_pair<P>(p, x.first, x.second, c);
    } else {
      using Tr = PairTraits<P>;
      const bool sentinel = (x.first == Tr::EMPTY) || (x.first == Tr::TOMB);
      bool r;
      if constexpr (PK == PK_VALID) {
        r = !sentinel;
      } else {
        const auto f = (p.field == HX_FIELD_VALUE) ? (uint64_t)x.second : (uint64_t)x.first;
        if constexpr (PK == PK_MOD_LT32) r = fastmod_u32((uint32_t)f, magic, (uint32_t)p.a) < p.b;  // 32-bit fields
        else r = (f & p.a) == p.b;
        if ((p.flags & HX_PRED_SKIP_SENTINELS) && sentinel) r = false;
      }
      return (p.flags & HX_PRED_NEGATE) ? !r : r;
    }
  }
};
template <>
struct ElemOps<P32> : PairOps<P32> {};
template <>
struct ElemOps<P64> : PairOps<P64> {};

// The kernel variant for a predicate (CLEAN passes always use the generic one).
template <class T>
inline int pred_kind(const hx_pred& p) {
  if (p.op == HX_PRED_MASK_EQ) return PK_MASK_EQ;
  if constexpr (std::is_same<T, uint32_t>::value) {
    if (p.op == HX_PRED_MOD_LT && (uint32_t)p.a != 0) return PK_MOD_LT32;
  } else {
    if (p.op == HX_PRED_VALID) return PK_VALID;
    if (std::is_same<T, P32>::value && p.op == HX_PRED_MOD_LT && p.a != 0 && p.a <= 0xFFFFFFFFull) return PK_MOD_LT32;
  }
  return PK_GENERIC;
}

template <class T>
__device__ __forceinline__ void load_vec(const T* p, T (&v)[16 / sizeof(T)]) {
  uint4 q = __ldcs(reinterpret_cast<const uint4*>(p));
  memcpy(&v[0], &q, 16);
}

// What a selected element writes: the element itself, or (O = its key type)
// only the key of a bucket pair (extractKeysByPattern).
template <class T, class O>
__device__ __forceinline__ O project(const T& x) {
  if constexpr (std::is_same<T, O>::value) return x;
  else return x.first;
}

// clean_tombstones mode (CLEAN): the input is the bucket array itself. Every
// TOMBSTONE bucket and every selected (moved) bucket is rewritten to
// (EMPTY, 0) after it has been read, the last tile takes the moved count off
// fill, and the whole pass is skipped when *skip is set. The
// phase-partitioned kernel decides "not home" from the bucket's index
// (home(Y) != i) and reads no other bucket. The look-back kernel reads the
// home bucket; one that another CTA rewrites at the same time cannot change
// its decision: a key Y is "not home" iff bucket[home(Y)] holds a key other
// than Y, and that bucket only ever changes between keys other than Y and
// EMPTY.
struct CleanArgs {
  const unsigned* skip;
  unsigned long long* fill;
};

template <class T, int R>
__device__ __forceinline__ void compact_load(const T* in, uint64_t n, uint64_t chunk, int lane, bool vec,
                                             T (&x)[R][16 / sizeof(T)]) {
  constexpr int E = 16 / sizeof(T);
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const uint64_t e = chunk + ((uint64_t)r * 32 + lane) * E;
    if (vec && e + E <= n) {
      load_vec<T>(in + e, x[r]);
    } else {
#pragma unroll
      for (int q = 0; q < E; ++q)
        if (e + q < n) x[r][q] = in[e + q];
    }
  }
}

// One tile = S sub-tiles of BLOCK*R*E elements. The CTA walks its sub-tiles
// in order, loading sub-tile s+1 while it selects from sub-tile s and stages
// the selected elements (or their keys) in shared memory at their tile-local
// output index; one look-back per tile then places the staged run in the
// output with coalesced stores. Registers hold two sub-tiles whatever S is,
// and the look-back, which bounds how many tiles per second the GPU can
// retire, is paid once per S sub-tiles.
template <class T, class O, int BLOCK, int R, int S, bool CLEAN, int PK>
__global__ void __launch_bounds__(BLOCK) k_compact(const T* __restrict__ in, O* __restrict__ out, uint64_t n,
                                                  hx_pred pr, uint64_t magic, typename ElemOps<T>::Ctx ctx,
                                                  uint64_t capacity, unsigned long long* d_count, ScanScratch sc,
                                                  bool vec, CleanArgs cl) {
  constexpr int E = ElemOps<T>::E;
  constexpr int WARPS = BLOCK / 32;
  constexpr uint64_t SUB = (uint64_t)BLOCK * R * E;
  constexpr uint64_t TILE = SUB * S;
  __shared__ unsigned s_warp[WARPS];
  __shared__ unsigned long long s_tile, s_prefix;
  __shared__ unsigned s_sub;
  extern __shared__ __align__(16) unsigned char s_raw[];
  O* s_out = reinterpret_cast<O*>(s_raw);

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if constexpr (CLEAN) {
    if (*cl.skip) return;
  }
  if (threadIdx.x == 0) s_tile = atomicAdd(sc.ticket, 1u);
  __syncthreads();
  const unsigned long long tile = s_tile;
  const uint64_t tile0 = tile * TILE;
  const uint64_t wchunk = (uint64_t)warp * 32 * R * E;

  T x[R][E], nx[R][E];
  compact_load<T, R>(in, n, tile0 + wchunk, lane, vec, x);
  unsigned staged = 0;  // selected elements of the earlier sub-tiles (block-uniform)
#pragma unroll 1
  for (int sub = 0; sub < S; ++sub) {
    const uint64_t chunk = tile0 + (uint64_t)sub * SUB + wchunk;
    if (sub + 1 < S) compact_load<T, R>(in, n, chunk + SUB, lane, vec, nx);
    unsigned f[R];  // selection bits of each held uint4
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const uint64_t e = chunk + ((uint64_t)r * 32 + lane) * E;
      unsigned bits = 0;
#pragma unroll
      for (int q = 0; q < E; ++q)
        if (e + q < n && ElemOps<T>::template pred<PK>(pr, x[r][q], ctx, magic)) bits |= 1u << q;
      f[r] = bits;
      if constexpr (CLEAN) {
        using Tr = PairTraits<T>;
#pragma unroll
        for (int q = 0; q < E; ++q)
          if (e + q < n && ((bits >> q) & 1u || x[r][q].first == Tr::TOMB)) {
            T empty;
            empty.first = Tr::EMPTY;
            empty.second = 0;
            const_cast<T*>(in)[e + q] = empty;
          }
      }
    }
    unsigned pre[R];
    unsigned acc = 0;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const unsigned c = __popc(f[r]);
      const unsigned incl = warp_incl_scan(c, lane);
      pre[r] = acc + incl - c;
      acc += __shfl_sync(0xffffffffu, incl, 31);
    }
    if (lane == 0) s_warp[warp] = acc;
    __syncthreads();
    if (warp == 0) {
      const unsigned wt = (lane < WARPS) ? s_warp[lane] : 0u;
      const unsigned wincl = warp_incl_scan(wt, lane);
      if (lane < WARPS) s_warp[lane] = wincl - wt;
      if (lane == 31) s_sub = wincl;
    }
    __syncthreads();
    unsigned o = staged + s_warp[warp];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      unsigned p = o + pre[r];
#pragma unroll
      for (int q = 0; q < E; ++q)
        if (f[r] & (1u << q)) s_out[p++] = project<T, O>(x[r][q]);
    }
    staged += s_sub;
    if (sub + 1 < S) {
#pragma unroll
      for (int r = 0; r < R; ++r)
#pragma unroll
        for (int q = 0; q < E; ++q) x[r][q] = nx[r][q];
    }
    __syncthreads();  // s_warp and s_sub are rewritten by the next sub-tile
  }
  if (warp == 0) {
    const unsigned long long tp = lookback(sc, tile, staged, lane);
    if (lane == 0) {
      s_prefix = tp;
      if (tile0 + TILE >= n) {  // last tile
        if (d_count) *d_count = tp + staged;
        if constexpr (CLEAN) atomicAdd(cl.fill, 0ull - (tp + staged));
      }
    }
  }
  __syncthreads();
  const unsigned long long prefix = s_prefix;
  for (unsigned i = threadIdx.x; i < staged; i += BLOCK) {
    const unsigned long long dst = prefix + i;
    if (dst < capacity) out[dst] = s_out[i];
  }
}

// ---- host launch helpers ---------------------------------------------------
constexpr int kScanBlock = 256;
constexpr int kScanR = 12;     // register kernel: 256 threads x 12 uint4 = 12288 u32 per tile (sweep of 4..16)
constexpr int kCompactBlock = 256;
constexpr int kCompactR = 4;  // 256 threads x 4 uint4 = 16 KiB per sub-tile
#ifndef HX_COMPACT_S
#define HX_COMPACT_S 4
#endif
constexpr int kCompactS = HX_COMPACT_S;  // sub-tiles per tile

// Tiles of the register-staged scan (the path for buffers that are not
// 16-byte aligned).
inline uint64_t scan_tiles(uint64_t n) {
  const uint64_t t = (uint64_t)kScanBlock * kScanR * 4;
  return (n + t - 1) / t;
}
template <class T>
inline uint64_t compact_tile_elems() {
  return (uint64_t)kCompactBlock * kCompactR * (16 / sizeof(T)) * kCompactS;
}
template <class T>
inline uint64_t compact_tiles(uint64_t n) {
  const uint64_t t = compact_tile_elems<T>();
  return (n + t - 1) / t;
}
// Scratch a scan or a compaction of n elements needs, whichever kernel runs:
// the look-back statuses of the register-staged kernels, or the count slots
// of the phase-partitioned kernels (hx_stream.cuh).
inline uint64_t scan_scratch_need(uint64_t n) {
  const uint64_t a = scan_scratch_bytes(scan_tiles(n)), b = hxs::scratch_need(n, 4);
  return a > b ? a : b;
}
template <class T>
inline uint64_t compact_scratch_need(uint64_t n) {
  const uint64_t a = scan_scratch_bytes(compact_tiles<T>(n)), b = hxs::scratch_need(n, sizeof(T));
  return a > b ? a : b;
}
inline ScanScratch carve_scratch(void* p, uint64_t tiles) {
  ScanScratch sc;
  sc.ticket = reinterpret_cast<unsigned int*>(p);
  sc.error = sc.ticket + 1;
  sc.status = reinterpret_cast<unsigned long long*>(reinterpret_cast<char*>(p) + 256);
  (void)tiles;
  return sc;
}
// Where each kernel family keeps its error word in the scratch.
inline unsigned* scan_error_word(void* scratch, bool stream_kernel) {
  return stream_kernel ? hxs::carve(scratch).error : carve_scratch(scratch, 0).error;
}
inline bool aligned16(const void* p) { return ((uintptr_t)p % 16) == 0; }

// Raise a kernel's dynamic shared-memory limit once (per kernel and device)
// when it needs more than the default 48 KiB.
template <class Kern>
inline cudaError_t allow_dynamic_smem(Kern kern, size_t smem) {
  if (smem <= 48 * 1024) return cudaSuccess;
  static std::mutex mu;
  static std::set<std::pair<const void*, int>> done;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> g(mu);
  const auto key = std::make_pair(reinterpret_cast<const void*>(kern), dev);
  if (done.count(key)) return cudaSuccess;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) done.insert(key);
  return e;
}

// Launch one exclusive scan (n > 0) with scratch of scan_scratch_need(n)
// bytes, which is zeroed here: the phase-partitioned kernel when both
// buffers are 16-byte aligned, else the register kernel over every tile.
// Returns through *stream_kernel which one ran (for its error word).
inline cudaError_t launch_scan(const uint32_t* in, uint32_t* out, uint64_t n, void* scratch, cudaStream_t s,
                               bool* stream_kernel = nullptr) {
  const bool sk = aligned16(in) && aligned16(out);
  if (stream_kernel) *stream_kernel = sk;
  if (sk)
    return hxs::launch<uint32_t, uint32_t, hxs::ScanSel, true>(in, out, n, hxs::ScanSel{}, 0,
                                                                          hxs::Done{}, scratch, s);
  const uint64_t tiles = scan_tiles(n);
  cudaError_t e = cudaMemsetAsync(scratch, 0, scan_scratch_bytes(tiles), s);
  if (e != cudaSuccess) return e;
  k_scan_u32<kScanBlock, kScanR><<<(unsigned)tiles, kScanBlock, 0, s>>>(in, out, n, carve_scratch(scratch, tiles),
                                                                       false);
  return cudaGetLastError();
}

// The predicate of a compaction for the phase-partitioned kernel: one
// compiled predicate kind (PK_*), and in clean_tombstones mode (CLEAN) the
// rewrite of every TOMBSTONE and every selected bucket to (EMPTY, 0) after
// it has been read (see CleanArgs).
template <class T, int PK, bool CLEAN>
struct PredSel {
  hx_pred pr;
  uint64_t magic;
  typename ElemOps<T>::Ctx ctx;
  uint64_t thresh = 0;  // PK_MOD_LT_THRESH: floor(s * magic / 2^32)
  static constexpr bool kRewrites = CLEAN;
  // generic pair rules may be HX_PRED_NOT_HOME, which compares a bucket's
  // index with its key's home bucket
  static constexpr bool kIndexed = PK == PK_GENERIC && !std::is_same<T, uint32_t>::value;
  __device__ __forceinline__ bool at(const T& x, uint64_t i) const {
    if constexpr (kIndexed) return pred_pair_at<T>(pr, x.first, x.second, i, ctx.sp);
    else return (*this)(x);
  }
  __device__ __forceinline__ bool operator()(const T& x) const {
    if constexpr (PK == PK_MOD_LT_THRESH) {
      uint32_t f;
      if constexpr (std::is_same<T, uint32_t>::value) f = x;
      else f = (uint32_t)(pr.field == HX_FIELD_VALUE ? x.second : x.first);
      const uint32_t hi = __umulhi((uint32_t)magic, f) + (uint32_t)(magic >> 32) * f;
      bool r = hi < (uint32_t)thresh;
      if constexpr (!std::is_same<T, uint32_t>::value) {
        using Tr = PairTraits<T>;
        if ((pr.flags & HX_PRED_SKIP_SENTINELS) && (x.first == Tr::EMPTY || x.first == Tr::TOMB)) r = false;
      }
      return (pr.flags & HX_PRED_NEGATE) ? !r : r;
    } else {
      return ElemOps<T>::template pred<PK>(pr, x, ctx, magic);
    }
  }
  __device__ __forceinline__ void rewrite(T* in, uint64_t i, const T& x, bool selected) const {
    if constexpr (CLEAN) {
      using Tr = PairTraits<T>;
      if (selected || x.first == Tr::TOMB) {
        T empty;
        empty.first = Tr::EMPTY;
        empty.second = 0;
        in[i] = empty;
      }
    }
  }
};

// Launch one compaction pass (n > 0) with scratch of compact_scratch_need<T>(n)
// bytes, which is zeroed here: the phase-partitioned kernel when the input
// is 16-byte aligned, else the look-back kernel k_compact.
template <class T, bool CLEAN, class O = T>
inline cudaError_t launch_compact(const T* in, O* out, uint64_t n, const hx_pred& pr,
                                  typename ElemOps<T>::Ctx ctx, uint64_t capacity, unsigned long long* d_count,
                                  void* scratch, CleanArgs cl, cudaStream_t s, bool* stream_kernel = nullptr) {
  const bool sk = aligned16(in);
  if (stream_kernel) *stream_kernel = sk;
  if (sk) {
    const hxs::Done done{d_count, CLEAN ? cl.fill : nullptr, CLEAN ? cl.skip : nullptr};
    auto go = [&](auto sel) -> cudaError_t {
      return hxs::launch<T, O, decltype(sel), false>(in, out, n, sel, capacity, done, scratch, s);
    };
    if constexpr (CLEAN) {
      return go(PredSel<T, PK_GENERIC, true>{pr, 0, ctx});
    } else {
      switch (pred_kind<T>(pr)) {
        case PK_MOD_LT32:
          if (mod_lt_thresh_ok(pr.a, pr.b)) {
            const uint64_t m = fastmod_magic((uint32_t)pr.a);
            return go(PredSel<T, PK_MOD_LT_THRESH, false>{pr, m, ctx, (pr.b * m) >> 32});
          }
          return go(PredSel<T, PK_MOD_LT32, false>{pr, fastmod_magic((uint32_t)pr.a), ctx});
        case PK_MASK_EQ:
          return go(PredSel<T, PK_MASK_EQ, false>{pr, 0, ctx});
        case PK_VALID:
          if constexpr (!std::is_same<T, uint32_t>::value) return go(PredSel<T, PK_VALID, false>{pr, 0, ctx});
          [[fallthrough]];
        default:
          return go(PredSel<T, PK_GENERIC, false>{pr, 0, ctx});
      }
    }
  }
  const uint64_t tiles = compact_tiles<T>(n);
  cudaError_t e = cudaMemsetAsync(scratch, 0, scan_scratch_bytes(tiles), s);
  if (e != cudaSuccess) return e;
  const size_t smem = (size_t)compact_tile_elems<T>() * sizeof(O);
  const ScanScratch sc = carve_scratch(scratch, tiles);
  const unsigned grid = (unsigned)tiles;
  auto launch = [&](auto kern, uint64_t magic) -> cudaError_t {
    cudaError_t err = allow_dynamic_smem(kern, smem);
    if (err != cudaSuccess) return err;
    kern<<<grid, kCompactBlock, smem, s>>>(in, out, n, pr, magic, ctx, capacity, d_count, sc, false, cl);
    return cudaGetLastError();
  };
  if constexpr (CLEAN) {
    return launch(k_compact<T, O, kCompactBlock, kCompactR, kCompactS, true, PK_GENERIC>, 0);
  } else {
    switch (pred_kind<T>(pr)) {
      case PK_MOD_LT32:
        return launch(k_compact<T, O, kCompactBlock, kCompactR, kCompactS, false, PK_MOD_LT32>,
                      fastmod_magic((uint32_t)pr.a));
      case PK_MASK_EQ:
        return launch(k_compact<T, O, kCompactBlock, kCompactR, kCompactS, false, PK_MASK_EQ>, 0);
      case PK_VALID:
        if constexpr (!std::is_same<T, uint32_t>::value)
          return launch(k_compact<T, O, kCompactBlock, kCompactR, kCompactS, false, PK_VALID>, 0);
        [[fallthrough]];
      default:
        return launch(k_compact<T, O, kCompactBlock, kCompactR, kCompactS, false, PK_GENERIC>, 0);
    }
  }
}

}  // namespace hx
