// hx_stream.cuh — phase-partitioned streaming kernels: stable stream
// compaction (copy_if, extractPattern, the clean_tombstones pass) and the
// exclusive u32 scan, for 16-byte-aligned inputs.
//
// Header-only so that the drop-in C++ header can instantiate the same
// compaction for a caller's own `Rule` functor in the caller's translation
// unit; libhx instantiates it for its predicate descriptors.
//
// Shape. One cooperative launch of G co-resident CTAs (G = resident CTAs per
// SM x SMs). The input is cut into slices (one stage of shared memory, 64 KiB
// by default); phase p gives slice p*G + b to CTA b, so
// a phase is G consecutive slices. Each CTA keeps STAGES slices in flight,
// each filled by one bulk copy (cp.async.bulk, completion on an mbarrier).
//   pass 1, phase p: read the slice from shared memory, evaluate the rule (or
//     sum, for the scan), write the CTA-local result back into the same stage
//     (the selected elements packed at the front, or the local exclusive
//     sums), and publish the CTA's count for phase p in a slot of scratch.
//   pass 2, phase p - D (D phases later): read every CTA's count of that
//     phase, which by then are almost always published, add up those of the
//     CTAs before this one and of all earlier phases, write the stage's result
//     to global memory at that offset, and refill the stage with a later slice.
// So the input is read once, the output written once, the only exchange
// between CTAs is one count per CTA per phase, and its latency is hidden
// behind D phases of work instead of sitting on every tile's critical path
// as in a decoupled look-back.
//
// Co-residency: every CTA waits for the counts of every other, so the launch
// is cooperative (the runtime guarantees all CTAs resident). Every wait is
// still bounded: an mbarrier wait or a count wait that runs out (about one
// second) sets the scratch error word; every CTA that sees the error word
// stops, waits (bounded) for the bulk copies it issued, and returns.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <map>
#include <mutex>
#include <type_traits>
#include <utility>

namespace hxs {

// ---- PTX helpers --------------------------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
constexpr unsigned long long kWaitNs = 1000000000ull;  // about one second per wait
// Waits for the phase of `bar` with `parity`; false after about a second.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
  if (mbar_try(bar, parity)) return true;
  const unsigned long long t0 = globaltimer();
  for (unsigned i = 0; i < (1u << 26); ++i) {
    if (mbar_try(bar, parity)) return true;
    if ((i & 255) == 255 && globaltimer() - t0 > kWaitNs) return false;
  }
  return false;
}
// One bulk copy of `bytes` (a multiple of 16, both addresses 16-byte aligned)
// from global into shared memory, completing `bytes` transactions on `bar`.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned ld_relaxed_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned warp_incl_scan(unsigned x, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  return x;
}

// ---- geometry and scratch -------------------------------------------------
// Tuned on GB300 over slices of 8-64 KiB, 3-6 stages, deferral 1-3 and
// 256/512/768/1024-thread blocks (2^28 u32 copy_if and scan).
#ifndef HX_STREAM_BLOCK
#define HX_STREAM_BLOCK 512
#endif
#ifndef HX_STREAM_R
#define HX_STREAM_R 8  // uint4 per thread per slice: 512 threads x 8 x 16 B = 64 KiB slices
#endif
#ifndef HX_STREAM_STAGES
#define HX_STREAM_STAGES 3
#endif
#ifndef HX_STREAM_DEFER
#define HX_STREAM_DEFER 1
#endif
#ifndef HX_STREAM_LANE_CHUNKS
#define HX_STREAM_LANE_CHUNKS 0  // compaction: each lane owns kR consecutive uint4s (see the kernel)
#endif
#ifndef HX_STREAM_MINB
#define HX_STREAM_MINB 1  // CTAs per SM the register allocation must allow
#endif
constexpr int kBlock = HX_STREAM_BLOCK;
static_assert(kBlock % 32 == 0 && kBlock <= 1024, "whole warps, at most 32 of them");
constexpr int kR = HX_STREAM_R;
constexpr int kStages = HX_STREAM_STAGES;
constexpr int kDefer = HX_STREAM_DEFER;
constexpr bool kLaneChunks = HX_STREAM_LANE_CHUNKS != 0;
static_assert(kDefer >= 1 && kDefer < kStages, "a stage must be free to load while D phases wait");
// Count slots per CTA. In phase p a CTA publishes its count of p, then
// reads every CTA's count of p - D; so when it publishes p it has read every
// count of p - 1 - D, every CTA has published p - 1 - D, and every CTA has
// therefore read every count of the phases up to p - 2 - 2D. The row of
// phase p is the row of phase p - kSlots, so kSlots = 2D + 2.
constexpr int kSlots = 2 * kDefer + 2;
constexpr int kMaxGrid = 1024;  // CTAs at most (GB300: 152 SMs x 1-2 CTAs); a larger device runs 1024
constexpr int kSlotLoads = (kMaxGrid + kBlock - 1) / kBlock;  // count slots each thread reads per phase
constexpr unsigned kSliceBytes = kBlock * kR * 16;

// Scratch: [error word u32][pad .. 256 B][count slots u64 x kSlots x grid].
// The launcher zeroes the part it uses.
constexpr uint64_t kScratchBytes = 256 + 8ull * kSlots * kMaxGrid;
inline uint64_t scratch_bytes_used(unsigned grid) { return 256 + 8ull * kSlots * grid; }
// Scratch a pass over n elements of elem_bytes each needs: its grid is at
// most one CTA per slice.
inline uint64_t scratch_need(uint64_t n, unsigned elem_bytes) {
  uint64_t slices = (n * elem_bytes + kSliceBytes - 1) / kSliceBytes;
  if (slices < 1) slices = 1;
  if (slices > (uint64_t)kMaxGrid) slices = kMaxGrid;
  return scratch_bytes_used((unsigned)slices);
}

struct Scratch {
  unsigned* error;
  unsigned long long* slots;
};
inline Scratch carve(void* p) {
  Scratch s;
  s.error = reinterpret_cast<unsigned*>(p);
  s.slots = reinterpret_cast<unsigned long long*>(static_cast<char*>(p) + 256);
  return s;
}

// What a selected element writes: the element, or only the key of a pair.
template <class T, class O>
__device__ __forceinline__ O project(const T& x) {
  if constexpr (std::is_same<T, O>::value) return x;
  else return x.first;
}

// Selector concept (compaction): a copyable struct with
//   __device__ bool operator()(const T& x) const;
//   static constexpr bool kRewrites;   // true: called as below for every element of the input
//   __device__ void rewrite(T* in, uint64_t i, const T& x, bool selected) const;
//   static constexpr bool kIndexed;    // true: the rule is called as at(x, i), i the element's index
// kRewrites lets the clean_tombstones pass empty the buckets it takes out;
// kIndexed lets a rule depend on where the element sits (a bucket's home).
template <class F>
struct FunctorSel {
  F f;
  static constexpr bool kRewrites = false;
  static constexpr bool kIndexed = false;
  template <class T>
  __device__ __forceinline__ bool operator()(const T& x) const {
    return f(x);
  }
  template <class T>
  __device__ __forceinline__ void rewrite(T*, uint64_t, const T&, bool) const {}
};
struct ScanSel {  // placeholder selector of the scan
  static constexpr bool kRewrites = false;
  static constexpr bool kIndexed = false;
  template <class T>
  __device__ __forceinline__ bool operator()(const T&) const {
    return true;
  }
  template <class T>
  __device__ __forceinline__ void rewrite(T*, uint64_t, const T&, bool) const {}
};

struct Done {                              // what the pass reports, and where it starts
  unsigned long long* d_count;              // if set, *d_count = min(total, count_max) (compaction)
  unsigned long long* sub_from;             // if set, *sub_from -= total (clean_tombstones' fill)
  const unsigned* skip;                     // if set and *skip != 0, the pass does nothing at all
  unsigned long long count_max = ~0ull;     // the largest count written to *d_count
  const unsigned long long* base_from = nullptr;  // if set, output starts at out[*base_from] (and
                                                  // the total counts it), after elements placed earlier
  const unsigned long long* n_from = nullptr;     // if set, the input has min(n, *n_from) elements,
                                                  // read on the device (n is then an upper bound)
};

// ---------------------------------------------------------------------------
// The kernel. SCAN: T = O = uint32_t, out[i] = sum of in[0..i) mod 2^32.
// Otherwise: out[0..c) = the selected elements (projected to O) in input
// order, writes beyond `capacity` dropped, c to *done.d_count.
// ---------------------------------------------------------------------------
template <class T, class O, class Sel, bool SCAN>
__global__ void __launch_bounds__(kBlock, HX_STREAM_MINB) k_stream(const T* __restrict__ in, O* __restrict__ out, uint64_t n,
                                                  Sel sel, uint64_t capacity, Done done, Scratch sc) {
  constexpr int E = 16 / sizeof(T);
  constexpr int WARPS = kBlock / 32;
  constexpr unsigned SU4 = kBlock * kR;  // uint4 per slice
  constexpr unsigned SE = SU4 * E;       // elements per slice
  static_assert(!SCAN || std::is_same<T, uint32_t>::value, "the scan is over uint32_t");
  static_assert(sizeof(O) <= sizeof(T), "the packed result fits in its stage");
  extern __shared__ __align__(128) uint4 s_stage[];  // kStages x SU4
  __shared__ __align__(8) uint64_t s_bar[kStages];
  __shared__ unsigned s_warp[WARPS];
  __shared__ unsigned s_cnt[kStages];
  __shared__ uint2 s_red[WARPS];  // per warp: (count before this CTA, phase total), both < 2^32
  __shared__ int s_abort;

  // Device-side inputs: the same values for every CTA, so every CTA runs the
  // same phases and none waits on a CTA that skipped.
  if (done.skip && *done.skip) return;
  if (done.n_from && *done.n_from < n) n = *done.n_from;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned G = gridDim.x, b = blockIdx.x;
  const uint64_t full_slices = n / SE;  // slices wholly inside [0, n)
  const unsigned phases = (unsigned)(((n + SE - 1) / SE + G - 1) / G);  // below 2^32 - kDefer (launch)
  unsigned pend = 0;                    // thread 0: stages with a bulk copy not yet seen complete
  unsigned par = 0;                     // parity of the next wait, bit per stage

  // Fill stage st with the slice of phase p (thread 0): a whole slice by one
  // bulk copy; the ragged last slice and slices past n are read later with
  // plain loads, so their barrier phase completes with no bytes.
  auto issue = [&](int st, unsigned p) {
    const uint64_t t = (uint64_t)p * G + b;
    if (t < full_slices) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // earlier reads of the stage come first
      mbar_expect_tx(&s_bar[st], kSliceBytes);
      bulk_load(s_stage + (size_t)st * SU4, in + t * SE, kSliceBytes, &s_bar[st]);
    } else {
      mbar_expect_tx(&s_bar[st], 0);
    }
    pend |= 1u << st;
  };
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) mbar_init(&s_bar[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_abort = 0;
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int s = 0; s < kStages && (unsigned)s < phases; ++s) issue(s, s);

  // result count (or sum) of the phases already written, after any elements placed before this pass
  unsigned long long base = done.base_from ? *done.base_from : 0ull;
  bool failed = false;
  // stage and count-slot row of phase p (pass 1) and of phase p - kDefer
  // (pass 2), advanced by one each phase instead of computed by division
  unsigned st1 = 0, st2 = 0, sl1 = 0, sl2 = 0;
  auto next = [](unsigned& i, unsigned m) { i = i + 1 == m ? 0u : i + 1; };
  for (unsigned p = 0; p < phases + kDefer; ++p) {
    // The count slots that pass 2 reads below were published kDefer phases
    // ago: load them now, so that their latency overlaps pass 1.
    unsigned long long pv[kSlotLoads];
    if (p >= (unsigned)kDefer) {
      const unsigned long long* row = sc.slots + sl2 * G;
#pragma unroll
      for (int k = 0; k < kSlotLoads; ++k) {
        const unsigned c = threadIdx.x + k * kBlock;
        pv[k] = c < G ? ld_relaxed(row + c) : 0ull;
      }
    }
    // ---- pass 1: phase p -------------------------------------------------
    if (p < phases) {
      const unsigned st = st1;
      const bool ok = mbar_wait(&s_bar[st], (par >> st) & 1u);
      if (ok) {  // a failed wait leaves par and pend as they were, for the drain below
        par ^= 1u << st;
        pend &= ~(1u << st);
      }
      const uint64_t t = (uint64_t)p * G + b;
      const bool whole = t < full_slices;
      const uint64_t e0 = t * SE;
      T x[kR][E];
      uint4* stage = s_stage + (size_t)st * SU4;
      const unsigned wbase = warp * 32 * kR;  // this warp's first uint4 of the slice
      // Where register row r comes from. By default row r of the warp is 32
      // consecutive uint4s, one per lane. With lane chunks (compaction only),
      // lane l owns the kR consecutive uint4s l*kR .. l*kR+kR-1 of the warp's
      // part and row r holds its uint4 (r + l) mod kR: rotated, so that with
      // kR = 8 the 8 lanes of a shared-memory wavefront read 8 different bank
      // groups.
      constexpr bool LANE = kLaneChunks && !SCAN && (kR & (kR - 1)) == 0 && kR * E <= 32;
      auto u_of = [&](int r) -> unsigned {
        if constexpr (LANE) return wbase + lane * kR + ((r + lane) & (kR - 1));
        else return wbase + r * 32 + lane;
      };
#pragma unroll
      for (int r = 0; r < kR; ++r) {
        const unsigned u = u_of(r);
        if (whole) {
          const uint4 q = stage[u];
          memcpy(&x[r][0], &q, 16);
        } else {
#pragma unroll
          for (int q = 0; q < E; ++q) {
            const uint64_t e = e0 + (uint64_t)u * E + q;
            if (e < n) x[r][q] = in[e];
            else memset(&x[r][q], 0, sizeof(T));
          }
        }
      }
      if (__syncthreads_or(!ok)) {  // stage st is read; a failed wait stops every thread here
        failed = true;
        break;
      }
      unsigned pre[kR];
      unsigned acc = 0;
      unsigned bits[kR];
      unsigned cnt[kR];
      unsigned lm = 0;  // lane chunks: the lane's selections, bit j*E + q for element q of its uint4 j
#pragma unroll
      for (int r = 0; r < kR; ++r) {
        unsigned c;
        if constexpr (SCAN) {
          c = x[r][0] + x[r][1] + x[r][2] + x[r][3];
          bits[r] = 0;
        } else {
          const uint64_t e = e0 + (uint64_t)u_of(r) * E;
          unsigned m = 0;
          if (whole) {  // block-uniform: no per-element bounds checks in a whole slice
#pragma unroll
            for (int q = 0; q < E; ++q) {
              bool s;
              if constexpr (Sel::kIndexed) s = sel.at(x[r][q], e + q);
              else s = sel(x[r][q]);
              m |= (unsigned)s << q;
              if constexpr (Sel::kRewrites) sel.rewrite(const_cast<T*>(in), e + q, x[r][q], s);
            }
          } else {
#pragma unroll
            for (int q = 0; q < E; ++q) {
              const bool in_range = e + q < n;
              bool s = false;
              if (in_range) {
                if constexpr (Sel::kIndexed) s = sel.at(x[r][q], e + q);
                else s = sel(x[r][q]);
              }
              if (s) m |= 1u << q;
              if constexpr (Sel::kRewrites) {
                if (in_range) sel.rewrite(const_cast<T*>(in), e + q, x[r][q], s);
              }
            }
          }
          bits[r] = m;
          if constexpr (LANE) lm |= m << (((r + lane) & (kR - 1)) * E);
          c = __popc(m);
        }
        cnt[r] = c;
        if constexpr (SCAN) {
          const unsigned incl = warp_incl_scan(c, lane);
          pre[r] = acc + incl - c;
          acc += __shfl_sync(0xffffffffu, incl, 31);
        }
      }
      unsigned lane_pre = 0;  // lane chunks: selections of the warp's lanes before this one
      if constexpr (LANE) {
        const unsigned c = __popc(lm);
        const unsigned incl = warp_incl_scan(c, lane);
        lane_pre = incl - c;
        acc = __shfl_sync(0xffffffffu, incl, 31);
      } else if constexpr (!SCAN) {
        // Ranks of the selections: a lane's count per uint4 is at most 4 and a
        // warp's sum at most 128, so four uint4s share one 32-bit word as byte
        // lanes with no carries between them: one warp scan per four uint4s.
        constexpr int NW = (kR + 3) / 4;
        unsigned packed_c[NW], incl_w[NW], tot_w[NW];
#pragma unroll
        for (int w = 0; w < NW; ++w) packed_c[w] = 0;
#pragma unroll
        for (int r = 0; r < kR; ++r) packed_c[r / 4] |= cnt[r] << (8 * (r % 4));
#pragma unroll
        for (int w = 0; w < NW; ++w) {
          incl_w[w] = warp_incl_scan(packed_c[w], lane);
          tot_w[w] = __shfl_sync(0xffffffffu, incl_w[w], 31);
        }
#pragma unroll
        for (int r = 0; r < kR; ++r) {
          const unsigned incl = (incl_w[r / 4] >> (8 * (r % 4))) & 0xffu;
          pre[r] = acc + incl - cnt[r];
          acc += (tot_w[r / 4] >> (8 * (r % 4))) & 0xffu;
        }
      }
      if (lane == 0) s_warp[warp] = acc;
      __syncthreads();
      if (warp == 0) {
        const unsigned wt = lane < WARPS ? s_warp[lane] : 0u;
        const unsigned wincl = warp_incl_scan(wt, lane);
        if (lane < WARPS) s_warp[lane] = wincl - wt;
        if (lane == 31) {
          s_cnt[st] = wincl;
          // publish this CTA's count (or sum, mod 2^32) of phase p, tagged with p + 1
          st_relaxed(sc.slots + sl1 * G + b, ((unsigned long long)(p + 1) << 32) | wincl);
        }
      }
      __syncthreads();
      // the CTA-local result, in place in the stage (every thread has read it)
      const unsigned woff = s_warp[warp];
      if constexpr (SCAN) {
#pragma unroll
        for (int r = 0; r < kR; ++r) {
          const unsigned o0 = woff + pre[r], o1 = o0 + x[r][0], o2 = o1 + x[r][1], o3 = o2 + x[r][2];
          stage[wbase + r * 32 + lane] = make_uint4(o0, o1, o2, o3);
        }
      } else {
        O* packed = reinterpret_cast<O*>(stage);
#pragma unroll
        for (int r = 0; r < kR; ++r) {
          if (!bits[r]) continue;  // nothing selected in this uint4: the common case for a sparse rule
          unsigned o;
          if constexpr (LANE) {
            const unsigned jb = ((r + lane) & (kR - 1)) * E;  // first bit of this uint4 in the lane's mask
            o = woff + lane_pre + __popc(lm & ((1u << jb) - 1u));
          } else {
            o = woff + pre[r];
          }
#pragma unroll
          for (int q = 0; q < E; ++q)
            if (bits[r] & (1u << q)) packed[o++] = hxs::project<T, O>(x[r][q]);
        }
      }
    }
    // ---- pass 2: phase p - D ---------------------------------------------
    if (p >= (unsigned)kDefer) {
      const unsigned q = p - kDefer;
      const unsigned st = st2;
      // Every CTA's count of phase q: the sum over CTAs before this one, and
      // the total. A phase holds at most kMaxGrid slices of at most 2^14
      // elements, so both fit 32 bits (the scan's sums are taken mod 2^32).
      unsigned before = 0, total = 0;
      bool ok = true;
#pragma unroll
      for (int k = 0; k < kSlotLoads; ++k) {
        const unsigned c = threadIdx.x + k * kBlock;
        if (c >= G) break;
        const unsigned long long* slot = sc.slots + sl2 * G + c;
        unsigned long long v = pv[k];
        if ((unsigned)(v >> 32) != q + 1) {
          const unsigned long long t0 = globaltimer();
          unsigned i = 0;
          while ((unsigned)(v >> 32) != q + 1) {
            if ((++i & 63) == 0) {
              if (ld_relaxed_u32(sc.error) || globaltimer() - t0 > kWaitNs) {
                ok = false;
                break;
              }
              __nanosleep(64);
            }
            v = ld_relaxed(slot);
          }
          if (!ok) break;
        }
        const unsigned cnt = (unsigned)v;
        total += cnt;
        if (c < b) before += cnt;
      }
      // only the warps that read a slot reduce; the others hold zeros
      const unsigned nw = G >= (unsigned)kBlock ? (unsigned)WARPS : (G + 31) / 32;
      if ((unsigned)warp < nw) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          before += __shfl_xor_sync(0xffffffffu, before, o);
          total += __shfl_xor_sync(0xffffffffu, total, o);
        }
        if (lane == 0) s_red[warp] = make_uint2(before, total);
      }
      if (__syncthreads_or(!ok)) {
        failed = true;
        break;
      }
      before = 0;
      total = 0;
      for (unsigned w = 0; w < nw; ++w) {
        const uint2 r = s_red[w];
        before += r.x;
        total += r.y;
      }
      const unsigned long long prefix = base + before;
      const uint4* stage = s_stage + (size_t)st * SU4;
      const uint64_t t = (uint64_t)q * G + b;
      if constexpr (SCAN) {
        const uint64_t e0 = t * SE;
        const unsigned add = (unsigned)prefix;
        const bool whole = t < full_slices;
        uint32_t* o32 = reinterpret_cast<uint32_t*>(out);
        for (unsigned u = threadIdx.x; u < SU4; u += kBlock) {
          const uint4 v = stage[u];
          const uint4 w = make_uint4(v.x + add, v.y + add, v.z + add, v.w + add);
          const uint64_t e = e0 + (uint64_t)u * 4;
          if (whole) {
            __stcs(reinterpret_cast<uint4*>(o32 + e), w);
          } else {
            const unsigned a[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
            for (int k = 0; k < 4; ++k)
              if (e + k < n) o32[e + k] = a[k];
          }
        }
      } else {
        const O* packed = reinterpret_cast<const O*>(stage);
        const unsigned cnt = s_cnt[st];
        for (unsigned i = threadIdx.x; i < cnt; i += kBlock) {
          const unsigned long long dst = prefix + i;
          if (dst < capacity) out[dst] = packed[i];
        }
      }
      base += total;
      __syncthreads();  // stage st is written out
      if (threadIdx.x == 0 && q + kStages < phases) issue(st, q + kStages);
      next(st2, kStages);
      next(sl2, kSlots);
    }
    next(st1, kStages);
    next(sl1, kSlots);
  }
  if (failed) {
    if (threadIdx.x == 0) {
      atomicExch(sc.error, 1u);
      // no copy is issued after a failure: give each one still in flight a
      // bounded wait before the CTA exits
      for (int s = 0; s < kStages; ++s)
        if ((pend >> s) & 1u) mbar_wait(&s_bar[s], (par >> s) & 1u);
    }
    return;
  }
  if (b == 0 && threadIdx.x == 0) {
    if (done.d_count) *done.d_count = base < done.count_max ? base : done.count_max;
    if (done.sub_from) atomicAdd(done.sub_from, 0ull - base);
  }
}

// ---- host side -------------------------------------------------------------
inline size_t smem_bytes() { return (size_t)kStages * kSliceBytes; }

// Co-resident CTAs of one kernel on the current device (SMs x CTAs per SM,
// at most kMaxGrid), with the kernel's shared-memory limit raised first.
// The limit is raised on every call (cheap, and it survives a device reset
// that would drop it); the occupancy query runs once per kernel and device.
// The cache is keyed by the kernel's host-side address, not by its template
// arguments alone: a kernel template instantiated in several translation
// units (libhx's, a caller's, the no-allocation scan's) is a separate
// function in each, while a static of an inline function is one object
// shared by all of them.
template <class Kern>
inline cudaError_t resident_grid(Kern kern, unsigned* grid) {
  const size_t smem = smem_bytes();
  cudaError_t e = cudaSuccess;
  if (smem > 48 * 1024) {
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  int dev = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, unsigned> cache;
  const auto key = std::make_pair(reinterpret_cast<const void*>(kern), dev);
  {
    std::lock_guard<std::mutex> g(mu);
    const auto it = cache.find(key);
    if (it != cache.end()) {
      *grid = it->second;
      return cudaSuccess;
    }
  }
  int per_sm = 0, sms = 0;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBlock, smem)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  long g = (long)per_sm * sms;
  if (g < 1) return cudaErrorInvalidConfiguration;
  if (g > kMaxGrid) g = kMaxGrid;
  {
    std::lock_guard<std::mutex> lk(mu);
    cache[key] = (unsigned)g;
  }
  *grid = (unsigned)g;
  return cudaSuccess;
}

// Launches one pass over n > 0 elements of a 16-byte-aligned `in` (and, for
// the scan, a 16-byte-aligned `out`). scratch: scratch_need(n, sizeof(T))
// bytes of device memory; the part this launch uses is zeroed here, on the
// stream. With done.n_from, n is an upper bound of the device-side count.
template <class T, class O, class Sel, bool SCAN>
inline cudaError_t launch(const T* in, O* out, uint64_t n, const Sel& sel, uint64_t capacity, Done done,
                          void* scratch, cudaStream_t s) {
  auto kern = k_stream<T, O, Sel, SCAN>;
  unsigned grid = 0;
  cudaError_t e = resident_grid(kern, &grid);
  if (e != cudaSuccess) return e;
  constexpr uint64_t SE = (uint64_t)kBlock * kR * (16 / sizeof(T));
  const uint64_t slices = (n + SE - 1) / SE;
  if (slices < grid) grid = (unsigned)slices;
  if (slices / grid >= 0xffff0000ull) return cudaErrorInvalidValue;  // phases are counted in 32 bits
  e = cudaMemsetAsync(scratch, 0, scratch_bytes_used(grid), s);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kBlock);
  cfg.dynamicSmemBytes = smem_bytes();
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, in, out, n, sel, capacity, done, carve(scratch));
}

}  // namespace hxs
