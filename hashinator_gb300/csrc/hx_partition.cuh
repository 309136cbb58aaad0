// hx_partition.cuh — reorders an insert batch by table region before it is
// inserted, so that the insert's random bucket updates fall into a few
// L2-resident regions at a time instead of the whole table.
//
// A region is a 2^rbits-th of the table: the keys whose home bucket shares
// its top rbits bits. Three launches:
//   k_region_hist   one pass over the keys: the number of keys per region
//                   (shared-memory histogram per CTA, added into global counts);
//   k_region_scan   one CTA: exclusive offsets of the regions (their cursors);
//   k_region_scatter  chunks of kChunk keys per CTA: rank each key within its
//                   region in shared memory, reserve the chunk's run in every
//                   region with one atomic per region, stage the chunk in
//                   shared memory in region order and write it out, so that
//                   consecutive threads write consecutive addresses.
// The permuted batch holds the same (key, value) pairs; inserting it gives the
// same mapping (for distinct keys the set of placements does not depend on the
// order; a key repeated in one batch keeps one of its values, which was
// already unspecified). The order inside a region is not kept.
#pragma once
#include "hx_device.cuh"

namespace hx {

constexpr int kPartBlock = 512;
constexpr int kPartChunk = 4096;      // keys per CTA per step of the scatter
constexpr int kPartMaxRegions = 2048;

// Region of a key in a table of 2^sp buckets split into 2^rbits regions.
template <class P>
__device__ __forceinline__ uint32_t region_of(typename PairTraits<P>::K key, int sp, int rbits) {
  return rbits ? (uint32_t)(home_slot(key, sp) >> (sp - rbits)) : 0u;
}

template <class P, bool PAIRS>
__global__ void __launch_bounds__(kPartBlock) k_region_hist(const typename PairTraits<P>::K* __restrict__ keys,
                                                            const P* __restrict__ pairs, uint64_t n, int sp,
                                                            int rbits, unsigned* __restrict__ counts) {
  __shared__ unsigned h[kPartMaxRegions];
  const int R = 1 << rbits;
  for (int i = threadIdx.x; i < R; i += blockDim.x) h[i] = 0;
  __syncthreads();
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    const auto k = PAIRS ? pairs[i].first : keys[i];
    atomicAdd(&h[region_of<P>(k, sp, rbits)], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < R; i += blockDim.x)
    if (h[i]) atomicAdd(&counts[i], h[i]);
}

// One CTA of kPartBlock threads: cursor[r] = counts[0] + ... + counts[r-1].
__global__ void __launch_bounds__(kPartBlock) k_region_scan(const unsigned* __restrict__ counts,
                                                            unsigned long long* __restrict__ cursor, int rbits) {
  __shared__ unsigned long long s_part[kPartBlock];
  const int R = 1 << rbits;
  constexpr int PER = kPartMaxRegions / kPartBlock;  // regions per thread
  unsigned long long v[PER], sum = 0;
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const int r = threadIdx.x * PER + j;
    v[j] = r < R ? counts[r] : 0ull;
    sum += v[j];
  }
  s_part[threadIdx.x] = sum;
  __syncthreads();
  for (int o = 1; o < kPartBlock; o <<= 1) {  // inclusive scan of the per-thread sums
    const unsigned long long add = threadIdx.x >= o ? s_part[threadIdx.x - o] : 0ull;
    __syncthreads();
    s_part[threadIdx.x] += add;
    __syncthreads();
  }
  unsigned long long run = s_part[threadIdx.x] - sum;
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const int r = threadIdx.x * PER + j;
    if (r < R) cursor[r] = run;
    run += v[j];
  }
}

// Scatter of keys and values (or pairs) into region order. vals == nullptr:
// the value of keys[i] is i (insertIndex).
template <class P, bool PAIRS>
__global__ void __launch_bounds__(kPartBlock) k_region_scatter(
    const typename PairTraits<P>::K* __restrict__ keys, const typename PairTraits<P>::V* __restrict__ vals,
    const P* __restrict__ pairs, uint64_t n, int sp, int rbits, unsigned long long* __restrict__ cursor,
    typename PairTraits<P>::K* __restrict__ out_keys, typename PairTraits<P>::V* __restrict__ out_vals,
    P* __restrict__ out_pairs) {
  using K = typename PairTraits<P>::K;
  using V = typename PairTraits<P>::V;
  constexpr int PER = kPartChunk / kPartBlock;
  // dynamic shared memory (part_scatter_smem<P>()): the chunk's run in each
  // region, the chunk's keys per region (then each region's start in the
  // staged chunk), and the staged keys, values and regions
  extern __shared__ __align__(16) unsigned char s_raw[];
  unsigned long long* s_base = reinterpret_cast<unsigned long long*>(s_raw);
  K* s_k = reinterpret_cast<K*>(s_base + kPartMaxRegions);
  V* s_v = reinterpret_cast<V*>(s_k + kPartChunk);
  unsigned* s_cnt = reinterpret_cast<unsigned*>(s_v + kPartChunk);
  unsigned short* s_reg = reinterpret_cast<unsigned short*>(s_cnt + kPartMaxRegions);
  const int R = 1 << rbits;
  for (uint64_t c0 = (uint64_t)blockIdx.x * kPartChunk; c0 < n; c0 += (uint64_t)gridDim.x * kPartChunk) {
    for (int i = threadIdx.x; i < R; i += blockDim.x) s_cnt[i] = 0;
    __syncthreads();
    K k[PER];
    V v[PER];
    uint32_t reg[PER], rank[PER];
#pragma unroll
    for (int j = 0; j < PER; ++j) {
      const uint64_t i = c0 + (uint64_t)j * kPartBlock + threadIdx.x;
      if (i < n) {
        if constexpr (PAIRS) {
          const P p = pairs[i];
          k[j] = p.first;
          v[j] = p.second;
        } else {
          k[j] = keys[i];
          v[j] = vals ? vals[i] : (V)i;
        }
        reg[j] = region_of<P>(k[j], sp, rbits);
        rank[j] = atomicAdd(&s_cnt[reg[j]], 1u);
      }
    }
    __syncthreads();
    // reserve each region's run, and turn the counts into the chunk-local starts
    for (int r = threadIdx.x; r < R; r += blockDim.x) {
      const unsigned c = s_cnt[r];
      s_base[r] = c ? atomicAdd(&cursor[r], (unsigned long long)c) : 0ull;
    }
    __syncthreads();
    if (threadIdx.x < 32) {  // exclusive scan of s_cnt by warp 0
      const int lane = threadIdx.x;
      unsigned carry = 0;
      for (int r0 = 0; r0 < R; r0 += 32) {
        const unsigned c = r0 + lane < R ? s_cnt[r0 + lane] : 0u;
        unsigned x = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
          if (lane >= o) x += y;
        }
        if (r0 + lane < R) s_cnt[r0 + lane] = carry + x - c;
        carry += __shfl_sync(0xffffffffu, x, 31);
      }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < PER; ++j) {
      const uint64_t i = c0 + (uint64_t)j * kPartBlock + threadIdx.x;
      if (i < n) {
        const unsigned slot = s_cnt[reg[j]] + rank[j];
        s_k[slot] = k[j];
        s_v[slot] = v[j];
        s_reg[slot] = (unsigned short)reg[j];
      }
    }
    __syncthreads();
    const uint64_t m = n - c0 < (uint64_t)kPartChunk ? n - c0 : (uint64_t)kPartChunk;
    for (unsigned s = threadIdx.x; s < m; s += blockDim.x) {
      const unsigned r = s_reg[s];
      const unsigned long long d = s_base[r] + (s - s_cnt[r]);
      if constexpr (PAIRS) {
        P p;
        p.first = s_k[s];
        p.second = s_v[s];
        out_pairs[d] = p;
      } else {
        out_keys[d] = s_k[s];
        out_vals[d] = s_v[s];
      }
    }
    __syncthreads();
  }
}

template <class P>
constexpr size_t part_scatter_smem() {
  using K = typename PairTraits<P>::K;
  using V = typename PairTraits<P>::V;
  return kPartMaxRegions * (sizeof(unsigned long long) + sizeof(unsigned)) + kPartChunk * (sizeof(K) + sizeof(V)) +
         kPartChunk * sizeof(unsigned short);
}

}  // namespace hx
