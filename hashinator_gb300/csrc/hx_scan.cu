// hx_scan.cu — split::tools replacements (exclusive scan, copy_if) and the
// host helpers shared by libhx.
#include <cstring>
#include <mutex>
#include "hx_host.h"
#include "hx_scan.cuh"

namespace hx {

static thread_local int t_last_cuda_error = 0;
static std::atomic<uint64_t> g_launches{0};

hx_status cuda_status(cudaError_t e) {
  t_last_cuda_error = (int)e;
  if (e == cudaErrorMemoryAllocation) return HX_ERR_OOM;
  return HX_ERR_CUDA;
}

hx_status after_launch() {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status(e);
  return HX_OK;
}

int sm_count() {
  static std::mutex mu;
  static int cache[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
  std::lock_guard<std::mutex> g(mu);
  if (cache[dev] == 0) {
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    cache[dev] = n > 0 ? n : 1;
  }
  return cache[dev];
}

hx_status Scratch::get(void* caller, uint64_t caller_bytes, uint64_t need, cudaStream_t stream) {
  s = stream;
  if (caller) {
    if (caller_bytes < need) return HX_ERR_INVALID_ARG;
    ptr = caller;
    owned = false;
    return HX_OK;
  }
  HX_CUDA(cudaMallocAsync(&ptr, need, stream));
  owned = true;
  return HX_OK;
}

Scratch::~Scratch() {
  if (owned && ptr) cudaFreeAsync(ptr, s);
}

// Reads the count and error word back for a synchronous call.
static hx_status finish_sync(cudaStream_t s, const unsigned long long* d_count, uint64_t* h_count,
                             const unsigned int* d_error, uint64_t capacity) {
  unsigned long long cnt = 0;
  unsigned int err = 0;
  HX_CUDA(cudaMemcpyAsync(&cnt, d_count, sizeof(cnt), cudaMemcpyDeviceToHost, s));
  HX_CUDA(cudaMemcpyAsync(&err, d_error, sizeof(err), cudaMemcpyDeviceToHost, s));
  HX_CUDA(cudaStreamSynchronize(s));
  *h_count = cnt;
  if (err) return HX_ERR_TIMEOUT;
  if (cnt > capacity) return HX_ERR_CAPACITY;
  return HX_OK;
}

// Scratch needed by a compaction over n elements of T, plus 256 B at its end
// for a device count word when the caller gives none.
template <class T>
static uint64_t compact_scratch_bytes(uint64_t n) {
  return (compact_scratch_need<T>(n) + 255) / 256 * 256 + 256;
}

template <class T>
static hx_status copy_if_t(const void* d_in, void* d_out, uint64_t n, const hx_pred& pr, uint64_t capacity,
                           uint64_t* d_count, uint64_t* h_count, void* d_scratch, uint64_t scratch_bytes,
                           cudaStream_t s) {
  const uint64_t need = compact_scratch_bytes<T>(n);
  Scratch sc;
  hx_status st = sc.get(d_scratch, scratch_bytes, need, s);
  if (st != HX_OK) return st;
  unsigned long long* cnt = d_count ? reinterpret_cast<unsigned long long*>(d_count)
                                    : reinterpret_cast<unsigned long long*>(static_cast<char*>(sc.ptr) + need - 256);
  bool sk = false;
  if (n == 0) {
    HX_CUDA(cudaMemsetAsync(cnt, 0, sizeof(*cnt), s));
    HX_CUDA(cudaMemsetAsync(sc.ptr, 0, 256, s));
  } else {
    typename ElemOps<T>::Ctx ctx{};
    cudaError_t e = launch_compact<T, false>(static_cast<const T*>(d_in), static_cast<T*>(d_out), n, pr, ctx,
                                             capacity, cnt, sc.ptr, CleanArgs{nullptr, nullptr}, s, &sk);
    if (e != cudaSuccess) return cuda_status(e);
    st = after_launch();
    if (st != HX_OK) return st;
  }
  if (h_count) return finish_sync(s, cnt, h_count, scan_error_word(sc.ptr, sk), capacity);
  return HX_OK;
}

// Random 32-byte sector reads over a buffer of 2^k sectors: the random-access
// ceiling of the memory system, against which the probe kernels (one random
// sector per key at least) are measured. U independent reads per thread.
__device__ __forceinline__ uint64_t diag_mix(uint64_t i) {
  uint64_t x = i * 0x9E3779B97F4A7C15ull;
  x ^= x >> 29;
  x *= 0xBF58476D1CE4E5B9ull;
  x ^= x >> 32;
  return x;
}
template <int U>
__global__ void __launch_bounds__(256) k_diag_random_sectors(const unsigned char* __restrict__ buf,
                                                             uint64_t sect_mask, uint64_t n,
                                                             unsigned long long* sink) {
  unsigned long long acc = 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t groups = (n + U - 1) / U;
  for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < groups; g += stride) {
    unsigned long long a[U], b[U], c[U], d[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint64_t sct = diag_mix(g * U + u) & sect_mask;
      asm volatile("ld.global.cg.v4.u64 {%0,%1,%2,%3}, [%4];"
                   : "=l"(a[u]), "=l"(b[u]), "=l"(c[u]), "=l"(d[u])
                   : "l"(buf + sct * 32));
    }
#pragma unroll
    for (int u = 0; u < U; ++u) acc += a[u] ^ b[u] ^ c[u] ^ d[u];
  }
  if (acc == 0x9E3779B97F4A7C15ull) *sink = acc;  // keeps the loads alive
}
// Random 64-bit CAS on word 0 of random 32-byte sectors: the ceiling of the
// insert kernels, which publish each new pair with one CAS.
__global__ void __launch_bounds__(256) k_diag_random_cas(unsigned long long* __restrict__ buf, uint64_t sect_mask,
                                                         uint64_t n, unsigned long long* sink) {
  unsigned long long acc = 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride)
    acc += atomicCAS(buf + (diag_mix(i) & sect_mask) * 4, 0ull, (unsigned long long)i + 1);
  if (acc == 0x9E3779B97F4A7C15ull) *sink = acc;
}

}  // namespace hx

using namespace hx;

extern "C" {

const char* hx_status_string(hx_status st) {
  switch (st) {
    case HX_OK: return "ok";
    case HX_ERR_OVERFLOW: return "table overflow: not every key found a bucket";
    case HX_ERR_OOM: return "device allocation failed";
    case HX_ERR_INVALID_ARG: return "invalid argument";
    case HX_ERR_CUDA: return "CUDA runtime error";
    case HX_ERR_TIMEOUT: return "a bounded device-side wait ran out";
    case HX_ERR_CAPACITY: return "output buffer smaller than the result count";
  }
  return "unknown status";
}

int hx_last_cuda_error(void) { return t_last_cuda_error; }

uint64_t hx_kernel_launch_count(void) { return g_launches.load(); }

hx_status hx_diag_random_access(void* d_buf, uint64_t bytes, uint64_t n_ops, int mode, hx_stream stream) {
  if (!d_buf || ((uintptr_t)d_buf % 32) || bytes < 64 || (mode != 0 && mode != 1)) return HX_ERR_INVALID_ARG;
  uint64_t nsect = 1;
  while (nsect * 2 <= bytes / 32) nsect *= 2;  // largest power of two that fits
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // The sink is never written unless an accumulated 64-bit sum hits a fixed
  // constant; it points at the buffer's first word.
  unsigned long long* sink = static_cast<unsigned long long*>(d_buf);
  if (mode == 0) {
    auto kern = k_diag_random_sectors<4>;
    const unsigned grid = (unsigned)(sm_count() * blocks_per_sm(kern, 256));
    kern<<<grid, 256, 0, s>>>(static_cast<const unsigned char*>(d_buf), nsect - 1, n_ops, sink);
  } else {
    const unsigned grid = (unsigned)(sm_count() * blocks_per_sm(k_diag_random_cas, 256));
    k_diag_random_cas<<<grid, 256, 0, s>>>(static_cast<unsigned long long*>(d_buf), nsect - 1, n_ops, sink);
  }
  return after_launch();
}

hx_status hx_scratch_bytes(int op, uint64_t n, uint64_t* bytes) {
  if (!bytes) return HX_ERR_INVALID_ARG;
  if (op == HX_SCRATCH_SCAN) {
    *bytes = scan_scratch_need(n);
  } else if (op == HX_SCRATCH_COPY_IF) {
    // the largest of the three element widths' needs
    uint64_t a = compact_scratch_bytes<uint32_t>(n), b = compact_scratch_bytes<P32>(n),
             c = compact_scratch_bytes<P64>(n);
    *bytes = a > b ? (a > c ? a : c) : (b > c ? b : c);
  } else {
    return HX_ERR_INVALID_ARG;
  }
  return HX_OK;
}

hx_status hx_exclusive_scan_u32(const uint32_t* d_in, uint32_t* d_out, uint64_t n, void* d_scratch,
                                uint64_t scratch_bytes, hx_stream stream) {
  HX_RANGE("hx_exclusive_scan_u32");
  if (n == 0) return HX_OK;
  if (!d_in || !d_out) return HX_ERR_INVALID_ARG;
  if (misaligned(d_in, 4) || misaligned(d_out, 4)) return HX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const uint64_t tiles = scan_tiles(n);
  if (tiles > 0xFFFFFFFFull) return HX_ERR_INVALID_ARG;
  Scratch sc;
  hx_status st = sc.get(d_scratch, scratch_bytes, scan_scratch_need(n), s);
  if (st != HX_OK) return st;
  HX_CUDA(launch_scan(d_in, d_out, n, sc.ptr, s));
  return after_launch();
}

hx_status hx_copy_if(const void* d_in, void* d_out, uint64_t n, int elem_bytes, const hx_pred* pred,
                     uint64_t capacity, uint64_t* d_count, uint64_t* h_count, void* d_scratch,
                     uint64_t scratch_bytes, hx_stream stream) {
  HX_RANGE("hx_copy_if");
  if (!pred || (n && (!d_in || !d_out))) return HX_ERR_INVALID_ARG;
  if (pred->op == HX_PRED_MOD_LT && pred->a == 0) return HX_ERR_INVALID_ARG;
  if (pred->op > HX_PRED_NOT_HOME) return HX_ERR_INVALID_ARG;
  if (pred->op == HX_PRED_NOT_HOME) return HX_ERR_INVALID_ARG;  // needs a map: hx_extract_pattern
  if ((elem_bytes == 4 || elem_bytes == 8 || elem_bytes == 16) &&
      (misaligned(d_in, (unsigned)elem_bytes) || misaligned(d_out, (unsigned)elem_bytes)))
    return HX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  switch (elem_bytes) {
    case 4:
      if (pred->op == HX_PRED_VALID) return HX_ERR_INVALID_ARG;
      return copy_if_t<uint32_t>(d_in, d_out, n, *pred, capacity, d_count, h_count, d_scratch, scratch_bytes, s);
    case 8:
      return copy_if_t<P32>(d_in, d_out, n, *pred, capacity, d_count, h_count, d_scratch, scratch_bytes, s);
    case 16:
      return copy_if_t<P64>(d_in, d_out, n, *pred, capacity, d_count, h_count, d_scratch, scratch_bytes, s);
    default:
      return HX_ERR_INVALID_ARG;
  }
}

}  // extern "C"
