// hx_noalloc.cu — an exclusive u32 scan that allocates no device memory.
//
// Some callers cannot allocate at the point where they need a scan: code that
// runs inside a host framework which owns all device memory and hands out
// none per call (a plugin's execute step, a serving loop with a fixed memory
// budget), or a tight time-stepping loop where cudaMalloc/cudaFree would
// synchronise the device. hx_exclusive_scan_u32 needs a few hundred KiB of
// look-back scratch and either takes it from the caller or allocates it; this
// entry point takes it from a fixed array compiled into the library instead.
//
// The array lives in device global memory for every GPU that loads libhx,
// from module load until the process exits. All calls share it, so calls
// that overlap on the GPU corrupt each other's results: order them on one
// stream (or otherwise serialise them).
#include <mutex>

#include "hx_host.h"
#include "hx_scan.cuh"

namespace hx {

constexpr uint64_t kNoAllocTileElems = (uint64_t)kScanBlock * kScanTmaR * 4;  // the smaller scan tiles
constexpr uint64_t kNoAllocTiles = (HX_NOALLOC_SCAN_MAX_N + kNoAllocTileElems - 1) / kNoAllocTileElems;
static_assert(256 + 8 * kNoAllocTiles <= HX_NOALLOC_SCAN_SCRATCH_BYTES, "ticket/error words + tile statuses fit");

// Look-back scratch of the no-allocation scan: 256 B of ticket and error
// words, then one 8-byte status word per tile of 4096 elements (524,544 B for
// the largest scan, 2^28 elements).
static __device__ __align__(256) unsigned char g_noalloc_scan_scratch[HX_NOALLOC_SCAN_SCRATCH_BYTES];

// Device address of the array, looked up once per device with that device
// current. In host code the array's name is only a host-side stand-in, so the
// address must come from cudaGetSymbolAddress.
static void* noalloc_scratch(int dev, cudaError_t* err) {
  static std::mutex mu;
  static void* addr[64] = {nullptr};
  *err = cudaSuccess;
  if (dev < 0 || dev >= 64) {
    *err = cudaErrorInvalidDevice;
    return nullptr;
  }
  std::lock_guard<std::mutex> g(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    *err = cudaGetSymbolAddress(&p, g_noalloc_scan_scratch);
    if (*err != cudaSuccess) return nullptr;
    addr[dev] = p;
  }
  return addr[dev];
}

}  // namespace hx

using namespace hx;

extern "C" hx_status hx_exclusive_scan_u32_noalloc(const uint32_t* d_in, uint32_t* d_out, uint64_t n,
                                                   hx_stream stream) {
  HX_RANGE("hx_exclusive_scan_u32_noalloc");
  if (n == 0) return HX_OK;
  if (!d_in || !d_out) return HX_ERR_INVALID_ARG;
  if (n > HX_NOALLOC_SCAN_MAX_N) return HX_ERR_INVALID_ARG;  // beyond the fixed scratch: nothing launched
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int dev = 0;
  HX_CUDA(cudaGetDevice(&dev));
  cudaError_t e;
  void* sc = noalloc_scratch(dev, &e);
  if (!sc) return cuda_status(e);
  const uint64_t tiles = scan_tiles(n);
  // The previous call left its tickets and statuses behind: reset the part used.
  HX_CUDA(cudaMemsetAsync(sc, 0, scan_scratch_bytes(tiles), s));
  HX_CUDA(launch_scan(d_in, d_out, n, sc, s));
  return after_launch();
}
