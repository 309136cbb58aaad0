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
#include <cuda.h>

#include <mutex>

#include "hx_host.h"
#include "hx_scan.cuh"

namespace hx {

// Both scan kernels fit the array at the largest n: the register-staged one
// (one status word per tile of 12288 elements) and the phase-partitioned one
// (count slots for its largest grid).
constexpr uint64_t kNoAllocTileElems = (uint64_t)kScanBlock * kScanR * 4;
constexpr uint64_t kNoAllocTiles = (HX_NOALLOC_SCAN_MAX_N + kNoAllocTileElems - 1) / kNoAllocTileElems;
static_assert(256 + 8 * kNoAllocTiles <= HX_NOALLOC_SCAN_SCRATCH_BYTES, "ticket/error words + tile statuses fit");
static_assert(hxs::kScratchBytes <= HX_NOALLOC_SCAN_SCRATCH_BYTES, "error word + count slots fit");

// Scratch of the no-allocation scan, HX_NOALLOC_SCAN_SCRATCH_BYTES
// (524,544 B): room for either scan kernel's words at n = 2^28.
static __device__ __align__(256) unsigned char g_noalloc_scan_scratch[HX_NOALLOC_SCAN_SCRATCH_BYTES];

// The current context's driver-assigned id (unique for the life of the
// process), through the runtime's driver entry points so that libhx does not
// link libcuda. 0 when the driver does not provide it.
static unsigned long long current_context_id() {
  using GetCurrent = CUresult (*)(CUcontext*);
  using GetId = CUresult (*)(CUcontext, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void* f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(f);
  });
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS)
    return 0;
  return id;
}

// Device address of the array in the current device's context. In host code
// the array's name is only a host-side stand-in, so the address comes from
// cudaGetSymbolAddress, called with the device current. It is looked up once
// per device and context: a cudaDeviceReset ends the context, the module is
// loaded again in the next one and the array may then sit elsewhere, so an
// address is reused only while the context that it was looked up in is the
// current one (when the driver cannot name contexts, it is looked up on
// every call).
static void* noalloc_scratch(int dev, cudaError_t* err) {
  static std::mutex mu;
  static void* addr[64] = {nullptr};
  static unsigned long long ctx_of[64] = {0};
  *err = cudaSuccess;
  if (dev < 0 || dev >= 64) {
    *err = cudaErrorInvalidDevice;
    return nullptr;
  }
  // Make the device's primary context current (cudaSetDevice initialises it),
  // so that the id below names the context the kernel will run in.
  if ((*err = cudaSetDevice(dev)) != cudaSuccess) return nullptr;
  const unsigned long long ctx = current_context_id();
  std::lock_guard<std::mutex> g(mu);
  if (!addr[dev] || ctx == 0 || ctx_of[dev] != ctx) {
    void* p = nullptr;
    *err = cudaGetSymbolAddress(&p, g_noalloc_scan_scratch);
    if (*err != cudaSuccess) return nullptr;
    addr[dev] = p;
    ctx_of[dev] = ctx;
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
  if (misaligned(d_in, 4) || misaligned(d_out, 4)) return HX_ERR_INVALID_ARG;
  if (n > HX_NOALLOC_SCAN_MAX_N) return HX_ERR_INVALID_ARG;  // beyond the fixed scratch: nothing launched
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int dev = 0;
  HX_CUDA(cudaGetDevice(&dev));
  cudaError_t e;
  void* sc = noalloc_scratch(dev, &e);
  if (!sc) return cuda_status(e);
  // The previous call left its words behind: launch_scan resets the part it uses.
  HX_CUDA(launch_scan(d_in, d_out, n, sc, s));
  return after_launch();
}
