// hx_host.h — host-side helpers shared by the libhx translation units.
#pragma once
#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>
#include "../../include/hx.h"

// NVTX ranges name each C-ABI call in Nsight Systems timelines and for
// `ncu --nvtx` filters. NVTX v3 is header-only; with no tool attached a range
// costs one call that returns at once. Build with -DHX_NVTX=0 to compile
// them out.
#ifndef HX_NVTX
#define HX_NVTX 1
#endif
#if HX_NVTX
#include <nvtx3/nvToolsExt.h>
#endif

namespace hx {

#if HX_NVTX
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};
#define HX_RANGE(name) ::hx::NvtxRange hx_nvtx_range_(name)
#else
#define HX_RANGE(name) ((void)0)
#endif

// Records the CUDA error for hx_last_cuda_error() and maps it to a status.
hx_status cuda_status(cudaError_t e);
#define HX_CUDA(call)                                   \
  do {                                                  \
    cudaError_t hx_e_ = (call);                         \
    if (hx_e_ != cudaSuccess) return ::hx::cuda_status(hx_e_); \
  } while (0)
// Checks the launch that was just issued and counts it.
hx_status after_launch();

int sm_count();  // SMs of the current device (cached per device)

// A device array of elements of `align` bytes must start at a multiple of
// `align`: the kernels load and store whole elements (and pairs as one 8- or
// 16-byte access), so a misaligned pointer is rejected before any launch.
inline bool misaligned(const void* p, unsigned align) {
  return (reinterpret_cast<uintptr_t>(p) % align) != 0;
}

// Blocks per SM for a kernel at a block size (cached by the caller).
template <class F>
int blocks_per_sm(F kernel, int block, size_t smem = 0) {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, block, smem) != cudaSuccess || nb < 1) nb = 1;
  return nb;
}

// Stream-ordered scratch: a caller buffer when given, else cudaMallocAsync
// on the stream, released stream-ordered by the destructor.
struct Scratch {
  void* ptr = nullptr;
  bool owned = false;
  cudaStream_t s = nullptr;
  hx_status get(void* caller, uint64_t caller_bytes, uint64_t need, cudaStream_t stream);
  ~Scratch();
};

}  // namespace hx
