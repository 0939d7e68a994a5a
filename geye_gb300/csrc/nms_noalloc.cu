// nms_noalloc.cu -- greedy NMS on caller-owned device buffers, allocating nothing.
//
// Some callers cannot call cudaMalloc: their device memory belongs to another
// allocator (a framework's caching pool, or a fixed per-process budget that
// must not grow), or they run a real-time loop where cudaMalloc/cudaFree's
// latency and implicit device synchronisation are not acceptable.  This entry
// point gives them the library's NMS (the same kernel as geye_nms, exact
// reference tie order and kept set) with its working memory in a file-scope
// __device__ array instead of an allocation.
//
// The array holds scratch for up to GEYE_NMS_NOALLOC_MAX_BOXES boxes (about
// 2.8 MB).  Every GPU that loads the library holds it until the process exits.
// All calls share it and it keeps the last call's contents; the kernel writes
// every scratch word it reads, and the two counters that must start at zero are
// cleared at the start of each call.  Calls that overlap on the GPU (two
// streams, or two host threads at once) race on the array.
//
// Host code cannot use the array's name as a device address (there it names a
// host-side stand-in), so the first call on each device, with that device
// current, looks the address up with cudaGetSymbolAddress and caches it; make
// that first call before any stream capture.  The cache is keyed on the
// current CUDA context's unique id (cuCtxGetId), not on the device ordinal: a
// context created after cudaDeviceReset, or a caller's own non-primary context
// on the same device, has its own copy of the array at its own address, and
// its first call looks that address up again.
#include <cuda.h>

#include <map>
#include <mutex>
#include <string>

#include "runtime.h"

namespace {

constexpr int kMaxBoxes = GEYE_NMS_NOALLOC_MAX_BOXES;            // a multiple of 32
constexpr size_t kScratchF = (size_t)kMaxBoxes * 6;              // sort keys + sorted boxes/areas
constexpr size_t kScratchI = (size_t)kMaxBoxes * 5 + 64;         // order, ranks, flags, segment queue
constexpr size_t kCounters = 64;                                 // [0] box count, [1] error flags
static_assert(kMaxBoxes % 32 == 0, "capacity must keep the int2 queue aligned");

static __device__ __align__(256) float g_nms_noalloc_scratch[kScratchF + kScratchI + kCounters];

__global__ void k_noalloc_begin(int *counters, int num) {
  counters[0] = num;
  counters[1] = 0;
}

__global__ void k_noalloc_end(const int *counters, int *d_kept) {
  if (counters[1] != 0) *d_kept = -1;
}

std::mutex g_mu;
std::map<unsigned long long, float *> g_base;   // context id -> the array's device address there

// the current context's unique id (making the device's primary context current
// through the runtime when the thread has none yet).  The two driver calls are
// looked up through the runtime, so the library keeps no link-time dependency
// on the driver library (it loads on machines without a GPU driver).
using CtxGetCurrentFn = CUresult (*)(CUcontext *);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long *);
geye_status current_context_id(unsigned long long *id) {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  if (!get_current || !get_id) {
    void *f1 = nullptr, *f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    // the driver ABI of CUDA 12.0, where cuCtxGetId first appeared
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
        q2 != cudaDriverEntryPointSuccess)
      return GEYE_ERR_CUDA;
    get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
    get_id = reinterpret_cast<CtxGetIdFn>(f2);
  }
  CUcontext cur = nullptr;
  if (get_current(&cur) != CUDA_SUCCESS) return GEYE_ERR_CUDA;
  if (!cur) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_nms_noalloc_scratch) != cudaSuccess) return GEYE_ERR_CUDA;
    if (get_current(&cur) != CUDA_SUCCESS || !cur) return GEYE_ERR_CUDA;
  }
  return get_id(cur, id) == CUDA_SUCCESS ? GEYE_OK : GEYE_ERR_CUDA;
}

}  // namespace

extern "C" geye_status geye_nms_noalloc(const float *d_boxes, int num, int numpart0, float overlap, float *d_out,
                                        int *d_kept, void *cuda_stream) {
  if (num < 0 || numpart0 < 0 || numpart0 > geye::kMaxParts || !d_kept || (num > 0 && (!d_boxes || !d_out))) {
    geye::set_error("geye_nms_noalloc: bad argument");
    return GEYE_ERR_ARG;
  }
  if (num > kMaxBoxes) {
    geye::set_error("geye_nms_noalloc: " + std::to_string(num) + " boxes exceed the fixed scratch capacity of " +
                    std::to_string(kMaxBoxes));
    return GEYE_ERR_ARG;
  }
  unsigned long long ctx_id = 0;
  std::lock_guard<std::mutex> lock(g_mu);
  if (current_context_id(&ctx_id) != GEYE_OK) {
    geye::set_error("geye_nms_noalloc: no usable CUDA context on the current device");
    return GEYE_ERR_CUDA;
  }
  cudaError_t e = cudaSuccess;
  float *base = nullptr;
  {
    auto it = g_base.find(ctx_id);
    if (it == g_base.end()) {
      void *p = nullptr;
      e = cudaGetSymbolAddress(&p, g_nms_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        geye::set_error(std::string("geye_nms_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        return GEYE_ERR_CUDA;
      }
      it = g_base.emplace(ctx_id, static_cast<float *>(p)).first;
    }
    base = it->second;
  }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(cuda_stream);
  float *scratch_f = base;
  int *scratch_i = reinterpret_cast<int *>(base + kScratchF);
  int *counters = reinterpret_cast<int *>(base + kScratchF + kScratchI);
  const int GL = (numpart0 + 1) * 4 + 3;
  const int cap = num > 0 ? (num + 31) & ~31 : 32;
  k_noalloc_begin<<<1, 1, 0, s>>>(counters, num);
  geye::launch_nms(d_boxes, counters, 1, GL, overlap, cap, scratch_f, scratch_i, d_out, d_kept, counters + 1, s);
  k_noalloc_end<<<1, 1, 0, s>>>(counters, d_kept);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    geye::set_error(std::string("geye_nms_noalloc: launch: ") + cudaGetErrorString(e));
    return GEYE_ERR_CUDA;
  }
  return GEYE_OK;
}
