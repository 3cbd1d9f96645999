// vl1_eval_mixed_noalloc: the tensor-core list-1 evaluation for callers that
// cannot allocate device memory.
//
// vl1_eval_mixed needs a per-call scratch area (density digits, scale
// exponents, displacement sums) that its caller allocates.  Some callers have
// no way to do that: host codes that own every byte of device memory through
// their own pool and hand a solver plugin only the arrays it computes on, and
// latency-critical loops where a cudaMalloc (which may synchronise the whole
// device, or fail when memory is fragmented) is not acceptable between steps.
// This entry point takes the same inputs and outputs but uses a fixed scratch
// array compiled into this library instead of caller-provided workspace; it
// calls no cudaMalloc, cudaFree or other allocating routine.
//
// The array is a file-scope __device__ object of VL1_NOALLOC_SCRATCH_BYTES
// bytes: every GPU on which the library's module is loaded holds it until the
// process exits.  Its device address is looked up on the first call made on a
// device (with that device current), and again whenever the CUDA context
// current on that device has changed since (a context the caller created
// with the driver API, or the primary context re-created after
// cudaDeviceReset): the address belongs to the context in which it was looked
// up.  A first call in a context should therefore come before any stream
// capture.  All calls share the one array: calls whose work overlaps on the
// GPU (different streams, or different host threads) race on it and must be
// serialised by the caller.  Each call re-initialises every scratch value it
// reads.
#include <cuda.h>

#include <mutex>

#include "vl1_internal.cuh"

namespace vl1 {
namespace {

constexpr int64_t kNoallocBytes = VL1_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

std::mutex g_noalloc_mutex;
void *g_noalloc_addr[kMaxDevices] = {};
CUcontext g_noalloc_ctx[kMaxDevices] = {};

using CtxGetCurrentFn = CUresult (*)(CUcontext *);

// The driver's cuCtxGetCurrent, found through the runtime (the library does
// not link the driver library itself); nullptr when unavailable.
CtxGetCurrentFn ctx_get_current() {
  static CtxGetCurrentFn fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<CtxGetCurrentFn>(p);
  }();
  return fn;
}

// Device address of the scratch array on `dev` (the current device) in the
// current context.
int32_t noalloc_scratch_address(int dev, void **out) {
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("device ordinal %d outside the supported range", dev);
    return VL1_E_ARG;
  }
  CUcontext ctx = nullptr;
  CtxGetCurrentFn get = ctx_get_current();
  if (get && get(&ctx) != CUDA_SUCCESS) ctx = nullptr;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_addr[dev] || !get || ctx != g_noalloc_ctx[dev]) {
    void *ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(noalloc scratch)");
    g_noalloc_addr[dev] = ptr;
    g_noalloc_ctx[dev] = ctx;
  }
  *out = g_noalloc_addr[dev];
  return VL1_OK;
}

}  // namespace
}  // namespace vl1

using namespace vl1;

extern "C" int32_t vl1_eval_mixed_noalloc(vl1_plan *plan, const vl1_tree_view *tree,
                                          const vl1_mixed_schedule *schedule,
                                          const double *coefs, int32_t nrhs, void *result,
                                          void *stream) {
  if (!plan || !tree || !schedule || nrhs < 1) {
    set_error("vl1_eval_mixed_noalloc: null plan/tree/schedule or nrhs < 1");
    return VL1_E_ARG;
  }
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev != plan->device) {
    set_error("vl1_eval_mixed_noalloc: the current device (%d) is not the plan's (%d)", dev,
              plan->device);
    return VL1_E_ARG;
  }
  const int64_t need =
      mixed_workspace_bytes(plan, tree->nboxes, tree->n_target_boxes, nrhs);
  if (need > kNoallocBytes) {
    set_error("vl1_eval_mixed_noalloc: this problem needs %lld bytes of scratch, above the "
              "fixed %lld-byte array; use vl1_eval_mixed with a caller-provided workspace",
              (long long)need, (long long)kNoallocBytes);
    return VL1_E_ARG;
  }
  void *scratch = nullptr;
  int32_t st = noalloc_scratch_address(dev, &scratch);
  if (st) return st;
  return vl1_eval_mixed(plan, tree, schedule, coefs, nrhs, result, scratch, kNoallocBytes,
                        stream);
}
