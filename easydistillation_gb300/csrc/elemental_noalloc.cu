// ed_elemental_run_noalloc: one elemental timeslice without any caller workspace.
//
// Some callers cannot allocate device memory at the point where they need
// elementals: a host application whose GPU memory is entirely owned by
// another allocator (a framework's memory pool that forbids raw cudaMalloc
// next to it), or a plugin entry point invoked from code that must not
// allocate.  For them this entry point runs the same computation as
// ed_elemental_run with its scratch taken from a fixed array compiled into
// the library, so nothing is allocated per call.
//
// Limits and behaviour:
//   * the array holds ED_NOALLOC_SCRATCH_BYTES (32 MiB); plans whose
//     workspace is larger are rejected with ED_ERR_WORKSPACE.  Every GPU that
//     loads the library keeps the array until the process exits;
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress, with that device current) and caches it; make
//     that first call before any stream capture on the device;
//   * all calls share the one array and a call leaves its contents behind.
//     Every scratch byte a run reads is written earlier in the same run
//     (the tensor-core modes clear their accumulators explicitly), so the
//     leftovers never leak into a result; but two calls that overlap on the
//     GPU (different streams, or different host threads) race on the array
//     and must be serialised by the caller.
#include <mutex>

#include "elemental.cuh"

static __device__ __align__(256) unsigned char g_noalloc_scratch[ED_NOALLOC_SCRATCH_BYTES];

namespace ed {
int elemental_run(const ed_elemental_plan* P, const void* links, long long dir_stride, long long site_stride,
                  int evec_prec, const void* evecs, const double* blend, void* out, void* ws, size_t ws_bytes,
                  cudaStream_t stream);
}  // namespace ed

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device (looked up once per device).
int scratch_address(void** addr) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return ed::cuda_status(e, "ed_elemental_run_noalloc: cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) {
    ed::set_error("ed_elemental_run_noalloc: device ordinal %d is out of range", dev);
    return ED_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return ed::cuda_status(e, "ed_elemental_run_noalloc: cudaGetSymbolAddress");
    g_scratch_addr[dev] = p;
  }
  *addr = g_scratch_addr[dev];
  return ED_OK;
}
}  // namespace

extern "C" int ed_elemental_run_noalloc(const ed_elemental_plan* plan, const void* links, long long dir_stride,
                                        long long site_stride, int evec_prec, const void* evecs, const double* blend,
                                        void* out, void* stream) {
  ED_CHECK_ARG(plan && !plan->custom, "ed_elemental_run_noalloc: needs a plan from ed_elemental_plan_create");
  ED_CHECK_ARG(links && evecs && out, "ed_elemental_run_noalloc: null pointer");
  ED_CHECK_ARG(evec_prec == ED_C128 || evec_prec == ED_C64, "ed_elemental_run_noalloc: bad eigenvector precision");
  ED_CHECK_ARG(dir_stride >= 0 && site_stride >= 0, "ed_elemental_run_noalloc: negative stride");
  if (plan->ws_bytes > (size_t)ED_NOALLOC_SCRATCH_BYTES) {
    ed::set_error(
        "ed_elemental_run_noalloc: this plan needs %zu bytes of scratch, more than the built-in %zu; "
        "use ed_elemental_run with a caller workspace",
        plan->ws_bytes, (size_t)ED_NOALLOC_SCRATCH_BYTES);
    return ED_ERR_WORKSPACE;
  }
  void* scratch = nullptr;
  int rc = scratch_address(&scratch);
  if (rc != ED_OK) return rc;
  return ed::elemental_run(plan, links, dir_stride, site_stride, evec_prec, evecs, blend, out, scratch,
                           (size_t)ED_NOALLOC_SCRATCH_BYTES, (cudaStream_t)stream);
}
