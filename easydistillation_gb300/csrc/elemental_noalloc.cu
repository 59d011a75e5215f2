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
//     (cudaGetSymbolAddress, with that device current) and caches it.  With
//     lazy module loading (CUDA_MODULE_LOADING=LAZY, the default of recent
//     CUDA releases) that lookup is also what loads the library's module on
//     the device and commits the 32 MiB there, so the first call does take
//     device memory: make it at an initialisation point where that is
//     allowed, and before any stream capture on the device;
//   * the tensor-core modes report a bounded device wait that gave up in a
//     status word inside the array; ed_elemental_status_noalloc reads it
//     (a run whose status is not 0 returned invalid elementals);
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
int tc_read_status(const ed_elemental_plan* P, const void* workspace, int* status, cudaStream_t stream);
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

extern "C" int ed_elemental_status_noalloc(const ed_elemental_plan* plan, int* code, void* stream) {
  ED_CHECK_ARG(plan && !plan->custom && code, "ed_elemental_status_noalloc: null pointer or a pair plan");
  ED_CHECK_ARG(plan->ws_bytes <= (size_t)ED_NOALLOC_SCRATCH_BYTES,
               "ed_elemental_status_noalloc: this plan cannot run in the built-in scratch array");
  void* scratch = nullptr;
  int rc = scratch_address(&scratch);
  if (rc != ED_OK) return rc;
  rc = ed::tc_read_status(plan, scratch, code, (cudaStream_t)stream);
  if (rc != ED_OK) return rc;
  if (*code != 0) {
    ed::set_error("elemental (no-allocation entry point): a bounded device wait gave up (code %d); the output of "
                  "that run is invalid", *code);
    return ED_ERR_TIMEOUT;
  }
  return ED_OK;
}
