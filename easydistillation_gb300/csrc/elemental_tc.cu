// Tensor-core (tcgen05) split-precision pair contractions.
#include "elemental.cuh"

namespace ed {

bool mode_supported(int mode) { return mode == ED_MODE_FP64; }

size_t tc_extra_workspace(const ed_elemental_plan* P) { return 0; }

int tc_plan_check(ed_elemental_plan* P) {
  P->tc_kind = 0;
  P->tc_bytes = 0;
  return ED_OK;
}

int launch_pair_gemm_tc(const ed_elemental_plan* P, const cplx<float>* chains, const cplx<double>* phases,
                        cplx<double>* G, void* extra, cudaStream_t stream) {
  set_error("tensor-core elemental modes are not built");
  return ED_ERR_UNSUPPORTED;
}

}  // namespace ed
