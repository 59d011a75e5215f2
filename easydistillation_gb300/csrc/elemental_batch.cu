// Batched elementals: several timeslices of one lattice in one pass.
//
// A batched plan repeats the pair groups of one timeslice for every timeslice
// of the batch (chain and G offsets per timeslice), so the chains of all
// timeslices are built first and ONE pair-contraction launch then covers the
// whole batch: the tiles of all timeslices share the GPU, which removes the
// partial last wave a single timeslice leaves (1376 tiles = 9.05 waves of 152
// CTAs at 32^3, Ne = 200, 27 momenta).  All launches are stream-ordered and
// allocation-free, so the whole batch can be captured in a CUDA graph.
#include <vector>

#include "elemental.cuh"

namespace ed {
int plan_build(ed_elemental_plan* P);
int elemental_run_batch(const ed_elemental_plan* P, int nb, const void* const* links, long long dir_stride,
                        long long site_stride, int evec_prec, const void* const* evecs, const double* blend,
                        void* const* outs, void* ws, size_t ws_bytes, cudaStream_t stream);
int elemental_run_batch_begin(const ed_elemental_plan* P, int nb, const void* const* links, long long dir_stride,
                              long long site_stride, int evec_prec, const void* const* evecs, void* ws,
                              cudaStream_t stream);
int elemental_run_batch_gemm(const ed_elemental_plan* P, int nb, void* ws, cudaStream_t stream);
int elemental_run_batch_end(const ed_elemental_plan* P, int nb, const double* blend, void* const* outs, void* ws,
                            cudaStream_t stream);
int launch_pair_gemm_tc_multi(int nplans, const ed_elemental_plan* const* plans, const int* nbs, void* const* ws,
                              cudaStream_t stream);
constexpr int kMaxMultiPlans = 4;  // volumes of one multi-volume GEMM launch (kMaxVol of tc_pair_gemm.cuh)
}  // namespace ed

extern "C" int ed_elemental_plan_create_batched(ed_elemental_plan** plan, int Lx, int Ly, int Lz, int Ne,
                                                int num_nabla, const int* moms, int nmom, int mode, int max_batch) {
  ED_CHECK_ARG(plan, "ed_elemental_plan_create_batched: null plan pointer");
  *plan = nullptr;
  ED_CHECK_ARG(Lx > 0 && Ly > 0 && Lz > 0 && Ne > 0 && nmom > 0 && max_batch > 0,
               "ed_elemental_plan_create_batched: sizes must be positive");
  ED_CHECK_ARG(num_nabla >= 0 && num_nabla <= 2, "ed_elemental_plan_create_batched: num_nabla must be 0, 1 or 2");
  ED_CHECK_ARG(moms, "ed_elemental_plan_create_batched: null momentum list");
  ED_CHECK_ARG(ed::mode_flags_valid(mode), "ed_elemental_plan_create_batched: unknown mode %d", mode);
  ED_CHECK_ARG((long long)Lx * Ly * Lz <= (1LL << 26), "ed_elemental_plan_create_batched: lattice too large");
  auto* P = new ed_elemental_plan();
  P->Lx = Lx;
  P->Ly = Ly;
  P->Lz = Lz;
  P->Ne = Ne;
  P->num_nabla = num_nabla;
  P->nmom = nmom;
  P->mode = mode & 0xff;
  ed::set_mode_flags(P, mode);
  P->use_herm = true;
  P->nbatch = max_batch;
  P->moms.assign(moms, moms + 3 * nmom);
  int rc = ed::plan_build(P);
  if (rc == ED_OK) rc = ed::tc_plan_check(P);
  if (rc != ED_OK) {
    delete P;
    return rc;
  }
  *plan = P;
  return ED_OK;
}

extern "C" int ed_elemental_run_batch(const ed_elemental_plan* plan, int nbatch, const void* const* links,
                                      long long dir_stride, long long site_stride, int evec_prec,
                                      const void* const* evecs, const double* blend, void* const* outs,
                                      void* workspace, size_t workspace_bytes, void* stream) {
  ED_CHECK_ARG(plan && !plan->custom, "ed_elemental_run_batch: needs an elemental plan");
  ED_CHECK_ARG(nbatch > 0 && nbatch <= plan->nbatch, "ed_elemental_run_batch: batch of %d timeslices, plan holds %d",
               nbatch, plan->nbatch);
  ED_CHECK_ARG(links && evecs && outs && workspace, "ed_elemental_run_batch: null pointer");
  for (int b = 0; b < nbatch; ++b)
    ED_CHECK_ARG(links[b] && evecs[b] && outs[b], "ed_elemental_run_batch: null pointer for timeslice %d", b);
  ED_CHECK_ARG(evec_prec == ED_C128 || evec_prec == ED_C64, "ed_elemental_run_batch: bad eigenvector precision");
  ED_CHECK_ARG(dir_stride >= 0 && site_stride >= 0, "ed_elemental_run_batch: negative stride");
  ED_CHECK_ARG(((uintptr_t)workspace % 256) == 0, "ed_elemental_run_batch: workspace must be 256-byte aligned");
  if (workspace_bytes < plan->ws_bytes) {
    ed::set_error("ed_elemental_run_batch: workspace of %zu bytes is smaller than the %zu the plan needs",
                  workspace_bytes, plan->ws_bytes);
    return ED_ERR_WORKSPACE;
  }
  return ed::elemental_run_batch(plan, nbatch, links, dir_stride, site_stride, evec_prec, evecs, blend, outs,
                                 workspace, workspace_bytes, (cudaStream_t)stream);
}

// ---- several batched plans (lattice volumes with their own Ne) with one pair-contraction launch

static int check_ws(const ed_elemental_plan* plan, const void* workspace, size_t workspace_bytes, const char* fn) {
  ED_CHECK_ARG(workspace, "%s: null workspace", fn);
  ED_CHECK_ARG(((uintptr_t)workspace % 256) == 0, "%s: workspace must be 256-byte aligned", fn);
  if (workspace_bytes < plan->ws_bytes) {
    ed::set_error("%s: workspace of %zu bytes is smaller than the %zu the plan needs", fn, workspace_bytes,
                  plan->ws_bytes);
    return ED_ERR_WORKSPACE;
  }
  return ED_OK;
}

extern "C" int ed_elemental_run_batch_begin(const ed_elemental_plan* plan, int nbatch, const void* const* links,
                                            long long dir_stride, long long site_stride, int evec_prec,
                                            const void* const* evecs, void* workspace, size_t workspace_bytes,
                                            void* stream) {
  ED_CHECK_ARG(plan && !plan->custom, "ed_elemental_run_batch_begin: needs an elemental plan");
  ED_CHECK_ARG(nbatch > 0 && nbatch <= plan->nbatch,
               "ed_elemental_run_batch_begin: batch of %d timeslices, plan holds %d", nbatch, plan->nbatch);
  ED_CHECK_ARG(links && evecs, "ed_elemental_run_batch_begin: null pointer");
  for (int b = 0; b < nbatch; ++b)
    ED_CHECK_ARG(links[b] && evecs[b], "ed_elemental_run_batch_begin: null pointer for timeslice %d", b);
  ED_CHECK_ARG(evec_prec == ED_C128 || evec_prec == ED_C64, "ed_elemental_run_batch_begin: bad eigenvector precision");
  ED_CHECK_ARG(dir_stride >= 0 && site_stride >= 0, "ed_elemental_run_batch_begin: negative stride");
  int rc = check_ws(plan, workspace, workspace_bytes, "ed_elemental_run_batch_begin");
  if (rc) return rc;
  return ed::elemental_run_batch_begin(plan, nbatch, links, dir_stride, site_stride, evec_prec, evecs, workspace,
                                       (cudaStream_t)stream);
}

extern "C" int ed_elemental_gemm_multi(int nplans, const ed_elemental_plan* const* plans, const int* nbatch,
                                       void* const* workspaces, const size_t* workspace_bytes, int* launches,
                                       void* stream) {
  ED_CHECK_ARG(nplans > 0 && plans && nbatch && workspaces && workspace_bytes,
               "ed_elemental_gemm_multi: null pointer or no plans");
  // the plans on the on-chip-phase tensor-core path with the split kind and form of the first such plan share
  // one launch (up to kMaxMultiPlans of them); every other plan (factorised, FP64, another kind) gets its own
  std::vector<const ed_elemental_plan*> mp;
  std::vector<int> mb, mi;
  std::vector<void*> mw;
  std::vector<int> single;
  const ed_elemental_plan* first = nullptr;
  for (int v = 0; v < nplans; ++v) {
    const ed_elemental_plan* P = plans[v];
    ED_CHECK_ARG(P && !P->custom, "ed_elemental_gemm_multi: plan %d is not an elemental plan", v);
    ED_CHECK_ARG(nbatch[v] > 0 && nbatch[v] <= P->nbatch,
                 "ed_elemental_gemm_multi: batch of %d timeslices for plan %d, which holds %d", nbatch[v], v,
                 P->nbatch);
    int rc = check_ws(P, workspaces[v], workspace_bytes[v], "ed_elemental_gemm_multi");
    if (rc) return rc;
    const bool onchip = P->tc_kind != 0 && P->tc_kind != ed::TC_OZAKI && !P->fac;
    if (onchip && !first) first = P;
    if (onchip && (int)mp.size() < ed::kMaxMultiPlans && P->tc_kind == first->tc_kind &&
        (P->tc_stack == 2) == (first->tc_stack == 2)) {
      mp.push_back(P);
      mb.push_back(nbatch[v]);
      mw.push_back(workspaces[v]);
      mi.push_back(v);
    } else {
      single.push_back(v);
    }
  }
  if (mp.size() == 1) {  // a lone on-chip plan runs its own batched GEMM
    single.push_back(mi[0]);
    mp.clear();
  }
  if (launches) *launches = (mp.empty() ? 0 : 1) + (int)single.size();
  if (!mp.empty()) {
    const int rc = ed::launch_pair_gemm_tc_multi((int)mp.size(), mp.data(), mb.data(), mw.data(), (cudaStream_t)stream);
    if (rc) return rc;
  }
  for (int v : single) {
    const int rc = ed::elemental_run_batch_gemm(plans[v], nbatch[v], workspaces[v], (cudaStream_t)stream);
    if (rc) return rc;
  }
  return ED_OK;
}

extern "C" int ed_elemental_run_batch_end(const ed_elemental_plan* plan, int nbatch, const double* blend,
                                          void* const* outs, void* workspace, size_t workspace_bytes, void* stream) {
  ED_CHECK_ARG(plan && !plan->custom, "ed_elemental_run_batch_end: needs an elemental plan");
  ED_CHECK_ARG(nbatch > 0 && nbatch <= plan->nbatch,
               "ed_elemental_run_batch_end: batch of %d timeslices, plan holds %d", nbatch, plan->nbatch);
  ED_CHECK_ARG(outs, "ed_elemental_run_batch_end: null pointer");
  for (int b = 0; b < nbatch; ++b) ED_CHECK_ARG(outs[b], "ed_elemental_run_batch_end: null output %d", b);
  int rc = check_ws(plan, workspace, workspace_bytes, "ed_elemental_run_batch_end");
  if (rc) return rc;
  return ed::elemental_run_batch_end(plan, nbatch, blend, outs, workspace, (cudaStream_t)stream);
}
