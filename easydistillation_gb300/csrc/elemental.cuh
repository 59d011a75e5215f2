// Elemental plan: host-side description of one timeslice of elementals.
#pragma once

#include <vector>

#include "common.cuh"

namespace ed {

enum TcKind { TC_F16 = 1, TC_BF16 = 2, TC_TF32 = 3, TC_OZAKI = 4 };  // ed_elemental_plan::tc_kind
constexpr int kMaxJobs = 64;   // pair groups (one per left chain and timeslice of a batch)
constexpr int kMaxTerms = 64;  // subset terms over all operators (43 for num_nabla = 2)
constexpr int kMaxDeriv = 13;  // operators for num_nabla = 2
constexpr int kMaxMom = 256;   // momenta for which p -> -p lookup is tabulated

// One GEMM group: left chain `left` against right chains [right0, right0+nright).
struct Job {
  int left, right0, nright;
  long long g_off;  // offset of G[nmom][Ne][nright*Ne] in complex elements
};

// One subset term of an operator: coeff * G_p(left, right), or, when herm,
// coeff * conj(G_{-p}(right, left))^T read from group `job`.
struct Term {
  int coeff, job, roff, herm;
};

}  // namespace ed

struct ed_elemental_plan {
  int Lx, Ly, Lz, V3, Ne, num_nabla, nderiv, nmom, mode;
  bool use_herm, herm;
  bool custom = false;  // generic pair plan (caller-built chains, no operator terms)
  int nbatch = 1;       // timeslices per run (batched plans)
  int jobs_per_t = 0;   // pair groups of one timeslice
  long long g_per_t = 0;  // G elements of one timeslice
  std::vector<int> moms, negidx;
  int nchain;
  std::vector<int> chain_parent, chain_dir;
  std::vector<ed::Job> jobs;
  std::vector<ed::Term> terms;
  std::vector<int> term_start;
  long long g_elems;
  int npairs;
  size_t off_links, off_links32, off_phase, off_chain, off_g, off_extra, ws_bytes;
  // tensor-core path parameters (filled by tc_plan_check)
  int tc_kind;        // 0 = none
  int tc_scale_exp;   // power-of-two scale applied before fp16 splitting
  size_t tc_bytes;    // extra workspace
  // factorised phases: momenta = {(px,py)} x {pz} up to a few unused combinations, or every momentum's phase
  // on the left side (ED_MODE_FLAG_LEFT_FACTOR: left factors = the momenta, one right factor = 1)
  bool no_factor = false;       // ED_MODE_FLAG_NO_FACTOR given at creation
  bool force_factor = false;    // ED_MODE_FLAG_FORCE_FACTOR: factorise however many combinations go unused
  bool left_factor = false;     // ED_MODE_FLAG_LEFT_FACTOR
  bool fac = false;             // the factorised-phase GEMM serves this plan
  int fac_pxy = 0, fac_pz = 0;  // left factors (distinct (px, py) pairs) and right factors (distinct pz)
  std::vector<int> fac_l, fac_r;  // their momenta, 3 ints each: phase_p = phase_{fac_l[a]} phase_{fac_r[c]}
  std::vector<signed char> fac_pidx;    // momentum index of (a, c), -1 if not in the list
  std::vector<int> fac_lchain;          // left-chain slots of one timeslice -> chain index
  std::vector<int> fac_lslot;           // chain index -> left-chain slot (-1 if never a left chain)
  cudaEvent_t prof_start = nullptr, prof_stop = nullptr;  // optional events around the pair GEMM
  // launch settings (ed_elemental_set_tuning); 0 everywhere is the built-in default
  int f64_tile = 0;    // FP64 pair GEMM tile, rows x cols: 0 = 64x64, 1 = 32x64, 2 = 64x32, 3 = 32x32
  int tc_slab_kb = 0;  // k-blocks per lock-step slab of the factorised GEMM (0 = TC_FLUSH_KB)
  int tc_grid = 0;     // CTAs of the persistent factorised GEMM (0 = every co-resident CTA)
  int tc_stages = 0;   // operand stages of the factorised GEMM (0 = the default of the GEMM form)
  int tc_pair = 0;     // factorised GEMM on single SMs (1) or on SM pairs (2); 0 = the built-in default
  int tc_kpb = 0;      // k-blocks accumulated per TMEM buffer of the factorised GEMM: 1, 2 or 4 (0: the form's default)
  bool gauss = false;  // factorised split GEMM in the Gauss three-multiplication form (ED_MODE_FLAG_GAUSS)
  int tc_stack = 0;    // factorised GEMM on single SMs: 0/1 = stacked [re | im] B operand (N = 256), 2 = four products
  int f64_ksplit = 1;  // K-split partial buffers the FP64 pair GEMM may use (sized at plan build)
  int f64_df = 0;      // FP64 pair GEMM in double-float arithmetic on the FP32 pipe (ED_TUNE_F64_DF)
};

namespace ed {
bool mode_supported(int mode);
bool mode_flags_valid(int mode);
void set_mode_flags(ed_elemental_plan* P, int mode);
void tc_fac_setup(ed_elemental_plan* P);
size_t tc_extra_workspace(const ed_elemental_plan* P);
size_t f64_extra_workspace(ed_elemental_plan* P);
int tc_plan_check(ed_elemental_plan* P);
int launch_pair_gemm_tc(const ed_elemental_plan* P, const cplx<float>* chains, const cplx<double>* phases,
                        cplx<double>* G, void* extra, cudaStream_t stream, int nb);
int tc_read_status(const ed_elemental_plan* P, const void* workspace, int* status, cudaStream_t stream);
}  // namespace ed
