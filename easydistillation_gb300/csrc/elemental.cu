// Elemental contraction E[d, p, i, j] (reference lattice/generator/elemental.py:290-338).
//
// The reference evaluates, for every derivative operator d and each of the
// 2^len(d) left/right subsets, a fresh pair of covariant-derivative chains and
// one zgemm per momentum.  Here one timeslice is planned once:
//   1. chains: every direction sequence s of length <= num_nabla is built once
//      (chain id = derivative index of s, derivative.py:23-33), each from its
//      parent by one hop kernel;
//   2. pair contractions G_p(X, Y)[i, j] = sum_k conj(X_i[k]) phase_p(k) Y_j[k]
//      for the distinct (left, right) chain pairs, grouped by left chain with a
//      contiguous range of right chains (one GEMM per group and momentum);
//      when the momentum list is closed under p -> -p, pairs with left > right
//      come from G_p(X, Y) = G_{-p}(Y, X)^dagger instead of a second GEMM;
//   3. combine: E[d, p] = sum_subsets (-1)^{#right} G_p(left, right), times the
//      blending coefficients when present (elemental.py:309-337).
#include <algorithm>
#include <map>
#include <vector>

#include "common.cuh"
#include "df.cuh"
#include "elemental.cuh"
#include "tc_config.cuh"

namespace ed {

int launch_links_to_soa(int out_prec, Latt L, int nt, const void* in, long long ts, long long ds, long long ss,
                        void* out, cudaStream_t stream);
int launch_to_planes(int ip, int op, int round_c64, long long nvec, int V3, const void* in, void* out,
                     cudaStream_t stream);
int launch_phases(Latt L, const int* moms, int nmom, cplx<double>* out, cudaStream_t stream);
int launch_hop(int in_prec, int out_prec, Latt L, int d, int nvec, const void* links_c128, const void* in,
               void* out, cudaStream_t stream);
int launch_hop_f32(Latt L, int d, int nvec, const void* links_c64, const void* in, void* out, cudaStream_t stream);

// ------------------------------------------------------------ plan (host)

static std::vector<int> derivative_seq(int n) {
  int len = 0, block = 1;
  while (n >= block) {
    n -= block;
    ++len;
    block *= 3;
  }
  std::vector<int> d(len);
  for (int k = len - 1; k >= 0; --k) {
    d[k] = n % 3;
    n /= 3;
  }
  return d;
}

static int chain_id(const std::vector<int>& s) {
  int base = 0, p3 = 1;
  for (size_t k = 0; k < s.size(); ++k) {
    base += p3;
    p3 *= 3;
  }
  int v = 0;
  for (int d : s) v = v * 3 + d;
  return base + v;
}

int plan_build(ed_elemental_plan* P) {
  P->V3 = P->Lx * P->Ly * P->Lz;
  P->nderiv = 0;
  for (int k = 0, p3 = 1; k <= P->num_nabla; ++k, p3 *= 3) P->nderiv += p3;
  P->nchain = P->nderiv;
  P->chain_parent.assign(P->nchain, -1);
  P->chain_dir.assign(P->nchain, -1);
  for (int c = 1; c < P->nchain; ++c) {
    std::vector<int> s = derivative_seq(c);
    P->chain_dir[c] = s.back();
    s.pop_back();
    P->chain_parent[c] = chain_id(s);
  }
  // momentum negation table
  P->negidx.assign(P->nmom, -1);
  bool closed = true;
  for (int a = 0; a < P->nmom; ++a) {
    for (int b = 0; b < P->nmom; ++b)
      if (P->moms[3 * b] == -P->moms[3 * a] && P->moms[3 * b + 1] == -P->moms[3 * a + 1] &&
          P->moms[3 * b + 2] == -P->moms[3 * a + 2]) {
        P->negidx[a] = b;
        break;
      }
    if (P->negidx[a] < 0) closed = false;
  }
  P->herm = closed && P->use_herm && P->nmom <= kMaxMom;

  // terms (elemental.py:309-321): bit k of `pick` sends direction k right
  struct RawTerm {
    int d, coeff, X, Y;
  };
  std::vector<RawTerm> raw;
  for (int d = 0; d < P->nderiv; ++d) {
    std::vector<int> dv = derivative_seq(d);
    for (int pick = 0; pick < (1 << dv.size()); ++pick) {
      std::vector<int> right, left;
      for (size_t k = 0; k < dv.size(); ++k) ((pick >> k) & 1 ? right : left).push_back(dv[k]);
      std::reverse(left.begin(), left.end());
      raw.push_back({d, (right.size() % 2) ? -1 : 1, chain_id(left), chain_id(right)});
    }
  }
  // needed (left, right) pairs, canonical under hermiticity
  std::map<int, std::pair<int, int>> range;  // left -> [ymin, ymax]
  for (auto& r : raw) {
    int X = r.X, Y = r.Y;
    if (P->herm && X > Y) std::swap(X, Y);
    auto it = range.find(X);
    if (it == range.end())
      range[X] = {Y, Y};
    else
      it->second = {std::min(it->second.first, Y), std::max(it->second.second, Y)};
  }
  P->jobs.clear();
  long long goff = 0;
  for (auto& kv : range) {
    Job j;
    j.left = kv.first;
    j.right0 = kv.second.first;
    j.nright = kv.second.second - kv.second.first + 1;
    j.g_off = goff;
    goff += (long long)P->nmom * P->Ne * j.nright * P->Ne;
    P->jobs.push_back(j);
  }
  P->g_elems = goff;
  if ((int)P->jobs.size() > kMaxJobs) {
    set_error("elemental plan: %d pair groups exceed the limit %d", (int)P->jobs.size(), kMaxJobs);
    return ED_ERR_UNSUPPORTED;
  }
  auto job_of = [&](int X) {
    for (size_t k = 0; k < P->jobs.size(); ++k)
      if (P->jobs[k].left == X) return (int)k;
    return -1;
  };
  P->terms.clear();
  P->term_start.assign(P->nderiv + 1, 0);
  for (int d = 0; d < P->nderiv; ++d) {
    P->term_start[d] = (int)P->terms.size();
    for (auto& r : raw) {
      if (r.d != d) continue;
      Term t;
      t.coeff = r.coeff;
      if (P->herm && r.X > r.Y) {
        t.job = job_of(r.Y);
        t.roff = r.X - P->jobs[t.job].right0;
        t.herm = 1;
      } else {
        t.job = job_of(r.X);
        t.roff = r.Y - P->jobs[t.job].right0;
        t.herm = 0;
      }
      P->terms.push_back(t);
    }
  }
  P->term_start[P->nderiv] = (int)P->terms.size();
  if ((int)P->terms.size() > kMaxTerms) {
    set_error("elemental plan: %d terms exceed the limit %d", (int)P->terms.size(), kMaxTerms);
    return ED_ERR_UNSUPPORTED;
  }
  P->npairs = 0;
  for (auto& j : P->jobs) P->npairs += j.nright;

  // Batch of timeslices: timeslice b owns chains [b*nchain, (b+1)*nchain) and
  // G block b; its groups repeat the first timeslice's with those offsets, so
  // one pair-contraction launch covers the whole batch.
  P->jobs_per_t = (int)P->jobs.size();
  P->g_per_t = P->g_elems;
  if ((long long)P->jobs_per_t * P->nbatch > kMaxJobs) {
    set_error("elemental plan: %d timeslices x %d pair groups exceed the limit %d", P->nbatch, P->jobs_per_t,
              kMaxJobs);
    return ED_ERR_UNSUPPORTED;
  }
  for (int b = 1; b < P->nbatch; ++b)
    for (int k = 0; k < P->jobs_per_t; ++k) {
      Job j = P->jobs[k];
      j.left += b * P->nchain;
      j.right0 += b * P->nchain;
      j.g_off += b * P->g_per_t;
      P->jobs.push_back(j);
    }
  P->g_elems = P->g_per_t * P->nbatch;
  tc_fac_setup(P);

  // workspace layout (256-byte aligned sections)
  auto up = [](size_t v) { return (v + 255) / 256 * 256; };
  const size_t B = (size_t)P->nbatch;
  size_t off = 0;
  P->off_links = off;
  off = up(off + B * 27ull * P->V3 * 16);
  P->off_links32 = off;
  if (P->mode != ED_MODE_FP64) off = up(off + B * 27ull * P->V3 * 8);
  P->off_phase = off;
  off = up(off + (size_t)P->nmom * P->V3 * 16);
  P->off_chain = off;
  const size_t chain_elt = P->mode == ED_MODE_FP64 ? 16 : 8;
  off = up(off + B * (size_t)P->nchain * P->Ne * 3 * P->V3 * chain_elt);
  P->off_g = off;
  off = up(off + (size_t)P->g_elems * 16);
  P->off_extra = off;
  off = up(off + tc_extra_workspace(P) + f64_extra_workspace(P));
  P->ws_bytes = off;
  return ED_OK;
}

// ------------------------------------------------------------ FP64 pair GEMM

struct GemmJobDev {
  int left, right0, nright, tile0, mt, nt;
  long long g_off;
};
struct GemmTable {
  int njobs;
  GemmJobDev j[kMaxJobs];
};

constexpr int F64_BK = 8;
constexpr long long F64_MIN_KCHUNK = 1024;  // k per K-split partial, at least
constexpr long long F64_SPLIT_TARGET = 320;  // CTAs the K split aims at (about two per SM)
constexpr int F64_KSPLIT_MAX = 16;

// One CTA = a (16*TM) x (16*TN) tile of G_p(X, Y-range) for one (group,
// momentum).  256 threads as 16x16, each owning TM x TN complex outputs.  The
// left operand is multiplied by the phase while staged:
// A[i][k] = conj(X_i[k]) * phase_p(k mod V3).  The tile shape is a plan
// setting (ED_TUNE_F64_TILE): smaller tiles waste less on an Ne that is not a
// multiple of 64 and give more CTAs for small Ne.
template <int TM, int TN>
__global__ void __launch_bounds__(256) pair_gemm_f64_kernel(GemmTable tab, int Ne, int V3, int nmom,
                                                            const cplx<double>* __restrict__ chains,
                                                            const cplx<double>* __restrict__ phases,
                                                            cplx<double>* __restrict__ G, long long kchunk,
                                                            long long part_stride) {
  constexpr int BM = 16 * TM, BN = 16 * TN;
  __shared__ cplx<double> As[F64_BK][BM + 1];
  __shared__ cplx<double> Bs[F64_BK][BN + 1];
  int tile = blockIdx.x;
  int jb = 0;
  while (jb + 1 < tab.njobs && tile >= tab.j[jb + 1].tile0) ++jb;
  const GemmJobDev J = tab.j[jb];
  int local = tile - J.tile0;
  const int per_p = J.mt * J.nt;
  const int p = local / per_p;
  local -= p * per_p;
  const int mtile = local / J.nt;
  const int ntile = local - mtile * J.nt;
  const long long K = 3LL * V3;
  // K split: CTA (tile, blockIdx.y) sums k in [k_begin, k_end) into partial blockIdx.y (one partial: G itself)
  const long long k_begin = blockIdx.y * kchunk, k_end = min(K, k_begin + kchunk);
  G += blockIdx.y * part_stride;
  const int M = Ne, N = J.nright * Ne;
  const cplx<double>* Lc = chains + (long long)J.left * Ne * K;
  const cplx<double>* Rc = chains + (long long)J.right0 * Ne * K;
  const cplx<double>* ph = phases + (long long)p * V3;

  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int lk = tid & 7, lr = tid >> 3;  // loader: 8 consecutive k per row, 32 rows per pass
  cplx<double> acc[TM][TN];
#pragma unroll
  for (int a = 0; a < TM; ++a)
#pragma unroll
    for (int b = 0; b < TN; ++b) acc[a][b] = mk(0.0, 0.0);

  for (long long k0 = k_begin; k0 < k_end; k0 += F64_BK) {
    const long long k = k0 + lk;
    cplx<double> phk = mk(0.0, 0.0);
    if (k < k_end) phk = ld(ph + (k % V3));
#pragma unroll
    for (int pass = 0; pass < BM / 32; ++pass) {
      const int r = lr + 32 * pass;
      const int gi = mtile * BM + r;
      cplx<double> a = mk(0.0, 0.0);
      if (gi < M && k < k_end) a = cmul_conj(ld(Lc + (long long)gi * K + k), phk);
      As[lk][r] = a;
    }
#pragma unroll
    for (int pass = 0; pass < BN / 32; ++pass) {
      const int r = lr + 32 * pass;
      const int gj = ntile * BN + r;
      cplx<double> b = mk(0.0, 0.0);
      if (gj < N && k < k_end) b = ld(Rc + (long long)gj * K + k);
      Bs[lk][r] = b;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < F64_BK; ++kk) {
      cplx<double> av[TM], bv[TN];
#pragma unroll
      for (int a = 0; a < TM; ++a) av[a] = As[kk][ty + 16 * a];
#pragma unroll
      for (int b = 0; b < TN; ++b) bv[b] = Bs[kk][tx + 16 * b];
#pragma unroll
      for (int a = 0; a < TM; ++a)
#pragma unroll
        for (int b = 0; b < TN; ++b) cfma(acc[a][b], av[a], bv[b]);
    }
    __syncthreads();
  }
  cplx<double>* Gp = G + J.g_off + (long long)p * M * N;
#pragma unroll
  for (int a = 0; a < TM; ++a) {
    const int gi = mtile * BM + ty + 16 * a;
    if (gi >= M) continue;
#pragma unroll
    for (int b = 0; b < TN; ++b) {
      const int gj = ntile * BN + tx + 16 * b;
      if (gj < N) Gp[(long long)gi * N + gj] = acc[a][b];
    }
  }
}

// The same pair GEMM in double-float arithmetic on the FP32 pipe (ED_TUNE_F64_DF): the staged operands are
// float4 {re_hi, im_hi, re_lo, im_lo} (df.cuh), split from the complex128 chains and phases by integer
// operations on their bits; the left operand conj(X_i) phase_p is formed in double-float while staged; every
// complex multiply-add is four exact FP32 product splits with cross terms and two-sum accumulation (~2^-47 per
// product); results are written as complex128.  On this part the FP32 pipe runs ~60x the FP64 rate.
__device__ __forceinline__ float4 df_cmul_conj(float4 x, float4 p) {  // conj(x) * p
  DF re{0.f, 0.f}, im{0.f, 0.f};
  df_acc(re, x.x, x.z, p.x, p.z);
  df_acc(re, x.y, x.w, p.y, p.w);
  df_acc(im, x.x, x.z, p.y, p.w);
  df_sub(im, x.y, x.w, p.x, p.z);
  return make_float4(re.hi, im.hi, re.lo, im.lo);
}

template <int TM, int TN>
__global__ void __launch_bounds__(256) pair_gemm_df_kernel(GemmTable tab, int Ne, int V3, int nmom,
                                                           const cplx<double>* __restrict__ chains,
                                                           const cplx<double>* __restrict__ phases,
                                                           cplx<double>* __restrict__ G, long long kchunk,
                                                           long long part_stride) {
  constexpr int BM = 16 * TM, BN = 16 * TN;
  __shared__ float4 As[F64_BK][BM + 1];
  __shared__ float4 Bs[F64_BK][BN + 1];
  int tile = blockIdx.x;
  int jb = 0;
  while (jb + 1 < tab.njobs && tile >= tab.j[jb + 1].tile0) ++jb;
  const GemmJobDev J = tab.j[jb];
  int local = tile - J.tile0;
  const int per_p = J.mt * J.nt;
  const int p = local / per_p;
  local -= p * per_p;
  const int mtile = local / J.nt;
  const int ntile = local - mtile * J.nt;
  const long long K = 3LL * V3;
  const long long k_begin = blockIdx.y * kchunk, k_end = min(K, k_begin + kchunk);
  G += blockIdx.y * part_stride;
  const int M = Ne, N = J.nright * Ne;
  const cplx<double>* Lc = chains + (long long)J.left * Ne * K;
  const cplx<double>* Rc = chains + (long long)J.right0 * Ne * K;
  const cplx<double>* ph = phases + (long long)p * V3;

  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int lk = tid & 7, lr = tid >> 3;
  DF are[TM][TN], aim[TM][TN];
#pragma unroll
  for (int a = 0; a < TM; ++a)
#pragma unroll
    for (int b = 0; b < TN; ++b) are[a][b] = aim[a][b] = DF{0.f, 0.f};
  const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);

  for (long long k0 = k_begin; k0 < k_end; k0 += F64_BK) {
    const long long k = k0 + lk;
    float4 phk = zero;
    if (k < k_end) {
      const cplx<double> pv = ld(ph + (k % V3));
      phk = split_c128_bits(make_double2(pv.re, pv.im));
    }
#pragma unroll
    for (int pass = 0; pass < BM / 32; ++pass) {
      const int r = lr + 32 * pass;
      const int gi = mtile * BM + r;
      float4 a = zero;
      if (gi < M && k < k_end) {
        const cplx<double> xv = ld(Lc + (long long)gi * K + k);
        a = df_cmul_conj(split_c128_bits(make_double2(xv.re, xv.im)), phk);
      }
      As[lk][r] = a;
    }
#pragma unroll
    for (int pass = 0; pass < BN / 32; ++pass) {
      const int r = lr + 32 * pass;
      const int gj = ntile * BN + r;
      float4 b = zero;
      if (gj < N && k < k_end) {
        const cplx<double> yv = ld(Rc + (long long)gj * K + k);
        b = split_c128_bits(make_double2(yv.re, yv.im));
      }
      Bs[lk][r] = b;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < F64_BK; ++kk) {
      float4 av[TM], bv[TN];
#pragma unroll
      for (int a = 0; a < TM; ++a) av[a] = As[kk][ty + 16 * a];
#pragma unroll
      for (int b = 0; b < TN; ++b) bv[b] = Bs[kk][tx + 16 * b];
#pragma unroll
      for (int a = 0; a < TM; ++a)
#pragma unroll
        for (int b = 0; b < TN; ++b) {  // (ar + i ai)(br + i bi)
          df_acc(are[a][b], av[a].x, av[a].z, bv[b].x, bv[b].z);
          df_sub(are[a][b], av[a].y, av[a].w, bv[b].y, bv[b].w);
          df_acc(aim[a][b], av[a].x, av[a].z, bv[b].y, bv[b].w);
          df_acc(aim[a][b], av[a].y, av[a].w, bv[b].x, bv[b].z);
        }
    }
    // K runs to 3 V3 (98304 at 32^3): renormalise the sums once per stage of F64_BK terms
#pragma unroll
    for (int a = 0; a < TM; ++a)
#pragma unroll
      for (int b = 0; b < TN; ++b) {
        df_renorm(are[a][b]);
        df_renorm(aim[a][b]);
      }
    __syncthreads();
  }
  cplx<double>* Gp = G + J.g_off + (long long)p * M * N;
#pragma unroll
  for (int a = 0; a < TM; ++a) {
    const int gi = mtile * BM + ty + 16 * a;
    if (gi >= M) continue;
#pragma unroll
    for (int b = 0; b < TN; ++b) {
      const int gj = ntile * BN + tx + 16 * b;
      if (gj < N) Gp[(long long)gi * N + gj] = mk(df_value(are[a][b]), df_value(aim[a][b]));
    }
  }
}

// ------------------------------------------------------------ combine

struct CombineTable {
  int nderiv, herm, nmom, Ne;
  int start[kMaxDeriv + 1];
  Term t[kMaxTerms];
  long long g_off[kMaxJobs];
  int nright[kMaxJobs];
  short negidx[kMaxMom];
};

// The term table travels as a kernel argument (about 2 KB).
__global__ void combine_kernel(const CombineTable tab, const cplx<double>* __restrict__ G,
                               const double* __restrict__ blend, cplx<double>* __restrict__ out) {
  const int Ne = tab.Ne;
  const long long total = (long long)tab.nderiv * tab.nmom * Ne * Ne;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(idx % Ne);
    const int i = (int)((idx / Ne) % Ne);
    const int p = (int)((idx / ((long long)Ne * Ne)) % tab.nmom);
    const int d = (int)(idx / ((long long)Ne * Ne * tab.nmom));
    cplx<double> acc = mk(0.0, 0.0);
    for (int q = tab.start[d]; q < tab.start[d + 1]; ++q) {
      const Term T = tab.t[q];
      const int N = tab.nright[T.job] * Ne;
      cplx<double> v;
      if (!T.herm) {
        v = G[tab.g_off[T.job] + ((long long)p * Ne + i) * N + T.roff * Ne + j];
      } else {
        const int np = tab.negidx[p];
        cplx<double> w = G[tab.g_off[T.job] + ((long long)np * Ne + j) * N + T.roff * Ne + i];
        v = mk(w.re, -w.im);
      }
      acc.re += T.coeff * v.re;
      acc.im += T.coeff * v.im;
    }
    if (blend) {
      const double c = blend[(long long)i * Ne + j];
      acc.re *= c;
      acc.im *= c;
    }
    out[idx] = acc;
  }
}

// ------------------------------------------------------------ run

// G[i] = sum over the K-split partials, in a fixed order (results do not depend on scheduling)
__global__ void f64_reduce_kernel(const cplx<double>* __restrict__ part, long long stride, int nsplit, long long n,
                                  cplx<double>* __restrict__ G) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    cplx<double> s = part[i];
    for (int q = 1; q < nsplit; ++q) s = s + part[q * stride + i];
    G[i] = s;
  }
}

int launch_pair_gemm_f64(const ed_elemental_plan* P, const cplx<double>* chains, const cplx<double>* phases,
                         cplx<double>* G, cudaStream_t stream, int njobs, void* extra) {
  // tile shapes of ED_TUNE_F64_TILE: rows x cols = 64x64, 32x64, 64x32, 32x32
  static const int kBM[4] = {64, 32, 64, 32}, kBN[4] = {64, 64, 32, 32};
  const int shape = P->f64_tile;
  GemmTable tab;
  tab.njobs = njobs;
  int tiles = 0;
  for (int k = 0; k < tab.njobs; ++k) {
    const Job& j = P->jobs[k];
    GemmJobDev& d = tab.j[k];
    d.left = j.left;
    d.right0 = j.right0;
    d.nright = j.nright;
    d.g_off = j.g_off;
    d.mt = ceil_div(P->Ne, kBM[shape]);
    d.nt = ceil_div((long long)j.nright * P->Ne, kBN[shape]);
    d.tile0 = tiles;
    tiles += d.mt * d.nt * P->nmom;
  }
  auto kern = P->f64_df ? (shape == 0   ? pair_gemm_df_kernel<4, 4>
                           : shape == 1 ? pair_gemm_df_kernel<2, 4>
                           : shape == 2 ? pair_gemm_df_kernel<4, 2>
                                        : pair_gemm_df_kernel<2, 2>)
                        : (shape == 0   ? pair_gemm_f64_kernel<4, 4>
                           : shape == 1 ? pair_gemm_f64_kernel<2, 4>
                           : shape == 2 ? pair_gemm_f64_kernel<4, 2>
                                        : pair_gemm_f64_kernel<2, 2>);
  // Few output tiles (few momenta, small Ne) leave most SMs idle over a long K: split K into partials, summed in
  // a fixed order afterwards, up to the plan's partial buffers and at least F64_MIN_KCHUNK k per part.
  const long long K = 3LL * P->V3;
  int nsplit = std::min<long long>(P->f64_ksplit, std::max<long long>(1, K / F64_MIN_KCHUNK));
  nsplit = std::max(1, std::min(nsplit, ceil_div(2LL * num_sms(), tiles)));
  const long long kchunk = (ceil_div(K, nsplit) + F64_BK - 1) / F64_BK * F64_BK;
  nsplit = ceil_div(K, kchunk);
  const long long g_used = njobs > 0 ? P->jobs[njobs - 1].g_off +
                                           (long long)P->nmom * P->Ne * P->jobs[njobs - 1].nright * P->Ne
                                     : 0;
  cplx<double>* part = nsplit > 1 ? (cplx<double>*)extra : G;
  if (P->prof_start) cudaEventRecord(P->prof_start, stream);
  kern<<<dim3(tiles, nsplit), 256, 0, stream>>>(tab, P->Ne, P->V3, P->nmom, chains, phases, part, kchunk, g_used);
  ED_RETURN_LAUNCH("pair GEMM (fp64)");
  if (nsplit > 1) {
    const int grid = (int)std::min<long long>(ceil_div(g_used, 256), 4LL * 1024 * num_sms());
    f64_reduce_kernel<<<grid, 256, 0, stream>>>(part, g_used, nsplit, g_used, G);
    ED_RETURN_LAUNCH("pair GEMM (fp64) partial sum");
  }
  if (P->prof_stop) cudaEventRecord(P->prof_stop, stream);
  return ED_OK;
}

// K-split partial buffers an FP64 plan reserves: as many as it takes to give about 320 CTAs with the
// 64 x 64 tiles (the fewest), at most 16, none when the tiles already fill the device.
size_t f64_extra_workspace(ed_elemental_plan* P) {
  P->f64_ksplit = 1;
  if (P->mode != ED_MODE_FP64) return 0;
  long long tiles = 0;
  for (size_t k = 0; k < P->jobs.size(); ++k)
    tiles += (long long)ceil_div(P->Ne, 64) * ceil_div((long long)P->jobs[k].nright * P->Ne, 64) * P->nmom;
  if (tiles >= F64_SPLIT_TARGET || 3LL * P->V3 < 2 * F64_MIN_KCHUNK) return 0;
  P->f64_ksplit = (int)std::min<long long>(F64_KSPLIT_MAX, ceil_div(F64_SPLIT_TARGET, std::max(1LL, tiles)));
  return (size_t)P->f64_ksplit * (size_t)P->g_elems * sizeof(cplx<double>);
}

int launch_combine(const ed_elemental_plan* P, const cplx<double>* G, const double* blend, cplx<double>* out,
                   cudaStream_t stream) {
  CombineTable tab;
  memset(&tab, 0, sizeof(tab));
  tab.nderiv = P->nderiv;
  tab.herm = P->herm;
  tab.nmom = P->nmom;
  tab.Ne = P->Ne;
  for (int d = 0; d <= P->nderiv; ++d) tab.start[d] = P->term_start[d];
  for (size_t q = 0; q < P->terms.size(); ++q) tab.t[q] = P->terms[q];
  for (int k = 0; k < P->jobs_per_t; ++k) {  // offsets within one timeslice's G block
    tab.g_off[k] = P->jobs[k].g_off;
    tab.nright[k] = P->jobs[k].nright;
  }
  for (int p = 0; p < P->nmom && p < kMaxMom; ++p) tab.negidx[p] = (short)P->negidx[p];
  const long long total = (long long)P->nderiv * P->nmom * P->Ne * P->Ne;
  const int grid = (int)std::min<long long>(ceil_div(total, 256), 4LL * 1024 * num_sms());
  combine_kernel<<<grid, 256, 0, stream>>>(tab, G, blend, out);
  ED_RETURN_LAUNCH("combine");
  return ED_OK;
}


// The three parts of a batched run: the phases and the chains of the nb timeslices (begin), the pair
// contraction (one launch for the whole batch), and the combine into the caller's outputs (end).
int elemental_run_batch_begin(const ed_elemental_plan* P, int nb, const void* const* links, long long dir_stride,
                              long long site_stride, int evec_prec, const void* const* evecs, void* ws,
                              cudaStream_t stream) {
  char* W = (char*)ws;
  const Latt L{P->Lx, P->Ly, P->Lz};
  int rc;
  cplx<double>* phases = (cplx<double>*)(W + P->off_phase);
  rc = launch_phases(L, P->moms.data(), P->nmom, phases, stream);
  if (rc) return rc;
  const int cprec = P->mode == ED_MODE_FP64 ? ED_C128 : ED_C64;
  const size_t celt = cprec == ED_C128 ? 16 : 8;
  const size_t chain_bytes = (size_t)P->Ne * 3 * P->V3 * celt;
  for (int b = 0; b < nb; ++b) {
    void* links_soa = W + P->off_links + (size_t)b * 27 * P->V3 * 16;
    void* links32 = W + P->off_links32 + (size_t)b * 27 * P->V3 * 8;
    char* chains = W + P->off_chain + (size_t)b * P->nchain * chain_bytes;
    if (cprec == ED_C128 || P->nchain == 1) {
      rc = launch_links_to_soa(ED_C128, L, 1, links[b], 0, dir_stride, site_stride, links_soa, stream);
      if (rc) return rc;
    }
    rc = launch_to_planes(evec_prec, cprec, 1, P->Ne, P->V3, evecs[b], chains, stream);
    if (rc) return rc;
    if (cprec == ED_C64 && P->nchain > 1) {
      rc = launch_links_to_soa(ED_C64, L, 1, links[b], 0, dir_stride, site_stride, links32, stream);
      if (rc) return rc;
    }
    for (int c = 1; c < P->nchain; ++c) {
      const void* src = chains + P->chain_parent[c] * chain_bytes;
      void* dst = chains + c * chain_bytes;
      if (cprec == ED_C64)
        rc = launch_hop_f32(L, P->chain_dir[c], P->Ne, links32, src, dst, stream);
      else
        rc = launch_hop(cprec, cprec, L, P->chain_dir[c], P->Ne, links_soa, src, dst, stream);
      if (rc) return rc;
    }
  }
  return ED_OK;
}

int elemental_run_batch_gemm(const ed_elemental_plan* P, int nb, void* ws, cudaStream_t stream) {
  char* W = (char*)ws;
  const cplx<double>* phases = (const cplx<double>*)(W + P->off_phase);
  cplx<double>* G = (cplx<double>*)(W + P->off_g);
  if (P->mode == ED_MODE_FP64)
    return launch_pair_gemm_f64(P, (const cplx<double>*)(W + P->off_chain), phases, G, stream, nb * P->jobs_per_t,
                                W + P->off_extra);
  return launch_pair_gemm_tc(P, (const cplx<float>*)(W + P->off_chain), phases, G, W + P->off_extra, stream, nb);
}

int elemental_run_batch_end(const ed_elemental_plan* P, int nb, const double* blend, void* const* outs, void* ws,
                            cudaStream_t stream) {
  cplx<double>* G = (cplx<double>*)((char*)ws + P->off_g);
  for (int b = 0; b < nb; ++b) {
    const int rc = launch_combine(P, G + (size_t)b * P->g_per_t, blend, (cplx<double>*)outs[b], stream);
    if (rc) return rc;
  }
  return ED_OK;
}

int elemental_run_batch(const ed_elemental_plan* P, int nb, const void* const* links, long long dir_stride,
                        long long site_stride, int evec_prec, const void* const* evecs, const double* blend,
                        void* const* outs, void* ws, size_t ws_bytes, cudaStream_t stream) {
  (void)ws_bytes;
  int rc = elemental_run_batch_begin(P, nb, links, dir_stride, site_stride, evec_prec, evecs, ws, stream);
  if (rc == ED_OK) rc = elemental_run_batch_gemm(P, nb, ws, stream);
  if (rc == ED_OK) rc = elemental_run_batch_end(P, nb, blend, outs, ws, stream);
  return rc;
}

int elemental_run(const ed_elemental_plan* P, const void* links, long long dir_stride, long long site_stride,
                  int evec_prec, const void* evecs, const double* blend, void* out, void* ws, size_t ws_bytes,
                  cudaStream_t stream) {
  return elemental_run_batch(P, 1, &links, dir_stride, site_stride, evec_prec, &evecs, blend, &out, ws, ws_bytes,
                             stream);
}

}  // namespace ed

// ------------------------------------------------------------ C ABI

namespace ed {
// an arithmetic mode with at most one of the GEMM-form flags (no / forced / left factorisation) and the Gauss flag
bool mode_flags_valid(int mode) {
  const int form = mode & (ED_MODE_FLAG_NO_FACTOR | ED_MODE_FLAG_FORCE_FACTOR | ED_MODE_FLAG_LEFT_FACTOR);
  return mode_supported(mode & 0xff) &&
         (mode & ~(0xff | ED_MODE_FLAG_NO_FACTOR | ED_MODE_FLAG_FORCE_FACTOR | ED_MODE_FLAG_GAUSS |
                   ED_MODE_FLAG_LEFT_FACTOR)) == 0 &&
         (form & (form - 1)) == 0;
}
void set_mode_flags(ed_elemental_plan* P, int mode) {
  P->no_factor = (mode & ED_MODE_FLAG_NO_FACTOR) != 0;
  P->force_factor = (mode & ED_MODE_FLAG_FORCE_FACTOR) != 0;
  P->left_factor = (mode & ED_MODE_FLAG_LEFT_FACTOR) != 0;
  P->gauss = (mode & ED_MODE_FLAG_GAUSS) != 0;
}
}  // namespace ed

extern "C" int ed_elemental_plan_create(ed_elemental_plan** plan, int Lx, int Ly, int Lz, int Ne, int num_nabla,
                                        const int* moms, int nmom, int mode) {
  ED_CHECK_ARG(plan, "ed_elemental_plan_create: null plan pointer");
  *plan = nullptr;
  ED_CHECK_ARG(Lx > 0 && Ly > 0 && Lz > 0 && Ne > 0 && nmom > 0, "ed_elemental_plan_create: sizes must be positive");
  ED_CHECK_ARG(num_nabla >= 0 && num_nabla <= 2, "ed_elemental_plan_create: num_nabla must be 0, 1 or 2");
  ED_CHECK_ARG(moms, "ed_elemental_plan_create: null momentum list");
  ED_CHECK_ARG(ed::mode_flags_valid(mode), "ed_elemental_plan_create: unknown mode %d", mode);
  ED_CHECK_ARG((long long)Lx * Ly * Lz <= (1LL << 26), "ed_elemental_plan_create: lattice too large");
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

extern "C" int ed_elemental_plan_destroy(ed_elemental_plan* plan) {
  delete plan;
  return ED_OK;
}

extern "C" int ed_elemental_workspace_size(const ed_elemental_plan* plan, size_t* bytes) {
  ED_CHECK_ARG(plan && bytes, "ed_elemental_workspace_size: null pointer");
  *bytes = plan->ws_bytes;
  return ED_OK;
}

extern "C" int ed_elemental_num_pairs(const ed_elemental_plan* plan, int* npairs) {
  ED_CHECK_ARG(plan && npairs, "ed_elemental_num_pairs: null pointer");
  *npairs = plan->npairs;
  return ED_OK;
}

extern "C" int ed_elemental_run(const ed_elemental_plan* plan, const void* links, long long dir_stride,
                                long long site_stride, int evec_prec, const void* evecs, const double* blend,
                                void* out, void* workspace, size_t workspace_bytes, void* stream) {
  ED_CHECK_ARG(plan && !plan->custom, "ed_elemental_run: needs a plan from ed_elemental_plan_create");
  ED_CHECK_ARG(links && evecs && out && workspace, "ed_elemental_run: null pointer");
  ED_CHECK_ARG(evec_prec == ED_C128 || evec_prec == ED_C64, "ed_elemental_run: bad eigenvector precision");
  ED_CHECK_ARG(dir_stride >= 0 && site_stride >= 0, "ed_elemental_run: negative stride");
  ED_CHECK_ARG(((uintptr_t)workspace % 256) == 0, "ed_elemental_run: workspace must be 256-byte aligned");
  if (workspace_bytes < plan->ws_bytes) {
    ed::set_error("ed_elemental_run: workspace of %zu bytes is smaller than the %zu the plan needs", workspace_bytes,
                  plan->ws_bytes);
    return ED_ERR_WORKSPACE;
  }
  return ed::elemental_run(plan, links, dir_stride, site_stride, evec_prec, evecs, blend, out, workspace,
                           workspace_bytes, (cudaStream_t)stream);
}

extern "C" int ed_elemental_status(const ed_elemental_plan* plan, const void* workspace, int* code, void* stream) {
  ED_CHECK_ARG(plan && workspace && code, "ed_elemental_status: null pointer");
  int rc = ed::tc_read_status(plan, workspace, code, (cudaStream_t)stream);
  if (rc != ED_OK) return rc;
  if (*code == 7) {  // TC_ERR_CLUSTER: an SM-pair GEMM ran without its two-CTA cluster and stopped at once
    ed::set_error("elemental: the SM-pair GEMM was launched without its two-CTA cluster; the output is invalid");
    return ED_ERR_CUDA;
  }
  if (*code != 0) {
    ed::set_error("elemental: a bounded device wait gave up (code %d); the output of that run is invalid", *code);
    return ED_ERR_TIMEOUT;
  }
  return ED_OK;
}

extern "C" int ed_elemental_set_profile_events(ed_elemental_plan* plan, void* start, void* stop) {
  ED_CHECK_ARG(plan, "ed_elemental_set_profile_events: null plan");
  ED_CHECK_ARG((start == nullptr) == (stop == nullptr), "ed_elemental_set_profile_events: give both events or none");
  plan->prof_start = (cudaEvent_t)start;
  plan->prof_stop = (cudaEvent_t)stop;
  return ED_OK;
}

extern "C" int ed_elemental_describe(const ed_elemental_plan* plan, int* ngroups, int* left, int* nright, int* herm) {
  ED_CHECK_ARG(plan && ngroups && herm, "ed_elemental_describe: null pointer");
  *ngroups = (int)plan->jobs.size();
  *herm = plan->herm ? 1 : 0;
  for (size_t g = 0; g < plan->jobs.size(); ++g) {
    if (left) left[g] = plan->jobs[g].left;
    if (nright) nright[g] = plan->jobs[g].nright;
  }
  return ED_OK;
}

extern "C" int ed_elemental_factorised(const ed_elemental_plan* plan, int* factorised, int* pxy, int* pz) {
  ED_CHECK_ARG(plan && factorised, "ed_elemental_factorised: null pointer");
  *factorised = plan->fac ? 1 : 0;
  if (pxy) *pxy = plan->fac_pxy;
  if (pz) *pz = plan->fac_pz;
  return ED_OK;
}

extern "C" int ed_elemental_set_tuning(ed_elemental_plan* plan, int key, int value) {
  ED_CHECK_ARG(plan, "ed_elemental_set_tuning: null plan");
  switch (key) {
    case ED_TUNE_F64_TILE:
      ED_CHECK_ARG(value >= 0 && value <= 3, "ed_elemental_set_tuning: FP64 tile shape %d not in 0..3", value);
      plan->f64_tile = value;
      return ED_OK;
    case ED_TUNE_TC_SLAB_KB:
      ED_CHECK_ARG(value >= 0 && value <= TC_FLUSH_KB && (value & (value - 1)) == 0,
                   "ed_elemental_set_tuning: slab of %d k-blocks (need 0 or a power of two <= %d)", value,
                   TC_FLUSH_KB);
      plan->tc_slab_kb = value;
      return ED_OK;
    case ED_TUNE_TC_GRID:
      ED_CHECK_ARG(value >= 0 && value <= (1 << 20), "ed_elemental_set_tuning: grid of %d CTAs", value);
      plan->tc_grid = value;
      return ED_OK;
    case ED_TUNE_TC_STAGES:
      ED_CHECK_ARG(value == 0 || value == 2 || value == 3 || value == 4,
                   "ed_elemental_set_tuning: %d stages (0, 2, 3 or 4)", value);
      plan->tc_stages = value;
      return ED_OK;
    case ED_TUNE_TC_PAIR:
      ED_CHECK_ARG(value >= 0 && value <= 3, "ed_elemental_set_tuning: SM pairing %d (0, 1, 2 or 3)", value);
      plan->tc_pair = value;
      // the stacked SM-pair form keeps a second double-float plane: the workspace size follows the setting
      // (query it again; a run with a smaller workspace is refused with ED_ERR_WORKSPACE)
      plan->ws_bytes = plan->off_extra + ed::tc_extra_workspace(plan) + ed::f64_extra_workspace(plan);
      return ED_OK;
    case ED_TUNE_TC_KPB:
      ED_CHECK_ARG(value == 0 || value == 1 || value == 2 || value == 4,
                   "ed_elemental_set_tuning: %d k-blocks per TMEM buffer (0, 1, 2 or 4)", value);
      plan->tc_kpb = value;
      return ED_OK;
    case ED_TUNE_TC_STACK:
      ED_CHECK_ARG(value >= 0 && value <= 2, "ed_elemental_set_tuning: operand form %d (0, 1 or 2)", value);
      plan->tc_stack = value;
      return ED_OK;
    case ED_TUNE_F64_DF:
      ED_CHECK_ARG(value == 0 || value == 1, "ed_elemental_set_tuning: double-float switch %d (0 or 1)", value);
      plan->f64_df = value;
      return ED_OK;
    default:
      ED_CHECK_ARG(false, "ed_elemental_set_tuning: unknown key %d", key);
  }
  return ED_ERR_ARG;
}

extern "C" int ed_elemental_get_tuning(const ed_elemental_plan* plan, int key, int* value) {
  ED_CHECK_ARG(plan && value, "ed_elemental_get_tuning: null pointer");
  switch (key) {
    case ED_TUNE_F64_TILE:
      *value = plan->f64_tile;
      return ED_OK;
    case ED_TUNE_TC_SLAB_KB:
      *value = plan->tc_slab_kb;
      return ED_OK;
    case ED_TUNE_TC_GRID:
      *value = plan->tc_grid;
      return ED_OK;
    case ED_TUNE_TC_STAGES:
      *value = plan->tc_stages;
      return ED_OK;
    case ED_TUNE_TC_PAIR:
      *value = plan->tc_pair;
      return ED_OK;
    case ED_TUNE_TC_KPB:
      *value = plan->tc_kpb;
      return ED_OK;
    case ED_TUNE_TC_STACK:
      *value = plan->tc_stack;
      return ED_OK;
    case ED_TUNE_F64_DF:
      *value = plan->f64_df;
      return ED_OK;
    default:
      ED_CHECK_ARG(false, "ed_elemental_get_tuning: unknown key %d", key);
  }
  return ED_ERR_ARG;
}

// ------------------------------------------------------------ generic pair contractions
// G_p[i][r*Ne + j] = sum_k conj(X_i[k]) phase_p(k) Y_{right0+r, j}[k] for caller-built
// chains (colour planes), e.g. the displaced vectors of the displacement elemental.

namespace ed {
static int pair_plan_build(ed_elemental_plan* P, int left, int right0, int nright) {
  P->V3 = P->Lx * P->Ly * P->Lz;
  P->nderiv = 0;
  P->custom = true;
  P->negidx.assign(P->nmom, -1);
  P->herm = false;
  P->jobs.clear();
  Job j;
  j.left = left;
  j.right0 = right0;
  j.nright = nright;
  j.g_off = 0;
  P->jobs.push_back(j);
  P->g_elems = (long long)P->nmom * P->Ne * nright * P->Ne;
  P->terms.clear();
  P->term_start.assign(1, 0);
  P->npairs = nright;
  P->nbatch = 1;
  P->jobs_per_t = 1;
  P->g_per_t = P->g_elems;
  auto up = [](size_t v) { return (v + 255) / 256 * 256; };
  P->off_links = P->off_links32 = P->off_chain = P->off_g = 0;
  P->off_phase = 0;
  size_t off = up((size_t)P->nmom * P->V3 * 16);
  P->off_extra = off;
  P->ws_bytes = off;  // tc_plan_check adds the tensor-core extra below
  return ED_OK;
}
}  // namespace ed

extern "C" int ed_pair_plan_create(ed_elemental_plan** plan, int Lx, int Ly, int Lz, int Ne, int nchain,
                                   const int* moms, int nmom, int mode, int left, int right0, int nright) {
  ED_CHECK_ARG(plan, "ed_pair_plan_create: null plan pointer");
  *plan = nullptr;
  ED_CHECK_ARG(Lx > 0 && Ly > 0 && Lz > 0 && Ne > 0 && nmom > 0 && nchain > 0 && nright > 0,
               "ed_pair_plan_create: sizes must be positive");
  ED_CHECK_ARG(ed::lattice_ok(Lx, Ly, Lz), "ed_pair_plan_create: Lx*Ly*Lz above 2^28");
  ED_CHECK_ARG(left >= 0 && left < nchain && right0 >= 0 && right0 + nright <= nchain,
               "ed_pair_plan_create: chain indices out of range");
  ED_CHECK_ARG(moms, "ed_pair_plan_create: null momentum list");
  ED_CHECK_ARG(ed::mode_supported(mode), "ed_pair_plan_create: unknown mode %d", mode);
  auto* P = new ed_elemental_plan();
  P->Lx = Lx;
  P->Ly = Ly;
  P->Lz = Lz;
  P->Ne = Ne;
  P->num_nabla = 0;
  P->nmom = nmom;
  P->mode = mode;
  P->use_herm = false;
  P->nchain = nchain;
  P->moms.assign(moms, moms + 3 * nmom);
  int rc = ed::pair_plan_build(P, left, right0, nright);
  if (rc == ED_OK) rc = ed::tc_plan_check(P);
  if (rc == ED_OK) P->ws_bytes = P->off_extra + ed::tc_extra_workspace(P) + ed::f64_extra_workspace(P);
  if (rc != ED_OK) {
    delete P;
    return rc;
  }
  *plan = P;
  return ED_OK;
}

extern "C" int ed_pair_run(const ed_elemental_plan* plan, const void* chains, void* G, void* workspace,
                           size_t workspace_bytes, void* stream) {
  ED_CHECK_ARG(plan && plan->custom, "ed_pair_run: needs a plan from ed_pair_plan_create");
  ED_CHECK_ARG(chains && G && workspace, "ed_pair_run: null pointer");
  ED_CHECK_ARG(((uintptr_t)workspace % 256) == 0, "ed_pair_run: workspace must be 256-byte aligned");
  if (workspace_bytes < plan->ws_bytes) {
    ed::set_error("ed_pair_run: workspace of %zu bytes is smaller than the %zu the plan needs", workspace_bytes,
                  plan->ws_bytes);
    return ED_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  char* W = (char*)workspace;
  ed::cplx<double>* phases = (ed::cplx<double>*)(W + plan->off_phase);
  int rc = ed::launch_phases(ed::Latt{plan->Lx, plan->Ly, plan->Lz}, plan->moms.data(), plan->nmom, phases, s);
  if (rc) return rc;
  if (plan->mode == ED_MODE_FP64)
    return ed::launch_pair_gemm_f64(plan, (const ed::cplx<double>*)chains, phases, (ed::cplx<double>*)G, s, 1,
                                    W + plan->off_extra);
  return ed::launch_pair_gemm_tc(plan, (const ed::cplx<float>*)chains, phases, (ed::cplx<double>*)G,
                                 W + plan->off_extra, s, 1);
}
