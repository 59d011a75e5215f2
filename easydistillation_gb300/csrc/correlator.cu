// Meson two-point contraction of one source timeslice (the einsum
// "tijab,xjk,xtbc,tklcd,yli,yad->t" of lattice/correlator/one_particle.py:64-72).
//
// Every gamma matrix of the reference's insertion table is monomial (one
// non-zero per row), so with tau_bw(t)[i][j] = g5_ii g5_jj conj(taub(t)[j][i])^T
// (one_particle.py:59-63) the contraction of one operator is a sum of terms
//   coef * Tr[ A phi_x(t) B psi_y^T ],  A = conj(taub(t)[j][i])^T,  B = tau(t)[k][l],
//   phi_x(t) = E_x(t_src + t),  psi_y = conj(E_y(t_src)),
// one per (part x, part y, spin i, spin k), with j and l fixed by the gammas
// and coef the product of the two gamma entries and the two g5 signs (the host
// builds the term table).  One CTA computes a 32 x 32 tile (a, c) of both
// P = A phi and Q = B psi^T for one (term, t) and adds coef * sum_{a,c} P[a,c] Q[c,a]
// into out[t]: neither product goes to HBM.  256 threads as 16 x 16, each owning
// 2 x 2 (a, c) pairs; the Ne-long reductions run in stages of 16 through shared
// memory.  FP64 throughout (the FP64 pipe bounds it).

#include "common.cuh"

namespace ed {
namespace {

constexpr int TP_T = 32, TP_K = 16;

__global__ void __launch_bounds__(256) twopoint_trace_kernel(int Ne, int Lt, int t_src, int nparts,
                                                             const int* __restrict__ idx,
                                                             const double2* __restrict__ coef,
                                                             const cplx<double>* __restrict__ tau,
                                                             const cplx<double>* __restrict__ taub,
                                                             const cplx<double>* __restrict__ el,
                                                             double2* __restrict__ out) {
  __shared__ cplx<double> As[TP_T][TP_K + 1];  // A[a][r] = conj(taub[t][j][i][r][a])
  __shared__ cplx<double> Ps[TP_K][TP_T + 1];  // phi[r][c]
  __shared__ cplx<double> Bs[TP_T][TP_K + 1];  // B[c][r] = tau[t][k][l][c][r]
  __shared__ cplx<double> Qs[TP_T][TP_K + 1];  // psi[a][r] = conj(E_y(t_src)[a][r])
  __shared__ double red[2][8];
  const int e = blockIdx.y, t = blockIdx.z;
  const int ntile = (Ne + TP_T - 1) / TP_T;
  const int a0 = (blockIdx.x / ntile) * TP_T, c0 = (blockIdx.x % ntile) * TP_T;
  const int x = idx[6 * e], y = idx[6 * e + 1], i = idx[6 * e + 2], j = idx[6 * e + 3], k = idx[6 * e + 4],
            l = idx[6 * e + 5];
  // a term naming a part or spin index out of range contributes nothing
  if (x < 0 || x >= nparts || y < 0 || y >= nparts || (unsigned)i > 3u || (unsigned)j > 3u || (unsigned)k > 3u ||
      (unsigned)l > 3u)
    return;
  const long long blk = (long long)Ne * Ne;
  const cplx<double>* Ablk = taub + (((long long)t * 4 + j) * 4 + i) * blk;  // taub[t][j][i]
  const cplx<double>* Bblk = tau + (((long long)t * 4 + k) * 4 + l) * blk;   // tau[t][k][l]
  const cplx<double>* phi = el + ((long long)x * Lt + (t_src + t) % Lt) * blk;
  const cplx<double>* psi = el + ((long long)y * Lt + t_src) * blk;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  cplx<double> P[2][2], Q[2][2];
#pragma unroll
  for (int u = 0; u < 2; ++u)
#pragma unroll
    for (int v = 0; v < 2; ++v) P[u][v] = Q[u][v] = mk(0.0, 0.0);
  for (int r0 = 0; r0 < Ne; r0 += TP_K) {
    // stage the 16-long slices: two elements per thread and array
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int lin = tid + 256 * q;  // 0..511
      {  // As / Qs: 32 rows (a) x 16 (r); A read column-wise from taub (a fastest in memory)
        const int al = lin & 31, r = lin >> 5, a = a0 + al, rr = r0 + r;
        cplx<double> v = mk(0.0, 0.0), w = mk(0.0, 0.0);
        if (a < Ne && rr < Ne) {
          const cplx<double> av = ld(Ablk + (long long)rr * Ne + a);
          v = mk(av.re, -av.im);
        }
        As[al][r] = v;
        const int al2 = lin >> 4, r2 = lin & 15, a2 = a0 + al2, rr2 = r0 + r2;
        if (a2 < Ne && rr2 < Ne) {
          const cplx<double> pv = ld(psi + (long long)a2 * Ne + rr2);
          w = mk(pv.re, -pv.im);
        }
        Qs[al2][r2] = w;
      }
      {  // Ps: 16 (r) x 32 (c), phi rows; Bs: 32 (c) x 16 (r), tau rows
        const int cl = lin & 31, r = lin >> 5, c = c0 + cl, rr = r0 + r;
        Ps[r][cl] = (c < Ne && rr < Ne) ? ld(phi + (long long)rr * Ne + c) : mk(0.0, 0.0);
        const int cl2 = lin >> 4, r2 = lin & 15, c2 = c0 + cl2, rr2 = r0 + r2;
        Bs[cl2][r2] = (c2 < Ne && rr2 < Ne) ? ld(Bblk + (long long)c2 * Ne + rr2) : mk(0.0, 0.0);
      }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < TP_K; ++r) {
      cplx<double> av[2], pv[2], bv[2], qv[2];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        av[u] = As[ty + 16 * u][r];
        qv[u] = Qs[ty + 16 * u][r];
        pv[u] = Ps[r][tx + 16 * u];
        bv[u] = Bs[tx + 16 * u][r];
      }
#pragma unroll
      for (int u = 0; u < 2; ++u)
#pragma unroll
        for (int v = 0; v < 2; ++v) {
          cfma(P[u][v], av[u], pv[v]);  // P[a_u][c_v] += A[a_u][r] phi[r][c_v]
          cfma(Q[u][v], bv[v], qv[u]);  // Q[c_v][a_u] += B[c_v][r] psi[a_u][r]
        }
    }
    __syncthreads();
  }
  double sre = 0.0, sim = 0.0;
#pragma unroll
  for (int u = 0; u < 2; ++u)
#pragma unroll
    for (int v = 0; v < 2; ++v) {
      const cplx<double> pr = P[u][v] * Q[u][v];
      sre += pr.re;
      sim += pr.im;
    }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sre += __shfl_xor_sync(0xffffffffu, sre, o);
    sim += __shfl_xor_sync(0xffffffffu, sim, o);
  }
  if ((tid & 31) == 0) {
    red[0][tid >> 5] = sre;
    red[1][tid >> 5] = sim;
  }
  __syncthreads();
  if (tid == 0) {
    double tr = 0.0, ti = 0.0;
    for (int w = 0; w < 8; ++w) {
      tr += red[0][w];
      ti += red[1][w];
    }
    const double2 cf = coef[e];
    atomicAdd(&out[t].x, cf.x * tr - cf.y * ti);
    atomicAdd(&out[t].y, cf.x * ti + cf.y * tr);
  }
}

}  // namespace
}  // namespace ed

extern "C" int ed_twopoint_trace(int T, int Ne, int Lt, int t_src, int nparts, int nterm, const int* term_idx,
                                 const double* term_coef, const void* tau, const void* taub, const void* el,
                                 void* out, void* stream) {
  ED_CHECK_ARG(T > 0 && Ne > 0 && Lt > 0 && nparts > 0 && nterm >= 0, "ed_twopoint_trace: sizes must be positive");
  ED_CHECK_ARG(T <= 65535 && nterm <= 65535, "ed_twopoint_trace: at most 65535 sink times and terms");
  ED_CHECK_ARG(t_src >= 0 && t_src < Lt, "ed_twopoint_trace: source timeslice out of range");
  ED_CHECK_ARG(term_idx && term_coef && tau && taub && el && out, "ed_twopoint_trace: null pointer");
  ED_CHECK_ARG(((uintptr_t)tau % 16) == 0 && ((uintptr_t)taub % 16) == 0 && ((uintptr_t)el % 16) == 0 &&
                   ((uintptr_t)out % 16) == 0 && ((uintptr_t)term_coef % 16) == 0,
               "ed_twopoint_trace: complex buffers must be 16-byte aligned");
  if (nterm == 0) return ED_OK;
  const int ntile = ed::ceil_div(Ne, ed::TP_T);
  dim3 grid((unsigned)(ntile * ntile), (unsigned)nterm, (unsigned)T);
  ed::twopoint_trace_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(
      Ne, Lt, t_src, nparts, term_idx, (const double2*)term_coef, (const ed::cplx<double>*)tau,
      (const ed::cplx<double>*)taub, (const ed::cplx<double>*)el, (double2*)out);
  ED_RETURN_LAUNCH("two-point trace");
  return ED_OK;
}
