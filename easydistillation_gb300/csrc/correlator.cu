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

// ---------------------------------------------------------------- two-point profile
// The eigenvector-resolved form of the same contraction (one_particle.py:80-135):
//   out[t][a][d] = sum_terms coef (A phi_x(t) B)[a][d] psi_y[a][d]
// with the terms, A and B of the trace kernel above and phi_x(t) = E_x(sink_t[t]).  The coefficient
// factorises, coef = lc[k][x] rc[i][y] (lc = gamma_x[j][k] g5[j], rc = G_y[l][i] g5[i], j = j(x, k) the row of
// gamma_x holding column k, l = l(y, i) the row of G_y holding column i), so
//   L[t][i][k] = sum_x lc[k][x] A_{i, j(x,k)}(t) phi_x(t)                     (profile_left_kernel)
//   out[t]     = sum_{i,y} rc[i][y] psi_y o (sum_k L[t][i][k] B_{k, l(y,i)}(t))   (profile_right_kernel)
// where o is the elementwise product: 16 left blocks of X Ne^3 and up to 16 right blocks of 4 Ne^3 per sink
// time.  Both are FP64 tiled GEMMs with the layout of twopoint_trace_kernel (32 x 32 tiles, 16-deep stages, 2 x
// 2 results per thread); the right kernel keeps the output tile in registers over every (i, l), so the result
// is written once, without atomics.

__global__ void __launch_bounds__(256) profile_left_kernel(int Ne, int nparts, const int* __restrict__ sink_t,
                                                           const int* __restrict__ ltab,
                                                           const double2* __restrict__ lcoef,
                                                           const cplx<double>* __restrict__ taub,
                                                           const cplx<double>* __restrict__ el, int Lt,
                                                           cplx<double>* __restrict__ L) {
  __shared__ cplx<double> As[TP_T][TP_K + 1];  // coef * A[a][r] = coef * conj(taub[t][j][i][r][a])
  __shared__ cplx<double> Ps[TP_K][TP_T + 1];  // phi_x[r][c]
  const int ik = blockIdx.y, i = ik >> 2, k = ik & 3, t = blockIdx.z;
  const int ntile = (Ne + TP_T - 1) / TP_T;
  const int a0 = (blockIdx.x / ntile) * TP_T, c0 = (blockIdx.x % ntile) * TP_T;
  const long long blk = (long long)Ne * Ne;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  cplx<double> P[2][2];
#pragma unroll
  for (int u = 0; u < 2; ++u)
#pragma unroll
    for (int v = 0; v < 2; ++v) P[u][v] = mk(0.0, 0.0);
  for (int x = 0; x < nparts; ++x) {
    const int j = ltab[k * nparts + x];
    if ((unsigned)j > 3u) continue;
    const double2 cf = lcoef[k * nparts + x];
    const cplx<double> cfx = mk(cf.x, cf.y);
    const cplx<double>* Ablk = taub + (((long long)t * 4 + j) * 4 + i) * blk;
    const cplx<double>* phi = el + ((long long)x * Lt + sink_t[t]) * blk;
    for (int r0 = 0; r0 < Ne; r0 += TP_K) {
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int lin = tid + 256 * q;
        {
          const int al = lin & 31, r = lin >> 5, a = a0 + al, rr = r0 + r;
          cplx<double> v = mk(0.0, 0.0);
          if (a < Ne && rr < Ne) {
            const cplx<double> av = ld(Ablk + (long long)rr * Ne + a);
            v = cfx * mk(av.re, -av.im);
          }
          As[al][r] = v;
        }
        {
          const int cl = lin & 31, r = lin >> 5, c = c0 + cl, rr = r0 + r;
          Ps[r][cl] = (c < Ne && rr < Ne) ? ld(phi + (long long)rr * Ne + c) : mk(0.0, 0.0);
        }
      }
      __syncthreads();
#pragma unroll
      for (int r = 0; r < TP_K; ++r) {
        cplx<double> av[2], pv[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          av[u] = As[ty + 16 * u][r];
          pv[u] = Ps[r][tx + 16 * u];
        }
#pragma unroll
        for (int u = 0; u < 2; ++u)
#pragma unroll
          for (int v = 0; v < 2; ++v) cfma(P[u][v], av[u], pv[v]);
      }
      __syncthreads();
    }
  }
  cplx<double>* Lb = L + ((long long)t * 16 + ik) * blk;
#pragma unroll
  for (int u = 0; u < 2; ++u)
#pragma unroll
    for (int v = 0; v < 2; ++v) {
      const int a = a0 + ty + 16 * u, c = c0 + tx + 16 * v;
      if (a < Ne && c < Ne) Lb[(long long)a * Ne + c] = P[u][v];
    }
}

__global__ void __launch_bounds__(256) profile_right_kernel(int Ne, int nparts, int Lt, int t_src,
                                                            const int* __restrict__ rtab,
                                                            const double2* __restrict__ rcoef,
                                                            const cplx<double>* __restrict__ L,
                                                            const cplx<double>* __restrict__ tau,
                                                            const cplx<double>* __restrict__ el,
                                                            double2* __restrict__ out) {
  __shared__ cplx<double> Ls[TP_T][TP_K + 1];  // L[t][i][k][a][r]
  __shared__ cplx<double> Bs[TP_K][TP_T + 1];  // tau[t][k][l][r][d]
  const int t = blockIdx.z;
  const int ntile = (Ne + TP_T - 1) / TP_T;
  const int a0 = (blockIdx.x / ntile) * TP_T, d0 = (blockIdx.x % ntile) * TP_T;
  const long long blk = (long long)Ne * Ne;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  cplx<double> acc[2][2];
#pragma unroll
  for (int u = 0; u < 2; ++u)
#pragma unroll
    for (int v = 0; v < 2; ++v) acc[u][v] = mk(0.0, 0.0);
  for (int i = 0; i < 4; ++i) {
    for (int l = 0; l < 4; ++l) {
      bool used = false;  // some source part y has l(y, i) == l (uniform over the block)
      for (int y = 0; y < nparts; ++y) used |= rtab[i * nparts + y] == l;
      if (!used) continue;
      cplx<double> Q[2][2];
#pragma unroll
      for (int u = 0; u < 2; ++u)
#pragma unroll
        for (int v = 0; v < 2; ++v) Q[u][v] = mk(0.0, 0.0);
      for (int k = 0; k < 4; ++k) {
        const cplx<double>* Lb = L + ((long long)t * 16 + i * 4 + k) * blk;
        const cplx<double>* Bb = tau + (((long long)t * 4 + k) * 4 + l) * blk;
        for (int r0 = 0; r0 < Ne; r0 += TP_K) {
#pragma unroll
          for (int q = 0; q < 2; ++q) {
            const int lin = tid + 256 * q;
            {
              const int al = lin >> 4, r = lin & 15, a = a0 + al, rr = r0 + r;
              Ls[al][r] = (a < Ne && rr < Ne) ? ld(Lb + (long long)a * Ne + rr) : mk(0.0, 0.0);
            }
            {
              const int dl = lin & 31, r = lin >> 5, d = d0 + dl, rr = r0 + r;
              Bs[r][dl] = (d < Ne && rr < Ne) ? ld(Bb + (long long)rr * Ne + d) : mk(0.0, 0.0);
            }
          }
          __syncthreads();
#pragma unroll
          for (int r = 0; r < TP_K; ++r) {
            cplx<double> lv[2], bv[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
              lv[u] = Ls[ty + 16 * u][r];
              bv[u] = Bs[r][tx + 16 * u];
            }
#pragma unroll
            for (int u = 0; u < 2; ++u)
#pragma unroll
              for (int v = 0; v < 2; ++v) cfma(Q[u][v], lv[u], bv[v]);
          }
          __syncthreads();
        }
      }
      // acc += sum over the source parts y with l(y, i) == l of rc[i][y] psi_y o Q
      for (int y = 0; y < nparts; ++y) {
        if (rtab[i * nparts + y] != l) continue;
        const double2 cf = rcoef[i * nparts + y];
        const cplx<double> cfy = mk(cf.x, cf.y);
        const cplx<double>* src = el + ((long long)y * Lt + t_src) * blk;
#pragma unroll
        for (int u = 0; u < 2; ++u)
#pragma unroll
          for (int v = 0; v < 2; ++v) {
            const int a = a0 + ty + 16 * u, d = d0 + tx + 16 * v;
            if (a < Ne && d < Ne) {
              const cplx<double> pv = ld(src + (long long)a * Ne + d);
              acc[u][v] = acc[u][v] + cfy * mk(pv.re, -pv.im) * Q[u][v];
            }
          }
      }
    }
  }
  double2* o = out + (long long)t * blk;
#pragma unroll
  for (int u = 0; u < 2; ++u)
#pragma unroll
    for (int v = 0; v < 2; ++v) {
      const int a = a0 + ty + 16 * u, d = d0 + tx + 16 * v;
      if (a < Ne && d < Ne) o[(long long)a * Ne + d] = make_double2(acc[u][v].re, acc[u][v].im);
    }
}

// The diagonal profile (is_diagonal, one_particle.py:113-121):
//   out[t][a] = sum_terms coef psi_y[a][a] sum_b conj(taub[t][j][i][b][a]) phi_x(t)[b][b] tau[t][k][l][b][a]
// one warp per (t, a), lanes over b, every term of the table in turn.
__global__ void __launch_bounds__(256) profile_diag_kernel(int Ne, int Lt, int t_src, int nparts, int nterm,
                                                           const int* __restrict__ sink_t,
                                                           const int* __restrict__ idx,
                                                           const double2* __restrict__ coef,
                                                           const cplx<double>* __restrict__ tau,
                                                           const cplx<double>* __restrict__ taub,
                                                           const cplx<double>* __restrict__ el,
                                                           double2* __restrict__ out) {
  const int t = blockIdx.y;
  const int a = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (a >= Ne) return;
  const long long blk = (long long)Ne * Ne;
  cplx<double> tot = mk(0.0, 0.0);
  for (int e = 0; e < nterm; ++e) {
    const int x = idx[6 * e], y = idx[6 * e + 1], i = idx[6 * e + 2], j = idx[6 * e + 3], k = idx[6 * e + 4],
              l = idx[6 * e + 5];
    if (x < 0 || x >= nparts || y < 0 || y >= nparts || (unsigned)i > 3u || (unsigned)j > 3u || (unsigned)k > 3u ||
        (unsigned)l > 3u)
      continue;
    const cplx<double>* Ab = taub + (((long long)t * 4 + j) * 4 + i) * blk;
    const cplx<double>* Bb = tau + (((long long)t * 4 + k) * 4 + l) * blk;
    const cplx<double>* phi = el + ((long long)x * Lt + sink_t[t]) * blk;
    cplx<double> s = mk(0.0, 0.0);
    for (int b = lane; b < Ne; b += 32) {
      const cplx<double> av = ld(Ab + (long long)b * Ne + a);
      s = s + mk(av.re, -av.im) * ld(phi + (long long)b * Ne + b) * ld(Bb + (long long)b * Ne + a);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      s.re += __shfl_xor_sync(0xffffffffu, s.re, o);
      s.im += __shfl_xor_sync(0xffffffffu, s.im, o);
    }
    const double2 cf = coef[e];
    const cplx<double> pv = ld(el + ((long long)y * Lt + t_src) * blk + (long long)a * Ne + a);
    tot = tot + mk(cf.x, cf.y) * mk(pv.re, -pv.im) * s;
  }
  if (lane == 0) out[(long long)t * Ne + a] = make_double2(tot.re, tot.im);
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

extern "C" int ed_twopoint_profile(int T, int Ne, int Lt, int t_src, int nparts, const int* sink_t, const int* ltab,
                                   const double* lcoef, const int* rtab, const double* rcoef, const void* tau,
                                   const void* taub, const void* el, void* work, void* out, void* stream) {
  ED_CHECK_ARG(T > 0 && Ne > 0 && Lt > 0 && nparts > 0, "ed_twopoint_profile: sizes must be positive");
  ED_CHECK_ARG(T <= 65535, "ed_twopoint_profile: at most 65535 sink times");
  ED_CHECK_ARG(t_src >= 0 && t_src < Lt, "ed_twopoint_profile: source timeslice out of range");
  ED_CHECK_ARG(sink_t && ltab && lcoef && rtab && rcoef && tau && taub && el && work && out,
               "ed_twopoint_profile: null pointer");
  ED_CHECK_ARG(((uintptr_t)tau % 16) == 0 && ((uintptr_t)taub % 16) == 0 && ((uintptr_t)el % 16) == 0 &&
                   ((uintptr_t)work % 16) == 0 && ((uintptr_t)out % 16) == 0 && ((uintptr_t)lcoef % 16) == 0 &&
                   ((uintptr_t)rcoef % 16) == 0,
               "ed_twopoint_profile: complex buffers must be 16-byte aligned");
  const int ntile = ed::ceil_div(Ne, ed::TP_T);
  cudaStream_t st = (cudaStream_t)stream;
  ed::profile_left_kernel<<<dim3((unsigned)(ntile * ntile), 16, (unsigned)T), 256, 0, st>>>(
      Ne, nparts, sink_t, ltab, (const double2*)lcoef, (const ed::cplx<double>*)taub, (const ed::cplx<double>*)el, Lt,
      (ed::cplx<double>*)work);
  ED_RETURN_LAUNCH("two-point profile, left blocks");
  ed::profile_right_kernel<<<dim3((unsigned)(ntile * ntile), 1, (unsigned)T), 256, 0, st>>>(
      Ne, nparts, Lt, t_src, rtab, (const double2*)rcoef, (const ed::cplx<double>*)work,
      (const ed::cplx<double>*)tau, (const ed::cplx<double>*)el, (double2*)out);
  ED_RETURN_LAUNCH("two-point profile, right blocks");
  return ED_OK;
}

extern "C" int ed_twopoint_profile_diag(int T, int Ne, int Lt, int t_src, int nparts, int nterm, const int* sink_t,
                                        const int* term_idx, const double* term_coef, const void* tau,
                                        const void* taub, const void* el, void* out, void* stream) {
  ED_CHECK_ARG(T > 0 && Ne > 0 && Lt > 0 && nparts > 0 && nterm >= 0, "ed_twopoint_profile_diag: bad sizes");
  ED_CHECK_ARG(T <= 65535, "ed_twopoint_profile_diag: at most 65535 sink times");
  ED_CHECK_ARG(t_src >= 0 && t_src < Lt, "ed_twopoint_profile_diag: source timeslice out of range");
  ED_CHECK_ARG(sink_t && term_idx && term_coef && tau && taub && el && out, "ed_twopoint_profile_diag: null pointer");
  ED_CHECK_ARG(((uintptr_t)tau % 16) == 0 && ((uintptr_t)taub % 16) == 0 && ((uintptr_t)el % 16) == 0 &&
                   ((uintptr_t)out % 16) == 0 && ((uintptr_t)term_coef % 16) == 0,
               "ed_twopoint_profile_diag: complex buffers must be 16-byte aligned");
  ed::profile_diag_kernel<<<dim3((unsigned)ed::ceil_div(Ne, 8), (unsigned)T), 256, 0, (cudaStream_t)stream>>>(
      Ne, Lt, t_src, nparts, nterm, sink_t, term_idx, (const double2*)term_coef, (const ed::cplx<double>*)tau,
      (const ed::cplx<double>*)taub, (const ed::cplx<double>*)el, (double2*)out);
  ED_RETURN_LAUNCH("two-point diagonal profile");
  return ED_OK;
}
