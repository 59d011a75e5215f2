// Link gradients of the covariant-derivative hop and of the Laplacian.
//
// With the loss convention dL = Re sum conj(grad) dX (torch's complex
// autograd), a stencil term  W(x) += alpha * U_d(x) F(x+d)  contributes
// alpha * Wbar(x) F(x+d)^dag to grad U_d(x), and a term
// W(x) += beta * U_d(x-d)^dag F(x-d) contributes beta * F(x) Wbar(x+d)^dag,
// summed over the vectors.  The covariant-derivative hop of
// lattice/generator/elemental.py:282-287 has (alpha, beta) = (1, -1); the
// Laplacian of lattice/generator/eigenvector.py:11-26 has (-1, -1).
// One thread per site accumulates the 3x3 outer products of all vectors into
// the SoA gradient [dir][row][col][V3] (read-modify-write, no atomics: each
// site's link belongs to one thread).
#include "common.cuh"

namespace ed {

__global__ void __launch_bounds__(128) link_grad_kernel(Latt L, int d, int nvec, double alpha, double beta,
                                                        const cplx<double>* __restrict__ wbar,
                                                        const cplx<double>* __restrict__ f,
                                                        cplx<double>* __restrict__ grad) {
  const int V3 = L.V3();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= V3) return;
  const int x = s % L.Lx, y = (s / L.Lx) % L.Ly, z = s / (L.Lx * L.Ly);
  int sp;
  if (d == 0)
    sp = s - x + wrap_inc(x, L.Lx);
  else if (d == 1)
    sp = s + (wrap_inc(y, L.Ly) - y) * L.Lx;
  else
    sp = s + (wrap_inc(z, L.Lz) - z) * L.Lx * L.Ly;
  cplx<double> g[9];
#pragma unroll
  for (int e = 0; e < 9; ++e) g[e] = mk(0.0, 0.0);
  for (int v = 0; v < nvec; ++v) {
    const cplx<double>* Wv = wbar + (long long)v * 3 * V3;
    const cplx<double>* Fv = f + (long long)v * 3 * V3;
    cplx<double> w0[3], fp[3], f0[3], wp[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      w0[c] = ld(Wv + c * V3 + s);
      fp[c] = ld(Fv + c * V3 + sp);
      f0[c] = ld(Fv + c * V3 + s);
      wp[c] = ld(Wv + c * V3 + sp);
    }
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        // alpha * w0[a] conj(fp[b]) + beta * f0[a] conj(wp[b])
        const cplx<double> t1 = cmul_conj(fp[b], w0[a]);
        const cplx<double> t2 = cmul_conj(wp[b], f0[a]);
        g[a * 3 + b].re += alpha * t1.re + beta * t2.re;
        g[a * 3 + b].im += alpha * t1.im + beta * t2.im;
      }
  }
#pragma unroll
  for (int e = 0; e < 9; ++e) {
    cplx<double>* p = grad + (long long)(d * 9 + e) * V3 + s;
    cplx<double> o = *p;
    *p = o + g[e];
  }
}

// Adjoint seeds of the pair contraction G_p(X, Y)[i, j] = sum_k conj(X_i[k]) phase_p(k) Y_j[k]
// (the GEMM of lattice/generator/elemental.py:324-329).  With the gradient Gbar of a pair,
//   grad Y_j[k] = sum_p sum_i Gbar_p[i][j] X_i[k] conj(phase_p(k))
//   grad X_i[k] = sum_p sum_j conj(Gbar_p[i][j]) Y_j[k] phase_p(k).
// Both are one gather-GEMM  out[a][k] += sum_r M[r][a] * Z_r[k] * psi_r(k)  over rows r, each
// naming a chain vector Z_r = chains[cx[r]][ir[r]] and a phase psi_r = phase_p (pr[r] = p) or
// conj(phase_p) (pr[r] = -p - 1); M[r][a] carries Gbar (or its conjugate transpose) and the
// rows of every (partner chain, momentum) a chain takes part in are stacked into one call.
// 256 threads as 16 x 16, each owning 4 x 4 complex outputs of a 64 (a) x 64 (k) tile; 8 rows
// per shared-memory stage.  FP64 arithmetic, the FP64 pipe bounds it like the forward GEMM.
constexpr int ADJ_BK = 8, ADJ_TM = 4, ADJ_TN = 4, ADJ_BM = 16 * ADJ_TM, ADJ_BN = 16 * ADJ_TN;

__global__ void __launch_bounds__(256) chain_adjoint_kernel(int Ne, int V3, int nchain, int nmom, int R,
                                                            const cplx<double>* __restrict__ M,
                                                            const int* __restrict__ cx, const int* __restrict__ ir,
                                                            const int* __restrict__ pr,
                                                            const cplx<double>* __restrict__ chains,
                                                            const cplx<double>* __restrict__ phases,
                                                            cplx<double>* __restrict__ out) {
  __shared__ cplx<double> Ms[ADJ_BK][ADJ_BM + 1];
  __shared__ cplx<double> Zs[ADJ_BK][ADJ_BN + 1];
  const long long K = 3LL * V3;
  const int a0 = blockIdx.y * ADJ_BM;
  const long long k0 = (long long)blockIdx.x * ADJ_BN;
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int lr = tid >> 5, lc = tid & 31;  // loader: row lr of the stage, 32 consecutive columns x 2 passes
  cplx<double> acc[ADJ_TM][ADJ_TN];
#pragma unroll
  for (int u = 0; u < ADJ_TM; ++u)
#pragma unroll
    for (int v = 0; v < ADJ_TN; ++v) acc[u][v] = mk(0.0, 0.0);
  for (int r0 = 0; r0 < R; r0 += ADJ_BK) {
    const int r = r0 + lr;
    bool rok = r < R;
    const cplx<double>* zrow = nullptr;
    int p = 0;
    bool cj = false;
    if (rok) {
      const int c = cx[r], i = ir[r], q = pr[r];
      cj = q < 0;
      p = cj ? -q - 1 : q;
      // a row naming a chain, vector or momentum out of range contributes nothing
      rok = c >= 0 && c < nchain && i >= 0 && i < Ne && p < nmom;
      if (rok) zrow = chains + ((long long)c * Ne + i) * K;
    }
#pragma unroll
    for (int pass = 0; pass < 2; ++pass) {
      const int c = lc + 32 * pass;
      const int a = a0 + c;
      Ms[lr][c] = (rok && a < Ne) ? ld(M + (long long)r * Ne + a) : mk(0.0, 0.0);
      const long long k = k0 + c;
      cplx<double> z = mk(0.0, 0.0);
      if (rok && k < K) {
        const cplx<double> ph = ld(phases + (long long)p * V3 + (k % V3));
        const cplx<double> x = ld(zrow + k);
        z = cj ? cmul_conj(ph, x) : x * ph;
      }
      Zs[lr][c] = z;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < ADJ_BK; ++kk) {
      cplx<double> mv[ADJ_TM], zv[ADJ_TN];
#pragma unroll
      for (int u = 0; u < ADJ_TM; ++u) mv[u] = Ms[kk][ty + 16 * u];
#pragma unroll
      for (int v = 0; v < ADJ_TN; ++v) zv[v] = Zs[kk][tx + 16 * v];
#pragma unroll
      for (int u = 0; u < ADJ_TM; ++u)
#pragma unroll
        for (int v = 0; v < ADJ_TN; ++v) cfma(acc[u][v], mv[u], zv[v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < ADJ_TM; ++u) {
    const int a = a0 + ty + 16 * u;
    if (a >= Ne) continue;
#pragma unroll
    for (int v = 0; v < ADJ_TN; ++v) {
      const long long k = k0 + tx + 16 * v;
      if (k < K) {
        cplx<double>* o = out + (long long)a * K + k;
        *o = *o + acc[u][v];
      }
    }
  }
}

}  // namespace ed

extern "C" int ed_chain_adjoint(int Lx, int Ly, int Lz, int Ne, int nchain, int nmom, int R, const void* M,
                                const int* cx, const int* ir, const int* pr, const void* chains, const void* phases,
                                void* out, void* stream) {
  ED_CHECK_ARG(Lx > 0 && Ly > 0 && Lz > 0 && Ne > 0 && nchain > 0 && nmom > 0 && R >= 0,
               "ed_chain_adjoint: sizes must be positive");
  ED_CHECK_ARG(ed::lattice_ok(Lx, Ly, Lz), "ed_chain_adjoint: Lx*Ly*Lz above 2^28");
  ED_CHECK_ARG(M && cx && ir && pr && chains && phases && out, "ed_chain_adjoint: null pointer");
  ED_CHECK_ARG(((uintptr_t)M % 16) == 0 && ((uintptr_t)chains % 16) == 0 && ((uintptr_t)phases % 16) == 0 &&
                   ((uintptr_t)out % 16) == 0,
               "ed_chain_adjoint: complex buffers must be 16-byte aligned");
  if (R == 0) return ED_OK;
  const long long K = 3LL * Lx * Ly * Lz;
  ED_CHECK_ARG(K / ed::ADJ_BN + 1 < (1LL << 31) && Ne <= 65535 * ed::ADJ_BM, "ed_chain_adjoint: too large");
  dim3 grid((unsigned)ed::ceil_div(K, ed::ADJ_BN), (unsigned)ed::ceil_div(Ne, ed::ADJ_BM));
  ed::chain_adjoint_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(
      Ne, Lx * Ly * Lz, nchain, nmom, R, (const ed::cplx<double>*)M, cx, ir, pr, (const ed::cplx<double>*)chains,
      (const ed::cplx<double>*)phases, (ed::cplx<double>*)out);
  ED_RETURN_LAUNCH("chain adjoint");
  return ED_OK;
}

extern "C" int ed_link_grad(int Lx, int Ly, int Lz, int dir, int nvec, double alpha, double beta, const void* wbar,
                            const void* f, void* grad_links, void* stream) {
  ED_CHECK_ARG(Lx > 0 && Ly > 0 && Lz > 0 && nvec > 0, "ed_link_grad: sizes must be positive");
  ED_CHECK_ARG(ed::lattice_ok(Lx, Ly, Lz), "ed_link_grad: Lx*Ly*Lz above 2^28");
  ED_CHECK_ARG(dir >= 0 && dir < 3, "ed_link_grad: dir must be 0, 1 or 2");
  ED_CHECK_ARG(wbar && f && grad_links, "ed_link_grad: null pointer");
  const int V3 = Lx * Ly * Lz;
  ed::link_grad_kernel<<<ed::ceil_div(V3, 128), 128, 0, (cudaStream_t)stream>>>(
      ed::Latt{Lx, Ly, Lz}, dir, nvec, alpha, beta, (const ed::cplx<double>*)wbar, (const ed::cplx<double>*)f,
      (ed::cplx<double>*)grad_links);
  ED_RETURN_LAUNCH("link gradient");
  return ED_OK;
}
