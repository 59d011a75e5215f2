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

}  // namespace ed

extern "C" int ed_link_grad(int Lx, int Ly, int Lz, int dir, int nvec, double alpha, double beta, const void* wbar,
                            const void* f, void* grad_links, void* stream) {
  ED_CHECK_ARG(Lx > 0 && Ly > 0 && Lz > 0 && nvec > 0, "ed_link_grad: sizes must be positive");
  ED_CHECK_ARG(dir >= 0 && dir < 3, "ed_link_grad: dir must be 0, 1 or 2");
  ED_CHECK_ARG(wbar && f && grad_links, "ed_link_grad: null pointer");
  const int V3 = Lx * Ly * Lz;
  ed::link_grad_kernel<<<ed::ceil_div(V3, 128), 128, 0, (cudaStream_t)stream>>>(
      ed::Latt{Lx, Ly, Lz}, dir, nvec, alpha, beta, (const ed::cplx<double>*)wbar, (const ed::cplx<double>*)f,
      (ed::cplx<double>*)grad_links);
  ED_RETURN_LAUNCH("link gradient");
  return ED_OK;
}
