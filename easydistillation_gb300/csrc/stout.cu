// One 3D stout-smearing step of the spatial links (FP64).
//
// Reference: lattice/generator/stout_smear.cu:159-245 (CUDA) and the numpy
// form lattice/generator/eigenvector.py:123-190.  For every spatial link
// U_mu(x), mu in {x, y, z}:
//   C     = sum_{nu != mu, nu spatial} [ U_nu(x) U_mu(x+nu) U_nu(x+mu)^dag
//                                      + U_nu(x-nu)^dag U_mu(x-nu) U_nu(x-nu+mu) ]
//   Omega = rho * C * U_mu(x)^dag
//   Q     = (i/2) (Omega^dag - Omega) - tr(.)/3            (traceless Hermitian)
//   U'    = exp(iQ) U_mu(x),  exp(iQ) = f0 + f1 Q + f2 Q^2 by Cayley-Hamilton with
//           the coefficients of C. Morningstar and M. Peardon, "Analytic smearing of
//           SU(3) link variables in lattice QCD", Phys. Rev. D 69, 054501 (2004),
//           hep-lat/0311018 (c0 = tr Q^3 / 3, c1 = tr Q^2 / 2).
// The step is out of place (every thread reads the unsmeared field).
// Layout: the generators' spatial links [3][nt][V3][3][3] complex128.
#include "common.cuh"

namespace ed {

using C = cplx<double>;

struct M3 {
  C a[9];
};

__device__ __forceinline__ M3 ldm(const C* __restrict__ p) {
  M3 m;
#pragma unroll
  for (int e = 0; e < 9; ++e) m.a[e] = ld(p + e);
  return m;
}
__device__ __forceinline__ M3 mul(const M3& A, const M3& B) {
  M3 R;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      C s = mk(0.0, 0.0);
#pragma unroll
      for (int k = 0; k < 3; ++k) cfma(s, A.a[i * 3 + k], B.a[k * 3 + j]);
      R.a[i * 3 + j] = s;
    }
  return R;
}
// A * B^dag
__device__ __forceinline__ M3 mul_nd(const M3& A, const M3& B) {
  M3 R;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      C s = mk(0.0, 0.0);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const C b = B.a[j * 3 + k];
        cfma(s, A.a[i * 3 + k], mk(b.re, -b.im));
      }
      R.a[i * 3 + j] = s;
    }
  return R;
}
// A^dag * B
__device__ __forceinline__ M3 mul_dn(const M3& A, const M3& B) {
  M3 R;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      C s = mk(0.0, 0.0);
#pragma unroll
      for (int k = 0; k < 3; ++k) cfma_conj(s, A.a[k * 3 + i], B.a[k * 3 + j]);
      R.a[i * 3 + j] = s;
    }
  return R;
}
__device__ __forceinline__ void add_to(M3& A, const M3& B) {
#pragma unroll
  for (int e = 0; e < 9; ++e) A.a[e] = A.a[e] + B.a[e];
}

__global__ void __launch_bounds__(128) stout_step_kernel(Latt L, int nt, double rho, const C* __restrict__ Uin,
                                                         C* __restrict__ Uout) {
  const int V3 = L.V3();
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nlinks = 3LL * nt * V3;
  if (idx >= nlinks) return;
  const int mu = (int)(idx / ((long long)nt * V3));
  const long long rem = idx - (long long)mu * nt * V3;
  const int t = (int)(rem / V3);
  const int s = (int)(rem - (long long)t * V3);
  const int x = s % L.Lx, y = (s / L.Lx) % L.Ly, z = s / (L.Lx * L.Ly);

  auto link = [&](int d, int xx, int yy, int zz) -> const C* {
    const int ss = xx + L.Lx * (yy + L.Ly * zz);
    return Uin + (((long long)d * nt + t) * V3 + ss) * 9;
  };
  auto shift = [&](int d, int& xx, int& yy, int& zz, int step) {
    if (d == 0) xx = (xx + step + L.Lx) % L.Lx;
    else if (d == 1) yy = (yy + step + L.Ly) % L.Ly;
    else zz = (zz + step + L.Lz) % L.Lz;
  };

  M3 Cst;
#pragma unroll
  for (int e = 0; e < 9; ++e) Cst.a[e] = mk(0.0, 0.0);
  for (int nu = 0; nu < 3; ++nu) {
    if (nu == mu) continue;
    // forward staple U_nu(x) U_mu(x+nu) U_nu(x+mu)^dag
    int x1 = x, y1 = y, z1 = z;
    shift(nu, x1, y1, z1, 1);
    int x2 = x, y2 = y, z2 = z;
    shift(mu, x2, y2, z2, 1);
    add_to(Cst, mul_nd(mul(ldm(link(nu, x, y, z)), ldm(link(mu, x1, y1, z1))), ldm(link(nu, x2, y2, z2))));
    // backward staple U_nu(x-nu)^dag U_mu(x-nu) U_nu(x-nu+mu)
    int x3 = x, y3 = y, z3 = z;
    shift(nu, x3, y3, z3, -1);
    int x4 = x3, y4 = y3, z4 = z3;
    shift(mu, x4, y4, z4, 1);
    add_to(Cst, mul(mul_dn(ldm(link(nu, x3, y3, z3)), ldm(link(mu, x3, y3, z3))), ldm(link(nu, x4, y4, z4))));
  }
  const M3 U = ldm(link(mu, x, y, z));
  M3 Om = mul_nd(Cst, U);
  // Q = (i/2)(Om^dag - Om), then remove the trace
  M3 Q;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const C a = Om.a[j * 3 + i];  // (Om^dag)_{ij} = conj(Om_{ji})
      const C d = mk(rho * a.re - rho * Om.a[i * 3 + j].re, -rho * a.im - rho * Om.a[i * 3 + j].im);
      Q.a[i * 3 + j] = mk(-0.5 * d.im, 0.5 * d.re);  // (i/2) * d
    }
  {
    const C tr = Q.a[0] + Q.a[4] + Q.a[8];
    const C t3 = mk(tr.re / 3.0, tr.im / 3.0);
    Q.a[0] = Q.a[0] - t3;
    Q.a[4] = Q.a[4] - t3;
    Q.a[8] = Q.a[8] - t3;
  }
  const M3 Q2 = mul(Q, Q);
  // c0 = Re tr(Q^3) / 3 needs only the diagonal of Q Q^2: sum_ik Re(Q_ik (Q^2)_ki)
  double tr3 = 0.0;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k) tr3 += Q.a[i * 3 + k].re * Q2.a[k * 3 + i].re - Q.a[i * 3 + k].im * Q2.a[k * 3 + i].im;
  const double c0_signed = tr3 / 3.0;
  const double c1 = (Q2.a[0].re + Q2.a[4].re + Q2.a[8].re) / 2.0;
  C f0, f1, f2;
  if (c1 <= 1e-300) {  // Q = 0: exp(iQ) = 1
    f0 = mk(1.0, 0.0);
    f1 = mk(0.0, 0.0);
    f2 = mk(0.0, 0.0);
  } else {
    const bool parity = c0_signed < 0;
    const double c0 = fabs(c0_signed);
    const double r = sqrt(c1 / 3.0);
    const double c0max = 2.0 * (c1 / 3.0) * r;
    const double theta = acos(fmin(1.0, c0 / c0max));
    double st, ct;
    sincos(theta / 3.0, &st, &ct);
    const double u = r * ct;
    const double w = sqrt(c1) * st;
    const double u2 = u * u, w2 = w * w;
    double su, cu, sw, cw;
    sincos(u, &su, &cu);
    sincos(w, &sw, &cw);
    // e^{2iu} from e^{iu} (double-angle identities)
    const double s2u = 2.0 * su * cu, c2u = (cu - su) * (cu + su);
    const double sinc = fabs(w) > 0.05 ? sw / w : 1.0 - w2 / 6.0 * (1.0 - w2 / 20.0 * (1.0 - w2 / 42.0 * (1.0 - w2 / 72.0)));
    const double den = 1.0 / (9.0 * u2 - w2);
    // e^{-iu} = cu - i su; e^{2iu} = c2u + i s2u
    f0 = mk(((u2 - w2) * c2u + cu * 8.0 * u2 * cw + su * 2.0 * u * (3.0 * u2 + w2) * sinc) * den,
            ((u2 - w2) * s2u - su * 8.0 * u2 * cw + cu * 2.0 * u * (3.0 * u2 + w2) * sinc) * den);
    f1 = mk((2.0 * u * c2u - cu * 2.0 * u * cw + su * (3.0 * u2 - w2) * sinc) * den,
            (2.0 * u * s2u + su * 2.0 * u * cw + cu * (3.0 * u2 - w2) * sinc) * den);
    f2 = mk((c2u - cu * cw - su * 3.0 * u * sinc) * den, (s2u + su * cw - cu * 3.0 * u * sinc) * den);
    if (parity) {
      f0.im = -f0.im;
      f1.re = -f1.re;
      f2.im = -f2.im;
    }
  }
  M3 E;
#pragma unroll
  for (int e = 0; e < 9; ++e) E.a[e] = f1 * Q.a[e] + f2 * Q2.a[e];
  E.a[0] = E.a[0] + f0;
  E.a[4] = E.a[4] + f0;
  E.a[8] = E.a[8] + f0;
  const M3 R = mul(E, U);
  C* o = Uout + idx * 9;
#pragma unroll
  for (int e = 0; e < 9; ++e) o[e] = R.a[e];
}

// Projection back onto U(3) by the averaged inverse iteration U <- (U + U^-dag) / 2 of
// lattice/generator/eigenvector.py:55-65 (and elemental.py:107-118), one thread per link, until
// max |U - U^-dag| and max |U U^dag - 1| are both <= tol for that link (the reference tests the whole
// field at once; a link that has converged is a fixed point of the iteration up to rounding).
// U^-dag = conj(cof(U)) / conj(det U) with the cofactor matrix cof.
__global__ void project_su3_kernel(long long n, C* __restrict__ U, double tol, int max_iter) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n) return;
  C* p = U + idx * 9;
  M3 A = ldm(p);
  for (int it = 0; it < max_iter; ++it) {
    C cof[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
        cof[i * 3 + j] = A.a[i1 * 3 + j1] * A.a[i2 * 3 + j2] - A.a[i1 * 3 + j2] * A.a[i2 * 3 + j1];
      }
    const C det = A.a[0] * cof[0] + A.a[1] * cof[1] + A.a[2] * cof[2];
    // 1 / conj(det) = det / |det|^2
    const double n2 = det.re * det.re + det.im * det.im;
    const C inv = mk(det.re / n2, det.im / n2);
    double dmax = 0.0, umax = 0.0;
    M3 Bm;
#pragma unroll
    for (int e = 0; e < 9; ++e) {
      Bm.a[e] = mk(cof[e].re, -cof[e].im) * inv;  // U^-dag
      dmax = fmax(dmax, hypot(A.a[e].re - Bm.a[e].re, A.a[e].im - Bm.a[e].im));
    }
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        C s = mk(0.0, 0.0);
#pragma unroll
        for (int k = 0; k < 3; ++k) cfma_conj(s, A.a[j * 3 + k], A.a[i * 3 + k]);  // (U U^dag)[i][j]
        umax = fmax(umax, hypot(s.re - (i == j ? 1.0 : 0.0), s.im));
      }
    if (dmax <= tol && umax <= tol) break;
#pragma unroll
    for (int e = 0; e < 9; ++e) A.a[e] = mk(0.5 * (A.a[e].re + Bm.a[e].re), 0.5 * (A.a[e].im + Bm.a[e].im));
  }
#pragma unroll
  for (int e = 0; e < 9; ++e) p[e] = A.a[e];
}

}  // namespace ed

extern "C" int ed_project_su3(long long nlinks, void* U, double tol, int max_iter, void* stream) {
  ED_CHECK_ARG(nlinks >= 0 && tol >= 0.0 && max_iter > 0, "ed_project_su3: bad arguments");
  ED_CHECK_ARG(U || nlinks == 0, "ed_project_su3: null pointer");
  if (nlinks == 0) return ED_OK;
  ed::project_su3_kernel<<<ed::ceil_div(nlinks, 128), 128, 0, (cudaStream_t)stream>>>(nlinks, (ed::C*)U, tol,
                                                                                       max_iter);
  ED_RETURN_LAUNCH("SU(3) projection");
  return ED_OK;
}

extern "C" int ed_stout_smear_step(int Lx, int Ly, int Lz, int nt, double rho, const void* U_in, void* U_out,
                                   void* stream) {
  ED_CHECK_ARG(Lx > 0 && Ly > 0 && Lz > 0 && nt > 0, "ed_stout_smear_step: sizes must be positive");
  ED_CHECK_ARG(ed::lattice_ok(Lx, Ly, Lz), "ed_stout_smear_step: Lx*Ly*Lz above 2^28");
  ED_CHECK_ARG(U_in && U_out && U_in != U_out, "ed_stout_smear_step: null or aliasing pointers");
  const long long n = 3LL * nt * Lx * Ly * Lz;
  ed::stout_step_kernel<<<ed::ceil_div(n, 128), 128, 0, (cudaStream_t)stream>>>(
      ed::Latt{Lx, Ly, Lz}, nt, rho, (const ed::C*)U_in, (ed::C*)U_out);
  ED_RETURN_LAUNCH("stout smearing step");
  return ED_OK;
}
