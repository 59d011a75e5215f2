// Lowest eigenpairs of batched real symmetric "arrowhead + tridiagonal"
// matrices: the projected matrices of thick-restart Lanczos.
//
// The reference's eigensolver is ARPACK (scipy eigsh) or cupyx's
// thick-restart Lanczos (lattice/generator/eigenvector.py:234-257); both
// diagonalise the small projected matrix with a dense LAPACK/cuSOLVER call
// every restart.  On GB300 a cuSOLVER syevd of a few hundred rows is a chain
// of host-synchronised launches (about 140 ms for eight 300x300 matrices), so
// this file diagonalises the batch in three kernels, all FP64, using the
// structure of the matrix:
//
//   T[j][j] = d[j]                       (0 <= j < m)
//   T[j][ka] = T[ka][j] = s[j]            (0 <= j < ka: the kept Ritz values' border)
//   T[j][j+1] = T[j+1][j] = e[j]          (ka <= j < m-1: the Lanczos recurrence)
//
// (ka = 0: a plain tridiagonal matrix).  Eliminating the ka arrow rows first
// leaves a tridiagonal system whose first diagonal entry is shifted by
// sum_j s_j^2 / (d_j - x), so every LDL^T factorisation of T - xI costs O(m):
//
// 1. arrow_bisect_kernel: eigenvalue i by bisection on the Sturm count (the
//    number of negative pivots of T - xI), one thread per (matrix, i), to an
//    interval of 2 eps max(|lo|, |hi|) + eps ||T||.
// 2. arrow_invit_kernel: eigenvector i by inverse iteration (three solves
//    with T - lambda_i I, the tridiagonal part by Gaussian elimination with
//    partial pivoting, zero pivots replaced by eps ||T||).  Eigenvalues closer
//    than 1e-7 ||T|| form a cluster that one thread processes in order,
//    orthogonalising every member against the earlier ones after each solve.
// 3. arrow_mgs_kernel: one block per matrix re-orthonormalises the vectors in
//    eigenvalue order (two classical Gram-Schmidt passes per vector) and
//    writes them as the columns of evecs [m][nwant].
//
// The bisection and inverse-iteration steps are the textbook methods
// (Sturm-sequence bisection; inverse iteration with partial pivoting as in
// LAPACK's stein), restated for the arrow structure.

#include <cfloat>
#include <cmath>

#include "common.cuh"

namespace ed {
namespace {

constexpr double kClusterRel = 1e-7;  // eigenvalues closer than this times ||T|| are treated as a cluster
constexpr int kInvIters = 3;

struct Arrow {
  const double* d;  // [m]
  const double* s;  // [ka]
  const double* e;  // [m-1], used for j >= ka
  int m, ka;
};

__device__ __forceinline__ Arrow arrow_of(int b, int m, int ka, const double* d, const double* s, const double* e) {
  Arrow A;
  A.d = d + (long long)b * m;
  A.s = ka > 0 ? s + (long long)b * ka : nullptr;
  A.e = e + (long long)b * (m > 1 ? m - 1 : 1);
  A.m = m;
  A.ka = ka;
  return A;
}

// Gershgorin interval [lo, hi] and ||T|| bound max(|lo|, |hi|).
__device__ void gershgorin(const Arrow& A, double& lo, double& hi) {
  double sabs = 0.0;
  for (int j = 0; j < A.ka; ++j) sabs += fabs(A.s[j]);
  lo = INFINITY;
  hi = -INFINITY;
  for (int j = 0; j < A.m; ++j) {
    double r;
    if (j < A.ka) {
      r = fabs(A.s[j]);
    } else {
      r = (j == A.ka ? sabs : fabs(A.e[j - 1])) + (j + 1 < A.m ? fabs(A.e[j]) : 0.0);
    }
    lo = fmin(lo, A.d[j] - r);
    hi = fmax(hi, A.d[j] + r);
  }
}

// Number of eigenvalues of T below x: negative pivots of the LDL^T
// factorisation of T - xI (arrow rows first).  |pivot| < pivmin counts as -pivmin.
__device__ int sturm_count(const Arrow& A, double x, double pivmin) {
  int neg = 0;
  double q = A.d[A.ka] - x;
  for (int j = 0; j < A.ka; ++j) {
    double p = A.d[j] - x;
    if (fabs(p) < pivmin) p = -pivmin;
    neg += p < 0.0;
    q -= A.s[j] * A.s[j] / p;
  }
  if (fabs(q) < pivmin) q = -pivmin;
  neg += q < 0.0;
  for (int j = A.ka + 1; j < A.m; ++j) {
    const double ej = A.e[j - 1];
    q = (A.d[j] - x) - ej * ej / q;
    if (fabs(q) < pivmin) q = -pivmin;
    neg += q < 0.0;
  }
  return neg;
}

__global__ void arrow_bisect_kernel(int B, int m, int ka, int nwant, const double* __restrict__ d,
                                    const double* __restrict__ s, const double* __restrict__ e,
                                    double* __restrict__ evals) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= B * nwant) return;
  const int b = idx / nwant, i = idx - b * nwant;
  const Arrow A = arrow_of(b, m, ka, d, s, e);
  double lo, hi;
  gershgorin(A, lo, hi);
  const double tnorm = fmax(fmax(fabs(lo), fabs(hi)), DBL_MIN);
  const double pivmin = DBL_MIN * fmax(1.0, tnorm * tnorm);
  const double atol = DBL_EPSILON * tnorm;
  lo -= 2.0 * atol + 2.0 * pivmin;
  hi += 2.0 * atol + 2.0 * pivmin;
  for (int it = 0; it < 256; ++it) {
    if (hi - lo <= 2.0 * DBL_EPSILON * fmax(fabs(lo), fabs(hi)) + atol) break;
    const double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) break;  // the interval is down to adjacent doubles
    if (sturm_count(A, mid, pivmin) > i)
      hi = mid;
    else
      lo = mid;
  }
  evals[idx] = 0.5 * (lo + hi);
}

// Work arrays of one (matrix, column): five fields of length m.
struct LuView {
  double *dd, *du1, *du2, *ml, *sw;
};
__device__ __forceinline__ LuView lu_view(double* work, int b, int c, int nwant, int m) {
  double* w = work + ((long long)b * nwant + c) * 5LL * m;
  LuView L;
  L.dd = w;
  L.du1 = w + m;
  L.du2 = w + 2 * m;
  L.ml = w + 3 * m;
  L.sw = w + 4 * m;
  return L;
}

__device__ __forceinline__ double guard(double p, double tiny) { return fabs(p) < tiny ? (p < 0.0 ? -tiny : tiny) : p; }

// Gaussian elimination with partial pivoting of the tridiagonal part of
// T - lam I (rows ka .. m-1, first diagonal entry already shifted by the
// arrow); n = m - ka rows, factors into L (fields dd, du1, du2, ml, sw).
__device__ void tri_factor(const Arrow& A, double lam, double tiny, const LuView& L) {
  const int n = A.m - A.ka, k0 = A.ka;
  double shift = 0.0;
  for (int j = 0; j < A.ka; ++j) shift += A.s[j] * A.s[j] / guard(A.d[j] - lam, tiny);
  for (int k = 0; k < n; ++k) {
    L.dd[k] = A.d[k0 + k] - lam - (k == 0 ? shift : 0.0);
    L.du1[k] = k + 1 < n ? A.e[k0 + k] : 0.0;
    L.du2[k] = 0.0;
  }
  for (int k = 0; k + 1 < n; ++k) {
    const double sub = A.e[k0 + k];  // T is symmetric: the subdiagonal equals the superdiagonal
    if (fabs(L.dd[k]) >= fabs(sub)) {
      L.sw[k] = 0.0;
      const double piv = guard(L.dd[k], tiny);
      L.dd[k] = piv;
      const double mlt = sub / piv;
      L.ml[k] = mlt;
      L.dd[k + 1] -= mlt * L.du1[k];
    } else {
      // rows k and k+1 trade places; row k+1's entry two columns right becomes fill-in
      L.sw[k] = 1.0;
      const double mlt = L.dd[k] / sub;
      L.ml[k] = mlt;
      const double next_d = L.dd[k + 1], next_u = L.du1[k + 1];
      L.dd[k] = sub;
      L.dd[k + 1] = L.du1[k] - mlt * next_d;
      L.du1[k] = next_d;
      L.du2[k] = next_u;
      L.du1[k + 1] = -mlt * next_u;
    }
  }
  L.dd[n - 1] = guard(L.dd[n - 1], tiny);
}

// y <- (T - lam I)^{-1} y in place (y: m entries with stride 1).
__device__ void arrow_solve(const Arrow& A, double lam, double tiny, const LuView& L, double* y) {
  const int n = A.m - A.ka, k0 = A.ka;
  double r0 = y[k0];
  for (int j = 0; j < A.ka; ++j) r0 -= A.s[j] * y[j] / guard(A.d[j] - lam, tiny);
  y[k0] = r0;
  double* x = y + k0;
  for (int k = 0; k + 1 < n; ++k) {
    if (L.sw[k] != 0.0) {
      const double t = x[k];
      x[k] = x[k + 1];
      x[k + 1] = t;
    }
    x[k + 1] -= L.ml[k] * x[k];
  }
  x[n - 1] /= L.dd[n - 1];
  if (n >= 2) x[n - 2] = (x[n - 2] - L.du1[n - 2] * x[n - 1]) / L.dd[n - 2];
  for (int k = n - 3; k >= 0; --k) x[k] = (x[k] - L.du1[k] * x[k + 1] - L.du2[k] * x[k + 2]) / L.dd[k];
  const double xk = x[0];
  for (int j = 0; j < A.ka; ++j) y[j] = (y[j] - A.s[j] * xk) / guard(A.d[j] - lam, tiny);
}

__device__ __forceinline__ double start_value(int j, int c) {
  // deterministic pseudo-random start vector in [-1, 1): integer hash of (j, c)
  uint32_t h = (uint32_t)j * 0x9E3779B1u ^ ((uint32_t)c + 0x7F4A7C15u) * 0x85EBCA77u;
  h ^= h >> 15;
  h *= 0x2C1B3C6Du;
  h ^= h >> 12;
  h *= 0x297A2D39u;
  h ^= h >> 15;
  return (double)(h >> 8) * (2.0 / 16777216.0) - 1.0;
}

__global__ void arrow_invit_kernel(int B, int m, int ka, int nwant, const double* __restrict__ d,
                                   const double* __restrict__ s, const double* __restrict__ e,
                                   const double* __restrict__ evals, double* __restrict__ Q,
                                   double* __restrict__ work) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= B * nwant) return;
  const int b = idx / nwant, i = idx - b * nwant;
  const Arrow A = arrow_of(b, m, ka, d, s, e);
  double lo, hi;
  gershgorin(A, lo, hi);
  const double tnorm = fmax(fmax(fabs(lo), fabs(hi)), DBL_MIN);
  const double tiny = DBL_EPSILON * tnorm;
  const double ctol = kClusterRel * tnorm;
  const double* ev = evals + (long long)b * nwant;
  if (i > 0 && ev[i] - ev[i - 1] <= ctol) return;  // a member of the cluster led by an earlier thread
  const LuView L = lu_view(work, b, i, nwant, m);
  for (int c = i; c < nwant; ++c) {
    if (c > i && ev[c] - ev[c - 1] > ctol) break;
    const double lam = ev[c];
    double* y = Q + ((long long)b * nwant + c) * m;
    tri_factor(A, lam, tiny, L);
    for (int j = 0; j < m; ++j) y[j] = start_value(j, c);
    for (int it = 0; it < kInvIters; ++it) {
      arrow_solve(A, lam, tiny, L, y);
      for (int p = i; p < c; ++p) {  // earlier members of the cluster
        const double* q = Q + ((long long)b * nwant + p) * m;
        double h = 0.0;
        for (int j = 0; j < m; ++j) h += q[j] * y[j];
        for (int j = 0; j < m; ++j) y[j] -= h * q[j];
      }
      double big = 0.0;
      for (int j = 0; j < m; ++j) big = fmax(big, fabs(y[j]));
      const double sc = big > 0.0 ? 1.0 / big : 1.0;
      double nrm = 0.0;
      for (int j = 0; j < m; ++j) {
        y[j] *= sc;
        nrm += y[j] * y[j];
      }
      nrm = sqrt(nrm);
      for (int j = 0; j < m; ++j) y[j] /= nrm;
    }
  }
}

// Two classical Gram-Schmidt passes per vector, in eigenvalue order; one
// block per matrix.  Q [nwant][m] (vector-contiguous) -> evecs [m][nwant].
constexpr int MGS_THREADS = 1024;
__global__ void __launch_bounds__(MGS_THREADS) arrow_mgs_kernel(int m, int nwant, double* __restrict__ Q,
                                                                double* __restrict__ evecs) {
  extern __shared__ double h[];  // [nwant] projections, then 32 partial sums
  __shared__ double red[MGS_THREADS / 32];
  const int b = blockIdx.x;
  double* Qb = Q + (long long)b * nwant * m;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = MGS_THREADS / 32;
  for (int c = 0; c < nwant; ++c) {
    double* y = Qb + (long long)c * m;
    for (int pass = 0; pass < 2 && c > 0; ++pass) {
      for (int p = warp; p < c; p += nwarps) {
        const double* q = Qb + (long long)p * m;
        double acc = 0.0;
        for (int j = lane; j < m; j += 32) acc += q[j] * y[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) h[p] = acc;
      }
      __syncthreads();
      for (int j = threadIdx.x; j < m; j += MGS_THREADS) {
        double v = y[j];
        for (int p = 0; p < c; ++p) v -= h[p] * Qb[(long long)p * m + j];
        y[j] = v;
      }
      __syncthreads();
    }
    double acc = 0.0;
    for (int j = threadIdx.x; j < m; j += MGS_THREADS) acc += y[j] * y[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) red[warp] = acc;
    __syncthreads();
    double nrm = 0.0;
    for (int w = 0; w < nwarps; ++w) nrm += red[w];
    const double inv = nrm > 0.0 ? 1.0 / sqrt(nrm) : 0.0;
    for (int j = threadIdx.x; j < m; j += MGS_THREADS) y[j] *= inv;
    __syncthreads();
  }
  double* out = evecs + (long long)b * m * nwant;
  for (long long t = threadIdx.x; t < (long long)m * nwant; t += MGS_THREADS) {
    const int j = (int)(t / nwant), c = (int)(t - (long long)j * nwant);
    out[t] = Qb[(long long)c * m + j];
  }
}

size_t workspace_bytes(int B, int m, int nwant) {
  return (size_t)B * nwant * m * 6 * sizeof(double);  // five factor fields + the vectors
}

}  // namespace
}  // namespace ed

extern "C" int ed_arrow_eigh_workspace(int B, int m, int nwant, size_t* bytes) {
  ED_CHECK_ARG(bytes, "ed_arrow_eigh_workspace: null pointer");
  ED_CHECK_ARG(B > 0 && m > 0 && nwant > 0 && nwant <= m, "ed_arrow_eigh_workspace: bad sizes");
  *bytes = ed::workspace_bytes(B, m, nwant);
  return ED_OK;
}

extern "C" int ed_arrow_eigh(int B, int m, int ka, int nwant, const double* d, const double* s, const double* e,
                             double* evals, double* evecs, void* workspace, size_t workspace_bytes, void* stream) {
  ED_CHECK_ARG(B > 0 && m > 0 && m <= 8192, "ed_arrow_eigh: need B > 0 and 0 < m <= 8192");
  ED_CHECK_ARG(nwant > 0 && nwant <= m, "ed_arrow_eigh: need 0 < nwant <= m");
  ED_CHECK_ARG(ka >= 0 && ka < m, "ed_arrow_eigh: need 0 <= ka < m");
  ED_CHECK_ARG(d && e && evals && evecs && workspace && (ka == 0 || s), "ed_arrow_eigh: null pointer");
  ED_CHECK_ARG(((uintptr_t)workspace % 8) == 0, "ed_arrow_eigh: workspace must be 8-byte aligned");
  ED_CHECK_ARG((size_t)nwant * sizeof(double) <= 48 * 1024, "ed_arrow_eigh: nwant too large");
  if (workspace_bytes < ed::workspace_bytes(B, m, nwant)) {
    ed::set_error("ed_arrow_eigh: workspace of %zu bytes is smaller than the %zu needed", workspace_bytes,
                  ed::workspace_bytes(B, m, nwant));
    return ED_ERR_WORKSPACE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  double* work = (double*)workspace;
  double* Q = work + (size_t)B * nwant * m * 5;
  const int n = B * nwant, threads = 64;
  ed::arrow_bisect_kernel<<<(n + threads - 1) / threads, threads, 0, st>>>(B, m, ka, nwant, d, s, e, evals);
  ED_RETURN_LAUNCH("arrow eigensolver: bisection");
  ed::arrow_invit_kernel<<<(n + threads - 1) / threads, threads, 0, st>>>(B, m, ka, nwant, d, s, e, evals, Q, work);
  ED_RETURN_LAUNCH("arrow eigensolver: inverse iteration");
  ed::arrow_mgs_kernel<<<B, ed::MGS_THREADS, (size_t)nwant * sizeof(double), st>>>(m, nwant, Q, evecs);
  ED_RETURN_LAUNCH("arrow eigensolver: orthonormalisation");
  return ED_OK;
}
