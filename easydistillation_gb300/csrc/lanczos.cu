// Native thick-restart Lanczos for the lowest eigenpairs of the 3D covariant
// Laplacian, batched over timeslices (ed_lanczos_tr).
//
// This is the eigensolve of EigenvectorGenerator.calc
// (lattice/generator/eigenvector.py:234-257: scipy / cupyx
// eigsh(LinearOperator, k=Ne, which="SA", tol), with the QUDA path's Chebyshev
// acceleration at :295-299), written as a host loop over the library's
// kernels: one FP64 stencil launch per Lanczos step for all timeslices
// (launch_laplacian), the three-term recurrence and one classical
// Gram-Schmidt pass per step (two at the first step after a restart) by
// ed_cgs_pass, the projected arrowhead + tridiagonal matrix diagonalised by
// ed_arrow_eigh at each restart, the restart rotation Y^T V by the library's
// own batched kernel (lz_rotate_kernel: FP64, or double-float on the FP32 pipe
// in the double-float Gram-Schmidt mode).  Everything is FP64 on the GPU
// unless that mode is chosen; the host reads one convergence counter per
// restart.  Convergence follows
// ARPACK's rule: Ritz pair i is accepted when |beta_m y_{m,i}| <= tol |theta_i|.
//
// ed_lanczos_tr_ex adds a mixed-precision solve: phase 1 runs the same
// iteration with the complex64 stencil (the FP64 basis vector rounded to
// complex64, the result widened back; Gram-Schmidt, Rayleigh-Ritz and the
// convergence test in FP64) for at most 3 restarts or to a loose tolerance
// (1e-3, far above the stencil's ~1e-7 rounding); its Ritz values give the
// Chebyshev cut (15 %
// above the largest wanted one) and its Ritz vectors the start vector of
// phase 2, an FP64-stencil Chebyshev-filtered solve to the requested
// tolerance.  The final eigenpairs, their residual test and the Rayleigh
// quotients are FP64.
//
// With a Chebyshev degree the iteration runs on -T_deg((2L - (12 + cut)) /
// (12 - cut)) (sign flipped for even degree so the wanted modes are the
// smallest), which keeps L's eigenvectors and their order below the cut; the
// eigenvalues returned are then the Rayleigh quotients x^H L x.

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <type_traits>
#include <vector>

#include "common.cuh"
#include "df.cuh"

namespace ed {
int split_rows(int B, int nrow, long long n, const void* src, long long sb, void* dst, long long db,
               cudaStream_t st);
int cgs_pass_df(int B, int r, long long n, const void* Vs, long long vs_bstride, void* w, void* ws, void* h, int ldh,
                double* norm_part, cudaStream_t st);
namespace {

constexpr int LZ_THREADS = 256;
// Mixed solve (ed_lanczos_tr_ex with the complex64 stencil): phase-1 tolerance (well above the complex64
// stencil's rounding, ~1e-7 relative) and restart budget, and the default Chebyshev degree of the FP64
// phase 2.  Phase 1 only supplies the Chebyshev cut and a start vector: its largest wanted Ritz value
// bounds the wanted eigenvalue from above (Cauchy interlacing) whether or not it has converged.  Measured
// at 24^3, Ne = 100 (8 timeslices): phase 1 to 1e-4 took 12 restarts and the whole solve ran at 3.5
// timeslices/s, no faster than the plain FP64 solve.
constexpr double LZ_MIXED_TOL = 1e-3;
constexpr int LZ_MIXED_RESTARTS = 3;  // phase 1 only has to bound the wanted spectrum from above
constexpr int LZ_MIXED_DEG = 16;

// ED_OK, or the library's CUDA error status for a failed call
inline int lz_chk(cudaError_t e, const char* what) { return e == cudaSuccess ? ED_OK : cuda_status(e, what); }

__device__ __forceinline__ double block_sum(double v, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  for (int q = 0; q < LZ_THREADS / 32; ++q) t += red[q];
  __syncthreads();
  return t;
}

// sum of the nblk partials of problem b, in a fixed order (every block gets the same value); thread 0 sums,
// the block shares the result
__device__ __forceinline__ double sum_parts(const double* part, int b, int nblk) {
  __shared__ double total;
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < nblk; ++q) t += part[(long long)b * nblk + q];
    total = t;
  }
  __syncthreads();
  return total;
}

// w[b] = pseudo-random start vector (integer hash of (b, x), values in [-1, 1))
__global__ void lz_random_kernel(int B, long long n, double2* __restrict__ w, unsigned seed) {
  const int b = blockIdx.y;
  for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (long long)gridDim.x * blockDim.x) {
    uint32_t h = (uint32_t)x * 0x9E3779B1u ^ ((uint32_t)b * 0x85EBCA77u + seed);
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    h ^= h >> 15;
    uint32_t g = h * 0x9E3779B1u + 0x7F4A7C15u;
    g ^= g >> 13;
    g *= 0x5BD1E995u;
    g ^= g >> 15;
    w[(long long)b * n + x] = make_double2((double)(h >> 8) * (2.0 / 16777216.0) - 1.0,
                                           (double)(g >> 8) * (2.0 / 16777216.0) - 1.0);
  }
}

// part[b][blk] = partial of Re(sum_x conj(a[b][x]) c[b][x])
__global__ void __launch_bounds__(LZ_THREADS) lz_dot_kernel(long long n, const double2* __restrict__ a, long long ab,
                                                            const double2* __restrict__ c, long long cb,
                                                            double* __restrict__ part) {
  __shared__ double red[LZ_THREADS / 32];
  const int b = blockIdx.y;
  double acc = 0.0;
  for (long long x = (long long)blockIdx.x * LZ_THREADS + threadIdx.x; x < n; x += (long long)gridDim.x * LZ_THREADS) {
    const double2 u = a[(long long)b * ab + x], v = c[(long long)b * cb + x];
    acc = fma(u.x, v.x, fma(u.y, v.y, acc));
  }
  const double t = block_sum(acc, red);
  if (threadIdx.x == 0) part[(long long)b * gridDim.x + blockIdx.x] = t;
}

// dst[b] = src[b] / sqrt(sum of part[b])
__global__ void lz_normalise_kernel(long long n, const double2* __restrict__ src, const double* __restrict__ part,
                                    int nblk, double2* __restrict__ dst, long long db) {
  const int b = blockIdx.y;
  const double nrm = sqrt(sum_parts(part, b, nblk));
  const double inv = nrm > 0.0 ? 1.0 / nrm : 1.0;
  for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (long long)gridDim.x * blockDim.x) {
    const double2 v = src[(long long)b * n + x];
    dst[(long long)b * db + x] = make_double2(v.x * inv, v.y * inv);
  }
}

// alpha = sum of part[b] (= Re <v_j, w>); d[j] = alpha; w -= alpha v_j + e[j-1] v_{j-1}
__global__ void lz_three_term_kernel(long long n, const double2* __restrict__ V, long long vb, int j,
                                     double2* __restrict__ w, const double* __restrict__ part, int nblk,
                                     double* __restrict__ d, const double* __restrict__ e, int ncv) {
  const int b = blockIdx.y;
  const double alpha = sum_parts(part, b, nblk);
  const double beta = e[(long long)b * (ncv - 1) + j - 1];
  if (blockIdx.x == 0 && threadIdx.x == 0) d[(long long)b * ncv + j] = alpha;
  const double2* vj = V + (long long)b * vb + (long long)j * n;
  const double2* vm = vj - n;
  for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (long long)gridDim.x * blockDim.x) {
    double2 o = w[(long long)b * n + x];
    const double2 a = vj[x], c = vm[x];
    o.x -= alpha * a.x + beta * c.x;
    o.y -= alpha * a.y + beta * c.y;
    w[(long long)b * n + x] = o;
  }
}

// End of step j: beta = ||w|| (from the Gram-Schmidt norm partials);
// d[j] (+)= Re h[j] (+ Re h2[j]); e[j] = beta (or beta_last at the last step);
// V[j+1] = w / beta.
__global__ void lz_finish_kernel(long long n, double2* __restrict__ V, long long vb, int j, const double2* __restrict__ w,
                                 const double2* __restrict__ h, const double2* __restrict__ h2, int ldh,
                                 const double* __restrict__ npart, int nblk, double* __restrict__ d,
                                 double* __restrict__ e, double* __restrict__ beta_last, int ncv, int first) {
  const int b = blockIdx.y;
  const double beta = sqrt(sum_parts(npart, b, nblk));
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    double dj = h[(long long)b * ldh + j].x + (h2 ? h2[(long long)b * ldh + j].x : 0.0);
    if (!first) dj += d[(long long)b * ncv + j];
    d[(long long)b * ncv + j] = dj;
    if (j + 1 < ncv)
      e[(long long)b * (ncv - 1) + j] = beta;
    else
      beta_last[b] = beta;
  }
  const double inv = beta > 0.0 ? 1.0 / beta : 1.0;
  double2* dst = V + (long long)b * vb + (long long)(j + 1) * n;
  for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (long long)gridDim.x * blockDim.x) {
    const double2 v = w[(long long)b * n + x];
    dst[x] = make_double2(v.x * inv, v.y * inv);
  }
}

// Chebyshev recurrence step: out = s * (f (a Lx + c x) - prev) with f = 2 (or 1 and no prev for the first step);
// x and prev may be strided (xb, pb elements per problem), Lx and out are [B][n].
__global__ void lz_cheb_kernel(long long n, const double2* __restrict__ Lx, const double2* __restrict__ x, long long xb,
                               const double2* __restrict__ prev, long long pb, double2* __restrict__ out, double a,
                               double c, double f, double s) {
  const int b = blockIdx.y;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double2 l = Lx[(long long)b * n + i], v = x[(long long)b * xb + i];
    double re = f * (a * l.x + c * v.x), im = f * (a * l.y + c * v.y);
    if (prev) {
      const double2 p = prev[(long long)b * pb + i];
      re -= p.x;
      im -= p.y;
    }
    out[(long long)b * n + i] = make_double2(s * re, s * im);
  }
}

// Count the wanted Ritz pairs that fail |beta_last y_{m-1,i}| <= tol max(|theta_i|, eps^(2/3)).
__global__ void lz_converged_kernel(int B, int ncv, int kk, int nev, const double* __restrict__ theta,
                                    const double* __restrict__ Y, const double* __restrict__ beta_last, double tol,
                                    int* __restrict__ nbad) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= B * nev) return;
  const int b = idx / nev, i = idx - b * nev;
  const double r = fabs(beta_last[b] * Y[((long long)b * ncv + ncv - 1) * kk + i]);
  const double sc = fmax(fabs(theta[(long long)b * kk + i]), 3.6e-11 /* eps^(2/3) */);
  if (!(r <= tol * sc)) atomicAdd(nbad, 1);
}

// Thick restart: d[i] = theta_i, s[i] = beta_last y_{m-1,i} for the kk kept pairs.
__global__ void lz_restart_kernel(int B, int ncv, int kk, const double* __restrict__ theta,
                                  const double* __restrict__ Y, const double* __restrict__ beta_last,
                                  double* __restrict__ d, double* __restrict__ s) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= B * kk) return;
  const int b = idx / kk, i = idx - b * kk;
  d[(long long)b * ncv + i] = theta[(long long)b * kk + i];
  s[(long long)b * kk + i] = beta_last[b] * Y[((long long)b * ncv + ncv - 1) * kk + i];
}

// Rayleigh quotients Re(x^H L x) / ||x||^2, one block per (problem, vector).
__global__ void __launch_bounds__(LZ_THREADS) lz_rq_kernel(long long n, const double2* __restrict__ X,
                                                           const double2* __restrict__ LX, double* __restrict__ rq) {
  __shared__ double red[LZ_THREADS / 32];
  const long long v = blockIdx.x;
  double num = 0.0, den = 0.0;
  for (long long i = threadIdx.x; i < n; i += LZ_THREADS) {
    const double2 x = X[v * n + i], l = LX[v * n + i];
    num = fma(x.x, l.x, fma(x.y, l.y, num));
    den = fma(x.x, x.x, fma(x.y, x.y, den));
  }
  num = block_sum(num, red);
  den = block_sum(den, red);
  if (threadIdx.x == 0) rq[v] = den > 0.0 ? num / den : 0.0;
}

// Sort each problem's nev values ascending (insertion sort, one thread per problem) and record the order.
__global__ void lz_sort_kernel(int B, int nev, double* __restrict__ vals, int* __restrict__ perm) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  double* v = vals + (long long)b * nev;
  int* p = perm + (long long)b * nev;
  for (int i = 0; i < nev; ++i) p[i] = i;
  for (int i = 1; i < nev; ++i) {
    const double key = v[i];
    const int kp = p[i];
    int q = i - 1;
    while (q >= 0 && v[q] > key) {
      v[q + 1] = v[q];
      p[q + 1] = p[q];
      --q;
    }
    v[q + 1] = key;
    p[q + 1] = kp;
  }
}

// dst[b][i] = src[b][perm[b][i]] (vectors of n values)
__global__ void lz_gather_kernel(int nev, long long n, const double2* __restrict__ src, const int* __restrict__ perm,
                                 double2* __restrict__ dst) {
  const int b = blockIdx.z, i = blockIdx.y;
  const int from = perm[(long long)b * nev + i];
  const double2* s = src + ((long long)b * nev + from) * n;
  double2* o = dst + ((long long)b * nev + i) * n;
  for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (long long)gridDim.x * blockDim.x)
    o[x] = s[x];
}

// out[b][x] = complex64 rounding of in[b*ib + x] (the operand of the complex64 stencil)
__global__ void lz_to_c64_kernel(long long n, const double2* __restrict__ in, long long ib, float2* __restrict__ out) {
  const int b = blockIdx.y;
  for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (long long)gridDim.x * blockDim.x) {
    const double2 v = in[(long long)b * ib + x];
    out[(long long)b * n + x] = make_float2((float)v.x, (float)v.y);
  }
}

// out[b][x] = in[b][x] widened to complex128
__global__ void lz_from_c64_kernel(long long n, const float2* __restrict__ in, double2* __restrict__ out) {
  const int b = blockIdx.y;
  for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (long long)gridDim.x * blockDim.x) {
    const float2 v = in[(long long)b * n + x];
    out[(long long)b * n + x] = make_double2((double)v.x, (double)v.y);
  }
}

// w[b] = sum of the nvec vectors X[b][0..nvec) (a warm start made of earlier Ritz vectors)
__global__ void lz_sum_vectors_kernel(long long n, int nvec, const double2* __restrict__ X, double2* __restrict__ w) {
  const int b = blockIdx.y;
  for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (long long)gridDim.x * blockDim.x) {
    double re = 0.0, im = 0.0;
    for (int i = 0; i < nvec; ++i) {
      const double2 v = X[((long long)b * nvec + i) * n + x];
      re += v.x;
      im += v.y;
    }
    w[(long long)b * n + x] = make_double2(re, im);
  }
}

// Workspace carve-up (all offsets 256-byte aligned).
struct LzLayout {
  size_t V, w, t0, t1, t2, lbuf, rot, hA, hB, part, npart, d, e, s, bl, theta, Y, arrow, nbad, rq, perm, Vs, ws, Ls,
      total;
  size_t arrow_bytes;
};

size_t al(size_t v) { return (v + 255) / 256 * 256; }

LzLayout lz_layout(int B, long long n, int ncv, int kk, int nev, int nblk, bool gs_df = false) {
  LzLayout L;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t at = o;
    o += al(bytes);
    return at;
  };
  const size_t vec = (size_t)B * n * 16;
  L.V = take((size_t)B * (ncv + 1) * n * 16);
  L.w = take(vec);
  L.t0 = take(vec);
  L.t1 = take(vec);
  L.t2 = take(vec);
  L.lbuf = take(vec);
  L.rot = take((size_t)B * kk * n * 16);
  L.hA = take((size_t)B * (ncv + 1) * 16);
  L.hB = take((size_t)B * (ncv + 1) * 16);
  L.part = take((size_t)B * nblk * 8);
  L.npart = take((size_t)B * nblk * 8);
  L.d = take((size_t)B * ncv * 8);
  L.e = take((size_t)B * ncv * 8);  // [B][ncv-1] used: T[j][j+1], the layout ed_arrow_eigh reads
  L.s = take((size_t)B * kk * 8);
  L.bl = take((size_t)B * 8);
  L.theta = take((size_t)B * kk * 8);
  L.Y = take((size_t)B * ncv * kk * 8);
  size_t ab = 0;
  ed_arrow_eigh_workspace(B, ncv, kk, &ab);
  L.arrow_bytes = ab;
  L.arrow = take(ab);
  L.nbad = take(16);
  L.rq = take((size_t)B * nev * 8);
  L.perm = take((size_t)B * nev * 4);
  L.Vs = L.ws = L.Ls = 0;
  if (gs_df) {  // the basis and w in the split form of the double-float Gram-Schmidt pass, and the split links
    L.Vs = take((size_t)B * (ncv + 1) * n * 16);
    L.ws = take(vec);
    L.Ls = take((size_t)B * 9 * n * 16);  // [B][27][V3] float4 (n = 3 V3)
  }
  L.total = o;
  return L;
}

// Ritz pairs kept at a thick restart: the wanted ones and a tenth more (at least 8).  Measured on GB300 at
// 24^3, Ne = 100 (8 timeslices): keeping Ne + (ncv - Ne) / 2 = 200 of 300 took 4.05 s, Ne + 10 took 2.73 s (9
// restarts instead of 16: longer cycles, fewer FP64 basis rotations).
int lz_kept(int nev, int ncv) { return std::min(ncv - 1, nev + std::max(8, nev / 10)); }

// The restart rotation and the Ritz vectors: C[b][j] = sum_r Y[b][r][j] V[b][r] for j < nkeep, r < m, with
// Y real (the Ritz coefficients, row-major [m][ldy]) and V complex128 rows of n elements.  A block computes
// 32 output rows (j) x 64 elements (x) from stages of 32 basis rows held in shared memory; each thread owns
// 2 x 4 complex results.  FP64: bound by this part's FP64 pipe (~1.25 TFLOP/s; 4 flops per complex element
// and Ritz coefficient).  DF (the double-float Gram-Schmidt mode): the basis rows in their split form
// (df.cuh) and Y split on the fly, double-float sums on the FP32 pipe.
constexpr int ROT_J = 32, ROT_X = 64, ROT_R = 32, ROT_THREADS = 256;

template <bool DFM>
__global__ void __launch_bounds__(ROT_THREADS) lz_rotate_kernel(int m, int nkeep, long long n,
                                                                const double2* __restrict__ V, long long vb,
                                                                const float4* __restrict__ Vs, long long vsb,
                                                                const double* __restrict__ Y, int ldy, long long yb,
                                                                double2* __restrict__ C, long long cb) {
  using VT = typename std::conditional<DFM, float4, double2>::type;  // a basis element as staged
  using YT = typename std::conditional<DFM, float2, double>::type;   // a Ritz coefficient as staged
  __shared__ YT Ys[ROT_R][ROT_J];
  __shared__ VT Vt[ROT_R][ROT_X];
  const int b = blockIdx.z;
  const long long x0 = (long long)blockIdx.x * ROT_X;
  const int j0 = blockIdx.y * ROT_J;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const double* Yb = Y + (long long)b * yb;
  double2 acc[2][4];
  DF are[2][4], aim[2][4];
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      acc[p][q] = make_double2(0.0, 0.0);
      are[p][q] = DF{0.f, 0.f};
      aim[p][q] = DF{0.f, 0.f};
    }
  for (int r0 = 0; r0 < m; r0 += ROT_R) {
    // stage Y[r0 .. r0+31][j0 .. j0+31] and the basis rows r0 .. r0+31, elements x0 .. x0+63 (zeros outside)
#pragma unroll
    for (int u = 0; u < (ROT_R * ROT_J) / ROT_THREADS; ++u) {
      const int lin = tid + u * ROT_THREADS, rr = lin / ROT_J, jj = lin % ROT_J;
      const int r = r0 + rr, j = j0 + jj;
      const double y = (r < m && j < nkeep) ? Yb[(long long)r * ldy + j] : 0.0;
      if constexpr (DFM) {
        const float yh = __double2float_rn(y);
        Ys[rr][jj] = make_float2(yh, __double2float_rn(y - (double)yh));
      } else {
        Ys[rr][jj] = y;
      }
    }
#pragma unroll
    for (int u = 0; u < (ROT_R * ROT_X) / ROT_THREADS; ++u) {
      const int lin = tid + u * ROT_THREADS, rr = lin / ROT_X, xx = lin % ROT_X;
      const int r = r0 + rr;
      const long long x = x0 + xx;
      if constexpr (DFM) {
        Vt[rr][xx] = (r < m && x < n) ? Vs[(long long)b * vsb + (long long)r * n + x] : make_float4(0.f, 0.f, 0.f, 0.f);
      } else {
        Vt[rr][xx] = (r < m && x < n) ? V[(long long)b * vb + (long long)r * n + x] : make_double2(0.0, 0.0);
      }
    }
    __syncthreads();
#pragma unroll 4
    for (int rr = 0; rr < ROT_R; ++rr) {
      YT y[2];
      VT v[4];
#pragma unroll
      for (int p = 0; p < 2; ++p) y[p] = Ys[rr][ty + 16 * p];
#pragma unroll
      for (int q = 0; q < 4; ++q) v[q] = Vt[rr][tx + 16 * q];
#pragma unroll
      for (int p = 0; p < 2; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          if constexpr (DFM) {
            df_acc(are[p][q], y[p].x, y[p].y, v[q].x, v[q].z);
            df_acc(aim[p][q], y[p].x, y[p].y, v[q].y, v[q].w);
          } else {
            acc[p][q].x = fma(y[p], v[q].x, acc[p][q].x);
            acc[p][q].y = fma(y[p], v[q].y, acc[p][q].y);
          }
        }
    }
    if constexpr (DFM) {  // one renormalisation per stage of ROT_R basis rows
#pragma unroll
      for (int p = 0; p < 2; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          df_renorm(are[p][q]);
          df_renorm(aim[p][q]);
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int p = 0; p < 2; ++p) {
    const int j = j0 + ty + 16 * p;
    if (j >= nkeep) continue;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const long long x = x0 + tx + 16 * q;
      if (x >= n) continue;
      C[(long long)b * cb + (long long)j * n + x] =
          DFM ? make_double2(df_value(are[p][q]), df_value(aim[p][q])) : acc[p][q];
    }
  }
}

// C[b] (nkeep rows of n complex128, batch stride cb) = the first nkeep Ritz combinations of the first m
// basis rows; Vs (the split rows, batch stride vsb) selects the double-float kernel.
int lz_rotate(cudaStream_t st, int B, long long n, int m, int nkeep, const double2* V, long long vb,
              const float4* Vs, long long vsb, const double* Y, int ldy, long long yb, double2* C, long long cb) {
  const dim3 grid((unsigned)((n + ROT_X - 1) / ROT_X), (unsigned)((nkeep + ROT_J - 1) / ROT_J), (unsigned)B);
  if (Vs)
    lz_rotate_kernel<true><<<grid, ROT_THREADS, 0, st>>>(m, nkeep, n, V, vb, Vs, vsb, Y, ldy, yb, C, cb);
  else
    lz_rotate_kernel<false><<<grid, ROT_THREADS, 0, st>>>(m, nkeep, n, V, vb, Vs, vsb, Y, ldy, yb, C, cb);
  return lz_chk(cudaGetLastError(), "Lanczos restart rotation");
}

}  // namespace
}  // namespace ed

extern "C" int ed_lanczos_workspace(int Lx, int Ly, int Lz, int nt, int Ne, int ncv, size_t* bytes) {
  ED_CHECK_ARG(bytes, "ed_lanczos_workspace: null pointer");
  ED_CHECK_ARG(Lx > 0 && Ly > 0 && Lz > 0 && nt > 0 && nt <= 65535 && Ne > 0, "ed_lanczos_workspace: bad sizes");
  ED_CHECK_ARG(ed::lattice_ok(Lx, Ly, Lz), "ed_lanczos_workspace: Lx*Ly*Lz above 2^28");
  const long long n = 3LL * Lx * Ly * Lz;
  ED_CHECK_ARG(Ne < ncv && ncv <= n, "ed_lanczos_workspace: need Ne < ncv <= 3*Lx*Ly*Lz");
  const int nblk = (int)((n + ed::LZ_THREADS - 1) / ed::LZ_THREADS);
  *bytes = ed::lz_layout(nt, n, ncv, ed::lz_kept(Ne, ncv), Ne, nblk).total;
  return ED_OK;
}

namespace ed {
namespace {

// One thick-restart Lanczos solve (the body of ed_lanczos_tr and of each phase of ed_lanczos_tr_ex).  The operator
// applications use the FP64 stencil on `links` (stencil_prec ED_C128), or round the FP64 basis vector to complex64,
// apply the complex64 stencil on `links32` and widen the result (ED_C64).  Everything else is FP64.  With start_nvec
// > 0 the start vector of problem b is the sum of the start_nvec vectors start[b][..] (else a pseudo-random one).
// status: converged, restarts, operator applications.  Argument checks are the callers'.
struct LzArgs {
  int Lx, Ly, Lz, nt;
  const void* links;
  const void* links32;
  int stencil_prec;
  int Ne;
  double tol;
  int ncv, max_restarts, poly_deg;
  double lambda_cut;
  void* evecs;
  double* evals;
  const void* start;
  int start_nvec;
  int* status;
  void* workspace;
  cudaStream_t stream;
  bool gs_df = false;  // Gram-Schmidt passes in double-float arithmetic on the FP32 pipe
};

size_t lz_c64_bytes(int B, long long n) { return 2 * al((size_t)B * n * 8); }

int lanczos_solve(const LzArgs& a) {
  const int Lx = a.Lx, Ly = a.Ly, Lz = a.Lz, nt = a.nt, Ne = a.Ne, ncv = a.ncv, max_restarts = a.max_restarts,
            poly_deg = a.poly_deg;
  const void* links = a.links;
  const double tol = a.tol, lambda_cut = a.lambda_cut;
  void* evecs = a.evecs;
  double* evals = a.evals;
  int* status = a.status;
  const long long n = 3LL * Lx * Ly * Lz;
  const int B = nt, kk = lz_kept(Ne, ncv);
  // elementwise grids: one element per thread; the Gram-Schmidt update kernel writes its ||w||^2 partials on the
  // same grid (ceil(n / 256) blocks per problem)
  const int nblk = (int)((n + LZ_THREADS - 1) / LZ_THREADS);
  const LzLayout Lw = lz_layout(B, n, ncv, kk, Ne, nblk, a.gs_df);
  float4* const Vs = a.gs_df ? (float4*)((uint8_t*)a.workspace + Lw.Vs) : nullptr;  // split basis rows
  float4* const wsp = a.gs_df ? (float4*)((uint8_t*)a.workspace + Lw.ws) : nullptr;  // split w
  // the links in split form: the double-float mode applies its FP64-class stencil as ED_DF on the FP32 pipe
  float4* const Ls = (a.gs_df && a.stencil_prec == ED_C128) ? (float4*)((uint8_t*)a.workspace + Lw.Ls) : nullptr;
  const long long vsb = (long long)(ncv + 1) * n;
  uint8_t* const W = (uint8_t*)a.workspace;
  // complex64 operand and result of the FP32 stencil, after the FP64 layout
  float2* x32 = (float2*)(W + Lw.total);
  float2* y32 = (float2*)(W + Lw.total + al((size_t)B * n * 8));
  cudaStream_t st = a.stream;
  double2* V = (double2*)(W + Lw.V);
  double2* w = (double2*)(W + Lw.w);
  double2* t0 = (double2*)(W + Lw.t0);
  double2* t1 = (double2*)(W + Lw.t1);
  double2* t2 = (double2*)(W + Lw.t2);
  double2* lbuf = (double2*)(W + Lw.lbuf);
  double2* rot = (double2*)(W + Lw.rot);
  double2* hA = (double2*)(W + Lw.hA);
  double2* hB = (double2*)(W + Lw.hB);
  double* part = (double*)(W + Lw.part);
  double* npart = (double*)(W + Lw.npart);
  double* d = (double*)(W + Lw.d);
  double* e = (double*)(W + Lw.e);
  double* s = (double*)(W + Lw.s);
  double* bl = (double*)(W + Lw.bl);
  double* theta = (double*)(W + Lw.theta);
  double* Y = (double*)(W + Lw.Y);
  int* nbad = (int*)(W + Lw.nbad);
  double* rq = (double*)(W + Lw.rq);
  int* perm = (int*)(W + Lw.perm);
  const long long vb = (long long)(ncv + 1) * n;
  const dim3 vgrid((unsigned)nblk, (unsigned)B);
  int rc = ED_OK;
#define LZ_TRY(expr)               \
  do {                             \
    rc = (expr);                   \
    if (rc != ED_OK) return rc;    \
  } while (0)
#define LZ_LAUNCHED(what) LZ_TRY(lz_chk(cudaGetLastError(), what))
  if (Ls) LZ_TRY(ed_split_c128((long long)B * 9 * n, links, Ls, st));

  // the operator: L, or -(+)T_deg of the spectrum map [cut, 12] -> [-1, 1]
  const double ca = poly_deg ? 2.0 / (12.0 - lambda_cut) : 0.0, cc = poly_deg ? -(12.0 + lambda_cut) / (12.0 - lambda_cut) : 0.0;
  const double sgn = (poly_deg % 2 == 0) ? -1.0 : 1.0;
  long long matvecs = 0;
  cudaStream_t sr = st;  // the stream the Lanczos steps go to (a capture stream while a restart cycle is recorded)
  // L x for every problem: FP64 stencil, or the complex64 stencil between a rounding and a widening
  auto stencil = [&](const double2* x, long long xb, double2* out) -> int {
    if (a.stencil_prec == ED_C128)
      return Ls ? ed_laplacian(ED_DF, Lx, Ly, Lz, B, 1, Ls, x, xb, out, n, sr)
                : ed_laplacian(ED_C128, Lx, Ly, Lz, B, 1, links, x, xb, out, n, sr);
    lz_to_c64_kernel<<<vgrid, LZ_THREADS, 0, sr>>>(n, x, xb, x32);
    int r = lz_chk(cudaGetLastError(), "Lanczos operand rounding");
    if (r != ED_OK) return r;
    if ((r = ed_laplacian(ED_C64, Lx, Ly, Lz, B, 1, a.links32, x32, n, y32, n, sr)) != ED_OK) return r;
    lz_from_c64_kernel<<<vgrid, LZ_THREADS, 0, sr>>>(n, y32, out);
    return lz_chk(cudaGetLastError(), "Lanczos result widening");
  };
  auto apply = [&](const double2* x, long long xb, double2* out) -> int {
    int r = stencil(x, xb, poly_deg ? lbuf : out);
    if (r != ED_OK || poly_deg == 0) return r;
    // T_0 = x, T_1 = A x, T_{k+1} = 2 A T_k - T_{k-1} with A = a L + c; the last step writes out, signed
    double2* bufs[3] = {t0, t1, t2};
    int ci = 1, pi = -1;  // T_k in bufs[ci]; T_{k-1} in bufs[pi], or x itself while pi < 0
    lz_cheb_kernel<<<vgrid, LZ_THREADS, 0, sr>>>(n, lbuf, x, xb, nullptr, 0, poly_deg == 1 ? out : bufs[ci], ca, cc,
                                                  1.0, poly_deg == 1 ? sgn : 1.0);
    if ((r = lz_chk(cudaGetLastError(), "Chebyshev step")) != ED_OK) return r;
    for (int kd = 2; kd <= poly_deg; ++kd) {
      if ((r = stencil(bufs[ci], n, lbuf)) != ED_OK) return r;
      const int ni = pi < 0 ? (ci + 1) % 3 : 3 - ci - pi;
      const bool last = kd == poly_deg;
      lz_cheb_kernel<<<vgrid, LZ_THREADS, 0, sr>>>(n, lbuf, bufs[ci], n, pi < 0 ? x : bufs[pi], pi < 0 ? xb : n,
                                                    last ? out : bufs[ni], ca, cc, 2.0, last ? sgn : 1.0);
      if ((r = lz_chk(cudaGetLastError(), "Chebyshev step")) != ED_OK) return r;
      pi = ci;
      ci = ni;
    }
    return ED_OK;
  };

  // one Gram-Schmidt pass of w against rows 0..j: FP64, or double-float on the split rows (split_w: w changed
  // since the last pass, so its split form is refreshed first)
  auto gs = [&](int j, double2* h, double* np, bool split_w) -> int {
    if (!a.gs_df) return ed_cgs_pass(B, j + 1, n, V, vb, w, h, ncv + 1, np, sr);
    int r = split_w ? split_rows(B, 1, n, w, n, wsp, n, sr) : ED_OK;
    if (r == ED_OK) r = cgs_pass_df(B, j + 1, n, Vs, vsb, w, wsp, h, ncv + 1, np, sr);
    return r;
  };
  // the split form of basis rows j0 .. j0 + nrow - 1 after they were written
  auto split_basis = [&](int j0, int nrow, cudaStream_t s2) -> int {
    return a.gs_df ? split_rows(B, nrow, n, V + (long long)j0 * n, vb, Vs + (long long)j0 * n, vsb, s2) : ED_OK;
  };
  // Lanczos steps k .. ncv-1 on stream sr
  auto cycle = [&](int k) -> int {
    int r;
    for (int j = k; j < ncv; ++j) {
      if ((r = apply(V + (long long)j * n, vb, w)) != ED_OK) return r;
      if (j == k) {
        if ((r = gs(j, hA, nullptr, true)) != ED_OK) return r;
        if ((r = gs(j, hB, npart, false)) != ED_OK) return r;
        lz_finish_kernel<<<vgrid, LZ_THREADS, 0, sr>>>(n, V, vb, j, w, hA, hB, ncv + 1, npart, nblk, d, e, bl, ncv, 1);
        if ((r = lz_chk(cudaGetLastError(), "Lanczos step end")) != ED_OK) return r;
        if ((r = split_basis(j + 1, 1, sr)) != ED_OK) return r;
      } else {
        lz_dot_kernel<<<vgrid, LZ_THREADS, 0, sr>>>(n, V + (long long)j * n, vb, w, n, part);
        if ((r = lz_chk(cudaGetLastError(), "Lanczos alpha")) != ED_OK) return r;
        lz_three_term_kernel<<<vgrid, LZ_THREADS, 0, sr>>>(n, V, vb, j, w, part, nblk, d, e, ncv);
        if ((r = lz_chk(cudaGetLastError(), "Lanczos recurrence")) != ED_OK) return r;
        if ((r = gs(j, hA, npart, true)) != ED_OK) return r;
        lz_finish_kernel<<<vgrid, LZ_THREADS, 0, sr>>>(n, V, vb, j, w, hA, nullptr, ncv + 1, npart, nblk, d, e, bl,
                                                        ncv, 0);
        if ((r = lz_chk(cudaGetLastError(), "Lanczos step end")) != ED_OK) return r;
        if ((r = split_basis(j + 1, 1, sr)) != ED_OK) return r;
      }
    }
    return ED_OK;
  };

  // From the second restart on every cycle runs the same launches (steps kk .. ncv-1): they are recorded once
  // on a private stream into a CUDA graph and replayed on the caller's stream.
  // If recording fails (a caller stream that is itself being captured, for instance), the cycles run eagerly.
  struct GraphRes {
    cudaStream_t cs = nullptr;
    cudaGraph_t g = nullptr;
    cudaGraphExec_t x = nullptr;
    bool unusable = false;
    void release() {
      if (x) cudaGraphExecDestroy(x);
      if (g) cudaGraphDestroy(g);
      if (cs) cudaStreamDestroy(cs);
      x = nullptr;
      g = nullptr;
      cs = nullptr;
    }
    ~GraphRes() { release(); }
  } gr;
  auto record = [&](int k) -> bool {
    if (cudaStreamCreateWithFlags(&gr.cs, cudaStreamNonBlocking) != cudaSuccess) return false;
    if (cudaStreamBeginCapture(gr.cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return false;
    sr = gr.cs;
    const int r = cycle(k);
    sr = st;
    const bool ended = cudaStreamEndCapture(gr.cs, &gr.g) == cudaSuccess;
    return r == ED_OK && ended && cudaGraphInstantiate(&gr.x, gr.g, 0) == cudaSuccess;
  };
  auto cycle_replayed = [&](int k) -> int {
    if (!gr.x && !gr.unusable && !record(k)) {
      gr.release();
      gr.unusable = true;
      cudaGetLastError();  // clear the failed recording's error; the eager cycle reports real launch errors
    }
    if (!gr.x) return cycle(k);
    return lz_chk(cudaGraphLaunch(gr.x, st), "Lanczos graph launch");
  };

  // start vectors
  if (a.start_nvec > 0)
    lz_sum_vectors_kernel<<<vgrid, LZ_THREADS, 0, st>>>(n, a.start_nvec, (const double2*)a.start, w);
  else
    lz_random_kernel<<<vgrid, LZ_THREADS, 0, st>>>(B, n, w, 12345u);
  LZ_LAUNCHED("Lanczos start vector");
  lz_dot_kernel<<<vgrid, LZ_THREADS, 0, st>>>(n, w, n, w, n, part);
  LZ_LAUNCHED("Lanczos start norm");
  lz_normalise_kernel<<<vgrid, LZ_THREADS, 0, st>>>(n, w, part, nblk, V, vb);
  LZ_LAUNCHED("Lanczos start normalise");
  LZ_TRY(split_basis(0, 1, st));

  int k = 0, restarts = 0, converged = 0, restart_cycles = 0;
  for (restarts = 1; restarts <= max_restarts; ++restarts) {
    if (k == 0 || restart_cycles == 0)
      LZ_TRY(cycle(k));  // the first restart cycle also warms up what the graph records
    else
      LZ_TRY(cycle_replayed(k));
    if (k > 0) ++restart_cycles;
    matvecs += (long long)(ncv - k) * (poly_deg ? poly_deg : 1);
    LZ_TRY(ed_arrow_eigh(B, ncv, k, kk, d, k > 0 ? s : nullptr, e, theta, Y, W + Lw.arrow, Lw.arrow_bytes, st));
    LZ_TRY(lz_chk(cudaMemsetAsync(nbad, 0, sizeof(int), st), "Lanczos convergence counter"));
    lz_converged_kernel<<<(B * Ne + 127) / 128, 128, 0, st>>>(B, ncv, kk, Ne, theta, Y, bl, tol, nbad);
    LZ_LAUNCHED("Lanczos convergence test");
    int hbad = -1;
    LZ_TRY(lz_chk(cudaMemcpyAsync(&hbad, nbad, sizeof(int), cudaMemcpyDeviceToHost, st), "Lanczos counter read"));
    LZ_TRY(lz_chk(cudaStreamSynchronize(st), "Lanczos synchronise"));
    if (hbad == 0) {
      converged = 1;
      break;
    }
    if (restarts == max_restarts) break;
    // thick restart: V[:, :kk] = Y[:, :kk]^T V[:, :ncv], V[:, kk] = V[:, ncv]
    LZ_TRY(lz_rotate(st, B, n, ncv, kk, V, vb, Vs, vsb, Y, kk, (long long)ncv * kk, rot, (long long)kk * n));
    LZ_TRY(lz_chk(cudaMemcpy2DAsync(V, vb * 16, rot, (size_t)kk * n * 16, (size_t)kk * n * 16, B,
                                         cudaMemcpyDeviceToDevice, st),
                       "Lanczos restart copy"));
    LZ_TRY(lz_chk(cudaMemcpy2DAsync(V + (long long)kk * n, vb * 16, V + (long long)ncv * n, vb * 16, (size_t)n * 16,
                                         B, cudaMemcpyDeviceToDevice, st),
                       "Lanczos residual vector copy"));
    lz_restart_kernel<<<(B * kk + 127) / 128, 128, 0, st>>>(B, ncv, kk, theta, Y, bl, d, s);
    LZ_LAUNCHED("Lanczos restart");
    LZ_TRY(split_basis(0, kk + 1, st));  // the rotated rows and the moved residual row
    k = kk;
  }
  if (restarts > max_restarts) restarts = max_restarts;
  // Ritz vectors X = Y[:, :Ne]^T V and values
  LZ_TRY(lz_rotate(st, B, n, ncv, Ne, V, vb, Vs, vsb, Y, kk, (long long)ncv * kk, (double2*)evecs, (long long)Ne * n));
  if (poly_deg == 0) {
    LZ_TRY(lz_chk(cudaMemcpy2DAsync(evals, (size_t)Ne * 8, theta, (size_t)kk * 8, (size_t)Ne * 8, B,
                                         cudaMemcpyDeviceToDevice, st),
                       "Lanczos eigenvalues"));
  } else {
    // eigenvalues of L: Rayleigh quotients, then ascending order
    double2* LX = rot;  // [B][Ne][n] (Ne <= kk)
    LZ_TRY(ed_laplacian(ED_C128, Lx, Ly, Lz, B, Ne, links, evecs, (long long)Ne * n, LX, (long long)Ne * n, st));
    matvecs += Ne;
    lz_rq_kernel<<<(unsigned)(B * Ne), LZ_THREADS, 0, st>>>(n, (const double2*)evecs, LX, rq);
    LZ_LAUNCHED("Rayleigh quotients");
    lz_sort_kernel<<<(B + 63) / 64, 64, 0, st>>>(B, Ne, rq, perm);
    LZ_LAUNCHED("eigenvalue sort");
    lz_gather_kernel<<<dim3((unsigned)std::min<long long>((n + 255) / 256, 64), Ne, B), 256, 0, st>>>(
        Ne, n, (const double2*)evecs, perm, LX);
    LZ_LAUNCHED("eigenvector reorder");
    LZ_TRY(lz_chk(
        cudaMemcpyAsync(evecs, LX, (size_t)B * Ne * n * 16, cudaMemcpyDeviceToDevice, st), "eigenvector copy"));
    LZ_TRY(lz_chk(cudaMemcpyAsync(evals, rq, (size_t)B * Ne * 8, cudaMemcpyDeviceToDevice, st),
                       "eigenvalue copy"));
  }
  status[0] = converged;
  status[1] = restarts;
  status[2] = (int)std::min<long long>(matvecs, 2147483647LL);
#undef LZ_TRY
#undef LZ_LAUNCHED
  return ED_OK;
}

}  // namespace
}  // namespace ed

extern "C" int ed_lanczos_tr(int Lx, int Ly, int Lz, int nt, const void* links, int Ne, double tol, int ncv,
                             int max_restarts, int poly_deg, double lambda_cut, void* evecs, double* evals, int* status,
                             void* workspace, size_t workspace_bytes, void* stream) {
  using namespace ed;
  ED_CHECK_ARG(Lx > 0 && Ly > 0 && Lz > 0 && nt > 0 && nt <= 65535 && Ne > 0, "ed_lanczos_tr: bad sizes");
  ED_CHECK_ARG(ed::lattice_ok(Lx, Ly, Lz), "ed_lanczos_tr: Lx*Ly*Lz above 2^28");
  const long long n = 3LL * Lx * Ly * Lz;
  ED_CHECK_ARG(Ne < ncv && ncv <= n, "ed_lanczos_tr: need Ne < ncv <= 3*Lx*Ly*Lz");
  ED_CHECK_ARG(tol > 0.0 && max_restarts > 0, "ed_lanczos_tr: need tol > 0 and max_restarts > 0");
  ED_CHECK_ARG(poly_deg >= 0 && (poly_deg == 0 || (lambda_cut > 0.0 && lambda_cut < 12.0)),
               "ed_lanczos_tr: a Chebyshev degree needs 0 < lambda_cut < 12");
  ED_CHECK_ARG(links && evecs && evals && status && workspace, "ed_lanczos_tr: null pointer");
  ED_CHECK_ARG(((uintptr_t)workspace % 256) == 0 && ((uintptr_t)evecs % 16) == 0 && ((uintptr_t)links % 16) == 0,
               "ed_lanczos_tr: workspace must be 256-byte aligned, links and evecs 16-byte aligned");
  const int nblk = (int)((n + LZ_THREADS - 1) / LZ_THREADS);
  const size_t need = lz_layout(nt, n, ncv, lz_kept(Ne, ncv), Ne, nblk).total;
  if (workspace_bytes < need) {
    set_error("ed_lanczos_tr: workspace of %zu bytes is smaller than the %zu needed", workspace_bytes, need);
    return ED_ERR_WORKSPACE;
  }
  LzArgs a{Lx, Ly, Lz, nt, links, nullptr, ED_C128, Ne, tol, ncv, max_restarts, poly_deg, lambda_cut,
           evecs, evals, nullptr, 0, status, workspace, (cudaStream_t)stream};
  return lanczos_solve(a);
}

namespace ed {
namespace {
// Krylov dimension of the FP64 Chebyshev refinement of the mixed solve: 2 Ne, at least Ne + 32 (measured best for
// the Chebyshev-filtered iteration), at most the problem size
int lz_refine_ncv(int Ne, long long n) { return (int)std::min<long long>(std::max(2 * Ne, Ne + 32), n); }
}  // namespace
}  // namespace ed

extern "C" int ed_lanczos_workspace_ex(int Lx, int Ly, int Lz, int nt, int Ne, int ncv, int stencil_prec,
                                       size_t* bytes) {
  ED_CHECK_ARG(bytes, "ed_lanczos_workspace_ex: null pointer");
  const bool gs_df = (stencil_prec & ED_LANCZOS_GS_DF) != 0;
  const int sp = stencil_prec & ~ED_LANCZOS_GS_DF;
  ED_CHECK_ARG(sp == ED_C128 || sp == ED_C64, "ed_lanczos_workspace_ex: bad stencil precision");
  ED_CHECK_ARG(Lx > 0 && Ly > 0 && Lz > 0 && nt > 0 && nt <= 65535 && Ne > 0, "ed_lanczos_workspace_ex: bad sizes");
  ED_CHECK_ARG(ed::lattice_ok(Lx, Ly, Lz), "ed_lanczos_workspace_ex: Lx*Ly*Lz above 2^28");
  const long long n = 3LL * Lx * Ly * Lz;
  ED_CHECK_ARG(Ne < ncv && ncv <= n, "ed_lanczos_workspace_ex: need Ne < ncv <= 3*Lx*Ly*Lz");
  const int nblk = (int)((n + ed::LZ_THREADS - 1) / ed::LZ_THREADS);
  size_t need = ed::lz_layout(nt, n, ncv, ed::lz_kept(Ne, ncv), Ne, nblk, gs_df).total;
  if (sp == ED_C64) {
    const int ncv2 = ed::lz_refine_ncv(Ne, n);
    if (ncv2 > Ne) need = std::max(need, ed::lz_layout(nt, n, ncv2, ed::lz_kept(Ne, ncv2), Ne, nblk, gs_df).total);
    need += ed::lz_c64_bytes(nt, n);
  }
  *bytes = need;
  return ED_OK;
}

extern "C" int ed_lanczos_tr_ex(int Lx, int Ly, int Lz, int nt, const void* links, const void* links_c64,
                                int stencil_prec, int Ne, double tol, int ncv, int max_restarts, int poly_deg,
                                double lambda_cut, void* evecs, double* evals, int* status, void* workspace,
                                size_t workspace_bytes, void* stream) {
  using namespace ed;
  const bool gs_df = (stencil_prec & ED_LANCZOS_GS_DF) != 0;
  const int sp = stencil_prec & ~ED_LANCZOS_GS_DF;
  ED_CHECK_ARG(sp == ED_C128 || sp == ED_C64, "ed_lanczos_tr_ex: bad stencil precision");
  ED_CHECK_ARG(status, "ed_lanczos_tr_ex: null status");
  for (int q = 0; q < 6; ++q) status[q] = 0;
  if (sp == ED_C128 && !gs_df) {
    const int rc = ed_lanczos_tr(Lx, Ly, Lz, nt, links, Ne, tol, ncv, max_restarts, poly_deg, lambda_cut, evecs, evals,
                                 status, workspace, workspace_bytes, stream);
    status[4] = status[2];
    return rc;
  }
  if (sp == ED_C128) {  // FP64 stencil, double-float Gram-Schmidt
    ED_CHECK_ARG(Lx > 0 && Ly > 0 && Lz > 0 && nt > 0 && nt <= 65535 && Ne > 0, "ed_lanczos_tr_ex: bad sizes");
    ED_CHECK_ARG(ed::lattice_ok(Lx, Ly, Lz), "ed_lanczos_tr_ex: Lx*Ly*Lz above 2^28");
    const long long n = 3LL * Lx * Ly * Lz;
    ED_CHECK_ARG(Ne < ncv && ncv <= n, "ed_lanczos_tr_ex: need Ne < ncv <= 3*Lx*Ly*Lz");
    ED_CHECK_ARG(tol > 0.0 && max_restarts > 0, "ed_lanczos_tr_ex: need tol > 0 and max_restarts > 0");
    ED_CHECK_ARG(poly_deg >= 0 && (poly_deg == 0 || (lambda_cut > 0.0 && lambda_cut < 12.0)),
                 "ed_lanczos_tr_ex: a Chebyshev degree needs 0 < lambda_cut < 12");
    ED_CHECK_ARG(links && evecs && evals && workspace, "ed_lanczos_tr_ex: null pointer");
    ED_CHECK_ARG(((uintptr_t)workspace % 256) == 0 && ((uintptr_t)evecs % 16) == 0 && ((uintptr_t)links % 16) == 0,
                 "ed_lanczos_tr_ex: workspace must be 256-byte aligned, links and evecs 16-byte aligned");
    size_t need = 0;
    int rc = ed_lanczos_workspace_ex(Lx, Ly, Lz, nt, Ne, ncv, stencil_prec, &need);
    if (rc != ED_OK) return rc;
    if (workspace_bytes < need) {
      set_error("ed_lanczos_tr_ex: workspace of %zu bytes is smaller than the %zu needed", workspace_bytes, need);
      return ED_ERR_WORKSPACE;
    }
    LzArgs a{Lx, Ly, Lz, nt, links, nullptr, ED_C128, Ne, tol, ncv, max_restarts, poly_deg, lambda_cut,
             evecs, evals, nullptr, 0, status, workspace, (cudaStream_t)stream, true};
    rc = lanczos_solve(a);
    status[4] = status[2];
    return rc;
  }
  ED_CHECK_ARG(Lx > 0 && Ly > 0 && Lz > 0 && nt > 0 && nt <= 65535 && Ne > 0, "ed_lanczos_tr_ex: bad sizes");
  ED_CHECK_ARG(ed::lattice_ok(Lx, Ly, Lz), "ed_lanczos_tr_ex: Lx*Ly*Lz above 2^28");
  const long long n = 3LL * Lx * Ly * Lz;
  ED_CHECK_ARG(Ne < ncv && ncv <= n, "ed_lanczos_tr_ex: need Ne < ncv <= 3*Lx*Ly*Lz");
  ED_CHECK_ARG(tol > 0.0 && max_restarts > 0 && poly_deg >= 0, "ed_lanczos_tr_ex: need tol > 0, max_restarts > 0");
  ED_CHECK_ARG(links && links_c64 && evecs && evals && workspace, "ed_lanczos_tr_ex: null pointer");
  ED_CHECK_ARG(((uintptr_t)workspace % 256) == 0 && ((uintptr_t)evecs % 16) == 0 && ((uintptr_t)links % 16) == 0 &&
                   ((uintptr_t)links_c64 % 16) == 0,
               "ed_lanczos_tr_ex: workspace must be 256-byte aligned, links and evecs 16-byte aligned");
  ED_CHECK_ARG(Lx % 2 == 0, "ed_lanczos_tr_ex: the complex64 stencil needs an even Lx");
  size_t need = 0;
  int rc = ed_lanczos_workspace_ex(Lx, Ly, Lz, nt, Ne, ncv, stencil_prec, &need);
  if (rc != ED_OK) return rc;
  if (workspace_bytes < need) {
    set_error("ed_lanczos_tr_ex: workspace of %zu bytes is smaller than the %zu needed", workspace_bytes, need);
    return ED_ERR_WORKSPACE;
  }
  const int ncv2 = lz_refine_ncv(Ne, n);
  cudaStream_t st = (cudaStream_t)stream;
  // phase 1: complex64 stencil, FP64 basis, Gram-Schmidt and Rayleigh-Ritz, to the loose tolerance LZ_MIXED_TOL
  int st1[3] = {0, 0, 0};
  LzArgs a1{Lx, Ly, Lz, nt, links, links_c64, ED_C64, Ne, std::max(tol, LZ_MIXED_TOL), ncv,
            std::min(max_restarts, LZ_MIXED_RESTARTS), 0, 0.0, evecs, evals, nullptr, 0, st1, workspace, st, gs_df};
  if ((rc = lanczos_solve(a1)) != ED_OK) return rc;
  int lap_code = 0;  // a bounded wait of the TMA-staged complex64 stencil that gave up invalidates phase 1
  if ((rc = ed_laplacian_status(&lap_code, st)) != ED_OK) return rc;
  // the Chebyshev cut: 15 % above the largest wanted phase-1 eigenvalue of any timeslice (a caller's cut wins)
  double cut = lambda_cut;
  if (!(cut > 0.0)) {
    std::vector<double> ev((size_t)nt * Ne);
    rc = lz_chk(cudaMemcpyAsync(ev.data(), evals, ev.size() * 8, cudaMemcpyDeviceToHost, st), "phase-1 eigenvalues");
    if (rc == ED_OK) rc = lz_chk(cudaStreamSynchronize(st), "phase-1 synchronise");
    if (rc != ED_OK) return rc;
    double top = 0.0;
    for (int b = 0; b < nt; ++b) top = std::max(top, ev[(size_t)b * Ne + Ne - 1]);
    cut = 1.15 * top;
  }
  // phase 2: FP64 stencil, Chebyshev-filtered, started from the sum of the phase-1 Ritz vectors, which stay in
  // evecs (the solve reads them into its start vector first and writes evecs only at its end)
  int st2[3] = {0, 0, 0};
  const int deg = poly_deg > 0 ? poly_deg : LZ_MIXED_DEG;
  const bool cheb = cut > 0.0 && cut < 12.0 && ncv2 > Ne;
  LzArgs a2{Lx, Ly, Lz, nt, links, nullptr, ED_C128, Ne, cheb ? std::max(tol, 1e-12) : tol, cheb ? ncv2 : ncv,
            max_restarts, cheb ? deg : 0, cheb ? cut : 0.0, evecs, evals, evecs, Ne, st2, workspace, st, gs_df};
  if ((rc = lanczos_solve(a2)) != ED_OK) return rc;
  status[0] = st2[0];
  status[1] = st1[1] + st2[1];
  status[2] = (int)std::min<long long>((long long)st1[2] + st2[2], 2147483647LL);
  status[3] = st1[2];
  status[4] = st2[2];
  status[5] = st1[1];
  return ED_OK;
}
