// Classical Gram-Schmidt pass of thick-restart Lanczos, batched over
// timeslices, complex128:
//
//   h[b][i] = sum_x conj(V[b][i][x]) w[b][x]      (i < r)
//   w[b][x] -= sum_i h[b][i] V[b][i][x]
//
// This is the reorthogonalisation inside the eigensolve the reference
// delegates to ARPACK / cupyx eigsh (lattice/generator/eigenvector.py:234-257).
// Both halves stream the r basis rows once from HBM (the basis is far larger
// than L2: 8 timeslices x 300 rows x 3*24^3 sites = 1.6 GB): 16-byte loads,
// several independent rows per thread, enough blocks to fill every SM.  Each
// 16-byte element costs one complex multiply-add (8 flops), and GB300's FP64
// pipe (about 1.25 TFLOP/s) caps that at about 2.5 TB/s of basis: measured
// 2.1-2.3 TB/s at 8 x 250 x 41472, the same as cuBLAS's batched GEMV, so the
// pass is FP64-bound, not HBM-bound.  The update kernel also returns per-block
// partial sums of |w|^2, which saves the separate norm reduction.

#include "common.cuh"

namespace ed {
namespace {

constexpr int GS_ROWS = 4;       // basis rows per block of the projection
constexpr int GS_THREADS = 256;
constexpr int GS_HCHUNK = 1024;  // projections staged in shared memory per chunk of the update

__device__ __forceinline__ void cfma_conj(double2& acc, double2 v, double2 w) {
  // acc += conj(v) * w
  acc.x = fma(v.x, w.x, fma(v.y, w.y, acc.x));
  acc.y = fma(v.x, w.y, fma(-v.y, w.x, acc.y));
}

__global__ void __launch_bounds__(GS_THREADS) cgs_project_kernel(int r, long long n, const double2* __restrict__ V,
                                                                 long long vb, const double2* __restrict__ w,
                                                                 double2* __restrict__ h, int ldh) {
  const int b = blockIdx.y, i0 = blockIdx.x * GS_ROWS;
  const double2* Vb = V + (long long)b * vb + (long long)i0 * n;
  const double2* wb = w + (long long)b * n;
  const int nrows = min(GS_ROWS, r - i0);
  double2 acc[GS_ROWS];
#pragma unroll
  for (int q = 0; q < GS_ROWS; ++q) acc[q] = make_double2(0.0, 0.0);
  if (nrows == GS_ROWS) {
    for (long long x = threadIdx.x; x < n; x += GS_THREADS) {
      const double2 wx = wb[x];
      double2 v[GS_ROWS];
#pragma unroll
      for (int q = 0; q < GS_ROWS; ++q) v[q] = __ldcs(Vb + q * n + x);
#pragma unroll
      for (int q = 0; q < GS_ROWS; ++q) cfma_conj(acc[q], v[q], wx);
    }
  } else {
    for (long long x = threadIdx.x; x < n; x += GS_THREADS) {
      const double2 wx = wb[x];
      for (int q = 0; q < nrows; ++q) cfma_conj(acc[q], __ldcs(Vb + q * n + x), wx);
    }
  }
  __shared__ double2 part[GS_THREADS / 32][GS_ROWS];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int q = 0; q < GS_ROWS; ++q) {
    double re = acc[q].x, im = acc[q].y;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      re += __shfl_xor_sync(0xffffffffu, re, o);
      im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    if (lane == 0) part[warp][q] = make_double2(re, im);
  }
  __syncthreads();
  if (threadIdx.x < nrows) {
    double2 s = make_double2(0.0, 0.0);
    for (int wgp = 0; wgp < GS_THREADS / 32; ++wgp) {
      s.x += part[wgp][threadIdx.x].x;
      s.y += part[wgp][threadIdx.x].y;
    }
    h[(long long)b * ldh + i0 + threadIdx.x] = s;
  }
}

__global__ void __launch_bounds__(GS_THREADS) cgs_update_kernel(int r, long long n, const double2* __restrict__ V,
                                                                long long vb, const double2* __restrict__ h, int ldh,
                                                                double2* __restrict__ w, double* __restrict__ norm_part) {
  __shared__ double2 hs[GS_HCHUNK];
  const int b = blockIdx.y;
  const long long x = (long long)blockIdx.x * GS_THREADS + threadIdx.x;
  const double2* Vb = V + (long long)b * vb;
  double2 acc = make_double2(0.0, 0.0);
  for (int c0 = 0; c0 < r; c0 += GS_HCHUNK) {
    const int cn = min(GS_HCHUNK, r - c0);
    __syncthreads();
    for (int i = threadIdx.x; i < cn; i += GS_THREADS) hs[i] = h[(long long)b * ldh + c0 + i];
    __syncthreads();
    if (x < n) {
      const double2* col = Vb + (long long)c0 * n + x;
      int i = 0;
      for (; i + 4 <= cn; i += 4) {
        double2 v[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) v[q] = __ldcs(col + (long long)(i + q) * n);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const double2 hq = hs[i + q];
          acc.x = fma(hq.x, v[q].x, fma(-hq.y, v[q].y, acc.x));
          acc.y = fma(hq.x, v[q].y, fma(hq.y, v[q].x, acc.y));
        }
      }
      for (; i < cn; ++i) {
        const double2 v = __ldcs(col + (long long)i * n), hq = hs[i];
        acc.x = fma(hq.x, v.x, fma(-hq.y, v.y, acc.x));
        acc.y = fma(hq.x, v.y, fma(hq.y, v.x, acc.y));
      }
    }
  }
  double sq = 0.0;
  if (x < n) {
    double2* wx = w + (long long)b * n + x;
    double2 o = *wx;
    o.x -= acc.x;
    o.y -= acc.y;
    *wx = o;
    sq = o.x * o.x + o.y * o.y;
  }
  if (norm_part) {  // this block's share of ||w_new||^2 (summed by the caller in a fixed order)
    __shared__ double red[GS_THREADS / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sq;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int q = 0; q < GS_THREADS / 32; ++q) t += red[q];
      norm_part[(long long)b * gridDim.x + blockIdx.x] = t;
    }
  }
}

}  // namespace
}  // namespace ed

extern "C" int ed_cgs_pass(int B, int r, long long n, const void* V, long long v_bstride, void* w, void* h, int ldh,
                           double* norm_part, void* stream) {
  ED_CHECK_ARG(B > 0 && r > 0 && n > 0, "ed_cgs_pass: sizes must be positive");
  ED_CHECK_ARG(B <= 65535 && ldh >= r, "ed_cgs_pass: need B <= 65535 and ldh >= r");
  ED_CHECK_ARG(v_bstride >= (long long)r * n, "ed_cgs_pass: batch stride of V smaller than r*n");
  ED_CHECK_ARG(V && w && h, "ed_cgs_pass: null pointer");
  ED_CHECK_ARG(((uintptr_t)V % 16) == 0 && ((uintptr_t)w % 16) == 0 && ((uintptr_t)h % 16) == 0,
               "ed_cgs_pass: pointers must be 16-byte aligned");
  cudaStream_t st = (cudaStream_t)stream;
  const dim3 g1((r + ed::GS_ROWS - 1) / ed::GS_ROWS, B);
  ed::cgs_project_kernel<<<g1, ed::GS_THREADS, 0, st>>>(r, n, (const double2*)V, v_bstride, (const double2*)w,
                                                         (double2*)h, ldh);
  ED_RETURN_LAUNCH("Gram-Schmidt projection");
  const dim3 g2((unsigned)((n + ed::GS_THREADS - 1) / ed::GS_THREADS), B);
  ed::cgs_update_kernel<<<g2, ed::GS_THREADS, 0, st>>>(r, n, (const double2*)V, v_bstride, (const double2*)h, ldh,
                                                        (double2*)w, norm_part);
  ED_RETURN_LAUNCH("Gram-Schmidt update");
  return ED_OK;
}
