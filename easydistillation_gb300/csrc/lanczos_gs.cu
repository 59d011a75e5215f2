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

#include <algorithm>

#include "common.cuh"
#include "df.cuh"

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

// ---------------------------------------------------------------- double-float pass on the FP32 pipe
// The same pass with every complex128 value of V and w carried in the split form of df.cuh, the basis
// rows stored once in that form (Vs, written when a row is made) and the sums kept as (hi, lo) FP32 pairs:
// every operation runs on the FP32 pipe, so a pass streams its 16 bytes per element at HBM speed instead
// of the FP64 pipe's ~2.5 TB/s.

// dst rows (stride db elements per problem) <- split of src rows (stride sb); nrow rows of n elements
__global__ void split_rows_kernel(long long n, int nrow, const double2* __restrict__ src, long long sb,
                                  float4* __restrict__ dst, long long db) {
  const int b = blockIdx.z, row = blockIdx.y;
  if (row >= nrow) return;
  const double2* s = src + (long long)b * sb + (long long)row * n;
  float4* d = dst + (long long)b * db + (long long)row * n;
  for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (long long)gridDim.x * blockDim.x)
    d[x] = split_c128(s[x]);
}

__global__ void __launch_bounds__(GS_THREADS) cgs_project_df_kernel(int r, long long n, const float4* __restrict__ Vs,
                                                                    long long vb, const float4* __restrict__ ws,
                                                                    double2* __restrict__ h, int ldh) {
  const int b = blockIdx.y, i0 = blockIdx.x * GS_ROWS;
  const float4* Vb = Vs + (long long)b * vb + (long long)i0 * n;
  const float4* wb = ws + (long long)b * n;
  const int nrows = min(GS_ROWS, r - i0);
  DF re[GS_ROWS], im[GS_ROWS];
#pragma unroll
  for (int q = 0; q < GS_ROWS; ++q) re[q] = im[q] = DF{0.f, 0.f};
  for (long long x = threadIdx.x; x < n; x += GS_THREADS) {
    const float4 w = wb[x];
    float4 v[GS_ROWS];
#pragma unroll
    for (int q = 0; q < GS_ROWS; ++q) v[q] = q < nrows ? __ldcs(Vb + q * n + x) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int q = 0; q < GS_ROWS; ++q) {
      // conj(v) w: re = vr wr + vi wi, im = vr wi - vi wr
      df_acc(re[q], v[q].x, v[q].z, w.x, w.z);
      df_acc(re[q], v[q].y, v[q].w, w.y, w.w);
      df_acc(im[q], v[q].x, v[q].z, w.y, w.w);
      df_sub(im[q], v[q].y, v[q].w, w.x, w.z);
    }
  }
  // FP64 reduction of the (hi, lo) pairs: small next to the streamed rows
  __shared__ double2 part[GS_THREADS / 32][GS_ROWS];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int q = 0; q < GS_ROWS; ++q) {
    double a = (double)re[q].hi + (double)re[q].lo, c = (double)im[q].hi + (double)im[q].lo;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      c += __shfl_xor_sync(0xffffffffu, c, o);
    }
    if (lane == 0) part[warp][q] = make_double2(a, c);
  }
  __syncthreads();
  if (threadIdx.x < nrows) {
    double2 t = make_double2(0.0, 0.0);
    for (int wgp = 0; wgp < GS_THREADS / 32; ++wgp) {
      t.x += part[wgp][threadIdx.x].x;
      t.y += part[wgp][threadIdx.x].y;
    }
    h[(long long)b * ldh + i0 + threadIdx.x] = t;
  }
}

__global__ void __launch_bounds__(GS_THREADS) cgs_update_df_kernel(int r, long long n, const float4* __restrict__ Vs,
                                                                   long long vb, const double2* __restrict__ h, int ldh,
                                                                   double2* __restrict__ w, float4* __restrict__ ws,
                                                                   double* __restrict__ norm_part) {
  __shared__ float4 hs[GS_HCHUNK];
  const int b = blockIdx.y;
  const long long x = (long long)blockIdx.x * GS_THREADS + threadIdx.x;
  const float4* Vb = Vs + (long long)b * vb;
  DF re{0.f, 0.f}, im{0.f, 0.f};
  for (int c0 = 0; c0 < r; c0 += GS_HCHUNK) {
    const int cn = min(GS_HCHUNK, r - c0);
    __syncthreads();
    for (int i = threadIdx.x; i < cn; i += GS_THREADS) hs[i] = split_c128(h[(long long)b * ldh + c0 + i]);
    __syncthreads();
    if (x < n) {
      const float4* col = Vb + (long long)c0 * n + x;
      int i = 0;
      for (; i + 4 <= cn; i += 4) {
        float4 v[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) v[q] = __ldcs(col + (long long)(i + q) * n);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float4 hq = hs[i + q];  // h v: re = hr vr - hi vi, im = hr vi + hi vr
          df_acc(re, hq.x, hq.z, v[q].x, v[q].z);
          df_sub(re, hq.y, hq.w, v[q].y, v[q].w);
          df_acc(im, hq.x, hq.z, v[q].y, v[q].w);
          df_acc(im, hq.y, hq.w, v[q].x, v[q].z);
        }
      }
      for (; i < cn; ++i) {
        const float4 v = __ldcs(col + (long long)i * n), hq = hs[i];
        df_acc(re, hq.x, hq.z, v.x, v.z);
        df_sub(re, hq.y, hq.w, v.y, v.w);
        df_acc(im, hq.x, hq.z, v.y, v.w);
        df_acc(im, hq.y, hq.w, v.x, v.z);
      }
    }
  }
  double sq = 0.0;
  if (x < n) {
    double2* wx = w + (long long)b * n + x;
    double2 o = *wx;
    o.x -= (double)re.hi + (double)re.lo;
    o.y -= (double)im.hi + (double)im.lo;
    *wx = o;
    if (ws) ws[(long long)b * n + x] = split_c128(o);  // the updated w in split form, for a second pass
    sq = o.x * o.x + o.y * o.y;
  }
  if (norm_part) {
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

// Split nrow complex128 rows (batch stride sb) into the float4 form of the double-float pass (batch stride db).
int split_rows(int B, int nrow, long long n, const void* src, long long sb, void* dst, long long db,
               cudaStream_t st) {
  if (nrow <= 0) return ED_OK;
  const dim3 g((unsigned)std::min<long long>((n + GS_THREADS - 1) / GS_THREADS, 1024), (unsigned)nrow, (unsigned)B);
  split_rows_kernel<<<g, GS_THREADS, 0, st>>>(n, nrow, (const double2*)src, sb, (float4*)dst, db);
  ED_RETURN_LAUNCH("double-float split");
  return ED_OK;
}

// The double-float pass: ws holds w in split form on entry (split_rows) and on exit (the updated w).
int cgs_pass_df(int B, int r, long long n, const void* Vs, long long vs_bstride, void* w, void* ws, void* h, int ldh,
                double* norm_part, cudaStream_t st) {
  const dim3 g1((r + GS_ROWS - 1) / GS_ROWS, B);
  cgs_project_df_kernel<<<g1, GS_THREADS, 0, st>>>(r, n, (const float4*)Vs, vs_bstride, (const float4*)ws,
                                                   (double2*)h, ldh);
  ED_RETURN_LAUNCH("double-float Gram-Schmidt projection");
  const dim3 g2((unsigned)((n + GS_THREADS - 1) / GS_THREADS), B);
  cgs_update_df_kernel<<<g2, GS_THREADS, 0, st>>>(r, n, (const float4*)Vs, vs_bstride, (const double2*)h, ldh,
                                                  (double2*)w, (float4*)ws, norm_part);
  ED_RETURN_LAUNCH("double-float Gram-Schmidt update");
  return ED_OK;
}
}  // namespace ed

extern "C" int ed_cgs_pass_df(int B, int r, long long n, const void* V, long long v_bstride, void* w, void* h, int ldh,
                              double* norm_part, void* workspace, size_t workspace_bytes, void* stream) {
  ED_CHECK_ARG(B > 0 && r > 0 && n > 0, "ed_cgs_pass_df: sizes must be positive");
  ED_CHECK_ARG(B <= 65535 && r <= 65535 && ldh >= r, "ed_cgs_pass_df: need B, r <= 65535 and ldh >= r");
  ED_CHECK_ARG(v_bstride >= (long long)r * n, "ed_cgs_pass_df: batch stride of V smaller than r*n");
  ED_CHECK_ARG(V && w && h && workspace, "ed_cgs_pass_df: null pointer");
  ED_CHECK_ARG(((uintptr_t)V % 16) == 0 && ((uintptr_t)w % 16) == 0 && ((uintptr_t)h % 16) == 0 &&
                   ((uintptr_t)workspace % 16) == 0,
               "ed_cgs_pass_df: pointers must be 16-byte aligned");
  const size_t need = (size_t)B * (r + 1) * n * 16;
  if (workspace_bytes < need) {
    ed::set_error("ed_cgs_pass_df: workspace of %zu bytes is smaller than the %zu needed", workspace_bytes, need);
    return ED_ERR_WORKSPACE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  float4* Vs = (float4*)workspace;  // [B][r][n]
  float4* ws = Vs + (size_t)B * r * n;  // [B][n]
  int rc = ed::split_rows(B, r, n, V, v_bstride, Vs, (long long)r * n, st);
  if (rc == ED_OK) rc = ed::split_rows(B, 1, n, w, n, ws, n, st);
  if (rc == ED_OK) rc = ed::cgs_pass_df(B, r, n, Vs, (long long)r * n, w, ws, h, ldh, norm_part, st);
  return rc;
}

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
