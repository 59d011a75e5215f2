// 3D covariant Laplacian and single covariant-derivative hop on SoA links.
//
// Laplacian (reference lattice/generator/eigenvector.py:11-26):
//   (L F)(x) = 6 F(x) - sum_{mu=x,y,z} [ U_mu(x) F(x+mu) + U_mu(x-mu)^dag F(x-mu) ]
// Covariant derivative hop (reference lattice/generator/elemental.py:282-287):
//   (D_d F)(x) = U_d(x) F(x+d) - U_d(x-d)^dag F(x-d)           (no factor 1/2)
// Periodic boundaries in x, y, z.  Links are SoA per timeslice
// [dir][row][col][V3], vectors are colour planes [colour][V3].
//
// The Laplacian is HBM-bound: per application it moves 27 link + 3 input +
// 3 output complex numbers per site.  Every thread handles S consecutive
// x-sites so that every plane access is one 128-bit load (S=1 for c128 =
// double2, S=2 for c64 = float4).
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>

#include "common.cuh"
#include "df.cuh"

namespace ed {

// 1: complex64 Laplacians go through the TMA-staged kernel where it applies.
// Off by default: at 32^3 x 64 timeslices it reaches 68 % of the measured HBM
// copy bandwidth against 83 % for the kernel that reads neighbours through
// L1/L2 (the links, 27 of the 33 complex numbers per site, dominate the
// traffic, and the per-plane block barrier costs latency hiding).
static int g_stencil_tma = 2;  // ed_laplacian_config: 0 L1/L2, 1 TMA input planes, 2 TMA strips (default)

template <typename T, int S>
struct Pack;

template <>
struct Pack<double, 1> {
  __device__ __forceinline__ static void load(const cplx<double>* p, cplx<double> (&o)[1]) { o[0] = ld(p); }
  __device__ __forceinline__ static void store(cplx<double>* p, const cplx<double> (&o)[1]) {
    *reinterpret_cast<double2*>(p) = make_double2(o[0].re, o[0].im);
  }
};

template <>
struct Pack<float, 2> {
  __device__ __forceinline__ static void load(const cplx<float>* p, cplx<float> (&o)[2]) {
    float4 v = __ldg(reinterpret_cast<const float4*>(p));
    o[0] = mk(v.x, v.y);
    o[1] = mk(v.z, v.w);
  }
  __device__ __forceinline__ static void store(cplx<float>* p, const cplx<float> (&o)[2]) {
    *reinterpret_cast<float4*>(p) = make_float4(o[0].re, o[0].im, o[1].re, o[1].im);
  }
};

// y += U x  (U given as 9 row-major complex)
template <typename T>
__device__ __forceinline__ void mv_add(cplx<T> (&y)[3], const cplx<T> (&U)[9], const cplx<T> (&x)[3]) {
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) cfma(y[a], U[a * 3 + b], x[b]);
}
// y += U^dag x
template <typename T>
__device__ __forceinline__ void mvd_add(cplx<T> (&y)[3], const cplx<T> (&U)[9], const cplx<T> (&x)[3]) {
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) cfma_conj(y[a], U[b * 3 + a], x[b]);
}

// One launch covers nt timeslices x nvec vectors; grid (sites/S/128, nvec, nt).
template <typename T, int S>
__global__ void __launch_bounds__(128, 8) laplacian_kernel(Latt L, const cplx<T>* __restrict__ links,
                                                        const cplx<T>* __restrict__ in, cplx<T>* __restrict__ out,
                                                        long long link_tstride, long long in_tstride,
                                                        long long out_tstride, T diag) {
  const int V3 = L.V3();
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid * S >= V3) return;
  const int t = blockIdx.z;
  const cplx<T>* U = links + (long long)t * link_tstride;
  const long long voff = (long long)blockIdx.y * 3 * V3;
  const cplx<T>* F = in + (long long)t * in_tstride + voff;
  cplx<T>* O = out + (long long)t * out_tstride + voff;

  const int s0 = tid * S;
  const int x0 = s0 % L.Lx;
  const int yz = s0 / L.Lx;
  const int y = yz % L.Ly;
  const int z = yz / L.Ly;
  const int row = s0 - x0;  // site of (0, y, z)

  cplx<T> acc[S][3];
  {
    cplx<T> f[3][S];
#pragma unroll
    for (int c = 0; c < 3; ++c) Pack<T, S>::load(F + c * V3 + s0, f[c]);
#pragma unroll
    for (int s = 0; s < S; ++s)
#pragma unroll
      for (int c = 0; c < 3; ++c) acc[s][c] = mk(diag * f[c][s].re, diag * f[c][s].im);
  }
  cplx<T> hop[S][3];
#pragma unroll
  for (int s = 0; s < S; ++s)
#pragma unroll
    for (int c = 0; c < 3; ++c) hop[s][c] = mk(T(0), T(0));

  // ---------------- x direction (mu = 0)
  {
    const int xm = wrap_dec(x0, L.Lx);
    const int xp = (x0 + S) % L.Lx;
    cplx<T> uf[9][S];
#pragma unroll
    for (int e = 0; e < 9; ++e) Pack<T, S>::load(U + (0 * 9 + e) * V3 + s0, uf[e]);
    cplx<T> ff[3][S];
#pragma unroll
    for (int c = 0; c < 3; ++c) Pack<T, S>::load(F + c * V3 + s0, ff[c]);
    cplx<T> fxp[3], fxm[3], ubm[9];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      fxp[c] = ld(F + c * V3 + row + xp);
      fxm[c] = ld(F + c * V3 + row + xm);
    }
#pragma unroll
    for (int e = 0; e < 9; ++e) ubm[e] = ld(U + (0 * 9 + e) * V3 + row + xm);
#pragma unroll
    for (int s = 0; s < S; ++s) {
      cplx<T> u[9], fn[3];
#pragma unroll
      for (int e = 0; e < 9; ++e) u[e] = uf[e][s];
#pragma unroll
      for (int c = 0; c < 3; ++c) fn[c] = (s + 1 < S) ? ff[c][(s + 1) % S] : fxp[c];
      mv_add(hop[s], u, fn);
      cplx<T> ub[9], fb[3];
#pragma unroll
      for (int e = 0; e < 9; ++e) ub[e] = (s > 0) ? uf[e][(s + S - 1) % S] : ubm[e];
#pragma unroll
      for (int c = 0; c < 3; ++c) fb[c] = (s > 0) ? ff[c][(s + S - 1) % S] : fxm[c];
      mvd_add(hop[s], ub, fb);
    }
  }
  // ---------------- y and z directions (mu = 1, 2)
#pragma unroll
  for (int mu = 1; mu < 3; ++mu) {
    int sp, sm;
    if (mu == 1) {
      sp = s0 + (wrap_inc(y, L.Ly) - y) * L.Lx;
      sm = s0 + (wrap_dec(y, L.Ly) - y) * L.Lx;
    } else {
      sp = s0 + (wrap_inc(z, L.Lz) - z) * L.Lx * L.Ly;
      sm = s0 + (wrap_dec(z, L.Lz) - z) * L.Lx * L.Ly;
    }
    cplx<T> uf[9][S], ub[9][S], fp[3][S], fm[3][S];
#pragma unroll
    for (int e = 0; e < 9; ++e) {
      Pack<T, S>::load(U + (mu * 9 + e) * V3 + s0, uf[e]);
      Pack<T, S>::load(U + (mu * 9 + e) * V3 + sm, ub[e]);
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      Pack<T, S>::load(F + c * V3 + sp, fp[c]);
      Pack<T, S>::load(F + c * V3 + sm, fm[c]);
    }
#pragma unroll
    for (int s = 0; s < S; ++s) {
      cplx<T> u[9], v[9], a[3], b[3];
#pragma unroll
      for (int e = 0; e < 9; ++e) {
        u[e] = uf[e][s];
        v[e] = ub[e][s];
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        a[c] = fp[c][s];
        b[c] = fm[c][s];
      }
      mv_add(hop[s], u, a);
      mvd_add(hop[s], v, b);
    }
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    cplx<T> o[S];
#pragma unroll
    for (int s = 0; s < S; ++s) o[s] = acc[s][c] - hop[s][c];
    Pack<T, S>::store(O + c * V3 + s0, o);
  }
}

// Covariant-derivative hop in direction d for a block of vectors.  Links are
// held in registers (two 3x3 per site) and reused over VB vectors.  Math in
// the links' precision TM (double, or float for the complex64 chains of the
// split-precision elemental modes); input/output storage TI/TO.
template <typename TI, typename TO, typename TM, int VB>
__global__ void __launch_bounds__(128) hop_kernel(Latt L, int d, int nvec, const cplx<TM>* __restrict__ U,
                                                  const cplx<TI>* __restrict__ in, cplx<TO>* __restrict__ out) {
  const int V3 = L.V3();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= V3) return;
  const int x = s % L.Lx;
  const int yz = s / L.Lx;
  const int y = yz % L.Ly;
  const int z = yz / L.Ly;
  int sp, sm;
  if (d == 0) {
    sp = s - x + wrap_inc(x, L.Lx);
    sm = s - x + wrap_dec(x, L.Lx);
  } else if (d == 1) {
    sp = s + (wrap_inc(y, L.Ly) - y) * L.Lx;
    sm = s + (wrap_dec(y, L.Ly) - y) * L.Lx;
  } else {
    sp = s + (wrap_inc(z, L.Lz) - z) * L.Lx * L.Ly;
    sm = s + (wrap_dec(z, L.Lz) - z) * L.Lx * L.Ly;
  }
  cplx<TM> uf[9], ub[9];
#pragma unroll
  for (int e = 0; e < 9; ++e) {
    uf[e] = ld(U + (d * 9 + e) * V3 + s);
    ub[e] = ld(U + (d * 9 + e) * V3 + sm);
  }
  const int v0 = blockIdx.y * VB;
  const int v1 = min(nvec, v0 + VB);
  for (int v = v0; v < v1; ++v) {
    const cplx<TI>* F = in + (long long)v * 3 * V3;
    cplx<TM> a[3], b[3], r[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      a[c] = cvt<TM>(ld(F + c * V3 + sp));
      b[c] = cvt<TM>(ld(F + c * V3 + sm));
      r[c] = mk(TM(0), TM(0));
    }
    mv_add(r, uf, a);
    cplx<TM> q[3] = {mk(TM(0), TM(0)), mk(TM(0), TM(0)), mk(TM(0), TM(0))};
    mvd_add(q, ub, b);
    cplx<TO>* O = out + (long long)v * 3 * V3;
#pragma unroll
    for (int c = 0; c < 3; ++c) O[c * V3 + s] = cvt<TO>(r[c] - q[c]);
  }
}

// ------------------------------------------------------------ TMA-staged Laplacian (complex64)
// One block marches through a slab of z planes of one (timeslice, vector).
// The input colour planes of z-1, z and z+1 sit in a ring of four shared-memory
// slots that TMA fills (plane z+2 lands while z computes), so every input
// value is read from HBM once per slab (plus one halo plane at each end);
// links are read with 128-bit loads, the backward links of x and y from the
// neighbouring sites of the same plane and those of z from the plane just
// finished (both L1/L2 resident).  Waits on the slot barriers are bounded: a
// timeout sets the error word that ed_laplacian_status reports.

constexpr int LT_THREADS = 256, LT_SLOTS = 4;
constexpr long long LT_WAIT_CYCLES = 4000000000LL;  // ~2 s
__device__ int g_stencil_error = 0;

__device__ __forceinline__ uint32_t st_smem(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ bool st_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(st_smem(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool st_test_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(st_smem(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: false when the barrier has not flipped within `limit` cycles.  The staged kernels take
// the limit of their data waits as a launch argument (ed_laplacian_wait_limit, default LT_WAIT_CYCLES);
// the waits that drain their own copies in flight before a block leaves always use LT_WAIT_CYCLES.
// try_wait may suspend the thread until the phase completes (up to a hardware time limit), so a limit
// below LT_SHORT_WAIT is polled with the non-suspending test_wait: such a limit then runs out whenever
// the data is not there yet, however close it is.
constexpr long long LT_SHORT_WAIT = 100000;
__device__ __forceinline__ bool st_wait(uint64_t* bar, uint32_t parity, long long limit = LT_WAIT_CYCLES) {
  if (limit < LT_SHORT_WAIT) {
    const long long t0 = clock64();
    while (!st_test_wait(bar, parity))
      if (clock64() - t0 > limit) return false;
    return true;
  }
  if (st_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  while (!st_try_wait(bar, parity))
    if (clock64() - t0 > limit) return false;
  return true;
}
long long g_stencil_wait_cycles = LT_WAIT_CYCLES;  // host-side launch setting
// Host-side launch setting: when set, every block of the staged kernels first waits, with the data-wait
// limit, on a barrier of its own that nothing completes, so that the limit runs out whatever the copy
// latency (the test of the failure path).
int g_stencil_wait_probe = 0;

__global__ void __launch_bounds__(LT_THREADS) laplacian_tma_kernel(const __grid_constant__ CUtensorMap fmap, Latt L,
                                                                   int zb, const cplx<float>* __restrict__ links,
                                                                   long long link_tstride, cplx<float>* __restrict__ out,
                                                                   long long out_tstride, float diag, int slot_bytes,
                                                                   long long wait_cycles, int probe) {
  extern __shared__ __align__(128) uint8_t sm[];
  uint64_t* bar = (uint64_t*)(sm + LT_SLOTS * slot_bytes);
  __shared__ int failed;
  const int Lx = L.Lx, Ly = L.Ly, Lz = L.Lz, V3 = L.V3(), P = Lx * Ly;
  const int t = blockIdx.z, v = blockIdx.y;
  const int z0 = blockIdx.x * zb, z1 = min(Lz, z0 + zb);
  const int nplanes = (z1 - z0) + 2;  // plane j holds z = z0 - 1 + j (periodic)
  if (threadIdx.x == 0) {
    failed = 0;
    for (int s = 0; s <= LT_SLOTS; ++s)  // bar[LT_SLOTS]: the probe barrier, never arrived on
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(st_smem(&bar[s])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  auto issue = [&](int j) {
    const int z = (z0 - 1 + j + Lz) % Lz;
    const int s = j % LT_SLOTS;
    uint8_t* dst = sm + s * slot_bytes;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(st_smem(&bar[s])), "r"(3 * P * 8)
                 : "memory");
    for (int c = 0; c < 3; ++c)
      asm volatile(
          "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], "
          "[%2];" ::"r"(st_smem(dst + c * P * 8)),
          "l"(&fmap), "r"(st_smem(&bar[s])), "r"(0), "r"(((v * 3 + c) * Lz + z) * Ly), "r"(t)
          : "memory");
  };
  int issued_hi = -1;
  if (threadIdx.x == 0)
    for (int j = 0; j < LT_SLOTS && j < nplanes; ++j) {
      issue(j);
      issued_hi = j;
    }
  if (threadIdx.x == 0 && probe && !st_wait(&bar[LT_SLOTS], 0, wait_cycles)) failed = 1;
  const cplx<float>* U = links + (long long)t * link_tstride;
  cplx<float>* O = out + (long long)t * out_tstride + (long long)v * 3 * V3;
  for (int z = z0; z < z1; ++z) {
    const int jc = z - z0 + 1;
    if (threadIdx.x == 0)
      for (int j = jc - 1; j <= jc + 1; ++j)
        if (!st_wait(&bar[j % LT_SLOTS], (j / LT_SLOTS) & 1, wait_cycles)) failed = 1;
    __syncthreads();
    if (failed) break;
    const float2* Fm = (const float2*)(sm + ((jc - 1) % LT_SLOTS) * slot_bytes);  // [c][y][x]
    const float2* Fc = (const float2*)(sm + (jc % LT_SLOTS) * slot_bytes);
    const float2* Fp = (const float2*)(sm + ((jc + 1) % LT_SLOTS) * slot_bytes);
    const int zm = wrap_dec(z, Lz), zp = wrap_inc(z, Lz);
    for (int q = threadIdx.x; q < P / 2; q += LT_THREADS) {
      const int x0 = (2 * q) % Lx, y = (2 * q) / Lx;
      const int p0 = y * Lx + x0;  // in-plane index of the first of the two sites
      const int s0 = z * P + p0;
      const int xm = wrap_dec(x0, Lx), xp2 = (x0 + 2) % Lx;
      const int ym = wrap_dec(y, Ly), yp = wrap_inc(y, Ly);
      cplx<float> f[3][2], hop[2][3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float4 a = *reinterpret_cast<const float4*>(Fc + c * P + p0);
        f[c][0] = mk(a.x, a.y);
        f[c][1] = mk(a.z, a.w);
      }
#pragma unroll
      for (int s = 0; s < 2; ++s)
#pragma unroll
        for (int c = 0; c < 3; ++c) hop[s][c] = mk(0.f, 0.f);
      // ---- x: forward links at s0 (both sites), backward U_x(x0-1) for site 0, U_x(x0) for site 1
      {
        cplx<float> uf[9][2], ubm[9], fxp[3], fxm[3];
#pragma unroll
        for (int e = 0; e < 9; ++e) Pack<float, 2>::load(U + (0 * 9 + e) * V3 + s0, uf[e]);
#pragma unroll
        for (int e = 0; e < 9; ++e) ubm[e] = ld(U + (0 * 9 + e) * V3 + z * P + y * Lx + xm);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float2 a = Fc[c * P + y * Lx + xp2], b = Fc[c * P + y * Lx + xm];
          fxp[c] = mk(a.x, a.y);
          fxm[c] = mk(b.x, b.y);
        }
        cplx<float> u[9], w[3];
#pragma unroll
        for (int e = 0; e < 9; ++e) u[e] = uf[e][0];
#pragma unroll
        for (int c = 0; c < 3; ++c) w[c] = f[c][1];
        mv_add(hop[0], u, w);       // U_x(x0) F(x0+1)
        mvd_add(hop[0], ubm, fxm);  // U_x(x0-1)^dag F(x0-1)
#pragma unroll
        for (int c = 0; c < 3; ++c) w[c] = f[c][0];
        mvd_add(hop[1], u, w);      // U_x(x0)^dag F(x0)
#pragma unroll
        for (int e = 0; e < 9; ++e) u[e] = uf[e][1];
        mv_add(hop[1], u, fxp);     // U_x(x0+1) F(x0+2)
      }
      // ---- y and z: forward links at s0, backward links at the neighbour sites
#pragma unroll
      for (int mu = 1; mu < 3; ++mu) {
        const int sm_site = mu == 1 ? z * P + ym * Lx + x0 : zm * P + p0;
        const float2* Fpl = mu == 1 ? Fc + yp * Lx + x0 : Fp + p0;
        const float2* Fml = mu == 1 ? Fc + ym * Lx + x0 : Fm + p0;
        cplx<float> uf[9][2], ub[9][2], fp[3][2], fm[3][2];
#pragma unroll
        for (int e = 0; e < 9; ++e) {
          Pack<float, 2>::load(U + (mu * 9 + e) * V3 + s0, uf[e]);
          Pack<float, 2>::load(U + (mu * 9 + e) * V3 + sm_site, ub[e]);
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float4 a = *reinterpret_cast<const float4*>(Fpl + c * P);
          const float4 b = *reinterpret_cast<const float4*>(Fml + c * P);
          fp[c][0] = mk(a.x, a.y);
          fp[c][1] = mk(a.z, a.w);
          fm[c][0] = mk(b.x, b.y);
          fm[c][1] = mk(b.z, b.w);
        }
#pragma unroll
        for (int s = 0; s < 2; ++s) {
          cplx<float> u[9], w[9], a[3], b[3];
#pragma unroll
          for (int e = 0; e < 9; ++e) {
            u[e] = uf[e][s];
            w[e] = ub[e][s];
          }
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            a[c] = fp[c][s];
            b[c] = fm[c][s];
          }
          mv_add(hop[s], u, a);
          mvd_add(hop[s], w, b);
        }
      }
      (void)zp;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        cplx<float> o[2];
#pragma unroll
        for (int s = 0; s < 2; ++s) o[s] = mk(diag * f[c][s].re - hop[s][c].re, diag * f[c][s].im - hop[s][c].im);
        Pack<float, 2>::store(O + c * V3 + s0, o);
      }
    }
    __syncthreads();  // every thread is done with plane jc - 1
    if (threadIdx.x == 0 && jc - 1 + LT_SLOTS < nplanes) {
      issue(jc - 1 + LT_SLOTS);
      issued_hi = jc - 1 + LT_SLOTS;
    }
  }
  if (threadIdx.x == 0 && failed) {
    atomicExch(&g_stencil_error, 1);
    // let the copies still in flight land before the block's shared memory is released
    for (int j = issued_hi; j >= 0 && j > issued_hi - LT_SLOTS; --j) st_wait(&bar[j % LT_SLOTS], (j / LT_SLOTS) & 1);
  }
}

// ------------------------------------------------------------ strip-staged Laplacian (complex64, TMA links + input)
// One block owns a strip of R rows x Lx sites of a z slab of one (timeslice,
// vector) and marches through the slab.  For every plane TMA brings into a
// shared-memory slot: the 27 link streams of the strip, the U_y links of the
// row below the strip, the input rows of the strip and the two halo rows
// above and below (the plane below the slab brings only its U_z links and
// input rows, the plane above only its input rows).  Three slots: per plane
// the block first applies the backward z hop (slot of plane z-1), releases
// that slot to the load of plane z+2, then the x and y hops and the forward
// z hop.  Every link and input value reaches shared memory by a bulk copy,
// so the bytes in flight do not depend on registers; one thread per site
// reads everything from shared memory.  Waits are bounded (status word).

constexpr int LS_SLOTS = 3, LS_MAX_SITES = 128;

struct LsGeom {
  int links, uyh, fmain, fhlo, fhhi, bytes;  // byte offsets inside a slot, slot size
};
__host__ __device__ inline int ls_al(int v) { return (v + 127) / 128 * 128; }
__host__ __device__ inline LsGeom ls_geom(int RLx, int Lx) {
  LsGeom g;
  g.links = 0;
  g.uyh = g.links + ls_al(27 * RLx * 8);
  g.fmain = g.uyh + ls_al(9 * Lx * 8);
  g.fhlo = g.fmain + ls_al(3 * RLx * 8);
  g.fhhi = g.fhlo + ls_al(3 * Lx * 8);
  g.bytes = g.fhhi + ls_al(3 * Lx * 8);
  return g;
}

__device__ __forceinline__ void ls_tma2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
          st_smem(dst)),
      "l"(map), "r"(st_smem(bar)), "r"(x), "r"(y)
      : "memory");
}
__device__ __forceinline__ void ls_tma3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], [%2];" ::
          "r"(st_smem(dst)),
      "l"(map), "r"(st_smem(bar)), "r"(x), "r"(y), "r"(z)
      : "memory");
}

__device__ __forceinline__ cplx<float> ls_ld(const uint8_t* base, int idx) {
  const float2 v = reinterpret_cast<const float2*>(base)[idx];
  return mk(v.x, v.y);
}

__global__ void __launch_bounds__(LS_MAX_SITES, 2)
    laplacian_strip_kernel(const __grid_constant__ CUtensorMap mL27, const __grid_constant__ CUtensorMap mL9,
                           const __grid_constant__ CUtensorMap mLz, const __grid_constant__ CUtensorMap mF,
                           const __grid_constant__ CUtensorMap mFh, Latt L, int R, int zb,
                           cplx<float>* __restrict__ out, long long out_tstride, float diag, long long wait_cycles,
                           int probe) {
  extern __shared__ __align__(128) uint8_t sm[];
  const int Lx = L.Lx, Ly = L.Ly, Lz = L.Lz, V3 = L.V3(), P = Lx * Ly, RLx = R * Lx;
  const LsGeom g = ls_geom(RLx, Lx);
  uint64_t* bar = (uint64_t*)(sm + LS_SLOTS * g.bytes);
  const int nstrip = Ly / R;
  const int strip = blockIdx.x % nstrip, slab = blockIdx.x / nstrip;
  const int v = blockIdx.y, t = blockIdx.z;
  const int y0 = strip * R, ylo = wrap_dec(y0, Ly), yhi = (y0 + R) % Ly;
  const int z0 = slab * zb, z1 = min(Lz, z0 + zb);
  const int nplanes = (z1 - z0) + 2;  // plane j holds z = z0 - 1 + j (periodic)
  if (threadIdx.x == 0) {
    for (int q = 0; q <= LS_SLOTS; ++q)  // bar[LS_SLOTS]: the probe barrier, never arrived on
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(st_smem(&bar[q])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  auto issue = [&](int j) {  // thread 0 only
    const int z = (z0 - 1 + j + Lz) % Lz;
    const int q = j % LS_SLOTS;
    uint8_t* base = sm + q * g.bytes;
    const bool first = j == 0, last = j == nplanes - 1;
    uint32_t bytes = 3 * RLx * 8;
    if (first)
      bytes += 9 * RLx * 8;
    else if (!last)
      bytes += 27 * RLx * 8 + 9 * Lx * 8 + 6 * Lx * 8;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(st_smem(&bar[q])), "r"(bytes)
                 : "memory");
    ls_tma3d(base + g.fmain, &mF, &bar[q], z * P + y0 * Lx, v * 3, t);
    if (first) {
      ls_tma2d(base + g.links + 18 * RLx * 8, &mLz, &bar[q], z * P + y0 * Lx, t * 27 + 18);
    } else if (!last) {
      ls_tma2d(base + g.links, &mL27, &bar[q], z * P + y0 * Lx, t * 27);
      ls_tma2d(base + g.uyh, &mL9, &bar[q], z * P + ylo * Lx, t * 27 + 9);
      ls_tma3d(base + g.fhlo, &mFh, &bar[q], z * P + ylo * Lx, v * 3, t);
      ls_tma3d(base + g.fhhi, &mFh, &bar[q], z * P + yhi * Lx, v * 3, t);
    }
  };
  int issued_hi = -1;  // thread 0 only
  if (threadIdx.x == 0)
    for (int j = 0; j < LS_SLOTS && j < nplanes; ++j) {
      issue(j);
      issued_hi = j;
    }
  const int p = threadIdx.x;  // site of the strip
  const bool active = p < RLx;
  const int xx = active ? p % Lx : 0, yy = active ? p / Lx : 0;
  const int pxm = yy * Lx + wrap_dec(xx, Lx), pxp = yy * Lx + wrap_inc(xx, Lx);
  cplx<float>* O = out + (long long)t * out_tstride + (long long)v * 3 * V3;
  bool ok = true, failed = false;
  if (threadIdx.x == 0 && probe) ok = st_wait(&bar[LS_SLOTS], 0, wait_cycles);
  for (int z = z0; z < z1; ++z) {
    const int jc = z - z0 + 1;
    const uint8_t* Sm = sm + ((jc - 1) % LS_SLOTS) * g.bytes;
    const uint8_t* Sc = sm + (jc % LS_SLOTS) * g.bytes;
    const uint8_t* Sp = sm + ((jc + 1) % LS_SLOTS) * g.bytes;
    ok = ok && st_wait(&bar[(jc - 1) % LS_SLOTS], ((jc - 1) / LS_SLOTS) & 1, wait_cycles) &&
         st_wait(&bar[jc % LS_SLOTS], (jc / LS_SLOTS) & 1, wait_cycles);
    cplx<float> hop[3] = {mk(0.f, 0.f), mk(0.f, 0.f), mk(0.f, 0.f)};
    if (active && ok) {  // backward z: U_z(z-1)^dag F(z-1)
      cplx<float> u[9], f[3];
#pragma unroll
      for (int e = 0; e < 9; ++e) u[e] = ls_ld(Sm + g.links, (18 + e) * RLx + p);
#pragma unroll
      for (int c = 0; c < 3; ++c) f[c] = ls_ld(Sm + g.fmain, c * RLx + p);
      mvd_add(hop, u, f);
    }
    failed = __syncthreads_or(!ok) != 0;  // the slot of plane z-1 is free from here on
    if (failed) break;
    if (threadIdx.x == 0 && jc + 2 < nplanes) {
      issue(jc + 2);
      issued_hi = jc + 2;
    }
    ok = st_wait(&bar[(jc + 1) % LS_SLOTS], ((jc + 1) / LS_SLOTS) & 1, wait_cycles);
    if (active && ok) {
      cplx<float> u[9], f[3], f0[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) f0[c] = ls_ld(Sc + g.fmain, c * RLx + p);
      // x forward: U_x(x) F(x+1); x backward: U_x(x-1)^dag F(x-1)
#pragma unroll
      for (int e = 0; e < 9; ++e) u[e] = ls_ld(Sc + g.links, e * RLx + p);
#pragma unroll
      for (int c = 0; c < 3; ++c) f[c] = ls_ld(Sc + g.fmain, c * RLx + pxp);
      mv_add(hop, u, f);
#pragma unroll
      for (int e = 0; e < 9; ++e) u[e] = ls_ld(Sc + g.links, e * RLx + pxm);
#pragma unroll
      for (int c = 0; c < 3; ++c) f[c] = ls_ld(Sc + g.fmain, c * RLx + pxm);
      mvd_add(hop, u, f);
      // y forward: U_y(y) F(y+1) (the row above the strip comes from the halo)
#pragma unroll
      for (int e = 0; e < 9; ++e) u[e] = ls_ld(Sc + g.links, (9 + e) * RLx + p);
#pragma unroll
      for (int c = 0; c < 3; ++c)
        f[c] = yy + 1 < R ? ls_ld(Sc + g.fmain, c * RLx + p + Lx) : ls_ld(Sc + g.fhhi, c * Lx + xx);
      mv_add(hop, u, f);
      // y backward: U_y(y-1)^dag F(y-1) (links and input of the row below the strip from the halo)
#pragma unroll
      for (int e = 0; e < 9; ++e)
        u[e] = yy > 0 ? ls_ld(Sc + g.links, (9 + e) * RLx + p - Lx) : ls_ld(Sc + g.uyh, e * Lx + xx);
#pragma unroll
      for (int c = 0; c < 3; ++c)
        f[c] = yy > 0 ? ls_ld(Sc + g.fmain, c * RLx + p - Lx) : ls_ld(Sc + g.fhlo, c * Lx + xx);
      mvd_add(hop, u, f);
      // z forward: U_z(z) F(z+1)
#pragma unroll
      for (int e = 0; e < 9; ++e) u[e] = ls_ld(Sc + g.links, (18 + e) * RLx + p);
#pragma unroll
      for (int c = 0; c < 3; ++c) f[c] = ls_ld(Sp + g.fmain, c * RLx + p);
      mv_add(hop, u, f);
      const int site = z * P + (y0 + yy) * Lx + xx;
#pragma unroll
      for (int c = 0; c < 3; ++c)
        O[(long long)c * V3 + site] = mk(diag * f0[c].re - hop[c].re, diag * f0[c].im - hop[c].im);
    }
  }
  if (!failed) failed = __syncthreads_or(!ok) != 0;  // a wait of the last plane's second half
  if (threadIdx.x == 0 && failed) {
    atomicExch(&g_stencil_error, 1);
    for (int j = issued_hi; j >= 0 && j > issued_hi - LS_SLOTS; --j) st_wait(&bar[j % LS_SLOTS], (j / LS_SLOTS) & 1);
  }
}

using StEncodeFn = PFN_cuTensorMapEncodeTiled_v12000;
static StEncodeFn st_encoder() {
  static StEncodeFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (StEncodeFn)p;
  }
  return fn;
}

// The TMA path serves complex64 when four planes fit in shared memory and the
// plane rows meet the tensor-map limits; returns -1 when it does not apply.
static int launch_laplacian_tma(Latt L, int nt, int nvec, const void* links, const void* in, long long its,
                                void* out, long long ots, cudaStream_t stream) {
  const int P = L.Lx * L.Ly;
  const int slot_bytes = (3 * P * 8 + 127) / 128 * 128;
  const int smem = LT_SLOTS * slot_bytes + 64;
  if (L.Lx % 2 || 2 * L.Lx > 256 || L.Ly > 256 || smem > 200 * 1024 || (its * 8) % 16 || (P * 8) % 128) return -1;
  if ((long long)3 * nvec * L.Lz * L.Ly >= (1LL << 31)) return -1;
  StEncodeFn enc = st_encoder();
  if (!enc) return -1;
  CUtensorMap map;
  cuuint64_t gdim[3] = {(cuuint64_t)(2 * L.Lx), (cuuint64_t)(3LL * nvec * L.Lz * L.Ly), (cuuint64_t)nt};
  cuuint64_t gstride[2] = {(cuuint64_t)(8LL * L.Lx), (cuuint64_t)(its * 8)};
  cuuint32_t box[3] = {(cuuint32_t)(2 * L.Lx), (cuuint32_t)L.Ly, 1};
  cuuint32_t estride[3] = {1, 1, 1};
  if (enc(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void*>(in), gdim, gstride, box, estride,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return -1;
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(laplacian_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) !=
        cudaSuccess)
      return -1;
    attr = true;
  }
  // about two waves of blocks (two blocks per SM when the planes are small)
  const long long want = 4LL * num_sms();
  int zb = (int)std::max(1LL, std::min<long long>(L.Lz, (long long)L.Lz * nt * nvec / want));
  const int nslab = ceil_div(L.Lz, zb);
  dim3 grid(nslab, nvec, nt);
  laplacian_tma_kernel<<<grid, LT_THREADS, smem, stream>>>(map, L, zb, (const cplx<float>*)links, 27LL * L.V3(),
                                                           (cplx<float>*)out, ots, 6.0f, slot_bytes,
                                                           g_stencil_wait_cycles, g_stencil_wait_probe);
  ED_RETURN_LAUNCH("laplacian (TMA-staged)");
  return ED_OK;
}

// The strip-staged path serves complex64 when Lx is even and a strip of whole
// rows (R rows, R | Ly, R * Lx <= 128 sites) exists; returns -1 otherwise.
static int launch_laplacian_strip(Latt L, int nt, int nvec, const void* links, const void* in, long long its,
                                  void* out, long long ots, cudaStream_t stream) {
  const int Lx = L.Lx, Ly = L.Ly, Lz = L.Lz, V3 = L.V3();
  if (Lx % 2 || Lx > LS_MAX_SITES || its % 2 || ((uintptr_t)in % 16) || ((uintptr_t)links % 16)) return -1;
  int R = 0;
  for (int r = 1; r <= Ly && r * Lx <= LS_MAX_SITES; ++r)
    if (Ly % r == 0) R = r;
  // RLx % 8 keeps every TMA destination (the U_z rows start 18 * RLx * 8 bytes into a slot) 128-byte aligned
  if (R == 0 || (R * Lx) % 8 || (long long)27 * nt >= (1LL << 31) || (long long)3 * nvec >= (1LL << 31)) return -1;
  StEncodeFn enc = st_encoder();
  if (!enc) return -1;
  const int RLx = R * Lx;
  CUtensorMap mL27, mL9, mLz, mF, mFh;
  cuuint64_t ldim[2] = {(cuuint64_t)V3, (cuuint64_t)(27LL * nt)};
  cuuint64_t lstride[1] = {(cuuint64_t)(8LL * V3)};
  cuuint64_t fdim[3] = {(cuuint64_t)V3, (cuuint64_t)(3LL * nvec), (cuuint64_t)nt};
  cuuint64_t fstride[2] = {(cuuint64_t)(8LL * V3), (cuuint64_t)(8LL * its)};
  cuuint32_t es[3] = {1, 1, 1};
  auto enc2 = [&](CUtensorMap* m, cuuint32_t bx, cuuint32_t by) {
    cuuint32_t box[2] = {bx, by};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<void*>(links), ldim, lstride, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
  };
  auto enc3 = [&](CUtensorMap* m, cuuint32_t bx) {
    cuuint32_t box[3] = {bx, 3, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<void*>(in), fdim, fstride, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
  };
  if (!enc2(&mL27, RLx, 27) || !enc2(&mL9, Lx, 9) || !enc2(&mLz, RLx, 9) || !enc3(&mF, RLx) || !enc3(&mFh, Lx))
    return -1;
  const LsGeom geo = ls_geom(RLx, Lx);
  const int smem = LS_SLOTS * geo.bytes + 64;
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(laplacian_strip_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 110 * 1024) !=
        cudaSuccess)
      return -1;
    attr = true;
  }
  if (smem > 110 * 1024) return -1;
  // z slabs long enough to amortise their two halo planes, short enough for about four waves of two blocks per SM
  const int nstrip = Ly / R;
  const long long want = 8LL * num_sms();
  const int zb = (int)std::max(2LL, std::min<long long>(Lz, (long long)Lz * nstrip * nvec * nt / want));
  const int nslab = ceil_div(Lz, zb);
  if ((long long)nstrip * nslab >= (1LL << 31) || nvec > 65535 || nt > 65535) return -1;
  dim3 grid(nstrip * nslab, nvec, nt);
  const int threads = (RLx + 31) / 32 * 32;
  laplacian_strip_kernel<<<grid, threads, smem, stream>>>(mL27, mL9, mLz, mF, mFh, L, R, zb, (cplx<float>*)out, ots,
                                                          6.0f, g_stencil_wait_cycles, g_stencil_wait_probe);
  ED_RETURN_LAUNCH("laplacian (strip-staged)");
  return ED_OK;
}

// ------------------------------------------------------------ double-float Laplacian
// The FP64 operator at FP32-pipe speed (this part's FP64 pipe bounds the FP64 kernel above at ~1.2 TFLOP/s,
// about a fifth of what HBM would allow): links in the split form of df.cuh ([t][dir][row][col][V3] float4
// {re_hi, im_hi, re_lo, im_lo}, 16 bytes per complex like complex128, split once per solve), colour planes in
// and out as complex128, each input value split by integer operations on its bits (split_bits), every product
// an exact FP32 product split plus the cross terms, summed in (hi, lo) pairs; ~2^-47 relative per product.
// One site per thread.

// y += U x and y += U^dag x on split operands (re, im sums kept apart)
__device__ __forceinline__ void cmac_df(DF& re, DF& im, float4 u, float4 f) {
  df_acc(re, u.x, u.z, f.x, f.z);
  df_sub(re, u.y, u.w, f.y, f.w);
  df_acc(im, u.x, u.z, f.y, f.w);
  df_acc(im, u.y, u.w, f.x, f.z);
}
__device__ __forceinline__ void cmac_conj_df(DF& re, DF& im, float4 u, float4 f) {
  df_acc(re, u.x, u.z, f.x, f.z);
  df_acc(re, u.y, u.w, f.y, f.w);
  df_acc(im, u.x, u.z, f.y, f.w);
  df_sub(im, u.y, u.w, f.x, f.z);
}

__global__ void __launch_bounds__(128) laplacian_df_kernel(Latt L, const float4* __restrict__ links,
                                                           const double2* __restrict__ in, double2* __restrict__ out,
                                                           long long link_tstride, long long in_tstride,
                                                           long long out_tstride) {
  const int V3 = L.V3();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= V3) return;
  const int t = blockIdx.z;
  const float4* U = links + (long long)t * link_tstride;
  const long long voff = (long long)blockIdx.y * 3 * V3;
  const double2* F = in + (long long)t * in_tstride + voff;
  double2* O = out + (long long)t * out_tstride + voff;
  const int x = s % L.Lx, yz = s / L.Lx, y = yz % L.Ly, z = yz / L.Ly;
  DF hre[3], him[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) hre[c] = him[c] = DF{0.f, 0.f};
#pragma unroll
  for (int mu = 0; mu < 3; ++mu) {
    int sp, sm;
    if (mu == 0) {
      sp = s - x + wrap_inc(x, L.Lx);
      sm = s - x + wrap_dec(x, L.Lx);
    } else if (mu == 1) {
      sp = s + (wrap_inc(y, L.Ly) - y) * L.Lx;
      sm = s + (wrap_dec(y, L.Ly) - y) * L.Lx;
    } else {
      sp = s + (wrap_inc(z, L.Lz) - z) * L.Lx * L.Ly;
      sm = s + (wrap_dec(z, L.Lz) - z) * L.Lx * L.Ly;
    }
    {  // U_mu(x) F(x + mu)
      float4 u[9], f[3];
#pragma unroll
      for (int e = 0; e < 9; ++e) u[e] = __ldg(U + (long long)(mu * 9 + e) * V3 + s);
#pragma unroll
      for (int c = 0; c < 3; ++c) f[c] = split_c128_bits(__ldg(F + (long long)c * V3 + sp));
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) cmac_df(hre[a], him[a], u[a * 3 + b], f[b]);
    }
    {  // U_mu(x - mu)^dag F(x - mu)
      float4 u[9], f[3];
#pragma unroll
      for (int e = 0; e < 9; ++e) u[e] = __ldg(U + (long long)(mu * 9 + e) * V3 + sm);
#pragma unroll
      for (int c = 0; c < 3; ++c) f[c] = split_c128_bits(__ldg(F + (long long)c * V3 + sm));
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) cmac_conj_df(hre[a], him[a], u[b * 3 + a], f[b]);
    }
  }
  // out = 6 F(x) - hop, formed in double-float and widened once
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float4 f = split_c128_bits(__ldg(F + (long long)c * V3 + s));
    DF ore{-hre[c].hi, -hre[c].lo}, oim{-him[c].hi, -him[c].lo};
    df_acc(ore, 6.f, 0.f, f.x, f.z);
    df_acc(oim, 6.f, 0.f, f.y, f.w);
    O[(long long)c * V3 + s] = make_double2(f2d_bits(ore.hi) + f2d_bits(ore.lo), f2d_bits(oim.hi) + f2d_bits(oim.lo));
  }
}

__global__ void split_c128_kernel(long long n, const double2* __restrict__ src, float4* __restrict__ dst) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dst[i] = split_c128(src[i]);
}

// ------------------------------------------------------------ launchers

int launch_laplacian(int prec, Latt L, int nt, int nvec, const void* links, const void* in, long long its,
                     void* out, long long ots, cudaStream_t stream) {
  const int V3 = L.V3();
  const long long lts = 27LL * V3;
  if (prec == ED_C64 && g_stencil_tma == 1) {
    const int rc = launch_laplacian_tma(L, nt, nvec, links, in, its, out, ots, stream);
    if (rc != -1) return rc;
  }
  if (prec == ED_C64 && g_stencil_tma == 2) {
    const int rc = launch_laplacian_strip(L, nt, nvec, links, in, its, out, ots, stream);
    if (rc != -1) return rc;
  }
  if (prec == ED_DF) {
    dim3 grid(ceil_div(V3, 128), nvec, nt);
    laplacian_df_kernel<<<grid, 128, 0, stream>>>(L, (const float4*)links, (const double2*)in, (double2*)out, lts, its,
                                                   ots);
  } else if (prec == ED_C128) {
    dim3 grid(ceil_div(V3, 128), nvec, nt);
    laplacian_kernel<double, 1><<<grid, 128, 0, stream>>>(L, (const cplx<double>*)links, (const cplx<double>*)in,
                                                           (cplx<double>*)out, lts, its, ots, 6.0);
  } else {
    dim3 grid(ceil_div(V3 / 2, 128), nvec, nt);
    laplacian_kernel<float, 2><<<grid, 128, 0, stream>>>(L, (const cplx<float>*)links, (const cplx<float>*)in,
                                                          (cplx<float>*)out, lts, its, ots, 6.0f);
  }
  ED_RETURN_LAUNCH("laplacian");
  return ED_OK;
}

int launch_hop(int in_prec, int out_prec, Latt L, int d, int nvec, const void* links_c128, const void* in,
               void* out, cudaStream_t stream) {
  constexpr int VB = 8;
  const int V3 = L.V3();
  dim3 grid(ceil_div(V3, 128), ceil_div(nvec, VB));
  const cplx<double>* U = (const cplx<double>*)links_c128;
  if (in_prec == ED_C128 && out_prec == ED_C128)
    hop_kernel<double, double, double, VB><<<grid, 128, 0, stream>>>(L, d, nvec, U, (const cplx<double>*)in,
                                                                     (cplx<double>*)out);
  else if (in_prec == ED_C64 && out_prec == ED_C64)
    hop_kernel<float, float, double, VB><<<grid, 128, 0, stream>>>(L, d, nvec, U, (const cplx<float>*)in,
                                                                   (cplx<float>*)out);
  else if (in_prec == ED_C64 && out_prec == ED_C128)
    hop_kernel<float, double, double, VB><<<grid, 128, 0, stream>>>(L, d, nvec, U, (const cplx<float>*)in,
                                                                    (cplx<double>*)out);
  else
    hop_kernel<double, float, double, VB><<<grid, 128, 0, stream>>>(L, d, nvec, U, (const cplx<double>*)in,
                                                                    (cplx<float>*)out);
  ED_RETURN_LAUNCH("covariant derivative hop");
  return ED_OK;
}

// complex64 chains with FP32 links and FP32 math (split-precision elemental modes)
int launch_hop_f32(Latt L, int d, int nvec, const void* links_c64, const void* in, void* out, cudaStream_t stream) {
  constexpr int VB = 8;
  const int V3 = L.V3();
  dim3 grid(ceil_div(V3, 128), ceil_div(nvec, VB));
  hop_kernel<float, float, float, VB><<<grid, 128, 0, stream>>>(L, d, nvec, (const cplx<float>*)links_c64,
                                                                (const cplx<float>*)in, (cplx<float>*)out);
  ED_RETURN_LAUNCH("covariant derivative hop (fp32)");
  return ED_OK;
}

}  // namespace ed

// ------------------------------------------------------------ C ABI

extern "C" int ed_laplacian(int prec, int Lx, int Ly, int Lz, int nt, int nvec, const void* links, const void* in,
                            long long in_tstride, void* out, long long out_tstride, void* stream) {
  ED_CHECK_ARG(prec == ED_C128 || prec == ED_C64 || prec == ED_DF, "ed_laplacian: prec must be ED_C128, ED_C64 or ED_DF");
  ED_CHECK_ARG(Lx > 0 && Ly > 0 && Lz > 0 && nt > 0 && nvec > 0, "ed_laplacian: sizes must be positive");
  ED_CHECK_ARG(ed::lattice_ok(Lx, Ly, Lz), "ed_laplacian: Lx*Ly*Lz above 2^28");
  ED_CHECK_ARG(prec != ED_C64 || Lx % 2 == 0, "ed_laplacian: c64 path needs an even Lx");
  ED_CHECK_ARG(nvec <= 65535 && nt <= 65535, "ed_laplacian: nvec and nt must be <= 65535");
  ED_CHECK_ARG(links && in && out, "ed_laplacian: null pointer");
  ED_CHECK_ARG(in != out, "ed_laplacian: in and out must not alias");
  ED_CHECK_ARG(((uintptr_t)links % 16) == 0 && ((uintptr_t)in % 16) == 0 && ((uintptr_t)out % 16) == 0,
               "ed_laplacian: buffers must be 16-byte aligned");
  ED_CHECK_ARG(in_tstride >= 0 && out_tstride >= 0, "ed_laplacian: negative stride");
  const long long dflt = 3LL * Lx * Ly * Lz * nvec;
  if (in_tstride == 0) in_tstride = dflt;
  if (out_tstride == 0) out_tstride = dflt;
  ED_CHECK_ARG(prec != ED_C64 || (in_tstride % 2 == 0 && out_tstride % 2 == 0),
               "ed_laplacian: c64 strides must keep 16-byte alignment");
  return ed::launch_laplacian(prec, ed::Latt{Lx, Ly, Lz}, nt, nvec, links, in, in_tstride, out, out_tstride,
                              (cudaStream_t)stream);
}

extern "C" int ed_split_c128(long long n, const void* src, void* dst, void* stream) {
  ED_CHECK_ARG(n >= 0, "ed_split_c128: negative size");
  ED_CHECK_ARG((src && dst) || n == 0, "ed_split_c128: null pointer");
  ED_CHECK_ARG(((uintptr_t)src % 16) == 0 && ((uintptr_t)dst % 16) == 0, "ed_split_c128: 16-byte alignment");
  if (n == 0) return ED_OK;
  const int grid = (int)std::min<long long>(ed::ceil_div(n, 256), 8LL * 1024);
  ed::split_c128_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(n, (const double2*)src, (float4*)dst);
  ED_RETURN_LAUNCH("double-float split");
  return ED_OK;
}

extern "C" int ed_laplacian_config(int use_tma) {
  ED_CHECK_ARG(use_tma >= 0 && use_tma <= 2, "ed_laplacian_config: use_tma must be 0, 1 or 2");
  ed::g_stencil_tma = use_tma;
  return ED_OK;
}

extern "C" int ed_laplacian_wait_limit(long long cycles) {
  ED_CHECK_ARG(cycles >= 0, "ed_laplacian_wait_limit: negative limit");
  ed::g_stencil_wait_cycles = cycles > 0 ? cycles : ed::LT_WAIT_CYCLES;
  return ED_OK;
}

extern "C" int ed_laplacian_wait_probe(int on) {
  ed::g_stencil_wait_probe = on ? 1 : 0;
  return ED_OK;
}

extern "C" int ed_laplacian_status(int* code, void* stream) {
  ED_CHECK_ARG(code, "ed_laplacian_status: null pointer");
  cudaStream_t s = (cudaStream_t)stream;
  int zero = 0;
  cudaError_t e = cudaMemcpyFromSymbolAsync(code, ed::g_stencil_error, sizeof(int), 0, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess && *code != 0) e = cudaMemcpyToSymbolAsync(ed::g_stencil_error, &zero, sizeof(int), 0,
                                                                  cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return ed::cuda_status(e, "reading the stencil status word");
  if (*code != 0) {
    ed::set_error("laplacian: a bounded wait of the TMA-staged kernel gave up; that output is invalid");
    return ED_ERR_TIMEOUT;
  }
  return ED_OK;
}

extern "C" int ed_covariant_derivative(int in_prec, int out_prec, int Lx, int Ly, int Lz, int dir, int nvec,
                                       const void* links_c128, const void* in, void* out, void* stream) {
  ED_CHECK_ARG((in_prec == ED_C128 || in_prec == ED_C64) && (out_prec == ED_C128 || out_prec == ED_C64),
               "ed_covariant_derivative: bad precision");
  ED_CHECK_ARG(Lx > 0 && Ly > 0 && Lz > 0 && nvec > 0, "ed_covariant_derivative: sizes must be positive");
  ED_CHECK_ARG(ed::lattice_ok(Lx, Ly, Lz), "ed_covariant_derivative: Lx*Ly*Lz above 2^28");
  ED_CHECK_ARG(dir >= 0 && dir < 3, "ed_covariant_derivative: dir must be 0, 1 or 2");
  ED_CHECK_ARG(links_c128 && in && out, "ed_covariant_derivative: null pointer");
  ED_CHECK_ARG(in != out, "ed_covariant_derivative: in and out must not alias");
  ED_CHECK_ARG(ed::ceil_div(nvec, 8) <= 65535, "ed_covariant_derivative: too many vectors");
  return ed::launch_hop(in_prec, out_prec, ed::Latt{Lx, Ly, Lz}, dir, nvec, links_c128, in, out,
                        (cudaStream_t)stream);
}

// ------------------------------------------------------------ one-sided parallel transport
// out(x) = U_d(x) in(x+d)          (sign > 0)
// out(x) = U_d(x-d)^dag in(x-d)    (sign < 0)
// Straight-line displacement of DisplacementElementalGenerator._D
// (lattice/generator/displacement_elemental.py:53-71).  FP64 math, c128 storage.
namespace ed {
template <int VB>
__global__ void __launch_bounds__(128) transport_kernel(Latt L, int d, int sign, int nvec,
                                                        const cplx<double>* __restrict__ U,
                                                        const cplx<double>* __restrict__ in,
                                                        cplx<double>* __restrict__ out) {
  const int V3 = L.V3();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= V3) return;
  const int x = s % L.Lx, y = (s / L.Lx) % L.Ly, z = s / (L.Lx * L.Ly);
  int sn;  // neighbour site
  if (d == 0)
    sn = s - x + (sign > 0 ? wrap_inc(x, L.Lx) : wrap_dec(x, L.Lx));
  else if (d == 1)
    sn = s + ((sign > 0 ? wrap_inc(y, L.Ly) : wrap_dec(y, L.Ly)) - y) * L.Lx;
  else
    sn = s + ((sign > 0 ? wrap_inc(z, L.Lz) : wrap_dec(z, L.Lz)) - z) * L.Lx * L.Ly;
  const int ls = sign > 0 ? s : sn;  // site of the link
  cplx<double> u[9];
#pragma unroll
  for (int e = 0; e < 9; ++e) u[e] = ld(U + (d * 9 + e) * V3 + ls);
  const int v0 = blockIdx.y * VB;
  const int v1 = min(nvec, v0 + VB);
  for (int v = v0; v < v1; ++v) {
    const cplx<double>* F = in + (long long)v * 3 * V3;
    cplx<double> a[3], r[3] = {mk(0.0, 0.0), mk(0.0, 0.0), mk(0.0, 0.0)};
#pragma unroll
    for (int c = 0; c < 3; ++c) a[c] = ld(F + c * V3 + sn);
    if (sign > 0)
      mv_add(r, u, a);
    else
      mvd_add(r, u, a);
    cplx<double>* O = out + (long long)v * 3 * V3;
#pragma unroll
    for (int c = 0; c < 3; ++c) O[c * V3 + s] = r[c];
  }
}
}  // namespace ed

extern "C" int ed_parallel_transport(int Lx, int Ly, int Lz, int dir, int sign, int nvec, const void* links_c128,
                                     const void* in, void* out, void* stream) {
  ED_CHECK_ARG(Lx > 0 && Ly > 0 && Lz > 0 && nvec > 0, "ed_parallel_transport: sizes must be positive");
  ED_CHECK_ARG(ed::lattice_ok(Lx, Ly, Lz), "ed_parallel_transport: Lx*Ly*Lz above 2^28");
  ED_CHECK_ARG(dir >= 0 && dir < 3 && (sign == 1 || sign == -1), "ed_parallel_transport: bad direction or sign");
  ED_CHECK_ARG(links_c128 && in && out && in != out, "ed_parallel_transport: null or aliasing pointers");
  constexpr int VB = 8;
  const int V3 = Lx * Ly * Lz;
  ED_CHECK_ARG(ed::ceil_div(nvec, VB) <= 65535, "ed_parallel_transport: too many vectors");
  dim3 grid(ed::ceil_div(V3, 128), ed::ceil_div(nvec, VB));
  ed::transport_kernel<VB><<<grid, 128, 0, (cudaStream_t)stream>>>(
      ed::Latt{Lx, Ly, Lz}, dir, sign, nvec, (const ed::cplx<double>*)links_c128, (const ed::cplx<double>*)in,
      (ed::cplx<double>*)out);
  ED_RETURN_LAUNCH("parallel transport");
  return ED_OK;
}
