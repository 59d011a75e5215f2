// Tensor-core (tcgen05 + TMEM + TMA) split-precision pair contractions.
//
//   G_p(X, Y)[i, j] = sum_k conj(X_i[k]) phase_p(k) Y_j[k]       (k = colour*V3 + site)
//
// is computed as one real-embedded complex GEMM per pair group
// (left chain X, right chains Y0..Y0+nR-1), all momenta at once:
//   A (M side, 128 rows per CTA)  : right-chain vectors m = (r, j), loaded by TMA
//                                   from pre-split planes in HBM;
//   B (N side, 256 rows per CTA)  : n = (i, p) = i*Nmom + p, produced in shared
//                                   memory by producer warps as conj(X_i) * phase_p;
//   D[m][n] = G_p[i][m] accumulated in TMEM: D_re = Ar.Br - Ai.Bi, D_im = Ar.Bi + Ai.Br
//   (4 real products per complex product; the 3-multiplication Gauss form would
//   need three 256-column accumulators, more than TMEM's 512 columns).
// Every real operand is split into hi + lo parts of a narrow type and each real
// product is hi.hi + hi.lo + lo.hi (three MMAs, FP32 accumulation):
//   f16x3 : fp16 parts of the operand scaled by 2^e (fp16 range); error ~2^-22
//   bf16x3: bf16 parts, no scaling;                                 error ~2^-16
//   tf32x3: tf32 parts (kind::tf32);                                error ~2^-22
// Warp roles (192 threads, one CTA per SM): warp 0 issues TMA, warp 1 owns TMEM
// and issues tcgen05.mma from one lane, warps 2-5 produce B and afterwards
// drain the accumulators (tcgen05.ld) into the FP64 G buffer.
// Shared memory rows are 64 bytes with the 64-byte swizzle (TMA and UMMA agree
// on it; the producers apply it by hand).  Every mbarrier wait is bounded: on
// timeout the kernel records an error code in a status word and leaves.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cudaTypedefs.h>

#include <algorithm>

#include "elemental.cuh"

namespace ed {

int launch_phases(Latt L, const int* moms, int nmom, cplx<double>* out, cudaStream_t stream);

constexpr int TC_BM = 128;
constexpr int TC_BN = 256;
constexpr int TC_ROWB = 64;  // bytes of K per shared-memory row (64-byte swizzle)
constexpr int TC_STAGES = 2;
constexpr int TC_PWARPS = 4;
constexpr int TC_THREADS = 64 + 32 * TC_PWARPS;
constexpr int TC_A_BYTES = 4 * TC_BM * TC_ROWB;  // 4 planes
constexpr int TC_B_BYTES = 4 * TC_BN * TC_ROWB;
constexpr int TC_STAGE_BYTES = TC_A_BYTES + TC_B_BYTES;
constexpr int TC_SMEM = TC_STAGES * TC_STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
constexpr long long TC_WAIT_CYCLES = 4000000000LL;  // ~2 s at 2 GHz

// status codes written by the kernel
constexpr int TC_ERR_FULL = 1, TC_ERR_EMPTY = 2, TC_ERR_ACC = 3;

enum TcKind { TC_F16 = 1, TC_BF16 = 2, TC_TF32 = 3 };

struct TcJob {
  int left, right0, nright, tile0, mt, nt;
  long long g_off;
};
struct TcTable {
  int njobs;
  TcJob j[kMaxJobs];
};

// device scalars at the start of the extra workspace
struct TcScalars {
  unsigned int absmax_bits;  // max |re|,|im| over all chains (float bits)
  int scale_exp;             // e: operands are multiplied by 2^e before splitting
  int status;                // 0 = ok, else TC_ERR_*
  int pad[61];
};

// ------------------------------------------------------------ PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: false if the barrier did not flip within TC_WAIT_CYCLES, or,
// when abort_on_error, as soon as another role has reported an error.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* status, int code,
                                          bool abort_on_error = true) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  for (uint32_t it = 1;; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 255u) == 0) {
      if (abort_on_error && *status != 0) return false;
      if (clock64() - t0 > TC_WAIT_CYCLES) {
        atomicCAS((int*)status, 0, code);
        return false;
      }
    }
  }
}

// Warp-uniform bounded wait: lane 0 polls, the outcome is broadcast.
__device__ __forceinline__ bool warp_wait(uint64_t* bar, uint32_t parity, volatile int* status, int code,
                                          bool abort_on_error = true) {
  int ok = 0;
  if ((threadIdx.x & 31) == 0) ok = mbar_wait(bar, parity, status, code, abort_on_error) ? 1 : 0;
  return __shfl_sync(0xffffffffu, ok, 0) != 0;
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
          smem_u32(dst)),
      "l"(map), "r"(smem_u32(bar)), "r"(x), "r"(y)
      : "memory");
}

// UMMA shared-memory descriptor: K-major, 64-byte swizzle, 8-row groups 512 B apart.
__device__ __forceinline__ uint64_t umma_desc_sw64(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)1 << 16;              // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(512 >> 4) << 32;     // stride byte offset: 8 rows x 64 B
  d |= (uint64_t)1 << 46;              // descriptor version (sm_100 family)
  d |= (uint64_t)4 << 61;              // layout: 64-byte swizzle
  return d;
}

// Instruction descriptor: D fp32, A/B format `fmt` (f16 0, bf16 1, tf32 2), K-major,
// M = 128, N = 256, optional negation of A.
__host__ __device__ constexpr uint32_t umma_idesc(uint32_t fmt, bool neg_a) {
  return (1u << 4) | (fmt << 7) | (fmt << 10) | ((neg_a ? 1u : 0u) << 13) | ((uint32_t)(TC_BN >> 3) << 17) |
         ((uint32_t)(TC_BM >> 4) << 24);
}

template <int KIND>
__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  if constexpr (KIND == TC_TF32) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
  } else {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
  }
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int e = 0; e < 16; ++e) v[e] = __uint_as_float(r[e]);
}

// ------------------------------------------------------------ splitting
// hi/lo parts of v packed as 16-bit pairs (2 values per 32-bit word) or tf32 words.
template <int KIND>
struct Split;

template <>
struct Split<TC_F16> {
  static constexpr int ESZ = 2;
  __device__ __forceinline__ static void pair(float a, float b, uint32_t& hi, uint32_t& lo) {
    __half2 h = __floats2half2_rn(a, b);
    float2 hf = __half22float2(h);
    __half2 l = __floats2half2_rn(a - hf.x, b - hf.y);
    hi = *reinterpret_cast<uint32_t*>(&h);
    lo = *reinterpret_cast<uint32_t*>(&l);
  }
};
template <>
struct Split<TC_BF16> {
  static constexpr int ESZ = 2;
  __device__ __forceinline__ static void pair(float a, float b, uint32_t& hi, uint32_t& lo) {
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    float2 hf = __bfloat1622float2(h);
    __nv_bfloat162 l = __floats2bfloat162_rn(a - hf.x, b - hf.y);
    hi = *reinterpret_cast<uint32_t*>(&h);
    lo = *reinterpret_cast<uint32_t*>(&l);
  }
};
template <>
struct Split<TC_TF32> {
  static constexpr int ESZ = 4;
  __device__ __forceinline__ static void one(float a, uint32_t& hi, uint32_t& lo) {
    uint32_t h, l;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(a));
    const float r = a - __uint_as_float(h);
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l) : "f"(r));
    hi = h;
    lo = l;
  }
};

// ------------------------------------------------------------ preparation kernels

__global__ void tc_absmax_kernel(const float* __restrict__ x, long long n, TcScalars* sc) {
  float m = 0.f;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    m = fmaxf(m, fabsf(x[i]));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(&sc->absmax_bits, __float_as_uint(m));
}

// e = floor(log2(2^13 / absmax)): split operands of magnitude <= 2^13 (and
// phase-rotated ones <= 2^13.5) stay well inside the fp16 range.
__global__ void tc_scale_kernel(TcScalars* sc, int kind) {
  if (threadIdx.x == 0) {
    int e = 0;
    const float m = __uint_as_float(sc->absmax_bits);
    if (kind == TC_F16 && m > 0.f && isfinite(m)) {
      int ex;
      frexpf(m, &ex);  // m in [2^(ex-1), 2^ex)
      e = 13 - ex;
      e = max(-100, min(100, e));
    }
    sc->scale_exp = e;
  }
}

// right-chain planes: out[q][m][k], q = re_hi, re_lo, im_hi, im_lo
template <int KIND>
__global__ void tc_split_kernel(const cplx<float>* __restrict__ chains, long long R, long long K,
                                const TcScalars* __restrict__ sc, void* __restrict__ planes) {
  const float s = ldexpf(1.f, sc->scale_exp);
  const long long total2 = R * K / 2;  // pairs of consecutive k
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total2;
       t += (long long)gridDim.x * blockDim.x) {
    const float4 v = reinterpret_cast<const float4*>(chains)[t];  // two complex values
    const long long e0 = 2 * t;
    if constexpr (KIND == TC_TF32) {
      uint32_t* P = (uint32_t*)planes;
      const long long plane = R * K;
      uint32_t h, l;
      Split<TC_TF32>::one(v.x * s, h, l);
      P[e0] = h;
      P[plane + e0] = l;
      Split<TC_TF32>::one(v.z * s, h, l);
      P[e0 + 1] = h;
      P[plane + e0 + 1] = l;
      Split<TC_TF32>::one(v.y * s, h, l);
      P[2 * plane + e0] = h;
      P[3 * plane + e0] = l;
      Split<TC_TF32>::one(v.w * s, h, l);
      P[2 * plane + e0 + 1] = h;
      P[3 * plane + e0 + 1] = l;
    } else {
      uint32_t* P = (uint32_t*)planes;  // 16-bit elements, pairs as words
      const long long plane = R * K / 2;
      uint32_t h, l;
      Split<KIND>::pair(v.x * s, v.z * s, h, l);
      P[t] = h;
      P[plane + t] = l;
      Split<KIND>::pair(v.y * s, v.w * s, h, l);
      P[2 * plane + t] = h;
      P[3 * plane + t] = l;
    }
  }
}

// FP64 phases -> complex64 phases scaled by 2^e
__global__ void tc_phase_kernel(const cplx<double>* __restrict__ ph, long long n, const TcScalars* __restrict__ sc,
                                cplx<float>* __restrict__ out) {
  const double s = ldexp(1.0, sc->scale_exp);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = mk((float)(ph[i].re * s), (float)(ph[i].im * s));
}

// ------------------------------------------------------------ the GEMM kernel

template <int KIND>
__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_pair_gemm_kernel(const __grid_constant__ CUtensorMap amap, TcTable tab, int Ne, int nmom, int V3, long long R,
                        const cplx<float>* __restrict__ chains, const cplx<float>* __restrict__ phases,
                        TcScalars* __restrict__ sc, cplx<double>* __restrict__ G) {
  constexpr int ESZ = Split<KIND>::ESZ;
  constexpr int KE = TC_ROWB / ESZ;              // k elements per stage
  constexpr int EPC = 16 / ESZ;                  // k elements per 16-byte chunk
  constexpr int CPR = TC_ROWB / 16;              // chunks per row (4)
  constexpr int KINST = 32 / ESZ;                // k elements per MMA instruction
  constexpr uint32_t FMT = KIND == TC_F16 ? 0u : (KIND == TC_BF16 ? 1u : 2u);
  constexpr uint32_t IDESC = umma_idesc(FMT, false);
  constexpr uint32_t IDESC_NEG = umma_idesc(FMT, true);

  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + TC_STAGES * TC_STAGE_BYTES);
  uint64_t* empty = full + TC_STAGES;
  uint64_t* accf = empty + TC_STAGES;
  uint32_t* tmem_slot = (uint32_t*)(accf + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  volatile int* status = &sc->status;

  // ---- decode the tile: group, n tile (fast), m tile
  int tile = blockIdx.x;
  int jb = 0;
  while (jb + 1 < tab.njobs && tile >= tab.j[jb + 1].tile0) ++jb;
  const TcJob J = tab.j[jb];
  const int local = tile - J.tile0;
  const int mtile = local / J.nt;
  const int ntile = local - mtile * J.nt;
  const long long K = 3LL * V3;
  const int nkb = (int)(K / KE);
  const int Mrows = J.nright * Ne;
  const int Ncols = Ne * nmom;
  const long long row0 = (long long)J.right0 * Ne + (long long)mtile * TC_BM;  // first A row (all-chain index)
  const int n0 = ntile * TC_BN;

  if (threadIdx.x == 0) {
    for (int s = 0; s < TC_STAGES; ++s) {
      mbar_init(&full[s], 1 + TC_PWARPS);
      mbar_init(&empty[s], 1);
    }
    mbar_init(accf, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(tmem_slot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ===================== TMA producer for A (4 planes per stage)
    if (lane == 0) {
      int issued_last = -1;
      for (int kb = 0; kb < nkb; ++kb) {
        const int s = kb % TC_STAGES;
        if (kb >= TC_STAGES && !mbar_wait(&empty[s], ((kb / TC_STAGES) + 1) & 1, status, TC_ERR_EMPTY)) break;
        uint8_t* As = smem + s * TC_STAGE_BYTES;
        mbar_arrive_expect_tx(&full[s], TC_A_BYTES);
        for (int q = 0; q < 4; ++q)
          tma_load_2d(As + q * TC_BM * TC_ROWB, &amap, &full[s], kb * KE, (int)(q * R + row0));
        issued_last = kb;
      }
      // do not leave while our copies may still land in shared memory
      if (issued_last >= 0) {
        const int s = issued_last % TC_STAGES;
        mbar_wait(&full[s], (issued_last / TC_STAGES) & 1, status, TC_ERR_FULL, false);
      }
    }
  } else if (warp == 1) {
    // ===================== MMA issuer
    if (lane == 0) {
      const uint32_t d_re = tmem, d_im = tmem + TC_BN;
      bool ok = true;
      for (int kb = 0; kb < nkb && ok; ++kb) {
        const int s = kb % TC_STAGES;
        if (!mbar_wait(&full[s], (kb / TC_STAGES) & 1, status, TC_ERR_FULL)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t a0 = smem_u32(smem + s * TC_STAGE_BYTES);
        const uint32_t b0 = a0 + TC_A_BYTES;
#pragma unroll
        for (int ks = 0; ks < KE / KINST; ++ks) {
          uint64_t A[4], B[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            A[q] = umma_desc_sw64(a0 + q * TC_BM * TC_ROWB + ks * 32);
            B[q] = umma_desc_sw64(b0 + q * TC_BN * TC_ROWB + ks * 32);
          }
          const uint32_t acc = (kb > 0 || ks > 0) ? 1u : 0u;
          // D_re = Ar.Br - Ai.Bi
          umma<KIND>(d_re, A[0], B[0], IDESC, acc);
          umma<KIND>(d_re, A[0], B[1], IDESC, 1u);
          umma<KIND>(d_re, A[1], B[0], IDESC, 1u);
          umma<KIND>(d_re, A[2], B[2], IDESC_NEG, 1u);
          umma<KIND>(d_re, A[2], B[3], IDESC_NEG, 1u);
          umma<KIND>(d_re, A[3], B[2], IDESC_NEG, 1u);
          // D_im = Ar.Bi + Ai.Br
          umma<KIND>(d_im, A[0], B[2], IDESC, acc);
          umma<KIND>(d_im, A[0], B[3], IDESC, 1u);
          umma<KIND>(d_im, A[1], B[2], IDESC, 1u);
          umma<KIND>(d_im, A[2], B[0], IDESC, 1u);
          umma<KIND>(d_im, A[2], B[1], IDESC, 1u);
          umma<KIND>(d_im, A[3], B[0], IDESC, 1u);
        }
        umma_commit(&empty[s]);  // frees this stage when the MMAs above complete
      }
      // Always signal: the epilogue (and the TMEM release after it) must not
      // run while issued MMAs are still in flight.
      umma_commit(accf);
    }
  } else {
    // ===================== B producers (warps 2..5), then epilogue
    const int pt = threadIdx.x - 64;  // 0..127
    const float* Xb = reinterpret_cast<const float*>(chains + (long long)J.left * Ne * K);
    bool ok = true;
    for (int kb = 0; kb < nkb; ++kb) {
      const int s = kb % TC_STAGES;
      if (kb >= TC_STAGES && !warp_wait(&empty[s], ((kb / TC_STAGES) + 1) & 1, status, TC_ERR_EMPTY)) {
        ok = false;
        break;
      }
      uint8_t* Bs = smem + s * TC_STAGE_BYTES + TC_A_BYTES;
      const long long k0 = (long long)kb * KE;
      const int site0 = (int)(k0 % V3);
#pragma unroll 2
      for (int task = pt; task < TC_BN * CPR; task += 32 * TC_PWARPS) {
        const int row = task / CPR, c = task % CPR;
        const int n = n0 + row;
        uint32_t hre[4], lre[4], him[4], lim[4];
        if (n < Ncols) {
          const int i = n / nmom, p = n - i * nmom;
          const float* x = Xb + 2 * ((long long)i * K + k0 + c * EPC);
          const float* ph = reinterpret_cast<const float*>(phases) + 2 * ((long long)p * V3 + site0 + c * EPC);
          float br[EPC], bi[EPC];
#pragma unroll
          for (int e = 0; e < EPC; e += 2) {
            const float4 xv = __ldg(reinterpret_cast<const float4*>(x + 2 * e));
            const float4 pv = __ldg(reinterpret_cast<const float4*>(ph + 2 * e));
            // conj(x) * phase
            br[e] = xv.x * pv.x + xv.y * pv.y;
            bi[e] = xv.x * pv.y - xv.y * pv.x;
            br[e + 1] = xv.z * pv.z + xv.w * pv.w;
            bi[e + 1] = xv.z * pv.w - xv.w * pv.z;
          }
          if constexpr (KIND == TC_TF32) {
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              Split<TC_TF32>::one(br[e], hre[e], lre[e]);
              Split<TC_TF32>::one(bi[e], him[e], lim[e]);
            }
          } else {
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              Split<KIND>::pair(br[2 * e], br[2 * e + 1], hre[e], lre[e]);
              Split<KIND>::pair(bi[2 * e], bi[2 * e + 1], him[e], lim[e]);
            }
          }
        } else {
#pragma unroll
          for (int e = 0; e < 4; ++e) hre[e] = lre[e] = him[e] = lim[e] = 0u;
        }
        const uint32_t off = row * TC_ROWB + ((c ^ ((row >> 1) & 3)) << 4);
        uint8_t* dst = Bs + off;
        *reinterpret_cast<uint4*>(dst + 0 * TC_BN * TC_ROWB) = make_uint4(hre[0], hre[1], hre[2], hre[3]);
        *reinterpret_cast<uint4*>(dst + 1 * TC_BN * TC_ROWB) = make_uint4(lre[0], lre[1], lre[2], lre[3]);
        *reinterpret_cast<uint4*>(dst + 2 * TC_BN * TC_ROWB) = make_uint4(him[0], him[1], him[2], him[3]);
        *reinterpret_cast<uint4*>(dst + 3 * TC_BN * TC_ROWB) = make_uint4(lim[0], lim[1], lim[2], lim[3]);
      }
      fence_proxy_async();
      __syncwarp();
      if (lane == 0) mbar_arrive(&full[s]);
    }
    // ---- epilogue: TMEM -> FP64 G
    const bool acc_ok = warp_wait(accf, 0, status, TC_ERR_ACC, false);
    if (ok && acc_ok && *status == 0) {
      tc_fence_after();
      const int quarter = warp & 3;
      const int m = quarter * 32 + lane;  // accumulator row = TMEM lane
      const long long m_local = (long long)mtile * TC_BM + m;
      const double inv = ldexp(1.0, -2 * sc->scale_exp);
      const int N = J.nright * Ne;
      for (int cc = 0; cc < TC_BN / 16; ++cc) {
        float vr[16], vi[16];
        const uint32_t tl = tmem + ((uint32_t)(quarter * 32) << 16) + cc * 16;
        tmem_ld16(tl, vr);
        tmem_ld16(tl + TC_BN, vi);
        if (m_local < Mrows) {
#pragma unroll
          for (int e = 0; e < 16; ++e) {
            const int n = n0 + cc * 16 + e;
            if (n < Ncols) {
              const int i = n / nmom, p = n - i * nmom;
              G[J.g_off + ((long long)p * Ne + i) * N + m_local] = mk((double)vr[e] * inv, (double)vi[e] * inv);
            }
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
  }
}

// ------------------------------------------------------------ host side

static int tc_kind_of(int mode) {
  switch (mode) {
    case ED_MODE_F16X3:
      return TC_F16;
    case ED_MODE_BF16X3:
      return TC_BF16;
    case ED_MODE_TF32X3:
      return TC_TF32;
    default:
      return 0;
  }
}

bool mode_supported(int mode) { return mode == ED_MODE_FP64 || tc_kind_of(mode) != 0; }

static size_t tc_esz(int kind) { return kind == TC_TF32 ? 4 : 2; }

static size_t up256(size_t v) { return (v + 255) / 256 * 256; }

size_t tc_extra_workspace(const ed_elemental_plan* P) {
  const int kind = tc_kind_of(P->mode);
  if (!kind) return 0;
  const size_t R = (size_t)P->nchain * P->Ne;
  const size_t K = 3ull * P->V3;
  return up256(sizeof(TcScalars)) + up256((size_t)P->nmom * P->V3 * 8) + up256(4 * R * K * tc_esz(kind));
}

int tc_plan_check(ed_elemental_plan* P) {
  P->tc_kind = tc_kind_of(P->mode);
  if (!P->tc_kind) return ED_OK;
  if (P->V3 % 32 != 0) {
    set_error("tensor-core elemental modes need Lx*Ly*Lz divisible by 32 (got %d)", P->V3);
    return ED_ERR_UNSUPPORTED;
  }
  const long long rows = 4LL * P->nchain * P->Ne;
  if (rows >= (1LL << 31) || 3LL * P->V3 >= (1LL << 31)) {
    set_error("tensor-core elemental modes: problem too large for 32-bit TMA coordinates");
    return ED_ERR_UNSUPPORTED;
  }
  return ED_OK;
}

using EncodeFn = PFN_cuTensorMapEncodeTiled_v12000;

static EncodeFn get_encode() {
  static EncodeFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeFn)p;
  }
  return fn;
}

template <int KIND>
static int launch_kind(const ed_elemental_plan* P, const cplx<float>* chains, const cplx<double>* phases,
                       cplx<double>* G, void* extra, cudaStream_t stream) {
  constexpr int ESZ = Split<KIND>::ESZ;
  char* X = (char*)extra;
  TcScalars* sc = (TcScalars*)X;
  cplx<float>* ph32 = (cplx<float>*)(X + up256(sizeof(TcScalars)));
  void* planes = X + up256(sizeof(TcScalars)) + up256((size_t)P->nmom * P->V3 * 8);
  const long long R = (long long)P->nchain * P->Ne;
  const long long K = 3LL * P->V3;

  cudaError_t e = cudaMemsetAsync(sc, 0, sizeof(TcScalars), stream);
  if (e != cudaSuccess) return cuda_status(e, "tc scalars reset");
  const int sms = num_sms();
  tc_absmax_kernel<<<4 * sms, 256, 0, stream>>>((const float*)chains, 2 * R * K, sc);
  tc_scale_kernel<<<1, 32, 0, stream>>>(sc, KIND);
  tc_split_kernel<KIND><<<8 * sms, 256, 0, stream>>>(chains, R, K, sc, planes);
  tc_phase_kernel<<<2 * sms, 256, 0, stream>>>(phases, (long long)P->nmom * P->V3, sc, ph32);
  ED_RETURN_LAUNCH("tensor-core operand preparation");

  EncodeFn enc = get_encode();
  if (!enc) {
    set_error("cuTensorMapEncodeTiled is unavailable from the driver");
    return ED_ERR_CUDA;
  }
  CUtensorMap amap;
  cuuint64_t gdim[2] = {(cuuint64_t)K, (cuuint64_t)(4 * R)};
  cuuint64_t gstride[1] = {(cuuint64_t)(K * ESZ)};
  cuuint32_t box[2] = {(cuuint32_t)(TC_ROWB / ESZ), (cuuint32_t)TC_BM};
  cuuint32_t estride[2] = {1, 1};
  CUresult cr = enc(&amap, KIND == TC_TF32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_UINT16, 2,
                    planes, gdim, gstride, box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (cr != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d)", (int)cr);
    return ED_ERR_CUDA;
  }

  TcTable tab;
  tab.njobs = (int)P->jobs.size();
  int tiles = 0;
  for (int k = 0; k < tab.njobs; ++k) {
    const Job& j = P->jobs[k];
    TcJob& d = tab.j[k];
    d.left = j.left;
    d.right0 = j.right0;
    d.nright = j.nright;
    d.g_off = j.g_off;
    d.mt = ceil_div((long long)j.nright * P->Ne, TC_BM);
    d.nt = ceil_div((long long)P->Ne * P->nmom, TC_BN);
    d.tile0 = tiles;
    tiles += d.mt * d.nt;
  }
  static bool attr_set[4] = {false, false, false, false};
  if (!attr_set[KIND]) {
    e = cudaFuncSetAttribute(tc_pair_gemm_kernel<KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM);
    if (e != cudaSuccess) return cuda_status(e, "tc kernel smem attribute");
    attr_set[KIND] = true;
  }
  if (P->prof_start) cudaEventRecord(P->prof_start, stream);
  tc_pair_gemm_kernel<KIND><<<tiles, TC_THREADS, TC_SMEM, stream>>>(amap, tab, P->Ne, P->nmom, P->V3, R, chains,
                                                                    ph32, sc, G);
  if (P->prof_stop) cudaEventRecord(P->prof_stop, stream);
  ED_RETURN_LAUNCH("tensor-core pair GEMM");
  return ED_OK;
}

int launch_pair_gemm_tc(const ed_elemental_plan* P, const cplx<float>* chains, const cplx<double>* phases,
                        cplx<double>* G, void* extra, cudaStream_t stream) {
  switch (P->tc_kind) {
    case TC_F16:
      return launch_kind<TC_F16>(P, chains, phases, G, extra, stream);
    case TC_BF16:
      return launch_kind<TC_BF16>(P, chains, phases, G, extra, stream);
    case TC_TF32:
      return launch_kind<TC_TF32>(P, chains, phases, G, extra, stream);
    default:
      set_error("not a tensor-core mode");
      return ED_ERR_ARG;
  }
}

int tc_read_status(const ed_elemental_plan* P, const void* workspace, int* status, cudaStream_t stream) {
  *status = 0;
  if (!P->tc_kind) return ED_OK;
  const TcScalars* sc = (const TcScalars*)((const char*)workspace + P->off_extra);
  cudaError_t e = cudaMemcpyAsync(status, &sc->status, sizeof(int), cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return cuda_status(e, "reading the tensor-core status word");
  return ED_OK;
}

}  // namespace ed
