// Tensor-core (tcgen05 + TMEM + TMA) split-precision pair contractions.
//
//   G_p(X, Y)[i, j] = sum_k conj(X_i[k]) phase_p(k) Y_j[k]       (k = colour*V3 + site)
//
// is computed as one real-embedded complex GEMM per pair group
// (left chain X, right chains Y0..Y0+nR-1), all momenta at once:
//   A (M side, 128 rows per CTA)  : right-chain vectors m = (r, j), loaded by TMA
//                                   from pre-split planes in HBM;
//   B (N side, 128 rows per CTA)  : n = (i, p) = i*Nmom + p, produced in shared
//                                   memory by producer warps as conj(X_i) * phase_p;
//   D[m][n] = G_p[i][m] accumulated in TMEM: D_re = Ar.Br - Ai.Bi, D_im = Ar.Bi + Ai.Br
//   (4 real products per complex product; the 3-multiplication Gauss form would
//   need three 128-column accumulators per buffer, which does not fit two
//   buffers into TMEM's 512 columns).
// Every real operand is split into hi + lo parts of a narrow type and each real
// product is hi.hi + hi.lo + lo.hi (three MMAs, FP32 accumulation):
//   f16x3 : fp16 parts of the operand scaled by 2^e (fp16 range); error ~2^-22
//   bf16x3: bf16 parts, no scaling;                                 error ~2^-16
//   tf32x3: tf32 parts (kind::tf32);                                error ~2^-22
// Warp roles and the accumulation scheme are described in tc_pair_gemm.cuh.
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

#include "tc_config.cuh"


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
  unsigned int progress;     // steps started (the lock step of the persistent factorised GEMMs)
  long long wait_limit;      // cycles a bounded wait of the single-SM factorised GEMM may take (0: TC_WAIT_CYCLES)
  int probe;                 // nonzero: that GEMM's TMA role issues no copy (the failure-detection test hook)
  int pad[57];
};
static_assert(sizeof(TcScalars) == 256, "device scalars");

// Process-wide settings of the single-SM factorised GEMM's bounded waits (ed_elemental_wait_limit /
// ed_elemental_wait_probe), written into the device scalars of every run by tc_scale_kernel.
long long g_tc_wait_cycles = 0;
int g_tc_wait_probe = 0;

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
// Bounded wait: false if the barrier did not flip within `limit` cycles
// (TC_WAIT_CYCLES unless the kernel passes its run's setting), or, when
// abort_on_error, as soon as another role has reported an error.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* status, int code,
                                          bool abort_on_error = true, long long limit = TC_WAIT_CYCLES) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  for (uint32_t it = 1;; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 255u) == 0) {
      if (abort_on_error && *status != 0) return false;
      if (clock64() - t0 > limit) {
        atomicCAS((int*)status, 0, code);
        return false;
      }
    }
  }
}

// Warp-uniform bounded wait: lane 0 polls, the outcome is broadcast.
__device__ __forceinline__ bool warp_wait(uint64_t* bar, uint32_t parity, volatile int* status, int code,
                                          bool abort_on_error = true, long long limit = TC_WAIT_CYCLES) {
  int ok = 0;
  if ((threadIdx.x & 31) == 0) ok = mbar_wait(bar, parity, status, code, abort_on_error, limit) ? 1 : 0;
  return __shfl_sync(0xffffffffu, ok, 0) != 0;
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(
          smem_u32(dst)),
      "l"(map), "r"(smem_u32(bar)), "r"(x), "r"(y), "r"(z)
      : "memory");
}

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
// M = TC_BM, N = TC_BN, optional negation of A.
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

// max |x| over n floats (n % 4 == 0, x 16-byte aligned), 16-byte loads
__global__ void tc_absmax_kernel(const float* __restrict__ x, long long n, TcScalars* sc) {
  float m = 0.f;
  const float4* x4 = reinterpret_cast<const float4*>(x);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n / 4;
       i += (long long)gridDim.x * blockDim.x) {
    const float4 v = x4[i];
    m = fmaxf(m, fmaxf(fmaxf(fabsf(v.x), fabsf(v.y)), fmaxf(fabsf(v.z), fabsf(v.w))));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(&sc->absmax_bits, __float_as_uint(m));
}

// e = floor(log2(2^13 / absmax)): split operands of magnitude <= 2^13 (and
// phase-rotated ones <= 2^13.5) stay well inside the fp16 range.
__global__ void tc_scale_kernel(TcScalars* sc, int kind, long long wait_limit, int probe) {
  if (threadIdx.x == 0) {
    sc->wait_limit = wait_limit;
    sc->probe = probe;
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
__global__ void tc_split_kernel(const cplx<float>* __restrict__ chains, long long R_used, long long R, long long K,
                                const TcScalars* __restrict__ sc, void* __restrict__ planes) {
  // rows [0, R_used) are split; the planes keep the stride of R rows
  const float s = ldexpf(1.f, sc->scale_exp);
  const long long total2 = R_used * K / 2;  // pairs of consecutive k
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

// double-float pair results -> complex128; two 16-byte loads in flight per
// thread (elements i and i + stride) before the stores
__global__ void tc_df_to_c128_kernel(const float4* __restrict__ DF, long long n, cplx<double>* __restrict__ G) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + stride < n; i += 2 * stride) {
    const float4 a = DF[i], b = DF[i + stride];
    G[i] = mk((double)a.x + (double)a.y, (double)a.z + (double)a.w);
    G[i + stride] = mk((double)b.x + (double)b.y, (double)b.z + (double)b.w);
  }
  if (i < n) {
    const float4 d = DF[i];
    G[i] = mk((double)d.x + (double)d.y, (double)d.z + (double)d.w);
  }
}

// the same for the two double-float planes of the SM-pair stacked GEMM (plane 1 at DF + plane), added
__global__ void tc_df2_to_c128_kernel(const float4* __restrict__ DF, long long plane, long long n,
                                      cplx<double>* __restrict__ G) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float4 a = DF[i], b = DF[plane + i];
    G[i] = mk(((double)a.x + (double)a.y) + ((double)b.x + (double)b.y),
              ((double)a.z + (double)a.w) + ((double)b.z + (double)b.w));
  }
}

// FP64 phases -> complex64 phases scaled by 2^e
__global__ void tc_phase_kernel(const cplx<double>* __restrict__ ph, long long n, const TcScalars* __restrict__ sc,
                                cplx<float>* __restrict__ out) {
  const double s = ldexp(1.0, sc->scale_exp);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = mk((float)(ph[i].re * s), (float)(ph[i].im * s));
}

// ------------------------------------------------------------ the GEMM kernels

#include "tc_pair_gemm.cuh"
#include "tc_fac_gemm.cuh"
#include "tc_fac2_gemm.cuh"
#include "tc_ozaki_gemm.cuh"

// ------------------------------------------------------------ factorised-phase operands

// Rows of the left (B) and right (A) variant planes.  Left slot sl of the
// batch (timeslice sl / nl) holds chain lchain[sl % nl] of that timeslice;
// right slot sl is chain sl of the chain buffer.
struct TcFacSlots {
  int nl;      // left-chain slots per timeslice (0 for the right side)
  int nchain;  // chains per timeslice
  int lchain[kMaxDeriv];
};

// Chain elements each thread of the split kernel loads before its first
// store: four 16-byte loads in flight per thread for the right side (3 pz
// variants per element, read-heavy); one for the left side, whose 9 (px, py)
// variants per element make it write-bound (and four would spill).
constexpr int kSplitUnrollRight = 4, kSplitUnrollLeft = 1;

// Writes the nvar variants of the two complex elements v (k = 2*kp, 2*kp + 1)
// of chain row (slot, i) into the planes.
template <int KIND, bool LEFT, bool SUM>
__device__ __forceinline__ void tc_fac_split_emit(const float4 v, int kp, long long orow0, int Ne, int nvar,
                                                  const cplx<float>* __restrict__ fac, int V3, long long Rplane,
                                                  long long K, int K2, void* __restrict__ planes) {
  const int site = (2 * kp) % V3;  // V3 is even: both elements lie in one colour plane
  for (int a = 0; a < nvar; ++a) {
    const float4 f = *reinterpret_cast<const float4*>(fac + (long long)a * V3 + site);
    const float fr0 = f.x, fi0 = f.y, fr1 = f.z, fi1 = f.w;
    float re0, im0, re1, im1;
    if constexpr (LEFT) {  // conj(x) * f
      re0 = v.x * fr0 + v.y * fi0;
      im0 = v.x * fi0 - v.y * fr0;
      re1 = v.z * fr1 + v.w * fi1;
      im1 = v.z * fi1 - v.w * fr1;
    } else {  // f * y
      re0 = fr0 * v.x - fi0 * v.y;
      im0 = fr0 * v.y + fi0 * v.x;
      re1 = fr1 * v.z - fi1 * v.w;
      im1 = fr1 * v.w + fi1 * v.z;
    }
    const long long orow = orow0 + (long long)a * Ne;
    // k-block-major planes: element (row, k) of a plane at ((k / KB) * Rplane + row) * KB + k % KB,
    // KB = the k elements of one 64-byte TMA row, so each (128-row, k-block) box is contiguous
    if constexpr (KIND == TC_TF32) {
      uint32_t* P = (uint32_t*)planes;
      const long long plane = Rplane * K, e0 = ((2LL * kp / 16) * Rplane + orow) * 16 + (2 * kp) % 16;
      uint32_t h, l;
      Split<TC_TF32>::one(re0, h, l);
      P[e0] = h;
      P[plane + e0] = l;
      Split<TC_TF32>::one(re1, h, l);
      P[e0 + 1] = h;
      P[plane + e0 + 1] = l;
      Split<TC_TF32>::one(im0, h, l);
      P[2 * plane + e0] = h;
      P[3 * plane + e0] = l;
      Split<TC_TF32>::one(im1, h, l);
      P[2 * plane + e0 + 1] = h;
      P[3 * plane + e0 + 1] = l;
      if constexpr (SUM) {  // planes 4, 5: re + im (Gauss form)
        Split<TC_TF32>::one(re0 + im0, h, l);
        P[4 * plane + e0] = h;
        P[5 * plane + e0] = l;
        Split<TC_TF32>::one(re1 + im1, h, l);
        P[4 * plane + e0 + 1] = h;
        P[5 * plane + e0 + 1] = l;
      }
    } else {
      uint32_t* P = (uint32_t*)planes;  // 16-bit elements, pairs as words (16 words per 64-byte row)
      const long long plane = Rplane * K2, w = (((long long)kp / 16) * Rplane + orow) * 16 + kp % 16;
      uint32_t h, l;
      Split<KIND>::pair(re0, re1, h, l);
      P[w] = h;
      P[plane + w] = l;
      Split<KIND>::pair(im0, im1, h, l);
      P[2 * plane + w] = h;
      P[3 * plane + w] = l;
      if constexpr (SUM) {  // planes 4, 5: re + im (Gauss form)
        Split<KIND>::pair(re0 + im0, re1 + im1, h, l);
        P[4 * plane + w] = h;
        P[5 * plane + w] = l;
      }
    }
  }
}

// out row (slot*nvar + a)*Ne + i of the planes <- conj(X_i) f_a   (LEFT)
//                                              or f_a Y_i         (right)
// for input row (slot, i) of the chain buffer; f_a = factor table a in
// complex64, already scaled by 2^e (tc_phase_kernel).  A block covers
// UNROLL * blockDim.x element pairs of a row; each thread loads its UNROLL
// pairs (blockDim.x apart) before it writes any variant.
template <int KIND, bool LEFT, int UNROLL, bool SUM>
__global__ void __launch_bounds__(256, 3) tc_fac_split_kernel(const cplx<float>* __restrict__ chains, TcFacSlots sl, int nrows, int Ne,
                                    int nvar, const cplx<float>* __restrict__ fac, int V3, long long Rplane,
                                    void* __restrict__ planes) {
  const long long K = 3LL * V3;
  const int K2 = (int)(K / 2);
  const int span = UNROLL * blockDim.x;
  for (int row = blockIdx.y; row < nrows; row += gridDim.y) {
    const int slot = row / Ne, i = row - (row / Ne) * Ne;
    const int chain = LEFT ? (slot / sl.nl) * sl.nchain + sl.lchain[slot % sl.nl] : slot;
    const float4* src = reinterpret_cast<const float4*>(chains + ((long long)chain * Ne + i) * K);
    const long long orow0 = (long long)slot * nvar * Ne + i;
    for (int k0 = blockIdx.x * span + threadIdx.x; k0 < K2; k0 += gridDim.x * span) {
      float4 v[UNROLL];
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) {
        const int kp = k0 + u * blockDim.x;
        if (kp < K2) v[u] = src[kp];
      }
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) {
        const int kp = k0 + u * blockDim.x;
        if (kp < K2) tc_fac_split_emit<KIND, LEFT, SUM>(v[u], kp, orow0, Ne, nvar, fac, V3, Rplane, K, K2, planes);
      }
    }
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
    case ED_MODE_OZAKI_I8:
      return TC_OZAKI;
    default:
      return 0;
  }
}

bool mode_supported(int mode) { return mode == ED_MODE_FP64 || tc_kind_of(mode) != 0; }

static size_t tc_esz(int kind) { return kind == TC_TF32 ? 4 : 2; }

static size_t up256(size_t v) { return (v + 255) / 256 * 256; }

// Decide whether the factorised-phase GEMM serves the plan: every momentum
// is a distinct (px, py) x pz combination and at most a quarter of the
// Pxy * Pz combinations the GEMM forms are not requested.  With
// ED_MODE_FLAG_LEFT_FACTOR every momentum's whole phase is a left factor and
// the one right factor is 1 (Pxy = Nmom, Pz = 1): nothing formed goes unused,
// for any list of distinct momenta, at the price of Nmom left variants per
// left chain.
void tc_fac_setup(ed_elemental_plan* P) {
  P->fac = false;
  const bool ozaki = tc_kind_of(P->mode) == TC_OZAKI;  // runs on factorised operands only
  if (!tc_kind_of(P->mode) || P->custom || (P->no_factor && !ozaki) || P->nmom > 127) return;
  std::vector<int> lm, rm, ai(P->nmom), ci(P->nmom);  // left / right factor momenta, 3 ints each
  for (int m = 0; m < P->nmom; ++m) {
    const int px = P->moms[3 * m], py = P->moms[3 * m + 1], pz = P->moms[3 * m + 2];
    // (px, py, 0) x (0, 0, pz), or (px, py, pz) x (0, 0, 0)
    const int l[3] = {px, py, P->left_factor ? pz : 0}, r[3] = {0, 0, P->left_factor ? 0 : pz};
    int a = 0, c = 0;
    while (a < (int)lm.size() / 3 && !(lm[3 * a] == l[0] && lm[3 * a + 1] == l[1] && lm[3 * a + 2] == l[2])) ++a;
    if (a == (int)lm.size() / 3) lm.insert(lm.end(), {l[0], l[1], l[2]});
    while (c < (int)rm.size() / 3 && !(rm[3 * c] == r[0] && rm[3 * c + 1] == r[1] && rm[3 * c + 2] == r[2])) ++c;
    if (c == (int)rm.size() / 3) rm.insert(rm.end(), {r[0], r[1], r[2]});
    ai[m] = a;
    ci[m] = c;
  }
  const int pxy = (int)lm.size() / 3, pz = (int)rm.size() / 3;
  if (pxy * pz > kMaxFac || (!ozaki && !P->force_factor && 4 * pxy * pz > 5 * P->nmom)) return;
  if (ozaki && (pxy > OZ_MAX_VAR || pz > OZ_MAX_VAR)) return;  // the row-maximum kernel keeps <= 16 per row
  std::vector<signed char> pidx(pxy * pz, -1);
  for (int m = 0; m < P->nmom; ++m) {
    signed char& e = pidx[ai[m] * pz + ci[m]];
    if (e >= 0) return;  // a repeated momentum
    e = (signed char)m;
  }
  std::vector<int> lchain, lslot(P->nchain, -1);
  for (int k = 0; k < P->jobs_per_t; ++k) {
    const int l = P->jobs[k].left;
    if (lslot[l] < 0) {
      lslot[l] = (int)lchain.size();
      lchain.push_back(l);
    }
  }
  const long long rb = (long long)P->nbatch * (long long)lchain.size() * pxy * P->Ne;
  const long long ra = (long long)P->nbatch * P->nchain * pz * P->Ne;
  if (OZ_BP * rb >= (1LL << 31) || OZ_AP * ra >= (1LL << 31) || (int)lchain.size() > kMaxDeriv) return;
  P->fac = true;
  P->fac_pxy = pxy;
  P->fac_pz = pz;
  P->fac_l = lm;
  P->fac_r = rm;
  P->fac_pidx = pidx;
  P->fac_lchain = lchain;
  P->fac_lslot = lslot;
}

// Extra workspace of the factorised-phase GEMM, in this order: scalars, FP64
// factor tables f_a (Pxy x V3) and g_c (Pz x V3), their scaled complex64
// copies, B planes [4][RB][K], A planes [4][RA][K], double-float results.
struct FacLayout {
  long long rb, ra;
  size_t fxy, fz, fxy32, fz32, bpl, apl, df, total;
};
static FacLayout fac_layout(const ed_elemental_plan* P) {
  FacLayout L;
  const size_t K = 3ull * P->V3, esz = tc_esz(tc_kind_of(P->mode));
  L.rb = (long long)P->nbatch * (long long)P->fac_lchain.size() * P->fac_pxy * P->Ne;
  L.ra = (long long)P->nbatch * P->nchain * P->fac_pz * P->Ne;
  L.fxy = up256(sizeof(TcScalars));
  L.fz = L.fxy + up256((size_t)P->fac_pxy * P->V3 * 16);
  L.fxy32 = L.fz + up256((size_t)P->fac_pz * P->V3 * 16);
  L.fz32 = L.fxy32 + up256((size_t)P->fac_pxy * P->V3 * 8);
  L.bpl = L.fz32 + up256((size_t)P->fac_pz * P->V3 * 8);
  const size_t np = tcf_planes(P->gauss ? TCF_GAUSS : TCF_FOUR);  // re, im (and re + im) x hi, lo
  L.apl = L.bpl + up256(np * (size_t)L.rb * K * esz);
  L.df = L.apl + up256(np * (size_t)L.ra * K * esz);
  // the SM-pair stacked GEMM (ED_TUNE_TC_PAIR = 3) gives each CTA of a pair a plane of its own
  L.total = L.df + up256((P->tc_pair == 3 ? 2 : 1) * (size_t)P->g_elems * sizeof(float4));
  return L;
}

// Extra workspace of the Ozaki path: scalars, FP64 and complex64 factor
// tables (as fac_layout), per-row maxima of A and B, the A digit planes
// [8][RA][K] and B digit planes [12][RB][K] (int8).  The pair results go
// straight to the plan's complex128 G buffer.
struct OzLayout {
  long long rb, ra;
  size_t fxy, fz, fxy32, fz32, amax, bmax, apl, bpl, total;
};
static OzLayout oz_layout(const ed_elemental_plan* P) {
  OzLayout L;
  const size_t K = 3ull * P->V3;
  L.rb = (long long)P->nbatch * (long long)P->fac_lchain.size() * P->fac_pxy * P->Ne;
  L.ra = (long long)P->nbatch * P->nchain * P->fac_pz * P->Ne;
  L.fxy = up256(sizeof(TcScalars));
  L.fz = L.fxy + up256((size_t)P->fac_pxy * P->V3 * 16);
  L.fxy32 = L.fz + up256((size_t)P->fac_pz * P->V3 * 16);
  L.fz32 = L.fxy32 + up256((size_t)P->fac_pxy * P->V3 * 8);
  L.amax = L.fz32 + up256((size_t)P->fac_pz * P->V3 * 8);
  L.bmax = L.amax + up256((size_t)L.ra * 4);
  L.apl = L.bmax + up256((size_t)L.rb * 4);
  L.bpl = L.apl + up256((size_t)OZ_AP * L.ra * K);
  L.total = L.bpl + up256((size_t)OZ_BP * L.rb * K);
  return L;
}

size_t tc_extra_workspace(const ed_elemental_plan* P) {
  const int kind = tc_kind_of(P->mode);
  if (!kind) return 0;
  if (kind == TC_OZAKI) return P->fac ? oz_layout(P).total : 0;
  if (P->fac) return fac_layout(P).total;
  const size_t R = (size_t)P->nchain * P->nbatch * P->Ne;
  const size_t K = 3ull * P->V3;
  return up256(sizeof(TcScalars)) + up256((size_t)P->nmom * P->V3 * 8) + up256(4 * R * K * tc_esz(kind)) +
         up256((size_t)P->g_elems * sizeof(float4));
}

int tc_plan_check(ed_elemental_plan* P) {
  P->tc_kind = tc_kind_of(P->mode);
  if (P->gauss && (!P->tc_kind || P->tc_kind == TC_OZAKI || !P->fac)) {
    set_error("the Gauss form (ED_MODE_FLAG_GAUSS) needs f16x3, bf16x3 or tf32x3 with a factorised momentum list");
    return ED_ERR_UNSUPPORTED;
  }
  if (!P->tc_kind) return ED_OK;
  if (P->V3 % 32 != 0) {
    set_error("tensor-core elemental modes need Lx*Ly*Lz divisible by 32 (got %d)", P->V3);
    return ED_ERR_UNSUPPORTED;
  }
  if (P->tc_kind == TC_OZAKI) {
    if (!P->fac) {
      set_error("the Ozaki int8 mode needs a distinct momentum list of at most %d (px,py) x pz combinations "
                "(and not a generic pair plan)", kMaxFac);
      return ED_ERR_UNSUPPORTED;
    }
    if (3LL * P->V3 > OZ_MAX_K) {
      set_error("the Ozaki int8 mode keeps int32 sums exact for 3*Lx*Ly*Lz <= %lld (got %lld)", OZ_MAX_K,
                3LL * P->V3);
      return ED_ERR_UNSUPPORTED;
    }
  }
  const long long rows = 4LL * P->nchain * P->nbatch * P->Ne;
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

// The on-chip-phase tensor-core path of one batched plan, in three parts: the operands (scale, split
// planes, FP32 phases, cleared results) and the description of its GEMM launch (tensor map, job table),
// the GEMM, and the double-float -> complex128 conversion.  A multi-volume run issues the first and last
// part per plan and one GEMM launch for all of them.
template <int KIND>
static int tc_onchip_prepare(const ed_elemental_plan* P, const cplx<float>* chains, const cplx<double>* phases,
                             void* extra, cudaStream_t stream, int nb, TcMultiVol* d, bool* staged) {
  constexpr int ESZ = Split<KIND>::ESZ;
  char* X = (char*)extra;
  TcScalars* sc = (TcScalars*)X;
  cplx<float>* ph32 = (cplx<float>*)(X + up256(sizeof(TcScalars)));
  void* planes = X + up256(sizeof(TcScalars)) + up256((size_t)P->nmom * P->V3 * 8);
  // rows of all chains of the plan's batch (the plane stride), and of the nb timeslices in use
  const long long R = (long long)P->nchain * P->nbatch * P->Ne;
  const long long R_used = (long long)P->nchain * nb * P->Ne;
  const long long K = 3LL * P->V3;
  float4* DF = (float4*)((char*)planes + up256(4 * (size_t)R * K * ESZ));

  cudaError_t e = cudaMemsetAsync(sc, 0, sizeof(TcScalars), stream);
  if (e != cudaSuccess) return cuda_status(e, "tc scalars reset");
  const int sms = num_sms();
  tc_absmax_kernel<<<4 * sms, 256, 0, stream>>>((const float*)chains, 2 * R_used * K, sc);
  tc_scale_kernel<<<1, 32, 0, stream>>>(sc, KIND, g_tc_wait_cycles, g_tc_wait_probe);
  tc_split_kernel<KIND><<<8 * sms, 256, 0, stream>>>(chains, R_used, R, K, sc, planes);
  tc_phase_kernel<<<2 * sms, 256, 0, stream>>>(phases, (long long)P->nmom * P->V3, sc, ph32);
  ED_RETURN_LAUNCH("tensor-core operand preparation");

  EncodeFn enc = get_encode();
  if (!enc) {
    set_error("cuTensorMapEncodeTiled is unavailable from the driver");
    return ED_ERR_CUDA;
  }
  cuuint64_t gdim[2] = {(cuuint64_t)K, (cuuint64_t)(4 * R)};
  cuuint64_t gstride[1] = {(cuuint64_t)(K * ESZ)};
  cuuint32_t box[2] = {(cuuint32_t)(TC_ROWB / ESZ), (cuuint32_t)TC_BM};
  cuuint32_t estride[2] = {1, 1};
  CUresult cr = enc(&d->amap, KIND == TC_TF32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_UINT16, 2,
                    planes, gdim, gstride, box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (cr != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d)", (int)cr);
    return ED_ERR_CUDA;
  }

  TcTable& tab = d->tab;
  tab.njobs = nb * P->jobs_per_t;
  int tiles = 0;
  for (int k = 0; k < tab.njobs; ++k) {
    const Job& j = P->jobs[k];
    TcJob& t = tab.j[k];
    t.left = j.left;
    t.right0 = j.right0;
    t.nright = j.nright;
    t.g_off = j.g_off;
    t.mt = ceil_div((long long)j.nright * P->Ne, TC_BM);
    t.nt = ceil_div((long long)P->Ne * P->nmom, TC_BN);
    t.tile0 = tiles;
    tiles += t.mt * t.nt;
  }
  // stage the producers' rows in shared memory when they fit (see tc_pair_gemm.cuh)
  d->xr = std::min(P->Ne, (TC_BN - 1) / P->nmom + 2);
  *staged = (long long)(d->xr + P->nmom) * (long long)((TC_ROWB / ESZ) * 8 + TC_XP_PAD) <= TC_XP_BYTES;
  d->chains = chains;
  d->phases = ph32;
  d->sc = sc;
  d->DF = DF;
  d->R = R;
  d->Ne = P->Ne;
  d->nmom = P->nmom;
  d->V3 = P->V3;
  d->tile0 = tiles;  // the caller turns this count into the volume's first block
  // stacked form unless the four-product form is asked for; k-blocks per accumulator group (stacked form only)
  d->kpb = P->tc_stack == 2 ? 1 : (P->tc_kpb > 0 ? P->tc_kpb : 2);
  const long long g_used = (long long)nb * P->g_per_t;
  e = cudaMemsetAsync(DF, 0, (size_t)g_used * sizeof(float4), stream);
  if (e != cudaSuccess) return cuda_status(e, "clearing the pair results");
  return ED_OK;
}

static int tc_onchip_finish(const ed_elemental_plan* P, const TcMultiVol& d, cplx<double>* G, cudaStream_t stream,
                            int nb) {
  tc_df_to_c128_kernel<<<8 * num_sms(), 256, 0, stream>>>(d.DF, (long long)nb * P->g_per_t, G);
  ED_RETURN_LAUNCH("double-float to complex128");
  return ED_OK;
}

// the dynamic shared memory attribute of a pair-GEMM kernel, set once per kernel
static int tc_set_smem(const void* kern) {
  static const void* done[16] = {};
  for (const void* k : done)
    if (k == kern) return ED_OK;
  const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM);
  if (e != cudaSuccess) return cuda_status(e, "tc kernel smem attribute");
  for (const void*& k : done)
    if (!k) {
      k = kern;
      break;
    }
  return ED_OK;
}

template <int KIND>
static int launch_kind(const ed_elemental_plan* P, const cplx<float>* chains, const cplx<double>* phases,
                       cplx<double>* G, void* extra, cudaStream_t stream, int nb) {
  TcMultiVol d;
  bool staged = false;
  int rc = tc_onchip_prepare<KIND>(P, chains, phases, extra, stream, nb, &d, &staged);
  if (rc) return rc;
  const int tiles = d.tile0;
  const bool stack = P->tc_stack != 2;
  auto kern = staged ? (stack ? tc_pair_gemm_kernel<KIND, true, true> : tc_pair_gemm_kernel<KIND, true, false>)
                     : (stack ? tc_pair_gemm_kernel<KIND, false, true> : tc_pair_gemm_kernel<KIND, false, false>);
  rc = tc_set_smem((const void*)kern);
  if (rc) return rc;
  if (P->prof_start) cudaEventRecord(P->prof_start, stream);
  kern<<<tiles, TC_THREADS, TC_SMEM, stream>>>(d.amap, d.tab, d.Ne, d.nmom, d.V3, d.R, d.chains, d.phases, d.sc,
                                                d.DF, d.xr, d.kpb);
  if (P->prof_stop) cudaEventRecord(P->prof_stop, stream);
  ED_RETURN_LAUNCH("tensor-core pair GEMM");
  return tc_onchip_finish(P, d, G, stream, nb);
}

template <int KIND>
static int launch_multi_kind(int nplans, const ed_elemental_plan* const* plans, const int* nbs, void* const* ws,
                             cudaStream_t stream) {
  TcMulti M;  // the launch's parameters (about 9 KB, copied by the launch)
  M.nvol = nplans;
  bool all_staged = true;
  long long tiles = 0;
  for (int v = 0; v < nplans; ++v) {
    const ed_elemental_plan* P = plans[v];
    char* W = (char*)ws[v];
    bool staged = false;
    const int rc = tc_onchip_prepare<KIND>(P, (const cplx<float>*)(W + P->off_chain),
                                           (const cplx<double>*)(W + P->off_phase), W + P->off_extra, stream, nbs[v],
                                           &M.v[v], &staged);
    if (rc) return rc;
    all_staged = all_staged && staged;
    const int n = M.v[v].tile0;
    M.v[v].tile0 = (int)tiles;
    tiles += n;
  }
  if (tiles >= (1LL << 31)) {
    set_error("ed_elemental_gemm_multi: too many tiles for one launch");
    return ED_ERR_UNSUPPORTED;
  }
  const bool stack = plans[0]->tc_stack != 2;  // the caller groups plans of one form
  auto kern = all_staged ? (stack ? tc_pair_gemm_multi_kernel<KIND, true, true>
                                  : tc_pair_gemm_multi_kernel<KIND, true, false>)
                         : (stack ? tc_pair_gemm_multi_kernel<KIND, false, true>
                                  : tc_pair_gemm_multi_kernel<KIND, false, false>);
  int rc = tc_set_smem((const void*)kern);
  if (rc) return rc;
  if (tiles > 0) {
    kern<<<(unsigned)tiles, TC_THREADS, TC_SMEM, stream>>>(M);
    ED_RETURN_LAUNCH("tensor-core pair GEMM over several volumes");
  }
  for (int v = 0; v < nplans; ++v) {
    const ed_elemental_plan* P = plans[v];
    rc = tc_onchip_finish(P, M.v[v], (cplx<double>*)((char*)ws[v] + P->off_g), stream, nbs[v]);
    if (rc) return rc;
  }
  return ED_OK;
}

int launch_pair_gemm_tc_multi(int nplans, const ed_elemental_plan* const* plans, const int* nbs, void* const* ws,
                              cudaStream_t stream) {
  switch (plans[0]->tc_kind) {
    case TC_F16:
      return launch_multi_kind<TC_F16>(nplans, plans, nbs, ws, stream);
    case TC_BF16:
      return launch_multi_kind<TC_BF16>(nplans, plans, nbs, ws, stream);
    case TC_TF32:
      return launch_multi_kind<TC_TF32>(nplans, plans, nbs, ws, stream);
    default:
      set_error("ed_elemental_gemm_multi: not a tensor-core split mode");
      return ED_ERR_UNSUPPORTED;
  }
}

// Tensor map over four k-block-major planes of R rows: dimensions (k within
// the 64-byte row, row, plane*nkb + k-block); a box is 128 rows of one
// k-block, 8 KB contiguous in HBM.
static int encode_kmajor(CUtensorMap* map, int kind, void* base, long long K, long long R, int box_rows = TC_BM,
                         int nplanes = 4) {
  EncodeFn enc = get_encode();
  if (!enc) {
    set_error("cuTensorMapEncodeTiled is unavailable from the driver");
    return ED_ERR_CUDA;
  }
  const size_t esz = tc_esz(kind);
  const long long KB = TC_ROWB / (long long)esz, nkb = K / KB;
  cuuint64_t gdim[3] = {(cuuint64_t)KB, (cuuint64_t)R, (cuuint64_t)(nplanes * nkb)};
  cuuint64_t gstride[2] = {(cuuint64_t)TC_ROWB, (cuuint64_t)(R * TC_ROWB)};
  cuuint32_t box[3] = {(cuuint32_t)KB, (cuuint32_t)box_rows, 1};
  cuuint32_t estride[3] = {1, 1, 1};
  CUresult cr = enc(map, kind == TC_TF32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_UINT16, 3, base,
                    gdim, gstride, box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (cr != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d)", (int)cr);
    return ED_ERR_CUDA;
  }
  return ED_OK;
}

// The factorised-phase GEMMs on SM pairs, a cooperative launch of two-CTA clusters, every cluster co-resident:
// tc_fac2_gemm_kernel (four-product form, 256-row A tiles) or, with `stacked`, tc_fac2s_gemm_kernel (the
// single-SM tiles with the complex halves of A and B spread over the pair; two double-float planes).
template <int KIND>
static int launch_fac_pairs(const ed_elemental_plan* P, const FacLayout& lay, void* apl, void* bpl, TcScalars* sc,
                            float4* DF, cplx<double>* G, cudaStream_t stream, int nb, bool stacked) {
  const long long K = 3LL * P->V3;
  const int pxy = P->fac_pxy, pz = P->fac_pz, Ne = P->Ne, nl = (int)P->fac_lchain.size();
  int rc;
  CUtensorMap amap, bmap, bmap16;
  if ((rc = encode_kmajor(&amap, KIND, apl, K, lay.ra))) return rc;  // 128-row A boxes
  // B: 128-row boxes (stacked: a CTA holds every column of one plane) or 64-row halves
  if ((rc = encode_kmajor(&bmap, KIND, bpl, K, lay.rb, stacked ? TC_BN : TC_BN / 2))) return rc;
  if ((rc = encode_kmajor(&bmap16, KIND, bpl, K, lay.rb, 16))) return rc;  // narrow last column tile
  const int tile_rows = stacked ? TC_BM : TCP_BM;
  TcFacTable tab;
  tab.njobs = nb * P->jobs_per_t;
  tab.pxy = pxy;
  tab.pz = pz;
  for (int q = 0; q < kMaxFac; ++q) tab.pidx[q] = q < pxy * pz ? P->fac_pidx[q] : (signed char)-1;
  for (int k = 0; k < tab.njobs; ++k) {
    const Job& j = P->jobs[k];
    const int b = k / P->jobs_per_t;
    const int slot = b * nl + P->fac_lslot[P->jobs[k % P->jobs_per_t].left];
    TcFacJob& d = tab.j[k];
    d.arow0 = j.right0 * pz * Ne;
    d.brow0 = slot * pxy * Ne;
    d.nright = j.nright;
    d.g_off = j.g_off;
    d.mt = (int)ceil_div((long long)j.nright * pz * Ne, tile_rows);
    d.nt = (int)ceil_div((long long)pxy * Ne, TC_BN);
  }
  // a narrow last column tile: N rounded up to 32 (four-product: each CTA then holds N/2 rows of B, a
  // multiple of the 16-row box) or to 16 (stacked: each CTA holds the tile's columns of one plane)
  const int last_cols = pxy * Ne - (tab.j[0].nt - 1) * TC_BN;
  const int round_to = stacked ? 16 : 32;
  const bool narrow = ((last_cols + round_to - 1) & ~(round_to - 1)) < TC_BN;
  int tiles = 0, tiles_n = 0;
  for (int k = 0; k < tab.njobs; ++k) {
    TcFacJob& d = tab.j[k];
    d.tile0 = tiles;
    tiles += d.mt * (d.nt - (narrow ? 1 : 0));
    d.tile0n = tiles_n;
    tiles_n += narrow ? d.mt : 0;
  }
  tab.nfull = tiles;
  tiles += tiles_n;
  const int max_st = stacked ? TCS_MAX_STAGES : TCP_MAX_STAGES;
  const int nst = P->tc_stages > 0 ? std::min(P->tc_stages, max_st) : (stacked ? TCS_DEFAULT_STAGES : TCP_DEFAULT_STAGES);
  auto kern4 = tc_fac2_gemm_kernel<KIND>;
  auto kerns = tc_fac2s_gemm_kernel<KIND>;
  const void* kfn = stacked ? (const void*)kerns : (const void*)kern4;
  cudaError_t e;
  static bool attr_set[4][2] = {};
  if (!attr_set[KIND][stacked]) {
    e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             stacked ? tcs_smem(TCS_MAX_STAGES) : tcp_smem(TCP_MAX_STAGES));
    if (e != cudaSuccess) return cuda_status(e, "paired tc kernel smem attribute");
    attr_set[KIND][stacked] = true;
  }
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  attr[1].id = cudaLaunchAttributeCooperative;
  attr[1].val.cooperative = 1;
  cfg.blockDim = dim3(TC_THREADS);
  cfg.dynamicSmemBytes = stacked ? tcs_smem(nst) : tcp_smem(nst);
  cfg.stream = stream;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cfg.gridDim = dim3(2 * num_sms());
  int clusters = 0;
  e = cudaOccupancyMaxActiveClusters(&clusters, kfn, &cfg);
  if (e != cudaSuccess) return cuda_status(e, "paired tc kernel cluster occupancy");
  if (clusters < 1) {
    set_error("the paired factorised tensor-core GEMM does not fit on the device");
    return ED_ERR_UNSUPPORTED;
  }
  // persistent grid: every cluster co-resident (the step counter of the kernel relies on it)
  int pairs = std::min(tiles, clusters);
  if (P->tc_grid > 0) pairs = std::max(1, std::min(pairs, P->tc_grid / 2));
  cfg.gridDim = dim3(2 * pairs);
  cfg.numAttrs = 2;
  const int slab_kb = P->tc_slab_kb > 0 ? P->tc_slab_kb : TC_FLUSH_KB;
  const long long g_used = (long long)nb * P->g_per_t;
  const int planes = stacked ? 2 : 1;  // the stacked form's CTAs flush into planes of their own
  e = cudaMemsetAsync(DF, 0, (size_t)planes * g_used * sizeof(float4), stream);
  if (e != cudaSuccess) return cuda_status(e, "clearing the pair results");
  if (P->prof_start) cudaEventRecord(P->prof_start, stream);
  if (stacked) {
    const int kpb = P->tc_kpb > 0 ? P->tc_kpb : 2;
    e = cudaLaunchKernelEx(&cfg, kerns, amap, bmap, bmap16, tab, Ne, P->V3, sc, DF, g_used, tiles, slab_kb, nst, kpb);
  } else {
    const int kpb = P->tc_kpb > 0 ? P->tc_kpb : 1;
    e = cudaLaunchKernelEx(&cfg, kern4, amap, bmap, bmap16, tab, Ne, P->V3, sc, DF, tiles, slab_kb, nst, kpb);
  }
  if (P->prof_stop) cudaEventRecord(P->prof_stop, stream);
  if (e != cudaSuccess) return cuda_status(e, "paired factorised-phase GEMM launch");
  ED_RETURN_LAUNCH("paired factorised-phase GEMM");
  if (stacked)
    tc_df2_to_c128_kernel<<<8 * num_sms(), 256, 0, stream>>>(DF, g_used, g_used, G);
  else
    tc_df_to_c128_kernel<<<8 * num_sms(), 256, 0, stream>>>(DF, g_used, G);
  ED_RETURN_LAUNCH("double-float to complex128");
  return ED_OK;
}

// Factorised-phase path: factor tables, left/right variant planes, one GEMM
// launch over all groups of the nb timeslices, double-float -> complex128.
template <int KIND>
static int launch_fac(const ed_elemental_plan* P, const cplx<float>* chains, cplx<double>* G, void* extra,
                      cudaStream_t stream, int nb) {
  const FacLayout lay = fac_layout(P);
  char* X = (char*)extra;
  TcScalars* sc = (TcScalars*)X;
  cplx<double>* fxy = (cplx<double>*)(X + lay.fxy);
  cplx<double>* fz = (cplx<double>*)(X + lay.fz);
  cplx<float>* fxy32 = (cplx<float>*)(X + lay.fxy32);
  cplx<float>* fz32 = (cplx<float>*)(X + lay.fz32);
  void* bpl = X + lay.bpl;
  void* apl = X + lay.apl;
  float4* DF = (float4*)(X + lay.df);
  const long long K = 3LL * P->V3;
  const int nl = (int)P->fac_lchain.size(), pxy = P->fac_pxy, pz = P->fac_pz, Ne = P->Ne;
  const Latt L{P->Lx, P->Ly, P->Lz};

  cudaError_t e = cudaMemsetAsync(sc, 0, sizeof(TcScalars), stream);
  if (e != cudaSuccess) return cuda_status(e, "tc scalars reset");
  const int sms = num_sms();
  const long long R_used = (long long)P->nchain * nb * Ne;
  tc_absmax_kernel<<<4 * sms, 256, 0, stream>>>((const float*)chains, 2 * R_used * K, sc);
  tc_scale_kernel<<<1, 32, 0, stream>>>(sc, KIND, g_tc_wait_cycles, g_tc_wait_probe);
  ED_RETURN_LAUNCH("tensor-core operand scale");
  std::vector<int> m3;
  m3.assign(P->fac_l.begin(), P->fac_l.begin() + 3 * pxy);
  int rc = launch_phases(L, m3.data(), pxy, fxy, stream);
  if (rc) return rc;
  m3.clear();
  m3.assign(P->fac_r.begin(), P->fac_r.begin() + 3 * pz);
  rc = launch_phases(L, m3.data(), pz, fz, stream);
  if (rc) return rc;
  tc_phase_kernel<<<sms, 256, 0, stream>>>(fxy, (long long)pxy * P->V3, sc, fxy32);
  tc_phase_kernel<<<sms, 256, 0, stream>>>(fz, (long long)pz * P->V3, sc, fz32);
  ED_RETURN_LAUNCH("factor tables");

  TcFacSlots sl;
  sl.nl = nl;
  sl.nchain = P->nchain;
  for (int s = 0; s < nl; ++s) sl.lchain[s] = P->fac_lchain[s];
  const int kxl = (int)ceil_div(K / 2, 256 * kSplitUnrollLeft), kxr = (int)ceil_div(K / 2, 256 * kSplitUnrollRight);
  const int lrows = nb * nl * Ne, rrows = nb * P->nchain * Ne;
  if (P->gauss) {
    tc_fac_split_kernel<KIND, true, kSplitUnrollLeft, true><<<dim3(kxl, std::min(lrows, 65535)), 256, 0, stream>>>(
        chains, sl, lrows, Ne, pxy, fxy32, P->V3, lay.rb, bpl);
    tc_fac_split_kernel<KIND, false, kSplitUnrollRight, true><<<dim3(kxr, std::min(rrows, 65535)), 256, 0, stream>>>(
        chains, sl, rrows, Ne, pz, fz32, P->V3, lay.ra, apl);
  } else {
    tc_fac_split_kernel<KIND, true, kSplitUnrollLeft, false><<<dim3(kxl, std::min(lrows, 65535)), 256, 0, stream>>>(
        chains, sl, lrows, Ne, pxy, fxy32, P->V3, lay.rb, bpl);
    tc_fac_split_kernel<KIND, false, kSplitUnrollRight, false><<<dim3(kxr, std::min(rrows, 65535)), 256, 0, stream>>>(
        chains, sl, rrows, Ne, pz, fz32, P->V3, lay.ra, apl);
  }
  ED_RETURN_LAUNCH("variant planes");

  if (P->tc_pair >= 2 && !P->gauss)
    return launch_fac_pairs<KIND>(P, lay, apl, bpl, sc, DF, G, stream, nb, P->tc_pair == 3);

  const int form = P->gauss ? TCF_GAUSS : (P->tc_stack == 2 ? TCF_FOUR : TCF_STACKED);
  const int np = tcf_planes(form);
  CUtensorMap amap, bmap, bmap16;
  if ((rc = encode_kmajor(&amap, KIND, apl, K, lay.ra, TC_BM, np))) return rc;
  if ((rc = encode_kmajor(&bmap, KIND, bpl, K, lay.rb, TC_BN, np))) return rc;
  if ((rc = encode_kmajor(&bmap16, KIND, bpl, K, lay.rb, 16, np))) return rc;  // the narrow last column tile

  TcFacTable tab;
  tab.njobs = nb * P->jobs_per_t;
  tab.pxy = pxy;
  tab.pz = pz;
  for (int q = 0; q < kMaxFac; ++q) tab.pidx[q] = q < pxy * pz ? P->fac_pidx[q] : (signed char)-1;
  int tiles = 0;
  for (int k = 0; k < tab.njobs; ++k) {
    const Job& j = P->jobs[k];
    const int b = k / P->jobs_per_t;
    const int slot = b * nl + P->fac_lslot[P->jobs[k % P->jobs_per_t].left];
    TcFacJob& d = tab.j[k];
    d.arow0 = j.right0 * pz * Ne;
    d.brow0 = slot * pxy * Ne;
    d.nright = j.nright;
    d.g_off = j.g_off;
    d.mt = (int)ceil_div((long long)j.nright * pz * Ne, TC_BM);
    d.nt = (int)ceil_div((long long)pxy * Ne, TC_BN);
  }
  // a last column tile of at most 112 valid columns runs narrow (16-row B boxes, smaller MMA N); number the
  // full tiles first and the narrow ones after them
  const int last_cols = pxy * Ne - (tab.j[0].nt - 1) * TC_BN;
  const bool narrow = ((last_cols + 15) & ~15) < TC_BN;
  int tiles_n = 0;
  for (int k = 0; k < tab.njobs; ++k) {
    TcFacJob& d = tab.j[k];
    d.tile0 = tiles;
    tiles += d.mt * (d.nt - (narrow ? 1 : 0));
    d.tile0n = tiles_n;
    tiles_n += narrow ? d.mt : 0;
  }
  tab.nfull = tiles;
  tiles += tiles_n;
  // the stacked form unless the four-product or the Gauss form is asked for
  auto kern = form == TCF_GAUSS     ? tc_fac_gemm_kernel<KIND, TCF_GAUSS>
              : form == TCF_STACKED ? tc_fac_gemm_kernel<KIND, TCF_STACKED>
                                    : tc_fac_gemm_kernel<KIND, TCF_FOUR>;
  const int smax = tcf_smem(tcf_max_stages(form), form);
  static bool attr_set[4][3] = {};
  static int resident[4][3] = {};
  if (!attr_set[KIND][form]) {
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smax);
    if (e != cudaSuccess) return cuda_status(e, "tc kernel smem attribute");
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident[KIND][form], kern, TC_THREADS, smax);
    if (e != cudaSuccess) return cuda_status(e, "tc kernel occupancy");
    if (resident[KIND][form] < 1) {
      set_error("the factorised tensor-core GEMM does not fit on an SM");
      return ED_ERR_UNSUPPORTED;
    }
    attr_set[KIND][form] = true;
  }
  const long long g_used = (long long)nb * P->g_per_t;
  e = cudaMemsetAsync(DF, 0, (size_t)g_used * sizeof(float4), stream);
  if (e != cudaSuccess) return cuda_status(e, "clearing the pair results");
  // persistent grid: every CTA co-resident (the step counter of the kernel relies on it)
  int grid = std::min(tiles, resident[KIND][form] * sms);
  if (P->tc_grid > 0) grid = std::min(grid, P->tc_grid);
  const int slab_kb = P->tc_slab_kb > 0 ? P->tc_slab_kb : TC_FLUSH_KB;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(TC_THREADS);
  const int nst = std::min(P->tc_stages > 0 ? P->tc_stages : TCF_DEFAULT_STAGES, tcf_max_stages(form));
  cfg.dynamicSmemBytes = tcf_smem(nst, form);
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (P->prof_start) cudaEventRecord(P->prof_start, stream);
  const int kpb = P->tc_kpb > 0 ? P->tc_kpb : (form == TCF_FOUR ? 1 : 2);
  e = cudaLaunchKernelEx(&cfg, kern, amap, bmap, bmap16, tab, Ne, P->V3, sc, DF, tiles, slab_kb, nst, kpb);
  if (P->prof_stop) cudaEventRecord(P->prof_stop, stream);
  if (e != cudaSuccess) return cuda_status(e, "tensor-core factorised-phase GEMM launch");
  ED_RETURN_LAUNCH("tensor-core factorised-phase GEMM");
  tc_df_to_c128_kernel<<<8 * sms, 256, 0, stream>>>(DF, g_used, G);
  ED_RETURN_LAUNCH("double-float to complex128");
  return ED_OK;
}

// ---- Ozaki int8 path
// Per-row maxima of the variant rows: one block per input row (slot, i), all
// nvar variants of that row; max over k of |re|, |im| of the FP32 product.
template <bool LEFT>
__global__ void oz_rowmax_kernel(const cplx<float>* __restrict__ chains, TcFacSlots sl, int Ne, int nvar,
                                 const cplx<float>* __restrict__ fac, int V3, float* __restrict__ rowmax) {
  __shared__ float red[OZ_MAX_VAR][8];
  const int row = blockIdx.x;
  const int slot = row / Ne, i = row - (row / Ne) * Ne;
  const int chain = LEFT ? (slot / sl.nl) * sl.nchain + sl.lchain[slot % sl.nl] : slot;
  const float4* src = reinterpret_cast<const float4*>(chains + ((long long)chain * Ne + i) * 3LL * V3);
  const int K2 = 3 * V3 / 2;
  float m[OZ_MAX_VAR];
#pragma unroll
  for (int a = 0; a < OZ_MAX_VAR; ++a) m[a] = 0.f;
  for (int kp = threadIdx.x; kp < K2; kp += blockDim.x) {
    const float4 v = src[kp];
    const int site = (2 * kp) % V3;
#pragma unroll
    for (int a = 0; a < OZ_MAX_VAR; ++a) {
      if (a >= nvar) break;
      const float4 f = *reinterpret_cast<const float4*>(fac + (long long)a * V3 + site);
      float r0, i0, r1, i1;
      if constexpr (LEFT) {
        r0 = v.x * f.x + v.y * f.y;
        i0 = v.x * f.y - v.y * f.x;
        r1 = v.z * f.z + v.w * f.w;
        i1 = v.z * f.w - v.w * f.z;
      } else {
        r0 = f.x * v.x - f.y * v.y;
        i0 = f.x * v.y + f.y * v.x;
        r1 = f.z * v.z - f.w * v.w;
        i1 = f.z * v.w + f.w * v.z;
      }
      m[a] = fmaxf(m[a], fmaxf(fmaxf(fabsf(r0), fabsf(i0)), fmaxf(fabsf(r1), fabsf(i1))));
    }
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int a = 0; a < OZ_MAX_VAR; ++a) {
    if (a >= nvar) break;
    float x = m[a];
    for (int o = 16; o > 0; o >>= 1) x = fmaxf(x, __shfl_xor_sync(0xffffffffu, x, o));
    if (lane == 0) red[a][warp] = x;
  }
  __syncthreads();
  if ((int)threadIdx.x < nvar) {
    float x = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) x = fmaxf(x, red[threadIdx.x][w]);
    rowmax[((long long)slot * nvar + threadIdx.x) * Ne + i] = x;
  }
}

// four signed 6-bit digits of v in (-1, 1): v = sum_s d_s 2^(-6(s+1)) up to
// 2^-25; every step is exact in FP32 (x - rint(x) keeps the fraction bits of x)
__device__ __forceinline__ void oz_digits(float v, int (&d)[OZ_S]) {
  float x = v * 64.f;
#pragma unroll
  for (int s = 0; s < OZ_S; ++s) {
    const float r = rintf(x);
    d[s] = (int)r;
    x = (x - r) * 64.f;
  }
}

// Digit planes of the variant rows: each thread handles 4 consecutive k of
// one input row and writes 4-byte words (4 int8 digits) per plane.
//   A (right, !LEFT): planes q = s*2 + {re, im};  B (LEFT): q = s*3 + {re, im, -im}
template <bool LEFT>
__global__ void oz_digit_kernel(const cplx<float>* __restrict__ chains, TcFacSlots sl, int nrows, int Ne, int nvar,
                                const cplx<float>* __restrict__ fac, int V3, const float* __restrict__ rowmax,
                                long long Rplane, int8_t* __restrict__ planes) {
  constexpr int NP = LEFT ? 3 : 2;
  const long long K = 3LL * V3;
  const int K4 = (int)(K / 4);
  for (int row = blockIdx.y; row < nrows; row += gridDim.y) {
    const int slot = row / Ne, i = row - (row / Ne) * Ne;
    const int chain = LEFT ? (slot / sl.nl) * sl.nchain + sl.lchain[slot % sl.nl] : slot;
    const float4* src = reinterpret_cast<const float4*>(chains + ((long long)chain * Ne + i) * K);
    for (int kq = blockIdx.x * blockDim.x + threadIdx.x; kq < K4; kq += gridDim.x * blockDim.x) {
      const float4 v0 = src[2 * kq], v1 = src[2 * kq + 1];
      const float xr[4] = {v0.x, v0.z, v1.x, v1.z}, xi[4] = {v0.y, v0.w, v1.y, v1.w};
      const int site = (4 * kq) % V3;  // 4 | V3: the four elements share a colour plane
      for (int a = 0; a < nvar; ++a) {
        const long long orow = ((long long)slot * nvar + a) * Ne + i;
        int e = 0;
        const float mx = rowmax[orow];
        if (mx > 0.f) frexpf(mx, &e);
        const float4 f0 = *reinterpret_cast<const float4*>(fac + (long long)a * V3 + site);
        const float4 f1 = *reinterpret_cast<const float4*>(fac + (long long)a * V3 + site + 2);
        const float fr[4] = {f0.x, f0.z, f1.x, f1.z}, fi[4] = {f0.y, f0.w, f1.y, f1.w};
        uint32_t wre[OZ_S] = {}, wim[OZ_S] = {}, wneg[OZ_S] = {};
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          float re, im;
          if constexpr (LEFT) {
            re = xr[u] * fr[u] + xi[u] * fi[u];
            im = xr[u] * fi[u] - xi[u] * fr[u];
          } else {
            re = fr[u] * xr[u] - fi[u] * xi[u];
            im = fr[u] * xi[u] + fi[u] * xr[u];
          }
          int dr[OZ_S], di[OZ_S];
          oz_digits(ldexpf(re, -e), dr);
          oz_digits(ldexpf(im, -e), di);
#pragma unroll
          for (int s = 0; s < OZ_S; ++s) {
            wre[s] |= (uint32_t)(dr[s] & 0xff) << (8 * u);
            wim[s] |= (uint32_t)(di[s] & 0xff) << (8 * u);
            wneg[s] |= (uint32_t)((-di[s]) & 0xff) << (8 * u);
          }
        }
        uint32_t* P = reinterpret_cast<uint32_t*>(planes);
        const long long w = orow * (K / 4) + kq, plane = Rplane * (K / 4);
#pragma unroll
        for (int s = 0; s < OZ_S; ++s) {
          P[(s * NP + 0) * plane + w] = wre[s];
          P[(s * NP + 1) * plane + w] = wim[s];
          if constexpr (LEFT) P[(s * NP + 2) * plane + w] = wneg[s];
        }
      }
    }
  }
}

static int encode_i8(CUtensorMap* map, void* base, long long K, long long rows) {
  EncodeFn enc = get_encode();
  if (!enc) {
    set_error("cuTensorMapEncodeTiled is unavailable from the driver");
    return ED_ERR_CUDA;
  }
  cuuint64_t gdim[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  cuuint64_t gstride[1] = {(cuuint64_t)K};
  cuuint32_t box[2] = {(cuuint32_t)OZ_KS, (cuuint32_t)OZ_BM};
  cuuint32_t estride[2] = {1, 1};
  CUresult cr = enc(map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, base, gdim, gstride, box, estride,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_32B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (cr != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d)", (int)cr);
    return ED_ERR_CUDA;
  }
  return ED_OK;
}

static int launch_ozaki(const ed_elemental_plan* P, const cplx<float>* chains, cplx<double>* G, void* extra,
                        cudaStream_t stream, int nb) {
  const OzLayout lay = oz_layout(P);
  char* X = (char*)extra;
  TcScalars* sc = (TcScalars*)X;
  cplx<double>* fxy = (cplx<double>*)(X + lay.fxy);
  cplx<double>* fz = (cplx<double>*)(X + lay.fz);
  cplx<float>* fxy32 = (cplx<float>*)(X + lay.fxy32);
  cplx<float>* fz32 = (cplx<float>*)(X + lay.fz32);
  float* amax = (float*)(X + lay.amax);
  float* bmax = (float*)(X + lay.bmax);
  int8_t* apl = (int8_t*)(X + lay.apl);
  int8_t* bpl = (int8_t*)(X + lay.bpl);
  const long long K = 3LL * P->V3;
  const int nl = (int)P->fac_lchain.size(), pxy = P->fac_pxy, pz = P->fac_pz, Ne = P->Ne;
  const Latt L{P->Lx, P->Ly, P->Lz};

  cudaError_t e = cudaMemsetAsync(sc, 0, sizeof(TcScalars), stream);  // scale 2^0, status 0
  if (e != cudaSuccess) return cuda_status(e, "tc scalars reset");
  const int sms = num_sms();
  std::vector<int> m3;
  m3.assign(P->fac_l.begin(), P->fac_l.begin() + 3 * pxy);
  int rc = launch_phases(L, m3.data(), pxy, fxy, stream);
  if (rc) return rc;
  m3.clear();
  m3.assign(P->fac_r.begin(), P->fac_r.begin() + 3 * pz);
  rc = launch_phases(L, m3.data(), pz, fz, stream);
  if (rc) return rc;
  tc_phase_kernel<<<sms, 256, 0, stream>>>(fxy, (long long)pxy * P->V3, sc, fxy32);
  tc_phase_kernel<<<sms, 256, 0, stream>>>(fz, (long long)pz * P->V3, sc, fz32);
  ED_RETURN_LAUNCH("factor tables");

  TcFacSlots sl;
  sl.nl = nl;
  sl.nchain = P->nchain;
  for (int s = 0; s < nl; ++s) sl.lchain[s] = P->fac_lchain[s];
  const int lrows = nb * nl * Ne, rrows = nb * P->nchain * Ne;
  oz_rowmax_kernel<true><<<lrows, 256, 0, stream>>>(chains, sl, Ne, pxy, fxy32, P->V3, bmax);
  oz_rowmax_kernel<false><<<rrows, 256, 0, stream>>>(chains, sl, Ne, pz, fz32, P->V3, amax);
  const int kx = (int)ceil_div(K / 4, 256);
  oz_digit_kernel<true><<<dim3(kx, std::min(lrows, 65535)), 256, 0, stream>>>(chains, sl, lrows, Ne, pxy, fxy32,
                                                                               P->V3, bmax, lay.rb, bpl);
  oz_digit_kernel<false><<<dim3(kx, std::min(rrows, 65535)), 256, 0, stream>>>(chains, sl, rrows, Ne, pz, fz32,
                                                                                P->V3, amax, lay.ra, apl);
  ED_RETURN_LAUNCH("Ozaki digit planes");

  CUtensorMap amap, bmap;
  if ((rc = encode_i8(&amap, apl, K, OZ_AP * lay.ra))) return rc;
  if ((rc = encode_i8(&bmap, bpl, K, OZ_BP * lay.rb))) return rc;

  TcFacTable tab;
  tab.njobs = nb * P->jobs_per_t;
  tab.pxy = pxy;
  tab.pz = pz;
  for (int q = 0; q < kMaxFac; ++q) tab.pidx[q] = q < pxy * pz ? P->fac_pidx[q] : (signed char)-1;
  int tiles = 0;
  for (int k = 0; k < tab.njobs; ++k) {
    const Job& j = P->jobs[k];
    const int b = k / P->jobs_per_t;
    const int slot = b * nl + P->fac_lslot[P->jobs[k % P->jobs_per_t].left];
    TcFacJob& d = tab.j[k];
    d.arow0 = j.right0 * pz * Ne;
    d.brow0 = slot * pxy * Ne;
    d.nright = j.nright;
    d.g_off = j.g_off;
    d.mt = (int)ceil_div((long long)j.nright * pz * Ne, OZ_BM);
    d.nt = (int)ceil_div((long long)pxy * Ne, OZ_BN);
    d.tile0 = tiles;
    tiles += d.mt * d.nt;
  }
  tab.nfull = tiles;  // every tile full-width (the Ozaki kernel numbers its tiles per group)
  static bool attr_set = false;
  if (!attr_set) {
    e = cudaFuncSetAttribute(tc_ozaki_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, OZ_SMEM);
    if (e != cudaSuccess) return cuda_status(e, "Ozaki kernel smem attribute");
    attr_set = true;
  }
  if (P->prof_start) cudaEventRecord(P->prof_start, stream);
  tc_ozaki_gemm_kernel<<<tiles, OZ_THREADS, OZ_SMEM, stream>>>(amap, bmap, tab, Ne, P->V3, (int)lay.ra, (int)lay.rb,
                                                              amax, bmax, sc, G);
  if (P->prof_stop) cudaEventRecord(P->prof_stop, stream);
  ED_RETURN_LAUNCH("Ozaki int8 pair GEMM");
  return ED_OK;
}

int launch_pair_gemm_tc(const ed_elemental_plan* P, const cplx<float>* chains, const cplx<double>* phases,
                        cplx<double>* G, void* extra, cudaStream_t stream, int nb) {
  if (P->tc_kind == TC_OZAKI) return launch_ozaki(P, chains, G, extra, stream, nb);
  if (P->fac) {
    switch (P->tc_kind) {
      case TC_F16:
        return launch_fac<TC_F16>(P, chains, G, extra, stream, nb);
      case TC_BF16:
        return launch_fac<TC_BF16>(P, chains, G, extra, stream, nb);
      case TC_TF32:
        return launch_fac<TC_TF32>(P, chains, G, extra, stream, nb);
      default:
        break;
    }
  }
  switch (P->tc_kind) {
    case TC_F16:
      return launch_kind<TC_F16>(P, chains, phases, G, extra, stream, nb);
    case TC_BF16:
      return launch_kind<TC_BF16>(P, chains, phases, G, extra, stream, nb);
    case TC_TF32:
      return launch_kind<TC_TF32>(P, chains, phases, G, extra, stream, nb);
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

extern "C" int ed_elemental_wait_limit(long long cycles) {
  ED_CHECK_ARG(cycles >= 0, "ed_elemental_wait_limit: negative limit");
  ed::g_tc_wait_cycles = cycles;
  return ED_OK;
}

extern "C" int ed_elemental_wait_probe(int on) {
  ed::g_tc_wait_probe = on ? 1 : 0;
  return ED_OK;
}
