// Ozaki-style integer-slice pair contraction (included by elemental_tc.cu).
//
// Same factorised operands as tc_fac_gemm.cuh (right variants g_c Y_j on the M
// side, left variants conj(X_i) f_a on the N side), but every operand row r
// is written as 2^e_r * sum_{s<4} d_s 2^(-6(s+1)) with e_r the power of two
// just above the row's largest |re|, |im| and signed 6-bit digits d_s
// (|d_0| <= 64, |d_s| <= 32 after), an exact decomposition of the FP32 value.
// The products of digit slices with s + t <= 3 are accumulated exactly in
// int32, one accumulator per weight w = s + t and per real/imaginary part:
//   re_w += sum_{s+t=w} ar_s br_t + ai_s (-bi)_t,   im_w += ar_s bi_t + ai_s br_t
// (|re_w|, |im_w| <= 12288 K < 2^31 for K <= 163840), and the epilogue forms
//   G = 2^(e_m + e_n) sum_w 2^(-6(w+2)) (re_w + i im_w)
// in FP64.  Dropped products (s + t >= 4) weigh <= 2^-30 of the leading one;
// the digits carry the 24-bit precision of the complex64 operands.
//
// The integer MMAs are the warp-level mma.sync.m16n8k32.s8 instructions:
// tcgen05.mma has no .kind::i8 on sm_103a.  Tile: 64 (M) x 64 (N) per CTA,
// 8 warps of 16 x 32 (four m16n8 fragments; 4 weights x 2 parts x 4 fragments
// x 4 = 128 int32 accumulators per thread).  Stages of 32 k (one MMA K) hold
// the 8 A digit planes and 12 B digit planes of the tile (40 KB), loaded by
// TMA with the 32-byte swizzle (conflict-free ldmatrix), 4 stages deep.

constexpr int OZ_BM = 64, OZ_BN = 64, OZ_KS = 32;  // tile rows, cols, k per stage (bytes)
constexpr int OZ_S = 4;                              // digit slices
constexpr int OZ_AP = OZ_S * 2;                      // A planes: slice x (re, im)
constexpr int OZ_BP = OZ_S * 3;                      // B planes: slice x (re, im, -im)
constexpr int OZ_A_BYTES = OZ_AP * OZ_BM * OZ_KS;    // 16 KB
constexpr int OZ_B_BYTES = OZ_BP * OZ_BN * OZ_KS;    // 24 KB
constexpr int OZ_STAGE_BYTES = OZ_A_BYTES + OZ_B_BYTES;
constexpr int OZ_STAGES = 4;
constexpr int OZ_THREADS = 256;
constexpr int OZ_SMEM = OZ_STAGES * OZ_STAGE_BYTES + 1024 + 256;
static_assert(OZ_SMEM <= 232448, "shared memory per block");
constexpr long long OZ_MAX_K = 163840;  // int32 accumulation stays exact below this K
constexpr int OZ_MAX_VAR = 16;          // variants per operand row handled by the row-maximum kernel

// byte offset of (row, 16-byte chunk) in a 32-byte-row plane written by TMA with the 32-byte swizzle
__device__ __forceinline__ uint32_t oz_swz(int row, int chunk) {
  return (uint32_t)(row * 32 + ((chunk ^ ((row >> 2) & 1)) << 4));
}

__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(addr));
}

__device__ __forceinline__ void imma(int (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
      : "+r"(c[0]), "+r"(c[1]), "+r"(c[2]), "+r"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// 2^e with e from frexp of the row maximum (|value| * 2^-e < 1)
__device__ __forceinline__ int oz_exp(float rowmax) {
  int e = 0;
  if (rowmax > 0.f) frexpf(rowmax, &e);
  return e;
}

__global__ void __launch_bounds__(OZ_THREADS, 1)
    tc_ozaki_gemm_kernel(const __grid_constant__ CUtensorMap amap, const __grid_constant__ CUtensorMap bmap,
                         const __grid_constant__ TcFacTable tab, int Ne, int V3, int RA, int RB,
                         const float* __restrict__ amax, const float* __restrict__ bmax, TcScalars* __restrict__ sc,
                         cplx<double>* __restrict__ G) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + OZ_STAGES * OZ_STAGE_BYTES);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  volatile int* status = &sc->status;

  const int tile = blockIdx.x;
  int jb = 0;
  while (jb + 1 < tab.njobs && tile >= tab.j[jb + 1].tile0) ++jb;
  const TcFacJob& J = tab.j[jb];
  const int local = tile - J.tile0;
  const int mtile = local / J.nt;
  const int ntile = local - mtile * J.nt;
  const long long K = 3LL * V3;
  const int nks = (int)(K / OZ_KS);
  const int ay = J.arow0 + mtile * OZ_BM;
  const int by = J.brow0 + ntile * OZ_BN;

  if (threadIdx.x == 0) {
    for (int s = 0; s < OZ_STAGES; ++s) mbar_init(&full[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  auto issue = [&](int ks) {
    const int s = ks % OZ_STAGES;
    uint8_t* As = smem + s * OZ_STAGE_BYTES;
    uint8_t* Bs = As + OZ_A_BYTES;
    mbar_arrive_expect_tx(&full[s], OZ_STAGE_BYTES);
    for (int q = 0; q < OZ_AP; ++q) tma_load_2d(As + q * OZ_BM * OZ_KS, &amap, &full[s], ks * OZ_KS, q * RA + ay);
    for (int q = 0; q < OZ_BP; ++q) tma_load_2d(Bs + q * OZ_BN * OZ_KS, &bmap, &full[s], ks * OZ_KS, q * RB + by);
  };
  int issued_hi = -1;  // thread 0: highest k step whose copies were issued
  if (threadIdx.x == 0)
    for (int ks = 0; ks < OZ_STAGES && ks < nks; ++ks) {
      issue(ks);
      issued_hi = ks;
    }

  // warp tile: rows wm*16 .. +15, cols wn*32 .. +31 (four n8 fragments)
  const int wm = warp & 3, wn = warp >> 2;
  int acc[4][2][4][4];  // [weight][re/im][n fragment][mma register]
#pragma unroll
  for (int w = 0; w < 4; ++w)
#pragma unroll
    for (int p = 0; p < 2; ++p)
#pragma unroll
      for (int f = 0; f < 4; ++f)
#pragma unroll
        for (int r = 0; r < 4; ++r) acc[w][p][f][r] = 0;

  // ldmatrix row addresses: A (x4 over 16 rows x 2 chunks), B (x4 over two n8 fragments x 2 chunks)
  const int a_row = wm * 16 + (lane & 7) + ((lane >> 3) & 1) * 8, a_chunk = lane >> 4;
  const int b_row = wn * 32 + (lane & 7) + ((lane >> 4) & 1) * 8, b_chunk = (lane >> 3) & 1;
  const uint32_t a_off = oz_swz(a_row, a_chunk);
  const uint32_t b_off0 = oz_swz(b_row, b_chunk), b_off1 = oz_swz(b_row + 16, b_chunk);

  bool ok = true;
  for (int ks = 0; ks < nks; ++ks) {
    const int s = ks % OZ_STAGES;
    if (!warp_wait(&full[s], (ks / OZ_STAGES) & 1, status, TC_ERR_FULL)) {
      ok = false;
    }
    if (__syncthreads_or(!ok)) {
      ok = false;
      break;
    }
    const uint32_t As = smem_u32(smem + s * OZ_STAGE_BYTES);
    const uint32_t Bs = As + OZ_A_BYTES;
    // slice pairs (sl, t), sl + t <= 3; operands reloaded from shared memory per
    // pair to keep the 128 accumulators plus one A and one B slice in registers
#pragma unroll
    for (int sl = 0; sl < OZ_S; ++sl) {
      uint32_t a[2][4];  // [re, im]
#pragma unroll
      for (int p = 0; p < 2; ++p)
        ldsm_x4(As + (sl * 2 + p) * OZ_BM * OZ_KS + a_off, a[p][0], a[p][1], a[p][2], a[p][3]);
#pragma unroll
      for (int t = 0; sl + t < OZ_S; ++t) {
        const int w = sl + t;
        uint32_t b[3][4][2];  // [re, im, -im][n fragment][reg]
#pragma unroll
        for (int p = 0; p < 3; ++p) {
          const uint32_t pb = Bs + (t * 3 + p) * OZ_BN * OZ_KS;
          ldsm_x4(pb + b_off0, b[p][0][0], b[p][0][1], b[p][1][0], b[p][1][1]);
          ldsm_x4(pb + b_off1, b[p][2][0], b[p][2][1], b[p][3][0], b[p][3][1]);
        }
#pragma unroll
        for (int f = 0; f < 4; ++f) {
          imma(acc[w][0][f], a[0], b[0][f][0], b[0][f][1]);  // ar br
          imma(acc[w][0][f], a[1], b[2][f][0], b[2][f][1]);  // ai (-bi)
          imma(acc[w][1][f], a[0], b[1][f][0], b[1][f][1]);  // ar bi
          imma(acc[w][1][f], a[1], b[0][f][0], b[0][f][1]);  // ai br
        }
      }
    }
    __syncthreads();  // every warp is done with stage s
    if (threadIdx.x == 0 && ks + OZ_STAGES < nks) {
      issue(ks + OZ_STAGES);
      issued_hi = ks + OZ_STAGES;
    }
  }
  if (!ok) {
    // wait (bounded, not aborting) until the copies of the last issued use of
    // every stage have landed, then leave without writing results
    if (threadIdx.x == 0)
      for (int ks = issued_hi; ks >= 0 && ks > issued_hi - OZ_STAGES; --ks)
        mbar_wait(&full[ks % OZ_STAGES], (ks / OZ_STAGES) & 1, status, TC_ERR_FULL, false);
    __syncthreads();
    return;
  }

  // ---- epilogue: exact int32 sums -> FP64, scaled by the row exponents, into G
  const int Mrows = J.nright * tab.pz * Ne;
  const int Ncols = tab.pxy * Ne;
  const int N = J.nright * Ne;
  const int per_r = tab.pz * Ne;
  const int g = lane >> 2, t4 = lane & 3;
#pragma unroll
  for (int half = 0; half < 2; ++half) {  // mma rows g and g + 8
    const int m_local = mtile * OZ_BM + wm * 16 + g + half * 8;
    if (m_local >= Mrows) continue;
    const int r_local = m_local / per_r;
    const int rem = m_local - r_local * per_r;
    const int c = rem / Ne;
    const int j = rem - c * Ne;
    const int ea = oz_exp(amax[J.arow0 + m_local]);
#pragma unroll
    for (int f = 0; f < 4; ++f)
#pragma unroll
      for (int col = 0; col < 2; ++col) {
        const int n = ntile * OZ_BN + wn * 32 + f * 8 + t4 * 2 + col;
        if (n >= Ncols) continue;
        const int a = n / Ne, i = n - (n / Ne) * Ne;
        const int p = tab.pidx[a * tab.pz + c];
        if (p < 0) continue;
        const int reg = half * 2 + col;
        double re = 0.0, im = 0.0;
#pragma unroll
        for (int w = 0; w < 4; ++w) {
          const double sw = ldexp(1.0, -6 * (w + 2));
          re += sw * (double)acc[w][0][f][reg];
          im += sw * (double)acc[w][1][f][reg];
        }
        const double s = ldexp(1.0, ea + oz_exp(bmax[J.brow0 + n]));
        G[J.g_off + ((long long)p * Ne + i) * N + (long long)r_local * Ne + j] = mk(re * s, im * s);
      }
  }
}
