// The tcgen05 pair-contraction kernel (included by elemental_tc.cu).
//
// Tile: 128 A rows (right-chain vectors m) x 128 B rows (n = (i, p)).
// Accumulation.  The tensor core adds each MMA's products into its FP32
// accumulator with truncation, which biases a long K reduction towards zero
// by ~0.5 ulp per accumulating MMA.  So no TMEM accumulator ever lives longer
// than one k-block (32 fp16 / 16 tf32 elements of K): the MMA warp writes
// each k-block into a fresh TMEM buffer (two buffers of 256 columns: real and
// imaginary 128 x 128 FP32 tiles) issuing the small hi.lo / lo.hi correction
// products first and the four dominant hi.hi products last, so only those
// four additions round at the partial's full magnitude.  Eight drain warps
// read every finished buffer (tcgen05.ld), add it into FP32 register sums
// (round-to-nearest) and hand the buffer back; every TC_FLUSH_KB k-blocks the register
// sums are added into a double-float (hi, lo FP32 pair) result in global
// memory with two-sum arithmetic (FP64 units are too slow on this part for a
// per-flush FP64 update), converted to complex128 after the kernel.
//
// Warp roles (512 threads, one CTA per SM):
//   warp 0      : TMA of the four A planes of each stage
//   warp 1      : TMEM owner, tcgen05.mma issue (one lane)
//   warps 2-7   : B producers: conj(X_i) * phase_p, split into hi/lo planes
//   warps 8-15  : drain (two warps per TMEM lane quarter, 64 columns each)
// Register split: warpgroups 0-1 drop to 80 registers, 2-3 rise to 176
// (256*80 + 256*176 = 512*128, the block's launch allocation).


// (hi, lo) += x in double-float arithmetic (Knuth two-sum, then renormalise):
// keeps ~46 significant bits with FP32 instructions only.
__device__ __forceinline__ void df_add(float& hi, float& lo, float x) {
  const float s = __fadd_rn(hi, x);
  const float bb = __fsub_rn(s, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(x, bb));
  const float l = __fadd_rn(lo, err);
  const float t = __fadd_rn(s, l);
  lo = __fsub_rn(l, __fsub_rn(t, s));
  hi = t;
}

// Add this thread's 64 register sums into the double-float result
// DF[elem] = (re_hi, re_lo, im_hi, im_lo) and clear them.  The
// read-modify-writes go in pairs (both loads before the stores).
__device__ __forceinline__ void flush_sums(float (&sre)[64], float (&sim)[64], float4* __restrict__ DF,
                                           long long gbase, int N, int n0c, int Ncols, int nmom, int Ne,
                                           long long m_local, int Mrows, float inv) {
  constexpr int G = 2;
  const bool row_ok = m_local < Mrows;
#pragma unroll
  for (int q0 = 0; q0 < 64; q0 += G) {
    long long off[G];
    float4 d[G];
#pragma unroll
    for (int u = 0; u < G; ++u) {
      const int n = n0c + q0 + u;
      off[u] = -1;
      if (row_ok && n < Ncols) {
        const int i = n / nmom, p = n - (n / nmom) * nmom;
        off[u] = gbase + ((long long)p * Ne + i) * N + m_local;
        d[u] = DF[off[u]];
      }
    }
#pragma unroll
    for (int u = 0; u < G; ++u) {
      if (off[u] >= 0) {
        df_add(d[u].x, d[u].y, sre[q0 + u] * inv);
        df_add(d[u].z, d[u].w, sim[q0 + u] * inv);
        DF[off[u]] = d[u];
      }
      sre[q0 + u] = 0.f;
      sim[q0 + u] = 0.f;
    }
  }
}

__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// STAGED: the left-chain rows and all phase rows of a k-block fit the staging
// area (xr + nmom rows); the TMA warp then copies them into shared memory and
// the producers read them there instead of from global memory.
// The body of one CTA: tile `tile` of the job table `tab` (the kernels below pass their tensor map and table
// from the launch's parameter space).
//
// STACK (the default form): the producers write the B planes of a stage as [re_hi; im_hi], [re_lo; im_lo]
// (256 rows each), so one M = 128, N = 256 MMA per split product computes A [Br | Bi]: acc1 = A_re [Br | Bi]
// and acc2 = A_im [Br | Bi] fill the 512 TMEM columns, single, and the drain forms re = acc1[:, :128] -
// acc2[:, 128:], im = acc1[:, 128:] + acc2[:, :128].  The MMAs of each k-block go accumulator by accumulator
// and accumulate `kpb` k-blocks per group (the drain reads acc1 while the acc2 MMAs run); the same scheme as
// the stacked form of tc_fac_gemm.cuh.  Without STACK: four real products into double-buffered [re], [im]
// buffers, one k-block each.
template <int KIND, bool STAGED, bool STACK>
__device__ __forceinline__ void tc_pair_gemm_body(const CUtensorMap* amap, const TcTable& tab, int Ne, int nmom,
                                                  int V3, long long R, const cplx<float>* __restrict__ chains,
                                                  const cplx<float>* __restrict__ phases, TcScalars* __restrict__ sc,
                                                  float4* __restrict__ DF, int xr, int tile, int kpb) {
  constexpr int ESZ = Split<KIND>::ESZ;
  constexpr int KE = TC_ROWB / ESZ;  // k elements per stage
  constexpr int EPC = 16 / ESZ;      // k elements per 16-byte chunk
  constexpr int CPR = TC_ROWB / 16;  // chunks per row (4)
  constexpr int KINST = 32 / ESZ;    // k elements per MMA instruction
  constexpr uint32_t FMT = KIND == TC_F16 ? 0u : (KIND == TC_BF16 ? 1u : 2u);
  constexpr uint32_t IDESC = umma_idesc(FMT, false);
  constexpr uint32_t IDESC_NEG = umma_idesc(FMT, true);

  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + TC_STAGES * TC_STAGE_BYTES);
  uint64_t* empty = full + TC_STAGES;
  uint64_t* accf = empty + TC_STAGES;  // 2: accumulator buffer ready to drain
  uint64_t* acce = accf + 2;           // 2: accumulator buffer drained
  uint64_t* mma_done = acce + 2;       // every issued MMA has completed
  uint64_t* xfull = mma_done + 1;      // TC_STAGES: staged left-chain/phase rows have landed
  uint64_t* xempty = xfull + TC_STAGES;  // TC_STAGES: the producers are done with a staging slot
  uint32_t* tmem_slot = (uint32_t*)(xempty + TC_STAGES);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  volatile int* status = &sc->status;

  // ---- decode the tile: group, n tile (fast), m tile
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
  const long long row0 = (long long)J.right0 * Ne + (long long)mtile * TC_BM;
  const int n0 = ntile * TC_BN;
  // staged rows: left-chain rows i_lo .. i_lo+nX-1, then all nmom phase rows (at row xr)
  constexpr int XROWB = KE * 8;                 // bytes of one complex64 row chunk
  constexpr int XSTRIDE = XROWB + TC_XP_PAD;    // padded row stride in shared memory
  const int i_lo = n0 / nmom;
  const int nX = min(Ne, (min(n0 + TC_BN, Ncols) - 1) / nmom + 1) - i_lo;

  if (threadIdx.x == 0) {
    for (int s = 0; s < TC_STAGES; ++s) {
      mbar_init(&full[s], 1 + TC_BWARPS);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], TC_DWARPS);
    }
    mbar_init(mma_done, 1);
    for (int st = 0; st < TC_STAGES; ++st) {
      mbar_init(&xfull[st], 1);
      mbar_init(&xempty[st], TC_BWARPS);
    }
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

  if (warp < 2 + TC_PWARPS) {
    // warpgroups 0-1: TMA, MMA and B producers give registers to the drain
    asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(TC_REGS_LOW));
  if (warp == 0) {
    // ===================== TMA producer of the A planes
    if (lane == 0) {
      int issued_last = -1;
      for (int kb = 0; kb < nkb; ++kb) {
        const int s = kb % TC_STAGES;
        if (kb >= TC_STAGES && !mbar_wait(&empty[s], ((kb / TC_STAGES) + 1) & 1, status, TC_ERR_EMPTY)) break;
        uint8_t* As = smem + s * TC_STAGE_BYTES;
        mbar_arrive_expect_tx(&full[s], TC_A_BYTES);
        for (int q = 0; q < 4; ++q)
          tma_load_2d(As + q * TC_BM * TC_ROWB, amap, &full[s], kb * KE, (int)(q * R + row0));
        issued_last = kb;
      }
      if (issued_last >= 0)  // do not leave while our copies may still land in shared memory
        mbar_wait(&full[issued_last % TC_STAGES], (issued_last / TC_STAGES) & 1, status, TC_ERR_FULL, false);
    }
  } else if (warp == 2) {
    // ===================== staging of the producers' input rows (left chain, phases):
    // one 1D bulk copy per row chunk, spread over the lanes.  A slot is reused
    // as soon as the producers have read it, independently of the MMA, so the
    // copies run up to TC_STAGES k-blocks ahead of the producers.
    if constexpr (STAGED) {
      int issued_last = -1;
      for (int kb = 0; kb < nkb; ++kb) {
        const int d = kb % TC_STAGES;
        if (kb >= TC_STAGES && !warp_wait(&xempty[d], ((kb / TC_STAGES) + 1) & 1, status, TC_ERR_EMPTY)) break;
        if (lane == 0) mbar_arrive_expect_tx(&xfull[d], (uint32_t)((nX + nmom) * XROWB));
        __syncwarp();
        uint8_t* XP = smem + d * TC_STAGE_BYTES + TC_A_BYTES + TC_B_BYTES;
        const long long k0 = (long long)kb * KE;
        const long long site0 = k0 % V3;
        const cplx<float>* Xrow = chains + ((long long)J.left * Ne + i_lo) * K + k0;
        for (int r = lane; r < nX + nmom; r += 32) {
          if (r < nX)
            bulk_copy_g2s(XP + r * XSTRIDE, Xrow + (long long)r * K, XROWB, &xfull[d]);
          else
            bulk_copy_g2s(XP + (xr + r - nX) * XSTRIDE, phases + (long long)(r - nX) * V3 + site0, XROWB,
                          &xfull[d]);
        }
        issued_last = kb;
      }
      if (issued_last >= 0)
        warp_wait(&xfull[issued_last % TC_STAGES], (issued_last / TC_STAGES) & 1, status, TC_ERR_XFULL, false);
    }
  } else if (warp == 1) {
    // ===================== MMA issuer
    if (lane == 0 && STACK) {
      constexpr uint32_t ID = (IDESC & ~(0x3Fu << 17)) | ((uint32_t)((2 * TC_BN) >> 3) << 17);  // N = 256
      bool ok = true;
      for (int kb = 0; kb < nkb && ok; ++kb) {
        const int s = kb % TC_STAGES;
        const int gb = kb / kpb;  // accumulator group
        const bool first = kb % kpb == 0, last = kb % kpb == kpb - 1 || kb == nkb - 1;
        if (!mbar_wait(&full[s], (kb / TC_STAGES) & 1, status, TC_ERR_FULL)) break;
        const uint32_t a0 = smem_u32(smem + s * TC_STAGE_BYTES);
        const uint32_t b0 = a0 + TC_A_BYTES;
#pragma unroll
        for (int h = 0; h < 2; ++h) {  // acc1 = Ar [Br | Bi], then acc2 = Ai [Br | Bi]
          if (first && gb >= 1 && !mbar_wait(&acce[h], (uint32_t)((gb - 1) & 1), status, TC_ERR_ACCE)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t d = tmem + h * 256;
#pragma unroll
          for (int ks = 0; ks < KE / KINST; ++ks) {  // correction products first
            const uint32_t acc = (ks > 0 || !first) ? 1u : 0u;
            const uint32_t ao = a0 + 2 * h * TC_BM * TC_ROWB + ks * 32, bo = b0 + ks * 32;
            umma<KIND>(d, umma_desc_sw64(ao), umma_desc_sw64(bo + 2 * TC_BN * TC_ROWB), ID, acc);
            umma<KIND>(d, umma_desc_sw64(ao + TC_BM * TC_ROWB), umma_desc_sw64(bo), ID, 1u);
          }
#pragma unroll
          for (int ks = 0; ks < KE / KINST; ++ks) {
            const uint32_t ao = a0 + 2 * h * TC_BM * TC_ROWB + ks * 32, bo = b0 + ks * 32;
            umma<KIND>(d, umma_desc_sw64(ao), umma_desc_sw64(bo), ID, 1u);
          }
          if (last) umma_commit(&accf[h]);  // this accumulator is ready to drain
        }
        if (!ok) break;
        umma_commit(&empty[s]);  // frees the stage when these MMAs complete
      }
      umma_commit(mma_done);  // arrives once every MMA issued above has completed (also on early exit)
    } else if (lane == 0) {
      int kb = 0;
      for (; kb < nkb; ++kb) {
        const int s = kb % TC_STAGES;
        const int b = kb & 1;
        if (!mbar_wait(&full[s], (kb / TC_STAGES) & 1, status, TC_ERR_FULL)) break;
        if (kb >= 2 && !mbar_wait(&acce[b], ((kb >> 1) + 1) & 1, status, TC_ERR_ACCE)) break;
        tc_fence_after();
        const uint32_t a0 = smem_u32(smem + s * TC_STAGE_BYTES);
        const uint32_t b0 = a0 + TC_A_BYTES;
        const uint32_t d_re = tmem + b * 256, d_im = d_re + TC_BN;
        uint64_t A[KE / KINST][4], B[KE / KINST][4];
#pragma unroll
        for (int ks = 0; ks < KE / KINST; ++ks)
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            A[ks][q] = umma_desc_sw64(a0 + q * TC_BM * TC_ROWB + ks * 32);
            B[ks][q] = umma_desc_sw64(b0 + q * TC_BN * TC_ROWB + ks * 32);
          }
        // small hi.lo / lo.hi products first (the first one starts the buffer afresh) ...
#pragma unroll
        for (int ks = 0; ks < KE / KINST; ++ks) {
          const uint32_t acc = ks > 0 ? 1u : 0u;
          umma<KIND>(d_re, A[ks][0], B[ks][1], IDESC, acc);
          umma<KIND>(d_re, A[ks][1], B[ks][0], IDESC, 1u);
          umma<KIND>(d_re, A[ks][2], B[ks][3], IDESC_NEG, 1u);
          umma<KIND>(d_re, A[ks][3], B[ks][2], IDESC_NEG, 1u);
          umma<KIND>(d_im, A[ks][0], B[ks][3], IDESC, acc);
          umma<KIND>(d_im, A[ks][1], B[ks][2], IDESC, 1u);
          umma<KIND>(d_im, A[ks][2], B[ks][1], IDESC, 1u);
          umma<KIND>(d_im, A[ks][3], B[ks][0], IDESC, 1u);
        }
        // ... then the dominant hi.hi products
#pragma unroll
        for (int ks = 0; ks < KE / KINST; ++ks) {
          umma<KIND>(d_re, A[ks][0], B[ks][0], IDESC, 1u);
          umma<KIND>(d_re, A[ks][2], B[ks][2], IDESC_NEG, 1u);
          umma<KIND>(d_im, A[ks][0], B[ks][2], IDESC, 1u);
          umma<KIND>(d_im, A[ks][2], B[ks][0], IDESC, 1u);
        }
        umma_commit(&empty[s]);  // frees the stage when these MMAs complete
        umma_commit(&accf[b]);   // the buffer is ready to drain
      }
      // arrives once every MMA issued above has completed (also on early exit)
      umma_commit(mma_done);
    }
  } else {
    // ===================== B producers
    // Each thread owns up to NT fixed (row, chunk) tasks; their row pointers
    // are resolved once per tile, so the K loop only adds offsets.
    constexpr int NT = (TC_BN * CPR + 32 * TC_BWARPS - 1) / (32 * TC_BWARPS);
    const int pt = threadIdx.x - 96;  // 0..159
    const float* Xb = reinterpret_cast<const float*>(chains + (long long)J.left * Ne * K);
    const float* Pb = reinterpret_cast<const float*>(phases);
    const float* xrow[NT];
    const float* prow[NT];
    uint32_t soff[NT];
    int tstate[NT];  // 0: no task, 1: zero row (beyond the tile), 2: data row
#pragma unroll
    for (int t = 0; t < NT; ++t) {
      const int task = pt + t * 32 * TC_BWARPS;
      const int row = task / CPR, c = task % CPR;
      const int n = n0 + row;
      tstate[t] = task >= TC_BN * CPR ? 0 : (n < Ncols ? 2 : 1);
      const int i = n < Ncols ? n / nmom : 0, p = n < Ncols ? n - (n / nmom) * nmom : 0;
      xrow[t] = Xb + 2 * ((long long)i * K + c * EPC);
      prow[t] = Pb + 2 * ((long long)p * V3 + c * EPC);
      soff[t] = row * TC_ROWB + ((c ^ ((row >> 1) & 3)) << 4);
    }
    // shared-memory offsets of each task's staged rows (chunk c of row i - i_lo and of phase row p)
    uint32_t xs_off[NT], ps_off[NT];
#pragma unroll
    for (int t = 0; t < NT; ++t) {
      const int task = pt + t * 32 * TC_BWARPS;
      const int row = task / CPR, c = task % CPR;
      const int n = min(n0 + row, Ncols - 1);
      const int i = n / nmom, p = n - i * nmom;
      xs_off[t] = (i - i_lo) * XSTRIDE + c * EPC * 8;
      ps_off[t] = (xr + p) * XSTRIDE + c * EPC * 8;
    }
    for (int kb = 0; kb < nkb; ++kb) {
      const int s = kb % TC_STAGES;
      if (STAGED && !warp_wait(&xfull[s], (kb / TC_STAGES) & 1, status, TC_ERR_XFULL)) break;
      if (kb >= TC_STAGES && !warp_wait(&empty[s], ((kb / TC_STAGES) + 1) & 1, status, TC_ERR_EMPTY)) break;
      uint8_t* Bs = smem + s * TC_STAGE_BYTES + TC_A_BYTES;
      const uint8_t* XP = Bs + TC_B_BYTES;
      const long long k0 = (long long)kb * KE;
      const int site0 = (int)(k0 % V3);
#pragma unroll
      for (int t = 0; t < NT; ++t) {
        if (tstate[t] == 0) continue;
        uint32_t hre[4], lre[4], him[4], lim[4];
        if (tstate[t] == 2) {
          const float* x = xrow[t] + 2 * k0;
          const float* ph = prow[t] + 2 * site0;
          float br[EPC], bi[EPC];
#pragma unroll
          for (int e = 0; e < EPC; e += 2) {
            float4 xv, pv;
            if constexpr (STAGED) {
              xv = *reinterpret_cast<const float4*>(XP + xs_off[t] + e * 8);
              pv = *reinterpret_cast<const float4*>(XP + ps_off[t] + e * 8);
            } else {
              xv = __ldg(reinterpret_cast<const float4*>(x + 2 * e));
              pv = __ldg(reinterpret_cast<const float4*>(ph + 2 * e));
            }
            br[e] = xv.x * pv.x + xv.y * pv.y;  // conj(x) * phase
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
        uint8_t* dst = Bs + soff[t];
        // planes re_hi, re_lo, im_hi, im_lo; stacked: re_hi, im_hi, re_lo, im_lo
        constexpr int PL = STACK ? 2 : 1, PI = STACK ? 1 : 2;
        *reinterpret_cast<uint4*>(dst + 0 * TC_BN * TC_ROWB) = make_uint4(hre[0], hre[1], hre[2], hre[3]);
        *reinterpret_cast<uint4*>(dst + PL * TC_BN * TC_ROWB) = make_uint4(lre[0], lre[1], lre[2], lre[3]);
        *reinterpret_cast<uint4*>(dst + PI * TC_BN * TC_ROWB) = make_uint4(him[0], him[1], him[2], him[3]);
        *reinterpret_cast<uint4*>(dst + 3 * TC_BN * TC_ROWB) = make_uint4(lim[0], lim[1], lim[2], lim[3]);
      }
      fence_proxy_async();
      __syncwarp();
      if (lane == 0) {
        mbar_arrive(&full[s]);
        if constexpr (STAGED) mbar_arrive(&xempty[s]);
      }
    }
  }
  } else {
    asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(TC_REGS_HIGH));
    // ===================== drain: TMEM -> FP32 register sums -> double-float result
    const int dw = warp - (2 + TC_PWARPS);  // 0..7
    const int quarter = warp & 3;           // TMEM lane quarter this warp may access
    const int half = dw >> 2;               // which 64 of the 128 columns
    const int m = quarter * 32 + lane;
    const long long m_local = (long long)mtile * TC_BM + m;
    const int N = J.nright * Ne;
    const int n0c = n0 + half * 64;
    const float inv = ldexpf(1.f, -2 * sc->scale_exp);
    float sre[64], sim[64];
#pragma unroll
    for (int c = 0; c < 64; ++c) sre[c] = sim[c] = 0.f;
    bool ok = true;
    if constexpr (STACK) {
      for (int kb0 = 0, g = 0; kb0 < nkb && ok; kb0 += kpb, ++g) {  // one group of kpb k-blocks
        const int kbl = min(nkb, kb0 + kpb) - 1;                      // its last k-block
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          if (!warp_wait(&accf[h], (uint32_t)(g & 1), status, TC_ERR_ACC)) {
            ok = false;
            break;
          }
          tc_fence_after();
          // acc1: re += [0, 128), im += [128, 256); acc2: im += [0, 128), re -= [128, 256)
          const uint32_t tl = tmem + ((uint32_t)(quarter * 32) << 16) + h * 256 + half * 64;
#pragma unroll
          for (int cc = 0; cc < 4; ++cc) {
            float v[16];
            tmem_ld16(tl + cc * 16, v);
            if (h == 0) {
#pragma unroll
              for (int e = 0; e < 16; ++e) sre[cc * 16 + e] += v[e];
            } else {
#pragma unroll
              for (int e = 0; e < 16; ++e) sim[cc * 16 + e] += v[e];
            }
            tmem_ld16(tl + TC_BN + cc * 16, v);
            if (h == 0) {
#pragma unroll
              for (int e = 0; e < 16; ++e) sim[cc * 16 + e] += v[e];
            } else {
#pragma unroll
              for (int e = 0; e < 16; ++e) sre[cc * 16 + e] -= v[e];
            }
          }
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&acce[h]);
        }
        if (ok && (kb0 / TC_FLUSH_KB != (kbl + 1) / TC_FLUSH_KB || kbl == nkb - 1))
          flush_sums(sre, sim, DF, J.g_off, N, n0c, Ncols, nmom, Ne, m_local, Mrows, inv);
      }
    }
    for (int kb = 0; kb < (STACK ? 0 : nkb); ++kb) {
      const int b = kb & 1;
      if (!warp_wait(&accf[b], (kb >> 1) & 1, status, TC_ERR_ACC)) {
        ok = false;
        break;
      }
      tc_fence_after();
      const uint32_t tl = tmem + ((uint32_t)(quarter * 32) << 16) + b * 256 + half * 64;
#pragma unroll
      for (int cc = 0; cc < 4; ++cc) {
        float v[16];
        tmem_ld16(tl + cc * 16, v);
#pragma unroll
        for (int e = 0; e < 16; ++e) sre[cc * 16 + e] += v[e];
        tmem_ld16(tl + TC_BN + cc * 16, v);
#pragma unroll
        for (int e = 0; e < 16; ++e) sim[cc * 16 + e] += v[e];
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&acce[b]);
      if ((kb & (TC_FLUSH_KB - 1)) == TC_FLUSH_KB - 1 || kb == nkb - 1)
        flush_sums(sre, sim, DF, J.g_off, N, n0c, Ncols, nmom, Ne, m_local, Mrows, inv);
    }
    if (!ok) {
      // wait (without aborting on the error flag) until every issued MMA is
      // done before the block releases TMEM
      warp_wait(mma_done, 0, status, TC_ERR_ACC, false);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
  }
}

template <int KIND, bool STAGED, bool STACK>
__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_pair_gemm_kernel(const __grid_constant__ CUtensorMap amap, const __grid_constant__ TcTable tab, int Ne,
                        int nmom, int V3, long long R, const cplx<float>* __restrict__ chains,
                        const cplx<float>* __restrict__ phases, TcScalars* __restrict__ sc, float4* __restrict__ DF,
                        int xr, int kpb) {
  tc_pair_gemm_body<KIND, STAGED, STACK>(&amap, tab, Ne, nmom, V3, R, chains, phases, sc, DF, xr, (int)blockIdx.x,
                                         kpb);
}

// Several lattice volumes (batched plans with their own Ne, V3, chains and results) in ONE launch: the tiles
// of volume v are blocks tile0[v] .. tile0[v+1]-1, so the small volumes' tiles share the waves of the large
// ones instead of running as launches of their own.
constexpr int kMaxVol = 4;
struct TcMultiVol {
  CUtensorMap amap;
  TcTable tab;
  const cplx<float>* chains;
  const cplx<float>* phases;
  TcScalars* sc;
  float4* DF;
  long long R;
  int Ne, nmom, V3, xr, tile0, kpb;
};
struct TcMulti {
  TcMultiVol v[kMaxVol];
  int nvol;
};

template <int KIND, bool STAGED, bool STACK>
__global__ void __launch_bounds__(TC_THREADS, 1) tc_pair_gemm_multi_kernel(const __grid_constant__ TcMulti M) {
  int v = 0;
  while (v + 1 < M.nvol && (int)blockIdx.x >= M.v[v + 1].tile0) ++v;
  const TcMultiVol& D = M.v[v];
  tc_pair_gemm_body<KIND, STAGED, STACK>(&D.amap, D.tab, D.Ne, D.nmom, D.V3, D.R, D.chains, D.phases, D.sc, D.DF,
                                         D.xr, (int)blockIdx.x - D.tile0, D.kpb);
}
