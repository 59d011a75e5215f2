// Factorised-phase pair contraction on SM pairs (included by elemental_tc.cu).
//
// The same GEMM as tc_fac_gemm.cuh (A = right variants g_c Y_j, B = left
// variants conj(X_i) f_a, hi/lo split planes in HBM, per-k-block TMEM
// buffers summed into FP32 registers, double-float results flushed once per
// lock step) with tiles of 256 A rows x 128 B rows computed by a cluster of
// two CTAs on two SMs through tcgen05.mma.cta_group::2 (M = 256):
//   * CTA rank r of the pair holds A rows [128 r, 128 r + 128) of the tile
//     and B rows [N/2 r, N/2 r + N/2) in its shared memory; one MMA reads
//     both CTAs' operands, so each SM takes in 32 KB of A and 16 KB of B per
//     k-block (48 KB instead of the 64 KB of the single-SM tile), and its
//     shared memory serves 6 KB per M=256 K=16 MMA half instead of 8 KB;
//   * each CTA's TMEM holds the accumulators of its own 128 rows (two
//     buffers of [re | im] x 128 columns, as in the single-SM kernel) and its
//     drain warps sum and flush its own rows;
//   * the leader CTA (rank 0) issues the MMAs; both CTAs' TMA loads signal the
//     leader's stage barrier (cp.async.bulk.tensor .cta_group::2 with the
//     leader's barrier address from mapa), whose expected byte count covers
//     both halves; the MMA completions are committed to both CTAs' barriers
//     (multicast mask 0b11); the drain warps of both CTAs arrive on the
//     leader's buffer-empty barrier (remote mbarrier.arrive, release.cluster).
// TMEM is allocated and released with .cta_group::2 by one warp of each CTA.
// Every wait is bounded (TC_WAIT_CYCLES) and reports through the status word;
// a CTA leaves only after its copies in flight have landed, the MMAs that
// read its shared memory or write its TMEM have completed, and the pair has
// met at the closing cluster barrier.

constexpr int TCP_BM = 2 * TC_BM;                   // A rows per pair tile
constexpr int TCP_A_BYTES = 4 * TC_BM * TC_ROWB;    // per CTA: 4 planes x 128 rows x 64 B = 32 KB
constexpr int TCP_B_BYTES = 4 * (TC_BN / 2) * TC_ROWB;  // per CTA: 4 planes x 64 rows x 64 B = 16 KB
constexpr int TCP_STAGE_BYTES = TCP_A_BYTES + TCP_B_BYTES;  // 48 KB
constexpr int TCP_MAX_STAGES = 4, TCP_DEFAULT_STAGES = 3;
__host__ __device__ constexpr int tcp_smem(int nst) { return nst * TCP_STAGE_BYTES + 1024 + 256; }
static_assert(tcp_smem(TCP_MAX_STAGES) <= 232448, "shared memory per block");

__device__ __forceinline__ uint32_t cluster_nctarank() {
  uint32_t n;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(n));
  return n;
}
__device__ __forceinline__ uint32_t cluster_ctarank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
// shared::cluster address of the same shared-memory location in CTA `rank` of the cluster
__device__ __forceinline__ uint32_t mapa_shared(uint32_t saddr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(saddr), "r"(rank));
  return r;
}
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// arrive on an mbarrier of another CTA of the cluster (shared::cluster address)
__device__ __forceinline__ void mbar_arrive_remote(uint32_t cluster_addr) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(cluster_addr) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait_cluster(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait with cluster-scope acquire (barriers that the peer CTA arrives on)
__device__ __forceinline__ bool mbar_wait_cluster(uint64_t* bar, uint32_t parity, volatile int* status, int code,
                                                  bool abort_on_error = true) {
  if (mbar_try_wait_cluster(bar, parity)) return true;
  const long long t0 = clock64();
  for (uint32_t it = 1;; ++it) {
    if (mbar_try_wait_cluster(bar, parity)) return true;
    if ((it & 255u) == 0) {
      if (abort_on_error && *status != 0) return false;
      if (clock64() - t0 > TC_WAIT_CYCLES) {
        atomicCAS((int*)status, 0, code);
        return false;
      }
    }
  }
}
// TMA load of this CTA's operand half, completing bytes on the leader CTA's barrier
__device__ __forceinline__ void tma_load_3d_pair(void* dst, const CUtensorMap* map, uint32_t bar_cluster, int x,
                                                 int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, "
      "%5}], [%2];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(bar_cluster), "r"(x), "r"(y), "r"(z)
      : "memory");
}
template <int KIND>
__device__ __forceinline__ void umma2(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  if constexpr (KIND == TC_TF32) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::2.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
  } else {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
  }
}
// commit the MMAs issued so far to the barrier at the same offset in both CTAs of the pair
__device__ __forceinline__ void umma2_commit_both(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(
          smem_u32(bar)),
      "h"((uint16_t)0x3)
      : "memory");
}

template <int KIND>
__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_fac2_gemm_kernel(const __grid_constant__ CUtensorMap amap, const __grid_constant__ CUtensorMap bmap,
                        const __grid_constant__ CUtensorMap bmap16, const __grid_constant__ TcFacTable tab, int Ne,
                        int V3, TcScalars* __restrict__ sc, float4* __restrict__ DF, int ntiles, int slab_kb,
                        int nst, int kpb) {
  constexpr int ESZ = Split<KIND>::ESZ;
  constexpr int KE = TC_ROWB / ESZ;
  constexpr int KINST = 32 / ESZ;
  constexpr uint32_t FMT = KIND == TC_F16 ? 0u : (KIND == TC_BF16 ? 1u : 2u);
  // M = 256 (cta_group::2), N set per tile below
  constexpr uint32_t IDESC = (umma_idesc(FMT, false) & ~(0x1Fu << 24)) | ((uint32_t)(TCP_BM >> 4) << 24);
  constexpr uint32_t IDESC_NEG = (umma_idesc(FMT, true) & ~(0x1Fu << 24)) | ((uint32_t)(TCP_BM >> 4) << 24);

  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + nst * TCP_STAGE_BYTES);
  uint64_t* empty = full + TCP_MAX_STAGES;
  uint64_t* accf = empty + TCP_MAX_STAGES;  // 2: accumulator buffer ready to drain (both CTAs)
  uint64_t* acce = accf + 2;                // 2: accumulator buffer drained (leader; arrivals from both CTAs)
  uint64_t* mma_done = acce + 2;            // every issued MMA has completed (both CTAs)
  uint32_t* tmem_slot = (uint32_t*)(mma_done + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // every CTA must sit in a two-CTA cluster: the pair's MMAs, multicast commits and remote arrivals address the
  // peer CTA.  A launch without that cluster shape (for instance by a tool that replays the kernel) stops here,
  // before any barrier, TMEM allocation or cluster access, and reports TC_ERR_CLUSTER.
  if (cluster_nctarank() != 2 || (gridDim.x & 1u) != 0u) {
    if (threadIdx.x == 0) atomicCAS(&sc->status, 0, TC_ERR_CLUSTER);
    return;
  }
  const uint32_t rank = cluster_ctarank();
  const bool leader = rank == 0;
  volatile int* status = &sc->status;
  unsigned int* progress = &sc->progress;

  const int G = gridDim.x, cta = blockIdx.x;
  const int pair = cta >> 1, npairs = G >> 1;
  const int J = (ntiles + npairs - 1) / npairs;  // tiles per pair (steps per slab)
  const long long K = 3LL * V3;
  const int nkb = (int)(K / KE);
  const int NS = (nkb + slab_kb - 1) / slab_kb;
  const int nsteps = NS * J;
  auto step_tile = [&](int q) { return (q % J) * npairs + pair; };
  auto step_kb0 = [&](int q) { return (q / J) * slab_kb; };
  auto step_kb1 = [&](int q) { return min(nkb, (q / J + 1) * slab_kb); };
  const bool has_narrow = tab.nfull < ntiles;
  auto decode = [&](int tile, int& jb, int& mtile, int& ntile) {
    jb = 0;
    if (tile < tab.nfull) {
      while (jb + 1 < tab.njobs && tile >= tab.j[jb + 1].tile0) ++jb;
      const int local = tile - tab.j[jb].tile0;
      const int ntc = tab.j[jb].nt - (has_narrow ? 1 : 0);
      mtile = local / ntc;
      ntile = local - mtile * ntc;
    } else {
      const int t2 = tile - tab.nfull;
      while (jb + 1 < tab.njobs && t2 >= tab.j[jb + 1].tile0n) ++jb;
      mtile = t2 - tab.j[jb].tile0n;
      ntile = tab.j[jb].nt - 1;
    }
  };
  // MMA N of a tile: all TC_BN columns, or for the last column tile of a group its valid columns rounded up
  // to 32 (each CTA then holds N/2 rows of B, a multiple of the 16-row narrow box)
  const int Ncols = tab.pxy * Ne;
  auto tile_cols = [&](int ntile) { return min(TC_BN, (min(TC_BN, Ncols - ntile * TC_BN) + 31) & ~31); };

  if (threadIdx.x == 0) {
    for (int s = 0; s < nst; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], 2 * TC_DWARPS);
    }
    mbar_init(mma_done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(tmem_slot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  cluster_sync_all();  // barriers initialised and TMEM allocated in both CTAs before any cross-CTA use
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp < 8) {
    asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(TCF_REGS_LOW));
    if (warp == 0) {
      // ===================== TMA of this CTA's A and B halves, step by step
      if (lane == 0) {
        long long g = 0, issued_last = -1;
        bool ok = true;
        for (int q = 0; q < nsteps && ok; ++q) {
          atomicAdd(progress, 1u);
          if (q > 0) {
            const unsigned int need = (unsigned int)q * (unsigned int)G;
            const long long t0 = clock64();
            while (*(volatile unsigned int*)progress < need) {
              if (*status != 0 || clock64() - t0 > TC_WAIT_CYCLES) {
                atomicCAS((int*)status, 0, TC_ERR_SYNC);
                ok = false;
                break;
              }
            }
            if (!ok) break;
          }
          const int tile = step_tile(q);
          if (tile >= ntiles) continue;
          int jb, mtile, ntile;
          decode(tile, jb, mtile, ntile);
          const int ncol = tile_cols(ntile);
          const int ay = tab.j[jb].arow0 + mtile * TCP_BM + (int)rank * TC_BM;
          const int by = tab.j[jb].brow0 + ntile * TC_BN + (int)rank * (ncol / 2);
          const int kb1 = step_kb1(q);
          for (int kb = step_kb0(q); kb < kb1; ++kb, ++g) {
            const int s = (int)(g % nst);
            if (g >= nst && !mbar_wait(&empty[s], (uint32_t)(((g / nst) + 1) & 1), status, TC_ERR_EMPTY)) {
              ok = false;
              break;
            }
            uint8_t* As = smem + s * TCP_STAGE_BYTES;
            uint8_t* Bs = As + TCP_A_BYTES;
            const uint32_t fbar = mapa_shared(smem_u32(&full[s]), 0);  // the leader's stage barrier
            if (leader) mbar_arrive_expect_tx(&full[s], 2 * TCP_A_BYTES + 4 * ncol * TC_ROWB);
            for (int p = 0; p < 4; ++p) {
              tma_load_3d_pair(As + p * TC_BM * TC_ROWB, &amap, fbar, 0, ay, p * nkb + kb);
              if (ncol == TC_BN) {
                tma_load_3d_pair(Bs + p * (TC_BN / 2) * TC_ROWB, &bmap, fbar, 0, by, p * nkb + kb);
              } else {
                for (int r = 0; r < ncol / 2; r += 16)
                  tma_load_3d_pair(Bs + p * (TC_BN / 2) * TC_ROWB + r * TC_ROWB, &bmap16, fbar, 0, by + r,
                                   p * nkb + kb);
              }
            }
            issued_last = g;
          }
        }
        // do not leave while our copies may still land: the leader's stage barrier completes once both
        // halves of the last issued stage have landed; the empty barrier (committed to both CTAs after the
        // MMAs that read the stage) covers the peer
        if (issued_last >= 0) {
          const int s = (int)(issued_last % nst);
          if (leader)
            mbar_wait(&full[s], (uint32_t)((issued_last / nst) & 1), status, TC_ERR_FULL, false);
        }
      }
    } else if (warp == 1) {
      // ===================== MMA issuer (leader CTA only; same product order as the single-SM kernel)
      if (leader && lane == 0) {
        long long g = 0;   // stages consumed
        long long gb = 0;  // TMEM buffers filled (kpb k-blocks each, fewer at the end of a step)
        bool ok = true;
        for (int q = 0; q < nsteps && ok; ++q) {
          const int tile = step_tile(q);
          if (tile >= ntiles) continue;
          int jb, mtile, ntile;
          decode(tile, jb, mtile, ntile);
          const uint32_t nfield = (uint32_t)(tile_cols(ntile) >> 3) << 17;
          const uint32_t ID = (IDESC & ~(0x3Fu << 17)) | nfield, ID_NEG = (IDESC_NEG & ~(0x3Fu << 17)) | nfield;
          const int kb1 = step_kb1(q);
          const int kb0s = step_kb0(q);
          for (int kb = kb0s; kb < kb1; ++kb, ++g) {
            const int s = (int)(g % nst);
            const int b = (int)(gb & 1);
            const bool first = (kb - kb0s) % kpb == 0;  // the first k-block of a TMEM buffer
            const bool last = (kb - kb0s) % kpb == kpb - 1 || kb == kb1 - 1;
            if (!mbar_wait_cluster(&full[s], (uint32_t)((g / nst) & 1), status, TC_ERR_FULL) ||
                (first && gb >= 2 &&
                 !mbar_wait_cluster(&acce[b], (uint32_t)(((gb >> 1) + 1) & 1), status, TC_ERR_ACCE))) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t a0 = smem_u32(smem + s * TCP_STAGE_BYTES);
            const uint32_t b0 = a0 + TCP_A_BYTES;
            const uint32_t d_re = tmem + b * 256, d_im = d_re + TC_BN;
#pragma unroll
            for (int ks = 0; ks < KE / KINST; ++ks) {
              const uint32_t acc = (ks > 0 || !first) ? 1u : 0u;
              const uint32_t ao = a0 + ks * 32, bo = b0 + ks * 32;
              const uint64_t A0 = umma_desc_sw64(ao), A1 = umma_desc_sw64(ao + TC_BM * TC_ROWB);
              const uint64_t A2 = umma_desc_sw64(ao + 2 * TC_BM * TC_ROWB),
                             A3 = umma_desc_sw64(ao + 3 * TC_BM * TC_ROWB);
              const uint64_t B0 = umma_desc_sw64(bo), B1 = umma_desc_sw64(bo + (TC_BN / 2) * TC_ROWB);
              const uint64_t B2 = umma_desc_sw64(bo + 2 * (TC_BN / 2) * TC_ROWB),
                             B3 = umma_desc_sw64(bo + 3 * (TC_BN / 2) * TC_ROWB);
              umma2<KIND>(d_re, A0, B1, ID, acc);
              umma2<KIND>(d_re, A1, B0, ID, 1u);
              umma2<KIND>(d_re, A2, B3, ID_NEG, 1u);
              umma2<KIND>(d_re, A3, B2, ID_NEG, 1u);
              umma2<KIND>(d_im, A0, B3, ID, acc);
              umma2<KIND>(d_im, A1, B2, ID, 1u);
              umma2<KIND>(d_im, A2, B1, ID, 1u);
              umma2<KIND>(d_im, A3, B0, ID, 1u);
            }
#pragma unroll
            for (int ks = 0; ks < KE / KINST; ++ks) {
              const uint32_t ao = a0 + ks * 32, bo = b0 + ks * 32;
              const uint64_t A0 = umma_desc_sw64(ao), A2 = umma_desc_sw64(ao + 2 * TC_BM * TC_ROWB);
              const uint64_t B0 = umma_desc_sw64(bo), B2 = umma_desc_sw64(bo + 2 * (TC_BN / 2) * TC_ROWB);
              umma2<KIND>(d_re, A0, B0, ID, 1u);
              umma2<KIND>(d_re, A2, B2, ID_NEG, 1u);
              umma2<KIND>(d_im, A0, B2, ID, 1u);
              umma2<KIND>(d_im, A2, B0, ID, 1u);
            }
            umma2_commit_both(&empty[s]);  // frees the stage in both CTAs when these MMAs complete
            if (last) {
              umma2_commit_both(&accf[b]);  // both CTAs' halves of the buffer are ready to drain
              ++gb;
            }
          }
        }
        umma2_commit_both(mma_done);  // arrives in both CTAs once every MMA issued above has completed
      }
    }
  } else {
    asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(TCF_REGS_HIGH));
    // ===================== drain: TMEM -> FP32 register sums -> double-float results, this CTA's rows
    const int dw = warp - 8;
    const int quarter = warp & 3;
    const int half = dw >> 2;
    const int m = quarter * 32 + lane;
    const float inv = ldexpf(1.f, -2 * sc->scale_exp);
    const uint32_t acce_leader[2] = {mapa_shared(smem_u32(&acce[0]), 0), mapa_shared(smem_u32(&acce[1]), 0)};
    float sre[64], sim[64];
    bool ok = true;
    long long g = 0;
    for (int q = 0; q < nsteps && ok; ++q) {
      const int tile = step_tile(q);
      if (tile >= ntiles) continue;
      int jb, mtile, ntile;
      decode(tile, jb, mtile, ntile);
      const TcFacJob& Jb = tab.j[jb];
      const int m_local = mtile * TCP_BM + (int)rank * TC_BM + m;
      const int n0c = ntile * TC_BN + half * 64;
      const int Mrows = Jb.nright * tab.pz * Ne;
#pragma unroll
      for (int c = 0; c < 64; ++c) sre[c] = sim[c] = 0.f;
      const int kb1 = step_kb1(q);
      for (int kb = step_kb0(q); kb < kb1; kb += kpb, ++g) {  // one TMEM buffer of kpb k-blocks
        const int b = (int)(g & 1);
        if (!warp_wait(&accf[b], (uint32_t)((g >> 1) & 1), status, TC_ERR_ACC)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t tl = tmem + ((uint32_t)(quarter * 32) << 16) + b * 256 + half * 64;
        {
          uint32_t r0[32], r1[32];
          tmem_ld32(tl, r0);
          tmem_ld32(tl + 32, r1);
          tmem_wait_ld();
#pragma unroll
          for (int e = 0; e < 32; ++e) {
            sre[e] += __uint_as_float(r0[e]);
            sre[32 + e] += __uint_as_float(r1[e]);
          }
        }
        {
          uint32_t r0[32], r1[32];
          tmem_ld32(tl + TC_BN, r0);
          tmem_ld32(tl + TC_BN + 32, r1);
          tmem_wait_ld();
#pragma unroll
          for (int e = 0; e < 32; ++e) {
            sim[e] += __uint_as_float(r0[e]);
            sim[32 + e] += __uint_as_float(r1[e]);
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive_remote(acce_leader[b]);
      }
      if (ok) flush_sums_fac(sre, sim, DF, tab, Jb, Ne, n0c, m_local, Mrows, inv);
    }
    // every MMA the leader issued has completed before this CTA releases its TMEM and shared memory (the
    // leader's final commit reaches both CTAs; waited without aborting on the error flag)
    warp_wait(mma_done, 0, status, TC_ERR_ACC, false);
  }
  tc_fence_before();
  __syncthreads();
  cluster_sync_all();  // neither CTA releases TMEM or leaves while its peer may still use the pair's MMAs
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
  }
}

// ---------------------------------------------------------------------------
// Stacked-operand form on SM pairs (ED_TUNE_TC_PAIR = 3).
//
// The tile is the single-SM one (128 A rows x up to 128 B columns), computed
// by a two-CTA cluster with the complex halves of both operands spread over the
// pair: CTA rank r holds the rows of plane r of the tile (r = 0: Ar, Br;
// r = 1: Ai, Bi), hi and lo parts, so one M = 256 (cta_group::2),
// N = 2 * ncol MMA computes [Ar; Ai] [Br | Bi] with
//   TMEM of rank 0: [Ar Br | Ar Bi]   (re +=, im +=)
//   TMEM of rank 1: [Ai Br | Ai Bi]   (im +=, re -=)
// Each CTA's accumulator is 256 columns wide, so both CTAs keep two TMEM
// buffers and the MMAs of a group never wait for the drain of the previous
// one (the single-SM stacked form needs both 256-column accumulators for one
// group and hands them over at every group boundary).  Per SM and k-block:
// 32 KB of operands for six 128 x 256 x 16 MMA halves (the single-SM stacked
// form: 64 KB for twelve), the same bytes per MMA.  Every accumulator column
// takes 6 accumulating MMAs per k-block, as in the single-SM stacked form.
// Each CTA flushes its own FP32 sums into its own double-float plane
// (DF + rank * df_plane); the two planes are added when they are converted to
// complex128.  Barriers, TMEM allocation and the exit protocol are those of
// tc_fac2_gemm_kernel.
constexpr int TCS_A_BYTES = 2 * TC_BM * TC_ROWB;          // per CTA: hi, lo x 128 rows x 64 B = 16 KB
constexpr int TCS_B_BYTES = 2 * TC_BN * TC_ROWB;          // per CTA: hi, lo x up to 128 rows = 16 KB
constexpr int TCS_STAGE_BYTES = TCS_A_BYTES + TCS_B_BYTES;  // 32 KB
constexpr int TCS_MAX_STAGES = 4, TCS_DEFAULT_STAGES = 4;
__host__ __device__ constexpr int tcs_smem(int nst) { return nst * TCS_STAGE_BYTES + 1024 + 256; }
static_assert(tcs_smem(TCS_MAX_STAGES) <= 232448, "shared memory per block");

template <int KIND>
__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_fac2s_gemm_kernel(const __grid_constant__ CUtensorMap amap, const __grid_constant__ CUtensorMap bmap,
                         const __grid_constant__ CUtensorMap bmap16, const __grid_constant__ TcFacTable tab, int Ne,
                         int V3, TcScalars* __restrict__ sc, float4* __restrict__ DF, long long df_plane, int ntiles,
                         int slab_kb, int nst, int kpb) {
  constexpr int ESZ = Split<KIND>::ESZ;
  constexpr int KE = TC_ROWB / ESZ;
  constexpr int KINST = 32 / ESZ;
  constexpr uint32_t FMT = KIND == TC_F16 ? 0u : (KIND == TC_BF16 ? 1u : 2u);
  // M = 256 (cta_group::2), N set per tile below
  constexpr uint32_t IDESC = (umma_idesc(FMT, false) & ~(0x1Fu << 24)) | ((uint32_t)(TCP_BM >> 4) << 24);

  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + nst * TCS_STAGE_BYTES);
  uint64_t* empty = full + TCS_MAX_STAGES;
  uint64_t* accf = empty + TCS_MAX_STAGES;  // 2: accumulator buffer ready to drain (both CTAs)
  uint64_t* acce = accf + 2;                // 2: accumulator buffer drained (leader; arrivals from both CTAs)
  uint64_t* mma_done = acce + 2;            // every issued MMA has completed (both CTAs)
  uint32_t* tmem_slot = (uint32_t*)(mma_done + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // every CTA must sit in a two-CTA cluster: the pair's MMAs, multicast commits and remote arrivals address the
  // peer CTA.  A launch without that cluster shape (for instance by a tool that replays the kernel) stops here,
  // before any barrier, TMEM allocation or cluster access, and reports TC_ERR_CLUSTER.
  if (cluster_nctarank() != 2 || (gridDim.x & 1u) != 0u) {
    if (threadIdx.x == 0) atomicCAS(&sc->status, 0, TC_ERR_CLUSTER);
    return;
  }
  const uint32_t rank = cluster_ctarank();
  const bool leader = rank == 0;
  volatile int* status = &sc->status;
  unsigned int* progress = &sc->progress;

  const int G = gridDim.x, cta = blockIdx.x;
  const int pair = cta >> 1, npairs = G >> 1;
  const int J = (ntiles + npairs - 1) / npairs;  // tiles per pair (steps per slab)
  const long long K = 3LL * V3;
  const int nkb = (int)(K / KE);
  const int NS = (nkb + slab_kb - 1) / slab_kb;
  const int nsteps = NS * J;
  auto step_tile = [&](int q) { return (q % J) * npairs + pair; };
  auto step_kb0 = [&](int q) { return (q / J) * slab_kb; };
  auto step_kb1 = [&](int q) { return min(nkb, (q / J + 1) * slab_kb); };
  const bool has_narrow = tab.nfull < ntiles;
  auto decode = [&](int tile, int& jb, int& mtile, int& ntile) {
    jb = 0;
    if (tile < tab.nfull) {
      while (jb + 1 < tab.njobs && tile >= tab.j[jb + 1].tile0) ++jb;
      const int local = tile - tab.j[jb].tile0;
      const int ntc = tab.j[jb].nt - (has_narrow ? 1 : 0);
      mtile = local / ntc;
      ntile = local - mtile * ntc;
    } else {
      const int t2 = tile - tab.nfull;
      while (jb + 1 < tab.njobs && t2 >= tab.j[jb + 1].tile0n) ++jb;
      mtile = t2 - tab.j[jb].tile0n;
      ntile = tab.j[jb].nt - 1;
    }
  };
  // B rows per CTA of a tile: all TC_BN, or for the last column tile of a group its valid columns rounded up
  // to 16 (16-row B boxes); the MMA's N is twice that
  const int Ncols = tab.pxy * Ne;
  auto tile_cols = [&](int ntile) { return min(TC_BN, (min(TC_BN, Ncols - ntile * TC_BN) + 15) & ~15); };

  if (threadIdx.x == 0) {
    for (int s = 0; s < nst; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], 2 * TC_DWARPS);
    }
    mbar_init(mma_done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(tmem_slot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  cluster_sync_all();  // barriers initialised and TMEM allocated in both CTAs before any cross-CTA use
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp < 8) {
    asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(TCF_STACK_REGS_LOW));
    if (warp == 0) {
      // ===================== TMA of this CTA's plane (hi, lo) of the tile's A and B rows, step by step
      if (lane == 0) {
        long long g = 0, issued_last = -1;
        bool ok = true;
        const int p_hi = 2 * (int)rank, p_lo = p_hi + 1;  // planes re_hi, re_lo (rank 0) / im_hi, im_lo (rank 1)
        for (int q = 0; q < nsteps && ok; ++q) {
          atomicAdd(progress, 1u);
          if (q > 0) {
            const unsigned int need = (unsigned int)q * (unsigned int)G;
            const long long t0 = clock64();
            while (*(volatile unsigned int*)progress < need) {
              if (*status != 0 || clock64() - t0 > TC_WAIT_CYCLES) {
                atomicCAS((int*)status, 0, TC_ERR_SYNC);
                ok = false;
                break;
              }
            }
            if (!ok) break;
          }
          const int tile = step_tile(q);
          if (tile >= ntiles) continue;
          int jb, mtile, ntile;
          decode(tile, jb, mtile, ntile);
          const int ncol = tile_cols(ntile);
          const int ay = tab.j[jb].arow0 + mtile * TC_BM;
          const int by = tab.j[jb].brow0 + ntile * TC_BN;
          const int kb1 = step_kb1(q);
          for (int kb = step_kb0(q); kb < kb1; ++kb, ++g) {
            const int s = (int)(g % nst);
            if (g >= nst && !mbar_wait(&empty[s], (uint32_t)(((g / nst) + 1) & 1), status, TC_ERR_EMPTY)) {
              ok = false;
              break;
            }
            uint8_t* As = smem + s * TCS_STAGE_BYTES;
            uint8_t* Bs = As + TCS_A_BYTES;
            const uint32_t fbar = mapa_shared(smem_u32(&full[s]), 0);  // the leader's stage barrier
            if (leader) mbar_arrive_expect_tx(&full[s], 2 * (TCS_A_BYTES + 2 * ncol * TC_ROWB));
            tma_load_3d_pair(As, &amap, fbar, 0, ay, p_hi * nkb + kb);
            tma_load_3d_pair(As + TC_BM * TC_ROWB, &amap, fbar, 0, ay, p_lo * nkb + kb);
            if (ncol == TC_BN) {
              tma_load_3d_pair(Bs, &bmap, fbar, 0, by, p_hi * nkb + kb);
              tma_load_3d_pair(Bs + TC_BN * TC_ROWB, &bmap, fbar, 0, by, p_lo * nkb + kb);
            } else {
              for (int r = 0; r < ncol; r += 16) {
                tma_load_3d_pair(Bs + r * TC_ROWB, &bmap16, fbar, 0, by + r, p_hi * nkb + kb);
                tma_load_3d_pair(Bs + (TC_BN + r) * TC_ROWB, &bmap16, fbar, 0, by + r, p_lo * nkb + kb);
              }
            }
            issued_last = g;
          }
        }
        // do not leave while our copies may still land (as in tc_fac2_gemm_kernel)
        if (issued_last >= 0) {
          const int s = (int)(issued_last % nst);
          if (leader)
            mbar_wait(&full[s], (uint32_t)((issued_last / nst) & 1), status, TC_ERR_FULL, false);
        }
      }
    } else if (warp == 1) {
      // ===================== MMA issuer (leader CTA only): correction products first, then hi x hi
      if (leader && lane == 0) {
        long long g = 0;   // stages consumed
        long long gb = 0;  // TMEM buffers filled (kpb k-blocks each, fewer at the end of a step)
        bool ok = true;
        for (int q = 0; q < nsteps && ok; ++q) {
          const int tile = step_tile(q);
          if (tile >= ntiles) continue;
          int jb, mtile, ntile;
          decode(tile, jb, mtile, ntile);
          const uint32_t nfield = (uint32_t)((2 * tile_cols(ntile)) >> 3) << 17;
          const uint32_t ID = (IDESC & ~(0x3Fu << 17)) | nfield;
          const int kb1 = step_kb1(q);
          const int kb0s = step_kb0(q);
          for (int kb = kb0s; kb < kb1; ++kb, ++g) {
            const int s = (int)(g % nst);
            const int b = (int)(gb & 1);
            const bool first = (kb - kb0s) % kpb == 0;  // the first k-block of a TMEM buffer
            const bool last = (kb - kb0s) % kpb == kpb - 1 || kb == kb1 - 1;
            if (!mbar_wait_cluster(&full[s], (uint32_t)((g / nst) & 1), status, TC_ERR_FULL) ||
                (first && gb >= 2 &&
                 !mbar_wait_cluster(&acce[b], (uint32_t)(((gb >> 1) + 1) & 1), status, TC_ERR_ACCE))) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t a0 = smem_u32(smem + s * TCS_STAGE_BYTES);
            const uint32_t b0 = a0 + TCS_A_BYTES;
            const uint32_t d = tmem + b * 256;
#pragma unroll
            for (int ks = 0; ks < KE / KINST; ++ks) {
              const uint32_t acc = (ks > 0 || !first) ? 1u : 0u;
              const uint32_t ao = a0 + ks * 32, bo = b0 + ks * 32;
              umma2<KIND>(d, umma_desc_sw64(ao), umma_desc_sw64(bo + TC_BN * TC_ROWB), ID, acc);  // hi x lo
              umma2<KIND>(d, umma_desc_sw64(ao + TC_BM * TC_ROWB), umma_desc_sw64(bo), ID, 1u);  // lo x hi
            }
#pragma unroll
            for (int ks = 0; ks < KE / KINST; ++ks) {
              const uint32_t ao = a0 + ks * 32, bo = b0 + ks * 32;
              umma2<KIND>(d, umma_desc_sw64(ao), umma_desc_sw64(bo), ID, 1u);  // hi x hi
            }
            umma2_commit_both(&empty[s]);  // frees the stage in both CTAs when these MMAs complete
            if (last) {
              umma2_commit_both(&accf[b]);  // both CTAs' halves of the buffer are ready to drain
              ++gb;
            }
          }
        }
        umma2_commit_both(mma_done);  // arrives in both CTAs once every MMA issued above has completed
      }
    }
  } else {
    asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(TCF_STACK_REGS_HIGH));
    // ===================== drain: TMEM -> FP32 register sums -> this CTA's double-float plane
    const int dw = warp - 8;
    const int quarter = warp & 3;
    const int half = dw >> 2;
    const int m = quarter * 32 + lane;
    const float inv = ldexpf(1.f, -2 * sc->scale_exp);
    const uint32_t acce_leader[2] = {mapa_shared(smem_u32(&acce[0]), 0), mapa_shared(smem_u32(&acce[1]), 0)};
    float4* const DFr = DF + (long long)rank * df_plane;
    float s0[64], s1[64];
    bool ok = true;
    long long g = 0;
    for (int q = 0; q < nsteps && ok; ++q) {
      const int tile = step_tile(q);
      if (tile >= ntiles) continue;
      int jb, mtile, ntile;
      decode(tile, jb, mtile, ntile);
      const TcFacJob& Jb = tab.j[jb];
      const int ncol = tile_cols(ntile);
      const int m_local = mtile * TC_BM + m;
      const int n0c = ntile * TC_BN + half * 64;
      const int Mrows = Jb.nright * tab.pz * Ne;
#pragma unroll
      for (int c = 0; c < 64; ++c) s0[c] = s1[c] = 0.f;
      const int kb1 = step_kb1(q);
      for (int kb = step_kb0(q); kb < kb1; kb += kpb, ++g) {  // one TMEM buffer of kpb k-blocks
        const int b = (int)(g & 1);
        if (!warp_wait(&accf[b], (uint32_t)((g >> 1) & 1), status, TC_ERR_ACC)) {
          ok = false;
          break;
        }
        tc_fence_after();
        // columns [0, ncol) hold A_r Br, [ncol, 2 ncol) A_r Bi: s0 and s1 sum them for either rank
        const uint32_t tl = tmem + ((uint32_t)(quarter * 32) << 16) + b * 256 + half * 64;
        {
          uint32_t r0[32], r1[32];
          tmem_ld32(tl, r0);
          tmem_ld32(tl + 32, r1);
          tmem_wait_ld();
#pragma unroll
          for (int e = 0; e < 32; ++e) {
            s0[e] += __uint_as_float(r0[e]);
            s0[32 + e] += __uint_as_float(r1[e]);
          }
        }
        {
          uint32_t r0[32], r1[32];
          tmem_ld32(tl + ncol, r0);
          tmem_ld32(tl + ncol + 32, r1);
          tmem_wait_ld();
#pragma unroll
          for (int e = 0; e < 32; ++e) {
            s1[e] += __uint_as_float(r0[e]);
            s1[32 + e] += __uint_as_float(r1[e]);
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive_remote(acce_leader[b]);
      }
      // rank 0: re += Ar Br, im += Ar Bi; rank 1: re -= Ai Bi, im += Ai Br
      if (ok) flush_sums_fac(s0, s1, DFr, tab, Jb, Ne, n0c, m_local, Mrows, inv, rank != 0);
    }
    // every MMA the leader issued has completed before this CTA releases its TMEM and shared memory
    warp_wait(mma_done, 0, status, TC_ERR_ACC, false);
  }
  tc_fence_before();
  __syncthreads();
  cluster_sync_all();  // neither CTA releases TMEM or leaves while its peer may still use the pair's MMAs
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
  }
}
