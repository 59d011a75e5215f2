// Factorised-phase pair contraction (included by elemental_tc.cu).
//
// When the momentum list is (close to) a product set {(px, py)} x {pz}, the
// phase factorises, phase_p(x, y, z) = f_a(x, y) * g_c(z) with a = (px, py)
// and c = pz, and
//   G_p(X, Y)[i, j] = sum_k (conj(X_i) f_a)[k] * (g_c Y_j)[k]
// becomes one plain complex GEMM between
//   B, the left variants  conj(X_i) f_a   (N side, rows n = a*Ne + i) and
//   A, the right variants g_c Y_j         (M side, rows m = (r*Pz + c)*Ne + j),
// covering all Pxy x Pz momenta of a chain pair at once.  Both operands are
// formed and split into hi/lo planes once per timeslice (tc_fac_split_kernel)
// and reach shared memory by TMA, so the K loop has no producer warps.  The
// accumulation scheme (per-k-block TMEM buffers, FP32 register sums,
// double-float flushes) is the one of tc_pair_gemm.cuh.
//
// Warp roles (512 threads, one CTA per SM):
//   warp 0      : TMA of the four A and the four B planes of each stage
//   warp 1      : TMEM owner, tcgen05.mma issue (one lane)
//   warps 2-7   : idle
//   warps 8-15  : drain (two warps per TMEM lane quarter, 64 + 64 columns each)
// Register split: warpgroups 0-1 drop to 56 registers and the drain
// warpgroups rise to 200 (256*56 + 256*200 = 512*128), enough to keep two
// 32-column TMEM loads in flight per wait.

// Operand stages of 64 KB in the shared-memory ring: 2 or 3, a launch setting (ED_TUNE_TC_STAGES).  Measured
// at 32^3, Ne = 200, 4 timeslices: 2 stages 144-146 ms, 3 stages 152 ms per launch.
constexpr int TCF_MAX_STAGES = 3, TCF_DEFAULT_STAGES = 2;
constexpr int TCF_STAGE_BYTES = TC_A_BYTES + TC_B_BYTES;  // 64 KB
// Forms of the kernel: four real products per complex one (FORM 0), stacked [re | im] B operand (FORM 1),
// Gauss three multiplications on re, im and re + im planes (FORM 2, six planes per operand: 96 KB stages).
constexpr int TCF_FOUR = 0, TCF_STACKED = 1, TCF_GAUSS = 2;
__host__ __device__ constexpr int tcf_planes(int form) { return form == TCF_GAUSS ? 6 : 4; }
__host__ __device__ constexpr int tcf_stage_bytes(int form) { return tcf_planes(form) * (TC_BM + TC_BN) * TC_ROWB; }
__host__ __device__ constexpr int tcf_max_stages(int form) { return form == TCF_GAUSS ? 2 : TCF_MAX_STAGES; }
__host__ __device__ constexpr int tcf_smem(int nst, int form = TCF_FOUR) {
  return nst * tcf_stage_bytes(form) + 1024 /*align*/ + 256 /*barriers*/;
}
static_assert(tcf_smem(TCF_MAX_STAGES) <= 232448, "shared memory per block");
static_assert(tcf_smem(tcf_max_stages(TCF_GAUSS), TCF_GAUSS) <= 232448, "shared memory per block");
constexpr int TCF_REGS_LOW = 56, TCF_REGS_HIGH = 200;
static_assert(256 * TCF_REGS_LOW + 256 * TCF_REGS_HIGH == TC_THREADS * TC_LAUNCH_REGS, "register split");
// the stacked form's drain holds the same sums but reads four 64-column slices per k-block group:
// 48 / 208 compiles without spills (56 / 200 spilled 176 bytes)
constexpr int TCF_STACK_REGS_LOW = 48, TCF_STACK_REGS_HIGH = 208;
static_assert(256 * TCF_STACK_REGS_LOW + 256 * TCF_STACK_REGS_HIGH == TC_THREADS * TC_LAUNCH_REGS, "register split");
constexpr int kMaxFac = 128;  // Pxy * Pz

struct TcFacJob {
  int arow0;   // first A row (right variants of the group's first right chain) within a plane
  int brow0;   // first B row (left variants of the group's left chain) within a plane
  int nright;  // right chains of the group
  int tile0, mt, nt;
  int tile0n;  // first of the group's narrow last-column tiles (numbered after every full tile)
  long long g_off;
};
struct TcFacTable {
  int njobs, pxy, pz;
  int nfull;  // tiles below nfull are full-width; the rest are the groups' narrow last-column tiles
  TcFacJob j[kMaxJobs];
  signed char pidx[kMaxFac];  // momentum index of (a, c) = pidx[a*pz + c], -1 if not requested
};

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Add the 64 register sums of one drain thread (row m, columns n0c..n0c+63)
// into the double-float results and clear them (with `swap`, sre holds the
// imaginary parts and -sim the real ones).  The read-modify-writes go
// in groups of 8: all loads of a group are issued before its stores, so a
// flush waits for 8 memory round trips instead of 64.
__device__ __forceinline__ void flush_sums_fac(float (&sre)[64], float (&sim)[64], float4* __restrict__ DF,
                                               const TcFacTable& tab, const TcFacJob& J, int Ne, int n0c,
                                               int m_local, int Mrows, float inv, bool swap = false) {
  constexpr int G = 8;
  const int Ncols = tab.pxy * Ne;
  const int N = J.nright * Ne;  // row length of G_p[i][.] within the group
  const bool row_ok = m_local < Mrows;
  const int per_r = tab.pz * Ne;
  const int r_local = m_local / per_r;
  const int rem = m_local - r_local * per_r;
  const int c = rem / Ne;
  const int j = rem - c * Ne;
  float4* const base = DF + J.g_off + (long long)r_local * Ne + j;
#pragma unroll
  for (int q0 = 0; q0 < 64; q0 += G) {
    long long off[G];
    float4 d[G];
#pragma unroll
    for (int u = 0; u < G; ++u) {
      const int n = n0c + q0 + u;
      off[u] = -1;
      if (row_ok && n < Ncols) {
        const int a = n / Ne, i = n - (n / Ne) * Ne;
        const int p = tab.pidx[a * tab.pz + c];
        if (p >= 0) off[u] = ((long long)p * Ne + i) * N;
      }
      if (off[u] >= 0) d[u] = base[off[u]];
    }
#pragma unroll
    for (int u = 0; u < G; ++u) {
      if (off[u] >= 0) {
        // swap: the sums hold (im, -re) (the second CTA of a pair in tc_fac2s_gemm_kernel)
        const float re = swap ? -sim[q0 + u] : sre[q0 + u], im = swap ? sre[q0 + u] : sim[q0 + u];
        df_add(d[u].x, d[u].y, re * inv);
        df_add(d[u].z, d[u].w, im * inv);
        base[off[u]] = d[u];
      }
      sre[q0 + u] = 0.f;
      sim[q0 + u] = 0.f;
    }
  }
}

// Persistent schedule.  The grid is one co-resident CTA per SM (cooperative
// launch).  The work is the list of steps (K slab s, tile): CTA c owns tiles
// c, c + G, c + 2G, ... and walks step q = s*J + j (tile j*G + c, the k-blocks
// of slab s).  At any moment the G CTAs work on the same K slab of G
// consecutive tiles, which share their A and B operand rows, so those rows
// come from HBM once and from L2 for the other CTAs; with every CTA running
// one tile over the whole K instead, the CTAs drift apart along K and the
// operand streams were re-read from HBM (736 GB per 4-timeslice launch at
// 32^3, Ne = 200).  To keep the CTAs in step, the TMA warp of each CTA counts
// every step it starts on a global counter and starts step q only when every
// CTA has started step q - 1 (a bounded wait).  The FP32 register sums are
// flushed into the double-float results at the end of every step, so a tile
// is only ever touched by its owner CTA.
//
// Stacked form (FORM = TCF_STACKED).  The B stage holds the real and imaginary
// planes of each precision part back to back, [Br_hi; Bi_hi] and
// [Br_lo; Bi_lo], so one M = 128, N = 2 * ncol MMA computes A * [Br | Bi].
// Two accumulators of 256 columns fill TMEM: acc1 = Ar [Br | Bi] and
// acc2 = Ai [Br | Bi], so Re = acc1[:, :ncol] - acc2[:, ncol:] and
// Im = acc1[:, ncol:] + acc2[:, :ncol], formed by the drain in FP32.  Half as
// many MMAs, each twice as wide (N = 256 ran at the full per-clock tensor rate
// in a probe of this part, N = 128 at 78 %), and no negated products; the
// operand bytes per k-block are unchanged.  Each accumulator is single: in
// every k-block the acc1 MMAs go first and the acc2 MMAs after them, so the
// drain reads acc1 while the acc2 MMAs run, and the MMAs of the next TMEM
// group into acc1 wait only for that read.  Every accumulator column takes
// 6 accumulating MMAs per k-block (12 in the 4-product form).
//
// Gauss form (FORM = TCF_GAUSS).  The split also writes the planes of
// re + im of both operands, so with X = Ar Br, Y = Ai Bi and
// Z = (Ar + Ai)(Br + Bi), three M = N = 128 accumulators (384 TMEM columns)
// give re = X - Y and im = Z - X - Y, formed by the drain in FP32: 9 MMAs per
// split product and K step instead of 12, for 96 KB of operands per k-block
// instead of 64.  As in the stacked form every accumulator is single and the
// MMAs of a k-block go accumulator by accumulator, so each one is drained
// while the next is computed.
template <int KIND, int FORM>
__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_fac_gemm_kernel(const __grid_constant__ CUtensorMap amap, const __grid_constant__ CUtensorMap bmap,
                       const __grid_constant__ CUtensorMap bmap16, const __grid_constant__ TcFacTable tab, int Ne,
                       int V3, TcScalars* __restrict__ sc,
                       float4* __restrict__ DF, int ntiles, int slab_kb, int nst, int kpb) {
  constexpr int ESZ = Split<KIND>::ESZ;
  constexpr int KE = TC_ROWB / ESZ;   // k elements per stage
  constexpr int KINST = 32 / ESZ;     // k elements per MMA instruction
  constexpr uint32_t FMT = KIND == TC_F16 ? 0u : (KIND == TC_BF16 ? 1u : 2u);
  constexpr uint32_t IDESC = umma_idesc(FMT, false);
  constexpr uint32_t IDESC_NEG = umma_idesc(FMT, true);
  constexpr bool STACK = FORM == TCF_STACKED, GAUSS = FORM == TCF_GAUSS;
  constexpr int NPL = tcf_planes(FORM);          // planes per operand
  constexpr int SB = tcf_stage_bytes(FORM);      // bytes per stage
  constexpr int AB = NPL * TC_BM * TC_ROWB;      // A bytes per stage
  constexpr int NACC = GAUSS ? 3 : 2;            // accumulators (buffers) in TMEM

  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + nst * SB);
  uint64_t* empty = full + TCF_MAX_STAGES;
  uint64_t* accf = empty + TCF_MAX_STAGES;  // 3: accumulator (buffer) ready to drain
  uint64_t* acce = accf + 3;            // 3: accumulator (buffer) drained
  uint64_t* mma_done = acce + 3;        // every issued MMA has completed
  uint32_t* tmem_slot = (uint32_t*)(mma_done + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  volatile int* status = &sc->status;
  unsigned int* progress = &sc->progress;  // zeroed with the scalars
  // the limit of every bounded wait of this run, and the test hook that makes the TMA role issue nothing (so the
  // first stage wait runs out whatever the copy latency): both set per run by tc_scale_kernel
  const long long wl = sc->wait_limit > 0 ? sc->wait_limit : TC_WAIT_CYCLES;
  const bool probe = sc->probe != 0;

  const int G = gridDim.x, cta = blockIdx.x;
  const int J = (ntiles + G - 1) / G;  // tiles per CTA (steps per slab)
  const long long K = 3LL * V3;
  const int nkb = (int)(K / KE);
  const int NS = (nkb + slab_kb - 1) / slab_kb;
  const int nsteps = NS * J;
  // tile of step q (>= ntiles: nothing to do) and its k-block range
  auto step_tile = [&](int q) { return (q % J) * G + cta; };
  auto step_kb0 = [&](int q) { return (q / J) * slab_kb; };
  auto step_kb1 = [&](int q) { return min(nkb, (q / J + 1) * slab_kb); };
  // Tile numbering: the full-width tiles of every group (column tile fastest), then, when the groups' last
  // column tile is narrow, those narrow tiles; grouped like this they share lock steps, which then run faster.
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
  // columns the MMAs of a tile cover: all TC_BN, or for the last column tile of a group its valid columns
  // rounded up to 16 (e.g. 16 for the 8 left over by 9 x 200 = 1800 = 14 x 128 + 8); its B rows then come in
  // 16-row boxes and the MMA runs with that N
  const int Ncols = tab.pxy * Ne;
  auto tile_cols = [&](int ntile) { return min(TC_BN, (min(TC_BN, Ncols - ntile * TC_BN) + 15) & ~15); };

  if (threadIdx.x == 0) {
    for (int s = 0; s < nst; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < NACC; ++b) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], TC_DWARPS);
    }
    mbar_init(mma_done, 1);
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

  if (warp < 8) {
    asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(FORM != TCF_FOUR ? TCF_STACK_REGS_LOW : TCF_REGS_LOW));
    if (warp == 0) {
      // ===================== TMA of the A and B planes, step by step
      if (lane == 0 && !probe) {
        long long g = 0, issued_last = -1;
        bool ok = true;
        for (int q = 0; q < nsteps && ok; ++q) {
          atomicAdd(progress, 1u);  // this CTA starts step q
          if (q > 0) {              // ... once every CTA has started step q - 1
            const unsigned int need = (unsigned int)q * (unsigned int)G;
            const long long t0 = clock64();
            while (*(volatile unsigned int*)progress < need) {
              if (*status != 0 || clock64() - t0 > wl) {
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
          const int ay = tab.j[jb].arow0 + mtile * TC_BM;
          const int by = tab.j[jb].brow0 + ntile * TC_BN;
          const int ncol = tile_cols(ntile);
          const int kb1 = step_kb1(q);
          for (int kb = step_kb0(q); kb < kb1; ++kb, ++g) {
            const int s = (int)(g % nst);
            if (g >= nst &&
                !mbar_wait(&empty[s], (uint32_t)(((g / nst) + 1) & 1), status, TC_ERR_EMPTY, true, wl)) {
              ok = false;
              break;
            }
            uint8_t* As = smem + s * SB;
            uint8_t* Bs = As + AB;
            mbar_arrive_expect_tx(&full[s], AB + NPL * ncol * TC_ROWB);
            for (int p = 0; p < NPL; ++p) {  // k-block-major planes: one contiguous 8 KB box each
              tma_load_3d(As + p * TC_BM * TC_ROWB, &amap, &full[s], 0, ay, p * nkb + kb);
              // planes re_hi, re_lo, im_hi, im_lo; stacked: [re_hi; im_hi] then [re_lo; im_lo], ncol rows each
              uint8_t* bd = STACK ? Bs + (p & 1) * 2 * TC_BN * TC_ROWB + (p >> 1) * ncol * TC_ROWB
                                  : Bs + p * TC_BN * TC_ROWB;
              if (ncol == TC_BN) {
                tma_load_3d(bd, &bmap, &full[s], 0, by, p * nkb + kb);
              } else {
                for (int r = 0; r < ncol; r += 16)
                  tma_load_3d(bd + r * TC_ROWB, &bmap16, &full[s], 0, by + r, p * nkb + kb);
              }
            }
            issued_last = g;
          }
        }
        if (issued_last >= 0)  // do not leave while our copies may still land in shared memory
          mbar_wait(&full[issued_last % nst], (uint32_t)((issued_last / nst) & 1), status,
                    TC_ERR_FULL, false, wl);
      }
    } else if (warp == 1) {
      // ===================== MMA issuer (same product order as tc_pair_gemm_kernel)
      if (lane == 0) {
        long long g = 0;   // stages consumed
        long long gb = 0;  // TMEM buffers filled (kpb k-blocks each, fewer at the end of a step)
        bool ok = true;
        for (int q = 0; q < nsteps && ok; ++q) {
          const int tile = step_tile(q);
          if (tile >= ntiles) continue;
          int jb, mtile, ntile;
          decode(tile, jb, mtile, ntile);
          const int ncol = tile_cols(ntile);
          const uint32_t nfield = (uint32_t)((STACK ? 2 * ncol : ncol) >> 3) << 17;  // the instruction's N
          const uint32_t ID = (IDESC & ~(0x3Fu << 17)) | nfield, ID_NEG = (IDESC_NEG & ~(0x3Fu << 17)) | nfield;
          const int kb1 = step_kb1(q);
          const int kb0s = step_kb0(q);
          if constexpr (STACK) {
            for (int kb = kb0s; kb < kb1 && ok; ++kb, ++g) {
              const int s = (int)(g % nst);
              const bool first = (kb - kb0s) % kpb == 0;
              const bool last = (kb - kb0s) % kpb == kpb - 1 || kb == kb1 - 1;
              if (!mbar_wait(&full[s], (uint32_t)((g / nst) & 1), status, TC_ERR_FULL, true, wl)) {
                ok = false;
                break;
              }
              const uint32_t a0 = smem_u32(smem + s * SB);
              const uint32_t b0 = a0 + AB;
#pragma unroll
              for (int h = 0; h < 2; ++h) {  // acc1 = Ar [Br | Bi], then acc2 = Ai [Br | Bi]
                if (first && gb >= 1 &&
                    !mbar_wait(&acce[h], (uint32_t)((gb - 1) & 1), status, TC_ERR_ACCE, true, wl)) {
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
              if (last) ++gb;
            }
            continue;
          }
          if constexpr (GAUSS) {
            for (int kb = kb0s; kb < kb1 && ok; ++kb, ++g) {
              const int s = (int)(g % nst);
              const bool first = (kb - kb0s) % kpb == 0;
              const bool last = (kb - kb0s) % kpb == kpb - 1 || kb == kb1 - 1;
              if (!mbar_wait(&full[s], (uint32_t)((g / nst) & 1), status, TC_ERR_FULL, true, wl)) {
                ok = false;
                break;
              }
              const uint32_t a0 = smem_u32(smem + s * SB);
              const uint32_t b0 = a0 + AB;
#pragma unroll
              for (int h = 0; h < 3; ++h) {  // X = Ar Br, Y = Ai Bi, Z = (Ar + Ai)(Br + Bi): planes 2h, 2h + 1
                if (first && gb >= 1 &&
                    !mbar_wait(&acce[h], (uint32_t)((gb - 1) & 1), status, TC_ERR_ACCE, true, wl)) {
                  ok = false;
                  break;
                }
                tc_fence_after();
                const uint32_t d = tmem + h * TC_BN;
#pragma unroll
                for (int ks = 0; ks < KE / KINST; ++ks) {  // correction products first
                  const uint32_t acc = (ks > 0 || !first) ? 1u : 0u;
                  const uint32_t ao = a0 + 2 * h * TC_BM * TC_ROWB + ks * 32, bo = b0 + 2 * h * TC_BN * TC_ROWB + ks * 32;
                  umma<KIND>(d, umma_desc_sw64(ao), umma_desc_sw64(bo + TC_BN * TC_ROWB), ID, acc);
                  umma<KIND>(d, umma_desc_sw64(ao + TC_BM * TC_ROWB), umma_desc_sw64(bo), ID, 1u);
                }
#pragma unroll
                for (int ks = 0; ks < KE / KINST; ++ks) {
                  const uint32_t ao = a0 + 2 * h * TC_BM * TC_ROWB + ks * 32, bo = b0 + 2 * h * TC_BN * TC_ROWB + ks * 32;
                  umma<KIND>(d, umma_desc_sw64(ao), umma_desc_sw64(bo), ID, 1u);
                }
                if (last) umma_commit(&accf[h]);  // this accumulator is ready to drain
              }
              if (!ok) break;
              umma_commit(&empty[s]);  // frees the stage when these MMAs complete
              if (last) ++gb;
            }
            continue;
          }
          for (int kb = kb0s; kb < kb1; ++kb, ++g) {
            const int s = (int)(g % nst);
            const int b = (int)(gb & 1);
            const bool first = (kb - kb0s) % kpb == 0;  // the first k-block of a TMEM buffer
            const bool last = (kb - kb0s) % kpb == kpb - 1 || kb == kb1 - 1;
            if (!mbar_wait(&full[s], (uint32_t)((g / nst) & 1), status, TC_ERR_FULL, true, wl) ||
                (first && gb >= 2 && !mbar_wait(&acce[b], (uint32_t)(((gb >> 1) + 1) & 1), status, TC_ERR_ACCE, true, wl))) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t a0 = smem_u32(smem + s * SB);
            const uint32_t b0 = a0 + AB;
            const uint32_t d_re = tmem + b * 256, d_im = d_re + TC_BN;
#pragma unroll
            for (int ks = 0; ks < KE / KINST; ++ks) {
              const uint32_t acc = (ks > 0 || !first) ? 1u : 0u;
              const uint32_t ao = a0 + ks * 32, bo = b0 + ks * 32;
              const uint64_t A0 = umma_desc_sw64(ao), A1 = umma_desc_sw64(ao + TC_BM * TC_ROWB);
              const uint64_t A2 = umma_desc_sw64(ao + 2 * TC_BM * TC_ROWB), A3 = umma_desc_sw64(ao + 3 * TC_BM * TC_ROWB);
              const uint64_t B0 = umma_desc_sw64(bo), B1 = umma_desc_sw64(bo + TC_BN * TC_ROWB);
              const uint64_t B2 = umma_desc_sw64(bo + 2 * TC_BN * TC_ROWB), B3 = umma_desc_sw64(bo + 3 * TC_BN * TC_ROWB);
              umma<KIND>(d_re, A0, B1, ID, acc);
              umma<KIND>(d_re, A1, B0, ID, 1u);
              umma<KIND>(d_re, A2, B3, ID_NEG, 1u);
              umma<KIND>(d_re, A3, B2, ID_NEG, 1u);
              umma<KIND>(d_im, A0, B3, ID, acc);
              umma<KIND>(d_im, A1, B2, ID, 1u);
              umma<KIND>(d_im, A2, B1, ID, 1u);
              umma<KIND>(d_im, A3, B0, ID, 1u);
            }
#pragma unroll
            for (int ks = 0; ks < KE / KINST; ++ks) {
              const uint32_t ao = a0 + ks * 32, bo = b0 + ks * 32;
              const uint64_t A0 = umma_desc_sw64(ao), A2 = umma_desc_sw64(ao + 2 * TC_BM * TC_ROWB);
              const uint64_t B0 = umma_desc_sw64(bo), B2 = umma_desc_sw64(bo + 2 * TC_BN * TC_ROWB);
              umma<KIND>(d_re, A0, B0, ID, 1u);
              umma<KIND>(d_re, A2, B2, ID_NEG, 1u);
              umma<KIND>(d_im, A0, B2, ID, 1u);
              umma<KIND>(d_im, A2, B0, ID, 1u);
            }
            umma_commit(&empty[s]);  // frees the stage when these MMAs complete
            if (last) {
              umma_commit(&accf[b]);  // the buffer is ready to drain
              ++gb;
            }
          }
        }
        umma_commit(mma_done);  // arrives once every MMA issued above has completed
      }
    }
  } else {
    asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(FORM != TCF_FOUR ? TCF_STACK_REGS_HIGH : TCF_REGS_HIGH));
    // ===================== drain: TMEM -> FP32 register sums -> double-float result per step
    const int dw = warp - 8;         // 0..7
    const int quarter = warp & 3;    // TMEM lane quarter this warp may access
    const int half = dw >> 2;        // which 64 of the 128 columns
    const int m = quarter * 32 + lane;
    const float inv = ldexpf(1.f, -2 * sc->scale_exp);
    float sre[64], sim[64];
    bool ok = true;
    long long g = 0;
    for (int q = 0; q < nsteps && ok; ++q) {
      const int tile = step_tile(q);
      if (tile >= ntiles) continue;
      int jb, mtile, ntile;
      decode(tile, jb, mtile, ntile);
      const TcFacJob& J = tab.j[jb];
      const int m_local = mtile * TC_BM + m;
      const int n0c = ntile * TC_BN + half * 64;
      const int Mrows = J.nright * tab.pz * Ne;
#pragma unroll
      for (int c = 0; c < 64; ++c) sre[c] = sim[c] = 0.f;
      const int kb1 = step_kb1(q);
      if constexpr (GAUSS) {
        for (int kb = step_kb0(q); kb < kb1; kb += kpb, ++g) {  // one group of kpb k-blocks
#pragma unroll
          for (int h = 0; h < 3; ++h) {  // X: re += x, im -= x; Y: re -= y, im -= y; Z: im += z
            if (!warp_wait(&accf[h], (uint32_t)(g & 1), status, TC_ERR_ACC, true, wl)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t tl = tmem + ((uint32_t)(quarter * 32) << 16) + h * TC_BN + half * 64;
            uint32_t r0[32], r1[32];
            tmem_ld32(tl, r0);
            tmem_ld32(tl + 32, r1);
            tmem_wait_ld();
            if (h == 0) {
#pragma unroll
              for (int e = 0; e < 32; ++e) {
                const float x0 = __uint_as_float(r0[e]), x1 = __uint_as_float(r1[e]);
                sre[e] += x0;
                sre[32 + e] += x1;
                sim[e] -= x0;
                sim[32 + e] -= x1;
              }
            } else if (h == 1) {
#pragma unroll
              for (int e = 0; e < 32; ++e) {
                const float y0 = __uint_as_float(r0[e]), y1 = __uint_as_float(r1[e]);
                sre[e] -= y0;
                sre[32 + e] -= y1;
                sim[e] -= y0;
                sim[32 + e] -= y1;
              }
            } else {
#pragma unroll
              for (int e = 0; e < 32; ++e) {
                sim[e] += __uint_as_float(r0[e]);
                sim[32 + e] += __uint_as_float(r1[e]);
              }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&acce[h]);
          }
          if (!ok) break;
        }
        if (ok) flush_sums_fac(sre, sim, DF, tab, J, Ne, n0c, m_local, Mrows, inv);
        continue;
      }
      if constexpr (STACK) {
        const int ncol = tile_cols(ntile);
        for (int kb = step_kb0(q); kb < kb1; kb += kpb, ++g) {  // one group of kpb k-blocks
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            if (!warp_wait(&accf[h], (uint32_t)(g & 1), status, TC_ERR_ACC, true, wl)) {
              ok = false;
              break;
            }
            tc_fence_after();
            // acc1: Re += [0, ncol), Im += [ncol, 2 ncol); acc2: Im += [0, ncol), Re -= [ncol, 2 ncol)
            const uint32_t tl = tmem + ((uint32_t)(quarter * 32) << 16) + h * 256 + half * 64;
            {
              uint32_t r0[32], r1[32];
              tmem_ld32(tl, r0);
              tmem_ld32(tl + 32, r1);
              tmem_wait_ld();
              if (h == 0) {
#pragma unroll
                for (int e = 0; e < 32; ++e) {
                  sre[e] += __uint_as_float(r0[e]);
                  sre[32 + e] += __uint_as_float(r1[e]);
                }
              } else {
#pragma unroll
                for (int e = 0; e < 32; ++e) {
                  sim[e] += __uint_as_float(r0[e]);
                  sim[32 + e] += __uint_as_float(r1[e]);
                }
              }
            }
            {
              uint32_t r0[32], r1[32];
              tmem_ld32(tl + ncol, r0);
              tmem_ld32(tl + ncol + 32, r1);
              tmem_wait_ld();
              if (h == 0) {
#pragma unroll
                for (int e = 0; e < 32; ++e) {
                  sim[e] += __uint_as_float(r0[e]);
                  sim[32 + e] += __uint_as_float(r1[e]);
                }
              } else {
#pragma unroll
                for (int e = 0; e < 32; ++e) {
                  sre[e] -= __uint_as_float(r0[e]);
                  sre[32 + e] -= __uint_as_float(r1[e]);
                }
              }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&acce[h]);
          }
          if (!ok) break;
        }
        if (ok) flush_sums_fac(sre, sim, DF, tab, J, Ne, n0c, m_local, Mrows, inv);
        continue;
      }
      for (int kb = step_kb0(q); kb < kb1; kb += kpb, ++g) {  // one TMEM buffer of kpb k-blocks
        const int b = (int)(g & 1);
        if (!warp_wait(&accf[b], (uint32_t)((g >> 1) & 1), status, TC_ERR_ACC, true, wl)) {
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
        if (lane == 0) mbar_arrive(&acce[b]);
      }
      if (ok) flush_sums_fac(sre, sim, DF, tab, J, Ne, n0c, m_local, Mrows, inv);
    }
    if (!ok) {
      // wait (without aborting on the error flag) until every issued MMA is
      // done before the block releases TMEM
      warp_wait(mma_done, 0, status, TC_ERR_ACC, false, wl);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
  }
}
