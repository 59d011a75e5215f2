// Tile, pipeline and register-split constants of the tcgen05 pair GEMM.
#pragma once

constexpr int TC_BM = 128;
constexpr int TC_BN = 128;
constexpr int TC_ROWB = 64;  // bytes of K per shared-memory row (64-byte swizzle)
constexpr int TC_STAGES = 3;
constexpr int TC_PWARPS = 6;               // warps 2..7
constexpr int TC_BWARPS = TC_PWARPS - 1;   // warps 3..7 produce B; warp 2 stages their input rows
constexpr int TC_DWARPS = 8;
constexpr int TC_THREADS = 32 * (2 + TC_PWARPS + TC_DWARPS);  // 512
constexpr int TC_A_BYTES = 4 * TC_BM * TC_ROWB;                // 4 planes, 32 KB
constexpr int TC_B_BYTES = 4 * TC_BN * TC_ROWB;                // 32 KB
// Per-stage staging of the left-chain and phase row chunks the producers
// read (complex64, one k-block each), rows padded by 16 bytes so that rows of
// consecutive momenta fall in different shared-memory banks.
constexpr int TC_XP_BYTES = 10240;
constexpr int TC_XP_PAD = 16;
constexpr int TC_STAGE_BYTES = TC_A_BYTES + TC_B_BYTES + TC_XP_BYTES;
constexpr int TC_SMEM = TC_STAGES * TC_STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
static_assert(TC_SMEM <= 232448, "shared memory per block");
constexpr int TC_LAUNCH_REGS = 65536 / TC_THREADS;  // 128
constexpr int TC_REGS_LOW = 80, TC_REGS_HIGH = 176;
static_assert(256 * TC_REGS_LOW + 256 * TC_REGS_HIGH == TC_THREADS * TC_LAUNCH_REGS, "register split");
// k-blocks between flushes of the FP32 register sums into the double-float
// results (power of 2).  Measured at 32^3, Ne = 200, f16x3: 64 -> 256 cuts the
// factorised GEMM from 173 to 155 ms per 4 timeslices (fewer read-modify-writes
// of the results) and moves the error against FP64 from 1.82e-7 to 2.01e-7.
constexpr int TC_FLUSH_KB = 256;
constexpr long long TC_WAIT_CYCLES = 4000000000LL;  // ~2 s at 2 GHz

// status codes written by the kernel
constexpr int TC_ERR_FULL = 1, TC_ERR_EMPTY = 2, TC_ERR_ACC = 3, TC_ERR_ACCE = 4, TC_ERR_XFULL = 5,
              TC_ERR_SYNC = 6, TC_ERR_CLUSTER = 7;
