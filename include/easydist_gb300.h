/*
 * easydist_gb300.h -- C ABI of the GB300 (sm_103a) distillation hot path.
 *
 * The library replaces the array arithmetic of two EasyDistillation
 * generators: the 3D covariant Laplacian inside EigenvectorGenerator's
 * per-timeslice eigensolve, and ElementalGenerator's displaced,
 * momentum-projected contraction.  Every call:
 *   - takes caller-owned DEVICE pointers (plain addresses) and sizes;
 *   - is ordered on the CUDA stream passed as `stream` (a cudaStream_t, NULL
 *     for the legacy default stream) and returns without synchronising;
 *   - returns ED_OK (0) or a negative ED_ERR_* code; the message of the last
 *     error on the calling host thread is available from ed_last_error();
 *   - allocates no device memory: scratch comes from a caller-provided
 *     workspace whose size is queried first.
 * There is no CPU fallback: without a usable sm_103a device the calls return
 * ED_ERR_CUDA.
 *
 * Lattice sizes are positive with V3 = Lx*Ly*Lz <= 2^28 (sites and colour
 * entries are numbered with 32-bit integers; elemental plans take V3 <= 2^26);
 * larger lattices are rejected with ED_ERR_ARG.
 *
 * Data layouts (V3 = Lx*Ly*Lz, site = x + Lx*(y + Ly*z), x fastest):
 *   reference links   : complex128, element (mu, site, a, b) at
 *                       mu*dir_stride + site*site_stride + 3*a + b
 *                       (ILDG order of one timeslice: dir_stride 9,
 *                        site_stride 36; the generators' transposed order
 *                        U[:3, t]: dir_stride 9*V3, site_stride 9)
 *   SoA links         : [dir 3][row 3][col 3][V3] complex (c128 or c64)
 *   reference vectors : [nvec][V3][3] complex, colour fastest
 *   colour planes     : [nvec][3][V3] complex (c128 or c64)
 *   elementals        : [Nderiv][Nmom][Ne][Ne] complex128
 */
#ifndef EASYDIST_GB300_H
#define EASYDIST_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes */
#define ED_OK 0
#define ED_ERR_ARG (-1)         /* invalid argument (sizes, pointers, alignment) */
#define ED_ERR_CUDA (-2)        /* a CUDA runtime error (launch, device) */
#define ED_ERR_UNSUPPORTED (-3) /* valid request this build does not serve */
#define ED_ERR_WORKSPACE (-4)   /* workspace too small */
#define ED_ERR_TIMEOUT (-5)     /* a bounded device-side wait gave up */

/* ---- storage precisions */
#define ED_C128 0 /* complex128: double2 */
#define ED_C64 1  /* complex64:  float2  */
#define ED_DF 2   /* double-float (ed_laplacian only): links in the split form of ed_split_c128, vectors
                   * complex128; FP64-class results (~2^-47 per product) computed on the FP32 pipe */
#define ED_BIG_ENDIAN 0x10 /* flag on a source precision of ed_decode_*: stored big-endian */

/* ---- elemental arithmetic modes */
#define ED_MODE_FP64 0   /* plain FP64 SIMT contraction (V rounded to c64, all else c128) */
#define ED_MODE_F16X3 1  /* tcgen05: scaled fp16 hi/lo split, 3 products per real product */
#define ED_MODE_BF16X3 2 /* tcgen05: bf16 hi/lo split, 3 products per real product */
#define ED_MODE_TF32X3 3 /* tcgen05 kind::tf32: tf32 hi/lo split, 3 products per real product */
#define ED_MODE_OZAKI_I8 4 /* Ozaki scheme: per-row scaled operands cut into four signed 6-bit
                            * int8 slices, slice products with s+t <= 3 accumulated exactly in
                            * int32 (mma.sync s8), recombined in FP64.  Needs a momentum list that
                            * factorises into distinct (px,py) x pz combinations (at most 128)
                            * and 3*Lx*Ly*Lz <= 163840. */
/* Flag OR-ed into a tensor-core mode at plan creation: keep the GEMM whose
 * phase-weighted operand is formed inside the kernel even when the momentum
 * list factorises into {(px,py)} x {pz} (by default such plans use the
 * factorised-phase GEMM, whose operands are both prepared in HBM). */
#define ED_MODE_FLAG_NO_FACTOR 0x100
/* Flag OR-ed into a tensor-core mode at plan creation: use the factorised-phase
 * GEMM whenever the momentum list fits {(px,py)} x {pz} (at most 128
 * combinations), however many of those combinations the list leaves unused
 * (by default at most a quarter may go unused).  Excludes
 * ED_MODE_FLAG_NO_FACTOR.  An autotuner measures both forms. */
#define ED_MODE_FLAG_FORCE_FACTOR 0x200
/* Flag OR-ed into f16x3 / bf16x3 / tf32x3 at plan creation: run the
 * factorised-phase GEMM in the Gauss three-multiplication form (X = Ar Br,
 * Y = Ai Bi, Z = (Ar + Ai)(Br + Bi); re = X - Y, im = Z - X - Y): 9 MMAs per
 * split product and K step instead of 12, on six operand planes per side
 * (re, im, re + im; the split-plane workspace grows by half).  Needs a
 * factorised plan (ED_ERR_UNSUPPORTED otherwise); runs on single SMs
 * whatever ED_TUNE_TC_PAIR / ED_TUNE_TC_STACK say. */
#define ED_MODE_FLAG_GAUSS 0x400
/* Flag OR-ed into a tensor-core mode at plan creation: factorise with every
 * momentum's whole phase on the left operand, phase_p = phase_p * 1 (Pxy =
 * Nmom left factors of three components, Pz = 1): the factorised GEMM then
 * forms exactly the requested momenta, for any list of at most 127 distinct
 * momenta, at the price of Nmom left variants per left chain in the split
 * planes (e.g. the 7 momenta with |p|^2 <= 1, which as a (px,py) x pz set
 * would leave 8 of 15 combinations unused).  Excludes the two flags above. */
#define ED_MODE_FLAG_LEFT_FACTOR 0x800

/* ---- launch settings of a plan (ed_elemental_set_tuning keys) */
#define ED_TUNE_F64_TILE 1   /* FP64 pair GEMM tile, rows x cols: 0 = 64x64 (default), 1 = 32x64,
                              * 2 = 64x32, 3 = 32x32 */
#define ED_TUNE_TC_SLAB_KB 2 /* k-blocks (of 32 fp16 / 16 tf32 elements) per lock-step slab of the
                              * persistent factorised tensor-core GEMM: 0 (default, 256) or a power
                              * of two <= 256.  The FP32 register sums are flushed to the
                              * double-float results once per slab, so smaller slabs also shorten
                              * the FP32 sums. */
#define ED_TUNE_TC_GRID 3    /* CTAs of the persistent factorised GEMM: 0 (default: every CTA that
                              * fits on the device at once) or an upper bound on that number */
#define ED_TUNE_TC_STAGES 4  /* operand stages in the factorised GEMM's shared-memory ring: 0 (the
                              * default of the GEMM form), 2 or 3 (64 KB stages on single SMs), up to
                              * 4 (48 KB stages on SM pairs, 32 KB in the stacked SM-pair form) */
#define ED_TUNE_TC_PAIR 5    /* factorised GEMM form: 0 (built-in default), 1 = one CTA per SM with
                              * 128 x 128 tiles, 2 = two-CTA clusters on SM pairs with 256 x 128
                              * tiles (tcgen05.mma.cta_group::2, four real products per complex
                              * one), 3 = two-CTA clusters with the stacked operands spread over
                              * the pair: 128 x 128 tiles, CTA r holds plane r (re / im) of the
                              * tile's A and B rows, one M = 256, N = 256 MMA per split product
                              * and K step computes [Ar; Ai] [Br | Bi], and each CTA keeps two
                              * 256-column TMEM buffers, so the MMAs of a k-block group never wait
                              * for the drain of the previous one (ED_TUNE_TC_KPB default 2;
                              * 2 to 4 operand stages of 32 KB, default 4) */
#define ED_TUNE_TC_KPB 6     /* k-blocks the factorised GEMM accumulates in one TMEM buffer before the
                              * drain warps read it: 0 (the form's default: 2 for the stacked form,
                              * 1 otherwise), 1, 2 or 4.  The tensor core's FP32 accumulation
                              * truncates, so longer buffers trade accuracy for fewer hand-overs
                              * (measured at 32^3, Ne = 200, f16x3 vs FP64: four-product form
                              * 2.0e-7 with 1, 5.1e-7 with 2; stacked form 2.6e-7 with 2,
                              * 5.8e-7 with 4).  4 is meant for the stacked and Gauss forms: the
                              * four-product form with 4 exceeded 1e-6 at K = 9216. */
#define ED_TUNE_F64_DF 8     /* FP64 mode's pair GEMM arithmetic: 0 (default) FP64 on the FP64 pipe, 1 =
                              * double-float on the FP32 pipe (each complex128 operand as two complex64
                              * parts, exact FP32 product splits with two-sum accumulation: ~2^-47 relative
                              * per product instead of 2^-53, FP64-class results at several times the
                              * FP64 pipe's speed).  The autotuner never changes it. */
#define ED_TUNE_TC_STACK 7   /* single-SM factorised GEMM operand form: 0 (default) or 1 = stacked:
                              * B = [Br; Bi] in shared memory, two M = 128, N = 256 MMAs
                              * A_re [Br | Bi] and A_im [Br | Bi] per split product into single
                              * 256-column accumulators, re / im formed by the drain (143 ms per
                              * 4 timeslices at 32^3, Ne = 200, f16x3); 2 = four real products
                              * per complex one, M = N = 128 MMAs into double-buffered [re], [im]
                              * accumulators (165-172 ms).  SM pairs take their form from
                              * ED_TUNE_TC_PAIR (2: four products, 3: stacked).  The on-chip-phase
                              * GEMM (lists that do not
                              * factorise) takes the same two forms: stacked with ED_TUNE_TC_KPB
                              * k-blocks per group (default 2), or four products, one k-block per
                              * double-buffered TMEM buffer. */

/* Library version as 10000*major + 100*minor + patch. */
int ed_version(void);

/* Copy the last error message of this host thread into buf (NUL-terminated,
 * truncated to len).  Returns the length of the full message. */
int ed_last_error(char* buf, size_t len);

/* Convert nt timeslices of spatial links from the reference layout into SoA.
 * Replaces the per-timeslice slice `U[:3, t]` of
 * lattice/generator/eigenvector.py:242-243 and elemental.py:103,320-321.
 * in: complex128 with element (t, mu, site, a, b) at
 *     t*t_stride + mu*dir_stride + site*site_stride + 3a + b   (complex units)
 * out: [nt][3][3][3][V3] of precision out_prec. */
int ed_links_to_soa(int out_prec, int Lx, int Ly, int Lz, int nt, const void* in, long long t_stride,
                    long long dir_stride, long long site_stride, void* out, void* stream);

/* Reference vectors [nvec][V3][3] (in_prec) -> colour planes [nvec][3][V3]
 * (out_prec).  round_c64 != 0 rounds every value through complex64 first,
 * as ElementalGenerator's complex64 buffer does (elemental.py:55,297-298). */
int ed_vectors_to_planes(int in_prec, int out_prec, int round_c64, long long nvec, int V3, const void* in,
                         void* out, void* stream);

/* Colour planes [nvec][3][V3] -> reference vectors [nvec][V3][3]. */
int ed_vectors_from_planes(int in_prec, int out_prec, long long nvec, int V3, const void* in, void* out,
                           void* stream);

/* Momentum phase tables exp(+2*pi*i*(px*x/Lx + py*y/Ly + pz*z/Lz)), FP64.
 * Replaces MomentumPhase.get (lattice/insertion/phase.py:11-13,41-46).
 * moms: HOST array [nmom][3] of ints; out: device [nmom][V3] complex128. */
int ed_momentum_phases(int Lx, int Ly, int Lz, const int* moms, int nmom, void* out, void* stream);

/* 3D covariant Laplacian on nt timeslices x nvec vectors.
 * Replaces _Laplacian (lattice/generator/eigenvector.py:11-26).
 * links: SoA [nt][27][V3] (prec); in/out: colour planes, vector v of
 * timeslice t at base + t*tstride + v*3*V3 (complex units; a stride of 0
 * means the packed 3*V3*nvec).  ED_C64 needs an even Lx and even strides.
 * ED_DF: links split by ed_split_c128 (same layout, 16 bytes per complex),
 * in/out complex128; the products and sums run in double-float arithmetic on
 * the FP32 pipe.  in and out must not alias. */
int ed_laplacian(int prec, int Lx, int Ly, int Lz, int nt, int nvec, const void* links, const void* in,
                 long long in_tstride, void* out, long long out_tstride, void* stream);

/* Split n complex128 values into double-float form: dst[i] = float4 {re_hi,
 * im_hi, re_lo, im_lo} with hi the value rounded to FP32 and lo the rest
 * rounded to FP32 (48 significant bits); for the links of ed_laplacian's
 * ED_DF mode.  No counterpart in the reference. */
int ed_split_c128(long long n, const void* src, void* dst, void* stream);

/* Choose the complex64 Laplacian kernel: use_tma = 1 stages the input colour
 * planes of z-1, z, z+1 through TMA into shared memory (when 4 planes fit, Lx
 * is even, Lx <= 128, Ly <= 256 and Lx*Ly is a multiple of 16); 2 stages, per
 * strip of whole rows (at most 128 sites), the 27 link streams, the halo links
 * and the input rows with their halo rows through TMA (Lx even, Lx <= 128,
 * a strip of R | Ly rows with R*Lx <= 128 and R*Lx % 8 == 0): the default, 87 %
 * of the measured HBM bandwidth at 32^3 x 64 against 85 % for 0, which reads
 * every neighbour through L1/L2.  A staged kernel whose limits a shape misses
 * falls back to 0.  Process-wide setting.  No counterpart in the reference. */
int ed_laplacian_config(int use_tma);

/* Cycle limit of the TMA-staged Laplacian kernels' waits for their data
 * (process-wide launch setting; 0 restores the default of 4e9 cycles, about
 * 2 s).  A wait that runs out sets the status word of ed_laplacian_status and
 * the block stops computing; it still waits for its own copies in flight,
 * with the default limit, before it leaves.  A tiny limit makes the waits run
 * out on purpose (a test of the timeout path).  No counterpart in the
 * reference. */
int ed_laplacian_wait_limit(long long cycles);

/* Test of the failure path (process-wide launch setting, 0 = off): when on,
 * every block of the TMA-staged Laplacian kernels first waits, with the
 * data-wait limit, on a barrier of its own that nothing completes, so the
 * limit runs out whatever the copy latency; the launch then reports
 * ED_ERR_TIMEOUT through ed_laplacian_status after its blocks have drained
 * their own copies.  No counterpart in the reference. */
int ed_laplacian_wait_probe(int on);

/* Cycle limit of every bounded wait of the single-SM factorised tensor-core
 * GEMM (tc_fac_gemm_kernel, the default GEMM of the split modes for product
 * momentum lists; process-wide, read at each run; 0 restores the default of
 * 4e9 cycles, about 2 s).  A wait that runs out sets the plan's status word
 * (ed_elemental_status: ED_ERR_TIMEOUT) and every role of the kernel stops:
 * the MMA issuer after the MMAs it has issued, the copy issuer after waiting
 * for its copies in flight, the drain warps after waiting for every issued
 * MMA, before TMEM is released.  No counterpart in the reference. */
int ed_elemental_wait_limit(long long cycles);

/* Test of that failure path (process-wide, 0 = off): when on, the copy issuer
 * of tc_fac_gemm_kernel issues no copy at all, so the first operand-stage
 * wait of the MMA issuer (and the drain warps' first wait) runs out after the
 * limit of ed_elemental_wait_limit, no MMA is issued, and the run reports
 * ED_ERR_TIMEOUT.  Other GEMM kernels ignore it.  No counterpart in the
 * reference. */
int ed_elemental_wait_probe(int on);

/* Status of the TMA-staged Laplacian's bounded waits since the last call
 * (synchronises `stream`): ED_OK, or ED_ERR_TIMEOUT when a wait gave up (the
 * output of that launch is invalid).  The status word is cleared. */
int ed_laplacian_status(int* code, void* stream);

/* ---- projected eigenproblem of thick-restart Lanczos (eigenvector.py:234-257: the
 *      dense eigensolve inside ARPACK / cupyx eigsh at every restart) */

/* Lowest nwant eigenpairs of B real symmetric matrices of order m with the
 * arrowhead + tridiagonal structure of a thick-restart Lanczos matrix:
 *   T[j][j] = d[j];  T[j][ka] = T[ka][j] = s[j] (j < ka);
 *   T[j][j+1] = T[j+1][j] = e[j] (ka <= j < m-1);  every other entry 0.
 * ka = 0 is a plain tridiagonal matrix.  Device arrays, FP64: d [B][m],
 * s [B][ka] (NULL when ka = 0), e [B][m-1] (entries below ka ignored).
 * Out: evals [B][nwant] ascending, evecs [B][m][nwant] (column i is the unit
 * eigenvector of evals[i]; the columns are orthonormal).  Bisection on Sturm
 * counts, inverse iteration (clusters closer than 1e-7 ||T|| orthogonalised
 * in order), two Gram-Schmidt passes; no host synchronisation.
 * workspace: ed_arrow_eigh_workspace bytes of device memory, 8-byte aligned. */
/* One classical Gram-Schmidt pass of the Lanczos reorthogonalisation, batched
 * over B problems, complex128 (double2):
 *   h[b][i] = sum_x conj(V[b][i][x]) w[b][x]   (i < r),  then
 *   w[b][x] -= sum_i h[b][i] V[b][i][x].
 * V: r rows of length n per problem, problem b at V + b*v_bstride (rows
 * contiguous, row stride n); w [B][n] updated in place; h [B][ldh].  Pointers
 * 16-byte aligned.  norm_part (optional, NULL to skip): [B][ceil(n/256)]
 * partial sums of |w_new|^2, whose row sums are ||w_new||^2.  Two kernels,
 * each streaming V once; on GB300 they are bound by the FP64 pipe (8 flops
 * per 16-byte element: about 2.5 TB/s at the FP64 peak), not by HBM. */
int ed_cgs_pass(int B, int r, long long n, const void* V, long long v_bstride, void* w, void* h, int ldh,
                double* norm_part, void* stream);
/* ed_cgs_pass in double-float arithmetic on the FP32 pipe (the pass
 * ED_LANCZOS_GS_DF selects inside the solver): V and w are split into two
 * complex64 parts each (into `workspace`, at least B*(r+1)*n*16 bytes), the
 * sums are (hi, lo) FP32 pairs; h, the updated w and the norm partials are
 * complex128 / double as in ed_cgs_pass.  Product error ~2^-47 relative. */
int ed_cgs_pass_df(int B, int r, long long n, const void* V, long long v_bstride, void* w, void* h, int ldh,
                   double* norm_part, void* workspace, size_t workspace_bytes, void* stream);

/* Lowest Ne eigenpairs of the FP64 3D covariant Laplacian of nt timeslices by
 * batched thick-restart Lanczos: the eigsh call of
 * lattice/generator/eigenvector.py:234-257 (and, with poly_deg > 0, the QUDA
 * path's Chebyshev acceleration of :295-299).  links: complex128 SoA
 * [nt][27][V3] (ed_links_to_soa); evecs out: complex128 colour planes
 * [nt][Ne][3][V3], unit norm; evals out: [nt][Ne] ascending; status (host,
 * int[3]): converged (1/0), restarts, operator applications.  ncv: Krylov
 * dimension (Ne < ncv <= 3*V3; 9/4 Ne plain and 2 Ne with Chebyshev
 * acceleration measured best); the kept Ritz pairs at a restart are
 * min(ncv-1, Ne + max(8, Ne/10)).  Convergence: |beta y_m,i| <= tol
 * |theta_i| for every wanted pair (ARPACK's test).  poly_deg > 0 iterates on
 * the Chebyshev filter of degree poly_deg that maps [lambda_cut, 12] to
 * [-1, 1] and returns Rayleigh quotients as eigenvalues.  Synchronises the
 * stream once per restart.  Needs ed_lanczos_workspace bytes (256-byte
 * aligned). */
int ed_lanczos_workspace(int Lx, int Ly, int Lz, int nt, int Ne, int ncv, size_t* bytes);
int ed_lanczos_tr(int Lx, int Ly, int Lz, int nt, const void* links, int Ne, double tol, int ncv, int max_restarts,
                  int poly_deg, double lambda_cut, void* evecs, double* evals, int* status, void* workspace,
                  size_t workspace_bytes, void* stream);

/* ed_lanczos_tr with a choice of stencil precision.  stencil_prec = ED_C128 is
 * ed_lanczos_tr (links_c64 unused).  ED_C64 is a mixed-precision solve of the
 * same eigenpairs: phase 1 runs the thick-restart iteration with the complex64
 * stencil on links_c64 (complex64 SoA [nt][27][V3], ed_links_to_soa) applied
 * to the FP64 basis vectors (rounded to complex64, the result widened),
 * while Gram-Schmidt, Rayleigh-Ritz and the convergence test stay FP64, for at
 * most 3 restarts or to a tolerance of max(tol, 1e-3) (it only has to bound
 * the wanted spectrum from above); phase 2 refines every pair in FP64: a
 * Chebyshev-filtered FP64-stencil solve (degree poly_deg, 16 when 0; Krylov
 * dimension max(2 Ne, Ne + 32)) whose cut is lambda_cut, or when lambda_cut
 * <= 0, 1.15 x the largest phase-1 eigenvalue of any timeslice, started from
 * the sum of the phase-1 Ritz vectors, to tol.  ncv is the Krylov dimension of
 * phase 1.  The outputs are those of ed_lanczos_tr (FP64 eigenpairs;
 * eigenvalues are FP64 Rayleigh quotients after phase 2).  status (host,
 * int[6]): converged, total restarts, total operator applications, phase-1
 * (complex64) applications, phase-2 (FP64) applications, phase-1 restarts.
 * Lx must be even for ED_C64.  Synchronises the stream once per restart and
 * once between the phases.  The reference's eigsh is FP64 throughout
 * (lattice/generator/eigenvector.py:234-257); the precision split has no
 * counterpart there.  Needs ed_lanczos_workspace_ex bytes.
 *
 * ED_LANCZOS_GS_DF OR-ed into stencil_prec (both calls): the Gram-Schmidt
 * passes, the restart rotation and the FP64-class stencil applications run in
 * double-float arithmetic on the FP32 pipe (ed_cgs_pass_df, the rotation
 * kernel, ed_laplacian's ED_DF on links split once per solve) instead of
 * FP64: the basis stays FP64 and gets a split copy (two complex64 parts per
 * value; the workspace grows by the basis and the links), the products err by
 * ~2^-47 relative instead of 2^-53, and a pass streams the basis at HBM speed
 * instead of the FP64 pipe's ~2.5 TB/s.  The recurrence, the projected
 * eigenproblem, the convergence test and the final Rayleigh quotients stay
 * FP64. */
#define ED_LANCZOS_GS_DF 0x100
int ed_lanczos_workspace_ex(int Lx, int Ly, int Lz, int nt, int Ne, int ncv, int stencil_prec, size_t* bytes);
int ed_lanczos_tr_ex(int Lx, int Ly, int Lz, int nt, const void* links, const void* links_c64, int stencil_prec,
                     int Ne, double tol, int ncv, int max_restarts, int poly_deg, double lambda_cut, void* evecs,
                     double* evals, int* status, void* workspace, size_t workspace_bytes, void* stream);

int ed_arrow_eigh_workspace(int B, int m, int nwant, size_t* bytes);
int ed_arrow_eigh(int B, int m, int ka, int nwant, const double* d, const double* s, const double* e,
                  double* evals, double* evecs, void* workspace, size_t workspace_bytes, void* stream);

/* In-place projection of nlinks 3x3 complex128 links [nlinks][3][3] back onto
 * U(3) by the averaged inverse iteration U <- (U + U^-dag) / 2 of
 * lattice/generator/eigenvector.py:55-65 (EigenvectorGenerator.project_SU3)
 * and elemental.py:107-118, until max|U - U^-dag| and max|U U^dag - 1| are
 * both <= tol for the link (the reference uses 1e-15 over the whole field),
 * at most max_iter iterations.  FP64, one thread per link. */
int ed_project_su3(long long nlinks, void* U, double tol, int max_iter, void* stream);

/* One covariant-derivative hop D_dir on nvec colour-plane vectors:
 * out = U_d(x) in(x+d) - U_d(x-d)^dag in(x-d).
 * Replaces one iteration of ElementalGenerator._nD (elemental.py:282-287).
 * links_c128: SoA complex128 [27][V3]; math in FP64. */
int ed_covariant_derivative(int in_prec, int out_prec, int Lx, int Ly, int Lz, int dir, int nvec,
                            const void* links_c128, const void* in, void* out, void* stream);

/* One 3D stout-smearing step of the spatial links, FP64, out of place.
 * Replaces the CUDA kernel stout_smear<double> (lattice/generator/stout_smear.cu:159-245)
 * and its numpy form (lattice/generator/eigenvector.py:123-190).
 * U_in/U_out: [3][nt][V3][3][3] complex128 (the generators' spatial links);
 * they must not alias. */
int ed_stout_smear_step(int Lx, int Ly, int Lz, int nt, double rho, const void* U_in, void* U_out, void* stream);

/* One-sided parallel transport of nvec colour-plane vectors (c128, FP64):
 * sign = +1: out(x) = U_dir(x) in(x+dir); sign = -1: out(x) = U_dir(x-dir)^dag in(x-dir).
 * Replaces one straight-line step of DisplacementElementalGenerator._D
 * (lattice/generator/displacement_elemental.py:53-71). links: SoA c128 [27][V3]. */
int ed_parallel_transport(int Lx, int Ly, int Lz, int dir, int sign, int nvec, const void* links_c128,
                          const void* in, void* out, void* stream);

/* out[i] = mean over k < nsrc of src[k*src_stride + i], complex128, i < n
 * (the `.mean(0)` of displacement_elemental.py:64,71). */
int ed_mean_c128(int nsrc, long long n, long long src_stride, const void* src, void* out, void* stream);

/* Adjoint (link gradient) of a stencil direction, accumulated into
 * grad_links (SoA c128 [27][V3], direction `dir` only):
 *   grad U_dir(x) += sum_v alpha * wbar_v(x) f_v(x+dir)^dag + beta * f_v(x) wbar_v(x+dir)^dag
 * where wbar is the adjoint seed of the stencil output and f its input
 * (colour planes, c128, nvec vectors).  (alpha, beta) = (1, -1) gives the
 * covariant-derivative hop of elemental.py:282-287, (-1, -1) the Laplacian of
 * eigenvector.py:11-26; gradient convention dL = Re sum conj(grad) dU.
 * No counterpart in the reference (it has no gradients). */
int ed_link_grad(int Lx, int Ly, int Lz, int dir, int nvec, double alpha, double beta, const void* wbar,
                 const void* f, void* grad_links, void* stream);

/* Adjoint seeds of the pair contraction (the backward pass of the GEMM of
 * lattice/generator/elemental.py:324-329; the reference has no gradients):
 *   out[a][k] += sum_{r < R} M[r][a] * chains[cx[r]][ir[r]][k] * psi_r(k)
 * with psi_r = phase_p (pr[r] = p >= 0) or conj(phase_p) (pr[r] = -p-1), and
 * k = colour*V3 + site.  For G_p(X, Y)[i][j] = sum_k conj(X_i[k]) phase_p(k) Y_j[k]
 * and a loss gradient Gbar_p: grad Y = rows (X, p, i) with M = Gbar_p[i][.]
 * and conj phases; grad X = rows (Y, p, j) with M = conj(Gbar_p[.][j]) and
 * phases.  M: device [R][Ne] complex128; cx, ir, pr: device int[R] (rows
 * naming anything out of range contribute nothing); chains: colour planes
 * [nchain][Ne][3][V3] complex128; phases: [nmom][V3] complex128; out:
 * [Ne][3][V3] complex128, accumulated.  FP64. */
int ed_chain_adjoint(int Lx, int Ly, int Lz, int Ne, int nchain, int nmom, int R, const void* M, const int* cx,
                     const int* ir, const int* pr, const void* chains, const void* phases, void* out, void* stream);

/* ---- correlators (lattice/correlator/one_particle.py) */

/* One source timeslice of the meson two-point contraction
 * "tijab,xjk,xtbc,tklcd,yli,yad->t" of lattice/correlator/one_particle.py:64-72,
 * accumulated into out[t] (complex128, t < T) without the overall minus sign:
 *   out[t] += sum_terms coef * Tr[ conj(taub[t][j][i])^T E_x(t_src + t mod Lt) tau[t][k][l] conj(E_y(t_src))^T ]
 * tau, taub: device [T][4][4][Ne][Ne] complex128 (the perambulator of the
 * source at the sink times, and the one of the backward propagator: tau
 * itself, or perambulator_bw); el: device [nparts][Lt][Ne][Ne] complex128
 * (the operator's assembled elementals, lattice/data.py:7-33); term_idx:
 * device int[nterm][6] = (x, y, i, j, k, l), term_coef: device
 * [nterm][2] doubles: one term per (part x, part y, spin i, spin k), with j
 * the row of the sink gamma whose non-zero is in column k, l the row of the
 * source gamma g4 Gamma^dag g4 whose non-zero is in column i, and coef the
 * product of those two entries and of g5[i][i] g5[j][j] (every gamma of the
 * reference's table is monomial).  Terms naming an index out of range
 * contribute nothing.  FP64. */
int ed_twopoint_trace(int T, int Ne, int Lt, int t_src, int nparts, int nterm, const int* term_idx,
                      const double* term_coef, const void* tau, const void* taub, const void* el, void* out,
                      void* stream);

/* Eigenvector-resolved two-point function of one source timeslice and one
 * operator: the contraction "tijab,xjk,xtbc,tklcd,yli,yad->tad" of
 * twopoint_profile (lattice/correlator/one_particle.py:80-135, :122-130):
 *   out[t][a][d] = sum_terms coef (conj(taub[t][j][i])^T E_x(sink_t[t]) tau[t][k][l])[a][d] conj(E_y(t_src))[a][d]
 * over the terms of ed_twopoint_trace, given in factorised form: for the
 * sink part x and spin k, ltab[k][x] = j and lcoef[k][x] = gamma_x[j][k]
 * g5[j][j] (device int[4][nparts], double[4][nparts][2]); for the source part
 * y and spin i, rtab[i][y] = l and rcoef[i][y] = G_y[l][i] g5[i][i].
 * sink_t: device int[T], the elemental timeslice of each sink time; tau, taub:
 * [T][4][4][Ne][Ne] at those sink times; el as for ed_twopoint_trace; work:
 * device scratch of T*16*Ne*Ne complex128; out: device [T][Ne][Ne]
 * complex128, overwritten.  FP64, written once per element (no atomics). */
int ed_twopoint_profile(int T, int Ne, int Lt, int t_src, int nparts, const int* sink_t, const int* ltab,
                        const double* lcoef, const int* rtab, const double* rcoef, const void* tau, const void* taub,
                        const void* el, void* work, void* out, void* stream);

/* The diagonal form (is_diagonal: "tijab,xjk,xtbb,tklba,yli,yaa->ta",
 * one_particle.py:113-121): out[t][a] = sum_terms coef conj(E_y(t_src))[a][a]
 * sum_b conj(taub[t][j][i][b][a]) E_x(sink_t[t])[b][b] tau[t][k][l][b][a], the
 * terms and arguments as for ed_twopoint_trace plus sink_t; out: device
 * [T][Ne] complex128, overwritten.  FP64. */
int ed_twopoint_profile_diag(int T, int Ne, int Lt, int t_src, int nparts, int nterm, const int* sink_t,
                             const int* term_idx, const double* term_coef, const void* tau, const void* taub,
                             const void* el, void* out, void* stream);

/* ---- elementals (ElementalGenerator.calc, lattice/generator/elemental.py:290-338) */
typedef struct ed_elemental_plan ed_elemental_plan;

/* Plan one timeslice of elementals: derivative operators 0..Nderiv-1 with
 * Nderiv = (3^(num_nabla+1)-1)/2 (elemental.py:48-49, derivative.py:23-33),
 * the momenta moms[nmom][3] (host ints), Ne eigenvectors, mode ED_MODE_*.
 * The plan is host-only state (no device memory). */
int ed_elemental_plan_create(ed_elemental_plan** plan, int Lx, int Ly, int Lz, int Ne, int num_nabla,
                             const int* moms, int nmom, int mode);
int ed_elemental_plan_destroy(ed_elemental_plan* plan);

/* Device workspace the plan needs, in bytes. */
int ed_elemental_workspace_size(const ed_elemental_plan* plan, size_t* bytes);

/* Number of distinct (left chain, right chain) contractions per momentum the
 * plan executes (the reference evaluates 2^len subsets per operator). */
int ed_elemental_num_pairs(const ed_elemental_plan* plan, int* npairs);

/* Run one timeslice.
 * links: reference-layout complex128 spatial links of this timeslice
 *        (see the layout note above, dir_stride/site_stride in complex units);
 * evecs: reference vectors [Ne][V3][3] of precision evec_prec (rounded to
 *        complex64 as the reference does);
 * blend: NULL or device [Ne][Ne] float64 stochastic blending coefficients,
 *        multiplied elementwise into every (operator, momentum) block
 *        (elemental.py:61-100,330-337);
 * out:   device [Nderiv][Nmom][Ne][Ne] complex128 (overwritten). */
int ed_elemental_run(const ed_elemental_plan* plan, const void* links, long long dir_stride, long long site_stride,
                     int evec_prec, const void* evecs, const double* blend, void* out, void* workspace,
                     size_t workspace_bytes, void* stream);

/* Batched elementals: a plan for up to max_batch timeslices of one lattice,
 * run with one pair-contraction launch for the whole batch (the reference
 * calls ElementalGenerator.calc once per timeslice, elemental.py:290).
 * links/evecs/outs are HOST arrays of nbatch device pointers (each as in
 * ed_elemental_run); nbatch <= max_batch.  The workspace (from
 * ed_elemental_workspace_size) grows with max_batch. */
int ed_elemental_plan_create_batched(ed_elemental_plan** plan, int Lx, int Ly, int Lz, int Ne, int num_nabla,
                                     const int* moms, int nmom, int mode, int max_batch);
int ed_elemental_run_batch(const ed_elemental_plan* plan, int nbatch, const void* const* links, long long dir_stride,
                           long long site_stride, int evec_prec, const void* const* evecs, const double* blend,
                           void* const* outs, void* workspace, size_t workspace_bytes, void* stream);

/* ed_elemental_run_batch in three parts, so that several batched plans (lattice
 * volumes with their own Ne, each with its own workspace) share ONE
 * pair-contraction launch: for every plan ed_elemental_run_batch_begin (the
 * phase table and the chains of its nbatch timeslices), then one
 * ed_elemental_gemm_multi over all plans, then ed_elemental_run_batch_end per
 * plan (the combine into the outputs).  The three parts of a plan run in
 * stream order on the same stream and together equal one
 * ed_elemental_run_batch; they allocate nothing, so the sequence can be
 * captured in a CUDA graph.  ed_elemental_gemm_multi issues one launch whose
 * blocks cover the tiles of the plans (up to 4) that take the on-chip-phase
 * tensor-core path with the split mode and form of the first such plan
 * (f16x3, bf16x3 or tf32x3, a momentum list that is not factorised), and one
 * launch for each other plan (factorised, FP64, another mode).  *launches
 * (may be NULL) receives the number of GEMM launches.  The
 * reference computes each (volume, timeslice) by its own
 * ElementalGenerator.calc(t) (lattice/generator/elemental.py:290-338). */
int ed_elemental_run_batch_begin(const ed_elemental_plan* plan, int nbatch, const void* const* links,
                                 long long dir_stride, long long site_stride, int evec_prec, const void* const* evecs,
                                 void* workspace, size_t workspace_bytes, void* stream);
int ed_elemental_gemm_multi(int nplans, const ed_elemental_plan* const* plans, const int* nbatch,
                            void* const* workspaces, const size_t* workspace_bytes, int* launches, void* stream);
int ed_elemental_run_batch_end(const ed_elemental_plan* plan, int nbatch, const double* blend, void* const* outs,
                               void* workspace, size_t workspace_bytes, void* stream);

/* Generic pair contraction on caller-built chains (the GEMM stage of
 * elemental.py:324-329 / displacement_elemental.py:94-95):
 *   G[p][i][r*Ne + j] = sum_k conj(X_i[k]) phase_p(k) Y_{right0+r, j}[k]
 * with X = chain `left`.  chains: colour planes [nchain][Ne][3][V3], complex128
 * for ED_MODE_FP64, complex64 for the tensor-core modes.  The plan is queried
 * with ed_elemental_workspace_size and released with ed_elemental_plan_destroy. */
int ed_pair_plan_create(ed_elemental_plan** plan, int Lx, int Ly, int Lz, int Ne, int nchain, const int* moms,
                        int nmom, int mode, int left, int right0, int nright);
int ed_pair_run(const ed_elemental_plan* plan, const void* chains, void* G, void* workspace, size_t workspace_bytes,
                void* stream);

/* Size of the scratch array built into the library for
 * ed_elemental_run_noalloc (32 MiB, held on every GPU that loads it). */
#define ED_NOALLOC_SCRATCH_BYTES (32u << 20)

/* Same as ed_elemental_run, for callers that cannot allocate device memory
 * (their GPU memory is owned by another allocator, or they are called from
 * code that must not allocate): scratch comes from a fixed array inside the
 * library instead of a caller workspace.  No counterpart in the reference
 * (it is an addition of this library).  Plans needing more than
 * ED_NOALLOC_SCRATCH_BYTES are rejected with ED_ERR_WORKSPACE.  The first call
 * on a device resolves the array's address and should precede any stream
 * capture; under lazy module loading (CUDA_MODULE_LOADING=LAZY, the default
 * of recent CUDA releases) that first call also loads the library's module on
 * the device and commits the 32 MiB there, so make it where allocating is
 * still allowed (at initialisation).  All calls share the array, so calls
 * that overlap on the GPU race and must be serialised by the caller.  In the
 * tensor-core modes a bounded device wait that gave up leaves a status word in
 * the array: read it with ed_elemental_status_noalloc. */
int ed_elemental_run_noalloc(const ed_elemental_plan* plan, const void* links, long long dir_stride,
                             long long site_stride, int evec_prec, const void* evecs, const double* blend, void* out,
                             void* stream);

/* ed_elemental_status for runs of ed_elemental_run_noalloc: synchronise
 * `stream` and report the status word the last run left in the built-in
 * scratch array (ED_OK, or ED_ERR_TIMEOUT when a bounded wait inside the
 * tensor-core kernel gave up; *code receives the raw word, 0 = ok).  No
 * counterpart in the reference. */
int ed_elemental_status_noalloc(const ed_elemental_plan* plan, int* code, void* stream);

/* Describe the plan's pair groups: *ngroups groups (one per left chain); for
 * group g, left[g] is its left chain and nright[g] its number of right chains
 * (arrays of at least 32 ints, may be NULL); *herm = 1 when the momentum list
 * is closed under p -> -p and hermiticity halves the work. */
int ed_elemental_describe(const ed_elemental_plan* plan, int* ngroups, int* left, int* nright, int* herm);

/* *factorised = 1 when the plan runs the factorised-phase tensor-core GEMM:
 * its momenta are (up to a quarter of unused combinations) the product set
 * of *pxy distinct (px, py) pairs and *pz distinct pz values, and both GEMM
 * operands (conj(X) f_(px,py) and g_pz Y) are prepared in HBM.  pxy and pz
 * may be NULL.  No counterpart in the reference (an execution detail). */
int ed_elemental_factorised(const ed_elemental_plan* plan, int* factorised, int* pxy, int* pz);

/* Set / read one launch setting of a plan (ED_TUNE_* key).  Settings change
 * how later runs are launched, never what they compute beyond rounding: the
 * FP64 tile shape leaves every sum in the same order (bit-identical results);
 * the slab length changes where the tensor-core path's FP32 sums are cut
 * (results agree to the mode's tolerance).  Host-side only, no device call.
 * ED_ERR_ARG for an unknown key or a value out of range.  No counterpart in
 * the reference (its GEMMs are library calls); the project's autotuner
 * (easydistillation_gb300/tune.py) picks the values by measurement. */
int ed_elemental_set_tuning(ed_elemental_plan* plan, int key, int value);
int ed_elemental_get_tuning(const ed_elemental_plan* plan, int key, int* value);

/* Record the CUDA events `start` / `stop` (cudaEvent_t, or NULL to disable)
 * on the run's stream immediately before and after the pair-contraction
 * kernel of every later ed_elemental_run with this plan, so a caller can time
 * that kernel alone.  The plan keeps only the handles. */
int ed_elemental_set_profile_events(ed_elemental_plan* plan, void* start, void* stop);

/* Synchronise `stream` and report the device-side status of the last run on
 * this workspace: ED_OK, or ED_ERR_TIMEOUT when a bounded wait inside the
 * tensor-core kernel gave up (its output is then invalid).  *code receives
 * the raw status word (0 = ok). */
int ed_elemental_status(const ed_elemental_plan* plan, const void* workspace, int* code, void* stream);

/* ---- on-disk formats (lattice/filedata/ildg.py:70, lattice/filedata/timeslice.py:96,
 *      lattice/generator/elemental.py:103: the readers' byte-order and precision
 *      conversion and the generators' link transpose, on the device) */

/* n complex numbers from a file's byte image in device memory (src_prec
 * ED_C128 or ED_C64, | ED_BIG_ENDIAN when stored big-endian) to native
 * complex numbers of dst_prec (ED_C128 widens exactly; ED_C64 rounds to
 * nearest, as numpy's astype).  src aligned to its element size, dst to its;
 * the two ranges must not overlap.  n = 0 is a no-op. */
int ed_decode_complex(int src_prec, long long n, const void* src, int dst_prec, void* dst, void* stream);

/* Spatial links from the ILDG site order: src [sites][4][3][3] complex (the
 * file's byte image, src_prec as above, sites = Lt*Lz*Ly*Lx), dst
 * [3][sites][3][3] complex128, the generators' [dir][t][z][y][x][3][3]
 * layout (the time links are dropped).  dst 16-byte aligned, no overlap. */
int ed_decode_links(int src_prec, long long sites, const void* src, void* dst, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* EASYDIST_GB300_H */
