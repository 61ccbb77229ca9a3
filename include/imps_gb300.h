/*
 * imps_gb300 -- C ABI of the GB300 (sm_103a) implementation of the IMPS_CPP_tools hot path:
 * the block-sparse effective-Hamiltonian applies (H_AC, H_C), transfer-matrix applies and
 * the Krylov solves (Lanczos eigensolve, GMRES environment solve) that drive VUMPS.
 *
 * Conventions
 *  - Every function returns an int status: 0 = OK, > 0 warning, < 0 error (IMPS_* below).
 *  - Vectors use the reference's layout unchanged: blocks concatenated in std::map key
 *    order (s-major for MPS tensors), each block column-major (MPSBlockMat.hpp:448-465,
 *    BlockObj.hpp:767-780, 1712), so vectors can be handed to/from ARPACK without permutation.
 *  - A "layout" is the sector table of one block-sparse object (the reference's
 *    GetSizesVector(), MPSBlockMat.hpp:336-347): per block (Qin, Qout, rows, cols, group),
 *    group = physical index s for an MPS tensor, i*d+j for a RedOp grid (OperatorTypes.hpp:
 *    160-187, row-major), 0 for BlockDiagMat/BlockMat.  Blocks must be ordered by group, then
 *    by Qin (lexicographic), as the reference's std::map iteration yields them.
 *  - mem = IMPS_MEM_HOST: pointers are host memory (copied through device staging);
 *    mem = IMPS_MEM_DEVICE: pointers are device memory on the context's device.
 *  - One context = one device + one CUDA stream; calls on one context are serialised on its
 *    stream, no call retains a caller pointer after it returns (except imps_plan_bind).
 *  - Contexts share no mutable state (each has its own stream, Krylov workspace, scratch and
 *    pinned staging; the launch-shape cache of imps_plan_autotune is locked): calls on plans of
 *    different contexts may run at the same time from different host threads, the caller
 *    ordering their streams (events).  Calls on one context, or on the plans of one context,
 *    come from one thread at a time.  Plan creation uploads its tables by synchronous copies on
 *    the legacy default stream: synchronise the device before a plan's first launch on a
 *    non-blocking stream.
 */
#ifndef IMPS_GB300_H
#define IMPS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define IMPS_OK 0
#define IMPS_WARN_NOT_CONVERGED 1
#define IMPS_ERR_BAD_ARG -1
#define IMPS_ERR_BAD_TABLE -2
#define IMPS_ERR_CUDA -3
#define IMPS_ERR_NAN -4
#define IMPS_ERR_TIMEOUT -5
#define IMPS_ERR_NO_DEVICE -6
#define IMPS_ERR_OOM -7
#define IMPS_ERR_UNSUPPORTED -8
#define IMPS_ERR_TOO_LARGE -9 /* problem exceeds the fixed scratch of imps_tm_apply_noalloc */

#define IMPS_MEM_HOST 0
#define IMPS_MEM_DEVICE 1

#define IMPS_DIR_LEFT 0
#define IMPS_DIR_RIGHT 1

#define IMPS_PREC_FP64 0
#define IMPS_PREC_BF16X6 1

typedef struct imps_ctx imps_ctx;
typedef struct imps_layout imps_layout;
typedef struct imps_plan imps_plan;

/* ---- library / context ------------------------------------------------------------------ */
const char* imps_status_string(int status);
int imps_version(void);
/* number of GPU kernels this library has launched in the process so far */
int64_t imps_launch_count(void);
int imps_ctx_create(int device, imps_ctx** out);
int imps_ctx_destroy(imps_ctx* ctx);
/* launch on an existing cudaStream_t (e.g. torch's current stream), used as given:
 * NULL is the CUDA legacy default stream.  imps_ctx_use_own_stream restores the context's
 * own non-blocking stream (the default after imps_ctx_create). */
int imps_ctx_set_stream(imps_ctx* ctx, void* cuda_stream);
int imps_ctx_use_own_stream(imps_ctx* ctx);
int imps_ctx_synchronize(imps_ctx* ctx);

/* ---- sector tables (replaces the std::map sector bookkeeping of BlockObj.hpp:506-600,
 *      1360-1467 and MPSBlockMat.hpp:41-175) -------------------------------------------------- */
int imps_layout_create(int nsym, int nblocks, const int32_t* qin, const int32_t* qout,
                       const int32_t* rows, const int32_t* cols, const int32_t* group,
                       imps_layout** out);
int imps_layout_destroy(imps_layout* L);
int64_t imps_layout_nelem(const imps_layout* L);
int imps_layout_nblocks(const imps_layout* L);
int imps_layout_nsym(const imps_layout* L);
/* export the table (arrays sized nblocks*nsym for keys, nblocks otherwise; NULL skips) */
int imps_layout_get(const imps_layout* L, int32_t* qin, int32_t* qout, int32_t* rows,
                    int32_t* cols, int32_t* group, int64_t* off);
/* GetMl (side 0) / GetMr (side 1) of an MPS tensor as a BlockDiagMat layout
 * (MPSBlockMat.hpp:281-326) */
int imps_layout_bond(const imps_layout* A, int side, imps_layout** out);

/* ---- contraction plans: sector matching compiled once into grouped-GEMM tables ----------- */
/* ApplyHA / ApplyHAvec (VUMPS_helpers.hpp:38-88).  Slots: 0 in, 1 out, 2 EHL, 3 EHR, 4 HL, 5 HR */
int imps_plan_hac(imps_ctx* ctx, const imps_layout* AC, const imps_layout* EHL,
                  const imps_layout* EHR, const imps_layout* HL, const imps_layout* HR, int d,
                  imps_plan** out);
/* ApplyHC / ApplyHCvec (VUMPS_helpers.hpp:91-133), h given as its nonzeros (row, col, value)
 * in armadillo SpMat iteration order.  Slots: 0 in, 1 out, 2 EHL, 3 EHR, 4 AL, 5 AR; call
 * imps_plan_prepare after binding/changing AL, AR. */
int imps_plan_hc(imps_ctx* ctx, const imps_layout* C, const imps_layout* EHL,
                 const imps_layout* EHR, const imps_layout* AL, const imps_layout* AR, int d,
                 int nnz, const int32_t* hrow, const int32_t* hcol, const double* hval,
                 imps_plan** out);
/* ApplyTMLeft / ApplyTMRight on a unit cell (TMBlockFunctions.hpp:33-84, 155-205, 542-625).
 * Slots: 0 in, 1 out, 2.. 2+nsites-1 A[k]. */
int imps_plan_tm(imps_ctx* ctx, int nsites, const imps_layout* const* A, int dir,
                 const imps_layout* in, const imps_layout* out, imps_plan** plan);
/* Mixed transfer matrix of two unit cells on a general BlockMat (one block per incoming
 * charge, a fixed charge offset): ApplyTMmixedLeft(A, B, X) / ApplyTMmixedRight(A, B, X)
 * (TMBlockFunctions.hpp:336-344, 474-482; unit-cell chains :669-676 in site order, :737-744
 * in reverse).  dir 0: out(Qout(B_s) -> Qout(A_s)) += B_s^T X A_s; dir 1:
 * out(Qin(A_s) -> Qin(B_s)) += A_s X B_s^T.  A is the lower, B the upper layer.  Apply with
 * imps_tm_apply (real vectors; a complex vector is applied plane by plane).
 * Slots: 0 in, 1 out, 2.. A[k], 2+nsites.. B[k]. */
int imps_plan_tm_mixed(imps_ctx* ctx, int nsites, const imps_layout* const* A, const imps_layout* const* B,
                       int dir, const imps_layout* in, const imps_layout* out, imps_plan** plan);
/* A grouped-GEMM program from explicit tables (all slots external, bound with
 * imps_plan_bind, executed in stage order by imps_plan_run).  stage_nouts[s] output blocks per
 * stage; per output block 7 int64 (c_slot, c_off, c_ld, M, N, accumulate, nterms) followed in
 * `terms` by its nterms terms of 9 int64 (a_slot, a_off, a_ld, a_trans, b_slot, b_off, b_ld,
 * b_trans, k) with `alphas`: C (+)= sum alpha op(A) op(B).  Output blocks of one stage must not
 * overlap.  Every region is bounds-checked against the slot sizes (IMPS_ERR_BAD_TABLE). */
int imps_plan_program(imps_ctx* ctx, int nslots, const int64_t* slot_nelem, int nstages,
                      const int32_t* stage_nouts, const int64_t* outs, const int64_t* terms,
                      const double* alphas, imps_plan** plan);
/* ReducedOp (MPSBlockUtilities.hpp:37-74).  Slots: 0 A, 1 out (derived layout 0). */
int imps_plan_redop(imps_ctx* ctx, const imps_layout* A, int d, int nnz, const int32_t* hrow,
                    const int32_t* hcol, const double* hval, int dir, imps_plan** out);
/* ApplyOpTMLeftDiag / ApplyOpTMRightDiag on the 2-site product A0*A1 (TMBlockFunctions.hpp:
 * 797-836, MPSBlockMat.hpp:934-947).  Slots: 0 A0, 1 A1, 2 out. */
int imps_plan_optm(imps_ctx* ctx, const imps_layout* A0, const imps_layout* A1, int d, int nnz,
                   const int32_t* hrow, const int32_t* hcol, const double* hval, int dir,
                   const imps_layout* out, imps_plan** plan);
/* MPS x BlockDiagMat (side bit0 = 1: A*op(X); 0: op(X)*A; side bit1: op(X) = X^T), scaled by
 * alpha (MPSBlockMat.hpp:1021-1043).  Slots: 0 A, 1 X, 2 out. */
int imps_plan_mps_bd(imps_ctx* ctx, const imps_layout* A, const imps_layout* X, int side,
                     double alpha, imps_plan** out);
/* Tangent-space gradient of GradNormRight (VUMPS_helpers.hpp:145-153).
 * Slots: 0 Y = H_AC(C*AR), 1 AR, 2 G (output, AR layout). */
int imps_plan_grad_right(imps_ctx* ctx, const imps_layout* Y, const imps_layout* AR,
                         imps_plan** out);
int imps_plan_destroy(imps_plan* P);
int imps_plan_derived_layout(const imps_plan* P, int which, imps_layout** out);
int imps_plan_info(const imps_plan* P, int64_t* flops_apply, int64_t* flops_prep,
                   int64_t* dropped, int* nslots, int* nstages);
int imps_plan_slot_info(const imps_plan* P, int slot, int* kind, int64_t* nelem);
/* A plan applying `src` to `copies` inputs at once (no counterpart in the reference): every stage
 * of src repeated per copy in one launch, the input, output and scratch slots `copies` times as
 * long (copy c at offset c x src's length), the operator slots shared (bindings copied).  src
 * must have no prepare stages (TM and mixed-TM plans).  Destroy with imps_plan_destroy. */
int imps_plan_replicate(const imps_plan* src, int copies, imps_plan** out);
/* bind a device pointer to an external slot (kept until rebound or the plan is destroyed) */
int imps_plan_bind(imps_plan* P, int slot, double* device_ptr);
int imps_plan_prepare(imps_plan* P);
int imps_plan_run(imps_plan* P);
/* export the sector-matching table of one stage: per output block its tag and term range;
 * per term (a_slot, a_off, b_slot, b_off, k, alpha).  Pass NULL arrays to query sizes. */
int imps_plan_table(const imps_plan* P, int prep, int stage, int64_t* n_outs, int64_t* n_terms,
                    int32_t* out_tag, int32_t* out_t0, int32_t* out_t1, int32_t* term_aslot,
                    int64_t* term_aoff, int32_t* term_bslot, int64_t* term_boff,
                    int32_t* term_k, double* term_alpha);
/* Tile-shape autotuner of the FP64 grouped GEMM (no counterpart in the reference, whose
 * products are per-block dgemm calls).  A stage's launch shape (tile 16 or 32, split-K 1..8)
 * is keyed on the histogram of its output blocks (rows, cols, summed K, terms).  For every
 * apply stage of `plan` whose key has no cached shape, each candidate is timed (median of
 * `reps` launches with CUDA events on the context's stream, on zero-filled stand-ins of the
 * caller's slots: no bound buffer is touched, nothing needs to be bound) and the fastest is
 * cached for the process; cached shapes are installed.  Plans
 * created later pick cached shapes up; stages without one use a makespan estimate.
 * Synchronises the stream.  n_tuned (optional): stages timed by this call. */
int imps_plan_autotune(imps_plan* plan, int reps, int* n_tuned);
/* the launch shape of an apply stage and its histogram key */
int imps_plan_stage_shape(const imps_plan* plan, int stage, int* tile, int* splits, uint64_t* key);
/* forget every cached shape */
int imps_autotune_clear(void);
/* select the GEMM engine of a plan: IMPS_PREC_FP64 (DFMA) or IMPS_PREC_BF16X6 (tcgen05) */
int imps_plan_set_precision(imps_plan* P, int prec);

/* ---- reference-facing functors (the std::function<void(T*,T*)> handed to ARPACK) --------- */
/* ApplyHAvec (VUMPS_helpers.hpp:55-88): operators bound to slots 2..5 beforehand */
int imps_hac_apply(imps_plan* hac, const double* in, double* out, int mem);
/* ApplyHCvec (VUMPS_helpers.hpp:114-133) */
int imps_hc_apply(imps_plan* hc, const double* in, double* out, int mem);
/* TMMultDiag with ApplyTMLeft/Right on the unit cell (EigsBlockFunctions.hpp:50-66) */
int imps_tm_apply(imps_plan* tm, const double* in, double* out, int mem);
/* InvEfun_proj (InvEBlockFunctions.hpp:12-47): out = in - T(in) + tr(in*rho_in)*rho_out */
int imps_tm_proj_apply(imps_plan* tm, const double* in, const double* rho_in,
                       const double* rho_out, double* out, int mem);

/* ---- solvers ----------------------------------------------------------------------------- */
/* eigs_rs(..., nev=1, "SA", tol, x0) (eigs.cpp:369-494) for a symmetric plan (H_AC or H_C):
 * thick-restarted Lanczos with CGS2 re-orthogonalisation on the device.  x holds x0 on
 * entry and the normalised eigenvector on exit.  ncv = 0 selects max(20, 2) capped at n. */
int imps_eigs_rs(imps_plan* op, double* x, int mem, double tol, int ncv, int maxit,
                 double* eval, int* n_applies);
/* Operator given by the caller for imps_eigs_rs_op: out = A in on device vectors of length n,
 * enqueued on the context's stream; return < 0 to abort the solve. */
typedef int (*imps_apply_fn)(void* user, const double* in, double* out);
/* eigs_rs(fun, N, vals, vecs, nev, "SA", tol, x0) (eigs.cpp:369-494) for a symmetric operator
 * given as a callback: the nev lowest eigenpairs by the device thick-restart Lanczos.  x holds
 * x0 on entry and the normalised lowest Ritz vector on exit; evals (host, nev); evecs (device,
 * n x nev column-major, optional).  A complex Hermitian operator is passed in its real form on
 * [re; im] (every eigenvalue twice; a Lanczos run from one start vector finds each once). */
int imps_eigs_rs_op(imps_ctx* ctx, int64_t n, imps_apply_fn fn, void* user, double* x, int mem, int nev,
                    double tol, int ncv, int maxit, double* evals, double* evecs, int* n_applies);
/* The lowest nev eigenpairs of P independent symmetric operators at once (Excitations_main.cpp:
 * 255-297 solves one eigs_n per momentum; here all momenta advance together): P thick-restart
 * Lanczos runs in lockstep, every step one callback fn(user, in, out) applying all P operators to
 * P vectors of length n stored one after the other (device).  X (device, P x n): start vectors
 * on entry, the normalised lowest Ritz vector of each system on exit; evals (host, P x nev);
 * converged (host, P, optional).  Returns IMPS_OK when every system converged. */
int imps_eigs_rs_batch_op(imps_ctx* ctx, int P, int64_t n, imps_apply_fn fn, void* user, double* X, int nev,
                          double tol, int ncv, int maxit, double* evals, int* n_applies, int* converged);
/* eigs_n(fun, N, vals, vecs, nev, whch, tol, x0) (eigs.cpp:193-342, real nonsymmetric
 * operator, ARPACK dnaupd/dneupd) on the device: Arnoldi with CGS2 orthogonalisation and a
 * Krylov-Schur restart, convergence as dnaupd (Ritz estimate <= tol max(eps^(2/3), |theta|)),
 * ncv = 0: min(max(20, 2 nev + 1), N), maxit = 0: N restart cycles.  which: IMPS_WHICH_LM
 * (largest modulus), IMPS_WHICH_LR (largest real part), IMPS_WHICH_SR (smallest real part).
 * evals (host, 2 nev doubles: re, im interleaved as std::complex) sorted by `which`, conjugate
 * pairs adjacent (+im first); evecs_re / evecs_im (mem, n x nev column-major, either may be
 * NULL): the Ritz vectors, unit 2-norm, largest-modulus component real and positive.  x0 (mem,
 * n) or NULL for a fixed pseudo-random start.  imps_eigs_n takes any square plan (TM, mixed
 * TM, H_AC, H_C); imps_eigs_n_op an operator callback as imps_eigs_rs_op. */
#define IMPS_WHICH_LM 0
#define IMPS_WHICH_LR 1
#define IMPS_WHICH_SR 2
int imps_eigs_n(imps_plan* op, const double* x0, int mem, int nev, int which, double tol, int ncv, int maxit,
                double* evals, double* evecs_re, double* evecs_im, int* n_applies);
int imps_eigs_n_op(imps_ctx* ctx, int64_t n, imps_apply_fn fn, void* user, const double* x0, int mem, int nev,
                   int which, double tol, int ncv, int maxit, double* evals, double* evecs_re, double* evecs_im,
                   int* n_applies);
/* InvertE_proj (InvEBlockFunctions.hpp:201-266) on a TM plan: solves
 *  dir l: y (1 - T + |R)(L|) = x (1 - |R)(L|),  dir r: (1 - T + |R)(L|) y = (1 - |R)(L|) x
 * with restarted GMRES (Krylov size `krylov`, 0 = 80); y holds y0 on entry (NULL = zeros). */
int imps_invert_e_proj(imps_plan* tm, const double* x, const double* L, const double* R,
                       int dir, double* y, int mem, double tol, int maxit, int krylov,
                       int* iters, double* relres);
/* InvertE_fac(A, B, x, dir, fac) (InvEBlockFunctions.hpp:413-451, operator InvEfun_fac
 * :166-197): solves (1 - fac T) y = x for the mixed TM plan `tmx` (direction fixed by the
 * plan), complex x and y given as separate real / imaginary planes in the plan's in-layout
 * order; y holds y0 on entry.  Restarted GMRES(krylov) on the device (0: 80), stop
 * |r| < tol |b|.  Status 1 = not converged (y returned). */
int imps_invert_e_fac(imps_plan* tmx, const double* x_re, const double* x_im, double fac_re, double fac_im,
                      double* y_re, double* y_im, int mem, double tol, int maxit, int krylov, int* iters,
                      double* relres);
/* InvertE_proj_fac(A, B, x, L, R, dir, fac) (InvEBlockFunctions.hpp:277-330, operator
 * InvEfun_proj_fac :90-125): (1 - fac T + |rho_out)(rho_in|) y = x - tr(x rho_in) rho_out with
 * (rho_in, rho_out) = (R, L) for dir 0, (L, R) for dir 1 (dir must match the plan); L, R are
 * real BlockMats whose blocks pair with x's in order (tr(x rho) = sum_b tr(x_b rho_b)). */
int imps_invert_e_proj_fac(imps_plan* tmx, const double* x_re, const double* x_im, const double* L,
                           const double* R, int dir, double fac_re, double fac_im, double* y_re, double* y_im,
                           int mem, double tol, int maxit, int krylov, int* iters, double* relres);
/* InvertE_fac (InvEBlockFunctions.hpp:346-476) for P systems (1 - f_j T) y_j = x_j at once, one
 * per momentum of the excitation ansatz (Excitations_main.cpp:255-297 runs them one momentum at a
 * time): P restarted GMRES runs in lockstep, each on its own Krylov basis of [re_j; im_j], every
 * iteration applying T to all 2P planes in one launch per stage of `rep`, a plan made by
 * imps_plan_replicate(tm, 2P) from the mixed TM plan.  x_*, y_* (device, P pointers each, n
 * elements): right-hand sides; initial guesses on entry, solutions on exit.  fac_re / fac_im
 * (host, P).  Each system stops at |r_j| <= tol |x_j| (or stagnation, as imps_invert_e_fac);
 * iters: lockstep iterations; relres: the largest relative residual. */
int imps_invert_e_fac_batch(imps_plan* rep, int P, const double* const* x_re, const double* const* x_im,
                            const double* fac_re, const double* fac_im, double* const* y_re, double* const* y_im,
                            double tol, int maxit, int krylov, int* iters, double* relres);
/* TMDominantEig (EigsBlockFunctions.hpp:91-172) for a left/right-isometric unit cell: the
 * dominant eigenvalue is 1 and the fixed point solves (1 - T + |x0)(1|) v = x0; v is
 * normalised to unit trace as in the reference.  x0 may be NULL (identity). */
int imps_tm_dominant(imps_plan* tm, const double* x0, double* V, int mem, double tol,
                     int maxit, double* eval, int* iters);
/* GradNormRight (VUMPS_helpers.hpp:145-153): F = norm_scaled(Y N_R^T), from Y = H_AC(C*AR)
 * already stored in the grad plan's slot 0 and AR in slot 1. */
int imps_grad_norm_right(imps_plan* grad, double* F);

/* ---- transfer-matrix apply without device allocation ------------------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc when they apply
 * the transfer matrix (device memory fully reserved up front by another allocator, or a
 * latency-critical loop that must not pay cudaMalloc's implicit device synchronisation):
 * Y = sum_s A_s^T X A_s (dir 0, as ApplyTMLeft) or sum_s A_s X A_s^T (dir 1, as
 * ApplyTMRight) for one MPS tensor A (layout A, device data A_data) and BlockDiagMat X, Y
 * (layouts in / out, device pointers), launched on cuda_stream.  Scratch and task tables live
 * in fixed file-scope device arrays: A may hold at most 1,048,576 elements (8 MiB of
 * scratch) and each of the two stages at most 8192 output tiles / 8192 GEMM terms; larger
 * problems return IMPS_ERR_TOO_LARGE.  The first call on a device looks up the arrays'
 * device address (do it before any stream capture).  All calls share the arrays: calls that
 * overlap on the GPU race, and calls from several host threads must be serialised. */
int imps_tm_apply_noalloc(const imps_layout* A, const imps_layout* in, const imps_layout* out, int dir,
                          const double* A_data, const double* X, double* Y, void* cuda_stream);

/* ---- per-sector decompositions ------------------------------------------------------------ */
/* Sector tables of GetDenseMat (MPSBlockMat.hpp:468-526): dir l groups blocks by outgoing
 * charge (rows stacked over s), dir r by incoming charge (columns stacked over s).  A is an
 * MPS layout or a BlockDiagMat layout.  Derived layout 0 = A's layout (Q / isometry),
 * derived layout 1 = BlockDiagMat over the sectors (R / DiagIso). */
int imps_plan_decomp(imps_ctx* ctx, const imps_layout* A, int dir, imps_plan** out);
/* qr(R, MPS, dir) / qr(R, BlockDiagMat, dir) with qr_pos sign convention, diag(R) >= 0
 * (MPSBlockUtilities.hpp:181-244, BlockObj.hpp:2422-2459, helpers.hpp:181-195).  Device
 * pointers only; every sector needs stacked dimension >= sector dimension. */
int imps_sector_qr(imps_plan* dec, const double* A, double* Q, double* R, int mem);
/* Nullspace(A, l) (MPSBlockUtilities.hpp:247-300) on a dir-l decomposition plan of a
 * left-isometric A: N_L (layout: imps_plan_derived_layout(plan, 2)) with orthonormal columns
 * orthogonal to A's, per right sector (sectors without a null space omitted).  Device memory. */
int imps_sector_nullspace(imps_plan* plan, const double* A, double* NL, int mem);
/* svd(S, DiagIso, MPS, dir) (MPSBlockUtilities.hpp:78-153): U = MPSIso (A's layout), S =
 * singular values per sector concatenated in sector order (descending), Viso = DiagIso
 * (V^T for dir l, U for dir r).  Any output may be NULL.  Column-pivoted QR, then one-sided
 * Jacobi on R^T (first sweeps in FP32, finished and tested in FP64); FP64 results. */
int imps_sector_svd(imps_plan* dec, const double* A, double* U, double* S, double* Viso, int mem);
/* Several independent sector SVDs (each as imps_sector_svd, on its own decomposition plan of
 * one context; at most 4) in one launch: the two polar steps of a site update,
 * svd(AC CR^T, l) and svd(CL^T AC, r) (VUMPS_main.cpp:213-220), fill twice the SMs of one.
 * Arrays of np pointers; entries of U, S, Viso may be NULL. */
int imps_sector_svd_batch(int np, imps_plan* const* plans, const double* const* A, double* const* U,
                          double* const* S, double* const* Viso, int mem);
/* X_q[:, j] *= S_q[j]^power on a BlockDiagMat decomposition plan (BlockDiagMat << BlockLam,
 * BlockObj.hpp:2316), e.g. U * sqrt(S) in randMPS_LR (MPSBlockUtilities.hpp:1116-1118) */
int imps_sector_colscale(imps_plan* dec, double* X, const double* S, double power, int mem);

/* ---- Krylov BLAS-1 (K5) and device-vector helpers for drivers ---------------------------- */
int imps_dot(imps_ctx* ctx, const double* x, const double* y, int64_t n, double* result);
/* sum over BlockDiagMat sectors of trace(X_q * Y_q) (InvEBlockFunctions.hpp:28-33) */
int imps_bd_trace_prod(imps_ctx* ctx, imps_layout* L, const double* X, const double* Y,
                       double* result);
/* max_i |x_i| (norm_inf, helpers.hpp:148-151) */
int imps_absmax(imps_ctx* ctx, const double* x, int64_t n, double* result);
/* y = a*x + b*y */
int imps_axpby(imps_ctx* ctx, double a, const double* x, double b, double* y, int64_t n);
/* x /= sign(x[0]) (VUMPS_main.cpp:201-202) */
int imps_sign_normalize(imps_ctx* ctx, double* x, int64_t n);

#ifdef __cplusplus
}
#endif
#endif /* IMPS_GB300_H */
