/*
 * sl1x1.h -- C ABI of libsl1x1gpu.so, a GB300 (sm_103a) implementation of
 * ScaLAPACK's dense LU path on a 1x1 BLACS grid.
 *
 * The Fortran-callable entry points keep the reference's names, argument
 * order and meaning (gfortran "Add_" mangling, all arguments by reference,
 * 32-bit INTEGER, hidden CHARACTER lengths last), so a program linked against
 * ScaLAPACK can link against this library instead when it runs on one process
 * with one GPU.  Every call computes on the GPU; there is no CPU fallback.
 *
 * Descriptor layout (DLEN_ = 9, SRC/pdgetrf.f:137-141, TOOLS/descinit.f:177-186):
 *   DESC = { DTYPE_=1, CTXT_, M_, N_, MB_, NB_, RSRC_, CSRC_, LLD_ }
 *
 * INFO conventions (as the reference, plus one class for the GPU):
 *   INFO = 0       success
 *   INFO = -i      the i-th scalar argument is illegal
 *   INFO = -(i*100+j)  entry j of the i-th (array) argument is illegal
 *   INFO = K > 0   U(K,K) is exactly zero (factorization completed)
 *   INFO <= -10000 GPU failure: -10000 - cudaError_t for a CUDA runtime error,
 *                  -20000 - s for a device status s (2: a bounded wait on
 *                  data another CTA publishes timed out), -30000 when the
 *                  problem exceeds a documented size limit of the GPU path.
 */
#ifndef SL1X1_H
#define SL1X1_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- ScaLAPACK LU driver and computational routines ---------------------- */

/* Replaces PDGETRF, SRC/pdgetrf.f:1-312 (signature at :1-2). */
void pdgetrf_(const int* M, const int* N, double* A, const int* IA, const int* JA,
              const int* DESCA, int* IPIV, int* INFO);

/* Replaces PDGETRS, SRC/pdgetrs.f:1-292 (signature at :1-2). TRANS = 'N','T','C'. */
void pdgetrs_(const char* TRANS, const int* N, const int* NRHS, const double* A, const int* IA,
              const int* JA, const int* DESCA, const int* IPIV, double* B, const int* IB,
              const int* JB, const int* DESCB, int* INFO, size_t TRANS_len);

/* Replaces PDGESV, SRC/pdgesv.f:1-245 (signature at :1-2). */
void pdgesv_(const int* N, const int* NRHS, double* A, const int* IA, const int* JA,
             const int* DESCA, int* IPIV, double* B, const int* IB, const int* JB,
             const int* DESCB, int* INFO);

/* ---- Routines on the LU factors ------------------------------------------ */

/* Replaces PDLANGE, SRC/pdlange.f:1: 'M' max |a|, '1'/'O' max column sum,
 * 'I' max row sum, 'F'/'E' Frobenius norm of sub(A), computed on the GPU
 * (NaN if no GPU is usable). */
double pdlange_(const char* NORM, const int* M, const int* N, const double* A, const int* IA,
                const int* JA, const int* DESCA, double* WORK, size_t NORM_len);

/* Replaces PDGECON, SRC/pdgecon.f:1-2: reciprocal condition number estimate
 * (1-norm or infinity-norm) from the LU factors of PDGETRF, with the same
 * validation, workspace query (LWORK/LIWORK = -1) and quick returns. */
void pdgecon_(const char* NORM, const int* N, const double* A, const int* IA, const int* JA,
              const int* DESCA, const double* ANORM, double* RCOND, double* WORK,
              const int* LWORK, int* IWORK, const int* LIWORK, int* INFO, size_t NORM_len);

/* Replaces PDGETRI, SRC/pdgetri.f:1-2: inverse of sub(A) from the LU factors
 * and pivots of PDGETRF; INFO = i > 0 when U(i,i) is exactly zero. */
void pdgetri_(const int* N, double* A, const int* IA, const int* JA, const int* DESCA,
              const int* IPIV, double* WORK, const int* LWORK, int* IWORK, const int* LIWORK,
              int* INFO);

/* ---- Expert driver and its parts (refinement, error bounds, scaling) ----- */

/* Replaces PDGERFS, SRC/pdgerfs.f:1-4: iterative refinement of X for
 * op(sub(A)) X = sub(B) with the factors of PDGETRF, the componentwise
 * backward error BERR and the forward error bound FERR of every column (FERR
 * and BERR indexed from JB, as the reference does). Same argument checks,
 * workspace query and N <= 1 quick return; residuals, solves and the norm
 * estimate run on the GPU. */
void pdgerfs_(const char* TRANS, const int* N, const int* NRHS, const double* A, const int* IA,
              const int* JA, const int* DESCA, const double* AF, const int* IAF, const int* JAF,
              const int* DESCAF, const int* IPIV, const double* B, const int* IB, const int* JB,
              const int* DESCB, double* X, const int* IX, const int* JX, const int* DESCX,
              double* FERR, double* BERR, double* WORK, const int* LWORK, int* IWORK,
              const int* LIWORK, int* INFO, size_t TRANS_len);

/* Replaces PDGESVX, SRC/pdgesvx.f:1-4: FACT = 'E' equilibrates (PDGEEQU,
 * PDLAQGE), 'N' or 'E' factors into AF, 'F' takes AF and IPIV; then RCOND
 * (PDLANGE + PDGECON; INFO = IA+N when RCOND < eps), PDGETRS, PDGERFS and the
 * back-transformation of X and FERR. One deliberate difference: with
 * FACT = 'F', TRANS = 'N' and EQUED = 'C' or 'B' the reference multiplies X
 * by a workspace that it never filled with C; this library multiplies by C. */
void pdgesvx_(const char* FACT, const char* TRANS, const int* N, const int* NRHS, double* A,
              const int* IA, const int* JA, const int* DESCA, double* AF, const int* IAF,
              const int* JAF, const int* DESCAF, int* IPIV, char* EQUED, double* R, double* C,
              double* B, const int* IB, const int* JB, const int* DESCB, double* X, const int* IX,
              const int* JX, const int* DESCX, double* RCOND, double* FERR, double* BERR,
              double* WORK, const int* LWORK, int* IWORK, const int* LIWORK, int* INFO,
              size_t FACT_len, size_t TRANS_len, size_t EQUED_len);

/* Replaces PDGEEQU, SRC/pdgeequ.f:1-2: row scale factors R(IA:IA+M-1) and
 * column scale factors C(JA:JA+N-1) that bring the largest entry of every row
 * and column of diag(R) sub(A) diag(C) to 1; INFO = i (zero row) or M+j (zero
 * column). Computed on the GPU; bit-identical to the reference's arithmetic. */
void pdgeequ_(const int* M, const int* N, const double* A, const int* IA, const int* JA,
              const int* DESCA, double* R, double* C, double* ROWCND, double* COLCND,
              double* AMAX, int* INFO);

/* Replaces PDLAQGE, SRC/pdlaqge.f:1-2: scales sub(A) by R and/or C when
 * ROWCND, COLCND and AMAX call for it (threshold 0.1) and reports EQUED. */
void pdlaqge_(const int* M, const int* N, double* A, const int* IA, const int* JA,
              const int* DESCA, const double* R, const double* C, const double* ROWCND,
              const double* COLCND, const double* AMAX, char* EQUED, size_t EQUED_len);

/* ---- Redistribution in front of the LU (REDIST) ------------------------- */

/* Replaces PDGEMR2D, REDIST/SRC/pdgemr.c:1-20 (SUBROUTINE PDGEMR2D(M, N, A,
 * IA, JA, DESCA, B, IB, JB, DESCB, ICTXT)): copies sub(A) into sub(B). This
 * library's contexts are 1x1 grids, so on one process it is a submatrix copy
 * between two descriptors; a process outside a context passes CTXT = -1 for
 * it. Between processes, the sl1x1_redist_* pieces below do the per-pair work
 * and a transport moves the buffers. */
void pdgemr2d_(const int* M, const int* N, const double* A, const int* IA, const int* JA,
               const int* DESCA, double* B, const int* IB, const int* JB, const int* DESCB,
               const int* ICTXT);

/* Redistribution between two 2D block-cyclic layouts, one process pair at a
 * time (no counterpart symbol in the reference; it is the pack / unpack step
 * of PDGEMR2D). sub(A) = A(ia:ia+m-1, ja:ja+n-1) laid out by desca on a
 * p0 x q0 grid, sub(B) by descb on a p1 x q1 grid; (sr, sc) is the source
 * process in A's grid, (dr, dc) the destination in B's. The buffer holds the
 * elements of sub(A) owned by both, column-major in submatrix coordinates.
 * Each returns the element count (-1 for an invalid descriptor or grid). */
long long sl1x1_redist_count(int m, int n, int ia, int ja, const int* desca, int p0, int q0,
                             int sr, int sc, int ib, int jb, const int* descb, int p1, int q1,
                             int dr, int dc);
/* Copies the pair's elements from the source's local array A into buf. */
long long sl1x1_redist_pack(int m, int n, int ia, int ja, const int* desca, int p0, int q0, int sr,
                            int sc, int ib, int jb, const int* descb, int p1, int q1, int dr,
                            int dc, const double* A, double* buf);
/* Copies buf into the destination's local array B. */
long long sl1x1_redist_unpack(int m, int n, int ia, int ja, const int* desca, int p0, int q0,
                              int sr, int sc, int ib, int jb, const int* descb, int p1, int q1,
                              int dr, int dc, const double* buf, double* B);

/* ---- TOOLS used by callers of the LU path ------------------------------- */

/* Replaces DESCINIT, TOOLS/descinit.f:1-192. */
void descinit_(int* DESC, const int* M, const int* N, const int* MB, const int* NB,
               const int* IRSRC, const int* ICSRC, const int* ICTXT, const int* LLD, int* INFO);

/* Replaces NUMROC, TOOLS/numroc.f:1-82. */
int numroc_(const int* N, const int* NB, const int* IPROC, const int* ISRCPROC,
            const int* NPROCS);

/* ---- 1x1 BLACS shim (replaces the BLACS/SRC entry points named) ---------- */
/* A context is valid only for a 1x1 grid; BLACS_GRIDINFO on any other
 * context returns NPROW = NPCOL = MYROW = MYCOL = -1, which the LU routines
 * report as INFO = -(600+CTXT_) / -(700+CTXT_) like the reference. */
void blacs_pinfo_(int* MYPNUM, int* NPROCS);                         /* BLACS/SRC/blacs_pinfo_.c:6 */
void blacs_get_(const int* ICTXT, const int* WHAT, int* VAL);        /* BLACS/SRC/blacs_get_.c */
void blacs_gridinit_(int* ICTXT, const char* ORDER, const int* NPROW, const int* NPCOL,
                     size_t ORDER_len);                              /* BLACS/SRC/blacs_init_.c:6 */
void blacs_gridinfo_(const int* ICTXT, int* NPROW, int* NPCOL, int* MYROW,
                     int* MYCOL);                                    /* BLACS/SRC/blacs_info_.c:6 */
void blacs_gridexit_(const int* ICTXT);                              /* BLACS/SRC/blacs_grid_.c */
void blacs_exit_(const int* CONTINUE);                               /* BLACS/SRC/blacs_exit_.c */

/* ---- Device-resident C entry points ------------------------------------ */
/* Same semantics as PDGETRF/PDGETRS on a whole matrix (IA=JA=1), with the
 * matrix already in GPU memory: dA is m x n column-major with leading
 * dimension ldda, dipiv receives min(m,n) 1-based pivot rows (LAPACK/ScaLAPACK
 * convention for IA=1), stream is a cudaStream_t (NULL = legacy default).
 * Returns INFO. The call returns after the work on `stream` has finished. */
int sl1x1_dgetrf_dev(int m, int n, double* dA, long long ldda, int* dipiv, int nb, void* stream);
int sl1x1_dgetrs_dev(char trans, int n, int nrhs, const double* dA, long long ldda,
                     const int* dipiv, double* dB, long long lddb, void* stream);
int sl1x1_dgesv_dev(int n, int nrhs, double* dA, long long ldda, int* dipiv, double* dB,
                    long long lddb, int nb, void* stream);

/* Low-precision trailing update on device data, the PDGEMM step of the
 * mixed-precision factorization: C (m x n) -= L (m x k) * U (k x n), FP32
 * column-major, with L and U rounded to BF16 (fmt 0) or FP16 (fmt 1) -- U per
 * column scaled by a power of two -- multiplied on tcgen05 tensor cores with
 * FP32 accumulation. Returns 0 or a negative INFO. */
int sl1x1_lowp_update_dev(int fmt, int m, int n, int k, const float* dL, long long ldl,
                          const float* dU, long long ldu, float* dC, long long ldc, void* stream);

/* Mixed-precision solve with iterative refinement (no routine of this form
 * exists in the reference; the interface follows LAPACK DSGESV). A (FP64,
 * n x n, device) is factored in FP32 with the trailing updates on tcgen05
 * tensor cores in BF16 (fmt 0), FP16 (fmt 1) or split BF16x3 (fmt 2) with FP32
 * accumulation; X is
 * refined in FP64 (classical refinement, then GMRES-IR when a step fails to
 * halve the scaled residual) until ||b-Ax||/(||A|| ||x|| N eps) <= tol
 * (tol <= 0: 1.0). If refinement stalls (a classical step that does not
 * halve the scaled residual, then a GMRES-IR step that does not cut it by
 * 10 %), or when GMRES's convergence rate predicts more remaining time than
 * the plain FP64 solve would take (estimated as 3.5 x the measured
 * low-precision factorization time), the FP64 factorization is used.
 * dipiv receives the pivots of the factorization that produced X (0-based
 * rows). keep_a = 1 keeps A intact in every case (an FP64 copy is made for the
 * fallback); keep_a = 0 lets the fallback factor A in place (DSGESV).
 * *iter (DSGESV convention): >= 0 refinement steps taken; -1 the low-precision
 * factorization failed; -3 refinement did not converge (fallback used).
 * stats[8] = {classical steps, GMRES-IR outer steps, GMRES inner iterations,
 * fell back (0; 1 after a stall; 2 on the predicted cost), final scaled
 * residual, ||A||_inf, factor ms, refine ms}.
 * Returns INFO (> 0: A is exactly singular in FP64). */
int sl1x1_dgesv_ir_dev(int n, int nrhs, double* dA, long long ldda, int* dipiv, const double* dB,
                       long long lddb, double* dX, long long lddx, int fmt, int nb, double tol,
                       int keep_a, int* iter, double* stats, void* stream);

/* Cost rule of sl1x1_dgesv_ir_dev: the plain FP64 solve is estimated at
 * `ratio` times the measured low-precision factorization time (default 3.5,
 * the ratio measured at N=32768 on GB300); refinement falls back to it once
 * GMRES's convergence rate predicts a longer remaining time. ratio <= 0 turns
 * the rule off (refinement then stops only on a stall). No counterpart in the
 * reference. */
void sl1x1_set_ir_cost_ratio(double ratio);

/* ---- Batched solver (no single routine of the reference; each system is a
 * PDGESV on a 1x1 grid). A plan describes `batch` independent systems
 * A_i X_i = B_i with 1 <= n[i] <= 512 and 1 <= nrhs[i] <= 8, each A_i, B_i,
 * X_i a column-major device array (host arrays of device pointers and leading
 * dimensions). A_i and B_i are not modified. mode 0 factors and solves in
 * FP64; mode 1 factors in FP32 and refines in FP64 until the scaled residual
 * ||b-Ax||/(||A|| ||x|| n eps) <= tol (tol <= 0: 1.0), re-solving in FP64 any
 * system that does not get there in 10 steps. Plan creation sorts the systems
 * by size, allocates the workspace, optionally autotunes the kernel shape
 * (threads per CTA, GEMM column chunk, CTAs per SM) on this batch, and
 * captures the execution (one persistent launch per pass) in a CUDA graph.
 * Results per system: INFO (> 0: exactly singular), refinement steps (-1:
 * solved by the FP64 pass after refinement stalled) and the scaled residual. */
typedef struct sl1x1_batch_plan_s* sl1x1_batch_plan;
int sl1x1_batch_plan_create(sl1x1_batch_plan* plan, int batch, const int* n, const int* nrhs,
                            const double* const* dA, const int* lda, const double* const* dB,
                            const int* ldb, double* const* dX, const int* ldx, int mode, double tol,
                            int autotune, void* stream);
int sl1x1_batch_plan_execute(sl1x1_batch_plan plan, void* stream);
int sl1x1_batch_plan_results(sl1x1_batch_plan plan, int* info, int* iters, double* sresid,
                             void* stream);
int sl1x1_batch_plan_shape(sl1x1_batch_plan plan, int* threads, int* chunk, int* ctas_per_sm);
void sl1x1_batch_plan_destroy(sl1x1_batch_plan plan);

/* Allocation-free FP64 LU (no counterpart in the reference): the
 * factorization of sl1x1_dgetrf_dev for callers that may not allocate GPU
 * memory (memory pools or arenas that own the device heap, loops that must not
 * allocate after start-up). Its scratch is a static 1 MiB device array held by
 * every GPU that loads this library until exit; the sliced tensor-core update,
 * whose scratch grows with the matrix, does not fit there, so this entry point
 * always runs the FP64 DMMA update: its factors, pivots and INFO are those of
 * sl1x1_dgetrf_dev with sl1x1_set_f64_update(0), and agree with the default
 * (sliced) factorization to rounding, with the same pivots.
 * The first call on a device looks up that array's address (make it before
 * any stream capture); every call reads its status back and synchronizes its
 * stream before it returns; calls whose GPU work overlaps race on the shared
 * array. M above (SMs of the device) x 768 rows (152 x 768 on GB300) is
 * rejected with -30000 before any launch. */
int sl1x1_dgetrf_noalloc(int m, int n, double* dA, long long ldda, int* dipiv, int nb,
                         void* stream);

/* Device forms of PDLANGE, PDGECON and PDGETRI (dipiv 1-based, as returned
 * by sl1x1_dgetrf_dev). dgecon/dgetri return INFO. */
double sl1x1_dlange_dev(char norm, int m, int n, const double* dA, long long ldda, void* stream);
int sl1x1_dgecon_dev(char norm, int n, const double* dLU, long long ldda, double anorm,
                     double* rcond, void* stream);
int sl1x1_dgetri_dev(int n, double* dA, long long ldda, const int* dipiv, void* stream);
/* PDGEEQU on device data: dR (m) and dC (n) device arrays, scalars on the
 * host; returns INFO as PDGEEQU. */
int sl1x1_dgeequ_dev(int m, int n, const double* dA, long long ldda, double* dR, double* dC,
                     double* rowcnd, double* colcnd, double* amax, void* stream);
/* PDGERFS on device data (dipiv 1-based as LAPACK); ferr and berr are host
 * arrays of nrhs entries. Returns 0 or a negative INFO. */
int sl1x1_dgerfs_dev(char trans, int n, int nrhs, const double* dA, long long ldda,
                     const double* dAF, long long lddaf, const int* dipiv, const double* dB,
                     long long lddb, double* dX, long long lddx, double* ferr, double* berr,
                     void* stream);

/* ---- Library control ----------------------------------------------------- */
/* Free every device buffer the library holds (also done by blacs_exit_). */
void sl1x1_finalize(void);
/* Block size NB used by the device entry points when nb <= 0 (default 256). */
void sl1x1_set_default_nb(int nb);
/* Look-ahead in the factorizations (default on): the next panel is factored
 * on a second stream while the trailing update runs. Same pivots (except
 * where two candidates tie to rounding) and factors equal to rounding either
 * way: the U12 solve balances its slices by the columns it is given. */
void sl1x1_set_lookahead(int on);
/* Split look-ahead step (default on; needs the look-ahead): after each panel,
 * the panel's stream brings the next panel's columns up to date itself
 * (interchanges, U12 solve, update) and factors it, while the caller's stream
 * handles the other columns. Results as for sl1x1_set_lookahead. */
void sl1x1_set_split_step(int on);
/* Column chunks of A's host-to-device copy in pdgetrf_ / pdgesv_ (1..16,
 * default 8; 1 = one copy before the factorization): with more than one, A
 * goes over in chunks of whole panels on a copy stream and step 0 of the
 * factorization (panel 0, then its interchanges, U12 solve and update chunk by
 * chunk) starts as soon as its columns are in place. Same results either way. */
void sl1x1_set_copy_chunks(int chunks);
/* Test hook for the failure paths: the k-th next growth of a library-owned
 * device buffer (k = 0: the next one) fails as if the device were out of
 * memory, without allocating; the hook then disarms itself (k < 0 disarms it
 * at once). Calls that need the buffer return INFO = -10002
 * (-10000 - cudaErrorMemoryAllocation) and leave the library usable; the
 * sliced-product scratch and the solve's block inverses are optional, and
 * without them the FP64 DMMA update and the substitution solves run instead.
 * Returns the hook's previous state: -1 once it has fired (or when it was
 * off), else the growths it was still waiting for. */
int sl1x1_debug_fail_alloc(int k);
/* SMs that the factorization's look-ahead trailing update leaves free for
 * the next panel's kernels: at least min_sms (default 24: the panel kernel's
 * CTAs must all be resident to make progress) and, when the update is small
 * enough to finish within about one panel period on fewer SMs, up to max_sms
 * (default 88). (0, 0) lets the update take every SM. Values are clamped to
 * 0..120. Changes only the speed. */
void sl1x1_set_update_reserve(int min_sms, int max_sms);
/* The estimate behind that rule: sliced-product flops one SM takes within a
 * panel period (default 3.2e8; larger values leave the panel more SMs; <= 1e6
 * restores the default). Changes only the speed. */
void sl1x1_set_update_share(double flops_per_sm);
/* Grid caps of the split look-ahead step, a bit mask (default 7): 1 the
 * next panel's in-panel sliced products and 2 its update keep to the SMs the
 * trailing update beside them leaves (each CTA then loops over more tiles);
 * 4 the caller's stream's U12 solve and row interchanges keep to the
 * update's own SMs. Changes only the speed. */
void sl1x1_set_inpanel_cap(int mask);
/* Test hook for the bounded device waits: the number of polls a panel CTA
 * makes for another CTA's published pivot candidates before it gives up
 * (polls < 0 restores the default, 2^24; 0 makes every wait run out at its
 * first poll). A panel that gives up records a device timeout, writes the
 * identity for the pivots it has not chosen and returns; the call then
 * returns INFO = -20002 and the library stays usable. No counterpart in the
 * reference, whose panel has no device waits. */
void sl1x1_debug_set_spin_limit(long long polls);
/* Smallest row slice per CTA of the cooperative panel kernel (8..768; 0, the
 * default, picks 256 rows for the FP32 panel and 128 for the FP64 one, with
 * about 64 CTAs for tall panels): larger slices mean fewer CTAs in each
 * column's pivot exchange but a longer rank-1 update per CTA. Changes only the
 * speed, not the results. */
void sl1x1_set_panel_rows(int rows);
/* CTAs (8..224, default 64) that the cooperative panel kernel spreads a tall
 * panel's rows over, before the minimum slice above applies. Changes only the
 * speed, not the results. */
void sl1x1_set_panel_ctas(int ctas);
/* 32-column sub-panels per in-panel block of the FP64 panel factorization
 * (1..8, default 2): inside a block only the next sub-panel's columns are
 * updated after each sub-panel, the columns beyond the block once at its end.
 * Same pivots except where candidates tie to rounding; factors equal to
 * rounding. */
void sl1x1_set_panel_ib(int subpanels);
/* Pipeline depth of the tcgen05 low-precision update used by the mixed
 * factorization and sl1x1_lowp_update_dev: 2 (default; two CTAs per SM, one's
 * epilogue overlapping the other's main loop) or 3 (one CTA per SM). Changes
 * only the speed, not the results. */
void sl1x1_set_lowp_stages(int stages);
/* Arithmetic of the FP64 factorization's trailing update (PDGEMM step of
 * SRC/pdgetrf.f:288-290): 1 (default) = the product formed exactly on the
 * BF16 tensor cores (tcgen05) from 7-bit integer slices of the operands (8
 * slices, row and column power-of-two scales, diagonals d <= 6 of the slice
 * products summed exactly as integers), accurate to a few units of 2^-53 of
 * max|L21(i,:)| max|U12(:,j)| and independent of the summation order; 0 =
 * FP64 DMMA (mma.sync m16n8k4). The sliced form needs device scratch of about
 * 4 KB per row plus 4 KB per column of the matrix; where it cannot be had
 * (sl1x1_dgetrf_noalloc) the DMMA form runs. */
void sl1x1_set_f64_update(int mode);
int sl1x1_get_f64_update(void);
/* Output tiles (128 x 64) each CTA of the sliced product takes in turn
 * (default 4; 1..4096): more overlap one tile's epilogue with the next
 * tile's products, fewer free SMs more often for the look-ahead panel's
 * kernels. Changes only the speed, not the results. */
void sl1x1_set_ozgemm_tiles(int tiles_per_cta);
/* dC (m x n) += alpha * dA (m x k) * dB (k x n), FP64, column-major device
 * arrays, through the sliced tensor-core product above (any k: passes of 256).
 * Returns 0, -i for an illegal i-th argument, <= -10000 for a CUDA error,
 * <= -20000 for a device timeout. */
int sl1x1_ozgemm_dev(int m, int n, int k, double alpha, const double* dA, long long ldda,
                     const double* dB, long long lddb, double* dC, long long lddc, void* stream);
/* Passes of the sliced FP64 product (trailing updates, U12 and PDGETRS
 * products, sl1x1_ozgemm_dev) that the error-budget test sent to the FP64
 * route on the current device since the library was loaded; -1 if the count
 * cannot be read. Operands whose large entries a power-of-two balancing along
 * k cannot line up take that route (no counterpart in the reference, whose
 * DGEMM is FP64 throughout). */
long long sl1x1_ozgemm_fp64_routes(void);
/* 1 if the library found a usable sm_103 device, else 0. */
int sl1x1_device_ok(void);
/* Version string. */
const char* sl1x1_version(void);

/* ---- Phase timers (the GPU counterpart of SLTIMER, TOOLS/sltimer.f:47) ---- */
/* Phases: 0 panel (PDGETF2), 1 row interchanges (PDLASWP), 2 U12 solve
 * (PDTRSM), 3 trailing update (PDGEMM, FP64), 4 solve (PDGETRS), 5 mixed
 * trailing update, 6 mixed panel, 7 refinement, 8 batched solver.
 * sl1x1_prof_enable(1) clears and starts event timing of every phase launch;
 * sl1x1_prof_read returns launches, summed device milliseconds and the
 * algorithmic flops and bytes of a phase (0 on success). */
void sl1x1_prof_enable(int on);
int sl1x1_prof_read(int phase, long long* launches, double* ms, double* flops, double* bytes);
/* Number of kernels this library has launched since it was loaded. */
long long sl1x1_launch_count(void);
/* FP64 tensor (DMMA) throughput of this device from a register-only loop,
 * TFLOP/s: the roofline denominator of the FP64 trailing update. */
double sl1x1_dmma_peak_tflops(void);

#ifdef __cplusplus
}
#endif

#endif /* SL1X1_H */
