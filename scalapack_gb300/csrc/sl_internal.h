// Internal interfaces shared by the sl1x1 translation units (not exported).
#pragma once
#include <cuda_runtime.h>

#include <functional>
#include <stddef.h>

#ifndef SL_TRY
#define SL_TRY(x)                     \
  do {                                \
    cudaError_t _e = (x);             \
    if (_e != cudaSuccess) return _e; \
  } while (0)
#endif

namespace sl {

int num_sms();

// ---- phase timers and launch counter (prof.cpp) ----
enum Phase {
  kPhPanel = 0,   // PDGETF2: sub-panel kernels and the in-panel swap/solve/update
  kPhLaswp = 1,   // PDLASWP on the left and right column blocks
  kPhTrsm = 2,    // PDTRSM for the U12 block row
  kPhGemm = 3,    // PDGEMM trailing update (sliced FP64 product, or FP64 DMMA)
  kPhSolve = 4,   // PDGETRS
  kPhMixedGemm = 5,  // low-precision trailing update (tcgen05)
  kPhMixedPanel = 6, // FP32 panel, swaps and solves of the mixed factorization
  kPhRefine = 7,     // FP64 residuals, corrections and GMRES of the refinement
  kPhBatched = 8,    // batched solver
  kPhResidual = 9,   // FP64 residuals and matrix-vector products of the refinement
  kPhPrecond = 10,   // low-precision solves applied during the refinement
  // parts of kPhPanel (timed inside it): the cooperative sub-panel kernels,
  // the in-panel interchanges, strip solves and sliced products, and the
  // inverse of L11 with the interchange plan
  kPhPanelKernel = 11,
  kPhPanelUpdate = 12,
  kPhPanelInverse = 13,
  kNumPhases = 14
};
void count_launches(int n);
void phase_begin(int phase, cudaStream_t s);
void phase_end(int phase, cudaStream_t s, double flops, double bytes);
void prof_enable(bool on);
bool prof_read(int phase, long long* launches, double* ms, double* flops, double* bytes);
long long launch_count();

// Scratch for the split-K partials of long skinny products (grown by the
// library with the refinement workspace; a null pointer disables split-K).
struct SplitKScratch {
  void* ptr = nullptr;
  size_t bytes = 0;
};
SplitKScratch& splitk_scratch();

// Scratch of the sliced FP64 product (ozgemm_f64.cu): BF16 slices of both
// operands and their row / column scales. One per stream that runs products
// concurrently; when it is absent or too small the DMMA product is used.
struct OzScratch {
  void* ptr = nullptr;
  size_t bytes = 0;
};
size_t oz_scratch_bytes(int m, int n, int k);
// Output tiles each CTA of the sliced product takes in turn (default 4).
void oz_set_tiles_per_cta(int t);
bool oz_fits(const OzScratch& sc, int m, int n, int k);
// C (m x n) += alpha * A (m x k) * B (k x n), FP64, column-major, on the BF16
// tensor cores through exact 7-bit slices (needs oz_fits), balanced by the
// column maxima of A; a pass whose slices would exceed the error budget is
// computed in FP64 arithmetic by the same launches. B may alias C (same
// pointer and leading dimension): the slices are cut before C is written, and
// the FP64 route takes whole column blocks per CTA.
// max_ctas > 0 caps the grid (each CTA then takes more tiles), leaving SMs
// to concurrent streams.
cudaError_t oz_dgemm(const OzScratch& sc, int m, int n, int k, double alpha, const double* A,
                     long long lda, const double* B, long long ldb, double* C, long long ldc,
                     int* status, cudaStream_t s, int max_ctas = 0);
// The same balanced by the row maxima of B, with the budget tested per
// column: for A = inv(T) - I of a unit-lower diagonal block T and B the rows
// it updates (the U12 solve), whose rows carry the pivots' scales.
cudaError_t oz_dgemm_bside(const OzScratch& sc, int m, int n, int k, double alpha,
                           const double* A, long long lda, const double* B, long long ldb,
                           double* C, long long ldc, int* status, cudaStream_t s, int max_ctas = 0);
// The same (side A) with the balancing keys of its single pass (k <= 256)
// already published with `epoch` (from oz_new_epoch) into oz_ckeys(sc) and
// oz_hkeys(sc) by the kernels that produced A and B: one launch fewer.
cudaError_t oz_dgemm_keyed(const OzScratch& sc, unsigned long long epoch, int m, int n, int k,
                           double alpha, const double* A, long long lda, const double* B,
                           long long ldb, double* C, long long ldc, int* status, cudaStream_t s,
                           int max_ctas = 0);
unsigned long long oz_new_epoch();
unsigned long long* oz_ckeys(const OzScratch& sc);
unsigned long long* oz_hkeys(const OzScratch& sc);
// Sliced-product passes that took the FP64 route on the current device.
long long oz_fp64_routes();
// Trailing-update arithmetic of the FP64 factorization: 0 = FP64 DMMA,
// 1 = sliced BF16 tensor-core product (when its scratch is present).
void f64_update_set(int mode);
int f64_update_get();

// Register-only DMMA throughput loop (FP64 tensor peak calibration), TFLOP/s.
double dmma_peak_tflops(cudaStream_t s);

// C = alpha * op(A) * B + beta * C, FP64, column-major (dgemm_f64.cu).
cudaError_t dgemm(bool transa, int m, int n, int k, double alpha, const double* A, long long lda,
                  const double* B, long long ldb, double beta, double* C, long long ldc,
                  cudaStream_t s);

// Device workspace used by the FP64 factorization / solve (sized by the
// caller through lu_workspace_bytes).
struct LuWork {
  int* status;       // 1 int: device status word (DevStatus)
  int* info_col;     // 1 int: first zero-pivot column (0-based), INT_MAX if none
  double* cand;      // exchange area of the panel kernel (kPanelCandDoubles words)
  int* swap_plan = nullptr;  // kSwapPlanInts: composite form of a panel's interchanges
  int* perm;         // n ints: composed row permutation (solve)
  double* bswap;     // n * nrhs doubles: gathered right-hand sides (solve)
  size_t perm_len;
  size_t bswap_len;
  // Look-ahead resources (null: the factorization runs on the caller's
  // stream only): a high-priority stream for the next panel and two events.
  cudaStream_t aux = nullptr;
  cudaEvent_t ev_next = nullptr;
  cudaEvent_t ev_panel = nullptr;
  // Sliced-product scratch for the caller's stream and for the panel's
  // stream, and 64x64 FP64 blocks for the U12 solve (kDinv64Doubles).
  OzScratch oz, oz_aux;
  double* dinv64 = nullptr;
  // Solve: inverses of the 64x64 diagonal blocks of L then of U
  // (kSolveInvDoubles(n) doubles), or null for the substitution solves.
  double* dinv_solve = nullptr;
  size_t dinv_solve_len = 0;
  // Columns still arriving (ncol_chunks = 0: all of A is in place). Chunk c
  // holds columns [c ? col_end[c-1] : 0, col_end[c]) and is in place once
  // ev_cols[c] has completed; step 0 of the factorization follows the chunks
  // (needs the look-ahead resources and dinv64_step0, a second
  // kDinv64Doubles block; otherwise the factorization waits for all of them).
  int ncol_chunks = 0;
  const int* col_end = nullptr;
  const cudaEvent_t* ev_cols = nullptr;
  double* dinv64_step0 = nullptr;
  // Rows of panels taller than the SMs' shared memory holds (FP64; null: such
  // panels are rejected): ptile_len doubles.
  double* ptile = nullptr;
  size_t ptile_len = 0;
  // Second inverse block (kDinv64Doubles) and interchange plan
  // (kSwapPlanInts) for the split look-ahead step, in which the next panel's
  // columns are brought up to date on the panel's stream (with oz_aux, which
  // then holds an m x nb x nb product) while the caller's stream handles the
  // other columns: consecutive panels alternate between the two sets. Null:
  // the next panel's columns go first on the caller's stream.
  double* dinv64_alt = nullptr;
  int* swap_plan_alt = nullptr;
  // Grid cap of the in-panel products on the panel's stream (0: none): the
  // SMs the trailing update beside them leaves free.
  int inpanel_ctas = 0;
};
// Most column chunks a streamed factorization takes.
constexpr int kMaxColChunks = 16;
// 64x64 inverses of the diagonal blocks of L and U, then two 32-bit column
// keys per column (padded to 64).
// Bytes of balancing words at the start of a sliced-product scratch buffer.
// They are epoch-tagged atomicMax words, so a buffer must start with them
// zeroed (a stale word of a larger epoch would never be replaced).
constexpr int kOzKinfoBytes = 8192;
inline size_t kSolveInvDoubles(int n) {
  return (size_t)2 * (size_t)((n + 63) / 64) * 64 * 64 + (size_t)((n + 63) / 64) * 64;
}
// Doubles of the U12 solve's diagonal-block inverses: NB <= 1024 in 64-row blocks.
constexpr size_t kDinv64Doubles = (size_t)16 * 64 * 64;

size_t panel_cand_doubles();
// 8-byte words of the panel kernel's exchange area (2 diagonal rows of 2 x 32
// words, 2 x 224 x 4 key words, 224 CTAs x 2 parities x 64 row words);
// panel_cand_doubles() returns it.
constexpr size_t kPanelCandDoubles = (size_t)4 * 32 + (size_t)8 * 224 + (size_t)224 * 2 * 2 * 32;
// Ints of a panel's interchange plan (count + 2 x 512 (row, src) pairs).
constexpr size_t kSwapPlanInts = 1 + 4 * 256 + 15;
// Largest M whose FP64 panel rows fit the SMs' shared memory on this device;
// taller panels need LuWork::ptile (panel_tile_doubles(m) doubles).
int panel_max_rows();
size_t panel_tile_doubles(int m);
// Smallest row slice per CTA of the cooperative panel (tunable; 0, the
// default, means 256 rows for FP32 and 128 for FP64).
int panel_min_rows();
int panel_ctas();
void set_panel_ib(int ib);
void set_panel_ctas(int g);
void set_panel_min_rows(int rows);
// Polls a panel CTA makes for another CTA's published words before it gives
// up (kSpinLimit by default; a test lowers it to make the waits run out).
long long spin_limit();
void set_spin_limit(long long polls);
// SMs (at least min_sms, at most max_sms) that the look-ahead trailing update
// leaves to the panel's stream; (0, 0) lets it take every SM.
void set_update_reserve(int min_sms, int max_sms);
// Sliced-product flops an SM takes in about one panel period (the rule's
// estimate; larger values leave the panel more SMs).
void set_update_share(double flops_per_sm);
// Split step: the in-panel products keep to the SMs the update leaves.
void set_inpanel_cap(int on);
// Block size used when a caller passes nb <= 0.
int default_nb();
// While an instance lives on a thread, phase timers record nothing on it
// (they would create CUDA events).
struct ProfSuppress {
  ProfSuppress();
  ~ProfSuppress();
};

// FP64 LU of the m x n column-major matrix dA (leading dimension ldda),
// right-looking, block size nb. dipiv receives min(m,n) 0-based pivot rows
// relative to dA. ws->info_col receives the first zero-pivot column.
cudaError_t dgetrf_device(int m, int n, double* dA, long long ldda, int* dipiv, int nb,
                          const LuWork& ws, cudaStream_t s);

// FP64 solve with the factors of dgetrf_device (trans = 'N', 'T' or 'C').
cudaError_t dgetrs_device(char trans, int n, int nrhs, const double* dA, long long ldda,
                          const int* dipiv, double* dB, long long lddb, const LuWork& ws,
                          cudaStream_t s);

// ---- low-precision trailing update (mixed_gemm.cu) ----
// Pack L21 (m x k FP32 col-major) and U12 (k x n FP32 col-major, per-column
// power-of-two scaled) into 16-bit K-major operands of k rounded up to 64.
// fmt: 0 BF16, 1 FP16, 2 BF16x3 (hi/lo split, 3 products along a K of 3*kpad).
int lowp_kpad(int k);
int lowp_kmult(int fmt);
size_t lowp_gemm_smem_bytes();
// Pipeline depth of the tcgen05 update: 3 (one CTA per SM) or 2 (two per SM).
void lowp_set_stages(int stages);
cudaError_t lowp_pack(int fmt, const float* L, long long lda, int m, const float* U,
                      long long ldu, int n, int k, unsigned short* A16, unsigned short* B16,
                      int* col_exp, cudaStream_t s);
// C (m x n FP32 col-major) -= (A16 B16^T) .* 2^col_exp (tcgen05, FP32 accumulate).
cudaError_t lowp_gemm(int fmt, int m, int n, int k, const unsigned short* A16,
                      const unsigned short* B16, const int* col_exp, float* C, long long ldc,
                      int* status, cudaStream_t s);

// ---- mixed-precision LU-IR (mixed.cu) ----
struct MixedWork {
  float* F = nullptr;          // FP32 working matrix, n x n, leading dimension ldf
  long long ldf = 0;
  unsigned short* A16 = nullptr;  // 16-bit GEMM operands (rows x kpad)
  unsigned short* B16 = nullptr;
  int* col_exp = nullptr;      // per-column exponents of U12
  int* perm = nullptr;         // composed pivot permutation (n)
  double* R = nullptr;         // residuals n x nrhs
  double* D = nullptr;         // GMRES correction (n)
  float* Xf = nullptr;         // FP32 right-hand sides n x nrhs
  float* Xtmp = nullptr;       // n x nrhs
  double* colmax = nullptr;    // 2*nrhs + 8
  double* V = nullptr;         // Krylov basis n x (gmres_m + 1)
  double* w = nullptr;         // n
  double* Ax = nullptr;        // n
  double* h = nullptr;         // gmres_m + 8
  double* Acopy = nullptr;     // optional FP64 copy of A for the fallback (keeps A)
  long long ldacopy = 0;
  int* chain = nullptr;        // chained solves: ticket (16 ints) + n x 8 x 2 tagged words
  float* dinv = nullptr;       // inverses of the 64x64 diagonal blocks of L, of U, then M_b of L, of U (4 x ceil(n/64) x 4096)
  int* epoch = nullptr;        // host-side counter of chained-solve epochs
  int* status = nullptr;       // device status word
};
struct IrOptions {
  int fmt = 0;              // 0: BF16 trailing update, 1: FP16, 2: BF16x3 split
  int nb = 256;             // block size of the low-precision factorization
  int nb_fp64 = 256;        // block size of the FP64 fallback
  int max_ir = 10;          // classical refinement steps
  int max_gmres_outer = 10; // GMRES-IR outer steps
  int gmres_m = 100;        // GMRES iterations per outer step
  double gmres_rtol = 1e-10;
  double tol = 1.0;         // target scaled residual
  // Estimated time of the plain FP64 solve as a multiple of the measured
  // low-precision factorization time: refinement gives up (and the FP64
  // solve runs) once its predicted remaining time exceeds that estimate.
  double fp64_cost_ratio = 3.5;
};
struct IrStats {
  int classical = 0, gmres_outer = 0, gmres_inner = 0, fell_back = 0, converged = 0;
  int gave_up = 0;  // refinement stopped on its predicted cost, not on a stall
  int info = 0, dev_status = 0;
  double sresid = 0.0, anorm = 0.0, factor_ms = 0.0, refine_ms = 0.0;
};
cudaError_t sgetrf_mixed_device(int n, float* F, long long ldf, int* dipiv, int nb, int fmt,
                                const LuWork& ws, const MixedWork& mw, cudaStream_t s);
cudaError_t dgesv_ir_device(int n, int nrhs, double* dA, long long lda, const double* dB,
                            long long ldb, double* dX, long long ldx, int* dipiv,
                            const IrOptions& opt, IrStats* st, const LuWork& ws,
                            const MixedWork& mw, cudaStream_t s);

// ---- batched solver (batched.cu) ----
struct BatchPlan;
cudaError_t batch_plan_create(BatchPlan** out, int batch, const int* n, const int* nrhs,
                              const double* const* A, const int* lda, const double* const* B,
                              const int* ldb, double* const* X, const int* ldx, int mode,
                              double tol, int autotune, cudaStream_t s);
cudaError_t batch_plan_execute(BatchPlan* p, cudaStream_t s);
cudaError_t batch_plan_results(BatchPlan* p, int* info, int* iters, double* sresid,
                               cudaStream_t s);
void batch_plan_shape(const BatchPlan* p, int* threads, int* chunk, int* ctas);
void batch_plan_destroy(BatchPlan* p);

// ---- norms, condition estimate, inverse (aux.cu) ----
cudaError_t dlange_device(char norm, int m, int n, const double* A, long long lda, double* work,
                          double* result, cudaStream_t s);
cudaError_t dgecon_device(bool onenrm, int n, const double* LU, long long lda, double anorm,
                          double* rcond, double* work, int* iw, cudaStream_t s);
// Operator of the 1-norm estimator: apply(true, x) -> B x, apply(false, x) -> B^T x.
using LaconApply = std::function<cudaError_t(bool, double*)>;
// PDLACON's estimate of ||B||_1 (n >= 2); work 3n + 4 doubles, iw 2 ints.
cudaError_t lacon_estimate(int n, const LaconApply& apply, double* work, int* iw, cudaStream_t s,
                           double* est);

// ---- refinement, error bounds, equilibration (refine.cu) ----
// Device workspace of dgerfs_device in doubles.
size_t refine_work_doubles(int n);
// PDGERFS on device data: X refined in place; ferr/berr are host arrays of
// nrhs entries (ferr[k] is left unchanged when column k of X is zero, as the
// reference does). dipiv is 0-based.
cudaError_t dgerfs_device(char trans, int n, int nrhs, const double* A, long long lda,
                          const double* AF, long long ldaf, const int* dipiv, const double* B,
                          long long ldb, double* X, long long ldx, double* ferr, double* berr,
                          const LuWork& ws, double* work, int* iw, cudaStream_t s);
// PDGEEQU: R (m) and C (n) device arrays; scalars and INFO on the host.
// work holds max(m, n) + 4 doubles, iw 1 int.
cudaError_t dgeequ_device(int m, int n, const double* A, long long lda, double* R, double* C,
                          double* rowcnd, double* colcnd, double* amax, int* info, double* work,
                          int* iw, cudaStream_t s);
// PDLAQGE's decision: 'N', 'R', 'C' or 'B'.
char dlaqge_equed(double rowcnd, double colcnd, double amax);
cudaError_t dlaqge_device(int m, int n, double* A, long long lda, const double* R, const double* C,
                          char equed, cudaStream_t s);
// X(i, c) *= v_i for c < ncols.
cudaError_t scale_rows_device(int n, int ncols, double* X, long long ldx, const double* v,
                              cudaStream_t s);
cudaError_t dgetri_device(int n, double* dA, long long lda, const int* dipiv, double* X,
                          const LuWork& ws, int* dflag, int* info, cudaStream_t s);

// perm[i] = original row ending in row i after the n interchanges i <-> ipiv[i].
cudaError_t perm_compose(const int* dipiv, int n, int* perm, cudaStream_t s);

// dst[i] = src[i] + delta, n entries (device arrays).
cudaError_t ipiv_shift(const int* src, int* dst, int n, int delta, cudaStream_t s);

}  // namespace sl
