// Internal interface of the host layer shared by api.cpp (LU, solve, norms,
// condition, inverse, BLACS shim) and expert_api.cpp (PDGERFS, PDGESVX,
// PDGEEQU, PDLAQGE): descriptor indices, the library-owned device state,
// argument checks with the reference's INFO encoding and the staging helpers.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <mutex>

#include "sl_internal.h"

namespace sl {
namespace host {

// Descriptor entries (0-based C indices of the Fortran DESC(1..9)).
enum { DTYPE_ = 0, CTXT_ = 1, M_ = 2, N_ = 3, MB_ = 4, NB_ = 5, RSRC_ = 6, CSRC_ = 7, LLD_ = 8 };
// Fortran positions of the descriptor entries (DESC(k) has k = index + 1).
enum { FDTYPE = 1, FCTXT = 2, FM = 3, FN = 4, FMB = 5, FNB = 6, FRSRC = 7, FCSRC = 8, FLLD = 9 };

extern std::mutex g_mu;  // device state and every entry point that uses it

struct DevState {
  bool init = false;
  bool ok = false;
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t aux = nullptr;       // look-ahead stream (higher priority)
  cudaEvent_t ev_next = nullptr, ev_panel = nullptr;
  cudaStream_t h2d = nullptr;       // host-to-device copies of A in column chunks
  cudaEvent_t ev_h2d = nullptr, ev_cols[sl::kMaxColChunks] = {};
  double* dA = nullptr; size_t capA = 0;
  double* dB = nullptr; size_t capB = 0;
  int* dipiv = nullptr; size_t capP = 0;
  int* dsmall = nullptr;      // [2] status, [3] first zero-pivot column, [4] mixed status
  double* dcand = nullptr;
  int* dplan = nullptr;       // a panel's interchange plan (kSwapPlanInts)
  int* dperm = nullptr; size_t capPerm = 0;
  double* dbswap = nullptr; size_t capBs = 0;
  // mixed-precision workspace
  float* dF = nullptr; size_t capF = 0;
  int* dpermx = nullptr; size_t capPermx = 0;
  double* dR = nullptr; size_t capR = 0;
  double* dD = nullptr; size_t capD = 0;
  float* dXf = nullptr; size_t capXf = 0;
  float* dXt = nullptr; size_t capXt = 0;
  double* dcm = nullptr; size_t capCm = 0;
  double* dV = nullptr; size_t capV = 0;
  double* dw = nullptr; size_t capW = 0;
  double* dAx = nullptr; size_t capAx = 0;
  double* dh = nullptr; size_t capH = 0;
  double* dAcopy = nullptr; size_t capAcopy = 0;
  int* dchain = nullptr; size_t capChain = 0;
  float* ddinv = nullptr; size_t capDinv = 0;
  double* dsplitk = nullptr; size_t capSplitk = 0;
  double* daux = nullptr; size_t capAux = 0;
  unsigned char* doz = nullptr; size_t capOz = 0;    // sliced-product scratch, caller's stream (bytes)
  unsigned char* doz2 = nullptr; size_t capOz2 = 0;  // sliced-product scratch, panel stream (bytes)
  double* ddinv64 = nullptr;  // U12 solve: inverses of L11's 64x64 blocks, then a copy for step 0
  double* dptile = nullptr; size_t capPtile = 0;  // rows of panels taller than shared memory holds
  double* ddinvs = nullptr; size_t capDinvs = 0;      // solve: inverses of the diagonal blocks
  int chain_epoch = 0;
  unsigned short* dA16 = nullptr; size_t capA16 = 0;
  unsigned short* dB16 = nullptr; size_t capB16 = 0;
  int* dcolexp = nullptr; size_t capCe = 0;
  // expert drivers (PDGERFS / PDGESVX / PDGEEQU): second matrix, solution,
  // refinement workspace, scale factors
  double* dA2 = nullptr; size_t capA2 = 0;
  double* dX = nullptr; size_t capX = 0;
  double* drw = nullptr; size_t capRw = 0;
  double* drc = nullptr; size_t capRc = 0;
  int* dipiv2 = nullptr; size_t capP2 = 0;
};
extern DevState g_dev;
extern int g_default_nb;
extern bool g_lookahead;

// Grows the sliced-update scratch for an m x n factorization with block nb
// (failure leaves the DMMA update in use).
void ensure_oz(int m, int n, int nb);

// Grid query (1x1 only; any other grid reads as NPROW = -1).
void gridinfo(int ictxt, int* nprow, int* npcol, int* myrow, int* mycol);
// TOOLS/numroc.f
int numroc(int n, int nb, int iproc, int isrcproc, int nprocs);
// PXERBLA message (PBLAS/SRC/PTZBLAS/pxerbla.f:57-58)
void pxerbla(int ictxt, const char* name, int info);
// TOOLS/chk1mat.f, folding into *info with the reference's encoding
void chk1mat(int ma, int mapos0, int na, int napos0, int ia, int ja, const int* desca,
             int descapos0, int* info);
// INFO class of a CUDA error: -10000 - code
int cuda_info(cudaError_t e);
// Creates the streams and small buffers on first use; false without an sm_103 GPU.
bool ensure_device();
sl::LuWork make_work();
cudaError_t ensure_solve_ws(int n, int nrhs);
// INFO after a factorization (>0 singular, <= -20000 device status)
int read_factor_info(cudaStream_t s, int mn, int* out_info);
// Device leading dimension for m rows (multiple of 32)
long long round_ld(long long m);
// Stages sub(A) into g_dev.dA, factors it, copies L\U and IPIV back.
int factor_host(int m, int n, double* A, int ia, int ja, const int* desca, int* ipiv,
                cudaStream_t s, long long* ldda_out, cudaStream_t copy_stream = nullptr);

// Test hook (sl1x1_debug_fail_alloc): the growth that finds it at 0 fails
// as an exhausted device would; -1 is off.
extern int g_fail_alloc_in;

// Grows a library-owned device buffer to at least `need` elements. On
// failure the buffer is gone (null, capacity 0).
template <class T>
cudaError_t grow(T** p, size_t* cap, size_t need) {
  if (need <= *cap && *p) return cudaSuccess;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  if (g_fail_alloc_in >= 0 && g_fail_alloc_in-- == 0) return cudaErrorMemoryAllocation;
  size_t n = need < 1 ? 1 : need;
  cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
  if (e == cudaSuccess) *cap = n;
  return e;
}

}  // namespace host
}  // namespace sl
