// sl1x1_dgetrf_noalloc: the FP64 LU factorization for callers that cannot
// allocate GPU memory.
//
// Who needs it: code that runs where cudaMalloc is not allowed or not safe --
// a caller inside a memory pool or arena that owns the whole device heap, a
// real-time or embedded loop that may not allocate after start-up, or a
// framework that hands this library only the matrix and pivot buffers. The
// other entry points grow library-owned device buffers on demand; this one
// allocates nothing.
//
// The factorization's only scratch -- the device status word, the
// first-zero-pivot column, the panel kernel's exchange area and the plan of a
// panel's row interchanges -- lives in the file-scope array below, a fixed 1 MiB that every GPU
// which loads this library holds until the process exits. The caller passes
// the matrix and the pivot array as usual. The LuWork below carries no
// sliced-product scratch (its size grows with the matrix), so the trailing
// update and the U12 solve run in FP64 (DMMA and the strip solve): the
// results are those of sl1x1_dgetrf_dev with sl1x1_set_f64_update(0).
//
// Set-up: the first call on each device looks up the device address of that
// array (cudaGetSymbolAddress, with that device current) and caches it; make
// that first call before any stream capture. Every call reads its status
// words back and synchronizes its stream before it returns. Every call
// shares the one array:
// the call re-initializes the status and zero-pivot words and every panel
// launch clears its exchange area,
// but two calls whose GPU work overlaps (on different streams or from
// different host threads) race on it and must not be issued.
#include <cuda_runtime.h>

#include <climits>
#include <cstdio>
#include <mutex>

#include "../../include/sl1x1.h"
#include "sl_internal.h"

namespace {

// Stated maximum of the static scratch: 1 MiB. It holds 4 ints at offset 0
// (two spare words, status word, first zero-pivot column), from offset 256 the
// panel kernel's exchange area, then the plan of a panel's row interchanges.
constexpr size_t kScratchBytes = (size_t)1 << 20;
constexpr size_t kCandOffset = 256;
constexpr size_t kPlanOffset = (kCandOffset + sl::kPanelCandDoubles * sizeof(double) + 255) / 256 * 256;
static_assert(kPlanOffset + sl::kSwapPlanInts * sizeof(int) <= kScratchBytes,
              "the panel exchange area and the interchange plan must fit the static scratch");

static __device__ __align__(256) unsigned char g_dgetrf_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
void* g_scratch_addr[kMaxDevices];  // device address per device, set once
std::mutex g_na_mu;

int cuda_info(cudaError_t e) { return -10000 - (int)e; }

}  // namespace

extern "C" int sl1x1_dgetrf_noalloc(int m, int n, double* dA, long long ldda, int* dipiv, int nb,
                                    void* stream) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (ldda < (m > 1 ? m : 1)) return -4;
  if (m > 0 && n > 0) {
    const int max_rows = sl::panel_max_rows();
    if (m > max_rows) {
      std::fprintf(stderr,
                   "sl1x1_dgetrf_noalloc: M=%d exceeds the supported maximum of %d rows "
                   "(the panel's rows held in the %d SMs' shared memory); nothing was launched\n",
                   m, max_rows, sl::num_sms());
      return -30000;
    }
  }
  if (m == 0 || n == 0) return 0;
  if (dA == nullptr) return -3;
  if (dipiv == nullptr) return -5;

  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_info(e);
  if (dev < 0 || dev >= kMaxDevices) return -30000;
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_scratch_addr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_dgetrf_scratch);
      if (e != cudaSuccess) return cuda_info(e);
      g_scratch_addr[dev] = p;
    }
    base = g_scratch_addr[dev];
  }

  sl::LuWork w;
  w.status = static_cast<int*>(base) + 2;
  w.info_col = static_cast<int*>(base) + 3;
  w.cand = reinterpret_cast<double*>(static_cast<unsigned char*>(base) + kCandOffset);
  w.swap_plan = reinterpret_cast<int*>(static_cast<unsigned char*>(base) + kPlanOffset);
  w.perm = nullptr;
  w.bswap = nullptr;
  w.perm_len = 0;
  w.bswap_len = 0;

  cudaStream_t s = static_cast<cudaStream_t>(stream);
  sl::ProfSuppress no_events;  // phase timers would create CUDA events
  // dgetrf_device zeroes the status word and resets the zero-pivot column,
  // and every panel launch clears its exchange area, before use.
  e = sl::dgetrf_device(m, n, dA, ldda, dipiv, nb > 0 ? nb : sl::default_nb(), w, s);
  if (e == cudaErrorInvalidValue) return -30000;
  if (e != cudaSuccess) return cuda_info(e);
  int h[2] = {0, 0};
  e = cudaMemcpyAsync(h, w.status, 2 * sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_info(e);
  if (h[0] != 0) return -20000 - h[0];
  const int mn = m < n ? m : n;
  const int info = (h[1] >= 0 && h[1] < mn) ? h[1] + 1 : 0;
  e = sl::ipiv_shift(dipiv, dipiv, mn, 1, s);  // 0-based rows -> 1-based, as LAPACK
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_info(e);
  return info;
}
