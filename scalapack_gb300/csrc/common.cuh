// Shared device helpers for the sl1x1 GB300 LU library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace sl {

// Error codes written by kernels into the device status word. They are turned
// into INFO = -(10000 + code) by the host layer.
enum DevStatus : int {
  kOk = 0,
  kBarrierTimeout = 1,   // reserved: a bounded grid barrier gave up (no kernel uses one now)
  kFlagTimeout = 2,      // a bounded wait on another CTA's published data gave up
  kBadArgument = 3,      // kernel-side argument check failed
};

// Upper bound on spin iterations of any device-side wait: each iteration is at
// least one L2 round trip, so this is several seconds of waiting, after which
// the kernel records an error and returns instead of hanging the GPU.
constexpr long long kSpinLimit = 1LL << 24;

__device__ __forceinline__ int ld_acquire_gpu(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release_gpu(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}


// Balancing keys of the sliced FP64 product (ozgemm_f64.cu), also published
// by kernels that produce its operands: (epoch << 12) | (frexp exponent +
// kOzEbias) of a finite nonzero value, 0 for zero or non-finite values.
constexpr int kOzEbias = 1100;  // frexp exponents -1073 .. 1024 -> 27 .. 2124 (< 4096)
__device__ __forceinline__ unsigned long long oz_key_word(double x, unsigned long long epoch) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffULL;
  if (b == 0ULL || b >= 0x7ff0000000000000ULL) return 0ULL;
  const int bexp = (int)(b >> 52);
  const int ex = bexp ? bexp - 1022 : (63 - __clzll((long long)b)) - 1073;
  return (epoch << 12) | (unsigned long long)(ex + kOzEbias);
}

// The balancing keys a kernel publishes for a following sliced product:
// column maxima of L (lrows x lcols from L, column-major) into ckeys, row
// maxima of the kernel's own output into hkeys, with one epoch; a null
// ckeys / hkeys turns that part off.
struct OzKeyJob {
  unsigned long long* ckeys = nullptr;
  unsigned long long* hkeys = nullptr;
  unsigned long long epoch = 0ULL;
  const double* L = nullptr;
  long long ldl = 0;
  int lrows = 0, lcols = 0;
};

// IDAMAX ordering key. Reference BLAS IDAMAX keeps the first maximal |x| and a
// NaN never replaces the running maximum, so NaN entries are mapped below every
// real magnitude. (The first element is handled separately by the callers.)
__device__ __forceinline__ double amax_key(double v) {
  double a = fabs(v);
  return (a != a) ? -1.0 : a;
}

// Combine two (key,row) candidates: larger key wins, ties go to the lower row.
__device__ __forceinline__ void amax_combine(double& k, int& r, double k2, int r2) {
  if (k2 > k || (k2 == k && r2 < r)) { k = k2; r = r2; }
}

__device__ __forceinline__ void warp_amax(double& k, int& r) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    double k2 = __shfl_xor_sync(0xffffffffu, k, off);
    int r2 = __shfl_xor_sync(0xffffffffu, r, off);
    amax_combine(k, r, k2, r2);
  }
}

}  // namespace sl
