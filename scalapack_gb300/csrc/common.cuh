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
