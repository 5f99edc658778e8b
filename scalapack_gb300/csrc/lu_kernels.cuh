// Type-generic LU kernels (T = double for the plain FP64 path, float for the
// FP32 panel of the mixed-precision path) and their launch helpers.
//
//   panel_kernel<T>      PDGETF2 (SRC/pdgetf2.f:206-237) on a <=32-column sub-panel
//   laswp_kernel<T>      PDLASWP (SRC/pdlaswp.f:163-172)
//   trsm_strip_kernel<T> PDTRSM diagonal-block solves (PB_CptrsmAB.c)
//   permute_rows_kernel<T>, gemm_skinny_kernel<T>  PDLAPIV and the narrow
//                        off-diagonal updates of PDGETRS
#pragma once
#include <algorithm>
#include <climits>
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "common.cuh"
#include "sl_internal.h"

namespace sl {

namespace {
// Dynamic shared-memory opt-in, once per kernel and translation unit. Kernels
// are registered per translation unit, so the record of which kernels were
// raised must not be shared between units: it lives in an unnamed namespace.
inline cudaError_t smem_attr_once(const void* kern, int bytes) {
  static std::mutex mu;
  static const void* done_k[64];
  static int done_b[64];
  static int ndone = 0;
  std::lock_guard<std::mutex> lk(mu);
  for (int i = 0; i < ndone; ++i)
    if (done_k[i] == kern && done_b[i] >= bytes) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess && ndone < 64) {
    done_k[ndone] = kern;
    done_b[ndone] = bytes;
    ++ndone;
  }
  return e;
}
}  // namespace

constexpr int PW = 32;       // sub-panel width held in shared memory (<= 64)
constexpr int PMAXG = 224;   // max CTAs of the panel kernel (warp 7 reads the diagonal row)
// Exchange area of the panel kernel, in 8-byte tagged words: the diagonal
// rows [2 parities][2*PW], the candidate keys [2 parities][PMAXG][4] (|x| key
// lo, key hi, row, spare: one 32-byte sector per CTA, so that CTAs do not
// write into each other's sectors) and the candidate rows
// [PMAXG][2 parities][2*PW].
constexpr int PX_DIAG = 0;
constexpr int PX_KEYS = 4 * PW;
constexpr int PX_VALS = PX_KEYS + 8 * PMAXG;
constexpr int PX_WORDS = PX_VALS + PMAXG * 2 * 2 * PW;
constexpr int PT = 256;      // threads per panel CTA
constexpr int PLD = PW + 1;  // shared row stride: conflict-free row and column walks

// Factor rows [r0, m) x columns [c0, c0+w) (w <= 32) of A in place (the
// panel kernel below): writes ipiv[c0+k] = r0 + pivot (0-based rows of A) for
// k < min(w, m-r0) and the first exactly-zero pivot column into *info_col.
//
// Tagged 8-byte words {32-bit payload, 32-bit tag} carry the per-column
// exchange between the panel's CTAs: a word is valid once its tag equals the
// column's tag, so readers poll the data itself and no separate grid barrier
// or fence is needed (each aligned 8-byte access is single-copy atomic).
__device__ __forceinline__ void st_tagged(unsigned long long* p, uint32_t v, uint32_t tag) {
  const unsigned long long wd = ((unsigned long long)tag << 32) | v;
  asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(wd) : "memory");
}
__device__ __forceinline__ unsigned long long ld_tagged(const unsigned long long* p) {
  unsigned long long wd;
  asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(wd) : "l"(p) : "memory");
  return wd;
}
__device__ __forceinline__ void ld_tagged2(const unsigned long long* p, unsigned long long& a,
                                           unsigned long long& b) {
  asm volatile("ld.relaxed.gpu.global.v2.b64 {%0, %1}, [%2];" : "=l"(a), "=l"(b) : "l"(p) : "memory");
}
__device__ __forceinline__ bool tag_ok(unsigned long long wd, uint32_t tag) {
  return (uint32_t)(wd >> 32) == tag;
}
__device__ __forceinline__ uint32_t payload(unsigned long long wd) { return (uint32_t)wd; }
__device__ __forceinline__ unsigned long long join(unsigned long long lo, unsigned long long hi) {
  return ((unsigned long long)payload(hi) << 32) | payload(lo);
}

// Value v of a row as tagged words (FP32: one word, FP64: two).
template <typename T>
__device__ __forceinline__ void st_value(unsigned long long* p, int j, T v, uint32_t tag) {
  if constexpr (sizeof(T) == 4) {
    st_tagged(p + j, __float_as_uint(v), tag);
  } else {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    st_tagged(p + 2 * j, (uint32_t)b, tag);
    st_tagged(p + 2 * j + 1, (uint32_t)(b >> 32), tag);
  }
}

// Polls value j of a published row until its tag matches, at most `limit`
// times; false on timeout.
template <typename T>
__device__ __forceinline__ bool ld_value(const unsigned long long* p, int j, uint32_t tag, T& v,
                                         long long limit) {
  for (long long spins = 0; spins < limit; ++spins) {
    if constexpr (sizeof(T) == 4) {
      const unsigned long long a = ld_tagged(p + j);
      if (tag_ok(a, tag)) { v = __uint_as_float(payload(a)); return true; }
    } else {
      unsigned long long a0, a1;
      ld_tagged2(p + 2 * j, a0, a1);
      if (tag_ok(a0, tag) && tag_ok(a1, tag)) { v = __longlong_as_double((long long)join(a0, a1)); return true; }
    }
  }
  return false;
}

// IDAMAX key of a value: the bit pattern of |x| as an integer (monotonic in
// |x| for IEEE formats, +0 and -0 equal), -1 for NaN so that NaN never wins.
// Integer keys keep the pivot search off the FP64 pipe.
__device__ __forceinline__ long long amax_ikey(double v) {
  const long long b = __double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFLL;
  return b > 0x7FF0000000000000LL ? -1LL : b;
}
__device__ __forceinline__ long long amax_ikey(float v) {
  const int b = __float_as_int(v) & 0x7FFFFFFF;
  return b > 0x7F800000 ? -1LL : (long long)b;
}
// Larger key wins, ties go to the lower row (IDAMAX returns the first max).
__device__ __forceinline__ void ikey_combine(long long& k, int& r, long long k2, int r2) {
  if (k2 > k || (k2 == k && r2 < r)) { k = k2; r = r2; }
}
__device__ __forceinline__ void warp_ikey(long long& k, int& r) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const long long k2 = __shfl_xor_sync(0xffffffffu, k, off);
    const int r2 = __shfl_xor_sync(0xffffffffu, r, off);
    ikey_combine(k, r, k2, r2);
  }
}

// Cooperative unblocked LU of a sub-panel (PDGETF2, SRC/pdgetf2.f:206-237)
// over rows r0..m-1 and columns c0..c0+w-1 of A, w <= PW. CTA b owns rows
// r0 + b*rpc .. +rpc-1 in shared memory. Per column k:
//   1. each CTA's IDAMAX candidate (first max, NaN never wins --
//      PBLAS/SRC/pdamax_.c:414-486 through idamax_) is published as tagged
//      words: its key and row, and the candidate row itself; the owner of the
//      diagonal row publishes that row too;
//   2. every CTA polls all keys (thread q reads CTA q's sector) until the
//      tags match, reduces to the global winner (largest |x|, lowest row on
//      ties) and then reads the pivot row from the winner's slot;
//   3. rows d and piv are exchanged inside the sub-panel, the column is scaled
//      by the reciprocal of the pivot and the rank-1 update is applied
//      (PDSWAP/PDSCAL/PDGER, pdgetf2.f:218-233) with one thread per row, which
//      also forms the next column's IDAMAX key.
// Column k's words carry tag k+1 and the launch zeroes the area first. A word
// of parity k&1 is rewritten only at column k+2, after every CTA has read
// column k+1 -- which it can only do after finishing column k -- so two
// parities suffice. Every poll is bounded (at most spin_limit polls); a CTA
// that gives up records kFlagTimeout and returns, and block 0 then writes the
// identity for the pivots it has not chosen, so the interchanges launched
// after it stay inside the matrix.
//
// GTILE: for panels taller than the CTAs' shared memory holds (more than 768
// FP64 rows per CTA on every SM), each CTA's rows live in a global buffer
// instead (gtile, column-major per CTA: rpc rows x PW columns, so a warp's
// row walk is one coalesced access); the algorithm is unchanged.
template <typename T, bool GTILE = false>
__global__ void __launch_bounds__(PT)
panel_kernel(T* A, long long lda, int m, int r0, int c0, int w, int rpc, int* ipiv,
             int* info_col, double* cand, int* status, long long spin_limit, T* gtile) {
  extern __shared__ __align__(16) unsigned char panel_smem[];
  // element (r, c) of this CTA's rows: [rpc][PLD] in shared memory, or
  // column-major rpc x PW in the global buffer
  T* tile = GTILE ? gtile + (size_t)blockIdx.x * (size_t)rpc * PW : reinterpret_cast<T*>(panel_smem);
  auto tix = [&](int r, int c) -> size_t {
    return GTILE ? (size_t)c * (size_t)rpc + (size_t)r : (size_t)r * PLD + (size_t)c;
  };
  __shared__ T s_U[PW];
  __shared__ T s_D[PW];
  __shared__ long long s_wk[PT / 32];
  __shared__ int s_wr[PT / 32];
  __shared__ int s_lrow, s_row, s_fail, s_scale;
  __shared__ long long s_lkey, s_gkey;
  __shared__ T s_rinv;

  const int G = gridDim.x, b = blockIdx.x, tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int R = m - r0;
  const int kw = min(w, R);
  const int lo = b * rpc;                   // first local row (relative to r0)
  const int nr = max(0, min(rpc, R - lo));  // rows owned
  unsigned long long* words = reinterpret_cast<unsigned long long*>(cand);
  unsigned long long* diagw = words + PX_DIAG;
  unsigned long long* keyw = words + PX_KEYS;
  unsigned long long* valw = words + PX_VALS;
  // block 0 on a timeout at column k: pivots k.. become the diagonal rows
  auto give_up = [&](int k) {
    if (b == 0)
      for (int q = k + tid; q < kw; q += PT) ipiv[c0 + q] = r0 + q;
  };

  // Sub-panel rows into shared memory, all w columns' loads in flight at once.
  for (int r = tid; r < nr; r += PT) {
    const T* src = A + (long long)(r0 + lo + r) + (long long)c0 * lda;
    T v[PW];
#pragma unroll
    for (int c = 0; c < PW; ++c) v[c] = (c < w) ? src[(long long)c * lda] : (T)0;
#pragma unroll
    for (int c = 0; c < PW; ++c)
      if (c < w) tile[tix(r, c)] = v[c];
  }
  if (tid == 0) s_fail = 0;

  // Per-warp IDAMAX candidates of column 0; those of column k+1 come out of
  // column k's rank-1 update.
  {
    long long key = -2;
    int row = INT_MAX;
    for (int r = tid; r < nr; r += PT) ikey_combine(key, row, amax_ikey(tile[tix(r, 0)]), lo + r);  // own rows
    warp_ikey(key, row);
    if (lane == 0) { s_wk[warp] = key; s_wr[warp] = row; }
  }
  __syncthreads();

  // Column k's rank-1 update is applied in two parts: right after its pivot,
  // only column k+1 (which gives the next pivot search its keys); the rest
  // (columns k+2..) after column k+1's key has been published, while the
  // other CTAs' keys are on their way. Every element still receives the
  // updates of columns 0, 1, ... in order, as one fma each.
  auto finish_update = [&](int kp) {  // columns kp+2 .. w-1 of the rows below kp
    for (int r = max(0, kp + 1 - lo) + tid; r < nr; r += PT) {
      const T l = tile[tix(r, kp)];
#pragma unroll 4
      for (int j = kp + 2; j < w; ++j) tile[tix(r, j)] = fma(-l, s_U[j], tile[tix(r, j)]);
    }
  };

  for (int k = 0; k < kw; ++k) {
    const int d = k;  // diagonal row relative to r0
    const int par = k & 1;
    const uint32_t tag = (uint32_t)(k + 1);
    // --- this CTA's candidate: IDAMAX over its rows >= d; its key goes out
    //     at once ---
    if (warp == 0) {
      long long key = lane < PT / 32 ? s_wk[lane] : -2;
      int row = lane < PT / 32 ? s_wr[lane] : INT_MAX;
      warp_ikey(key, row);
      if (lane == 0) {
        s_lrow = row;
        s_lkey = key;
        const unsigned long long kb = (unsigned long long)key;
        unsigned long long* kw4 = keyw + ((size_t)par * PMAXG + b) * 4;
        st_tagged(kw4 + 0, (uint32_t)kb, tag);
        st_tagged(kw4 + 1, (uint32_t)(kb >> 32), tag);
        st_tagged(kw4 + 2, (uint32_t)row, tag);
      }
    }
    __syncthreads();
    {
      // the rest of column k-1's update, then the candidate row and the
      // diagonal row (if owned), each published by its owner warp
      if (k > 0) finish_update(k - 1);
      // finish_update(k-1) hands row r (of this CTA) to thread (r - st) % PT
      const int st = max(0, k - lo);
      const int lr = s_lrow;
      if (lr != INT_MAX && lr - lo >= st && lr - lo < nr && (((lr - lo - st) % PT) >> 5) == warp) {
        __syncwarp();
        for (int c = lane; c < w; c += 32)
          st_value<T>(valw + ((size_t)b * 2 + par) * 2 * PW, c, tile[tix(lr - lo, c)], tag);
      }
      if (d - lo >= st && d - lo < nr && (((d - lo - st) % PT) >> 5) == warp) {
        __syncwarp();
        for (int c = lane; c < w; c += 32) st_value<T>(diagw + par * 2 * PW, c, tile[tix(d - lo, c)], tag);
      }
    }

    // --- poll every CTA's key (thread q <- CTA q) and the diagonal row (warp 7);
    //     the polls spin without sleeping (a sleep costs more than it saves
    //     here), bounded by spin_limit ---
    long long key = -2;
    int row = INT_MAX;
    if (tid < G) {
      long long spins = 0;
      for (;;) {
        if (spins++ >= spin_limit) { atomicExch(status, (int)kFlagTimeout); s_fail = 1; break; }
        unsigned long long w0, w1, w2, w3;
        ld_tagged2(keyw + ((size_t)tid + (size_t)par * PMAXG) * 4, w0, w1);
        ld_tagged2(keyw + ((size_t)tid + (size_t)par * PMAXG) * 4 + 2, w2, w3);
        if (tag_ok(w0, tag) && tag_ok(w1, tag) && tag_ok(w2, tag)) {
          key = (long long)join(w0, w1);
          const uint32_t rr = payload(w2);
          row = rr >= (uint32_t)INT_MAX ? INT_MAX : (int)rr;
          break;
        }
      }
    } else if (warp == PT / 32 - 1) {
      for (int c = lane; c < w; c += 32) {
        T v;
        if (ld_value<T>(diagw + par * 2 * PW, c, tag, v, spin_limit)) s_D[c] = v;
        else { atomicExch(status, (int)kFlagTimeout); s_fail = 1; }
      }
    }
    warp_ikey(key, row);
    if (lane == 0) { s_wk[warp] = key; s_wr[warp] = row; }
    __syncthreads();
    if (s_fail) { give_up(k); return; }
    if (warp == 0) {
      key = lane < PT / 32 ? s_wk[lane] : -2;
      row = lane < PT / 32 ? s_wr[lane] : INT_MAX;
      warp_ikey(key, row);
      if (lane == 0) { s_row = row; s_gkey = key; }
    }
    __syncthreads();
    // IDAMAX keeps the first element when it is NaN; AMAX == 0 selects the
    // diagonal row (PBLAS/SRC/pdamax_.c:486).
    const int piv = (amax_ikey(s_D[k]) < 0 || s_gkey == 0) ? d : s_row;
    // U = the pivot row: the diagonal row, or the winner's published row
    if (tid < w) {
      if (piv == d) {
        s_U[tid] = s_D[tid];
      } else {
        T v;
        if (ld_value<T>(valw + ((size_t)(piv / rpc) * 2 + par) * 2 * PW, tid, tag, v, spin_limit)) s_U[tid] = v;
        else { atomicExch(status, (int)kFlagTimeout); s_fail = 1; }
      }
    }
    __syncthreads();
    if (s_fail) { give_up(k); return; }
    // --- row interchange inside the sub-panel (PDSWAP, pdgetf2.f:218) ---
    if (piv != d && tid < w) {
      if (d >= lo && d < lo + nr) tile[tix(d - lo, tid)] = s_U[tid];
      if (piv >= lo && piv < lo + nr) tile[tix(piv - lo, tid)] = s_D[tid];
    }
    if (tid == 0) {
      const T gmax = s_U[k];
      s_scale = (gmax != (T)0);
      s_rinv = (gmax != (T)0) ? (T)1 / gmax : (T)0;  // ONE/GMAX (pdgetf2.f:224)
      if (b == 0) {
        ipiv[c0 + k] = r0 + piv;
        if (gmax == (T)0) atomicMin(info_col, c0 + k);
      }
    }
    __syncthreads();
    // --- scale (PDSCAL) and the first column of the rank-1 update (PDGER),
    //     one thread per row; the row's next-column entry gives its IDAMAX
    //     key for column k+1 ---
    const bool scale = s_scale != 0;
    const T rinv = s_rinv;
    const int kn = k + 1;
    long long nkey = -2;
    int nrow = INT_MAX;
    for (int r = max(0, d + 1 - lo) + tid; r < nr; r += PT) {
      T l = tile[tix(r, k)];
      if (scale) l *= rinv;
      tile[tix(r, k)] = l;
      if (kn < w) tile[tix(r, kn)] = fma(-l, s_U[kn], tile[tix(r, kn)]);
      if (kn < kw) ikey_combine(nkey, nrow, amax_ikey(tile[tix(r, kn)]), lo + r);
    }
    if (kn < kw) {
      warp_ikey(nkey, nrow);
      if (lane == 0) { s_wk[warp] = nkey; s_wr[warp] = nrow; }
    }
    __syncthreads();
  }
  // the last column's remaining update (columns beyond kw when the panel has
  // fewer rows than columns)
  if (kw > 0) finish_update(kw - 1);
  __syncthreads();

  for (int r = tid; r < nr; r += PT) {
    T* dst = A + (long long)(r0 + lo + r) + (long long)c0 * lda;
    T v[PW];
#pragma unroll
    for (int c = 0; c < PW; ++c) v[c] = (c < w) ? tile[tix(r, c)] : (T)0;
#pragma unroll
    for (int c = 0; c < PW; ++c)
      if (c < w) dst[(long long)c * lda] = v[c];
  }
}

// Sequential row interchanges k1..k2-1 (rows i <-> ipiv[i]) on the columns
// [cb1,ce1) and [cb2,ce2); one thread per column (PDLASWP 'Forward','Rows').
// Used when the interchanges outnumber the composite form's table.
template <typename T>
__global__ void __launch_bounds__(256)
laswp_seq_kernel(T* A, long long lda, int k1, int k2, const int* __restrict__ ipiv, int cb1,
                 int ce1, int cb2, int ce2) {
  const int npiv = k2 - k1;
  const long long n1 = ce1 - cb1, n2 = ce2 - cb2;
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n1 + n2) return;
  long long col = idx < n1 ? cb1 + idx : cb2 + (idx - n1);
  T* a = A + col * lda;
  for (int i = 0; i < npiv; ++i) {
    int p = ipiv[k1 + i];
    int r = k1 + i;
    if (p != r) {
      T t = a[r];
      a[r] = a[p];
      a[p] = t;
    }
  }
}

// The same interchanges applied as one composite permutation (PDLASWP
// 'Forward','Rows', SRC/pdlaswp.f:163-172): warp 0 of each CTA replays the
// swaps on row labels in shared memory -- entries for rows k1..k2-1 plus the
// pivot rows below them -- giving, for every touched row, the row whose
// original content ends up there. Then one warp per column loads all moved
// values at once and stores them, so a column costs one round trip instead of
// k2-k1 dependent ones. The result is bitwise that of the sequential swaps.
constexpr int LSW_MAXP = 256;
template <typename T>
__global__ void __launch_bounds__(256)
laswp_kernel(T* A, long long lda, int k1, int k2, const int* __restrict__ ipiv, int cb1, int ce1,
             int cb2, int ce2) {
  __shared__ int s_piv[LSW_MAXP];
  __shared__ int s_row[2 * LSW_MAXP];  // touched row of entry e
  __shared__ int s_src[2 * LSW_MAXP];  // row whose original content lands in s_row[e]
  __shared__ int s_cnt;
  const int npiv = k2 - k1;  // <= LSW_MAXP (checked by the launcher)
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i < npiv; i += blockDim.x) {
    s_piv[i] = ipiv[k1 + i];
    s_row[i] = k1 + i;
    s_src[i] = k1 + i;
  }
  __syncthreads();
  if (warp == 0) {
    int cnt = npiv;
    for (int i = 0; i < npiv; ++i) {
      const int p = s_piv[i];
      if (p == k1 + i) continue;
      int e;
      if (p >= k1 && p < k2) {
        e = p - k1;
      } else {
        e = -1;
        for (int base = npiv; base < cnt && e < 0; base += 32) {
          const int q = base + lane;
          const unsigned hit = __ballot_sync(0xffffffffu, q < cnt && s_row[q] == p);
          if (hit) e = base + __ffs(hit) - 1;
        }
        if (e < 0) {
          e = cnt++;
          if (lane == 0) { s_row[e] = p; s_src[e] = p; }
        }
      }
      __syncwarp();
      if (lane == 0) {
        const int t = s_src[i];
        s_src[i] = s_src[e];
        s_src[e] = t;
      }
      __syncwarp();
    }
    if (lane == 0) s_cnt = cnt;
  }
  __syncthreads();
  const int cnt = s_cnt;
  const long long n1 = ce1 - cb1, ncols = n1 + (ce2 - cb2);
  constexpr int PER = 2 * LSW_MAXP / 32;
  for (long long ci = (long long)blockIdx.x * 8 + warp; ci < ncols; ci += (long long)gridDim.x * 8) {
    const long long col = ci < n1 ? cb1 + ci : cb2 + (ci - n1);
    T* a = A + col * lda;
    T v[PER];
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int e = lane + 32 * q;
      v[q] = (e < cnt && s_src[e] != s_row[e]) ? a[s_src[e]] : (T)0;
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int e = lane + 32 * q;
      if (e < cnt && s_src[e] != s_row[e]) a[s_row[e]] = v[q];
    }
  }
}

// Plan of the interchanges k1..k2-1 (k2-k1 <= LSW_MAXP) in composite form:
// plan[0] = number of pairs, then (row, src) pairs for every touched row whose
// content changes (row receives the original content of src). The touched
// rows are k1..k2-1, then each row outside them in the order the interchanges
// first reach it; every thread walks the interchanges backwards for its rows
// (interchange i moves the content followed from ipiv[k1+i] to k1+i or the
// other way), so the cost is npiv shared-memory reads per row, in parallel.
// The pairs come out in the order of a sequential replay. Computed once per
// panel, on the panel's stream; laswp_apply_kernel then only moves data.
static __device__ __noinline__ void laswp_plan_block(int k1, int k2, const int* __restrict__ ipiv,
                                                    int* plan) {
  __shared__ int s_piv[LSW_MAXP], s_first[LSW_MAXP], s_rank[LSW_MAXP];
  __shared__ int s_row[2 * LSW_MAXP], s_src[2 * LSW_MAXP];
  __shared__ int s_cnt;
  const int npiv = k2 - k1, tid = threadIdx.x, nt = blockDim.x;
  for (int i = tid; i < npiv; i += nt) s_piv[i] = ipiv[k1 + i];
  __syncthreads();
  // interchange i reaches an outside row for the first time
  for (int i = tid; i < npiv; i += nt) {
    const int p = s_piv[i];
    bool first = p < k1 || p >= k2;
    for (int i2 = 0; first && i2 < i; ++i2) first = s_piv[i2] != p;
    s_first[i] = first ? 1 : 0;
  }
  __syncthreads();
  if (tid == 0) {
    int c = 0;
    for (int i = 0; i < npiv; ++i) {
      s_rank[i] = c;
      c += s_first[i];
    }
    s_cnt = npiv + c;
  }
  __syncthreads();
  for (int i = tid; i < npiv; i += nt) {
    s_row[i] = k1 + i;
    if (s_first[i]) s_row[npiv + s_rank[i]] = s_piv[i];
  }
  __syncthreads();
  const int cnt = s_cnt;
  for (int e = tid; e < cnt; e += nt) {
    int q = s_row[e];
    for (int i = npiv - 1; i >= 0; --i) {
      const int p = s_piv[i];
      q = (q == k1 + i) ? p : ((q == p) ? k1 + i : q);
    }
    s_src[e] = q;
  }
  __syncthreads();
  if (tid == 0) {
    int np = 0;
    for (int e = 0; e < cnt; ++e)
      if (s_src[e] != s_row[e]) {
        plan[1 + 2 * np] = s_row[e];
        plan[2 + 2 * np] = s_src[e];
        ++np;
      }
    plan[0] = np;
  }
}

static __global__ void laswp_plan_kernel(int k1, int k2, const int* __restrict__ ipiv, int* plan) {
  laswp_plan_block(k1, k2, ipiv, plan);
}

// Applies a plan of laswp_plan_kernel to the columns [cb1,ce1) and
// [cb2,ce2): one warp per column loads every moved value, then stores them.
template <typename T>
__global__ void __launch_bounds__(256)
laswp_apply_kernel(T* A, long long lda, const int* __restrict__ plan, int cb1, int ce1, int cb2,
                   int ce2) {
  __shared__ int s_row[2 * LSW_MAXP], s_src[2 * LSW_MAXP];
  const int np = plan[0];
  for (int e = threadIdx.x; e < np; e += blockDim.x) {
    s_row[e] = plan[1 + 2 * e];
    s_src[e] = plan[2 + 2 * e];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long n1 = ce1 - cb1, ncols = n1 + (ce2 - cb2);
  constexpr int PER = 2 * LSW_MAXP / 32;
  for (long long ci = (long long)blockIdx.x * 8 + warp; ci < ncols; ci += (long long)gridDim.x * 8) {
    const long long col = ci < n1 ? cb1 + ci : cb2 + (ci - n1);
    T* a = A + col * lda;
    T v[PER];
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int e = lane + 32 * q;
      v[q] = (e < np) ? a[s_src[e]] : (T)0;
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int e = lane + 32 * q;
      if (e < np) a[s_row[e]] = v[q];
    }
  }
}

// op(T) X = B for a w x w triangle (w <= 256) and a strip of NC columns of B
// per CTA, held in shared memory. FORWARD solves top-down (lower, or upper^T),
// otherwise bottom-up. The triangle is staged in shared memory eb (<= 32)
// columns at a time (all loads of a block in flight together), so the w
// dependent steps read only shared memory. Non-unit diagonals divide
// (reference DTRSM semantics).
constexpr int TRSM_EB = 32;
template <typename T, bool UPPER, bool TRANS, bool UNIT, int NC>
__global__ void __launch_bounds__(256)
trsm_strip_kernel(int w, int ncols, int eb, const T* __restrict__ Tm, long long ldt, T* B,
                  long long ldb, OzKeyJob kj) {
  constexpr bool FORWARD = (UPPER == TRANS);
  const int nsolve = (ncols + NC - 1) / NC;
  if ((int)blockIdx.x >= nsolve) {
    // extra blocks: column maxima of kj.L, 32 rows each (warp w: columns w,
    // w+8, ...; one coalesced load per column)
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const int i = ((int)blockIdx.x - nsolve) * 32 + lane;
    for (int c = wp; c < kj.lcols; c += 8) {
      const unsigned long long v = (i < kj.lrows) ? oz_key_word(kj.L[i + (long long)c * kj.ldl], kj.epoch) : 0ULL;
      const unsigned hi = __reduce_max_sync(0xffffffffu, (unsigned)(v >> 12 == kj.epoch ? (v & 4095ULL) : 0ULL));
      if (lane == 0 && hi) atomicMax(kj.ckeys + c, (kj.epoch << 12) | hi);
    }
    return;
  }
  constexpr int RG = 256 / NC;  // row groups
  extern __shared__ __align__(16) unsigned char strip_smem[];
  T* Bs = reinterpret_cast<T*>(strip_smem);  // [w][NC+1]
  const int LD = NC + 1;
  T* Es = Bs + (size_t)w * LD;                // [eb][w+1]: Es[ii*(w+1) + r] = op(T)(r, i(ii))
  const int LE = w + 1;
  const int tid = threadIdx.x;
  const int c = tid % NC, rg = tid / NC;
  const long long col0 = (long long)blockIdx.x * NC;
  const int nc = (int)min((long long)NC, ncols - col0);
  for (int i = tid; i < w * NC; i += 256) {
    int r = i % w, cc = i / w;
    Bs[r * LD + cc] = cc < nc ? B[r + (col0 + cc) * ldb] : (T)0;
  }
  for (int s0 = 0; s0 < w; s0 += eb) {
    const int nb = min(eb, w - s0);
    __syncthreads();  // the previous block's steps are done with Es
    for (int idx = tid; idx < nb * w; idx += 256) {
      int ii, r;
      if (!TRANS) { r = idx % w; ii = idx / w; }    // coalesced along r
      else { ii = idx % nb; r = idx / nb; }         // coalesced along i
      const int i = FORWARD ? s0 + ii : w - 1 - (s0 + ii);
      Es[ii * LE + r] = TRANS ? Tm[i + (long long)r * ldt] : Tm[r + (long long)i * ldt];
    }
    __syncthreads();
    for (int ii = 0; ii < nb; ++ii) {
      const int i = FORWARD ? s0 + ii : w - 1 - (s0 + ii);
      const T* Ei = Es + ii * LE;
      if (!UNIT) {
        if (tid < NC) Bs[i * LD + tid] = Bs[i * LD + tid] / Ei[i];
        __syncthreads();
      }
      const T xi = Bs[i * LD + c];
      if (FORWARD) {
        for (int r = i + 1 + rg; r < w; r += RG) Bs[r * LD + c] = fma(-Ei[r], xi, Bs[r * LD + c]);
      } else {
        for (int r = rg; r < i; r += RG) Bs[r * LD + c] = fma(-Ei[r], xi, Bs[r * LD + c]);
      }
      __syncthreads();
    }
  }
  for (int i = tid; i < w * NC; i += 256) {
    int r = i % w, cc = i / w;
    if (cc < nc) B[r + (col0 + cc) * ldb] = Bs[r * LD + cc];
  }
  // row maxima of this strip of the solution: the balancing keys of the
  // product that takes it as its right operand
  if constexpr (sizeof(T) == 8) {
    if (kj.hkeys != nullptr)
      for (int r = tid; r < w; r += 256) {
        unsigned long long km = 0ULL;
        for (int cc = 0; cc < nc; ++cc) {
          const unsigned long long v = oz_key_word(Bs[r * LD + cc], kj.epoch);
          km = v > km ? v : km;
        }
        if (km) atomicMax(kj.hkeys + r, km);
      }
  }
}

// op(T) x = b for a w x w diagonal block (w <= 128) and few right-hand sides:
// one CTA per right-hand side stages the block's triangle in shared memory
// (row stride w+1, conflict-free) with all its warps, then warp 0 solves the
// column with its 4 rows per lane held in registers;
// x_i is broadcast with a shuffle, so no block-wide barrier sits on the
// dependency chain. Non-unit diagonals divide (reference DTRSM semantics).
template <typename T, bool UPPER, bool TRANS, bool UNIT>
__global__ void __launch_bounds__(256)
trsv_warp_kernel(int w, int ncols, const T* __restrict__ Tm, long long ldt, T* B, long long ldb) {
  extern __shared__ __align__(16) unsigned char trsv_smem[];
  T* Ts = reinterpret_cast<T*>(trsv_smem);  // Ts[r*(w+1) + i] = op(T)(r, i)
  const int W1 = w + 1;
  constexpr bool FORWARD = (UPPER == TRANS);
  // stage only the triangle the solve reads (the diagonal too when non-unit),
  // many loads in flight per thread
#pragma unroll 8
  for (int idx = threadIdx.x; idx < w * w; idx += blockDim.x) {
    int r, i;
    if (!TRANS) { r = idx % w; i = idx / w; }  // coalesced along r
    else { i = idx % w; r = idx / w; }         // coalesced along i
    const bool need = FORWARD ? (r > i || (!UNIT && r == i)) : (r < i || (!UNIT && r == i));
    if (need) Ts[r * W1 + i] = TRANS ? Tm[i + (long long)r * ldt] : Tm[r + (long long)i * ldt];
  }
  __syncthreads();
  // one right-hand side per CTA, solved by warp 0: GB300's FP64 pipe is narrow
  // per SM, so the columns' solves are spread over as many SMs as there are
  // columns; the other warps only help staging
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long col = blockIdx.x;
  if (warp != 0 || col >= ncols) return;
  T x[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    int r = lane + 32 * q;
    x[q] = r < w ? B[r + col * ldb] : (T)0;
  }
  for (int s = 0; s < w; ++s) {
    const int i = FORWARD ? s : w - 1 - s;
    const int qi = i >> 5, li = i & 31;
    if (!UNIT && lane == li) {
      const T dinv = Ts[i * W1 + i];
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (q == qi) x[q] = x[q] / dinv;
    }
    T own = x[0];
#pragma unroll
    for (int q = 1; q < 4; ++q)
      if (q == qi) own = x[q];
    const T xi = __shfl_sync(0xffffffffu, own, li);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int r = lane + 32 * q;
      if (r < w && (FORWARD ? r > i : r < i)) x[q] = fma(-Ts[r * W1 + i], xi, x[q]);
    }
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    int r = lane + 32 * q;
    if (r < w) B[r + col * ldb] = x[q];
  }
}

// Single-launch blocked triangular solve for few right-hand sides (nrhs <=
// NRM), FP32: FORWARD solves with the unit-lower L, otherwise with the
// non-unit upper U, of an n x n LU factor, X (n x nrhs) overwritten in place.
//
// Each CTA takes the next 64-row block (in solve order) from an atomic
// ticket, so every block it depends on belongs to a CTA that has already
// started: the waits below always end (no residency assumption). Solved
// blocks are published as tagged words {x bits, epoch} in xt, so a consumer
// polls the values themselves (one round trip, no flag and no fence). A CTA
// stages the inverse of its diagonal block (precomputed once per factorization,
// diag_inv) and M_b = inv(T_bb) T_bp for its immediate predecessor p in
// shared memory, consumes the earlier solved blocks in chunks as they appear
// (4 thread groups of 64 rows x 16 columns apply the 64x64 blocks of the
// factor), forms y_b = inv(T_bb) v_b before the predecessor is solved, and
// when x_p arrives one 64x64 product from shared memory remains on the chain,
// x_b = y_b - M_b x_p (no serial substitution). Waits are bounded
// (kSpinLimit); on timeout the CTA records kFlagTimeout in *status and stops.
// TM: storage of the factor and of the diagonal-block inverses (FP32). TV:
// the arithmetic and the vectors: FP32, or FP64 for a preconditioner applied
// in the working precision (the FP32 factors and inverses then define the
// operator exactly and only FP64 rounding enters). An FP64 value travels as
// two tagged words (low and high halves).
template <typename TM, typename TV, bool FORWARD, int NRM>
__global__ void __launch_bounds__(256)
trsv_chain_kernel(const TM* __restrict__ A, long long lda, int n, TV* X, long long ldx, int nrhs,
                  const TM* __restrict__ Dinv, const TM* __restrict__ Mp, int* ticket,
                  unsigned long long* xt, int epoch, int* status) {
  static_assert(sizeof(TM) == 4, "FP32 factors");
  constexpr int VW = sizeof(TV) / 4;  // tagged words per value
  constexpr int KB = 64;
  constexpr int kChunk = NRM > 4 ? 1 : (NRM > 1 ? 4 : 8);  // static shared memory under 48 KB
  __shared__ TM Ds[KB][KB + 1];         // inverse of the diagonal block, Ds[r][i]
  __shared__ TM Ms[KB][KB + 1];         // M_b = inv(T_bb) T_bp, Ms[r][i]
  __shared__ TV xs[kChunk * KB][NRM];   // x of the blocks being applied
  __shared__ TV part[4][KB][NRM];       // partial sums of the 4 column groups
  __shared__ int s_b, s_fail, s_bad[kChunk];
  const uint32_t tag = (uint32_t)epoch;
  auto word = [&](int c, long long row) { return xt + ((size_t)c * n + row) * VW; };
  // reads one published value; false while its tag(s) are not the current one
  auto read_val = [&](const unsigned long long* p, TV& v) -> bool {
    if constexpr (VW == 1) {
      unsigned long long wd;
      asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(wd) : "l"(p) : "memory");
      v = __uint_as_float((uint32_t)wd);
      return (uint32_t)(wd >> 32) == tag;
    } else {
      unsigned long long lo, hi;
      asm volatile("ld.relaxed.gpu.global.v2.b64 {%0, %1}, [%2];" : "=l"(lo), "=l"(hi) : "l"(p) : "memory");
      v = __longlong_as_double((long long)(((unsigned long long)(uint32_t)hi << 32) | (uint32_t)lo));
      return (uint32_t)(lo >> 32) == tag && (uint32_t)(hi >> 32) == tag;
    }
  };
  auto publish = [&](unsigned long long* p, TV v) {
    if constexpr (VW == 1) {
      const unsigned long long wd = ((unsigned long long)tag << 32) | __float_as_uint(v);
      asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(wd) : "memory");
    } else {
      const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
      const unsigned long long lo = ((unsigned long long)tag << 32) | (uint32_t)bits;
      const unsigned long long hi = ((unsigned long long)tag << 32) | (uint32_t)(bits >> 32);
      asm volatile("st.relaxed.gpu.global.v2.b64 [%0], {%1, %2};" ::"l"(p), "l"(lo), "l"(hi) : "memory");
    }
  };
  const int tid = threadIdx.x;
  const int nblk = (n + KB - 1) / KB;
  if (tid == 0) { s_b = atomicAdd(ticket, 1); s_fail = 0; }
  __syncthreads();
  const int sidx = s_b;
  if (sidx >= nblk) return;
  const int b = FORWARD ? sidx : nblk - 1 - sidx;
  const int r0 = b * KB, rb = min(KB, n - r0);
  const int kp = FORWARD ? b - 1 : b + 1;  // predecessor in solve order
  const int wp = (sidx > 0) ? min(KB, n - kp * KB) : 0;
  const TM* Db = Dinv + (size_t)b * KB * KB;  // row-major [KB][KB]
  const TM* Mb = Mp + (size_t)b * KB * KB;
  for (int idx = tid; idx < KB * KB; idx += 256) {
    Ds[idx / KB][idx % KB] = Db[idx];
    Ms[idx / KB][idx % KB] = (sidx > 0) ? Mb[idx] : (TM)0;
  }
  const int r = tid & (KB - 1), q = tid >> 6;
  const int warp = tid >> 5, lane = tid & 31;
  // the block's right-hand side, read now rather than on the chain (warp c
  // owns column c; only this CTA writes these rows)
  TV bx0 = (TV)0, bx1 = (TV)0;
  if (warp < nrhs) {
    if (lane < rb) bx0 = X[(r0 + lane) + (long long)warp * ldx];
    if (lane + 32 < rb) bx1 = X[(r0 + lane + 32) + (long long)warp * ldx];
  }
  TV acc[NRM];
#pragma unroll
  for (int c = 0; c < NRM; ++c) acc[c] = (TV)0;
  // Blocks 0 .. sidx-2 in solve order: chunks of the consecutive solved blocks
  // that are already published (at least the first one, waited for).
  int t = 0;
  long long spins = 0;
  while (t < sidx - 1) {
    const int want = min(kChunk, sidx - 1 - t);
    const int kfirst = FORWARD ? t : nblk - 1 - (t + want - 1);  // lowest block of the chunk
    const int k0 = kfirst * KB;
    const int kn = min(want * KB, n - k0);
    if (tid == 0) {
      // one thread watches the chunk's first block (its last value) before the
      // whole chunk is read, so waiting CTAs do not stream through L2
      const int kb0 = FORWARD ? t : nblk - 1 - t;
      const unsigned long long* p = word(0, kb0 * KB + min(KB, n - kb0 * KB) - 1);
      for (long long sp = 0;; ++sp) {
        TV v;
        if (read_val(p, v)) break;
        if (sp > kSpinLimit) { s_fail = 1; break; }
      }
    }
    if (tid < kChunk) s_bad[tid] = 0;
    __syncthreads();
    if (s_fail) {
      if (tid == 0) atomicExch(status, (int)kFlagTimeout);
      return;
    }
    for (int idx = tid; idx < kn * nrhs; idx += 256) {
      const int i = idx % kn, c = idx / kn;
      TV v;
      if (!read_val(word(c, k0 + i), v)) {
        const int blk = i / KB;                                  // chunk block, matrix order
        s_bad[FORWARD ? blk : want - 1 - blk] = 1;               // solve order
      }
      xs[i][c] = v;
    }
    __syncthreads();
    int av = 0;
    while (av < want && s_bad[av] == 0) ++av;
    if (av == 0) {  // the watched value arrived before the rest of its block
      if (++spins > kSpinLimit) {
        if (tid == 0) atomicExch(status, (int)kFlagTimeout);
        return;
      }
      __syncthreads();  // everyone has read s_bad before it is reset
      continue;
    }
    // columns of the av complete blocks, in matrix order
    const int c0 = FORWARD ? 0 : (want - av) * KB;
    const int c1 = FORWARD ? min(av * KB, kn) : kn;
    if (r < rb) {
      for (int g0 = c0 + q * 16; g0 < c1; g0 += 64) {
        const int g1 = min(g0 + 16, c1);
        for (int kk = g0; kk < g1; ++kk) {
          const TV a = (TV)A[(r0 + r) + (long long)(k0 + kk) * lda];
#pragma unroll
          for (int c = 0; c < NRM; ++c)
            if (c < nrhs) acc[c] = fma(a, xs[kk][c], acc[c]);
        }
      }
    }
    __syncthreads();
    t += av;
  }
#pragma unroll
  for (int c = 0; c < NRM; ++c) part[q][r][c] = acc[c];
  __syncthreads();
  // v = b - sum of the partials (warp c owns column c, lanes rows lane and
  // lane+32), then y = inv(T_bb) v by all four thread groups
  __shared__ TV vs[NRM][KB];
  if (warp < nrhs) {
    const int c = warp;
    TV v0 = (TV)0, v1 = (TV)0;
    if (lane < rb) v0 = bx0 - (part[0][lane][c] + part[1][lane][c] + part[2][lane][c] + part[3][lane][c]);
    if (lane + 32 < rb)
      v1 = bx1 - (part[0][lane + 32][c] + part[1][lane + 32][c] + part[2][lane + 32][c] + part[3][lane + 32][c]);
    vs[c][lane] = v0;
    vs[c][lane + 32] = v1;
  }
  __syncthreads();
  {
#pragma unroll
    for (int c = 0; c < NRM; ++c) acc[c] = (TV)0;
#pragma unroll
    for (int i = q * 16; i < q * 16 + 16; ++i) {
      const TV d = (TV)Ds[r][i];
#pragma unroll
      for (int c = 0; c < NRM; ++c)
        if (c < nrhs) acc[c] = fma(d, vs[c][i], acc[c]);
    }
#pragma unroll
    for (int c = 0; c < NRM; ++c) part[q][r][c] = acc[c];
  }
  __syncthreads();
  TV x0 = (TV)0, x1 = (TV)0;
  if (warp < nrhs) {
    const int c = warp;
    x0 = part[0][lane][c] + part[1][lane][c] + part[2][lane][c] + part[3][lane][c];
    x1 = part[0][lane + 32][c] + part[1][lane + 32][c] + part[2][lane + 32][c] + part[3][lane + 32][c];
  }
  // The predecessor: poll its x (the chain's one round trip), x -= M_b x_p.
  if (sidx > 0) {
    for (int idx = tid; idx < wp * nrhs; idx += 256) {
      const int i = idx % wp, c = idx / wp;
      const unsigned long long* p = word(c, kp * KB + i);
      TV v = (TV)0;
      for (long long sp = 0;; ++sp) {
        if (read_val(p, v)) break;
        if (sp > kSpinLimit) { s_fail = 1; break; }
      }
      xs[i][c] = v;
    }
    __syncthreads();  // also orders the reads of part above before the writes below
    if (s_fail) {
      if (tid == 0) atomicExch(status, (int)kFlagTimeout);
      return;
    }
#pragma unroll
    for (int c = 0; c < NRM; ++c) acc[c] = (TV)0;
#pragma unroll 4
    for (int kk = q * 16; kk < q * 16 + 16; ++kk) {
      if (kk < wp) {
        const TV m = (TV)Ms[r][kk];
#pragma unroll
        for (int c = 0; c < NRM; ++c)
          if (c < nrhs) acc[c] = fma(m, xs[kk][c], acc[c]);
      }
    }
#pragma unroll
    for (int c = 0; c < NRM; ++c) part[q][r][c] = acc[c];
    __syncthreads();
    if (warp < nrhs) {
      const int c = warp;
      x0 -= part[0][lane][c] + part[1][lane][c] + part[2][lane][c] + part[3][lane][c];
      x1 -= part[0][lane + 32][c] + part[1][lane + 32][c] + part[2][lane + 32][c] + part[3][lane + 32][c];
    }
  }
  // publish: tagged words for the consumers, plain values for the result
  if (warp < nrhs) {
    const int c = warp;
    if (lane < rb) {
      publish(word(c, r0 + lane), x0);
      X[(r0 + lane) + (long long)c * ldx] = x0;
    }
    if (lane + 32 < rb) {
      publish(word(c, r0 + lane + 32), x1);
      X[(r0 + lane + 32) + (long long)c * ldx] = x1;
    }
  }
}

// Launch the chained solve; `sync` holds 1 ticket int (64 bytes reserved)
// followed by the tagged words: n x nrhs values of 1 (FP32) or 2 (FP64) words
// (zeroed once; epoch must differ from every earlier one).
template <typename TM, typename TV, bool FORWARD>
inline cudaError_t trsv_chain(const TM* A, long long lda, int n, TV* X, long long ldx, int nrhs,
                              const TM* Dinv, const TM* Mp, int* sync, int epoch, int* status,
                              cudaStream_t s) {
  if (n <= 0 || nrhs <= 0) return cudaSuccess;
  const int nblk = (n + 63) / 64;
  SL_TRY(cudaMemsetAsync(sync, 0, sizeof(int), s));
  unsigned long long* xt = reinterpret_cast<unsigned long long*>(sync + 16);
  if (nrhs <= 1)
    trsv_chain_kernel<TM, TV, FORWARD, 1><<<nblk, 256, 0, s>>>(A, lda, n, X, ldx, nrhs, Dinv, Mp, sync, xt, epoch, status);
  else if constexpr (sizeof(TV) == 8)
    return cudaErrorInvalidValue;  // FP64 vectors: one right-hand side (GMRES)
  else if (nrhs <= 4)
    trsv_chain_kernel<TM, TV, FORWARD, 4><<<nblk, 256, 0, s>>>(A, lda, n, X, ldx, nrhs, Dinv, Mp, sync, xt, epoch, status);
  else
    trsv_chain_kernel<TM, TV, FORWARD, 8><<<nblk, 256, 0, s>>>(A, lda, n, X, ldx, nrhs, Dinv, Mp, sync, xt, epoch, status);
  count_launches(1);
  return cudaGetLastError();
}

// dst(i, c) = src(perm[i], c) (forward) or dst(perm[i], c) = src(i, c) (inverse).
template <typename TS, typename TD>
__global__ void permute_rows_kernel(const TS* __restrict__ src, long long lds, TD* dst,
                                    long long ldd, const int* __restrict__ perm, int n, int nrhs,
                                    int inverse) {
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)n * nrhs) return;
  int i = (int)(idx % n), c = (int)(idx / n);
  int p = perm[i];
  if (!inverse) dst[i + c * ldd] = (TD)src[p + c * lds];
  else dst[p + c * ldd] = (TD)src[i + c * lds];
}

// C (m x n) += alpha * op(A) (m x k) * B (k x n) for n <= NC <= 16 and any k:
// one thread per row of C, B staged in 64-row chunks through shared memory.
// Used for the narrow off-diagonal updates of the triangular solves and for
// residuals b - A x with a few right-hand sides.
template <typename T, bool TRANSA, int NC>
__global__ void __launch_bounds__(256)
gemm_skinny_kernel(int m, int n, int k, T alpha, const T* __restrict__ A, long long lda,
                   const T* __restrict__ B, long long ldb, T* C, long long ldc) {
  __shared__ T Bs[64][NC];
  const long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  T acc[NC];
#pragma unroll
  for (int j = 0; j < NC; ++j) acc[j] = (T)0;
  for (int k0 = 0; k0 < k; k0 += 64) {
    const int kc = min(64, k - k0);
    __syncthreads();
    for (int c = threadIdx.x; c < 64 * NC; c += blockDim.x) {
      int kk = c % 64, nn = c / 64;
      Bs[kk][nn] = (kk < kc && nn < n) ? B[(k0 + kk) + (long long)nn * ldb] : (T)0;
    }
    __syncthreads();
    if (row < m) {
#pragma unroll 16
      for (int kk = 0; kk < kc; ++kk) {
        T a = TRANSA ? A[(k0 + kk) + row * lda] : A[row + (long long)(k0 + kk) * lda];
#pragma unroll
        for (int j = 0; j < NC; ++j) acc[j] = fma(a, Bs[kk][j], acc[j]);
      }
    }
  }
  if (row < m) {
#pragma unroll
    for (int j = 0; j < NC; ++j)
      if (j < n) C[row + (long long)j * ldc] += alpha * acc[j];
  }
}

// ------------------------------------------------------------ launch helpers

template <typename T>
inline cudaError_t launch_panel(T* A, long long lda, int m, int r0, int c0, int w, int* ipiv,
                                const LuWork& ws, cudaStream_t s) {
  const int R = m - r0;
  // Rows per CTA: about 64 CTAs per panel, and at least the type's minimum
  // (FP32 256, FP64 128, or the tuning knob). Fewer CTAs make the per-column
  // exchange cheaper (fewer keys to poll, less cross-die skew); more rows per
  // CTA make the rank-1 update longer -- on GB300's FP64 pipe sooner than on
  // the FP32 one.
  // Tall panels beyond 64 CTAs' shared memory spread over every SM instead;
  // beyond every SM's shared memory the rows go to the global buffer ws.ptile.
  const int rpc_max = (int)((200 * 1024) / (sizeof(T) * PLD)) & ~7;
  int rpc = (R + panel_ctas() - 1) / panel_ctas();
  const int lo_rows = panel_min_rows() > 0 ? panel_min_rows() : (sizeof(T) == 4 ? 256 : 128);
  if (rpc < lo_rows) rpc = lo_rows;
  if (rpc > rpc_max) rpc = (R + num_sms() - 1) / num_sms();
  rpc = (rpc + 7) & ~7;
  int G = (R + rpc - 1) / rpc;
  size_t smem = sizeof(T) * (size_t)rpc * PLD;
  const bool global_tile = smem > 200 * 1024 || G > PMAXG;
  T* gtile = nullptr;
  if (global_tile) {
    if constexpr (sizeof(T) != 8) {
      return cudaErrorInvalidValue;  // M beyond the FP32 panel limit
    } else {
      G = std::min(PMAXG, num_sms());
      rpc = ((R + G - 1) / G + 7) & ~7;
      G = (R + rpc - 1) / rpc;
      if (!ws.ptile || ws.ptile_len < (size_t)G * rpc * PW) return cudaErrorInvalidValue;
      gtile = ws.ptile;
      smem = 0;
    }
  }
  if (!global_tile) SL_TRY(smem_attr_once((const void*)panel_kernel<T, false>, 200 * 1024));
  // zero the diagonal rows and the G slots used (stale tags must not match)
  cudaError_t e = cudaMemsetAsync(ws.cand, 0, sizeof(unsigned long long) * ((size_t)PX_VALS + (size_t)G * 2 * 2 * PW), s);
  if (e != cudaSuccess) return e;
  long long limit = spin_limit();
  void* args[] = {&A, &lda, &m, &r0, &c0, &w, (void*)&rpc, &ipiv, (void*)&ws.info_col,
                  (void*)&ws.cand, (void*)&ws.status, (void*)&limit, (void*)&gtile};
  count_launches(1);
  if (global_tile)
    return cudaLaunchCooperativeKernel((void*)panel_kernel<T, true>, dim3(G), dim3(PT), args, 0, s);
  return cudaLaunchCooperativeKernel((void*)panel_kernel<T, false>, dim3(G), dim3(PT), args, smem, s);
}

template <typename T>
inline cudaError_t laswp(T* A, long long lda, int k1, int k2, const int* ipiv, int cb1, int ce1,
                         int cb2, int ce2, cudaStream_t s) {
  const long long ncols = (long long)(ce1 - cb1) + (ce2 - cb2);
  if (ncols <= 0 || k2 <= k1) return cudaSuccess;
  if (k2 - k1 > LSW_MAXP) {
    dim3 grid((unsigned)((ncols + 255) / 256));
    laswp_seq_kernel<T><<<grid, 256, 0, s>>>(A, lda, k1, k2, ipiv, cb1, ce1, cb2, ce2);
  } else {
    // one warp per column, at most 4 CTAs per SM's worth of CTAs
    const long long want = (ncols + 7) / 8;
    const long long cap = 4LL * num_sms();
    laswp_kernel<T><<<(unsigned)(want < cap ? want : cap), 256, 0, s>>>(A, lda, k1, k2, ipiv, cb1,
                                                                         ce1, cb2, ce2);
  }
  count_launches(1);
  return cudaGetLastError();
}

// Plan of a panel's interchanges (k2 - k1 <= LSW_MAXP), see laswp_plan_kernel.
inline cudaError_t laswp_plan(int k1, int k2, const int* ipiv, int* plan, cudaStream_t s) {
  if (k2 - k1 > LSW_MAXP) return cudaErrorInvalidValue;
  if (k2 <= k1) return cudaMemsetAsync(plan, 0, sizeof(int), s);
  laswp_plan_kernel<<<1, 256, 0, s>>>(k1, k2, ipiv, plan);
  count_launches(1);
  return cudaGetLastError();
}

// Row interchanges from a plan when one is available, else as laswp().
template <typename T>
inline cudaError_t laswp_planned(T* A, long long lda, int k1, int k2, const int* ipiv,
                                 const int* plan, int cb1, int ce1, int cb2, int ce2,
                                 cudaStream_t s, int max_ctas = 0) {
  const long long ncols = (long long)(ce1 - cb1) + (ce2 - cb2);
  if (ncols <= 0 || k2 <= k1) return cudaSuccess;
  if (!plan || k2 - k1 > LSW_MAXP) return laswp<T>(A, lda, k1, k2, ipiv, cb1, ce1, cb2, ce2, s);
  const long long want = (ncols + 7) / 8;
  const long long cap = max_ctas > 0 ? (long long)max_ctas : 4LL * num_sms();
  laswp_apply_kernel<T><<<(unsigned)(want < cap ? want : cap), 256, 0, s>>>(A, lda, plan, cb1, ce1,
                                                                            cb2, ce2);
  count_launches(1);
  return cudaGetLastError();
}

template <typename T, bool UPPER, bool TRANS, bool UNIT, int NC = 8>
inline cudaError_t trsm_strip(int w, int ncols, const T* Tm, long long ldt, T* B, long long ldb,
                              cudaStream_t s, const OzKeyJob& kj = OzKeyJob()) {
  if (w <= 0 || ncols <= 0) return cudaSuccess;
  // staged triangle columns per block: up to 32, within 200 KB of shared memory
  constexpr size_t kBudget = 200 * 1024;
  const size_t bbytes = sizeof(T) * (size_t)w * (NC + 1);
  const size_t ecol = sizeof(T) * (size_t)(w + 1);
  if (bbytes + ecol > kBudget) return cudaErrorInvalidValue;
  const int eb = (int)std::min<size_t>(TRSM_EB, (kBudget - bbytes) / ecol);
  const size_t smem = bbytes + (size_t)eb * ecol;
  auto kern = trsm_strip_kernel<T, UPPER, TRANS, UNIT, NC>;
  SL_TRY(smem_attr_once((const void*)kern, (int)kBudget));
  dim3 grid((ncols + NC - 1) / NC + (kj.ckeys ? (kj.lrows + 31) / 32 : 0));
  kern<<<grid, 256, smem, s>>>(w, ncols, eb, Tm, ldt, B, ldb, kj);
  count_launches(1);
  return cudaGetLastError();
}

// The same product with each row tile split across NC/4 column groups of 4
// (64 rows per CTA for NC = 16, 128 for NC = 8): 4x more CTAs than
// gemm_skinny_kernel, so that a product with few rows still fills every SM
// (the off-diagonal updates of a blocked triangular solve with 8-16 right-hand
// sides).
template <typename T, bool TRANSA, int NC>
__global__ void __launch_bounds__(256)
gemm_skinny_rt_kernel(int m, int n, int k, T alpha, const T* __restrict__ A, long long lda,
                      const T* __restrict__ B, long long ldb, T* C, long long ldc) {
  static_assert(NC % 4 == 0 && NC >= 8, "column groups of 4");
  constexpr int G = NC / 4;    // column groups
  constexpr int RT = 256 / G;  // rows per CTA
  __shared__ T Bs[64][NC];
  const int g = threadIdx.x / RT, rl = threadIdx.x % RT;
  const long long row = (long long)blockIdx.x * RT + rl;
  T acc[4] = {(T)0, (T)0, (T)0, (T)0};
  for (int k0 = 0; k0 < k; k0 += 64) {
    const int kc = min(64, k - k0);
    __syncthreads();
    for (int c = threadIdx.x; c < 64 * NC; c += blockDim.x) {
      int kk = c % 64, nn = c / 64;
      Bs[kk][nn] = (kk < kc && nn < n) ? B[(k0 + kk) + (long long)nn * ldb] : (T)0;
    }
    __syncthreads();
    if (row < m) {
#pragma unroll 16
      for (int kk = 0; kk < kc; ++kk) {
        const T a = TRANSA ? A[(k0 + kk) + row * lda] : A[row + (long long)(k0 + kk) * lda];
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[j] = fma(a, Bs[kk][g * 4 + j], acc[j]);
      }
    }
  }
  if (row < m) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = g * 4 + j;
      if (c < n) C[row + (long long)c * ldc] += alpha * acc[j];
    }
  }
}

template <typename T, bool TA, int NC>
inline cudaError_t launch_skinny(int m, int n, int k, T alpha, const T* A, long long lda,
                                 const T* B, long long ldb, T* C, long long ldc, cudaStream_t s) {
  dim3 grid((m + 255) / 256);
  gemm_skinny_kernel<T, TA, NC><<<grid, 256, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, C, ldc);
  count_launches(1);
  return cudaGetLastError();
}

// Split-K form for long k (matrix-vector products of the refinement): CTA
// (bx, by) computes rows 256*bx.. of op(A)[:, kslice(by)] * B into its own
// partial slot; gemm_skinny_reduce adds the ksplit partials in a fixed order.
template <typename T, int NC>
__global__ void __launch_bounds__(256)
gemm_skinny_splitk_kernel(int m, int n, int k, int kslice, const T* __restrict__ A, long long lda,
                          const T* __restrict__ B, long long ldb, T* part) {
  __shared__ T Bs[64][NC];
  const long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int kbeg = blockIdx.y * kslice, kend = min(k, kbeg + kslice);
  T acc[2][NC];
#pragma unroll
  for (int j = 0; j < NC; ++j) { acc[0][j] = (T)0; acc[1][j] = (T)0; }
  for (int k0 = kbeg; k0 < kend; k0 += 64) {
    const int kc = min(64, kend - k0);
    __syncthreads();
    for (int c = threadIdx.x; c < 64 * NC; c += blockDim.x) {
      int kk = c % 64, nn = c / 64;
      Bs[kk][nn] = (kk < kc && nn < n) ? B[(k0 + kk) + (long long)nn * ldb] : (T)0;
    }
    __syncthreads();
    if (row < m) {
      int kk = 0;
      for (; kk + 1 < kc; kk += 2) {  // two independent accumulator chains
        const T a0 = A[row + (long long)(k0 + kk) * lda];
        const T a1 = A[row + (long long)(k0 + kk + 1) * lda];
#pragma unroll
        for (int j = 0; j < NC; ++j) {
          acc[0][j] = fma(a0, Bs[kk][j], acc[0][j]);
          acc[1][j] = fma(a1, Bs[kk + 1][j], acc[1][j]);
        }
      }
      if (kk < kc) {
        const T a0 = A[row + (long long)(k0 + kk) * lda];
#pragma unroll
        for (int j = 0; j < NC; ++j) acc[0][j] = fma(a0, Bs[kk][j], acc[0][j]);
      }
    }
  }
  if (row < m) {
#pragma unroll
    for (int j = 0; j < NC; ++j)
      if (j < n) part[((long long)blockIdx.y * n + j) * m + row] = acc[0][j] + acc[1][j];
  }
}

template <typename T>
__global__ void gemm_skinny_reduce_kernel(int m, int n, int ksplit, T alpha, const T* part, T* C,
                                          long long ldc) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)m * n) return;
  const int row = (int)(idx % m), j = (int)(idx / m);
  T s = (T)0;
  for (int q = 0; q < ksplit; ++q) s += part[((long long)q * n + j) * m + row];
  C[row + (long long)j * ldc] += alpha * s;
}

// C += alpha * op(A) * B for n <= 16 columns.
template <typename T>
inline cudaError_t gemm_skinny(bool transa, int m, int n, int k, T alpha, const T* A,
                               long long lda, const T* B, long long ldb, T* C, long long ldc,
                               cudaStream_t s) {
  if (m <= 0 || n <= 0 || k <= 0) return cudaSuccess;
  if (!transa && n <= 4 && k >= 4096) {
    // long products: spread k over ksplit CTA columns so every SM works
    const int rb = (m + 255) / 256;
    int ksplit = (4 * num_sms() + rb - 1) / rb;
    if (ksplit > 32) ksplit = 32;
    if (ksplit > 1) {
      SplitKScratch& sc = splitk_scratch();
      const size_t need = sizeof(T) * (size_t)ksplit * n * m;
      if (sc.ptr && sc.bytes >= need) {
        const int kslice = ((k + ksplit - 1) / ksplit + 63) / 64 * 64;
        ksplit = (k + kslice - 1) / kslice;
        dim3 grid(rb, ksplit);
        T* part = reinterpret_cast<T*>(sc.ptr);
        if (n == 1) gemm_skinny_splitk_kernel<T, 1><<<grid, 256, 0, s>>>(m, n, k, kslice, A, lda, B, ldb, part);
        else gemm_skinny_splitk_kernel<T, 4><<<grid, 256, 0, s>>>(m, n, k, kslice, A, lda, B, ldb, part);
        const long long tot = (long long)m * n;
        gemm_skinny_reduce_kernel<T><<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(m, n, ksplit, alpha, part, C, ldc);
        count_launches(2);
        return cudaGetLastError();
      }
    }
  }
  if (n > 4 && (m + 255) / 256 < 2 * num_sms()) {
    // few rows: split each row tile over column groups so that every SM works
    const int nc = n <= 8 ? 8 : 16;
    const int rt = 256 / (nc / 4);
    dim3 grid((unsigned)((m + rt - 1) / rt));
    if (nc == 8) {
      if (transa) gemm_skinny_rt_kernel<T, true, 8><<<grid, 256, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, C, ldc);
      else gemm_skinny_rt_kernel<T, false, 8><<<grid, 256, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, C, ldc);
    } else {
      if (transa) gemm_skinny_rt_kernel<T, true, 16><<<grid, 256, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, C, ldc);
      else gemm_skinny_rt_kernel<T, false, 16><<<grid, 256, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, C, ldc);
    }
    count_launches(1);
    return cudaGetLastError();
  }
#define SL_SK(NC)                                                                              \
  return transa ? launch_skinny<T, true, NC>(m, n, k, alpha, A, lda, B, ldb, C, ldc, s)        \
                : launch_skinny<T, false, NC>(m, n, k, alpha, A, lda, B, ldb, C, ldc, s)
  if (n == 1) { SL_SK(1); }
  if (n <= 2) { SL_SK(2); }
  if (n <= 4) { SL_SK(4); }
  if (n <= 8) { SL_SK(8); }
  SL_SK(16);
#undef SL_SK
}

template <typename TS, typename TD>
inline cudaError_t permute_rows(const TS* src, long long lds, TD* dst, long long ldd,
                                const int* perm, int n, int nrhs, int inverse, cudaStream_t s) {
  const long long total = (long long)n * nrhs;
  if (total <= 0) return cudaSuccess;
  permute_rows_kernel<TS, TD><<<(unsigned)((total + 255) / 256), 256, 0, s>>>(
      src, lds, dst, ldd, perm, n, nrhs, inverse);
  count_launches(1);
  return cudaGetLastError();
}

// C += alpha op(A) B for the off-diagonal blocks of the solves (defined per
// type: FP64 in lu_f64.cu with DMMA for wide B, FP32 in mixed.cu).
template <typename T>
cudaError_t gemm_update(bool transa, int m, int n, int k, T alpha, const T* A, long long lda,
                        const T* B, long long ldb, T* C, long long ldc, cudaStream_t s);
template <>
cudaError_t gemm_update<double>(bool, int, int, int, double, const double*, long long,
                                const double*, long long, double*, long long, cudaStream_t);
template <>
cudaError_t gemm_update<float>(bool, int, int, int, float, const float*, long long, const float*,
                               long long, float*, long long, cudaStream_t);

template <typename T, bool UPPER, bool TRANS, bool UNIT>
inline cudaError_t diag_solve(int kb, int nrhs, const T* Td, long long lda, T* X, long long ldx,
                              cudaStream_t s) {
  if (kb <= 128 && nrhs <= 16) {
    // Few right-hand sides: one warp per column, the block in shared memory.
    auto kern = trsv_warp_kernel<T, UPPER, TRANS, UNIT>;
    SL_TRY(smem_attr_once((const void*)kern, 140 * 1024));
    const size_t smem = sizeof(T) * (size_t)kb * (kb + 1);
    kern<<<nrhs, 256, smem, s>>>(kb, nrhs, Td, lda, X, ldx);
    count_launches(1);
    return cudaGetLastError();
  }
  return trsm_strip<T, UPPER, TRANS, UNIT, 8>(kb, nrhs, Td, lda, X, ldx, s);
}

// Blocked triangular solve op(T) X = X with the n x n LU factors in A:
// lower = unit-lower L, otherwise non-unit upper U; trans solves with T^T.
// Diagonal blocks (256 wide for large n, 64 otherwise) are solved in shared
// memory; off-diagonal blocks are applied with gemm_update.
template <typename T>
inline cudaError_t tri_solve(bool lower, bool trans, bool unit, int n, int nrhs, const T* A,
                             long long lda, T* X, long long ldx, cudaStream_t s) {
  const int KB = nrhs <= 16 ? 128 : (n >= 2048 ? 256 : 64);
  const bool forward = (lower != trans);
  const int nblk = (n + KB - 1) / KB;
  for (int bi = 0; bi < nblk; ++bi) {
    const int b = forward ? bi : nblk - 1 - bi;
    const int k0 = b * KB;
    const int kb = (n - k0) < KB ? (n - k0) : KB;
    const T* Td = A + k0 + (long long)k0 * lda;
    if (lower && !trans) SL_TRY((diag_solve<T, false, false, true>(kb, nrhs, Td, lda, X + k0, ldx, s)));
    else if (!lower && !trans) {
      if (unit) SL_TRY((diag_solve<T, true, false, true>(kb, nrhs, Td, lda, X + k0, ldx, s)));
      else SL_TRY((diag_solve<T, true, false, false>(kb, nrhs, Td, lda, X + k0, ldx, s)));
    } else if (!lower && trans) SL_TRY((diag_solve<T, true, true, false>(kb, nrhs, Td, lda, X + k0, ldx, s)));
    else SL_TRY((diag_solve<T, false, true, true>(kb, nrhs, Td, lda, X + k0, ldx, s)));
    if (forward) {
      const int rest = n - k0 - kb;
      if (rest > 0) {
        // X[k0+kb:] -= op(T)[k0+kb:, k0:k0+kb] * X[k0:k0+kb]
        const T* Aoff = trans ? A + k0 + (long long)(k0 + kb) * lda : A + (k0 + kb) + (long long)k0 * lda;
        SL_TRY(gemm_update<T>(trans, rest, nrhs, kb, (T)-1, Aoff, lda, X + k0, ldx, X + k0 + kb, ldx, s));
      }
    } else if (k0 > 0) {
      // X[0:k0] -= op(T)[0:k0, k0:k0+kb] * X[k0:k0+kb]
      const T* Aoff = trans ? A + k0 : A + (long long)k0 * lda;
      SL_TRY(gemm_update<T>(trans, k0, nrhs, kb, (T)-1, Aoff, lda, X + k0, ldx, X, ldx, s));
    }
  }
  return cudaSuccess;
}

}  // namespace sl
