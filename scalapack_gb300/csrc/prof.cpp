// Phase timers of the sl1x1 library: the GPU counterpart of the reference's
// SLTIMER wall-clock timers (TOOLS/sltimer.f:47-113), which the LU tester
// wraps around PDGETRF and PDGETRS (TESTING/traditional/LIN/pdludriver.f:
// 376-383, 706-713). When enabled, every launch of a timed phase is bracketed
// by CUDA events on the launching stream, and the algorithmic flop and byte
// counts of each launch are accumulated, so a caller can compute achieved
// TFLOP/s or GB/s per phase without a profiler. A launch counter is always on.
#include <cuda_runtime.h>

#include <mutex>
#include <vector>

#include "sl_internal.h"

namespace sl {
namespace {

struct PhaseRec {
  std::vector<cudaEvent_t> begin, end;
  double flops = 0.0, bytes = 0.0;
  long long launches = 0;
};

std::mutex g_pm;
bool g_on = false;
// Per host thread: a ProfSuppress on one thread leaves the timers of calls on
// other threads untouched, so it needs no lock.
thread_local bool g_suppressed = false;
PhaseRec g_ph[kNumPhases];
std::vector<cudaEvent_t> g_pool;
long long g_launches = 0;
int g_open_phase = -1;

cudaEvent_t get_event() {
  if (!g_pool.empty()) {
    cudaEvent_t e = g_pool.back();
    g_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

void recycle_all() {
  for (auto& p : g_ph) {
    for (auto e : p.begin) g_pool.push_back(e);
    for (auto e : p.end) g_pool.push_back(e);
    p = PhaseRec();
  }
}

}  // namespace

void count_launches(int n) {
  std::lock_guard<std::mutex> lk(g_pm);
  g_launches += n;
}

ProfSuppress::ProfSuppress() { g_suppressed = true; }
ProfSuppress::~ProfSuppress() { g_suppressed = false; }

void phase_begin(int phase, cudaStream_t s) {
  if (g_suppressed) return;
  std::lock_guard<std::mutex> lk(g_pm);
  if (!g_on || phase < 0 || phase >= kNumPhases) return;
  cudaEvent_t e = get_event();
  cudaEventRecord(e, s);
  g_ph[phase].begin.push_back(e);
  g_open_phase = phase;
}

void phase_end(int phase, cudaStream_t s, double flops, double bytes) {
  if (g_suppressed) return;
  std::lock_guard<std::mutex> lk(g_pm);
  if (!g_on || phase < 0 || phase >= kNumPhases) return;
  cudaEvent_t e = get_event();
  cudaEventRecord(e, s);
  g_ph[phase].end.push_back(e);
  g_ph[phase].flops += flops;
  g_ph[phase].bytes += bytes;
  g_ph[phase].launches += 1;
  g_open_phase = -1;
}

void prof_enable(bool on) {
  std::lock_guard<std::mutex> lk(g_pm);
  cudaDeviceSynchronize();
  recycle_all();
  g_on = on;
}

bool prof_read(int phase, long long* launches, double* ms, double* flops, double* bytes) {
  std::lock_guard<std::mutex> lk(g_pm);
  if (phase < 0 || phase >= kNumPhases) return false;
  PhaseRec& p = g_ph[phase];
  double total = 0.0;
  size_t n = p.begin.size() < p.end.size() ? p.begin.size() : p.end.size();
  for (size_t i = 0; i < n; ++i) {
    float t = 0.f;
    if (cudaEventSynchronize(p.end[i]) == cudaSuccess &&
        cudaEventElapsedTime(&t, p.begin[i], p.end[i]) == cudaSuccess)
      total += t;
  }
  *launches = p.launches;
  *ms = total;
  *flops = p.flops;
  *bytes = p.bytes;
  return true;
}

long long launch_count() {
  std::lock_guard<std::mutex> lk(g_pm);
  return g_launches;
}

}  // namespace sl
