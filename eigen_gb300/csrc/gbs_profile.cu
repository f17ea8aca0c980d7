// Phase profiler and launch counter (see gbs_profile.cuh).
#include <atomic>
#include <mutex>
#include <vector>

#include "gb300solve.h"
#include "gbs_profile.cuh"

namespace gbs {

static std::atomic<uint64_t> g_launches{0};
static std::atomic<int> g_enabled{0};

struct Rec {
  cudaEvent_t b, e;
  cudaStream_t stream;
  int phase;
  double flops, bytes;
  bool closed;
};
static std::mutex g_mu;
static std::vector<Rec> g_recs;
static std::vector<cudaEvent_t> g_free;
static thread_local std::vector<size_t> t_open;   // indices of open records (stack)

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
bool profiling() { return g_enabled.load(std::memory_order_relaxed) != 0; }

static cudaEvent_t take_event()
{
  if (!g_free.empty()) {
    cudaEvent_t e = g_free.back();
    g_free.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

void prof_begin(cudaStream_t s, int phase)
{
  if (!profiling()) return;
  std::lock_guard<std::mutex> lk(g_mu);
  Rec r;
  r.b = take_event();
  r.e = take_event();
  r.phase = phase;
  r.stream = s;
  r.flops = r.bytes = 0;
  r.closed = false;
  cudaEventRecord(r.b, s);
  g_recs.push_back(r);
  t_open.push_back(g_recs.size() - 1);
}

void prof_end(cudaStream_t s, int phase, double flops, double bytes)
{
  if (!profiling() || t_open.empty()) return;
  std::lock_guard<std::mutex> lk(g_mu);
  size_t i = t_open.back();
  t_open.pop_back();
  if (i >= g_recs.size()) return;
  Rec& r = g_recs[i];
  r.flops = flops;
  r.bytes = bytes;
  r.closed = true;
  (void)phase;
  cudaEventRecord(r.e, s);
}

}  // namespace gbs

using namespace gbs;

extern "C" uint64_t gbs_kernel_launch_count(void) { return g_launches.load(); }

extern "C" int gbs_profile_enable(int on)
{
  g_enabled.store(on ? 1 : 0);
  return GBS_SUCCESS;
}

extern "C" int gbs_profile_reset(void)
{
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto& r : g_recs) {
    g_free.push_back(r.b);
    g_free.push_back(r.e);
  }
  g_recs.clear();
  return GBS_SUCCESS;
}

extern "C" int gbs_profile_timeline(int* phase, int* stream, double* start_ms, double* end_ms, int cap)
{
  std::lock_guard<std::mutex> lk(g_mu);
  std::vector<cudaStream_t> seen;
  int cnt = 0;
  for (auto& r : g_recs) {
    if (!r.closed) continue;
    if (cudaEventSynchronize(r.e) != cudaSuccess) return -(100 + GBS_CUDA_ERROR);
    if (cnt < cap) {
      float t0 = 0, t1 = 0;
      if (cudaEventElapsedTime(&t0, g_recs[0].b, r.b) != cudaSuccess ||
          cudaEventElapsedTime(&t1, g_recs[0].b, r.e) != cudaSuccess)
        return -(100 + GBS_CUDA_ERROR);
      int si = 0;
      while (si < (int)seen.size() && seen[si] != r.stream) ++si;
      if (si == (int)seen.size()) seen.push_back(r.stream);
      if (phase) phase[cnt] = r.phase;
      if (stream) stream[cnt] = si;
      if (start_ms) start_ms[cnt] = t0;
      if (end_ms) end_ms[cnt] = t1;
    }
    ++cnt;
  }
  return cnt;
}

extern "C" int gbs_profile_collect(int phase, double* ms_total, int64_t* launches, double* flops, double* bytes)
{
  std::lock_guard<std::mutex> lk(g_mu);
  double ms = 0, f = 0, b = 0;
  int64_t cnt = 0;
  for (auto& r : g_recs) {
    if (r.phase != phase || !r.closed) continue;
    if (cudaEventSynchronize(r.e) != cudaSuccess) return GBS_CUDA_ERROR;
    float t = 0;
    if (cudaEventElapsedTime(&t, r.b, r.e) != cudaSuccess) return GBS_CUDA_ERROR;
    ms += t;
    f += r.flops;
    b += r.bytes;
    ++cnt;
  }
  if (ms_total) *ms_total = ms;
  if (launches) *launches = cnt;
  if (flops) *flops = f;
  if (bytes) *bytes = b;
  return GBS_SUCCESS;
}
