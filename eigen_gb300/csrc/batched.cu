// Batched factor + solve of many small, uneven systems (LLT for SPD, LU with
// partial pivoting for general matrices), one right-hand side each.
//
// The reference has no batch API: its CPU path is one LLT / PartialPivLU per
// matrix (LLT.h:305-328 for n < 32; PartialPivLU.h:365-496).  Here the plan
// groups the items by (kind, size class), sorts each group by cost (largest
// first) and gives every group one persistent launch; the launches are forked
// onto side streams (one CUDA graph per call) so that their tails overlap.
// Inside a launch, warps take the next items with one atomicAdd (no waits).
// Each group runs one of two kernel families:
//   * one warp per system (batched_kernel below): the matrix in the warp's
//     shared-memory slice, lanes own rows (one or two per lane);
//   * G lanes per system, G in {1, 2, 4, 8, 16} (batched_lane.cuh): 32 / G
//     systems per warp, which keeps the FP64 units busy on small n.
// Both follow the reference's arithmetic: LLT left-looking (x = a_kk -
// ||l_k||^2, fail if x <= 0 with the failing column untouched), LU with the
// first maximum of |a_ik| as pivot, whole-row interchanges, division by the
// pivot, rank-1 updates -- the same pivots and failing columns.  The variant
// per group comes from the autotuner (gbs_batched_autotune), cached per
// (GPU, kind, size class, dtype).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <numeric>
#include <sstream>
#include <string>
#include <vector>

#include "batched_lane.cuh"
#include "dense_driver.cuh"
#include "gbs_common.cuh"
#include "gbs_profile.cuh"

namespace gbs {
namespace {

using Item = BatchItem;

// b[k / 32] without a dynamic register index (which would go to local memory)
template <typename T, int RPL>
__device__ __forceinline__ T pick(const T (&b)[RPL], int k)
{
  T v = b[0];
#pragma unroll
  for (int q = 1; q < RPL; ++q)
    if (k >= 32 * q) v = b[q];
  return v;
}

// MAXN: bucket bound (32 or 64); RPL: rows per lane = MAXN / 32.
template <typename T, int MAXN>
__global__ void batched_kernel(const Item* __restrict__ items, int count, int maxn, T* __restrict__ A,
                               T* __restrict__ Bv, int* __restrict__ info, int* __restrict__ piv, int* __restrict__ counter)
{
  (void)maxn;
  constexpr int RPL = MAXN / 32;
  constexpr int LD = MAXN + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T* S = (T*)smem_raw + (size_t)warp * MAXN * LD;
  for (;;) {
    int idx = 0;
    if (lane == 0) idx = atomicAdd(counter, 1);
    idx = __shfl_sync(0xffffffffu, idx, 0);
    if (idx >= count) break;
    const Item it = items[idx];
    const int n = it.n;
    T* a = A + it.a_off;
    T* bv = Bv + it.b_off;
    for (int c = 0; c < n; ++c)                                   // S[col*LD + row], coalesced per column
      for (int r = lane; r < n; r += 32) S[c * LD + r] = a[c * n + r];
    T b[RPL];
#pragma unroll
    for (int q = 0; q < RPL; ++q) {
      const int r = lane + 32 * q;
      b[q] = r < n ? bv[r] : T(0);
    }
    __syncwarp();
    int status = -1;
    if (it.kind == 0) {
      // ---------------- LLT, left-looking (LLT.h:305-328)
      for (int k = 0; k < n; ++k) {
        T p = T(0);
        for (int j = lane; j < k; j += 32) { const T l = S[j * LD + k]; p = fma(l, l, p); }
        p = warp_sum(p);
        T x = S[k * LD + k] - p;
        if (x <= T(0)) { status = k; break; }
        x = sqrt(x);
        const T rx = T(1) / x;           // one reciprocal per column: an FP64 division costs ~10 FMAs
#pragma unroll
        for (int q = 0; q < RPL; ++q) {
          const int i = lane + 32 * q;
          if (i > k && i < n) {
            T s = T(0);
            for (int j = 0; j < k; ++j) s = fma(S[j * LD + i], S[j * LD + k], s);
            S[k * LD + i] = (S[k * LD + i] - s) * rx;
          }
        }
        __syncwarp();
        if (lane == 0) S[k * LD + k] = x;
        __syncwarp();
      }
      if (status < 0) {
        // L y = b, then L^T x = y (lane = row); reciprocals of the diagonal per row, in parallel
        T rd[RPL];
#pragma unroll
        for (int q = 0; q < RPL; ++q) {
          const int i = lane + 32 * q;
          rd[q] = i < n ? T(1) / S[i * LD + i] : T(0);
        }
        for (int k = 0; k < n; ++k) {
          const T yk = __shfl_sync(0xffffffffu, pick(b, k), k % 32) * __shfl_sync(0xffffffffu, pick(rd, k), k % 32);
#pragma unroll
          for (int q = 0; q < RPL; ++q) {
            const int i = lane + 32 * q;
            if (i > k && i < n) b[q] = fma(-S[k * LD + i], yk, b[q]);
            if (i == k) b[q] = yk;
          }
        }
        for (int k = n - 1; k >= 0; --k) {
          const T xk = __shfl_sync(0xffffffffu, pick(b, k), k % 32) * __shfl_sync(0xffffffffu, pick(rd, k), k % 32);
#pragma unroll
          for (int q = 0; q < RPL; ++q) {
            const int i = lane + 32 * q;
            if (i < k) b[q] = fma(-S[i * LD + k], xk, b[q]);
            if (i == k) b[q] = xk;
          }
        }
      }
      // write back the lower triangle (the strict upper part is the caller's)
      for (int c = 0; c < n; ++c)
        for (int r = c + lane; r < n; r += 32) a[c * n + r] = S[c * LD + r];
    } else {
      // ---------------- LU with partial pivoting (PartialPivLU.h:365-409)
      using U = typename PivotKey<T>::U;
      int* pv = piv + it.b_off;
      for (int k = 0; k < n; ++k) {
        U bk = 0;                        // integer pivot keys: no FP64 compares
        int bi = 0x7fffffff;
#pragma unroll
        for (int q = 0; q < RPL; ++q) {
          const int i = lane + 32 * q;
          if (i >= k && i < n) {
            const U key = pivot_key(S[k * LD + i], i == k);
            if (key > bk) { bk = key; bi = i; }
          }
        }
        group_argmax<32>(bk, bi, 0xffffffffu);
        const int p = bi;
        const bool nz = bk != U(2);
        __syncwarp();                    // every lane has finished the previous update
        if (lane == 0) pv[k] = p;
        if (nz) {
          if (p != k) {
            for (int c = lane; c < n; c += 32) {
              const T t = S[c * LD + k]; S[c * LD + k] = S[c * LD + p]; S[c * LD + p] = t;
            }
            // the right-hand side row follows (P b, PartialPivLU.h:233)
            const T bk2 = __shfl_sync(0xffffffffu, pick(b, k), k % 32);
            const T bp = __shfl_sync(0xffffffffu, pick(b, p), p % 32);
#pragma unroll
            for (int q = 0; q < RPL; ++q) {
              const int i = lane + 32 * q;
              if (i == k) b[q] = bp;
              if (i == p) b[q] = bk2;
            }
          }
          __syncwarp();
          const T d = S[k * LD + k];
#pragma unroll
          for (int q = 0; q < RPL; ++q) {
            const int i = lane + 32 * q;
            if (i > k && i < n) S[k * LD + i] = S[k * LD + i] / d;
          }
        } else if (status < 0) {
          status = k;
        }
        __syncwarp();
        // trailing update, four columns at a time (loads of a block before its stores)
        T l[RPL];
        bool act[RPL];
#pragma unroll
        for (int q = 0; q < RPL; ++q) {
          const int i = lane + 32 * q;
          act[q] = i > k && i < n;
          l[q] = act[q] ? S[k * LD + i] : T(0);
        }
        int j = k + 1;
        for (; j + 4 <= n; j += 4) {
          const T u0 = S[j * LD + k], u1 = S[(j + 1) * LD + k], u2 = S[(j + 2) * LD + k], u3 = S[(j + 3) * LD + k];
#pragma unroll
          for (int q = 0; q < RPL; ++q) {
            if (act[q]) {
              T* ar = S + j * LD + lane + 32 * q;
              const T a0 = ar[0], a1 = ar[LD], a2 = ar[2 * LD], a3 = ar[3 * LD];
              ar[0] = fma(-l[q], u0, a0);
              ar[LD] = fma(-l[q], u1, a1);
              ar[2 * LD] = fma(-l[q], u2, a2);
              ar[3 * LD] = fma(-l[q], u3, a3);
            }
          }
        }
        for (; j < n; ++j) {
          const T u = S[j * LD + k];
#pragma unroll
          for (int q = 0; q < RPL; ++q)
            if (act[q]) S[j * LD + lane + 32 * q] = fma(-l[q], u, S[j * LD + lane + 32 * q]);
        }
      }
      __syncwarp();
      // L y = P b (unit), U x = y; the reciprocals of U's diagonal per row, in parallel
      T rd[RPL];
#pragma unroll
      for (int q = 0; q < RPL; ++q) {
        const int i = lane + 32 * q;
        rd[q] = i < n ? T(1) / S[i * LD + i] : T(0);
      }
      for (int k = 0; k < n; ++k) {
        const T yk = __shfl_sync(0xffffffffu, pick(b, k), k % 32);
#pragma unroll
        for (int q = 0; q < RPL; ++q) {
          const int i = lane + 32 * q;
          if (i > k && i < n) b[q] = fma(-S[k * LD + i], yk, b[q]);
        }
      }
      for (int k = n - 1; k >= 0; --k) {
        const T xk = __shfl_sync(0xffffffffu, pick(b, k), k % 32) * __shfl_sync(0xffffffffu, pick(rd, k), k % 32);
#pragma unroll
        for (int q = 0; q < RPL; ++q) {
          const int i = lane + 32 * q;
          if (i < k) b[q] = fma(-S[k * LD + i], xk, b[q]);
          if (i == k) b[q] = xk;
        }
      }
      for (int c = 0; c < n; ++c)
        for (int r = lane; r < n; r += 32) a[c * n + r] = S[c * LD + r];
    }
#pragma unroll
    for (int q = 0; q < RPL; ++q) {
      const int r = lane + 32 * q;
      if (r < n && (it.kind == 1 || status < 0)) bv[r] = b[q];
    }
    if (lane == 0) info[it.id] = status;
    __syncwarp();
  }
}

template <typename T, int MAXN>
size_t smem_per_warp() { return sizeof(T) * MAXN * (MAXN + 1); }

// ------------------------------------------------------------------ variants
// A size bucket runs one of: one warp per system (batched_kernel, lanes = 32,
// warps per CTA from kWarpChoices) or G lanes per system (lu_group_kernel,
// llt_lane_kernel; one warp per CTA).
const int kWarpChoices[] = {1, 2, 4, 8};

template <typename T>
const void* kernel_for(int kind, int lanes, int maxn)
{
  if (lanes == 32) return maxn <= 32 ? (const void*)batched_kernel<T, 32> : (const void*)batched_kernel<T, 64>;
  if (kind == 0) return lanes == 1 ? (const void*)llt_lane_kernel<T> : nullptr;
  switch (lanes) {
    case 1: return (const void*)lu_group_kernel<T, 1>;
    case 2: return (const void*)lu_group_kernel<T, 2>;
    case 4: return (const void*)lu_group_kernel<T, 4>;
    case 8: return (const void*)lu_group_kernel<T, 8>;
    case 16: return (const void*)lu_group_kernel<T, 16>;
  }
  return nullptr;
}

template <typename T>
size_t smem_for(int kind, int lanes, int maxn, int warps)
{
  if (lanes == 32) return (maxn <= 32 ? smem_per_warp<T, 32>() : smem_per_warp<T, 64>()) * warps;
  return kind == 0 ? llt_lane_smem<T>(maxn) : lu_group_smem<T>(maxn, lanes);
}

// size classes (upper bounds) and the variants tried for each
const int kLltClasses[] = {8, 12, 16, 20, 24, 32, 64};
const int kLuClasses[] = {8, 12, 16, 24, 32, 48, 64};

std::vector<int> lane_choices(int kind, int hi)
{
  if (kind == 0) return hi <= 32 ? std::vector<int>{1, 32} : std::vector<int>{32};
  if (hi <= 16) return {1, 2, 32};
  if (hi <= 32) return {2, 4, 8, 32};
  return {8, 16, 32};
}

// defaults (before autotuning) from per-bucket timings on GB300: one lane
// per system for LLT up to n = 32, one warp per system for LU except
// n = 33..48, where 16 lanes per system win
int default_lanes(int kind, int hi)
{
  if (kind == 0) return hi <= 32 ? 1 : 32;
  return hi == 48 ? 16 : 32;
}

// ------------------------------------------------------------------ autotuner
// The best (lanes per system, warps per CTA) per (GPU, kind, size class,
// dtype) is cached in a small JSON-lines file.
struct TuneEntry {
  int lanes, warps;
};
std::mutex g_tune_mu;
std::map<std::string, TuneEntry> g_tune;
bool g_tune_loaded = false;

std::string cache_path()
{
  const char* p = getenv("GBS_AUTOTUNE_CACHE");
  if (p && *p) return p;
  const char* h = getenv("HOME");
  return std::string(h && *h ? h : "/tmp") + "/.gb300solve_autotune.jsonl";
}

void load_cache()
{
  if (g_tune_loaded) return;
  g_tune_loaded = true;
  std::ifstream f(cache_path());
  std::string line;
  while (std::getline(f, line)) {
    auto k0 = line.find("\"key\": \""), w0 = line.find("\"warps\": "), l0 = line.find("\"lanes\": ");
    if (k0 == std::string::npos || w0 == std::string::npos || l0 == std::string::npos) continue;
    k0 += 8;
    auto k1 = line.find('"', k0);
    g_tune[line.substr(k0, k1 - k0)] = {atoi(line.c_str() + l0 + 9), atoi(line.c_str() + w0 + 9)};
  }
}

void store_cache(const std::string& key, TuneEntry e, double us)
{
  g_tune[key] = e;
  std::ofstream f(cache_path(), std::ios::app);
  if (f) f << "{\"key\": \"" << key << "\", \"lanes\": " << e.lanes << ", \"warps\": " << e.warps << ", \"us\": " << us << "}\n";
}

std::string tune_key(int kind, int hi, int dtype)
{
  cudaDeviceProp p;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaGetDeviceProperties(&p, dev);
  std::ostringstream s;
  s << p.name << "|sm" << p.major << p.minor << "|" << (kind ? "lu" : "llt") << "|n<=" << hi << "|"
    << (dtype == GBS_F64 ? "f64" : "f32");
  return s.str();
}

constexpr int kSideStreams = 4;

}  // namespace
}  // namespace gbs

using namespace gbs;

struct BucketPlan {
  int kind, lo, hi;      // item kind and size class lo..hi
  int first, count;      // its range of the sorted work list
  int maxn;              // largest n present
  int lanes;             // lanes per system (32: one warp per system)
  int warps;             // warps per CTA
  int grid;
  double cost;           // sum of n^3 (LU counted twice), for the launch order
};

struct gbs_batched {
  int dtype = GBS_F64;
  int64_t count = 0;
  int64_t total_a = 0, total_b = 0;
  std::vector<int> sizes, kinds;
  std::vector<int64_t> a_off, b_off;
  std::vector<BucketPlan> buckets;
  DevBuf items, counters;
  cudaStream_t stream = nullptr;
  cudaStream_t side[kSideStreams] = {};
  cudaEvent_t ev_fork = nullptr;
  std::vector<cudaEvent_t> ev_join;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  void* g_a = nullptr;           // buffers the graph was captured with
  void* g_b = nullptr;
  void* g_info = nullptr;
  void* g_piv = nullptr;
  int use_graph = 1;
  // gbs_batched_solve_host: parts of consecutive items, each with a plan of
  // its own, the batch's device copy, and the streams that move it
  std::vector<gbs_batched*> parts;
  std::vector<int64_t> part_first;     // part q holds the items [part_first[q], part_first[q + 1])
  DevBuf da, db, dinfo, dpiv;
  cudaStream_t hin = nullptr, hrun = nullptr, hout = nullptr;
  std::vector<cudaEvent_t> ev_in, ev_run;
};

static void drop_graph(gbs_batched* p)
{
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  p->exec = nullptr;
  p->graph = nullptr;
}

// grid of a bucket: co-resident CTAs of its variant (raises the kernel's
// shared-memory limit first); called outside any stream capture.
template <typename T>
static int bucket_grid(BucketPlan& b)
{
  b.grid = 0;
  if (b.count <= 0) return GBS_SUCCESS;
  const void* fn = kernel_for<T>(b.kind, b.lanes, b.maxn);
  if (!fn) return GBS_INVALID_ARGUMENT;
  const size_t smem = smem_for<T>(b.kind, b.lanes, b.maxn, b.warps);
  int optin = 0, dev = 0;
  GBS_CUDA_TRY(cudaGetDevice(&dev));
  GBS_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  if (smem > (size_t)optin) return GBS_INVALID_ARGUMENT;
  // the limit, not this bucket's size: several buckets may share the kernel
  GBS_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
  int per_sm = 0;
  GBS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 32 * b.warps, smem));
  per_sm = std::max(per_sm, 1);
  const int per_cta = b.lanes == 32 ? b.warps : 32 / b.lanes;    // systems a CTA takes at once
  b.grid = std::min<int>(per_sm * device_sm_count(), (b.count + per_cta - 1) / per_cta);
  return GBS_SUCCESS;
}

static int prepare(gbs_batched* p)
{
  for (BucketPlan& b : p->buckets) GBS_TRY(p->dtype == GBS_F64 ? bucket_grid<double>(b) : bucket_grid<float>(b));
  return GBS_SUCCESS;
}

template <typename T>
static int launch_bucket(const BucketPlan& b, cudaStream_t s, const Item* items, void* A, void* B, int* info,
                         int* piv, int* counter)
{
  if (b.count <= 0) return GBS_SUCCESS;
  const Item* it = items + b.first;
  int count = b.count, maxn = b.maxn;
  T* a = (T*)A;
  T* bb = (T*)B;
  void* args[] = {(void*)&it, (void*)&count, (void*)&maxn, (void*)&a, (void*)&bb, (void*)&info, (void*)&piv, (void*)&counter};
  count_launch();
  GBS_CUDA_TRY(cudaLaunchKernel(kernel_for<T>(b.kind, b.lanes, b.maxn), dim3(b.grid), dim3(32 * b.warps), args,
                                smem_for<T>(b.kind, b.lanes, b.maxn, b.warps), s));
  return GBS_SUCCESS;
}

// only >= 0: that bucket alone (autotuning); else every bucket, forked onto
// side streams so that the buckets' tails overlap, joined back into s.
static int enqueue(gbs_batched* p, cudaStream_t s, void* d_a, void* d_b, int* d_info, int* d_piv, int only = -1)
{
  const int nb = (int)p->buckets.size();
  GBS_CUDA_TRY(cudaMemsetAsync(p->counters.p, 0, sizeof(int) * std::max(nb, 1), s));
  const Item* it = p->items.as<Item>();
  int* ctr = p->counters.as<int>();
  PhaseScope ps(s, PH_BATCHED, 0.0, 0.0);
  auto launch = [&](int b, cudaStream_t st) {
    return p->dtype == GBS_F64 ? launch_bucket<double>(p->buckets[b], st, it, d_a, d_b, d_info, d_piv, ctr + b)
                               : launch_bucket<float>(p->buckets[b], st, it, d_a, d_b, d_info, d_piv, ctr + b);
  };
  if (only >= 0) return launch(only, s);
  if (nb == 1) return launch(0, s);
  GBS_CUDA_TRY(cudaEventRecord(p->ev_fork, s));
  for (int b = 0; b < nb; ++b) {
    cudaStream_t st = p->side[b % kSideStreams];
    if (b < kSideStreams) GBS_CUDA_TRY(cudaStreamWaitEvent(st, p->ev_fork, 0));
    GBS_TRY(launch(b, st));
  }
  for (int k = 0; k < std::min(nb, kSideStreams); ++k) {
    GBS_CUDA_TRY(cudaEventRecord(p->ev_join[k], p->side[k]));
    GBS_CUDA_TRY(cudaStreamWaitEvent(s, p->ev_join[k], 0));
  }
  return GBS_SUCCESS;
}

extern "C" int gbs_batched_destroy(gbs_batched* p);

extern "C" int gbs_batched_create(gbs_batched** out, int dtype, int64_t count, const int* sizes, const int* kinds,
                                  int use_graph)
{
  if (!out || count < 0 || (count > 0 && (!sizes || !kinds)) || (dtype != GBS_F64 && dtype != GBS_F32))
    return GBS_INVALID_ARGUMENT;
  *out = nullptr;
  GBS_TRY(ensure_device());
  gbs_batched* p = new gbs_batched();
  p->dtype = dtype;
  p->count = count;
  p->use_graph = use_graph;
  p->sizes.assign(sizes, sizes + count);
  p->kinds.assign(kinds, kinds + count);
  p->a_off.resize((size_t)count);
  p->b_off.resize((size_t)count);
  int64_t ao = 0, bo = 0;
  for (int64_t i = 0; i < count; ++i) {
    const int n = sizes[i];
    if (n < 1 || n > 64 || (kinds[i] != 0 && kinds[i] != 1)) {
      delete p;
      gbs_set_last_message("gbs_batched_create: sizes must be in [1, 64] and kinds 0 (LLT) or 1 (LU)");
      return GBS_INVALID_ARGUMENT;
    }
    p->a_off[(size_t)i] = ao;
    p->b_off[(size_t)i] = bo;
    ao += (int64_t)n * n;
    bo += n;
  }
  p->total_a = ao;
  p->total_b = bo;
  // size class of an item: index into kLltClasses / kLuClasses
  auto cls = [&](int64_t i) {
    const int* c = kinds[i] ? kLuClasses : kLltClasses;
    int k = 0;
    while (sizes[i] > c[k]) ++k;
    return k;
  };
  // work list: grouped by (kind, size class), each group sorted by cost
  // (largest first); warps take consecutive items, so a warp's systems have
  // nearly equal sizes
  std::vector<Item> items((size_t)count);
  std::vector<int64_t> order((size_t)count);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int64_t x, int64_t y) {
    const int gx = kinds[x] * 16 + cls(x), gy = kinds[y] * 16 + cls(y);
    if (gx != gy) return gx < gy;
    return sizes[x] > sizes[y];
  });
  for (int64_t k = 0; k < count; ++k) {
    const int64_t i = order[(size_t)k];
    Item& it = items[(size_t)k];
    it.a_off = p->a_off[(size_t)i];
    it.b_off = p->b_off[(size_t)i];
    it.n = sizes[i];
    it.kind = kinds[i];
    it.id = (int)i;
    it.pad = 0;
    const int c = cls(i);
    const int* cl = kinds[i] ? kLuClasses : kLltClasses;
    if (p->buckets.empty() || p->buckets.back().kind != kinds[i] || p->buckets.back().hi != cl[c]) {
      BucketPlan b{};
      b.kind = kinds[i];
      b.lo = c ? cl[c - 1] + 1 : 1;
      b.hi = cl[c];
      b.first = (int)k;
      b.maxn = sizes[i];
      b.lanes = default_lanes(b.kind, b.hi);
      b.warps = 1;                       // one-warp CTAs pack best (33 KB each for n <= 64)
      p->buckets.push_back(b);
    }
    BucketPlan& b = p->buckets.back();
    b.count++;
    b.cost += (double)sizes[i] * sizes[i] * sizes[i] * (kinds[i] ? 2.0 : 1.0);
  }
  const int nb = (int)p->buckets.size();
  int rc;
  if ((rc = p->items.reserve(sizeof(Item) * (size_t)std::max<int64_t>(count, 1))) != GBS_SUCCESS ||
      (rc = p->counters.reserve(sizeof(int) * (size_t)std::max(nb, 1))) != GBS_SUCCESS) {
    delete p;
    return rc;
  }
  bool ok = cudaStreamCreateWithFlags(&p->stream, cudaStreamDefault) == cudaSuccess &&
            cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming) == cudaSuccess;
  for (int k = 0; ok && k < kSideStreams; ++k) {
    cudaEvent_t e = nullptr;
    ok = cudaStreamCreateWithFlags(&p->side[k], cudaStreamNonBlocking) == cudaSuccess &&
         cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
    p->ev_join.push_back(e);
  }
  if (!ok || (count > 0 && cudaMemcpy(p->items.p, items.data(), sizeof(Item) * count, cudaMemcpyHostToDevice) != cudaSuccess)) {
    gbs_batched_destroy(p);
    return GBS_CUDA_ERROR;
  }
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    load_cache();
    for (BucketPlan& b : p->buckets) {
      auto f = g_tune.find(tune_key(b.kind, b.hi, dtype));
      if (f == g_tune.end()) continue;
      const std::vector<int> ch = lane_choices(b.kind, b.hi);
      if (std::find(ch.begin(), ch.end(), f->second.lanes) == ch.end()) continue;
      b.lanes = f->second.lanes;
      b.warps = b.lanes == 32 ? f->second.warps : 1;
    }
  }
  // largest total work first: its tail overlaps the smaller buckets
  std::stable_sort(p->buckets.begin(), p->buckets.end(), [](const BucketPlan& x, const BucketPlan& y) { return x.cost > y.cost; });
  if ((rc = prepare(p)) != GBS_SUCCESS) {
    gbs_batched_destroy(p);
    return rc;
  }
  *out = p;
  return GBS_SUCCESS;
}

extern "C" int gbs_batched_destroy(gbs_batched* p)
{
  if (!p) return GBS_SUCCESS;
  for (cudaStream_t hs : {p->hin, p->hrun, p->hout})
    if (hs) cudaStreamSynchronize(hs);
  for (gbs_batched* q : p->parts) gbs_batched_destroy(q);
  for (cudaEvent_t e : p->ev_in)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : p->ev_run)
    if (e) cudaEventDestroy(e);
  for (cudaStream_t hs : {p->hin, p->hrun, p->hout})
    if (hs) cudaStreamDestroy(hs);
  if (p->stream) cudaStreamSynchronize(p->stream);
  for (int k = 0; k < kSideStreams; ++k)
    if (p->side[k]) cudaStreamSynchronize(p->side[k]);
  drop_graph(p);
  for (cudaEvent_t e : p->ev_join)
    if (e) cudaEventDestroy(e);
  if (p->ev_fork) cudaEventDestroy(p->ev_fork);
  for (int k = 0; k < kSideStreams; ++k)
    if (p->side[k]) cudaStreamDestroy(p->side[k]);
  if (p->stream) cudaStreamDestroy(p->stream);
  delete p;
  return GBS_SUCCESS;
}

extern "C" int64_t gbs_batched_matrix_elements(const gbs_batched* p) { return p ? p->total_a : 0; }
extern "C" int64_t gbs_batched_rhs_elements(const gbs_batched* p) { return p ? p->total_b : 0; }

extern "C" int gbs_batched_offsets(const gbs_batched* p, int64_t* a_off, int64_t* b_off)
{
  if (!p) return GBS_INVALID_ARGUMENT;
  if (a_off) std::copy(p->a_off.begin(), p->a_off.end(), a_off);
  if (b_off) std::copy(p->b_off.begin(), p->b_off.end(), b_off);
  return GBS_SUCCESS;
}

extern "C" int gbs_batched_solve(gbs_batched* p, void* d_a, void* d_b, int* d_info, int* d_piv, void* stream)
{
  if (!p || (p->count > 0 && (!d_a || !d_b || !d_info || !d_piv))) return GBS_INVALID_ARGUMENT;
  if (p->count == 0) return GBS_SUCCESS;
  cudaStream_t s = (cudaStream_t)stream;     // NULL: the legacy default stream
  if (!p->use_graph) return enqueue(p, s, d_a, d_b, d_info, d_piv);
  if (p->exec && (p->g_a != d_a || p->g_b != d_b || p->g_info != d_info || p->g_piv != d_piv)) drop_graph(p);
  if (!p->exec) {
    // capture on the plan's own stream (counter reset + the bucket kernels)
    GBS_CUDA_TRY(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue(p, p->stream, d_a, d_b, d_info, d_piv);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(p->stream, &g);
    if (rc != GBS_SUCCESS) { if (g) cudaGraphDestroy(g); return rc; }
    GBS_CUDA_TRY(e);
    GBS_CUDA_TRY(cudaGraphInstantiate(&p->exec, g, 0));
    p->graph = g;
    p->g_a = d_a;
    p->g_b = d_b;
    p->g_info = d_info;
    p->g_piv = d_piv;
  }
  count_launch();
  GBS_CUDA_TRY(cudaGraphLaunch(p->exec, s));
  return GBS_SUCCESS;
}

// Coordinate descent over the buckets' variants (lanes per system, and warps
// per CTA for one warp per system) on the whole concurrent batch: each bucket
// in turn tries every allowed variant and keeps one that lowers the batch's
// time by more than 1 %.  Every timed run starts from the caller's input
// (kept in a scratch copy), and the buffers hold that input again on return.
extern "C" int gbs_batched_autotune(gbs_batched* p, void* d_a, void* d_b, int* d_info, int* d_piv, int persist)
{
  if (!p || p->count == 0 || !d_a || !d_b || !d_info || !d_piv) return GBS_INVALID_ARGUMENT;
  cudaStream_t s = p->stream;
  const size_t esz = p->dtype == GBS_F64 ? 8 : 4;
  const size_t abytes = (size_t)p->total_a * esz, bbytes = (size_t)p->total_b * esz;
  DevBuf a0, b0;
  GBS_TRY(a0.reserve(abytes));
  GBS_TRY(b0.reserve(bbytes));
  GBS_CUDA_TRY(cudaMemcpyAsync(a0.p, d_a, abytes, cudaMemcpyDeviceToDevice, s));
  GBS_CUDA_TRY(cudaMemcpyAsync(b0.p, d_b, bbytes, cudaMemcpyDeviceToDevice, s));
  cudaEvent_t e0, e1;
  GBS_CUDA_TRY(cudaEventCreate(&e0));
  GBS_CUDA_TRY(cudaEventCreate(&e1));
  int rc = GBS_SUCCESS;
  auto restore = [&]() {
    if (rc == GBS_SUCCESS && (cudaMemcpyAsync(d_a, a0.p, abytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
                              cudaMemcpyAsync(d_b, b0.p, bbytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess))
      rc = GBS_CUDA_ERROR;
  };
  // best of `reps` runs of the whole batch, in ms
  auto time_batch = [&](int reps) {
    float best = 1e30f, ms = 0;
    for (int r = 0; r < reps && rc == GBS_SUCCESS; ++r) {
      restore();
      if (rc == GBS_SUCCESS && cudaEventRecord(e0, s) != cudaSuccess) rc = GBS_CUDA_ERROR;
      if (rc == GBS_SUCCESS) rc = enqueue(p, s, d_a, d_b, d_info, d_piv);
      if (rc == GBS_SUCCESS && (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                                cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
        rc = GBS_CUDA_ERROR;
      best = std::min(best, ms);
    }
    return best;
  };
  time_batch(1);                                     // warm-up
  float best = time_batch(3);
  for (int bi = 0; bi < (int)p->buckets.size() && rc == GBS_SUCCESS; ++bi) {
    BucketPlan& b = p->buckets[bi];
    BucketPlan keep = b;
    for (int lanes : lane_choices(b.kind, b.hi)) {
      for (int w : kWarpChoices) {
        if ((lanes != 32 && w != 1) || (lanes == keep.lanes && w == keep.warps)) continue;
        b = keep;
        b.lanes = lanes;
        b.warps = w;
        if ((p->dtype == GBS_F64 ? bucket_grid<double>(b) : bucket_grid<float>(b)) != GBS_SUCCESS) {
          cudaGetLastError();
          continue;                                  // does not fit
        }
        const float t = time_batch(3);
        if (rc == GBS_SUCCESS && t < 0.99f * best) {
          best = t;
          keep = b;
        }
      }
    }
    b = keep;
    if (rc == GBS_SUCCESS && persist) {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      store_cache(tune_key(b.kind, b.hi, p->dtype), {b.lanes, b.warps}, best * 1e3);
    }
  }
  restore();
  if (rc == GBS_SUCCESS && cudaStreamSynchronize(s) != cudaSuccess) rc = GBS_CUDA_ERROR;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  GBS_TRY(rc);
  GBS_TRY(prepare(p));
  drop_graph(p);
  return GBS_SUCCESS;
}

// Warps per CTA of the first bucket with n <= 32 and of the first with n > 32.
extern "C" int gbs_batched_config(const gbs_batched* p, int* warps_small, int* warps_large)
{
  if (!p) return GBS_INVALID_ARGUMENT;
  int ws = 4, wl = 4;
  bool fs = false, fl = false;
  for (const BucketPlan& b : p->buckets) {
    if (b.hi <= 32 && !fs) { ws = b.warps; fs = true; }
    if (b.hi > 32 && !fl) { wl = b.warps; fl = true; }
  }
  if (warps_small) *warps_small = ws;
  if (warps_large) *warps_large = wl;
  return GBS_SUCCESS;
}

// The plan's buckets, 7 ints each: kind, smallest and largest size of the
// class, items, largest size present, lanes per system, warps per CTA.
extern "C" int gbs_batched_buckets(const gbs_batched* p, int capacity, int* count, int* desc)
{
  if (!p || !count || capacity < 0 || (capacity > 0 && !desc)) return GBS_INVALID_ARGUMENT;
  *count = (int)p->buckets.size();
  for (int i = 0; i < std::min(capacity, *count); ++i) {
    const BucketPlan& b = p->buckets[i];
    const int v[7] = {b.kind, b.lo, b.hi, b.count, b.maxn, b.lanes, b.warps};
    std::copy(v, v + 7, desc + 7 * i);
  }
  return GBS_SUCCESS;
}

// Sets the variant of bucket i (as listed by gbs_batched_buckets).
extern "C" int gbs_batched_set_variant(gbs_batched* p, int bucket, int lanes, int warps)
{
  if (!p || bucket < 0 || bucket >= (int)p->buckets.size()) return GBS_INVALID_ARGUMENT;
  BucketPlan& b = p->buckets[bucket];
  const std::vector<int> ch = lane_choices(b.kind, b.hi);
  if (std::find(ch.begin(), ch.end(), lanes) == ch.end()) return GBS_INVALID_ARGUMENT;
  if (lanes == 32 ? std::find(std::begin(kWarpChoices), std::end(kWarpChoices), warps) == std::end(kWarpChoices)
                  : warps != 1)
    return GBS_INVALID_ARGUMENT;
  const BucketPlan keep = b;
  b.lanes = lanes;
  b.warps = warps;
  const int rc = p->dtype == GBS_F64 ? bucket_grid<double>(b) : bucket_grid<float>(b);
  if (rc != GBS_SUCCESS) {
    b = keep;
    return rc;
  }
  drop_graph(p);
  return GBS_SUCCESS;
}

// ------------------------------------------------------------------ host buffers
namespace {
constexpr int kHostParts = 4;                         // parts of a large batch
constexpr int64_t kHostPartMinBytes = 16 << 20;       // smaller batches use fewer parts

// The parts' plans run the variants of the whole plan's buckets, so every item
// is solved by the same kernel as by gbs_batched_solve.
int sync_part_variants(gbs_batched* p)
{
  for (gbs_batched* q : p->parts)
    for (size_t i = 0; i < q->buckets.size(); ++i) {
      const BucketPlan& qb = q->buckets[i];
      for (const BucketPlan& b : p->buckets)
        if (b.kind == qb.kind && b.hi == qb.hi && (b.lanes != qb.lanes || b.warps != qb.warps))
          GBS_TRY(gbs_batched_set_variant(q, (int)i, b.lanes, b.warps));
    }
  return GBS_SUCCESS;
}

void drop_parts(gbs_batched* p)
{
  for (gbs_batched* q : p->parts) gbs_batched_destroy(q);
  for (cudaEvent_t e : p->ev_in)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : p->ev_run)
    if (e) cudaEventDestroy(e);
  for (cudaStream_t* hs : {&p->hin, &p->hrun, &p->hout}) {
    if (*hs) cudaStreamDestroy(*hs);
    *hs = nullptr;
  }
  p->parts.clear();
  p->part_first.clear();
  p->ev_in.clear();
  p->ev_run.clear();
}

int build_parts(gbs_batched* p);

int make_parts(gbs_batched* p)
{
  const int rc = build_parts(p);
  if (rc != GBS_SUCCESS) drop_parts(p);
  return rc;
}

int build_parts(gbs_batched* p)
{
  const size_t es = p->dtype == GBS_F64 ? sizeof(double) : sizeof(float);
  const int64_t bytes = (p->total_a + p->total_b) * (int64_t)es;
  const int nparts = (int)std::max<int64_t>(1, std::min<int64_t>(kHostParts, bytes / kHostPartMinBytes));
  p->part_first.assign(1, 0);
  for (int q = 1; q < nparts; ++q) {            // equal bytes per part, cut at item boundaries
    const int64_t target = (p->total_a + p->total_b) * q / nparts;
    int64_t i = p->part_first.back();
    while (i < p->count && p->a_off[(size_t)i] + p->b_off[(size_t)i] < target) ++i;
    if (i > p->part_first.back() && i < p->count) p->part_first.push_back(i);
  }
  p->part_first.push_back(p->count);
  for (size_t q = 0; q + 1 < p->part_first.size(); ++q) {
    const int64_t i0 = p->part_first[q], i1 = p->part_first[q + 1];
    gbs_batched* part = nullptr;
    GBS_TRY(gbs_batched_create(&part, p->dtype, i1 - i0, p->sizes.data() + i0, p->kinds.data() + i0, p->use_graph));
    p->parts.push_back(part);
    cudaEvent_t ei = nullptr, er = nullptr;
    GBS_CUDA_TRY(cudaEventCreateWithFlags(&ei, cudaEventDisableTiming));
    p->ev_in.push_back(ei);
    GBS_CUDA_TRY(cudaEventCreateWithFlags(&er, cudaEventDisableTiming));
    p->ev_run.push_back(er);
  }
  for (cudaStream_t* hs : {&p->hin, &p->hrun, &p->hout})
    GBS_CUDA_TRY(cudaStreamCreateWithFlags(hs, cudaStreamNonBlocking));
  return GBS_SUCCESS;
}
}  // namespace

extern "C" int gbs_batched_solve_host(gbs_batched* p, const void* a, const void* b, void* x, int* info, int* piv)
{
  if (!p || (p->count > 0 && (!a || !b || !x || !info))) return GBS_INVALID_ARGUMENT;
  if (p->count == 0) return GBS_SUCCESS;
  const size_t es = p->dtype == GBS_F64 ? sizeof(double) : sizeof(float);
  if (p->parts.empty()) GBS_TRY(make_parts(p));
  GBS_TRY(sync_part_variants(p));
  GBS_TRY(p->da.reserve(es * (size_t)p->total_a));
  GBS_TRY(p->db.reserve(es * (size_t)p->total_b));
  GBS_TRY(p->dinfo.reserve(sizeof(int) * (size_t)p->count));
  GBS_TRY(p->dpiv.reserve(sizeof(int) * (size_t)p->total_b));
  char* da = (char*)p->da.p;
  char* db = (char*)p->db.p;
  const char* ha = (const char*)a;
  const char* hb = (const char*)b;
  char* hx = (char*)x;
  int rc = GBS_SUCCESS;
  for (size_t q = 0; q < p->parts.size() && rc == GBS_SUCCESS; ++q) {
    const int64_t i0 = p->part_first[q], i1 = p->part_first[q + 1];
    const int64_t a0 = p->a_off[(size_t)i0], a1 = i1 < p->count ? p->a_off[(size_t)i1] : p->total_a;
    const int64_t b0 = p->b_off[(size_t)i0], b1 = i1 < p->count ? p->b_off[(size_t)i1] : p->total_b;
    // part q crosses in while part q - 1 is solved, and out while part q + 1 is
    cudaError_t e = cudaMemcpyAsync(da + es * a0, ha + es * a0, es * (a1 - a0), cudaMemcpyHostToDevice, p->hin);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(db + es * b0, hb + es * b0, es * (b1 - b0), cudaMemcpyHostToDevice, p->hin);
    if (e == cudaSuccess) e = cudaEventRecord(p->ev_in[q], p->hin);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(p->hrun, p->ev_in[q], 0);
    if (e != cudaSuccess) {
      gbs_set_last_cuda_error(e, "gbs_batched_solve_host", __FILE__, __LINE__);
      rc = GBS_CUDA_ERROR;
      break;
    }
    rc = gbs_batched_solve(p->parts[q], da + es * a0, db + es * b0, p->dinfo.as<int>() + i0, p->dpiv.as<int>() + b0,
                           p->hrun);
    if (rc != GBS_SUCCESS) break;
    e = cudaEventRecord(p->ev_run[q], p->hrun);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(p->hout, p->ev_run[q], 0);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(hx + es * b0, db + es * b0, es * (b1 - b0), cudaMemcpyDeviceToHost, p->hout);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(info + i0, p->dinfo.as<int>() + i0, sizeof(int) * (i1 - i0), cudaMemcpyDeviceToHost,
                          p->hout);
    if (e == cudaSuccess && piv)
      e = cudaMemcpyAsync(piv + b0, p->dpiv.as<int>() + b0, sizeof(int) * (b1 - b0), cudaMemcpyDeviceToHost,
                          p->hout);
    if (e != cudaSuccess) {
      gbs_set_last_cuda_error(e, "gbs_batched_solve_host", __FILE__, __LINE__);
      rc = GBS_CUDA_ERROR;
    }
  }
  // nothing of the three streams outlives the call
  for (cudaStream_t hs : {p->hin, p->hrun, p->hout}) {
    const cudaError_t e = cudaStreamSynchronize(hs);
    if (e != cudaSuccess && rc == GBS_SUCCESS) {
      gbs_set_last_cuda_error(e, "gbs_batched_solve_host", __FILE__, __LINE__);
      rc = GBS_CUDA_ERROR;
    }
  }
  return rc;
}
