// Batched factor + solve of many small, uneven systems (LLT for SPD, LU with
// partial pivoting for general matrices), one right-hand side each.
//
// The reference has no batch API: its CPU path is one LLT / PartialPivLU per
// matrix (LLT.h:305-328 for n < 32; PartialPivLU.h:365-496).  Here one
// persistent launch per size bucket serves the whole batch:
//   * the work list is sorted by cost (largest first) at plan time;
//   * every warp takes the next matrix with one atomicAdd (no waits);
//   * the matrix lives in the warp's own shared-memory slice, lanes own rows;
//   * LLT follows the reference's left-looking column order (x = a_kk -
//     ||l_k||^2, fail if x <= 0, column below scaled by 1/x after the dot
//     products), so info() and the failing column match;
//   * LU pivots on the first maximum of |a_ik| (warp-shuffle argmax), swaps
//     whole rows, scales, rank-1 updates -- the reference's pivot sequence;
//   * the solve (P, L, U or L, L^T) runs in the same warp, lane = row.
// The two buckets (n <= 32, one row per lane; n <= 64, two rows per lane) run
// as two kernel nodes of one CUDA graph; threads per CTA per bucket come from
// the autotuner (batched_autotune), cached per (bucket, dtype, GPU).
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

#include "dense_driver.cuh"
#include "gbs_common.cuh"
#include "gbs_profile.cuh"

namespace gbs {
namespace {

struct Item {
  int64_t a_off;   // element offset of the matrix (column-major n x n, ld = n)
  int64_t b_off;   // element offset of its right-hand side (n)
  int n;
  int kind;        // 0 = LLT, 1 = LU
  int id;          // position in the caller's batch
  int pad;
};

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
__global__ void batched_kernel(const Item* __restrict__ items, int count, T* __restrict__ A, T* __restrict__ Bv,
                               int* __restrict__ info, int* __restrict__ piv, int* __restrict__ counter)
{
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
    for (int e = lane; e < n * n; e += 32) S[(e / n) * LD + (e % n)] = a[e];   // S[col*LD + row]
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
#pragma unroll
        for (int q = 0; q < RPL; ++q) {
          const int i = lane + 32 * q;
          if (i > k && i < n) {
            T s = T(0);
            for (int j = 0; j < k; ++j) s = fma(S[j * LD + i], S[j * LD + k], s);
            S[k * LD + i] = (S[k * LD + i] - s) / x;
          }
        }
        __syncwarp();
        if (lane == 0) S[k * LD + k] = x;
        __syncwarp();
      }
      if (status < 0) {
        // L y = b, then L^T x = y (lane = row)
        for (int k = 0; k < n; ++k) {
          T yk = __shfl_sync(0xffffffffu, pick(b, k), k % 32);
          yk = yk / S[k * LD + k];
#pragma unroll
          for (int q = 0; q < RPL; ++q) {
            const int i = lane + 32 * q;
            if (i > k && i < n) b[q] = fma(-S[k * LD + i], yk, b[q]);
            if (i == k) b[q] = yk;
          }
        }
        for (int k = n - 1; k >= 0; --k) {
          T xk = __shfl_sync(0xffffffffu, pick(b, k), k % 32);
          xk = xk / S[k * LD + k];
#pragma unroll
          for (int q = 0; q < RPL; ++q) {
            const int i = lane + 32 * q;
            if (i < k) b[q] = fma(-S[i * LD + k], xk, b[q]);
            if (i == k) b[q] = xk;
          }
        }
      }
      // write back the lower triangle (the strict upper part is the caller's)
      for (int e = lane; e < n * n; e += 32) {
        const int r = e % n, c = e / n;
        if (r >= c) a[e] = S[c * LD + r];
      }
    } else {
      // ---------------- LU with partial pivoting (PartialPivLU.h:365-409)
      int* pv = piv + it.b_off;
      int nbt = 0;
      for (int k = 0; k < n; ++k) {
        T bs = T(-2);
        int bi = 0x7fffffff;
#pragma unroll
        for (int q = 0; q < RPL; ++q) {
          const int i = lane + 32 * q;
          if (i >= k && i < n) {
            const T x = S[k * LD + i];
            const T s = (i == k) ? ((x != x) ? T(INFINITY) : gbs_abs(x)) : pivot_score(x);
            if (better(s, i, bs, bi)) { bs = s; bi = i; }
          }
        }
        warp_argmax(bs, bi);
        const int p = bi;
        const T pivv = S[k * LD + p];
        const bool nz = pivv != T(0);
        __syncwarp();                    // every lane has read the pivot before rows move
        if (lane == 0) pv[k] = p;
        if (nz) {
          if (p != k) {
            for (int c = lane; c < n; c += 32) {
              const T t = S[c * LD + k]; S[c * LD + k] = S[c * LD + p]; S[c * LD + p] = t;
            }
            ++nbt;
            // the right-hand side row follows (P b, PartialPivLU.h:233)
            const T bk = __shfl_sync(0xffffffffu, pick(b, k), k % 32);
            const T bp = __shfl_sync(0xffffffffu, pick(b, p), p % 32);
#pragma unroll
            for (int q = 0; q < RPL; ++q) {
              const int i = lane + 32 * q;
              if (i == k) b[q] = bp;
              if (i == p) b[q] = bk;
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
#pragma unroll
        for (int q = 0; q < RPL; ++q) {
          const int i = lane + 32 * q;
          if (i > k && i < n) {
            const T l = S[k * LD + i];
            for (int j = k + 1; j < n; ++j) S[j * LD + i] = fma(-l, S[j * LD + k], S[j * LD + i]);
          }
        }
        __syncwarp();
      }
      (void)nbt;
      // L y = P b (unit), U x = y
      for (int k = 0; k < n; ++k) {
        const T yk = __shfl_sync(0xffffffffu, pick(b, k), k % 32);
#pragma unroll
        for (int q = 0; q < RPL; ++q) {
          const int i = lane + 32 * q;
          if (i > k && i < n) b[q] = fma(-S[k * LD + i], yk, b[q]);
        }
      }
      for (int k = n - 1; k >= 0; --k) {
        T xk = __shfl_sync(0xffffffffu, pick(b, k), k % 32);
        xk = xk / S[k * LD + k];
#pragma unroll
        for (int q = 0; q < RPL; ++q) {
          const int i = lane + 32 * q;
          if (i < k) b[q] = fma(-S[k * LD + i], xk, b[q]);
          if (i == k) b[q] = xk;
        }
      }
      for (int e = lane; e < n * n; e += 32) a[e] = S[(e / n) * LD + (e % n)];
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

// ------------------------------------------------------------------ autotuner
// Candidate CTA shapes (warps per CTA); the best per (bucket, dtype, GPU) is
// cached in a small JSON-lines file.
const int kWarpChoices[] = {1, 2, 4, 8};

std::mutex g_tune_mu;
std::map<std::string, int> g_tune;   // key -> warps per CTA
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
    auto k0 = line.find("\"key\": \""), w0 = line.find("\"warps\": ");
    if (k0 == std::string::npos || w0 == std::string::npos) continue;
    k0 += 8;
    auto k1 = line.find('"', k0);
    g_tune[line.substr(k0, k1 - k0)] = atoi(line.c_str() + w0 + 9);
  }
}

void store_cache(const std::string& key, int warps, double us)
{
  g_tune[key] = warps;
  std::ofstream f(cache_path(), std::ios::app);
  if (f) f << "{\"key\": \"" << key << "\", \"warps\": " << warps << ", \"us\": " << us << "}\n";
}

std::string tune_key(int bucket, int dtype)
{
  cudaDeviceProp p;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaGetDeviceProperties(&p, dev);
  std::ostringstream s;
  s << p.name << "|sm" << p.major << p.minor << "|n<=" << bucket << "|" << (dtype == GBS_F64 ? "f64" : "f32");
  return s.str();
}

}  // namespace
}  // namespace gbs

using namespace gbs;

struct gbs_batched {
  int dtype = GBS_F64;
  int64_t count = 0;
  int64_t total_a = 0, total_b = 0;
  std::vector<int> sizes, kinds;
  std::vector<int64_t> a_off, b_off;
  int nb[2] = {0, 0};            // items per bucket
  int warps[2] = {4, 4};         // warps per CTA per bucket
  int grid[2] = {0, 0};
  DevBuf items, counters;
  cudaStream_t stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  void* g_a = nullptr;           // buffers the graph was captured with
  void* g_b = nullptr;
  void* g_info = nullptr;
  void* g_piv = nullptr;
  int use_graph = 1;
};

// grid for a bucket: co-resident CTAs of this shape (sets the smem limit
// first); called outside any stream capture.
template <typename T, int MAXN>
static int bucket_grid(int count, int warps, int* grid)
{
  *grid = 0;
  if (count <= 0) return GBS_SUCCESS;
  const size_t smem = smem_per_warp<T, MAXN>() * warps;
  GBS_CUDA_TRY(cudaFuncSetAttribute(batched_kernel<T, MAXN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  GBS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batched_kernel<T, MAXN>, 32 * warps, smem));
  per_sm = std::max(per_sm, 1);
  *grid = std::min<int>(per_sm * device_sm_count(), (count + warps - 1) / warps);
  return GBS_SUCCESS;
}

template <typename T, int MAXN>
static int launch_bucket(cudaStream_t s, const Item* items, int count, int warps, int grid, T* A, T* B, int* info,
                         int* piv, int* counter)
{
  if (count <= 0) return GBS_SUCCESS;
  const size_t smem = smem_per_warp<T, MAXN>() * warps;
  count_launch();
  batched_kernel<T, MAXN><<<grid, 32 * warps, smem, s>>>(items, count, A, B, info, piv, counter);
  GBS_CUDA_TRY(cudaGetLastError());
  return GBS_SUCCESS;
}

static int prepare(gbs_batched* p)
{
  if (p->dtype == GBS_F64) {
    GBS_TRY((bucket_grid<double, 32>(p->nb[0], p->warps[0], &p->grid[0])));
    GBS_TRY((bucket_grid<double, 64>(p->nb[1], p->warps[1], &p->grid[1])));
  } else {
    GBS_TRY((bucket_grid<float, 32>(p->nb[0], p->warps[0], &p->grid[0])));
    GBS_TRY((bucket_grid<float, 64>(p->nb[1], p->warps[1], &p->grid[1])));
  }
  return GBS_SUCCESS;
}

static int enqueue(gbs_batched* p, cudaStream_t s, void* d_a, void* d_b, int* d_info, int* d_piv)
{
  GBS_CUDA_TRY(cudaMemsetAsync(p->counters.p, 0, 2 * sizeof(int), s));
  const Item* it = p->items.as<Item>();
  int* ctr = p->counters.as<int>();
  PhaseScope ps(s, PH_BATCHED, 0.0, 0.0);
  if (p->dtype == GBS_F64) {
    GBS_TRY((launch_bucket<double, 32>(s, it, p->nb[0], p->warps[0], p->grid[0], (double*)d_a, (double*)d_b, d_info, d_piv, ctr)));
    GBS_TRY((launch_bucket<double, 64>(s, it + p->nb[0], p->nb[1], p->warps[1], p->grid[1], (double*)d_a, (double*)d_b, d_info,
                                      d_piv, ctr + 1)));
  } else {
    GBS_TRY((launch_bucket<float, 32>(s, it, p->nb[0], p->warps[0], p->grid[0], (float*)d_a, (float*)d_b, d_info, d_piv, ctr)));
    GBS_TRY((launch_bucket<float, 64>(s, it + p->nb[0], p->nb[1], p->warps[1], p->grid[1], (float*)d_a, (float*)d_b, d_info,
                                     d_piv, ctr + 1)));
  }
  return GBS_SUCCESS;
}

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
  // work list: bucket by size, each bucket sorted by cost (largest first)
  std::vector<Item> items((size_t)count);
  std::vector<int64_t> order((size_t)count);
  std::iota(order.begin(), order.end(), 0);
  auto cost = [&](int64_t i) { return (double)sizes[i] * sizes[i] * sizes[i] * (kinds[i] ? 2.0 : 1.0); };
  std::stable_sort(order.begin(), order.end(), [&](int64_t x, int64_t y) {
    const int bx = sizes[x] > 32, by = sizes[y] > 32;
    if (bx != by) return bx < by;
    return cost(x) > cost(y);
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
    p->nb[sizes[i] > 32]++;
  }
  int rc;
  if ((rc = p->items.reserve(sizeof(Item) * (size_t)std::max<int64_t>(count, 1))) != GBS_SUCCESS ||
      (rc = p->counters.reserve(2 * sizeof(int))) != GBS_SUCCESS) {
    delete p;
    return rc;
  }
  if (cudaStreamCreateWithFlags(&p->stream, cudaStreamDefault) != cudaSuccess) {
    delete p;
    return GBS_CUDA_ERROR;
  }
  if (count > 0 && cudaMemcpy(p->items.p, items.data(), sizeof(Item) * count, cudaMemcpyHostToDevice) != cudaSuccess) {
    delete p;
    return GBS_CUDA_ERROR;
  }
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    load_cache();
    for (int b = 0; b < 2; ++b) {
      auto f = g_tune.find(tune_key(b ? 64 : 32, dtype));
      if (f != g_tune.end()) p->warps[b] = f->second;
    }
  }
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
  if (p->stream) cudaStreamSynchronize(p->stream);
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
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
  if (p->exec && (p->g_a != d_a || p->g_b != d_b || p->g_info != d_info || p->g_piv != d_piv)) {
    cudaGraphExecDestroy(p->exec);
    cudaGraphDestroy(p->graph);
    p->exec = nullptr;
    p->graph = nullptr;
  }
  if (!p->exec) {
    // capture on the plan's own stream (counter reset + both bucket kernels)
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

// Times each candidate CTA shape per bucket on the caller's batch (the data
// are re-factored, so pass scratch copies) and keeps the fastest.
extern "C" int gbs_batched_autotune(gbs_batched* p, void* d_a, void* d_b, int* d_info, int* d_piv, int persist)
{
  if (!p || p->count == 0) return GBS_INVALID_ARGUMENT;
  cudaStream_t s = p->stream;
  cudaEvent_t e0, e1;
  GBS_CUDA_TRY(cudaEventCreate(&e0));
  GBS_CUDA_TRY(cudaEventCreate(&e1));
  int chosen[2] = {p->warps[0], p->warps[1]};
  for (int b = 0; b < 2; ++b) {
    if (p->nb[b] == 0) continue;
    double best = 1e30;
    int best_w = chosen[b];
    for (int w : kWarpChoices) {
      p->warps[0] = b == 0 ? w : chosen[0];
      p->warps[1] = b == 1 ? w : chosen[1];
      const size_t smem = (b == 0 ? (p->dtype == GBS_F64 ? smem_per_warp<double, 32>() : smem_per_warp<float, 32>())
                                  : (p->dtype == GBS_F64 ? smem_per_warp<double, 64>() : smem_per_warp<float, 64>())) *
                          w;
      if (smem > 200 * 1024) continue;
      GBS_TRY(prepare(p));
      float ms = 0, tot = 0;
      for (int rep = 0; rep < 3; ++rep) {
        GBS_CUDA_TRY(cudaEventRecord(e0, s));
        GBS_TRY(enqueue(p, s, d_a, d_b, d_info, d_piv));
        GBS_CUDA_TRY(cudaEventRecord(e1, s));
        GBS_CUDA_TRY(cudaEventSynchronize(e1));
        GBS_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
        if (rep) tot += ms;
      }
      if (tot < best) { best = tot; best_w = w; }
    }
    chosen[b] = best_w;
    if (persist) {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      store_cache(tune_key(b ? 64 : 32, p->dtype), best_w, best * 500.0);
    }
  }
  p->warps[0] = chosen[0];
  p->warps[1] = chosen[1];
  GBS_TRY(prepare(p));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (p->exec) {
    cudaGraphExecDestroy(p->exec);
    cudaGraphDestroy(p->graph);
    p->exec = nullptr;
    p->graph = nullptr;
  }
  return GBS_SUCCESS;
}

extern "C" int gbs_batched_config(const gbs_batched* p, int* warps_small, int* warps_large)
{
  if (!p) return GBS_INVALID_ARGUMENT;
  if (warps_small) *warps_small = p->warps[0];
  if (warps_large) *warps_large = p->warps[1];
  return GBS_SUCCESS;
}
