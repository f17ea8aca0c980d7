// Host drivers of the plain factor-and-solve path: the blocked LU and LLT
// loops, triangular solves, ||A||_1 and the Hager/Higham rcond estimator,
// all stream-ordered on device buffers.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "dense_driver.cuh"
#include "dense_kernels.cuh"
#include "gbs_profile.cuh"

// ------------------------------------------------------------------ errors
static thread_local std::string g_last_error = "";

void gbs_set_last_cuda_error(cudaError_t e, const char* what, const char* file, int line)
{
  char buf[512];
  snprintf(buf, sizeof(buf), "CUDA error %d (%s) in %s at %s:%d", (int)e, cudaGetErrorString(e), what, file, line);
  g_last_error = buf;
}

void gbs_set_last_message(const char* msg) { g_last_error = msg; }

extern "C" const char* gbs_last_error(void) { return g_last_error.c_str(); }
extern "C" const char* gbs_version(void) { return "gb300solve 0.1 (sm_103a)"; }

namespace gbs {

// ------------------------------------------------------------------ device
static std::once_flag g_dev_once;
static int g_dev_status = GBS_NO_DEVICE;
static int g_sm_count = 0;

static void probe_devices()
{
  int cnt = 0;
  if (cudaGetDeviceCount(&cnt) != cudaSuccess || cnt <= 0) {
    cudaGetLastError();
    gbs_set_last_message("no CUDA device");
    return;
  }
  int usable = 0;
  for (int d = 0; d < cnt; ++d) {
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, d) != cudaSuccess) continue;
    if (p.major == 10 && p.minor == 3) {
      ++usable;
      if (g_sm_count == 0) g_sm_count = p.multiProcessorCount;
    }
  }
  if (usable > 0) g_dev_status = GBS_SUCCESS;
  else gbs_set_last_message("no sm_103 (GB300) device: this library is built for sm_103a only");
}

int ensure_device()
{
  std::call_once(g_dev_once, probe_devices);
  if (g_dev_status != GBS_SUCCESS) gbs_set_last_message("no usable sm_103a device");
  return g_dev_status;
}

int device_sm_count()
{
  ensure_device();
  return g_sm_count > 0 ? g_sm_count : 1;
}

// ------------------------------------------------------------------ buffers
int DevBuf::reserve(size_t b)
{
  if (b <= bytes && p) return GBS_SUCCESS;
  if (borrowed) {
    gbs_set_last_message("workspace request exceeds a fixed (borrowed) device buffer");
    return GBS_INVALID_ARGUMENT;
  }
  release();
  size_t want = std::max<size_t>(b, 256);
  cudaError_t e = cudaMalloc(&p, want);
  if (e != cudaSuccess) {
    cudaGetLastError();
    p = nullptr;
    bytes = 0;
    gbs_set_last_cuda_error(e, "cudaMalloc", __FILE__, __LINE__);
    return e == cudaErrorMemoryAllocation ? GBS_OUT_OF_MEMORY : GBS_CUDA_ERROR;
  }
  bytes = want;
  return GBS_SUCCESS;
}

void DevBuf::release()
{
  if (p && !borrowed) cudaFree(p);
  p = nullptr;
  bytes = 0;
}

int HostBuf::reserve(size_t b)
{
  if (b <= bytes && p) return GBS_SUCCESS;
  release();
  size_t want = std::max<size_t>(b, 256);
  cudaError_t e = cudaMallocHost(&p, want);
  if (e != cudaSuccess) {
    cudaGetLastError();
    p = nullptr;
    bytes = 0;
    gbs_set_last_cuda_error(e, "cudaMallocHost", __FILE__, __LINE__);
    return GBS_OUT_OF_MEMORY;
  }
  bytes = want;
  return GBS_SUCCESS;
}

void HostBuf::release()
{
  if (p) cudaFreeHost(p);
  p = nullptr;
  bytes = 0;
}

static std::mutex g_pool_mu;
static std::vector<Workspace*> g_pool;

WorkspaceLease::WorkspaceLease()
{
  status = ensure_device();
  if (status != GBS_SUCCESS) return;
  {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (!g_pool.empty()) {
      ws = g_pool.back();
      g_pool.pop_back();
    }
  }
  if (!ws) {
    ws = new Workspace();
    cudaError_t e = cudaStreamCreateWithFlags(&ws->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      gbs_set_last_cuda_error(e, "cudaStreamCreate", __FILE__, __LINE__);
      delete ws;
      ws = nullptr;
      status = GBS_CUDA_ERROR;
    }
  }
}

WorkspaceLease::~WorkspaceLease()
{
  if (!ws) return;
  std::lock_guard<std::mutex> lk(g_pool_mu);
  g_pool.push_back(ws);
}

// ------------------------------------------------------------------ status
static std::atomic<uint64_t> g_wait_limit_ns{kSpinDeadlineNs};

uint64_t wait_limit_ns() { return g_wait_limit_ns.load(std::memory_order_relaxed); }

void set_wait_limit_ns(uint64_t ns) { g_wait_limit_ns.store(ns ? ns : kSpinDeadlineNs, std::memory_order_relaxed); }

int reset_status(DeviceStatus* d_st, cudaStream_t s)
{
  DeviceStatus h;
  memset(&h, 0, sizeof(h));
  h.info = -1;
  h.limit_ns = wait_limit_ns();
  // the status word is tiny: a kernel-free 32-byte upload per factorization
  GBS_CUDA_TRY(cudaMemcpyAsync(d_st, &h, sizeof(h), cudaMemcpyHostToDevice, s));
  GBS_CUDA_TRY(cudaStreamSynchronize(s));
  return GBS_SUCCESS;
}

int read_status(const DeviceStatus* d_st, DeviceStatus* h_st, cudaStream_t s)
{
  GBS_CUDA_TRY(cudaMemcpyAsync(h_st, d_st, sizeof(DeviceStatus), cudaMemcpyDeviceToHost, s));
  GBS_CUDA_TRY(cudaStreamSynchronize(s));
  if (h_st->timeout) {
    gbs_set_last_message("an inter-CTA wait timed out; the factorization was abandoned");
    return GBS_TIMEOUT;
  }
  return GBS_SUCCESS;
}

static inline int ceil_div(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

// ------------------------------------------------------------------ GEMM launch
template <typename T>
static int gemm_sub(cudaStream_t s, int phase, int M, int N, int K, const T* A, int64_t a_rs, int64_t a_cs,
                    const T* B, int64_t b_rs, int64_t b_cs, T* C, int64_t ldc, int lower, const int* stop_flag)
{
  if (M <= 0 || N <= 0 || K <= 0) return GBS_SUCCESS;
  constexpr int BM = 64, BN = 64, BK = 16, TM = 4, TN = 4;
  dim3 grid(ceil_div(N, BN), ceil_div(M, BM));
  if (grid.y > 65535) {
    gbs_set_last_message("matrix too tall for the GEMM grid");
    return GBS_INVALID_ARGUMENT;
  }
  const double flops = (lower ? 1.0 : 2.0) * M * (double)N * K + (lower ? (double)M * K : 0.0);
  const double bytes = sizeof(T) * ((double)M * K + (double)K * N + (lower ? 1.0 : 2.0) * M * (double)N);
  PhaseScope ps(s, phase, flops, bytes);
  const int64_t sms = device_sm_count();
  if ((int64_t)grid.x * grid.y < sms) {
    // fewer 64 x 64 tiles than SMs: smaller tiles spread the update over more
    // SMs (an SM's FP64 rate, not bandwidth, bounds it).  Per-SM work in units
    // of one 64 x 64 tile: ceil(tiles / SMs) x (tile area / 64^2); the smaller
    // tile size wins ties.  Each element's sum runs over K in the same order
    // whatever the tile, so the results are identical.
    const int64_t t32 = (int64_t)ceil_div(N, 32) * ceil_div(M, 32), t16 = (int64_t)ceil_div(N, 16) * ceil_div(M, 16);
    const double w32 = (double)((t32 + sms - 1) / sms) / 4.0, w16 = (double)((t16 + sms - 1) / sms) / 16.0;
    if (w16 <= w32) {
      dim3 g3(ceil_div(N, 16), ceil_div(M, 16));
      gemm_sub_kernel<T, 16, 16, BK, 1, 1><<<g3, 256, 0, s>>>(M, N, K, A, a_rs, a_cs, B, b_rs, b_cs, C, ldc, lower,
                                                             stop_flag);
    } else {
      dim3 g2(ceil_div(N, 32), ceil_div(M, 32));
      gemm_sub_kernel<T, 32, 32, BK, 2, 2><<<g2, 256, 0, s>>>(M, N, K, A, a_rs, a_cs, B, b_rs, b_cs, C, ldc, lower,
                                                             stop_flag);
    }
  } else {
    gemm_sub_kernel<T, BM, BN, BK, TM, TN><<<grid, (BM / TM) * (BN / TN), 0, s>>>(
        M, N, K, A, a_rs, a_cs, B, b_rs, b_cs, C, ldc, lower, stop_flag);
  }
  GBS_CUDA_TRY(cudaGetLastError());
  return GBS_SUCCESS;
}

template <typename T>
int gemm_sub_device(cudaStream_t s, int phase, int M, int N, int K, const T* A, int64_t a_rs, int64_t a_cs, const T* B,
                    int64_t b_rs, int64_t b_cs, T* C, int64_t ldc)
{
  return gemm_sub<T>(s, phase, M, N, K, A, a_rs, a_cs, B, b_rs, b_cs, C, ldc, 0, nullptr);
}

template <typename T>
int syrk_sub_device(cudaStream_t s, int phase, int n, int K, const T* A, int64_t a_rs, int64_t a_cs, const T* B,
                    int64_t b_rs, int64_t b_cs, T* C, int64_t ldc)
{
  return gemm_sub<T>(s, phase, n, n, K, A, a_rs, a_cs, B, b_rs, b_cs, C, ldc, 1, nullptr);
}

// B(kb x ncols) <- L^{-1} B for a unit-lower L of kb <= 128 rows with many
// columns: 32-row blocks solved one column per thread, SIMT updates between.
template <typename T>
int trsm_lunit_wide(cudaStream_t s, int kb, int ncols, const T* L, int64_t ldl, T* B, int64_t ldb)
{
  for (int b0 = 0; b0 < kb; b0 += kPanelNB) {
    const int bb = std::min(kPanelNB, kb - b0);
    {
      PhaseScope ps(s, PH_TRSM_LU, (double)bb * bb * ncols, sizeof(T) * 2.0 * bb * ncols);
      trsm_lunit_kernel<T, kPanelNB><<<ceil_div(ncols, 128), 128, 0, s>>>(L + b0 * ldl + b0, ldl, bb, B + b0, ldb,
                                                                         ncols);
      GBS_CUDA_TRY(cudaGetLastError());
    }
    const int rest = kb - b0 - bb;
    if (rest > 0)
      GBS_TRY(gemm_sub<T>(s, PH_TRSM_LU, rest, ncols, bb, L + b0 * ldl + b0 + bb, 1, ldl, B + b0, 1, ldb,
                          B + b0 + bb, ldb, 0, nullptr));
  }
  return GBS_SUCCESS;
}

// Row interchanges tr[i0..i1) (applied in order) on the columns [c0,c1) and
// [c2,c3), as ONE gather: each CTA replays the swaps on a row map in shared
// memory, then every column reads its affected rows once (independent loads)
// and writes them to their final places.
// map[0] = cnt; map[1..1+cnt) = touched rows; map[257..257+cnt) = source row
// now at each.  One warp replays the interchanges in order, finding rows with
// a ballot over the list.
__global__ void laswp_map_kernel(const int* __restrict__ tr, int i0, int i1, int* __restrict__ map)
{
  griddep_launch_dependents();
  griddep_wait();
  __shared__ int rows[256], src[256];
  const int lane = threadIdx.x;
  int cnt = 0;
  for (int i = i0; i < i1; ++i) {
    const int r1 = i, r2 = tr[i];
    if (r1 == r2) continue;          // no interchange for this row
    int u1 = -1, u2 = -1;
    for (int b = 0; b < cnt; b += 32) {
      const int u = b + lane;
      const bool in = u < cnt;
      const unsigned m1 = __ballot_sync(0xffffffffu, in && rows[u] == r1);
      const unsigned m2 = __ballot_sync(0xffffffffu, in && rows[u] == r2);
      if (m1 && u1 < 0) u1 = b + __ffs(m1) - 1;
      if (m2 && u2 < 0) u2 = b + __ffs(m2) - 1;
    }
    if (u1 < 0) { u1 = cnt; if (lane == 0) { rows[cnt] = r1; src[cnt] = r1; } ++cnt; }
    if (u2 < 0) { u2 = cnt; if (lane == 0) { rows[cnt] = r2; src[cnt] = r2; } ++cnt; }
    __syncwarp();
    if (lane == 0) { const int t = src[u1]; src[u1] = src[u2]; src[u2] = t; }
    __syncwarp();
  }
  for (int u = lane; u < cnt; u += 32) {
    map[1 + u] = rows[u];
    map[257 + u] = src[u];
  }
  if (lane == 0) map[0] = cnt;
}

// Applies the row map to the columns [c0,c1) and [c2,c3): one warp per column
// reads every affected row once (independent loads), then writes them back
// to their final rows.
template <typename T>
__global__ void laswp_gather_kernel(T* __restrict__ a, int64_t lda, const int* __restrict__ map, int c0, int c1,
                                    int c2, int c3)
{
  griddep_launch_dependents();
  griddep_wait();
  __shared__ int rows[256], src[256];
  const int cnt = map[0];
  for (int u = threadIdx.x; u < cnt; u += blockDim.x) {
    rows[u] = map[1 + u];
    src[u] = map[257 + u];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  const int n1 = c1 - c0, ntot = n1 + (c3 - c2);
  for (int t = wid; t < ntot; t += nw) {
    const int col = t < n1 ? c0 + t : c2 + (t - n1);
    T* ac = a + (int64_t)col * lda;
    T v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int u = q * 32 + lane;
      if (u < cnt) v[q] = ac[src[u]];
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int u = q * 32 + lane;
      if (u < cnt) ac[rows[u]] = v[q];
    }
    __syncwarp();
  }
}

template <typename T>
int laswp_map_apply(cudaStream_t s, T* A, int64_t lda, const int* map, int c0, int c1, int c2, int c3)
{
  const int nc = (c1 - c0) + (c3 - c2);
  if (nc <= 0) return GBS_SUCCESS;
  PhaseScope ps(s, PH_LASWP, 0.0, 2.0 * sizeof(T) * (double)nc * 2 * kPanelNB);
  const int grid = std::min(ceil_div(nc, 8), 8 * device_sm_count());
  GBS_CUDA_TRY(launch_pdl(laswp_gather_kernel<T>, dim3(grid), dim3(256), 0, s, A, lda, map, c0, c1, c2, c3));
  GBS_CUDA_TRY(cudaGetLastError());
  return GBS_SUCCESS;
}

// The same row map for up to 128 interchanges of rows in [i0, m): the source
// row of every row of [i0, m) in shared memory, the interchanges replayed on
// it by one thread (constant time each), then the moved rows collected in
// parallel (the gather does not depend on the order of the entries).
__global__ void laswp_block_map_kernel(const int* __restrict__ tr, int i0, int i1, int m, int* __restrict__ map)
{
  griddep_launch_dependents();
  griddep_wait();
  extern __shared__ int src_of[];          // [m - i0]: source row now at row i0 + r
  __shared__ int s_tr[128];
  __shared__ int cnt;
  const int span = m - i0;
  for (int r = threadIdx.x; r < span; r += blockDim.x) src_of[r] = i0 + r;
  for (int i = threadIdx.x; i < i1 - i0; i += blockDim.x) s_tr[i] = tr[i0 + i];
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 0; i < i1 - i0; ++i) {
      const int p = s_tr[i] - i0;          // rows >= i0 + i
      if (p > i && p < span) {
        const int t = src_of[i];
        src_of[i] = src_of[p];
        src_of[p] = t;
      }
    }
  }
  __syncthreads();
  for (int r = threadIdx.x; r < span; r += blockDim.x) {
    const int src = src_of[r];
    if (src != i0 + r) {
      const int u = atomicAdd(&cnt, 1);
      if (u < 256) {                       // 128 interchanges move at most 256 rows
        map[1 + u] = i0 + r;
        map[257 + u] = src;
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) map[0] = min(cnt, 256);
}

template <typename T>
int laswp_block_device(cudaStream_t s, T* A, int64_t lda, int m, const int* tr, int i0, int i1, int c0, int c1,
                       int c2, int c3, DevBuf& map)
{
  const int nc = (c1 - c0) + (c3 - c2);
  if (nc <= 0 || i1 <= i0) return GBS_SUCCESS;
  const size_t smem = sizeof(int) * (size_t)(m - i0);
  if (i1 - i0 > 128 || smem > kBlockMapSmemMax)
    return laswp_gather_device<T>(s, A, lda, tr, i0, i1, c0, c1, c2, c3, map);
  static const cudaError_t attr = cudaFuncSetAttribute(laswp_block_map_kernel,
                                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                        (int)kBlockMapSmemMax);
  GBS_CUDA_TRY(attr);
  GBS_TRY(map.reserve(sizeof(int) * kLaswpMapInts));
  PhaseScope ps(s, PH_LASWP, 0.0, 2.0 * sizeof(T) * (double)nc * 2 * (i1 - i0));
  GBS_CUDA_TRY(launch_pdl(laswp_block_map_kernel, dim3(1), dim3(1024), smem, s, tr, i0, i1, m, map.as<int>()));
  count_launch();
  const int grid = std::min(ceil_div(nc, 8), 8 * device_sm_count());
  GBS_CUDA_TRY(launch_pdl(laswp_gather_kernel<T>, dim3(grid), dim3(256), 0, s, A, lda, (const int*)map.as<int>(), c0, c1,
                          c2, c3));
  GBS_CUDA_TRY(cudaGetLastError());
  return GBS_SUCCESS;
}

template <typename T>
int laswp_gather_device(cudaStream_t s, T* A, int64_t lda, const int* tr, int i0, int i1, int c0, int c1, int c2,
                        int c3, DevBuf& map)
{
  const int nc = (c1 - c0) + (c3 - c2);
  if (nc <= 0 || i1 <= i0) return GBS_SUCCESS;
  if (i1 - i0 > 128) {
    gbs_set_last_message("laswp_gather: at most 128 interchanges per call");
    return GBS_INVALID_ARGUMENT;
  }
  GBS_TRY(map.reserve(sizeof(int) * kLaswpMapInts));
  PhaseScope ps(s, PH_LASWP, 0.0, 2.0 * sizeof(T) * (double)nc * (i1 - i0));
  GBS_CUDA_TRY(launch_pdl(laswp_map_kernel, dim3(1), dim3(32), 0, s, tr, i0, i1, map.as<int>()));
  count_launch();
  const int grid = std::min(ceil_div(nc, 8), 8 * device_sm_count());
  GBS_CUDA_TRY(launch_pdl(laswp_gather_kernel<T>, dim3(grid), dim3(256), 0, s, A, lda, (const int*)map.as<int>(), c0, c1,
                          c2, c3));
  GBS_CUDA_TRY(cudaGetLastError());
  return GBS_SUCCESS;
}

// ------------------------------------------------------------------ LU
template <typename T>
int laswp_device(cudaStream_t s, T* B, int64_t ldb, int ncols, const int* dTr, int i0, int i1, int reverse)
{
  if (ncols <= 0 || i1 <= i0) return GBS_SUCCESS;
  PhaseScope ps(s, PH_LASWP, 0.0, 2.0 * sizeof(T) * (double)ncols * (i1 - i0));
  laswp_kernel<T><<<ceil_div(ncols, 128), 128, 0, s>>>(B, ldb, dTr, i0, i1, 0, ncols, 0, 0, reverse);
  GBS_CUDA_TRY(cudaGetLastError());
  return GBS_SUCCESS;
}

template <typename T>
int getrf_device(cudaStream_t s, int m, int n, T* dA, int64_t lda, int* dTr, DeviceStatus* dSt, DevBuf& scratch)
{
  const int size = std::min(m, n);
  for (int k = 0; k < size; k += kPanelNB) {
    const int kb = std::min(kPanelNB, size - k);
    T* Akk = dA + (int64_t)k * lda + k;
    const int* map = nullptr;
    GBS_TRY(panel_factor<T>(s, Akk, lda, m - k, kb, k, dTr + k, scratch, dSt, &map));
    // apply the panel's interchanges to A_0 (left) and A_2 (right): one gather
    // of the panel's row map, or the interchanges in order
    const int left = k, right0 = k + kb, nright = n - right0;
    if (map) {
      GBS_TRY(laswp_map_apply<T>(s, dA, lda, map, 0, left, right0, n));
    } else if (left + nright > 0) {
      PhaseScope ps(s, PH_LASWP, 0.0, 2.0 * sizeof(T) * (double)(left + nright) * kb);
      laswp_kernel<T><<<ceil_div(left + nright, 128), 128, 0, s>>>(dA, lda, dTr, k, k + kb, 0, left, right0, n, 0);
      GBS_CUDA_TRY(cudaGetLastError());
    }
    if (nright > 0) {
      T* A12 = dA + (int64_t)right0 * lda + k;
      {
        PhaseScope ps(s, PH_TRSM_LU, (double)kb * kb * nright, sizeof(T) * 2.0 * kb * nright);
        trsm_lunit_kernel<T, kPanelNB><<<ceil_div(nright, 128), 128, 0, s>>>(Akk, lda, kb, A12, lda, nright);
        GBS_CUDA_TRY(cudaGetLastError());
      }
      const int trows = m - k - kb;
      if (trows > 0) {
        const T* A21 = Akk + kb;
        T* A22 = dA + (int64_t)right0 * lda + k + kb;
        GBS_TRY(gemm_sub<T>(s, PH_GEMM, trows, nright, kb, A21, 1, lda, A12, 1, lda, A22, lda, 0, nullptr));
      }
    }
  }
  return GBS_SUCCESS;
}

template <typename T>
int getrf_preload()
{
  cudaFuncAttributes fa;
  const void* kernels[] = {
      (const void*)laswp_map_kernel,
      (const void*)laswp_gather_kernel<T>,
      (const void*)laswp_kernel<T>,
      (const void*)trsm_lunit_kernel<T, kPanelNB>,
      (const void*)gemm_sub_kernel<T, 64, 64, 16, 4, 4>,
      (const void*)gemm_sub_kernel<T, 32, 32, 16, 2, 2>,
      (const void*)gemm_sub_kernel<T, 16, 16, 16, 1, 1>,
  };
  for (const void* k : kernels) GBS_CUDA_TRY(cudaFuncGetAttributes(&fa, k));
  return panel_preload<T>();
}

// ------------------------------------------------------------------ LLT
template <typename T>
static int potrf_lower(cudaStream_t s, int n, T* dA, int64_t lda, DeviceStatus* dSt)
{
  constexpr int max_bs = 128;
  static const cudaError_t attr = [] {         // once per process (thread-safe static initialisation)
    cudaError_t e = cudaFuncSetAttribute(potrf_diag_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)potrf_diag_smem<T>(max_bs));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(trsm_rlt_blocked_kernel<T, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)(sizeof(T) * (max_bs * (max_bs + 1) + max_bs * 32 + max_bs)));
    return e;
  }();
  GBS_CUDA_TRY(attr);
  if (n < 32) {
    PhaseScope ps(s, PH_POTRF_DIAG, (double)n * n * n / 3.0, sizeof(T) * (double)n * n);
    potrf_diag_kernel<T><<<1, 256, potrf_diag_smem<T>(n), s>>>(dA, lda, n, 0, dSt);
    GBS_CUDA_TRY(cudaGetLastError());
    return GBS_SUCCESS;
  }
  // the reference's block size (LLT.h:338-340): identical blocking keeps the
  // matrix contents identical to the reference's after an early failure.
  // Plain launches: programmatic dependent launch measured slower on this
  // FP64 chain (LLT n = 512: 874 -> 824 solves/s).
  int bs = n / 8;
  bs = (bs / 16) * 16;
  bs = std::min(std::max(bs, 8), max_bs);
  for (int k = 0; k < n; k += bs) {
    const int b = std::min(bs, n - k);
    const int rs = n - k - b;
    T* Akk = dA + (int64_t)k * lda + k;
    {
      PhaseScope ps(s, PH_POTRF_DIAG, (double)b * b * b / 3.0, sizeof(T) * (double)b * b);
      potrf_diag_kernel<T><<<1, 256, potrf_diag_smem<T>(b), s>>>(Akk, lda, b, k, dSt);
      GBS_CUDA_TRY(cudaGetLastError());
    }
    if (rs > 0) {
      T* A21 = Akk + b;
      {
      PhaseScope ps(s, PH_TRSM_LLT, (double)rs * b * b, sizeof(T) * 2.0 * rs * b);
      trsm_rlt_blocked_kernel<T, 32><<<ceil_div(rs, 32), 256, sizeof(T) * (b * (b + 1) + b * 32 + b), s>>>(
          Akk, lda, b, A21, lda, rs, dSt);
      GBS_CUDA_TRY(cudaGetLastError());
      }
      T* A22 = A21 + (int64_t)b * lda;
      GBS_TRY(gemm_sub<T>(s, PH_SYRK, rs, rs, b, A21, 1, lda, A21, lda, 1, A22, lda, 1, &dSt->info));
    }
  }
  return GBS_SUCCESS;
}

template <typename T>
int potrf_device(cudaStream_t s, int n, T* dA, int64_t lda, int upper, DeviceStatus* dSt, DevBuf& tmp)
{
  if (n <= 0) return GBS_SUCCESS;
  if (!upper) return potrf_lower<T>(s, n, dA, lda, dSt);
  // Upper: the reference factors the transposed view with the lower
  // algorithm (LLT.h:362-383); same here on a transposed copy.
  GBS_TRY(tmp.reserve(sizeof(T) * (size_t)n * n));
  T* L = tmp.as<T>();
  int64_t tot = (int64_t)n * n;
  int grid = (int)std::min<int64_t>((tot + 255) / 256, 65535 * 4);
  {
    PhaseScope ps(s, PH_COPY, 0.0, sizeof(T) * (double)n * n);
    transpose_triangle_kernel<T><<<grid, 256, 0, s>>>(dA, lda, L, n, n, 1);
    GBS_CUDA_TRY(cudaGetLastError());
  }
  GBS_TRY(potrf_lower<T>(s, n, L, n, dSt));
  {
    PhaseScope ps(s, PH_COPY, 0.0, sizeof(T) * (double)n * n);
    transpose_triangle_kernel<T><<<grid, 256, 0, s>>>(L, n, dA, lda, n, 0);
    GBS_CUDA_TRY(cudaGetLastError());
  }
  return GBS_SUCCESS;
}

// ------------------------------------------------------------------ solves
template <typename T>
int tri_solve_device(cudaStream_t s, int n, int nrhs, const T* tri, int64_t ld, int lower, int trans, int unit,
                     T* B, int64_t ldb, SolveWork& w, const T* dinv)
{
  if (n <= 0 || nrhs <= 0) return GBS_SUCCESS;
  // FP64: 32-row blocks keep the per-block DFMA work on the critical path
  // short; FP32: 64-row blocks.
  constexpr int NB = tri_solve_nb<T>();
  constexpr int RC = 16;
  const int64_t rs = trans ? ld : 1, cs = trans ? 1 : ld;   // op(Tri)(i,j) = tri[i*rs + j*cs]
  const int forward = (lower != 0) != (trans != 0);
  const int nblk = ceil_div(n, NB);
  GBS_TRY(w.flags.reserve(sizeof(int) * (size_t)(nblk + 2)));
  GBS_TRY(solve_err_slot(s, w));
  const uint64_t limit = wait_limit_ns();
  const int grid = std::min(nblk, 2 * device_sm_count());
  constexpr size_t smem = trsm_persistent_smem<T, NB, RC>();
  static const cudaError_t attr = cudaFuncSetAttribute(trsm_persistent_kernel<T, NB, RC>,
                                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  GBS_CUDA_TRY(attr);
  for (int c0 = 0; c0 < nrhs; c0 += RC) {
    const int nc = std::min(RC, nrhs - c0);
    GBS_CUDA_TRY(cudaMemsetAsync(w.flags.p, 0, sizeof(int) * (size_t)(nblk + 2), s));
    PhaseScope ps(s, PH_TRI_SOLVE, (double)n * n * nc, sizeof(T) * (0.5 * (double)n * n + 2.0 * n * nc));
    trsm_persistent_kernel<T, NB, RC><<<grid, RC * 32, smem, s>>>(n, nc, tri, rs, cs, forward, unit,
                                                                   B + (int64_t)c0 * ldb, ldb, w.flags.as<int>(),
                                                                   dinv, w.err.as<int>(), limit);
    GBS_CUDA_TRY(cudaGetLastError());
  }
  return GBS_SUCCESS;
}

int solve_err_slot(cudaStream_t s, SolveWork& w)
{
  if (w.err.p) return GBS_SUCCESS;
  GBS_TRY(w.err.reserve(16));
  GBS_CUDA_TRY(cudaMemsetAsync(w.err.p, 0, 16, s));
  return GBS_SUCCESS;
}

int solve_status(cudaStream_t s, SolveWork& w)
{
  GBS_CUDA_TRY(cudaStreamSynchronize(s));
  if (!w.err.p) return GBS_SUCCESS;
  int h = 0;
  GBS_CUDA_TRY(cudaMemcpy(&h, w.err.p, sizeof(h), cudaMemcpyDeviceToHost));
  if (h) {
    GBS_CUDA_TRY(cudaMemset(w.err.p, 0, sizeof(h)));    // the next solve on this workspace starts clean
    gbs_set_last_message("a triangular-solve wait timed out");
    return GBS_TIMEOUT;
  }
  return GBS_SUCCESS;
}

// Failure-detection diagnostics.  The persistent solve of an n x n system
// (identity triangle, one right-hand side) with the ticket counter started at
// 1: no CTA ever takes block 0, so its ready flag is never published and every
// CTA's first wait runs out; after the first timeout the others see the flag
// and leave, so the launch ends after about one wait limit.
int tri_solve_timeout_selftest(cudaStream_t s, int n)
{
  constexpr int NB = tri_solve_nb<double>();
  constexpr int RC = 16;
  if (n < 2 * NB) n = 2 * NB;
  const int nblk = ceil_div(n, NB);
  DevBuf tri, b;
  SolveWork w;
  GBS_TRY(tri.reserve(sizeof(double) * (size_t)n * n));
  GBS_TRY(b.reserve(sizeof(double) * (size_t)n));
  GBS_TRY(w.flags.reserve(sizeof(int) * (size_t)(nblk + 2)));
  GBS_TRY(w.err.reserve(16));
  GBS_CUDA_TRY(cudaMemsetAsync(tri.p, 0, sizeof(double) * (size_t)n * n, s));
  GBS_CUDA_TRY(cudaMemsetAsync(b.p, 0, sizeof(double) * (size_t)n, s));
  GBS_CUDA_TRY(cudaMemsetAsync(w.flags.p, 0, sizeof(int) * (size_t)(nblk + 2), s));
  GBS_CUDA_TRY(cudaMemsetAsync(w.err.p, 0, 16, s));
  static const int one = 1;
  GBS_CUDA_TRY(cudaMemcpyAsync(w.flags.p, &one, sizeof(int), cudaMemcpyHostToDevice, s));
  const int grid = std::min(nblk, 2 * device_sm_count());
  constexpr size_t smem = trsm_persistent_smem<double, NB, RC>();
  GBS_CUDA_TRY(cudaFuncSetAttribute(trsm_persistent_kernel<double, NB, RC>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  count_launch();
  trsm_persistent_kernel<double, NB, RC><<<grid, RC * 32, smem, s>>>(n, 1, tri.as<double>(), 1, n, 1, 1,
                                                                    b.as<double>(), n, w.flags.as<int>(), nullptr,
                                                                    w.err.as<int>(), wait_limit_ns());
  GBS_CUDA_TRY(cudaGetLastError());
  return solve_status(s, w);
}

// Two CTAs meet at a grid barrier that counts three arrivals.
__global__ void barrier_selftest_kernel(DeviceStatus* st) { grid_barrier(st, gridDim.x + 1); }

int barrier_timeout_selftest(cudaStream_t s)
{
  DevBuf st;
  GBS_TRY(st.reserve(sizeof(DeviceStatus)));
  GBS_TRY(reset_status(st.as<DeviceStatus>(), s));
  count_launch();
  barrier_selftest_kernel<<<2, 32, 0, s>>>(st.as<DeviceStatus>());
  GBS_CUDA_TRY(cudaGetLastError());
  DeviceStatus h;
  return read_status(st.as<DeviceStatus>(), &h, s);
}

template <typename T>
int lu_solve_device(cudaStream_t s, int n, int nrhs, const T* dLU, int64_t ld, const int* dTr, T* B, int64_t ldb,
                    int transpose, SolveWork& w)
{
  if (!transpose) {
    GBS_TRY(laswp_device<T>(s, B, ldb, nrhs, dTr, 0, n, 0));
    GBS_TRY(tri_solve_device<T>(s, n, nrhs, dLU, ld, 1, 0, 1, B, ldb, w));
    GBS_TRY(tri_solve_device<T>(s, n, nrhs, dLU, ld, 0, 0, 0, B, ldb, w));
  } else {
    GBS_TRY(tri_solve_device<T>(s, n, nrhs, dLU, ld, 0, 1, 0, B, ldb, w));
    GBS_TRY(tri_solve_device<T>(s, n, nrhs, dLU, ld, 1, 1, 1, B, ldb, w));
    GBS_TRY(laswp_device<T>(s, B, ldb, nrhs, dTr, 0, n, 1));
  }
  return GBS_SUCCESS;
}

template <typename T>
int llt_solve_device(cudaStream_t s, int n, int nrhs, const T* dL, int64_t ld, int upper, T* B, int64_t ldb,
                     SolveWork& w)
{
  if (!upper) {
    GBS_TRY(tri_solve_device<T>(s, n, nrhs, dL, ld, 1, 0, 0, B, ldb, w));
    GBS_TRY(tri_solve_device<T>(s, n, nrhs, dL, ld, 1, 1, 0, B, ldb, w));
  } else {
    GBS_TRY(tri_solve_device<T>(s, n, nrhs, dL, ld, 0, 1, 0, B, ldb, w));
    GBS_TRY(tri_solve_device<T>(s, n, nrhs, dL, ld, 0, 0, 0, B, ldb, w));
  }
  return GBS_SUCCESS;
}

template <typename T>
int copy_matrix_device(cudaStream_t s, const T* a, int64_t lda, T* b, int64_t ldb, int m, int n)
{
  if (m <= 0 || n <= 0) return GBS_SUCCESS;
  GBS_CUDA_TRY(cudaMemcpy2DAsync(b, ldb * sizeof(T), a, lda * sizeof(T), (size_t)m * sizeof(T), n,
                                 cudaMemcpyDeviceToDevice, s));
  return GBS_SUCCESS;
}

// ------------------------------------------------------------------ norms
template <typename T>
int l1_norm_device(cudaStream_t s, const T* dA, int64_t lda, int m, int n, int sym, int upper, double* d_out,
                   double* h_out)
{
  GBS_CUDA_TRY(cudaMemsetAsync(d_out, 0, sizeof(double), s));
  if (m > 0 && n > 0) {
    PhaseScope ps(s, PH_NORM, (double)m * n, sizeof(T) * (double)m * n);
    const int wpb = 8;
    if (sym) sym_l1_norm_kernel<T><<<ceil_div(n, wpb), 32 * wpb, 0, s>>>(dA, lda, n, upper, d_out);
    else l1_norm_kernel<T><<<ceil_div(n, wpb), 32 * wpb, 0, s>>>(dA, lda, m, n, d_out);
    GBS_CUDA_TRY(cudaGetLastError());
  }
  if (h_out) {
    GBS_CUDA_TRY(cudaMemcpyAsync(h_out, d_out, sizeof(double), cudaMemcpyDeviceToHost, s));
    GBS_CUDA_TRY(cudaStreamSynchronize(s));
  }
  return GBS_SUCCESS;
}

// ------------------------------------------------------------------ rcond
// ConditionEstimator.h:56-142.  The control flow (sign vectors, argmax, bound
// comparisons) runs on the host on n-vectors read back after each solve.
template <typename T>
static int dec_solve(cudaStream_t s, int kind, int n, const T* dF, int64_t ld, const int* dTr, T* v, int adjoint,
                     SolveWork& w)
{
  if (kind == 0) GBS_TRY(lu_solve_device<T>(s, n, 1, dF, ld, dTr, v, n, adjoint, w));
  else if (kind == 3) GBS_TRY(ldlt_solve_device<T>(s, n, 1, dF, ld, dTr, v, n, w));   // self-adjoint
  else GBS_TRY(llt_solve_device<T>(s, n, 1, dF, ld, kind == 2, v, n, w));
  return solve_status(s, w);
}

template <typename T>
int inv_l1_estimate_device(cudaStream_t s, int kind, int n, const T* dF, int64_t ld, const int* dTr, DevBuf& vec,
                           HostBuf& hvec, SolveWork& w, double* est)
{
  if (n == 0) { *est = 0; return GBS_SUCCESS; }
  GBS_TRY(vec.reserve(sizeof(T) * (size_t)n));
  GBS_TRY(hvec.reserve(sizeof(T) * (size_t)n * 3));
  T* dv = vec.as<T>();
  T* hv = (T*)hvec.p;
  T* sgn = hv + n;
  T* old_sgn = hv + 2 * (size_t)n;
  auto upload = [&]() -> int {
    GBS_CUDA_TRY(cudaMemcpyAsync(dv, hv, sizeof(T) * n, cudaMemcpyHostToDevice, s));
    return GBS_SUCCESS;
  };
  auto download = [&]() -> int {
    GBS_CUDA_TRY(cudaMemcpyAsync(hv, dv, sizeof(T) * n, cudaMemcpyDeviceToHost, s));
    GBS_CUDA_TRY(cudaStreamSynchronize(s));
    return GBS_SUCCESS;
  };
  auto l1 = [&]() {
    T acc = 0;
    for (int i = 0; i < n; ++i) acc += hv[i] < 0 ? -hv[i] : hv[i];
    return acc;
  };
  for (int i = 0; i < n; ++i) hv[i] = T(1) / T(n);
  GBS_TRY(upload());
  GBS_TRY(dec_solve<T>(s, kind, n, dF, ld, dTr, dv, 0, w));
  GBS_TRY(download());
  T lower_bound = l1();
  if (n == 1) { *est = (double)lower_bound; return GBS_SUCCESS; }
  T old_lower_bound = lower_bound;
  int vmax = -1, old_vmax = -1;
  for (int k = 0; k < 4; ++k) {
    for (int i = 0; i < n; ++i) sgn[i] = hv[i] < T(0) ? T(-1) : T(1);
    if (k > 0 && memcmp(sgn, old_sgn, sizeof(T) * n) == 0) break;
    for (int i = 0; i < n; ++i) hv[i] = sgn[i];
    GBS_TRY(upload());
    GBS_TRY(dec_solve<T>(s, kind, n, dF, ld, dTr, dv, 1, w));
    GBS_TRY(download());
    vmax = 0;
    T best = hv[0] < 0 ? -hv[0] : hv[0];
    for (int i = 1; i < n; ++i) {
      T t = hv[i] < 0 ? -hv[i] : hv[i];
      if (t > best) { best = t; vmax = i; }
    }
    if (vmax == old_vmax) break;
    for (int i = 0; i < n; ++i) hv[i] = T(0);
    hv[vmax] = T(1);
    GBS_TRY(upload());
    GBS_TRY(dec_solve<T>(s, kind, n, dF, ld, dTr, dv, 0, w));
    GBS_TRY(download());
    lower_bound = l1();
    if (lower_bound <= old_lower_bound) break;
    memcpy(old_sgn, sgn, sizeof(T) * n);
    old_vmax = vmax;
    old_lower_bound = lower_bound;
  }
  T alt = 1;
  for (int i = 0; i < n; ++i) {
    hv[i] = alt * (T(1) + (T(i) / T(n - 1)));
    alt = -alt;
  }
  GBS_TRY(upload());
  GBS_TRY(dec_solve<T>(s, kind, n, dF, ld, dTr, dv, 0, w));
  GBS_TRY(download());
  T alternate = (T(2) * l1()) / (T(3) * T(n));
  *est = (double)(lower_bound > alternate ? lower_bound : alternate);
  return GBS_SUCCESS;
}

// ConditionEstimator.h:157-169, evaluated in the scalar type of the factor.
double rcond_from_estimate(int64_t n, double matrix_norm, double inv_norm, bool single)
{
  if (n == 0) return 1.0;
  if (single) {
    float mn = (float)matrix_norm, inv = (float)inv_norm;
    if (mn == 0.0f) return 0.0;
    if (n == 1) return 1.0;
    return inv == 0.0f ? 0.0 : (double)((1.0f / inv) / mn);
  }
  if (matrix_norm == 0.0) return 0.0;
  if (n == 1) return 1.0;
  return inv_norm == 0.0 ? 0.0 : (1.0 / inv_norm) / matrix_norm;
}

// ------------------------------------------------------------------ instantiations
#define GBS_INSTANTIATE(T)                                                                                      \
  template int getrf_device<T>(cudaStream_t, int, int, T*, int64_t, int*, DeviceStatus*, DevBuf&);               \
  template int getrf_preload<T>();                                                                              \
  template int potrf_device<T>(cudaStream_t, int, T*, int64_t, int, DeviceStatus*, DevBuf&);                     \
  template int tri_solve_device<T>(cudaStream_t, int, int, const T*, int64_t, int, int, int, T*, int64_t,       \
                                   SolveWork&, const T*);                                                    \
  template int laswp_device<T>(cudaStream_t, T*, int64_t, int, const int*, int, int, int);                       \
  template int lu_solve_device<T>(cudaStream_t, int, int, const T*, int64_t, const int*, T*, int64_t, int,       \
                                  SolveWork&);                                                               \
  template int llt_solve_device<T>(cudaStream_t, int, int, const T*, int64_t, int, T*, int64_t, SolveWork&);     \
  template int l1_norm_device<T>(cudaStream_t, const T*, int64_t, int, int, int, int, double*, double*);         \
  template int inv_l1_estimate_device<T>(cudaStream_t, int, int, const T*, int64_t, const int*, DevBuf&, HostBuf&, \
                                         SolveWork&, double*);                                                               \
  template int copy_matrix_device<T>(cudaStream_t, const T*, int64_t, T*, int64_t, int, int);                   \
  template int gemm_sub_device<T>(cudaStream_t, int, int, int, int, const T*, int64_t, int64_t, const T*, int64_t, \
                                  int64_t, T*, int64_t);                                                       \
  template int syrk_sub_device<T>(cudaStream_t, int, int, int, const T*, int64_t, int64_t, const T*, int64_t,     \
                                  int64_t, T*, int64_t);                                                       \
  template int trsm_lunit_wide<T>(cudaStream_t, int, int, const T*, int64_t, T*, int64_t);                     \
  template int laswp_gather_device<T>(cudaStream_t, T*, int64_t, const int*, int, int, int, int, int, int, DevBuf&); \
  template int laswp_map_apply<T>(cudaStream_t, T*, int64_t, const int*, int, int, int, int);                 \
  template int laswp_block_device<T>(cudaStream_t, T*, int64_t, int, const int*, int, int, int, int, int, int,  \
                                     DevBuf&);

GBS_INSTANTIATE(double)
GBS_INSTANTIATE(float)

}  // namespace gbs
