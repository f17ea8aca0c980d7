// gbs_dgetrf_noalloc: the LU factorization for callers that cannot let a
// library call cudaMalloc (see include/gb300solve.h).
//
// The factorization is the one gbs_dgetrf runs (getrf_device: cooperative panel
// kernel, row interchanges, TRSM, DFMA trailing update).  The only global
// memory it needs beyond the caller's matrix and pivot array is the panel's
// candidate-exchange scratch and the 32-byte device status word.  Here both
// live in one file-scope __device__ array of fixed size instead of buffers
// from cudaMalloc.
#include <mutex>
#include <vector>

#include "dense_driver.cuh"
#include "dense_kernels.cuh"
#include "gbs_profile.cuh"

namespace {

using namespace gbs;

// Stated maximum: 256 KiB, held by every GPU that loads the library until the
// process exits.  Bytes [0, 256) hold the device status word, the rest the
// panel scratch.
constexpr size_t kScratchBytes = 256 * 1024;
constexpr size_t kStatusBytes = 256;
constexpr int kMaxDim = 65536;   // largest m and n accepted (panel scratch fits for m <= 124,672)

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// The status word keeps the previous call's contents: start every call from
// zero (barrier counters, timeout flag, swap count) with info = -1.
__global__ void noalloc_reset_status(DeviceStatus* st, unsigned long long limit_ns)
{
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    st->limit_ns = limit_ns;
    st->bar_count = 0;
    st->bar_gen = 0;
    st->timeout = 0;
    st->info = -1;
    st->nb_transpositions = 0;
  }
}

// 0-based absolute transpositions -> LAPACK's 1-based ipiv, and the LAPACK info.
__global__ void noalloc_finish(const DeviceStatus* st, int* ipiv, int size, int* info)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < size) ipiv[i] += 1;
  if (i == 0) {
    if (st->timeout) *info = -(100 + GBS_TIMEOUT);
    else *info = st->info >= 0 ? st->info + 1 : 0;
  }
}

// Host code may not use g_noalloc_scratch as an address: it names a host-side
// stand-in.  The device address comes from cudaGetSymbolAddress, once per
// device, with that device current.
std::mutex g_addr_mu;
std::vector<void*> g_addr;

int scratch_address(void** out)
{
  int dev = 0;
  GBS_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_addr_mu);
  if ((int)g_addr.size() <= dev) g_addr.resize(dev + 1, nullptr);
  if (!g_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      gbs_set_last_cuda_error(e, "cudaGetSymbolAddress(g_noalloc_scratch)", __FILE__, __LINE__);
      return GBS_CUDA_ERROR;
    }
    // Kernels load lazily on their first launch, which can take device
    // memory.  Load here every kernel a call of any shape can launch (the
    // cluster or the cooperative panel, each GEMM tile size, the interchange
    // kernels), so later calls of other shapes load nothing.
    cudaFuncAttributes fa;
    GBS_CUDA_TRY(cudaFuncGetAttributes(&fa, (const void*)noalloc_reset_status));
    GBS_CUDA_TRY(cudaFuncGetAttributes(&fa, (const void*)noalloc_finish));
    GBS_TRY(getrf_preload<double>());
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return GBS_SUCCESS;
}

}  // namespace

extern "C" int gbs_dgetrf_noalloc(int m, int n, double* d_a, int lda, int* d_ipiv, int* d_info, void* stream)
{
  if (m < 0 || n < 0 || lda < (m > 1 ? m : 1) || !d_info || ((m > 0 && n > 0) && (!d_a || !d_ipiv))) {
    gbs_set_last_message("gbs_dgetrf_noalloc: invalid argument");
    return GBS_INVALID_ARGUMENT;
  }
  if (m > kMaxDim || n > kMaxDim) {
    gbs_set_last_message("gbs_dgetrf_noalloc: m and n must not exceed 65536 (fixed scratch of 256 KiB)");
    return GBS_INVALID_ARGUMENT;
  }
  GBS_TRY(ensure_device());
  cudaStream_t s = (cudaStream_t)stream;
  void* base = nullptr;
  GBS_TRY(scratch_address(&base));
  DeviceStatus* st = (DeviceStatus*)base;
  const int size = m < n ? m : n;

  // The panel scratch needed by the tallest panel (m rows) is at most
  // panel_scratch_bytes(ceil(m / 256)); every later panel needs less.
  const int p_max = (m + kPanelThreads - 1) / kPanelThreads;
  if (panel_scratch_bytes<double, kPanelNB>(p_max > 0 ? p_max : 1) > kScratchBytes - kStatusBytes) {
    gbs_set_last_message("gbs_dgetrf_noalloc: panel scratch exceeds the fixed 256 KiB array");
    return GBS_INVALID_ARGUMENT;
  }

  count_launch();
  noalloc_reset_status<<<1, 32, 0, s>>>(st, wait_limit_ns());
  GBS_CUDA_TRY(cudaGetLastError());
  int rc = GBS_SUCCESS;
  if (size > 0) {
    // A borrowed view of the static array, which is large enough for every
    // panel of this call (checked above).
    DevBuf view;
    view.borrowed = true;      // reserve() refuses to grow it, release() never frees it
    view.p = (unsigned char*)base + kStatusBytes;
    view.bytes = kScratchBytes - kStatusBytes;
    rc = getrf_device<double>(s, m, n, d_a, lda, d_ipiv, st, view);
  }
  if (rc != GBS_SUCCESS) return rc;
  count_launch();
  noalloc_finish<<<(size + 255) / 256 > 0 ? (size + 255) / 256 : 1, 256, 0, s>>>(st, d_ipiv, size, d_info);
  GBS_CUDA_TRY(cudaGetLastError());
  return GBS_SUCCESS;
}
