// C-ABI of the low-precision tiers: the standalone tensor-core update and
// (below) the mixed-precision factor + iterative-refinement solvers.
#include <algorithm>

#include "dense_driver.cuh"
#include "tc_gemm.cuh"

using namespace gbs;

extern "C" int gbs_tc_gemm_sub(int kind, int m, int n, int k, const float* d_a, int64_t lda, const float* d_b,
                               int64_t ldb, float* d_c, int64_t ldc, int lower, void* stream)
{
  if (m < 0 || n < 0 || k < 0 || kind < TC_BF16 || kind > TC_TF32X3) return GBS_INVALID_ARGUMENT;
  if ((m > 0 && lda < m) || (k > 0 && ldb < k) || (m > 0 && ldc < m) || (lower && m != n)) return GBS_INVALID_ARGUMENT;
  if (m == 0 || n == 0 || k == 0) return GBS_SUCCESS;
  WorkspaceLease lease;
  if (lease.status != GBS_SUCCESS) return lease.status;
  Workspace& w = *lease.ws;
  cudaStream_t s = stream ? (cudaStream_t)stream : w.stream;
  GBS_TRY(w.status.reserve(sizeof(DeviceStatus)));
  GBS_TRY(reset_status(w.status.as<DeviceStatus>(), s));
  static thread_local TcWorkspace tws;
  GBS_TRY(tc_gemm_sub(s, kind, m, n, k, d_a, 1, lda, d_b, 1, ldb, d_c, ldc, lower, w.status.as<DeviceStatus>(), tws));
  DeviceStatus h;
  return read_status(w.status.as<DeviceStatus>(), &h, s);
}
