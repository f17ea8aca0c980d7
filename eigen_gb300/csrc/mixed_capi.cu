// C-ABI of the low-precision tiers: the standalone tensor-core update and
// (below) the mixed-precision factor + iterative-refinement solvers.
#include <algorithm>

#include "dense_driver.cuh"
#include "mixed_driver.cuh"
#include "tc_gemm.cuh"

using namespace gbs;

static void fill_info(gbs_refine_info* info, const MixedResult& r)
{
  if (!info) return;
  info->tier_used = r.tier;
  info->iterations = r.iterations;
  info->fell_back = r.fell_back;
  info->singular = r.singular;
  info->backward_error = r.backward_error;
}

static int check_mixed_args(int n, int nrhs, int lda, int ldb, int ldx, int tier, int max_iter)
{
  if (n < 0 || nrhs < 0 || lda < std::max(1, n) || ldb < std::max(1, n) || ldx < std::max(1, n) ||
      tier < GBS_TIER_FP64 || tier > GBS_TIER_FP16 || max_iter < 0) {
    gbs_set_last_message("gbs_dgesv_mixed: invalid argument");
    return GBS_INVALID_ARGUMENT;
  }
  return GBS_SUCCESS;
}

extern "C" int gbs_dgesv_mixed_device(int n, int nrhs, const double* d_a, int lda, const double* d_b, int ldb,
                                      double* d_x, int ldx, int tier, double tol, int max_iter, gbs_refine_info* info,
                                      void* stream)
{
  GBS_TRY(check_mixed_args(n, nrhs, lda, ldb, ldx, tier, max_iter));
  GBS_TRY(ensure_device());
  MixedOptions opt;
  opt.tier = tier;
  opt.tol = tol;
  opt.max_iter = max_iter;
  MixedResult r;
  WorkspaceLease lease;
  if (lease.status != GBS_SUCCESS) return lease.status;
  cudaStream_t s = stream ? (cudaStream_t)stream : lease.ws->stream;
  GBS_TRY(mixed_lu_solve(s, n, nrhs, d_a, lda, d_b, ldb, d_x, ldx, opt, &r));
  fill_info(info, r);
  return GBS_SUCCESS;
}

extern "C" int gbs_dgesv_mixed(int n, int nrhs, const double* a, int lda, const double* b, int ldb, double* x, int ldx,
                               int tier, double tol, int max_iter, gbs_refine_info* info)
{
  GBS_TRY(check_mixed_args(n, nrhs, lda, ldb, ldx, tier, max_iter));
  if (n == 0 || nrhs == 0) return GBS_SUCCESS;
  WorkspaceLease lease;
  if (lease.status != GBS_SUCCESS) return lease.status;
  Workspace& w = *lease.ws;
  cudaStream_t s = w.stream;
  GBS_TRY(w.a.reserve(sizeof(double) * (size_t)n * n));
  GBS_TRY(w.b.reserve(sizeof(double) * (size_t)n * nrhs * 2));
  double* dA = w.a.as<double>();
  double* dB = w.b.as<double>();
  double* dX = dB + (size_t)n * nrhs;
  GBS_CUDA_TRY(cudaMemcpy2DAsync(dA, sizeof(double) * n, a, sizeof(double) * lda, sizeof(double) * n, n,
                                 cudaMemcpyHostToDevice, s));
  GBS_CUDA_TRY(cudaMemcpy2DAsync(dB, sizeof(double) * n, b, sizeof(double) * ldb, sizeof(double) * n, nrhs,
                                 cudaMemcpyHostToDevice, s));
  MixedOptions opt;
  opt.tier = tier;
  opt.tol = tol;
  opt.max_iter = max_iter;
  MixedResult r;
  GBS_TRY(mixed_lu_solve(s, n, nrhs, dA, n, dB, n, dX, n, opt, &r));
  GBS_CUDA_TRY(cudaMemcpy2DAsync(x, sizeof(double) * ldx, dX, sizeof(double) * n, sizeof(double) * n, nrhs,
                                 cudaMemcpyDeviceToHost, s));
  GBS_CUDA_TRY(cudaStreamSynchronize(s));
  fill_info(info, r);
  return GBS_SUCCESS;
}

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
