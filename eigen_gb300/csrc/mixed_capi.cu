// C-ABI of the low-precision tiers: the standalone tensor-core update and the
// mixed-precision factor + FP64 refinement solvers (gbs_d{ge,po}sv_mixed*).
#include <algorithm>

#include "dense_driver.cuh"
#include "mixed_driver.cuh"
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
  cudaStream_t s = (cudaStream_t)stream;     // NULL: the legacy default stream
  GBS_TRY(w.status.reserve(sizeof(DeviceStatus)));
  GBS_TRY(reset_status(w.status.as<DeviceStatus>(), s));
  static thread_local TcWorkspace tws;
  GBS_TRY(tc_gemm_sub(s, kind, m, n, k, d_a, 1, lda, d_b, 1, ldb, d_c, ldc, lower, w.status.as<DeviceStatus>(), tws));
  DeviceStatus h;
  return read_status(w.status.as<DeviceStatus>(), &h, s);
}

extern "C" void gbs_refine_options_default(gbs_refine_options* o)
{
  if (!o) return;
  MixedOptions d;
  o->tier = d.tier;
  o->refine = d.refine;
  o->tol = d.tol;
  o->max_iter = d.max_iter;
  o->gmres_restart = d.gmres_restart;
  o->gmres_tol = d.gmres_tol;
  o->shift_factor = d.shift_factor;
  o->lookahead = d.lookahead;
  o->residual = d.residual;
  o->pivoting = d.pivoting;
}

static int to_options(const gbs_refine_options* o, MixedOptions* m)
{
  MixedOptions d;
  if (o) {
    d.tier = o->tier;
    d.refine = o->refine;
    d.tol = o->tol;
    d.max_iter = o->max_iter;
    d.gmres_restart = o->gmres_restart;
    d.gmres_tol = o->gmres_tol;
    d.shift_factor = o->shift_factor;
    d.lookahead = o->lookahead;
    d.residual = o->residual;
    d.pivoting = o->pivoting;
  }
  if (d.tier < GBS_TIER_FP64 || d.tier > GBS_TIER_FP16 || d.refine < GBS_REFINE_AUTO || d.refine > GBS_REFINE_GMRES ||
      d.max_iter < 0 || d.gmres_restart < 1 || d.gmres_restart > 200 || !(d.tol >= 0) || !(d.shift_factor >= 0) ||
      d.residual < GBS_RESID_AUTO || d.residual > GBS_RESID_OZAKI || d.pivoting < GBS_PIVOT_AUTO ||
      d.pivoting > GBS_PIVOT_PARTIAL) {
    gbs_set_last_message("invalid gbs_refine_options");
    return GBS_INVALID_ARGUMENT;
  }
  *m = d;
  return GBS_SUCCESS;
}

static void fill_info(gbs_refine_info* info, const MixedResult& r)
{
  if (!info) return;
  info->tier_used = r.tier;
  info->solver = r.solver;
  info->iterations = r.iterations;
  info->inner_iterations = r.inner_iterations;
  info->fell_back = r.fell_back;
  info->singular = r.singular;
  info->backward_error = r.backward_error;
  info->shift = r.shift;
}

static int check_dims(int n, int nrhs, int lda, int ldb, int ldx)
{
  if (n < 0 || nrhs < 0 || lda < std::max(1, n) || ldb < std::max(1, n) || ldx < std::max(1, n)) {
    gbs_set_last_message("mixed solver: invalid size or leading dimension");
    return GBS_INVALID_ARGUMENT;
  }
  return GBS_SUCCESS;
}

typedef int (*MixedFn)(cudaStream_t, int, int, const double*, int64_t, const double*, int64_t, double*, int64_t,
                       const MixedOptions&, MixedResult*);

static int run_device(MixedFn fn, int n, int nrhs, const double* d_a, int lda, const double* d_b, int ldb, double* d_x,
                      int ldx, const gbs_refine_options* opt, gbs_refine_info* info, void* stream)
{
  GBS_TRY(check_dims(n, nrhs, lda, ldb, ldx));
  MixedOptions o;
  GBS_TRY(to_options(opt, &o));
  GBS_TRY(ensure_device());
  WorkspaceLease lease;
  if (lease.status != GBS_SUCCESS) return lease.status;
  cudaStream_t s = (cudaStream_t)stream;     // NULL: the legacy default stream
  MixedResult r;
  const int rc = fn(s, n, nrhs, d_a, lda, d_b, ldb, d_x, ldx, o, &r);
  fill_info(info, r);
  return rc;
}

constexpr int kLowerCopyCols = 512;    // column blocks of the SPD solve's lower-triangle copy

static int run_host(MixedFn fn, int n, int nrhs, const double* a, int lda, const double* b, int ldb, double* x, int ldx,
                    const gbs_refine_options* opt, gbs_refine_info* info)
{
  GBS_TRY(check_dims(n, nrhs, lda, ldb, ldx));
  MixedOptions o;
  GBS_TRY(to_options(opt, &o));
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
  GBS_CUDA_TRY(cudaMemcpy2DAsync(dB, sizeof(double) * n, b, sizeof(double) * ldb, sizeof(double) * n, nrhs,
                                 cudaMemcpyHostToDevice, s));
  MixedResult r;
  int rc;
  if (fn == mixed_lu_solve) {     // A's copy overlaps the factorization
    rc = mixed_lu_solve_host(s, n, nrhs, a, lda, dA, dB, n, dX, n, o, &r);
  } else if (fn == mixed_llt_solve) {
    // the SPD solve reads A's lower triangle only (LLT.h:50-51, UpLo = Lower): copy the lower
    // trapezoid of each block of kLowerCopyCols columns, about half of A
    for (int c0 = 0; c0 < n; c0 += kLowerCopyCols) {
      const int nc = std::min(kLowerCopyCols, n - c0);
      GBS_CUDA_TRY(cudaMemcpy2DAsync(dA + (size_t)c0 * n + c0, sizeof(double) * n, a + (size_t)c0 * lda + c0,
                                     sizeof(double) * lda, sizeof(double) * (n - c0), nc, cudaMemcpyHostToDevice,
                                     s));
    }
    rc = fn(s, n, nrhs, dA, n, dB, n, dX, n, o, &r);
  } else {
    GBS_CUDA_TRY(cudaMemcpy2DAsync(dA, sizeof(double) * n, a, sizeof(double) * lda, sizeof(double) * n, n,
                                   cudaMemcpyHostToDevice, s));
    rc = fn(s, n, nrhs, dA, n, dB, n, dX, n, o, &r);
  }
  fill_info(info, r);
  if (rc != GBS_SUCCESS) return rc;
  GBS_CUDA_TRY(cudaMemcpy2DAsync(x, sizeof(double) * ldx, dX, sizeof(double) * n, sizeof(double) * n, nrhs,
                                 cudaMemcpyDeviceToHost, s));
  GBS_CUDA_TRY(cudaStreamSynchronize(s));
  return GBS_SUCCESS;
}

extern "C" int gbs_dgesv_mixed_device(int n, int nrhs, const double* d_a, int lda, const double* d_b, int ldb,
                                      double* d_x, int ldx, const gbs_refine_options* opt, gbs_refine_info* info,
                                      void* stream)
{
  return run_device(mixed_lu_solve, n, nrhs, d_a, lda, d_b, ldb, d_x, ldx, opt, info, stream);
}

extern "C" int gbs_dgesv_mixed(int n, int nrhs, const double* a, int lda, const double* b, int ldb, double* x, int ldx,
                               const gbs_refine_options* opt, gbs_refine_info* info)
{
  return run_host(mixed_lu_solve, n, nrhs, a, lda, b, ldb, x, ldx, opt, info);
}

extern "C" int gbs_dposv_mixed_device(int n, int nrhs, const double* d_a, int lda, const double* d_b, int ldb,
                                      double* d_x, int ldx, const gbs_refine_options* opt, gbs_refine_info* info,
                                      void* stream)
{
  return run_device(mixed_llt_solve, n, nrhs, d_a, lda, d_b, ldb, d_x, ldx, opt, info, stream);
}

extern "C" int gbs_dposv_mixed(int n, int nrhs, const double* a, int lda, const double* b, int ldb, double* x, int ldx,
                               const gbs_refine_options* opt, gbs_refine_info* info)
{
  return run_host(mixed_llt_solve, n, nrhs, a, lda, b, ldb, x, ldx, opt, info);
}

extern "C" int gbs_dgeresid_device(int n, int nrhs, const double* d_a, int lda, const double* d_x, int ldx,
                                   const double* d_b, int ldb, double* d_r, int ldr, int method, void* stream)
{
  const int ld_min = n > 1 ? n : 1;
  if (n < 0 || nrhs < 0 || lda < ld_min || ldx < ld_min || (d_b && ldb < ld_min) || ldr < ld_min ||
      method < GBS_RESID_AUTO || method > GBS_RESID_OZAKI) {
    gbs_set_last_message("gbs_dgeresid_device: invalid argument");
    return GBS_INVALID_ARGUMENT;
  }
  GBS_TRY(ensure_device());
  return residual_device((cudaStream_t)stream, n, nrhs, d_a, lda, d_x, ldx, d_b, ldb, d_r, ldr, method);
}

extern "C" int gbs_streamed_input_plan(int n, int cap, int* col, int* iter, int* rolling)
{
  if (cap < 0) return -(100 + GBS_INVALID_ARGUMENT);
  return streamed_input_plan(n, cap, col, iter, rolling);
}
