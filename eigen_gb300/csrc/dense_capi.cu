// C-ABI of the plain factor-and-solve path (include/gb300solve.h):
// decomposition objects, the Eigen plug-in level and the LAPACK level.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "dense_driver.cuh"
#include "gbs_profile.cuh"

using namespace gbs;

namespace {

inline size_t esize(int dtype) { return dtype == GBS_F64 ? sizeof(double) : sizeof(float); }

int upload_matrix(cudaStream_t s, const void* h, int64_t ldh, void* d, int64_t ldd, int64_t m, int64_t n, size_t es)
{
  if (m <= 0 || n <= 0) return GBS_SUCCESS;
  GBS_CUDA_TRY(cudaMemcpy2DAsync(d, ldd * es, h, ldh * es, m * es, n, cudaMemcpyHostToDevice, s));
  return GBS_SUCCESS;
}

int download_matrix(cudaStream_t s, const void* d, int64_t ldd, void* h, int64_t ldh, int64_t m, int64_t n, size_t es)
{
  if (m <= 0 || n <= 0) return GBS_SUCCESS;
  GBS_CUDA_TRY(cudaMemcpy2DAsync(h, ldh * es, d, ldd * es, m * es, n, cudaMemcpyDeviceToHost, s));
  return GBS_SUCCESS;
}

int sync(cudaStream_t s)
{
  GBS_CUDA_TRY(cudaStreamSynchronize(s));
  return GBS_SUCCESS;
}

int check_dims(int64_t n, int64_t lda)
{
  if (n < 0 || lda < std::max<int64_t>(1, n) || n > 0x7fffffff) {
    gbs_set_last_message("invalid size or leading dimension");
    return GBS_INVALID_ARGUMENT;
  }
  return GBS_SUCCESS;
}

}  // namespace

extern "C" int gbs_device_count(void)
{
  if (ensure_device() != GBS_SUCCESS) return 0;
  int c = 0;
  cudaGetDeviceCount(&c);
  int usable = 0;
  for (int d = 0; d < c; ++d) {
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, d) == cudaSuccess && p.major == 10 && p.minor == 3) ++usable;
  }
  return usable;
}

extern "C" double gbs_set_wait_limit(double seconds)
{
  const double prev = (double)wait_limit_ns() * 1e-9;
  set_wait_limit_ns(seconds > 0 ? (uint64_t)(seconds * 1e9 + 0.5) : 0);
  return prev;
}

namespace {

// Runs one diagnostic on a private stream that is destroyed afterwards.
template <typename F>
int on_private_stream(F&& f)
{
  GBS_TRY(ensure_device());
  cudaStream_t s;
  GBS_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  const int rc = f(s);
  cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  return rc;
}

}  // namespace

extern "C" int gbs_selftest_solve_timeout(int n)
{
  return on_private_stream([n](cudaStream_t s) { return tri_solve_timeout_selftest(s, n); });
}

extern "C" int gbs_selftest_barrier_timeout(void)
{
  return on_private_stream([](cudaStream_t s) { return barrier_timeout_selftest(s); });
}

// =================================================================== LLT object
struct gbs_llt {
  int dtype = GBS_F64;
  int uplo = GBS_LOWER;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int64_t n = 0;
  DevBuf A, st, tmp, vec, rhs, norm;
  HostBuf hvec;
  SolveWork sw;
  double l1 = 0;
  bool initialized = false;
  int info = GBS_NOT_INITIALIZED;
  int64_t failed_col = -1;
};

extern "C" int gbs_llt_create(gbs_llt** out, int dtype, int uplo)
{
  if (!out || (dtype != GBS_F64 && dtype != GBS_F32) || (uplo != GBS_LOWER && uplo != GBS_UPPER))
    return GBS_INVALID_ARGUMENT;
  *out = nullptr;
  GBS_TRY(ensure_device());
  gbs_llt* o = new gbs_llt();
  o->dtype = dtype;
  o->uplo = uplo;
  cudaError_t e = cudaStreamCreateWithFlags(&o->stream, cudaStreamDefault);
  if (e != cudaSuccess) {
    gbs_set_last_cuda_error(e, "cudaStreamCreate", __FILE__, __LINE__);
    delete o;
    return GBS_CUDA_ERROR;
  }
  o->own_stream = true;
  *out = o;
  return GBS_SUCCESS;
}

extern "C" int gbs_llt_destroy(gbs_llt* o)
{
  if (!o) return GBS_SUCCESS;
  if (o->stream) cudaStreamSynchronize(o->stream);
  if (o->own_stream && o->stream) cudaStreamDestroy(o->stream);
  delete o;
  return GBS_SUCCESS;
}

extern "C" int gbs_llt_set_stream(gbs_llt* o, void* stream)
{
  if (!o) return GBS_INVALID_ARGUMENT;
  if (o->own_stream && o->stream) {
    cudaStreamSynchronize(o->stream);
    cudaStreamDestroy(o->stream);
  }
  o->stream = (cudaStream_t)stream;
  o->own_stream = false;
  return GBS_SUCCESS;
}

static int llt_factor_current(gbs_llt* o)
{
  const int n = (int)o->n;
  cudaStream_t s = o->stream;
  GBS_TRY(reset_status(o->st.as<DeviceStatus>(), s));
  GBS_TRY(o->norm.reserve(sizeof(double)));
  const int up = o->uplo == GBS_UPPER;
  if (o->dtype == GBS_F64) {
    GBS_TRY(l1_norm_device<double>(s, o->A.as<double>(), n, n, n, 1, up, o->norm.as<double>(), &o->l1));
    GBS_TRY(potrf_device<double>(s, n, o->A.as<double>(), n, up, o->st.as<DeviceStatus>(), o->tmp));
  } else {
    GBS_TRY(l1_norm_device<float>(s, o->A.as<float>(), n, n, n, 1, up, o->norm.as<double>(), &o->l1));
    GBS_TRY(potrf_device<float>(s, n, o->A.as<float>(), n, up, o->st.as<DeviceStatus>(), o->tmp));
  }
  DeviceStatus h;
  int rc = read_status(o->st.as<DeviceStatus>(), &h, s);
  o->initialized = true;
  if (rc != GBS_SUCCESS) {
    o->info = rc;
    return rc;
  }
  o->failed_col = h.info;
  o->info = h.info >= 0 ? GBS_NUMERICAL_ISSUE : GBS_SUCCESS;
  return GBS_SUCCESS;
}

static int llt_prepare(gbs_llt* o, int64_t n)
{
  GBS_TRY(ensure_device());
  o->n = n;
  o->initialized = false;
  o->info = GBS_NOT_INITIALIZED;
  o->failed_col = -1;
  GBS_TRY(o->A.reserve(esize(o->dtype) * (size_t)std::max<int64_t>(n * n, 1)));
  GBS_TRY(o->st.reserve(sizeof(DeviceStatus)));
  return GBS_SUCCESS;
}

extern "C" int gbs_llt_compute(gbs_llt* o, int64_t n, const void* a, int64_t lda)
{
  if (!o || (n > 0 && !a)) return GBS_INVALID_ARGUMENT;
  GBS_TRY(check_dims(n, lda));
  GBS_TRY(llt_prepare(o, n));
  GBS_TRY(upload_matrix(o->stream, a, lda, o->A.p, n, n, n, esize(o->dtype)));
  return llt_factor_current(o);
}

extern "C" int gbs_llt_compute_device(gbs_llt* o, int64_t n, const void* d_a, int64_t lda)
{
  if (!o || (n > 0 && !d_a)) return GBS_INVALID_ARGUMENT;
  GBS_TRY(check_dims(n, lda));
  GBS_TRY(llt_prepare(o, n));
  if (n > 0)
    GBS_CUDA_TRY(cudaMemcpy2DAsync(o->A.p, n * esize(o->dtype), d_a, lda * esize(o->dtype), n * esize(o->dtype), n,
                                   cudaMemcpyDeviceToDevice, o->stream));
  return llt_factor_current(o);
}

extern "C" int gbs_llt_info(const gbs_llt* o)
{
  if (!o || !o->initialized) return GBS_NOT_INITIALIZED;
  return o->info;
}

extern "C" int64_t gbs_llt_failed_column(const gbs_llt* o) { return o ? o->failed_col : -1; }

static int llt_ready(const gbs_llt* o)
{
  if (!o || !o->initialized) {
    gbs_set_last_message("LLT is not initialized.");
    return GBS_NOT_INITIALIZED;
  }
  if (o->info != GBS_SUCCESS) {
    gbs_set_last_message("LLT failed because matrix appears to be negative");
    return GBS_NUMERICAL_ISSUE;
  }
  return GBS_SUCCESS;
}

static int llt_solve_inplace(gbs_llt* o, int nrhs, void* dX, int64_t ldx)
{
  const int n = (int)o->n;
  const int up = o->uplo == GBS_UPPER;
  if (o->dtype == GBS_F64)
    return llt_solve_device<double>(o->stream, n, nrhs, o->A.as<double>(), n, up, (double*)dX, ldx, o->sw);
  return llt_solve_device<float>(o->stream, n, nrhs, o->A.as<float>(), n, up, (float*)dX, ldx, o->sw);
}

extern "C" int gbs_llt_solve(gbs_llt* o, int64_t nrhs, const void* b, int64_t ldb, void* x, int64_t ldx)
{
  GBS_TRY(llt_ready(o));
  const int64_t n = o->n;
  if (nrhs < 0 || ldb < std::max<int64_t>(1, n) || ldx < std::max<int64_t>(1, n)) return GBS_INVALID_ARGUMENT;
  if (n == 0 || nrhs == 0) return GBS_SUCCESS;
  const size_t es = esize(o->dtype);
  GBS_TRY(o->rhs.reserve(es * (size_t)n * nrhs));
  GBS_TRY(upload_matrix(o->stream, b, ldb, o->rhs.p, n, n, nrhs, es));
  GBS_TRY(llt_solve_inplace(o, (int)nrhs, o->rhs.p, n));
  GBS_TRY(solve_status(o->stream, o->sw));
  GBS_TRY(download_matrix(o->stream, o->rhs.p, n, x, ldx, n, nrhs, es));
  return sync(o->stream);
}

extern "C" int gbs_llt_solve_device(gbs_llt* o, int64_t nrhs, const void* d_b, int64_t ldb, void* d_x, int64_t ldx)
{
  GBS_TRY(llt_ready(o));
  const int64_t n = o->n;
  if (nrhs < 0 || ldb < std::max<int64_t>(1, n) || ldx < std::max<int64_t>(1, n)) return GBS_INVALID_ARGUMENT;
  if (n == 0 || nrhs == 0) return GBS_SUCCESS;
  const size_t es = esize(o->dtype);
  if (d_x != d_b)
    GBS_CUDA_TRY(cudaMemcpy2DAsync(d_x, ldx * es, d_b, ldb * es, n * es, nrhs, cudaMemcpyDeviceToDevice, o->stream));
  return llt_solve_inplace(o, (int)nrhs, d_x, ldx);
}

extern "C" int gbs_llt_rcond(gbs_llt* o, double* rcond)
{
  GBS_TRY(llt_ready(o));
  if (!rcond) return GBS_INVALID_ARGUMENT;
  const int n = (int)o->n;
  const int kind = o->uplo == GBS_UPPER ? 2 : 1;
  const bool single = o->dtype == GBS_F32;
  if (n == 0 || o->l1 == 0.0 || n == 1) {
    *rcond = rcond_from_estimate(n, o->l1, 1.0, single);
    return GBS_SUCCESS;
  }
  double est = 0;
  if (o->dtype == GBS_F64)
    GBS_TRY(inv_l1_estimate_device<double>(o->stream, kind, n, o->A.as<double>(), n, nullptr, o->vec, o->hvec, o->sw, &est));
  else
    GBS_TRY(inv_l1_estimate_device<float>(o->stream, kind, n, o->A.as<float>(), n, nullptr, o->vec, o->hvec, o->sw, &est));
  *rcond = rcond_from_estimate(n, o->l1, est, single);
  return GBS_SUCCESS;
}

extern "C" int gbs_llt_l1_norm(const gbs_llt* o, double* l1)
{
  if (!o || !o->initialized || !l1) return GBS_NOT_INITIALIZED;
  *l1 = o->l1;
  return GBS_SUCCESS;
}

extern "C" int gbs_llt_matrix(gbs_llt* o, void* out, int64_t ld)
{
  if (!o || !o->initialized) return GBS_NOT_INITIALIZED;
  if (ld < std::max<int64_t>(1, o->n)) return GBS_INVALID_ARGUMENT;
  GBS_TRY(download_matrix(o->stream, o->A.p, o->n, out, ld, o->n, o->n, esize(o->dtype)));
  return sync(o->stream);
}

extern "C" void* gbs_llt_device_matrix(gbs_llt* o, int64_t* ld)
{
  if (!o || !o->initialized) return nullptr;
  if (ld) *ld = o->n;
  return o->A.p;
}

// LLT::rankUpdate (LLT.h:461-472): info() becomes NumericalIssue when a
// downdate would make the matrix indefinite (the factor is then left as the
// reference leaves it, updated up to the failing column), else Success.  The
// stored ||A||_1 is not changed, as in the reference.
static int llt_rank_update_common(gbs_llt* o, const void* d_v, double sigma)
{
  int failed = -1;
  const int up = o->uplo == GBS_UPPER;
  const int n = (int)o->n;
  if (o->dtype == GBS_F64)
    GBS_TRY(llt_rank_update_device<double>(o->stream, n, o->A.as<double>(), n, up, (const double*)d_v, sigma, o->tmp,
                                           &failed));
  else
    GBS_TRY(llt_rank_update_device<float>(o->stream, n, o->A.as<float>(), n, up, (const float*)d_v, sigma, o->tmp,
                                          &failed));
  o->failed_col = failed;
  o->info = failed >= 0 ? GBS_NUMERICAL_ISSUE : GBS_SUCCESS;
  return GBS_SUCCESS;
}

extern "C" int gbs_llt_rank_update(gbs_llt* o, const void* v, double sigma)
{
  if (!o || !o->initialized) return GBS_NOT_INITIALIZED;
  if (o->n > 0 && !v) return GBS_INVALID_ARGUMENT;
  const size_t es = esize(o->dtype);
  GBS_TRY(o->rhs.reserve(es * (size_t)std::max<int64_t>(o->n, 1)));
  if (o->n > 0) GBS_CUDA_TRY(cudaMemcpyAsync(o->rhs.p, v, es * o->n, cudaMemcpyHostToDevice, o->stream));
  return llt_rank_update_common(o, o->rhs.p, sigma);
}

extern "C" int gbs_llt_rank_update_device(gbs_llt* o, const void* d_v, double sigma)
{
  if (!o || !o->initialized) return GBS_NOT_INITIALIZED;
  if (o->n > 0 && !d_v) return GBS_INVALID_ARGUMENT;
  return llt_rank_update_common(o, d_v, sigma);
}

extern "C" int gbs_llt_synchronize(gbs_llt* o)
{
  if (!o) return GBS_INVALID_ARGUMENT;
  return solve_status(o->stream, o->sw);
}

// =================================================================== LU object
struct gbs_lu {
  int dtype = GBS_F64;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int64_t n = 0;
  DevBuf A, tr, st, scratch, vec, rhs, norm;
  HostBuf hvec;
  SolveWork sw;
  double l1 = 0;
  bool initialized = false;
  int64_t first_zero = -1;
  int nbt = 0;
};

extern "C" int gbs_lu_create(gbs_lu** out, int dtype)
{
  if (!out || (dtype != GBS_F64 && dtype != GBS_F32)) return GBS_INVALID_ARGUMENT;
  *out = nullptr;
  GBS_TRY(ensure_device());
  gbs_lu* o = new gbs_lu();
  o->dtype = dtype;
  cudaError_t e = cudaStreamCreateWithFlags(&o->stream, cudaStreamDefault);
  if (e != cudaSuccess) {
    gbs_set_last_cuda_error(e, "cudaStreamCreate", __FILE__, __LINE__);
    delete o;
    return GBS_CUDA_ERROR;
  }
  o->own_stream = true;
  *out = o;
  return GBS_SUCCESS;
}

extern "C" int gbs_lu_destroy(gbs_lu* o)
{
  if (!o) return GBS_SUCCESS;
  if (o->stream) cudaStreamSynchronize(o->stream);
  if (o->own_stream && o->stream) cudaStreamDestroy(o->stream);
  delete o;
  return GBS_SUCCESS;
}

extern "C" int gbs_lu_set_stream(gbs_lu* o, void* stream)
{
  if (!o) return GBS_INVALID_ARGUMENT;
  if (o->own_stream && o->stream) {
    cudaStreamSynchronize(o->stream);
    cudaStreamDestroy(o->stream);
  }
  o->stream = (cudaStream_t)stream;
  o->own_stream = false;
  return GBS_SUCCESS;
}

static int lu_prepare(gbs_lu* o, int64_t n)
{
  GBS_TRY(ensure_device());
  o->n = n;
  o->initialized = false;
  o->first_zero = -1;
  o->nbt = 0;
  GBS_TRY(o->A.reserve(esize(o->dtype) * (size_t)std::max<int64_t>(n * n, 1)));
  GBS_TRY(o->tr.reserve(sizeof(int) * (size_t)std::max<int64_t>(n, 1)));
  GBS_TRY(o->st.reserve(sizeof(DeviceStatus)));
  GBS_TRY(o->norm.reserve(sizeof(double)));
  return GBS_SUCCESS;
}

static int lu_factor_current(gbs_lu* o)
{
  const int n = (int)o->n;
  cudaStream_t s = o->stream;
  GBS_TRY(reset_status(o->st.as<DeviceStatus>(), s));
  if (o->dtype == GBS_F64) {
    GBS_TRY(l1_norm_device<double>(s, o->A.as<double>(), n, n, n, 0, 0, o->norm.as<double>(), &o->l1));
    GBS_TRY(getrf_device<double>(s, n, n, o->A.as<double>(), n, o->tr.as<int>(), o->st.as<DeviceStatus>(),
                                 o->scratch));
  } else {
    GBS_TRY(l1_norm_device<float>(s, o->A.as<float>(), n, n, n, 0, 0, o->norm.as<double>(), &o->l1));
    GBS_TRY(getrf_device<float>(s, n, n, o->A.as<float>(), n, o->tr.as<int>(), o->st.as<DeviceStatus>(),
                                o->scratch));
  }
  DeviceStatus h;
  GBS_TRY(read_status(o->st.as<DeviceStatus>(), &h, s));
  o->first_zero = h.info;
  o->nbt = h.nb_transpositions;
  o->initialized = true;
  return GBS_SUCCESS;
}

extern "C" int gbs_lu_compute(gbs_lu* o, int64_t n, const void* a, int64_t lda)
{
  if (!o || (n > 0 && !a)) return GBS_INVALID_ARGUMENT;
  GBS_TRY(check_dims(n, lda));
  GBS_TRY(lu_prepare(o, n));
  GBS_TRY(upload_matrix(o->stream, a, lda, o->A.p, n, n, n, esize(o->dtype)));
  return lu_factor_current(o);
}

extern "C" int gbs_lu_compute_device(gbs_lu* o, int64_t n, const void* d_a, int64_t lda)
{
  if (!o || (n > 0 && !d_a)) return GBS_INVALID_ARGUMENT;
  GBS_TRY(check_dims(n, lda));
  GBS_TRY(lu_prepare(o, n));
  if (n > 0)
    GBS_CUDA_TRY(cudaMemcpy2DAsync(o->A.p, n * esize(o->dtype), d_a, lda * esize(o->dtype), n * esize(o->dtype), n,
                                   cudaMemcpyDeviceToDevice, o->stream));
  return lu_factor_current(o);
}

static int lu_ready(const gbs_lu* o)
{
  if (!o || !o->initialized) {
    gbs_set_last_message("PartialPivLU is not initialized.");
    return GBS_NOT_INITIALIZED;
  }
  return GBS_SUCCESS;
}

extern "C" int64_t gbs_lu_first_zero_pivot(const gbs_lu* o) { return o ? o->first_zero : -1; }
extern "C" int gbs_lu_nb_transpositions(const gbs_lu* o) { return o ? o->nbt : 0; }

static int lu_solve_inplace(gbs_lu* o, int nrhs, void* dX, int64_t ldx, int transpose)
{
  const int n = (int)o->n;
  if (o->dtype == GBS_F64)
    return lu_solve_device<double>(o->stream, n, nrhs, o->A.as<double>(), n, o->tr.as<int>(), (double*)dX, ldx,
                                   transpose, o->sw);
  return lu_solve_device<float>(o->stream, n, nrhs, o->A.as<float>(), n, o->tr.as<int>(), (float*)dX, ldx, transpose, o->sw);
}

extern "C" int gbs_lu_solve(gbs_lu* o, int64_t nrhs, const void* b, int64_t ldb, void* x, int64_t ldx, int transpose)
{
  GBS_TRY(lu_ready(o));
  const int64_t n = o->n;
  if (nrhs < 0 || ldb < std::max<int64_t>(1, n) || ldx < std::max<int64_t>(1, n)) return GBS_INVALID_ARGUMENT;
  if (n == 0 || nrhs == 0) return GBS_SUCCESS;
  const size_t es = esize(o->dtype);
  GBS_TRY(o->rhs.reserve(es * (size_t)n * nrhs));
  GBS_TRY(upload_matrix(o->stream, b, ldb, o->rhs.p, n, n, nrhs, es));
  GBS_TRY(lu_solve_inplace(o, (int)nrhs, o->rhs.p, n, transpose));
  GBS_TRY(solve_status(o->stream, o->sw));
  GBS_TRY(download_matrix(o->stream, o->rhs.p, n, x, ldx, n, nrhs, es));
  return sync(o->stream);
}

extern "C" int gbs_lu_solve_device(gbs_lu* o, int64_t nrhs, const void* d_b, int64_t ldb, void* d_x, int64_t ldx,
                                   int transpose)
{
  GBS_TRY(lu_ready(o));
  const int64_t n = o->n;
  if (nrhs < 0 || ldb < std::max<int64_t>(1, n) || ldx < std::max<int64_t>(1, n)) return GBS_INVALID_ARGUMENT;
  if (n == 0 || nrhs == 0) return GBS_SUCCESS;
  const size_t es = esize(o->dtype);
  if (d_x != d_b)
    GBS_CUDA_TRY(cudaMemcpy2DAsync(d_x, ldx * es, d_b, ldb * es, n * es, nrhs, cudaMemcpyDeviceToDevice, o->stream));
  return lu_solve_inplace(o, (int)nrhs, d_x, ldx, transpose);
}

template <typename T>
__global__ void identity_kernel(T* x, int64_t ld, int64_t n)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * n) return;
  const int64_t r = t % n, c = t / n;
  x[c * ld + r] = r == c ? T(1) : T(0);
}

// A^-1 = solve(I) (PartialPivLU.h:197-201): the identity solved in place at d_x
static int lu_inverse_into(gbs_lu* o, void* d_x, int64_t ldx)
{
  const int64_t n = o->n;
  count_launch();
  const int grid = (int)std::min<int64_t>((n * n + 255) / 256, 1 << 30);
  if (o->dtype == GBS_F64) identity_kernel<double><<<grid, 256, 0, o->stream>>>((double*)d_x, ldx, n);
  else identity_kernel<float><<<grid, 256, 0, o->stream>>>((float*)d_x, ldx, n);
  GBS_CUDA_TRY(cudaGetLastError());
  return lu_solve_inplace(o, (int)n, d_x, ldx, 0);
}

extern "C" int gbs_lu_inverse(gbs_lu* o, void* x, int64_t ldx)
{
  GBS_TRY(lu_ready(o));
  const int64_t n = o->n;
  if (!x && n > 0) return GBS_INVALID_ARGUMENT;
  if (ldx < std::max<int64_t>(1, n)) return GBS_INVALID_ARGUMENT;
  if (n == 0) return GBS_SUCCESS;
  const size_t es = esize(o->dtype);
  GBS_TRY(o->rhs.reserve(es * (size_t)n * n));
  GBS_TRY(lu_inverse_into(o, o->rhs.p, n));
  GBS_TRY(solve_status(o->stream, o->sw));
  GBS_TRY(download_matrix(o->stream, o->rhs.p, n, x, ldx, n, n, es));
  return sync(o->stream);
}

extern "C" int gbs_lu_inverse_device(gbs_lu* o, void* d_x, int64_t ldx)
{
  GBS_TRY(lu_ready(o));
  const int64_t n = o->n;
  if (!d_x && n > 0) return GBS_INVALID_ARGUMENT;
  if (ldx < std::max<int64_t>(1, n)) return GBS_INVALID_ARGUMENT;
  if (n == 0) return GBS_SUCCESS;
  return lu_inverse_into(o, d_x, ldx);
}

extern "C" int gbs_lu_rcond(gbs_lu* o, double* rcond)
{
  GBS_TRY(lu_ready(o));
  if (!rcond) return GBS_INVALID_ARGUMENT;
  const int n = (int)o->n;
  const bool single = o->dtype == GBS_F32;
  if (n == 0 || o->l1 == 0.0 || n == 1) {
    *rcond = rcond_from_estimate(n, o->l1, 1.0, single);
    return GBS_SUCCESS;
  }
  double est = 0;
  if (o->dtype == GBS_F64)
    GBS_TRY(inv_l1_estimate_device<double>(o->stream, 0, n, o->A.as<double>(), n, o->tr.as<int>(), o->vec, o->hvec,
                                           o->sw, &est));
  else
    GBS_TRY(inv_l1_estimate_device<float>(o->stream, 0, n, o->A.as<float>(), n, o->tr.as<int>(), o->vec, o->hvec,
                                          o->sw, &est));
  *rcond = rcond_from_estimate(n, o->l1, est, single);
  return GBS_SUCCESS;
}

extern "C" int gbs_lu_l1_norm(const gbs_lu* o, double* l1)
{
  if (!o || !o->initialized || !l1) return GBS_NOT_INITIALIZED;
  *l1 = o->l1;
  return GBS_SUCCESS;
}

extern "C" int gbs_lu_matrix(gbs_lu* o, void* out, int64_t ld)
{
  GBS_TRY(lu_ready(o));
  if (ld < std::max<int64_t>(1, o->n)) return GBS_INVALID_ARGUMENT;
  GBS_TRY(download_matrix(o->stream, o->A.p, o->n, out, ld, o->n, o->n, esize(o->dtype)));
  return sync(o->stream);
}

extern "C" int gbs_lu_transpositions(gbs_lu* o, int* out)
{
  GBS_TRY(lu_ready(o));
  if (o->n == 0) return GBS_SUCCESS;
  GBS_CUDA_TRY(cudaMemcpyAsync(out, o->tr.p, sizeof(int) * o->n, cudaMemcpyDeviceToHost, o->stream));
  return sync(o->stream);
}

// permutationP().indices(): identity, then for k = n-1 .. 0 swap(idx[k], idx[t[k]])
// (PermutationMatrix.h:82-88).
extern "C" int gbs_lu_permutation(gbs_lu* o, int* out)
{
  GBS_TRY(lu_ready(o));
  const int64_t n = o->n;
  if (n == 0) return GBS_SUCCESS;
  std::vector<int> t((size_t)n);
  GBS_TRY(gbs_lu_transpositions(o, t.data()));
  for (int64_t i = 0; i < n; ++i) out[i] = (int)i;
  for (int64_t k = n - 1; k >= 0; --k) std::swap(out[k], out[t[(size_t)k]]);
  return GBS_SUCCESS;
}

// determinant = (-1)^{nb_transpositions} * prod(diag(U)) (PartialPivLU.h:531,539-543)
extern "C" int gbs_lu_determinant(gbs_lu* o, double* det)
{
  GBS_TRY(lu_ready(o));
  const int64_t n = o->n;
  const size_t es = esize(o->dtype);
  std::vector<double> dd((size_t)std::max<int64_t>(n, 1));
  std::vector<float> df((size_t)std::max<int64_t>(n, 1));
  if (n > 0) {
    void* dst = o->dtype == GBS_F64 ? (void*)dd.data() : (void*)df.data();
    GBS_CUDA_TRY(cudaMemcpy2DAsync(dst, es, o->A.p, (n + 1) * es, es, n, cudaMemcpyDeviceToHost, o->stream));
    GBS_TRY(sync(o->stream));
  }
  if (o->dtype == GBS_F64) {
    double p = (o->nbt % 2) ? -1.0 : 1.0;
    for (int64_t i = 0; i < n; ++i) p *= dd[(size_t)i];
    *det = p;
  } else {
    float p = (o->nbt % 2) ? -1.0f : 1.0f;
    for (int64_t i = 0; i < n; ++i) p *= df[(size_t)i];
    *det = p;
  }
  return GBS_SUCCESS;
}

extern "C" void* gbs_lu_device_matrix(gbs_lu* o, int64_t* ld)
{
  if (!o || !o->initialized) return nullptr;
  if (ld) *ld = o->n;
  return o->A.p;
}

extern "C" int gbs_lu_synchronize(gbs_lu* o)
{
  if (!o) return GBS_INVALID_ARGUMENT;
  return solve_status(o->stream, o->sw);
}

// =================================================================== plug-in level
template <typename T>
static int64_t partial_lu_blocked(int64_t rows, int64_t cols, T* a, int64_t lda, int* tr, int* nbt)
{
  if (rows < 0 || cols < 0 || lda < std::max<int64_t>(1, rows) || rows > 0x7fffffff || cols > 0x7fffffff)
    return -(100 + GBS_INVALID_ARGUMENT);
  if (nbt) *nbt = 0;
  const int64_t size = std::min(rows, cols);
  if (size == 0) return -1;
  WorkspaceLease lease;
  if (lease.status != GBS_SUCCESS) return -(100 + lease.status);
  Workspace& w = *lease.ws;
  cudaStream_t s = w.stream;
  int rc;
  if ((rc = w.a.reserve(sizeof(T) * (size_t)rows * cols)) != GBS_SUCCESS) return -(100 + rc);
  if ((rc = w.piv.reserve(sizeof(int) * (size_t)size)) != GBS_SUCCESS) return -(100 + rc);
  if ((rc = w.status.reserve(sizeof(DeviceStatus))) != GBS_SUCCESS) return -(100 + rc);
  if ((rc = upload_matrix(s, a, lda, w.a.p, rows, rows, cols, sizeof(T))) != GBS_SUCCESS) return -(100 + rc);
  if ((rc = reset_status(w.status.as<DeviceStatus>(), s)) != GBS_SUCCESS) return -(100 + rc);
  if ((rc = getrf_device<T>(s, (int)rows, (int)cols, w.a.as<T>(), rows, w.piv.as<int>(), w.status.as<DeviceStatus>(),
                            w.scratch)) != GBS_SUCCESS)
    return -(100 + rc);
  DeviceStatus h;
  if ((rc = read_status(w.status.as<DeviceStatus>(), &h, s)) != GBS_SUCCESS) return -(100 + rc);
  if ((rc = download_matrix(s, w.a.p, rows, a, lda, rows, cols, sizeof(T))) != GBS_SUCCESS) return -(100 + rc);
  cudaError_t e = cudaMemcpyAsync(tr, w.piv.p, sizeof(int) * size, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    gbs_set_last_cuda_error(e, "download pivots", __FILE__, __LINE__);
    return -(100 + GBS_CUDA_ERROR);
  }
  if (nbt) *nbt = h.nb_transpositions;
  return h.info;
}

extern "C" int64_t gbs_partial_lu_blocked_d(int64_t rows, int64_t cols, double* a, int64_t lda, int* tr, int* nbt)
{
  return partial_lu_blocked<double>(rows, cols, a, lda, tr, nbt);
}

extern "C" int64_t gbs_partial_lu_blocked_s(int64_t rows, int64_t cols, float* a, int64_t lda, int* tr, int* nbt)
{
  return partial_lu_blocked<float>(rows, cols, a, lda, tr, nbt);
}

template <typename T>
static int64_t llt_blocked(int64_t n, T* a, int64_t lda, int upper)
{
  if (n < 0 || lda < std::max<int64_t>(1, n) || n > 0x7fffffff) return -(100 + GBS_INVALID_ARGUMENT);
  if (n == 0) return -1;
  WorkspaceLease lease;
  if (lease.status != GBS_SUCCESS) return -(100 + lease.status);
  Workspace& w = *lease.ws;
  cudaStream_t s = w.stream;
  int rc;
  if ((rc = w.a.reserve(sizeof(T) * (size_t)n * n)) != GBS_SUCCESS) return -(100 + rc);
  if ((rc = w.status.reserve(sizeof(DeviceStatus))) != GBS_SUCCESS) return -(100 + rc);
  if ((rc = upload_matrix(s, a, lda, w.a.p, n, n, n, sizeof(T))) != GBS_SUCCESS) return -(100 + rc);
  if ((rc = reset_status(w.status.as<DeviceStatus>(), s)) != GBS_SUCCESS) return -(100 + rc);
  if ((rc = potrf_device<T>(s, (int)n, w.a.as<T>(), n, upper, w.status.as<DeviceStatus>(), w.scratch)) != GBS_SUCCESS)
    return -(100 + rc);
  DeviceStatus h;
  if ((rc = read_status(w.status.as<DeviceStatus>(), &h, s)) != GBS_SUCCESS) return -(100 + rc);
  if ((rc = download_matrix(s, w.a.p, n, a, lda, n, n, sizeof(T))) != GBS_SUCCESS) return -(100 + rc);
  if ((rc = sync(s)) != GBS_SUCCESS) return -(100 + rc);
  return h.info;
}

extern "C" int64_t gbs_llt_blocked_d(int64_t n, double* a, int64_t lda, int upper)
{
  return llt_blocked<double>(n, a, lda, upper);
}

extern "C" int64_t gbs_llt_blocked_s(int64_t n, float* a, int64_t lda, int upper)
{
  return llt_blocked<float>(n, a, lda, upper);
}

// =================================================================== LAPACK level
// Argument checks and info codes of lapack/lu.cpp:14-89 and lapack/cholesky.cpp:14-72.
template <typename T>
static int getrf_impl(const int* m, const int* n, T* a, const int* lda, int* ipiv, int* info)
{
  *info = 0;
  if (*m < 0) *info = -1;
  else if (*n < 0) *info = -2;
  else if (*lda < std::max(1, *m)) *info = -4;
  if (*info != 0) return 0;
  if (*m == 0 || *n == 0) return 0;
  int nbt = 0;
  int64_t ret = partial_lu_blocked<T>(*m, *n, a, *lda, ipiv, &nbt);
  if (ret < -1) return (int)(-ret - 100);
  for (int i = 0; i < std::min(*m, *n); ++i) ipiv[i]++;
  if (ret >= 0) *info = (int)ret + 1;
  return 0;
}

extern "C" int gbs_dgetrf(const int* m, const int* n, double* a, const int* lda, int* ipiv, int* info)
{
  return getrf_impl<double>(m, n, a, lda, ipiv, info);
}

extern "C" int gbs_sgetrf(const int* m, const int* n, float* a, const int* lda, int* ipiv, int* info)
{
  return getrf_impl<float>(m, n, a, lda, ipiv, info);
}

static int trans_op(char c)
{
  if (c == 'N' || c == 'n') return 0;
  if (c == 'T' || c == 't' || c == 'C' || c == 'c') return 1;   // real scalars: adjoint == transpose
  return -1;
}

template <typename T>
static int getrs_impl(const char* trans, const int* n, const int* nrhs, const T* a, const int* lda, const int* ipiv,
                      T* b, const int* ldb, int* info)
{
  *info = 0;
  const int op = trans_op(*trans);
  if (op < 0) *info = -1;
  else if (*n < 0) *info = -2;
  else if (*nrhs < 0) *info = -3;
  else if (*lda < std::max(1, *n)) *info = -5;
  else if (*ldb < std::max(1, *n)) *info = -8;
  if (*info != 0) return 0;
  if (*n == 0 || *nrhs == 0) return 0;
  WorkspaceLease lease;
  if (lease.status != GBS_SUCCESS) return lease.status;
  Workspace& w = *lease.ws;
  cudaStream_t s = w.stream;
  const int N = *n, R = *nrhs;
  GBS_TRY(w.a.reserve(sizeof(T) * (size_t)N * N));
  GBS_TRY(w.b.reserve(sizeof(T) * (size_t)N * R));
  GBS_TRY(w.piv.reserve(sizeof(int) * (size_t)N));
  std::vector<int> tr((size_t)N);
  for (int i = 0; i < N; ++i) tr[(size_t)i] = ipiv[i] - 1;
  GBS_TRY(upload_matrix(s, a, *lda, w.a.p, N, N, N, sizeof(T)));
  GBS_TRY(upload_matrix(s, b, *ldb, w.b.p, N, N, R, sizeof(T)));
  GBS_CUDA_TRY(cudaMemcpyAsync(w.piv.p, tr.data(), sizeof(int) * N, cudaMemcpyHostToDevice, s));
  GBS_TRY(lu_solve_device<T>(s, N, R, w.a.as<T>(), N, w.piv.as<int>(), w.b.as<T>(), N, op, w.sw));
  GBS_TRY(solve_status(s, w.sw));
  GBS_TRY(download_matrix(s, w.b.p, N, b, *ldb, N, R, sizeof(T)));
  return sync(s);
}

extern "C" int gbs_dgetrs(const char* trans, const int* n, const int* nrhs, const double* a, const int* lda,
                          const int* ipiv, double* b, const int* ldb, int* info)
{
  return getrs_impl<double>(trans, n, nrhs, a, lda, ipiv, b, ldb, info);
}

extern "C" int gbs_sgetrs(const char* trans, const int* n, const int* nrhs, const float* a, const int* lda,
                          const int* ipiv, float* b, const int* ldb, int* info)
{
  return getrs_impl<float>(trans, n, nrhs, a, lda, ipiv, b, ldb, info);
}

static int uplo_op(char c)
{
  if (c == 'U' || c == 'u') return 1;
  if (c == 'L' || c == 'l') return 0;
  return -1;
}

template <typename T>
static int potrf_impl(const char* uplo, const int* n, T* a, const int* lda, int* info)
{
  *info = 0;
  const int up = uplo_op(*uplo);
  if (up < 0) *info = -1;
  else if (*n < 0) *info = -2;
  else if (*lda < std::max(1, *n)) *info = -4;
  if (*info != 0) return 0;
  int64_t ret = llt_blocked<T>(*n, a, *lda, up);
  if (ret < -1) return (int)(-ret - 100);
  if (ret >= 0) *info = (int)ret + 1;
  return 0;
}

extern "C" int gbs_dpotrf(const char* uplo, const int* n, double* a, const int* lda, int* info)
{
  return potrf_impl<double>(uplo, n, a, lda, info);
}

extern "C" int gbs_spotrf(const char* uplo, const int* n, float* a, const int* lda, int* info)
{
  return potrf_impl<float>(uplo, n, a, lda, info);
}

template <typename T>
static int potrs_impl(const char* uplo, const int* n, const int* nrhs, const T* a, const int* lda, T* b,
                      const int* ldb, int* info)
{
  *info = 0;
  const int up = uplo_op(*uplo);
  if (up < 0) *info = -1;
  else if (*n < 0) *info = -2;
  else if (*nrhs < 0) *info = -3;
  else if (*lda < std::max(1, *n)) *info = -5;
  else if (*ldb < std::max(1, *n)) *info = -7;
  if (*info != 0) return 0;
  if (*n == 0 || *nrhs == 0) return 0;
  WorkspaceLease lease;
  if (lease.status != GBS_SUCCESS) return lease.status;
  Workspace& w = *lease.ws;
  cudaStream_t s = w.stream;
  const int N = *n, R = *nrhs;
  GBS_TRY(w.a.reserve(sizeof(T) * (size_t)N * N));
  GBS_TRY(w.b.reserve(sizeof(T) * (size_t)N * R));
  GBS_TRY(upload_matrix(s, a, *lda, w.a.p, N, N, N, sizeof(T)));
  GBS_TRY(upload_matrix(s, b, *ldb, w.b.p, N, N, R, sizeof(T)));
  GBS_TRY(llt_solve_device<T>(s, N, R, w.a.as<T>(), N, up, w.b.as<T>(), N, w.sw));
  GBS_TRY(solve_status(s, w.sw));
  GBS_TRY(download_matrix(s, w.b.p, N, b, *ldb, N, R, sizeof(T)));
  return sync(s);
}

extern "C" int gbs_dpotrs(const char* uplo, const int* n, const int* nrhs, const double* a, const int* lda, double* b,
                          const int* ldb, int* info)
{
  return potrs_impl<double>(uplo, n, nrhs, a, lda, b, ldb, info);
}

extern "C" int gbs_spotrs(const char* uplo, const int* n, const int* nrhs, const float* a, const int* lda, float* b,
                          const int* ldb, int* info)
{
  return potrs_impl<float>(uplo, n, nrhs, a, lda, b, ldb, info);
}
