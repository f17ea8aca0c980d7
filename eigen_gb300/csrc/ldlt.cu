// LDLT: Eigen's Cholesky with diagonal pivoting, A = P^T L D L^T P
// (Eigen/src/Cholesky/LDLT.h), on the GPU, and its gbs_ldlt_* C ABI.
//
// The reference's pivot at step k is the first maximum of |a_ii| over the
// positions i >= k of the diagonal as permuted so far (LDLT.h:305-317).  Its
// left-looking algorithm updates a_kk only at step k, so every pivot choice
// reads an input diagonal value: the whole transposition sequence is a
// function of the input's diagonal.  It is replayed exactly on the host (a
// segment tree over positions, O(n log n)), and the factorization then runs
// without pivot searches on the symmetrically permuted matrix P A P^T:
//   * one CTA factors each 32 x 32 diagonal block in shared memory;
//   * a panel kernel forms Z = A21 L11^-T and L21 = Z D1^-1 (one row per thread);
//   * the trailing update A22 -= Z L21^T is the lower-triangle DFMA/FFMA GEMM
//     of the plain path.
// A zero (or NaN) pivot leaves its column unscaled and contributes nothing to
// later columns, as in the reference (LDLT.h:354-360).  info and the sign
// follow the reference's step-by-step rules, evaluated on the host from D and
// one "column below is zero" flag per zero pivot.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

#include "dense_driver.cuh"
#include "gbs_profile.cuh"

namespace gbs {

namespace {

constexpr int kLdltNB = 32;      // block width of the factorization

inline int cdiv(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

// W(i, j) = A(perm[i], perm[j]) for i >= j, read from the used triangle of A
// (upper: A(min, max)); W column-major, ld n.
template <typename T>
__global__ void ldlt_permute_kernel(const T* __restrict__ A, int64_t lda, int n, int upper,
                                    const int* __restrict__ perm, T* __restrict__ W)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int pi = perm[i];
  for (int j = blockIdx.y; j <= i; j += gridDim.y) {
    const int pj = perm[j];
    const int r = pi > pj ? pi : pj, c = pi > pj ? pj : pi;
    W[(int64_t)j * n + i] = upper ? A[(int64_t)r * lda + c] : A[(int64_t)c * lda + r];
  }
}

// LDL^T of one b x b diagonal block (b <= kLdltNB) in shared memory,
// right-looking: for each column j, l = a / d and z = a (or z = a d when the
// pivot d is zero or NaN: no scaling, and no contribution to later columns),
// then a(i, k) -= z_i l_k for j < k <= i.
template <typename T>
__global__ void __launch_bounds__(256) ldlt_diag_kernel(T* __restrict__ W, int64_t ld, int b)
{
  __shared__ T a[kLdltNB][kLdltNB + 1];   // a[col][row]
  __shared__ T lcol[kLdltNB], zcol[kLdltNB];
  const int tid = threadIdx.x;
  for (int e = tid; e < b * b; e += blockDim.x) {
    const int r = e % b, c = e / b;
    if (r >= c) a[c][r] = W[(int64_t)c * ld + r];
  }
  __syncthreads();
  for (int j = 0; j < b; ++j) {
    const T d = a[j][j];
    const bool valid = fabs((double)d) > 0.0;
    for (int i = j + 1 + tid; i < b; i += blockDim.x) {
      const T x = a[j][i];
      lcol[i] = valid ? x / d : x;
      zcol[i] = valid ? x : x * d;
    }
    __syncthreads();
    const int t = b - 1 - j;
    for (int e = tid; e < t * t; e += blockDim.x) {
      const int kk = e / t, ii = e % t;
      if (ii < kk) continue;
      const int i = j + 1 + ii, k = j + 1 + kk;
      a[k][i] = fma(-zcol[i], lcol[k], a[k][i]);
    }
    for (int i = j + 1 + tid; i < b; i += blockDim.x) a[j][i] = lcol[i];
    __syncthreads();
  }
  for (int e = tid; e < b * b; e += blockDim.x) {
    const int r = e % b, c = e / b;
    if (r >= c) W[(int64_t)c * ld + r] = a[c][r];
  }
}

// Rows of the panel below a factored diagonal block: z = a L11^-T (unit
// lower), L21 row = z / d (z where d is zero or NaN), and Z row = z (z d where
// d is zero or NaN) for the trailing update.  W at the diagonal block.
template <typename T>
__global__ void __launch_bounds__(128) ldlt_panel_kernel(T* __restrict__ W, int64_t ld, int b, int rs,
                                                         T* __restrict__ Z, int64_t ldz)
{
  __shared__ T L[kLdltNB][kLdltNB + 1];   // L[col][row]
  __shared__ T dd[kLdltNB];
  const int tid = threadIdx.x;
  for (int e = tid; e < kLdltNB * kLdltNB; e += blockDim.x) {
    const int r = e % kLdltNB, c = e / kLdltNB;
    L[c][r] = (r > c && r < b && c < b) ? W[(int64_t)c * ld + r] : T(0);
  }
  if (tid < kLdltNB) dd[tid] = tid < b ? W[(int64_t)tid * ld + tid] : T(1);
  __syncthreads();
  const int r = blockIdx.x * blockDim.x + tid;
  if (r >= rs) return;
  T* row = W + b + r;
  T x[kLdltNB];
#pragma unroll
  for (int c = 0; c < kLdltNB; ++c) x[c] = c < b ? row[(int64_t)c * ld] : T(0);
#pragma unroll
  for (int j = 0; j < kLdltNB; ++j) {
#pragma unroll
    for (int jj = j + 1; jj < kLdltNB; ++jj) x[jj] = fma(-x[j], L[j][jj], x[jj]);
  }
#pragma unroll
  for (int c = 0; c < kLdltNB; ++c) {
    if (c < b) {
      const T d = dd[c];
      const bool valid = fabs((double)d) > 0.0;
      Z[r + (int64_t)c * ldz] = valid ? x[c] : x[c] * d;
      row[(int64_t)c * ld] = valid ? x[c] / d : x[c];
    }
  }
}

// flag[j] = 1 when column j's pivot is valid or its entries below the
// diagonal are all exactly zero (a NaN is not zero), else 0; check_all: test
// every column.
template <typename T>
__global__ void ldlt_zero_column_kernel(const T* __restrict__ W, int64_t ld, int n, int* __restrict__ flag,
                                        int check_all)
{
  const int lane = threadIdx.x & 31;
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (j >= n) return;
  const T* col = W + (int64_t)j * ld;
  const T d = col[j];
  int ok = 1;
  if (check_all || !(fabs((double)d) > 0.0)) {
    for (int i = j + 1 + lane; i < n; i += 32)
      if (!(col[i] == T(0))) ok = 0;
    ok = __all_sync(0xffffffffu, ok);
  }
  if (lane == 0) flag[j] = ok;
}

// dst rows from src rows: dst[i] = src[perm[i]] (inverse: dst[perm[i]] = src[i]).
template <typename T>
__global__ void ldlt_permute_rows_kernel(const T* __restrict__ src, int64_t lds, T* __restrict__ dst, int64_t ldd,
                                         int n, int nrhs, const int* __restrict__ perm, int inverse)
{
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)n * nrhs) return;
  const int i = (int)(e % n), c = (int)(e / n);
  if (inverse) dst[(int64_t)c * ldd + perm[i]] = src[(int64_t)c * lds + i];
  else dst[(int64_t)c * ldd + i] = src[(int64_t)c * lds + perm[i]];
}

// x_i <- x_i / d_i where |d_i| > 1 / highest, else 0 (LDLT.h:555-565).
template <typename T>
__global__ void ldlt_dinv_kernel(const T* __restrict__ W, int64_t ld, int n, int nrhs, T* __restrict__ X, int64_t ldx)
{
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)n * nrhs) return;
  const int i = (int)(e % n), c = (int)(e / n);
  const T tol = sizeof(T) == 8 ? T(1.0 / DBL_MAX) : T(1.0f / FLT_MAX);
  const T d = W[(int64_t)i * ld + i];
  T& x = X[(int64_t)c * ldx + i];
  x = fabs((double)d) > (double)tol ? x / d : T(0);
}

// Lower triangle of W into the used triangle of A (upper: transposed).
template <typename T>
__global__ void ldlt_store_kernel(const T* __restrict__ W, int n, int upper, T* __restrict__ A, int64_t lda)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int j = blockIdx.y; j <= i; j += gridDim.y) {
    const T v = W[(int64_t)j * n + i];
    if (upper) A[(int64_t)i * lda + j] = v;
    else A[(int64_t)j * lda + i] = v;
  }
}

// The reference's transpositions (LDLT.h:305-317) from the input diagonal:
// step k takes the first maximum of |d| over positions k..n-1 of the diagonal
// as permuted so far; a NaN at position k wins, a NaN elsewhere never does.
// perm[i] = the input row at position i after all interchanges.
struct PivotTree {
  int P = 1;
  std::vector<double> val;
  std::vector<int> idx;       // position, -1 = no valid (non-NaN) entry
  void build(const std::vector<double>& a)
  {
    const int n = (int)a.size();
    while (P < n) P *= 2;
    val.assign(2 * P, 0.0);
    idx.assign(2 * P, -1);
    for (int i = 0; i < n; ++i) set(i, a[i], false);
    for (int v = P - 1; v >= 1; --v) pull(v);
  }
  void pull(int v)
  {
    const int l = 2 * v, r = 2 * v + 1;
    if (idx[r] >= 0 && (idx[l] < 0 || val[r] > val[l])) { val[v] = val[r]; idx[v] = idx[r]; }
    else { val[v] = val[l]; idx[v] = idx[l]; }
  }
  void set(int i, double x, bool up)
  {
    int v = P + i;
    val[v] = x;
    idx[v] = std::isnan(x) ? -1 : i;
    if (up)
      for (v >>= 1; v >= 1; v >>= 1) pull(v);
  }
  // first maximum over positions [lo, P)
  int query(int lo) const
  {
    int best = -1;
    double bv = 0.0;
    auto take = [&](int v) {
      if (idx[v] >= 0 && (best < 0 || val[v] > bv || (val[v] == bv && idx[v] < best))) { bv = val[v]; best = idx[v]; }
    };
    for (int l = lo + P, r = 2 * P; l < r; l >>= 1, r >>= 1) {
      if (l & 1) take(l++);
      if (r & 1) take(--r);
    }
    return best;
  }
};

void ldlt_pivots(const std::vector<double>& absdiag, std::vector<int>& tr, std::vector<int>& perm)
{
  const int n = (int)absdiag.size();
  std::vector<double> a = absdiag;
  perm.resize(n);
  tr.resize(n);
  for (int i = 0; i < n; ++i) perm[i] = i;
  PivotTree t;
  t.build(a);
  for (int k = 0; k < n; ++k) {
    int p = std::isnan(a[k]) ? k : t.query(k);
    if (p < 0) p = k;
    tr[k] = p;
    if (p != k) {
      std::swap(a[k], a[p]);
      std::swap(perm[k], perm[p]);
      t.set(k, a[k], true);
      t.set(p, a[p], true);
    }
  }
}

}  // namespace

template <typename T>
int ldlt_solve_device(cudaStream_t s, int n, int nrhs, const T* W, int64_t ld, const int* perm, T* B, int64_t ldb,
                      SolveWork& w)
{
  if (n <= 0 || nrhs <= 0) return GBS_SUCCESS;
  const int64_t tot = (int64_t)n * nrhs;
  GBS_TRY(w.tmp.reserve(sizeof(T) * (size_t)tot));
  T* t = w.tmp.as<T>();
  const int grid = cdiv(tot, 256);
  {
    PhaseScope ps(s, PH_LASWP, 0.0, 2.0 * sizeof(T) * (double)tot);
    GBS_CUDA_TRY(cudaMemcpy2DAsync(t, sizeof(T) * n, B, sizeof(T) * ldb, sizeof(T) * n, nrhs,
                                   cudaMemcpyDeviceToDevice, s));
    ldlt_permute_rows_kernel<T><<<grid, 256, 0, s>>>(t, n, B, ldb, n, nrhs, perm, 0);
    GBS_CUDA_TRY(cudaGetLastError());
  }
  GBS_TRY(tri_solve_device<T>(s, n, nrhs, W, ld, 1, 0, 1, B, ldb, w));
  count_launch();
  ldlt_dinv_kernel<T><<<grid, 256, 0, s>>>(W, ld, n, nrhs, B, ldb);
  GBS_CUDA_TRY(cudaGetLastError());
  GBS_TRY(tri_solve_device<T>(s, n, nrhs, W, ld, 1, 1, 1, B, ldb, w));
  {
    PhaseScope ps(s, PH_LASWP, 0.0, 2.0 * sizeof(T) * (double)tot);
    GBS_CUDA_TRY(cudaMemcpy2DAsync(t, sizeof(T) * n, B, sizeof(T) * ldb, sizeof(T) * n, nrhs,
                                   cudaMemcpyDeviceToDevice, s));
    ldlt_permute_rows_kernel<T><<<grid, 256, 0, s>>>(t, n, B, ldb, n, nrhs, perm, 1);
    GBS_CUDA_TRY(cudaGetLastError());
  }
  return GBS_SUCCESS;
}

template int ldlt_solve_device<double>(cudaStream_t, int, int, const double*, int64_t, const int*, double*, int64_t,
                                       SolveWork&);
template int ldlt_solve_device<float>(cudaStream_t, int, int, const float*, int64_t, const int*, float*, int64_t,
                                      SolveWork&);

// Blocked LDL^T of the lower triangle of W (n x n, ld n), no pivoting.  Z:
// n x kLdltNB scratch.
template <typename T>
static int ldlt_factor_permuted(cudaStream_t s, int n, T* W, T* Z)
{
  for (int k = 0; k < n; k += kLdltNB) {
    const int b = std::min(kLdltNB, n - k);
    const int rs = n - k - b;
    T* Wkk = W + (int64_t)k * n + k;
    {
      PhaseScope ps(s, PH_POTRF_DIAG, (double)b * b * b / 3.0, sizeof(T) * (double)b * b);
      ldlt_diag_kernel<T><<<1, 256, 0, s>>>(Wkk, n, b);
      GBS_CUDA_TRY(cudaGetLastError());
    }
    if (rs > 0) {
      {
        PhaseScope ps(s, PH_TRSM_LLT, (double)rs * b * b, sizeof(T) * 3.0 * rs * b);
        ldlt_panel_kernel<T><<<cdiv(rs, 128), 128, 0, s>>>(Wkk, n, b, rs, Z, rs);
        GBS_CUDA_TRY(cudaGetLastError());
      }
      T* L21 = Wkk + b;
      T* A22 = L21 + (int64_t)b * n;
      // A22 -= Z L21^T (lower): op(B)(kk, j) = L21(j, kk)
      GBS_TRY(syrk_sub_device<T>(s, PH_SYRK, rs, b, Z, 1, rs, L21, n, 1, A22, n));
    }
  }
  return GBS_SUCCESS;
}

}  // namespace gbs

using namespace gbs;

// =================================================================== LDLT object
struct gbs_ldlt {
  int dtype = GBS_F64;
  int uplo = GBS_LOWER;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int64_t n = 0;
  DevBuf A;        // matrixLDLT(): the factor in the used triangle, the other triangle as given
  DevBuf W;        // the lower factor of P A P^T (the solves' operand)
  DevBuf perm, flags, Z, rhs, vec, norm;
  HostBuf hvec;
  SolveWork sw;
  double l1 = 0;
  bool initialized = false;
  int info = GBS_NOT_INITIALIZED;
  int sign = 2;    // LDLT.h:22 SignMatrix: 0 PositiveSemiDef, 1 NegativeSemiDef, 2 ZeroSign, 3 Indefinite
  std::vector<int> tr;
};

namespace {

inline size_t es_of(int dtype) { return dtype == GBS_F64 ? sizeof(double) : sizeof(float); }

template <typename T>
int ldlt_factor_current(gbs_ldlt* o)
{
  const int n = (int)o->n;
  cudaStream_t s = o->stream;
  const int up = o->uplo == GBS_UPPER;
  T* A = o->A.as<T>();
  GBS_TRY(o->norm.reserve(sizeof(double)));
  GBS_TRY(l1_norm_device<T>(s, A, n, n, n, 1, up, o->norm.as<double>(), &o->l1));
  o->tr.assign(n, 0);
  o->sign = 2;
  if (n == 0) {
    o->info = GBS_SUCCESS;
    o->initialized = true;
    return GBS_SUCCESS;
  }
  // the diagonal, to the host
  std::vector<T> hd(n);
  GBS_CUDA_TRY(cudaMemcpy2DAsync(hd.data(), sizeof(T), A, sizeof(T) * (n + 1), sizeof(T), n,
                                 cudaMemcpyDeviceToHost, s));
  GBS_CUDA_TRY(cudaStreamSynchronize(s));
  std::vector<double> ad(n);
  for (int i = 0; i < n; ++i) ad[i] = std::fabs((double)hd[i]);
  std::vector<int> tr, perm;
  ldlt_pivots(ad, tr, perm);
  const double d0 = ad[tr[0]];
  const bool special = n >= 2 && !(d0 > 0.0);   // the whole diagonal zero (or a NaN first): LDLT.h:345-353
  if (special || n == 1) {
    for (int i = 0; i < n; ++i) { tr[i] = i; perm[i] = i; }
  }
  GBS_TRY(o->perm.reserve(sizeof(int) * (size_t)n));
  GBS_CUDA_TRY(cudaMemcpyAsync(o->perm.p, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
  GBS_TRY(o->W.reserve(sizeof(T) * (size_t)n * n));
  T* W = o->W.as<T>();
  {
    PhaseScope ps(s, PH_COPY, 0.0, sizeof(T) * (double)n * n);
    dim3 grid(cdiv(n, 256), std::min(n, 65535));
    ldlt_permute_kernel<T><<<grid, 256, 0, s>>>(A, n, n, up, o->perm.as<int>(), W);
    GBS_CUDA_TRY(cudaGetLastError());
  }
  GBS_TRY(o->flags.reserve(sizeof(int) * (size_t)n));
  std::vector<int> hflag(n, 1);
  if (special) {
    // the matrix stays as given; Success when its used triangle is zero off the diagonal
    count_launch();
    ldlt_zero_column_kernel<T><<<cdiv((int64_t)n * 32, 256), 256, 0, s>>>(W, n, n, o->flags.as<int>(), 1);
    GBS_CUDA_TRY(cudaGetLastError());
    GBS_CUDA_TRY(cudaMemcpyAsync(hflag.data(), o->flags.p, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
    GBS_CUDA_TRY(cudaStreamSynchronize(s));
    bool ret = true;
    for (int j = 0; j < n; ++j) ret = ret && hflag[j];
    o->tr = tr;
    o->sign = 2;
    o->info = ret ? GBS_SUCCESS : GBS_NUMERICAL_ISSUE;
    o->initialized = true;
    return GBS_SUCCESS;
  }
  if (n == 1) {
    o->tr = tr;
    o->sign = hd[0] > T(0) ? 0 : hd[0] < T(0) ? 1 : 2;
    o->info = GBS_SUCCESS;
    o->initialized = true;
    return GBS_SUCCESS;
  }
  GBS_TRY(o->Z.reserve(sizeof(T) * (size_t)n * kLdltNB));
  GBS_TRY(ldlt_factor_permuted<T>(s, n, W, o->Z.as<T>()));
  count_launch();
  ldlt_zero_column_kernel<T><<<cdiv((int64_t)n * 32, 256), 256, 0, s>>>(W, n, n, o->flags.as<int>(), 0);
  GBS_CUDA_TRY(cudaGetLastError());
  {
    PhaseScope ps(s, PH_COPY, 0.0, sizeof(T) * (double)n * n);
    dim3 grid(cdiv(n, 256), std::min(n, 65535));
    ldlt_store_kernel<T><<<grid, 256, 0, s>>>(W, n, up, A, n);
    GBS_CUDA_TRY(cudaGetLastError());
  }
  GBS_CUDA_TRY(cudaMemcpy2DAsync(hd.data(), sizeof(T), W, sizeof(T) * (n + 1), sizeof(T), n,
                                 cudaMemcpyDeviceToHost, s));
  GBS_CUDA_TRY(cudaMemcpyAsync(hflag.data(), o->flags.p, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
  GBS_CUDA_TRY(cudaStreamSynchronize(s));
  // the reference's per-step bookkeeping (LDLT.h:354-369)
  bool ret = true, found_zero = false;
  int sign = 2;
  for (int k = 0; k < n; ++k) {
    const T d = hd[k];
    const bool valid = std::fabs((double)d) > 0.0;
    if (k < n - 1 && !valid) ret = ret && hflag[k];
    if (found_zero && valid) ret = false;
    else if (!valid) found_zero = true;
    if (sign == 0) { if (d < T(0)) sign = 3; }
    else if (sign == 1) { if (d > T(0)) sign = 3; }
    else if (sign == 2) { if (d > T(0)) sign = 0; else if (d < T(0)) sign = 1; }
  }
  o->tr = tr;
  o->sign = sign;
  o->info = ret ? GBS_SUCCESS : GBS_NUMERICAL_ISSUE;
  o->initialized = true;
  return GBS_SUCCESS;
}

int ldlt_prepare(gbs_ldlt* o, int64_t n)
{
  GBS_TRY(ensure_device());
  o->n = n;
  o->initialized = false;
  o->info = GBS_NOT_INITIALIZED;
  GBS_TRY(o->A.reserve(es_of(o->dtype) * (size_t)std::max<int64_t>(n * n, 1)));
  return GBS_SUCCESS;
}

int ldlt_factor(gbs_ldlt* o)
{
  return o->dtype == GBS_F64 ? ldlt_factor_current<double>(o) : ldlt_factor_current<float>(o);
}

int ldlt_ready(const gbs_ldlt* o)
{
  if (!o || !o->initialized) {
    gbs_set_last_message("LDLT is not initialized.");
    return GBS_NOT_INITIALIZED;
  }
  return GBS_SUCCESS;
}

int check_n(int64_t n, int64_t lda)
{
  if (n < 0 || lda < std::max<int64_t>(1, n) || n > (1 << 26)) {   // one warp per column in int thread indexes
    gbs_set_last_message("invalid size or leading dimension");
    return GBS_INVALID_ARGUMENT;
  }
  return GBS_SUCCESS;
}

}  // namespace

extern "C" int gbs_ldlt_create(gbs_ldlt** out, int dtype, int uplo)
{
  if (!out || (dtype != GBS_F64 && dtype != GBS_F32) || (uplo != GBS_LOWER && uplo != GBS_UPPER))
    return GBS_INVALID_ARGUMENT;
  *out = nullptr;
  GBS_TRY(ensure_device());
  gbs_ldlt* o = new gbs_ldlt();
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

extern "C" int gbs_ldlt_destroy(gbs_ldlt* o)
{
  if (!o) return GBS_SUCCESS;
  if (o->stream) cudaStreamSynchronize(o->stream);
  if (o->own_stream && o->stream) cudaStreamDestroy(o->stream);
  delete o;
  return GBS_SUCCESS;
}

extern "C" int gbs_ldlt_set_stream(gbs_ldlt* o, void* stream)
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

extern "C" int gbs_ldlt_compute(gbs_ldlt* o, int64_t n, const void* a, int64_t lda)
{
  if (!o || (n > 0 && !a)) return GBS_INVALID_ARGUMENT;
  GBS_TRY(check_n(n, lda));
  GBS_TRY(ldlt_prepare(o, n));
  const size_t es = es_of(o->dtype);
  if (n > 0)
    GBS_CUDA_TRY(cudaMemcpy2DAsync(o->A.p, n * es, a, lda * es, n * es, n, cudaMemcpyHostToDevice, o->stream));
  return ldlt_factor(o);
}

extern "C" int gbs_ldlt_compute_device(gbs_ldlt* o, int64_t n, const void* d_a, int64_t lda)
{
  if (!o || (n > 0 && !d_a)) return GBS_INVALID_ARGUMENT;
  GBS_TRY(check_n(n, lda));
  GBS_TRY(ldlt_prepare(o, n));
  const size_t es = es_of(o->dtype);
  if (n > 0)
    GBS_CUDA_TRY(cudaMemcpy2DAsync(o->A.p, n * es, d_a, lda * es, n * es, n, cudaMemcpyDeviceToDevice, o->stream));
  return ldlt_factor(o);
}

extern "C" int gbs_ldlt_info(const gbs_ldlt* o)
{
  if (!o || !o->initialized) return GBS_NOT_INITIALIZED;
  return o->info;
}

extern "C" int gbs_ldlt_sign(const gbs_ldlt* o)
{
  if (!o || !o->initialized) return -1;
  return o->sign;
}

extern "C" int gbs_ldlt_is_positive(const gbs_ldlt* o)
{
  if (!o || !o->initialized) return -1;
  return o->sign == 0 || o->sign == 2;
}

extern "C" int gbs_ldlt_is_negative(const gbs_ldlt* o)
{
  if (!o || !o->initialized) return -1;
  return o->sign == 1 || o->sign == 2;
}

static int ldlt_solve_inplace(gbs_ldlt* o, int nrhs, void* dX, int64_t ldx)
{
  const int n = (int)o->n;
  if (o->dtype == GBS_F64)
    return ldlt_solve_device<double>(o->stream, n, nrhs, o->W.as<double>(), n, o->perm.as<int>(), (double*)dX, ldx,
                                     o->sw);
  return ldlt_solve_device<float>(o->stream, n, nrhs, o->W.as<float>(), n, o->perm.as<int>(), (float*)dX, ldx, o->sw);
}

extern "C" int gbs_ldlt_solve(gbs_ldlt* o, int64_t nrhs, const void* b, int64_t ldb, void* x, int64_t ldx)
{
  GBS_TRY(ldlt_ready(o));
  const int64_t n = o->n;
  if (nrhs < 0 || ldb < std::max<int64_t>(1, n) || ldx < std::max<int64_t>(1, n) || (n > 0 && nrhs > 0 && (!b || !x)))
    return GBS_INVALID_ARGUMENT;
  if (n == 0 || nrhs == 0) return GBS_SUCCESS;
  const size_t es = es_of(o->dtype);
  GBS_TRY(o->rhs.reserve(es * (size_t)n * nrhs));
  GBS_CUDA_TRY(cudaMemcpy2DAsync(o->rhs.p, n * es, b, ldb * es, n * es, nrhs, cudaMemcpyHostToDevice, o->stream));
  GBS_TRY(ldlt_solve_inplace(o, (int)nrhs, o->rhs.p, n));
  GBS_TRY(solve_status(o->stream, o->sw));
  GBS_CUDA_TRY(cudaMemcpy2DAsync(x, ldx * es, o->rhs.p, n * es, n * es, nrhs, cudaMemcpyDeviceToHost, o->stream));
  GBS_CUDA_TRY(cudaStreamSynchronize(o->stream));
  return GBS_SUCCESS;
}

extern "C" int gbs_ldlt_solve_device(gbs_ldlt* o, int64_t nrhs, const void* d_b, int64_t ldb, void* d_x, int64_t ldx)
{
  GBS_TRY(ldlt_ready(o));
  const int64_t n = o->n;
  if (nrhs < 0 || ldb < std::max<int64_t>(1, n) || ldx < std::max<int64_t>(1, n)) return GBS_INVALID_ARGUMENT;
  if (n == 0 || nrhs == 0) return GBS_SUCCESS;
  const size_t es = es_of(o->dtype);
  if (d_x != d_b)
    GBS_CUDA_TRY(cudaMemcpy2DAsync(d_x, ldx * es, d_b, ldb * es, n * es, nrhs, cudaMemcpyDeviceToDevice, o->stream));
  return ldlt_solve_inplace(o, (int)nrhs, d_x, ldx);
}

extern "C" int gbs_ldlt_rcond(gbs_ldlt* o, double* rcond)
{
  GBS_TRY(ldlt_ready(o));
  if (!rcond) return GBS_INVALID_ARGUMENT;
  const int n = (int)o->n;
  const bool single = o->dtype == GBS_F32;
  if (n == 0 || o->l1 == 0.0 || n == 1) {
    *rcond = rcond_from_estimate(n, o->l1, 1.0, single);
    return GBS_SUCCESS;
  }
  double est = 0;
  if (o->dtype == GBS_F64)
    GBS_TRY(inv_l1_estimate_device<double>(o->stream, 3, n, o->W.as<double>(), n, o->perm.as<int>(), o->vec, o->hvec,
                                           o->sw, &est));
  else
    GBS_TRY(inv_l1_estimate_device<float>(o->stream, 3, n, o->W.as<float>(), n, o->perm.as<int>(), o->vec, o->hvec,
                                          o->sw, &est));
  *rcond = rcond_from_estimate(n, o->l1, est, single);
  return GBS_SUCCESS;
}

extern "C" int gbs_ldlt_l1_norm(const gbs_ldlt* o, double* l1)
{
  if (!o || !o->initialized || !l1) return GBS_NOT_INITIALIZED;
  *l1 = o->l1;
  return GBS_SUCCESS;
}

extern "C" int gbs_ldlt_matrix(gbs_ldlt* o, void* out, int64_t ld)
{
  GBS_TRY(ldlt_ready(o));
  if (ld < std::max<int64_t>(1, o->n) || (o->n > 0 && !out)) return GBS_INVALID_ARGUMENT;
  if (o->n == 0) return GBS_SUCCESS;
  const size_t es = es_of(o->dtype);
  GBS_CUDA_TRY(cudaMemcpy2DAsync(out, ld * es, o->A.p, o->n * es, o->n * es, o->n, cudaMemcpyDeviceToHost, o->stream));
  GBS_CUDA_TRY(cudaStreamSynchronize(o->stream));
  return GBS_SUCCESS;
}

extern "C" int gbs_ldlt_vector_d(gbs_ldlt* o, void* out)
{
  GBS_TRY(ldlt_ready(o));
  if (o->n > 0 && !out) return GBS_INVALID_ARGUMENT;
  if (o->n == 0) return GBS_SUCCESS;
  const size_t es = es_of(o->dtype);
  GBS_CUDA_TRY(cudaMemcpy2DAsync(out, es, o->A.p, (o->n + 1) * es, es, o->n, cudaMemcpyDeviceToHost, o->stream));
  GBS_CUDA_TRY(cudaStreamSynchronize(o->stream));
  return GBS_SUCCESS;
}

extern "C" int gbs_ldlt_transpositions(gbs_ldlt* o, int* out)
{
  GBS_TRY(ldlt_ready(o));
  if (o->n > 0 && !out) return GBS_INVALID_ARGUMENT;
  for (int64_t i = 0; i < o->n; ++i) out[i] = o->tr[i];
  return GBS_SUCCESS;
}

extern "C" void* gbs_ldlt_device_matrix(gbs_ldlt* o, int64_t* ld)
{
  if (!o || !o->initialized) return nullptr;
  if (ld) *ld = o->n;
  return o->A.p;
}

extern "C" int gbs_ldlt_synchronize(gbs_ldlt* o)
{
  if (!o) return GBS_INVALID_ARGUMENT;
  return solve_status(o->stream, o->sw);
}
