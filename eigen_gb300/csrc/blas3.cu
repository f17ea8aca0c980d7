// BLAS level 3 on the GPU with the semantics of the reference's BLAS shim
// (blas/level3_impl.h): ?gemm, ?trsm, ?syrk, host-buffer and device-buffer
// entry points; and LLT::rankUpdate (LLT.h:231-299, 461-472) on a gbs_llt.
//
//   gemm   C = alpha op(A) op(B) + beta C; beta = 0 sets C to zero without
//          reading it (level3_impl.h:52-58); k = 0 only scales
//   trsm   op(A) X = B (side 'L') or X op(A) = B (side 'R'), then X *= alpha
//          (level3_impl.h:157-174); with diag 'U' the diagonal of A is not
//          read, nor is the other triangle
//   syrk   C = alpha op(A) op(A)^T + beta C on the uplo triangle only
//          (level3_impl.h:396-430)
// Argument checks return the position of the first invalid argument, the
// number the reference passes to xerbla (level3_impl.h:46-54, 146-154,
// 386-394).
//
// One SIMT tile kernel does every product: C tiles of 64 x 64 (32 x 32 or
// 16 x 16 when that spreads the work over more SMs), K in steps of 16 through
// shared memory, 4 x 4 register tiles, FMA on the FP64/FP32 pipes; beta is
// applied in its epilogue, so C is read and written once.  The triangular
// solve is blocked by 32: a diagonal block is solved with one right-hand-side
// column per thread (the block in shared memory), then the rows below (above)
// are updated by the product kernel.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "dense_driver.cuh"
#include "gbs_profile.cuh"

namespace gbs {

namespace {

inline int cdiv(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

constexpr int kTrsmNB = 32;

// C(M x N) = beta' C + alpha op(A) op(B) with op(A)(i,k) = A[i a_rs + k a_cs],
// op(B)(k,j) = B[k b_rs + j b_cs]; beta' C is 0 when beta == 0 (C not read).
// tri: 0 the whole of C, 1 only i >= j, 2 only i <= j.
template <typename T, int BM, int BN, int BK, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
blas_gemm_kernel(int M, int N, int K, T alpha, const T* __restrict__ A, int64_t a_rs, int64_t a_cs,
                 const T* __restrict__ B, int64_t b_rs, int64_t b_cs, T beta, T* __restrict__ C, int64_t ldc, int tri)
{
  constexpr int TX = BN / TN, TY = BM / TM, NT = TX * TY;
  const int bm = blockIdx.y * BM, bn = blockIdx.x * BN;
  if (tri == 1 && bn >= bm + BM) return;              // tile strictly above the diagonal
  if (tri == 2 && bm >= bn + BN) return;              // tile strictly below the diagonal
  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][BN + 1];
  const int tid = threadIdx.x;
  const int tx = tid % TX, ty = tid / TX;
  T acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = T(0);

  for (int k0 = 0; k0 < K; k0 += BK) {
    for (int e = tid; e < BM * BK; e += NT) {
      const int i = e % BM, kk = e / BM;
      const int gi = bm + i, gk = k0 + kk;
      As[kk][i] = (gi < M && gk < K) ? A[(int64_t)gi * a_rs + (int64_t)gk * a_cs] : T(0);
    }
    for (int e = tid; e < BN * BK; e += NT) {
      const int kk = e % BK, j = e / BK;
      const int gj = bn + j, gk = k0 + kk;
      Bs[kk][j] = (gj < N && gk < K) ? B[(int64_t)gk * b_rs + (int64_t)gj * b_cs] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      T af[TM], bf[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) af[i] = As[kk][ty + i * TY];
#pragma unroll
      for (int j = 0; j < TN; ++j) bf[j] = Bs[kk][tx + j * TX];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = fma(af[i], bf[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < TN; ++j) {
    const int gj = bn + tx + j * TX;
    if (gj >= N) continue;
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      const int gi = bm + ty + i * TY;
      if (gi >= M) continue;
      if ((tri == 1 && gi < gj) || (tri == 2 && gi > gj)) continue;
      T* c = C + (int64_t)gj * ldc + gi;
      const T c0 = beta == T(0) ? T(0) : (beta == T(1) ? *c : beta * *c);
      *c = fma(alpha, acc[i][j], c0);
    }
  }
}

template <typename T>
int blas_gemm_launch(cudaStream_t s, int M, int N, int K, T alpha, const T* A, int64_t a_rs, int64_t a_cs, const T* B,
                     int64_t b_rs, int64_t b_cs, T beta, T* C, int64_t ldc, int tri)
{
  if (M <= 0 || N <= 0) return GBS_SUCCESS;
  const double flops = (tri ? 1.0 : 2.0) * M * (double)N * K;
  const double bytes = sizeof(T) * ((double)M * K + (double)K * N + (tri ? 1.0 : 2.0) * M * (double)N);
  PhaseScope ps(s, PH_GEMM, flops, bytes);
  const int64_t sms = device_sm_count();
  const int64_t t64 = (int64_t)cdiv(N, 64) * cdiv(M, 64);
  if (cdiv(M, 16) > 65535) {
    gbs_set_last_message("matrix too tall for the product grid");
    return GBS_INVALID_ARGUMENT;
  }
  if (t64 < sms) {
    const int64_t t32 = (int64_t)cdiv(N, 32) * cdiv(M, 32), t16 = (int64_t)cdiv(N, 16) * cdiv(M, 16);
    const double w32 = (double)((t32 + sms - 1) / sms) / 4.0, w16 = (double)((t16 + sms - 1) / sms) / 16.0;
    if (w16 <= w32)
      blas_gemm_kernel<T, 16, 16, 16, 1, 1><<<dim3(cdiv(N, 16), cdiv(M, 16)), 256, 0, s>>>(
          M, N, K, alpha, A, a_rs, a_cs, B, b_rs, b_cs, beta, C, ldc, tri);
    else
      blas_gemm_kernel<T, 32, 32, 16, 2, 2><<<dim3(cdiv(N, 32), cdiv(M, 32)), 256, 0, s>>>(
          M, N, K, alpha, A, a_rs, a_cs, B, b_rs, b_cs, beta, C, ldc, tri);
  } else {
    blas_gemm_kernel<T, 64, 64, 16, 4, 4><<<dim3(cdiv(N, 64), cdiv(M, 64)), 256, 0, s>>>(
        M, N, K, alpha, A, a_rs, a_cs, B, b_rs, b_cs, beta, C, ldc, tri);
  }
  GBS_CUDA_TRY(cudaGetLastError());
  return GBS_SUCCESS;
}

// C = beta C on the tri part (0 whole, 1 lower, 2 upper); zero_if_zero: beta =
// 0 writes zeros without reading C (gemm / syrk), else a plain product (trsm's
// alpha, where 0 * NaN stays NaN).
template <typename T>
__global__ void blas_scale_kernel(int m, int n, T* __restrict__ C, int64_t ldc, T beta, int tri, int zero_if_zero)
{
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)m * n) return;
  const int i = (int)(e % m), j = (int)(e / m);
  if ((tri == 1 && i < j) || (tri == 2 && i > j)) return;
  T& c = C[(int64_t)j * ldc + i];
  c = (zero_if_zero && beta == T(0)) ? T(0) : beta * c;
}

template <typename T>
int blas_scale(cudaStream_t s, int m, int n, T* C, int64_t ldc, T beta, int tri, int zero_if_zero)
{
  if (m <= 0 || n <= 0) return GBS_SUCCESS;
  count_launch();
  blas_scale_kernel<T><<<cdiv((int64_t)m * n, 256), 256, 0, s>>>(m, n, C, ldc, beta, tri, zero_if_zero);
  GBS_CUDA_TRY(cudaGetLastError());
  return GBS_SUCCESS;
}

// X = op(A_kk)^-1 X for one nb x nb diagonal block (nb <= kTrsmNB) of a
// triangle that is lower in op(A) (lower_eff) or upper; op(A)(i,j) =
// A[i a_rs + j a_cs]; one column of X (ld ldx, ncols columns) per thread.
// Only the block's triangle is read, and its diagonal only when !unit.
template <typename T>
__global__ void __launch_bounds__(128) blas_trsm_block_kernel(const T* __restrict__ A, int64_t a_rs, int64_t a_cs,
                                                              int nb, int lower_eff, int unit, T* __restrict__ X,
                                                              int64_t ldx, int ncols)
{
  __shared__ T L[kTrsmNB][kTrsmNB + 1];     // L[i][j] = op(A)(i, j)
  __shared__ T rdiag[kTrsmNB];
  for (int e = threadIdx.x; e < kTrsmNB * kTrsmNB; e += blockDim.x) {
    const int i = e % kTrsmNB, j = e / kTrsmNB;
    const bool in = i < nb && j < nb && (lower_eff ? i > j : i < j);
    L[i][j] = in ? A[(int64_t)i * a_rs + (int64_t)j * a_cs] : T(0);
  }
  if (threadIdx.x < kTrsmNB) {
    const int i = threadIdx.x;
    rdiag[i] = (unit || i >= nb) ? T(1) : T(1) / A[(int64_t)i * a_rs + (int64_t)i * a_cs];
  }
  __syncthreads();
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncols) return;
  T* col = X + (int64_t)c * ldx;
  T x[kTrsmNB];
#pragma unroll
  for (int i = 0; i < kTrsmNB; ++i) x[i] = i < nb ? col[i] : T(0);
  if (lower_eff) {
#pragma unroll
    for (int j = 0; j < kTrsmNB; ++j) {
      x[j] = x[j] * rdiag[j];
#pragma unroll
      for (int i = j + 1; i < kTrsmNB; ++i) x[i] = fma(-L[i][j], x[j], x[i]);
    }
  } else {
#pragma unroll
    for (int j = kTrsmNB - 1; j >= 0; --j) {
      x[j] = x[j] * rdiag[j];
#pragma unroll
      for (int i = 0; i < j; ++i) x[i] = fma(-L[i][j], x[j], x[i]);
    }
  }
#pragma unroll
  for (int i = 0; i < kTrsmNB; ++i)
    if (i < nb) col[i] = x[i];
}

// op(A) X = B in place on B (m x n, ld ldb), op(A) m x m with the strides
// above and lower_eff its triangle.
template <typename T>
int trsm_left(cudaStream_t s, int m, int n, const T* A, int64_t a_rs, int64_t a_cs, int lower_eff, int unit, T* B,
              int64_t ldb)
{
  const int nblk = cdiv(m, kTrsmNB);
  for (int q = 0; q < nblk; ++q) {
    const int bi = lower_eff ? q : nblk - 1 - q;
    const int k0 = bi * kTrsmNB, kb = std::min(kTrsmNB, m - k0);
    {
      PhaseScope ps(s, PH_TRSM_LU, (double)kb * kb * n, sizeof(T) * 2.0 * kb * n);
      blas_trsm_block_kernel<T><<<cdiv(n, 128), 128, 0, s>>>(A + (int64_t)k0 * a_rs + (int64_t)k0 * a_cs, a_rs, a_cs,
                                                             kb, lower_eff, unit, B + k0, ldb, n);
      GBS_CUDA_TRY(cudaGetLastError());
    }
    if (lower_eff && k0 + kb < m) {        // rows below: B2 -= op(A)(below, block) X_block
      const int r0 = k0 + kb;
      GBS_TRY(blas_gemm_launch<T>(s, m - r0, n, kb, T(-1), A + (int64_t)r0 * a_rs + (int64_t)k0 * a_cs, a_rs, a_cs,
                                  B + k0, 1, ldb, T(1), B + r0, ldb, 0));
    } else if (!lower_eff && k0 > 0) {     // rows above
      GBS_TRY(blas_gemm_launch<T>(s, k0, n, kb, T(-1), A + (int64_t)k0 * a_cs, a_rs, a_cs, B + k0, 1, ldb, T(1), B,
                                  ldb, 0));
    }
  }
  return GBS_SUCCESS;
}

template <typename T>
__global__ void blas_transpose_kernel(const T* __restrict__ S, int64_t lds, int rows, int cols, T* __restrict__ D,
                                      int64_t ldd)
{
  __shared__ T tile[32][33];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int r = r0 + threadIdx.x, c = c0 + k;
    if (r < rows && c < cols) tile[k][threadIdx.x] = S[(int64_t)c * lds + r];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int r = r0 + k, c = c0 + threadIdx.x;     // D(c, r) = S(r, c)
    if (r < rows && c < cols) D[(int64_t)r * ldd + c] = tile[threadIdx.x][k];
  }
}

template <typename T>
int transpose(cudaStream_t s, const T* S, int64_t lds, int rows, int cols, T* D, int64_t ldd)
{
  if (rows <= 0 || cols <= 0) return GBS_SUCCESS;
  PhaseScope ps(s, PH_COPY, 0.0, 2.0 * sizeof(T) * (double)rows * cols);
  blas_transpose_kernel<T><<<dim3(cdiv(cols, 32), cdiv(rows, 32)), dim3(32, 8), 0, s>>>(S, lds, rows, cols, D, ldd);
  GBS_CUDA_TRY(cudaGetLastError());
  return GBS_SUCCESS;
}

inline bool op_ok(char c) { return c == 'N' || c == 'n' || c == 'T' || c == 't' || c == 'C' || c == 'c'; }
inline bool op_notrans(char c) { return c == 'N' || c == 'n'; }
inline bool side_ok(char c) { return c == 'L' || c == 'l' || c == 'R' || c == 'r'; }
inline bool uplo_ok(char c) { return c == 'U' || c == 'u' || c == 'L' || c == 'l'; }
inline bool diag_ok(char c) { return c == 'U' || c == 'u' || c == 'N' || c == 'n'; }

}  // namespace

// ------------------------------------------------------------------ device drivers
template <typename T>
static int gemm_device(char opa, char opb, int m, int n, int k, T alpha, const T* A, int lda, const T* B, int ldb, T beta,
                       T* C, int ldc, cudaStream_t s)
{
  if (m == 0 || n == 0) return GBS_SUCCESS;
  if (k == 0) return beta == T(1) ? GBS_SUCCESS : blas_scale<T>(s, m, n, C, ldc, beta, 0, 1);
  const bool na = op_notrans(opa), nb = op_notrans(opb);
  return blas_gemm_launch<T>(s, m, n, k, alpha, A, na ? 1 : lda, na ? lda : 1, B, nb ? 1 : ldb, nb ? ldb : 1, beta, C,
                             ldc, 0);
}

template <typename T>
static int trsm_device(char side, char uplo, char opa, char diag, int m, int n, T alpha, const T* A, int lda, T* B,
                       int ldb, cudaStream_t s, DevBuf& tmp)
{
  if (m == 0 || n == 0) return GBS_SUCCESS;
  const bool left = side == 'L' || side == 'l', lower = uplo == 'L' || uplo == 'l';
  const bool notrans = op_notrans(opa), unit = diag == 'U' || diag == 'u';
  const int64_t a_rs = notrans ? 1 : lda, a_cs = notrans ? lda : 1;    // op(A)(i,j) = A[i a_rs + j a_cs]
  const int lower_eff = lower == notrans;                               // op(A) lower?
  if (left) {
    GBS_TRY(trsm_left<T>(s, m, n, A, a_rs, a_cs, lower_eff, unit, B, ldb));
  } else {
    // X op(A) = B  <=>  op(A)^T X^T = B^T
    GBS_TRY(tmp.reserve(sizeof(T) * (size_t)m * n));
    T* Bt = tmp.as<T>();
    GBS_TRY(transpose<T>(s, B, ldb, m, n, Bt, n));
    GBS_TRY(trsm_left<T>(s, n, m, A, a_cs, a_rs, !lower_eff, unit, Bt, n));
    GBS_TRY(transpose<T>(s, Bt, n, n, m, B, ldb));
  }
  if (alpha != T(1)) GBS_TRY(blas_scale<T>(s, m, n, B, ldb, alpha, 0, 0));
  return GBS_SUCCESS;
}

template <typename T>
static int syrk_device(char uplo, char op, int n, int k, T alpha, const T* A, int lda, T beta, T* C, int ldc,
                       cudaStream_t s)
{
  const int tri = (uplo == 'U' || uplo == 'u') ? 2 : 1;
  if (n == 0) return GBS_SUCCESS;
  if (k == 0) return beta == T(1) ? GBS_SUCCESS : blas_scale<T>(s, n, n, C, ldc, beta, tri, 1);
  const bool na = op_notrans(op);
  const int64_t a_rs = na ? 1 : lda, a_cs = na ? lda : 1;               // op(A)(i,kk)
  return blas_gemm_launch<T>(s, n, n, k, alpha, A, a_rs, a_cs, A, a_cs, a_rs, beta, C, ldc, tri);
}

// ------------------------------------------------------------------ LLT rank update
// LLT.h:231-299 on the lower factor, element (i, j) at L[i rs + j cs] (upper:
// the transposed view, LLT.h:386-390).  One CTA: per column, thread 0 forms
// the rotation (sigma > 0, Jacobi.h:226-258) or the downdate's scalars, then
// every thread updates its rows of the column and of t.  t: n scratch;
// *fail: the first column whose new diagonal would not be positive, or -1.
template <typename T>
__global__ void __launch_bounds__(1024) llt_rank_update_kernel(T* __restrict__ L, int64_t rs, int64_t cs, int n,
                                                               const T* __restrict__ v, T sigma, T* __restrict__ t,
                                                               int* __restrict__ fail)
{
  __shared__ T sc[4];
  __shared__ int sskip;
  const int tid = threadIdx.x;
  auto at = [&](int i, int j) -> T& { return L[(int64_t)i * rs + (int64_t)j * cs]; };
  if (sigma > T(0)) {
    const T ss = sqrt(sigma);
    for (int i = tid; i < n; i += blockDim.x) t[i] = ss * v[i];
    __syncthreads();
    for (int i = 0; i < n; ++i) {
      if (tid == 0) {
        const T p = at(i, i), q = -t[i];
        T c, s, r;
        if (q == T(0)) { c = p < T(0) ? T(-1) : T(1); s = T(0); r = fabs(p); }
        else if (p == T(0)) { c = T(0); s = q < T(0) ? T(1) : T(-1); r = fabs(q); }
        else if (fabs(p) > fabs(q)) {
          const T tt = q / p;
          T u = sqrt(T(1) + tt * tt);
          if (p < T(0)) u = -u;
          c = T(1) / u; s = -tt * c; r = p * u;
        } else {
          const T tt = p / q;
          T u = sqrt(T(1) + tt * tt);
          if (q < T(0)) u = -u;
          s = T(-1) / u; c = -tt * s; r = q * u;
        }
        at(i, i) = r;
        sc[0] = c;
        sc[1] = s;
        sskip = (c == T(1) && s == T(0));
      }
      __syncthreads();
      if (!sskip) {
        const T c = sc[0], s = sc[1];
        for (int k = i + 1 + tid; k < n; k += blockDim.x) {
          const T xi = at(k, i), yi = t[k];
          at(k, i) = c * xi + s * yi;
          t[k] = -s * xi + c * yi;
        }
      }
      __syncthreads();
    }
    if (tid == 0) *fail = -1;
    return;
  }
  for (int i = tid; i < n; i += blockDim.x) t[i] = v[i];
  __syncthreads();
  T beta = T(1);                                  // thread 0's
  for (int j = 0; j < n; ++j) {
    if (tid == 0) {
      const T ljj = at(j, j), dj = ljj * ljj, wj = t[j];
      const T swj2 = sigma * wj * wj, gamma = dj * beta + swj2;
      const T x = dj + swj2 / beta;
      if (x <= T(0)) {
        sskip = -1;
        *fail = j;
      } else {
        const T nljj = sqrt(x);
        at(j, j) = nljj;
        beta += swj2 / dj;
        sc[0] = wj / ljj;
        sc[1] = nljj / ljj;
        sc[2] = nljj * sigma * wj / gamma;
        sskip = gamma != T(0) ? 1 : 0;
      }
    }
    __syncthreads();
    const int mode = sskip;
    if (mode < 0) return;
    const T f = sc[0], g1 = sc[1], g2 = sc[2];
    for (int k = j + 1 + tid; k < n; k += blockDim.x) {
      const T tk = t[k] - f * at(k, j);
      t[k] = tk;
      if (mode) at(k, j) = g1 * at(k, j) + g2 * tk;
    }
    __syncthreads();
  }
  if (tid == 0) *fail = -1;
}

template <typename T>
int llt_rank_update_device(cudaStream_t s, int n, T* A, int64_t lda, int upper, const T* d_v, double sigma,
                           DevBuf& tmp, int* failed)
{
  if (n <= 0) { *failed = -1; return GBS_SUCCESS; }
  GBS_TRY(tmp.reserve(sizeof(T) * (size_t)n + 256));
  int* d_fail = (int*)((unsigned char*)tmp.p + ((sizeof(T) * (size_t)n + 15) / 16) * 16);
  {
    PhaseScope ps(s, PH_TRI_SOLVE, 6.0 * n * (double)n / 2, sizeof(T) * 2.0 * n * (double)n / 2);
    llt_rank_update_kernel<T><<<1, 1024, 0, s>>>(A, upper ? lda : 1, upper ? 1 : lda, n, d_v, (T)sigma, tmp.as<T>(),
                                                 d_fail);
    GBS_CUDA_TRY(cudaGetLastError());
  }
  GBS_CUDA_TRY(cudaMemcpyAsync(failed, d_fail, sizeof(int), cudaMemcpyDeviceToHost, s));
  GBS_CUDA_TRY(cudaStreamSynchronize(s));
  return GBS_SUCCESS;
}

template int llt_rank_update_device<double>(cudaStream_t, int, double*, int64_t, int, const double*, double, DevBuf&,
                                            int*);
template int llt_rank_update_device<float>(cudaStream_t, int, float*, int64_t, int, const float*, double, DevBuf&,
                                           int*);

}  // namespace gbs

using namespace gbs;

// ------------------------------------------------------------------ C ABI
namespace {

int gemm_check(const char* opa, const char* opb, const int* m, const int* n, const int* k, const void* alpha,
               const int* lda, const int* ldb, const void* beta, const int* ldc)
{
  if (!opa || !opb || !m || !n || !k || !alpha || !lda || !ldb || !beta || !ldc) return 1;
  if (!op_ok(*opa)) return 1;
  if (!op_ok(*opb)) return 2;
  if (*m < 0) return 3;
  if (*n < 0) return 4;
  if (*k < 0) return 5;
  if (*lda < std::max(1, op_notrans(*opa) ? *m : *k)) return 8;
  if (*ldb < std::max(1, op_notrans(*opb) ? *k : *n)) return 10;
  if (*ldc < std::max(1, *m)) return 13;
  return 0;
}

int trsm_check(const char* side, const char* uplo, const char* opa, const char* diag, const int* m, const int* n,
               const void* alpha, const int* lda, const int* ldb)
{
  if (!side || !uplo || !opa || !diag || !m || !n || !alpha || !lda || !ldb) return 1;
  if (!side_ok(*side)) return 1;
  if (!uplo_ok(*uplo)) return 2;
  if (!op_ok(*opa)) return 3;
  if (!diag_ok(*diag)) return 4;
  if (*m < 0) return 5;
  if (*n < 0) return 6;
  if (*lda < std::max(1, (*side == 'L' || *side == 'l') ? *m : *n)) return 9;
  if (*ldb < std::max(1, *m)) return 11;
  return 0;
}

int syrk_check(const char* uplo, const char* op, const int* n, const int* k, const void* alpha, const int* lda,
               const void* beta, const int* ldc)
{
  if (!uplo || !op || !n || !k || !alpha || !lda || !beta || !ldc) return 1;
  if (!uplo_ok(*uplo)) return 1;
  if (!op_ok(*op)) return 2;
  if (*n < 0) return 3;
  if (*k < 0) return 4;
  if (*lda < std::max(1, op_notrans(*op) ? *n : *k)) return 7;
  if (*ldc < std::max(1, *n)) return 10;
  return 0;
}

int arg_error(const char* name, int info)
{
  char buf[96];
  snprintf(buf, sizeof(buf), "%s: argument %d is invalid", name, info);
  gbs_set_last_message(buf);
  return info;
}

int lib_error(int status) { return status == GBS_SUCCESS ? 0 : -(100 + status); }

template <typename T>
int gemm_host(const char* opa, const char* opb, const int* m, const int* n, const int* k, const T* alpha, const T* a,
              const int* lda, const T* b, const int* ldb, const T* beta, T* c, const int* ldc, const char* name)
{
  const int info = gemm_check(opa, opb, m, n, k, alpha, lda, ldb, beta, ldc);
  if (info) return arg_error(name, info);
  if (*m == 0 || *n == 0 || (*k == 0 && *beta == T(1))) return 0;
  WorkspaceLease L;
  if (L.status != GBS_SUCCESS) return lib_error(L.status);
  Workspace& w = *L.ws;
  cudaStream_t s = w.stream;
  const bool na = op_notrans(*opa), nb = op_notrans(*opb);
  const int ar = na ? *m : *k, ac = na ? *k : *m, br = nb ? *k : *n, bc = nb ? *n : *k;
  const size_t es = sizeof(T);
  int rc = w.a.reserve(es * ((size_t)ar * ac + 1));
  if (rc == GBS_SUCCESS) rc = w.b.reserve(es * ((size_t)br * bc + 1));
  if (rc == GBS_SUCCESS) rc = w.scratch.reserve(es * ((size_t)*m * *n + 1));
  if (rc != GBS_SUCCESS) return lib_error(rc);
  T *dA = w.a.as<T>(), *dB = w.b.as<T>(), *dC = w.scratch.as<T>();
  auto up = [&](void* d, const void* h, int64_t ldh, int rows, int cols) {
    return (rows > 0 && cols > 0) ? cudaMemcpy2DAsync(d, rows * es, h, ldh * es, rows * es, cols,
                                                      cudaMemcpyHostToDevice, s) : cudaSuccess;
  };
  if (*k > 0 && (up(dA, a, *lda, ar, ac) != cudaSuccess || up(dB, b, *ldb, br, bc) != cudaSuccess))
    return lib_error(GBS_CUDA_ERROR);
  if (*beta != T(0) && up(dC, c, *ldc, *m, *n) != cudaSuccess) return lib_error(GBS_CUDA_ERROR);
  rc = gemm_device<T>(*opa, *opb, *m, *n, *k, *alpha, dA, ar, dB, br, *beta, dC, *m, s);
  if (rc != GBS_SUCCESS) return lib_error(rc);
  if (cudaMemcpy2DAsync(c, *ldc * es, dC, *m * es, *m * es, *n, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return lib_error(GBS_CUDA_ERROR);
  return 0;
}

template <typename T>
int trsm_host(const char* side, const char* uplo, const char* opa, const char* diag, const int* m, const int* n,
              const T* alpha, const T* a, const int* lda, T* b, const int* ldb, const char* name)
{
  const int info = trsm_check(side, uplo, opa, diag, m, n, alpha, lda, ldb);
  if (info) return arg_error(name, info);
  if (*m == 0 || *n == 0) return 0;
  WorkspaceLease L;
  if (L.status != GBS_SUCCESS) return lib_error(L.status);
  Workspace& w = *L.ws;
  cudaStream_t s = w.stream;
  const int na = (*side == 'L' || *side == 'l') ? *m : *n;
  const size_t es = sizeof(T);
  int rc = w.a.reserve(es * (size_t)na * na);
  if (rc == GBS_SUCCESS) rc = w.b.reserve(es * (size_t)*m * *n);
  if (rc != GBS_SUCCESS) return lib_error(rc);
  if (cudaMemcpy2DAsync(w.a.p, na * es, a, *lda * es, na * es, na, cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemcpy2DAsync(w.b.p, *m * es, b, *ldb * es, *m * es, *n, cudaMemcpyHostToDevice, s) != cudaSuccess)
    return lib_error(GBS_CUDA_ERROR);
  rc = trsm_device<T>(*side, *uplo, *opa, *diag, *m, *n, *alpha, w.a.as<T>(), na, w.b.as<T>(), *m, s, w.scratch);
  if (rc != GBS_SUCCESS) return lib_error(rc);
  if (cudaMemcpy2DAsync(b, *ldb * es, w.b.p, *m * es, *m * es, *n, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return lib_error(GBS_CUDA_ERROR);
  return 0;
}

template <typename T>
int syrk_host(const char* uplo, const char* op, const int* n, const int* k, const T* alpha, const T* a, const int* lda,
              const T* beta, T* c, const int* ldc, const char* name)
{
  const int info = syrk_check(uplo, op, n, k, alpha, lda, beta, ldc);
  if (info) return arg_error(name, info);
  if (*n == 0) return 0;
  WorkspaceLease L;
  if (L.status != GBS_SUCCESS) return lib_error(L.status);
  Workspace& w = *L.ws;
  cudaStream_t s = w.stream;
  const bool na = op_notrans(*op);
  const int ar = na ? *n : *k, ac = na ? *k : *n;
  const size_t es = sizeof(T);
  int rc = w.a.reserve(es * ((size_t)ar * ac + 1));
  if (rc == GBS_SUCCESS) rc = w.scratch.reserve(es * (size_t)*n * *n);
  if (rc != GBS_SUCCESS) return lib_error(rc);
  // C is uploaded whole (the other triangle comes back unchanged)
  if ((*k > 0 && ar > 0 && ac > 0 &&
       cudaMemcpy2DAsync(w.a.p, ar * es, a, *lda * es, ar * es, ac, cudaMemcpyHostToDevice, s) != cudaSuccess) ||
      cudaMemcpy2DAsync(w.scratch.p, *n * es, c, *ldc * es, *n * es, *n, cudaMemcpyHostToDevice, s) != cudaSuccess)
    return lib_error(GBS_CUDA_ERROR);
  rc = syrk_device<T>(*uplo, *op, *n, *k, *alpha, w.a.as<T>(), ar, *beta, w.scratch.as<T>(), *n, s);
  if (rc != GBS_SUCCESS) return lib_error(rc);
  if (cudaMemcpy2DAsync(c, *ldc * es, w.scratch.p, *n * es, *n * es, *n, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return lib_error(GBS_CUDA_ERROR);
  return 0;
}

// device entry points: scratch for the right-side trsm from a pooled workspace
template <typename T>
int trsm_dev(const char* side, const char* uplo, const char* opa, const char* diag, const int* m, const int* n,
             const T* alpha, const T* a, const int* lda, T* b, const int* ldb, void* stream, const char* name)
{
  const int info = trsm_check(side, uplo, opa, diag, m, n, alpha, lda, ldb);
  if (info) return arg_error(name, info);
  if (*m == 0 || *n == 0) return 0;
  WorkspaceLease L;
  if (L.status != GBS_SUCCESS) return lib_error(L.status);
  return lib_error(trsm_device<T>(*side, *uplo, *opa, *diag, *m, *n, *alpha, a, *lda, b, *ldb, (cudaStream_t)stream,
                                  L.ws->scratch));
}

}  // namespace

#define GBS_BLAS_ENTRY(PRE, T)                                                                                       \
  extern "C" int gbs_##PRE##gemm(const char* transa, const char* transb, const int* m, const int* n, const int* k,  \
                                 const T* alpha, const T* a, const int* lda, const T* b, const int* ldb,           \
                                 const T* beta, T* c, const int* ldc)                                              \
  {                                                                                                                 \
    if (ensure_device() != GBS_SUCCESS) return lib_error(GBS_NO_DEVICE);                                           \
    return gemm_host<T>(transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, "gbs_" #PRE "gemm");        \
  }                                                                                                                 \
  extern "C" int gbs_##PRE##gemm_device(const char* transa, const char* transb, const int* m, const int* n,        \
                                        const int* k, const T* alpha, const T* d_a, const int* lda, const T* d_b,  \
                                        const int* ldb, const T* beta, T* d_c, const int* ldc, void* stream)       \
  {                                                                                                                 \
    if (ensure_device() != GBS_SUCCESS) return lib_error(GBS_NO_DEVICE);                                           \
    const int info = gemm_check(transa, transb, m, n, k, alpha, lda, ldb, beta, ldc);                              \
    if (info) return arg_error("gbs_" #PRE "gemm_device", info);                                                  \
    return lib_error(gemm_device<T>(*transa, *transb, *m, *n, *k, *alpha, d_a, *lda, d_b, *ldb, *beta, d_c, *ldc,  \
                                    (cudaStream_t)stream));                                                         \
  }                                                                                                                 \
  extern "C" int gbs_##PRE##trsm(const char* side, const char* uplo, const char* transa, const char* diag,         \
                                 const int* m, const int* n, const T* alpha, const T* a, const int* lda, T* b,     \
                                 const int* ldb)                                                                    \
  {                                                                                                                 \
    if (ensure_device() != GBS_SUCCESS) return lib_error(GBS_NO_DEVICE);                                           \
    return trsm_host<T>(side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb, "gbs_" #PRE "trsm");               \
  }                                                                                                                 \
  extern "C" int gbs_##PRE##trsm_device(const char* side, const char* uplo, const char* transa, const char* diag,  \
                                        const int* m, const int* n, const T* alpha, const T* d_a, const int* lda,  \
                                        T* d_b, const int* ldb, void* stream)                                      \
  {                                                                                                                 \
    if (ensure_device() != GBS_SUCCESS) return lib_error(GBS_NO_DEVICE);                                           \
    return trsm_dev<T>(side, uplo, transa, diag, m, n, alpha, d_a, lda, d_b, ldb, stream, "gbs_" #PRE "trsm_device"); \
  }                                                                                                                 \
  extern "C" int gbs_##PRE##syrk(const char* uplo, const char* trans, const int* n, const int* k, const T* alpha,  \
                                 const T* a, const int* lda, const T* beta, T* c, const int* ldc)                  \
  {                                                                                                                 \
    if (ensure_device() != GBS_SUCCESS) return lib_error(GBS_NO_DEVICE);                                           \
    return syrk_host<T>(uplo, trans, n, k, alpha, a, lda, beta, c, ldc, "gbs_" #PRE "syrk");                       \
  }                                                                                                                 \
  extern "C" int gbs_##PRE##syrk_device(const char* uplo, const char* trans, const int* n, const int* k,           \
                                        const T* alpha, const T* d_a, const int* lda, const T* beta, T* d_c,       \
                                        const int* ldc, void* stream)                                              \
  {                                                                                                                 \
    if (ensure_device() != GBS_SUCCESS) return lib_error(GBS_NO_DEVICE);                                           \
    const int info = syrk_check(uplo, trans, n, k, alpha, lda, beta, ldc);                                         \
    if (info) return arg_error("gbs_" #PRE "syrk_device", info);                                                  \
    return lib_error(syrk_device<T>(*uplo, *trans, *n, *k, *alpha, d_a, *lda, *beta, d_c, *ldc,                    \
                                    (cudaStream_t)stream));                                                         \
  }

GBS_BLAS_ENTRY(d, double)
GBS_BLAS_ENTRY(s, float)
