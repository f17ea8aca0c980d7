// Mixed-precision LU + FP64 iterative refinement (the LAPACK dsgesv idea,
// with the factorization's trailing updates on the tcgen05 tensor cores).
//
//   1. A32 = fp32(A)                                     (HBM-bound cast)
//   2. P A32 = L U: 128-column outer panels; each panel is factored by the
//      cooperative register kernel (32 columns at a time) with its inner
//      updates and the outer trailing update A22 -= A21 A12 on tensor cores
//      in the tier's precision (BF16 / FP16 / TF32 / 3xTF32)
//   3. x = U^-1 L^-1 P b in FP32 (persistent triangular solves)
//   4. repeat: r = b - A x in FP64 (split-K DFMA, deterministic reduction);
//      stop when max_j ||r_j||_inf / (||A||_inf ||x_j||_inf + ||b_j||_inf)
//      <= tol; d = LU^-1 (r / s) in FP32 with s = ||r_j||_inf per column;
//      x += s d in FP64
//   5. refinement that stops decreasing (or runs out of iterations) falls
//      back to the plain FP64 factorization, which then decides the result.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include "dense_driver.cuh"
#include "dense_kernels.cuh"
#include "gbs_profile.cuh"
#include "mixed_driver.cuh"
#include "tc_gemm.cuh"

namespace gbs {

static inline int cdiv(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

// ------------------------------------------------------------------ kernels
// R = B - A X, FP64.  Grid (row blocks of 128, K splits); each thread owns one
// row and RC right-hand sides; X's K-chunk is staged in shared memory.
// Partial sums go to part[split][col][row]; residual_reduce adds them in
// split order (deterministic).
constexpr int kResRows = 128, kResRC = 16, kResKC = 64;

__global__ void __launch_bounds__(kResRows)
residual_partial_kernel(int n, int nrhs, const double* __restrict__ A, int64_t lda, const double* __restrict__ X,
                        int64_t ldx, int kspan, double* __restrict__ part)
{
  __shared__ double sx[kResKC][kResRC];
  const int row = blockIdx.x * kResRows + threadIdx.x;
  const int split = blockIdx.y;
  const int k0 = split * kspan, k1 = min(n, k0 + kspan);
  double acc[kResRC];
#pragma unroll
  for (int c = 0; c < kResRC; ++c) acc[c] = 0.0;
  for (int kc = k0; kc < k1; kc += kResKC) {
    __syncthreads();
    for (int e = threadIdx.x; e < kResKC * kResRC; e += kResRows) {
      const int kk = e % kResKC, c = e / kResKC;
      sx[kk][c] = (kc + kk < k1 && c < nrhs) ? X[(int64_t)c * ldx + kc + kk] : 0.0;
    }
    __syncthreads();
    if (row < n) {
      const int kend = min(kResKC, k1 - kc);
      const double* ap = A + (int64_t)kc * lda + row;
      for (int kk = 0; kk < kend; ++kk) {
        const double a = ap[(int64_t)kk * lda];
#pragma unroll
        for (int c = 0; c < kResRC; ++c) acc[c] = fma(a, sx[kk][c], acc[c]);
      }
    }
  }
  if (row < n) {
    for (int c = 0; c < nrhs; ++c) part[((int64_t)split * nrhs + c) * n + row] = acc[c];
  }
}

__global__ void residual_reduce_kernel(int n, int nrhs, int splits, const double* __restrict__ part,
                                       const double* __restrict__ B, int64_t ldb, double* __restrict__ R)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * nrhs) return;
  const int row = (int)(t % n), c = (int)(t / n);
  double s = 0.0;
  for (int k = 0; k < splits; ++k) s += part[((int64_t)k * nrhs + c) * n + row];
  R[(int64_t)c * n + row] = B[(int64_t)c * ldb + row] - s;
}

// out[c] = max_i |V(i, c)| for the three matrices (R, X, B) of one refinement
// step, stored as out[0..nrhs) = R, [nrhs..2nrhs) = X, [2nrhs..3nrhs) = B.
__global__ void col_absmax3_kernel(int n, int nrhs, const double* R, int64_t ldr, const double* X, int64_t ldx,
                                   const double* B, int64_t ldb, double* out)
{
  const int which = blockIdx.y;   // 0 = R, 1 = X, 2 = B
  const int c = blockIdx.x;
  const double* V = which == 0 ? R : which == 1 ? X : B;
  const int64_t ld = which == 0 ? ldr : which == 1 ? ldx : ldb;
  double m = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double v = fabs(V[(int64_t)c * ld + i]);
    m = (v > m || v != v) ? v : m;
  }
  m = warp_max(m);
  __shared__ double sm[32];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = threadIdx.x < (blockDim.x >> 5) ? sm[threadIdx.x] : 0.0;
    m = warp_max(m);
    if (threadIdx.x == 0) out[which * nrhs + c] = m;
  }
}

// ||A||_inf = max_i sum_j |a_ij| : one thread per row, coalesced over rows.
__global__ void row_abs_sum_kernel(int n, const double* __restrict__ A, int64_t lda, double* __restrict__ rows)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int j = 0; j < n; ++j) s += fabs(A[(int64_t)j * lda + i]);
  rows[i] = s;
}

// W32 = fp32(R / s_c), s_c = max_i |R(i,c)| (1 when zero); W packed n x nrhs
__global__ void scale_to_f32_kernel(int n, int nrhs, const double* __restrict__ R, int64_t ldr,
                                    const double* __restrict__ scale, float* __restrict__ W)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * nrhs) return;
  const int row = (int)(t % n), c = (int)(t / n);
  const double s = scale[c] > 0.0 ? scale[c] : 1.0;
  W[t] = (float)(R[(int64_t)c * ldr + row] / s);
}

// X += s_c * W32 (FP64); init != 0: X = s_c * W32
__global__ void update_from_f32_kernel(int n, int nrhs, const float* __restrict__ W, const double* __restrict__ scale,
                                       double* __restrict__ X, int64_t ldx, int init)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * nrhs) return;
  const int row = (int)(t % n), c = (int)(t / n);
  const double s = scale[c] > 0.0 ? scale[c] : 1.0;
  const double d = s * (double)W[t];
  double* xp = X + (int64_t)c * ldx + row;
  *xp = init ? d : *xp + d;
}

// ------------------------------------------------------------------ workspace pool
struct MixedWork {
  cudaStream_t stream = nullptr;
  DevBuf a32, tr, st, scratch, r, part, w32, stats, rows, a64, x64, map;
  SolveWork sw;
  TcWorkspace tc;
  HostBuf hstats;
  Workspace plain;
};

static std::mutex g_mpool_mu;
static std::vector<MixedWork*> g_mpool;

struct MixedLease {
  MixedWork* w = nullptr;
  int status = GBS_SUCCESS;
  MixedLease()
  {
    status = ensure_device();
    if (status != GBS_SUCCESS) return;
    {
      std::lock_guard<std::mutex> lk(g_mpool_mu);
      if (!g_mpool.empty()) {
        w = g_mpool.back();
        g_mpool.pop_back();
      }
    }
    if (!w) {
      w = new MixedWork();
      if (cudaStreamCreateWithFlags(&w->stream, cudaStreamDefault) != cudaSuccess) {
        delete w;
        w = nullptr;
        status = GBS_CUDA_ERROR;
      }
    }
  }
  ~MixedLease()
  {
    if (!w) return;
    std::lock_guard<std::mutex> lk(g_mpool_mu);
    g_mpool.push_back(w);
  }
};

// ------------------------------------------------------------------ factorization
constexpr int kMixedNB = 128;

int mixed_getrf(cudaStream_t s, int n, float* A, int64_t lda, int* tr, DeviceStatus* st, DevBuf& scratch, int kind,
                TcWorkspace& tcw, SolveWork& sw, DevBuf& map)
{
  for (int k = 0; k < n; k += kMixedNB) {
    const int kb = std::min(kMixedNB, n - k);
    // ---- panel [k:n, k:k+kb]
    for (int j = k; j < k + kb; j += kPanelNB) {
      const int jb = std::min(kPanelNB, k + kb - j);
      float* Ajj = A + (int64_t)j * lda + j;
      GBS_TRY(panel_factor<float>(s, Ajj, lda, n - j, jb, j, tr + j, scratch, st));
      GBS_TRY(laswp_gather_device<float>(s, A, lda, tr, j, j + jb, k, j, j + jb, k + kb, map));
      const int rest = k + kb - (j + jb);
      if (rest > 0) {
        float* A12 = A + (int64_t)(j + jb) * lda + j;
        {
          PhaseScope ps(s, PH_TRSM_LU, (double)jb * jb * rest, 8.0 * jb * rest);
          trsm_lunit_kernel<float, kPanelNB><<<cdiv(rest, 128), 128, 0, s>>>(Ajj, lda, jb, A12, lda, rest);
          GBS_CUDA_TRY(cudaGetLastError());
        }
        const int rows = n - (j + jb);
        if (rows > 0)
          GBS_TRY(tc_gemm_sub(s, kind, rows, rest, jb, Ajj + jb, 1, lda, A12, 1, lda, A12 + jb, lda, 0, st, tcw));
      }
    }
    // ---- interchanges outside the panel, TRSM of A12, trailing update
    GBS_TRY(laswp_gather_device<float>(s, A, lda, tr, k, k + kb, 0, k, k + kb, n, map));
    const int nr = n - k - kb;
    if (nr > 0) {
      float* Akk = A + (int64_t)k * lda + k;
      float* A12 = A + (int64_t)(k + kb) * lda + k;
      GBS_TRY(trsm_lunit_wide<float>(s, kb, nr, Akk, lda, A12, lda));
      GBS_TRY(tc_gemm_sub(s, kind, nr, nr, kb, Akk + kb, 1, lda, A12, 1, lda, A12 + kb, lda, 0, st, tcw));
    }
  }
  return GBS_SUCCESS;
}

// ------------------------------------------------------------------ refinement
static int residual(cudaStream_t s, int n, int nrhs, const double* A, int64_t lda, const double* X, int64_t ldx,
                    const double* B, int64_t ldb, double* R, MixedWork& w)
{
  const int splits = std::max(1, std::min(32, cdiv((int64_t)device_sm_count() * 4, cdiv(n, kResRows))));
  const int kspan = cdiv(cdiv(n, splits), kResKC) * kResKC;
  const int used = cdiv(n, kspan);
  GBS_TRY(w.part.reserve(sizeof(double) * (size_t)used * n * nrhs));
  {
    PhaseScope ps(s, PH_RESIDUAL, 2.0 * n * (double)n * nrhs, 8.0 * ((double)n * n + 2.0 * n * nrhs));
    residual_partial_kernel<<<dim3(cdiv(n, kResRows), used), kResRows, 0, s>>>(n, nrhs, A, lda, X, ldx, kspan,
                                                                               w.part.as<double>());
    GBS_CUDA_TRY(cudaGetLastError());
  }
  count_launch();
  residual_reduce_kernel<<<cdiv((int64_t)n * nrhs, 256), 256, 0, s>>>(n, nrhs, used, w.part.as<double>(), B, ldb, R);
  GBS_CUDA_TRY(cudaGetLastError());
  return GBS_SUCCESS;
}

static double host_backward_error(int nrhs, const double* st, double anorm, double* worst_out)
{
  double worst = 0.0;
  for (int c = 0; c < nrhs; ++c) {
    const double rn = st[c], xn = st[nrhs + c], bn = st[2 * nrhs + c];
    const double den = anorm * xn + bn;
    double e = den > 0 ? rn / den : rn;
    if (e != e) e = INFINITY;
    worst = std::max(worst, e);
  }
  if (worst_out) *worst_out = worst;
  return worst;
}

int mixed_lu_solve(cudaStream_t s, int n, int nrhs, const double* A, int64_t lda, const double* B, int64_t ldb,
                   double* X, int64_t ldx, const MixedOptions& opt, MixedResult* res)
{
  MixedResult out;
  out.tier = opt.tier;
  if (n <= 0 || nrhs <= 0) {
    if (res) *res = out;
    return GBS_SUCCESS;
  }
  if (nrhs > kResRC) {
    // refine independent 16-column groups
    MixedResult worst;
    for (int c0 = 0; c0 < nrhs; c0 += kResRC) {
      MixedResult r;
      const int nc = std::min(kResRC, nrhs - c0);
      GBS_TRY(mixed_lu_solve(s, n, nc, A, lda, B + (int64_t)c0 * ldb, ldb, X + (int64_t)c0 * ldx, ldx, opt, &r));
      worst.iterations = std::max(worst.iterations, r.iterations);
      worst.fell_back |= r.fell_back;
      worst.backward_error = std::max(worst.backward_error, r.backward_error);
      worst.tier = r.tier;
    }
    if (res) *res = worst;
    return GBS_SUCCESS;
  }
  MixedLease lease;
  if (lease.status != GBS_SUCCESS) return lease.status;
  MixedWork& w = *lease.w;
  const size_t nn = (size_t)n * n;
  GBS_TRY(w.a32.reserve(sizeof(float) * nn));
  GBS_TRY(w.tr.reserve(sizeof(int) * (size_t)n));
  GBS_TRY(w.st.reserve(sizeof(DeviceStatus)));
  GBS_TRY(w.r.reserve(sizeof(double) * (size_t)n * nrhs));
  GBS_TRY(w.w32.reserve(sizeof(float) * (size_t)n * nrhs));
  GBS_TRY(w.stats.reserve(sizeof(double) * (3 * nrhs + 1)));
  GBS_TRY(w.rows.reserve(sizeof(double) * (size_t)n));
  GBS_TRY(w.hstats.reserve(sizeof(double) * (3 * nrhs + 1)));
  DeviceStatus* st = w.st.as<DeviceStatus>();
  float* A32 = w.a32.as<float>();
  double* R = w.r.as<double>();
  float* W = w.w32.as<float>();
  double* stats = w.stats.as<double>();
  double* hst = (double*)w.hstats.p;

  // ||A||_inf (once)
  count_launch();
  row_abs_sum_kernel<<<cdiv(n, 256), 256, 0, s>>>(n, A, lda, w.rows.as<double>());
  GBS_CUDA_TRY(cudaGetLastError());
  std::vector<double> hrows((size_t)n);
  GBS_CUDA_TRY(cudaMemcpyAsync(hrows.data(), w.rows.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));

  GBS_TRY(reset_status(st, s));
  double anorm = 0;
  for (double v : hrows) anorm = std::max(anorm, v);

  bool converged = false;
  if (opt.tier != GBS_TIER_FP64) {
    {
      PhaseScope ps(s, PH_COPY, 0.0, 12.0 * nn);
      copy_matrix_kernel<double, float><<<std::min<int64_t>(cdiv(nn, 256), 65535 * 8), 256, 0, s>>>(A, lda, A32, n, n, n);
      GBS_CUDA_TRY(cudaGetLastError());
    }
    const int kind = opt.tier == GBS_TIER_BF16 ? TC_BF16 : opt.tier == GBS_TIER_FP16 ? TC_FP16
                   : opt.tier == GBS_TIER_TF32 ? TC_TF32 : TC_TF32X3;
    GBS_TRY(mixed_getrf(s, n, A32, n, w.tr.as<int>(), st, w.scratch, kind, w.tc, w.sw, w.map));
    DeviceStatus h;
    GBS_TRY(read_status(st, &h, s));
    if (h.info < 0) {
      // x0 = LU^-1 b in FP32, scaled per column
      count_launch();
      col_absmax3_kernel<<<dim3(nrhs, 3), 256, 0, s>>>(n, nrhs, B, ldb, B, ldb, B, ldb, stats);
      count_launch();
      scale_to_f32_kernel<<<cdiv((int64_t)n * nrhs, 256), 256, 0, s>>>(n, nrhs, B, ldb, stats, W);
      GBS_CUDA_TRY(cudaGetLastError());
      GBS_TRY(lu_solve_device<float>(s, n, nrhs, A32, n, w.tr.as<int>(), W, n, 0, w.sw));
      count_launch();
      update_from_f32_kernel<<<cdiv((int64_t)n * nrhs, 256), 256, 0, s>>>(n, nrhs, W, stats, X, ldx, 1);
      GBS_CUDA_TRY(cudaGetLastError());
      double prev = INFINITY;
      int stalls = 0;
      for (int it = 0; it <= opt.max_iter; ++it) {
        GBS_TRY(residual(s, n, nrhs, A, lda, X, ldx, B, ldb, R, w));
        count_launch();
        col_absmax3_kernel<<<dim3(nrhs, 3), 256, 0, s>>>(n, nrhs, R, n, X, ldx, B, ldb, stats);
        GBS_CUDA_TRY(cudaGetLastError());
        GBS_CUDA_TRY(cudaMemcpyAsync(hst, stats, sizeof(double) * 3 * nrhs, cudaMemcpyDeviceToHost, s));
        GBS_TRY(solve_status(s, w.sw));
        double be = host_backward_error(nrhs, hst, anorm, nullptr);
        out.backward_error = be;
        out.iterations = it;
        if (be <= opt.tol) { converged = true; break; }
        if (!(be < 0.5 * prev)) { if (++stalls >= 2) break; } else stalls = 0;
        prev = std::min(prev, be);
        if (it == opt.max_iter) break;
        count_launch();
        scale_to_f32_kernel<<<cdiv((int64_t)n * nrhs, 256), 256, 0, s>>>(n, nrhs, R, n, stats, W);
        GBS_CUDA_TRY(cudaGetLastError());
        GBS_TRY(lu_solve_device<float>(s, n, nrhs, A32, n, w.tr.as<int>(), W, n, 0, w.sw));
        count_launch();
        update_from_f32_kernel<<<cdiv((int64_t)n * nrhs, 256), 256, 0, s>>>(n, nrhs, W, stats, X, ldx, 0);
        GBS_CUDA_TRY(cudaGetLastError());
      }
    }
  }
  if (!converged) {
    // plain FP64 factorization decides the result
    out.fell_back = opt.tier != GBS_TIER_FP64;
    out.tier = GBS_TIER_FP64;
    GBS_TRY(w.a64.reserve(sizeof(double) * nn));
    GBS_TRY(w.tr.reserve(sizeof(int) * (size_t)n));
    GBS_TRY(copy_matrix_device<double>(s, A, lda, w.a64.as<double>(), n, n, n));
    GBS_TRY(reset_status(st, s));
    GBS_TRY(getrf_device<double>(s, n, n, w.a64.as<double>(), n, w.tr.as<int>(), st, w.scratch));
    DeviceStatus h;
    GBS_TRY(read_status(st, &h, s));
    GBS_TRY(copy_matrix_device<double>(s, B, ldb, X, ldx, n, nrhs));
    GBS_TRY(lu_solve_device<double>(s, n, nrhs, w.a64.as<double>(), n, w.tr.as<int>(), X, ldx, 0, w.sw));
    GBS_TRY(residual(s, n, nrhs, A, lda, X, ldx, B, ldb, R, w));
    count_launch();
    col_absmax3_kernel<<<dim3(nrhs, 3), 256, 0, s>>>(n, nrhs, R, n, X, ldx, B, ldb, stats);
    GBS_CUDA_TRY(cudaMemcpyAsync(hst, stats, sizeof(double) * 3 * nrhs, cudaMemcpyDeviceToHost, s));
    GBS_TRY(solve_status(s, w.sw));
    out.backward_error = host_backward_error(nrhs, hst, anorm, nullptr);
    if (h.info >= 0) out.singular = 1;
  }
  if (res) *res = out;
  return GBS_SUCCESS;
}

}  // namespace gbs
