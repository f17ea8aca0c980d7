// Batches of medium general systems (n <= 512): one CTA per matrix, matrix in
// global memory (L2-resident while its CTA works on it).
//
//   mbatch_lu_rcond   FP64 PartialPivLU (first max wins, PartialPivLU.h:365-409)
//                     + ||A||_1 + Hager/Higham rcond (ConditionEstimator.h:56-169)
//                     + solve of one right-hand side: the plain FP64 tier and the
//                     label generator of the precision router
//   mbatch_ir         FP32 LU of a working copy + FP64 iterative refinement to the
//                     backward-error bound; flags the items that did not reach it
//   mbatch_features   router features: size, diagonal and row-norm statistics and
//                     four power-iteration estimates of ||A||_2 / ||A||_F
// Every item is independent; a CTA loops over items (grid-stride).
#include <algorithm>
#include <cmath>
#include <vector>

#include "dense_driver.cuh"
#include "gbs_common.cuh"
#include "gbs_profile.cuh"
#include "mbatch_lu.cuh"

namespace gbs {
namespace {

constexpr int kMB = 256;          // threads per CTA
constexpr int kMaxN = 512;

struct MItem {
  int64_t a_off;   // element offset of the n x n column-major matrix (ld = n)
  int64_t v_off;   // element offset of its n-vectors (rhs / solution / pivots)
  int n;
  int pad;
};

template <typename T>
__device__ T block_sum(T v, T* red)
{
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  T s = T(0);
  for (int i = 0; i < kMB / 32; ++i) s += red[i];
  return s;
}

template <typename T>
__device__ T block_max(T v, T* red)
{
  v = warp_max(v);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  T s = red[0];
  for (int i = 1; i < kMB / 32; ++i) s = red[i] > s ? red[i] : s;
  return s;
}

// first maximum of score over the CTA (lowest index on ties)
template <typename T>
__device__ void block_argmax(T& s, int& i, T* rv, int* ri)
{
  warp_argmax(s, i);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) { rv[warp] = s; ri[warp] = i; }
  __syncthreads();
  s = rv[0];
  i = ri[0];
  for (int w = 1; w < kMB / 32; ++w)
    if (better(rv[w], ri[w], s, i)) { s = rv[w]; i = ri[w]; }
}

constexpr int kNB64 = 16;        // panel width of the FP64 LU
constexpr int kNB32 = 32;        // panel width of the FP32 LU

// x <- A^-1 x (trans = 0) or A^-T x (trans = 1) with PA = LU in a; x in shared
// memory; one barrier per column (the rcond estimator's transposed solves)
template <typename T>
__device__ void cta_lu_solve(const T* a, int n, const int* piv, T* x, int trans)
{
  if (!trans) {
    if (threadIdx.x == 0)
      for (int k = 0; k < n; ++k) {
        const int p = piv[k];
        if (p != k) { const T t = x[k]; x[k] = x[p]; x[p] = t; }
      }
    __syncthreads();
    for (int j = 0; j < n; ++j) {            // unit lower, column-oriented
      const T xj = x[j];
      for (int i = j + 1 + threadIdx.x; i < n; i += kMB) x[i] = fma(-a[(int64_t)j * n + i], xj, x[i]);
      __syncthreads();
    }
    for (int j = n - 1; j >= 0; --j) {       // upper
      if (threadIdx.x == 0) x[j] = x[j] / a[(int64_t)j * n + j];
      __syncthreads();
      const T xj = x[j];
      for (int i = threadIdx.x; i < j; i += kMB) x[i] = fma(-a[(int64_t)j * n + i], xj, x[i]);
      __syncthreads();
    }
  } else {
    for (int j = 0; j < n; ++j) {            // U^T y = b: forward, row j of U^T = column j of U
      if (threadIdx.x == 0) x[j] = x[j] / a[(int64_t)j * n + j];
      __syncthreads();
      const T xj = x[j];
      for (int i = j + 1 + threadIdx.x; i < n; i += kMB) x[i] = fma(-a[(int64_t)i * n + j], xj, x[i]);
      __syncthreads();
    }
    for (int j = n - 1; j >= 0; --j) {       // L^T z = y: backward, unit
      const T xj = x[j];
      for (int i = threadIdx.x; i < j; i += kMB) x[i] = fma(-a[(int64_t)i * n + j], xj, x[i]);
      __syncthreads();
    }
    if (threadIdx.x == 0)
      for (int k = n - 1; k >= 0; --k) {
        const int p = piv[k];
        if (p != k) { const T t = x[k]; x[k] = x[p]; x[p] = t; }
      }
    __syncthreads();
  }
}

// Factor kernels: one CTA per item, the blocked LU's shared memory (two CTAs
// per SM).  The FP64 one records ||A||_1 (needed by rcond) in anorm1 before the
// matrix is overwritten; the FP32 one converts its FP64 item into the working
// copy first.  info[it] = first exactly-zero pivot or -1.
__global__ void __launch_bounds__(kMB, 2)
mbatch_getrf64_kernel(const MItem* __restrict__ items, const int* __restrict__ sel, int count, int total,
                      double* __restrict__ A, int* __restrict__ piv, double* __restrict__ anorm1,
                      int* __restrict__ info)
{
  __shared__ double rv[kMB / 32];
  extern __shared__ __align__(16) char dsm[];
  for (int t = blockIdx.x; t < count; t += gridDim.x) {
    const int it = sel[t];
    if (it < 0 || it >= total) continue;      // ignore out-of-range indices (uniform over the CTA)
    const MItem m = items[it];
    const int n = m.n;
    double* a = A + m.a_off;
    if (anorm1) {
      double best = 0.0;
      for (int c = threadIdx.x >> 5; c < n; c += kMB / 32) {
        double s = 0.0;
#pragma unroll 4
        for (int i = threadIdx.x & 31; i < n; i += 32) s += fabs(a[(int64_t)c * n + i]);
        s = warp_sum(s);
        best = s > best ? s : best;
      }
      best = block_max(best, rv);
      if (threadIdx.x == 0) anorm1[it] = best;
    }
    const int fz = mb::cta_blocked_getrf<double, kNB64>(a, n, piv + m.v_off, dsm);
    if (threadIdx.x == 0) info[it] = fz;
  }
}

__global__ void __launch_bounds__(kMB, 2)
mbatch_getrf32_kernel(const MItem* __restrict__ items, const int* __restrict__ sel, int count, int total,
                      const double* __restrict__ A, float* __restrict__ W, int* __restrict__ piv,
                      int* __restrict__ info)
{
  extern __shared__ __align__(16) char dsm[];
  for (int t = blockIdx.x; t < count; t += gridDim.x) {
    const int it = sel[t];
    if (it < 0 || it >= total) continue;
    const MItem m = items[it];
    const int n = m.n;
    const double* a = A + m.a_off;
    float* w = W + m.a_off;
    const int nn = n * n;
#pragma unroll 4
    for (int e = threadIdx.x; e < nn; e += kMB) w[e] = (float)a[e];
    __syncthreads();
    const int fz = mb::cta_blocked_getrf<float, kNB32>(w, n, piv + m.v_off, dsm);
    if (threadIdx.x == 0) info[it] = fz;
  }
}

// b - A x for the CTA's rows (FP64); 16 columns of loads issued together per
// row.  Returns the thread's max |r_i| and max |x_i|.
__device__ __forceinline__ void cta_residual(const double* __restrict__ a, int n, const double* __restrict__ b,
                                             const double* x, double* r, double& rn, double& xn)
{
  for (int i = threadIdx.x; i < n; i += kMB) {
    double s[4] = {b[i], 0.0, 0.0, 0.0};
    for (int j0 = 0; j0 < n; j0 += 16) {
      double v[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) v[q] = j0 + q < n ? a[(int64_t)(j0 + q) * n + i] : 0.0;
#pragma unroll
      for (int q = 0; q < 16; ++q)
        if (j0 + q < n) s[q & 3] = fma(-v[q], x[j0 + q], s[q & 3]);
    }
    const double t = (s[0] + s[1]) + (s[2] + s[3]);
    r[i] = t;
    rn = fmax(rn, fabs(t));
    xn = fmax(xn, fabs(x[i]));
  }
}

// max_i sum_j |a(i, j)| over the CTA's rows, 16 loads issued together
__device__ __forceinline__ double cta_row_abs_max(const double* __restrict__ a, int n)
{
  double best = 0.0;
  for (int i = threadIdx.x; i < n; i += kMB) {
    double s[4] = {0.0, 0.0, 0.0, 0.0};
    for (int j0 = 0; j0 < n; j0 += 16) {
      double v[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) v[q] = j0 + q < n ? a[(int64_t)(j0 + q) * n + i] : 0.0;
#pragma unroll
      for (int q = 0; q < 16; ++q) s[q & 3] += fabs(v[q]);
    }
    best = fmax(best, (s[0] + s[1]) + (s[2] + s[3]));
  }
  return best;
}

// Solve + rcond of items factored by mbatch_getrf64_kernel (no dynamic shared
// memory: several CTAs per SM hide the triangular solves' latency).
// rcond: ConditionEstimator.h:56-169 (Hager / Higham), ||A||_1 from anorm1.
__global__ void __launch_bounds__(kMB, 3)
mbatch_solve_rcond_kernel(const MItem* __restrict__ items, const int* __restrict__ sel, int count, int total,
                          const double* __restrict__ A, const int* __restrict__ piv, double* __restrict__ rhs,
                          double* __restrict__ rcond)
{
  __shared__ double x[kMaxN], sgn[kMaxN], osgn[kMaxN];
  __shared__ double rv[kMB / 32];
  __shared__ int ri[kMB / 32];
  for (int t = blockIdx.x; t < count; t += gridDim.x) {
    const int it = sel[t];
    if (it < 0 || it >= total) continue;
    const MItem m = items[it];
    const int n = m.n;
    const double* a = A + m.a_off;
    const int* pv = piv + m.v_off;
    if (rhs) {
      for (int i = threadIdx.x; i < n; i += kMB) x[i] = rhs[m.v_off + i];
      __syncthreads();
      mb::cta_lu_solve_blocked(a, n, pv, x);
      for (int i = threadIdx.x; i < n; i += kMB) rhs[m.v_off + i] = x[i];
      __syncthreads();
    }
    if (!rcond) continue;        // uniform over the CTA
    const double anorm = rcond[it];
    // rcond (ConditionEstimator.h:56-169)
    double rc;
    if (n == 0) rc = 1.0;
    else if (anorm == 0.0) rc = 0.0;
    else if (n == 1) rc = 1.0;
    else {
      for (int i = threadIdx.x; i < n; i += kMB) x[i] = 1.0 / n;
      __syncthreads();
      mb::cta_lu_solve_blocked(a, n, pv, x);
      double lb = block_sum([&] { double s = 0; for (int i = threadIdx.x; i < n; i += kMB) s += fabs(x[i]); return s; }(), rv);
      double old_lb = lb;
      int old_v = -1;
      for (int k = 0; k < 4; ++k) {
        int same = 1;
        for (int i = threadIdx.x; i < n; i += kMB) {
          const double sg = x[i] < 0 ? -1.0 : 1.0;
          if (k > 0 && sg != osgn[i]) same = 0;
          sgn[i] = sg;
        }
        same = __syncthreads_and(same);
        if (k > 0 && same) break;
        for (int i = threadIdx.x; i < n; i += kMB) x[i] = sgn[i];
        __syncthreads();
        cta_lu_solve(a, n, pv, x, 1);
        double s = -1.0;
        int vi = 0x7fffffff;
        for (int i = threadIdx.x; i < n; i += kMB) {
          const double t = fabs(x[i]);
          if (better(t, i, s, vi)) { s = t; vi = i; }
        }
        block_argmax(s, vi, rv, ri);
        if (vi == old_v) break;
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += kMB) x[i] = i == vi ? 1.0 : 0.0;
        __syncthreads();
        mb::cta_lu_solve_blocked(a, n, pv, x);
        lb = block_sum([&] { double t = 0; for (int i = threadIdx.x; i < n; i += kMB) t += fabs(x[i]); return t; }(), rv);
        if (lb <= old_lb) break;
        for (int i = threadIdx.x; i < n; i += kMB) osgn[i] = sgn[i];
        old_v = vi;
        old_lb = lb;
        __syncthreads();
      }
      __syncthreads();
      for (int i = threadIdx.x; i < n; i += kMB) x[i] = ((i & 1) ? -1.0 : 1.0) * (1.0 + (double)i / (double)(n - 1));
      __syncthreads();
      mb::cta_lu_solve_blocked(a, n, pv, x);
      const double alt =
          2.0 * block_sum([&] { double t = 0; for (int i = threadIdx.x; i < n; i += kMB) t += fabs(x[i]); return t; }(), rv) /
          (3.0 * n);
      const double est = lb > alt ? lb : alt;
      rc = est == 0.0 ? 0.0 : (1.0 / est) / anorm;
    }
    if (threadIdx.x == 0) rcond[it] = rc;
    __syncthreads();
  }
}

// FP64 refinement of items factored in FP32 by mbatch_getrf32_kernel.
// status[it] on entry: -1 when the FP32 factors are usable (the factor
// kernel's info for a factorization without a zero pivot); on exit: refinement
// steps taken (>= 0) when the backward error reached tol, -1 when it did not,
// -2 when the FP32 factorization had a zero pivot (the caller re-solves both in
// FP64).  X is written only on success.
__global__ void __launch_bounds__(kMB, 4)
mbatch_ir_kernel(const MItem* __restrict__ items, const int* __restrict__ sel, int count, int total,
                 const double* __restrict__ A, const float* __restrict__ W, const int* __restrict__ piv,
                 const double* __restrict__ rhs, double* __restrict__ X, double tol, int max_iter,
                 int* __restrict__ status)
{
  __shared__ double x[kMaxN], r[kMaxN];
  __shared__ float d[kMaxN];
  __shared__ double rvd[kMB / 32];
  for (int t = blockIdx.x; t < count; t += gridDim.x) {
    const int it = sel[t];
    if (it < 0 || it >= total) continue;
    const MItem m = items[it];
    const int n = m.n;
    const double* a = A + m.a_off;
    const float* w = W + m.a_off;
    const int* pv = piv + m.v_off;
    const double* b = rhs + m.v_off;
    const int fz = status[it];
    __syncthreads();
    int result = fz == -1 ? -1 : -2;
    if (fz == -1) {
      const double anorm = block_max(cta_row_abs_max(a, n), rvd);      // ||A||_inf
      double bmax = 0.0;
      for (int i = threadIdx.x; i < n; i += kMB) { x[i] = 0.0; r[i] = b[i]; bmax = fmax(bmax, fabs(r[i])); }
      bmax = block_max(bmax, rvd);
      for (int step = 0; step <= max_iter; ++step) {
        // correction d = LU^-1 (r / s) in FP32, x += s d
        double rm = 0.0;
        for (int i = threadIdx.x; i < n; i += kMB) rm = fmax(rm, fabs(r[i]));
        rm = block_max(rm, rvd);
        const double sc = rm > 0 ? rm : 1.0;
        for (int i = threadIdx.x; i < n; i += kMB) d[i] = (float)(r[i] / sc);
        __syncthreads();
        mb::cta_lu_solve_blocked<float>(w, n, pv, d);
        for (int i = threadIdx.x; i < n; i += kMB) x[i] += sc * (double)d[i];
        __syncthreads();
        // r = b - A x (FP64), backward error
        double rn = 0.0, xn = 0.0;
        cta_residual(a, n, b, x, r, rn, xn);
        rn = block_max(rn, rvd);
        xn = block_max(xn, rvd);
        const double den = anorm * xn + bmax;
        const double be = den > 0 ? rn / den : rn;
        if (be <= tol) { result = step; break; }
        if (!(be == be)) break;
      }
      if (result >= 0)
        for (int i = threadIdx.x; i < n; i += kMB) X[m.v_off + i] = x[i];
    }
    if (threadIdx.x == 0) status[it] = result;
    __syncthreads();
  }
}

// ------------------------------------------------------------------ GMRES-IR
// FP64 GMRES (restarted every outer step, CGS2 Arnoldi, Givens rotations) on
// M^-1 A d = M^-1 r with the FP32 LU as M, inside FP64 iterative refinement
// (Carson & Higham's GMRES-IR).  Reaches the FP64 backward-error bound for
// condition numbers well past the FP32 factorization's own limit.
constexpr int kMaxKrylov = 16;

// vout = M^-1 vin with the FP32 factors applied in FP64 arithmetic (vin, vout
// FP64 shared vectors, may alias)
__device__ void cta_precond(const float* __restrict__ w32, int n, const int* __restrict__ pv, const double* vin,
                            double* vout)
{
  if (vin != vout) {
    for (int i = threadIdx.x; i < n; i += kMB) vout[i] = vin[i];
    __syncthreads();
  }
  mb::cta_lu_solve_blocked<double, float>(w32, n, pv, vout);
}

// y = A v (FP64, v in shared memory), 16 loads in flight per row
__device__ __forceinline__ void cta_matvec(const double* __restrict__ a, int n, const double* v, double* y)
{
  for (int i = threadIdx.x; i < n; i += kMB) {
    double s[4] = {0.0, 0.0, 0.0, 0.0};
    for (int j0 = 0; j0 < n; j0 += 16) {
      double q16[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) q16[q] = j0 + q < n ? a[(int64_t)(j0 + q) * n + i] : 0.0;
#pragma unroll
      for (int q = 0; q < 16; ++q)
        if (j0 + q < n) s[q & 3] = fma(q16[q], v[j0 + q], s[q & 3]);
    }
    y[i] = (s[0] + s[1]) + (s[2] + s[3]);
  }
}

// status[it] on entry and exit as for mbatch_ir_kernel (so a refinement
// failure, -1, may be handed straight to this kernel); on exit outer steps
// taken (>= 0) when the backward error reached tol.  inner[it]: total
// GMRES iterations.  V: Krylov basis, (kMaxKrylov + 1) vectors per item at
// element offset v_off * (kMaxKrylov + 1).
__global__ void __launch_bounds__(kMB, 3)
mbatch_gmres_kernel(const MItem* __restrict__ items, const int* __restrict__ sel, int count, int total,
                    const double* __restrict__ A, const float* __restrict__ W, const int* __restrict__ piv,
                    const double* __restrict__ rhs, double* __restrict__ X, double* __restrict__ V, double tol,
                    int max_outer, int restart, double inner_tol, int* __restrict__ status, int* __restrict__ inner)
{
  __shared__ double x[kMaxN], r[kMaxN], wv[kMaxN];
  __shared__ double H[(kMaxKrylov + 1) * kMaxKrylov];
  __shared__ double cs[kMaxKrylov], sn[kMaxKrylov], g[kMaxKrylov + 1], yv[kMaxKrylov];
  __shared__ double hcol[kMaxKrylov + 1];
  __shared__ double red[kMB / 32][kMaxKrylov + 1];
  __shared__ double rvd[kMB / 32];
  __shared__ int s_stop;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int t = blockIdx.x; t < count; t += gridDim.x) {
    const int it = sel[t];
    if (it < 0 || it >= total) continue;
    const MItem m = items[it];
    const int n = m.n;
    const double* a = A + m.a_off;
    const float* w32 = W + m.a_off;
    const int* pv = piv + m.v_off;
    const double* b = rhs + m.v_off;
    double* Vb = V + m.v_off * (int64_t)(kMaxKrylov + 1);
    const int fz = status[it];
    __syncthreads();
    int result = fz == -1 ? -1 : -2, inner_total = 0;
    if (fz == -1) {
      const double anorm = block_max(cta_row_abs_max(a, n), rvd);
      double bmax = 0.0;
      for (int i = tid; i < n; i += kMB) { x[i] = 0.0; r[i] = b[i]; bmax = fmax(bmax, fabs(b[i])); }
      bmax = block_max(bmax, rvd);
      for (int outer = 0; outer < max_outer; ++outer) {
        cta_precond(w32, n, pv, r, wv);                               // z = M^-1 r
        double ss = 0.0;
        for (int i = tid; i < n; i += kMB) ss += wv[i] * wv[i];
        const double beta = sqrt(block_sum(ss, rvd));
        if (!(beta > 0.0)) break;
        for (int i = tid; i < n; i += kMB) Vb[i] = wv[i] / beta;
        if (tid == 0) {
          g[0] = beta;
          for (int q = 1; q <= kMaxKrylov; ++q) g[q] = 0.0;
        }
        __syncthreads();
        int kdone = 0;
        for (int k = 0; k < restart; ++k) {
          for (int i = tid; i < n; i += kMB) wv[i] = Vb[(int64_t)k * n + i];
          __syncthreads();
          cta_matvec(a, n, wv, r);                                   // r <- A v_k (r is rebuilt after the cycle)
          __syncthreads();
          cta_precond(w32, n, pv, r, wv);                             // w = M^-1 A v_k
          // classical Gram-Schmidt, twice
          for (int pass = 0; pass < 2; ++pass) {
            double part[kMaxKrylov + 1];
#pragma unroll
            for (int q = 0; q <= kMaxKrylov; ++q) part[q] = 0.0;
            for (int i = tid; i < n; i += kMB) {
              const double wi = wv[i];
#pragma unroll
              for (int q = 0; q <= kMaxKrylov; ++q)
                if (q <= k) part[q] = fma(Vb[(int64_t)q * n + i], wi, part[q]);
            }
#pragma unroll
            for (int q = 0; q <= kMaxKrylov; ++q)
              if (q <= k) {
                const double v = warp_sum(part[q]);
                if (lane == 0) red[warp][q] = v;
              }
            __syncthreads();
            if (tid <= k) {
              double h = 0.0;
              for (int w8 = 0; w8 < kMB / 32; ++w8) h += red[w8][tid];
              hcol[tid] = pass == 0 ? h : hcol[tid] + h;
              yv[tid] = h;                                            // this pass's coefficients
            }
            __syncthreads();
            for (int i = tid; i < n; i += kMB) {
              double s0 = wv[i];
              for (int q = 0; q <= k; ++q) s0 = fma(-Vb[(int64_t)q * n + i], yv[q], s0);
              wv[i] = s0;
            }
            __syncthreads();
          }
          double s2 = 0.0;
          for (int i = tid; i < n; i += kMB) s2 += wv[i] * wv[i];
          const double hnext = sqrt(block_sum(s2, rvd));
          if (tid == 0) {
            for (int q = 0; q < k; ++q) {                               // earlier rotations
              const double h0 = hcol[q], h1 = hcol[q + 1];
              hcol[q] = cs[q] * h0 + sn[q] * h1;
              hcol[q + 1] = -sn[q] * h0 + cs[q] * h1;
            }
            const double hk = hcol[k];
            const double rr = sqrt(hk * hk + hnext * hnext);
            const double c = rr > 0 ? hk / rr : 1.0, sgn = rr > 0 ? hnext / rr : 0.0;
            cs[k] = c;
            sn[k] = sgn;
            hcol[k] = rr;
            g[k + 1] = -sgn * g[k];
            g[k] = c * g[k];
            for (int q = 0; q <= k; ++q) H[q + (kMaxKrylov + 1) * k] = hcol[q];
            s_stop = !(hnext > 0.0) || !(rr > 0.0) || fabs(g[k + 1]) <= inner_tol * beta;
          }
          __syncthreads();
          kdone = k + 1;
          if (s_stop) break;
          if (k + 1 < restart)
            for (int i = tid; i < n; i += kMB) Vb[(int64_t)(k + 1) * n + i] = wv[i] / hnext;
          __syncthreads();
        }
        inner_total += kdone;
        if (tid == 0) {                                               // y = H^-1 g (upper triangular)
          for (int q = kdone - 1; q >= 0; --q) {
            double s0 = g[q];
            for (int l = q + 1; l < kdone; ++l) s0 -= H[q + (kMaxKrylov + 1) * l] * yv[l];
            yv[q] = s0 / H[q + (kMaxKrylov + 1) * q];
          }
        }
        __syncthreads();
        for (int i = tid; i < n; i += kMB) {
          double s0 = x[i];
          for (int q = 0; q < kdone; ++q) s0 = fma(Vb[(int64_t)q * n + i], yv[q], s0);
          x[i] = s0;
        }
        __syncthreads();
        double rn = 0.0, xn = 0.0;
        cta_residual(a, n, b, x, r, rn, xn);
        rn = block_max(rn, rvd);
        xn = block_max(xn, rvd);
        const double den = anorm * xn + bmax;
        const double be = den > 0 ? rn / den : rn;
        if (be <= tol) { result = outer; break; }
        if (!(be == be)) break;
      }
      if (result >= 0)
        for (int i = tid; i < n; i += kMB) X[m.v_off + i] = x[i];
    }
    if (tid == 0) {
      status[it] = result;
      if (inner) inner[it] = inner_total;
    }
    __syncthreads();
  }
}

// Router features (kFeat floats per matrix, scale invariant):
//  0 log2(n)/9           1 ||diag||_2/||A||_F       2 min|a_ii|/mean|a_ii|   3 max|a_ii|/mean|a_ii|
//  4 min row norm/mean   5 max row norm/mean        6 std row norm/mean
//  7..10 power-iteration estimates rho_k = ||A^T A x_k||^(1/2) / ||A||_F, x_{k+1} = A^T A x_k / ||.||
//  11..13 log of rho_{k+1}/rho_k (convergence rate of the power iteration)   14 1.0 (bias)  15 0
constexpr int kFeat = 16;

__global__ void __launch_bounds__(kMB)
mbatch_features_kernel(const MItem* __restrict__ items, const int* __restrict__ sel, int count, int total,
                       const double* __restrict__ A, float* __restrict__ F)
{
  __shared__ float x[kMaxN], y[kMaxN];
  __shared__ float rv[kMB / 32];
  for (int t = blockIdx.x; t < count; t += gridDim.x) {
    const int it = sel[t];
    if (it < 0 || it >= total) continue;      // ignore out-of-range indices (uniform over the CTA)
    const MItem m = items[it];
    const int n = m.n;
    const double* a = A + m.a_off;
    // FP32 arithmetic: the features are estimates, and FP64 here would cost more
    // than the low-precision attempt the router is meant to save
    float fro = 0.f, dsq = 0.f, dmin = INFINITY, dmax = 0.f, dsum = 0.f, rmin = INFINITY, rmax = 0.f, rsum = 0.f,
          rsq = 0.f;
    for (int i = threadIdx.x; i < n; i += kMB) {
      float rs = 0.f;
      for (int j = 0; j < n; ++j) { const float v = (float)a[(int64_t)j * n + i]; rs = fmaf(v, v, rs); }
      const float dv = fabsf((float)a[(int64_t)i * n + i]);
      fro += rs;
      dsq += dv * dv;
      dmin = fmin(dmin, dv); dmax = fmax(dmax, dv); dsum += dv;
      const float rn = sqrtf(rs);
      rmin = fmin(rmin, rn); rmax = fmax(rmax, rn); rsum += rn; rsq += rn * rn;
    }
    fro = block_sum(fro, rv);
    dsq = block_sum(dsq, rv);
    dsum = block_sum(dsum, rv);
    rsum = block_sum(rsum, rv);
    rsq = block_sum(rsq, rv);
    dmax = block_max(dmax, rv);
    rmax = block_max(rmax, rv);
    dmin = -block_max(-dmin, rv);
    rmin = -block_max(-rmin, rv);
    const float fnorm = sqrtf(fro) > 0 ? sqrtf(fro) : 1.f;
    const float dmean = dsum / n > 0 ? dsum / n : 1.f, rmean = rsum / n > 0 ? rsum / n : 1.f;
    const float rstd = sqrtf(fmaxf(rsq / n - rmean * rmean, 0.f));
    // power iteration on A^T A from a fixed start vector
    for (int i = threadIdx.x; i < n; i += kMB) x[i] = rsqrtf((float)n) * ((i % 3) ? 1.f : -1.f);
    __syncthreads();
    float rho[4];
    for (int k = 0; k < 4; ++k) {
      for (int i = threadIdx.x; i < n; i += kMB) {
        float s = 0.f;
        for (int j = 0; j < n; ++j) s = fmaf((float)a[(int64_t)j * n + i], x[j], s);
        y[i] = s;
      }
      __syncthreads();
      float nn = 0.f;
      for (int j = threadIdx.x; j < n; j += kMB) {
        float s = 0.f;
        for (int i = 0; i < n; ++i) s = fmaf((float)a[(int64_t)j * n + i], y[i], s);
        x[j] = s;
        nn = fmaf(s, s, nn);
      }
      nn = sqrtf(block_sum(nn, rv));
      rho[k] = sqrtf(nn) / fnorm;
      const float inv = nn > 0 ? 1.f / nn : 0.f;
      for (int j = threadIdx.x; j < n; j += kMB) x[j] *= inv;
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      float* f = F + (int64_t)it * kFeat;
      f[0] = (float)(log2((double)n) / 9.0);
      f[1] = (float)(sqrt(dsq) / fnorm);
      f[2] = (float)(dmin / dmean);
      f[3] = (float)(dmax / dmean);
      f[4] = (float)(rmin / rmean);
      f[5] = (float)(rmax / rmean);
      f[6] = (float)(rstd / rmean);
      for (int k = 0; k < 4; ++k) f[7 + k] = (float)rho[k];
      for (int k = 0; k < 3; ++k) f[11 + k] = (rho[k] > 0 ? 10.f * logf(rho[k + 1] / rho[k]) : 0.f);
      f[14] = 1.0f;
      f[15] = 0.0f;
    }
    __syncthreads();
  }
}

}  // namespace
}  // namespace gbs

using namespace gbs;

struct gbs_mbatch {
  int64_t count = 0;
  std::vector<int> sizes;
  std::vector<int64_t> a_off, v_off;
  int64_t total_a = 0, total_v = 0;
  DevBuf items;
  DevBuf order;      // item indices by decreasing n: the default processing order
  DevBuf krylov;     // GMRES-IR basis, reserved on first use
};

// One CTA per selected item: the block scheduler hands the next item to the
// first CTA slot that frees up, and the default order (largest first) keeps
// the tail of the launch short.
static int mb_grid(int64_t count) { return (int)std::min<int64_t>(count, 0x7fffffff); }

template <typename K>
static int mb_smem(K kernel, size_t bytes)
{
  GBS_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  return GBS_SUCCESS;
}

extern "C" int gbs_mbatch_create(gbs_mbatch** out, int64_t count, const int* sizes)
{
  if (!out || count < 0 || (count > 0 && !sizes)) return GBS_INVALID_ARGUMENT;
  *out = nullptr;
  GBS_TRY(ensure_device());
  gbs_mbatch* p = new gbs_mbatch();
  p->count = count;
  p->sizes.assign(sizes, sizes + count);
  p->a_off.resize((size_t)count);
  p->v_off.resize((size_t)count);
  std::vector<MItem> items((size_t)count);
  int64_t ao = 0, vo = 0;
  for (int64_t i = 0; i < count; ++i) {
    const int n = sizes[i];
    if (n < 1 || n > kMaxN) {
      delete p;
      gbs_set_last_message("gbs_mbatch_create: sizes must be in [1, 512]");
      return GBS_INVALID_ARGUMENT;
    }
    items[(size_t)i] = MItem{ao, vo, n, 0};
    p->a_off[(size_t)i] = ao;
    p->v_off[(size_t)i] = vo;
    ao += (int64_t)n * n;
    vo += n;
  }
  p->total_a = ao;
  p->total_v = vo;
  std::vector<int> order((size_t)count);
  for (int64_t i = 0; i < count; ++i) order[(size_t)i] = (int)i;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return sizes[x] > sizes[y]; });
  int rc = p->items.reserve(sizeof(MItem) * (size_t)std::max<int64_t>(count, 1));
  if (rc == GBS_SUCCESS) rc = p->order.reserve(sizeof(int) * (size_t)std::max<int64_t>(count, 1));
  if (rc == GBS_SUCCESS && count > 0 &&
      (cudaMemcpy(p->items.p, items.data(), sizeof(MItem) * count, cudaMemcpyHostToDevice) != cudaSuccess ||
       cudaMemcpy(p->order.p, order.data(), sizeof(int) * count, cudaMemcpyHostToDevice) != cudaSuccess))
    rc = GBS_CUDA_ERROR;
  if (rc != GBS_SUCCESS) {
    delete p;
    return rc;
  }
  *out = p;
  return GBS_SUCCESS;
}

extern "C" int gbs_mbatch_destroy(gbs_mbatch* p)
{
  delete p;
  return GBS_SUCCESS;
}

extern "C" int64_t gbs_mbatch_matrix_elements(const gbs_mbatch* p) { return p ? p->total_a : 0; }
extern "C" int64_t gbs_mbatch_vector_elements(const gbs_mbatch* p) { return p ? p->total_v : 0; }

extern "C" int gbs_mbatch_offsets(const gbs_mbatch* p, int64_t* a_off, int64_t* v_off)
{
  if (!p) return GBS_INVALID_ARGUMENT;
  if (a_off) std::copy(p->a_off.begin(), p->a_off.end(), a_off);
  if (v_off) std::copy(p->v_off.begin(), p->v_off.end(), v_off);
  return GBS_SUCCESS;
}

// d_items: device list of n_items item indices to process (NULL: all items,
// largest first)
static int mb_select(const gbs_mbatch* p, const int* d_items, int64_t n_items, int* count, const int** sel)
{
  if (d_items) {
    if (n_items < 0 || n_items > p->count) return GBS_INVALID_ARGUMENT;
    *count = (int)n_items;
    *sel = d_items;
  } else {
    *count = (int)p->count;
    *sel = p->order.as<int>();
  }
  return GBS_SUCCESS;
}

extern "C" int gbs_mbatch_lu_rcond(gbs_mbatch* p, const int* d_items, int64_t n_items, double* d_a, int* d_piv,
                                   double* d_rhs, double* d_rcond, int* d_info, void* stream)
{
  if (!p) return GBS_INVALID_ARGUMENT;
  int count = 0;
  const int* sel = nullptr;
  GBS_TRY(mb_select(p, d_items, n_items, &count, &sel));
  if (count == 0) return GBS_SUCCESS;
  if (!d_a || !d_piv || !d_info) return GBS_INVALID_ARGUMENT;
  cudaStream_t s = (cudaStream_t)stream;
  constexpr size_t smem = mb::Layout<double, kNB64>::bytes;
  GBS_TRY(mb_smem(mbatch_getrf64_kernel, smem));
  {
    PhaseScope ps(s, PH_BATCHED, 0.0, 0.0);
    mbatch_getrf64_kernel<<<mb_grid(count), kMB, smem, s>>>(p->items.as<MItem>(), sel, count, (int)p->count, d_a,
                                                           d_piv, d_rcond, d_info);
    GBS_CUDA_TRY(cudaGetLastError());
  }
  if (d_rhs || d_rcond) {
    PhaseScope ps(s, PH_TRI_SOLVE, 0.0, 0.0);
    mbatch_solve_rcond_kernel<<<mb_grid(count), kMB, 0, s>>>(p->items.as<MItem>(), sel, count, (int)p->count, d_a,
                                                            d_piv, d_rhs, d_rcond);
    GBS_CUDA_TRY(cudaGetLastError());
  }
  return GBS_SUCCESS;
}

extern "C" int gbs_mbatch_ir(gbs_mbatch* p, const int* d_items, int64_t n_items, const double* d_a, float* d_work,
                             int* d_piv, const double* d_rhs, double* d_x, double tol, int max_iter, int factored,
                             int* d_status, void* stream)
{
  if (!p || max_iter < 0) return GBS_INVALID_ARGUMENT;
  int count = 0;
  const int* sel = nullptr;
  GBS_TRY(mb_select(p, d_items, n_items, &count, &sel));
  if (count == 0) return GBS_SUCCESS;
  if (!d_a || !d_work || !d_piv || !d_rhs || !d_x || !d_status) return GBS_INVALID_ARGUMENT;
  cudaStream_t s = (cudaStream_t)stream;
  if (!factored) {
    constexpr size_t smem = mb::Layout<float, kNB32>::bytes;
    GBS_TRY(mb_smem(mbatch_getrf32_kernel, smem));
    PhaseScope ps(s, PH_BATCHED, 0.0, 0.0);
    mbatch_getrf32_kernel<<<mb_grid(count), kMB, smem, s>>>(p->items.as<MItem>(), sel, count, (int)p->count, d_a,
                                                           d_work, d_piv, d_status);
    GBS_CUDA_TRY(cudaGetLastError());
  }
  {
    PhaseScope ps(s, PH_RESIDUAL, 0.0, 0.0);
    mbatch_ir_kernel<<<mb_grid(count), kMB, 0, s>>>(p->items.as<MItem>(), sel, count, (int)p->count, d_a, d_work,
                                                   d_piv, d_rhs, d_x, tol, max_iter, d_status);
    GBS_CUDA_TRY(cudaGetLastError());
  }
  return GBS_SUCCESS;
}

extern "C" int gbs_mbatch_gmres_ir(gbs_mbatch* p, const int* d_items, int64_t n_items, const double* d_a,
                                   float* d_work, int* d_piv, const double* d_rhs, double* d_x, double tol,
                                   int max_outer, int restart, int factored, int* d_status, int* d_inner,
                                   void* stream)
{
  if (!p || max_outer < 0 || restart < 1 || restart > kMaxKrylov) return GBS_INVALID_ARGUMENT;
  int count = 0;
  const int* sel = nullptr;
  GBS_TRY(mb_select(p, d_items, n_items, &count, &sel));
  if (count == 0) return GBS_SUCCESS;
  if (!d_a || !d_work || !d_piv || !d_rhs || !d_x || !d_status) return GBS_INVALID_ARGUMENT;
  GBS_TRY(p->krylov.reserve(sizeof(double) * (size_t)p->total_v * (kMaxKrylov + 1)));
  cudaStream_t s = (cudaStream_t)stream;
  if (!factored) {
    constexpr size_t smem = mb::Layout<float, kNB32>::bytes;
    GBS_TRY(mb_smem(mbatch_getrf32_kernel, smem));
    PhaseScope ps(s, PH_BATCHED, 0.0, 0.0);
    mbatch_getrf32_kernel<<<mb_grid(count), kMB, smem, s>>>(p->items.as<MItem>(), sel, count, (int)p->count, d_a,
                                                           d_work, d_piv, d_status);
    GBS_CUDA_TRY(cudaGetLastError());
  }
  {
    PhaseScope ps(s, PH_RESIDUAL, 0.0, 0.0);
    mbatch_gmres_kernel<<<mb_grid(count), kMB, 0, s>>>(p->items.as<MItem>(), sel, count, (int)p->count, d_a, d_work,
                                                      d_piv, d_rhs, d_x, p->krylov.as<double>(), tol, max_outer,
                                                      restart, 1e-10, d_status, d_inner);
    GBS_CUDA_TRY(cudaGetLastError());
  }
  return GBS_SUCCESS;
}

extern "C" int gbs_mbatch_features(gbs_mbatch* p, const int* d_items, int64_t n_items, const double* d_a,
                                   float* d_feat, void* stream)
{
  if (!p) return GBS_INVALID_ARGUMENT;
  int count = 0;
  const int* sel = nullptr;
  GBS_TRY(mb_select(p, d_items, n_items, &count, &sel));
  if (count == 0) return GBS_SUCCESS;
  if (!d_a || !d_feat) return GBS_INVALID_ARGUMENT;
  cudaStream_t s = (cudaStream_t)stream;
  PhaseScope ps(s, PH_ROUTER, 0.0, 0.0);
  mbatch_features_kernel<<<mb_grid(count), kMB, 0, s>>>(p->items.as<MItem>(), sel, count, (int)p->count, d_a, d_feat);
  GBS_CUDA_TRY(cudaGetLastError());
  return GBS_SUCCESS;
}

extern "C" int gbs_router_feature_count(void) { return kFeat; }
