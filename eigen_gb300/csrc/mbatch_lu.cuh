// CTA-level blocked PartialPivLU and triangular solves for one n x n matrix
// (n <= 512, column-major, ld = n) per thread block of kMB threads.
//
// Right-looking blocked LU with NB-column panels, the order of
// partial_lu_impl::blocked_lu (PartialPivLU.h:426-496):
//   1. panel rows [k0, n) x NB columns in registers (two rows per thread);
//      per column: first-max pivot search (warp shuffles + one block
//      exchange), row exchange inside the panel, division by the pivot and the
//      rank-1 update of the panel's later columns (unblocked_lu,
//      PartialPivLU.h:365-409);
//   2. the panel's row transpositions applied to every other column as one
//      gather per column (warp per column);
//   3. U12 = L11^-1 A12, one column per thread (L11 from shared memory);
//   4. A22 -= L21 U12 in 64-column chunks, each warp an 8-column slab,
//      each lane four rows a pass, K = NB fully unrolled (L21 transposed in
//      shared memory, the U12 chunk in shared memory, A22 read and written once
//      per panel).
// The last panel (fewer than NB columns) has no trailing matrix, so steps 3
// and 4 always run with the full NB.
#pragma once

#include "gbs_common.cuh"

namespace gbs {
namespace mb {

constexpr int kMB = 256;          // threads per CTA
constexpr int kMaxN = 512;        // two rows per thread in the panel
constexpr int kCW = 64;           // trailing-update chunk width (8 warps x 8 columns)

template <typename T, int NB>
struct Layout {                   // dynamic shared memory of the blocked LU
  static constexpr size_t lt = 0;                                        // T[NB][kMaxN]  L panel, transposed
  static constexpr size_t ub = lt + sizeof(T) * NB * kMaxN;              // T[NB][kCW+1]  U12 chunk
  static constexpr size_t prow = ub + sizeof(T) * NB * (kCW + 1);        // T[NB]         pivot row
  static constexpr size_t krow = prow + sizeof(T) * NB;                  // T[NB]         row k
  static constexpr size_t perm = krow + sizeof(T) * NB;                  // int[kMaxN]
  static constexpr size_t spiv = perm + sizeof(int) * kMaxN;             // int[NB]
  static constexpr size_t red = spiv + sizeof(int) * NB;                 // T[8] + int[8]
  static constexpr size_t bytes = red + (sizeof(T) + sizeof(int)) * (kMB / 32) + 16;
};

// first maximum over the CTA (lowest index on ties), result in every thread
template <typename T>
__device__ __forceinline__ void cta_argmax(T& s, int& i, T* rv, int* ri)
{
  warp_argmax(s, i);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) { rv[warp] = s; ri[warp] = i; }
  __syncthreads();
  s = rv[0];
  i = ri[0];
#pragma unroll
  for (int w = 1; w < kMB / 32; ++w)
    if (better(rv[w], ri[w], s, i)) { s = rv[w]; i = ri[w]; }
}

// In-place LU of a; 0-based pivots to piv.  Returns the first exactly-zero
// pivot or -1 (same value in every thread).  smem: Layout<T, NB>::bytes.
template <typename T, int NB>
__device__ int cta_blocked_getrf(T* __restrict__ a, int n, int* __restrict__ piv, char* smem)
{
  using Ly = Layout<T, NB>;
  T(*lt)[kMaxN] = reinterpret_cast<T(*)[kMaxN]>(smem + Ly::lt);
  T(*ub)[kCW + 1] = reinterpret_cast<T(*)[kCW + 1]>(smem + Ly::ub);
  T* prow = reinterpret_cast<T*>(smem + Ly::prow);
  T* krow = reinterpret_cast<T*>(smem + Ly::krow);
  int* perm = reinterpret_cast<int*>(smem + Ly::perm);
  int* spiv = reinterpret_cast<int*>(smem + Ly::spiv);
  T* rv = reinterpret_cast<T*>(smem + Ly::red);
  int* ri = reinterpret_cast<int*>(smem + Ly::red + sizeof(T) * (kMB / 32));
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int first_zero = -1;

  for (int k0 = 0; k0 < n; k0 += NB) {
    const int nb = min(NB, n - k0);
    // ---- 1. panel in registers
    int rows[2] = {k0 + tid, k0 + tid + kMB};
    T v[2][NB];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < NB; ++j)
        v[i][j] = (rows[i] < n && j < nb) ? a[(int64_t)(k0 + j) * n + rows[i]] : T(0);
#pragma unroll
    for (int j = 0; j < NB; ++j) {       // unrolled: every register index and update mask is static
      if (j >= nb) break;
      const int kk = k0 + j;
      T s = T(-2);
      int idx = 0x7fffffff;
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int r = rows[i];
        if (r >= kk && r < n) {
          const T x = v[i][j];
          const T sc = (r == kk) ? ((x != x) ? T(INFINITY) : gbs_abs(x)) : pivot_score(x);
          if (better(sc, r, s, idx)) { s = sc; idx = r; }
        }
      }
      cta_argmax(s, idx, rv, ri);
      const int p = idx;
      // the two rows involved are published by their owners only: row kk
      // lives in thread j (slot 0), row p in thread (p - k0) mod kMB
      const int p_owner = (p - k0) & (kMB - 1);
      const bool p_hi = (p - k0) >= kMB;
      if (tid == p_owner) {
#pragma unroll
        for (int jj = 0; jj < NB; ++jj) prow[jj] = p_hi ? v[1][jj] : v[0][jj];
      }
      if (tid == j) {
#pragma unroll
        for (int jj = 0; jj < NB; ++jj) krow[jj] = v[0][jj];
      }
      __syncthreads();
      const T pv = prow[j];
      const bool swap = pv != T(0);
      if (tid == 0) spiv[j] = p;
      if (!swap && first_zero < 0) first_zero = kk;
      const T* u = swap ? prow : krow;
      if (swap && p != kk) {
        if (tid == j) {
#pragma unroll
          for (int jj = 0; jj < NB; ++jj) v[0][jj] = prow[jj];
        }
        if (tid == p_owner) {
          if (p_hi) {
#pragma unroll
            for (int jj = 0; jj < NB; ++jj) v[1][jj] = krow[jj];
          } else {
#pragma unroll
            for (int jj = 0; jj < NB; ++jj) v[0][jj] = krow[jj];
          }
        }
      }
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        if (rows[i] > kk && rows[i] < n) {
          if (swap) v[i][j] = v[i][j] / pv;
          const T l = v[i][j];
#pragma unroll
          for (int jj = j + 1; jj < NB; ++jj) v[i][jj] = fma(-l, u[jj], v[i][jj]);
        }
      }
      // prow / krow are rewritten only after the next column's argmax, whose
      // first barrier orders these reads before those writes
    }
    // write the panel back; L (and L11) transposed to shared memory
#pragma unroll
    for (int i = 0; i < 2; ++i)
      if (rows[i] < n)
#pragma unroll
        for (int j = 0; j < NB; ++j)
          if (j < nb) {
            a[(int64_t)(k0 + j) * n + rows[i]] = v[i][j];
            lt[j][rows[i]] = v[i][j];
          }
    for (int r = k0 + tid; r < n; r += kMB) perm[r] = r;
    __syncthreads();
    if (tid < nb) piv[k0 + tid] = spiv[tid];
    if (tid == 0)
      for (int j = 0; j < nb; ++j) {
        const int p = spiv[j];
        const int t = perm[k0 + j];
        perm[k0 + j] = perm[p];
        perm[p] = t;
      }
    __syncthreads();
    // ---- 2. row exchanges on the other columns: new row r = old row perm[r]
    // for the panel's rows and for the pivot rows below it; each warp moves
    // kSwapCols columns at a time (all loads issued before the stores)
    {
      constexpr int Q = (2 * NB + 31) / 32;
      constexpr int kSwapCols = 8;
      int dst[Q], src[Q];
#pragma unroll
      for (int q = 0; q < Q; ++q) {
        const int t = lane + 32 * q;
        int row = -1;
        if (t < nb) row = k0 + t;
        else if (t >= NB && t - NB < nb && spiv[t - NB] >= k0 + nb) row = spiv[t - NB];
        dst[q] = row;
        src[q] = row >= 0 ? perm[row] : 0;
      }
      const int ncols = n - nb;
      for (int cc0 = warp * kSwapCols; cc0 < ncols; cc0 += kSwapCols * (kMB / 32)) {
        T val[kSwapCols][Q];
#pragma unroll
        for (int b = 0; b < kSwapCols; ++b) {
          const int cc = cc0 + b;
          const int c = cc < k0 ? cc : cc + nb;
#pragma unroll
          for (int q = 0; q < Q; ++q)
            val[b][q] = (cc < ncols && dst[q] >= 0) ? a[(int64_t)c * n + src[q]] : T(0);
        }
        __syncwarp();
#pragma unroll
        for (int b = 0; b < kSwapCols; ++b) {
          const int cc = cc0 + b;
          const int c = cc < k0 ? cc : cc + nb;
#pragma unroll
          for (int q = 0; q < Q; ++q)
            if (cc < ncols && dst[q] >= 0) a[(int64_t)c * n + dst[q]] = val[b][q];
        }
        __syncwarp();
      }
    }
    if (k0 + nb >= n) break;            // last panel: no trailing matrix
    __syncthreads();
    // ---- 3. U12 = L11^-1 A12 (unit lower), one column per thread
    for (int c = k0 + NB + tid; c < n; c += kMB) {
      T* col = a + (int64_t)c * n + k0;
      T x[NB];
#pragma unroll
      for (int j = 0; j < NB; ++j) x[j] = col[j];
#pragma unroll
      for (int j = 0; j < NB; ++j) {
        asm volatile("" ::: "memory");   // keep each step's L11 loads next to their use (register pressure)
#pragma unroll
        for (int i = j + 1; i < NB; ++i) x[i] = fma(-lt[j][k0 + i], x[j], x[i]);
      }
#pragma unroll
      for (int j = 0; j < NB; ++j) col[j] = x[j];
    }
    __syncthreads();
    // ---- 4. A22 -= L21 U12
    const int r_begin = k0 + NB;
    for (int c0 = r_begin; c0 < n; c0 += kCW) {
      const int cw = min(kCW, n - c0);
      for (int e = tid; e < NB * kCW; e += kMB) {
        const int kq = e % NB, c = e / NB;
        ub[kq][c] = c < cw ? a[(int64_t)(c0 + c) * n + k0 + kq] : T(0);
      }
      __syncthreads();
      const int cb = warp * 8;
      if (cb < cw) {
        for (int r0 = r_begin; r0 < n; r0 += 128) {
          const int ng = min(4, (n - r0 + 31) >> 5);      // 32-row groups inside the matrix (warp-uniform)
          T acc[4][8];
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int r = r0 + lane + 32 * i;
#pragma unroll
            for (int c = 0; c < 8; ++c)
              acc[i][c] = (i < ng && r < n && cb + c < cw) ? a[(int64_t)(c0 + cb + c) * n + r] : T(0);
          }
#pragma unroll
          for (int kq = 0; kq < NB; ++kq) {
            asm volatile("" ::: "memory");
            T bv[8];
#pragma unroll
            for (int c = 0; c < 8; ++c) bv[c] = ub[kq][cb + c];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
              if (i < ng) {
                const int r = r0 + lane + 32 * i;
                const T av = r < n ? lt[kq][r] : T(0);
#pragma unroll
                for (int c = 0; c < 8; ++c) acc[i][c] = fma(-av, bv[c], acc[i][c]);
              }
            }
          }
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int r = r0 + lane + 32 * i;
            if (i < ng && r < n)
#pragma unroll
              for (int c = 0; c < 8; ++c)
                if (cb + c < cw) a[(int64_t)(c0 + cb + c) * n + r] = acc[i][c];
          }
        }
      }
      __syncthreads();
    }
  }
  __syncthreads();
  return first_zero;
}

// x[i] - sum_{j < nb} a(i, b0 + j) x[b0 + j], the nb <= 32 loads issued together
template <typename TA, typename T>
__device__ __forceinline__ T block_dot_sub(const TA* __restrict__ a, int n, int i, int b0, int nb, const T* x)
{
  T v[32];
#pragma unroll
  for (int j = 0; j < 32; ++j) v[j] = j < nb ? T(a[(int64_t)(b0 + j) * n + i]) : T(0);
  T s[4] = {x[i], T(0), T(0), T(0)};
#pragma unroll
  for (int j = 0; j < 32; ++j)
    if (j < nb) s[j & 3] = fma(-v[j], x[b0 + j], s[j & 3]);
  return (s[0] + s[1]) + (s[2] + s[3]);
}

// x <- U^-1 L^-1 P x for PA = LU in a (ld n); x in shared memory.  Blocked by
// 32 rows: warp 0 solves each diagonal block with shuffles from a register copy
// of its rows, then every thread updates the rows beyond it.  The arithmetic
// is T's; the factors may be stored narrower (TA = float with T = double: FP32
// factors applied in FP64, as GMRES-IR's preconditioner needs).
template <typename T, typename TA = T>
__device__ void cta_lu_solve_blocked(const TA* __restrict__ a, int n, const int* __restrict__ piv, T* x)
{
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (warp == 0)                        // row interchanges in order, pivots fetched 32 at a time
    for (int k0 = 0; k0 < n; k0 += 32) {
      const int pl = k0 + lane < n ? piv[k0 + lane] : 0;
      const int cnt = min(32, n - k0);
      for (int q = 0; q < cnt; ++q) {
        const int p = __shfl_sync(0xffffffffu, pl, q);
        if (lane == 0 && p != k0 + q) { const T t = x[k0 + q]; x[k0 + q] = x[p]; x[p] = t; }
      }
    }
  __syncthreads();
  // forward: unit lower
  for (int b0 = 0; b0 < n; b0 += 32) {
    const int nb = min(32, n - b0);
    if (warp == 0) {
      T row[32];
#pragma unroll
      for (int j = 0; j < 32; ++j) row[j] = (lane < nb && j < lane) ? T(a[(int64_t)(b0 + j) * n + b0 + lane]) : T(0);
      T xi = lane < nb ? x[b0 + lane] : T(0);
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const T xj = __shfl_sync(0xffffffffu, xi, j);
        if (j < nb && lane > j) xi = fma(-row[j], xj, xi);
      }
      if (lane < nb) x[b0 + lane] = xi;
    }
    __syncthreads();
    for (int i = b0 + nb + tid; i < n; i += kMB) x[i] = block_dot_sub<TA, T>(a, n, i, b0, nb, x);
    __syncthreads();
  }
  // backward: upper, non-unit
  for (int b1 = n; b1 > 0; b1 -= 32) {
    const int b0 = max(0, b1 - 32), nb = b1 - b0;
    if (warp == 0) {
      T row[32];
#pragma unroll
      for (int j = 0; j < 32; ++j) row[j] = (lane < nb && j >= lane && j < nb) ? T(a[(int64_t)(b0 + j) * n + b0 + lane]) : T(0);
      T xi = lane < nb ? x[b0 + lane] : T(0);
#pragma unroll
      for (int j = 31; j >= 0; --j) {
        if (j < nb) {
          if (lane == j) xi = xi / row[j];
          const T xj = __shfl_sync(0xffffffffu, xi, j);
          if (lane < j) xi = fma(-row[j], xj, xi);
        }
      }
      if (lane < nb) x[b0 + lane] = xi;
    }
    __syncthreads();
    for (int i = tid; i < b0; i += kMB) x[i] = block_dot_sub<TA, T>(a, n, i, b0, nb, x);
    __syncthreads();
  }
}

}  // namespace mb
}  // namespace gbs
