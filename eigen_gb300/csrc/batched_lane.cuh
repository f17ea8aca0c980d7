// Small-system kernels with G lanes per system (G in {1, 2, 4, 8, 16}): a
// warp factors and solves 32 / G systems at once.
//
// On GB300 an FP64 warp instruction holds its sub-partition's FP64 unit for
// 64 cycles whatever the number of active lanes (about 19 cycles per warp
// instruction for the SM once all four sub-partitions issue), so the cost of
// a small factorization is its count of FP64 warp instructions.  With one
// warp per system (batched_kernel), every per-column step (square root,
// division, pivot reduction) is a full warp instruction serving one system,
// and lanes beyond n idle; with G lanes per system the same instruction
// serves 32 / G systems and the trailing updates keep almost every lane busy.
//
// Layout: each warp has its own shared-memory slice; the element (r, c) of
// the warp's system s sits at ((c * R + r / G) * kLS + s * G + r % G), R =
// ceil(maxn / G) rows per lane, so lane s * G + g owns rows g, g + G, ...
// Accesses of one (row slot, column) by all lanes are consecutive (no bank
// conflicts).  Each lane loads and stores its own rows.
//
// Arithmetic follows the reference's unblocked algorithms:
//  * LU: unblocked_lu (PartialPivLU.h:365-409): first maximum of |a_ik|
//    (Visitor.h:173-186) as the pivot, whole-row interchanges, column
//    divided by the pivot, rank-1 update; a zero pivot is recorded and the
//    column left unscaled.  The pivot search compares the magnitudes' bit
//    patterns as integers (same order as the FP64 comparison, no FP64
//    instruction).
//  * LLT: left-looking like the reference's unblocked LLT (LLT.h:305-328):
//    x = a_kk - ||l_k||^2 is checked before column k changes, so a failing
//    column and the columns right of it keep their input values; the column
//    is scaled by the reciprocal of its diagonal.
//  * the solves use the reciprocals of the diagonal computed once per system.
#pragma once

#include <cstdint>

#include "gbs_common.cuh"

namespace gbs {

constexpr int kLS = 33;   // lane stride of the interleaved layouts (32 lanes + 1 pad)

struct BatchItem {
  int64_t a_off;   // element offset of the matrix (column-major n x n, ld = n)
  int64_t b_off;   // element offset of its right-hand side (n)
  int n;
  int kind;        // 0 = LLT, 1 = LU
  int id;          // position in the caller's batch
  int pad;
};

template <typename T>
struct PivotKey;
template <>
struct PivotKey<double> {
  using U = unsigned long long;
  static constexpr U kAbs = 0x7fffffffffffffffull, kInf = 0x7ff0000000000000ull;
  static __device__ __forceinline__ U bits(double x) { return (U)__double_as_longlong(x); }
};
template <>
struct PivotKey<float> {
  using U = unsigned;
  static constexpr U kAbs = 0x7fffffffu, kInf = 0x7f800000u;
  static __device__ __forceinline__ U bits(float x) { return __float_as_uint(x); }
};

// Pivot key of a(r, k), larger wins and ties go to the lower row: |a| + 2 for
// numbers (the bit pattern of a non-negative float orders like its value), 1
// for a NaN, except in row k itself, where a NaN scores as +inf (pivot_score
// and the first-element rule of the reference's visitor).  0 = no candidate;
// key 2 is an exact zero.
template <typename T>
__device__ __forceinline__ typename PivotKey<T>::U pivot_key(T x, bool first)
{
  using K = PivotKey<T>;
  const typename K::U m = K::bits(x) & K::kAbs;
  if (m > K::kInf) return first ? K::kInf + 2 : 1;
  return m + 2;
}

template <int G, typename U>
__device__ __forceinline__ void group_argmax(U& key, int& idx, unsigned gmask)
{
#pragma unroll
  for (int off = G / 2; off > 0; off >>= 1) {
    const U ko = __shfl_xor_sync(gmask, key, off);
    const int io = __shfl_xor_sync(gmask, idx, off);
    if (ko > key || (ko == key && io < idx)) { key = ko; idx = io; }
  }
}

template <int G>
__device__ __forceinline__ void group_sync(unsigned gmask)
{
  if constexpr (G > 1) __syncwarp(gmask);
}

// Shared memory of one warp of lu_group_kernel: the matrices, the right-hand
// sides and the reciprocals of U's diagonal.
template <typename T>
__host__ __device__ inline size_t lu_group_smem(int maxn, int G)
{
  const int R = (maxn + G - 1) / G;
  return (size_t)(maxn * R + 2 * R) * kLS * sizeof(T);
}

// Shared memory of one warp of llt_lane_kernel: packed lower triangles, the
// right-hand sides and the reciprocals of L's diagonal.
template <typename T>
__host__ __device__ inline size_t llt_lane_smem(int maxn)
{
  return (size_t)(maxn * (maxn + 1) / 2 + 2 * maxn) * kLS * sizeof(T);
}

// PartialPivLU + solve, G lanes per system, one warp per CTA.  The warp takes
// 32 / G consecutive items of the (cost-sorted) list per atomicAdd.
template <typename T, int G>
__global__ void __launch_bounds__(32)
lu_group_kernel(const BatchItem* __restrict__ items, int count, int maxn, T* __restrict__ A, T* __restrict__ Bv,
                int* __restrict__ info, int* __restrict__ piv, int* __restrict__ counter)
{
  using U = typename PivotKey<T>::U;
  constexpr int SPW = 32 / G;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int s = lane / G, g = lane % G;
  const unsigned gmask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (s * G));
  const int R = (maxn + G - 1) / G;
  const int cs = R * kLS;                          // column stride
  T* S = (T*)smem_raw;
  T* Bs = S + (size_t)maxn * cs;
  T* Ds = Bs + cs;
  // own row slot t of column c: S[c * cs + t * kLS + lane]; row r of the
  // system (any lane): S[c * cs + (r / G) * kLS + s * G + r % G].  A lane
  // loads and stores its own rows, so only the group's lanes synchronise.
  for (;;) {
    int base = 0;
    if (lane == 0) base = atomicAdd(counter, SPW);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= count) break;
    const bool act = base + s < count;
    const BatchItem it = items[act ? base + s : base];
    const int n = act ? it.n : 0;
    // each lane loads its own rows g, g + G, ... (a group reads G consecutive rows)
    {
      const T* a = A + it.a_off + g;
      for (int c = 0; c < n; ++c)
        for (int t = 0; t < R && g + G * t < n; ++t) S[c * cs + t * kLS + lane] = a[c * n + G * t];
      for (int t = 0; t < R && g + G * t < n; ++t) Bs[t * kLS + lane] = Bv[it.b_off + g + G * t];
    }
    int* pv = piv + it.b_off;
    int status = -1;
    for (int k = 0; k < n; ++k) {
      const int tk = k >= g ? (k - g + G - 1) / G : 0;             // first own slot with row >= k
      U bk = 0;
      int bi = 0x7fffffff;
      for (int t = tk; t < R; ++t) {
        const int r = g + G * t;
        if (r >= n) break;
        const U key = pivot_key(S[k * cs + t * kLS + lane], r == k);
        if (key > bk) { bk = key; bi = r; }
      }
      group_argmax<G>(bk, bi, gmask);
      const int p = bi;
      const bool nz = bk != U(2);
      if (g == 0) pv[k] = p;
      group_sync<G>(gmask);                                         // the previous update is visible
      if (nz && p != k) {
        const int ok = (k / G) * kLS + s * G + k % G, op = (p / G) * kLS + s * G + p % G;
        for (int c = g; c < n; c += G) {
          const T x = S[c * cs + ok];
          S[c * cs + ok] = S[c * cs + op];
          S[c * cs + op] = x;
        }
        if (g == 0) {                                               // P b (PartialPivLU.h:233)
          const T x = Bs[ok];
          Bs[ok] = Bs[op];
          Bs[op] = x;
        }
      }
      group_sync<G>(gmask);                                         // row k is final
      const int t1 = k + 1 > g ? (k + 1 - g + G - 1) / G : 0;       // first own slot with row > k
      if (nz) {
        const T d = S[k * cs + (k / G) * kLS + s * G + k % G];
        for (int t = t1; t < R && g + G * t < n; ++t) S[k * cs + t * kLS + lane] /= d;
      } else if (status < 0) {
        status = k;
      }
      // trailing update, four columns at a time: all loads of a block before
      // its stores (the compiler cannot tell that the rows do not alias)
      const T* uk = S + (k / G) * kLS + s * G + k % G;             // row k: column c at uk[c * cs]
      int c = k + 1;
      for (; c + 4 <= n; c += 4) {
        const T u0 = uk[c * cs], u1 = uk[(c + 1) * cs], u2 = uk[(c + 2) * cs], u3 = uk[(c + 3) * cs];
        for (int t = t1; t < R && g + G * t < n; ++t) {
          const T l = S[k * cs + t * kLS + lane];
          T* ar = S + c * cs + t * kLS + lane;
          const T a0 = ar[0], a1 = ar[cs], a2 = ar[2 * cs], a3 = ar[3 * cs];
          ar[0] = fma(-l, u0, a0);
          ar[cs] = fma(-l, u1, a1);
          ar[2 * cs] = fma(-l, u2, a2);
          ar[3 * cs] = fma(-l, u3, a3);
        }
      }
      for (; c < n; ++c) {
        const T u = uk[c * cs];
        for (int t = t1; t < R && g + G * t < n; ++t) {
          T* ar = S + c * cs + t * kLS + lane;
          *ar = fma(-S[k * cs + t * kLS + lane], u, *ar);
        }
      }
    }
    // reciprocals of U's diagonal (own rows)
    for (int t = 0; t < R && g + G * t < n; ++t) {
      const int r = g + G * t;
      Ds[t * kLS + lane] = T(1) / S[r * cs + t * kLS + lane];
    }
    group_sync<G>(gmask);
    // L y = P b (unit lower; b was permuted with the rows)
    for (int k = 0; k < n; ++k) {
      const T yk = Bs[(k / G) * kLS + s * G + k % G];
      const int t1 = k + 1 > g ? (k + 1 - g + G - 1) / G : 0;
      for (int t = t1; t < R && g + G * t < n; ++t)
        Bs[t * kLS + lane] = fma(-S[k * cs + t * kLS + lane], yk, Bs[t * kLS + lane]);
      group_sync<G>(gmask);
    }
    // U x = y
    for (int k = n - 1; k >= 0; --k) {
      const int ok = (k / G) * kLS + s * G + k % G;
      if (g == k % G) Bs[ok] *= Ds[ok];
      group_sync<G>(gmask);
      const T xk = Bs[ok];
      for (int t = 0; t < R && g + G * t < k; ++t) Bs[t * kLS + lane] = fma(-S[k * cs + t * kLS + lane], xk, Bs[t * kLS + lane]);
    }
    if (act && g == 0) info[it.id] = status;
    {
      T* a = A + it.a_off + g;
      for (int c = 0; c < n; ++c)
        for (int t = 0; t < R && g + G * t < n; ++t) a[c * n + G * t] = S[c * cs + t * kLS + lane];
      for (int t = 0; t < R && g + G * t < n; ++t) Bv[it.b_off + g + G * t] = Bs[t * kLS + lane];
    }
    __syncwarp();                                                   // the group's reads are done before the next loads
  }
}

// LLT + solve, one lane per system (32 systems per warp), packed lower
// triangles: element (r, c), r >= c, at slot c * maxn - c (c - 1) / 2 + r - c.
// Every lane works on its own system only: it loads and stores its matrix
// itself (no warp synchronisation), and the inner loops accumulate four rows
// in registers over two columns at a time (loads ahead of the FMAs).
// One system of llt_lane_kernel, entirely in this lane's slots L[slot * kLS].
template <typename T>
__device__ __forceinline__ void llt_lane_system(const BatchItem& it, int maxn, T* const L, T* __restrict__ A,
                                                T* __restrict__ Bv, int* __restrict__ info)
{
  T* const b = L + (size_t)(maxn * (maxn + 1) / 2) * kLS;
  T* const Ds = b + (size_t)maxn * kLS;
  auto col = [maxn](int c) { return c * maxn - (c * (c - 1)) / 2; };
  const int n = it.n;
  T* const a = A + it.a_off;
  T* const bv = Bv + it.b_off;
  // lower triangle, column by column (slots of a column are consecutive)
  for (int c = 0; c < n; ++c) {
    const T* src = a + c * n + c;
    T* d = L + col(c) * kLS;
    const int m = n - c;
    int r = 0;
    for (; r + 4 <= m; r += 4) {
      const T x0 = src[r], x1 = src[r + 1], x2 = src[r + 2], x3 = src[r + 3];
      d[r * kLS] = x0;
      d[(r + 1) * kLS] = x1;
      d[(r + 2) * kLS] = x2;
      d[(r + 3) * kLS] = x3;
    }
    for (; r < m; ++r) d[r * kLS] = src[r];
  }
  for (int r = 0; r < n; ++r) b[r * kLS] = bv[r];
  int status = -1;
  const int step0 = (maxn - 1) * kLS;                             // slot(k, j + 1) - slot(k, j) = (maxn - 1 - j) kLS
  for (int k = 0; k < n; ++k) {
    // x = a_kk - ||l_k||^2 first: a failing column is left as it was
    T p0 = T(0), p1 = T(0);
    const T* pj = L + k * kLS;                                    // L(k, 0)
    int st = step0;
    int j = 0;
    for (; j + 2 <= k; j += 2) {
      const T l0 = pj[0];
      pj += st;
      st -= kLS;
      const T l1 = pj[0];
      pj += st;
      st -= kLS;
      p0 = fma(l0, l0, p0);
      p1 = fma(l1, l1, p1);
    }
    if (j < k) p0 = fma(pj[0], pj[0], p0);
    T* ck = L + col(k) * kLS;                                     // (k + i, k) at ck[i * kLS]
    const T d = ck[0] - (p0 + p1);
    if (d <= T(0)) { status = k; break; }                         // a NaN goes on, as in the reference
    const T x = sqrt(d);
    const T rx = T(1) / x;
    ck[0] = x;
    Ds[k * kLS] = rx;
    // a_ik -= sum_j l_ij l_kj for rows k+i0 .. k+i0+3
    for (int i0 = 1; i0 < n - k; i0 += 4) {
      const int m = n - k - i0;
      T a0 = ck[i0 * kLS];
      T a1 = m > 1 ? ck[(i0 + 1) * kLS] : T(0);
      T a2 = m > 2 ? ck[(i0 + 2) * kLS] : T(0);
      T a3 = m > 3 ? ck[(i0 + 3) * kLS] : T(0);
      const T* q = L + k * kLS;                                   // L(k, jj); rows below at q[i * kLS]
      int sq = step0;
      int jj = 0;
      for (; jj + 2 <= k; jj += 2) {
        const T* q1 = q + sq;
        const T l0 = q[0], l1 = q1[0];
        const T* r0 = q + i0 * kLS;
        const T* r1 = q1 + i0 * kLS;
        const T c00 = r0[0], c01 = r0[kLS], c02 = r0[2 * kLS], c03 = r0[3 * kLS];
        const T c10 = r1[0], c11 = r1[kLS], c12 = r1[2 * kLS], c13 = r1[3 * kLS];
        a0 = fma(-c00, l0, a0);
        a1 = fma(-c01, l0, a1);
        a2 = fma(-c02, l0, a2);
        a3 = fma(-c03, l0, a3);
        a0 = fma(-c10, l1, a0);
        a1 = fma(-c11, l1, a1);
        a2 = fma(-c12, l1, a2);
        a3 = fma(-c13, l1, a3);
        q = q1 + (sq - kLS);
        sq -= 2 * kLS;
      }
      if (jj < k) {
        const T l0 = q[0];
        const T* r0 = q + i0 * kLS;
        a0 = fma(-r0[0], l0, a0);
        a1 = fma(-r0[kLS], l0, a1);
        a2 = fma(-r0[2 * kLS], l0, a2);
        a3 = fma(-r0[3 * kLS], l0, a3);
      }
      ck[i0 * kLS] = a0 * rx;
      if (m > 1) ck[(i0 + 1) * kLS] = a1 * rx;
      if (m > 2) ck[(i0 + 2) * kLS] = a2 * rx;
      if (m > 3) ck[(i0 + 3) * kLS] = a3 * rx;
    }
  }
  if (status < 0) {
    // L y = b: y_i = (b_i - sum_{j<i} l_ij y_j) / l_ii, column-oriented
    for (int k = 0; k < n; ++k) {
      const T* ck = L + col(k) * kLS;
      const T yk = b[k * kLS] * Ds[k * kLS];
      b[k * kLS] = yk;
      int i = 1;
      for (; i + 4 <= n - k; i += 4) {
        const T c0 = ck[i * kLS], c1 = ck[(i + 1) * kLS], c2 = ck[(i + 2) * kLS], c3 = ck[(i + 3) * kLS];
        const T b0 = b[(k + i) * kLS], b1 = b[(k + i + 1) * kLS], b2 = b[(k + i + 2) * kLS], b3 = b[(k + i + 3) * kLS];
        b[(k + i) * kLS] = fma(-c0, yk, b0);
        b[(k + i + 1) * kLS] = fma(-c1, yk, b1);
        b[(k + i + 2) * kLS] = fma(-c2, yk, b2);
        b[(k + i + 3) * kLS] = fma(-c3, yk, b3);
      }
      for (; i < n - k; ++i) b[(k + i) * kLS] = fma(-ck[i * kLS], yk, b[(k + i) * kLS]);
    }
    // L^T x = y: x_k = (y_k - sum_{i>k} l_ik x_i) / l_kk, a dot product down column k
    for (int k = n - 1; k >= 0; --k) {
      const T* ck = L + col(k) * kLS;
      T s0 = b[k * kLS], s1 = T(0);
      int i = 1;
      for (; i + 2 <= n - k; i += 2) {
        const T c0 = ck[i * kLS], c1 = ck[(i + 1) * kLS];
        const T x0 = b[(k + i) * kLS], x1 = b[(k + i + 1) * kLS];
        s0 = fma(-c0, x0, s0);
        s1 = fma(-c1, x1, s1);
      }
      if (i < n - k) s0 = fma(-ck[i * kLS], b[(k + i) * kLS], s0);
      b[k * kLS] = (s0 + s1) * Ds[k * kLS];
    }
  }
  info[it.id] = status;
  // write back the lower triangle (the strict upper part is the caller's)
  for (int c = 0; c < n; ++c) {
    T* dst = a + c * n + c;
    const T* sl = L + col(c) * kLS;
    const int m = n - c;
    int r = 0;
    for (; r + 4 <= m; r += 4) {
      const T x0 = sl[r * kLS], x1 = sl[(r + 1) * kLS], x2 = sl[(r + 2) * kLS], x3 = sl[(r + 3) * kLS];
      dst[r] = x0;
      dst[r + 1] = x1;
      dst[r + 2] = x2;
      dst[r + 3] = x3;
    }
    for (; r < m; ++r) dst[r] = sl[r * kLS];
  }
  if (status < 0)
    for (int r = 0; r < n; ++r) bv[r] = b[r * kLS];
}

template <typename T>
__global__ void __launch_bounds__(32)
llt_lane_kernel(const BatchItem* __restrict__ items, int count, int maxn, T* __restrict__ A, T* __restrict__ Bv,
                int* __restrict__ info, int* __restrict__ piv, int* __restrict__ counter)
{
  (void)piv;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  T* const L = (T*)smem_raw + lane;                                 // this lane's slots, stride kLS
  for (;;) {
    int base = 0;
    if (lane == 0) base = atomicAdd(counter, 32);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= count) break;
    if (base + lane < count) llt_lane_system(items[base + lane], maxn, L, A, Bv, info);
  }
}

}  // namespace gbs
